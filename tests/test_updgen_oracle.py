"""The oracle's genealogy update (ora_ug_run, the no-migration model of
updategenealogy, update_gtree.cpp:723-966) against the reference's own runs
by the harness: IS and HKY loci (golden_ug.npz), and stepwise loci among them
with finishSWupdateA's allele proposals (golden_ug_sw.npz): every proposal's
decision, topology and tmrca flags, G.pdg and p(G), and the final
genealogies and alleles, on host threads too."""
import numpy as np
import pytest

from ima2p_gb300 import popmodel
from ima2p_gb300.synth import Genealogy, LabelledGenealogy
from oracle import pyoracle as O
from tests._golden import load


class _Hky:
    def __init__(self, seq, mult, totsites):
        self.seq, self.mult, self.totsites = seq, mult, totsites


def _case(name="golden_ug.npz"):
    d = load(name)
    npops, tree = int(d["npops"]), str(d["tree"])
    pm = popmodel.build(tree, npops, nomig=True)
    kinds = [str(k) for k in d["kinds"]]
    off = d["node_off"]
    base = []
    for l in range(len(kinds)):
        sl = slice(off[l], off[l + 1])
        down = d["base_down"][sl].astype(np.int32)
        g = Genealogy(d["base_up0"][sl].astype(np.int32), d["base_up1"][sl].astype(np.int32), down,
                      d["base_time"][sl].copy(), int(np.flatnonzero(down == -1)[0]))
        base.append(LabelledGenealogy(g, d["base_pop"][sl].astype(np.int32), [[] for _ in range(len(down))]))
    loci = []
    nch = len(d["betas"])
    alleles = {}
    for l, k in enumerate(kinds):
        if k == "is":
            seq = d["seq_%d" % l]
            loci.append(("is", seq, O.is_sumlogk(seq, base[l].g)[1]))
        elif k == "hky":
            loci.append(("hky", _Hky(d["seq_%d" % l], d["mult_%d" % l], int(d["totsites_%d" % l]))))
        else:
            lo, hi = (int(v) for v in d["arange_%d" % l])
            loci.append(("sw", len(base[l].pop) // 2 + 1, lo, hi))
            for c in range(nch):
                alleles[(c, l)] = d["alleles_%d" % l]
    samps = d["samps"].astype(np.int32)
    ul = O.UgLoci(loci, np.ones(len(kinds)), samps)
    u = np.tile(d["us"], nch)
    kap = np.tile([float(d["kappa"]) if k == "hky" else 1.0 for k in kinds], nch)
    pi = np.array([d["pi_%d" % l] if k == "hky" else np.zeros(4) for l, k in enumerate(kinds)] * nch)
    th_max, th_min, _, _, _ = popmodel.priors(pm, float(d["thetaprior"]), 0.0)
    gens = [[base[l] for l in range(len(kinds))] for _ in range(nch)]
    return d, pm, ul, u, kap, pi, th_max, th_min, gens, alleles


@pytest.mark.parametrize("nthreads", [1, 3])
@pytest.mark.parametrize("fixture", ["golden_ug.npz", "golden_ug_sw.npz"])
def test_oracle_updategenealogy_matches_reference(nthreads, fixture):
    d, pm, ul, u, kap, pi, th_max, th_min, gens, alleles = _case(fixture)
    nch, nl, ns = len(d["betas"]), len(d["kinds"]), int(d["nsweeps"])
    rngs = [O.UgRng(int(s)) for s in d["seeds"]]
    tv = np.tile(d["tv0"], (nch, 1))
    st, res, resd, pdg, probg, fin = O.ug_run(pm, th_max, th_min, ul, gens, tv, d["betas"], u, kap, pi, ns, rngs,
                                              nthreads=nthreads, alleles=alleles)
    assert st == 0
    ref = d["res"]
    # the harness runs chain by chain, each chain's sweeps in order
    got = np.concatenate([np.column_stack([np.full(ns * nl, c), np.tile(np.arange(nl), ns),
                                           res[c].reshape(-1, 3), resd[c].reshape(-1, 2)]) for c in range(nch)])
    assert np.array_equal(got[:, :5], ref[:, :5])
    # the IS restatement agrees with the reference's likelihoodIS to an ulp
    # or two (the oracle's own golden bar is 1e-13 relative)
    np.testing.assert_allclose(got[:, 5], ref[:, 5], rtol=1e-13, atol=0)
    np.testing.assert_allclose(got[:, 6], ref[:, 6], rtol=1e-13, atol=0)
    for k, f in enumerate(("up0", "up1", "down", "pop")):
        np.testing.assert_array_equal(fin[(0, 1, 2, 4)[k]], d["final_" + f])
    edge = fin[2] != -1  # the root edge's time is a placeholder (the harness writes TIMEMAX)
    np.testing.assert_array_equal(fin[3][edge], d["final_time"][edge])
    if "final_A" in d.files:  # the stepwise loci's alleles, chain-locus order
        kinds = [str(k) for k in d["kinds"]]
        off = d["node_off"]
        got, k = [], 0
        for c in range(nch):
            for l in range(nl):
                m = int(off[l + 1] - off[l])
                if kinds[l] == "sw":
                    got.append(fin[5][k:k + m])
                k += m
        np.testing.assert_array_equal(np.concatenate(got), d["final_A"])


def test_oracle_generator_state_carries_over():
    """Two calls of 5 sweeps = one call of 10: the generators (MT position,
    normdev's cached deviate, bitran's register) come back advanced."""
    d, pm, ul, u, kap, pi, th_max, th_min, gens, _ = _case()
    nch, nl = len(d["betas"]), len(d["kinds"])
    tv = np.tile(d["tv0"], (nch, 1))
    r1 = [O.UgRng(int(s)) for s in d["seeds"]]
    st, res10, _, _, pg10, fin10 = O.ug_run(pm, th_max, th_min, ul, gens, tv, d["betas"], u, kap, pi, 10, r1)
    assert st == 0
    r2 = [O.UgRng(int(s)) for s in d["seeds"]]
    st, res5, _, _, _, fin5 = O.ug_run(pm, th_max, th_min, ul, gens, tv, d["betas"], u, kap, pi, 5, r2)
    assert st == 0
    np.testing.assert_array_equal(res5, res10[:, :5])
    assert r2[0].mti != O.UgRng(int(d["seeds"][0])).mti
