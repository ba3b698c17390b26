"""The oracle's genealogy update (ora_ug_run, the no-migration model of
updategenealogy, update_gtree.cpp:723-966) against the reference's own run
by the harness (golden_ug.npz): every proposal's decision, topology and tmrca
flags, G.pdg and p(G), and the final genealogies, on host threads too."""
import numpy as np
import pytest

from ima2p_gb300 import popmodel
from ima2p_gb300.synth import Genealogy, LabelledGenealogy
from oracle import pyoracle as O
from tests._golden import load


class _Hky:
    def __init__(self, seq, mult, totsites):
        self.seq, self.mult, self.totsites = seq, mult, totsites


def _case():
    d = load("golden_ug.npz")
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
    for l, k in enumerate(kinds):
        if k == "is":
            seq = d["seq_%d" % l]
            loci.append(("is", seq, O.is_sumlogk(seq, base[l].g)[1]))
        else:
            loci.append(("hky", _Hky(d["seq_%d" % l], d["mult_%d" % l], int(d["totsites_%d" % l]))))
    nch = len(d["betas"])
    samps = d["samps"].astype(np.int32)
    ul = O.UgLoci(loci, np.ones(len(kinds)), samps)
    u = np.tile(d["us"], nch)
    kap = np.tile([float(d["kappa"]) if k == "hky" else 1.0 for k in kinds], nch)
    pi = np.array([d["pi_%d" % l] if k == "hky" else np.zeros(4) for l, k in enumerate(kinds)] * nch)
    th_max, th_min, _, _, _ = popmodel.priors(pm, float(d["thetaprior"]), 0.0)
    gens = [[base[l] for l in range(len(kinds))] for _ in range(nch)]
    return d, pm, ul, u, kap, pi, th_max, th_min, gens


@pytest.mark.parametrize("nthreads", [1, 3])
def test_oracle_updategenealogy_matches_reference(nthreads):
    d, pm, ul, u, kap, pi, th_max, th_min, gens = _case()
    nch, nl, ns = len(d["betas"]), len(d["kinds"]), int(d["nsweeps"])
    rngs = [O.UgRng(int(s)) for s in d["seeds"]]
    tv = np.tile(d["tv0"], (nch, 1))
    st, res, resd, pdg, probg, fin = O.ug_run(pm, th_max, th_min, ul, gens, tv, d["betas"], u, kap, pi, ns, rngs,
                                              nthreads=nthreads)
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


def test_oracle_generator_state_carries_over():
    """Two calls of 5 sweeps = one call of 10: the generators (MT position,
    normdev's cached deviate, bitran's register) come back advanced."""
    d, pm, ul, u, kap, pi, th_max, th_min, gens = _case()
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
