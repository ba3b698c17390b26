"""The genealogy update of the no-migration model on the device
(ima_gpu_updategenealogy_sweep) against the reference's own updategenealogy
(update_gtree.cpp:723-966), run by the harness on 3 chains x 5 loci (IS and
HKY, golden_ug.npz; SW among IS and HKY, golden_ug_sw.npz), 10 sweeps per
chain from a seed of its own: the same
accepted proposals per chain-locus, the same final genealogies (topology and
population labels exact, times to the last bits of the device's log and
sqrt in the slide's normal deviate), G.pdg and p(G)."""
import numpy as np
import pytest

from ima2p_gb300 import api, popmodel
from tests._golden import load

pytestmark = pytest.mark.gpu


class UgCase:
    def __init__(self, name="golden_ug.npz"):
        d = load(name)
        self.d = d
        self.npops = int(d["npops"])
        self.tree = str(d["tree"])
        self.pm = popmodel.build(self.tree, self.npops, nomig=True)
        self.kinds = [str(k) for k in d["kinds"]]
        self.nl = len(self.kinds)
        self.us = d["us"]
        self.kappa = float(d["kappa"])
        self.betas = d["betas"]
        self.seeds = [int(s) for s in d["seeds"]]
        self.nch = len(self.betas)
        self.nsweeps = int(d["nsweeps"])
        self.samps = d["samps"].astype(np.int32)
        self.off = d["node_off"]
        self.res = d["res"]

    def base(self, li, f):
        return self.d["base_" + f][self.off[li]:self.off[li + 1]]

    def final(self, ci, li, f):
        lens = [self.off[k + 1] - self.off[k] for k in range(self.nl)] * self.nch
        start = sum(lens[:ci * self.nl + li])
        return self.d["final_" + f][start:start + lens[ci * self.nl + li]]

    def context(self):
        from ima2p_gb300.synth import Genealogy, LabelledGenealogy
        ctx = api.Context(0)
        for li, kind in enumerate(self.kinds):
            if kind == "is":
                ctx.add_locus_is(self.d["seq_%d" % li])
            elif kind == "hky":
                ctx.add_locus_hky(self.d["seq_%d" % li], self.d["mult_%d" % li], int(self.d["totsites_%d" % li]))
            else:
                ctx.add_locus_sw(int(self.off[li + 1] - self.off[li] + 1) // 2, 1)
        ctx.set_chains(1, self.nch)
        th_max, th_min, _, _, _ = popmodel.priors(self.pm, float(self.d["thetaprior"]), 0.0)
        ctx.set_popmodel(self.pm, th_max, th_min)
        ci = np.repeat(np.arange(self.nch, dtype=np.int32), self.nl)
        li = np.tile(np.arange(self.nl, dtype=np.int32), self.nch)
        flat = []
        for c in range(self.nch):
            for l in range(self.nl):
                down = self.base(l, "down").astype(np.int32)
                g = Genealogy(self.base(l, "up0").astype(np.int32), self.base(l, "up1").astype(np.int32), down,
                              self.base(l, "time").copy(), int(np.flatnonzero(down == -1)[0]))
                flat.append(LabelledGenealogy(g, self.base(l, "pop").astype(np.int32), [[] for _ in range(len(down))]))
        ctx.set_genealogies(ci, li, np.concatenate([g.g.up0 for g in flat]), np.concatenate([g.g.up1 for g in flat]),
                            np.concatenate([g.g.down for g in flat]), np.concatenate([g.g.time for g in flat]),
                            length=np.full(len(flat), -1.0))
        ctx.set_labels(ci, li, flat)
        ctx.set_locus_pops(np.ones(self.nl), self.samps)
        for c in range(self.nch):
            for l, kind in enumerate(self.kinds):
                if kind == "hky":
                    ctx.set_pi(c, l, self.d["pi_%d" % l])
                elif kind == "sw":
                    ctx.set_alleles(c, l, self.d["alleles_%d" % l])
        ctx.set_betas(self.betas)
        return ctx

    def allele_range(self):
        if "sw" not in self.kinds:
            return None
        return np.array([self.d["arange_%d" % l] if k == "sw" else [0, 0] for l, k in enumerate(self.kinds)],
                        np.int32)

    def rates(self):
        u = np.tile(self.us, self.nch)
        kap = np.where(np.array([k == "hky" for k in self.kinds] * self.nch), self.kappa, 1.0)
        return u, kap


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_FAST])
@pytest.mark.parametrize("fixture", ["golden_ug.npz", "golden_ug_sw.npz"])
def test_updategenealogy_follows_the_reference(precision, fixture):
    """golden_ug_sw.npz puts stepwise loci among them: finishSWupdateA's
    allele proposals and branch terms, and the final alleles."""
    case = UgCase(fixture)
    ctx = case.context()
    u, kap = case.rates()
    rngs = [api.UgRng(s) for s in case.seeds]
    tv = np.tile(case.d["tv0"], (case.nch, 1))
    acc, top, probg = ctx.updategenealogy_sweep(np.arange(case.nch), tv, case.nsweeps, rngs, u, kap,
                                                precision=precision, allele_range=case.allele_range())
    ref_acc = np.zeros((case.nch, case.nl), np.int64)
    ref_top = np.zeros((case.nch, case.nl), np.int64)
    last_pdg = np.zeros((case.nch, case.nl))
    last_probg = np.zeros(case.nch)
    for ci, li, a, t, _, pdg, pg in case.res:
        ci, li = int(ci), int(li)
        ref_acc[ci, li] += int(a)
        ref_top[ci, li] += int(a) * int(t)
        last_pdg[ci, li] = pdg
        last_probg[ci] = pg
    assert np.array_equal(acc, ref_acc)
    assert np.array_equal(top, ref_top)
    np.testing.assert_allclose(probg, last_probg, rtol=0, atol=1e-9)
    pdg = ctx.get_pdg().reshape(case.nch, case.nl)
    tol = 1e-9 if precision == api.PREC_FP64 else 1e-5
    np.testing.assert_allclose(pdg, last_pdg, rtol=0, atol=tol)
    for ci in range(case.nch):
        for li in range(case.nl):
            nlines = int(case.off[li + 1] - case.off[li])
            up0, up1, down, t, pop = ctx.get_genealogy(ci, li, nlines)
            assert np.array_equal(up0, case.final(ci, li, "up0"))
            assert np.array_equal(up1, case.final(ci, li, "up1"))
            assert np.array_equal(down, case.final(ci, li, "down"))
            assert np.array_equal(pop, case.final(ci, li, "pop"))
            edge = down != -1
            np.testing.assert_allclose(t[edge], case.final(ci, li, "time")[edge], rtol=1e-12, atol=0)
    if "final_A" in case.d.files:
        got = [ctx.get_alleles(ci, li, int(case.off[li + 1] - case.off[li]))
               for ci in range(case.nch) for li in range(case.nl) if case.kinds[li] == "sw"]
        assert np.array_equal(np.concatenate(got), case.d["final_A"])
    ctx.close()


def test_updategenealogy_state_carries_between_calls():
    """Ten one-sweep calls give the reference's ten-sweep run: the
    generators, genealogies, partials and p(G) carry over, and an
    evaluation after the sweeps reads the accepted genealogies."""
    case = UgCase()
    ctx = case.context()
    u, kap = case.rates()
    rngs = [api.UgRng(s) for s in case.seeds]
    tv = np.tile(case.d["tv0"], (case.nch, 1))
    acc = np.zeros((case.nch, case.nl), np.int64)
    for _ in range(case.nsweeps):
        a, _, probg = ctx.updategenealogy_sweep(np.arange(case.nch), tv, 1, rngs, u, kap, precision=api.PREC_FP64)
        acc += a
    ref_acc = np.zeros((case.nch, case.nl), np.int64)
    for ci, li, a, *_ in case.res:
        ref_acc[int(ci), int(li)] += int(a)
    assert np.array_equal(acc, ref_acc)
    last_probg = {int(r[0]): r[6] for r in case.res}
    np.testing.assert_allclose(probg, [last_probg[c] for c in range(case.nch)], rtol=0, atol=1e-9)
    ci = np.repeat(np.arange(case.nch, dtype=np.int32), case.nl)
    li = np.tile(np.arange(case.nl, dtype=np.int32), case.nch)
    r, st = ctx.eval(ci, li, u, kap, precision=api.PREC_FP64)
    last = {(int(x[0]), int(x[1])): x[5] for x in case.res}
    np.testing.assert_allclose(r, [last[(int(a), int(b))] for a, b in zip(ci, li)], rtol=0, atol=1e-9)
    ctx.close()


def test_updategenealogy_checkpoint_round_trip(tmp_path):
    """Four sweeps, ima_gpu_checkpoint_write, a fresh context restored from
    the file, six more sweeps: the accepted proposals, final genealogies,
    p(G) and HKY G.pdg of the uninterrupted ten-sweep run (the file carries
    the topologies and level schedules the device changed).  An IS locus's
    G.pdg moves by a constant: the reference takes sum log k! from the first
    genealogy a process evaluates (calc_prob_data.cpp:760-765), and after a
    restart that is the restored one; differences of G.pdg, and with them
    the decisions, do not move."""
    case = UgCase()
    u, kap = case.rates()
    tv = np.tile(case.d["tv0"], (case.nch, 1))
    chains = np.arange(case.nch)
    ctx = case.context()
    rngs = [api.UgRng(s) for s in case.seeds]
    whole, _, pg_whole = ctx.updategenealogy_sweep(chains, tv, 10, rngs, u, kap, precision=api.PREC_FP64)
    want = [ctx.get_genealogy(ci, li, int(case.off[li + 1] - case.off[li]))
            for ci in range(case.nch) for li in range(case.nl)]
    pdg_whole = ctx.get_pdg()
    ctx.close()

    path = str(tmp_path / "ug.ckp")
    ctx = case.context()
    rngs = [api.UgRng(s) for s in case.seeds]
    first, _, _ = ctx.updategenealogy_sweep(chains, tv, 4, rngs, u, kap, precision=api.PREC_FP64)
    ctx.checkpoint_write(path)
    ctx.close()
    ctx = case.context()
    ctx.checkpoint_read(path)
    rest, _, pg = ctx.updategenealogy_sweep(chains, tv, 6, rngs, u, kap, precision=api.PREC_FP64)
    assert np.array_equal(first + rest, whole)
    np.testing.assert_allclose(pg, pg_whole, rtol=0, atol=1e-9)
    hky = np.array([k == "hky" for k in case.kinds])
    np.testing.assert_allclose(ctx.get_pdg()[:, hky], pdg_whole[:, hky], rtol=0, atol=1e-9)
    k = 0
    for ci in range(case.nch):
        for li in range(case.nl):
            got = ctx.get_genealogy(ci, li, int(case.off[li + 1] - case.off[li]))
            for f in (0, 1, 2, 4):
                assert np.array_equal(got[f], want[k][f])
            edge = got[2] != -1
            assert np.array_equal(got[3][edge], want[k][3][edge])
            k += 1
    ctx.close()


def test_updategenealogy_refuses_what_it_does_not_model():
    """Models with migration and SW loci of several markers stay with the
    host: IMA_ERR_STATE / IMA_ERR_ARG before anything runs (an SW locus also
    needs its allele range); no sweeps returns the chains' p(G) summed
    afresh."""
    case = UgCase()
    u, kap = case.rates()
    tv = np.tile(case.d["tv0"], (case.nch, 1))
    ctx = case.context()
    rngs = [api.UgRng(s) for s in case.seeds]
    before = [r.mt.mti for r in rngs]
    acc, top, pg = ctx.updategenealogy_sweep(np.arange(case.nch), tv, 0, rngs, u, kap, precision=api.PREC_FP64)
    assert not acc.any() and not top.any()
    assert [r.mt.mti for r in rngs] == before
    assert np.all(np.isfinite(pg))
    ctx.close()
    # a model with migration
    ctx = api.Context(0)
    for li, kind in enumerate(case.kinds):
        if kind == "is":
            ctx.add_locus_is(case.d["seq_%d" % li])
        else:
            ctx.add_locus_hky(case.d["seq_%d" % li], case.d["mult_%d" % li], int(case.d["totsites_%d" % li]))
    ctx.set_chains(1, case.nch)
    pm = popmodel.build(case.tree, case.npops)
    ctx.set_popmodel(pm, *popmodel.priors(pm, 10.0, 1.0))
    with pytest.raises(api.ImaError) as e:
        ctx.updategenealogy_sweep(np.arange(case.nch), tv, 1, rngs, u, kap)
    assert e.value.code == api.IMA_ERR_STATE
    ctx.close()
    # an SW locus of two linked markers, and one without its allele range
    for markers, rng_ in ((2, np.array([[0, 40]], np.int32)), (1, None)):
        ctx = api.Context(0)
        ctx.add_locus_sw(10, markers)
        ctx.set_chains(1, 2)
        pm = popmodel.build(case.tree, case.npops, nomig=True)
        ctx.set_popmodel(pm, *popmodel.priors(pm, 10.0, 0.0)[:2])
        with pytest.raises(api.ImaError) as e:
            ctx.updategenealogy_sweep(np.arange(2), tv[:2], 1, rngs[:2], np.ones(2), None, allele_range=rng_)
        assert e.value.code == api.IMA_ERR_ARG
        ctx.close()


@pytest.mark.parametrize("kind", ["sw", "hky"])
def test_updategenealogy_matches_the_oracle_on_many_chains(kind):
    """Many chains and more loci than the ring of step slots, so proposals,
    weights (three streams by turns), likelihoods (two) and decisions run
    steps ahead of one another: 48 chains x 9 loci x 3 sweeps on the
    stepwise workload's shapes (5-population tree, 3 sampled) or the HKY
    one's (2 populations), against the oracle's restatement run chain by
    chain.  Accepted proposals per chain-locus, final topologies, population
    labels and alleles exact; node times and p(G) to the last bits of the
    device's log and sqrt in the slide's normal deviate."""
    from ima2p_gb300 import workloads
    from oracle import pyoracle as O

    nch, nsw = 48, 3
    if kind == "sw":
        w = workloads.make_updgen_sw(nloci=9, nch=nch, per_pop=12)
    else:
        w = workloads.make_updgen(nloci=9, nch=nch, ncopies=10, nbases=300)
    nl = len(w.loci)
    pm = popmodel.build(w.tree, w.npops, nomig=True)
    th_max, th_min, _, _, _ = popmodel.priors(pm, 30.0, 0.0)
    ctx = api.Context(0)
    for l, loc in enumerate(w.loci):
        if kind == "sw":
            ctx.add_locus_sw(len(w.base[l].pop) // 2 + 1, 1)
        else:
            ctx.add_locus_hky(loc.seq, loc.mult, loc.totsites)
    ctx.set_chains(1, nch)
    ctx.set_popmodel(pm, th_max, th_min)
    ci = np.repeat(np.arange(nch, dtype=np.int32), nl)
    li = np.tile(np.arange(nl, dtype=np.int32), nch)
    flat = [w.base[l] for _ in range(nch) for l in range(nl)]
    ctx.set_genealogies(ci, li, np.concatenate([g.g.up0 for g in flat]), np.concatenate([g.g.up1 for g in flat]),
                        np.concatenate([g.g.down for g in flat]), np.concatenate([g.g.time for g in flat]),
                        length=np.full(len(flat), -1.0))
    ctx.set_labels(ci, li, flat)
    ctx.set_locus_pops(np.ones(nl), w.samppop)
    for c in range(nch):
        for l in range(nl):
            if kind == "sw":
                ctx.set_alleles(c, l, w.alleles[l])
            else:
                ctx.set_pi(c, l, w.loci[l].pi)
    betas = 1.0 / (1.0 + 0.05 * np.arange(nch))
    ctx.set_betas(betas)
    tv = np.tile(w.tvals, (nch, 1))
    u, kap = np.tile(w.u, nch), np.tile(w.kappa, nch)
    rngs = [api.UgRng(500 + c) for c in range(nch)]
    acc, _, probg = ctx.updategenealogy_sweep(np.arange(nch), tv, nsw, rngs, u, kap, precision=api.PREC_FP64,
                                              allele_range=w.arange)
    if kind == "sw":
        loci = O.UgLoci([("sw", len(w.base[l].pop) // 2 + 1, int(w.arange[l][0]), int(w.arange[l][1]))
                         for l in range(nl)], np.ones(nl), w.samppop)
        al = {(c, l): w.alleles[l] for c in range(nch) for l in range(nl)}
        pis = np.zeros((nch * nl, 4))
    else:
        loci = O.UgLoci([("hky", loc) for loc in w.loci], np.ones(nl), w.samppop)
        al = None
        pis = np.array([w.loci[l].pi for _ in range(nch) for l in range(nl)])
    ro = [O.UgRng(500 + c) for c in range(nch)]
    st, res, _, _, pg, fin = O.ug_run(pm, th_max, th_min, loci, [[w.base[l] for l in range(nl)]] * nch, tv, betas,
                                      u, kap, pis, nsw, ro, nthreads=8, alleles=al)
    assert st == 0
    np.testing.assert_array_equal(acc, res[..., 0].sum(axis=1))
    assert 0 < acc.sum() < nch * nl * nsw
    np.testing.assert_allclose(probg, pg, rtol=0, atol=1e-9)
    o = 0
    for k in range(nch * nl):
        c, l = int(ci[k]), int(li[k])
        nlines = len(flat[k].pop)
        got = ctx.get_genealogy(c, l, nlines)
        sl = slice(o, o + nlines)
        for j in (0, 1, 2, 4):
            np.testing.assert_array_equal(got[j], fin[j][sl])
        nonroot = fin[2][sl] != -1
        np.testing.assert_allclose(got[3][nonroot], fin[3][sl][nonroot], rtol=1e-12)
        if kind == "sw":
            np.testing.assert_array_equal(ctx.get_alleles(c, l, nlines), fin[5][sl])
        o += nlines
    ctx.close()
