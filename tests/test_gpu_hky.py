"""HKY pruning on the GPU: full and dirty-node evaluations with
accept/reject of the partial likelihoods, against the reference's golden
values.  FP64 form: 1e-12 relative.  Float-float form (IMA_PREC_FAST:
partials, coefficients and products as float pairs, exact power-of-two
rescaling, FP64 root sums): per-locus |error| <= HKY_FF_ATOL = 1e-6 absolute.
FP32 form (IMA_PREC_FP32): within HKY_FP32_RTOL of |log L|; bench.py
reports both forms' measured error distributions."""
import numpy as np
import pytest

from ima2p_gb300 import api, synth
from ima2p_gb300.synth import HKYLocus
from oracle import pyoracle as O
from tests._golden import load, trees
from tests._gpu import ctx_with

pytestmark = pytest.mark.gpu

# float-float: absolute per locus
HKY_FF_ATOL = 1e-6
# FP32, relative to |log L|: FP32 rounding of ~depth*10 operations per pattern
HKY_FP32_RTOL = 2e-6


def _run_golden(precision):
    d = load("golden_hky.npz")
    for c in range(int(d["ncases"])):
        p = "c%d_" % c
        loc = HKYLocus(d[p + "seq"], d[p + "mult"], int(d[p + "totsites"]), d[p + "pi"])
        ts = trees(d, p)
        u, kappa = float(d[p + "u"]), float(d[p + "kappa"])
        ctx = ctx_with([("hky", loc)])
        ctx.set_pi(0, 0, loc.pi)
        ctx.set_genealogy(0, 0, ts[0])
        got = [ctx.eval([0], [0], [u], [kappa], precision=precision)[0][0]]
        ctx.commit([0], [0], [1])
        for t, e, acc in zip(ts[1:], d[p + "e"], d[p + "acc"]):
            ctx.set_genealogy(0, 0, t)
            got.append(ctx.eval([0], [0], [u], [kappa], edits=[e], precision=precision)[0][0])
            ctx.commit([0], [0], [acc])
        ctx.close()
        yield np.array(got), d[p + "ref"]


def test_hky_fp64_golden():
    for got, ref in _run_golden(api.PREC_FP64):
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0)


def test_hky_ff_golden():
    for got, ref in _run_golden(api.PREC_FAST):
        np.testing.assert_allclose(got, ref, rtol=0, atol=HKY_FF_ATOL)


def test_hky_fp32_golden():
    for got, ref in _run_golden(api.PREC_FP32):
        np.testing.assert_allclose(got, ref, rtol=HKY_FP32_RTOL, atol=0)


def test_hky_reference_mirror_calls():
    d = load("golden_hky.npz")
    p = "c1_"
    loc = HKYLocus(d[p + "seq"], d[p + "mult"], int(d[p + "totsites"]), d[p + "pi"])
    ts = trees(d, p)
    u, kappa = float(d[p + "u"]), float(d[p + "kappa"])
    ctx = ctx_with([("hky", loc)])
    ctx.set_pi(0, 0, loc.pi)
    ctx.set_genealogy(0, 0, ts[0])
    got = [ctx.likelihoodHKY(0, 0, u, kappa, -1, -1, -1, -1)]
    ctx.copyfraclike(0, 0)
    ctx.storescalefactors(0, 0)
    for t, e, acc in zip(ts[1:], d[p + "e"], d[p + "acc"]):
        ctx.set_genealogy(0, 0, t)
        got.append(ctx.likelihoodHKY(0, 0, u, kappa, *[int(v) for v in e]))
        if acc:
            ctx.copyfraclike(0, 0)
            ctx.storescalefactors(0, 0)
        else:
            ctx.restorescalefactors(0, 0)
    np.testing.assert_allclose(got, d[p + "ref"], rtol=0, atol=HKY_FF_ATOL)


def test_hky_batch_many_chains_vs_oracle():
    rng = np.random.default_rng(11)
    nloci, nch = 3, 5
    locs, base = [], []
    for li in range(nloci):
        g = synth.two_pop_tree(rng, 8 + 4 * li, 8 + 4 * li, theta=10.0, mig=0.2, tsplit=1.5)
        locs.append(synth.hky_data(rng, g, 400 + 300 * li, 1.0, rng.uniform(2, 8), rng.dirichlet([5] * 4)))
        base.append(g)
    ctx = ctx_with([("hky", L) for L in locs], 1, nch)
    ci, li, u, kap, want = [], [], [], [], []
    for c in range(nch):
        for l in range(nloci):
            t = synth.jitter_times(rng, base[l], 0.3)
            ctx.set_genealogy(c, l, t)
            ctx.set_pi(c, l, locs[l].pi)
            uu, kk = float(rng.lognormal(0, 0.5)), float(rng.uniform(2, 8))
            st = O.HKYState(*locs[l].seq.shape)
            want.append(st.likelihood(locs[l], t, uu, kk))
            ci.append(c), li.append(l), u.append(uu), kap.append(kk)
    r64, _ = ctx.eval(ci, li, u, kap, precision=api.PREC_FP64)
    rff, _ = ctx.eval(ci, li, u, kap, precision=api.PREC_FAST)
    r32, _ = ctx.eval(ci, li, u, kap, precision=api.PREC_FP32)
    np.testing.assert_allclose(r64, want, rtol=1e-12)
    np.testing.assert_allclose(rff, want, rtol=0, atol=HKY_FF_ATOL)
    np.testing.assert_allclose(r32, want, rtol=HKY_FP32_RTOL)


def test_hky_ff_config2_shaped_batch():
    """Loci of the 50-locus benchmark's shape (20 + 20 copies, 1000 bp, kappa
    ~ U(2, 8), pi ~ Dirichlet(5, 5, 5, 5), lognormal rates), a few chains:
    every per-locus log likelihood of the float-float form within 1e-6 of the
    FP64 form (itself 1e-12 from the reference's arithmetic), full and
    dirty-node evaluations; the FP32 form is far outside that bar on the
    same loci, which is why the float-float form is the default."""
    from ima2p_gb300 import workloads
    wl = workloads.make_hky(nloci=8, nch=4)
    ctx = api.Context(0)
    for _, loc in wl.loci:
        ctx.add_locus_hky(loc.seq, loc.mult, loc.totsites)
    ctx.set_chains(1, wl.nchains)
    wl.upload(ctx)
    ci, li = wl.pairs()
    u, kap = wl.u[ci, li], wl.par[ci, li]
    # FP32 first: the fast partial slots hold the float-float evaluation's
    # values when they are committed below
    r32, _ = ctx.eval(ci, li, u, kap, precision=api.PREC_FP32)
    r64, _ = ctx.eval(ci, li, u, kap, precision=api.PREC_FP64)
    rff, st = ctx.eval(ci, li, u, kap, precision=api.PREC_FAST)
    assert np.all(st == 0)
    err = np.abs(rff - r64)
    assert err.max() <= HKY_FF_ATOL, err.max()
    assert np.abs(r32 - r64).max() > 10 * err.max()
    # accept, then move one internal node's time on every chain-locus and
    # re-evaluate its path from the edit list
    ctx.commit(ci, li, np.ones(len(ci), np.uint8))
    edits = []
    for c, l in zip(ci, li):
        h = wl.tree(int(c), int(l)).copy()
        k = h.n + 7
        a, b = int(h.up0[k]), int(h.up1[k])
        lo = max(h.time[h.up0[a]] if h.up0[a] >= 0 else 0.0, h.time[h.up0[b]] if h.up0[b] >= 0 else 0.0)
        h.time[a] = h.time[b] = 0.5 * (lo + h.time[a])
        ctx.set_genealogy(int(c), int(l), h)
        edits.append([k, -1, -1, -1])
    rff, _ = ctx.eval(ci, li, u, kap, edits=edits, precision=api.PREC_FAST)
    r64, _ = ctx.eval(ci, li, u, kap, edits=edits, precision=api.PREC_FP64)
    assert np.abs(rff - r64).max() <= HKY_FF_ATOL
    ctx.close()


def test_hky_large_locus_uses_global_partials():
    """A chain-locus whose partials exceed the shared-memory cache (100 copies,
    3000 bp) takes the global-memory path; full and dirty-node evaluations
    agree with the oracle."""
    rng = np.random.default_rng(13)
    g = synth.two_pop_tree(rng, 50, 50, theta=10.0, mig=0.2, tsplit=1.5)
    loc = synth.hky_data(rng, g, 3000, 1.0, 4.0, rng.dirichlet([5] * 4))
    assert (loc.seq.shape[0] - 1) * loc.seq.shape[1] * 20 > 64 * 1024
    ctx = ctx_with([("hky", loc)])
    ctx.set_pi(0, 0, loc.pi)
    ctx.set_genealogy(0, 0, g)
    st = O.HKYState(*loc.seq.shape)
    want = st.likelihood(loc, g, 1.0, 4.0)
    st.accept()
    got = ctx.eval([0], [0], [1.0], [4.0])[0][0]
    ctx.commit([0], [0], [1])
    assert abs(got - want) <= HKY_FF_ATOL
    k = g.n + 7
    h = g.copy()
    a, b = int(h.up0[k]), int(h.up1[k])
    lo = max(h.time[h.up0[a]] if h.up0[a] >= 0 else 0.0, h.time[h.up0[b]] if h.up0[b] >= 0 else 0.0)
    h.time[a] = h.time[b] = 0.5 * (lo + h.time[a])
    ctx.set_genealogy(0, 0, h)
    got = ctx.eval([0], [0], [1.0], [4.0], edits=[[k, -1, -1, -1]])[0][0]
    want = st.likelihood(loc, h, 1.0, 4.0, (k, -1, -1, -1))
    assert abs(got - want) <= HKY_FF_ATOL
    ctx.close()
