"""The batch autotuner (ima_gpu_batch_autotune) on a small config-4-shaped
mixed workload: every launch variant of the fast kernels gives the plain
FP64 form's likelihoods (float-float HKY within 1e-6 per locus, SW within
1e-8), every variant of the FP32 HKY kernel within 2e-6 relative, and the
variants agree with one another up to the order of the final FP64
reduction; the tuned batch replays as a graph with the chosen shapes."""
import numpy as np
import pytest

from ima2p_gb300 import api, workloads
from tests._gpu import ctx_with

pytestmark = pytest.mark.gpu

HKY_VARIANTS, SW_VARIANTS = 6, 3


def _mixed_ctx():
    wl = workloads.make_mixed(seed=9, n_hky=12, n_sw=6, nruns=2, cpr=8)
    ctx = ctx_with(wl.loci, wl.nruns, wl.cpr)
    wl.upload(ctx)
    ci, li = wl.pairs()
    return wl, ctx, ci, li, wl.u.ravel(), wl.par.ravel()


def _check(res, ref, is_hky, prec):
    if prec == api.PREC_FP32:
        np.testing.assert_allclose(res[is_hky], ref[is_hky], rtol=2e-6)
    else:
        assert np.max(np.abs(res[is_hky] - ref[is_hky])) <= 1e-6
    assert np.max(np.abs(res[~is_hky] - ref[~is_hky])) <= 1e-8


@pytest.mark.parametrize("prec", [api.PREC_FAST, api.PREC_FP32])
def test_every_variant_matches_fp64_and_autotune_picks_one(prec):
    wl, ctx, ci, li, u, par = _mixed_ctx()
    is_hky = li < 12
    ref_b = ctx.batch_create(ci, li, u, par, precision=api.PREC_FP64)
    ref_b.run(use_graph=False)
    ref = ref_b.results()[0]
    b = ctx.batch_create(ci, li, u, par, precision=prec)
    outs = []
    for v in range(HKY_VARIANTS):
        b.set_variants(v, v % SW_VARIANTS)
        b.run(use_graph=True)
        r = b.results()[0]
        _check(r, ref, is_hky, prec)
        outs.append(r)
    for r in outs[1:]:
        np.testing.assert_allclose(r, outs[0], rtol=1e-12)
    hv, sv = b.autotune(reps=3)
    assert 0 <= hv < HKY_VARIANTS and 0 <= sv < SW_VARIANTS
    b.run(use_graph=True)
    np.testing.assert_allclose(b.results()[0], outs[0], rtol=1e-12)


def test_variants_out_of_range_are_rejected():
    wl, ctx, ci, li, u, par = _mixed_ctx()
    b = ctx.batch_create(ci, li, u, par, precision=api.PREC_FAST)
    with pytest.raises(api.ImaError):
        b.set_variants(HKY_VARIANTS, 0)
    with pytest.raises(api.ImaError):
        b.set_variants(0, SW_VARIANTS)


def test_sweep_graph_matches_separate_calls():
    """ima_gpu_batch_sweep as one graph launch per sweep (evaluation, commit,
    swaps) leaves the same betas, committed likelihoods and swap counts as the
    same sweeps made call by call (batch run, commit, swapchains on the same
    Philox stream), with an accept mask that changes between sweeps."""
    out = []
    for graph in (True, False):
        wl, ctx, ci, li, u, par = _mixed_ctx()
        ctx.setheat(0.9, 0.8, 1)
        ctx.set_probg(np.linspace(-30.0, -20.0, wl.nchains))
        b = ctx.batch_create(ci, li, u, par, precision=api.PREC_FAST)
        rng = np.random.default_rng(4)
        for s in range(6):
            acc = (rng.uniform(size=len(ci)) < 0.7).astype(np.uint8)
            if graph:
                b.sweep(3, accept=acc, seed=11, use_graph=True)
            else:
                b.run(use_graph=False)
                ctx.commit(ci, li, acc)
                ctx.swapchains(3, True, seed=11)
        ctx.synchronize()
        counts = [ctx.get_swapcounts(r) for r in range(wl.nruns)]
        out.append((ctx.get_betas(), ctx.get_pdg(), counts))
        ctx.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    for (a, b_), (c, d) in zip(out[0][2], out[1][2]):
        assert np.array_equal(a, c) and np.array_equal(b_, d)
