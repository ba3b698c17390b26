"""The tensor-core path: a bf16 tile through TMA, tcgen05.mma and tcgen05.ld
checked element by element against CUDA cores, then the tensor-core-screened
surface against the exact FP64 log-sum-exp of the oracle (2e-9 relative, the
tolerance of the CUDA-core screen, plus 3e-7 absolute: the weights
exp(p - max) are FP32 exponentials, within 2 ulp)."""
import numpy as np
import pytest

from ima2p_gb300 import api, synth
from oracle import pyoracle as O
from tests._gpu import ctx_with

pytestmark = pytest.mark.gpu


def test_tcgen05_tile_is_exact():
    ctx = ctx_with([("sw", 2, 1)])
    bad, err = ctx.tc_selftest()
    assert bad == 0 and err == 0.0, (bad, err)


@pytest.mark.parametrize("mt", [0, 1, 2])
def test_surface_tensor_core_screen_vs_oracle(mt):
    rng = np.random.default_rng(41 + mt)
    rows, lognorm, off = synth.surface_stats(rng, 30000, 5, 8, 2)
    pts = synth.surface_points(rng, 300)
    ctx = ctx_with([("sw", 2, 1)])
    ln = lognorm if mt == 0 else None
    ctx.surface_load(rows, 5, 8, 3, lognorm=ln)
    q, ess = ctx.surface_eval(pts, modeltype=mt, method=api.SURF_TC)
    q2, _ = ctx.surface_eval(pts, modeltype=mt, method=api.SURF_FAST)
    np.testing.assert_allclose(q, q2, rtol=2e-9, atol=3e-7)
    for k in range(0, len(pts), 13):
        qo, eo = O.jointp(rows, 5, 8, 3, pts[k], modeltype=mt, lognorm=ln)
        assert abs(q[k] - qo) <= 2e-9 * abs(qo) + 3e-7, (k, q[k], qo)
        assert abs(ess[k] - eo) <= 1e-4 * eo


def test_surface_row_operands_reused_across_evaluations():
    """The row-derived operands are prepared once per (rows, model type) and
    reused; switching model type, method or point count, or reloading rows,
    must give what a fresh context gives, bit for bit: the screened candidate
    set and the sums do not depend on timing."""
    rng = np.random.default_rng(77)
    rows, lognorm, off = synth.surface_stats(rng, 20000, 5, 8, 2)
    pts = synth.surface_points(rng, 400)

    def fresh(mt, method, n):
        c = ctx_with([("sw", 2, 1)])
        c.surface_load(rows, 5, 8, 3, lognorm=lognorm if mt == 0 else None)
        return c.surface_eval(pts[:n], modeltype=mt, method=method)[0]

    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(rows, 5, 8, 3, lognorm=None)
    seq = [(1, api.SURF_TC, 400), (1, api.SURF_TC, 150), (2, api.SURF_TC, 400), (1, api.SURF_FAST, 300),
           (1, api.SURF_FP64, 50), (1, api.SURF_TC, 400), (2, api.SURF_FAST, 200), (1, api.SURF_TC, 100)]
    for mt, method, n in seq:
        q = ctx.surface_eval(pts[:n], modeltype=mt, method=method)[0]
        np.testing.assert_array_equal(q, fresh(mt, method, n), err_msg=str((mt, method, n)))
    # reloading other rows invalidates the prepared operands
    rows2 = rows.copy()
    rows2[:, off["fc"]] *= 1.5
    ctx.surface_load(rows2, 5, 8, 3, lognorm=None)
    q = ctx.surface_eval(pts, modeltype=1, method=api.SURF_TC)[0]
    c2 = ctx_with([("sw", 2, 1)])
    c2.surface_load(rows2, 5, 8, 3, lognorm=None)
    np.testing.assert_array_equal(q, c2.surface_eval(pts, modeltype=1, method=api.SURF_TC)[0])


@pytest.mark.parametrize("method", [api.SURF_TC, api.SURF_FAST])
def test_surface_repeat_calls_bitwise(method):
    """The same points evaluated again give the same bits (densities and
    effective sample sizes): neither which terms pass the screen nor the order
    of their sums follows timing.  Enough genealogies for several chunks and
    the max-only pre-pass.  With the points in another order each point's
    density is unchanged."""
    rng = np.random.default_rng(5)
    rows, lognorm, _ = synth.surface_stats(rng, 70000, 5, 8, 2)
    pts = synth.surface_points(rng, 700)
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(rows, 5, 8, 3, lognorm=lognorm)
    q0, e0 = ctx.surface_eval(pts, modeltype=0, method=method)
    for _ in range(3):
        q1, e1 = ctx.surface_eval(pts, modeltype=0, method=method)
        np.testing.assert_array_equal(q1, q0)
        np.testing.assert_array_equal(e1, e0)
    perm = rng.permutation(len(pts))
    q2, _ = ctx.surface_eval(pts[perm], modeltype=0, method=method)
    # a point's terms and sums do not depend on the other points of its tile
    np.testing.assert_allclose(q2, q0[perm], rtol=1e-12, atol=0)


# Fewer than four 256-genealogy tiles: no max-only pre-pass runs, and a
# point's reference is the best of its 32 exact seed samples (genealogies
# floor(i G / 32)), so a term can lie far above it
G_NO_PREPASS = 700
G_STAR = 256 + 17  # between the seed samples 262 and 284


def test_surface_tc_term_far_above_prepass_bound():
    """One genealogy 300 nats above every other, away from the seed samples,
    with no pre-pass: its weight relative to the seeds' bound leaves the
    fixed-point range, so every point is taken a second time relative to its
    exact maximum.  The densities agree with the FP64 form and the oracle,
    and repeat bit for bit."""
    rng = np.random.default_rng(8)
    G = G_NO_PREPASS
    rows, lognorm, _ = synth.surface_stats(rng, G, 5, 8, 2)
    lognorm = lognorm.copy()
    g_star = G_STAR
    lognorm[g_star] = lognorm.max() + 300.0
    pts = synth.surface_points(rng, 200)
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(rows, 5, 8, 3, lognorm=lognorm)
    q, ess = ctx.surface_eval(pts, modeltype=0, method=api.SURF_TC)
    assert ctx.surface_retaken() == len(pts)
    q64, ess64 = ctx.surface_eval(pts, modeltype=0, method=api.SURF_FP64)
    assert np.all(np.abs(q - q64) <= 2e-9 * np.abs(q64) + 3e-7), np.max(np.abs(q - q64))
    np.testing.assert_allclose(ess, ess64, rtol=1e-4)
    for k in range(0, len(pts), 37):
        qo, _ = O.jointp(rows, 5, 8, 3, pts[k], modeltype=0, lognorm=lognorm)
        assert abs(q[k] - qo) <= 2e-9 * abs(qo) + 3e-7, (k, q[k], qo)
    q2, _ = ctx.surface_eval(pts, modeltype=0, method=api.SURF_TC)
    np.testing.assert_array_equal(q2, q)


@pytest.mark.parametrize("lead", [20.0, 40.0, 46.0, 50.0, 54.0, 60.0])
def test_surface_tc_dominant_genealogy_sample_size(lead):
    """One genealogy `lead` nats above every other, away from the seed
    samples, with no pre-pass: terms up to 55 nats above the seeds' bound
    stay in the first pass's fixed-point sums, larger ones send the point to
    the second pass.  Either way the densities and the effective sample
    sizes (here close to 1) agree with the FP64 form -- the squared weights
    of the largest terms exceed FP32's range and must still be counted."""
    rng = np.random.default_rng(9)
    G = G_NO_PREPASS
    rows, lognorm, _ = synth.surface_stats(rng, G, 5, 8, 2)
    lognorm = lognorm.copy()
    lognorm[G_STAR] = lognorm.max() + lead
    pts = synth.surface_points(rng, 100)
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(rows, 5, 8, 3, lognorm=lognorm)
    q, ess = ctx.surface_eval(pts, modeltype=0, method=api.SURF_TC)
    q64, ess64 = ctx.surface_eval(pts, modeltype=0, method=api.SURF_FP64)
    assert np.all(np.abs(q - q64) <= 2e-9 * np.abs(q64) + 3e-7), np.max(np.abs(q - q64))
    np.testing.assert_allclose(ess, ess64, rtol=1e-4)
