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
    must give what a fresh context gives.  Two runs agree to ~4e-10, not
    bitwise: the order in which candidates are folded depends on timing, and
    each term's weight is an FP32 exponential taken against the running
    maximum at that moment.  Stale operands would be off by far more than
    the 1e-8 allowed here."""
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
        np.testing.assert_allclose(q, fresh(mt, method, n), rtol=0, atol=1e-8, err_msg=str((mt, method, n)))
    # reloading other rows invalidates the prepared operands
    rows2 = rows.copy()
    rows2[:, off["fc"]] *= 1.5
    ctx.surface_load(rows2, 5, 8, 3, lognorm=None)
    q = ctx.surface_eval(pts, modeltype=1, method=api.SURF_TC)[0]
    c2 = ctx_with([("sw", 2, 1)])
    c2.surface_load(rows2, 5, 8, 3, lognorm=None)
    np.testing.assert_allclose(q, c2.surface_eval(pts, modeltype=1, method=api.SURF_TC)[0], rtol=0, atol=1e-8)
