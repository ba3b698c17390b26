"""L-mode surface on the GPU: the truncated reference form against the
golden jointp values, and the FP64 exact log-sum-exp against the oracle."""
import numpy as np
import pytest

from ima2p_gb300 import api, synth
from oracle import pyoracle as O
from tests._golden import load
from tests._gpu import ctx_with

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["a", "b1", "b2"])
def test_surface_compat_golden(case):
    d = load("golden_jointp.npz")
    if case == "a":
        rows, pts, ref, np_, nm, npops, mt = d["a_rows"], d["a_pts"], d["a_ref"], 3, 2, 2, 0
    else:
        mt = int(case[1])
        rows, pts, ref, np_, nm, npops = d["b_rows"], d["b_pts"], d["b_ref%d" % mt], 5, 8, 3
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(rows, np_, nm, npops)
    q, ess = ctx.surface_eval(pts, modeltype=mt, method=api.SURF_COMPAT)
    np.testing.assert_allclose(q, ref[:, 0], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(ess, ref[:, 1], rtol=1e-9)
    if case == "a":
        q1, e1 = ctx.jointp(pts[0])
        assert abs(q1 - ref[0, 0]) <= 1e-12 * abs(ref[0, 0])


def test_surface_fp64_exact_vs_oracle():
    rng = np.random.default_rng(21)
    rows, lognorm, off = synth.surface_stats(rng, 5000, 5, 8, 2)
    pts = synth.surface_points(rng, 40)
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(rows, 5, 8, 3, lognorm=lognorm)
    q, ess = ctx.surface_eval(pts, modeltype=0, method=api.SURF_FP64)
    for k in range(len(pts)):
        qo, eo = O.jointp(rows, 5, 8, 3, pts[k], modeltype=0, lognorm=lognorm)
        assert abs(q[k] - qo) <= 1e-12 * abs(qo)
        assert abs(ess[k] - eo) <= 1e-9 * eo


@pytest.mark.parametrize("mt", [0, 1, 2])
def test_surface_fast_split_precision_vs_oracle(mt):
    """Screen + exact float-float recomputation: within 2e-9 relative plus
    3e-7 absolute of the exact FP64 log-sum-exp (the target is 1e-7
    relative); what remains is the FP32 exp (<= 2 ulp) of each term's offset
    from the running maximum."""
    rng = np.random.default_rng(31 + mt)
    rows, lognorm, off = synth.surface_stats(rng, 20000, 5, 8, 2)
    pts = synth.surface_points(rng, 150)
    ctx = ctx_with([("sw", 2, 1)])
    ln = lognorm if mt == 0 else None
    ctx.surface_load(rows, 5, 8, 3, lognorm=ln)
    q, ess = ctx.surface_eval(pts, modeltype=mt, method=api.SURF_FAST)
    for k in range(0, len(pts), 7):
        qo, eo = O.jointp(rows, 5, 8, 3, pts[k], modeltype=mt, lognorm=ln)
        assert abs(q[k] - qo) <= 2e-9 * abs(qo) + 3e-7, (k, q[k], qo)
        assert abs(ess[k] - eo) <= 1e-4 * eo


def test_surface_fast_two_populations_golden_rows():
    d = load("golden_jointp.npz")
    rows, pts = d["a_rows"], d["a_pts"]
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(rows, 3, 2, 2)
    q, _ = ctx.surface_eval(pts, modeltype=0, method=api.SURF_FAST)
    want = [O.jointp(rows, 3, 2, 2, x)[0] for x in pts]
    np.testing.assert_allclose(q, want, rtol=2e-9, atol=3e-7)
