"""1-D marginal densities on the GPU (ima_gpu_margincalc, ima_gpu_fillvec)
against the reference's margincalc (golden_margin.npz) and the oracle.  The
sums are FP64 without a shift, as the reference's; only the order of the
additions differs (per-chunk partial sums), so values agree to 1e-12
relative."""
import numpy as np
import pytest

from ima2p_gb300 import api, synth
from oracle import pyoracle as O
from tests._golden import load
from tests._gpu import ctx_with

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.mark.parametrize("expo", [False, True])
def test_margincalc_vs_reference(expo):
    d = load("golden_margin.npz")
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(d["rows"], 3, 2, 2)
    em = d["expo_mean"] if expo else None
    want = d["ref_expo"] if expo else d["ref"]
    pts = d["points"]
    plain = pts[:, 2] == 0
    # one call per (logi, yadjust) group, as the reference's callers make them
    got = ctx.margincalc(pts[plain, 0].astype(int), pts[plain, 1], 0.0, 0, expo_mean=em)
    np.testing.assert_allclose(got, want[plain], rtol=RTOL)
    got = ctx.margincalc(pts[~plain, 0].astype(int), pts[~plain, 1], 1.92, 1, expo_mean=em)
    np.testing.assert_allclose(got, want[~plain], rtol=RTOL)


def test_fillvec_full_grid_vs_oracle():
    """fillvec on GRIDSIZE = 1000 points per parameter over 20,000
    genealogies (several chunks per point), against the oracle's margincalc
    on a sample of grid points; a migration rate with a zero prior is skipped."""
    rng = np.random.default_rng(8)
    rows, _, off = synth.surface_stats(rng, 20000, 3, 2, 1)
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(rows, 3, 2, 2)
    pmin = np.zeros(5)
    pmax = np.array([20.0, 12.0, 30.0, 3.0, 1e-7])
    xs, ys = ctx.fillvec(pmin, pmax, 1000)
    for p in range(4):
        for j in range(0, 1000, 97):
            assert xs[p, j] == ((j + 0.5) * (pmax[p] - pmin[p])) / 1000
            want = O.margincalc(rows, 3, 2, p, xs[p, j])
            assert abs(ys[p, j] - want) <= RTOL * abs(want), (p, j, ys[p, j], want)
    assert np.all(ys[4] == 0.0)


def test_margincalc_rejects_bad_points():
    d = load("golden_margin.npz")
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(d["rows"], 3, 2, 2)
    with pytest.raises(api.ImaError):
        ctx.margincalc([5], [1.0])
    with pytest.raises(api.ImaError):
        ctx.margincalc([0], [0.0])
