"""2NM densities on the GPU (ima_gpu_popmig, ima_gpu_popmig_curves) against
golden_popmig.npz, made by the unmodified reference's calc_popmig and
calc_pop_expomig (popmig.cpp:9-172), and against the oracle.

Tolerance: the per-genealogy terms follow the reference's operation order
(compiled without FMA contraction) on the device's log/exp/pow, and the sum
over genealogies is taken in chunks, so values agree to rounding: 1e-11
relative at the fixture's points.  One more effect widens it on dense grids:
uppergamma is gln + log(1 - P(a, x)), which saturates at -1e200 when P
rounds to 1, and calc_popmig switches to the lower functions only when its
two upper terms are EQUAL (popmig.cpp:64-68).  Where P is within a few ulps
of 1 an ulp of the host's or the device's exp/log decides whether both terms
saturate, i.e. which branch one genealogy takes; its share of the sum is the
difference (1.3e-10 relative on the curves here).  Curves and the 300,000-row
case are compared at 1e-9."""
import os

import numpy as np
import pytest

from ima2p_gb300 import api
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_popmig.npz"))
RTOL = 1e-11
RTOL_GRID = 1e-9


def _ctx(rows):
    ctx = api.Context(0)
    ctx.surface_load(rows, 3, 2, 2)
    return ctx


def test_points_match_the_reference():
    ctx = _ctx(GOLD["rows"])
    p = GOLD["points"]
    th, mi, x, pl = p[:, 0].astype(int), p[:, 1].astype(int), p[:, 2], p[:, 3].astype(int)
    for form in (0, 1):
        sel = pl == form
        y = ctx.popmig(th[sel], mi[sel], x[sel], GOLD["qmax"], GOLD["mmax"], prob_or_like=form)
        np.testing.assert_allclose(y, GOLD["ref"][sel], rtol=RTOL)
        ye = ctx.popmig(th[sel], mi[sel], x[sel], GOLD["qmax"], GOLD["mmax"], mig_mean=GOLD["mean"],
                        prob_or_like=form)
        np.testing.assert_allclose(ye, GOLD["ref_expo"][sel], rtol=RTOL)
    ctx.close()


def test_curves_follow_the_reference_grid_rule():
    """popmig_curves: the scan from the top for the first density above 1e-9
    and the curve on (0, maxx], against the oracle; the scan grid itself is
    the fixture's curve points (term (1, 1), 50 points)."""
    rows = GOLD["rows"]
    ctx = _ctx(rows)
    q, m, mean = GOLD["qmax"], GOLD["mmax"], GOLD["mean"]
    terms = [(0, 0), (1, 1)]
    grid = 50
    for mig_mean in (None, mean):
        xs, ys, mx = ctx.popmig_curves(terms, q, m, mig_mean=mig_mean, gridsize=grid)
        for t, (ti, mj) in enumerate(terms):
            pmmax = 20 * mean[mj] if mig_mean is not None else q[ti] * m[mj] / 2.0
            scan = [(j + 0.5) * pmmax / grid for j in range(grid)]
            dens = [O.popmig(rows, 3, 2, ti, mj, v, q[ti], m[mj],
                             mmean=None if mig_mean is None else mean[mj]) for v in scan]
            above = [j for j in range(grid) if dens[j] > 1e-9]
            want = scan[above[-1]] if above else pmmax
            assert mx[t] == want
            assert np.array_equal(xs[t], [(j + 0.5) * want / grid for j in range(grid)])
            ref = [O.popmig(rows, 3, 2, ti, mj, v, q[ti], m[mj], mmean=None if mig_mean is None else mean[mj])
                   for v in xs[t]]
            np.testing.assert_allclose(ys[t], ref, rtol=RTOL_GRID)
    # the fixture's grid points for term (1, 1) are the scan grid: same values
    p = GOLD["points"]
    cur = (p[:, 0] == 1) & (p[:, 1] == 1) & (np.arange(len(p)) >= len(p) - int(GOLD["grid"]))
    y = ctx.popmig(p[cur, 0].astype(int), p[cur, 1].astype(int), p[cur, 2], q, m)
    np.testing.assert_allclose(y, GOLD["ref"][cur], rtol=RTOL_GRID)
    ctx.close()


def test_many_genealogies_average_like_one_copy():
    """calc_popmig averages over genealogies: the fixture's 200 rows repeated
    1500 times (300,000 rows, the reference's MAXGENEALOGIESTOSAVE) give the
    fixture's densities, through many chunks and CTAs."""
    rows = np.tile(GOLD["rows"], (1500, 1))
    ctx = _ctx(rows)
    p = GOLD["points"][:28]
    for form in (0, 1):
        sel = p[:, 3] == form
        y = ctx.popmig(p[sel, 0].astype(int), p[sel, 1].astype(int), p[sel, 2], GOLD["qmax"], GOLD["mmax"],
                       prob_or_like=form)
        np.testing.assert_allclose(y, GOLD["ref"][:28][sel], rtol=RTOL_GRID)
        ye = ctx.popmig(p[sel, 0].astype(int), p[sel, 1].astype(int), p[sel, 2], GOLD["qmax"], GOLD["mmax"],
                        mig_mean=GOLD["mean"], prob_or_like=form)
        np.testing.assert_allclose(ye, GOLD["ref_expo"][:28][sel], rtol=RTOL_GRID)
    ctx.close()


def test_bad_requests_are_refused():
    ctx = api.Context(0)
    with pytest.raises(api.ImaError):  # no surface
        ctx.popmig([0], [0], [1.0], GOLD["qmax"], GOLD["mmax"])
    ctx.surface_load(GOLD["rows"], 3, 2, 2)
    for th, mi, x in ((3, 0, 1.0), (0, 2, 1.0), (0, 0, 0.0), (-1, 0, 1.0)):
        with pytest.raises(api.ImaError):
            ctx.popmig([th], [mi], [x], GOLD["qmax"], GOLD["mmax"])
    with pytest.raises(api.ImaError):  # a non-positive prior mean
        ctx.popmig([0], [0], [1.0], GOLD["qmax"], GOLD["mmax"], mig_mean=np.array([0.8, 0.0]))
    y = ctx.popmig([0], [0], [0.7], GOLD["qmax"], GOLD["mmax"])  # still usable
    assert np.isfinite(y[0])
    ctx.close()


def test_likelihood_curves_under_both_priors():
    """popmig_curves with prob_or_like = 1 (each density divided by the prior
    density of 2NM), uniform and exponential migration priors, against the
    oracle on the curve the device chose."""
    rows = GOLD["rows"]
    ctx = _ctx(rows)
    q, m, mean = GOLD["qmax"], GOLD["mmax"], GOLD["mean"]
    for mig_mean in (None, mean):
        xs, ys, mx = ctx.popmig_curves([(0, 0), (2, 1)], q, m, mig_mean=mig_mean, prob_or_like=1, gridsize=40)
        for t, (ti, mj) in enumerate([(0, 0), (2, 1)]):
            ref = [O.popmig(rows, 3, 2, ti, mj, v, q[ti], m[mj], mmean=None if mig_mean is None else mean[mj],
                            prob_or_like=1) for v in xs[t]]
            np.testing.assert_allclose(ys[t], ref, rtol=RTOL_GRID)
    ctx.close()
