"""findmarginpeaks' numbers on the GPU (ima_gpu_findmarginpeaks: every
parameter's, term's and genealogy range's search advancing together, each
round's points in batched launches) against golden_peaks.npz, made by the
unmodified reference.

Tolerances: each search follows the reference's sequence of points given
its values, and the device's densities agree with the reference's to
rounding (another summation order), so a golden-section comparison of two
nearly equal values near convergence can go the other way: peak locations
within 1e-5 relative (the search's own tolerance is 1e-7), the densities
at the peaks 1e-9 relative, the tests (2 log of a density ratio at the
peak) 1e-6 absolute, and the 95% limits within the bisection's tolerance,
1e-4.  Which parameters have no peak (-1) is exact."""
import os

import numpy as np
import pytest

from ima2p_gb300 import api

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_peaks.npz"))


def _run(rows, expo):
    ctx = api.Context(0)
    ctx.surface_load(rows, 3, 2, 2)
    o = ctx.findmarginpeaks(np.zeros(3), GOLD["qmax"], np.zeros(2), GOLD["mmax"],
                            mig_mean=GOLD["mean"] if expo else None, terms=GOLD["terms"])
    ctx.close()
    return o


@pytest.mark.parametrize("name", ["branch", "interior"])
@pytest.mark.parametrize("expo", [False, True])
def test_findmarginpeaks_matches_the_reference(name, expo):
    tag = name + ("_expo" if expo else "")
    g = {k: GOLD["%s_%s" % (tag, k)] for k in ("mlval", "peakloc", "migtest", "lo95", "hi95", "pm_mlval",
                                               "pm_peakloc", "pm_test")}
    o = _run(GOLD[name + "_rows"], expo)
    assert o["rounds"] > 0
    assert np.array_equal(o["peakloc"] < 0, g["peakloc"] < 0)
    ok = g["peakloc"] >= 0
    np.testing.assert_allclose(o["peakloc"][ok], g["peakloc"][ok], rtol=1e-5)
    np.testing.assert_allclose(o["mlval"][ok], g["mlval"][ok], rtol=1e-9)
    np.testing.assert_allclose(o["migtest"], g["migtest"], rtol=0, atol=1e-6)
    assert np.array_equal(np.isnan(o["lo95"]), np.isnan(g["lo95"]))
    fin = ~np.isnan(g["lo95"])
    np.testing.assert_allclose(o["lo95"][fin], g["lo95"][fin], rtol=0, atol=1e-4)
    np.testing.assert_allclose(o["hi95"][fin], g["hi95"][fin], rtol=0, atol=1e-4)
    np.testing.assert_allclose(o["pm_peakloc"], g["pm_peakloc"], rtol=1e-5)
    np.testing.assert_allclose(o["pm_mlval"], g["pm_mlval"], rtol=1e-9)
    np.testing.assert_allclose(o["pm_test"], g["pm_test"], rtol=0, atol=1e-6)
    want_hold = np.where(g["peakloc"][2] < 0, 1e-7, g["peakloc"][2]).astype(np.float32)
    np.testing.assert_allclose(o["holdpeakloc"], want_hold, rtol=1e-5)


def test_too_few_genealogies_and_no_terms():
    ctx = api.Context(0)
    ctx.surface_load(GOLD["interior_rows"][:10], 3, 2, 2)
    o = ctx.findmarginpeaks(np.zeros(3), GOLD["qmax"], np.zeros(2), GOLD["mmax"])
    assert (o["holdpeakloc"] == -1).all() and o["rounds"] == 0
    ctx.surface_load(GOLD["interior_rows"], 3, 2, 2)
    o = ctx.findmarginpeaks(np.zeros(3), GOLD["qmax"], np.zeros(2), GOLD["mmax"])  # no 2NM terms
    np.testing.assert_allclose(o["peakloc"], GOLD["interior_peakloc"], rtol=1e-5)
    with pytest.raises(api.ImaError):  # a term outside the parameters
        ctx.findmarginpeaks(np.zeros(3), GOLD["qmax"], np.zeros(2), GOLD["mmax"], terms=[(0, 2)])
    ctx.close()


def test_prior_minima_against_the_oracle():
    """Non-zero prior minima: marginp is off-scale below them as above the
    maxima, which moves the brackets; the device's searches against the
    oracle's (pinned to the reference on the golden cases)."""
    from oracle import pyoracle as O
    rows = GOLD["interior_rows"]
    tmin, mmin = np.array([0.5, 1.0, 2.0]), np.array([0.05, 0.3])
    want = O.findmarginpeaks(rows, 3, 2, tmin, GOLD["qmax"], mmin, GOLD["mmax"], terms=GOLD["terms"])
    ctx = api.Context(0)
    ctx.surface_load(rows, 3, 2, 2)
    got = ctx.findmarginpeaks(tmin, GOLD["qmax"], mmin, GOLD["mmax"], terms=GOLD["terms"])
    ctx.close()
    assert np.array_equal(got["peakloc"] < 0, want["peakloc"] < 0)
    ok = want["peakloc"] >= 0
    np.testing.assert_allclose(got["peakloc"][ok], want["peakloc"][ok], rtol=1e-5)
    np.testing.assert_allclose(got["mlval"][ok], want["mlval"][ok], rtol=1e-9)
    np.testing.assert_allclose(got["migtest"], want["migtest"], rtol=0, atol=1e-6)
    fin = ~np.isnan(want["lo95"])
    np.testing.assert_allclose(got["lo95"][fin], want["lo95"][fin], rtol=0, atol=1e-4)
    np.testing.assert_allclose(got["hi95"][fin], want["hi95"][fin], rtol=0, atol=1e-4)
    np.testing.assert_allclose(got["pm_peakloc"], want["pm_peakloc"], rtol=1e-5)
