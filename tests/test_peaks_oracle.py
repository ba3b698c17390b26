"""The oracle's findmarginpeaks numbers (marginalopt, the migration tests,
margin95, marginalopt_popmig and its test) against golden_peaks.npz, made
by the unmodified reference (surface_call_functions.cpp:178-734,
surface_search_functions.cpp:42-200, popmig.cpp:181-428): equal bit for bit
on rows reaching every branch of the 2NM term and on rows whose peaks lie
inside the priors, under uniform and exponential migration priors."""
import os

import numpy as np
import pytest

from oracle import pyoracle as O

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_peaks.npz"))
KEYS = ("mlval", "peakloc", "migtest", "lo95", "hi95", "pm_mlval", "pm_peakloc", "pm_test")


@pytest.mark.parametrize("name", ["branch", "interior"])
@pytest.mark.parametrize("expo", [False, True])
def test_findmarginpeaks_matches_the_reference(name, expo):
    tag = name + ("_expo" if expo else "")
    o = O.findmarginpeaks(GOLD[name + "_rows"], 3, 2, np.zeros(3), GOLD["qmax"], np.zeros(2), GOLD["mmax"],
                          mg_mean=GOLD["mean"] if expo else None, terms=GOLD["terms"])
    for k in KEYS:
        assert np.array_equal(o[k], GOLD["%s_%s" % (tag, k)], equal_nan=True), k


def test_interior_peaks_are_found_inside_the_priors():
    pk = GOLD["interior_peakloc"]
    assert (pk > 0).all() and (pk[:, :3] < 20).all() and (pk[:, 3:] < GOLD["mmax"]).all()
    assert (GOLD["interior_pm_peakloc"] > 0).all()


def test_too_few_genealogies():
    rows = GOLD["interior_rows"][:10]
    assert O.findmarginpeaks(rows, 3, 2, np.zeros(3), GOLD["qmax"], np.zeros(2), GOLD["mmax"]) is None
