"""The oracle's calc_popmig / calc_pop_expomig (2NM densities) against
golden_popmig.npz, made by the unmodified reference (popmig.cpp:9-172):
equal bit for bit, both forms, posterior and likelihood, every branch of the
per-genealogy term (tests/golden/make_golden.py:popmig_rows)."""
import os

import numpy as np

from oracle import pyoracle as O

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_popmig.npz"))


def test_calc_popmig_matches_the_reference():
    rows, q, m = GOLD["rows"], GOLD["qmax"], GOLD["mmax"]
    got = [O.popmig(rows, 3, 2, int(t), int(mi), x, q[int(t)], m[int(mi)], prob_or_like=int(pl))
           for t, mi, x, pl in GOLD["points"]]
    assert np.array_equal(np.array(got), GOLD["ref"])


def test_calc_pop_expomig_matches_the_reference():
    rows, q, mean = GOLD["rows"], GOLD["qmax"], GOLD["mean"]
    got = [O.popmig(rows, 3, 2, int(t), int(mi), x, q[int(t)], 0.0, mmean=mean[int(mi)], prob_or_like=int(pl))
           for t, mi, x, pl in GOLD["points"]]
    assert np.array_equal(np.array(got), GOLD["ref_expo"])


def test_fixture_reaches_every_branch():
    rows = GOLD["rows"]
    # columns: cc 0-2, fc 3-5, hcc 6-8, mc 9-10, fm 11-12
    cc0, fc0, mc0, fm0 = rows[:, 0], rows[:, 3], rows[:, 9], rows[:, 11]
    assert ((cc0 == 0) & (fc0 == 0) & (fm0 > 0)).any()          # no coalescences
    assert ((mc0 == 0) & (fm0 == 0) & (fc0 > 0)).any()          # no migrations
    assert ((rows[:, 1] == 0) & (rows[:, 4] == 0) & (rows[:, 10] == 0) & (rows[:, 12] == 0)).any()  # neither
    assert (GOLD["ref"] < 0).any()  # x beyond theta_max * m_max / 2: the likelihood's prior term turns negative


def test_popmig_terms_follow_the_parameter_names():
    """popmodel.popmig_terms: for every population but the root, each
    migration parameter whose name starts with it, in (thetai, mi) order, as
    print_populationmigrationrate_histograms picks them
    (histograms.cpp:754-773)."""
    from ima2p_gb300 import popmodel
    pm = popmodel.build("(0,1):2", 2)
    assert [(t, m) for t, m, _ in popmodel.popmig_terms(pm)] == [(0, 0), (1, 1)]
    pm = popmodel.build("((0,1):3,2):4", 3)
    terms = popmodel.popmig_terms(pm)
    assert [(t, m) for t, m, _ in terms] == [(0, 0), (0, 2), (1, 1), (1, 4), (2, 3), (2, 5), (2, 6), (3, 7)]
    for t, m, label in terms:
        src = int(pm.mg_names[m][1:].split(">")[0])
        assert src == t and t < 2 * pm.npops - 2 and label == "2N%d%s" % (t, pm.mg_names[m])
    assert all(any(m == mm for _, mm, _ in terms) for m in range(len(pm.mg_names)))
