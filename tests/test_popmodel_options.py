"""The parameter maps of the -j model options against the reference's own
setup_iparams and set_nomigrationchecklist (initialize.cpp:202-809), run by
the harness on 9 population trees x 19 option sets (golden_iparams.npz):
theta and migration cells, names, first and last periods, priors, and the
cells a model forbids."""
import json

import numpy as np
import pytest

from ima2p_gb300 import popmodel
from tests._golden import load

CASES = json.loads(str(load("golden_iparams.npz")["cases"]))


def _options(flags):
    return popmodel.ModelOptions(**{f: True for f in flags if f not in ("no_migration", "expo_migration_prior")})


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s|%s" % (c["tree"], "+".join(c["flags"]) or "default"))
def test_maps_match_reference(case):
    n, flags = case["npops"], case["flags"]
    nomig = "no_migration" in flags
    pm = popmodel.build(case["tree"], n, nomig=nomig, options=_options(flags), varrank=case["varrank"])
    ref = case["ref"]
    assert [[popmodel.toff(n, p) + r for p, r in t[3]] for t in ref["theta"]] == pm.th_cells
    assert [t[0] for t in ref["theta"]] == pm.th_names
    assert [(t[1], t[2]) for t in ref["theta"]] == pm.th_be
    mg = [[popmodel.moff(n, p) + a * (n - p) + b for p, a, b in m[3]] for m in ref["mig"]]
    assert mg == pm.mg_cells
    assert [m[0] for m in ref["mig"]] == pm.mg_names
    assert [(m[1], m[2]) for m in ref["mig"]] == pm.mg_be
    assert [popmodel.moff(n, p) + a * (n - p) + b for p, a, b in ref["chk"]] == pm.chk_cells
    th_max, th_min, mg_max, mg_min, mg_mean = popmodel.priors(pm, 10.0, 5.0, "expo_migration_prior" in flags)
    np.testing.assert_array_equal(th_max, [t[4] for t in ref["theta"]])
    np.testing.assert_array_equal(th_min, [t[5] for t in ref["theta"]])
    np.testing.assert_array_equal(mg_max, [m[4] for m in ref["mig"]])
    np.testing.assert_array_equal(mg_min, [m[5] for m in ref["mig"]])
    np.testing.assert_array_equal(mg_mean, [m[6] for m in ref["mig"]])


def test_conflicting_options_are_refused():
    with pytest.raises(ValueError):
        popmodel.build("((0,1):3,2):4", 3, options=popmodel.ModelOptions(parameters_by_period=True,
                                                                         ancestral_sizes_largest_sampled=True))
    with pytest.raises(ValueError):
        popmodel.build("((0,1):3,2):4", 3, options=popmodel.ModelOptions(one_migration_parameter=True,
                                                                         single_migration_both_directions=True))
    with pytest.raises(ValueError):
        popmodel.build("((0,1):3,2):4", 3, nomig=True, options=popmodel.ModelOptions(one_migration_parameter=True))
