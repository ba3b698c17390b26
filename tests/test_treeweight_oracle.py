"""Genealogy weights and p(G) integrals: the oracle restatement
(ora_treeweight, ora_tree_prob, ora_iterm) and the host-side population
tables (ima2p_gb300.popmodel) against golden_tw.npz, made by the unmodified
reference's treeweight / sum_treeinfo / initialize_integrate_tree_prob /
setup_iparams (update_gtree_common.cpp:108-304, :1680-2134; ginfo.cpp:209;
initialize.cpp:202-727).  Integer and FP64 results are compared bit for
bit.  CPU only."""
import numpy as np
import pytest

from ima2p_gb300 import popmodel
from oracle import pyoracle as O
from tests._golden import load, tw_cases

CASES = tw_cases()


@pytest.mark.parametrize("c", range(len(CASES)))
def test_parameter_maps_match_setup_iparams(c):
    cs = CASES[c]
    pm = cs.pm
    assert [[popmodel.toff(cs.npops, p) + r for p, r in wp] for wp in cs.th_wp] == pm.th_cells
    assert [[popmodel.moff(cs.npops, p) + a * (cs.npops - p) + b for p, a, b in wp] for wp in cs.mg_wp] == pm.mg_cells


@pytest.mark.parametrize("c", range(len(CASES)))
def test_oracle_weights_and_integrals_bit_exact(c):
    cs = CASES[c]
    pm = cs.pm
    nth, nmg = len(pm.th_cells), len(pm.mg_cells)
    for ci in range(cs.nch):
        ws = []
        for li, (ng, h, samp) in enumerate(cs.loci):
            st, w = O.treeweight(pm, cs.tvals[ci], cs.gen(ci, li), samp, h)
            assert st == 0
            i = ci * cs.nl + li
            for f in ("cc", "hcc", "fc") + (() if pm.nomig else ("mc", "fm")):
                assert np.array_equal(w[f], cs.ref[f][i]), (ci, li, f)
            if pm.nomig:  # the reference keeps no migration cells then
                assert not w["mc"].any() and not w["fm"].any()
            assert [w["mignum"], w["length"], w["tlength"]] == list(cs.ref["scal"][i])
            ws.append(w)
        tot = O.sum_weights(ws, pm)
        st, pg, q, m = O.tree_prob(pm, tot, cs.th_pr[:, 0], cs.th_pr[:, 1], cs.mg_pr[:, 0], cs.mg_pr[:, 1],
                                   cs.mg_pr[:, 2], expo=cs.expo)
        assert st == 0
        ours = np.concatenate([[pg], q, [] if pm.nomig else m])
        assert np.array_equal(ours, cs.ref["pg"][ci])


def test_integral_terms_bit_exact_and_stops():
    d = load("golden_tw.npz")
    for line, want in zip(d["iterm_lines"], d["iterm_ref"]):
        v, st = O.iterm(*line)
        assert st == 0 and v == want, (line, v, want)
    for line in d["iterm_stop"]:  # the reference stops with IM_err on these
        assert O.iterm(*line)[1] != 0


def test_oracle_rejects_a_genealogy_the_model_cannot_hold():
    cs = CASES[1]
    lg = cs.gen(0, 0)
    bad = type(lg)(lg.g, lg.pop.copy(), lg.mig)
    # a coalescence placed in an ancestral population before it exists
    bad.pop[cs.loci[0][0]] = cs.npops + cs.npops - 2
    st, _ = O.treeweight(cs.pm, cs.tvals[0], bad, cs.loci[0][2], cs.loci[0][1])
    assert st == 1


def test_tree_string_checks():
    with pytest.raises(ValueError):
        popmodel.build("((0,1):3,2)", 3)
    with pytest.raises(ValueError):
        popmodel.build("((0,1):4,2):3", 3)
    with pytest.raises(ValueError):
        popmodel.build("((0,0):3,2):4", 3)
