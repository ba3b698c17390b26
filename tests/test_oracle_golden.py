"""The CPU oracle against golden vectors produced by the compiled reference
(tests/golden/make_golden.py).  This pins the restatement before it is used
to check any kernel."""
import numpy as np
import pytest

from oracle import pyoracle as O
from ima2p_gb300.synth import HKYLocus
from tests._golden import load, trees


def test_is_matches_reference():
    d = load("golden_is.npz")
    for c in range(int(d["ncases"])):
        p = "c%d_" % c
        seq, ts, ref = d[p + "seq"], trees(d, p), d[p + "ref"]
        st, slk_first, _ = O.is_sumlogk(seq, ts[0])
        assert st == 0
        assert slk_first == ref[0, 1]          # cached constant from the first genealogy
        for t, L, u, r in zip(ts, d[p + "length"], d[p + "u"], ref):
            v, status, _ = O.is_likelihood(seq, t, float(L), float(u), slk_first)
            if r[0] == -1e9:
                assert status == 1 and v == -1e9
            else:
                assert status == 0
                assert abs(v - r[0]) <= 1e-12 * abs(r[0])
            st2, own, _ = O.is_sumlogk(seq, t)
            assert own == r[2]                  # mutation counts -> sum log k!, bit-exact


def test_hky_matches_reference():
    d = load("golden_hky.npz")
    for c in range(int(d["ncases"])):
        p = "c%d_" % c
        loc = HKYLocus(d[p + "seq"], d[p + "mult"], int(d[p + "totsites"]), d[p + "pi"])
        ts = trees(d, p)
        u, kappa = float(d[p + "u"]), float(d[p + "kappa"])
        n, S = loc.seq.shape
        st = O.HKYState(n, S)
        got = [st.likelihood(loc, ts[0], u, kappa)]
        st.accept()
        for t, e, acc in zip(ts[1:], d[p + "e"], d[p + "acc"]):
            got.append(st.likelihood(loc, t, u, kappa, e))
            st.accept() if acc else st.reject()
        np.testing.assert_allclose(got, d[p + "ref"], rtol=1e-12, atol=0)


def test_sw_matches_reference():
    d = load("golden_sw.npz")
    for t, A, u, r in zip(trees(d), d["A"], d["u"], d["ref"]):
        v, dl = O.sw_likelihood(A, t, float(u))
        if r[0] == -np.finfo(np.float64).max:
            assert v == r[0]
        else:
            assert abs(v - r[0]) <= 1e-12 * abs(r[0])
        np.testing.assert_allclose(dl, r[1:], rtol=1e-12, atol=1e-300)


def test_swap_matches_reference_bit_exact():
    d = load("golden_swap.npz")
    for c in range(int(d["ncases"])):
        p = "c%d_" % c
        nch, nl, tries, steps, mode, seed = (int(v) for v in d[p + "params"])
        h1, h2 = d[p + "h"]
        st, beta, allb = O.setheat(nch, h1, h2, mode)
        S = O.chain_sums(d[p + "pdg"], d[p + "probg"])
        u = O.mt_uniforms(seed, 200000)
        k = 0
        sc = np.zeros((nch, nch), np.int32)
        tc = np.zeros((nch, nch), np.int32)
        for s in range(steps):
            ok, used, _ = O.swapchains(S, beta, allb, tries, u[k:], sc, tc)
            k += used
            assert ok == d[p + "ok"][s]
            assert np.array_equal(beta, d[p + "betas"][s])
        assert np.array_equal(sc, d[p + "swapcount"])
        assert np.array_equal(tc, d[p + "tempcount"])


@pytest.mark.parametrize("case", ["a", "b1", "b2"])
def test_jointp_compat_matches_reference(case):
    d = load("golden_jointp.npz")
    if case == "a":
        rows, pts, ref, np_, nm, npops, mt = d["a_rows"], d["a_pts"], d["a_ref"], 3, 2, 2, 0
    else:
        mt = int(case[1])
        rows, pts, ref, np_, nm, npops = d["b_rows"], d["b_pts"], d["b_ref%d" % mt], 5, 8, 3
    for x, r in zip(pts, ref):
        q, ess = O.jointp(rows, np_, nm, npops, x, modeltype=mt, compat=True)
        assert abs(q - r[0]) <= 1e-12 * max(1.0, abs(r[0]))
        assert abs(ess - r[1]) <= 1e-10 * r[1]


def test_mt19937_known_answer():
    # first outputs of init_genrand(5489), the generator's published check values
    assert list(O.mt_u32(5489, 3)) == [3499211612, 581869302, 3890346734]


DE_CASES = ["full", "theta", "mig", "nested"]


def _de_active(mt, np_=3, nm=2):
    lo, hi = {0: (0, np_ + nm), 1: (0, np_), 2: (np_, np_ + nm)}[mt]
    return list(range(lo, hi)) + [np_ + nm]


@pytest.mark.parametrize("case", DE_CASES)
def test_de_peak_search_matches_reference_bit_exact(case):
    """modelloop (jointfind.cpp:746-812) with the truncated jointp, seeded
    MT19937: the restated search takes the reference's trajectory draw for
    draw, so the peak, its density and ESS are identical."""
    d = load("golden_de.npz")
    npops, mt, seed, nested = (int(v) for v in d[case + "_case"])
    xmap = d[case + "_xmap"] if nested else None
    best, ess, gens, runs, _ = O.modelloop(d["rows"], 3, 2, npops, d["upper"], mt, int(d["multiplier"]), seed,
                                           xmap=xmap, nested=nested, compat=True)
    idx = _de_active(mt)
    if nested:  # the constant m21 is part of the mapped peak too
        idx = list(range(6))
    assert np.array_equal(best[idx], d[case + "_best"][idx]), (best, d[case + "_best"])
    assert ess == float(d[case + "_ess"])
    assert gens > 10 and 2 <= runs <= 10


def test_de_rejects_nested_migration_model():
    d = load("golden_de.npz")
    best, ess, gens, runs, _ = O.modelloop(d["rows"], 3, 2, 3, d["upper"], 2, 30, 1, xmap=np.array([0.0, 0, 0, 0, 1]),
                                           nested=2)
    assert gens == -1


@pytest.mark.parametrize("expo", [False, True])
def test_margincalc_matches_reference_bit_exact(expo):
    """margincalc (surface_call_functions.cpp:119-175): plain sums on
    fillvec's grid and log'd values less yadjust, uniform and exponential
    migration priors."""
    d = load("golden_margin.npz")
    em = d["expo_mean"] if expo else None
    want = d["ref_expo"] if expo else d["ref"]
    got = np.array([O.margincalc(d["rows"], 3, 2, int(p), x, ya, int(lg), expo_mean=em)
                    for p, x, lg, ya in d["points"]])
    assert np.array_equal(got, want)
