"""Stepwise-mutation likelihood on the GPU against the reference's golden
values: per-locus totals and per-branch dlikeA, including a zero Bessel term
(total -DBL_MAX) and x > 700.  The fast form must stay within SW_FAST_ATOL of
the reference per locus (the 1e-6 target, with margin) and SW_BRANCH_ATOL
per branch (float-float terms, about 1e-11 each; short branches take the
series of log(1 + u) with its tail in FP32); the FP64 form within 1e-12
relative."""
import numpy as np
import pytest

from ima2p_gb300 import api, synth
from oracle import pyoracle as O
from tests._golden import load, trees
from tests._gpu import ctx_with

pytestmark = pytest.mark.gpu

SW_FAST_ATOL = 1e-8      # per-locus |log L - reference|
SW_BRANCH_ATOL = 2e-10   # per-branch |dlikeA - reference|
DBLMAX = np.finfo(np.float64).max


@pytest.mark.parametrize("prec", [api.PREC_FAST, api.PREC_FP64])
def test_sw_golden(prec):
    d = load("golden_sw.npz")
    ts = trees(d)
    n = ts[0].n
    ctx = ctx_with([("sw", n, 1)], 1, len(ts))
    for ci, (t, A) in enumerate(zip(ts, d["A"])):
        ctx.set_genealogy(ci, 0, t)
        ctx.set_alleles(ci, 0, A)
    res, st = ctx.eval(np.arange(len(ts)), np.zeros(len(ts)), d["u"], precision=prec)
    for ci, r in enumerate(d["ref"]):
        if r[0] == -DBLMAX:
            assert res[ci] == -DBLMAX and st[ci] == api.EVAL_SW_ZERO
            continue
        if prec == api.PREC_FAST:
            assert abs(res[ci] - r[0]) <= SW_FAST_ATOL, (ci, res[ci], r[0])
        else:
            assert abs(res[ci] - r[0]) <= 1e-12 * abs(r[0])
        dl = ctx.get_dlikeA(ci, 0)
        if prec == api.PREC_FP64:
            np.testing.assert_allclose(dl, r[1:], rtol=1e-11, atol=1e-11)
        else:
            np.testing.assert_allclose(dl, r[1:], rtol=0, atol=SW_BRANCH_ATOL)


def test_sw_config3_shape_vs_oracle():
    rng = np.random.default_rng(5)
    nloci, nch = 6, 4
    base = [synth.three_pop_tree(rng, [30, 30, 30], theta=4.0, mig=0.05) for _ in range(nloci)]
    ctx = ctx_with([("sw", 90, 1)] * nloci, 1, nch)
    ci, li, u, want = [], [], [], []
    worst = 0.0
    for c in range(nch):
        for l in range(nloci):
            t = synth.jitter_times(rng, base[l], 0.2)
            A = synth.sw_alleles(rng, t, float(rng.lognormal(0, 0.5)))
            ctx.set_genealogy(c, l, t)
            ctx.set_alleles(c, l, A)
            uu = float(rng.lognormal(0, 0.5))
            want.append(O.sw_likelihood(A, t, uu)[0])
            ci.append(c), li.append(l), u.append(uu)
    fast, _ = ctx.eval(ci, li, u, precision=api.PREC_FAST)
    slow, _ = ctx.eval(ci, li, u, precision=api.PREC_FP64)
    np.testing.assert_allclose(slow, want, rtol=1e-12)
    assert np.max(np.abs(fast - np.array(want))) <= SW_FAST_ATOL


def test_sw_bessel_edge_terms():
    """Single-branch genealogies sweep |d| and x across the A&S / Miller
    regimes and the float-float fallbacks."""
    cases = []
    for d in (0, 1, 2, 3, 5, 9, 17, 30):
        for x in (1e-12, 1e-6, 0.01, 0.3, 1.0, 3.7499, 3.75, 10.0, 80.0, 699.0, 701.0):
            cases.append((d, x))
    n = 2
    ctx = ctx_with([("sw", n, 1)], 1, len(cases))
    for ci, (d, x) in enumerate(cases):
        g = synth.Genealogy(np.array([-1, -1, 0]), np.array([-1, -1, 1]), np.array([2, 2, -1]),
                            np.array([x, x, -1.0]), 2)
        ctx.set_genealogy(ci, 0, g)
        ctx.set_alleles(ci, 0, np.array([20 + d, 20, 20]))
    res, st = ctx.eval(np.arange(len(cases)), np.zeros(len(cases)), np.ones(len(cases)))
    for k, (d, x) in enumerate(cases):
        want = O.lib().ora_sw_branch_term(d, x, 1.0) + O.lib().ora_sw_branch_term(0, x, 1.0)
        if want <= -1e99:
            assert st[k] == api.EVAL_SW_ZERO
        else:
            assert abs(res[k] - want) <= 2 * SW_BRANCH_ATOL + 1e-9 * abs(want), (d, x, res[k], want)


@pytest.mark.parametrize("prec", [api.PREC_FAST, api.PREC_FP64])
def test_sw_allele_edit_list_gives_update_delta(prec):
    """finishSWupdateA (update_gtree_common.cpp:2219-2362) proposes a new
    allele for one internal node and returns likeadj - oldlikeadj, the change
    of the branch terms that touch it.  Shipped as an edit list, the change is
    the difference of the batched evaluations after and before the edits; it
    must equal the oracle's difference of full likelihoods."""
    rng = np.random.default_rng(23)
    nloci, nch = 3, 8
    ctx = ctx_with([("sw", 40, 1)] * nloci, 1, nch)
    trees_, alle, ci, li, u = {}, {}, [], [], []
    for c in range(nch):
        for l in range(nloci):
            t = synth.three_pop_tree(rng, [14, 13, 13], theta=4.0, mig=0.05)
            A = synth.sw_alleles(rng, t, 1.0)
            ctx.set_genealogy(c, l, t)
            ctx.set_alleles(c, l, A)
            trees_[c, l], alle[c, l] = t, A
            ci.append(c), li.append(l), u.append(float(rng.lognormal(0, 0.3)))
    before, _ = ctx.eval(ci, li, u, precision=prec)
    # one moved node per chain-locus: an internal node, its allele stepped by -3..3
    node = [int(rng.integers(40, 79)) for _ in ci]
    newA = [int(alle[c, l][v] + rng.integers(-3, 4)) for c, l, v in zip(ci, li, node)]
    ctx.set_allele_edits(ci, li, node, newA)
    after, _ = ctx.eval(ci, li, u, precision=prec)
    tol = 2 * SW_FAST_ATOL if prec == api.PREC_FAST else 1e-10
    for k, (c, l) in enumerate(zip(ci, li)):
        A2 = alle[c, l].copy()
        A2[node[k]] = newA[k]
        want = O.sw_likelihood(A2, trees_[c, l], u[k])[0] - O.sw_likelihood(alle[c, l], trees_[c, l], u[k])[0]
        assert abs((after[k] - before[k]) - want) <= tol, (k, after[k] - before[k], want)
    # an invalid entry rejects the whole list
    with pytest.raises(api.ImaError):
        ctx.set_allele_edits([0, 0], [0, 0], [40, 999], [20, 20])


@pytest.mark.parametrize("prec", [api.PREC_FAST, api.PREC_FP64])
def test_sw_linked_markers(prec):
    """A locus of three linked stepwise markers (L[li].nlinked = 3): each
    marker ai has its own allele states on the same genealogy, and
    likelihoodSW(ci, li, ai, u, tr) evaluates one marker with its own rate.
    Every (chain, marker) request in one batch, against the oracle; dlikeA per
    marker; an edit of one marker leaves the others' terms unchanged."""
    rng = np.random.default_rng(29)
    nch, nm = 6, 3
    ctx = ctx_with([("sw", 36, nm)], 1, nch)
    trees_, alle = {}, {}
    for c in range(nch):
        t = synth.three_pop_tree(rng, [12, 12, 12], theta=4.0, mig=0.05)
        ctx.set_genealogy(c, 0, t)
        trees_[c] = t
        for a in range(nm):
            A = synth.sw_alleles(rng, t, float(rng.lognormal(0, 0.4)))
            ctx.set_alleles(c, 0, A, ai=a)
            alle[c, a] = A
    ci = np.repeat(np.arange(nch), nm)
    ai = np.tile(np.arange(nm), nch)
    u = rng.lognormal(0, 0.4, size=len(ci))
    tr = rng.uniform(0.5, 2.0, size=len(ci))
    res, st = ctx.eval(ci, np.zeros(len(ci), np.int32), u, tr, ai=ai, precision=prec)
    tol = SW_FAST_ATOL if prec == api.PREC_FAST else 1e-12
    for k in range(len(ci)):
        want, dl_want = O.sw_likelihood(alle[ci[k], ai[k]], trees_[ci[k]], u[k], tr[k])
        assert abs(res[k] - want) <= tol * (1 if prec == api.PREC_FAST else abs(want)), (k, res[k], want)
    # dlikeA of the last evaluation of each (chain, marker)
    for k in range(len(ci)):
        dl = ctx.get_dlikeA(int(ci[k]), 0, int(ai[k]))
        dl_want = O.sw_likelihood(alle[ci[k], ai[k]], trees_[ci[k]], u[k], tr[k])[1]
        np.testing.assert_allclose(dl, dl_want, rtol=0 if prec == api.PREC_FAST else 1e-11,
                                   atol=SW_BRANCH_ATOL if prec == api.PREC_FAST else 1e-11)
    # an edit of marker 1 on chain 0 changes only that marker's evaluation
    node = 40
    ctx.set_allele_edits([0], [0], [node], [int(alle[0, 1][node]) + 2], ai=[1])
    res2, _ = ctx.eval(ci, np.zeros(len(ci), np.int32), u, tr, ai=ai, precision=prec)
    changed = np.flatnonzero(res2 != res)
    assert list(changed) == [1]
