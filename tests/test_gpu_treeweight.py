"""Genealogy weights and p(G) integrals on the GPU (ima_gpu_treeweight,
ima_gpu_tree_prob) against golden_tw.npz, made by the unmodified reference
(treeweight, sum_treeinfo, initialize_integrate_tree_prob, savegsampinf;
update_gtree_common.cpp:1680-2134, ginfo.cpp:209-377), and against the
oracle.

Tolerances: the weights (cc, mc counts; hcc, fc, fm sums; length, tlength)
are the reference's bit for bit.  The integrals q, m and probg run the
reference's incomplete gamma functions on the device's log/exp, which may
round differently from the host's by an ulp; LogDiff can amplify that when
its two arguments are close, so they are compared at 1e-10 absolute (values
are O(1-100))."""
import numpy as np
import pytest

from ima2p_gb300 import api
from oracle import pyoracle as O
from tests._golden import tw_cases

pytestmark = pytest.mark.gpu

CASES = tw_cases()
ATOL_INT = 1e-10


def _load(ctx, cs):
    pm = cs.pm
    nmg = len(pm.mg_cells)
    ctx.set_popmodel(pm, cs.th_pr[:, 0], cs.th_pr[:, 1],
                     cs.mg_pr[:, 0] if nmg else None, cs.mg_pr[:, 1] if nmg else None,
                     cs.mg_pr[:, 2] if nmg else None, expo=cs.expo)


def _inputs(cs, reps=1):
    gens = cs.gens * reps
    packed = api.pack_labelled(gens)
    gl = np.tile(np.tile(np.arange(cs.nl), cs.nch), reps)
    gt = np.tile(np.repeat(np.arange(cs.nch), cs.nl), reps)
    hval = np.array([h for _, h, _ in cs.loci])
    samp = np.array([s for _, _, s in cs.loci], np.int32)
    return packed, gl, gt, hval, samp


@pytest.mark.parametrize("c", range(len(CASES)))
def test_weights_bit_exact_and_integrals(c):
    cs = CASES[c]
    ctx = api.Context(0)
    _load(ctx, cs)
    packed, gl, gt, hval, samp = _inputs(cs)
    w = ctx.treeweight(packed, gl, gt, hval, samp, cs.tvals)
    for f in ("cc", "hcc", "fc") + (() if cs.nomig else ("mc", "fm")):
        assert np.array_equal(w[f], cs.ref[f]), f
    if cs.nomig:
        assert not w["mc"].any() and not w["fm"].any()
    assert np.array_equal(w["mignum"], cs.ref["scal"][:, 0].astype(np.int32))
    assert np.array_equal(w["lens"], cs.ref["scal"][:, 1:])
    # p(G) per chain: loci summed in locus order
    off = np.arange(cs.nch + 1, dtype=np.int32) * cs.nl
    pdg = np.linspace(-300.0, -200.0, cs.nch)
    probg, q, m, rows = ctx.tree_prob(off, pdg=pdg, group_tv=np.arange(cs.nch), rows=True)
    ref = cs.ref["pg"]
    nth = q.shape[1]
    np.testing.assert_allclose(probg, ref[:, 0], rtol=0, atol=ATOL_INT)
    np.testing.assert_allclose(q, ref[:, 1:1 + nth], rtol=0, atol=ATOL_INT)
    np.testing.assert_allclose(m, ref[:, 1 + nth:], rtol=0, atol=ATOL_INT)
    # the gsampinf rows savegsampinf would write, against the oracle's
    for ci in range(cs.nch):
        ws = [dict(cc=w["cc"][i], hcc=w["hcc"][i], fc=w["fc"][i], mc=w["mc"][i], fm=w["fm"][i])
              for i in range(ci * cs.nl, (ci + 1) * cs.nl)]
        tot = O.sum_weights(ws, cs.pm)
        want = O.gsamp_row(cs.pm, tot, q[ci], m[ci], pdg[ci], probg[ci], cs.tvals[ci])
        assert np.array_equal(rows[ci], want)


OPTION_SETS = [
    dict(parameters_by_period=True),
    dict(ancestral_sizes_largest_sampled=True, no_migration_between_nonsisters=True),
    dict(one_migration_parameter=True),
    dict(migration_between_sampled=True, single_migration_both_directions=True),
]


@pytest.mark.parametrize("opts", range(len(OPTION_SETS)))
@pytest.mark.parametrize("c", [c for c in range(len(CASES)) if CASES[c].npops >= 3 and not CASES[c].nomig])
def test_model_option_integrals(c, opts):
    """p(G) under the -j model options' maps (popmodel.build, pinned to the
    reference's setup_iparams by test_popmodel_options) against the oracle,
    including the chains a forbidden migration cell sends to -DBL_MAX."""
    from ima2p_gb300 import popmodel
    cs = CASES[c]
    opt = popmodel.ModelOptions(**OPTION_SETS[opts])
    pm = popmodel.build(cs.tree, cs.npops, options=opt, varrank=np.arange(cs.npops)[::-1] * 1.0)
    pr = popmodel.priors(pm, cs.thetaprior, cs.mprior, cs.expo)
    ctx = api.Context(0)
    ctx.set_popmodel(pm, *pr, expo=cs.expo)
    packed, gl, gt, hval, samp = _inputs(cs)
    w = ctx.treeweight(packed, gl, gt, hval, samp, cs.tvals)
    off = np.arange(cs.nch + 1, dtype=np.int32) * cs.nl
    probg, q, m = ctx.tree_prob(off, group_tv=np.arange(cs.nch))[:3]
    for ci in range(cs.nch):
        ws = [dict(cc=w["cc"][i], hcc=w["hcc"][i], fc=w["fc"][i], mc=w["mc"][i], fm=w["fm"][i])
              for i in range(ci * cs.nl, (ci + 1) * cs.nl)]
        st, pg, q_o, m_o = O.tree_prob(pm, O.sum_weights(ws, pm), *pr, expo=cs.expo, chk=pm.chk_cells)
        if pg == -np.finfo(np.float64).max:
            assert probg[ci] == pg
            continue
        np.testing.assert_allclose(probg[ci], pg, rtol=0, atol=ATOL_INT)
        np.testing.assert_allclose(q[ci], q_o, rtol=0, atol=ATOL_INT)
        np.testing.assert_allclose(m[ci], m_o, rtol=0, atol=ATOL_INT)


def test_many_genealogies_and_long_groups():
    """The 3-population case repeated 400 times (9600 genealogies, 2400 warps'
    worth of blocks): every copy gives the reference's weights, and a chain
    of 400 x 6 loci sums in locus order as sum_treeinfo does."""
    cs = CASES[1]
    reps = 400
    ctx = api.Context(0)
    _load(ctx, cs)
    packed, gl, gt, hval, samp = _inputs(cs, reps)
    w = ctx.treeweight(packed, gl, gt, hval, samp, cs.tvals)
    n1 = cs.nch * cs.nl
    for f in ("cc", "hcc", "fc", "mc", "fm"):
        assert np.array_equal(w[f], np.tile(cs.ref[f], (reps, 1))), f
    # group: every copy of chain 0's genealogies, in order
    idx = np.concatenate([r * n1 + np.arange(cs.nl) for r in range(reps)])
    sel = api.pack_labelled([cs.gens[i % n1] for i in idx])
    w2 = ctx.treeweight(sel, np.tile(np.arange(cs.nl), reps), np.zeros(len(idx), np.int32), hval, samp,
                        cs.tvals)
    probg, q, m, _ = ctx.tree_prob(np.array([0, len(idx)], np.int32), group_tv=np.zeros(1, np.int32))
    ws = [dict(cc=w2["cc"][i], hcc=w2["hcc"][i], fc=w2["fc"][i], mc=w2["mc"][i], fm=w2["fm"][i])
          for i in range(len(idx))]
    tot = O.sum_weights(ws, cs.pm)
    st, pg, oq, om = O.tree_prob(cs.pm, tot, cs.th_pr[:, 0], cs.th_pr[:, 1], cs.mg_pr[:, 0], cs.mg_pr[:, 1],
                                 cs.mg_pr[:, 2], expo=cs.expo)
    assert st == 0
    np.testing.assert_allclose(q[0], oq, rtol=0, atol=ATOL_INT)
    np.testing.assert_allclose(m[0], om, rtol=0, atol=ATOL_INT)
    np.testing.assert_allclose(probg[0], pg, rtol=0, atol=ATOL_INT * 10)


def test_genealogy_the_model_cannot_hold_is_rejected():
    cs = CASES[1]
    ctx = api.Context(0)
    _load(ctx, cs)
    packed, gl, gt, hval, samp = _inputs(cs)
    node_off, up0, time, pop, mig_off, mig_t, mig_p = packed
    bad = pop.copy()
    ng0 = cs.loci[0][0]
    bad[ng0] = 2 * cs.npops - 2  # the first coalescence placed in the root population
    with pytest.raises(api.ImaError):
        ctx.treeweight((node_off, up0, time, bad, mig_off, mig_t, mig_p), gl, gt, hval, samp, cs.tvals)
    # the context stays usable
    w = ctx.treeweight(packed, gl, gt, hval, samp, cs.tvals)
    assert np.array_equal(w["fc"], cs.ref["fc"])
    with pytest.raises(api.ImaError):  # samppop that does not match the genealogy
        ctx.treeweight(packed, gl, gt, hval, samp + 1, cs.tvals)
    # migration offsets that decrease inside a genealogy (its end points intact):
    # node j of genealogy 0 gets a negative count
    j = next(i for i in range(node_off[0] + 1, node_off[1] - 1) if mig_off[i] > mig_off[node_off[0]])
    bad_off = mig_off.copy()
    bad_off[j + 1] = mig_off[j] - 1
    with pytest.raises(api.ImaError):
        ctx.treeweight((node_off, up0, time, pop, bad_off, mig_t, mig_p), gl, gt, hval, samp, cs.tvals)
    assert np.array_equal(ctx.treeweight(packed, gl, gt, hval, samp, cs.tvals)["fc"], cs.ref["fc"])
    with pytest.raises(api.ImaError):  # groups beyond the genealogies
        ctx.tree_prob(np.array([0, len(gl) + 1], np.int32))


def test_mmode_rows_feed_the_resident_surface():
    """Sampling steps on the device: each step's gsampinf rows (one per
    chain here) are appended to the resident surface, which the L-mode
    functions then read -- against the oracle's jointp and margincalc on the
    same rows copied to the host."""
    cs = CASES[1]  # 3 populations: 5 theta, 8 migration parameters, rowlen 48
    ctx = api.Context(0)
    _load(ctx, cs)
    packed, gl, gt, hval, samp = _inputs(cs)
    off = np.arange(cs.nch + 1, dtype=np.int32) * cs.nl
    host_rows = []
    for step in range(3):
        ctx.treeweight(packed, gl, gt, hval, samp, cs.tvals)
        pdg = np.linspace(-250.0, -210.0, cs.nch) - step
        _, _, _, rows = ctx.tree_prob(off, pdg=pdg, group_tv=np.arange(cs.nch), rows=True)
        order = [3, 0, 2, 1] if step == 1 else list(range(cs.nch))
        ctx.surface_append_tree_rows(order[:2])
        ctx.surface_append_tree_rows(order[2:])
        host_rows += [rows[i] for i in order]
    host_rows = np.array(host_rows, np.float32)
    G, np_, nm, npops = ctx.surface_info()
    assert (G, np_, nm, npops) == (len(host_rows), 5, 8, 3)
    assert np.array_equal(ctx.surface_get_rows(), host_rows)
    rng = np.random.default_rng(6)
    pts = np.column_stack([rng.uniform(0.5, 10.0, (6, 5)), rng.uniform(0.05, 1.5, (6, 8))])
    q, _ = ctx.surface_eval(pts, method=api.SURF_FP64)
    want = np.array([O.jointp(host_rows, 5, 8, 3, x)[0] for x in pts])
    np.testing.assert_allclose(q, want, rtol=1e-12)
    for p_, x in ((0, 2.5), (4, 7.0), (7, 0.4)):
        assert abs(ctx.margincalc(p_, x)[0] - O.margincalc(host_rows, 5, 8, p_, x)) <= 1e-12 * abs(O.margincalc(host_rows, 5, 8, p_, x))
    with pytest.raises(api.ImaError):  # the caller's row width must be the surface's
        ctx.surface_get_rows(rowlen=47)
    # rows of a model with another shape are refused
    other = CASES[0]
    _load(ctx, other)
    p2, gl2, gt2, hv2, sp2 = _inputs(other)
    ctx.treeweight(p2, gl2, gt2, hv2, sp2, other.tvals)
    ctx.tree_prob(np.arange(other.nch + 1, dtype=np.int32) * other.nl)
    with pytest.raises(api.ImaError):
        ctx.surface_append_tree_rows([0])
