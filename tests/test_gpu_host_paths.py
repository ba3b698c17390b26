"""Host paths of the boundary on the GPU: set_genealogies splits long lists
over host threads (results must be those of one-by-one uploads, bitwise), and
ima_gpu_eval reuses its staged requests when a call repeats the previous
request arrays (new genealogies must still be seen, changed rates must not be
missed)."""
import numpy as np
import pytest

from ima2p_gb300 import api, workloads
from tests._gpu import ctx_with

pytestmark = pytest.mark.gpu


def _hky_ctx(wl):
    ctx = ctx_with(wl.loci, wl.nruns, wl.cpr)
    return ctx


def test_parallel_upload_matches_one_by_one():
    wl = workloads.make_hky(seed=31, nloci=12, nch=32, ncopies=10, nbases=300)   # 384 pairs: parallel path
    ci, li = wl.pairs()
    pci, pli, up0, up1, down, tm = wl.packed()
    u, par = wl.u.ravel(), wl.par.ravel()
    a = _hky_ctx(wl)
    wl.upload(a)  # set_genealogies over all 384 pairs at once
    b = _hky_ctx(wl)
    for (c, l), p in wl.pi.items():
        b.set_pi(c, l, p)
    for c, l in zip(pci, pli):
        b.set_genealogy(int(c), int(l), wl.tree(int(c), int(l)))
    ra, _ = a.eval(ci, li, u, par)
    rb, _ = b.eval(ci, li, u, par)
    assert np.array_equal(ra, rb)
    # re-timed (topology kept) and re-shaped lists go through the same path
    scaled = np.where(tm > 0, tm * 1.01, tm)
    a.set_genealogies(pci, pli, up0, up1, down, scaled)
    off = 0
    for k, (c, l) in enumerate(zip(pci, pli)):
        g = wl.tree(int(c), int(l)).copy()
        nl = len(g.up0)
        g.time = scaled[off:off + nl].copy()
        off += nl
        b.set_genealogy(int(c), int(l), g)
    assert np.array_equal(a.eval(ci, li, u, par)[0], b.eval(ci, li, u, par)[0])


@pytest.mark.parametrize("kind", ["hky", "is", "is_long", "is_huge"])
def test_set_times_matches_set_genealogies(kind):
    """The times-only upload (long lists over the host threads, short ones
    on the caller's) gives the bits of a full upload with the same times,
    tree lengths included (the infinite-sites likelihood reads them), and
    refuses a pair that holds no genealogy."""
    if kind == "hky":
        wl = workloads.make_hky(seed=33, nloci=12, nch=32, ncopies=10, nbases=300)   # 384 pairs
    elif kind == "is":
        wl = workloads.make_is(seed=34)
    elif kind == "is_long":
        wl = workloads.make_is(seed=38, nloci=10, nch=200)   # 78,000 nodes: lengths summed later
    else:
        wl = workloads.make_is(seed=41, nloci=10, nch=12000)   # 4.7 M nodes: the copy engine's path
    ci, li = wl.pairs()
    pci, pli, up0, up1, down, tm = wl.packed()
    u, par = wl.u.ravel(), wl.par.ravel()
    a, b = _hky_ctx(wl), _hky_ctx(wl)
    wl.upload(a)
    wl.upload(b)
    a.eval(ci, li, u, par)
    b.eval(ci, li, u, par)
    nl = np.array([2 * wl.tree(int(c), int(l)).n - 1 for c, l in zip(pci, pli)])
    ends = np.cumsum(nl)
    starts = ends - nl
    rng = np.random.default_rng(7)
    # every pair in item order (copies started while the host stages), the
    # first five, every pair shuffled (staged, copied at the evaluation), and
    # one pair of the first kind followed by a full upload of another
    for case in ("all", "five", "shuffled", "mixed"):
        f = np.repeat(rng.uniform(0.9, 1.1, size=len(nl)), nl)   # one factor per genealogy keeps the order
        scaled = np.where(tm > 0, tm * f, tm)
        order = {"all": np.arange(len(pci)), "five": np.arange(5),
                 "shuffled": rng.permutation(len(pci)), "mixed": np.arange(len(pci))}[case]
        idx = np.concatenate([np.arange(starts[k], ends[k]) for k in order])
        a.set_times(pci[order], pli[order], scaled[idx])
        b.set_genealogies(pci[order], pli[order], up0[idx], up1[idx], down[idx], scaled[idx])
        if case == "mixed":
            k = len(pci) // 2
            g = wl.tree(int(pci[k]), int(pli[k])).copy()
            g.time = np.where(g.time > 0, g.time * 1.05, g.time)
            a.set_genealogy(int(pci[k]), int(pli[k]), g)
            b.set_genealogy(int(pci[k]), int(pli[k]), g)
        ra, sa = a.eval(ci, li, u, par)
        rb, sb = b.eval(ci, li, u, par)
        assert np.array_equal(ra, rb) and np.array_equal(sa, sb), case
    fresh = _hky_ctx(wl)
    with pytest.raises(api.ImaError):
        fresh.set_times([0], [0], tm[:nl[0]])


@pytest.mark.parametrize("kind", ["sw", "is", "is_long", "sw_long", "mixed_long", "is_huge"])
def test_eval_times_matches_set_times_then_eval(kind):
    """The one-call re-timing and evaluation gives the bits of set_times
    followed by eval, for a run of pairs in item order (read in place where
    the device reads host memory) and for a shuffled list, with and without
    given lengths.  is_long has more nodes than the one-kernel short-run
    path takes: its lengths are summed later, before the infinite-sites
    evaluation reads them.  sw_long and mixed_long are long enough that the
    run is read in two parts, each part's evaluation waiting for its own
    times only."""
    if kind == "sw":
        wl = workloads.make_sw(seed=35, nloci=10, nch=16, per_pop=10)
    elif kind == "is":
        wl = workloads.make_is(seed=36)
    elif kind == "is_long":
        wl = workloads.make_is(seed=37, nloci=10, nch=200)   # 78,000 nodes
    elif kind == "sw_long":
        wl = workloads.make_sw(seed=39, nloci=24, nch=64, per_pop=30)   # 275,000 nodes
    elif kind == "mixed_long":
        wl = workloads.make_mixed(seed=40, n_hky=12, n_sw=8, nruns=2, cpr=64)
    else:
        wl = workloads.make_is(seed=42, nloci=10, nch=12000)   # 4.7 M nodes: the copy engine's path
    ci, li = wl.pairs()
    pci, pli, up0, up1, down, tm = wl.packed()
    u, par = wl.u.ravel(), wl.par.ravel()
    a, b = _hky_ctx(wl), _hky_ctx(wl)
    wl.upload(a)
    wl.upload(b)
    nl = np.array([2 * wl.tree(int(c), int(l)).n - 1 for c, l in zip(pci, pli)])
    ends = np.cumsum(nl)
    starts = ends - nl
    rng = np.random.default_rng(8)
    for case in ("run", "shuffled", "run_lengths"):
        f = np.repeat(rng.uniform(0.9, 1.1, size=len(nl)), nl)
        scaled = np.where(tm > 0, tm * f, tm)
        order = rng.permutation(len(pci)) if case == "shuffled" else np.arange(len(pci))
        idx = np.concatenate([np.arange(starts[k], ends[k]) for k in order])
        lengths = rng.uniform(1.0, 3.0, size=len(order)) if case == "run_lengths" else None
        ra, sa = a.eval_times(pci[order], pli[order], scaled[idx], u[order], par[order], length=lengths)
        b.set_times(pci[order], pli[order], scaled[idx], length=lengths)
        rb, sb = b.eval(pci[order], pli[order], u[order], par[order])
        assert np.array_equal(ra, rb) and np.array_equal(sa, sb), case
        # and the state left behind is the same
        assert np.array_equal(a.eval(ci, li, u, par)[0], b.eval(ci, li, u, par)[0]), case


def test_parallel_upload_rejects_a_bad_genealogy():
    wl = workloads.make_hky(seed=32, nloci=10, nch=32, ncopies=10, nbases=200)
    pci, pli, up0, up1, down, tm = wl.packed()
    ctx = _hky_ctx(wl)
    bad_down = down.copy()
    nl = 2 * 20 - 1
    k = 150 * nl + nl - 1  # the root of pair 150 gets a parent: two parents link to it
    bad_down[k] = 21
    with pytest.raises(api.ImaError):
        ctx.set_genealogies(pci, pli, up0, up1, bad_down, tm)


def test_eval_reuses_requests_but_sees_new_data():
    wl = workloads.make_hky(seed=33, nloci=8, nch=32, ncopies=10, nbases=300)
    ci, li = wl.pairs()
    pci, pli, up0, up1, down, tm = wl.packed()
    u, par = wl.u.ravel().copy(), wl.par.ravel()
    ctx = _hky_ctx(wl)
    wl.upload(ctx)
    r0 = ctx.eval(ci, li, u, par)[0]
    # new genealogy times, identical request arrays: the cached requests see them
    scaled = np.where(tm > 0, tm * 1.2, tm)
    ctx.set_genealogies(pci, pli, up0, up1, down, scaled)
    r1 = ctx.eval(ci, li, u, par)[0]
    fresh = _hky_ctx(wl)
    wl.upload(fresh)
    fresh.set_genealogies(pci, pli, up0, up1, down, scaled)
    assert np.array_equal(r1, fresh.eval(ci, li, u, par)[0])
    assert not np.array_equal(r0, r1)
    # one changed rate is a different request list
    u[7] *= 1.5
    r2 = ctx.eval(ci, li, u, par)[0]
    assert r2[7] != r1[7] and np.array_equal(np.delete(r2, 7), np.delete(r1, 7))
