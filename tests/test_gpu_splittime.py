"""The split-time update (ima2p_gb300.splittime.changet_ry1) with its
weights, p(G) and infinite-sites likelihoods on the GPU
(ima_gpu_treeweight, ima_gpu_tree_prob, ima_gpu_eval) against
golden_ry.npz, made by the unmodified reference's changet_RY1 with the same
MT19937 seed: the same decision at every one of 90 steps over three chains,
split times and node and migration times bit for bit; probg within 1e-10
(device log/exp), pdg within 1e-12 relative (IS FP64)."""
import numpy as np
import pytest

from ima2p_gb300 import api, splittime
from tests._golden import load
from tests._splittime import RyCase, final_times, run_chain_set

pytestmark = pytest.mark.gpu


def _device_backend(case):
    ctx = api.Context(0)
    for q in case.seqs:
        ctx.add_locus_is(q)
    ctx.set_chains(1, case.nch)
    th_max, th_min, mg_max, mg_min, mg_mean = case.priors()
    ctx.set_popmodel(case.pm, th_max, th_min, mg_max, mg_min, mg_mean)
    return ctx, splittime.DeviceBackend(ctx, np.ones(case.nl), case.samps, case.us)


def test_device_driven_update_follows_the_reference():
    case = RyCase()
    ctx, backend = _device_backend(case)
    res, states = run_chain_set(case, backend, api.MT19937(case.seed))
    ref = case.res
    assert np.array_equal(res[:, 0], ref[:, 0])
    assert np.array_equal(res[:, 1], ref[:, 1])
    np.testing.assert_allclose(res[:, 2], ref[:, 2], rtol=0, atol=1e-10)
    np.testing.assert_allclose(res[:, 3], ref[:, 3], rtol=1e-12)
    t, m = final_times(case, states)
    root = np.concatenate([lg.g.down == -1 for st in states for lg in st.gens])
    assert np.array_equal(t[~root], case.times[~root])
    assert np.array_equal(m, case.migt)
    ctx.close()


def test_batched_sweep_follows_the_reference():
    """changet_ry1_sweep: every chain's proposal in one ima_gpu_treeweight /
    ima_gpu_tree_prob / ima_gpu_set_genealogies / ima_gpu_eval round; the
    generator draws in the sequential run's order."""
    from tests._splittime import run_sweeps
    case = RyCase()
    ctx = api.Context(0)
    for q in case.seqs:
        ctx.add_locus_is(q)
    ctx.set_chains(1, case.nch)
    ctx.set_popmodel(case.pm, *case.priors())
    backend = splittime.SweepBackend(ctx, np.ones(case.nl), case.samps, case.us)
    res, cs = run_sweeps(case, backend, api.MT19937(case.seed))
    ref = case.res
    assert np.array_equal(res[:, 0], ref[:, 0])
    assert np.array_equal(res[:, 1], ref[:, 1])
    np.testing.assert_allclose(res[:, 2], ref[:, 2], rtol=0, atol=1e-10)
    np.testing.assert_allclose(res[:, 3], ref[:, 3], rtol=1e-12)
    assert np.array_equal(cs.time[cs.edge], case.times[cs.edge])
    assert np.array_equal(cs.mig_t, case.migt)
    ctx.close()


def test_resident_sweep_follows_the_reference():
    """ResidentChainSet: genealogies, labels and times stay on the GPU; the
    rubber band moves them there (ima_gpu_rubber_band), the weights are
    computed in place (ima_gpu_chain_weights).  Same decisions and times as
    the reference's changet_RY1; then a host upload of one genealogy leaves
    every other chain-locus as the device had it."""
    case = RyCase()
    ctx = api.Context(0)
    for q in case.seqs:
        ctx.add_locus_is(q)
    ctx.set_chains(1, case.nch)
    ctx.set_popmodel(case.pm, *case.priors())
    cs = splittime.ResidentChainSet(ctx, case.fresh_gens(), [case.d["tv0"]] * case.nch, case.betas,
                                    np.ones(case.nl), case.samps, case.us)
    rng = api.MT19937(case.seed)
    res = []
    for s0 in range(0, len(case.steps), case.nch):
        periods = [case.steps[s0 + c][1] for c in range(case.nch)]
        acc = cs.sweep(periods, rng, case.tprior, case.npops)
        for c in range(case.nch):
            res.append((int(acc[c]), float(cs.tvals[c, periods[c]]), float(cs.probg[c]), float(cs.pdgsum[c])))
    res, ref = np.array(res), case.res
    assert np.array_equal(res[:, 0], ref[:, 0])
    assert np.array_equal(res[:, 1], ref[:, 1])
    np.testing.assert_allclose(res[:, 2], ref[:, 2], rtol=0, atol=1e-10)
    np.testing.assert_allclose(res[:, 3], ref[:, 3], rtol=1e-12)
    base = case.fresh_gens()
    off = 0
    moff = 0
    for ci in range(case.nch):
        for li in range(case.nl):
            g = base[ci][li]
            nl = len(g.pop)
            t, m = ctx.get_times(ci, li, nl)
            edge = g.g.down != -1
            assert np.array_equal(t[edge], case.times[off:off + nl][edge])
            assert np.array_equal(m, case.migt[moff:moff + len(m)])
            off += nl
            moff += len(m)
    # a host upload of the first and last chain-locus after device moves:
    # the range upload spans every other one, which must keep the device's
    # times and lengths
    before = cs._eval()
    ends = [(0, 0), (case.nch - 1, case.nl - 1)]
    gs = []
    for ci, li in ends:
        t_, _ = ctx.get_times(ci, li, len(base[ci][li].pop))
        g = base[ci][li].g.copy()
        g.time = t_
        gs.append(g)
    ctx.set_genealogies(np.array([e[0] for e in ends]), np.array([e[1] for e in ends]),
                        np.concatenate([g.up0 for g in gs]), np.concatenate([g.up1 for g in gs]),
                        np.concatenate([g.down for g in gs]), np.concatenate([g.time for g in gs]),
                        length=np.full(2, -1.0))
    after = cs._eval()
    mask = np.ones_like(before, bool)
    for ci, li in ends:
        mask[ci, li] = False
    assert np.array_equal(before[mask], after[mask])
    ctx.close()


def test_library_drawn_sweep_follows_the_reference():
    """ima_gpu_changet_ry1_sweep_mt: getnewt's and the acceptance draws made
    in the library from the caller's MT19937, split times from the context --
    the reference's decisions and times again, and the generator left where
    the reference leaves it."""
    case = RyCase()
    ctx = api.Context(0)
    for q in case.seqs:
        ctx.add_locus_is(q)
    ctx.set_chains(1, case.nch)
    ctx.set_popmodel(case.pm, *case.priors())
    cs = splittime.ResidentChainSet(ctx, case.fresh_gens(), [case.d["tv0"]] * case.nch, case.betas,
                                    np.ones(case.nl), case.samps, case.us)
    rng = api.MT19937(case.seed)
    res = []
    for s0 in range(0, len(case.steps), case.nch):
        periods = [case.steps[s0 + c][1] for c in range(case.nch)]
        acc = cs.sweep_device_mt(periods, rng, case.tprior)
        for c in range(case.nch):
            res.append((int(acc[c]), float(cs.tvals[c, periods[c]]), float(cs.probg[c]), float(cs.pdgsum[c])))
    res, ref = np.array(res), case.res
    assert np.array_equal(res[:, 0], ref[:, 0])
    assert np.array_equal(res[:, 1], ref[:, 1])
    np.testing.assert_allclose(res[:, 2], ref[:, 2], rtol=0, atol=1e-10)
    np.testing.assert_allclose(res[:, 3], ref[:, 3], rtol=1e-12)
    assert np.array_equal(ctx.get_split_times(), cs.tvals)
    # two draws per chain and step: the Python-driven run leaves the same state
    rng2 = api.MT19937(case.seed)
    for _ in range(2 * len(case.steps)):
        rng2.uniform()
    assert rng.uniform() == rng2.uniform()
    ctx.close()


def test_device_decided_sweep_follows_the_reference():
    """ima_gpu_changet_ry1_sweep: band, weights, likelihoods and the MH
    decision on the device in one call per sweep -- the reference's
    decisions and times again."""
    case = RyCase()
    ctx = api.Context(0)
    for q in case.seqs:
        ctx.add_locus_is(q)
    ctx.set_chains(1, case.nch)
    ctx.set_popmodel(case.pm, *case.priors())
    cs = splittime.ResidentChainSet(ctx, case.fresh_gens(), [case.d["tv0"]] * case.nch, case.betas,
                                    np.ones(case.nl), case.samps, case.us)
    rng = api.MT19937(case.seed)
    res = []
    for s0 in range(0, len(case.steps), case.nch):
        periods = [case.steps[s0 + c][1] for c in range(case.nch)]
        acc = cs.sweep_device(periods, rng, case.tprior, case.npops)
        for c in range(case.nch):
            res.append((int(acc[c]), float(cs.tvals[c, periods[c]]), float(cs.probg[c]), float(cs.pdgsum[c])))
    res, ref = np.array(res), case.res
    assert np.array_equal(res[:, 0], ref[:, 0])
    assert np.array_equal(res[:, 1], ref[:, 1])
    np.testing.assert_allclose(res[:, 2], ref[:, 2], rtol=0, atol=1e-10)
    np.testing.assert_allclose(res[:, 3], ref[:, 3], rtol=1e-12)
    base = case.fresh_gens()
    off = moff = 0
    for ci in range(case.nch):
        for li in range(case.nl):
            nl = len(base[ci][li].pop)
            t, m = ctx.get_times(ci, li, nl)
            edge = base[ci][li].g.down != -1
            assert np.array_equal(t[edge], case.times[off:off + nl][edge])
            assert np.array_equal(m, case.migt[moff:moff + len(m)])
            off += nl
            moff += len(m)
    ctx.close()


def _resident_context(case):
    ctx = api.Context(0)
    for q in case.seqs:
        ctx.add_locus_is(q)
    ctx.set_chains(1, case.nch)
    ctx.set_popmodel(case.pm, *case.priors())
    return ctx


def _run(cs, case, rng, sweeps):
    res = []
    for s0 in sweeps:
        periods = [case.steps[s0 + c][1] for c in range(case.nch)]
        acc = cs.sweep_device(periods, rng, case.tprior, case.npops)
        for c in range(case.nch):
            res.append((int(acc[c]), float(cs.tvals[c, periods[c]]), float(cs.probg[c]), float(cs.pdgsum[c])))
    return res


def test_checkpoint_resume_continues_the_run(tmp_path):
    """ima_gpu_checkpoint_write after 12 sweeps, then ima_gpu_checkpoint_read
    into a fresh context with the saved generator: the remaining 18 sweeps
    make the uninterrupted run's decisions, split times, p(G) and likelihood
    sums bit for bit (and so the reference's), and leave the same times on
    the device.  A file for other chains, a truncated file and a file that
    is not a checkpoint are refused."""
    case = RyCase()
    starts = list(range(0, len(case.steps), case.nch))
    ctx = _resident_context(case)
    cs = splittime.ResidentChainSet(ctx, case.fresh_gens(), [case.d["tv0"]] * case.nch, case.betas,
                                    np.ones(case.nl), case.samps, case.us)
    whole = _run(cs, case, api.MT19937(case.seed), starts)
    base = case.fresh_gens()
    want_t = [ctx.get_times(ci, li, len(base[ci][li].pop)) for ci in range(case.nch) for li in range(case.nl)]
    ctx.close()

    path = tmp_path / "chains.ckp"
    ctx = _resident_context(case)
    cs = splittime.ResidentChainSet(ctx, case.fresh_gens(), [case.d["tv0"]] * case.nch, case.betas,
                                    np.ones(case.nl), case.samps, case.us)
    rng = api.MT19937(case.seed)
    first = _run(cs, case, rng, starts[:12])
    ctx.checkpoint_write(path, rng)
    saved_tv, saved_pdg, saved_pg = cs.tvals.copy(), ctx.get_pdg(), ctx.get_probg()
    ctx.close()

    ctx = _resident_context(case)
    rng2 = api.MT19937(1)
    cs2 = splittime.ResidentChainSet.resume(ctx, path, case.us, rng=rng2)
    assert np.array_equal(cs2.tvals, saved_tv)
    assert np.array_equal(cs2.pdg, saved_pdg)
    assert np.array_equal(cs2.probg, saved_pg)
    assert np.array_equal(np.frombuffer(bytes(rng2), np.uint8), np.frombuffer(bytes(rng), np.uint8))
    rest = _run(cs2, case, rng2, starts[12:])
    assert first + rest == whole
    res, ref = np.array(whole), case.res
    assert np.array_equal(res[:, 0], ref[:, 0])
    assert np.array_equal(res[:, 1], ref[:, 1])
    k = 0
    for ci in range(case.nch):
        for li in range(case.nl):
            t, m = ctx.get_times(ci, li, len(base[ci][li].pop))
            edge = base[ci][li].g.down != -1
            assert np.array_equal(t[edge], want_t[k][0][edge])
            assert np.array_equal(m, want_t[k][1])
            k += 1
    ctx.close()

    other = api.Context(0)  # one chain fewer
    for q in case.seqs:
        other.add_locus_is(q)
    other.set_chains(1, case.nch - 1)
    other.set_popmodel(case.pm, *case.priors())
    with pytest.raises(api.ImaError):
        other.checkpoint_read(path)
    other.close()
    data = path.read_bytes()
    short = tmp_path / "short.ckp"
    short.write_bytes(data[:len(data) // 2])
    junk = tmp_path / "junk.ckp"
    junk.write_bytes(b"not a checkpoint" * 64)
    ctx = _resident_context(case)
    for bad in (short, junk):
        with pytest.raises(api.ImaError):
            ctx.checkpoint_read(bad)
    ctx.close()
    # a file whose population section does not match its loci (samppop of
    # locus 0 one gene too many) is refused before anything is replaced: the
    # context keeps its genealogies, p(G) and split times
    import ctypes
    bad = bytearray(data)
    ntv = case.nch * (case.npops - 1)
    off = len(bad) - ctypes.sizeof(api.MT19937) - ntv * 8 - case.nl * case.npops * 4
    v = int.from_bytes(bytes(bad[off:off + 4]), "little", signed=True) + 1
    bad[off:off + 4] = v.to_bytes(4, "little", signed=True)
    badp = tmp_path / "bad_pops.ckp"
    badp.write_bytes(bytes(bad))
    ctx = _resident_context(case)
    splittime.ResidentChainSet(ctx, case.fresh_gens(), [case.d["tv0"]] * case.nch, case.betas,
                               np.ones(case.nl), case.samps, case.us)
    keep_t = [ctx.get_times(ci, li, len(base[ci][li].pop)) for ci in range(case.nch) for li in range(case.nl)]
    keep_pg, keep_tv = ctx.get_probg(), ctx.get_split_times().copy()
    with pytest.raises(api.ImaError) as ei:
        ctx.checkpoint_read(badp)
    assert ei.value.code == api.IMA_ERR_DATA
    assert np.array_equal(ctx.get_probg(), keep_pg)
    assert np.array_equal(ctx.get_split_times(), keep_tv)
    k = 0
    for ci in range(case.nch):
        for li in range(case.nl):
            t, m = ctx.get_times(ci, li, len(base[ci][li].pop))
            assert np.array_equal(t, keep_t[k][0]) and np.array_equal(m, keep_t[k][1])
            k += 1
    ctx.close()


def test_chain_weights_on_a_subset_of_chains():
    """ima_gpu_chain_weights on chains given in any order and any subset:
    each chain's p(G) and integrals equal the all-chain call's."""
    case = RyCase()
    ctx = _resident_context(case)
    splittime.ResidentChainSet(ctx, case.fresh_gens(), [case.d["tv0"]] * case.nch, case.betas,
                               np.ones(case.nl), case.samps, case.us)
    tv = np.array([case.d["tv0"]] * case.nch, np.float64).reshape(case.nch, -1)
    allc = np.arange(case.nch, dtype=np.int32)
    p_all, q_all, m_all = ctx.chain_weights(allc, tv)
    for sub in ([case.nch - 1], [2, 0], [1]):
        sub = np.array(sub, np.int32)
        p, q, m = ctx.chain_weights(sub, tv[sub])
        assert np.array_equal(p, p_all[sub])
        assert np.array_equal(q, q_all[sub])
        assert np.array_equal(m, m_all[sub])
    # after the subset call only chain 1's genealogies hold weights: p(G) of
    # chain 1 again matches, a group over chain 0 is refused
    nl = case.nl
    p1, _, _, _ = ctx.tree_prob(np.array([nl, 2 * nl], np.int32))
    assert np.array_equal(p1, p_all[[1]])
    with pytest.raises(api.ImaError) as ei:
        ctx.tree_prob(np.array([0, nl], np.int32))
    assert ei.value.code == api.IMA_ERR_STATE
    ctx.close()


def test_library_drawn_sweep_of_one_chain():
    """ima_gpu_changet_ry1_sweep_mt on a subset of the chains (chain 1 alone,
    12 updates): each decision, split time, p(G) and likelihood sum equals the
    oracle-driven changet_RY1 of that chain with the same generator, the
    chain's final node and migration times are the oracle's, and the other
    chains' genealogies and split times are untouched."""
    from tests._splittime import OracleBackend
    case = RyCase()
    ctx = _resident_context(case)
    splittime.ResidentChainSet(ctx, case.fresh_gens(), [case.d["tv0"]] * case.nch, case.betas,
                               np.ones(case.nl), case.samps, case.us)
    base = case.fresh_gens()
    before = {(ci, li): ctx.get_times(ci, li, len(base[ci][li].pop)) for ci in range(case.nch) for li in range(case.nl)}
    tv0 = ctx.get_split_times().copy()
    backend = OracleBackend(case)
    g0 = case.fresh_gens()[0]  # sum log k! comes from chain 0's genealogies, evaluated first
    backend.likelihoods(0, g0, backend.weights(0, g0, np.array(case.d["tv0"], np.float64))[0])
    gens = case.fresh_gens()[1]
    tv = np.array(case.d["tv0"], np.float64)
    lens, probg = backend.weights(1, gens, tv)
    pdg = np.asarray(backend.likelihoods(1, gens, lens), np.float64)
    s = 0.0
    for v in pdg:
        s += float(v)
    state = splittime.ChainState(tv, float(case.betas[1]), gens, pdg, s, probg)
    rng_o, rng_g = api.MT19937(case.seed), api.MT19937(case.seed)
    periods = [k for ci, k in case.steps if ci == 1][:12]
    for k in periods:
        acc_o = splittime.changet_ry1(state, 1, k, rng_o, case.tprior, case.nl, case.npops, backend)
        acc, pdgsum, pg, newt = ctx.changet_ry1_sweep_mt(np.array([1], np.int32), np.array([k]), case.tprior, rng_g,
                                                       np.asarray(case.us, np.float64))
        assert bool(acc[0]) == acc_o
        assert ctx.get_split_times()[1, k] == state.tvals[k]
        assert abs(pg[0] - state.probg) <= 1e-10
        assert abs(pdgsum[0] - state.pdgsum) <= 1e-12 * abs(state.pdgsum)
    tv_now = ctx.get_split_times()
    assert np.array_equal(np.delete(tv_now, 1, axis=0), np.delete(tv0, 1, axis=0))
    for ci in range(case.nch):
        for li in range(case.nl):
            t, m = ctx.get_times(ci, li, len(base[ci][li].pop))
            edge = base[ci][li].g.down != -1
            if ci == 1:
                lg = state.gens[li]
                assert np.array_equal(t[edge], lg.g.time[edge])
                assert np.array_equal(m, np.array([e[0] for mm in lg.mig for e in mm]))
            else:
                assert np.array_equal(t, before[(ci, li)][0]) and np.array_equal(m, before[(ci, li)][1])
    ctx.close()


def test_long_runs_match_reference_marginals():
    """Statistical parity of whole runs: the device-resident split-time
    sampler (changet_ry1_sweep_mt: band, weights, p(G), likelihoods and the
    decision on the GPU) run for 4000 updates on chain 0 of the golden case,
    periods alternating, under six seeds of its own, against the compiled
    reference's runs of the same length under six other seeds: the thinned
    split times of each period pass a two-sample Kolmogorov-Smirnov test
    (p > 1e-3), their means agree within four standard errors of the
    difference (from per-seed means), and so do the acceptance rates."""
    stats = pytest.importorskip("scipy.stats")
    d = load("golden_ks.npz")
    steps, thin = int(d["steps"]), int(d["thin"])
    ref = {k: np.concatenate([d["t%d_%d" % (k, s)] for s in d["seeds"]]) for k in range(2)}
    ref_acc = np.array([d["acc_%d" % s].mean() for s in d["seeds"]])
    case = RyCase()
    ours = {0: [], 1: []}
    per_seed = {0: [], 1: []}
    acc_rate = []
    for seed in (201, 202, 203, 204, 205, 206):
        ctx = _resident_context(case)
        splittime.ResidentChainSet(ctx, case.fresh_gens(), [case.d["tv0"]] * case.nch, case.betas,
                                   np.ones(case.nl), case.samps, case.us)
        rng = api.MT19937(seed)
        tv = {0: [], 1: []}
        nacc = 0
        for k in range(steps):
            acc, _, _, _ = ctx.changet_ry1_sweep_mt(np.array([0], np.int32), np.array([k % 2]), case.tprior, rng,
                                                    np.asarray(case.us, np.float64))
            nacc += int(acc[0])
            tv[k % 2].append(float(ctx.get_split_times()[0, k % 2]))
        for p in range(2):
            x = np.array(tv[p])[::thin]
            ours[p].append(x)
            per_seed[p].append(x.mean())
        acc_rate.append(nacc / steps)
        ctx.close()
    for p in range(2):
        a, b = np.concatenate(ours[p]), ref[p]
        assert stats.ks_2samp(a, b).pvalue > 1e-3, (p, a.mean(), b.mean())
        rm = np.array([d["t%d_%d" % (p, s)].mean() for s in d["seeds"]])
        om = np.array(per_seed[p])
        se = np.sqrt(rm.var(ddof=1) / len(rm) + om.var(ddof=1) / len(om))
        assert abs(om.mean() - rm.mean()) <= 4 * se, (p, om.mean(), rm.mean(), se)
    se = np.sqrt(np.var(acc_rate, ddof=1) / 6 + ref_acc.var(ddof=1) / 6)
    assert abs(np.mean(acc_rate) - ref_acc.mean()) <= 4 * se + 1e-3, (np.mean(acc_rate), ref_acc.mean())
