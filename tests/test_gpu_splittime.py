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
