"""The split-time update driver (ima2p_gb300.splittime.changet_ry1) on the
oracle against golden_ry.npz, made by the unmodified reference's
changet_RY1 (update_t_RY.cpp:223-518) with the same MT19937 seed: the same
decision at every step, the same split times and node and migration times
bit for bit, probg and pdg to rounding.  CPU only."""
import numpy as np
import pytest

from ima2p_gb300 import api
from tests._splittime import OracleBackend, RyCase, final_times, run_chain_set

pytestmark = pytest.mark.skipif(not __import__("os").path.exists(api.LIB_PATH),
                                reason="library not built here (MT19937 lives in it)")


def test_oracle_driven_update_follows_the_reference():
    case = RyCase()
    res, states = run_chain_set(case, OracleBackend(case), api.MT19937(case.seed))
    ref = case.res
    assert np.array_equal(res[:, 0], ref[:, 0])          # decisions
    assert np.array_equal(res[:, 1], ref[:, 1])          # split times, bit for bit
    np.testing.assert_allclose(res[:, 2], ref[:, 2], rtol=0, atol=1e-10)   # probg
    np.testing.assert_allclose(res[:, 3], ref[:, 3], rtol=1e-12)           # pdg sums
    t, m = final_times(case, states)
    root = np.concatenate([lg.g.down == -1 for st in states for lg in st.gens])
    assert np.array_equal(t[~root], case.times[~root])   # every edge time, bit for bit
    assert np.array_equal(m, case.migt)


def test_batched_sweep_on_the_oracle_follows_the_reference():
    """changet_ry1_sweep (every chain's proposal in one batch) on the oracle:
    the reference's sequential run, decision for decision."""
    from tests._splittime import OracleSweepBackend, run_sweeps
    case = RyCase()
    res, cs = run_sweeps(case, OracleSweepBackend(case), api.MT19937(case.seed))
    ref = case.res
    assert np.array_equal(res[:, 0], ref[:, 0])
    assert np.array_equal(res[:, 1], ref[:, 1])
    np.testing.assert_allclose(res[:, 2], ref[:, 2], rtol=0, atol=1e-10)
    np.testing.assert_allclose(res[:, 3], ref[:, 3], rtol=1e-12)
    assert np.array_equal(cs.time[cs.edge], case.times[cs.edge])
    assert np.array_equal(cs.mig_t, case.migt)
