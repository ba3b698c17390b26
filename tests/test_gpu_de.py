"""The L-mode peak search on the GPU (ima_gpu_modelloop): every generation's
trial vectors are one batched surface evaluation.  With the reference's own
jointp (IMA_SURF_COMPAT) the search must follow the reference's modelloop
(golden_de.npz, made by the unmodified reference) and consume the same
MT19937 draws as the oracle; with the exact tensor-core surface it must find
the peak of the exact log-sum-exp that the oracle's search finds."""
import numpy as np
import pytest

from ima2p_gb300 import api
from oracle import pyoracle as O
from tests._golden import load
from tests._gpu import ctx_with

pytestmark = pytest.mark.gpu

DE_CASES = ["full", "theta", "mig", "nested"]


def _active(mt, nested):
    if nested:
        return list(range(6))
    lo, hi = {0: (0, 5), 1: (0, 3), 2: (3, 5)}[mt]
    return list(range(lo, hi)) + [5]


def _case(d, case):
    npops, mt, seed, nested = (int(v) for v in d[case + "_case"])
    return npops, mt, seed, nested, (d[case + "_xmap"] if nested else None)


@pytest.mark.parametrize("case", DE_CASES)
def test_peak_search_follows_reference(case):
    d = load("golden_de.npz")
    npops, mt, seed, nested, xmap = _case(d, case)
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(d["rows"], 3, 2, npops)
    best, ess, gens, runs, rng = ctx.modelloop(d["upper"], mt, seed=seed, multiplier=int(d["multiplier"]),
                                               xmap=xmap, nested=nested, method=api.SURF_COMPAT)
    ref = d[case + "_best"]
    idx = _active(mt, nested)
    # the compat surface agrees with the reference's jointp to ~1e-12, so every
    # selection goes the same way and the peak is the reference's
    np.testing.assert_allclose(best[idx], ref[idx], rtol=1e-9)
    assert abs(ess - float(d[case + "_ess"])) <= 1e-9 * float(d[case + "_ess"])
    # the same number of generations and restarts, and the same draws consumed
    ob, oe, og, orr, orng = O.modelloop(d["rows"], 3, 2, npops, d["upper"], mt, int(d["multiplier"]), seed,
                                        xmap=xmap, nested=nested, compat=True)
    assert (gens, runs) == (og, orr)
    assert list(rng.mt) == list(orng.mt) and rng.mti == orng.mti


def test_peak_search_exact_surface():
    """The exact surface (tensor-core screen): the peak of log-sum-exp over all
    genealogies, as the oracle's search with the exact FP64 objective finds it
    (trajectories may part where two values agree to 1e-10, so the peak is
    compared, not the path)."""
    d = load("golden_de.npz")
    npops, mt, seed, nested, xmap = _case(d, "full")
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(d["rows"], 3, 2, npops)
    best, ess, gens, runs, _ = ctx.modelloop(d["upper"], mt, seed=seed, multiplier=int(d["multiplier"]),
                                             method=api.SURF_TC)
    ob, oe, og, orr, _ = O.modelloop(d["rows"], 3, 2, npops, d["upper"], mt, int(d["multiplier"]), seed,
                                     compat=False)
    assert abs(best[5] - ob[5]) <= 1e-6
    np.testing.assert_allclose(best[:5], ob[:5], rtol=2e-2)
    assert abs(ess - oe) <= 1e-3 * oe


def test_rng_state_continues():
    """Two searches in a row draw from one stream: the second starts where the
    first stopped, as the reference's global generator does."""
    d = load("golden_de.npz")
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(d["rows"], 3, 2, 3)
    rng = api.MT19937(5)
    b1 = ctx.modelloop(d["upper"], 1, rng=rng, multiplier=10, method=api.SURF_COMPAT)[0]
    b2 = ctx.modelloop(d["upper"], 2, rng=rng, multiplier=10, method=api.SURF_COMPAT)[0]
    orng = O.MT(5)
    o1 = O.modelloop(d["rows"], 3, 2, 3, d["upper"], 1, 10, rng=orng)[0]
    o2 = O.modelloop(d["rows"], 3, 2, 3, d["upper"], 2, 10, rng=orng)[0]
    np.testing.assert_allclose(b1[[0, 1, 2, 5]], o1[[0, 1, 2, 5]], rtol=1e-9)
    np.testing.assert_allclose(b2[[3, 4, 5]], o2[[3, 4, 5]], rtol=1e-9)


def test_bad_arguments():
    d = load("golden_de.npz")
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(d["rows"], 3, 2, 3)
    with pytest.raises(api.ImaError):  # nested migration-only models are not accepted
        ctx.modelloop(d["upper"], 2, xmap=np.array([0.0, 0, 0, 0, 1]), nested=2)
    with pytest.raises(api.ImaError):  # a nested index beyond the nested model
        ctx.modelloop(d["upper"], 0, xmap=np.array([0.0, 1, 2, 3, 4]), nested=3)


def test_lmode_pipeline_from_ti_file(tmp_path):
    """.ti file -> resident surface -> peak search -> marginal densities, the
    whole L-mode path, against the oracle on the rows the reference's reader
    would load."""
    from tests.test_ti_io import parsed, write_ti
    d = load("golden_de.npz")
    path = str(tmp_path / "run.ti")
    write_ti(path, d["rows"])
    rows, total = api.ti_read([path], d["rows"].shape[1])
    assert total == len(d["rows"]) and np.array_equal(rows, parsed(d["rows"]))
    ctx = ctx_with([("sw", 2, 1)])
    ctx.surface_load(rows, 3, 2, 2)
    best, ess, gens, runs, _ = ctx.modelloop(d["upper"], 0, seed=77, multiplier=30, method=api.SURF_COMPAT)
    ob, oe, og, orr, _ = O.modelloop(rows, 3, 2, 2, d["upper"], 0, 30, 77, compat=True)
    np.testing.assert_allclose(best, ob, rtol=1e-9)
    xs, ys = ctx.fillvec(np.zeros(5), d["upper"], 200)
    for p in range(5):
        for j in (0, 77, 199):
            want = O.margincalc(rows, 3, 2, p, xs[p, j])
            assert abs(ys[p, j] - want) <= 1e-12 * abs(want)
