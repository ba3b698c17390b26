"""The oracle's batched C entry points (ora_*_batch, the CPU baselines'
timed path) give exactly the single-item restatement's numbers, on one and
on several host threads."""
import numpy as np
import pytest

from ima2p_gb300 import synth
from oracle import pyoracle as O


def _items(kind, rng, k=24):
    out = []
    if kind == "sw":
        for _ in range(k):
            g = synth.three_pop_tree(rng, [5, 6, 4])
            out.append(("sw", g, float(rng.lognormal(0, 0.5)), 1.0, synth.sw_alleles(rng, g, 1.0)))
    elif kind == "hky":
        locs = []
        for _ in range(3):
            g = synth.two_pop_tree(rng, 6, 7, theta=10.0, mig=0.2, tsplit=1.5)
            locs.append((synth.hky_data(rng, g, 300, 1.0, 4.0, rng.dirichlet([5] * 4)), g))
        for j in range(k):
            loc, g = locs[j % 3]
            out.append(("hky", synth.jitter_times(rng, g, 0.2), float(rng.lognormal(0, 0.5)),
                        float(rng.uniform(2, 8)), loc))
    else:
        g = synth.two_pop_tree(rng, 8, 8)
        seq = synth.is_data(rng, g, 1.0, min_sites=4)
        for _ in range(k):
            out.append(("is", synth.jitter_times(rng, g, 0.2), float(rng.lognormal(0, 0.5)), 1.0, seq))
    return out


def _single(it):
    kind, g, u, par, data = it
    if kind == "sw":
        return O.sw_likelihood(data, g, u, par)[0]
    if kind == "hky":
        return O.HKYState(*data.seq.shape).likelihood(data, g, u, par)
    return O.is_likelihood(data, g, g.length(), u, 0.0)[0]


@pytest.mark.parametrize("kind", ["sw", "hky", "is"])
@pytest.mark.parametrize("threads", [1, 4])
def test_batch_equals_single_items(kind, threads):
    items = _items(kind, np.random.default_rng(3))
    want = np.array([_single(it) for it in items])
    got = O.PackedItems(items).run(threads)
    assert np.array_equal(got, want)
