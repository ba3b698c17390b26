"""MC3 swaps on the GPU fed the reference's own MT19937 uniforms: every
decision, the betas after every step and both count matrices are bit-exact
against the golden output of the compiled reference."""
import numpy as np
import pytest

from ima2p_gb300 import api
from oracle import pyoracle as O
from tests._golden import load
from tests._gpu import ctx_with

pytestmark = pytest.mark.gpu


def test_swap_golden_bit_exact():
    d = load("golden_swap.npz")
    for c in range(int(d["ncases"])):
        p = "c%d_" % c
        nch, nl, tries, steps, mode, seed = (int(v) for v in d[p + "params"])
        h1, h2 = (float(v) for v in d[p + "h"])
        ctx = ctx_with([("sw", 2, 1)] * nl, 1, nch)
        ctx.setheat(h1, h2, mode)
        ctx.set_pdg(d[p + "pdg"])
        ctx.set_probg(d[p + "probg"])
        u = O.mt_uniforms(seed, 400000)
        k = 0
        for s in range(steps):
            ok, used = ctx.swapchains(tries, True, uniforms=u[k:k + 4 * tries + 64].reshape(1, -1))
            k += int(used[0])
            assert ok[0] == d[p + "ok"][s]
            assert np.array_equal(ctx.get_betas(), d[p + "betas"][s]), (c, s)
        sc, tc = ctx.get_swapcounts(0)
        assert np.array_equal(sc, d[p + "swapcount"])
        assert np.array_equal(tc, d[p + "tempcount"])
        ctx.close()


def test_swap_independent_runs_match_oracle():
    rng = np.random.default_rng(9)
    nruns, cpr, nl, tries = 8, 128, 4, 12
    ctx = ctx_with([("sw", 2, 1)] * nl, nruns, cpr)
    ctx.setheat(0.95, 0.8, 1)
    pdg = rng.normal(-100, 3, (nruns * cpr, nl))
    probg = rng.normal(-30, 2, nruns * cpr)
    ctx.set_pdg(pdg)
    ctx.set_probg(probg)
    U = np.stack([O.mt_uniforms(100 + r, 4096) for r in range(nruns)])
    ok, used = ctx.swapchains(tries, True, uniforms=U)
    betas = ctx.get_betas()
    for r in range(nruns):
        st, beta, allb = O.setheat(cpr, 0.95, 0.8, 1)
        S = O.chain_sums(pdg[r * cpr:(r + 1) * cpr], probg[r * cpr:(r + 1) * cpr])
        sc = np.zeros((cpr, cpr), np.int32)
        tc = np.zeros((cpr, cpr), np.int32)
        o, u_used, _ = O.swapchains(S, beta, allb, tries, U[r], sc, tc)
        assert used[r] == u_used and ok[r] == o
        assert np.array_equal(betas[r * cpr:(r + 1) * cpr], beta)
        gsc, gtc = ctx.get_swapcounts(r)
        assert np.array_equal(gsc, sc) and np.array_equal(gtc, tc)


def test_swap_philox_stream_is_deterministic():
    def run():
        ctx = ctx_with([("sw", 2, 1)], 2, 32)
        ctx.setheat(0.9, 0.8, 1)
        ctx.set_pdg(np.linspace(-50, -10, 64))
        ctx.set_probg(np.zeros(64))
        for _ in range(20):
            ctx.swapchains(3, True, seed=1234)
        b = ctx.get_betas()
        ctx.close()
        return b
    b1, b2 = run(), run()
    assert np.array_equal(b1, b2)
    assert sorted(b1[:32]) == sorted(O.setheat(32, 0.9, 0.8, 1)[1])  # a permutation of the ladder


def test_swap_callback_draws_like_the_reference():
    """ima_gpu_swapchains_cb with the reference's MT19937 drawn one value at a
    time (the library's copy of the generator, seeded as the harness seeds
    it): every decision, the betas after every step, both count matrices and
    the generator's final state match the compiled reference's golden run --
    no draw more, none fewer."""
    d = load("golden_swap.npz")
    for c in range(int(d["ncases"])):
        p = "c%d_" % c
        nch, nl, tries, steps, mode, seed = (int(v) for v in d[p + "params"])
        h1, h2 = (float(v) for v in d[p + "h"])
        ctx = ctx_with([("sw", 2, 1)] * nl, 1, nch)
        ctx.setheat(h1, h2, mode)
        ctx.set_pdg(d[p + "pdg"])
        ctx.set_probg(d[p + "probg"])
        rng = api.MT19937(seed)
        u = O.mt_uniforms(seed, 400000)
        k = 0
        for s in range(steps):
            ok, used = ctx.swapchains_cb(tries, rng.uniform)
            k += int(used[0])
            assert ok[0] == d[p + "ok"][s]
            assert np.array_equal(ctx.get_betas(), d[p + "betas"][s]), (c, s)
        # the next draw is the stream's k-th value: exactly k were taken
        assert rng.uniform() == u[k]
        sc, tc = ctx.get_swapcounts(0)
        assert np.array_equal(sc, d[p + "swapcount"])
        assert np.array_equal(tc, d[p + "tempcount"])
        ctx.close()
