"""The split-time update changet_RY1 (update_t_RY.cpp:223-518, Rannala and
Yang's rubber band) as a host driver over the C ABI.

The host keeps the proposal and the Metropolis-Hastings decision, as the
reference's host program does; the weights of every locus, p(G) and the data
likelihoods of the proposed state -- the work that makes the update costly --
go to the device in three calls (ima_gpu_treeweight, ima_gpu_tree_prob,
ima_gpu_eval).  The arithmetic that decides where each time moves and whether
the proposal is taken is the reference's, operation for operation:

* getnewt (update_gtree_common.cpp:2501-2519): one uniform, a window of
  (t_d_prior - t_u_prior) / (log(nloci + 1) (npops - period)), reflected at
  the prior bounds;
* beforesplit / aftersplit (update_t_RY.cpp:59-86): the linear maps of every
  node and migration time in (t_u, oldt] and (oldt, t_d), counted for the
  Hastings term (node times twice, once per daughter edge);
* the Metropolis-Hastings term (:394-406) and log(U) < min(1, term) (:408);
* on rejection, the inverse maps (:444-491): times go back through the same
  formulas with oldt and newt exchanged, not from a saved copy.

Given the same generator state, the same inputs and likelihoods that agree
with the reference's to rounding, the chain takes the reference's decisions
step for step.  The backend supplies the device (or any other) computation:
``weights(ci, gens, tvals) -> (lens, probg)`` and ``likelihoods(ci, gens,
lens) -> pdg per locus``.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import api

TIMEMAX = 1000000.0  # imamp.hpp:129


def beforesplit(tnode, oldt, newt, tau_u, ptime):
    """update_t_RY.cpp:72-86 (elementwise on arrays)."""
    if tnode == 0:
        return ptime * newt / oldt
    return tau_u + (ptime - tau_u) * (newt - tau_u) / (oldt - tau_u)


def aftersplit(tnode, lastperiod, oldt, newt, tau_d, ptime):
    """update_t_RY.cpp:59-70 (elementwise on arrays)."""
    if tnode == lastperiod - 1:
        return ptime + newt - oldt
    return tau_d - (tau_d - newt) * (tau_d - ptime) / (tau_d - oldt)


def getnewt(rng, period, t_u_prior, t_d_prior, oldt, nloci, npops):
    """update_gtree_common.cpp:2501-2519."""
    twin = (t_d_prior - t_u_prior) / (math.log(float(nloci) + 1) * (npops - period))
    U = rng.uniform()
    newt = (oldt - twin / 2) + U * twin
    if newt >= t_d_prior:
        newt = 2.0 * t_d_prior - newt
    elif newt <= t_u_prior:
        newt = 2.0 * t_u_prior - newt
    return newt


@dataclasses.dataclass
class ChainState:
    """One chain's state as changet_RY1 reads it: split times, heat, the
    labelled genealogies of every locus, per-locus likelihoods, their sum
    and p(G)."""
    tvals: np.ndarray
    beta: float
    gens: list
    pdg: np.ndarray
    pdgsum: float
    probg: float


def _move(gens, period, last, oldt, newt, t_u, t_d, count):
    """Apply the rubber band to every non-root edge time and migration time
    of the chain's genealogies; returns (ecd, ecu, emd, emu) when counting."""
    ecd = ecu = emd = emu = 0
    for lg in gens:
        t = lg.g.time
        edge = lg.g.down != -1
        lo = edge & (t <= oldt) & (t > t_u)
        hi = edge & ~lo & (t > oldt) & (t < t_d)
        t[lo] = beforesplit(period, oldt, newt, t_u, t[lo])
        t[hi] = aftersplit(period, last, oldt, newt, t_d, t[hi])
        ecu += int(lo.sum())
        ecd += int(hi.sum())
        for i, m in enumerate(lg.mig):
            if not m or not edge[i]:
                continue
            for j, (mt, mp) in enumerate(m):
                if t_u < mt <= oldt:
                    m[j] = (float(beforesplit(period, oldt, newt, t_u, mt)), mp)
                    emu += 1
                elif oldt < mt < t_d:
                    m[j] = (float(aftersplit(period, last, oldt, newt, t_d, mt)), mp)
                    emd += 1
    return (ecd, ecu, emd, emu) if count else None


def changet_ry1(state: ChainState, ci, period, rng, tprior, nloci, npops, backend, gbeta=1.0):
    """One split-time update of chain ci's period (changet_RY1); returns True
    when the proposal is accepted.  tprior[k] = (T[k].pr.min, T[k].pr.max)."""
    last = npops - 1
    tv = state.tvals
    t_u = 0.0 if period == 0 else float(tv[period - 1])
    t_d = TIMEMAX if period == last - 1 else float(tv[period + 1])
    t_d_prior = min(tprior[period][1], t_d)
    t_u_prior = max(tprior[period][0], t_u)
    oldt = float(tv[period])
    newt = getnewt(rng, period, t_u_prior, t_d_prior, oldt, nloci, npops)
    t_u_hterm = (newt - t_u) / (oldt - t_u)
    t_d_hterm = 1.0 if period == last - 1 else (t_d - newt) / (t_d - oldt)
    ecd, ecu, emd, emu = _move(state.gens, period, last, oldt, newt, t_u, t_d, True)
    tv[period] = newt
    lens, probg_new = backend.weights(ci, state.gens, tv)
    pdg_new = np.asarray(backend.likelihoods(ci, state.gens, lens), np.float64)
    pdgnewsum = 0.0
    for v in pdg_new:
        pdgnewsum += float(v)
    ecd //= 2
    ecu //= 2
    tpw = gbeta * (pdgnewsum - state.pdgsum)
    tpw += probg_new - state.probg
    mh = state.beta * tpw + (ecd + emd) * math.log(t_d_hterm) + (ecu + emu) * math.log(t_u_hterm)
    U = math.log(rng.uniform())
    if U < min(1.0, mh):
        state.pdg = pdg_new
        state.pdgsum = pdgnewsum
        state.probg = probg_new
        return True
    tv[period] = oldt
    _move(state.gens, period, last, newt, oldt, t_u, t_d, False)
    return False


class DeviceBackend:
    """Weights, p(G) and infinite-sites likelihoods on the device for
    changet_ry1: ctx must hold the loci (added in locus order), one chain
    per ChainState and the population model (ima_gpu_set_popmodel)."""

    def __init__(self, ctx: api.Context, loci_hval, loci_samppop, u, precision=api.PREC_FP64):
        self.ctx = ctx
        self.hval = np.asarray(loci_hval, np.float64)
        self.samp = np.asarray(loci_samppop, np.int32)
        self.u = np.asarray(u, np.float64)
        self.prec = precision

    def weights(self, ci, gens, tvals):
        nl = len(gens)
        w = self.ctx.treeweight(api.pack_labelled(gens), np.arange(nl, dtype=np.int32), np.zeros(nl, np.int32),
                                self.hval, self.samp, np.asarray(tvals, np.float64)[None, :])
        probg, _, _, _ = self.ctx.tree_prob(np.array([0, nl], np.int32))
        return w["lens"], float(probg[0])

    def likelihoods(self, ci, gens, lens):
        nl = len(gens)
        for li, lg in enumerate(gens):
            self.ctx.set_genealogy(ci, li, lg.g, length=float(lens[li, 0]))
        r, st = self.ctx.eval(np.full(nl, ci, np.int32), np.arange(nl, dtype=np.int32), self.u,
                              np.ones(nl), precision=self.prec)
        return r


class ChainSet:
    """Every chain's state packed for a batched sweep: the labelled
    genealogies of chains 0..nch-1 x loci 0..nl-1 (chain-major) as one CSR
    (api.pack_labelled order), split times [nch][npops-1], heats, per-locus
    likelihoods [nch][nl] and their sums, p(G) per chain."""

    def __init__(self, gens, tvals, betas):
        self.nch, self.nl = len(gens), len(gens[0])
        flat = [lg for row in gens for lg in row]
        (self.node_off, self.up0, self.time, self.pop, self.mig_off, self.mig_t,
         self.mig_p) = api.pack_labelled(flat)
        self.up1 = np.concatenate([lg.g.up1 for lg in flat]).astype(np.int32)
        self.down = np.concatenate([lg.g.down for lg in flat]).astype(np.int32)
        self.tvals = np.array(tvals, np.float64).reshape(self.nch, -1).copy()
        self.beta = np.asarray(betas, np.float64).copy()
        nn = np.diff(self.node_off)
        self.node_chain = np.repeat(np.arange(self.nch * self.nl) // self.nl, nn)
        self.edge = self.down != -1
        counts = np.diff(self.mig_off)
        self.mig_chain = np.repeat(self.node_chain, counts)
        self.pdg = np.zeros((self.nch, self.nl))
        self.pdgsum = np.zeros(self.nch)
        self.probg = np.zeros(self.nch)

    def packed(self):
        return self.node_off, self.up0, self.time, self.pop, self.mig_off, self.mig_t, self.mig_p


def _band(period, last, oldt, newt, t_u, t_d, t, sel_lo, sel_hi):
    """beforesplit on sel_lo, aftersplit on sel_hi; oldt..t_d per element."""
    out = t.copy()
    first = sel_lo & (period == 0)
    rest = sel_lo & (period != 0)
    out[first] = t[first] * newt[first] / oldt[first]
    out[rest] = t_u[rest] + (t[rest] - t_u[rest]) * (newt[rest] - t_u[rest]) / (oldt[rest] - t_u[rest])
    top = sel_hi & (period == last - 1)
    mid = sel_hi & (period != last - 1)
    out[top] = t[top] + newt[top] - oldt[top]
    out[mid] = t_d[mid] - (t_d[mid] - newt[mid]) * (t_d[mid] - t[mid]) / (t_d[mid] - oldt[mid])
    return out


class SweepBackend:
    """Device work of a batched sweep: weights and p(G) of every chain in one
    ima_gpu_treeweight + ima_gpu_tree_prob, likelihoods of every chain-locus
    in one ima_gpu_set_genealogies + ima_gpu_eval.  ctx holds the loci, nch
    chains in one run (ima_gpu_set_chains(1, nch)) and the population
    model."""

    def __init__(self, ctx, loci_hval, loci_samppop, u, kappa=None, precision=api.PREC_FP64):
        self.ctx = ctx
        self.hval = np.asarray(loci_hval, np.float64)
        self.samp = np.asarray(loci_samppop, np.int32)
        self.u = np.asarray(u, np.float64)
        self.kappa = np.ones(len(self.u)) if kappa is None else np.asarray(kappa, np.float64)
        self.prec = precision

    def weights(self, cs: ChainSet):
        n = cs.nch * cs.nl
        gl = np.tile(np.arange(cs.nl, dtype=np.int32), cs.nch)
        gt = np.repeat(np.arange(cs.nch, dtype=np.int32), cs.nl)
        w = self.ctx.treeweight(cs.packed(), gl, gt, self.hval, self.samp, cs.tvals)
        probg, _, _, _ = self.ctx.tree_prob((np.arange(cs.nch + 1) * cs.nl).astype(np.int32))
        return w["lens"], probg

    def likelihoods(self, cs: ChainSet, lens):
        n = cs.nch * cs.nl
        ci = np.repeat(np.arange(cs.nch, dtype=np.int32), cs.nl)
        li = np.tile(np.arange(cs.nl, dtype=np.int32), cs.nch)
        self.ctx.set_genealogies(ci, li, cs.up0, cs.up1, cs.down, cs.time, length=lens[:, 0].copy())
        r, _ = self.ctx.eval(ci, li, np.tile(self.u, cs.nch), np.tile(self.kappa, cs.nch), precision=self.prec)
        return r.reshape(cs.nch, cs.nl)

    def decide(self, cs: ChainSet, accept):
        """Commit the accepted chains' evaluations, revert the others'."""
        ci = np.repeat(np.arange(cs.nch, dtype=np.int32), cs.nl)
        li = np.tile(np.arange(cs.nl, dtype=np.int32), cs.nch)
        self.ctx.commit(ci, li, np.repeat(np.asarray(accept, np.uint8), cs.nl))


def setup_chainset(cs: ChainSet, backend):
    """The state finish_setup_C leaves: weights, p(G), likelihoods and
    their per-chain sums in locus order."""
    lens, probg = backend.weights(cs)
    pdg = np.asarray(backend.likelihoods(cs, lens), np.float64)
    backend.decide(cs, np.ones(cs.nch, bool))
    cs.pdg = pdg
    s = np.zeros(cs.nch)
    for li in range(cs.nl):
        s = s + pdg[:, li]
    cs.pdgsum = s
    cs.probg = np.asarray(probg, np.float64)


def changet_ry1_sweep(cs: ChainSet, periods, rng, tprior, npops, backend, gbeta=1.0):
    """One changet_RY1 per chain, chains in order, with the device work of
    all chains batched.  The generator draws are the sequential run's (for
    chain 0: getnewt's uniform, then the acceptance uniform; then chain 1,
    ...), since no draw depends on another chain.  Returns the accept flags."""
    nch, last = cs.nch, npops - 1
    periods = np.asarray(periods, np.int64)
    oldt = cs.tvals[np.arange(nch), periods].copy()
    t_u = np.where(periods == 0, 0.0, cs.tvals[np.arange(nch), np.maximum(periods - 1, 0)])
    t_d = np.where(periods == last - 1, TIMEMAX, cs.tvals[np.arange(nch), np.minimum(periods + 1, last - 1)])
    newt = np.zeros(nch)
    logU = np.zeros(nch)
    for c in range(nch):
        k = int(periods[c])
        t_d_prior = min(tprior[k][1], float(t_d[c]))
        t_u_prior = max(tprior[k][0], float(t_u[c]))
        newt[c] = getnewt(rng, k, t_u_prior, t_d_prior, float(oldt[c]), cs.nl, npops)
        logU[c] = math.log(rng.uniform())
    # the rubber band on every node and migration time, per chain's parameters
    nc, mc = cs.node_chain, cs.mig_chain

    def move(o, n, t, chain, edge):
        P, tu, td, ot, nt = periods[chain], t_u[chain], t_d[chain], o[chain], n[chain]
        lo = edge & (t <= ot) & (t > tu)
        hi = edge & ~lo & (t > ot) & (t < td)
        return _band(P, last, ot, nt, tu, td, t, lo, hi), lo, hi

    old_time, old_mig = cs.time.copy(), cs.mig_t.copy()
    cs.time, lo, hi = move(oldt, newt, cs.time, nc, cs.edge)
    ecu = np.bincount(nc[lo], minlength=nch) // 2
    ecd = np.bincount(nc[hi], minlength=nch) // 2
    medge = np.repeat(cs.edge, np.diff(cs.mig_off))
    cs.mig_t, mlo, mhi = move(oldt, newt, cs.mig_t, mc, medge)
    emu = np.bincount(mc[mlo], minlength=nch)
    emd = np.bincount(mc[mhi], minlength=nch)
    cs.tvals[np.arange(nch), periods] = newt
    lens, probg_new = backend.weights(cs)
    pdg_new = np.asarray(backend.likelihoods(cs, lens), np.float64)
    pdgnewsum = np.zeros(nch)
    for li in range(cs.nl):
        pdgnewsum = pdgnewsum + pdg_new[:, li]
    accept = np.zeros(nch, bool)
    for c in range(nch):
        t_u_hterm = (newt[c] - t_u[c]) / (oldt[c] - t_u[c])
        t_d_hterm = 1.0 if periods[c] == last - 1 else (t_d[c] - newt[c]) / (t_d[c] - oldt[c])
        tpw = gbeta * (float(pdgnewsum[c]) - float(cs.pdgsum[c]))
        tpw += float(probg_new[c]) - float(cs.probg[c])
        mh = (float(cs.beta[c]) * tpw + int(ecd[c] + emd[c]) * math.log(t_d_hterm)
              + int(ecu[c] + emu[c]) * math.log(t_u_hterm))
        accept[c] = logU[c] < min(1.0, mh)
    backend.decide(cs, accept)
    cs.pdg[accept] = pdg_new[accept]
    cs.pdgsum[accept] = pdgnewsum[accept]
    cs.probg[accept] = np.asarray(probg_new, np.float64)[accept]
    rej = ~accept
    if rej.any():
        # rejected chains: the inverse maps, as the reference moves them back
        cs.tvals[np.arange(nch)[rej], periods[rej]] = oldt[rej]
        back_t, _, _ = move(newt, oldt, cs.time, nc, cs.edge & rej[nc])
        back_m, _, _ = move(newt, oldt, cs.mig_t, mc, medge & rej[mc])
        cs.time = np.where(rej[nc], back_t, cs.time)
        cs.mig_t = np.where(rej[mc], back_m, cs.mig_t)
    return accept


class ResidentChainSet:
    """Every chain's state resident in a context for device sweeps: the
    genealogies and their population labels stay on the GPU and the rubber
    band moves their times there (ima_gpu_rubber_band); weights, p(G) and
    likelihoods are computed in place (ima_gpu_chain_weights, ima_gpu_eval);
    only the generator draws, the per-chain counts and sums and the
    decisions pass through the host.  ctx: the loci added, ima_gpu_set_chains
    (1, nch) and the population model set."""

    def __init__(self, ctx, gens, tvals, betas, hval, samppop, u, kappa=None, precision=api.PREC_FP64):
        self.ctx = ctx
        self.nch, self.nl = len(gens), len(gens[0])
        self.tvals = np.array(tvals, np.float64).reshape(self.nch, -1).copy()
        self.beta = np.asarray(betas, np.float64).copy()
        self.u = np.asarray(u, np.float64)
        self.kappa = np.ones(self.nl) if kappa is None else np.asarray(kappa, np.float64)
        self.prec = precision
        self.ci = np.repeat(np.arange(self.nch, dtype=np.int32), self.nl)
        self.li = np.tile(np.arange(self.nl, dtype=np.int32), self.nch)
        flat = [lg for row in gens for lg in row]
        ctx.set_genealogies(self.ci, self.li, np.concatenate([g.g.up0 for g in flat]),
                            np.concatenate([g.g.up1 for g in flat]), np.concatenate([g.g.down for g in flat]),
                            np.concatenate([g.g.time for g in flat]), length=np.full(len(flat), -1.0))
        ctx.set_labels(self.ci, self.li, flat)
        ctx.set_locus_pops(hval, samppop)
        self.chains = np.arange(self.nch, dtype=np.int32)
        self.probg, _, _ = ctx.chain_weights(self.chains, self.tvals)
        self.pdg = self._eval()
        ctx.commit(self.ci, self.li, np.ones(len(self.ci), np.uint8))
        self.pdgsum = self._sums(self.pdg)
        ctx.set_betas(self.beta)     # resident heats and p(G) for the device decisions
        ctx.set_probg(self.probg)

    @classmethod
    def resume(cls, ctx, path, u, kappa=None, precision=api.PREC_FP64, rng=None):
        """The chain set a checkpoint_write file holds, restored into ctx (the
        loci added, ima_gpu_set_chains and the population model set as when
        it was written); rng (may be None) takes the saved generator state.
        Split times, heats and p(G) come from the context; one full
        evaluation rebuilds the partial likelihoods the file does not hold
        and gives back the saved G.pdg."""
        self = cls.__new__(cls)
        ctx.checkpoint_read(path, rng)
        self.ctx = ctx
        self.nch, self.nl = ctx.nchains, len(ctx.loci)
        self.u = np.asarray(u, np.float64)
        self.kappa = np.ones(self.nl) if kappa is None else np.asarray(kappa, np.float64)
        self.prec = precision
        self.ci = np.repeat(np.arange(self.nch, dtype=np.int32), self.nl)
        self.li = np.tile(np.arange(self.nl, dtype=np.int32), self.nch)
        self.chains = np.arange(self.nch, dtype=np.int32)
        self.tvals = ctx.get_split_times()
        self.beta = ctx.get_betas()
        self.probg = ctx.get_probg()
        self.pdg = self._eval()
        ctx.commit(self.ci, self.li, np.ones(len(self.ci), np.uint8))
        self.pdgsum = self._sums(self.pdg)
        return self

    def _eval(self):
        r, _ = self.ctx.eval(self.ci, self.li, np.tile(self.u, self.nch), np.tile(self.kappa, self.nch),
                             precision=self.prec)
        return r.reshape(self.nch, self.nl)

    def _sums(self, pdg):
        s = np.zeros(self.nch)
        for li in range(self.nl):
            s = s + pdg[:, li]
        return s

    def sweep(self, periods, rng, tprior, npops, gbeta=1.0):
        """One changet_RY1 per chain, chains in order (draws as in the
        sequential run); returns the accept flags."""
        nch, last = self.nch, npops - 1
        periods = np.asarray(periods, np.int64)
        rows = np.arange(nch)
        oldt = self.tvals[rows, periods].copy()
        t_u = np.where(periods == 0, 0.0, self.tvals[rows, np.maximum(periods - 1, 0)])
        t_d = np.where(periods == last - 1, TIMEMAX, self.tvals[rows, np.minimum(periods + 1, last - 1)])
        newt, logU = np.zeros(nch), np.zeros(nch)
        for c in range(nch):
            k = int(periods[c])
            newt[c] = getnewt(rng, k, max(tprior[k][0], float(t_u[c])), min(tprior[k][1], float(t_d[c])),
                              float(oldt[c]), self.nl, npops)
            logU[c] = math.log(rng.uniform())
        counts = self.ctx.rubber_band(self.chains, periods, oldt, newt, t_u, t_d)
        tv_new = self.tvals.copy()
        tv_new[rows, periods] = newt
        probg_new, _, _ = self.ctx.chain_weights(self.chains, tv_new)
        pdg_new = self._eval()
        pdgnewsum = self._sums(pdg_new)
        accept = np.zeros(nch, bool)
        for c in range(nch):
            ecd, ecu, emd, emu = (int(v) for v in counts[c])
            ecd //= 2
            ecu //= 2
            t_u_hterm = (newt[c] - t_u[c]) / (oldt[c] - t_u[c])
            t_d_hterm = 1.0 if periods[c] == last - 1 else (t_d[c] - newt[c]) / (t_d[c] - oldt[c])
            tpw = gbeta * (float(pdgnewsum[c]) - float(self.pdgsum[c]))
            tpw += float(probg_new[c]) - float(self.probg[c])
            mh = float(self.beta[c]) * tpw + (ecd + emd) * math.log(t_d_hterm) + (ecu + emu) * math.log(t_u_hterm)
            accept[c] = logU[c] < min(1.0, mh)
        self.ctx.commit(self.ci, self.li, np.repeat(accept.astype(np.uint8), self.nl))
        self.pdg[accept] = pdg_new[accept]
        self.pdgsum[accept] = pdgnewsum[accept]
        self.probg[accept] = probg_new[accept]
        self.tvals[rows[accept], periods[accept]] = newt[accept]
        rej = np.flatnonzero(~accept)
        if len(rej):
            self.ctx.rubber_band(self.chains[rej], periods[rej], oldt[rej], newt[rej], t_u[rej], t_d[rej],
                                 inverse=True)
        return accept

    def sweep_device_mt(self, periods, rng, tprior, gbeta=1.0):
        """sweep_device with the draws in the library
        (ima_gpu_changet_ry1_sweep_mt): rng is the api.MT19937 the
        reference's uniform() would draw from."""
        nch = self.nch
        periods = np.asarray(periods, np.int64)
        acc, pdgsum, probg, newt = self.ctx.changet_ry1_sweep_mt(
            self.chains, periods, tprior, rng, np.tile(self.u, nch), np.tile(self.kappa, nch), gbeta, self.prec)
        rows = np.arange(nch)
        self.tvals[rows[acc], periods[acc]] = newt[acc]
        self.pdgsum = pdgsum
        self.probg = probg
        return acc

    def sweep_device(self, periods, rng, tprior, npops, gbeta=1.0):
        """sweep() with the decisions on the device (ima_gpu_changet_ry1_sweep):
        one call per sweep; the host draws and takes the two logs of the
        Hastings ratios, as the reference computes them."""
        nch, last = self.nch, npops - 1
        periods = np.asarray(periods, np.int64)
        rows = np.arange(nch)
        oldt = self.tvals[rows, periods].copy()
        t_u = np.where(periods == 0, 0.0, self.tvals[rows, np.maximum(periods - 1, 0)])
        t_d = np.where(periods == last - 1, TIMEMAX, self.tvals[rows, np.minimum(periods + 1, last - 1)])
        newt, logU, lhu, lhd = np.zeros(nch), np.zeros(nch), np.zeros(nch), np.zeros(nch)
        for c in range(nch):
            k = int(periods[c])
            newt[c] = getnewt(rng, k, max(tprior[k][0], float(t_u[c])), min(tprior[k][1], float(t_d[c])),
                              float(oldt[c]), self.nl, npops)
            logU[c] = math.log(rng.uniform())
            lhu[c] = math.log((newt[c] - t_u[c]) / (oldt[c] - t_u[c]))
            lhd[c] = 0.0 if k == last - 1 else math.log((t_d[c] - newt[c]) / (t_d[c] - oldt[c]))
        tv_new = self.tvals.copy()
        tv_new[rows, periods] = newt
        acc, pdgsum, probg = self.ctx.changet_ry1_sweep(
            self.chains, periods, oldt, newt, t_u, t_d, lhu, lhd, logU, tv_new,
            np.tile(self.u, nch), np.tile(self.kappa, nch), gbeta, self.prec)
        self.tvals[rows[acc], periods[acc]] = newt[acc]
        self.pdgsum = pdgsum
        self.probg = probg
        return acc
