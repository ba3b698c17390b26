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
