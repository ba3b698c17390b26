"""Shared pieces of the split-time update tests: the golden_ry.npz case as
chain states, and a backend for ima2p_gb300.splittime on the oracle."""
import copy

import numpy as np

from ima2p_gb300 import popmodel, splittime
from ima2p_gb300.synth import Genealogy, LabelledGenealogy
from oracle import pyoracle as O
from tests._golden import load


class RyCase:
    def __init__(self):
        d = load("golden_ry.npz")
        self.d = d
        self.npops = int(d["npops"])
        self.tree = str(d["tree"])
        self.pm = popmodel.build(self.tree, self.npops)
        self.thetaprior, self.mprior = (float(v) for v in d["priors"])
        self.samps = d["samps"].astype(np.int32)
        self.us = d["us"]
        self.nl = len(self.samps)
        self.betas = d["betas"]
        self.nch = len(self.betas)
        self.tprior = [tuple(r) for r in d["tprior"]]
        self.steps = [tuple(int(v) for v in s) for s in d["steps"]]
        self.seed = int(d["seed"])
        so, sh = d["seq_off"], d["seq_shape"]
        self.seqs = [d["seqs"][so[i]:so[i + 1]].reshape(sh[i]).astype(np.int8) for i in range(self.nl)]
        no, mo = d["node_off"], d["mig_off"]
        self.base = []
        for li in range(self.nl):
            a, b = int(no[li]), int(no[li + 1])
            root = int(np.flatnonzero(d["down"][a:b] == -1)[0])
            g = Genealogy(d["up0"][a:b].astype(np.int32), d["up1"][a:b].astype(np.int32),
                          d["down"][a:b].astype(np.int32), d["time"][a:b].copy(), root)
            mig = [[(float(d["mig_t"][e]), int(d["mig_p"][e])) for e in range(mo[j], mo[j + 1])] for j in range(a, b)]
            self.base.append(LabelledGenealogy(g, d["pop"][a:b].copy(), mig))
        self.res = d["res"]
        self.times = d["times"]
        self.migt = d["migt"]

    def fresh_gens(self):
        """Every chain starts from the same genealogies (deep copies)."""
        return [[copy.deepcopy(self.base[li]) for li in range(self.nl)] for _ in range(self.nch)]

    def priors(self):
        nth, nmg = len(self.pm.th_cells), len(self.pm.mg_cells)
        return ([self.thetaprior] * nth, [0.0] * nth, [max(self.mprior, 1e-6)] * nmg, [0.0] * nmg,
                [max(self.mprior, 1e-6) / 2] * nmg)


class OracleBackend:
    """treeweight, p(G) and likelihoodIS on the oracle."""

    def __init__(self, case):
        self.c = case
        self.slk = {}

    def weights(self, ci, gens, tvals):
        c = self.c
        ws, lens = [], []
        for li, lg in enumerate(gens):
            st, w = O.treeweight(c.pm, np.asarray(tvals, np.float64), lg, c.samps[li], 1.0)
            assert st == 0
            ws.append(w)
            lens.append([w["length"], w["tlength"]])
        st, pg, _, _ = O.tree_prob(c.pm, O.sum_weights(ws, c.pm), *c.priors())
        assert st == 0
        return np.array(lens), pg

    def likelihoods(self, ci, gens, lens):
        c = self.c
        out = []
        for li, lg in enumerate(gens):
            if li not in self.slk:  # the reference caches sum log k! from the first genealogy
                self.slk[li] = O.is_sumlogk(c.seqs[li], lg.g)[1]
            out.append(O.is_likelihood(c.seqs[li], lg.g, lens[li][0], c.us[li], self.slk[li])[0])
        return out


def run_chain_set(case, backend, rng):
    """The harness's run: set up every chain as finish_setup_C does, then the
    listed (chain, period) updates in order; returns (per-step results,
    states)."""
    gens = case.fresh_gens()
    states = []
    for ci in range(case.nch):
        tv = np.array(case.d["tv0"], np.float64)
        lens, probg = backend.weights(ci, gens[ci], tv)
        pdg = np.asarray(backend.likelihoods(ci, gens[ci], lens), np.float64)
        s = 0.0
        for v in pdg:
            s += float(v)
        states.append(splittime.ChainState(tv, float(case.betas[ci]), gens[ci], pdg, s, probg))
    res = []
    for ci, k in case.steps:
        acc = splittime.changet_ry1(states[ci], ci, k, rng, case.tprior, case.nl, case.npops, backend)
        st = states[ci]
        res.append((int(acc), float(st.tvals[k]), st.probg, st.pdgsum))
    return np.array(res), states


def final_times(case, states):
    t = np.concatenate([lg.g.time for st in states for lg in st.gens])
    m = np.array([e[0] for st in states for lg in st.gens for mm in lg.mig for e in mm])
    return t, m


class OracleSweepBackend:
    """The batched sweep's backend on the oracle."""

    def __init__(self, case):
        self.c = case
        self.one = OracleBackend(case)

    def _gens(self, cs):
        from ima2p_gb300.synth import Genealogy, LabelledGenealogy
        out = []
        for i in range(cs.nch * cs.nl):
            a, b = int(cs.node_off[i]), int(cs.node_off[i + 1])
            root = int(np.flatnonzero(cs.down[a:b] == -1)[0])
            g = Genealogy(cs.up0[a:b], cs.up1[a:b], cs.down[a:b], cs.time[a:b], root)
            mig = [[(float(cs.mig_t[e]), int(cs.mig_p[e])) for e in range(cs.mig_off[j], cs.mig_off[j + 1])]
                   for j in range(a, b)]
            out.append(LabelledGenealogy(g, cs.pop[a:b], mig))
        return out

    def weights(self, cs):
        gens = self._gens(cs)
        lens, probg = [], []
        for ci in range(cs.nch):
            l_, p_ = self.one.weights(ci, gens[ci * cs.nl:(ci + 1) * cs.nl], cs.tvals[ci])
            lens.append(l_)
            probg.append(p_)
        return np.concatenate(lens), np.array(probg)

    def likelihoods(self, cs, lens):
        gens = self._gens(cs)
        return np.array([self.one.likelihoods(ci, gens[ci * cs.nl:(ci + 1) * cs.nl], lens[ci * cs.nl:(ci + 1) * cs.nl])
                         for ci in range(cs.nch)])

    def decide(self, cs, accept):
        pass


def run_sweeps(case, backend, rng):
    """The fixture's steps as sweeps: chains 0, 1, 2 in order, 30 times."""
    from ima2p_gb300 import splittime
    cs = splittime.ChainSet(case.fresh_gens(), [case.d["tv0"]] * case.nch, case.betas)
    splittime.setup_chainset(cs, backend)
    res = []
    for s0 in range(0, len(case.steps), case.nch):
        periods = [case.steps[s0 + c][1] for c in range(case.nch)]
        assert [case.steps[s0 + c][0] for c in range(case.nch)] == list(range(case.nch))
        acc = splittime.changet_ry1_sweep(cs, periods, rng, case.tprior, case.npops, backend)
        for c in range(case.nch):
            res.append((int(acc[c]), float(cs.tvals[c, periods[c]]), float(cs.probg[c]), float(cs.pdgsum[c])))
    return np.array(res), cs
