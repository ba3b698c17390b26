"""Seeded synthetic workloads with the shapes of the benchmark configurations.

  is       2 populations, 5 IS loci x (10+10) copies, 4 geometric chains
  hky      2 populations, 50 HKY loci x (20+20) x 1000 bp, 32 chains
  sw       3 sampled populations (5-population tree), 100 SW loci x 30 copies
           per population, 64 chains
  mixed    300 loci (200 HKY of U(200,3000) bp, 100 SW), U(4,60) copies per
           population x 3 populations, 128 chains x 8 runs
  surface  G = 2^21 genealogy summaries, K = 48 row width, P = 2^16 points
  updgen   the hky shapes (50 HKY loci x (20+20) x 1000 bp) under the
           no-migration model, population-labelled genealogies, for the
           genealogy update

Every chain gets its own genealogy per locus: independent coalescent draws
for the smaller configurations, time-rescaled copies of a per-locus draw
(with perturbed internal microsatellite states) for the large ones.  Data
and parameters follow the distributions the configurations name.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import synth


@dataclasses.dataclass
class Workload:
    name: str
    describe: str
    loci: list            # ("is", seq) | ("hky", HKYLocus) | ("sw", n, 1)
    nruns: int
    cpr: int
    trees: dict            # (ci, li) -> Genealogy (or built on demand, see tree())
    u: np.ndarray          # [nchains, nloci]
    par: np.ndarray        # [nchains, nloci] kappa (HKY) / tr (SW) / unused
    pi: dict               # (ci, li) -> base frequencies (or per locus, see pi_of())
    alleles: dict          # (ci, li) -> int32 [2n-1]
    lazy: object = None    # optional (base trees, time factors, allele fn) for big runs

    @property
    def nchains(self):
        return self.nruns * self.cpr

    @property
    def nloci(self):
        return len(self.loci)

    def pairs(self):
        ci = np.repeat(np.arange(self.nchains), self.nloci).astype(np.int32)
        li = np.tile(np.arange(self.nloci), self.nchains).astype(np.int32)
        return ci, li

    def tree(self, c, l):
        if self.lazy is None:
            return self.trees[(c, l)]
        base, fac, _ = self.lazy
        g = base[l].copy()
        keep = g.time >= 0
        g.time[keep] *= fac[c, l]
        return g

    def allele(self, c, l):
        if self.lazy is None:
            return self.alleles.get((c, l))
        return self.lazy[2](c, l)

    def packed(self):
        """Node arrays of every chain-locus concatenated in pair order."""
        ci, li = self.pairs()
        if self.lazy is None:
            gs = [self.trees[(int(c), int(l))] for c, l in zip(ci, li)]
            cat = lambda f: np.concatenate([getattr(g, f) for g in gs])
            return ci, li, cat("up0").astype(np.int32), cat("up1").astype(np.int32), \
                cat("down").astype(np.int32), cat("time")
        base, fac, _ = self.lazy
        nl = np.array([len(g.up0) for g in base])
        rows = [np.tile(np.concatenate([base[l].up0 for l in range(self.nloci)]), self.nchains)]
        up0 = rows[0].astype(np.int32)
        up1 = np.tile(np.concatenate([g.up1 for g in base]), self.nchains).astype(np.int32)
        down = np.tile(np.concatenate([g.down for g in base]), self.nchains).astype(np.int32)
        bt = np.concatenate([g.time for g in base])
        f = np.repeat(fac.reshape(-1), np.tile(nl, self.nchains))
        t = np.tile(bt, self.nchains)
        time = np.where(t >= 0, t * f, t)
        return ci, li, up0, up1, down, time

    def upload(self, ctx):
        ci, li, up0, up1, down, time = self.packed()
        ctx.set_genealogies(ci, li, up0, up1, down, time)
        if self.lazy is None:
            for (c, l), p in self.pi.items():
                ctx.set_pi(c, l, p)
            for (c, l), A in self.alleles.items():
                ctx.set_alleles(c, l, A)
        else:
            for l, spec in enumerate(self.loci):
                for c in range(self.nchains):
                    if spec[0] == "hky":
                        ctx.set_pi(c, l, spec[1].pi)
                    elif spec[0] == "sw":
                        ctx.set_alleles(c, l, self.allele(c, l))


def _loci_u(rng, nloci):
    u = rng.lognormal(0.0, 0.5, nloci)
    return u / np.exp(np.mean(np.log(u)))  # product of the scalars = 1


def make_is(seed=1001, nloci=5, nch=4):
    rng = np.random.default_rng(seed)
    loci, trees = [], {}
    u = np.tile(_loci_u(rng, nloci), (nch, 1))
    for li in range(nloci):
        g0 = synth.two_pop_tree(rng, 10, 10, theta=5.0, mig=0.1, tsplit=1.0)
        loci.append(("is", synth.is_data(rng, g0, u[0, li] * 1.0, min_sites=3)))
        for ci in range(nch):
            trees[(ci, li)] = g0 if ci == 0 else synth.jitter_times(rng, g0, 0.1)
    return Workload("is", "config1-is: 2 pops, %d IS loci x (10+10) copies, 500 bp, %d chains" % (nloci, nch),
                    loci, 1, nch, trees, u, np.ones((nch, nloci)), {}, {})


def make_hky(seed=1002, nloci=50, nch=32, ncopies=20, nbases=1000):
    rng = np.random.default_rng(seed)
    loci, trees, pis = [], {}, {}
    ul = _loci_u(rng, nloci)
    kap = rng.uniform(2.0, 8.0, nloci)
    for li in range(nloci):
        g0 = synth.two_pop_tree(rng, ncopies, ncopies, theta=10.0, mig=0.2, tsplit=1.5)
        loc = synth.hky_data(rng, g0, nbases, float(ul[li]), float(kap[li]), rng.dirichlet([5, 5, 5, 5]))
        loci.append(("hky", loc))
        for ci in range(nch):
            trees[(ci, li)] = g0 if ci == 0 else synth.two_pop_tree(rng, ncopies, ncopies, 10.0, 0.2, 1.5)
            pis[(ci, li)] = loc.pi
    return Workload("hky", "config2-hky: 2 pops, %d HKY loci x (%d+%d) x %d bp, %d chains, "
                           "full re-evaluation of every chain-locus per step" % (nloci, ncopies, ncopies, nbases, nch),
                    loci, 1, nch, trees, np.tile(ul, (nch, 1)), np.tile(kap, (nch, 1)), pis, {})


def _perturb_alleles(rng, g, A, n):
    B = A.copy()
    internal = np.arange(n, 2 * n - 1)
    flip = rng.uniform(size=len(internal)) < 0.2
    B[internal[flip]] += rng.choice([-1, 1], size=int(flip.sum()))
    return np.maximum(B, 4).astype(np.int32)


def make_sw(seed=1003, nloci=100, nch=64, per_pop=30):
    rng = np.random.default_rng(seed)
    loci, trees, alleles = [], {}, {}
    ul = _loci_u(rng, nloci)
    n = 3 * per_pop
    for li in range(nloci):
        g0 = synth.three_pop_tree(rng, [per_pop] * 3, theta=4.0, mig=0.05)
        A0 = synth.sw_alleles(rng, g0, float(ul[li]))
        loci.append(("sw", n, 1))
        for ci in range(nch):
            trees[(ci, li)] = g0 if ci == 0 else synth.jitter_times(rng, g0, 0.15)
            alleles[(ci, li)] = A0 if ci == 0 else _perturb_alleles(rng, g0, A0, n)
    return Workload("sw", "config3-sw: 3 sampled pops (5-pop tree), %d SW loci x %d copies, %d chains, "
                          "full evaluation of every chain-locus per step" % (nloci, n, nch),
                    loci, 1, nch, trees, np.tile(ul, (nch, 1)), np.ones((nch, nloci)), {}, alleles)


def make_mixed(seed=1004, n_hky=200, n_sw=100, nruns=8, cpr=128):
    rng = np.random.default_rng(seed)
    loci, base, A0s = [], [], {}
    nloci = n_hky + n_sw
    ul = _loci_u(rng, nloci)
    kap = rng.uniform(2.0, 8.0, nloci)
    for li in range(nloci):
        samples = [int(v) for v in rng.integers(4, 61, 3)]
        g0 = synth.three_pop_tree(rng, samples, theta=10.0 if li < n_hky else 4.0, mig=0.05)
        base.append(g0)
        if li < n_hky:
            loc = synth.hky_data(rng, g0, int(rng.integers(200, 3001)), float(ul[li]), float(kap[li]),
                                 rng.dirichlet([5, 5, 5, 5]))
            loci.append(("hky", loc))
        else:
            loci.append(("sw", g0.n, 1))
            A0s[li] = synth.sw_alleles(rng, g0, float(ul[li]))
    nch = nruns * cpr
    fac = np.exp(rng.normal(0.0, 0.15, (nch, nloci)))

    def allele(c, l):
        if l not in A0s:
            return None
        r = np.random.default_rng(seed * 7919 + c * 1000 + l)
        return _perturb_alleles(r, base[l], A0s[l], base[l].n)

    par = np.tile(np.where(np.arange(nloci) < n_hky, kap, 1.0), (nch, 1))
    return Workload("mixed", "config4-mixed: 300 loci (200 HKY U(200,3000) bp + 100 SW), U(4,60) copies "
                             "x 3 pops, %d chains x %d runs" % (cpr, nruns),
                    loci, nruns, cpr, {}, np.tile(ul, (nch, 1)), par, {}, {},
                    lazy=(base, fac, allele))


def make(name):
    return {"is": make_is, "hky": make_hky, "sw": make_sw, "mixed": make_mixed}[name]()


@dataclasses.dataclass
class UgWorkload:
    """Population-labelled genealogies and data for the genealogy update:
    every chain starts from the locus's own coalescent draw."""
    describe: str
    tree: str
    npops: int
    tvals: list
    kind: str             # "hky" or "sw"
    loci: list            # HKYLocus per locus (hky)
    base: list            # synth.LabelledGenealogy per locus
    samppop: np.ndarray   # [nloci][npops]
    u: np.ndarray         # [nloci]
    kappa: np.ndarray     # [nloci]
    nch: int
    alleles: list = None       # sw: every node's allele per locus
    arange: np.ndarray = None  # sw: [nloci][2] allele range


def make_updgen(seed=1006, nloci=50, nch=32, ncopies=20, nbases=1000, tsplit=1.5, theta=10.0):
    """The hky workload's shapes under the no-migration model (two
    populations split at tsplit): kappa ~ U(2, 8), base frequencies ~
    Dirichlet(5, 5, 5, 5), lognormal(0, 0.5) rate scalars."""
    rng = np.random.default_rng(seed)
    ul = _loci_u(rng, nloci)
    kap = rng.uniform(2.0, 8.0, nloci)
    splits = [(tsplit, 0, 1, 2)]
    loci, base = [], []
    for li in range(nloci):
        lg = synth.sim_im_labeled(rng, [ncopies, ncopies], [theta] * 3, 0.0, splits)
        loci.append(synth.hky_data(rng, lg.g, nbases, float(ul[li]), float(kap[li]), rng.dirichlet([5, 5, 5, 5])))
        base.append(lg)
    return UgWorkload("genealogy update: 2 pops (no migration, split at %g), %d HKY loci x (%d+%d) x %d bp, "
                      "%d chains, one proposal per chain-locus per sweep" % (tsplit, nloci, ncopies, ncopies,
                                                                             nbases, nch),
                      "(0,1):2", 2, [tsplit], "hky", loci, base,
                      np.tile([ncopies, ncopies], (nloci, 1)).astype(np.int32), ul, kap, nch)


def make_updgen_sw(seed=1007, nloci=100, nch=64, per_pop=30, tvals=(0.8, 1.6), theta=4.0):
    """The sw workload's shapes under the no-migration model: 3 sampled
    populations of a 5-population tree, stepwise loci with alleles
    simulated on each locus's genealogy (root allele 20), lognormal(0, 0.5)
    rate scalars; each locus's allele range is its alleles' widened by 5."""
    rng = np.random.default_rng(seed)
    ul = _loci_u(rng, nloci)
    splits = [(tvals[0], 0, 1, 3), (tvals[1], 2, 3, 4)]
    base, alleles, ar = [], [], []
    for li in range(nloci):
        lg = synth.sim_im_labeled(rng, [per_pop] * 3, [theta] * 5, 0.0, splits)
        A = synth.sw_alleles(rng, lg.g, float(ul[li]))
        base.append(lg)
        alleles.append(A)
        ar.append([int(A.min()) - 5, int(A.max()) + 5])
    return UgWorkload("genealogy update: 3 sampled pops of a 5-pop tree (no migration), %d SW loci x %d copies, "
                      "%d chains, one proposal per chain-locus per sweep" % (nloci, 3 * per_pop, nch),
                      "((0,1):3,2):4", 3, list(tvals), "sw", [None] * nloci, base,
                      np.tile([per_pop] * 3, (nloci, 1)).astype(np.int32), ul, np.ones(nloci), nch, alleles,
                      np.array(ar, np.int32))
