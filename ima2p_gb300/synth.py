"""Seeded synthetic inputs with the shapes of IMa2p's hot paths.

An isolation-with-migration coalescent simulator writes genealogies in the
reference's edge layout (imamp.hpp:651-679): ``up0/up1`` daughters (-1 at
tips), ``down`` parent (-1 at the root), ``time[c]`` the time at the lower end
of edge ``c``; tips are ``0..n-1`` and internal nodes ``n..2n-2``.  Time is in
the reference's mutation-scaled units, so a pair of lineages in population
``i`` coalesces at rate ``2/theta_i`` and a branch of length ``t`` carries
Poisson(``t*u``) mutations for a locus rate scalar ``u``.

Data are simulated on those genealogies:

* infinite sites: one segregating site per mutation, coded 0/1 relative to
  the first sequence as readseqIS does (readata.cpp:347-495);
* HKY85: site patterns compressed in first-occurrence order with
  multiplicities (readata.cpp:202-222), empirical base frequencies
  (readata.cpp:247-345);
* stepwise microsatellites: +/-1 steps, root allele 20.

Surface inputs follow the ``gsampinf`` row layout (ginfo.cpp:288-316).
Nothing here is on a timed path.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Genealogy:
    up0: np.ndarray
    up1: np.ndarray
    down: np.ndarray
    time: np.ndarray
    root: int

    @property
    def n(self) -> int:
        return (len(self.up0) + 1) // 2

    def branch(self) -> np.ndarray:
        """Branch length of every edge (0 at the root)."""
        t = self.time.copy()
        internal = self.up0 >= 0
        t[internal] = self.time[internal] - self.time[self.up0[internal]]
        t[self.root] = 0.0
        return t

    def length(self) -> float:
        return float(self.branch().sum())

    def copy(self) -> "Genealogy":
        return Genealogy(self.up0.copy(), self.up1.copy(), self.down.copy(),
                         self.time.copy(), int(self.root))


def sim_im_genealogy(rng, samples, theta, mig, splits, theta_anc=None):
    """Structured coalescent with population splits.

    samples: lineages sampled per extant population.
    theta:   theta of every population id (extant then ancestral).
    mig:     per-lineage migration rate between co-existing populations.
    splits:  list of (time, pop_a, pop_b, new_pop) in increasing time.
    """
    n = int(sum(samples))
    nl = 2 * n - 1
    up0 = np.full(nl, -1, np.int32)
    up1 = np.full(nl, -1, np.int32)
    down = np.full(nl, -1, np.int32)
    time = np.zeros(nl, np.float64)
    lin = []  # (node, pop)
    k = 0
    for p, s in enumerate(samples):
        for _ in range(s):
            lin.append([k, p])
            k += 1
    active = set(range(len(samples)))
    nxt = n
    t = 0.0
    si = 0
    while len(lin) > 1:
        counts = {}
        for _, p in lin:
            counts[p] = counts.get(p, 0) + 1
        crate = {p: c * (c - 1) / theta[p] for p, c in counts.items() if c > 1}
        mrate = mig * len(lin) if len(active) > 1 else 0.0
        total = sum(crate.values()) + mrate
        wait = rng.exponential(1.0 / total) if total > 0 else np.inf
        tsplit = splits[si][0] if si < len(splits) else np.inf
        if t + wait >= tsplit:
            t = tsplit
            _, a, b, new = splits[si]
            for l in lin:
                if l[1] in (a, b):
                    l[1] = new
            active.discard(a)
            active.discard(b)
            active.add(new)
            si += 1
            continue
        t += wait
        r = rng.uniform(0, total)
        if r < mrate:
            li = int(rng.integers(len(lin)))
            others = sorted(active - {lin[li][1]})
            lin[li][1] = int(others[rng.integers(len(others))])
            continue
        r -= mrate
        pops = list(crate)
        p = pops[-1]
        for q in pops:
            if r < crate[q]:
                p = q
                break
            r -= crate[q]
        idx = [i for i, l in enumerate(lin) if l[1] == p]
        i, j = rng.choice(idx, 2, replace=False)
        a, b = lin[i][0], lin[j][0]
        node = nxt
        nxt += 1
        up0[node], up1[node] = a, b
        down[a] = down[b] = node
        time[a] = time[b] = t
        for x in sorted((i, j), reverse=True):
            lin.pop(x)
        lin.append([node, p])
    root = lin[0][0]
    time[root] = -1.0
    return Genealogy(up0, up1, down, time, int(root))


@dataclasses.dataclass
class LabelledGenealogy:
    """A genealogy with the population labels treeweight reads
    (update_gtree_common.cpp:1680-1937): ``pop[i]`` is the population at the
    lower end of edge ``i`` (the sampled population at a tip, the population
    of the coalescence otherwise) and ``mig[i]`` the migration events along
    the edge, oldest last, as (time, population moved to going back in time)
    pairs -- the reference's ``gtree[i].mig[]`` list (imamp.hpp:601-605).
    Population changes at splits are implicit, as in the reference."""
    g: Genealogy
    pop: np.ndarray
    mig: list

    @property
    def mignum(self) -> int:
        return sum(len(m) for m in self.mig)

    def packed_mig(self):
        """CSR form: per-node offsets (len nodes+1), times, destination pops."""
        off = np.zeros(len(self.mig) + 1, np.int32)
        off[1:] = np.cumsum([len(m) for m in self.mig])
        t = np.array([e[0] for m in self.mig for e in m], np.float64)
        p = np.array([e[1] for m in self.mig for e in m], np.int32)
        return off, t, p


def sim_im_labeled(rng, samples, theta, mig, splits):
    """The structured coalescent of sim_im_genealogy, recording where each
    lineage is: the population of every coalescence and every migration event
    with its time and destination.  ``splits`` as in sim_im_genealogy, with
    ``new_pop`` the ancestral population id of the reference's tree string
    (the split forming population npops+k happens at the k-th split time)."""
    n = int(sum(samples))
    nl = 2 * n - 1
    up0 = np.full(nl, -1, np.int32)
    up1 = np.full(nl, -1, np.int32)
    down = np.full(nl, -1, np.int32)
    time = np.zeros(nl, np.float64)
    pop = np.zeros(nl, np.int32)
    migs = [[] for _ in range(nl)]
    lin = []  # [node, current pop, events on the edge so far]
    k = 0
    for p, s in enumerate(samples):
        for _ in range(s):
            lin.append([k, p, []])
            pop[k] = p
            k += 1
    active = set(range(len(samples)))
    nxt = n
    t = 0.0
    si = 0
    while len(lin) > 1:
        counts = {}
        for _, p, _e in lin:
            counts[p] = counts.get(p, 0) + 1
        crate = {p: c * (c - 1) / theta[p] for p, c in counts.items() if c > 1}
        mrate = mig * len(lin) if len(active) > 1 else 0.0
        total = sum(crate.values()) + mrate
        wait = rng.exponential(1.0 / total) if total > 0 else np.inf
        tsplit = splits[si][0] if si < len(splits) else np.inf
        if t + wait >= tsplit:
            t = tsplit
            _, a, b, new = splits[si]
            for l in lin:
                if l[1] in (a, b):
                    l[1] = new
            active.discard(a)
            active.discard(b)
            active.add(new)
            si += 1
            continue
        t += wait
        r = rng.uniform(0, total)
        if r < mrate:
            li = int(rng.integers(len(lin)))
            others = sorted(active - {lin[li][1]})
            dest = int(others[rng.integers(len(others))])
            lin[li][1] = dest
            lin[li][2].append((t, dest))
            continue
        r -= mrate
        pops = list(crate)
        p = pops[-1]
        for q in pops:
            if r < crate[q]:
                p = q
                break
            r -= crate[q]
        idx = [i for i, l in enumerate(lin) if l[1] == p]
        i, j = rng.choice(idx, 2, replace=False)
        a, b = lin[i][0], lin[j][0]
        migs[a], migs[b] = lin[i][2], lin[j][2]
        node = nxt
        nxt += 1
        up0[node], up1[node] = a, b
        down[a] = down[b] = node
        time[a] = time[b] = t
        pop[node] = p
        for x in sorted((i, j), reverse=True):
            lin.pop(x)
        lin.append([node, p, []])
    root = lin[0][0]
    time[root] = -1.0
    return LabelledGenealogy(Genealogy(up0, up1, down, time, int(root)), pop, migs)


def splits_from_treestring(s: str, npops: int):
    """(daughter a, daughter b, ancestor) per split of an IMa2p population
    tree string such as "((0,1):3,2):4", ordered by ancestor id: the
    ancestor numbered npops+k forms at the k-th split time
    (build_poptree.cpp:508-629)."""
    pos = 0

    def node():
        nonlocal pos
        if s[pos] == "(":
            pos += 1
            a = node()
            assert s[pos] == ","
            pos += 1
            b = node()
            assert s[pos] == ")" and s[pos + 1] == ":"
            pos += 2
            j = pos
            while pos < len(s) and s[pos].isdigit():
                pos += 1
            anc = int(s[j:pos])
            out.append((a, b, anc))
            return anc
        j = pos
        while pos < len(s) and s[pos].isdigit():
            pos += 1
        return int(s[j:pos])

    out = []
    node()
    out.sort(key=lambda x: x[2])
    assert [x[2] for x in out] == list(range(npops, 2 * npops - 1))
    return out


def two_pop_tree(rng, n1, n2, theta=5.0, mig=0.1, tsplit=1.0):
    return sim_im_genealogy(rng, [n1, n2], [theta, theta, theta], mig,
                            [(tsplit, 0, 1, 2)])


def three_pop_tree(rng, samples, theta=4.0, mig=0.05, t1=1.0, t2=2.0):
    return sim_im_genealogy(rng, list(samples), [theta] * 5, mig,
                            [(t1, 0, 1, 3), (t2, 3, 2, 4)])


def jitter_times(rng, g: Genealogy, scale=0.1) -> Genealogy:
    """Same topology, internal times rescaled by one random factor."""
    h = g.copy()
    f = float(np.exp(rng.normal(0.0, scale)))
    keep = h.time >= 0
    h.time[keep] *= f
    return h


# ----------------------------------------------------------------- IS data
def is_data(rng, g: Genealogy, u: float, min_sites: int = 1):
    """Infinite-sites 0/1 matrix [n, S] compatible with g by construction."""
    n = g.n
    br = g.branch()
    below = _tips_below(g)
    cols = []
    for c in range(2 * n - 1):
        if c == g.root:
            continue
        for _ in range(rng.poisson(br[c] * u)):
            col = np.zeros(n, np.int8)
            col[below[c]] = 1
            cols.append(col)
    while len(cols) < min_sites:
        c = int(rng.integers(2 * n - 1))
        if c == g.root:
            continue
        col = np.zeros(n, np.int8)
        col[below[c]] = 1
        cols.append(col)
    rng.shuffle(cols)
    seq = np.stack(cols, axis=1) if cols else np.zeros((n, 0), np.int8)
    seq = np.where(seq[0:1, :] == 1, 1 - seq, seq).astype(np.int8)
    return np.ascontiguousarray(seq)


def _tips_below(g: Genealogy):
    n = g.n
    out = [None] * (2 * n - 1)
    order = postorder(g)
    for c in order:
        if g.up0[c] < 0:
            out[c] = [c]
        else:
            out[c] = out[g.up0[c]] + out[g.up1[c]]
    return out


def postorder(g: Genealogy):
    order = []
    stack = [(g.root, False)]
    while stack:
        c, seen = stack.pop()
        if g.up0[c] < 0 or seen:
            order.append(c)
            continue
        stack.append((c, True))
        stack.append((int(g.up1[c]), False))
        stack.append((int(g.up0[c]), False))
    return order


# ---------------------------------------------------------------- HKY data
def hky_standfactor(pi, kappa):
    p = 0.0
    for i in range(4):
        for j in range(4):
            if i != j:
                p += pi[i] * pi[j] * (kappa if (i + j) in (2, 4) else 1.0)
    return p


def hky_pmatrix(pi, kappa, b):
    P = np.zeros((4, 4))
    e1 = np.exp(-b)
    for k in range(4):
        Pk = pi[0] + pi[2] if k in (0, 2) else pi[1] + pi[3]
        A = 1.0 + Pk * (kappa - 1.0)
        e2 = np.exp(-b * A)
        for j in range(4):
            if j == k:
                P[j, k] = pi[k] + pi[k] * e1 * (1 / Pk - 1) + e2 * (Pk - pi[k]) / Pk
            elif j + k in (2, 4):
                P[j, k] = pi[k] + pi[k] * e1 * (1 / Pk - 1) - pi[k] / Pk * e2
            else:
                P[j, k] = pi[k] * (1 - e1)
    return P


@dataclasses.dataclass
class HKYLocus:
    seq: np.ndarray      # [n, S'] int8 patterns, states 0..3 (A C G T)
    mult: np.ndarray     # [S'] int32
    totsites: int
    pi: np.ndarray       # empirical base frequencies (used by the likelihood)


def hky_data(rng, g: Genealogy, nbases: int, u: float, kappa: float, pi_sim):
    n = g.n
    mu = u / (nbases * hky_standfactor(pi_sim, kappa))
    br = g.branch()
    states = np.zeros((2 * n - 1, nbases), np.int8)
    states[g.root] = rng.choice(4, size=nbases, p=pi_sim)
    for c in reversed(postorder(g)):
        if c == g.root:
            continue
        P = hky_pmatrix(pi_sim, kappa, mu * br[c])
        par = states[g.down[c]]
        cum = np.cumsum(P, axis=1)
        r = rng.uniform(size=nbases)
        states[c] = (r[:, None] > cum[par]).sum(axis=1).clip(0, 3)
    tips = states[:n]
    counts = np.bincount(tips.ravel(), minlength=4).astype(np.float64)
    pi_emp = counts / counts.sum()
    cols, inv = np.unique(tips.T, axis=0, return_inverse=True)
    inv = inv.ravel()
    first = np.full(len(cols), nbases)
    for s in range(nbases - 1, -1, -1):
        first[inv[s]] = s
    order = np.argsort(first)
    mult = np.bincount(inv, minlength=len(cols))[order].astype(np.int32)
    seq = np.ascontiguousarray(cols[order].T.astype(np.int8))
    return HKYLocus(seq, mult, nbases, pi_emp)


# ----------------------------------------------------------------- SW data
def sw_alleles(rng, g: Genealogy, u: float, root_allele=20, min_allele=4,
               max_tries=100):
    n = g.n
    br = g.branch()
    for _ in range(max_tries):
        A = np.zeros(2 * n - 1, np.int32)
        A[g.root] = root_allele
        for c in reversed(postorder(g)):
            if c == g.root:
                continue
            k = rng.poisson(br[c] * u)
            steps = int(2 * rng.binomial(k, 0.5) - k) if k else 0
            A[c] = A[g.down[c]] + steps
        if A.min() >= min_allele:
            return A
    return np.maximum(A, min_allele)


# ------------------------------------------------------------ surface data
def gsamp_layout(np_, nm, nsplit):
    """Column offsets of a gsampinf row (ginfo.cpp:288-316)."""
    off = dict(cc=0, fc=np_, hcc=2 * np_, mc=3 * np_, fm=3 * np_ + nm,
               qi=3 * np_ + 2 * nm, mi=4 * np_ + 2 * nm, pdg=4 * np_ + 3 * nm)
    off["probg"] = off["pdg"] + 1
    off["t"] = off["probg"] + 1
    off["rowlen"] = off["t"] + nsplit
    return off


def surface_stats(rng, G, np_=5, nm=8, nsplit=2):
    """Synthetic gsampinf rows and an FP64 per-genealogy log normaliser:
    cc ~ Poisson(8), fc ~ Gamma(4,1), mc ~ Poisson(1), fm ~ Gamma(2,1),
    normaliser ~ N(-200, 20)."""
    off = gsamp_layout(np_, nm, nsplit)
    rows = np.zeros((G, off["rowlen"]), np.float32)
    rows[:, off["cc"]:off["cc"] + np_] = rng.poisson(8.0, (G, np_))
    rows[:, off["fc"]:off["fc"] + np_] = rng.gamma(4.0, 1.0, (G, np_))
    rows[:, off["hcc"]:off["hcc"] + np_] = 0.0
    rows[:, off["mc"]:off["mc"] + nm] = rng.poisson(1.0, (G, nm))
    rows[:, off["fm"]:off["fm"] + nm] = rng.gamma(2.0, 1.0, (G, nm))
    rows[:, off["qi"]:off["qi"] + np_] = rng.normal(-20.0, 2.0, (G, np_))
    rows[:, off["mi"]:off["mi"] + nm] = rng.normal(-5.0, 1.0, (G, nm))
    lognorm = rng.normal(-200.0, 20.0, G)
    rows[:, off["pdg"]] = rng.normal(-100.0, 5.0, G)
    rows[:, off["probg"]] = (-lognorm).astype(np.float32)
    rows[:, off["t"]:off["t"] + nsplit] = rng.uniform(0.1, 3.0, (G, nsplit))
    return rows, lognorm, off


def peaked_stats(rng, G, np_=5, nm=8, nsplit=2):
    """Synthetic gsampinf rows whose marginal densities peak inside priors of
    theta <= 20 and m <= 2: cc ~ Poisson(15) with fc / cc ~ U(1, 5) (theta
    peaks near 2 fc / cc), mc ~ Poisson(4) with mc / fm ~ U(0.3, 2) (m peaks
    near mc / fm), log integrals ~ N(0, 1)."""
    off = gsamp_layout(np_, nm, nsplit)
    rows = np.zeros((G, off["rowlen"]), np.float32)
    cc = rng.poisson(15.0, (G, np_))
    rows[:, off["cc"]:off["cc"] + np_] = cc
    rows[:, off["fc"]:off["fc"] + np_] = cc * rng.uniform(1.0, 5.0, (G, np_))
    mc = rng.poisson(4.0, (G, nm))
    rows[:, off["mc"]:off["mc"] + nm] = mc
    rows[:, off["fm"]:off["fm"] + nm] = np.maximum(mc, 0.5) / rng.uniform(0.3, 2.0, (G, nm))
    rows[:, off["qi"]:off["qi"] + np_] = rng.normal(0.0, 1.0, (G, np_))
    rows[:, off["mi"]:off["mi"] + nm] = rng.normal(0.0, 1.0, (G, nm))
    rows[:, off["t"]:off["t"] + nsplit] = rng.uniform(0.1, 3.0, (G, nsplit))
    return rows


def surface_points(rng, P, np_=5, nm=8, theta_hi=20.0, m_hi=2.0):
    th = rng.uniform(0.1, theta_hi, (P, np_))
    m = rng.uniform(1e-7, m_hi, (P, nm))
    return np.ascontiguousarray(np.concatenate([th, m], axis=1))
