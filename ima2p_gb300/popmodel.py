"""Population-tree tables and parameter maps for the genealogy-weight path.

Host logic only.  The reference derives these once per run from the
population tree string:

* ``fillplist`` (build_poptree.cpp:391-450): period 0 holds the sampled
  populations 0..npops-1; at the k-th split (k = 1..npops-1) the two
  daughters (``droppops[k]``, in increasing id) leave and their ancestor
  (``addpop[k]``, id npops+k-1) joins; ``plist[k]`` lists the populations of
  period k in increasing id.  ``pop_e[p]`` is the period at which population
  p ends (-1 for the root) and ``pop_down[p]`` its ancestor.
* ``setup_iparams`` (initialize.cpp:202-727), default model options: one
  theta per tree population, collecting its (period, position) cells; one
  migration rate per ordered pair of populations first co-existing in a
  period (both sampled, or one of them new there), collecting the pair's
  cells in every later period both still exist.  ``-j`` model variants other
  than no-migration are not built.

Cells are addressed in the flat layout the device path uses:
``T = npops(npops+1)/2`` coalescent cells at ``k*npops - k(k-1)/2 + ii`` and
``M = sum_{k<npops-1} (npops-k)^2`` migration cells at
``moff(k) + ii*(npops-k) + jj``.
"""
from __future__ import annotations

import dataclasses

import numpy as np

MAXPOPS = 10  # imamp.hpp:122


def toff(npops: int, k: int) -> int:
    return k * npops - k * (k - 1) // 2


def moff(npops: int, k: int) -> int:
    return sum((npops - j) ** 2 for j in range(k))


def sizes(npops: int):
    return npops * (npops + 1) // 2, moff(npops, npops - 1)


def parse_treestring(s: str, npops: int):
    """(daughter a, daughter b, ancestor) per split of a tree string such as
    "((0,1):3,2):4", ordered by ancestor id (the ancestor npops+k-1 forms at
    the k-th split time; poptreeread, build_poptree.cpp:508-629)."""
    pos = 0
    out = []

    def number():
        nonlocal pos
        j = pos
        while pos < len(s) and s[pos].isdigit():
            pos += 1
        if j == pos:
            raise ValueError("population tree string: number expected at %d in %r" % (j, s))
        return int(s[j:pos])

    def node():
        nonlocal pos
        if pos < len(s) and s[pos] == "(":
            pos += 1
            a = node()
            if pos >= len(s) or s[pos] != ",":
                raise ValueError("population tree string: ',' expected in %r" % s)
            pos += 1
            b = node()
            if s[pos:pos + 2] != "):":
                raise ValueError("population tree string: '):' expected in %r" % s)
            pos += 2
            anc = number()
            out.append((a, b, anc))
            return anc
        return number()

    node()
    if pos != len(s):
        raise ValueError("population tree string: trailing text in %r" % s)
    out.sort(key=lambda x: x[2])
    if [x[2] for x in out] != list(range(npops, 2 * npops - 1)):
        raise ValueError("population tree string %r does not number its %d ancestors "
                         "npops..2npops-2" % (s, npops - 1))
    tips = sorted(v for a, b, _ in out for v in (a, b) if v < npops)
    if tips != list(range(npops)):
        raise ValueError("population tree string %r does not hold populations 0..%d once each"
                         % (s, npops - 1))
    return out


@dataclasses.dataclass
class PopModel:
    npops: int
    plist: np.ndarray      # [npops, npops]  (row k: npops-k entries, rest -1)
    droppops: np.ndarray   # [npops, 2]
    addpop: np.ndarray     # [npops]
    pop_e: np.ndarray      # [2npops-1]
    pop_down: np.ndarray   # [2npops-1]
    nomig: bool
    th_cells: list         # per theta parameter: flat T cells
    mg_cells: list         # per migration parameter: flat M cells
    th_names: list
    mg_names: list

    @property
    def T(self) -> int:
        return sizes(self.npops)[0]

    @property
    def M(self) -> int:
        return sizes(self.npops)[1]

    def th_csr(self):
        off = np.zeros(len(self.th_cells) + 1, np.int32)
        off[1:] = np.cumsum([len(c) for c in self.th_cells])
        idx = np.array([v for c in self.th_cells for v in c], np.int32)
        return off, idx

    def mg_csr(self):
        off = np.zeros(len(self.mg_cells) + 1, np.int32)
        off[1:] = np.cumsum([len(c) for c in self.mg_cells])
        idx = np.array([v for c in self.mg_cells for v in c], np.int32)
        return off, idx

    def period_of(self, tvals, t):
        """findperiod (update_gtree_common.cpp:1626)."""
        k = 0
        while k < self.npops - 1 and tvals[k] <= t:
            k += 1
        return k


def build(treestring: str, npops: int, nomig: bool = False) -> PopModel:
    if not 2 <= npops <= MAXPOPS:
        raise ValueError("npops must be in 2..%d" % MAXPOPS)
    splits = parse_treestring(treestring, npops)
    ntp = 2 * npops - 1
    pop_b = np.zeros(ntp, np.int32)
    pop_e = np.full(ntp, -1, np.int32)
    pop_down = np.full(ntp, -1, np.int32)
    for k, (a, b, anc) in enumerate(splits, start=1):
        pop_b[anc] = k
        for d in (a, b):
            pop_e[d] = k
            pop_down[d] = anc
    plist = np.full((npops, npops), -1, np.int32)
    droppops = np.full((npops, 2), -1, np.int32)
    addpop = np.full(npops, -1, np.int32)
    cur = set(range(npops))
    plist[0, :npops] = np.arange(npops)
    periods = [sorted(cur)]
    for k in range(1, npops):
        gone = sorted(j for j in range(ntp) if pop_e[j] == k)
        new = [j for j in range(ntp) if pop_b[j] == k]
        droppops[k] = gone
        addpop[k] = new[0]
        cur = (cur - set(gone)) | {new[0]}
        periods.append(sorted(cur))
        plist[k, :npops - k] = periods[k]

    # theta parameters: one per tree population (initialize.cpp:296-325)
    th_cells, th_names = [], []
    for p in range(ntp):
        th_cells.append([toff(npops, k) + ii for k in range(npops) for ii, q in enumerate(periods[k]) if q == p])
        th_names.append("q%d" % p)

    # migration parameters (initialize.cpp:375-660, default options)
    mg_cells, mg_names = [], []
    if not nomig:
        last = npops - 1
        for k in range(last):
            n_k = npops - k
            for i in range(n_k - 1):
                for j in range(i + 1, n_k):
                    pi, pj = periods[k][i], periods[k][j]
                    if k > 0 and pi in periods[k - 1] and pj in periods[k - 1]:
                        continue
                    for src, dst in ((pi, pj), (pj, pi)):
                        cells = []
                        for kk in range(k, last):
                            if pi not in periods[kk] or pj not in periods[kk]:
                                break
                            a = periods[kk].index(src)
                            b = periods[kk].index(dst)
                            cells.append(moff(npops, kk) + a * (npops - kk) + b)
                        mg_cells.append(cells)
                        mg_names.append("m%d>%d" % (src, dst))
    return PopModel(npops, plist, droppops, addpop, pop_e, pop_down, bool(nomig),
                    th_cells, mg_cells, th_names, mg_names)


def popmig_terms(pm: PopModel):
    """The 2NM terms print_populationmigrationrate_histograms draws for the
    default parameterisation (histograms.cpp:754-773): for every population
    but the root (thetai < numtreepops - 1), each migration parameter whose
    name starts with that population ("m<thetai>>..."), in (thetai, mi)
    order; returns [(thetai, mi, label)] with the reference's "2N<i>m<i>><j>"
    labels."""
    out = []
    for ti in range(2 * pm.npops - 2):
        for mi, name in enumerate(pm.mg_names):
            if int(name[1:].split(">")[0]) == ti:
                out.append((ti, mi, "2N%d%s" % (ti, name)))
    return out
