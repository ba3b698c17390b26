"""Population-tree tables and parameter maps for the genealogy-weight path.

Host logic only.  The reference derives these once per run from the
population tree string:

* ``fillplist`` (build_poptree.cpp:391-450): period 0 holds the sampled
  populations 0..npops-1; at the k-th split (k = 1..npops-1) the two
  daughters (``droppops[k]``, in increasing id) leave and their ancestor
  (``addpop[k]``, id npops+k-1) joins; ``plist[k]`` lists the populations of
  period k in increasing id.  ``pop_e[p]`` is the period at which population
  p ends (-1 for the root) and ``pop_down[p]`` its ancestor.
* ``setup_iparams`` (initialize.cpp:202-727): by default one theta per tree
  population, collecting its (period, position) cells, and one migration
  rate per ordered pair of populations first co-existing in a period (both
  sampled, or one of them new there), collecting the pair's cells in every
  later period both still exist.  The ``-j`` model options reshape these
  maps (``ModelOptions``): parameters by period, ancestral sizes tied to the
  largest sampled descendant, one migration parameter, migration only
  between sampled populations or only between sisters, one rate for both
  directions, no migration.
* ``set_nomigrationchecklist`` (initialize.cpp:761-809): the migration cells
  those options forbid (a genealogy with a migration there has p(G) = 0).

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
class ModelOptions:
    """The ``-j`` model options that shape the parameter maps (imamp.hpp:
    356-381 names them; ima_main_mpi.cpp rejects the combinations marked)."""
    parameters_by_period: bool = False       # PARAMETERSBYPERIOD (not with the next)
    ancestral_sizes_largest_sampled: bool = False  # ANCESTRALPOPSIZESSETTOLARGESTSAMPLED
    one_migration_parameter: bool = False    # ONEMIGRATIONPARAMETER (not with both directions)
    migration_between_sampled: bool = False  # MIGRATIONBETWEENSAMPLED
    no_migration_between_nonsisters: bool = False  # NOMIGBETWEENNONSISTERS
    single_migration_both_directions: bool = False  # SINGLEMIGRATIONBOTHDIRECTIONS

    def check(self, nomig: bool):
        if self.parameters_by_period and self.ancestral_sizes_largest_sampled:
            raise ValueError("parameters by period and ancestral sizes set to the largest sampled conflict")
        if self.one_migration_parameter and (self.single_migration_both_directions or nomig):
            raise ValueError("one migration parameter conflicts with one rate for both directions and "
                             "with no migration")


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
    th_be: list = dataclasses.field(default_factory=list)   # per theta: (first, last) period (i_param b, e)
    mg_be: list = dataclasses.field(default_factory=list)   # per migration rate: (first, last) period
    chk_cells: list = dataclasses.field(default_factory=list)  # flat M cells that must hold no migration

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


MPRIORMIN = 0.000001    # imamp.hpp:137
EXPOMIGPLOTSCALE = 20   # imamp.hpp:156


def priors(pm: PopModel, thetaprior: float, mprior: float, expo: bool = False):
    """The parameters' prior bounds as setup_iparams and setimigarray set
    them without a prior file (initialize.cpp:156-198, :225-240): theta on
    (0, thetaprior]; migration on (0, max(mprior, MPRIORMIN)] with mean
    max/2, or, under the exponential prior, mean mprior and plot range
    EXPOMIGPLOTSCALE * mprior.  Returns th_max, th_min, mg_max, mg_min,
    mg_mean."""
    nth, nmg = len(pm.th_cells), len(pm.mg_cells)
    th_max, th_min = np.full(nth, float(thetaprior)), np.zeros(nth)
    if expo:
        mean = np.full(nmg, float(mprior))
        mx = EXPOMIGPLOTSCALE * mean
    else:
        mx = np.full(nmg, max(float(mprior), MPRIORMIN))
        mean = (mx - 0.0) / 2.0
    return th_max, th_min, mx, np.zeros(nmg), mean


def build(treestring: str, npops: int, nomig: bool = False, options: ModelOptions | None = None,
          varrank=None) -> PopModel:
    """The population tables of a tree string and the parameter maps of a
    model.  varrank: each sampled population's polymorphism score (the
    reference's set_uvals fills it from the data); only the option that ties
    ancestral sizes to the largest sampled descendant reads it."""
    if not 2 <= npops <= MAXPOPS:
        raise ValueError("npops must be in 2..%d" % MAXPOPS)
    opt = options or ModelOptions()
    opt.check(nomig)
    splits = parse_treestring(treestring, npops)
    ntp = 2 * npops - 1
    pop_b = np.zeros(ntp, np.int32)
    pop_e = np.full(ntp, -1, np.int32)
    pop_down = np.full(ntp, -1, np.int32)
    ups = {}
    for k, (a, b, anc) in enumerate(splits, start=1):
        pop_b[anc] = k
        # the reference reads the tree string after rewriting it so that a
        # leaf comes before a subtree, and the smaller number first
        # otherwise (rewrite, build_poptree.cpp:258-389): up[0] is the
        # smaller id
        ups[anc] = (min(a, b), max(a, b))
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
    tcell = lambda k, i: toff(npops, k) + i
    mcell = lambda k, i, j: moff(npops, k) + i * (npops - k) + j

    # population sizes (initialize.cpp:207-366)
    th_cells, th_names, th_be = [], [], []
    if opt.parameters_by_period:
        for k in range(npops):
            for i, p in enumerate(periods[k]):
                th_cells.append([tcell(k, i)])
                th_names.append("q%d,%d" % (k, p))
                th_be.append((int(pop_b[p]), int(pop_e[p])))
    else:
        rep = list(range(ntp))  # the sampled population whose size a population takes
        if opt.ancestral_sizes_largest_sampled:
            vr = np.zeros(npops) if varrank is None else np.asarray(varrank, np.float64)

            def fill(p):  # fillvarranktree: the descendant record with the larger score, ties to up[0]
                if p < npops:
                    return p
                a, b = (fill(d) for d in ups[p])
                rep[p] = b if vr[a] < vr[b] else a
                return rep[p]

            fill(ntp - 1)
        nparam = npops if opt.ancestral_sizes_largest_sampled else ntp
        for q in range(nparam):
            th_cells.append([tcell(k, i) for k in range(npops) for i, p in enumerate(periods[k])
                             if p == q or (opt.ancestral_sizes_largest_sampled and rep[p] == q)])
            th_names.append("q%d" % q)
            th_be.append((int(pop_b[q]), int(pop_e[q])))

    # migration rates (initialize.cpp:367-660)
    def sisters(k, i, j):  # checkaresis: the two merge at a later split
        pair = {periods[k][i], periods[k][j]}
        return any(set(droppops[kk].tolist()) == pair for kk in range(k + 1, npops))

    def first_meeting(k, i, j):
        if k == 0:
            return True
        if opt.migration_between_sampled:
            return False
        pi, pj = periods[k][i], periods[k][j]
        return opt.parameters_by_period or pi not in periods[k - 1] or pj not in periods[k - 1]

    def later(k, i, j):  # the pair's positions in the later periods both still exist in
        pi, pj = periods[k][i], periods[k][j]
        kk = k + 1
        while kk < npops - 1 and pi in periods[kk] and pj in periods[kk]:
            yield kk, periods[kk].index(pi), periods[kk].index(pj)
            kk += 1

    mg_cells, mg_names, mg_be = [], [], []
    pad = []
    if not nomig:
        if opt.one_migration_parameter:
            mg_cells.append([])
            mg_names.append("m_all")
            mg_be.append((0, npops - 2))
        for k in range(npops - 1):
            for i in range(npops - k - 1):
                for j in range(i + 1, npops - k):
                    if not first_meeting(k, i, j):
                        continue
                    if opt.no_migration_between_nonsisters and not sisters(k, i, j):
                        continue
                    pi, pj = periods[k][i], periods[k][j]
                    cont = [] if opt.parameters_by_period else list(later(k, i, j))
                    last = cont[-1][0] if cont else k
                    both = opt.single_migration_both_directions
                    fwd = [mcell(k, i, j)] + ([mcell(k, j, i)] if both else [])
                    for kk, a, b in cont:
                        fwd += [mcell(kk, a, b)] + ([mcell(kk, b, a)] if both else [])
                    back = [] if both else [mcell(k, j, i)] + [mcell(kk, b, a) for kk, a, b in cont]
                    if opt.one_migration_parameter:
                        mg_cells[0] += fwd + back
                        if opt.parameters_by_period:
                            # the reference sizes this list counting the
                            # pair's later periods (its by-period test is
                            # skipped for one parameter) but fills only the
                            # first: the unfilled entries stay as malloc left
                            # them, which the harness reads as cell (0, 0, 0),
                            # a diagonal cell that holds no migration
                            nlater = len(list(later(k, i, j)))
                            pad.extend([mcell(0, 0, 0)] * (2 * nlater))
                        continue
                    arrow = "<>" if both else ">"
                    if opt.parameters_by_period:
                        mg_names.append("m%d,%d%s%d" % (k, pi, arrow, pj))
                    else:
                        mg_names.append("m%d%s%d" % (pi, arrow, pj))
                    mg_cells.append(fwd)
                    mg_be.append((k, last))
                    if not both:
                        mg_names.append("m%d,%d>%d" % (k, pj, pi) if opt.parameters_by_period
                                        else "m%d>%d" % (pj, pi))
                        mg_cells.append(back)
                        mg_be.append((k, last))

    if pad:
        mg_cells[0] += pad

    # cells the options forbid (initialize.cpp:761-809)
    chk = []
    for k in range(npops - 1):
        for i in range(npops - k - 1):
            for j in range(i + 1, npops - k):
                pi, pj = periods[k][i], periods[k][j]
                if (opt.migration_between_sampled and (pi >= npops or pj >= npops)) or \
                        (opt.no_migration_between_nonsisters and not sisters(k, i, j)):
                    chk += [mcell(k, i, j), mcell(k, j, i)]
    return PopModel(npops, plist, droppops, addpop, pop_e, pop_down, bool(nomig),
                    th_cells, mg_cells, th_names, mg_names, th_be, mg_be, chk)


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
