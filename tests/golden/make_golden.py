"""Generate the golden fixtures in this directory by running the UNMODIFIED
IMa2p reference (oracle/_ref/imaref, built by ``make -C oracle ref`` from the
reference source tree) on seeded inputs.

Run from the repository root:  python tests/golden/make_golden.py

Fixtures:
  golden_is.npz     likelihoodIS + calc_sumlogk on synthetic 2-population loci
                    and on loci of the reference's own Simulations/*.u files
                    (genealogies built as perfect phylogenies of their IS data)
  golden_hky.npz    likelihoodHKY full and dirty-node evaluations with
                    copyfraclike/storescalefactors/restorescalefactors
  golden_sw.npz     likelihoodSW totals and per-branch dlikeA, incl. zero-
                    probability branches and x > 700
  golden_swap.npz   setheat + swapchains (MT19937 seeded), betas and counts
  golden_jointp.npz jointp (truncated, eexp) values and ESS
  golden_de.npz     modelloop (the L-mode differential-evolution peak search,
                    MT19937 seeded) for the full model, theta-only and
                    migration-only model types and a nested model
  golden_margin.npz margincalc (1-D marginal densities) on fillvec's grids,
                    plain and log'd with yadjust, uniform and exponential
                    migration priors
  golden_tw.npz     treeweight (genealogy weights), sum_treeinfo and
                    initialize_integrate_tree_prob (p(G) integrals) on
                    population-labelled IM genealogies for 2-5 population
                    trees, with the reference's own parameter maps
                    (setup_iparams), and the integral terms on edge cases
  golden_ry.npz     the split-time update changet_RY1 (MT19937 seeded) on
                    three chains of four infinite-sites loci, 3 populations
                    with migration: decisions, split times, probg and pdg
                    per step, final node and migration times
  golden_ks.npz     long runs of the same update on chain 0 for six seeds:
                    thinned split times of both periods (the statistical
                    comparison of the device-resident sampler)

  golden_popmig.npz calc_popmig and calc_pop_expomig (2NM densities) over
                    gsampinf rows that reach every branch of the terms
                    (no coalescences, no migrations, neither), posterior
                    and likelihood forms, and a 2NM curve grid

  golden_peaks.npz  findmarginpeaks' numbers (marginalopt peaks over both
                    halves and all genealogies, migration tests, margin95
                    limits, marginalopt_popmig peaks and tests) on the
                    popmig rows and on rows whose peaks lie inside the
                    priors, uniform and exponential migration priors

Run with fixture names (is hky sw swap jointp de margin tw ry ks popmig peaks) to regenerate only those.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from ima2p_gb300 import synth  # noqa: E402
from oracle import pyoracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
SIMDIR = os.path.join(O.REFERENCE, "Simulations")


def pack_trees(trees):
    return dict(up0=np.stack([t.up0 for t in trees]), up1=np.stack([t.up1 for t in trees]),
                down=np.stack([t.down for t in trees]), time=np.stack([t.time for t in trees]),
                root=np.array([t.root for t in trees], np.int32))


# ------------------------------------------------------- .u IS loci
def read_u_is_loci(path):
    """Infinite-sites loci of a .u file as 0/1 matrices (readata.cpp:34-495:
    sites with exactly two ACGT states, coded against the first sequence)."""
    lines = [ln.rstrip("\n") for ln in open(path)]
    i = 1
    while lines[i].startswith("#"):
        i += 1
    i += 3  # npops, names, tree
    nloci = int(lines[i].split()[0])
    i += 1
    loci = []
    for _ in range(nloci):
        hdr = lines[i].split()
        n = int(hdr[1]) + int(hdr[2])
        nb = int(hdr[3])
        rows = [lines[i + 1 + k][10:].replace(" ", "")[:nb].lower() for k in range(n)]
        i += 1 + n
        cols = []
        for s in range(nb):
            col = [r[s] for r in rows]
            if any(c not in "acgt" for c in col):
                continue
            states = sorted(set(col))
            if len(states) != 2:
                continue
            cols.append([0 if c == col[0] else 1 for c in col])
        if cols:
            loci.append(np.array(cols, np.int8).T.copy())
    return loci


def perfect_phylogeny(rng, seq):
    """A binary genealogy on which every 0/1 column is a single mutation;
    polytomies are resolved at random, times are drawn to respect the nesting."""
    n = seq.shape[0]
    # columns are coded against the first sequence, so rooting on its side
    # makes every derived set a clade (four-gamete compatible data)
    splits = {frozenset(np.nonzero(c)[0]) for c in seq.T}
    full = frozenset(range(n))
    clades = sorted({s for s in splits if 1 < len(s) < n} | {full}, key=len)
    # every clade's children: maximal proper sub-clades plus leftover tips
    nl = 2 * n - 1
    up0 = np.full(nl, -1, np.int32)
    up1 = np.full(nl, -1, np.int32)
    down = np.full(nl, -1, np.int32)
    height = np.zeros(nl)
    node_of = {frozenset([t]): t for t in range(n)}
    nxt = [n]

    def join(a, b, h):
        k = nxt[0]
        nxt[0] += 1
        up0[k], up1[k] = a, b
        down[a] = down[b] = k
        height[k] = h
        return k

    for c in clades:
        subs = [s for s in node_of if s < c and len(s) < len(c)]
        maximal = [s for s in subs if not any(s < t for t in subs)]
        parts = [node_of[s] for s in maximal]
        covered = frozenset().union(*maximal) if maximal else frozenset()
        parts += [t for t in c if t not in covered]
        base = max(height[p] for p in parts)
        while len(parts) > 1:
            i, j = rng.choice(len(parts), 2, replace=False)
            base += rng.exponential(0.2)
            k = join(parts[i], parts[j], base)
            parts = [p for q, p in enumerate(parts) if q not in (i, j)] + [k]
        node_of[c] = parts[0]
        for s in maximal:
            del node_of[s]
        for t in c:
            node_of.pop(frozenset([t]), None)
    root = node_of[full]
    time = np.zeros(nl)
    for c in range(nl):
        time[c] = height[down[c]] if down[c] >= 0 else -1.0
    return synth.Genealogy(up0, up1, down, time, int(root))


def golden_is():
    rng = np.random.default_rng(1001)
    out = {}
    cases = []
    for k in range(3):
        g0 = synth.two_pop_tree(rng, 10, 10, theta=5.0, mig=0.1, tsplit=1.0)
        seq = synth.is_data(rng, g0, 1.0, min_sites=5)
        trees = [g0] + [synth.jitter_times(rng, g0, 0.2) for _ in range(4)]
        trees.append(synth.two_pop_tree(rng, 10, 10))  # mostly incompatible
        cases.append(("syn%d" % k, seq, trees))
    for fname in ("Sim1_5loci.u", "Sim2.u"):
        path = os.path.join(SIMDIR, fname)
        for li, seq in enumerate(read_u_is_loci(path)[:3]):
            g0 = perfect_phylogeny(rng, seq)
            trees = [g0] + [synth.jitter_times(rng, g0, 0.2) for _ in range(2)]
            cases.append(("%s_L%d" % (fname.split(".")[0], li), seq, trees))
    for ci, (name, seq, trees) in enumerate(cases):
        lengths = np.array([t.length() for t in trees])
        us = rng.lognormal(0.0, 0.5, len(trees))
        ref = O.ref_is(seq, trees, lengths, us)
        p = "c%d_" % ci
        out[p + "name"] = np.array(name)
        out[p + "seq"] = seq
        for k, v in pack_trees(trees).items():
            out[p + k] = v
        out[p + "length"] = lengths
        out[p + "u"] = us
        out[p + "ref"] = ref
    out["ncases"] = np.array(len(cases))
    np.savez_compressed(os.path.join(OUT, "golden_is.npz"), **out)


def time_edit(rng, g, k):
    """Move the coalescence that creates internal node k inside its window."""
    h = g.copy()
    a, b = int(h.up0[k]), int(h.up1[k])
    lo = max(h.time[h.up0[a]] if h.up0[a] >= 0 else 0.0, h.time[h.up0[b]] if h.up0[b] >= 0 else 0.0)
    hi = h.time[k] if h.down[k] >= 0 else h.time[a] * 1.5
    h.time[a] = h.time[b] = lo + (hi - lo) * rng.uniform(0.05, 0.95)
    return h


def tip_swap(rng, g):
    """Exchange two tips that hang from different parents (a topology edit)."""
    h = g.copy()
    n = h.n
    while True:
        i, j = rng.choice(n, 2, replace=False)
        if h.down[i] != h.down[j]:
            break
    pi, pj = int(h.down[i]), int(h.down[j])
    for p, old, new in ((pi, i, j), (pj, j, i)):
        if h.up0[p] == old:
            h.up0[p] = new
        else:
            h.up1[p] = new
    h.down[i], h.down[j] = pj, pi
    h.time[i], h.time[j] = h.time[j], h.time[i]
    return h, int(i), int(j)


def golden_hky():
    rng = np.random.default_rng(1002)
    out = {}
    cases = []
    for k, (n1, nb) in enumerate(((6, 300), (10, 1000), (20, 1000))):
        g = synth.two_pop_tree(rng, n1, n1, theta=10.0, mig=0.2, tsplit=1.5)
        pi_sim = rng.dirichlet([5, 5, 5, 5])
        kappa = rng.uniform(2, 8)
        u = float(rng.lognormal(0, 0.5))
        loc = synth.hky_data(rng, g, nb, u, kappa, pi_sim)
        n = g.n
        seqs = []  # (tree, e, accept)
        cur = g
        for step in range(6):
            if step % 3 == 2:
                h, i, j = tip_swap(rng, cur)
                e = (i, j, -1, -1)
            else:
                kk = int(rng.integers(n, 2 * n - 1))
                h = time_edit(rng, cur, kk)
                e = (kk, -1, -1, -1)
            acc = int(rng.uniform() < 0.5)
            seqs.append((h, e, acc))
            if acc:
                cur = h
        cases.append((loc, g, u, kappa, seqs))
    for ci, (loc, g, u, kappa, seqs) in enumerate(cases):
        ref = O.ref_hky(loc, [(g, u, kappa, seqs)])
        p = "c%d_" % ci
        out[p + "seq"] = loc.seq
        out[p + "mult"] = loc.mult
        out[p + "totsites"] = np.array(loc.totsites)
        out[p + "pi"] = loc.pi
        for kk, v in pack_trees([g] + [s[0] for s in seqs]).items():
            out[p + kk] = v
        out[p + "e"] = np.array([s[1] for s in seqs], np.int32)
        out[p + "acc"] = np.array([s[2] for s in seqs], np.int32)
        out[p + "u"] = np.array(u)
        out[p + "kappa"] = np.array(kappa)
        out[p + "ref"] = ref
    out["ncases"] = np.array(len(cases))
    np.savez_compressed(os.path.join(OUT, "golden_hky.npz"), **out)


def golden_sw():
    rng = np.random.default_rng(1003)
    g = synth.three_pop_tree(rng, [10, 10, 10], theta=4.0, mig=0.05)
    trees, alleles, us = [], [], []
    for k in range(8):
        h = synth.jitter_times(rng, g, 0.3)
        A = synth.sw_alleles(rng, h, float(rng.lognormal(0, 0.5)))
        if k == 5:  # a large jump across a short branch -> Miller recurrence
            A = A.copy()
            A[h.up0[h.root]] += 7
        if k == 6:  # zero-length branch with an allele change -> I_d(0) = 0
            A = A.copy()
            h = h.copy()
            c = int(h.up0[h.root])
            if h.up0[c] >= 0:
                h.time[h.up0[c]] = h.time[h.up1[c]] = h.time[c]
                A[c] = A[h.root] + 2
        trees.append(h)
        alleles.append(A)
        us.append(float(rng.lognormal(0, 0.5)) if k != 7 else 40.0)  # x > 700
    ref = O.ref_sw(trees, alleles, us)
    out = pack_trees(trees)
    out["A"] = np.stack(alleles)
    out["u"] = np.array(us)
    out["ref"] = ref
    np.savez_compressed(os.path.join(OUT, "golden_sw.npz"), **out)


def golden_swap():
    rng = np.random.default_rng(1004)
    out = {}
    cases = [(4, 5, 1, 200, 1, 0.9, 0.8, 0), (20, 10, 2, 200, 1, 0.96, 0.9, 7),
             (24, 3, 3, 100, 0, 0.05, 0.0, 11), (128, 6, 12, 60, 1, 0.95, 0.8, 5)]
    for ci, (nch, nl, tries, steps, mode, h1, h2, seed) in enumerate(cases):
        pdg = rng.normal(-100, 3, (nch, nl))
        probg = rng.normal(-30, 2, nch)
        ok, betas, sc, tc = O.ref_swap(pdg, probg, tries, steps, mode, h1, h2, seed)
        p = "c%d_" % ci
        out[p + "params"] = np.array([nch, nl, tries, steps, mode, seed])
        out[p + "h"] = np.array([h1, h2])
        out[p + "pdg"] = pdg
        out[p + "probg"] = probg
        out[p + "ok"] = ok
        out[p + "betas"] = betas
        out[p + "swapcount"] = sc
        out[p + "tempcount"] = tc
    out["ncases"] = np.array(len(cases))
    np.savez_compressed(os.path.join(OUT, "golden_swap.npz"), **out)


def golden_jointp():
    rng = np.random.default_rng(1005)
    out = {}
    # 2 populations (3 theta, 2 m), row width 21 as in a real .ti
    off = synth.gsamp_layout(3, 2, 1)
    G = 400
    rows = np.zeros((G, off["rowlen"]), np.float32)
    rows[:, 0:3] = rng.poisson(4, (G, 3))
    rows[:, 3:6] = rng.gamma(3, 1, (G, 3))
    rows[:, 6:9] = rng.normal(0, 1, (G, 3))
    rows[:, 9:11] = rng.poisson(1, (G, 2))
    rows[:, 11:13] = rng.gamma(2, 1, (G, 2))
    rows[:, off["probg"]] = rng.normal(15, 6, G)
    pts = np.concatenate([rng.uniform(0.1, 10, (12, 3)), rng.uniform(1e-3, 2, (12, 2))], 1)
    out["a_rows"] = rows
    out["a_pts"] = pts
    out["a_ref"] = O.ref_jointp(rows, 3, 2, 2, 0, pts)
    # 3 populations (5 theta, 8 m): theta-only and migration-only model types
    rows5, _, off5 = synth.surface_stats(rng, 300, 5, 8, 2)
    rows5[:, off5["qi"]:off5["qi"] + 5] = rng.normal(-4, 1, (300, 5))
    rows5[:, off5["mi"]:off5["mi"] + 8] = rng.normal(-2, 1, (300, 8))
    pts5 = synth.surface_points(rng, 8)
    out["b_rows"] = rows5
    out["b_pts"] = pts5
    out["b_ref1"] = O.ref_jointp(rows5, 5, 8, 3, 1, pts5)
    out["b_ref2"] = O.ref_jointp(rows5, 5, 8, 3, 2, pts5)
    np.savez_compressed(os.path.join(OUT, "golden_jointp.npz"), **out)


def de_rows(rng, G, np_, nm):
    """gsampinf rows close to one another, so the posterior spreads over many
    genealogies (a peak with an effective sample size in the hundreds)."""
    rows, _, off = synth.surface_stats(rng, G, np_, nm, 1)
    rows[:] = rows[0]
    rows[:, off["fc"]:off["fc"] + np_] *= (1 + 0.05 * rng.standard_normal((G, np_))).astype(np.float32)
    rows[:, off["fm"]:off["fm"] + nm] *= (1 + 0.05 * rng.standard_normal((G, nm))).astype(np.float32)
    rows[:, off["probg"]] = (200 + rng.normal(0, 0.5, G)).astype(np.float32)
    rows[:, off["qi"]:off["qi"] + np_] += rng.normal(0, 0.3, (G, np_)).astype(np.float32)
    rows[:, off["mi"]:off["mi"] + nm] += rng.normal(0, 0.3, (G, nm)).astype(np.float32)
    return rows


def golden_de():
    rng = np.random.default_rng(1006)
    rows = de_rows(rng, 400, 3, 2)
    upper = np.array([20.0, 20.0, 20.0, 2.0, 2.0])
    # (name, npops, modeltype, seed, xmap, nested); DE population 30 x params
    cases = [("full", 2, 0, 77, None, 0), ("theta", 3, 1, 78, None, 0), ("mig", 3, 2, 79, None, 0),
             ("nested", 2, 0, 80, [0.0, 0.0, 1.0, 2.0, -1e-7], 3)]
    out = {"rows": rows, "upper": upper, "multiplier": np.array(30)}
    for name, npops, mt, seed, xmap, nested in cases:
        best, ess = O.ref_de(rows, 3, 2, npops, upper, mt, 30, seed, xmap=xmap, nested=nested)
        out[name + "_case"] = np.array([npops, mt, seed, nested])
        out[name + "_xmap"] = np.array(xmap if xmap else [0.0] * 5)
        out[name + "_best"] = best
        out[name + "_ess"] = np.array(ess)
    np.savez_compressed(os.path.join(OUT, "golden_de.npz"), **out)


def golden_margin():
    rng = np.random.default_rng(1007)
    rows, _, off = synth.surface_stats(rng, 300, 3, 2, 1)
    pmax = np.array([20.0, 15.0, 25.0, 2.0, 5.0])
    grid = 40  # points per parameter on fillvec's grid (GRIDSIZE is 1000 in the reference)
    pts = []
    for p in range(5):
        for j in range(grid):
            pts.append((p, ((j + 0.5) * pmax[p]) / grid, 0, 0.0))
    for p in range(5):  # log'd with a y adjustment, as margin95's root search calls it
        for x in (0.05, 1.0, 4.0):
            pts.append((p, x, 1, 1.92))
    out = {"rows": rows, "pmax": pmax, "grid": np.array(grid), "points": np.array(pts)}
    out["ref"] = O.ref_margincalc(rows, 3, 2, pts)
    out["expo_mean"] = np.array([0.8, 1.7])
    out["ref_expo"] = O.ref_margincalc(rows, 3, 2, pts, expo_mean=out["expo_mean"])
    np.savez_compressed(os.path.join(OUT, "golden_margin.npz"), **out)


TW_CASES = [
    # (npops, tree string, chains, loci, migration rate, expo prior, no migration)
    (2, "(0,1):2", 4, 5, 0.5, False, False),
    (3, "((0,1):3,2):4", 4, 6, 0.3, True, False),
    (4, "((0,1):4,(2,3):5):6", 3, 4, 0.3, False, False),
    (3, "((0,2):3,1):4", 3, 4, 0.0, False, True),
    (5, "(((0,1):5,2):6,(3,4):7):8", 2, 3, 0.2, False, False),
]


def tw_case(rng, npops, ts, nch, nl, mrate, expo, nomig):
    from ima2p_gb300 import popmodel
    sp = popmodel.parse_treestring(ts, npops)
    loci = []
    for li in range(nl):
        samp = [int(v) for v in rng.integers(2, 13, npops)]
        loci.append((int(sum(samp)), float([1.0, 0.25, 0.75, 1.0][li % 4]), samp))
    # one chain has splits older than most roots, the others younger
    tvals = [np.sort(rng.uniform(0.2, 1.5 if ci else 6.0, npops - 1)) for ci in range(nch)]
    gens = []
    for ci in range(nch):
        row = []
        for ng, h, samp in loci:
            splits = [(tvals[ci][k], a, b, anc) for k, (a, b, anc) in enumerate(sp)]
            theta = list(rng.uniform(1.0, 6.0, 2 * npops - 1))
            row.append(synth.sim_im_labeled(rng, samp, theta, mrate, splits))
        gens.append(row)
    return loci, tvals, gens


def golden_tw():
    rng = np.random.default_rng(1010)
    out = {}
    for c, (npops, ts, nch, nl, mrate, expo, nomig) in enumerate(TW_CASES):
        loci, tvals, gens = tw_case(rng, npops, ts, nch, nl, mrate, expo, nomig)
        thetaprior, mprior = 12.0, 1.5
        r = O.ref_tw(npops, ts, loci, tvals, gens, thetaprior, mprior, expo=expo, nomig=nomig)
        k = "c%d_" % c
        out[k + "meta"] = np.array([npops, nch, nl, int(expo), int(nomig)])
        out[k + "tree"] = np.array(ts)
        out[k + "priors"] = np.array([thetaprior, mprior])
        out[k + "loci"] = np.array([[ng, h] + samp for ng, h, samp in loci], np.float64)
        out[k + "tvals"] = np.array(tvals)
        flat = [gens[ci][li] for ci in range(nch) for li in range(nl)]
        out[k + "node_off"] = np.concatenate([[0], np.cumsum([len(g.pop) for g in flat])]).astype(np.int32)
        for f in ("up0", "up1", "down", "time"):
            out[k + f] = np.concatenate([getattr(g.g, f) for g in flat])
        out[k + "pop"] = np.concatenate([g.pop for g in flat]).astype(np.int32)
        counts = [len(m) for g in flat for m in g.mig]
        out[k + "mig_off"] = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        out[k + "mig_t"] = np.array([e[0] for g in flat for m in g.mig for e in m], np.float64)
        out[k + "mig_p"] = np.array([e[1] for g in flat for m in g.mig for e in m], np.int32)
        gw = [r["gw"][(ci, li)] for ci in range(nch) for li in range(nl)]
        for f in ("cc", "hcc", "fc", "mc", "fm"):
            out[k + f] = np.array([w[f] for w in gw])
        out[k + "scal"] = np.array([[w["mignum"], w["length"], w["tlength"]] for w in gw])
        out[k + "pg"] = np.array([r["pg"][ci] for ci in range(nch)])
        out[k + "th_wp"] = np.array([len(wp) for wp, _, _ in r["theta"]] + [v for wp, _, _ in r["theta"] for pr in wp for v in pr], np.int32)
        out[k + "mg_wp"] = np.array([len(wp) for wp, _, _, _ in r["mig"]] + [v for wp, _, _, _ in r["mig"] for pr in wp for v in pr], np.int32)
        out[k + "th_pr"] = np.array([[mx, mn] for _, mx, mn in r["theta"]])
        out[k + "mg_pr"] = np.array([[mx, mn, mean] for _, mx, mn, mean in r["mig"]]).reshape(-1, 3)
    out["ncases"] = np.array(len(TW_CASES))
    lines, errs = [], []
    for cc in (0, 1, 2, 3, 7, 30, 150, 900):
        for fc in (1e-3, 0.05, 0.7, 3.0, 40.0, 900.0, 2e4):
            for mx, mn in ((10.0, 0.0), (50.0, 0.0), (10.0, 0.5), (3.0, 1.0)):
                h = float(rng.choice([0.0, -0.6931471805599453, 1.3]) * cc)
                (errs if O.iterm(0, cc, fc, h, mx, mn)[1] else lines).append((0, cc, fc, h, mx, mn))
    for cm in (0, 1, 2, 5, 40, 300):
        for fm in (1e-7, 1e-3, 0.3, 2.0, 25.0, 400.0):
            for mx, mn in ((2.0, 0.0), (10.0, 0.0), (0.000001, 0.0), (5.0, 0.2)):
                if cm > 0 and mx == 0.000001:
                    continue
                (errs if O.iterm(1, cm, fm, 0.0, mx, mn)[1] else lines).append((1, cm, fm, 0.0, mx, mn))
            lines.append((2, cm, fm, 0.0, 1.7, 0.0))
    out["iterm_lines"] = np.array(lines)
    out["iterm_ref"] = O.ref_iterm(lines)
    stopped = []
    for l in errs:  # the reference stops (IM_err) on each of these
        try:
            O.ref_iterm([l])
        except Exception:
            stopped.append(l)
    assert len(stopped) == len(errs)
    out["iterm_stop"] = np.array(errs)
    np.savez_compressed(os.path.join(OUT, "golden_tw.npz"), **out)


def golden_ry():
    from ima2p_gb300 import popmodel
    rng = np.random.default_rng(1011)
    npops, ts = 3, "((0,1):3,2):4"
    sp = popmodel.parse_treestring(ts, npops)
    nl, nch, tv0 = 4, 3, [0.45, 1.1]
    samps = [[int(v) for v in rng.integers(3, 7, npops)] for _ in range(nl)]
    splits = [(tv0[k], a, b, anc) for k, (a, b, anc) in enumerate(sp)]
    base = [synth.sim_im_labeled(rng, samps[li], list(rng.uniform(1.0, 3.0, 5)), 0.5, splits) for li in range(nl)]
    seqs = [synth.is_data(rng, base[li].g, 1.0, min_sites=4) for li in range(nl)]
    us = [0.8, 1.0, 1.2, 1.0]
    loci = [(sum(samps[li]), 1.0, samps[li], us[li], seqs[li]) for li in range(nl)]
    gens = [[base[li] for li in range(nl)] for _ in range(nch)]
    betas = [1.0, 0.7, 0.45]
    tprior = [(0.0, 3.0), (0.0, 5.0)]
    steps = [(s % nch, int(rng.integers(0, npops - 1))) for s in range(90)]
    res, times, migt = O.ref_ry(npops, ts, tprior, loci, [(tv0, b) for b in betas], gens, steps, 4321, 10.0, 1.0)
    out = {"npops": np.array(npops), "tree": np.array(ts), "tv0": np.array(tv0), "betas": np.array(betas),
           "tprior": np.array(tprior), "steps": np.array(steps), "seed": np.array(4321),
           "priors": np.array([10.0, 1.0]), "samps": np.array(samps), "us": np.array(us),
           "seq_off": np.concatenate([[0], np.cumsum([q.size for q in seqs])]),
           "seq_shape": np.array([q.shape for q in seqs]), "seqs": np.concatenate([q.ravel() for q in seqs]),
           "res": np.array(res)}
    packed_base = [b for b in base]
    out["node_off"] = np.concatenate([[0], np.cumsum([len(g.pop) for g in packed_base])]).astype(np.int32)
    for f in ("up0", "up1", "down", "time"):
        out[f] = np.concatenate([getattr(g.g, f) for g in packed_base])
    out["pop"] = np.concatenate([g.pop for g in packed_base]).astype(np.int32)
    out["mig_off"] = np.concatenate([[0], np.cumsum([len(m) for g in packed_base for m in g.mig])]).astype(np.int32)
    out["mig_t"] = np.array([e[0] for g in packed_base for m in g.mig for e in m])
    out["mig_p"] = np.array([e[1] for g in packed_base for m in g.mig for e in m], np.int32)
    out["times"] = np.concatenate([times[(ci, li)] for ci in range(nch) for li in range(nl)])
    out["migt"] = np.concatenate([migt[(ci, li)] for ci in range(nch) for li in range(nl)])
    np.savez_compressed(os.path.join(OUT, "golden_ry.npz"), **out)


def popmig_rows():
    """gsampinf rows (3 population sizes, 2 migration rates) with every
    branch of calc_popmig's term present: cc = fc = 0 (rows 0-19, theta 0),
    mc = fm = 0 (rows 20-39, migration 0), all four zero (rows 40-49, theta
    1 / migration 1)."""
    rng = np.random.default_rng(2024)
    rows, _, off = synth.surface_stats(rng, 200, 3, 2, 1)
    rows[0:20, off["cc"] + 0] = 0
    rows[0:20, off["fc"] + 0] = 0
    rows[20:40, off["mc"] + 0] = 0
    rows[20:40, off["fm"] + 0] = 0
    for c in ("cc", "fc"):
        rows[40:50, off[c] + 1] = 0
    for c in ("mc", "fm"):
        rows[40:50, off[c] + 1] = 0
    return rows


# long runs of the split-time update for the statistical comparison
KS_SEEDS, KS_STEPS, KS_THIN = (101, 102, 103, 104, 105, 106), 4000, 10


def golden_ks():
    """The reference's changet_RY1 run for KS_STEPS updates on chain 0 of the
    golden_ry case (periods alternating), for each of KS_SEEDS: every
    KS_THIN-th split time of each period after its update."""
    sys.path.insert(0, ROOT)
    from tests._splittime import RyCase
    c = RyCase()
    loci = [(int(c.samps[li].sum()), 1.0, [int(v) for v in c.samps[li]], float(c.us[li]), c.seqs[li])
            for li in range(c.nl)]
    tv0 = [float(v) for v in c.d["tv0"]]
    out = {"seeds": np.array(KS_SEEDS), "steps": np.array(KS_STEPS), "thin": np.array(KS_THIN)}
    for seed in KS_SEEDS:
        steps = [(0, k % 2) for k in range(KS_STEPS)]
        res, _, _ = O.ref_ry(c.npops, c.tree, c.tprior, loci, [(tv0, b) for b in c.betas], c.fresh_gens(), steps,
                             seed, c.thetaprior, c.mprior)
        tv = np.array([r[1] for r in res])
        for k in range(2):
            out["t%d_%d" % (k, seed)] = tv[k::2][::KS_THIN]
        out["acc_%d" % seed] = np.array([r[0] for r in res], np.int8)
    np.savez_compressed(os.path.join(OUT, "golden_ks.npz"), **out)


def golden_popmig():
    rows = popmig_rows()
    qmax, mmax, mean = np.array([20.0, 15.0, 25.0]), np.array([2.0, 5.0]), np.array([0.8, 1.7])
    pts = [(t, m, x, pl) for (t, m) in ((0, 0), (1, 1), (0, 1), (2, 0))
           for x in (0.01, 0.05, 0.7, 3.0, 9.0, 14.9, 40.0) for pl in (0, 1)]
    # a curve: the 2NM grid of term (1, 1) at 50 points on (0, qmax mmax / 2]
    grid = 50
    pmmax = qmax[1] * mmax[1] / 2.0
    pts += [(1, 1, (j + 0.5) * pmmax / grid, 0) for j in range(grid)]
    out = {"rows": rows, "qmax": qmax, "mmax": mmax, "mean": mean, "points": np.array(pts), "grid": np.array(grid)}
    out["ref"] = O.ref_popmig(rows, 3, 2, qmax, mmax, pts)
    out["ref_expo"] = O.ref_popmig(rows, 3, 2, qmax, mmax, pts, mmean=mean)
    np.savez_compressed(os.path.join(OUT, "golden_popmig.npz"), **out)


def interior_rows(G=2000, seed=2025):
    """gsampinf rows (3 population sizes, 2 migration rates) whose marginal
    peaks lie inside the priors: cc ~ Poisson(15) with fc / cc ~ U(1, 5)
    (theta peaks 2-10 of 20), mc ~ Poisson(4) with mc / fm ~ U(0.3, 2)
    (migration peaks inside 2 and 5), integrals ~ N(0, 1)."""
    rng = np.random.default_rng(seed)
    off = synth.gsamp_layout(3, 2, 1)
    rows = np.zeros((G, off["rowlen"]), np.float32)
    cc = rng.poisson(15.0, (G, 3))
    rows[:, off["cc"]:off["cc"] + 3] = cc
    rows[:, off["fc"]:off["fc"] + 3] = cc * rng.uniform(1.0, 5.0, (G, 3))
    mc = rng.poisson(4.0, (G, 2))
    rows[:, off["mc"]:off["mc"] + 2] = mc
    rows[:, off["fm"]:off["fm"] + 2] = np.maximum(mc, 0.5) / rng.uniform(0.3, 2.0, (G, 2))
    rows[:, off["qi"]:off["qi"] + 3] = rng.normal(0.0, 1.0, (G, 3))
    rows[:, off["mi"]:off["mi"] + 2] = rng.normal(0.0, 1.0, (G, 2))
    rows[:, off["t"]] = rng.uniform(0.1, 3.0, G)
    return rows


def golden_peaks():
    qmax, mmax, mean = np.array([20.0, 15.0, 25.0]), np.array([2.0, 5.0]), np.array([0.8, 1.7])
    terms = [(0, 0), (1, 1)]
    out = {"qmax": qmax, "mmax": mmax, "mean": mean, "terms": np.array(terms)}
    for name, rows in (("branch", popmig_rows()), ("interior", interior_rows())):
        out[name + "_rows"] = rows
        for tag, m in (("", None), ("_expo", mean)):
            r = O.ref_findmarginpeaks(rows, 3, 2, np.zeros(3), qmax, np.zeros(2), mmax, mg_mean=m, terms=terms)
            for k, v in r.items():
                out["%s%s_%s" % (name, tag, k)] = v
    np.savez_compressed(os.path.join(OUT, "golden_peaks.npz"), **out)


IPARAM_TREES = [
    (2, "(0,1):2"),
    (3, "((0,1):3,2):4"),
    (3, "((0,2):3,1):4"),
    (3, "(0,(1,2):3):4"),
    (4, "((0,1):4,(2,3):5):6"),
    (4, "(((0,1):4,2):5,3):6"),
    (4, "((0,(1,2):4):5,3):6"),
    (5, "(((0,1):5,2):6,(3,4):7):8"),
    (5, "((0,1):5,((2,3):6,4):7):8"),
]
IPARAM_OPTIONS = [
    (), ("parameters_by_period",), ("ancestral_sizes_largest_sampled",), ("one_migration_parameter",),
    ("migration_between_sampled",), ("no_migration_between_nonsisters",), ("single_migration_both_directions",),
    ("no_migration",), ("expo_migration_prior",),
    ("parameters_by_period", "single_migration_both_directions"),
    ("parameters_by_period", "one_migration_parameter"),
    ("parameters_by_period", "migration_between_sampled"),
    ("parameters_by_period", "no_migration_between_nonsisters"),
    ("ancestral_sizes_largest_sampled", "no_migration_between_nonsisters"),
    ("one_migration_parameter", "no_migration_between_nonsisters"),
    ("one_migration_parameter", "migration_between_sampled"),
    ("migration_between_sampled", "single_migration_both_directions"),
    ("no_migration_between_nonsisters", "single_migration_both_directions", "expo_migration_prior"),
    ("ancestral_sizes_largest_sampled", "no_migration"),
]


def golden_iparams():
    """The reference's parameter maps and no-migration checklist for every
    tree of IPARAM_TREES under every option set of IPARAM_OPTIONS (with
    seeded polymorphism scores for the ancestral-size option, ties
    included)."""
    rng = np.random.default_rng(1012)
    cases = []
    for npops, ts in IPARAM_TREES:
        for flags in IPARAM_OPTIONS:
            vr = rng.integers(0, 4, size=npops).astype(float)  # small integers: ties occur
            r = O.ref_iparams(npops, ts, flags, 10.0, 5.0, vr)
            cases.append({"npops": npops, "tree": ts, "flags": list(flags), "varrank": vr.tolist(), "ref": r})
    import json
    np.savez_compressed(os.path.join(OUT, "golden_iparams.npz"), cases=np.array(json.dumps(cases)))


def _golden_ug(name, kinds, seed, us):
    """The reference's genealogy update updategenealogy under the
    no-migration model: 3 chains x the given loci, 10 sweeps per chain from
    seeds of their own; every proposal's decision, G.pdg and p(G), and the
    final genealogies (with the SW loci's alleles)."""
    from ima2p_gb300 import popmodel
    rng = np.random.default_rng(seed)
    npops, ts = 3, "((0,1):3,2):4"
    sp = popmodel.parse_treestring(ts, npops)
    tv0 = [0.45, 1.1]
    splits = [(tv0[k], a, b, anc) for k, (a, b, anc) in enumerate(sp)]
    kappa, pi_sim = 2.0, np.array([0.3, 0.2, 0.2, 0.3])
    loci, base, samps, alleles = [], [], [], {}
    out = {"npops": np.array(npops), "tree": np.array(ts), "tv0": np.array(tv0), "kinds": np.array(kinds),
           "us": np.array(us), "kappa": np.array(kappa), "thetaprior": np.array(10.0)}
    betas, seeds, nsweeps = [1.0, 0.8, 0.5], [11, 12, 13], 10
    for li, kind in enumerate(kinds):
        samp = [int(v) for v in rng.integers(3, 7, npops)]
        lg = synth.sim_im_labeled(rng, samp, list(rng.uniform(1.0, 3.0, 5)), 0.0, splits)
        samps.append(samp)
        base.append(lg)
        if kind == "is":
            seq = synth.is_data(rng, lg.g, us[li], min_sites=4)
            loci.append(("is", sum(samp), 1.0, samp, us[li], seq))
            out["seq_%d" % li] = seq
        elif kind == "hky":
            hl = synth.hky_data(rng, lg.g, 300, us[li], kappa, pi_sim)
            loci.append(("hky", sum(samp), 1.0, samp, us[li], hl, kappa))
            out["seq_%d" % li] = hl.seq
            out["mult_%d" % li] = hl.mult
            out["totsites_%d" % li] = np.array(hl.totsites)
            out["pi_%d" % li] = hl.pi
        else:
            A = synth.sw_alleles(rng, lg.g, us[li])
            lo, hi = int(A.min()) - 3, int(A.max()) + 3
            loci.append(("sw", sum(samp), 1.0, samp, us[li], lo, hi))
            out["alleles_%d" % li] = A
            out["arange_%d" % li] = np.array([lo, hi])
            for ci in range(len(betas)):
                alleles[(ci, li)] = A
    chains = [(tv0, b, s) for b, s in zip(betas, seeds)]
    gens = [[base[li] for li in range(len(kinds))] for _ in chains]
    res, trees = O.ref_ug(npops, ts, 10.0, loci, chains, gens, nsweeps, alleles=alleles)
    out.update({"samps": np.array(samps), "betas": np.array(betas), "seeds": np.array(seeds),
                "nsweeps": np.array(nsweeps), "res": np.array(res)})
    for f in ("up0", "up1", "down", "time", "pop"):
        out["base_" + f] = np.concatenate([getattr(g.g, f) if f != "pop" else g.pop for g in base])
    out["node_off"] = np.concatenate([[0], np.cumsum([len(g.pop) for g in base])]).astype(np.int32)
    for k, f in enumerate(("up0", "up1", "down", "time", "pop")):
        out["final_" + f] = np.concatenate([trees[(ci, li)][k] for ci in range(len(chains))
                                            for li in range(len(kinds))])
    if "sw" in kinds:
        out["final_A"] = np.concatenate([trees[(ci, li)][5] for ci in range(len(chains))
                                         for li in range(len(kinds)) if kinds[li] == "sw"])
    np.savez_compressed(os.path.join(OUT, name), **out)


def golden_ug():
    _golden_ug("golden_ug.npz", ["is", "hky", "is", "hky", "is"], 2031, [1.0, 1.5, 0.8, 1.2, 1.1])


def golden_ug_sw():
    """The same with stepwise loci among them (finishSWupdateA's allele
    proposal and branch terms, update_gtree_common.cpp:2219-2362)."""
    _golden_ug("golden_ug_sw.npz", ["sw", "is", "sw", "hky", "sw"], 2032, [2.0, 1.0, 1.5, 1.2, 3.0])

if __name__ == "__main__":
    if not O.ref_available():
        sys.exit("build the reference harness first: make -C oracle ref")
    gens = {"is": golden_is, "hky": golden_hky, "sw": golden_sw, "swap": golden_swap,
            "jointp": golden_jointp, "de": golden_de, "margin": golden_margin,
            "tw": golden_tw, "ry": golden_ry, "ks": golden_ks, "popmig": golden_popmig,
            "peaks": golden_peaks, "iparams": golden_iparams, "ug": golden_ug, "ug_sw": golden_ug_sw}
    for name in (sys.argv[1:] or list(gens)):
        gens[name]()
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))
