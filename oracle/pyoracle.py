"""ctypes view of the CPU oracle (libima_oracle.so) and a runner for the
compiled reference harness (_ref/imaref).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU legs, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# the IMa2p source tree the harness and the link-level binding compile
REFERENCE = os.environ.get("IMA2P_REFERENCE", "/root/reference")
LIB_PATH = os.path.join(HERE, "libima_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "imaref")

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


P = C.c_void_p
I = C.c_int
D = C.c_double


def _declare(L):
    L.ora_sw_batch.argtypes = [I, P, P, P, P, P, P, P, P, P, I, P]
    L.ora_sw_batch.restype = I
    L.ora_hky_batch.argtypes = [I, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, I, P]
    L.ora_hky_batch.restype = I
    L.ora_is_batch.argtypes = [I, P, P, P, P, P, P, P, P, P, P, P, P, I, P, P]
    L.ora_is_batch.restype = I
    L.ora_jointp_batch.argtypes = [I, I, P, I, I, I, I, P, I, P, I, P, P]
    L.ora_jointp_batch.restype = I
    L.ora_is_sumlogk.argtypes = [I, I, P, P, P, P, P, P]
    L.ora_is_sumlogk.restype = I
    L.ora_is_likelihood.argtypes = [I, I, P, P, P, P, P, D, D, D, P, P]
    L.ora_is_likelihood.restype = D
    L.ora_hky_likelihood.argtypes = [I, I, I, P, P, P, P, P, P, I, P, D, D, P, P, P, P, P]
    L.ora_hky_likelihood.restype = D
    for f in ("ora_hky_copyfraclike", "ora_hky_storescalefactors", "ora_hky_restorescalefactors"):
        getattr(L, f).argtypes = [I, I, P, P]
        getattr(L, f).restype = None
    L.ora_bessi.argtypes = [I, D]
    L.ora_bessi.restype = D
    L.ora_sw_likelihood.argtypes = [I, P, P, P, P, D, D, P]
    L.ora_sw_likelihood.restype = D
    L.ora_sw_branch_term.argtypes = [I, D, D]
    L.ora_sw_branch_term.restype = D
    L.ora_mt_fill_u32.argtypes = [C.c_uint32, I, P]
    L.ora_mt_fill_u32.restype = None
    L.ora_setheat.argtypes = [I, D, D, I, P, P]
    L.ora_setheat.restype = I
    L.ora_swapchains.argtypes = [I, I, P, P, P, P, P, P, P, P]
    L.ora_swapchains.restype = I
    L.ora_chain_sums.argtypes = [I, I, P, P, I, P]
    L.ora_chain_sums.restype = None
    L.ora_surface_p.argtypes = [I, I, P, I, I, I, I, P, P, P]
    L.ora_surface_p.restype = None
    for f in ("ora_jointp_exact", "ora_jointp_compat"):
        getattr(L, f).argtypes = [I, I, P, I, I, I, I, P, P, P]
        getattr(L, f).restype = D
    L.ora_margincalc.argtypes = [I, I, P, I, I, I, D, D, I, P]
    L.ora_margincalc.restype = D
    L.ora_ti_load.argtypes = [C.c_char_p, I, P, I]
    L.ora_ti_load.restype = I
    L.ora_findmarginpeaks.argtypes = [I, I, P, I, I, P, P, P, P, P, I, P, P, P, P, P, P, P, P, P, P]
    L.ora_findmarginpeaks.restype = I
    for f in ("ora_popmig", "ora_pop_expomig"):
        getattr(L, f).argtypes = [I, I, P, I, I, I, I, D, D, D, I, P]
        getattr(L, f).restype = D
    L.ora_mt_seed.argtypes = [P, C.c_uint32]
    L.ora_mt_seed.restype = None
    L.ora_mt_uniform.argtypes = [P]
    L.ora_mt_uniform.restype = D
    L.ora_modelloop.argtypes = [I, I, P, I, I, I, P, I, I, P, I, P, I, P, P, P, P]
    L.ora_modelloop.restype = I
    L.ora_treeweight.argtypes = [I, P, P, P, P, P, P, I, I, P, D, P, P, P, P, P, P, P, P, P, P, P, P, P]
    L.ora_treeweight.restype = I
    L.ora_treeweight_batch.argtypes = [I, P, P, P, P, P, I, I] + [P] * 19
    L.ora_treeweight_batch.restype = I
    L.ora_iterm.argtypes = [I, I, D, D, D, D, P]
    L.ora_iterm.restype = D
    L.ora_tree_prob.argtypes = [I, I, P, P, P, P, P, I, P, P, P, P, I, P, P, P, P, P, I, P, P, P, P]
    L.ora_tree_prob.restype = I
    L.ora_gsamp_row.argtypes = [I, P, P, P, P, P, I, P, P, I, P, P, P, P, D, D, I, P, P]
    L.ora_gsamp_row.restype = None
    L.ora_ug_rng_seed.argtypes = [P, I]
    L.ora_ug_rng_seed.restype = None
    # model (npops + 5 tables), theta maps (nth + 4), loci (nloci + 12), chains
    # (nchains + 9), gbeta + 3 rate arrays, nsweeps, rng, nthreads, 4 outputs
    L.ora_ug_run.argtypes = ([I] + [P] * 5 + [I] + [P] * 4 + [I] + [P] * 12 + [I] + [P] * 9 + [D] + [P] * 3 +
                             [I, P, I] + [P] * 4)
    L.ora_ug_run.restype = I


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ----------------------------------------------------------------- IS
def is_sumlogk(seq, g):
    n, S = seq.shape
    seq = np.ascontiguousarray(seq, np.int8)
    out = np.zeros(1)
    counts = np.zeros(n - 1, np.int32)
    st = lib().ora_is_sumlogk(n, S, _p(seq), _p(_i32(g.up0)), _p(_i32(g.up1)),
                              _p(_i32(g.down)), _p(out), _p(counts))
    return st, float(out[0]), counts


def is_likelihood(seq, g, length, u, sumlogk):
    n, S = seq.shape
    seq = np.ascontiguousarray(seq, np.int8)
    node = np.zeros(max(S, 1), np.int32)
    st = np.zeros(1, np.int32)
    v = lib().ora_is_likelihood(n, S, _p(seq), _p(_i32(g.up0)), _p(_i32(g.up1)),
                                _p(_i32(g.down)), _p(_f64(g.time)), length, u,
                                sumlogk, _p(node), _p(st))
    return v, int(st[0]), node[:S]


# ---------------------------------------------------------------- HKY
class HKYState:
    """FP64 frac/newfrac/scalefactor buffers of one chain-locus."""

    def __init__(self, n, S):
        nl = 2 * n - 1
        self.n, self.S = n, S
        self.frac = np.zeros((nl, S, 4))
        self.newfrac = np.zeros((nl, S, 4))
        self.sf = np.zeros((nl, S))
        self.oldsf = np.zeros((nl, S))

    def likelihood(self, loc, g, u, kappa, e=(-1, -1, -1, -1)):
        e = _i32(e)
        return lib().ora_hky_likelihood(
            self.n, self.S, loc.totsites, _p(np.ascontiguousarray(loc.seq, np.int8)),
            _p(_i32(loc.mult)), _p(_f64(loc.pi)), _p(_i32(g.up0)), _p(_i32(g.up1)),
            _p(_i32(g.down)), int(g.root), _p(_f64(g.time)), u, kappa, _p(e),
            _p(self.frac), _p(self.newfrac), _p(self.sf), _p(self.oldsf))

    def accept(self):
        lib().ora_hky_copyfraclike(self.n, self.S, _p(self.newfrac), _p(self.frac))
        lib().ora_hky_storescalefactors(self.n, self.S, _p(self.sf), _p(self.oldsf))

    def reject(self):
        lib().ora_hky_restorescalefactors(self.n, self.S, _p(self.sf), _p(self.oldsf))


# ----------------------------------------------------------------- SW
def sw_likelihood(A, g, u, tr=1.0):
    n = g.n
    dl = np.zeros(2 * n - 1)
    v = lib().ora_sw_likelihood(n, _p(_i32(A)), _p(_i32(g.down)), _p(_i32(g.up0)),
                                _p(_f64(g.time)), u, tr, _p(dl))
    return v, dl


def bessi(n, x):
    return lib().ora_bessi(int(n), float(x))


# ------------------------------------------------------------ MT / MC3
def mt_u32(seed, count):
    out = np.zeros(count, np.uint32)
    lib().ora_mt_fill_u32(seed, count, _p(out))
    return out


def mt_uniforms(seed, count):
    return (mt_u32(seed, count).astype(np.float64) + 0.5) * 2.32830643653869628906e-10


def setheat(nchains, h1, h2, mode):
    beta = np.zeros(nchains)
    allb = np.zeros(nchains)
    st = lib().ora_setheat(nchains, h1, h2, mode, _p(beta), _p(allb))
    return st, beta, allb


def chain_sums(pdg, probg, include_probg=True):
    nch, nl = pdg.shape
    S = np.zeros(nch)
    lib().ora_chain_sums(nch, nl, _p(_f64(pdg)), _p(_f64(probg)), int(include_probg), _p(S))
    return S


def swapchains(S, beta, allbetas, swaptries, uniforms, swapcount, tempcount):
    """Mutates beta, swapcount, tempcount in place; returns (swap0ok, used, decisions)."""
    n = len(beta)
    used = np.zeros(1, np.int32)
    dec = np.zeros((swaptries, 3), np.int32)
    ok = lib().ora_swapchains(n, swaptries, _p(_f64(S)), _p(beta), _p(_f64(allbetas)),
                              _p(_f64(uniforms)), _p(used), _p(swapcount), _p(tempcount),
                              _p(dec))
    return ok, int(used[0]), dec


# ------------------------------------------------------------ surface
def surface_p(rows, np_, nm, npops, x, modeltype=0, lognorm=None):
    G, rl = rows.shape
    out = np.zeros(G)
    rows = np.ascontiguousarray(rows, np.float32)
    lib().ora_surface_p(G, rl, _p(rows), np_, nm, npops, modeltype,
                        _p(_f64(lognorm)) if lognorm is not None else None,
                        _p(_f64(x)), _p(out))
    return out


def jointp(rows, np_, nm, npops, x, modeltype=0, lognorm=None, compat=False):
    G, rl = rows.shape
    rows = np.ascontiguousarray(rows, np.float32)
    ess = np.zeros(1)
    f = lib().ora_jointp_compat if compat else lib().ora_jointp_exact
    q = f(G, rl, _p(rows), np_, nm, npops, modeltype,
          _p(_f64(lognorm)) if lognorm is not None else None, _p(_f64(x)), _p(ess))
    return q, float(ess[0])


# ------------------------------------------------- compiled reference
def ref_available():
    return os.path.exists(REF_BIN)


def _tree_txt(g):
    return " ".join(map(str, g.up0)) + "\n" + " ".join(map(str, g.up1)) + "\n" + \
        " ".join(map(str, g.down)) + "\n" + " ".join("%.17g" % t for t in g.time) + "\n"


def run_ref(mode, text):
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write(text)
        path = f.name
    try:
        out = subprocess.run([REF_BIN, mode, path], check=True, capture_output=True,
                             text=True).stdout
    finally:
        os.unlink(path)
    return out


IPARAM_FLAGS = ("parameters_by_period", "ancestral_sizes_largest_sampled", "one_migration_parameter",
                "migration_between_sampled", "no_migration_between_nonsisters",
                "single_migration_both_directions", "no_migration", "expo_migration_prior")


def ref_iparams(npops, treestr, flags, thetaprior, mprior, varrank):
    """The reference's setup_iparams and set_nomigrationchecklist
    (initialize.cpp:202-809) on a population tree, through oracle/_ref/imaref
    (this container only).  flags: the IPARAM_FLAGS that are set.  Returns
    {"theta": [(name, b, e, [(p, r)], max, min)], "mig": [(name, b, e,
    [(p, r, c)], max, min, mean)], "chk": [(p, r, c)]}."""
    t = ["%d %s" % (npops, treestr), " ".join("1" if f in flags else "0" for f in IPARAM_FLAGS),
         "%.17g %.17g" % (thetaprior, mprior), " ".join("%.17g" % v for v in varrank)]
    out = run_ref("iparams", "\n".join(t) + "\n")
    res = {"theta": [], "mig": [], "chk": []}
    for ln in out.splitlines():
        f = ln.split()
        if f[0] == "TH":
            n = int(f[5])
            wp = [(int(f[6 + 2 * j]), int(f[7 + 2 * j])) for j in range(n)]
            res["theta"].append((f[2], int(f[3]), int(f[4]), wp, float(f[6 + 2 * n]), float(f[7 + 2 * n])))
        elif f[0] == "MG":
            n = int(f[5])
            wp = [(int(f[6 + 3 * j]), int(f[7 + 3 * j]), int(f[8 + 3 * j])) for j in range(n)]
            res["mig"].append((f[2], int(f[3]), int(f[4]), wp, float(f[6 + 3 * n]), float(f[7 + 3 * n]),
                               float(f[8 + 3 * n])))
        elif f[0] == "CHK":
            n = int(f[1])
            res["chk"] = [(int(f[2 + 3 * j]), int(f[3 + 3 * j]), int(f[4 + 3 * j])) for j in range(n)]
    return res


def ref_is(seq, trees, lengths, us):
    n, S = seq.shape
    t = [f"{n} {S}", " ".join(map(str, seq.ravel())), str(len(trees))]
    for g, L, u in zip(trees, lengths, us):
        t.append(_tree_txt(g) + "%.17g %.17g" % (L, u))
    out = run_ref("is", "\n".join(t) + "\n")
    return np.array([[float(v) for v in line.split()] for line in out.strip().splitlines()])


def ref_hky(loc, items):
    """items: list of (g, u, kappa, edits) where edits = [(g2, (e1..e4), accept)]."""
    n, S = loc.seq.shape
    t = [f"{n} {S} {loc.totsites}", " ".join(map(str, loc.seq.ravel())),
         " ".join(map(str, loc.mult)), " ".join("%.17g" % p for p in loc.pi), str(len(items))]
    for g, u, kappa, edits in items:
        t.append(_tree_txt(g) + "%.17g %.17g %d" % (u, kappa, len(edits)))
        for g2, e, acc in edits:
            t.append(_tree_txt(g2) + " ".join(map(str, e)) + " %d" % acc)
    out = run_ref("hky", "\n".join(t) + "\n")
    return np.array([float(v) for v in out.split()])


def ref_sw(trees, alleles, us, tr=1.0):
    n = trees[0].n
    t = [f"{n} {len(trees)}"]
    for g, A, u in zip(trees, alleles, us):
        t.append(_tree_txt(g) + " ".join(map(str, A)) + "\n%.17g %.17g" % (u, tr))
    out = run_ref("sw", "\n".join(t) + "\n")
    return np.array([[float(v) for v in line.split()] for line in out.strip().splitlines()])


def ref_swap(pdg, probg, swaptries, nsteps, mode, h1, h2, seed):
    nch, nl = pdg.shape
    t = [f"{nch} {nl} {swaptries} {nsteps} {mode} %.17g %.17g {seed}" % (h1, h2),
         " ".join("%.17g" % v for v in pdg.ravel()), " ".join("%.17g" % v for v in probg)]
    out = run_ref("swap", "\n".join(t) + "\n").strip().splitlines()
    steps = [line.split() for line in out[:nsteps]]
    ok = np.array([int(s[0]) for s in steps])
    betas = np.array([[float(v) for v in s[1:]] for s in steps])
    sc = np.array([[int(v) for v in line.split()] for line in out[nsteps:nsteps + nch]])
    tc = np.array([[int(v) for v in line.split()] for line in out[nsteps + nch:nsteps + 2 * nch]])
    return ok, betas, sc, tc


def ref_jointp(rows, np_, nm, npops, modeltype, points):
    G, rl = rows.shape
    t = [f"{G} {rl} {np_} {nm} {npops} {modeltype}",
         "\n".join(" ".join("%.9g" % v for v in r) for r in rows), str(len(points))]
    t += [" ".join("%.17g" % v for v in x) for x in points]
    out = run_ref("jointp", "\n".join(t) + "\n")
    return np.array([[float(v) for v in line.split()] for line in out.strip().splitlines()])


# ------------------------------------------------------------ DE peak search
class MT(C.Structure):
    """MT19937 generator state (utilities.cpp:323-427): mt[624], mti."""
    _fields_ = [("mt", C.c_uint32 * 624), ("mti", C.c_int)]

    def __init__(self, seed):
        super().__init__()
        lib().ora_mt_seed(C.byref(self), seed)

    def uniform(self):
        return lib().ora_mt_uniform(C.byref(self))


def modelloop(rows, np_, nm, npops, upper, modeltype=0, multiplier=100, seed=1234, rng=None,
              xmap=None, nested=0, compat=True, lognorm=None):
    """modelloop (jointfind.cpp:746-812) restated; returns (best[n+1], ess,
    generations, restarts, rng)."""
    G, rl = rows.shape
    rows = np.ascontiguousarray(rows, np.float32)
    n = np_ + nm
    rng = rng if rng is not None else MT(seed)
    best = np.zeros(n + 1)
    ess = np.zeros(1)
    nrun = np.zeros(1, np.int32)
    gens = lib().ora_modelloop(G, rl, _p(rows), np_, nm, npops,
                               _p(_f64(lognorm)) if lognorm is not None else None, int(compat), modeltype,
                               _p(_f64(upper)), multiplier,
                               _p(_f64(xmap)) if xmap is not None else None, nested,
                               C.cast(C.pointer(rng), C.c_void_p), _p(best), _p(ess), _p(nrun))
    return best, float(ess[0]), gens, int(nrun[0]), rng


def ref_de(rows, np_, nm, npops, upper, modeltype=0, multiplier=100, seed=1234, xmap=None, nested=0):
    """The reference's own modelloop through oracle/_ref/imaref (this
    container only); returns (best[n+1], ess)."""
    G, rl = rows.shape
    lines = ["%d %d %d %d %d %d %d %d %d" % (G, rl, np_, nm, npops, modeltype, multiplier, seed, nested),
             " ".join("%.9g" % v for v in np.asarray(rows, np.float32).ravel()),
             " ".join("%.17g" % v for v in upper)]
    if nested:
        lines.append(" ".join("%.17g" % v for v in xmap))
    out = run_ref("de", "\n".join(lines) + "\n")
    best = ess = None
    for ln in out.splitlines():
        if ln.startswith("BEST"):
            best = np.array([float(v) for v in ln.split()[1:]])
        elif ln.startswith("ESS"):
            ess = float(ln.split()[1])
    return best, ess


# ------------------------------------------------------------ 1-D marginals
def margincalc(rows, np_, nm, pi, x, yadjust=0.0, logi=0, expo_mean=None):
    G, rl = rows.shape
    rows = np.ascontiguousarray(rows, np.float32)
    return lib().ora_margincalc(G, rl, _p(rows), np_, nm, int(pi), float(x), float(yadjust), int(logi),
                                _p(_f64(expo_mean)) if expo_mean is not None else None)


def ref_margincalc(rows, np_, nm, points, expo_mean=None):
    """The reference's margincalc through oracle/_ref/imaref (this container
    only); points: (pi, x, logi, yadjust) tuples."""
    G, rl = rows.shape
    lines = ["%d %d %d %d %d" % (G, rl, np_, nm, 1 if expo_mean is not None else 0),
             " ".join("%.9g" % v for v in np.asarray(rows, np.float32).ravel())]
    if expo_mean is not None:
        lines.append(" ".join("%.17g" % v for v in expo_mean))
    lines.append(str(len(points)))
    lines += ["%d %.17g %d %.17g" % (int(p), x, int(lg), ya) for p, x, lg, ya in points]
    out = run_ref("margin", "\n".join(lines) + "\n")
    return np.array([float(v) for v in out.split()])


# ------------------------------------------------------------- 2NM densities
def popmig(rows, np_, nm, thetai, mi, x, qmax, mmax, mmean=None, prob_or_like=0):
    """calc_popmig (calc_pop_expomig when mmean is given) at x; raises
    ValueError where the reference would stop in an incomplete gamma term."""
    G, rl = rows.shape
    rows = np.ascontiguousarray(rows, np.float32)
    st = C.c_int(0)
    if mmean is None:
        v = lib().ora_popmig(G, rl, _p(rows), np_, nm, int(thetai), int(mi), float(x), float(qmax),
                             float(mmax), int(prob_or_like), C.byref(st))
    else:
        v = lib().ora_pop_expomig(G, rl, _p(rows), np_, nm, int(thetai), int(mi), float(x), float(qmax),
                                  float(mmean), int(prob_or_like), C.byref(st))
    if st.value:
        raise ValueError("incomplete gamma term failed (%d)" % st.value)
    return v


def ref_popmig(rows, np_, nm, qmax, mmax, points, mmean=None):
    """The reference's calc_popmig / calc_pop_expomig through
    oracle/_ref/imaref (this container only); points: (thetai, mi, x,
    prob_or_like) tuples; qmax [np], mmax [nm], mmean [nm] or None."""
    G, rl = rows.shape
    lines = ["%d %d %d %d %d" % (G, rl, np_, nm, 1 if mmean is not None else 0),
             " ".join("%.9g" % v for v in np.asarray(rows, np.float32).ravel()),
             " ".join("%.17g" % v for v in qmax), " ".join("%.17g" % v for v in mmax),
             " ".join("%.17g" % v for v in (mmean if mmean is not None else np.zeros(nm)))]
    lines.append(str(len(points)))
    lines += ["%d %d %.17g %d" % (int(t), int(m), x, int(pl)) for t, m, x, pl in points]
    out = run_ref("popmig", "\n".join(lines) + "\n")
    return np.array([float(v) for v in out.split()])


# ------------------------------------------------------ findmarginpeaks
def _parse_peaks(out, nt):
    d = {}
    for ln in out.splitlines():
        f = ln.split()
        if not f:
            continue
        if f[0] == "TOOFEW":
            return None
        if f[0] in ("ML", "PK", "PML", "PPK"):
            d.setdefault(f[0], []).append([float(v) for v in f[2:]])
        else:
            d[f[0]] = [float(v) for v in f[1:]]
    o = {"mlval": np.array(d["ML"]), "peakloc": np.array(d["PK"]), "migtest": np.array(d["MT"]),
         "lo95": np.array(d["LO"]), "hi95": np.array(d["HI"])}
    if nt:
        o["pm_mlval"], o["pm_peakloc"], o["pm_test"] = np.array(d["PML"]), np.array(d["PPK"]), np.array(d["PT"])
    return o


def ti_load(path, rowlen, cap):
    """The reference's .ti value loop on one core: rows [n][rowlen] float32."""
    rows = np.zeros((cap, rowlen), np.float32)
    n = lib().ora_ti_load(os.fsencode(str(path)), int(rowlen), _p(rows), int(cap))
    if n < 0:
        raise OSError("cannot open %s" % path)
    return rows[:n]


def findmarginpeaks(rows, np_, nm, th_min, th_max, mg_min, mg_max, mg_mean=None, terms=()):
    """The oracle's findmarginpeaks numbers (same dict as ref_findmarginpeaks);
    None for 10 or fewer genealogies."""
    G, rl = rows.shape
    rows = np.ascontiguousarray(rows, np.float32)
    terms = np.asarray(list(terms), np.int32).reshape(-1, 2)
    nt, npar = len(terms), np_ + nm
    mpop, mterm = np.ascontiguousarray(terms[:, 0]), np.ascontiguousarray(terms[:, 1])
    o = {"mlval": np.zeros((3, npar)), "peakloc": np.zeros((3, npar)), "migtest": np.zeros(max(nm, 1)),
         "lo95": np.zeros(npar), "hi95": np.zeros(npar), "pm_mlval": np.zeros((3, max(nt, 1))),
         "pm_peakloc": np.zeros((3, max(nt, 1))), "pm_test": np.zeros(max(nt, 1))}
    f = [_f64(v) for v in (th_min, th_max, mg_min, mg_max)]
    mean = _f64(mg_mean) if mg_mean is not None else None
    st = lib().ora_findmarginpeaks(G, rl, _p(rows), np_, nm, *(_p(v) for v in f), _p(mean) if mean is not None else None,
                                   nt, _p(mpop), _p(mterm), *(_p(o[k]) for k in ("mlval", "peakloc", "migtest",
                                                                                  "lo95", "hi95", "pm_mlval",
                                                                                  "pm_peakloc", "pm_test")))
    if st == -1:
        return None
    if st:
        raise ValueError("incomplete gamma term failed (%d)" % st)
    o["migtest"] = o["migtest"][:nm]
    if nt:
        o["pm_mlval"], o["pm_peakloc"], o["pm_test"] = o["pm_mlval"][:, :nt], o["pm_peakloc"][:, :nt], o["pm_test"][:nt]
    else:
        for k in ("pm_mlval", "pm_peakloc", "pm_test"):
            del o[k]
    return o


def ref_findmarginpeaks(rows, np_, nm, th_min, th_max, mg_min, mg_max, mg_mean=None, terms=()):
    """The reference's findmarginpeaks numbers (marginalopt over the two
    halves and all genealogies, the migration tests, margin95, and for the
    2NM terms marginalopt_popmig and its test) through oracle/_ref/imaref
    (this container only)."""
    G, rl = rows.shape
    terms = list(terms)
    lines = ["%d %d %d %d %d" % (G, rl, np_, nm, 1 if mg_mean is not None else 0),
             " ".join("%.9g" % v for v in np.asarray(rows, np.float32).ravel())]
    for arr in (th_min, th_max, mg_min, mg_max, mg_mean if mg_mean is not None else np.zeros(nm)):
        lines.append(" ".join("%.17g" % v for v in arr))
    lines.append(str(len(terms)))
    lines.append(" ".join(str(t[0]) for t in terms))
    lines.append(" ".join(str(t[1]) for t in terms))
    return _parse_peaks(run_ref("peaks", "\n".join(lines) + "\n"), len(terms))


# ------------------------------------------------- treeweight + p(G) integral
def ref_tw(npops, treestr, loci, tvals, gens, thetaprior, mprior, expo=False, nomig=False):
    """The reference's treeweight, sum_treeinfo and
    initialize_integrate_tree_prob through oracle/_ref/imaref (this container
    only).  loci: (numgenes, hval, samppop) per locus; tvals: split times per
    chain; gens[ci][li]: LabelledGenealogy.  Returns a dict with the
    parameter maps ("theta": [(wp, max, min)], "mig": [(wp, max, min, mean)]),
    per chain-locus weights ("gw") and per chain integrals ("pg")."""
    nch, nl = len(gens), len(loci)
    t = ["%d %d %d %d %d" % (npops, nch, nl, int(expo), int(nomig)), treestr,
         "%.17g %.17g" % (thetaprior, mprior)]
    for ng, h, sp in loci:
        t.append("%d %.17g %s" % (ng, h, " ".join(map(str, sp))))
    for tv in tvals:
        t.append(" ".join("%.17g" % v for v in tv) if len(tv) else "")
    for ci in range(nch):
        for li in range(nl):
            lg = gens[ci][li]
            t.append(str(len(lg.pop)))
            t.append(_tree_txt(lg.g) + " ".join(map(str, lg.pop)))
            for m in lg.mig:
                t.append(" ".join([str(len(m))] + ["%.17g %d" % (mt, mp) for mt, mp in m]))
    out = run_ref("tw", "\n".join(t) + "\n")
    T = npops * (npops + 1) // 2
    M = 0 if nomig else sum((npops - k) ** 2 for k in range(npops - 1))
    res = {"theta": [], "mig": [], "gw": {}, "pg": {}}
    for ln in out.splitlines():
        f = ln.split()
        if f[0] == "TH":
            n = int(f[2])
            wp = [(int(f[3 + 2 * j]), int(f[4 + 2 * j])) for j in range(n)]
            res["theta"].append((wp, float(f[3 + 2 * n]), float(f[4 + 2 * n])))
        elif f[0] == "MG":
            n = int(f[2])
            wp = [(int(f[3 + 3 * j]), int(f[4 + 3 * j]), int(f[5 + 3 * j])) for j in range(n)]
            res["mig"].append((wp, float(f[3 + 3 * n]), float(f[4 + 3 * n]), float(f[5 + 3 * n])))
        elif f[0] == "GW":
            v = f[3:]
            o = 0
            d = {"mignum": int(v[0]), "length": float(v[1]), "tlength": float(v[2])}
            o = 3
            d["cc"] = np.array([int(x) for x in v[o:o + T]]); o += T
            d["hcc"] = np.array([float(x) for x in v[o:o + T]]); o += T
            d["fc"] = np.array([float(x) for x in v[o:o + T]]); o += T
            d["mc"] = np.array([int(x) for x in v[o:o + M]], dtype=np.int64); o += M
            d["fm"] = np.array([float(x) for x in v[o:o + M]]); o += M
            res["gw"][(int(f[1]), int(f[2]))] = d
        elif f[0] == "PG":
            res["pg"][int(f[1])] = np.array([float(x) for x in f[2:]])
    return res


def ref_iterm(lines):
    """Reference integral terms; lines: (kind, c, f, h, max, min) with kind 0
    coalescent, 1 migration, 2 migration under the exponential prior (max is
    then the prior mean)."""
    t = [str(len(lines))] + ["%d %d %.17g %.17g %.17g %.17g" % tuple(x) for x in lines]
    return np.array([float(v) for v in run_ref("iterm", "\n".join(t) + "\n").split()])


def treeweight(pm, tvals, lg, samppop, hval):
    """ora_treeweight on one LabelledGenealogy; returns (status, dict)."""
    T, M = pm.T, pm.M
    g = lg.g
    ng = g.n
    off, mt, mp = lg.packed_mig()
    cc = np.zeros(T, np.int32); hcc = np.zeros(T); fc = np.zeros(T)
    mc = np.zeros(max(M, 1), np.int32); fm = np.zeros(max(M, 1))
    out3 = np.zeros(2); mn = np.zeros(1, np.int32)
    st = lib().ora_treeweight(pm.npops, _p(_i32(pm.plist)), _p(_i32(pm.droppops)), _p(_i32(pm.addpop)),
                              _p(_i32(pm.pop_e)), _p(_i32(pm.pop_down)), _p(_f64(tvals)), int(pm.nomig),
                              ng, _p(_i32(samppop)), float(hval), _p(_i32(g.up0)), _p(_f64(g.time)),
                              _p(_i32(lg.pop)), _p(_i32(off)), _p(_f64(mt if len(mt) else np.zeros(1))),
                              _p(_i32(mp if len(mp) else np.zeros(1))), _p(cc), _p(hcc), _p(fc),
                              _p(mc), _p(fm), _p(out3), _p(mn))
    return st, {"cc": cc, "hcc": hcc, "fc": fc, "mc": mc[:M], "fm": fm[:M],
                "length": float(out3[0]), "tlength": float(out3[1]), "mignum": int(mn[0])}


def iterm(kind, c, f, h, mx, mn):
    st = np.zeros(1, np.int32)
    v = lib().ora_iterm(int(kind), int(c), float(f), float(h), float(mx), float(mn), _p(st))
    return v, int(st[0])


def sum_weights(ws, pm):
    """sum_treeinfo (ginfo.cpp:209-244) over loci in order, from zero."""
    tot = {"cc": np.zeros(pm.T, np.int32), "hcc": np.zeros(pm.T), "fc": np.zeros(pm.T),
           "mc": np.zeros(pm.M, np.int32), "fm": np.zeros(pm.M)}
    for w in ws:
        for k in tot:
            tot[k] = tot[k] + w[k]
    return tot


def tree_prob(pm, w, th_max, th_min, mg_max, mg_min, mg_mean, expo=False, chk=()):
    tho, thi = pm.th_csr()
    mgo, mgi = pm.mg_csr()
    nth, nmg = len(pm.th_cells), len(pm.mg_cells)
    q = np.zeros(max(nth, 1)); m = np.zeros(max(nmg, 1)); pg = np.zeros(1)
    chk = _i32(np.asarray(chk if len(chk) else [0]))
    st = lib().ora_tree_prob(int(pm.nomig), int(expo), _p(_i32(w["cc"])), _p(_f64(w["hcc"])), _p(_f64(w["fc"])),
                             _p(_i32(w["mc"] if pm.M else np.zeros(1))), _p(_f64(w["fm"] if pm.M else np.zeros(1))),
                             nth, _p(tho), _p(thi if len(thi) else np.zeros(1, np.int32)),
                             _p(_f64(th_max)), _p(_f64(th_min)),
                             nmg, _p(mgo), _p(mgi if len(mgi) else np.zeros(1, np.int32)),
                             _p(_f64(mg_max if nmg else np.zeros(1))), _p(_f64(mg_min if nmg else np.zeros(1))),
                             _p(_f64(mg_mean if nmg else np.zeros(1))), len(chk) if chk[0] or len(chk) > 1 else 0,
                             _p(chk), _p(pg), _p(q), _p(m))
    return st, float(pg[0]), q[:nth], m[:nmg]


def gsamp_row(pm, w, q, m, pdg, probg, tvals):
    tho, thi = pm.th_csr()
    mgo, mgi = pm.mg_csr()
    nth, nmg = len(pm.th_cells), len(pm.mg_cells)
    nm_eff = 0 if pm.nomig else nmg
    row = np.zeros(3 * nth + 2 * nm_eff + nth + nm_eff + 2 + pm.npops - 1, np.float32)
    lib().ora_gsamp_row(int(pm.nomig), _p(_i32(w["cc"])), _p(_f64(w["hcc"])), _p(_f64(w["fc"])),
                        _p(_i32(w["mc"] if pm.M else np.zeros(1))), _p(_f64(w["fm"] if pm.M else np.zeros(1))),
                        nth, _p(tho), _p(thi), nmg, _p(mgo), _p(mgi if len(mgi) else np.zeros(1, np.int32)),
                        _p(_f64(q)), _p(_f64(m if len(m) else np.zeros(1))), float(pdg), float(probg),
                        pm.npops - 1, _p(_f64(tvals)), _p(row))
    return row


def treeweight_batch(pm, packed, gen_locus, gen_tv, hval, samppop, tvals):
    """ora_treeweight_batch over the CSR inputs of ima_gpu_treeweight;
    returns (number rejected, dict of outputs)."""
    node_off, up0, time, pop, mig_off, mig_t, mig_p = packed
    ngen = len(node_off) - 1
    T, M = pm.T, pm.M
    out = {"cc": np.zeros((ngen, T), np.int32), "hcc": np.zeros((ngen, T)), "fc": np.zeros((ngen, T)),
           "mc": np.zeros((ngen, M), np.int32), "fm": np.zeros((ngen, M)), "lens": np.zeros((ngen, 2)),
           "mignum": np.zeros(ngen, np.int32)}
    keep = [_i32(node_off), _i32(up0), _f64(time), _i32(pop), _i32(mig_off),
            _f64(mig_t if len(mig_t) else np.zeros(1)), _i32(mig_p if len(mig_p) else np.zeros(1)),
            _i32(gen_locus), _i32(gen_tv), _f64(hval), _i32(samppop), _f64(tvals)]
    bad = lib().ora_treeweight_batch(pm.npops, _p(_i32(pm.plist)), _p(_i32(pm.droppops)), _p(_i32(pm.addpop)),
                                     _p(_i32(pm.pop_e)), _p(_i32(pm.pop_down)), int(pm.nomig), ngen,
                                     *(_p(a) for a in keep),
                                     *(_p(out[k]) for k in ("cc", "hcc", "fc", "mc", "fm", "lens", "mignum")))
    return bad, out


def ref_ry(npops, treestr, tprior, loci, chains, gens, steps, seed, thetaprior, mprior, expo=False):
    """The reference's split-time update changet_RY1 through
    oracle/_ref/imaref (this container only).  loci: (numgenes, hval,
    samppop, u, seq[n][S]) per infinite-sites locus; chains: (tvals, beta);
    gens[ci][li]: LabelledGenealogy; steps: (ci, period) in order.  Returns
    (per step (accepted, tval, probg, pdg), times[ci][li], migration
    times[ci][li])."""
    nch, nl = len(chains), len(loci)
    t = ["%d %d %d %d %d %d" % (npops, nch, nl, seed, len(steps), int(expo)), treestr,
         "%.17g %.17g" % (thetaprior, mprior)]
    t += ["%.17g %.17g" % tuple(p) for p in tprior]
    for ng, h, sp, u, seq in loci:
        seq = np.asarray(seq)
        t.append("%d %.17g %s %.17g %d" % (ng, h, " ".join(map(str, sp)), u, seq.shape[1]))
        t.append(" ".join(map(str, seq.ravel())))
    for tv, b in chains:
        t.append(" ".join("%.17g" % v for v in tv) + " %.17g" % b)
    for ci in range(nch):
        for li in range(nl):
            lg = gens[ci][li]
            t.append(str(len(lg.pop)))
            t.append(_tree_txt(lg.g) + " ".join(map(str, lg.pop)))
            for m in lg.mig:
                t.append(" ".join([str(len(m))] + ["%.17g %d" % (mt, mp) for mt, mp in m]))
    t += ["%d %d" % s for s in steps]
    out = run_ref("ry", "\n".join(t) + "\n")
    res, times, migt = [], {}, {}
    for ln in out.splitlines():
        f = ln.split()
        if f[0] == "STEP":
            res.append((int(f[1]), float(f[2]), float(f[3]), float(f[4])))
        elif f[0] == "TIMES":
            times[(int(f[1]), int(f[2]))] = np.array([float(v) for v in f[3:]])
        elif f[0] == "MIGT":
            migt[(int(f[1]), int(f[2]))] = np.array([float(v) for v in f[3:]])
    return res, times, migt


def ref_ug(npops, treestr, thetaprior, loci, chains, gens, nsweeps, alleles=None):
    """The reference's genealogy update updategenealogy under the
    no-migration model through oracle/_ref/imaref (this container only).
    loci: ("is", numgenes, hval, samppop, u, seq[n][S]), ("hky", numgenes,
    hval, samppop, u, HKYLocus, kappa) or ("sw", numgenes, hval, samppop, u,
    minA, maxA); chains: (tvals, beta, seed); gens[ci][li]:
    LabelledGenealogy (no migration events); alleles[(ci, li)]: the SW
    loci's alleles of every node.  Each chain runs nsweeps sweeps over its
    loci from setseeds(seed).  Returns (per proposal (ci, li, accepted,
    topolchange, tmrcachange, pdg, probg), final trees {(ci, li): (up0, up1,
    down, time, pop[, A])})."""
    nch, nl = len(chains), len(loci)
    t = ["%d %d %d %d" % (npops, nch, nl, nsweeps), treestr, "%.17g" % thetaprior]
    for loc in loci:
        kind, ng, h, sp, u = loc[:5]
        if kind == "sw":
            t.append("2 %d %.17g %s %.17g %d %d" % (ng, h, " ".join(map(str, sp)), u, loc[5], loc[6]))
        elif kind == "is":
            seq = np.asarray(loc[5])
            t.append("0 %d %.17g %s %.17g %d" % (ng, h, " ".join(map(str, sp)), u, seq.shape[1]))
            t.append(" ".join(map(str, seq.ravel())))
        else:
            hl, kappa = loc[5], loc[6]
            t.append("1 %d %.17g %s %.17g %d" % (ng, h, " ".join(map(str, sp)), u, hl.seq.shape[1]))
            t.append(" ".join(map(str, hl.seq.ravel())))
            t.append("%d %s %s %.17g" % (hl.totsites, " ".join(map(str, hl.mult)),
                                         " ".join("%.17g" % p for p in hl.pi), kappa))
    for tv, b, seed in chains:
        t.append(" ".join("%.17g" % v for v in tv) + " %.17g %d" % (b, seed))
    for ci in range(nch):
        for li in range(nl):
            lg = gens[ci][li]
            t.append(str(len(lg.pop)))
            t.append(_tree_txt(lg.g) + " ".join(map(str, lg.pop)))
            if loci[li][0] == "sw":
                t.append(" ".join(map(str, alleles[(ci, li)])))
    out = run_ref("ug", "\n".join(t) + "\n")
    res, trees = [], {}
    for ln in out.splitlines():
        f = ln.split()
        if f[0] == "UG":
            res.append((int(f[1]), int(f[2]), int(f[3]), int(f[4]), int(f[5]), float(f[6]), float(f[7])))
        elif f[0] == "TREE":
            ci, li = int(f[1]), int(f[2])
            k = 6 if loci[li][0] == "sw" else 5
            m = (len(f) - 3) // k
            v = f[3:]
            tr = (np.array(v[0:m], np.int32), np.array(v[m:2 * m], np.int32),
                  np.array(v[2 * m:3 * m], np.int32), np.array([float(x) for x in v[3 * m:4 * m]]),
                  np.array(v[4 * m:5 * m], np.int32))
            if k == 6:
                tr = tr + (np.array(v[5 * m:6 * m], np.int32),)
            trees[(ci, li)] = tr
    return res, trees


class UgRng(C.Structure):
    """ora_ug_rng: a chain's uniform() MT19937, normdev's cached deviate and
    bitran's register."""
    _fields_ = [("mt", C.c_uint32 * 624), ("mti", C.c_int), ("iset", C.c_int32), ("gset", C.c_double),
                ("iseed", C.c_uint64)]

    def __init__(self, seed=None):
        super().__init__()
        if seed is not None:
            lib().ora_ug_rng_seed(C.byref(self), int(seed))


class UgLoci:
    """The loci of an updategenealogy run packed for ora_ug_run: per locus
    ("is", seq, sumlogk), ("hky", HKYLocus-like (seq, mult, totsites)) or
    ("sw", numgenes, minA, maxA)."""

    def __init__(self, loci, hval, samppop):
        self.nloci = len(loci)
        self.model = _i32([{"is": 0, "hky": 1, "sw": 2}[l[0]] for l in loci])
        seqs = [np.zeros((l[1], 1), np.int8) if l[0] == "sw" else
                np.ascontiguousarray(l[1].seq if l[0] == "hky" else l[1], np.int8) for l in loci]
        self.n = _i32([q.shape[0] for q in seqs])
        self.S = _i32([q.shape[1] for q in seqs])
        self.arange = _i32([[l[2], l[3]] if l[0] == "sw" else [0, 0] for l in loci]).ravel()
        self.totsites = _i32([l[1].totsites if l[0] == "hky" else 0 for l in loci])
        self.seq_off = np.concatenate([[0], np.cumsum([q.size for q in seqs])[:-1]]).astype(np.int64)
        self.seq = np.concatenate([q.ravel() for q in seqs]).astype(np.int8)
        mults = [_i32(l[1].mult) if l[0] == "hky" else np.zeros(1, np.int32) for l in loci]
        self.mult_off = np.concatenate([[0], np.cumsum([m.size for m in mults])[:-1]]).astype(np.int64)
        self.mult = np.concatenate(mults).astype(np.int32)
        self.sumlogk = _f64([l[2] if l[0] == "is" else 0.0 for l in loci])
        self.hval = _f64(hval)
        self.samppop = _i32(samppop)


def ug_run(pm, th_max, th_min, loci, gens, tvals, betas, u, kappa, pi, nsweeps, rngs, gbeta=1.0, nthreads=1,
           record=True, alleles=None):
    """ora_ug_run: nsweeps genealogy updates (no-migration model) of every
    chain; gens[c][l] LabelledGenealogy (copied, not changed); alleles[(c,
    l)] the SW loci's alleles of every node; rngs UgRng per chain
    (advanced).  Returns (status, res [nch][nsweeps][nloci][3] or None, resd
    [...][2] or None, pdg [nch][nloci], probg [nch], final genealogies (up0,
    up1, down, time, pop, A) flat in chain-locus order)."""
    nch, nl = len(gens), loci.nloci
    flat = [lg for row in gens for lg in row]
    lens = [len(lg.pop) for lg in flat]
    node_off = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
    up0 = _i32(np.concatenate([lg.g.up0 for lg in flat])).copy()
    up1 = _i32(np.concatenate([lg.g.up1 for lg in flat])).copy()
    down = _i32(np.concatenate([lg.g.down for lg in flat])).copy()
    time = _f64(np.concatenate([lg.g.time for lg in flat])).copy()
    pop = _i32(np.concatenate([lg.pop for lg in flat])).copy()
    A = np.zeros(len(pop), np.int32)
    if alleles:
        k = 0
        for c in range(nch):
            for l in range(nl):
                m = len(gens[c][l].pop)
                if (c, l) in alleles:
                    A[k:k + m] = alleles[(c, l)]
                k += m
    tho, thi = pm.th_csr()
    arr = (UgRng * nch)(*rngs)
    res = np.zeros((nch, nsweeps, nl, 3), np.int32) if record else None
    resd = np.zeros((nch, nsweeps, nl, 2)) if record else None
    pdg, probg = np.zeros((nch, nl)), np.zeros(nch)
    tv = _f64(np.asarray(tvals, np.float64).reshape(nch, -1))
    st = lib().ora_ug_run(pm.npops, _p(_i32(pm.plist)), _p(_i32(pm.droppops)), _p(_i32(pm.addpop)),
                          _p(_i32(pm.pop_e)), _p(_i32(pm.pop_down)), len(pm.th_cells), _p(tho), _p(thi),
                          _p(_f64(th_max)), _p(_f64(th_min)), nl, _p(loci.model), _p(loci.n), _p(loci.S),
                          _p(loci.totsites), _p(loci.seq_off), _p(loci.mult_off), _p(loci.seq), _p(loci.mult),
                          _p(loci.hval), _p(loci.samppop), _p(loci.sumlogk), _p(loci.arange), nch, _p(node_off),
                          _p(up0), _p(up1), _p(down), _p(time), _p(pop), _p(A), _p(tv), _p(_f64(betas)), float(gbeta),
                          _p(_f64(np.asarray(u).reshape(-1))), _p(_f64(np.asarray(kappa).reshape(-1))),
                          _p(_f64(np.asarray(pi).reshape(-1))), int(nsweeps), C.cast(arr, P), int(nthreads),
                          _p(res), _p(resd), _p(pdg), _p(probg))
    for k in range(nch):
        C.memmove(C.addressof(rngs[k]), C.addressof(arr[k]), C.sizeof(UgRng))
    return st, res, resd, pdg, probg, (up0, up1, down, time, pop, A)


# ------------------------------------------------------------- batches
class PackedItems:
    """Chain-loci of one model packed into flat arrays for the batched C
    entry points (ora_*_batch): evaluating them costs one call, so timing
    them times the restated arithmetic, not per-item marshalling.

    items: (kind, genealogy, u, kappa / tr, data) with kind "is" | "hky" |
    "sw" (all the same); data is the IS seq, the HKYLocus or the alleles."""

    def __init__(self, items):
        kinds = {it[0] for it in items}
        assert len(kinds) == 1, kinds
        self.kind = kinds.pop()
        self.nitems = len(items)
        gs = [it[1] for it in items]
        self.n = _i32([g.n for g in gs])
        nl = np.array([len(g.up0) for g in gs], np.int64)
        self.node_off = np.concatenate([[0], np.cumsum(nl)[:-1]]).astype(np.int64)
        self.up0 = _i32(np.concatenate([g.up0 for g in gs]))
        self.up1 = _i32(np.concatenate([g.up1 for g in gs]))
        self.down = _i32(np.concatenate([g.down for g in gs]))
        self.time = _f64(np.concatenate([g.time for g in gs]))
        self.u = _f64([it[2] for it in items])
        self.par = _f64([it[3] for it in items])
        self.out = np.zeros(self.nitems)
        if self.kind == "sw":
            A = [_i32(it[4]) for it in items]
            self.al_off = np.concatenate([[0], np.cumsum([len(a) for a in A])[:-1]]).astype(np.int64)
            self.A = _i32(np.concatenate(A))
        else:
            # one copy of each distinct data table
            tabs, idx = [], {}
            for it in items:
                key = id(it[4])
                if key not in idx:
                    idx[key] = len(tabs)
                    tabs.append(it[4])
            seqs = [np.ascontiguousarray(t.seq if self.kind == "hky" else t, np.int8) for t in tabs]
            soff = np.concatenate([[0], np.cumsum([q.size for q in seqs])[:-1]]).astype(np.int64)
            self.seq = np.concatenate([q.ravel() for q in seqs]).astype(np.int8)
            tix = [idx[id(it[4])] for it in items]
            self.S = _i32([seqs[t].shape[1] for t in tix])
            self.seq_off = soff[tix]
            if self.kind == "hky":
                mults = [_i32(t.mult) for t in tabs]
                moff = np.concatenate([[0], np.cumsum([len(m) for m in mults])[:-1]]).astype(np.int64)
                self.mult = _i32(np.concatenate(mults))
                self.mult_off = moff[tix]
                self.totsites = _i32([tabs[t].totsites for t in tix])
                self.pi = _f64(np.concatenate([tabs[t].pi for t in tix]))
            else:
                self.length = _f64([g.length() for g in gs])
                self.sumlogk = np.zeros(self.nitems)
                self.status = np.zeros(self.nitems, np.int32)

    def run(self, nthreads=1):
        """Evaluate every item; returns the log likelihoods."""
        L = lib()
        if self.kind == "sw":
            L.ora_sw_batch(self.nitems, _p(self.n), _p(self.node_off), _p(self.up0), _p(self.down), _p(self.time),
                           _p(self.al_off), _p(self.A), _p(self.u), _p(self.par), int(nthreads), _p(self.out))
        elif self.kind == "hky":
            L.ora_hky_batch(self.nitems, _p(self.n), _p(self.node_off), _p(self.up0), _p(self.up1), _p(self.down),
                            _p(self.time), _p(self.S), _p(self.totsites), _p(self.seq_off), _p(self.seq),
                            _p(self.mult_off), _p(self.mult), _p(self.pi), _p(self.u), _p(self.par),
                            int(nthreads), _p(self.out))
        else:
            L.ora_is_batch(self.nitems, _p(self.n), _p(self.node_off), _p(self.up0), _p(self.up1), _p(self.down),
                           _p(self.time), _p(self.S), _p(self.seq_off), _p(self.seq), _p(self.length), _p(self.u),
                           _p(self.sumlogk), int(nthreads), _p(self.out), _p(self.status))
        return self.out


def jointp_batch(rows, np_, nm, npops, pts, modeltype=0, lognorm=None, nthreads=1):
    """ora_jointp_exact at every point, on nthreads host threads: (q, ess)."""
    rows = np.ascontiguousarray(rows, np.float32)
    pts = _f64(pts)
    q, ess = np.zeros(len(pts)), np.zeros(len(pts))
    ln = _f64(lognorm) if lognorm is not None else None
    lib().ora_jointp_batch(rows.shape[0], rows.shape[1], _p(rows), np_, nm, npops, modeltype,
                           _p(ln) if ln is not None else None, len(pts), _p(pts), int(nthreads), _p(q), _p(ess))
    return q, ess
