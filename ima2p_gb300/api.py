"""Python view of the C ABI in include/ima_gpu.h (libima2p_gb300.so).

The method names mirror the reference functions they replace
(likelihoodIS / likelihoodHKY / likelihoodSW, copyfraclike /
storescalefactors / restorescalefactors, setheat / swapchains, jointp), with
the same argument meaning, sentinels and error behaviour: a failing call
raises ImaError carrying the library's status code and message, where the
reference would print IM_err and exit.  There is no CPU fallback: without the
compiled library every call fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libima2p_gb300.so")

IMA_OK, IMA_ERR_ARG, IMA_ERR_CUDA, IMA_ERR_STATE, IMA_ERR_NOMEM, IMA_ERR_DATA = 0, -1, -2, -3, -4, -5
MODEL_IS, MODEL_HKY, MODEL_SW = 0, 1, 2
PREC_FAST, PREC_FP64, PREC_FP32 = 0, 1, 2
EVAL_OK, EVAL_IS_REJECT, EVAL_IS_FAIL, EVAL_SW_ZERO = 0, 1, 2, 3
SURF_FAST, SURF_FP64, SURF_COMPAT, SURF_TC = 0, 1, 2, 3
K_IS, K_IS_SUMLOGK, K_HKY_FAST, K_HKY_FP64, K_SW_FAST, K_SW_FP64, K_SWAP, K_SURF_FAST, \
    K_SURF_FP64, K_SURF_COMPAT, K_SURF_TC, K_MARGIN, K_TREEWEIGHT, K_TREE_PROB, K_POPMIG, K_HKY_FP32, K_TIMES, \
    K_UG = range(18)
KERNEL_NAMES = ["is", "is_sumlogk", "hky_fast", "hky_fp64", "sw_fast", "sw_fp64", "swap",
                "surf_fast", "surf_fp64", "surf_compat", "surf_tc", "margin", "treeweight", "tree_prob",
                "popmig", "hky_fp32", "times", "ug"]
REJECT_IS = -1000000000.0

# every symbol the header declares (checked by tests/test_abi.py)
EXPORTS = [
    "ima_gpu_create", "ima_gpu_destroy", "ima_gpu_error", "ima_gpu_synchronize",
    "ima_gpu_add_locus_is", "ima_gpu_add_locus_hky", "ima_gpu_add_locus_sw", "ima_gpu_set_chains",
    "ima_gpu_set_genealogy", "ima_gpu_set_genealogies", "ima_gpu_set_pi", "ima_gpu_set_alleles",
    "ima_gpu_set_allele_edits", "ima_gpu_likelihoodIS",
    "ima_gpu_likelihoodHKY", "ima_gpu_copyfraclike", "ima_gpu_storescalefactors",
    "ima_gpu_restorescalefactors", "ima_gpu_likelihoodSW", "ima_gpu_get_dlikeA", "ima_gpu_eval",
    "ima_gpu_commit", "ima_gpu_batch_create", "ima_gpu_batch_run", "ima_gpu_batch_results",
    "ima_gpu_batch_destroy", "ima_gpu_flush_genealogies", "ima_gpu_setheat", "ima_gpu_get_betas",
    "ima_gpu_set_betas", "ima_gpu_set_pdg", "ima_gpu_get_pdg", "ima_gpu_set_probg",
    "ima_gpu_swapchains", "ima_gpu_swapchains_cb", "ima_gpu_set_allbetas", "ima_gpu_surface_retaken",
    "ima_gpu_batch_sweep", "ima_gpu_set_times", "ima_gpu_eval_times", "ima_gpu_get_swapcounts", "ima_gpu_surface_load",
    "ima_gpu_surface_eval", "ima_gpu_jointp", "ima_gpu_surface_fp64_noalloc", "ima_gpu_tc_selftest",
    "ima_gpu_surface_info", "ima_mt19937_seed", "ima_mt19937_uniform", "ima_gpu_modelloop",
    "ima_gpu_batch_autotune", "ima_gpu_batch_set_variants", "ima_gpu_margincalc", "ima_gpu_fillvec",
    "ima_ti_read", "ima_ti_write_binary", "ima_ti_read_binary",
    "ima_gpu_timer_begin", "ima_gpu_timer_end",
    "ima_gpu_set_profiling", "ima_gpu_kernel_stats", "ima_gpu_launch_count", "ima_gpu_flush_l2",
    "ima_gpu_memory", "ima_gpu_set_popmodel", "ima_gpu_treeweight", "ima_gpu_tree_prob",
    "ima_gpu_surface_append_tree_rows", "ima_gpu_surface_get_rows",
    "ima_gpu_set_locus_pops", "ima_gpu_set_labels", "ima_gpu_get_times", "ima_gpu_rubber_band",
    "ima_gpu_chain_weights", "ima_gpu_changet_ry1_sweep", "ima_gpu_get_probg", "ima_gpu_get_split_times",
    "ima_gpu_checkpoint_write", "ima_gpu_checkpoint_read", "ima_gpu_popmig", "ima_gpu_popmig_curves",
    "ima_gpu_findmarginpeaks", "ima_gpu_changet_ry1_sweep_mt", "ima_ug_rng_seed",
    "ima_gpu_updategenealogy_sweep", "ima_gpu_get_genealogy", "ima_gpu_get_alleles",
]


def _ck_free(code, what):
    if code != IMA_OK:
        raise ImaError(code, what)


def ti_read(paths, rowlen, maxload=0):
    """Rows of the reference's .ti files (ima_ti_read): (rows [G][rowlen]
    float32, total genealogies in the files)."""
    lib = load_library()
    arr = (C.c_char_p * len(paths))(*[os.fsencode(p) for p in paths])
    loaded, total = I(), I()
    _ck_free(lib.ima_ti_read(len(paths), C.cast(arr, P), int(rowlen), int(maxload), None, 0,
                             C.byref(loaded), C.byref(total)), "ti_read (count)")
    rows = np.zeros((loaded.value, rowlen), np.float32)
    _ck_free(lib.ima_ti_read(len(paths), C.cast(arr, P), int(rowlen), int(maxload), _ptr(rows), loaded.value,
                             C.byref(loaded), C.byref(total)), "ti_read")
    return rows, total.value


def ti_write_binary(path, rows):
    rows = np.ascontiguousarray(rows, np.float32)
    _ck_free(load_library().ima_ti_write_binary(os.fsencode(path), rows.shape[0], rows.shape[1], _ptr(rows)),
             "ti_write_binary")


def ti_read_binary(path):
    lib = load_library()
    G, rl = I(), I()
    _ck_free(lib.ima_ti_read_binary(os.fsencode(path), C.byref(G), C.byref(rl), None, 0), "ti_read_binary")
    rows = np.zeros((G.value, rl.value), np.float32)
    G2, rl2 = I(), I(rl.value)
    _ck_free(lib.ima_ti_read_binary(os.fsencode(path), C.byref(G2), C.byref(rl2), _ptr(rows), G.value),
             "ti_read_binary")
    return rows[:G2.value]


class MT19937(C.Structure):
    """The reference's MT19937 generator state (ima_mt19937)."""
    _fields_ = [("mt", C.c_uint32 * 624), ("mti", C.c_int)]

    def __init__(self, seed=None):
        super().__init__()
        if seed is not None:
            load_library().ima_mt19937_seed(C.byref(self), int(seed))

    def uniform(self):
        return load_library().ima_mt19937_uniform(C.byref(self))


class UgRng(C.Structure):
    """A chain's generators for the genealogy update (ima_ug_rng): the
    MT19937 of uniform(), normdev's cached deviate and bitran's register."""
    _fields_ = [("mt", MT19937), ("iset", C.c_int32), ("gset", C.c_double), ("iseed", C.c_uint64)]

    def __init__(self, seed=None):
        super().__init__()
        if seed is not None:
            load_library().ima_ug_rng_seed(C.byref(self), int(seed))


# double uniform(void *arg): the caller's generator, drawn one value at a time
UNIFORM_FN = C.CFUNCTYPE(C.c_double, C.c_void_p)


class ImaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def load_library(path: str = LIB_PATH):
    """Loads the compiled library; fails loudly when it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImaError(IMA_ERR_STATE, f"{path} is missing: build it with ima2p_gb300.build "
                                      "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(path)
    _declare(lib)
    _lib = lib
    return lib


P = C.c_void_p
I = C.c_int
D = C.c_double


def _declare(L):
    sig = {
        "ima_gpu_create": (I, [I, C.POINTER(P)]),
        "ima_gpu_destroy": (None, [P]),
        "ima_gpu_error": (C.c_char_p, [P]),
        "ima_gpu_synchronize": (I, [P]),
        "ima_gpu_add_locus_is": (I, [P, I, I, P, C.POINTER(I)]),
        "ima_gpu_add_locus_hky": (I, [P, I, I, I, P, P, C.POINTER(I)]),
        "ima_gpu_add_locus_sw": (I, [P, I, I, C.POINTER(I)]),
        "ima_gpu_set_chains": (I, [P, I, I]),
        "ima_gpu_set_genealogy": (I, [P, I, I, P, P, P, P, D]),
        "ima_gpu_set_genealogies": (I, [P, I, P, P, P, P, P, P, P]),
        "ima_gpu_set_pi": (I, [P, I, I, P]),
        "ima_gpu_set_alleles": (I, [P, I, I, I, P]),
        "ima_gpu_likelihoodIS": (I, [P, I, I, D, P]),
        "ima_gpu_likelihoodHKY": (I, [P, I, I, D, D, I, I, I, I, P]),
        "ima_gpu_copyfraclike": (I, [P, I, I]),
        "ima_gpu_storescalefactors": (I, [P, I, I]),
        "ima_gpu_restorescalefactors": (I, [P, I, I]),
        "ima_gpu_likelihoodSW": (I, [P, I, I, I, D, D, P]),
        "ima_gpu_get_dlikeA": (I, [P, I, I, I, P]),
        "ima_gpu_eval": (I, [P, I, P, P, P, P, P, P, I, P, P]),
        "ima_gpu_commit": (I, [P, I, P, P, P]),
        "ima_gpu_batch_create": (I, [P, I, P, P, P, P, P, P, I, C.POINTER(I)]),
        "ima_gpu_batch_run": (I, [P, I, I]),
        "ima_gpu_batch_results": (I, [P, I, P, P]),
        "ima_gpu_batch_destroy": (I, [P, I]),
        "ima_gpu_flush_genealogies": (I, [P]),
        "ima_gpu_setheat": (I, [P, D, D, I]),
        "ima_gpu_get_betas": (I, [P, P]),
        "ima_gpu_set_betas": (I, [P, P]),
        "ima_gpu_set_pdg": (I, [P, P]),
        "ima_gpu_get_pdg": (I, [P, P]),
        "ima_gpu_set_probg": (I, [P, P]),
        "ima_gpu_get_probg": (I, [P, P]),
        "ima_gpu_get_split_times": (I, [P, P]),
        "ima_gpu_checkpoint_write": (I, [P, C.c_char_p, P]),
        "ima_gpu_checkpoint_read": (I, [P, C.c_char_p, P]),
        "ima_gpu_popmig": (I, [P, I, P, P, P, P, P, P, I, P]),
        "ima_gpu_popmig_curves": (I, [P, I, P, P, I, P, P, P, I, P, P, P]),
        "ima_gpu_changet_ry1_sweep_mt": (I, [P, I, P, P, P, P, P, D, P, P, I, P, P, P, P]),
        "ima_ug_rng_seed": (None, [P, C.c_int32]),
        "ima_gpu_updategenealogy_sweep": (I, [P, I, P, P, I, P, P, P, D, I, P, P, P, P]),
        "ima_gpu_get_genealogy": (I, [P, I, I, P, P, P, P, P]),
        "ima_gpu_get_alleles": (I, [P, I, I, I, P]),
        "ima_gpu_findmarginpeaks": (I, [P, P, P, P, P, P, I, P, P, P, P, P, P, P, P, P, P, P, C.POINTER(I)]),
        "ima_gpu_swapchains": (I, [P, I, I, P, I, C.c_uint64, P, P]),
        "ima_gpu_get_swapcounts": (I, [P, I, P, P]),
        "ima_gpu_surface_load": (I, [P, I, I, P, I, I, I, P]),
        "ima_gpu_surface_eval": (I, [P, I, P, I, I, P, P]),
        "ima_gpu_jointp": (I, [P, P, I, P, P]),
        "ima_gpu_batch_autotune": (I, [P, I, I, C.POINTER(I), C.POINTER(I)]),
        "ima_ti_read": (I, [I, P, I, I, P, I, C.POINTER(I), C.POINTER(I)]),
        "ima_ti_write_binary": (I, [C.c_char_p, I, I, P]),
        "ima_ti_read_binary": (I, [C.c_char_p, C.POINTER(I), C.POINTER(I), P, I]),
        "ima_gpu_margincalc": (I, [P, I, P, P, D, I, P, P]),
        "ima_gpu_set_popmodel": (I, [P, I, I, I, P, P, P, P, P, I, P, P, P, P, I, P, P, P, P, P, I, P]),
        "ima_gpu_treeweight": (I, [P, I, P, P, P, P, P, P, P, P, P, I, P, P, I, P, P, P, P, P, P, P, P]),
        "ima_gpu_tree_prob": (I, [P, I, P, P, P, P, P, P, P]),
        "ima_gpu_surface_append_tree_rows": (I, [P, I, P]),
        "ima_gpu_surface_get_rows": (I, [P, I, I, I, P]),
        "ima_gpu_set_locus_pops": (I, [P, P, P]),
        "ima_gpu_set_labels": (I, [P, I, P, P, P, P, P, P]),
        "ima_gpu_get_times": (I, [P, I, I, P, P, P]),
        "ima_gpu_rubber_band": (I, [P, I, P, P, P, P, P, P, I, P]),
        "ima_gpu_chain_weights": (I, [P, I, P, P, P, P, P]),
        "ima_gpu_changet_ry1_sweep": (I, [P, I, P, P, P, P, P, P, P, P, P, D, P, P, P, I, P, P, P]),
        "ima_gpu_fillvec": (I, [P, I, P, P, P, P, P]),
        "ima_gpu_batch_set_variants": (I, [P, I, I, I]),
        "ima_gpu_set_allele_edits": (I, [P, I, P, P, P, P, P]),
        "ima_gpu_surface_info": (I, [P, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(I)]),
        "ima_mt19937_seed": (None, [P, C.c_uint32]),
        "ima_mt19937_uniform": (D, [P]),
        "ima_gpu_modelloop": (I, [P, I, P, I, P, I, I, P, P, P, C.POINTER(I), C.POINTER(I)]),
        "ima_gpu_surface_fp64_noalloc": (I, [P, I, I, I, I, I, P, P, I, I, P, P, P]),
        "ima_gpu_swapchains_cb": (I, [P, I, I, UNIFORM_FN, P, P, P]),
        "ima_gpu_surface_retaken": (I, [P, C.POINTER(I)]),
        "ima_gpu_batch_sweep": (I, [P, I, P, I, I, C.c_uint64, I]),
        "ima_gpu_set_times": (I, [P, I, P, P, P, P]),
        "ima_gpu_eval_times": (I, [P, I, P, P, P, P, P, P, P, I, P, P]),
        "ima_gpu_tc_selftest": (I, [P, C.POINTER(I), C.POINTER(C.c_float)]),
        "ima_gpu_timer_begin": (I, [P]),
        "ima_gpu_timer_end": (I, [P, C.POINTER(C.c_float)]),
        "ima_gpu_set_profiling": (I, [P, I]),
        "ima_gpu_kernel_stats": (I, [P, I, C.POINTER(C.c_longlong), C.POINTER(D), C.POINTER(D)]),
        "ima_gpu_launch_count": (I, [P, C.POINTER(C.c_longlong)]),
        "ima_gpu_flush_l2": (I, [P]),
        "ima_gpu_memory": (I, [P, C.POINTER(C.c_size_t)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _addr(a):
    """The address as an int (cheaper per call than _ptr).  Only for arrays
    a caller holds in a variable for the duration of the call: unlike _ptr's
    pointer object, an int keeps no reference to a temporary array."""
    return None if a is None else a.ctypes.data


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class Context:
    """One device context: resident loci, chains, genealogies and surface."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = P()
        rc = self.lib.ima_gpu_create(device, C.byref(h))
        if rc != IMA_OK:
            raise ImaError(rc, "ima_gpu_create failed (no usable CUDA device?)")
        self.h = h
        self.loci = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.ima_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc):
        if rc != IMA_OK:
            raise ImaError(rc, self.lib.ima_gpu_error(self.h).decode())

    # ------------------------------------------------------------ loci
    def add_locus_is(self, seq):
        seq = np.ascontiguousarray(seq, np.int8)
        li = I()
        self._ck(self.lib.ima_gpu_add_locus_is(self.h, seq.shape[0], seq.shape[1], _ptr(seq), C.byref(li)))
        self.loci.append((MODEL_IS, seq.shape[0]))
        return li.value

    def add_locus_hky(self, seq, mult, totsites):
        seq = np.ascontiguousarray(seq, np.int8)
        mult = _i32(mult)
        li = I()
        self._ck(self.lib.ima_gpu_add_locus_hky(self.h, seq.shape[0], seq.shape[1], int(totsites),
                                                 _ptr(seq), _ptr(mult), C.byref(li)))
        self.loci.append((MODEL_HKY, seq.shape[0]))
        return li.value

    def add_locus_sw(self, numgenes, nlinked=1):
        li = I()
        self._ck(self.lib.ima_gpu_add_locus_sw(self.h, int(numgenes), int(nlinked), C.byref(li)))
        self.loci.append((MODEL_SW, numgenes))
        return li.value

    def set_chains(self, nruns, chains_per_run):
        self._ck(self.lib.ima_gpu_set_chains(self.h, int(nruns), int(chains_per_run)))
        self.nruns, self.cpr = nruns, chains_per_run
        self.nchains = nruns * chains_per_run

    # -------------------------------------------------------- genealogy
    def set_genealogy(self, ci, li, g, length=None):
        self._ck(self.lib.ima_gpu_set_genealogy(
            self.h, int(ci), int(li), _ptr(_i32(g.up0)), _ptr(_i32(g.up1)), _ptr(_i32(g.down)),
            _ptr(_f64(g.time)), -1.0 if length is None else float(length)))

    def set_genealogies(self, ci, li, up0, up1, down, time, length=None):
        """Packed form: node arrays of all pairs concatenated in pair order."""
        ci, li = _i32(ci), _i32(li)
        self._ck(self.lib.ima_gpu_set_genealogies(
            self.h, len(ci), _ptr(ci), _ptr(li), _ptr(_i32(up0)), _ptr(_i32(up1)), _ptr(_i32(down)),
            _ptr(_f64(time)), _ptr(_f64(length))))

    def set_times(self, ci, li, time, length=None):
        """New node times of genealogies whose topology is unchanged (packed as in set_genealogies)."""
        ci, li = _i32(ci), _i32(li)
        self._ck(self.lib.ima_gpu_set_times(self.h, len(ci), _ptr(ci), _ptr(li), _ptr(_f64(time)),
                                            _ptr(_f64(length))))

    def eval_times(self, ci, li, time, u, kappa=None, ai=None, length=None, precision=PREC_FAST):
        """set_times then eval of the same pairs in one call (full evaluations)."""
        ci, li, u = _i32(ci), _i32(li), _f64(u)
        n = len(ci)
        kappa, ai = _f64(kappa), _i32(ai)
        time, length = _f64(time), _f64(length)
        res = np.empty(n)
        st = np.empty(n, np.int32)
        self._ck(self.lib.ima_gpu_eval_times(self.h, n, _addr(ci), _addr(li), _addr(time), _addr(length), _addr(u),
                                             _addr(kappa), _addr(ai), int(precision), _addr(res), _addr(st)))
        return res, st

    def set_pi(self, ci, li, pi):
        self._ck(self.lib.ima_gpu_set_pi(self.h, int(ci), int(li), _ptr(_f64(pi))))

    def set_alleles(self, ci, li, A, ai=0):
        self._ck(self.lib.ima_gpu_set_alleles(self.h, int(ci), int(li), int(ai), _ptr(_i32(A))))

    def get_alleles(self, ci, li, nlines, ai=0):
        """The resident allele states of a stepwise chain-locus's marker."""
        A = np.zeros(nlines, np.int32)
        self._ck(self.lib.ima_gpu_get_alleles(self.h, int(ci), int(li), int(ai), _ptr(A)))
        return A

    def set_allele_edits(self, ci, li, node, A, ai=None):
        """Edit list of single allele states (ima_gpu_set_allele_edits)."""
        ci, li, node, A = _i32(ci), _i32(li), _i32(node), _i32(A)
        ai = _i32(np.zeros(len(ci)) if ai is None else ai)
        self._ck(self.lib.ima_gpu_set_allele_edits(self.h, len(ci), _ptr(ci), _ptr(li), _ptr(ai), _ptr(node),
                                                   _ptr(A)))

    def flush_genealogies(self):
        self._ck(self.lib.ima_gpu_flush_genealogies(self.h))

    # -------------------------------------------- reference mirrors
    def likelihoodIS(self, ci, li, mutrate):
        out = np.zeros(1)
        self._ck(self.lib.ima_gpu_likelihoodIS(self.h, int(ci), int(li), float(mutrate), _ptr(out)))
        return float(out[0])

    def likelihoodHKY(self, ci, li, mutrate, kappa, e1=-1, e2=-1, e3=-1, e4=-1):
        out = np.zeros(1)
        self._ck(self.lib.ima_gpu_likelihoodHKY(self.h, int(ci), int(li), float(mutrate), float(kappa),
                                                 int(e1), int(e2), int(e3), int(e4), _ptr(out)))
        return float(out[0])

    def copyfraclike(self, ci, li):
        self._ck(self.lib.ima_gpu_copyfraclike(self.h, int(ci), int(li)))

    def storescalefactors(self, ci, li):
        self._ck(self.lib.ima_gpu_storescalefactors(self.h, int(ci), int(li)))

    def restorescalefactors(self, ci, li):
        self._ck(self.lib.ima_gpu_restorescalefactors(self.h, int(ci), int(li)))

    def likelihoodSW(self, ci, li, ai, u, tr=1.0):
        out = np.zeros(1)
        self._ck(self.lib.ima_gpu_likelihoodSW(self.h, int(ci), int(li), int(ai), float(u), float(tr), _ptr(out)))
        return float(out[0])

    def get_dlikeA(self, ci, li, ai=0):
        n = self.loci[li][1]
        out = np.zeros(2 * n - 1)
        self._ck(self.lib.ima_gpu_get_dlikeA(self.h, int(ci), int(li), int(ai), _ptr(out)))
        return out

    # -------------------------------------------------------- batched
    def eval(self, ci, li, u, kappa=None, edits=None, ai=None, precision=PREC_FAST):
        ci, li, u = _i32(ci), _i32(li), _f64(u)
        n = len(ci)
        kappa, ai = _f64(kappa), _i32(ai)
        edits = None if edits is None else _i32(edits).reshape(n, 4)
        res = np.empty(n)
        st = np.empty(n, np.int32)
        self._ck(self.lib.ima_gpu_eval(self.h, n, _addr(ci), _addr(li), _addr(u), _addr(kappa), _addr(edits),
                                       _addr(ai), int(precision), _addr(res), _addr(st)))
        return res, st

    def commit(self, ci, li, accept):
        ci, li = _i32(ci), _i32(li)
        acc = np.ascontiguousarray(accept, np.uint8)
        self._ck(self.lib.ima_gpu_commit(self.h, len(ci), _ptr(ci), _ptr(li), _ptr(acc)))

    def batch_create(self, ci, li, u, kappa=None, edits=None, ai=None, precision=PREC_FAST):
        ci, li, u = _i32(ci), _i32(li), _f64(u)
        n = len(ci)
        kappa, ai = _f64(kappa), _i32(ai)
        edits = None if edits is None else _i32(edits).reshape(n, 4)
        b = I()
        self._ck(self.lib.ima_gpu_batch_create(self.h, n, _ptr(ci), _ptr(li), _ptr(u), _ptr(kappa),
                                               _ptr(edits), _ptr(ai), int(precision), C.byref(b)))
        return Batch(self, b.value, n)

    # ----------------------------------------------------------- MC3
    def setheat(self, hval1, hval2, heatmode):
        self._ck(self.lib.ima_gpu_setheat(self.h, float(hval1), float(hval2), int(heatmode)))

    def get_betas(self):
        out = np.zeros(self.nchains)
        self._ck(self.lib.ima_gpu_get_betas(self.h, _ptr(out)))
        return out

    def set_betas(self, beta):
        self._ck(self.lib.ima_gpu_set_betas(self.h, _ptr(_f64(beta))))

    def set_pdg(self, pdg):
        self._ck(self.lib.ima_gpu_set_pdg(self.h, _ptr(_f64(pdg))))

    def get_pdg(self):
        out = np.zeros((self.nchains, len(self.loci)))
        self._ck(self.lib.ima_gpu_get_pdg(self.h, _ptr(out)))
        return out

    def set_probg(self, probg):
        self._ck(self.lib.ima_gpu_set_probg(self.h, _ptr(_f64(probg))))

    def get_probg(self):
        out = np.zeros(self.nchains)
        self._ck(self.lib.ima_gpu_get_probg(self.h, _ptr(out)))
        return out

    def swapchains(self, swaptries, include_probg=True, uniforms=None, seed=0):
        """uniforms: [nruns, stride] per-run streams, or None for Philox."""
        used = np.zeros(self.nruns, np.int32)
        ok = np.zeros(self.nruns, np.int32)
        if uniforms is not None:
            uniforms = _f64(uniforms).reshape(self.nruns, -1)
            stride = uniforms.shape[1]
        else:
            stride = 0
        self._ck(self.lib.ima_gpu_swapchains(self.h, int(swaptries), int(include_probg), _ptr(uniforms),
                                             int(stride), int(seed), _ptr(used), _ptr(ok)))
        return ok, used

    def surface_retaken(self):
        """Points the last tensor-core surface evaluation took a second time."""
        n = I()
        self._ck(self.lib.ima_gpu_surface_retaken(self.h, C.byref(n)))
        return n.value

    def swapchains_cb(self, swaptries, uniform, include_probg=True):
        """Swap attempts drawing uniform() one value at a time, where the
        reference draws (ima_gpu_swapchains_cb): returns (swap0ok, draws)
        per run."""
        used = np.zeros(self.nruns, np.int32)
        ok = np.zeros(self.nruns, np.int32)
        cb = UNIFORM_FN(lambda _arg: float(uniform()))
        self._ck(self.lib.ima_gpu_swapchains_cb(self.h, int(swaptries), int(include_probg), cb, None, _ptr(used),
                                                _ptr(ok)))
        return ok, used

    def get_swapcounts(self, run=0):
        sc = np.zeros((self.cpr, self.cpr), np.int32)
        tc = np.zeros((self.cpr, self.cpr), np.int32)
        self._ck(self.lib.ima_gpu_get_swapcounts(self.h, int(run), _ptr(sc), _ptr(tc)))
        return sc, tc

    # ------------------------------------------------------- surface
    def surface_load(self, rows, numpopsizeparams, nummigrateparams, npops, lognorm=None):
        rows = np.ascontiguousarray(rows, np.float32)
        self.surf_npar = numpopsizeparams + nummigrateparams
        self._ck(self.lib.ima_gpu_surface_load(self.h, rows.shape[0], rows.shape[1], _ptr(rows),
                                               int(numpopsizeparams), int(nummigrateparams), int(npops),
                                               _ptr(_f64(lognorm))))

    def surface_eval(self, x, modeltype=0, method=SURF_TC):
        x = _f64(x).reshape(-1, self.surf_npar)
        q = np.zeros(len(x))
        ess = np.zeros(len(x))
        self._ck(self.lib.ima_gpu_surface_eval(self.h, len(x), _ptr(x), int(modeltype), int(method),
                                               _ptr(q), _ptr(ess)))
        return q, ess

    def tc_selftest(self):
        bad = I()
        err = C.c_float()
        self._ck(self.lib.ima_gpu_tc_selftest(self.h, C.byref(bad), C.byref(err)))
        return bad.value, err.value

    def jointp(self, x, calc_ess=1):
        q = np.zeros(1)
        e = np.zeros(1)
        self._ck(self.lib.ima_gpu_jointp(self.h, _ptr(_f64(x)), int(calc_ess), _ptr(e), _ptr(q)))
        return float(q[0]), float(e[0])

    def margincalc(self, param, x, yadjust=0.0, logi=0, expo_mean=None):
        param, x = _i32(np.atleast_1d(param)), _f64(np.atleast_1d(x))
        out = np.zeros(len(x))
        em = _f64(expo_mean) if expo_mean is not None else None
        self._ck(self.lib.ima_gpu_margincalc(self.h, len(x), _ptr(param), _ptr(x), float(yadjust), int(logi),
                                             _ptr(em) if em is not None else None, _ptr(out)))
        return out

    # ------------------------------------- genealogy weights and p(G)
    def set_popmodel(self, pm, th_max, th_min=None, mg_max=None, mg_min=None, mg_mean=None, expo=False,
                     chk=None):
        """Load a population model (ima2p_gb300.popmodel.PopModel) with the
        priors of its parameters (itheta[].pr, imig[].pr).  chk: the
        migration cells that must stay empty (default: the model's own,
        pm.chk_cells)."""
        if chk is None:
            chk = getattr(pm, "chk_cells", ())
        nth, nmg = len(pm.th_cells), len(pm.mg_cells)
        tho, thi = pm.th_csr()
        mgo, mgi = pm.mg_csr()
        th_max = _f64(np.broadcast_to(np.asarray(th_max, np.float64), (nth,)))
        th_min = _f64(np.zeros(nth) if th_min is None else np.broadcast_to(np.asarray(th_min, np.float64), (nth,)))
        z = np.zeros(max(nmg, 1))
        mg_max = _f64(z if mg_max is None else np.broadcast_to(np.asarray(mg_max, np.float64), (nmg,)))
        mg_min = _f64(z if mg_min is None else np.broadcast_to(np.asarray(mg_min, np.float64), (nmg,)))
        mg_mean = _f64(z if mg_mean is None else np.broadcast_to(np.asarray(mg_mean, np.float64), (nmg,)))
        chk = _i32(np.asarray(chk, np.int32) if len(chk) else np.zeros(1, np.int32))
        keep = [_i32(pm.plist.ravel()), _i32(pm.droppops.ravel()), _i32(pm.addpop), _i32(pm.pop_e),
                _i32(pm.pop_down), tho, _i32(thi if len(thi) else np.zeros(1)), mgo,
                _i32(mgi if len(mgi) else np.zeros(1))]
        self._ck(self.lib.ima_gpu_set_popmodel(
            self.h, pm.npops, int(pm.nomig), int(expo), *(_ptr(a) for a in keep[:5]), nth, _ptr(keep[5]),
            _ptr(keep[6]), _ptr(th_max), _ptr(th_min), nmg, _ptr(keep[7]), _ptr(keep[8]), _ptr(mg_max),
            _ptr(mg_min), _ptr(mg_mean), len(chk) if len(chk) > 1 or chk[0] else 0, _ptr(chk)))
        self._tw_pm = pm

    def treeweight(self, packed, gen_locus, gen_tv, hval, samppop, tvals):
        """treeweight for many genealogies.  packed: (node_off, up0, time, pop,
        mig_off, mig_t, mig_p) as pack_labelled() makes them.  Returns a dict
        of cc, hcc, fc [ngen][T], mc, fm [ngen][M], lens [ngen][2], mignum."""
        pm = self._tw_pm
        node_off, up0, time, pop, mig_off, mig_t, mig_p = packed
        ngen = len(node_off) - 1
        T, M = pm.T, pm.M
        out = {"cc": np.zeros((ngen, T), np.int32), "hcc": np.zeros((ngen, T)), "fc": np.zeros((ngen, T)),
               "mc": np.zeros((ngen, M), np.int32), "fm": np.zeros((ngen, M)), "lens": np.zeros((ngen, 2)),
               "mignum": np.zeros(ngen, np.int32)}
        ins = [_i32(node_off), _i32(up0), _f64(time), _i32(pop), _i32(mig_off),
               _f64(mig_t if len(mig_t) else np.zeros(1)), _i32(mig_p if len(mig_p) else np.zeros(1)),
               _i32(gen_locus), _i32(gen_tv)]
        hval, samppop, tvals = _f64(np.atleast_1d(hval)), _i32(samppop), _f64(np.atleast_2d(tvals))
        self._ck(self.lib.ima_gpu_treeweight(
            self.h, ngen, *(_ptr(a) for a in ins), len(hval), _ptr(hval), _ptr(samppop), len(tvals),
            _ptr(tvals), *(_ptr(out[k]) for k in ("cc", "hcc", "fc", "mc", "fm", "lens", "mignum"))))
        return out

    def tree_prob(self, group_off, pdg=None, group_tv=None, rows=False):
        """p(G) per chain over the genealogies of the last treeweight call:
        returns (probg, q [ngroups][nth], m [ngroups][nmg], rows or None)."""
        pm = self._tw_pm
        group_off = _i32(group_off)
        G = len(group_off) - 1
        nth, nmg = len(pm.th_cells), 0 if pm.nomig else len(pm.mg_cells)
        probg, q, m = np.zeros(G), np.zeros((G, nth)), np.zeros((G, max(nmg, 1)))
        rowbuf = np.zeros((G, 4 * nth + 3 * nmg + 2 + pm.npops - 1), np.float32) if rows else None
        pdg = _f64(pdg) if pdg is not None else None
        gtv = _i32(group_tv) if group_tv is not None else None
        self._ck(self.lib.ima_gpu_tree_prob(self.h, G, _ptr(group_off), _ptr(pdg) if pdg is not None else None,
                                            _ptr(gtv) if gtv is not None else None, _ptr(probg), _ptr(q),
                                            _ptr(m), _ptr(rowbuf) if rows else None))
        return probg, q, m[:, :nmg], rowbuf

    # -------------------- resident labels and the split-time update
    def set_locus_pops(self, hval, samppop):
        """L[li].hval and L[li].samppop of every locus, for the resident
        weights."""
        hval, samppop = _f64(hval), _i32(samppop)
        self._ck(self.lib.ima_gpu_set_locus_pops(self.h, _ptr(hval), _ptr(samppop)))

    def set_labels(self, ci, li, gens):
        """Population labels and migration events (LabelledGenealogy) of the
        chain-loci (ci[k], li[k]), kept on the device."""
        ci, li = _i32(np.atleast_1d(ci)), _i32(np.atleast_1d(li))
        pop = _i32(np.concatenate([g.pop for g in gens]))
        moff = []
        for g in gens:
            o = np.zeros(len(g.mig) + 1, np.int32)
            o[1:] = np.cumsum([len(m) for m in g.mig])
            moff.append(o)
        moff = _i32(np.concatenate(moff))
        mt = _f64(np.array([e[0] for g in gens for m in g.mig for e in m] or [0.0]))
        mp = _i32(np.array([e[1] for g in gens for m in g.mig for e in m] or [0]))
        self._ck(self.lib.ima_gpu_set_labels(self.h, len(ci), _ptr(ci), _ptr(li), _ptr(pop), _ptr(moff),
                                             _ptr(mt), _ptr(mp)))

    def get_times(self, ci, li, nlines):
        """Device node times and migration times (node order) of a chain-locus."""
        t = np.zeros(nlines)
        n = I()
        self._ck(self.lib.ima_gpu_get_times(self.h, int(ci), int(li), _ptr(t), C.byref(n), None))
        m = np.zeros(max(n.value, 1))
        self._ck(self.lib.ima_gpu_get_times(self.h, int(ci), int(li), _ptr(t), C.byref(n), _ptr(m)))
        return t, m[:n.value]

    def rubber_band(self, chains, period, oldt, newt, t_u, t_d, inverse=False):
        """changet_RY1's time moves on every locus of the chains; returns
        [nch][4] = (ecd, ecu, emd, emu) going forward (node counts per edge)."""
        chains, period = _i32(chains), _i32(period)
        arrs = [_f64(v) for v in (oldt, newt, t_u, t_d)]
        counts = np.zeros((len(chains), 4), np.int32)
        self._ck(self.lib.ima_gpu_rubber_band(self.h, len(chains), _ptr(chains), _ptr(period),
                                              *(_ptr(v) for v in arrs), int(inverse), _ptr(counts)))
        return counts

    def chain_weights(self, chains, tvals):
        """Resident weights of every locus of the chains (lengths updated on
        the device) and their p(G): (probg, q, m)."""
        pm = self._tw_pm
        chains = _i32(chains)
        tvals = _f64(np.asarray(tvals, np.float64).reshape(len(chains), -1))
        nth, nmg = len(pm.th_cells), 0 if pm.nomig else len(pm.mg_cells)
        probg, q, m = np.zeros(len(chains)), np.zeros((len(chains), nth)), np.zeros((len(chains), max(nmg, 1)))
        self._ck(self.lib.ima_gpu_chain_weights(self.h, len(chains), _ptr(chains), _ptr(tvals), _ptr(probg),
                                                _ptr(q), _ptr(m)))
        return probg, q, m[:, :nmg]

    def changet_ry1_sweep(self, chains, period, oldt, newt, t_u, t_d, log_hu, log_hd, logU, tvals, u,
                          kappa=None, gbeta=1.0, precision=PREC_FP64):
        """One device-decided changet_RY1 per chain: returns (accept,
        pdgsum, probg) after the decisions."""
        chains, period = _i32(chains), _i32(period)
        f = [_f64(v) for v in (oldt, newt, t_u, t_d, log_hu, log_hd, logU)]
        tvals, u = _f64(tvals), _f64(u)
        kap = _f64(kappa) if kappa is not None else None
        n = len(chains)
        acc, pdgsum, probg = np.zeros(n, np.uint8), np.zeros(n), np.zeros(n)
        self._ck(self.lib.ima_gpu_changet_ry1_sweep(
            self.h, n, _ptr(chains), _ptr(period), *(_ptr(v) for v in f), float(gbeta), _ptr(tvals), _ptr(u),
            _ptr(kap) if kap is not None else None, int(precision), _ptr(acc), _ptr(pdgsum), _ptr(probg)))
        return acc.astype(bool), pdgsum, probg

    def get_split_times(self):
        """The split times the resident labels follow, [nchains][npops-1]."""
        out = np.zeros((self.nchains, self._tw_pm.npops - 1))
        self._ck(self.lib.ima_gpu_get_split_times(self.h, _ptr(out)))
        return out

    def checkpoint_write(self, path, rng=None):
        """The resident chain state (and the generator, if given) to a file."""
        self._ck(self.lib.ima_gpu_checkpoint_write(self.h, os.fsencode(path),
                                                   C.byref(rng) if rng is not None else None))

    def checkpoint_read(self, path, rng=None):
        """Restore a checkpoint_write file into this context (same loci and
        chains; the population model set first when the file holds labels);
        rng, if given, takes the saved generator state."""
        self._ck(self.lib.ima_gpu_checkpoint_read(self.h, os.fsencode(path),
                                                  C.byref(rng) if rng is not None else None))

    def changet_ry1_sweep_mt(self, chains, period, tprior, rng, u, kappa=None, gbeta=1.0, precision=PREC_FP64):
        """changet_ry1_sweep with getnewt's and the acceptance draws made in
        the library from rng (MT19937); tprior [(lo, hi)] per split.
        Returns (accept, pdgsum, probg, newt)."""
        chains, period = _i32(chains), _i32(period)
        tp = np.asarray(tprior, np.float64).reshape(-1, 2)
        lo, hi = _f64(tp[:, 0]), _f64(tp[:, 1])
        u = _f64(u)
        kap = _f64(kappa) if kappa is not None else None
        n = len(chains)
        acc, pdgsum, probg, newt = np.zeros(n, np.uint8), np.zeros(n), np.zeros(n), np.zeros(n)
        self._ck(self.lib.ima_gpu_changet_ry1_sweep_mt(
            self.h, n, _ptr(chains), _ptr(period), _ptr(lo), _ptr(hi), C.byref(rng), float(gbeta), _ptr(u),
            _ptr(kap) if kap is not None else None, int(precision), _ptr(acc), _ptr(pdgsum), _ptr(probg),
            _ptr(newt)))
        return acc.astype(bool), pdgsum, probg, newt

    def updategenealogy_sweep(self, chains, tvals, nsweeps, rngs, u, kappa=None, gbeta=1.0, precision=PREC_FP64,
                              allele_range=None):
        """nsweeps device genealogy updates of every locus of the chains (the
        no-migration model); rngs: a UgRng per chain, advanced in place;
        allele_range [nloci][2]: the SW loci's (minA, maxA).  Returns
        (accepted, topology changes) [nch][nloci] and p(G) [nch]."""
        chains = _i32(chains)
        n, nl = len(chains), len(self.loci)
        tvals = _f64(np.asarray(tvals, np.float64).reshape(n, -1))
        u = _f64(np.asarray(u, np.float64).reshape(-1))
        kap = _f64(np.asarray(kappa, np.float64).reshape(-1)) if kappa is not None else None
        ar = _i32(np.asarray(allele_range).reshape(-1)) if allele_range is not None else None
        arr = (UgRng * n)(*rngs)
        acc, top, probg = np.zeros((n, nl), np.int32), np.zeros((n, nl), np.int32), np.zeros(n)
        self._ck(self.lib.ima_gpu_updategenealogy_sweep(
            self.h, n, _ptr(chains), _ptr(tvals), int(nsweeps), _ptr(u), _ptr(kap) if kap is not None else None,
            _ptr(ar) if ar is not None else None, float(gbeta), int(precision), C.cast(arr, P), _ptr(acc), _ptr(top),
            _ptr(probg)))
        for k in range(n):
            C.memmove(C.addressof(rngs[k]), C.addressof(arr[k]), C.sizeof(UgRng))
        return acc, top, probg

    def get_genealogy(self, ci, li, nlines):
        """The resident genealogy of a chain-locus: (up0, up1, down, time, pop)."""
        up0, up1, down, pop = (np.zeros(nlines, np.int32) for _ in range(4))
        t = np.zeros(nlines)
        self._ck(self.lib.ima_gpu_get_genealogy(self.h, int(ci), int(li), _ptr(up0), _ptr(up1), _ptr(down), _ptr(t),
                                                _ptr(pop)))
        return up0, up1, down, t, pop

    def surface_append_tree_rows(self, groups):
        """Append the gsampinf rows of these chains (last tree_prob) to the
        resident surface."""
        groups = _i32(np.atleast_1d(groups))
        self._ck(self.lib.ima_gpu_surface_append_tree_rows(self.h, len(groups), _ptr(groups)))
        _, np_, nm, _ = self.surface_info()
        self.surf_npar = np_ + nm

    def surface_get_rows(self, start=0, count=None, rowlen=None):
        """Surface rows [start, start+count) ([count][rowlen]; rowlen defaults
        to gsampinf's 4np + 3nm + 2 + npops-1)."""
        G, np_, nm, npops = self.surface_info()
        count = G - start if count is None else count
        rowlen = 4 * np_ + 3 * nm + 2 + npops - 1 if rowlen is None else rowlen
        out = np.zeros((count, rowlen), np.float32)
        self._ck(self.lib.ima_gpu_surface_get_rows(self.h, int(start), int(count), int(rowlen), _ptr(out)))
        return out

    def popmig(self, thetai, mi, x, theta_max, mig_max, mig_mean=None, prob_or_like=0):
        """calc_popmig (calc_pop_expomig with mig_mean) at the points: term
        (thetai[k], mi[k]) at x[k]."""
        x = _f64(np.atleast_1d(x))
        n = len(x)
        th = _i32(np.broadcast_to(np.asarray(thetai), (n,)).copy())
        mi = _i32(np.broadcast_to(np.asarray(mi), (n,)).copy())
        q, m = _f64(theta_max), _f64(mig_max)
        mean = _f64(mig_mean) if mig_mean is not None else None
        y = np.zeros(n)
        self._ck(self.lib.ima_gpu_popmig(self.h, n, _ptr(th), _ptr(mi), _ptr(x), _ptr(q), _ptr(m),
                                         _ptr(mean) if mean is not None else None, int(prob_or_like), _ptr(y)))
        return y

    def popmig_curves(self, terms, theta_max, mig_max, mig_mean=None, prob_or_like=0, gridsize=1000):
        """The 2NM curves of the (thetai, mi) terms: (x [nt][gridsize],
        y [nt][gridsize], maxx [nt])."""
        terms = np.asarray(terms, np.int32).reshape(-1, 2)
        nt = len(terms)
        th, mi = _i32(terms[:, 0]), _i32(terms[:, 1])
        q, m = _f64(theta_max), _f64(mig_max)
        mean = _f64(mig_mean) if mig_mean is not None else None
        xs, ys, mx = np.zeros((nt, gridsize)), np.zeros((nt, gridsize)), np.zeros(nt)
        self._ck(self.lib.ima_gpu_popmig_curves(self.h, nt, _ptr(th), _ptr(mi), int(gridsize), _ptr(q), _ptr(m),
                                                _ptr(mean) if mean is not None else None, int(prob_or_like),
                                                _ptr(xs), _ptr(ys), _ptr(mx)))
        return xs, ys, mx

    def findmarginpeaks(self, theta_min, theta_max, mig_min, mig_max, mig_mean=None, terms=()):
        """findmarginpeaks' numbers: dict of mlval, peakloc ([3][np+nm]),
        migtest, lo95, hi95, pm_mlval, pm_peakloc ([3][nterms]), pm_test,
        holdpeakloc and rounds; terms = [(thetai, mi)] 2NM terms."""
        _, np_, nm, _ = self.surface_info()
        terms = np.asarray(terms, np.int32).reshape(-1, 2)
        nt = len(terms)
        mpop, mterm = _i32(terms[:, 0]), _i32(terms[:, 1])
        f = lambda v: _f64(v) if v is not None else None  # noqa: E731
        tmin, tmax, mmin, mmax, mean = f(theta_min), f(theta_max), f(mig_min), f(mig_max), f(mig_mean)
        o = {"mlval": np.zeros((3, np_ + nm)), "peakloc": np.zeros((3, np_ + nm)), "migtest": np.zeros(max(nm, 1)),
             "lo95": np.zeros(np_ + nm), "hi95": np.zeros(np_ + nm), "pm_mlval": np.zeros((3, max(nt, 1))),
             "pm_peakloc": np.zeros((3, max(nt, 1))), "pm_test": np.zeros(max(nt, 1)),
             "holdpeakloc": np.zeros(np_ + nm, np.float32)}
        rounds = I()
        self._ck(self.lib.ima_gpu_findmarginpeaks(
            self.h, _ptr(tmin), _ptr(tmax), _ptr(mmin), _ptr(mmax), _ptr(mean), nt, _ptr(mpop), _ptr(mterm),
            _ptr(o["mlval"]), _ptr(o["peakloc"]), _ptr(o["migtest"]), _ptr(o["lo95"]), _ptr(o["hi95"]),
            _ptr(o["pm_mlval"]) if nt else None, _ptr(o["pm_peakloc"]) if nt else None,
            _ptr(o["pm_test"]) if nt else None, _ptr(o["holdpeakloc"]), C.byref(rounds)))
        o["migtest"] = o["migtest"][:nm]
        o["pm_mlval"], o["pm_peakloc"], o["pm_test"] = o["pm_mlval"][:, :nt], o["pm_peakloc"][:, :nt], o["pm_test"][:nt]
        o["rounds"] = rounds.value
        return o

    def fillvec(self, pmin, pmax, gridsize=1000, expo_mean=None):
        n = len(pmin)
        xs = np.zeros((n, gridsize))
        ys = np.zeros((n, gridsize))
        em = _f64(expo_mean) if expo_mean is not None else None
        self._ck(self.lib.ima_gpu_fillvec(self.h, int(gridsize), _ptr(_f64(pmin)), _ptr(_f64(pmax)),
                                          _ptr(em) if em is not None else None, _ptr(xs), _ptr(ys)))
        return xs, ys

    def surface_info(self):
        G, np_, nm, npops = I(), I(), I(), I()
        self._ck(self.lib.ima_gpu_surface_info(self.h, C.byref(G), C.byref(np_), C.byref(nm), C.byref(npops)))
        return G.value, np_.value, nm.value, npops.value

    def modelloop(self, upper, modeltype=0, rng=None, seed=1234, multiplier=100, xmap=None, nested=0,
                  method=SURF_COMPAT):
        """modelloop (jointfind.cpp:746-812): the DE peak search over the
        loaded surface.  rng: an MT19937 state (continues across calls);
        returns (best[n+1], ess, generations, restarts, rng)."""
        rng = rng if rng is not None else MT19937(seed)
        n = sum(self.surface_info()[1:3])
        best = np.zeros(n + 1)
        ess = np.zeros(1)
        gens, runs = I(), I()
        xm = _f64(xmap) if xmap is not None else None
        self._ck(self.lib.ima_gpu_modelloop(self.h, int(modeltype), _ptr(_f64(upper)), int(multiplier),
                                            _ptr(xm) if xm is not None else None, int(nested), int(method),
                                            C.byref(rng), _ptr(best), _ptr(ess), C.byref(gens), C.byref(runs)))
        return best, float(ess[0]), gens.value, runs.value, rng

    # --------------------------------------------------- measurement
    def synchronize(self):
        self._ck(self.lib.ima_gpu_synchronize(self.h))

    def timer_begin(self):
        self._ck(self.lib.ima_gpu_timer_begin(self.h))

    def timer_end(self):
        ms = C.c_float()
        self._ck(self.lib.ima_gpu_timer_end(self.h, C.byref(ms)))
        return ms.value

    def set_profiling(self, on):
        self._ck(self.lib.ima_gpu_set_profiling(self.h, int(on)))

    def kernel_stats(self, kind):
        n = C.c_longlong()
        ms = D()
        by = D()
        self._ck(self.lib.ima_gpu_kernel_stats(self.h, int(kind), C.byref(n), C.byref(ms), C.byref(by)))
        return n.value, ms.value, by.value

    def launch_count(self):
        n = C.c_longlong()
        self._ck(self.lib.ima_gpu_launch_count(self.h, C.byref(n)))
        return n.value

    def flush_l2(self):
        self._ck(self.lib.ima_gpu_flush_l2(self.h))

    def memory(self):
        n = C.c_size_t()
        self._ck(self.lib.ima_gpu_memory(self.h, C.byref(n)))
        return n.value


IMA_ERR_TOO_LARGE = -7


def surface_fp64_noalloc(rows_ptr, G, rowlen, np_, nm, npops, lognorm_ptr, x_ptr, npoints,
                         modeltype, q_ptr, ess_ptr, stream=None):
    """The allocation-free FP64 surface on caller-owned device pointers (ints);
    returns the library status code.  For callers that cannot allocate device
    memory; see include/ima_gpu.h for its scratch limit."""
    lib = load_library()
    return lib.ima_gpu_surface_fp64_noalloc(rows_ptr, G, rowlen, np_, nm, npops, lognorm_ptr, x_ptr,
                                            npoints, modeltype, q_ptr, ess_ptr, stream)


class Batch:
    """Requests staged on the device; run() replays them (optionally as a graph)."""

    def __init__(self, ctx, handle, n):
        self.ctx, self.handle, self.n = ctx, handle, n

    def autotune(self, reps=5):
        """ima_gpu_batch_autotune: returns the chosen (hky, sw) launch variants."""
        h, w = I(), I()
        self.ctx._ck(self.ctx.lib.ima_gpu_batch_autotune(self.ctx.h, self.handle, int(reps), C.byref(h), C.byref(w)))
        return h.value, w.value

    def set_variants(self, hky=0, sw=0):
        self.ctx._ck(self.ctx.lib.ima_gpu_batch_set_variants(self.ctx.h, self.handle, int(hky), int(sw)))

    def run(self, use_graph=True):
        self.ctx._ck(self.ctx.lib.ima_gpu_batch_run(self.ctx.h, self.handle, int(use_graph)))

    def sweep(self, swaptries, accept=None, include_probg=True, seed=0, use_graph=True):
        """ima_gpu_batch_sweep: every request evaluated, the accepted ones
        (all when accept is None) committed, then every run's swap attempts on
        the device's Philox stream -- one graph launch with use_graph."""
        acc = None if accept is None else np.ascontiguousarray(accept, np.uint8)
        self.ctx._ck(self.ctx.lib.ima_gpu_batch_sweep(self.ctx.h, self.handle, _ptr(acc), int(swaptries),
                                                      int(include_probg), int(seed), int(use_graph)))

    def results(self):
        res = np.zeros(self.n)
        st = np.zeros(self.n, np.int32)
        self.ctx._ck(self.ctx.lib.ima_gpu_batch_results(self.ctx.h, self.handle, _ptr(res), _ptr(st)))
        return res, st

    def destroy(self):
        if self.handle is not None:
            self.ctx._ck(self.ctx.lib.ima_gpu_batch_destroy(self.ctx.h, self.handle))
            self.handle = None


def pack_labelled(gens):
    """CSR arrays of ima_gpu_treeweight from a list of LabelledGenealogy:
    (node_off, up0, time, pop, mig_off, mig_t, mig_p)."""
    node_off = np.zeros(len(gens) + 1, np.int32)
    node_off[1:] = np.cumsum([len(g.pop) for g in gens])
    up0 = np.concatenate([g.g.up0 for g in gens]).astype(np.int32)
    time = np.concatenate([g.g.time for g in gens]).astype(np.float64)
    pop = np.concatenate([g.pop for g in gens]).astype(np.int32)
    counts = [len(m) for g in gens for m in g.mig]
    mig_off = np.zeros(len(counts) + 1, np.int32)
    mig_off[1:] = np.cumsum(counts)
    mig_t = np.array([e[0] for g in gens for m in g.mig for e in m], np.float64)
    mig_p = np.array([e[1] for g in gens for m in g.mig for e in m], np.int32)
    return node_off, up0, time, pop, mig_off, mig_t, mig_p
