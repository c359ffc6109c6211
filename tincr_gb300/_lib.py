"""ctypes binding of the C ABI declared in include/tincr_gb300.h.

The shared library is built in-tree (`tincr_gb300/lib/libtincr_gb300.so`, see build.py).  There
is no CPU fallback: if the library cannot be loaded every entry point raises.
"""

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libtincr_gb300.so")

OK, NOT_CONVERGED, NONFINITE, BAD_ARG, CUDA_ERR, NO_DEVICE, CG_MAXITER = range(7)
STATUS_NAMES = {0: "OK", 1: "NOT_CONVERGED", 2: "NONFINITE", 3: "BAD_ARG", 4: "CUDA_ERR", 5: "NO_DEVICE",
                6: "CG_MAXITER"}
PREC_FP64, PREC_BF16X3 = 0, 1
KF_AO_EXCHANGE, KF_AO_TRANSFORM, KF_SUBSPACE, KF_GRADIENT, KF_OTHER, KF_HOST, KF_EIGEN, KF_DIGITS = range(8)
KF_COUNT = 8
GRAD_REFERENCE, GRAD_EXACT = 0, 1
GRAD_SK_EXTRAPOLATE = 16   # flag OR-ed into a variant: SK splines extrapolated beyond their grid
SCC_LC, SCC_SK_EXTRAPOLATE, SCC_FP32_START = 1, 2, 4

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

# name -> (restype, argtypes); must match include/tincr_gb300.h
SIGNATURES = {
    "tincr_ctx_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "tincr_ctx_destroy": (C.c_int, [C.c_void_p]),
    "tincr_last_error": (C.c_char_p, [C.c_void_p]),
    "tincr_last_timing": (C.c_int, [C.c_void_p, _dp, C.POINTER(C.c_longlong)]),
    "tincr_tda_set_states": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp]),
    "tincr_last_solve_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), _ip, _dp]),
    "tincr_set_precision": (C.c_int, [C.c_void_p, C.c_int]),
    "tincr_tda_solve_batch": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_void_p]),
    "tincr_batch_tile_table": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, _dp]),
    "tincr_davidson_history": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, _ip, _dp, _ip, _ip]),
    "tincr_subspace_eigh": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _ip]),
    "tincr_gemm_fp64_tensor": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]),
    "tincr_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "tincr_debug_tc_first_wait": (C.c_int, [C.c_void_p, C.c_longlong]),
    "tincr_kernel_stats": (C.c_int, [C.c_void_p, C.c_int, _dp, C.POINTER(C.c_longlong), _dp, _dp]),
    "tincr_trans_charges": (C.c_int, [C.c_void_p, C.c_int, _ip, C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_int,
                                      C.c_int, _dp, _dp, _dp]),
    "tincr_tda_setup": (C.c_int, [C.c_void_p, C.c_int, _ip, C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, _dp, _dp,
                                  _dp]),
    "tincr_tda_products": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, C.c_int]),
    "tincr_tda_products_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "tincr_exciton_states": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                       C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_double, C.c_int, _dp, _dp, _dp,
                                       _ip]),
    "tincr_tda_solve": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, _dp, _dp, _dp, _dp, _dp,
                                  _ip]),
    "tincr_set_parameters": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, _ip, _ip, _dp, _dp, C.c_int, _dp, _dp,
                                       C.c_int, _ip, _dp, _dp, _dp]),
    "tincr_gradient": (C.c_int, [C.c_void_p, _ip, C.c_double, _dp, _dp, _dp, C.c_int, C.c_int, _dp, _dp, _ip]),
    "tincr_rpa_solve": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, _dp, _dp, _dp, _dp, _ip]),
    "tincr_scc_batch": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, _ip, _dp, _dp, C.c_void_p, _dp, C.c_double,
                                  C.c_int, C.c_double, C.c_int, C.c_double, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                  _ip, _ip, _dp]),
}

_lib = None


class TincrError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


def load(path=LIB_PATH):
    """Load the CUDA library (raises OSError when it is missing: no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError("tincr_gb300 CUDA library not built: %s (run tincr_gb300.build.build())" % path)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_ip)


def f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class Context:
    """Owns one `tincr_ctx` (one GPU, one system)."""

    def __init__(self, device=0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.tincr_ctx_create(C.byref(h), int(device))
        if rc != OK:
            raise TincrError(rc, "tincr_ctx_create(device=%d) failed" % device)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.tincr_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc, allow=(OK,)):
        if rc not in allow:
            raise TincrError(rc, (self.lib.tincr_last_error(self.h) or b"").decode())
        return rc

    def set_profiling(self, on=True):
        self.check(self.lib.tincr_set_profiling(self.h, 1 if on else 0))

    def kernel_stats(self, family):
        ms, fl, by = C.c_double(), C.c_double(), C.c_double()
        n = C.c_longlong()
        self.check(self.lib.tincr_kernel_stats(self.h, int(family), C.byref(ms), C.byref(n), C.byref(fl),
                                               C.byref(by)))
        return dict(ms=ms.value, launches=n.value, flops=fl.value, bytes=by.value)

    def last_solve_stats(self):
        n = C.c_longlong()
        k = C.c_int()
        r = C.c_double()
        self.check(self.lib.tincr_last_solve_stats(self.h, C.byref(n), C.byref(k), C.byref(r)))
        return dict(n_products=n.value, n_collapses=k.value, max_residual=r.value)

    def davidson_history(self):
        """Records of the last solve: list of dict(iter, n_sub, max_residual, roots_left, precision)."""
        n = C.c_int()
        self.check(self.lib.tincr_davidson_history(self.h, 0, C.byref(n), None, None, None, None, None))
        k = n.value
        it, ns, rl, pr = (np.zeros(k, np.int32) for _ in range(4))
        mr = np.zeros(k)
        self.check(self.lib.tincr_davidson_history(self.h, k, C.byref(n), iptr(it), iptr(ns), dptr(mr), iptr(rl),
                                                   iptr(pr)))
        return [dict(iter=int(it[i]), n_sub=int(ns[i]), max_residual=float(mr[i]), roots_left=int(rl[i]),
                     precision=int(pr[i])) for i in range(k)]

    TILE_SHAPES = ("64x64", "64x32", "32x64", "32x32")
    PLANE_STEPS = ("H", "F", "G", "AX")

    def batch_tile_table(self):
        """The batch autotuner's table: list of dict(n_atoms, n_orb, n_occ, n_virt, lc,
        shapes={step: shape or None}, us={step: {shape: microseconds}})."""
        n = C.c_int()
        self.check(self.lib.tincr_batch_tile_table(self.h, 0, C.byref(n), None, None))
        k = n.value
        ent = np.zeros((max(k, 1), 9), np.int32)
        us = np.zeros((max(k, 1), 4, 4))
        self.check(self.lib.tincr_batch_tile_table(self.h, k, C.byref(n), iptr(ent), dptr(us)))
        out = []
        for i in range(min(k, n.value)):
            e = ent[i]
            shapes = {st: (self.TILE_SHAPES[e[5 + p]] if e[5 + p] >= 0 else None)
                      for p, st in enumerate(self.PLANE_STEPS)}
            times = {st: {sh: float(us[i, p, q]) for q, sh in enumerate(self.TILE_SHAPES)}
                     for p, st in enumerate(self.PLANE_STEPS) if e[5 + p] >= 0}
            out.append(dict(n_atoms=int(e[0]), n_orb=int(e[1]), n_occ=int(e[2]), n_virt=int(e[3]), lc=bool(e[4]),
                            shapes=shapes, us=times))
        return out

    def subspace_eigh(self, a, k):
        """k lowest eigenpairs of the symmetric matrix a (upper triangle read): (w [k], y [k, m], on_device)."""
        a = f64(a)
        m = a.shape[0]
        w = np.zeros(k)
        y = np.zeros((k, m))
        dev = C.c_int()
        self.check(self.lib.tincr_subspace_eigh(self.h, m, int(k), dptr(a), dptr(w), dptr(y), C.byref(dev)))
        return w, y, bool(dev.value)

    def gemm_fp64_tensor(self, a, b):
        """a [M, K] @ b[N, K]^T with FP64-class accuracy on the tensor cores (N <= 32)."""
        a, b = f64(a), f64(b)
        c = np.zeros((a.shape[0], b.shape[0]))
        self.check(self.lib.tincr_gemm_fp64_tensor(self.h, a.shape[0], b.shape[0], a.shape[1], dptr(a), dptr(b),
                                                   dptr(c)))
        return c

    def last_timing(self):
        ms = C.c_double()
        n = C.c_longlong()
        self.lib.tincr_last_timing(self.h, C.byref(ms), C.byref(n))
        return ms.value, n.value
