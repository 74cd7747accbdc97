"""ctypes binding of librepeat_gb300.so (the C ABI in include/repeat_gb300.h).

There is no CPU fallback: if the library is missing or cannot be loaded, every
call raises.  Device buffers are torch CUDA tensors passed by data_ptr().
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librepeat_gb300.so")

RP_OK = 0
RP_E_ARG = -1
STATUS = {
    -1: "RP_E_ARG", -2: "RP_E_CUDA", -3: "RP_E_NOMEM", -4: "RP_E_SINGULAR", -5: "RP_E_TIMEOUT",
    -6: "RP_E_STATE", -7: "RP_E_UNSUPPORTED",
}
PREC_FP64 = 0
PREC_MIXED = 1
SOLVE_INFO_WORDS = 4   # residual, min |pivot|, max |pivot|, kappa
FIT_INFO_WORDS = 8     # residual, min |pivot|, max |pivot|, singular, kappa, path, precision, flags
FIT_ESCALATED = 1      # flag: a mixed-precision cube refitted in FP64 (kappa / (n+1) above the limit)
DEFAULT_KAPPA_LIMIT = 2e5
FIT_TWO_PASS = 2       # flag: a mixed-precision cube refitted in two passes after a clamp

# every symbol include/repeat_gb300.h declares
EXPORTS = ["rp_version", "rp_ctx_create", "rp_ctx_destroy", "rp_last_error", "rp_filter", "rp_ewald_setup",
           "rp_ewald_destroy", "rp_ewald_info", "rp_gram", "rp_solve", "rp_potential", "rp_fit",
           "rp_fit_batch", "rp_set_timing", "rp_stage_times", "rp_launch_count", "rp_solve_noalloc",
           "rp_batch_submit", "rp_batch_poll", "rp_batch_wait", "rp_qeq", "rp_set_kappa_limit", "rp_autotune",
           "rp_load_tiles"]


class RepeatError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class SingularError(RepeatError):
    pass


class RpGrid(ctypes.Structure):
    _fields_ = [("n_grid", ctypes.c_int * 3), ("axis", ctypes.c_double * 9)]


class RpFitDesc(ctypes.Structure):
    _fields_ = [("grid", RpGrid), ("V", ctypes.c_void_p), ("atoms", ctypes.c_void_p), ("Z", ctypes.c_void_p),
                ("N", ctypes.c_int), ("vdw_factor", ctypes.c_double), ("vdw_max", ctypes.c_double),
                ("cutoff", ctypes.c_double), ("qtot", ctypes.c_double), ("kmax", ctypes.c_int),
                ("n_groups", ctypes.c_int), ("group_ptr", ctypes.c_void_p), ("group_idx", ctypes.c_void_p),
                ("resp_s", ctypes.c_void_p), ("resp_t", ctypes.c_void_p), ("precision", ctypes.c_int)]


_lib = None


def load(path: str | None = None):
    """Load the CUDA library (building it in-tree first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from .build import build_cuda
        build_cuda()
    if not os.path.exists(path):
        raise ImportError(f"librepeat_gb300.so not found at {path}; run pyrepeat_gb300.build")
    L = ctypes.CDLL(path)
    P, I, D, L64, SZ = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int64, ctypes.c_size_t
    L.rp_version.restype = I
    L.rp_version.argtypes = []
    L.rp_ctx_create.restype = I
    L.rp_ctx_create.argtypes = [I, SZ, ctypes.POINTER(P)]
    L.rp_ctx_destroy.restype = I
    L.rp_ctx_destroy.argtypes = [P]
    L.rp_last_error.restype = I
    L.rp_last_error.argtypes = [P, ctypes.c_char_p, SZ]
    L.rp_filter.restype = I
    L.rp_filter.argtypes = [P, ctypes.POINTER(RpGrid), P, P, I, P, D, D, P, P, L64, ctypes.POINTER(L64), P, P]
    L.rp_ewald_setup.restype = I
    L.rp_ewald_setup.argtypes = [P, ctypes.POINTER(RpGrid), D, I, ctypes.POINTER(P)]
    L.rp_ewald_destroy.restype = I
    L.rp_ewald_destroy.argtypes = [P]
    L.rp_ewald_info.restype = I
    L.rp_ewald_info.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(D)]
    L.rp_gram.restype = I
    L.rp_gram.argtypes = [P, P, P, I, P, P, L64, I, P, P, P, P]
    L.rp_solve.restype = I
    L.rp_solve.argtypes = [P, P, P, I, I, P, P, P, P, D, P, P, P]
    L.rp_potential.restype = I
    L.rp_potential.argtypes = [P, P, P, P, I, P, L64, P, P]
    L.rp_fit.restype = I
    L.rp_fit.argtypes = [P, ctypes.POINTER(RpFitDesc), P, ctypes.POINTER(L64), P]
    L.rp_solve_noalloc.restype = I
    L.rp_solve_noalloc.argtypes = [P, P, I, I, P, P, P, P, D, P, P, P]
    L.rp_launch_count.restype = I
    L.rp_launch_count.argtypes = [ctypes.POINTER(ctypes.c_longlong)]
    L.rp_set_timing.restype = I
    L.rp_set_timing.argtypes = [P, I]
    L.rp_stage_times.restype = I
    L.rp_stage_times.argtypes = [P, ctypes.c_char_p, SZ, P, ctypes.POINTER(I)]
    L.rp_fit_batch.restype = I
    L.rp_fit_batch.argtypes = [P, I, P, P, P, P, P, P]
    L.rp_batch_submit.restype = I
    L.rp_batch_submit.argtypes = [P, I, P, P, P, P, P, ctypes.POINTER(ctypes.c_longlong)]
    L.rp_batch_poll.restype = I
    L.rp_batch_poll.argtypes = [P, ctypes.c_longlong, ctypes.POINTER(I), ctypes.POINTER(I)]
    L.rp_batch_wait.restype = I
    L.rp_batch_wait.argtypes = [P, ctypes.c_longlong, ctypes.POINTER(I)]
    L.rp_qeq.restype = I
    L.rp_qeq.argtypes = [P, P, P, I, P, P, D, P, P, P, P]
    L.rp_set_kappa_limit.restype = I
    L.rp_set_kappa_limit.argtypes = [P, D]
    L.rp_autotune.restype = I
    L.rp_autotune.argtypes = [P, I, P, P, ctypes.c_char_p]
    L.rp_load_tiles.restype = I
    L.rp_load_tiles.argtypes = [P, ctypes.c_char_p]
    _lib = L
    return L


def check(ctx_ptr, rc: int, what: str = ""):
    if rc == RP_OK:
        return
    buf = ctypes.create_string_buffer(1024)
    if ctx_ptr:
        load().rp_last_error(ctx_ptr, buf, 1024)
    msg = buf.value.decode(errors="replace") or what
    if rc == -4:
        raise SingularError(rc, msg)
    raise RepeatError(rc, msg)


def tile_key(N: int, M: int, kmax: int) -> int:
    """The autotuner's bucket of a fit (the C library's rp::tile_key)."""
    nb = 0 if N < 32 else 1 if N < 64 else 2 if N < 128 else 3 if N < 256 else 4 if N < 512 else 5
    mb = 0 if M < 32768 else 1 if M < 131072 else 2 if M < 524288 else 3
    return (nb * 4 + mb) * 64 + min(max(int(kmax), 0), 63)


def fit_info(row) -> dict:
    """One cube's FIT_INFO_WORDS record as a dict."""
    return {"residual": float(row[0]), "pivot_min": float(row[1]), "pivot_max": float(row[2]),
            "singular": bool(row[3]), "kappa": float(row[4]), "solve_path": int(row[5]),
            "precision": "fp64" if int(row[6]) == PREC_FP64 else "mixed",
            "escalated": bool(int(row[7]) & FIT_ESCALATED), "two_pass": bool(int(row[7]) & FIT_TWO_PASS)}


def solve_info(info) -> dict:
    """rp_solve's SOLVE_INFO_WORDS record as a dict."""
    return {"residual": float(info[0]), "pivot_min": float(info[1]), "pivot_max": float(info[2]),
            "kappa": float(info[3])}


def launch_count() -> int:
    v = ctypes.c_longlong(0)
    load().rp_launch_count(ctypes.byref(v))
    return int(v.value)


def make_grid(n_grid, axis) -> RpGrid:
    g = RpGrid()
    g.n_grid[:] = [int(v) for v in n_grid]
    g.axis[:] = [float(x) for row in axis for x in row]
    return g
