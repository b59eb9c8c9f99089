"""Python host API over the C ABI of libfednl_gpu.so (include/fednl_gpu.h).

Names follow the reference's operator surface (dopt): ``get_topk_from_upper_diagonal_part``,
``get_toplek_from_upper_diagonal_part``, ``generate_randk_items_in_upper_triangular_part``,
``generate_randseqk_items_in_upper_triangular_part``, ``apply_natural_compressor``,
``evaluate_gradient_and_hessian`` and ``cholesky_option_b_solve``, plus ``FedNL`` for whole runs
(the reference's ``train()`` loop).  Matrices are NumPy arrays in the reference's column-major
d x lda layout (flattened), indices are the reference's flat indices j * lda + i.

Errors raise ``FedNLError`` with the library's message; the native library is mandatory (there
is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

IDENTITY, RANDK, TOPK, RANDSEQK, TOPLEK, NATURAL, RANDK_PHILOX = 0, 1, 2, 3, 4, 5, 6
COMPRESSORS = {"identity": IDENTITY, "randk": RANDK, "topk": TOPK, "randseqk": RANDSEQK,
               "seqk": RANDSEQK, "toplek": TOPLEK, "natural": NATURAL, "randk_philox": RANDK_PHILOX}
STATUS = {0: "OK", -1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "ENOTPD", -5: "ETIMEOUT", -6: "ENODEV"}
# Newton solves of the mixed-precision form: FP64 cooperative Cholesky; FP32 Cholesky in one CTA's
# shared memory with one refinement step (d up to about 300); FP32 Cholesky on a cooperative grid
# with FP64-residual refinement to 2^-30 relative, six steps at most (d up to 1312)
SOLVERS = {"fp64": 0, "fp32_refined": 1, "fp32_coop": 2}
HESS_KERNELS = ["masks_smem", "masks_global", "lists"]   # fednl_gpu_hess_schedule kinds 0, 1, 2


class FedNLError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class ProblemDesc(C.Structure):
    _fields_ = [("d", C.c_int32), ("lda", C.c_int32), ("n_clients", C.c_int32),
                ("n_samples", C.POINTER(C.c_int32)), ("lambda_", C.c_double),
                ("compressor", C.c_int32), ("k", C.c_int32), ("alpha", C.c_double),
                ("workers", C.c_int32), ("seed_base", C.c_uint32), ("toplek_seed", C.c_uint32),
                ("feature_format", C.c_int32), ("clients_per_round", C.c_int32),
                ("client_seed", C.c_uint32), ("option_a", C.c_int32), ("line_search", C.c_int32),
                ("ls_c", C.c_double), ("ls_gamma", C.c_double), ("ls_max_steps", C.c_int32), ("track_f", C.c_int32),
                ("arith_order", C.c_int32), ("reserved", C.c_int32)]


# arithmetic order of the FP64 engine: its own fixed order, or the reference's (bit for bit)
ORDERS = {"fixed": 0, "reference": 1}


class RoundStats(C.Structure):
    _fields_ = [("round", C.c_int32), ("status", C.c_int32), ("grad_norm", C.c_double), ("l", C.c_double)]


# fednl_result_callback: (dimension, ||g||, ||g||^2/(2 mu), 2||g||^2/mu)
RESULT_CALLBACK = C.CFUNCTYPE(None, C.c_int, C.c_double, C.c_double, C.c_double)

# every symbol declared in include/fednl_gpu.h
EXPORTS = ["fednl_gpu_create", "fednl_gpu_destroy", "fednl_gpu_upload_client_data", "fednl_gpu_init_shifts",
           "fednl_gpu_round", "fednl_gpu_run", "fednl_gpu_get_x", "fednl_gpu_set_x", "fednl_gpu_get_grad",
           "fednl_gpu_get_H", "fednl_gpu_get_shift", "fednl_gpu_get_l", "fednl_gpu_get_lk",
           "fednl_gpu_get_message", "fednl_gpu_get_f", "fednl_gpu_get_ls_steps", "fednl_gpu_get_selected", "fednl_gpu_get_true_grad", "fednl_gpu_get_dir",
           "fednl_gpu_topk", "fednl_gpu_toplek", "fednl_gpu_randk",
           "fednl_gpu_randseqk", "fednl_gpu_natural", "fednl_gpu_logreg_oracle", "fednl_gpu_optionb_solve",
           "fednl_gpu_optionb_solve_noalloc", "fednl_gpu_time_rounds", "fednl_gpu_profile_kernels",
           "fednl_gpu_last_error", "fednl_gpu_execute_local", "fednl_gpu_load_libsvm",
           "fednl_gpu_weighted_gram_tf32", "fednl_mx_create", "fednl_mx_destroy", "fednl_mx_upload_client_data",
           "fednl_mx_init_shifts", "fednl_mx_run", "fednl_mx_time_rounds", "fednl_mx_get_x", "fednl_mx_get_grad",
           "fednl_mx_get_l", "fednl_mx_profile_kernels", "fednl_gpu_client_phase", "fednl_mx_client_phase",
           "fednl_gpu_solve_batch", "fednl_gpu_round_result", "fednl_mx_round_result", "fednl_gpu_mem_info",
           "fednl_mx_get_diff", "fednl_mx_get_selection", "fednl_mx_get_shift", "fednl_gpu_footprint",
           "fednl_mx_footprint", "fednl_server_create", "fednl_server_destroy", "fednl_server_submit",
           "fednl_server_tick", "fednl_server_status", "fednl_server_latencies", "fednl_gpu_optionb_solve_mixed", "fednl_gpu_optionb_solve32", "fednl_gpu_selftest_rn",
           "fednl_mx_set_solver", "fednl_gpu_encode_client_round", "fednl_gpu_get_client_grad", "fednl_gpu_get_diff",
           "fednl_gpu_autotune", "fednl_gpu_autotune_shapes", "fednl_mx_autotune", "doptExecuteLocal", "doptExecuteLocalPP",
           "fednl_gpu_shift_update", "fednl_gpu_aggregate", "fednl_gpu_compress_identity", "fednl_gpu_fp64_rate",
           "fednl_server_device_times", "fednl_gpu_stream", "fednl_mx_stream", "fednl_server_submit_ref",
           "fednl_gpu_hess_schedule", "fednl_gpu_set_hess_schedule", "fednl_gpu_upload_client_csr",
           "fednl_gpu_hit_lists"]

_lib = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Loads the in-tree libfednl_gpu.so (building it with nvcc if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB_PATH):
        if not build_if_missing:
            raise FedNLError(-6, f"native library missing: {_build.LIB_PATH}")
        _build.build()
    L = C.CDLL(_build.LIB_PATH)
    vp, dp, up, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.POINTER(C.c_int32)
    sig = {
        "fednl_gpu_create": [C.POINTER(ProblemDesc), C.POINTER(C.c_void_p)],
        "fednl_gpu_destroy": [vp],
        "fednl_gpu_upload_client_data": [vp, dp, dp],
        "fednl_gpu_init_shifts": [vp, dp],
        "fednl_gpu_round": [vp, C.POINTER(RoundStats)],
        "fednl_gpu_run": [vp, C.c_int32, dp],
        "fednl_gpu_get_x": [vp, dp], "fednl_gpu_set_x": [vp, dp], "fednl_gpu_get_grad": [vp, dp],
        "fednl_gpu_get_H": [vp, dp], "fednl_gpu_get_shift": [vp, C.c_int32, dp],
        "fednl_gpu_get_message": [vp, C.c_int32, up, dp, ip],
        "fednl_gpu_get_selected": [vp, ip, ip],
        "fednl_gpu_get_true_grad": [vp, dp],
        "fednl_gpu_get_dir": [vp, C.c_int32, dp, dp],
        "fednl_gpu_topk": [dp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, up],
        "fednl_gpu_toplek": [dp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, ip, up, up, ip],
        "fednl_gpu_randk": [up, C.c_int32, C.c_int32, C.c_int32, C.c_int32, up],
        "fednl_gpu_randseqk": [up, C.c_int32, C.c_int32, C.c_int32, C.c_int32, up],
        "fednl_gpu_natural": [dp, C.c_int64, dp, C.POINTER(C.c_uint8)],
        "fednl_gpu_fp64_rate": [C.c_int64, dp, dp, dp],
        "fednl_gpu_shift_update": [dp, dp, C.c_int32, C.c_int32, C.c_int32, up, ip, C.c_int32, C.c_double,
                                   C.c_double],
        "fednl_gpu_aggregate": [C.c_int32, C.c_int32, C.c_int32, dp, dp, up, dp, ip, C.c_int32, dp, dp, dp],
        "fednl_gpu_compress_identity": [dp, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double, dp, up, dp],
        "fednl_gpu_logreg_oracle": [dp, dp, C.c_int32, C.c_int32, C.c_int32, C.c_double, dp, dp, dp],
        "fednl_gpu_optionb_solve": [dp, C.c_int32, C.c_int32, C.c_double, dp, dp],
        "fednl_gpu_optionb_solve_mixed": [dp, C.c_int32, C.c_int32, C.c_double, dp, dp],
        "fednl_gpu_optionb_solve32": [dp, C.c_int32, C.c_int32, C.c_double, dp, dp, C.c_int32, C.c_int32],
        "fednl_gpu_selftest_rn": [C.c_int64, C.c_uint64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
        "fednl_gpu_optionb_solve_noalloc": [vp, C.c_int32, C.c_int32, C.c_double, vp, vp, vp],
        "fednl_gpu_time_rounds": [vp, C.c_int32, C.c_int64, dp, dp],
        "fednl_gpu_profile_kernels": [vp, C.c_int32, C.c_int64, ip, dp, C.c_char_p, C.c_int32],
        "fednl_gpu_hit_lists": [C.c_int32, C.c_int32, ip, ip, ip, C.POINTER(C.c_int64), ip,
                                C.POINTER(C.c_uint16), up, up, C.POINTER(C.c_uint16)],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.fednl_gpu_get_l.argtypes = [vp]
    L.fednl_gpu_get_l.restype = C.c_double
    L.fednl_gpu_get_lk.argtypes = [vp, C.c_int32]
    L.fednl_gpu_get_lk.restype = C.c_double
    L.fednl_gpu_get_f.argtypes = [vp]
    L.fednl_gpu_get_f.restype = C.c_double
    L.fednl_gpu_get_ls_steps.argtypes = [vp]
    L.fednl_gpu_get_ls_steps.restype = C.c_int32
    fp = C.POINTER(C.c_float)
    L.fednl_gpu_weighted_gram_tf32.argtypes = [fp, fp, ip, C.c_int32, C.c_int32, C.c_float, fp]
    L.fednl_gpu_weighted_gram_tf32.restype = C.c_int
    for name, args in {"fednl_mx_create": [C.POINTER(ProblemDesc), C.POINTER(C.c_void_p)], "fednl_mx_destroy": [vp],
                       "fednl_mx_upload_client_data": [vp, fp, dp], "fednl_mx_init_shifts": [vp, dp],
                       "fednl_mx_run": [vp, C.c_int32, dp], "fednl_mx_time_rounds": [vp, C.c_int32, C.c_int64, dp, dp],
                       "fednl_mx_get_x": [vp, dp], "fednl_mx_get_grad": [vp, dp],
                       "fednl_mx_profile_kernels": [vp, C.c_int32, dp, C.c_char_p, C.c_int32]}.items():
        getattr(L, name).argtypes = args
        getattr(L, name).restype = C.c_int
    for name, args in {"fednl_gpu_client_phase": [vp], "fednl_mx_client_phase": [vp],
                       "fednl_gpu_solve_batch": [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p), C.c_int32],
                       "fednl_gpu_round_result": [vp, C.POINTER(RoundStats)],
                       "fednl_mx_round_result": [vp, C.POINTER(RoundStats)],
                       "fednl_gpu_mem_info": [C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
                       "fednl_mx_get_diff": [vp, C.c_int32, fp], "fednl_mx_get_shift": [vp, C.c_int32, fp],
                       "fednl_mx_get_selection": [vp, C.c_int32, up, ip], "fednl_mx_set_solver": [vp, C.c_int32],
                       "fednl_gpu_encode_client_round": [vp, C.c_int32, C.c_int32, C.POINTER(C.c_uint8), C.c_int64,
                                                         C.POINTER(C.c_int64)],
                       "fednl_gpu_get_client_grad": [vp, C.c_int32, dp], "fednl_gpu_get_diff": [vp, C.c_int32, dp],
                       "fednl_gpu_autotune": [vp, ip, dp], "fednl_gpu_autotune_shapes": [vp, ip, ip, ip, dp],
                       "fednl_mx_autotune": [vp, ip, ip, dp], "fednl_gpu_hess_schedule": [vp, ip, ip, ip],
                       "fednl_gpu_set_hess_schedule": [vp, C.c_int32, C.c_int32],
                       "fednl_gpu_upload_client_csr": [vp, ip, ip, dp]}.items():
        getattr(L, name).argtypes = args
        getattr(L, name).restype = C.c_int
    L.fednl_mx_get_l.argtypes = [vp]
    L.fednl_mx_get_l.restype = C.c_double
    L.fednl_gpu_load_libsvm.argtypes = [C.c_char_p, C.c_int32, ip, ip, dp, dp]
    L.fednl_gpu_load_libsvm.restype = C.c_int
    L.fednl_gpu_execute_local.argtypes = [C.c_char_p, RESULT_CALLBACK]
    L.fednl_gpu_execute_local.restype = C.c_int
    L.doptExecuteLocal.argtypes = [C.c_char_p, RESULT_CALLBACK]
    L.doptExecuteLocal.restype = C.c_int
    L.doptExecuteLocalPP.argtypes = [C.c_char_p, C.CFUNCTYPE(None, C.c_int)]
    L.doptExecuteLocalPP.restype = C.c_int
    L.fednl_gpu_last_error.argtypes = []
    L.fednl_gpu_last_error.restype = C.c_char_p
    _lib = L
    return L


def _check(rc: int):
    if rc != 0:
        raise FedNLError(rc, load().fednl_gpu_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _up(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def hit_lists(d: int, n_samples, rowptr, colidx) -> dict:
    """The binary Hessian's common-sample lists for 0/1 features as CSR rows, built on the host by the
    library (fednl_gpu_hit_lists; no device): code [n_clients, ustr] (u16), seg [n_clients, nseg + 1],
    rec [records + 1] (u32), hits (u16) and maxrec."""
    L = load()
    ns = np.ascontiguousarray(n_samples, dtype=np.int32)
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    ci = np.ascontiguousarray(colidx, dtype=np.int32)
    if ci.size == 0:
        ci = np.zeros(1, np.int32)
    sizes = np.zeros(4, np.int64)
    mr = np.zeros(1, np.int32)
    i64 = C.POINTER(C.c_int64)
    u16 = C.POINTER(C.c_uint16)
    _check(L.fednl_gpu_hit_lists(d, ns.size, _ip(ns), _ip(rp), _ip(ci), sizes.ctypes.data_as(i64), _ip(mr),
                                 None, None, None, None))
    code = np.empty(int(sizes[0]), np.uint16)
    seg = np.empty(int(sizes[1]), np.uint32)
    rec = np.empty(int(sizes[2]), np.uint32)
    hits = np.empty(max(1, int(sizes[3])), np.uint16)
    _check(L.fednl_gpu_hit_lists(d, ns.size, _ip(ns), _ip(rp), _ip(ci), sizes.ctypes.data_as(i64), _ip(mr),
                                 code.ctypes.data_as(u16), _up(seg), _up(rec), hits.ctypes.data_as(u16)))
    return {"code": code.reshape(ns.size, -1), "seg": seg.reshape(ns.size, -1), "rec": rec,
            "hits": hits[:int(sizes[3])], "maxrec": int(mr[0])}


def reference_lda(d: int) -> int:
    return (d + 3) // 4 * 4


# ---- operator surface ------------------------------------------------------------------------

def get_topk_from_upper_diagonal_part(mats: np.ndarray, d: int, lda: int, k: int) -> np.ndarray:
    """mats: [n, d*lda] column-major matrices -> [n, k] ascending flat indices."""
    m = np.ascontiguousarray(mats, dtype=np.float64).reshape(-1, d * lda)
    U = d * (d + 1) // 2
    kk = min(k, U)
    out = np.zeros((m.shape[0], max(k, 1)), dtype=np.uint32)
    _check(load().fednl_gpu_topk(_dp(m), m.shape[0], d, lda, k, _up(out)))
    return out[:, :kk]


def get_toplek_from_upper_diagonal_part(mats: np.ndarray, d: int, lda: int, k: int, worker_states: np.ndarray,
                                        worker_of=None):
    """Returns a list of index arrays; worker_states (uint32[W]) is advanced in place."""
    m = np.ascontiguousarray(mats, dtype=np.float64).reshape(-1, d * lda)
    n = m.shape[0]
    out = np.zeros((n, k), dtype=np.uint32)
    counts = np.zeros(n, dtype=np.int32)
    wo = None if worker_of is None else np.ascontiguousarray(worker_of, dtype=np.int32)
    ws = worker_states
    assert ws.dtype == np.uint32 and ws.flags.c_contiguous
    _check(load().fednl_gpu_toplek(_dp(m), n, d, lda, k, ws.size,
                                   _ip(wo) if wo is not None else None, _up(ws), _up(out), _ip(counts)))
    return [out[t, :counts[t]].copy() for t in range(n)]


def generate_randk_items_in_upper_triangular_part(states: np.ndarray, d: int, lda: int, k: int) -> np.ndarray:
    assert states.dtype == np.uint32 and states.flags.c_contiguous
    out = np.zeros((states.size, k), dtype=np.uint32)
    _check(load().fednl_gpu_randk(_up(states), states.size, d, lda, k, _up(out)))
    return out


def generate_randseqk_items_in_upper_triangular_part(states: np.ndarray, d: int, lda: int, k: int) -> np.ndarray:
    assert states.dtype == np.uint32 and states.flags.c_contiguous
    out = np.zeros((states.size, k), dtype=np.uint32)
    _check(load().fednl_gpu_randseqk(_up(states), states.size, d, lda, k, _up(out)))
    return out


def apply_natural_compressor(values: np.ndarray, with_packed: bool = False):
    v = np.ascontiguousarray(values, dtype=np.float64).ravel()
    out = np.empty_like(v)
    packed = np.zeros(3 * (v.size // 2 + 1), dtype=np.uint8) if with_packed else None
    _check(load().fednl_gpu_natural(_dp(v), v.size, _dp(out),
                                    packed.ctypes.data_as(C.POINTER(C.c_uint8)) if with_packed else None))
    return (out, packed) if with_packed else out


def evaluate_gradient_and_hessian(features, labels, lam: float, x, lda: int | None = None):
    f = np.ascontiguousarray(features, dtype=np.float64)
    b = np.ascontiguousarray(labels, dtype=np.float64)
    n, d = f.shape
    lda = lda or reference_lda(d)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    g = np.empty(d)
    h = np.empty(d * lda)
    _check(load().fednl_gpu_logreg_oracle(_dp(f), _dp(b), n, d, lda, lam, _dp(xx), _dp(g), _dp(h)))
    return g, h


def cholesky_option_b_solve_mixed(H: np.ndarray, d: int, lda: int, l: float, g: np.ndarray) -> np.ndarray:
    """(H + l I) dx = g with the mixed-precision form's solve (FP32 factor, refined)."""
    Hc = np.ascontiguousarray(H, dtype=np.float64)
    gc = np.ascontiguousarray(g, dtype=np.float64)
    dx = np.empty(d)
    _check(load().fednl_gpu_optionb_solve_mixed(_dp(Hc), d, lda, float(l), _dp(gc), _dp(dx)))
    return dx


def selftest_rn(n: int, seed: int = 1) -> tuple:
    """Mismatch counts (sqrt, reciprocal) of the Cholesky's integer square root and reciprocal against
    the hardware operations over n generated inputs."""
    a = C.c_int64(0)
    b = C.c_int64(0)
    _check(load().fednl_gpu_selftest_rn(int(n), int(seed), C.byref(a), C.byref(b)))
    return a.value, b.value


def cholesky_option_b_solve32(H: np.ndarray, d: int, lda: int, l: float, g: np.ndarray, refine: int = 6,
                              grid: int = 0) -> np.ndarray:
    """(H + l I) dx = g with the FP32 cooperative factor and FP64 refinement (mixed solver 2)."""
    Hc = np.ascontiguousarray(H, dtype=np.float64)
    gc = np.ascontiguousarray(g, dtype=np.float64)
    dx = np.empty(d)
    _check(load().fednl_gpu_optionb_solve32(_dp(Hc), d, lda, float(l), _dp(gc), _dp(dx), int(refine), int(grid)))
    return dx


def cholesky_option_b_solve(H: np.ndarray, d: int, lda: int, l: float, g: np.ndarray) -> np.ndarray:
    hh = np.ascontiguousarray(H, dtype=np.float64).ravel()
    gg = np.ascontiguousarray(g, dtype=np.float64)
    dx = np.empty(d)
    _check(load().fednl_gpu_optionb_solve(_dp(hh), d, lda, l, _dp(gg), _dp(dx)))
    return dx


# ---- whole runs ------------------------------------------------------------------------------

class FedNL:
    """One FedNL problem resident on the GPU (reference: bin_fednl_local train()); with
    clients_per_round set, FedNL-PP (bin_fednl_local_pp train()) with that many sampled clients."""

    def __init__(self, prob, compressor, k: int, alpha: float, lda: int | None = None, workers: int = 1,
                 seed_base: int = 123, toplek_seed: int = 1234, x0=None, feature_format: int = 0,
                 clients_per_round: int = 0, client_seed: int = 1234, option_a: bool = False,
                 line_search=None, track_f: bool = False, order: str = "fixed", hess_schedule=None,
                 csr: bool = False):
        """order: "fixed" (the engine's own order, bit-identical to the test oracle) or "reference"
        (the reference's operation order, bit-identical to the reference's rounds).  hess_schedule:
        (kernel, threads) of the binary Hessian from the initial shifts on (see set_hess_schedule).
        csr: upload 0/1 features as CSR columns, packed into the bit layout on the device."""
        self.d = prob.d
        self.lda = lda or reference_lda(prob.d)
        self.n_clients = prob.n_clients
        self._ns = np.ascontiguousarray(prob.n_samples, dtype=np.int32)
        comp = COMPRESSORS[compressor] if isinstance(compressor, str) else int(compressor)
        self.compressor = comp
        desc = ProblemDesc(self.d, self.lda, self.n_clients, _ip(self._ns), float(prob.lam), comp, int(k),
                           float(alpha), int(workers), int(seed_base), int(toplek_seed), int(feature_format),
                           int(clients_per_round or 0), int(client_seed), 1 if option_a else 0,
                           1 if line_search else 0, float(line_search[0]) if line_search else 0.5,
                           float(line_search[1]) if line_search else 0.5, int(line_search[2]) if line_search else 5,
                           1 if track_f else 0, ORDERS[order], 0)
        self.pp = bool(clients_per_round)
        h = C.c_void_p()
        _check(load().fednl_gpu_create(C.byref(desc), C.byref(h)))
        self._h = h
        try:
            f = np.ascontiguousarray(prob.features, dtype=np.float64)
            b = np.ascontiguousarray(prob.labels, dtype=np.float64)
            if csr:
                rows, cols = np.nonzero(f)
                rp = np.zeros(f.shape[0] + 1, dtype=np.int32)
                np.add.at(rp, rows + 1, 1)
                rp = np.cumsum(rp).astype(np.int32)
                ci = np.ascontiguousarray(cols, dtype=np.int32)
                _check(load().fednl_gpu_upload_client_csr(self._h, _ip(rp), _ip(ci if ci.size else np.zeros(1, np.int32)),
                                                          _dp(b)))
            else:
                _check(load().fednl_gpu_upload_client_data(self._h, _dp(f), _dp(b)))
            if hess_schedule is not None:
                self.set_hess_schedule(*hess_schedule)
            xx = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
            _check(load().fednl_gpu_init_shifts(self._h, _dp(xx) if xx is not None else None))
        except Exception:
            self.close()
            raise

    def close(self):
        if getattr(self, "_h", None):
            load().fednl_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def round(self) -> float:
        st = RoundStats()
        _check(load().fednl_gpu_round(self._h, C.byref(st)))
        return st.grad_norm

    def run(self, rounds: int) -> np.ndarray:
        out = np.empty(rounds)
        _check(load().fednl_gpu_run(self._h, rounds, _dp(out)))
        return out

    def autotune(self) -> dict:
        """Measures the solve's CTA count and the binary Hessian's launch shape (per d and n_i
        bucket) on this problem and keeps the fastest (same results)."""
        g = np.zeros(1, dtype=np.int32)
        ms = np.zeros(1)
        _check(load().fednl_gpu_autotune(self._h, _ip(g), _dp(ms)))
        nt = np.zeros(1, dtype=np.int32)
        sm = np.zeros(1, dtype=np.int32)
        b = np.zeros(1, dtype=np.int32)
        hms = np.zeros(1)
        _check(load().fednl_gpu_autotune_shapes(self._h, _ip(nt), _ip(sm), _ip(b), _dp(hms)))
        out = {"chol_ctas": int(g[0]), "solve_ms": float(ms[0]), "hess_threads": int(nt[0]),
               "hess_masks_in_smem": bool(sm[0]), "ni_bucket": int(b[0]), "hess_ms": float(hms[0])}
        out["hess_kernel"] = self.hess_schedule()["kernel"]
        return out

    def hess_schedule(self) -> dict:
        """The binary Hessian's kernel ("masks_smem", "masks_global", "lists"), threads per block, and
        whether the common-sample lists were built at upload."""
        k = np.zeros(1, dtype=np.int32)
        nt = np.zeros(1, dtype=np.int32)
        built = np.zeros(1, dtype=np.int32)
        _check(load().fednl_gpu_hess_schedule(self._h, _ip(k), _ip(nt), _ip(built)))
        return {"kernel": HESS_KERNELS[int(k[0])] if k[0] >= 0 else None, "threads": int(nt[0]),
                "lists_built": bool(built[0])}

    def set_hess_schedule(self, kernel: str, threads: int = 256):
        """Overrides the binary Hessian's kernel and threads per block (results do not change)."""
        _check(load().fednl_gpu_set_hess_schedule(self._h, HESS_KERNELS.index(kernel), threads))

    def client_phase(self):
        """Launches the round up to the master's aggregation (no wait); solve_batch ends it."""
        _check(load().fednl_gpu_client_phase(self._h))

    def round_result(self) -> float:
        """||g|| of the round that solve_batch just ended (waits for it)."""
        st = RoundStats()
        _check(load().fednl_gpu_round_result(self._h, C.byref(st)))
        return st.grad_norm

    def time_rounds(self, rounds: int, flush_bytes: int = 0):
        """Device-timed rounds (CUDA events on the library's stream); returns (total_ms, per_round_ms)."""
        tot = C.c_double(0.0)
        per = np.empty(rounds)
        _check(load().fednl_gpu_time_rounds(self._h, rounds, flush_bytes, C.byref(tot), _dp(per)))
        return tot.value, per

    def profile_kernels(self, rounds: int, flush_bytes: int = 0):
        """Mean per-launch time of every kernel of a round: {name: ms}, in launch order."""
        n = np.zeros(1, dtype=np.int32)
        ms = np.zeros(64)
        buf = C.create_string_buffer(4096)
        _check(load().fednl_gpu_profile_kernels(self._h, rounds, flush_bytes, _ip(n), _dp(ms), buf, 4096))
        names = buf.value.decode().split(";")
        return [(names[t], float(ms[t])) for t in range(int(n[0]))]

    def x(self) -> np.ndarray:
        out = np.empty(self.d)
        _check(load().fednl_gpu_get_x(self._h, _dp(out)))
        return out

    def set_x(self, x):
        xx = np.ascontiguousarray(x, dtype=np.float64)
        _check(load().fednl_gpu_set_x(self._h, _dp(xx)))

    def grad(self) -> np.ndarray:
        out = np.empty(self.d)
        _check(load().fednl_gpu_get_grad(self._h, _dp(out)))
        return out

    def H(self) -> np.ndarray:
        out = np.empty(self.d * self.lda)
        _check(load().fednl_gpu_get_H(self._h, _dp(out)))
        return out

    def shift(self, c: int) -> np.ndarray:
        out = np.empty(self.d * self.lda)
        _check(load().fednl_gpu_get_shift(self._h, c, _dp(out)))
        return out

    def l(self) -> float:
        return load().fednl_gpu_get_l(self._h)

    def lk(self, c: int) -> float:
        return load().fednl_gpu_get_lk(self._h, c)

    def f(self) -> float:
        """f(x) at the last round's starting iterate (line search or track_f)."""
        return load().fednl_gpu_get_f(self._h)

    def ls_steps(self) -> int:
        return load().fednl_gpu_get_ls_steps(self._h)

    def selected(self) -> np.ndarray:
        """FedNL-PP: the last round's sampled clients, ascending."""
        out = np.empty(self.n_clients, dtype=np.int32)
        cnt = np.zeros(1, dtype=np.int32)
        _check(load().fednl_gpu_get_selected(self._h, _ip(out), _ip(cnt)))
        return out[:int(cnt[0])].copy()

    def true_grad(self) -> np.ndarray:
        out = np.empty(self.d)
        _check(load().fednl_gpu_get_true_grad(self._h, _dp(out)))
        return out

    def dir(self, c: int):
        dr, dd = np.empty(self.d), np.empty(self.d)
        _check(load().fednl_gpu_get_dir(self._h, c, _dp(dr), _dp(dd)))
        return dr, dd

    def encode_round(self, c: int, flags: int) -> bytes:
        """The bytes bin_fednl_distr_client sends its master for client c's last round."""
        n = C.c_int64(0)
        _check(load().fednl_gpu_encode_client_round(self._h, c, flags, None, 0, C.byref(n)))
        buf = (C.c_uint8 * max(1, n.value))()
        _check(load().fednl_gpu_encode_client_round(self._h, c, flags, buf, n.value, C.byref(n)))
        return bytes(buf)[: n.value]

    def client_grad(self, c: int) -> np.ndarray:
        out = np.empty(self.d)
        _check(load().fednl_gpu_get_client_grad(self._h, c, _dp(out)))
        return out

    def diff(self, c: int) -> np.ndarray:
        """H_c - shift_c of the last round, packed upper (j (j + 1) / 2 + i)."""
        U = self.d * (self.d + 1) // 2
        out = np.empty(U)
        _check(load().fednl_gpu_get_diff(self._h, c, _dp(out)))
        return out

    def message(self, c: int):
        U = self.d * (self.d + 1) // 2
        idx = np.empty(U, dtype=np.uint32)
        val = np.empty(U)
        cnt = np.zeros(1, dtype=np.int32)
        _check(load().fednl_gpu_get_message(self._h, c, _up(idx), _dp(val), _ip(cnt)))
        n = int(cnt[0])
        return idx[:n].copy(), val[:n].copy()


# ---- the reference's local driver ---------------------------------------------------------------

def execute_local(command: str):
    """doptExecuteLocal (bin_fednl_local/src/mainShared.cpp:15-38) on the GPU engine: runs the
    bin_fednl_local command line and returns (return code, callback values or None)."""
    got = []

    @RESULT_CALLBACK
    def cb(d, gnorm, fgap, xgap):
        got.append((int(d), float(gnorm), float(fgap), float(xgap)))

    rc = load().fednl_gpu_execute_local(command.encode(), cb)
    return rc, (got[0] if got else None)


def shift_update(shifts, diffs, d: int, lda: int, idx, counts, alpha: float, value_mult: float = 1.0):
    """fednl_gpu_shift_update: shifts [n, d*lda] updated in place; idx [n, k_stride]; counts [n]."""
    sh = np.ascontiguousarray(shifts, dtype=np.float64)
    df = np.ascontiguousarray(diffs, dtype=np.float64)
    ix = np.ascontiguousarray(idx, dtype=np.uint32)
    ct = np.ascontiguousarray(counts, dtype=np.int32)
    n = ct.size
    _check(load().fednl_gpu_shift_update(_dp(sh), _dp(df), n, d, lda, _up(ix), _ip(ct), ix.shape[1], float(alpha),
                                         float(value_mult)))
    return sh


def aggregate(grads, lks, d: int, lda: int, H, idx=None, vals=None, counts=None):
    """fednl_gpu_aggregate: returns (H updated, g, l)."""
    gr = np.ascontiguousarray(grads, dtype=np.float64)
    lk = np.ascontiguousarray(lks, dtype=np.float64)
    Hh = np.ascontiguousarray(H, dtype=np.float64).copy()
    n = lk.size
    g = np.empty(d)
    l = np.zeros(1)
    if idx is None:
        _check(load().fednl_gpu_aggregate(n, d, lda, _dp(gr), _dp(lk), None, None, None, 0, _dp(Hh), _dp(g), _dp(l)))
    else:
        ix = np.ascontiguousarray(idx, dtype=np.uint32)
        vv = np.ascontiguousarray(vals, dtype=np.float64)
        ct = np.ascontiguousarray(counts, dtype=np.int32)
        _check(load().fednl_gpu_aggregate(n, d, lda, _dp(gr), _dp(lk), _up(ix), _dp(vv), _ip(ct), ix.shape[1],
                                          _dp(Hh), _dp(g), _dp(l)))
    return Hh, g, float(l[0])


def compress_identity(diffs, d: int, lda: int, alpha: float, prescale: float, shifts=None):
    """fednl_gpu_compress_identity: returns (idx [n, U], vals [n, U], shifts updated or None)."""
    df = np.ascontiguousarray(diffs, dtype=np.float64).reshape(-1, d * lda)
    n = df.shape[0]
    U = d * (d + 1) // 2
    ix = np.empty((n, U), dtype=np.uint32)
    vv = np.empty((n, U))
    sh = None if shifts is None else np.ascontiguousarray(shifts, dtype=np.float64).reshape(n, d * lda).copy()
    _check(load().fednl_gpu_compress_identity(_dp(df), n, d, lda, float(alpha), float(prescale),
                                              _dp(sh) if sh is not None else None, _up(ix), _dp(vv)))
    return ix, vv, sh


def fp64_rate(iters: int = 1 << 16) -> dict:
    """This GPU's FP64 pipe: fma and add lane operations per second (G op/s, all SMs busy) and the
    cycles of one dependent add in a single warp."""
    a, b, c = np.zeros(1), np.zeros(1), np.zeros(1)
    _check(load().fednl_gpu_fp64_rate(int(iters), _dp(a), _dp(b), _dp(c)))
    return {"fma_gops": float(a[0]), "add_gops": float(b[0]), "add_latency_cycles": float(c[0])}


# the reference's exported callback types (FedNLLocalShared.h:8-11, FedNLPPLocalShared.h:8)
RESULT_CALLBACK_PP = C.CFUNCTYPE(None, C.c_int)


def dopt_execute_local(command: str):
    """The reference's own symbol doptExecuteLocal, exported by this library: returns (return code,
    callback values or None)."""
    got = []

    @RESULT_CALLBACK
    def cb(d, gnorm, fgap, xgap):
        got.append((int(d), float(gnorm), float(fgap), float(xgap)))

    rc = load().doptExecuteLocal(command.encode(), cb)
    return rc, (got[0] if got else None)


def dopt_execute_local_pp(command: str):
    """The reference's own symbol doptExecuteLocalPP (bin_fednl_local_pp): returns (return code,
    the dimension passed to the callback or None)."""
    got = []

    @RESULT_CALLBACK_PP
    def cb(d):
        got.append(int(d))

    rc = load().doptExecuteLocalPP(command.encode(), cb)
    return rc, (got[0] if got else None)


def load_libsvm(path: str, add_intercept: bool = False):
    """The reference's LIBSVM loader semantics: returns (features [n, d] row-major, labels +-1)."""
    L = load()
    n = np.zeros(1, dtype=np.int32)
    d = np.zeros(1, dtype=np.int32)
    _check(L.fednl_gpu_load_libsvm(path.encode(), int(add_intercept), _ip(n), _ip(d), None, None))
    feats = np.empty((int(n[0]), int(d[0])))
    labs = np.empty(int(n[0]))
    _check(L.fednl_gpu_load_libsvm(path.encode(), int(add_intercept), _ip(n), _ip(d), _dp(feats), _dp(labs)))
    return feats, labs


def weighted_gram_tf32(features, weights, n_samples, lam: float = 0.0) -> np.ndarray:
    """Tensor-core weighted Gram X_c^T diag(w) X_c + lam I per client (upper 128-tiles filled);
    features [sum n][d] FP32, weights [sum n] FP32."""
    f = np.ascontiguousarray(features, dtype=np.float32)
    w = np.ascontiguousarray(weights, dtype=np.float32)
    ns = np.ascontiguousarray(n_samples, dtype=np.int32)
    d = f.shape[1]
    out = np.zeros((len(ns), d, d), dtype=np.float32)
    fp = C.POINTER(C.c_float)
    _check(load().fednl_gpu_weighted_gram_tf32(f.ctypes.data_as(fp), w.ctypes.data_as(fp), _ip(ns), len(ns), d,
                                               float(lam), out.ctypes.data_as(fp)))
    return out


class MixedFedNL:
    """The mixed-precision FedNL round (FP32 features; RandK-Philox, TopK or TopLEK; Option B):
    client Hessians on the tensor cores, FP64 master and solve."""

    def __init__(self, prob, k: int, alpha: float, seed_base: int = 123, x0=None, compressor="randk_philox",
                 toplek_seed: int = 1234, solver: str = "fp64"):
        self.d = prob.d
        self.U = prob.d * (prob.d + 1) // 2
        self.n_clients = prob.n_clients
        self._ns = np.ascontiguousarray(prob.n_samples, dtype=np.int32)
        comp = COMPRESSORS[compressor] if isinstance(compressor, str) else int(compressor)
        desc = ProblemDesc(self.d, 0, self.n_clients, _ip(self._ns), float(prob.lam), comp, int(k),
                           float(alpha), 1, int(seed_base), int(toplek_seed), 2, 0, 1234, 0, 0, 0.5, 0.5, 5, 0, 0, 0)
        h = C.c_void_p()
        _check(load().fednl_mx_create(C.byref(desc), C.byref(h)))
        self._h = h
        try:
            f = np.ascontiguousarray(prob.features, dtype=np.float32)
            b = np.ascontiguousarray(prob.labels, dtype=np.float64)
            _check(load().fednl_mx_upload_client_data(self._h, f.ctypes.data_as(C.POINTER(C.c_float)), _dp(b)))
            xx = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
            _check(load().fednl_mx_init_shifts(self._h, _dp(xx) if xx is not None else None))
            _check(load().fednl_mx_set_solver(self._h, SOLVERS[solver]))
        except Exception:
            self.close()
            raise

    def close(self):
        if getattr(self, "_h", None):
            load().fednl_mx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, rounds: int) -> np.ndarray:
        out = np.empty(rounds)
        _check(load().fednl_mx_run(self._h, rounds, _dp(out)))
        return out

    def autotune(self) -> dict:
        """Measures the solves (the FP64 and FP32 cooperative solves over CTA counts; the FP32
        shared-memory solve where it fits) on this problem's current system and keeps the fastest."""
        sv = np.zeros(1, dtype=np.int32)
        g = np.zeros(1, dtype=np.int32)
        ms = np.zeros(1)
        _check(load().fednl_mx_autotune(self._h, _ip(sv), _ip(g), _dp(ms)))
        return {"solver": list(SOLVERS)[int(sv[0])], "chol_ctas": int(g[0]), "solve_ms": float(ms[0])}

    def client_phase(self):
        _check(load().fednl_mx_client_phase(self._h))

    def round_result(self) -> float:
        st = RoundStats()
        _check(load().fednl_mx_round_result(self._h, C.byref(st)))
        return st.grad_norm

    def time_rounds(self, rounds: int, flush_bytes: int = 0):
        tot = C.c_double(0.0)
        per = np.empty(rounds)
        _check(load().fednl_mx_time_rounds(self._h, rounds, flush_bytes, C.byref(tot), _dp(per)))
        return tot.value, per

    def profile_kernels(self, rounds: int):
        ms = np.zeros(16)
        buf = C.create_string_buffer(1024)
        _check(load().fednl_mx_profile_kernels(self._h, rounds, _dp(ms), buf, 1024))
        names = buf.value.decode().split(";")
        return [(names[t], float(ms[t])) for t in range(len(names))]

    def x(self) -> np.ndarray:
        out = np.empty(self.d)
        _check(load().fednl_mx_get_x(self._h, _dp(out)))
        return out

    def grad(self) -> np.ndarray:
        out = np.empty(self.d)
        _check(load().fednl_mx_get_grad(self._h, _dp(out)))
        return out

    def l(self) -> float:
        return load().fednl_mx_get_l(self._h)

    def diff(self, c: int) -> np.ndarray:
        """The last round's FP32 H_c - shift_c, packed upper [U]."""
        out = np.empty(self.U, dtype=np.float32)
        _check(load().fednl_mx_get_diff(self._h, c, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def shift(self, c: int) -> np.ndarray:
        out = np.empty(self.U, dtype=np.float32)
        _check(load().fednl_mx_get_shift(self._h, c, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def selection(self, c: int) -> np.ndarray:
        """Packed upper positions the last round selected for client c."""
        n = np.zeros(1, dtype=np.int32)
        out = np.empty(self.U, dtype=np.uint32)
        _check(load().fednl_mx_get_selection(self._h, c, _up(out), _ip(n)))
        return out[: int(n[0])].copy()


def solve_batch(problems):
    """Ends the current round of every problem (FedNL or MixedFedNL after client_phase) with one
    cooperative launch that solves all their Option-B systems."""
    f64 = [p._h for p in problems if isinstance(p, FedNL)]
    mx = [p._h for p in problems if isinstance(p, MixedFedNL)]
    a = (C.c_void_p * max(1, len(f64)))(*f64)
    b = (C.c_void_p * max(1, len(mx)))(*mx)
    _check(load().fednl_gpu_solve_batch(a, len(f64), b, len(mx)))


def mem_info():
    """(free, total) device memory in bytes."""
    f, t = C.c_int64(0), C.c_int64(0)
    _check(load().fednl_gpu_mem_info(C.byref(f), C.byref(t)))
    return f.value, t.value
