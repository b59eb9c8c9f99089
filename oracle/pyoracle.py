"""ctypes binding of the CPU oracle (oracle/fednl_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py, always as the oracle (or as the timed CPU port), never by the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

IDENTITY, RANDK, TOPK, RANDSEQK, TOPLEK, NATURAL, RANDK_PHILOX = 0, 1, 2, 3, 4, 5, 6
COMPRESSORS = {"identity": IDENTITY, "randk": RANDK, "topk": TOPK, "randseqk": RANDSEQK,
               "toplek": TOPLEK, "natural": NATURAL, "randk_philox": RANDK_PHILOX}


class Problem(C.Structure):
    _fields_ = [("d", C.c_int32), ("lda", C.c_int32), ("n_clients", C.c_int32),
                ("n_samples", C.POINTER(C.c_int32)), ("features", C.POINTER(C.c_double)),
                ("labels", C.POINTER(C.c_double)), ("lambda_", C.c_double),
                ("compressor", C.c_int32), ("k", C.c_int32), ("alpha", C.c_double),
                ("workers", C.c_int32), ("threads", C.c_int32), ("seed_base", C.c_uint32),
                ("toplek_seed", C.c_uint32), ("pp", C.c_int32), ("clients_per_round", C.c_int32),
                ("client_seed", C.c_uint32), ("option_a", C.c_int32), ("line_search", C.c_int32),
                ("ls_c", C.c_double), ("ls_gamma", C.c_double), ("ls_max_steps", C.c_int32),
                ("track_f", C.c_int32), ("ref_order", C.c_int32)]


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp, up, ip = C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.POINTER(C.c_int32)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(Problem), dp]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_round.restype = C.c_int
        L.orc_round.argtypes = [C.c_void_p, dp]
        for f in ("orc_get_x", "orc_get_H", "orc_get_grad"):
            getattr(L, f).argtypes = [C.c_void_p, dp]
        L.orc_get_shift.argtypes = [C.c_void_p, C.c_int32, dp]
        L.orc_get_l.restype = C.c_double
        L.orc_get_l.argtypes = [C.c_void_p]
        L.orc_get_lk.restype = C.c_double
        L.orc_get_lk.argtypes = [C.c_void_p, C.c_int32]
        L.orc_get_true_grad.argtypes = [C.c_void_p, dp]
        L.orc_get_selected.restype = C.c_int32
        L.orc_get_selected.argtypes = [C.c_void_p, ip]
        L.orc_get_dir.argtypes = [C.c_void_p, C.c_int32, dp, dp]
        L.orc_get_f.restype = C.c_double
        L.orc_get_f.argtypes = [C.c_void_p]
        L.orc_get_ls_steps.restype = C.c_int32
        L.orc_get_ls_steps.argtypes = [C.c_void_p]
        for f in ("orc_log", "orc_exp", "orc_exp_vcl", "orc_exp_cr", "orc_log_vcl"):
            getattr(L, f).restype = C.c_double
            getattr(L, f).argtypes = [C.c_double]
        L.orc_get_message.restype = C.c_int32
        L.orc_get_message.argtypes = [C.c_void_p, C.c_int32, up, dp]
        L.orc_upper_indices.argtypes = [C.c_int32, C.c_int32, up]
        L.orc_topk.restype = C.c_int32
        L.orc_topk.argtypes = [dp, C.c_int32, C.c_size_t, up, up]
        L.orc_toplek.restype = C.c_int32
        L.orc_toplek.argtypes = [dp, C.c_int32, C.c_int32, C.c_size_t, up, C.c_double, C.c_double, up, up]
        L.orc_randk.argtypes = [up, C.c_int32, C.c_size_t, up, up]
        L.orc_randseqk.argtypes = [up, C.c_int32, C.c_size_t, up, up]
        L.orc_randk_philox.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32, C.c_size_t, up, up]
        L.orc_philox4x32.argtypes = [up, up, up]
        L.orc_natural.restype = C.c_double
        L.orc_natural.argtypes = [C.c_double]
        L.orc_pack2_natural.restype = C.c_uint32
        L.orc_pack2_natural.argtypes = [C.c_double, C.c_double]
        L.orc_l2sq.restype = C.c_double
        L.orc_l2sq.argtypes = [dp, C.c_size_t]
        L.orc_ldlt.restype = C.c_int
        L.orc_ldlt.argtypes = [dp, C.c_int32, C.c_int32, C.c_double, dp]
        L.orc_solve_ldlt.argtypes = [dp, C.c_int32, C.c_int32, dp, dp]
        L.orc_cholesky_ref.restype = C.c_int
        L.orc_cholesky_ref.argtypes = [dp, C.c_int32, C.c_int32, C.c_double, dp]
        L.orc_solve_chol_ref.argtypes = [dp, C.c_int32, C.c_int32, dp, dp]
        L.orc_margin.argtypes = [dp, C.c_int32, C.c_int32, C.c_int32, dp, dp]
        L.orc_sigmoid.argtypes = [dp, C.c_int32, dp]
        L.orc_gradient.argtypes = [dp, C.c_int32, C.c_int32, C.c_int32, dp, dp, C.c_double, dp]
        L.orc_hessian.argtypes = [dp, C.c_int32, C.c_int32, C.c_int32, dp, C.c_double, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _up(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def upper_indices(d: int, lda: int) -> np.ndarray:
    out = np.empty(d * (d + 1) // 2, dtype=np.uint32)
    lib().orc_upper_indices(d, lda, _up(out))
    return out


def topk(m_full: np.ndarray, d: int, lda: int, k: int) -> np.ndarray:
    """m_full: column-major d x lda buffer (flattened, length d*lda)."""
    m = np.ascontiguousarray(m_full, dtype=np.float64)
    up = upper_indices(d, lda)
    out = np.empty(max(k, up.size), dtype=np.uint32)
    n = lib().orc_topk(_dp(m), k, up.size, _up(up), _up(out))
    return out[:n].copy()


def toplek(m_full: np.ndarray, d: int, lda: int, k: int, rng_state: np.ndarray) -> np.ndarray:
    """rng_state: uint32[1] worker generator state, advanced in place."""
    m = np.ascontiguousarray(m_full, dtype=np.float64)
    up = upper_indices(d, lda)
    out = np.empty(up.size, dtype=np.uint32)
    frob = lib().orc_l2sq(_dp(m), m.size)
    delta = float(k) * (1.0 / float(up.size))
    n = lib().orc_toplek(_dp(m), lda, k, up.size, _up(up), delta, frob, _up(rng_state), _up(out))
    return out[:n].copy()


def randk(rng_state: np.ndarray, d: int, lda: int, k: int) -> np.ndarray:
    up = upper_indices(d, lda)
    out = np.empty(k, dtype=np.uint32)
    lib().orc_randk(_up(rng_state), k, up.size, _up(up), _up(out))
    return out


def randseqk(rng_state: np.ndarray, d: int, lda: int, k: int) -> np.ndarray:
    up = upper_indices(d, lda)
    out = np.empty(k, dtype=np.uint32)
    lib().orc_randseqk(_up(rng_state), k, up.size, _up(up), _up(out))
    return out


def cholesky_solve(h_full: np.ndarray, d: int, lda: int, l: float, b: np.ndarray):
    h = np.ascontiguousarray(h_full, dtype=np.float64)
    ltr = np.zeros(d * lda)
    ok = lib().orc_ldlt(_dp(h), d, lda, l, _dp(ltr))
    x = np.zeros(d)
    if ok:
        bb = np.ascontiguousarray(b, dtype=np.float64)
        lib().orc_solve_ldlt(_dp(ltr), d, lda, _dp(bb), _dp(x))
    return bool(ok), x


class FedNL:
    """Whole FedNL run on the CPU oracle (master merges clients in order)."""

    def __init__(self, prob, compressor, k, alpha, lda=None, workers=1, threads=None,
                 seed_base=123, toplek_seed=1234, x0=None, clients_per_round=None, client_seed=1234,
                 option_a=False, line_search=None, track_f=False, ref_order=False):
        """clients_per_round set: FedNL-PP (bin_fednl_local_pp) with that many clients per round.
        option_a: Cholesky of H + lambda I (--fednl-option-a).  line_search = (c, gamma, max_steps):
        FedNL-LS (--line_search).  track_f: form f(x) every round (--tracking).  ref_order: the
        reference's own operation order (bit-exact with the reference's no-FMA AVX2 build)."""
        self.d = prob.d
        self.lda = lda if lda is not None else (prob.d + 3) // 4 * 4
        self._keep = [np.ascontiguousarray(prob.n_samples, dtype=np.int32),
                      np.ascontiguousarray(prob.features, dtype=np.float64),
                      np.ascontiguousarray(prob.labels, dtype=np.float64)]
        comp = COMPRESSORS[compressor] if isinstance(compressor, str) else int(compressor)
        p = Problem(self.d, self.lda, prob.n_clients,
                    self._keep[0].ctypes.data_as(C.POINTER(C.c_int32)),
                    _dp(self._keep[1]), _dp(self._keep[2]), prob.lam, comp, int(k), float(alpha),
                    int(workers), int(threads if threads else workers), seed_base, toplek_seed,
                    1 if clients_per_round else 0, int(clients_per_round or 0), client_seed,
                    1 if option_a else 0, 1 if line_search else 0,
                    float(line_search[0]) if line_search else 0.5, float(line_search[1]) if line_search else 0.5,
                    int(line_search[2]) if line_search else 5, 1 if track_f else 0, 1 if ref_order else 0)
        self.pp = bool(clients_per_round)
        x0 = np.zeros(self.d) if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
        self._h = lib().orc_create(C.byref(p), _dp(x0))
        self.n_clients = prob.n_clients

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def round(self) -> float:
        g = C.c_double(0.0)
        rc = lib().orc_round(self._h, C.byref(g))
        if rc != 0:
            raise RuntimeError("oracle: Cholesky failed (matrix not positive definite)")
        return g.value

    def x(self) -> np.ndarray:
        out = np.empty(self.d)
        lib().orc_get_x(self._h, _dp(out))
        return out

    def grad(self) -> np.ndarray:
        out = np.empty(self.d)
        lib().orc_get_grad(self._h, _dp(out))
        return out

    def H(self) -> np.ndarray:
        out = np.empty(self.d * self.lda)
        lib().orc_get_H(self._h, _dp(out))
        return out

    def shift(self, c: int) -> np.ndarray:
        out = np.empty(self.d * self.lda)
        lib().orc_get_shift(self._h, c, _dp(out))
        return out

    def l(self) -> float:
        return lib().orc_get_l(self._h)

    def true_grad(self) -> np.ndarray:
        out = np.empty(self.d)
        lib().orc_get_true_grad(self._h, _dp(out))
        return out

    def f(self) -> float:
        return lib().orc_get_f(self._h)

    def ls_steps(self) -> int:
        return lib().orc_get_ls_steps(self._h)

    def selected(self) -> np.ndarray:
        out = np.empty(self.n_clients, dtype=np.int32)
        n = lib().orc_get_selected(self._h, out.ctypes.data_as(C.POINTER(C.c_int32)))
        return out[:n].copy()

    def dir(self, c: int):
        dr, dd = np.empty(self.d), np.empty(self.d)
        lib().orc_get_dir(self._h, c, _dp(dr), _dp(dd))
        return dr, dd

    def lk(self, c: int) -> float:
        return lib().orc_get_lk(self._h, c)

    def message(self, c: int):
        U = self.d * (self.d + 1) // 2
        idx = np.empty(U, dtype=np.uint32)
        val = np.empty(U)
        n = lib().orc_get_message(self._h, c, _up(idx), _dp(val))
        return idx[:n].copy(), val[:n].copy()
