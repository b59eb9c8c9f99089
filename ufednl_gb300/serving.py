"""The serving loop from Python: a stream of independent FedNL problems, admitted by device memory
and advanced together one round per tick by the native server (fednl_server_* in the C ABI).

``draw_stream`` makes the request stream: Poisson arrivals at ``rate`` per second; each problem
draws d from {69, 124, 301, 1024}, a client count log-uniform in [16, 512], n_i uniform in
[50, 2000], Bernoulli(p) features (p uniform in [0.05, 0.5], d-1 attributes plus the intercept
column) or N(0,1) features (all d attributes), lambda from {1e-3, 1e-4} and a TopK, RandK or
TopLEK compressor with k = 8d.  Every problem runs on the mixed-precision engine (TF32
tensor-core client Hessians, FP32 shifts, FP64 master and solve; RandK draws from the Philox
stream); ``Request.engine`` set to PRECISION_FP64 puts a problem on the FP64 engine instead.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from . import fednl
from .fednl import ProblemDesc, _check, _dp, _ip, load

PRECISION_FP64, PRECISION_MIXED = 0, 1
QUEUED, LIVE, DONE, FAILED = 0, 1, 2, 3


class TickStats(C.Structure):
    _fields_ = [("live", C.c_int32), ("admitted", C.c_int32), ("retired", C.c_int32), ("pending", C.c_int32),
                ("tick_ms", C.c_double), ("device_ms", C.c_double), ("held_bytes", C.c_int64),
                ("device_free", C.c_int64), ("device_total", C.c_int64)]


class ProblemStatus(C.Structure):
    _fields_ = [("state", C.c_int32), ("rounds", C.c_int32), ("error", C.c_int32), ("d", C.c_int32),
                ("grad_norm", C.c_double), ("t_submit_ms", C.c_double), ("t_admit_ms", C.c_double),
                ("t_done_ms", C.c_double), ("bytes", C.c_int64)]


def _lib():
    L = load()
    if not getattr(L, "_serving_sigs", False):
        vp = C.c_void_p
        for name, args in {"fednl_server_create": [C.c_int64, C.c_int64, C.c_int32, C.POINTER(vp)],
                           "fednl_server_destroy": [vp],
                           "fednl_server_submit": [vp, C.POINTER(ProblemDesc), C.c_int32, vp, C.POINTER(C.c_double),
                                                   C.c_double, C.c_int32, C.POINTER(C.c_int64)],
                           "fednl_server_tick": [vp, C.POINTER(TickStats)],
                           "fednl_server_status": [vp, C.c_int64, C.POINTER(ProblemStatus), C.POINTER(C.c_double)],
                           "fednl_server_latencies": [vp, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_int64)],
                           "fednl_server_device_times": [vp, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_int64)],
                           "fednl_server_submit_ref": [vp, C.POINTER(ProblemDesc), C.c_int32, vp, C.POINTER(C.c_double),
                                                       C.c_double, C.c_int32, C.POINTER(C.c_int64)],
                           "fednl_gpu_footprint": [C.POINTER(ProblemDesc), C.POINTER(C.c_int64)],
                           "fednl_mx_footprint": [C.POINTER(ProblemDesc), C.POINTER(C.c_int64)]}.items():
            getattr(L, name).argtypes = args
            getattr(L, name).restype = C.c_int
        L._serving_sigs = True
    return L


@dataclass
class Request:
    pid: int
    arrival_s: float
    d: int
    n_samples: np.ndarray
    kind: str            # "bernoulli" or "normal"
    density: float
    lam: float
    compressor: str      # "topk", "randk", "toplek"
    k: int
    seed: int
    engine: int = PRECISION_MIXED

    @property
    def precision(self) -> int:
        return self.engine

    @property
    def n_clients(self) -> int:
        return int(self.n_samples.shape[0])


def draw_stream(count: int, rate: float = 200.0, seed: int = 4, dims=(69, 124, 301, 1024),
                clients=(16, 512), n_range=(50, 2000)) -> list[Request]:
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for pid in range(count):
        t += rng.exponential(1.0 / rate)
        d = int(rng.choice(dims))
        nc = int(round(np.exp(rng.uniform(np.log(clients[0]), np.log(clients[1])))))
        ns = rng.integers(n_range[0], n_range[1] + 1, nc).astype(np.int32)
        kind = "bernoulli" if rng.random() < 0.5 else "normal"
        density = float(rng.uniform(0.05, 0.5))
        lam = float(rng.choice([1e-3, 1e-4]))
        comp = str(rng.choice(["topk", "randk", "toplek"]))
        out.append(Request(pid, t, d, ns, kind, density, lam, comp, 8 * d, int(rng.integers(1 << 31))))
    return out


def make_data(req: Request):
    """Row-major features [S, d] (float32 for the mixed engine, float64 otherwise) and +-1 labels."""
    rng = np.random.default_rng(req.seed)
    S = int(req.n_samples.sum())
    d = req.d
    if req.kind == "bernoulli":
        a = np.empty((S, d), dtype=np.float32)
        a[:, : d - 1] = rng.random((S, d - 1), dtype=np.float32) < np.float32(req.density)
        a[:, d - 1] = 1.0
    else:
        a = rng.standard_normal((S, d), dtype=np.float32)
    w = rng.normal(0.0, 1.0 / np.sqrt(d), size=d).astype(np.float32)
    p = 1.0 / (1.0 + np.exp(-(a @ w).astype(np.float64)))
    y = np.where(rng.random(S) < p, 1.0, -1.0)
    if req.precision == PRECISION_FP64:
        a = a.astype(np.float64)
    return np.ascontiguousarray(a), y


def make_pool_payloads(reqs: list[Request], bernoulli_density: float = 0.275, chunk: int = 1 << 16):
    """Payloads for a long request stream without one feature matrix per problem: the problems of one
    (d, kind) take row prefixes of one shared FP32 pool (N(0,1), or Bernoulli {0,1} at
    ``bernoulli_density`` -- the mean of the stream's U(0.05, 0.5) -- with the intercept column
    last), each with its own labels from its own planted w*.  Returns {pid: (features, labels)};
    the features are views into the pools, valid while the returned dict lives."""
    need = {}
    for r in reqs:
        key = (r.d, r.kind)
        need[key] = max(need.get(key, 0), int(r.n_samples.sum()))
    pools = {}
    for (d, kind), rows in sorted(need.items()):
        rng = np.random.default_rng(1000003 * d + (1 if kind == "bernoulli" else 2))
        a = np.empty((rows, d), dtype=np.float32)
        for r0 in range(0, rows, chunk):
            r1 = min(rows, r0 + chunk)
            if kind == "bernoulli":
                a[r0:r1, : d - 1] = rng.random((r1 - r0, d - 1), dtype=np.float32) < np.float32(bernoulli_density)
                a[r0:r1, d - 1] = 1.0
            else:
                a[r0:r1] = rng.standard_normal((r1 - r0, d), dtype=np.float32)
        pools[(d, kind)] = a
    out = {}
    for r in reqs:
        S = int(r.n_samples.sum())
        a = pools[(r.d, r.kind)][:S]
        rng = np.random.default_rng(r.seed)
        w = rng.normal(0.0, 1.0 / np.sqrt(r.d), size=r.d).astype(np.float32)
        p = 1.0 / (1.0 + np.exp(-(a @ w).astype(np.float64)))
        out[r.pid] = (a, np.where(rng.random(S) < p, 1.0, -1.0))
    return out


def _desc(req: Request, ns: np.ndarray) -> ProblemDesc:
    d = req.d
    U = d * (d + 1) // 2
    comp = fednl.COMPRESSORS[req.compressor]
    if req.precision == PRECISION_MIXED and req.compressor == "randk":
        comp = fednl.RANDK_PHILOX
    k = min(req.k, U)
    alpha = k / U if req.compressor == "randk" else 1.0
    fmt = 1 if req.kind == "bernoulli" else 2
    if req.precision == PRECISION_MIXED:
        fmt = 2
    return ProblemDesc(d, 0, req.n_clients, _ip(ns), req.lam, comp, k, alpha, 1, 123 + req.pid, 1234, fmt,
                       0, 1234, 0, 0, 0.5, 0.5, 5, 0, 0, 0)


def footprint(req: Request) -> int:
    ns = np.ascontiguousarray(req.n_samples, dtype=np.int32)
    b = C.c_int64(0)
    f = _lib().fednl_mx_footprint if req.precision == PRECISION_MIXED else _lib().fednl_gpu_footprint
    _check(f(C.byref(_desc(req, ns)), C.byref(b)))
    return b.value


class Server:
    """The native serving loop: submit problems at any time, tick to run one round of every live one."""

    def __init__(self, budget_bytes: int = 0, reserve_bytes: int = 1 << 30, max_live: int = 0):
        h = C.c_void_p()
        _check(_lib().fednl_server_create(budget_bytes, reserve_bytes, max_live, C.byref(h)))
        self._h = h
        self.d = {}
        self._refs = {}

    def close(self):
        if getattr(self, "_h", None):
            _lib().fednl_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, req: Request, features=None, labels=None, tol: float = 1e-9, max_rounds: int = 30) -> int:
        if features is None:
            features, labels = make_data(req)
        ns = np.ascontiguousarray(req.n_samples, dtype=np.int32)
        want = np.float32 if req.precision == PRECISION_MIXED else np.float64
        f = np.ascontiguousarray(features, dtype=want)
        y = np.ascontiguousarray(labels, dtype=np.float64)
        pid = C.c_int64(0)
        _check(_lib().fednl_server_submit(self._h, C.byref(_desc(req, ns)), req.precision, f.ctypes.data_as(C.c_void_p),
                                          _dp(y), tol, max_rounds, C.byref(pid)))
        self.d[pid.value] = req.d
        return pid.value

    def submit_ref(self, req: Request, features, labels, tol: float = 1e-9, max_rounds: int = 30) -> int:
        """Submission without a copy (fednl_server_submit_ref): the server reads features and labels
        when it admits the problem; they must stay alive and unchanged until then (the server keeps a
        reference to them here)."""
        ns = np.ascontiguousarray(req.n_samples, dtype=np.int32)
        want = np.float32 if req.precision == PRECISION_MIXED else np.float64
        f = features if (features.dtype == want and features.flags.c_contiguous) else np.ascontiguousarray(features, dtype=want)
        y = np.ascontiguousarray(labels, dtype=np.float64)
        pid = C.c_int64(0)
        _check(_lib().fednl_server_submit_ref(self._h, C.byref(_desc(req, ns)), req.precision,
                                              f.ctypes.data_as(C.c_void_p), _dp(y), tol, max_rounds, C.byref(pid)))
        self.d[pid.value] = req.d
        self._refs[pid.value] = (f, y)
        return pid.value

    def submit_problem(self, prob, compressor: str, k: int, alpha: float, precision: int = PRECISION_FP64,
                       tol: float = 1e-9, max_rounds: int = 30, seed_base: int = 123) -> int:
        """A datagen.Problem as one request (the same desc FedNL / MixedFedNL would build)."""
        ns = np.ascontiguousarray(prob.n_samples, dtype=np.int32)
        comp = fednl.COMPRESSORS[compressor]
        fmt = 2 if precision == PRECISION_MIXED else 0
        desc = ProblemDesc(prob.d, 0, prob.n_clients, _ip(ns), float(prob.lam), comp, int(k), float(alpha), 1,
                           int(seed_base), 1234, fmt, 0, 1234, 0, 0, 0.5, 0.5, 5, 0, 0, 0)
        want = np.float32 if precision == PRECISION_MIXED else np.float64
        f = np.ascontiguousarray(prob.features, dtype=want)
        y = np.ascontiguousarray(prob.labels, dtype=np.float64)
        pid = C.c_int64(0)
        _check(_lib().fednl_server_submit(self._h, C.byref(desc), precision, f.ctypes.data_as(C.c_void_p), _dp(y),
                                          tol, max_rounds, C.byref(pid)))
        self.d[pid.value] = prob.d
        return pid.value

    def tick(self) -> TickStats:
        st = TickStats()
        _check(_lib().fednl_server_tick(self._h, C.byref(st)))
        return st

    def status(self, pid: int):
        st = ProblemStatus()
        x = np.full(self.d[pid], np.nan)
        _check(_lib().fednl_server_status(self._h, pid, C.byref(st), _dp(x)))
        return st, x

    def latencies(self) -> np.ndarray:
        n = C.c_int64(0)
        _check(_lib().fednl_server_latencies(self._h, None, 0, C.byref(n)))
        out = np.empty(n.value)
        _check(_lib().fednl_server_latencies(self._h, _dp(out), n.value, C.byref(n)))
        return out

    def device_times(self) -> np.ndarray:
        """Device time in ms of every tick that had live problems."""
        n = C.c_int64(0)
        _check(_lib().fednl_server_device_times(self._h, None, 0, C.byref(n)))
        out = np.empty(n.value)
        _check(_lib().fednl_server_device_times(self._h, _dp(out), n.value, C.byref(n)))
        return out

    def run_until_idle(self, timeout_s: float = 120.0) -> list[TickStats]:
        """Ticks until nothing is queued, being admitted or live (sleeping 1 ms between ticks
        that had nothing live, while the admission thread works), or until ``timeout_s``."""
        t0 = time.perf_counter()
        ticks = []
        while True:
            st = self.tick()
            ticks.append(st)
            if (st.live == st.retired and st.pending == 0) or time.perf_counter() - t0 > timeout_s:
                return ticks
            if st.live == 0:
                time.sleep(0.001)

    def wait_settled(self, pid: int, timeout_s: float = 10.0):
        """Ticks until the problem has left the queue (admitted and run, or refused)."""
        t0 = time.perf_counter()
        while True:
            self.tick()
            st = self.status(pid)[0]
            if st.state != QUEUED or time.perf_counter() - t0 > timeout_s:
                return st
            time.sleep(0.001)


def serve(reqs: list[Request], payloads: dict, server: Server, tol: float = 1e-9, max_rounds: int = 30,
          realtime: bool = True, max_ticks: int = 100000, borrow: bool = False):
    """Submits each request when its arrival time has passed (wall clock from the call, or all at
    once without ``realtime``) and ticks until every submitted problem has retired.  Returns the
    problem ids, the per-tick stats and the wall time in seconds."""
    t0 = time.perf_counter()
    ids = {}
    ticks = []
    nxt = 0
    live_or_queued = 0
    for _ in range(max_ticks):
        now = time.perf_counter() - t0
        while nxt < len(reqs) and (not realtime or reqs[nxt].arrival_s <= now):
            r = reqs[nxt]
            f, y = payloads[r.pid]
            if borrow:
                ids[r.pid] = server.submit_ref(r, f, y, tol=tol, max_rounds=max_rounds)
            else:
                ids[r.pid] = server.submit(r, f, y, tol=tol, max_rounds=max_rounds)
            nxt += 1
        st = server.tick()
        ticks.append((time.perf_counter() - t0, st.live, st.admitted, st.retired, st.pending, st.tick_ms,
                      st.held_bytes, st.device_free, st.device_total, st.device_ms))
        live_or_queued = st.live - st.retired + st.pending
        if nxt == len(reqs) and live_or_queued == 0 and st.admitted == 0:
            break
        if st.live == 0 and st.admitted == 0:
            # nothing on the device: wait for the next arrival or for the admission thread
            wait = 0.0005 if nxt >= len(reqs) else reqs[nxt].arrival_s - (time.perf_counter() - t0)
            time.sleep(max(0.0, min(0.002, wait)))
    return ids, ticks, time.perf_counter() - t0
