"""Benchmark of the FedNL round on GB300: rounds/s of the w8a-like workload (d=301, 142 clients,
n_i ~ U{200..600}, TopLEK k=8d, alpha=1, Option B, FP64 throughout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload w8a|a9a]

A step is one FedNL round over all clients.  Prints one JSON line (rank 0).  ``--impl reference``
times the reference algorithm's CPU implementation (the C port in oracle/, every host thread)
on the same workload.  Under torchrun every rank runs an independent replica on its own GPU
(the round has no cross-GPU exchange); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "FedNL rounds/s & time to ‖∇f‖≤1e-9 (mixed vs FP64 GPU vs host CPU); p99 round ms"
L2_FLUSH_BYTES = 256 << 20          # > 129 MB L2: every timed round starts cold
TOL = 1e-9


def workload(name: str):
    from ufednl_gb300 import datagen
    if name == "a9a":
        return datagen.workload_a9a_like(), "topk", 8 * 124
    return datagen.workload_w8a_like(), "toplek", 8 * 301


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws):
    if ws <= 1:
        return None
    import torch.distributed as td
    td.init_process_group("gloo")
    return td


def dist_max(td, v: float) -> float:
    if td is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(td):
    if td is not None:
        td.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"fednl_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.idx), "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        j = json.load(open(p))
        return float(j["hbm_gbs"]), float(j["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def algorithmic_bytes(kernel: str, prob, k: int) -> tuple[float, str]:
    """Algorithmic HBM bytes of one launch of a round kernel on this workload."""
    d = prob.d
    U = d * (d + 1) // 2
    nc = prob.n_clients
    S = prob.total_samples
    words = int(sum(d * ((int(n) + 63) // 64) for n in prob.n_samples))
    if kernel == "k_hess_hits":
        # read every client's shift, write its difference (packed upper FP64), read D
        return nc * U * 16.0 + S * 8.0, "shift read + diff write (packed upper, FP64) per client, D_s read"
    if kernel.startswith("k_hess"):
        # read every client's shift, write its difference (packed upper FP64), read bitmasks and D
        return nc * U * 16.0 + words * 8.0 + S * 8.0, "shift read + diff write (packed upper, FP64) per client"
    if kernel == "k_select":
        return nc * U * 8.0, "read every client's difference once"
    if kernel == "k_apply":
        return nc * (U + 31) // 32 * 4.0 + 2 * U * 8.0, "selection bitmaps + H read/write"
    if kernel == "k_chol_coop":
        return U * 8.0 + 2 * d * 8.0, "H read (packed upper) + g read + step write; latency-bound FP64 chain"
    return 0.0, "n/a"


def hess_fp64_ops(prob) -> float:
    """FP64 operations of one binary Hessian launch in the TopK / TopLEK round: for every client and
    upper entry (i, j) one add per sample after the first with both attributes set (the in-order sum
    of D_s; the first term is exact and costs none), the diagonal's + lambda (the intercept column is
    the attribute's D_s sum, already formed), then the difference (1 more; the squares of the norm
    are formed by the selection kernel)."""
    d = prob.d
    U = d * (d + 1) // 2
    tot = 0.0
    for c in range(prob.n_clients):
        a = prob.features[prob.client_slice(c)]
        g = a.T @ a
        off = np.triu(g, 1)
        if a.shape[0] and np.all(a[:, -1] == 1.0):
            off[:, -1] = 0.0
        tot += float(np.maximum(off - 1.0, 0.0).sum()) + d
    return tot + 1.0 * prob.n_clients * U


# what limits each FP64 round kernel, in words (the roofline entries give the numbers)
SLOWEST_BOUND = {
    "k_select": "latency (the reference heap's sequential root replacements and extractions, one warp per client; "
                "the launch lasts as long as its slowest client)",
    "k_chol_coop": "latency (per-column FP64 dependency chain and grid barriers)",
    "k_hess_binary": "instruction issue and the FP64 pipe (in-order sums over bit-mask intersections)",
    "k_hess_hits": "latency of the record sums and the FP64 pipe (differences and in-order sums), HBM third",
}


def kernel_roofline(name: str, ms: float, bound: str, work: float, peak: float, unit: str, what: str,
                    peak_source: str) -> dict:
    """achieved = algorithmic work per launch / mean launch time (CUDA events); frac = achieved / peak."""
    scale = 1e9 if unit in ("GB/s", "Gop/s") else 1e12
    ach = work / (ms * 1e-3) / scale if ms > 0 else 0.0
    return {"kernel": name, "bound": bound, "achieved": ach, "peak": peak, "unit": unit, "frac": ach / peak,
            "traffic": traffic_from_profiles(name), "work_per_launch": work, "work": what, "kernel_ms": ms,
            "peak_source": peak_source}


def traffic_from_profiles(kernel: str):
    """DRAM bytes per launch recorded from an ncu capture in profiles/<kernel>*.md, if any."""
    pdir = os.path.join(REPO, "profiles")
    if not os.path.isdir(pdir):
        return None
    for fn in sorted(os.listdir(pdir)):
        if fn.startswith(kernel) and fn.endswith(".md"):
            for line in open(os.path.join(pdir, fn)):
                if line.strip().startswith("traffic_bytes_per_launch:"):
                    try:
                        return float(line.split(":", 1)[1].split()[0])
                    except ValueError:
                        return None
    return None


def upload_bytes(prob) -> int:
    """Host->device bytes fednl_gpu_upload_client_data copies for binary features."""
    d = prob.d
    S = prob.total_samples
    words = int(sum(d * ((int(n) + 63) // 64) for n in prob.n_samples))
    nnz = int(np.count_nonzero(prob.features))
    return words * 8 + nnz * 4 + (S + 1) * 4 + prob.n_clients * 8 + S * 8


def cpu_port_rounds_per_s(prob, comp, k, threads: int, max_rounds: int, budget_s: float):
    from oracle import pyoracle
    pyoracle.build()
    orc = pyoracle.FedNL(prob, comp, k, 1.0, workers=threads, threads=threads)
    orc.round()                                           # warm-up round
    t0 = time.perf_counter()
    n = 0
    while n < max_rounds:
        orc.round()
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    orc.close()
    return n / dt, n, dt


# The port against the reference's own operators on the same 8 x86 cores (Xeon @ 2.70 GHz), measured
# with oracle/time_reference.py where the reference sources are available (reference built with its
# Release options -O3 -march=native, AVX-512 and FMA): the reference's round is faster than the port,
# so a GPU / port ratio overstates the GPU / reference ratio by the inverse of these factors.
PORT_CALIBRATION = {"port_over_reference_native": {"w8a-like d301 TopLEK": 0.339, "a9a-like d124 TopK": 0.492},
                    "measured": "8 threads each, x86 Xeon @ 2.70 GHz, oracle/time_reference.py, 16 rounds",
                    "reference_rounds_per_s": {"w8a-like d301 TopLEK": 19.76, "a9a-like d124 TopK": 94.83},
                    "port_rounds_per_s": {"w8a-like d301 TopLEK": 6.70, "a9a-like d124 TopK": 46.70}}


def cpu_port_time_to_tol(prob, comp, k, threads: int, cap: int = 60):
    """The CPU port from x0 = 0 until ||g|| <= TOL (or cap rounds): rounds and wall seconds."""
    from oracle import pyoracle
    pyoracle.build()
    orc = pyoracle.FedNL(prob, comp, k, 1.0, workers=threads, threads=threads)
    t0 = time.perf_counter()
    rounds = None
    for r in range(cap):
        if orc.round() <= TOL:
            rounds = r + 1
            break
    dt = time.perf_counter() - t0
    orc.close()
    return {"tol": TOL, "rounds": rounds, "seconds": dt if rounds else None, "cap": cap,
            "timed": "wall clock of rounds 1..R from x0 = 0"}


def reference_order_rounds(fednl, prob, comp, k, workers: int, n: int):
    """The workload in the reference's arithmetic order (desc.arith_order = reference: rounds
    bit-identical to the reference's own): device-timed rounds with a cold L2 before each, and the
    per-kernel breakdown."""
    fed = fednl.FedNL(prob, comp, k, 1.0, workers=workers, order="reference")
    fed.run(3)
    tot, per = fed.time_rounds(n, L2_FLUSH_BYTES)
    prof = fed.profile_kernels(min(n, 20), L2_FLUSH_BYTES)
    fed.close()
    return {"rounds_per_s": n / (tot / 1000.0), "round_ms_p50": float(np.percentile(per, 50)),
            "round_ms_p99": float(np.percentile(per, 99)), "rounds_timed": n, "kernels_ms": dict(prof)}


def mixed_accuracy(fednl, prob_mx, prob64, comp, k, alpha, cap: int, fp64_to_tol: bool, feature_format: int = 0):
    """The mixed-precision form run until its ||g|| <= TOL (or cap rounds), then the true FP64 gradient
    at its final iterate from the FP64 engine (one round from that iterate reports ||grad f(x)||), and,
    when fp64_to_tol, the FP64 GPU form run to TOL from x0 for the iterate comparison."""
    mx = fednl.MixedFedNL(prob_mx, k, alpha, compressor=comp)
    mx.autotune()
    g_mx, rounds = None, None
    for r in range(cap):
        g_mx = float(mx.run(1)[0])
        if g_mx <= TOL:
            rounds = r + 1
            break
    x_mx = mx.x()
    mx.close()
    f64 = fednl.FedNL(prob64, comp, k, alpha, feature_format=feature_format)
    f64.set_x(x_mx)
    g_true = float(f64.round())
    f64.close()
    out = {"compressor": comp, "k": k, "tol": TOL, "round_cap": cap, "mixed_rounds_to_tol": rounds,
           "mixed_grad_norm": g_mx, "fp64_grad_norm_at_mixed_iterate": g_true,
           "grad_norm_error_vs_fp64": abs(g_mx - g_true) / g_true if g_true > 0 else None,
           "meets_tol_in_fp64": g_true <= TOL}
    if fp64_to_tol:
        f64 = fednl.FedNL(prob64, comp, k, alpha, feature_format=feature_format)
        r64 = None
        for r in range(cap):
            if f64.round() <= TOL:
                r64 = r + 1
                break
        x64 = f64.x()
        f64.close()
        out["fp64_rounds_to_tol"] = r64
        out["iterate_rel_diff_vs_fp64"] = float(np.linalg.norm(x_mx - x64) / np.linalg.norm(x64))
    return out


def run_reference(args, ws, rank, td):
    prob, comp, k = workload(args.workload)
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    warm = max(0, args.warmup)
    from oracle import pyoracle
    pyoracle.build()
    orc = pyoracle.FedNL(prob, comp, k, 1.0, workers=threads, threads=threads)
    for _ in range(min(warm, 2)):
        orc.round()
    t0 = time.perf_counter()
    n = 0
    while n < args.steps:
        orc.round()
        n += 1
        if time.perf_counter() - t0 > 90.0:
            break
    dt = time.perf_counter() - t0
    orc.close()
    v = n / dt
    sample = (f"{n} full rounds of the workload (of {args.steps} requested; 90 s cap), "
              f"{threads} threads, C port of the reference round (oracle/fednl_oracle.c)")
    line = {"metric": METRIC, "value": v, "unit": "rounds/s", "n_gpus": args.gpus, "steps": n,
            "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": config_dict(prob, comp, k, threads),
            "cpu_baseline": {"value": v, "unit": "rounds/s", "cores": threads, "kind": "port", "sample": sample,
                             "calibration": PORT_CALIBRATION},
            "e2e": {"value": v, "unit": "rounds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def extra_workloads(fednl, threads: int, steps: int):
    """The other configurations of the reference's benchmark set, device-timed the same way (cold L2
    before every round) beside a bounded sample of the CPU port: the a9a-like FedNL TopK run and the
    phishing-like FedNL-PP runs (2048 clients x 6 samples, tau = 128; RandSeqK and Natural)."""
    from ufednl_gb300 import datagen
    from oracle import pyoracle
    out = {}
    U69 = 69 * 70 // 2
    cases = [("a9a-like d124 80x407 TopK k=8d", datagen.workload_a9a_like(), "topk", 8 * 124, 1.0, 0),
             ("phishing-like d69 2048x6 FedNL-PP tau=128 RandSeqK k=d", datagen.workload_phishing_pp(),
              "randseqk", 69, 69 / U69, 128),
             ("phishing-like d69 2048x6 FedNL-PP tau=128 Natural", datagen.workload_phishing_pp(),
              "natural", U69, 1.0 / (1.0 + 1.0 / 8.0), 128)]
    n = max(20, min(steps, 200))
    for name, prob, comp, k, alpha, tau in cases:
        fed = fednl.FedNL(prob, comp, k, alpha, workers=threads, clients_per_round=tau)
        fed.run(3)
        tot, per = fed.time_rounds(n, L2_FLUSH_BYTES)
        prof = fed.profile_kernels(min(n, 20), L2_FLUSH_BYTES)
        fed.close()
        orc = pyoracle.FedNL(prob, comp, k, alpha, workers=threads, threads=threads,
                             clients_per_round=tau or None)
        orc.round()
        t0 = time.perf_counter()
        m = 0
        while m < 200 and time.perf_counter() - t0 < 3.0:
            orc.round()
            m += 1
        cpu = m / (time.perf_counter() - t0)
        orc.close()
        top = max(prof, key=lambda t: t[1])
        out[name] = {"rounds_per_s": n / (tot / 1000.0), "round_ms_p50": float(np.percentile(per, 50)),
                     "round_ms_p99": float(np.percentile(per, 99)), "rounds_timed": n,
                     "top_kernel": {"name": top[0], "ms": top[1]}, "gpu_launches_per_round": len(prof),
                     "cpu_port_rounds_per_s": cpu, "cpu_port_sample": f"{m} rounds, {threads} threads"}
    return out


def mixed_workload(fednl, threads: int, tensor_peak_tflops: float, src: str):
    """The mixed-precision configuration: dense N(0,1) FP32 features, d=1024, 256 clients with
    n_i ~ U{512..4096} (seed 2), lambda 1e-4, RandK-Philox k=4d.  The mixed round (TF32 tensor-core
    Hessians) is device-timed; the mixed form then runs to ||g|| <= 1e-9 (or 400 rounds) and the FP64
    engine evaluates the true gradient at its final iterate; the FP64 GPU round and the CPU port are
    timed on a bounded sample of the same data (the FP64 form is not run to tolerance here: about
    3.6 s a round at this size)."""
    from ufednl_gb300 import datagen
    from oracle import pyoracle
    prob = datagen.workload_dense_fp32_1024()
    d, k = prob.d, 4 * prob.d
    U = d * (d + 1) // 2
    alpha = k / U
    mx = fednl.MixedFedNL(prob, k, alpha)
    mx.run(2)
    tuned = mx.autotune()
    tot, per = mx.time_rounds(20, L2_FLUSH_BYTES)
    prof = mx.profile_kernels(5)
    mx.close()
    gram_ms = dict(prof)["k_gram_tf32"]
    flops = float(prob.total_samples) * d * (d + 1)          # upper triangle incl. diagonal, 2 flops per MAC
    tf = flops / (gram_ms * 1e-3) / 1e12
    p64 = datagen.Problem(d, prob.n_samples, prob.features.astype(np.float64), prob.labels, prob.lam)
    acc = mixed_accuracy(fednl, prob, p64, "randk_philox", k, alpha, 400, False, feature_format=2)
    f64 = fednl.FedNL(p64, "randk_philox", k, alpha, feature_format=2)
    tot64, _ = f64.time_rounds(2)
    f64.close()
    orc = pyoracle.FedNL(p64, "randk_philox", k, alpha, workers=threads, threads=threads)
    t0 = time.perf_counter()
    orc.round()
    cpu_s = time.perf_counter() - t0
    orc.close()
    return {"rounds_per_s": 20 / (tot / 1000.0), "round_ms_p50": float(np.percentile(per, 50)),
            "round_ms_p99": float(np.percentile(per, 99)), "kernels_ms": dict(prof),
            "tensor": {"kernel": "k_gram_tf32", "precision": "tf32 x tf32 -> fp32 (tcgen05.mma kind::tf32)",
                       "flops_per_launch": flops, "achieved_tflops": tf, "peak_tflops": tensor_peak_tflops,
                       "frac": tf / tensor_peak_tflops,
                       "peak_source": f"{src}: MEASURED_PEAKS.json bf16_tflops / 2 (tf32 rate)"},
            "autotuned": tuned,
            "fp64_gpu_rounds_per_s": 2 / (tot64 / 1000.0), "cpu_port_rounds_per_s": 1.0 / cpu_s,
            "cpu_port_sample": f"1 round, {threads} threads",
            "accuracy_vs_fp64": acc}


def mixed_headline(fednl, prob, comp, k, steps: int, fp64_rounds_per_s: float, fp64_tol_s):
    """The mixed-precision form on the headline workload (w8a-like, d = 301 padded to 384 on the
    tensor cores, TopLEK k = 8d): device-timed rounds with a cold L2 before each, the rounds and
    device time to ||g|| <= 1e-9 from x0 = 0, and the speed-up over the FP64 GPU form."""
    mx = fednl.MixedFedNL(prob, k, 1.0, compressor=comp)
    mx.run(2)
    tuned = mx.autotune()                  # solver and CTA count for this d, cached for the process
    mx.close()
    mx = fednl.MixedFedNL(prob, k, 1.0, compressor=comp)
    mx.autotune()
    g = mx.run(200)
    mx.close()
    hit = np.nonzero(g <= TOL)[0]
    rounds_to_tol = int(hit[0]) + 1 if hit.size else None
    mx = fednl.MixedFedNL(prob, k, 1.0, compressor=comp)
    mx.autotune()
    tol_ms = mx.time_rounds(rounds_to_tol, L2_FLUSH_BYTES)[0] if rounds_to_tol else None
    mx.close()
    mx = fednl.MixedFedNL(prob, k, 1.0, compressor=comp)
    mx.autotune()
    mx.run(3)
    n = max(20, min(steps, 300))
    tot, per = mx.time_rounds(n, L2_FLUSH_BYTES)
    prof = mx.profile_kernels(10)
    mx.close()
    rps = n / (tot / 1000.0)
    # round-level bound: the slower of the tensor-core work (the padded client Gram matrices' upper
    # tiles in TF32) and the FP32 shift stream (read, difference written, shift written back)
    hbm, bf16, src = peaks()
    dp = (prob.d + 127) // 128 * 128
    tiles = (dp // 128) * (dp // 128 + 1) // 2
    gram_flops = 2.0 * prob.total_samples * 128 * 128 * tiles
    U = prob.d * (prob.d + 1) // 2
    shift_bytes = 3.0 * prob.n_clients * U * 4
    t_tensor = gram_flops / (bf16 / 2.0 * 1e12) * 1e3
    t_hbm = shift_bytes / (hbm * 1e9) * 1e3
    bound_ms = max(t_tensor, t_hbm)
    km = dict(prof)
    S = float(prob.total_samples)
    hsrc = f"{src} (MEASURED_PEAKS.json hbm_gbs)"
    mx_roof = [kernel_roofline("k_gram_tf32", km.get("k_gram_tf32", 0.0), "tensor", S * prob.d * (prob.d + 1),
                               bf16 / 2.0, "TFLOP/s", "client Gram upper triangles incl. diagonal, 2 flops per MAC",
                               f"{src}: MEASURED_PEAKS.json bf16_tflops / 2 (tf32 rate)"),
               kernel_roofline("k_mx_select", km.get("k_mx_select", 0.0), "hbm", prob.n_clients * U * 4.0, hbm,
                               "GB/s", "every client's FP32 difference read once", hsrc),
               kernel_roofline("k_mx_margin", km.get("k_mx_margin", 0.0), "hbm", S * prob.d * 4.0, hbm, "GB/s",
                               "the FP32 features read once", hsrc)]
    return {"rounds_per_s": rps, "round_ms_p50": float(np.percentile(per, 50)),
            "round_roofline": {"bound": "tensor" if t_tensor >= t_hbm else "hbm", "gram_tf32_flops": gram_flops,
                               "shift_stream_bytes": shift_bytes, "lower_bound_ms": bound_ms,
                               "round_ms": tot / n, "frac": bound_ms / (tot / n),
                               "peaks": f"{src}: tf32 = bf16_tflops / 2, hbm_gbs"},
            "round_ms_p99": float(np.percentile(per, 99)), "rounds_timed": n, "kernels_ms": dict(prof),
            "roofline_kernels": mx_roof,
            "gpu_launches_per_round": len(prof),
            "time_to_tol": {"tol": TOL, "rounds": rounds_to_tol,
                            "seconds": tol_ms / 1000.0 if tol_ms is not None else None},
            "speedup_vs_fp64_gpu_rounds_per_s": rps / fp64_rounds_per_s,
            "speedup_vs_fp64_gpu_time_to_tol": (fp64_tol_s / (tol_ms / 1000.0))
            if (fp64_tol_s and tol_ms) else None,
            "autotuned": tuned,
            "accuracy_vs_fp64": [mixed_accuracy(fednl, prob, prob, c_, k, 1.0, 200, True) for c_ in (comp, "topk")],
            "precision": "TF32 tensor-core client Hessians (FP32 accumulate), FP32 shifts and selection, "
                         "float-float margins/gradients, FP64 master; solve as autotuned (FP64 Cholesky; FP32 "
                         "Cholesky on a cooperative grid or cluster with FP64-residual refinement to 2^-30; or "
                         "FP32 one-CTA Cholesky with one float-float refinement step)"}


def serving_workload(fednl, count: int = 200, max_rounds: int = 40):
    """The serving loop on the request stream (Poisson arrivals at 200/s, seed 4; d in {69, 124, 301,
    1024}, 16-512 clients, n_i 50-2000, Bernoulli or N(0,1) features, TopK / RandK / TopLEK with
    k = 8d), every problem on the mixed-precision engine, retired at ||g|| <= 1e-9 or after max_rounds
    rounds.  Payloads are prepared before the clock (row prefixes of shared per-(d, kind) pools with
    per-problem labels; submitted without a copy); the clock covers submission at each arrival time,
    admission on the server's own thread (create, upload, initial shifts), every tick and retirement."""
    from ufednl_gb300 import serving
    reqs = serving.draw_stream(count, rate=200.0, seed=4)
    payloads = serving.make_pool_payloads(reqs)
    srv = serving.Server(reserve_bytes=8 << 30)
    ids, ticks, wall = serving.serve(reqs, payloads, srv, tol=TOL, max_rounds=max_rounds, realtime=True, borrow=True)
    lat = srv.latencies()
    dev = srv.device_times()
    sts = [srv.status(ids[r.pid])[0] for r in reqs]
    srv.close()
    done = [s for s in sts if s.state == serving.DONE]
    conv = [s for s in done if s.grad_norm <= TOL]
    resp = [s.t_done_ms - s.t_submit_ms for s in done]
    wait = [s.t_admit_ms - s.t_submit_ms for s in sts if s.t_admit_ms >= 0]
    held = [t[6] for t in ticks]
    total = ticks[-1][8] if ticks else 0

    def pct(v, q):
        return float(np.percentile(v, q)) if len(v) else None
    return {"problems": count, "done": len(done), "failed": sum(s.state == serving.FAILED for s in sts),
            "converged": len(conv), "capped": len(done) - len(conv),
            "problems_per_s": len(done) / wall, "converged_per_s": len(conv) / wall, "wall_s": wall,
            "ticks": len(ticks),
            "queue_wait_ms": {"p50": pct(wait, 50), "p99": pct(wait, 99)},
            "round_latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99),
                                 "measured": "host clock from the tick's first launch to the problem's result"},
            "tick_device_ms": {"p50": pct(dev, 50), "p99": pct(dev, 99),
                               "measured": "CUDA events: every live problem's client phase to the batched solve's "
                                           "end; admission runs on the server's own thread, outside the ticks"},
            "problem_latency_ms": {"p50": pct(resp, 50), "p99": pct(resp, 99)},
            "rounds_total": int(len(lat)), "max_live": int(max(t[1] for t in ticks)) if ticks else 0,
            "hbm_held_gb": {"max": max(held) / 1e9 if held else 0.0, "mean": float(np.mean(held)) / 1e9 if held else 0.0},
            "hbm_total_gb": total / 1e9,
            "max_rounds": max_rounds, "arrivals": "Poisson 200/s (seed 4), submitted at their arrival times",
            "data": "per-(d, kind) shared FP32 pools, problems take row prefixes; Bernoulli pools at density "
                    "0.275 (the mean of the stream's U(0.05, 0.5)); labels per problem from its own w*",
            "solve": "one batched launch per tick: FP64 cooperative Cholesky groups for the problems whose "
                     "autotuned solver is not the FP32 one-CTA factor, one FP32 one-CTA factor per problem "
                     "with d <= 304 otherwise"}


def config_dict(prob, comp, k, workers):
    return {"workload": prob.name, "d": prob.d, "clients": prob.n_clients, "samples": prob.total_samples,
            "compressor": comp, "k": k, "alpha": 1.0, "option": "B", "lambda": prob.lam, "workers": workers,
            "precision": "fp64", "l2": f"flushed before every timed round ({L2_FLUSH_BYTES >> 20} MB write)",
            "parallelism": "replicas"}


def run_ours(args, ws, rank, local, td):
    from ufednl_gb300 import build, fednl
    build.build()
    prob, comp, k = workload(args.workload)
    W = args.workers or (os.cpu_count() or 1)
    fed = fednl.FedNL(prob, comp, k, 1.0, workers=W)
    # convergence trace: rounds to ||g|| <= 1e-9 from x0 (device-timed below)
    gtrace = fed.run(max(args.warmup, 3))
    tuned = fed.autotune()                 # cooperative Cholesky CTA count (results do not depend on it)
    dist_barrier(td)
    with ClockSampler(local) as clk:
        total_ms, per = fed.time_rounds(args.steps, L2_FLUSH_BYTES)
    clocks = clk.summary()
    total_ms = dist_max(td, total_ms)
    dist_barrier(td)
    value = ws * args.steps / (total_ms / 1000.0)
    ms_per_step = total_ms / args.steps

    # per-kernel breakdown with CUDA events on the library's stream
    prof = fed.profile_kernels(min(args.steps, 50), L2_FLUSH_BYTES)
    kernels = {n: ms for n, ms in prof}
    hbm, bf16, src = peaks()
    fp64 = fednl.fp64_rate()              # this GPU's FP64 pipe, the FP64 kernels' denominator
    hsrc = f"{src} (MEASURED_PEAKS.json hbm_gbs)"
    fsrc = "measured by fednl_gpu_fp64_rate in this run (independent FP64 add chains, all SMs)"
    # the kernels the round's bound is about, by name (the same set whatever --steps is): the shift
    # stream (the binary Hessian reads every shift and writes every difference; k_select reads every
    # difference once) against HBM, the Hessian's in-order sums against the FP64 pipe, and the
    # Cholesky's latency chain in cycles per column
    hname = "k_hess_hits" if "k_hess_hits" in kernels else "k_hess_binary"
    hb, hwhat = algorithmic_bytes(hname, prob, k)
    hops = hess_fp64_ops(prob)
    sb, swhat = algorithmic_bytes("k_select", prob, k)
    r_hess_hbm = kernel_roofline(hname, kernels.get(hname, 0.0), "hbm", hb, hbm, "GB/s", hwhat, hsrc)
    r_hess_fp64 = kernel_roofline(hname, kernels.get(hname, 0.0), "fp64", hops, fp64["add_gops"],
                                  "Gop/s", "in-order D_s sums (one add per sample after the first with both attributes set) "
                                  "+ the difference per upper entry", fsrc)
    r_select = kernel_roofline("k_select", kernels.get("k_select", 0.0), "hbm", sb, hbm, "GB/s", swhat, hsrc)
    chol_ms = kernels.get("k_chol_coop", 0.0)
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    r_chol = {"kernel": "k_chol_coop", "bound": "latency (per-column FP64 dependency chain and grid barriers)",
              "kernel_ms": chol_ms, "cycles_per_column": chol_ms * 1e-3 * sm_mhz * 1e6 / prob.d,
              "sm_mhz": sm_mhz, "fp64_add_latency_cycles": fp64["add_latency_cycles"]}
    roof = dict(r_hess_hbm)
    roof["fp64"] = {k_: r_hess_fp64[k_] for k_ in ("achieved", "peak", "unit", "frac", "work_per_launch")}
    roof["note"] = (f"{hname} streams the shift matrices (shift read, difference written); bound by "
                    f"{SLOWEST_BOUND[hname]} (fp64.frac against the FP64 pipe, frac against HBM)")
    roof_list = [r_hess_hbm, r_hess_fp64, r_select, r_chol]
    slowest, slowest_ms = max(prof, key=lambda t: t[1])
    # round-level bound: the shift stream (every client's shift read and written once, packed
    # upper FP64) at the measured HBM bandwidth, against the measured time per round
    U = prob.d * (prob.d + 1) // 2
    shift_bytes = 2.0 * prob.n_clients * U * 8
    round_roof = {"bound": "hbm", "shift_stream_bytes": shift_bytes,
                  "lower_bound_ms": shift_bytes / (hbm * 1e9) * 1e3, "round_ms": ms_per_step,
                  "frac": shift_bytes / (hbm * 1e9) * 1e3 / ms_per_step}
    fed.close()

    # time to ||g|| <= 1e-9: a fresh run finds the round count, a second fresh run times exactly
    # those rounds on the device (early rounds cost more than converged ones: TopLEK extracts deeper)
    fed2 = fednl.FedNL(prob, comp, k, 1.0, workers=W)
    g = fed2.run(200)
    hit = np.nonzero(g <= TOL)[0]
    rounds_to_tol = int(hit[0]) + 1 if hit.size else None
    fed2.close()
    tol_ms = None
    if rounds_to_tol:
        fed2 = fednl.FedNL(prob, comp, k, 1.0, workers=W)
        fed2.autotune()
        tol_ms, _ = fed2.time_rounds(rounds_to_tol, L2_FLUSH_BYTES)
        fed2.close()

    # end to end through the C ABI with host buffers: create + upload + init + K rounds (each
    # returning its statistics to the host) + final iterate readback
    n_e2e = min(args.steps, 100)
    t0 = time.perf_counter()
    fed3 = fednl.FedNL(prob, comp, k, 1.0, workers=W)
    for _ in range(n_e2e):
        fed3.round()
    x = fed3.x()
    fed3.close()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": n_e2e / e2e_s, "unit": "rounds/s",
           "h2d_bytes_per_step": upload_bytes(prob) / n_e2e + 0.0,
           "d2h_bytes_per_step": 16 + 8 + prob.d * 8 / n_e2e,
           "rounds": n_e2e, "includes": "create + client-data upload + shift init + rounds + x readback"}

    line = {"metric": METRIC, "value": value, "unit": "rounds/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(prob, comp, k, W),
            "round_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99))},
            "time_to_tol": {"tol": TOL, "rounds": rounds_to_tol,
                            "seconds": tol_ms / 1000.0 if tol_ms is not None else None,
                            "timed": "device time of rounds 1..R from x0 = 0"},
            "roofline": roof, "roofline_kernels": roof_list,
            "slowest_kernel": {"kernel": slowest, "ms": slowest_ms, "bound": SLOWEST_BOUND.get(slowest, "latency")},
            "fp64_pipe": fp64, "round_roofline": round_roof, "kernels_ms": kernels,
            "gpu_launches": args.steps * len(prof),
            "reference_order": reference_order_rounds(fednl, prob, comp, k, W, min(args.steps, 60)),
            "autotuned": tuned,
            "clocks": clocks, "e2e": e2e}
    if ws == 1 and rank == 0:
        line["mixed_precision"] = mixed_headline(fednl, prob, comp, k, args.steps, value,
                                                 tol_ms / 1000.0 if tol_ms is not None else None)
        if not args.no_serving:
            line["serving"] = serving_workload(fednl)
    if ws == 1 and rank == 0 and not args.no_extra:
        line["extra_workloads"] = extra_workloads(fednl, os.cpu_count() or 1, args.steps)
        line["extra_workloads"]["dense FP32 d1024 256x(512-4096) RandK-Philox k=4d, mixed precision"] = \
            mixed_workload(fednl, os.cpu_count() or 1, bf16 / 2.0, src)
    if ws == 1 and rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, n, dt = cpu_port_rounds_per_s(prob, comp, k, threads, 20, 20.0)
        line["cpu_baseline"] = {"value": v, "unit": "rounds/s", "cores": threads, "kind": "port",
                                "sample": f"{n} full rounds of the workload after one warm-up round ({dt:.1f} s)",
                                "time_to_tol": cpu_port_time_to_tol(prob, comp, k, threads),
                                "caveat": "the oracle's C port of the reference round (scalar, fixed operation "
                                          "order, -O3 without -march) stands in for bin_fednl_local, whose "
                                          "sources and x86 SIMD build are not available on this host",
                                "calibration": PORT_CALIBRATION}
    if rank == 0:
        print(json.dumps(line))
    return 0


CASES = ("fp64-w8a", "fp64ref-w8a", "mixed-w8a", "mixed-dense1024")


def run_case(case: str, rounds: int) -> int:
    """A short fixed run of the round for profiling captures (no timing, no JSON line):
    fp64-w8a        the FP64 engine on the w8a-like workload (d=301, 142 clients, TopLEK k=8d)
    fp64ref-w8a     the same in the reference's arithmetic order
    mixed-w8a       the mixed-precision engine on the same workload (solve autotuned)
    mixed-dense1024 the mixed-precision engine, dense N(0,1) features, d=1024, 64 clients x 1024
                    samples (268 MB of features, larger than L2), RandK-Philox k=4d"""
    from ufednl_gb300 import build, datagen, fednl
    build.build()
    fednl.load()
    if case in ("fp64-w8a", "fp64ref-w8a"):
        prob = datagen.workload_w8a_like()
        run = fednl.FedNL(prob, "toplek", 8 * prob.d, 1.0, workers=16,
                          order="reference" if case == "fp64ref-w8a" else "fixed")
    elif case == "mixed-w8a":
        prob = datagen.workload_w8a_like()
        run = fednl.MixedFedNL(prob, 8 * prob.d, 1.0, compressor="toplek")
    else:
        d = 1024
        prob = datagen.dense_problem_fp32(7, d, [1024] * 64, 1e-4)
        k = 4 * d
        run = fednl.MixedFedNL(prob, k, k / (d * (d + 1) // 2))
    if case.startswith("mixed"):
        run.autotune()            # the solve and launch shape a benchmark run would use
    g = run.run(rounds)
    run.close()
    print(case, "||g|| per round:", np.array2string(g, precision=6))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["w8a", "a9a"], default="w8a")
    ap.add_argument("--workers", type=int, default=0, help="reference --workers (TopLEK streams); 0 = host cores")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--no-extra", action="store_true", help="skip the a9a-like and FedNL-PP side measurements")
    ap.add_argument("--case", choices=CASES, default=None,
                    help="run a short fixed case for a profiling capture instead of the benchmark")
    ap.add_argument("--case-rounds", type=int, default=3)
    args = ap.parse_args()
    if args.case:
        return run_case(args.case, args.case_rounds)
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_env()
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    td = dist_init(ws)
    try:
        if args.impl == "reference":
            return run_reference(args, ws, rank, td)
        return run_ours(args, ws, rank, local, td)
    finally:
        if td is not None:
            td.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
