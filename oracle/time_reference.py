"""Times the reference's round against the oracle's C port on the same host cores.

TEST / MEASUREMENT INFRASTRUCTURE: needs the reference sources (REF_ROOT) and runs only where they
are, never on the GPU host.  The reference side is oracle/ref_harness.cpp, which drives the
reference's own operators (margins, sigmoid, gradient, Hessian, compressors, Cholesky, solves) with
one persistent thread per reference worker and the master merging clients in order, compiled twice:
with the reference's Release options (-O3 -march=native: oracle/_ref/ref_harness_native) and with
the portable no-FMA options the golden fixtures use (oracle/_ref/ref_harness).  The port is
oracle/fednl_oracle.c (the CPU baseline bench.py times on the GPU host), in both arithmetic orders.
bin_fednl_local itself is not built: its main program needs a header that the reference's CMake
configure step generates.

    REF_ROOT=<dopt folder> python oracle/time_reference.py [--rounds R] [--threads T]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)

COMP = {"topk": 2, "toplek": 4}


def harness_rounds_per_s(binary, prob, comp, k, workers, rounds):
    """Mean rounds/s of the harness over rounds 1..R-1 (round 0 excluded: first touch of the data)."""
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([prob.d, prob.n_clients, COMP[comp], k, workers, rounds, 0], dtype="<i4").tofile(f)
            np.array([prob.lam, 1.0], dtype="<f8").tofile(f)
            prob.n_samples.astype("<i4").tofile(f)
            prob.features.astype("<f8").tofile(f)
            prob.labels.astype("<f8").tofile(f)
        subprocess.run([binary, "time", fin, fout], check=True)
        raw = open(fout, "rb").read()
    ends = np.frombuffer(raw[-8 * rounds:], dtype="<f8")
    return (rounds - 1) / (ends[-1] - ends[0])


def port_rounds_per_s(prob, comp, k, workers, threads, rounds, ref_order):
    from oracle import pyoracle
    orc = pyoracle.FedNL(prob, comp, k, 1.0, workers=workers, threads=threads, ref_order=ref_order)
    orc.round()
    t0 = time.perf_counter()
    for _ in range(rounds - 1):
        orc.round()
    dt = time.perf_counter() - t0
    orc.close()
    return (rounds - 1) / dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rounds", type=int, default=16)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    ref = os.environ.get("REF_ROOT")
    if not ref:
        ap.error("set REF_ROOT to the reference's dopt source folder")
    subprocess.run(["make", "-s", "-C", HERE, "ref", "refnative", f"REF_ROOT={ref}"], check=True)
    from oracle import pyoracle
    from ufednl_gb300 import datagen
    pyoracle.build()
    T = a.threads
    out = {"threads": T, "rounds": a.rounds, "cpu": subprocess.run(["sh", "-c", "lscpu | grep 'Model name'"],
                                                                  capture_output=True, text=True).stdout.strip()}
    for name, prob, comp, k in (("w8a-like d301 142 clients TopLEK k=8d", datagen.workload_w8a_like(), "toplek", 8 * 301),
                                ("a9a-like d124 80x407 TopK k=8d", datagen.workload_a9a_like(), "topk", 8 * 124)):
        row = {
            "reference_operators_native": harness_rounds_per_s(os.path.join(HERE, "_ref", "ref_harness_native"),
                                                               prob, comp, k, T, a.rounds),
            "reference_operators_nofma": harness_rounds_per_s(os.path.join(HERE, "_ref", "ref_harness"),
                                                              prob, comp, k, T, a.rounds),
            "port_fixed_order": port_rounds_per_s(prob, comp, k, T, T, a.rounds, False),
            "port_reference_order": port_rounds_per_s(prob, comp, k, T, T, a.rounds, True),
        }
        row["port_over_reference_native"] = row["port_fixed_order"] / row["reference_operators_native"]
        out[name] = row
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
