"""Small fixed runs of the round, for profiling captures that need a short deterministic command:

    python -m ufednl_gb300.cases <case> [--rounds R]

fp64-w8a        the FP64 engine on the w8a-like workload (d=301, 142 clients, TopLEK k=8d)
mixed-w8a       the mixed-precision engine on the same workload (solve autotuned)
mixed-dense1024 the mixed-precision engine, dense N(0,1) features, d=1024, 64 clients x 1024
                samples (268 MB of features, larger than L2), RandK-Philox k=4d
"""
from __future__ import annotations

import argparse

import numpy as np

from . import build, datagen, fednl


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["fp64-w8a", "mixed-w8a", "mixed-dense1024"])
    ap.add_argument("--rounds", type=int, default=3)
    a = ap.parse_args(argv)
    build.build()
    fednl.load()
    if a.case == "fp64-w8a":
        prob = datagen.workload_w8a_like()
        run = fednl.FedNL(prob, "toplek", 8 * prob.d, 1.0, workers=16)
    elif a.case == "mixed-w8a":
        prob = datagen.workload_w8a_like()
        run = fednl.MixedFedNL(prob, 8 * prob.d, 1.0, compressor="toplek")
    else:
        d = 1024
        prob = datagen.dense_problem_fp32(7, d, [1024] * 64, 1e-4)
        k = 4 * d
        run = fednl.MixedFedNL(prob, k, k / (d * (d + 1) // 2))
    if a.case != "fp64-w8a":
        run.autotune()            # the solve and launch shape a benchmark run would use
    g = run.run(a.rounds)
    run.close()
    print(a.case, "||g| per round:", np.array2string(g, precision=6))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
