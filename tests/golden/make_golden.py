"""Regenerates the golden fixtures in this folder by running the REFERENCE implementation.

The reference (u-FedNL / dopt) is compiled from its own sources into ``oracle/_ref/ref_harness``
by ``make -C oracle ref`` (needs the reference source tree; this script never runs on the GPU
box).  Each fixture stores seeded inputs and the reference's outputs:

* ``run_<name>.npz``   whole FedNL runs (Option B, clients merged in order): per-round iterate,
  ||g||, l and, for the first rounds, every client's message (indices and values) and Lk;
* ``pp_<name>.npz``    whole FedNL-PP runs (bin_fednl_local_pp, Option B): per-round iterate,
  ||true gradient||, l, sampled clients and, for the first rounds, each sampled client's message,
  Lk and direction;
* ``select_<name>.npz`` TopK / TopLEK index sets on given matrices (ties included);
* ``rand_<name>.npz``   RandK / RandSeqK index draws of one client generator;
* ``chol.npz``          Option-B Cholesky solves.

Usage:  python tests/golden/make_golden.py [--ref-root PATH]
"""
from __future__ import annotations

import argparse
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

sys.path.insert(0, os.path.dirname(HERE))

from ufednl_gb300 import datagen  # noqa: E402
from golden_runs import message_digest, problem_digest  # noqa: E402

COMP = {"identity": 0, "randk": 1, "topk": 2, "randseqk": 3, "toplek": 4, "natural": 5}
HARNESS = os.path.join(REPO, "oracle", "_ref", "ref_harness")
ONLY = None     # --only: fixture kind prefix to regenerate


def _skip(kind):
    return ONLY is not None and not kind.startswith(ONLY)


def run_case(name, prob, comp, k, alpha, workers, rounds, dump_rounds, ext=None, workload=None):
    """ext = dict(option_a, line_search, ls_max, track_f, ls_c, ls_gamma): the extended run
    (Option A / FedNL-LS / tracking), written as runx_<name>.npz with f(x_k) and line-search counts.
    workload = the datagen workload function's name: the fixture stores that name and a digest of
    the generated inputs instead of the inputs, and per-client message digests instead of the
    messages (the workload-sized runs)."""
    if _skip("runx" if ext else "run"):
        return
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([prob.d, prob.n_clients, COMP[comp], k, workers, rounds, dump_rounds],
                     dtype="<i4").tofile(f)
            np.array([prob.lam, alpha], dtype="<f8").tofile(f)
            if ext:
                np.array([ext["option_a"], ext["line_search"], ext["ls_max"], ext["track_f"]], dtype="<i4").tofile(f)
                np.array([ext["ls_c"], ext["ls_gamma"]], dtype="<f8").tofile(f)
            prob.n_samples.astype("<i4").tofile(f)
            prob.features.astype("<f8").tofile(f)
            prob.labels.astype("<f8").tofile(f)
        subprocess.run([HARNESS, "runx" if ext else "run", fin, fout], check=True)
        raw = open(fout, "rb").read()
    pos = 0

    def take(dt, n):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dt, count=n, offset=pos)
        pos += a.nbytes
        return a.copy()

    lda = int(take("<i4", 1)[0])
    d, nc = prob.d, prob.n_clients
    ok, gnorm, lval, xs, fks, lss = [], [], [], [], [], []
    msg_idx, msg_val, lks, msg_cnt = [], [], [], []
    for r in range(rounds):
        ok.append(int(take("<i4", 1)[0]))
        gnorm.append(float(take("<f8", 1)[0]))
        lval.append(float(take("<f8", 1)[0]))
        xs.append(take("<f8", d))
        if ext:
            fks.append(float(take("<f8", 1)[0]))
            lss.append(int(take("<i4", 1)[0]))
        if r < dump_rounds:
            for c in range(nc):
                cnt = int(take("<i4", 1)[0])
                msg_cnt.append(cnt)
                msg_idx.append(take("<u4", cnt))
                msg_val.append(take("<f8", cnt))
                lks.append(float(take("<f8", 1)[0]))
    misround = int(take("<i4", 1)[0])
    assert pos == len(raw)
    extra = {}
    if ext:
        extra = dict(f=np.array(fks), ls_steps=np.array(lss, dtype=np.int32), **{k_: v for k_, v in ext.items()})
    if workload:
        inputs = dict(workload=workload, inputs_sha256=problem_digest(prob), n_samples=prob.n_samples)
        msgs = dict(msg_digest=np.array([message_digest(i, v, lk) for i, v, lk in zip(msg_idx, msg_val, lks)]))
    else:
        inputs = dict(n_samples=prob.n_samples, features=prob.features, labels=prob.labels)
        msgs = dict(msg_idx=np.concatenate(msg_idx).astype(np.uint32), msg_val=np.concatenate(msg_val))
    np.savez_compressed(
        os.path.join(HERE, f"{'runx' if ext else 'run'}_{name}.npz"),
        d=d, lda=lda, lam=prob.lam, compressor=comp, k=k, alpha=alpha, workers=workers, rounds=rounds,
        dump_rounds=dump_rounds, ok=np.array(ok), gnorm=np.array(gnorm), l=np.array(lval),
        x=np.array(xs), msg_count=np.array(msg_cnt, dtype=np.int32), lk=np.array(lks),
        libm_first_misround=misround, **inputs, **msgs, **extra)


def pp_case(name, prob, comp, k, alpha, tau, rounds, dump_rounds, sel_seed=1234):
    if _skip("pp"):
        return
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([prob.d, prob.n_clients, COMP[comp], k, tau, rounds, dump_rounds], dtype="<i4").tofile(f)
            np.array([sel_seed], dtype="<u4").tofile(f)
            np.array([prob.lam, alpha], dtype="<f8").tofile(f)
            prob.n_samples.astype("<i4").tofile(f)
            prob.features.astype("<f8").tofile(f)
            prob.labels.astype("<f8").tofile(f)
        subprocess.run([HARNESS, "pp", fin, fout], check=True)
        raw = open(fout, "rb").read()
    pos = 0

    def take(dt, n):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dt, count=n, offset=pos)
        pos += a.nbytes
        return a.copy()

    lda = int(take("<i4", 1)[0])
    d = prob.d
    ok, gnorm, lval, xs, sels = [], [], [], [], []
    msg_idx, msg_val, lks, msg_cnt, dirs = [], [], [], [], []
    for r in range(rounds):
        ok.append(int(take("<i4", 1)[0]))
        gnorm.append(float(take("<f8", 1)[0]))
        lval.append(float(take("<f8", 1)[0]))
        xs.append(take("<f8", d))
        sels.append(take("<i4", tau))
        if r < dump_rounds:
            for _ in range(tau):
                cnt = int(take("<i4", 1)[0])
                msg_cnt.append(cnt)
                msg_idx.append(take("<u4", cnt))
                msg_val.append(take("<f8", cnt))
                lks.append(float(take("<f8", 1)[0]))
                dirs.append(take("<f8", d))
    assert pos == len(raw)
    np.savez_compressed(
        os.path.join(HERE, f"pp_{name}.npz"),
        d=d, lda=lda, n_samples=prob.n_samples, features=prob.features, labels=prob.labels,
        lam=prob.lam, compressor=comp, k=k, alpha=alpha, tau=tau, sel_seed=sel_seed, rounds=rounds,
        dump_rounds=dump_rounds, ok=np.array(ok), gnorm=np.array(gnorm), l=np.array(lval),
        x=np.array(xs), selected=np.array(sels), msg_count=np.array(msg_cnt, dtype=np.int32),
        msg_idx=np.concatenate(msg_idx).astype(np.uint32), msg_val=np.concatenate(msg_val),
        lk=np.array(lks), dir=np.array(dirs))


LIBSVM_TEXTS = {
    # tabs, CR/LF endings, an empty line, exponents, signs, repeated separators; the first line's
    # smallest index reappears later (the reference's statistics pass resets min/max per entry of
    # line 1)
    "mixed": "+1 1:0.5 3:1 7:2.25e-1\r\n-1 2:1\t4:0.125 7:1\n\n+1 1:1 2:3E2 5:-0.75\n"
             "-1   3:1e-2  6:1.5\r+1 4:0.1234567 7:10.0\n-1 1:2 5:+3.5e+1\n",
    # 0/1 labels and binary features (a9a-style)
    "binary01": "0 1:1 4:1 9:1\n1 2:1 3:1 9:1\n1 1:1 5:1 7:1 8:1\n0 4:1 6:1 9:1\n1 3:1 9:1\n",
}


def libsvm_case(name, text, add_intercept):
    if _skip("libsvm"):
        return
    src = os.path.join(HERE, f"libsvm_{name}.txt")
    with open(src, "w", newline="") as f:
        f.write(text)
    with tempfile.TemporaryDirectory() as td:
        fout = os.path.join(td, "out.bin")
        subprocess.run([HARNESS, "libsvm", src, fout, str(int(add_intercept))], check=True)
        raw = open(fout, "rb").read()
    ok = int(np.frombuffer(raw, "<i4", 1, 0)[0])
    assert ok == 1
    d, n = (int(v) for v in np.frombuffer(raw, "<i4", 2, 4))
    x = np.frombuffer(raw, "<f8", n * d, 12).reshape(n, d).copy()
    y = np.frombuffer(raw, "<f8", n, 12 + 8 * n * d).copy()
    np.savez_compressed(os.path.join(HERE, f"libsvm_{name}_{int(add_intercept)}.npz"), x=x, y=y,
                        add_intercept=int(add_intercept))


def select_case(name, mats, d, k, lek):
    if _skip("select"):
        return
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([d, k, len(mats)], dtype="<i4").tofile(f)
            for m in mats:
                m.astype("<f8").T.copy().tofile(f)          # column-major d x d
        subprocess.run([HARNESS, "toplek" if lek else "topk", fin, fout], check=True)
        raw = open(fout, "rb").read()
    lda = int(np.frombuffer(raw, "<i4", 1, 0)[0])
    pos = 4
    counts, idx = [], []
    for _ in mats:
        cnt = int(np.frombuffer(raw, "<i4", 1, pos)[0])
        pos += 4
        idx.append(np.frombuffer(raw, "<u4", cnt, pos).copy())
        pos += 4 * cnt
        counts.append(cnt)
    np.savez_compressed(os.path.join(HERE, f"select_{name}.npz"), d=d, lda=lda, k=k,
                        toplek=int(lek), mats=np.array(mats), counts=np.array(counts, dtype=np.int32),
                        idx=np.concatenate(idx).astype(np.uint32))


def rand_case(name, d, k, seed, draws, seq):
    if _skip("rand"):
        return
    with tempfile.TemporaryDirectory() as td:
        fout = os.path.join(td, "out.bin")
        subprocess.run([HARNESS, "randseqk" if seq else "randk", fout, str(d), str(k), str(seed),
                        str(draws)], check=True)
        raw = open(fout, "rb").read()
    lda = int(np.frombuffer(raw, "<i4", 1, 0)[0])
    idx = np.frombuffer(raw, "<u4", draws * k, 4).reshape(draws, k).copy()
    np.savez_compressed(os.path.join(HERE, f"rand_{name}.npz"), d=d, lda=lda, k=k, seed=seed,
                        draws=draws, seq=int(seq), idx=idx)


def chol_cases(rng):
    if _skip("chol"):
        return
    outs = []
    with tempfile.TemporaryDirectory() as td:
        for d, l in ((9, 0.1), (33, 1e-3), (70, 0.0)):
            a = rng.standard_normal((d, d + 4))
            h = a @ a.T / d
            b = rng.standard_normal(d)
            fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
            with open(fin, "wb") as f:
                np.array([d], dtype="<i4").tofile(f)
                np.array([l], dtype="<f8").tofile(f)
                h.astype("<f8").T.copy().tofile(f)
                b.astype("<f8").tofile(f)
            subprocess.run([HARNESS, "chol", fin, fout], check=True)
            raw = open(fout, "rb").read()
            ok = int(np.frombuffer(raw, "<i4", 1, 0)[0])
            x = np.frombuffer(raw, "<f8", d, 4).copy()
            outs.append((d, l, h, b, ok, x))
    np.savez_compressed(os.path.join(HERE, "chol.npz"),
                        **{f"h{i}": o[2] for i, o in enumerate(outs)},
                        **{f"b{i}": o[3] for i, o in enumerate(outs)},
                        **{f"x{i}": o[5] for i, o in enumerate(outs)},
                        l=np.array([o[1] for o in outs]), ok=np.array([o[4] for o in outs]),
                        n=len(outs))


def tie_matrices(rng, d, count, levels):
    mats = []
    for t in range(count):
        m = rng.integers(-levels, levels + 1, size=(d, d)).astype(np.float64) * 0.25
        m = np.triu(m) + np.triu(m, 1).T
        mats.append(m)
    return mats


def wire_case(name, rng):
    """The distributed client's packet framing (UsedTypes.h:1022-1125) through the reference's
    own dopt::MutableData: signal byte, LEB128 length, payload."""
    if _skip("wire"):
        return
    sizes = [0, 1, 8, 127, 128, 129, 2408 * 8, 16383, 16384, 300000, 2097152]
    sigs = [41 + (t % 9) for t in range(len(sizes))]
    payloads = [rng.integers(0, 256, n, dtype=np.uint8) if n <= 20000 else np.zeros(n, dtype=np.uint8) for n in sizes]
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<i", len(sizes)))
            for sg, pl in zip(sigs, payloads):
                f.write(struct.pack("<ii", sg, len(pl)))
                f.write(pl.tobytes())
        subprocess.run([HARNESS, "wire", fin, fout], check=True)
        framed = np.frombuffer(open(fout, "rb").read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, f"wire_{name}.npz"), sigs=np.array(sigs, dtype=np.int32),
                        sizes=np.array(sizes, dtype=np.int64), payload=np.concatenate(payloads), framed=framed)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=os.environ.get("REF_ROOT"),
                    help="the reference's dopt source folder (or set REF_ROOT)")
    ap.add_argument("--only", default=None, help="regenerate only fixtures whose kind starts with this (run, pp, ...)")
    args = ap.parse_args()
    if not args.ref_root:
        ap.error("the reference source folder is needed: --ref-root PATH or REF_ROOT=PATH")
    global ONLY
    ONLY = args.only
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", f"REF_ROOT={args.ref_root}"],
                   check=True)
    rng = np.random.default_rng(20241203)
    wire_case("frames", np.random.default_rng(7))

    # whole runs: uneven clients, LDA padding (d=13 -> LDA 16), every compressor
    small = datagen.binary_problem(11, 13, [20, 31, 17, 25, 40], 0.3, 1e-3)
    U = 13 * 14 // 2
    run_case("topk_d13", small, "topk", 26, 1.0, 2, 30, 4)
    run_case("toplek_d13", small, "toplek", 39, 1.0, 2, 30, 4)
    run_case("randk_d13", small, "randk", 26, 26 / U, 2, 12, 4)
    run_case("randseqk_d13", small, "randseqk", 13, 13 / U, 2, 12, 4)
    run_case("natural_d13", small, "natural", U, 1.0 / (1.0 + 1.0 / 8.0), 2, 12, 4)
    run_case("identity_d13", small, "identity", U, 1.0, 2, 12, 4)
    mid = datagen.binary_problem(12, 40, [60, 45, 80, 52, 71, 66, 49], 0.12, 1e-3)
    run_case("topk_d40", mid, "topk", 320, 1.0, 3, 40, 3)
    run_case("toplek_d40", mid, "toplek", 320, 1.0, 3, 60, 3)
    dense = datagen.dense_problem(13, 10, [30, 22, 41], 1e-2)
    run_case("topk_dense_d10", dense, "topk", 20, 1.0, 1, 8, 3)

    # the benchmark workloads at full size: a9a-like (d=124, 80 x 407, TopK k=8d) and w8a-like
    # (d=301, 142 clients n_i 200-600, TopLEK k=8d, 16 reference workers)
    run_case("topk_a9a_d124", datagen.workload_a9a_like(), "topk", 8 * 124, 1.0, 8, 12, 12,
             workload="workload_a9a_like")
    run_case("toplek_w8a_d301", datagen.workload_w8a_like(), "toplek", 8 * 301, 1.0, 16, 8, 8,
             workload="workload_w8a_like")

    # the reference's LIBSVM loader on tricky text
    for nm, txt in LIBSVM_TEXTS.items():
        libsvm_case(nm, txt, False)
        libsvm_case(nm, txt, True)

    # Option A, FedNL-LS and tracked objective values
    ls = dict(option_a=0, line_search=1, ls_max=5, track_f=1, ls_c=0.5, ls_gamma=0.5)
    run_case("ls_randk_d13", small, "randk", 26, 26 / U, 2, 12, 2, ext=ls)
    run_case("ls_natural_d13", small, "natural", U, 1.0 / (1.0 + 1.0 / 8.0), 2, 10, 2,
             ext=dict(ls, ls_c=0.25, ls_gamma=0.7, ls_max=3))
    run_case("ls_topk_d40", mid, "topk", 320, 1.0, 3, 40, 2, ext=ls)
    run_case("opta_randseqk_d13", small, "randseqk", 13, 13 / U, 2, 12, 2,
             ext=dict(option_a=1, line_search=0, ls_max=5, track_f=1, ls_c=0.5, ls_gamma=0.5))
    run_case("track_toplek_d13", small, "toplek", 39, 1.0, 2, 10, 2,
             ext=dict(option_a=0, line_search=0, ls_max=5, track_f=1, ls_c=0.5, ls_gamma=0.5))

    # FedNL-PP runs: uneven-free small federation (the reference's PP binary splits evenly), every
    # compressor; a phishing-shaped case (d = 69, n_i = 6)
    ppsmall = datagen.binary_problem(21, 13, [8] * 24, 0.45, 1e-3)
    pp_case("randseqk_d13", ppsmall, "randseqk", 13, 13 / U, 6, 20, 3)
    pp_case("randk_d13", ppsmall, "randk", 26, 26 / U, 6, 12, 2)
    pp_case("natural_d13", ppsmall, "natural", U, 1.0 / (1.0 + 1.0 / 8.0), 6, 12, 2)
    pp_case("identity_d13", ppsmall, "identity", U, 1.0, 6, 8, 2)
    pp_case("topk_d13", ppsmall, "topk", 26, 1.0, 6, 10, 2)
    pp_case("toplek_d13", ppsmall, "toplek", 39, 1.0, 6, 10, 2)
    ppphish = datagen.binary_problem(3, 69, [6] * 64, 0.45, 1e-3)
    pp_case("randseqk_d69", ppphish, "randseqk", 69, 69 / (69 * 70 // 2), 8, 10, 2)
    pp_case("natural_d69", ppphish, "natural", 69 * 70 // 2, 1.0 / (1.0 + 1.0 / 8.0), 8, 6, 1)

    # selections on tie-heavy and continuous matrices (one OS thread => one TopLEK stream)
    ties = tie_matrices(rng, 12, 12, 3)
    select_case("topk_ties_d12", ties, 12, 10, False)
    select_case("toplek_ties_d12", ties, 12, 10, True)
    cont = [np.triu(m) + np.triu(m, 1).T for m in rng.standard_normal((8, 30, 30))]
    select_case("topk_cont_d30", cont, 30, 60, False)
    select_case("toplek_cont_d30", cont, 30, 60, True)
    few = tie_matrices(rng, 9, 10, 1)                 # values in {-0.25, 0, 0.25}: huge tie classes
    select_case("topk_few_d9", few, 9, 7, False)
    select_case("toplek_few_d9", few, 9, 7, True)

    rand_case("randk_d20", 20, 40, 123, 6, False)
    rand_case("randk_d301", 301, 2408, 124, 3, False)
    rand_case("randseqk_d20", 20, 40, 125, 6, True)
    rand_case("randseqk_d69", 69, 69, 126, 8, True)
    chol_cases(rng)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
