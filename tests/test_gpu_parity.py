"""Parity of the GB300 kernels (through the C ABI) with the reference's own outputs (golden
fixtures) and with the CPU oracle on the same seeded inputs.

Bars: compressor index sets and RandK/RandSeqK draws bit-exact; shift updates and messages
bit-exact given identical input matrices; FP64 iterates within 1e-10 relative (the sigmoid's exp
differs between CUDA and glibc by at most an ulp, which is the only source of difference)."""
import glob
import os

import numpy as np
import pytest

import golden_runs
from conftest import golden_path
from ufednl_gb300 import datagen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from ufednl_gb300 import build, fednl
    build.build()
    fednl.load()
    return fednl


def _full(m, d, lda):
    full = np.zeros((d, lda))
    full[:, :d] = m.T
    return full.reshape(-1)


def _problem(z):
    return golden_runs.problem_of(z)


# ---- compressors against the reference's golden vectors -----------------------------------

@pytest.mark.parametrize("path", sorted(glob.glob(golden_path("select_*.npz"))), ids=os.path.basename)
def test_selection_golden(gpu, path):
    z = np.load(path)
    d, lda, k = int(z["d"]), int(z["lda"]), int(z["k"])
    mats = np.stack([_full(m, d, lda) for m in z["mats"]])
    pos = 0
    if int(z["toplek"]):
        ws = np.array([1234], dtype=np.uint32)         # one reference thread => one stream
        got = gpu.get_toplek_from_upper_diagonal_part(mats, d, lda, k, ws)
        for t, g in enumerate(got):
            cnt = int(z["counts"][t])
            np.testing.assert_array_equal(g, z["idx"][pos:pos + cnt])
            pos += cnt
    else:
        got = gpu.get_topk_from_upper_diagonal_part(mats, d, lda, k)
        for t in range(len(mats)):
            np.testing.assert_array_equal(got[t], z["idx"][pos:pos + k])
            pos += k


@pytest.mark.parametrize("path", sorted(glob.glob(golden_path("rand_*.npz"))), ids=os.path.basename)
def test_random_draws_golden(gpu, path):
    z = np.load(path)
    d, lda, k = int(z["d"]), int(z["lda"]), int(z["k"])
    st = np.array([int(z["seed"])], dtype=np.uint32)
    for t in range(int(z["draws"])):
        if int(z["seq"]):
            got = gpu.generate_randseqk_items_in_upper_triangular_part(st, d, lda, k)
        else:
            got = gpu.generate_randk_items_in_upper_triangular_part(st, d, lda, k)
        np.testing.assert_array_equal(got[0], z["idx"][t])


def test_cholesky_golden(gpu):
    z = np.load(golden_path("chol.npz"))
    for i in range(int(z["n"])):
        h = z[f"h{i}"]
        d = h.shape[0]
        dx = gpu.cholesky_option_b_solve(_full(h, d, d), d, d, float(z["l"][i]), z[f"b{i}"])
        ref = z[f"x{i}"]
        np.testing.assert_allclose(dx, ref, rtol=1e-10, atol=1e-10 * np.max(np.abs(ref)))


def test_cholesky_known_answer_and_not_pd(gpu):
    """CholeskyFactorizationGTest.cpp:11-40: L L^T with L = [[1,0,0],[4,7,0],[1,2,5]] is solved
    exactly; [[1,2],[2,1]] is rejected as not positive definite."""
    L = np.array([[1.0, 0, 0], [4, 7, 0], [1, 2, 5]])
    A = L @ L.T
    b = np.array([1.0, 2.0, 3.0])
    dx = gpu.cholesky_option_b_solve(A.T.copy().ravel(), 3, 3, 0.0, b)
    np.testing.assert_allclose(A @ dx, b, rtol=1e-14)
    with pytest.raises(gpu.FedNLError) as e:
        gpu.cholesky_option_b_solve(np.array([[1.0, 2.0], [2.0, 1.0]]).ravel(), 2, 2, 0.0, np.ones(2))
    assert e.value.code == -4


# ---- compressors against the oracle on larger, tie-heavy and continuous inputs -------------

@pytest.mark.parametrize("d,k,kind", [(124, 992, "ties"), (301, 2408, "cont"), (301, 2408, "ties"),
                                      (69, 69, "zeros"), (40, 1, "cont"), (40, 819, "cont"), (40, 820, "ties"),
                                      (33, 560, "few")])
def test_topk_toplek_vs_oracle(gpu, oracle, d, k, kind):
    rng = np.random.default_rng(d * 1000 + k)
    lda = (d + 3) // 4 * 4
    mats = []
    for t in range(6):
        if kind == "ties":
            m = rng.integers(-4, 5, size=(d, d)) * 0.125
        elif kind == "few":
            m = rng.integers(-1, 2, size=(d, d)) * 1.0
        elif kind == "zeros":
            m = rng.standard_normal((d, d)) * (rng.random((d, d)) < 0.02)
        else:
            m = rng.standard_normal((d, d))
        m = np.triu(m) + np.triu(m, 1).T
        mats.append(_full(m, d, lda))
    mats = np.stack(mats)
    got = gpu.get_topk_from_upper_diagonal_part(mats, d, lda, k)
    for t in range(len(mats)):
        np.testing.assert_array_equal(got[t], oracle.topk(mats[t], d, lda, k))
    # TopLEK with two worker streams, matrices alternating between them
    ws = np.array([1234, 1234], dtype=np.uint32)
    wo = np.arange(len(mats)) % 2
    got = gpu.get_toplek_from_upper_diagonal_part(mats, d, lda, k, ws, wo)
    st = [np.array([1234], dtype=np.uint32), np.array([1234], dtype=np.uint32)]
    for t in range(len(mats)):
        np.testing.assert_array_equal(got[t], oracle.toplek(mats[t], d, lda, k, st[t % 2]))
    assert ws[0] == st[0][0] and ws[1] == st[1][0]


@pytest.mark.parametrize("d,k", [(301, 2408), (124, 992), (1024, 4096), (13, 91)])
@pytest.mark.parametrize("seq", [False, True])
def test_randk_randseqk_vs_oracle(gpu, oracle, d, k, seq):
    lda = (d + 3) // 4 * 4
    g_states = np.array([123 + c for c in range(5)], dtype=np.uint32)
    o_states = [np.array([123 + c], dtype=np.uint32) for c in range(5)]
    for _ in range(3):
        if seq:
            got = gpu.generate_randseqk_items_in_upper_triangular_part(g_states, d, lda, k)
        else:
            got = gpu.generate_randk_items_in_upper_triangular_part(g_states, d, lda, k)
        for c in range(5):
            ref = oracle.randseqk(o_states[c], d, lda, k) if seq else oracle.randk(o_states[c], d, lda, k)
            np.testing.assert_array_equal(got[c], ref)
            assert g_states[c] == o_states[c][0]


def test_natural_vs_oracle(gpu, oracle):
    rng = np.random.default_rng(7)
    v = np.concatenate([rng.standard_normal(1001) * 10.0 ** rng.integers(-300, 300, 1001),
                        [0.0, -0.0, 5e-324, -1e-310, np.inf, -np.inf]])
    out, packed = gpu.apply_natural_compressor(v, with_packed=True)
    L = oracle.lib()
    ref = np.array([L.orc_natural(float(x)) for x in v])
    np.testing.assert_array_equal(out.view(np.uint64), ref.view(np.uint64))
    n = v.size
    words = packed.reshape(-1, 3).astype(np.uint32)
    words = words[:, 0] | (words[:, 1] << 8) | (words[:, 2] << 16)
    for q in range(n // 2):
        assert words[q] == L.orc_pack2_natural(float(v[2 * q]), float(v[2 * q + 1]))
    # trailing block: (last, second-to-last) for an odd count
    assert n % 2 == 1 and words[n // 2] == L.orc_pack2_natural(float(v[n - 1]), float(v[n - 2]))


# ---- logistic oracle ------------------------------------------------------------------------

@pytest.mark.parametrize("kind", ["binary", "dense"])
def test_logreg_oracle_vs_cpu(gpu, oracle, kind):
    d, n, lam = 37, 53, 1e-3
    p = (datagen.binary_problem(3, d, [n], 0.2, lam) if kind == "binary" else datagen.dense_problem(3, d, [n], lam))
    x = np.random.default_rng(1).standard_normal(d) * 0.3
    g, h = gpu.evaluate_gradient_and_hessian(p.features, p.labels, lam, x)
    lda = (d + 3) // 4 * 4
    import ctypes as C
    L = oracle.lib()
    dp = C.POINTER(C.c_double)
    atr = np.zeros((n, lda))
    atr[:, :d] = p.features * p.labels[:, None]
    atr = np.ascontiguousarray(atr.ravel())
    m = np.empty(n)
    sig = np.empty(n)
    L.orc_margin(atr.ctypes.data_as(dp), d, lda, n, x.ctypes.data_as(dp), m.ctypes.data_as(dp))
    L.orc_sigmoid(m.ctypes.data_as(dp), n, sig.ctypes.data_as(dp))
    gr = np.empty(d)
    hr = np.empty(d * lda)
    L.orc_gradient(atr.ctypes.data_as(dp), d, lda, n, x.ctypes.data_as(dp), sig.ctypes.data_as(dp), lam,
                   gr.ctypes.data_as(dp))
    L.orc_hessian(atr.ctypes.data_as(dp), d, lda, n, sig.ctypes.data_as(dp), lam, hr.ctypes.data_as(dp))
    np.testing.assert_allclose(g, gr, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(h, hr, rtol=1e-13, atol=1e-15)


# ---- whole runs -------------------------------------------------------------------------------

ALL_RUNS = sorted(glob.glob(golden_path("run_*.npz")) + glob.glob(golden_path("runx_*.npz")))


@pytest.mark.parametrize("path", [p for p in ALL_RUNS if "_a9a_" not in p and "_w8a_" not in p], ids=os.path.basename)
def test_run_golden(gpu, path):
    """Whole runs in the engine's fixed order against the reference's golden runs, same contract as
    the CPU oracle's (Option A, FedNL-LS and tracked objective values included)."""
    from test_oracle_golden import check_run_against_reference
    z = np.load(path)
    prob = _problem(z)
    fed = gpu.FedNL(prob, str(z["compressor"]), int(z["k"]), float(z["alpha"]), lda=int(z["lda"]),
                    workers=int(z["workers"]), **golden_runs.run_kwargs(z))
    check_run_against_reference(fed, z, prob)
    fed.close()


@pytest.mark.parametrize("path", ALL_RUNS, ids=os.path.basename)
def test_run_golden_reference_order(gpu, path):
    """Whole runs in the reference's arithmetic order reproduce the reference's golden runs bit for
    bit (iterates, ||g||, l, every client's message and Lk) up to the first round whose sigmoid
    glibc's exp misrounded, and within 1e-10 after it; the a9a-like (d=124, 80 x 407, TopK) and
    w8a-like (d=301, 142 clients, TopLEK with 16 reference workers) workloads at full size."""
    z = np.load(path)
    prob = _problem(z)
    fed = gpu.FedNL(prob, str(z["compressor"]), int(z["k"]), float(z["alpha"]), lda=int(z["lda"]),
                    workers=int(z["workers"]), order="reference", **golden_runs.run_kwargs(z))
    exact = golden_runs.check_run_bitexact(fed, z, prob.n_clients)
    fed.close()
    assert exact >= 1


def _compare_runs(gpu, oracle, prob, comp, k, alpha, rounds, workers, threads=None, order="fixed", **opts):
    """GPU and CPU oracle perform the same IEEE operations in the same order: every round's
    iterate, aggregated gradient, l and every client's message must agree bit for bit (and f(x_k)
    and the line-search evaluation count when those options are on).  order: the engine's fixed
    order or the reference's."""
    threads = threads or min(workers, os.cpu_count() or 1)
    orc = oracle.FedNL(prob, comp, k, alpha, workers=workers, threads=threads, ref_order=order == "reference",
                       **opts)
    fed = gpu.FedNL(prob, comp, k, alpha, workers=workers, order=order, **opts)
    for r in range(rounds):
        go = orc.round()
        gg = fed.round()
        np.testing.assert_array_equal(fed.x(), orc.x(), err_msg=f"round {r}: iterate")
        np.testing.assert_array_equal(fed.grad(), orc.grad(), err_msg=f"round {r}: gradient")
        assert fed.l() == orc.l(), f"round {r}: l"
        if opts.get("line_search") or opts.get("track_f"):
            assert fed.f() == orc.f(), f"round {r}: f(x_k)"
            assert fed.ls_steps() == orc.ls_steps(), f"round {r}: line-search evaluations"
        assert abs(gg - go) <= 1e-14 * go + 1e-300
        for c in range(0, prob.n_clients, max(1, prob.n_clients // 7)):
            io, vo = orc.message(c)
            ig, vg = fed.message(c)
            np.testing.assert_array_equal(ig, io, err_msg=f"round {r} client {c}: indices")
            np.testing.assert_array_equal(vg, vo, err_msg=f"round {r} client {c}: values")
            assert fed.lk(c) == orc.lk(c)
    np.testing.assert_array_equal(fed.shift(0), orc.shift(0))
    fed.close()
    orc.close()


@pytest.mark.parametrize("comp", ["topk", "toplek", "randk", "randseqk", "natural", "identity", "randk_philox"])
def test_run_vs_oracle_small(gpu, oracle, comp):
    prob = datagen.binary_problem(21, 30, [37, 52, 29, 61, 44, 33], 0.15, 1e-3)
    U = 30 * 31 // 2
    k = {"topk": 120, "toplek": 150, "randk": 60, "randseqk": 30, "natural": U, "identity": U,
         "randk_philox": 60}[comp]
    alpha = {"randk": k / U, "randseqk": k / U, "natural": 8 / 9, "randk_philox": k / U}.get(comp, 1.0)
    _compare_runs(gpu, oracle, prob, comp, k, alpha, 8, workers=4)


@pytest.mark.parametrize("opts", [dict(line_search=(0.5, 0.5, 5), track_f=True),
                                  dict(line_search=(0.3, 0.6, 3)),
                                  dict(option_a=True, track_f=True)], ids=["ls", "ls-short", "option-a"])
@pytest.mark.parametrize("comp", ["topk", "randk", "natural"])
def test_run_options_vs_oracle(gpu, oracle, comp, opts):
    """FedNL-LS (trial points, objective, Armijo test on the device), Option A and tracked
    objective values, bit for bit against the oracle."""
    prob = datagen.binary_problem(23, 30, [37, 52, 29, 61, 44, 33], 0.15, 1e-3)
    U = 30 * 31 // 2
    k = {"topk": 120, "randk": 60, "natural": U}[comp]
    alpha = {"randk": k / U, "natural": 8 / 9}.get(comp, 1.0)
    _compare_runs(gpu, oracle, prob, comp, k, alpha, 12, workers=4, **opts)


def test_run_options_vs_oracle_dense_and_w8a(gpu, oracle):
    prob = datagen.dense_problem(24, 18, [31, 27, 40], 1e-2)
    _compare_runs(gpu, oracle, prob, "topk", 36, 1.0, 6, workers=2, line_search=(0.5, 0.5, 5), track_f=True)
    prob = datagen.workload_w8a_like()
    _compare_runs(gpu, oracle, prob, "toplek", 8 * 301, 1.0, 3, workers=8, threads=os.cpu_count(),
                  line_search=(0.5, 0.5, 5))


def test_run_vs_oracle_dense(gpu, oracle):
    prob = datagen.dense_problem(22, 18, [31, 27, 40], 1e-2)
    _compare_runs(gpu, oracle, prob, "topk", 36, 1.0, 6, workers=2)


def test_run_vs_oracle_a9a_like_full_size(gpu, oracle):
    """The a9a-like workload at its full size (d=124, 80 x 407, TopK k=8d, alpha=1)."""
    prob = datagen.workload_a9a_like()
    _compare_runs(gpu, oracle, prob, "topk", 8 * 124, 1.0, 4, workers=8, threads=os.cpu_count())


def test_run_vs_oracle_w8a_like_full_size(gpu, oracle):
    """The w8a-like workload at its full size (d=301, 142 clients, n_i 200-600, TopLEK k=8d)."""
    prob = datagen.workload_w8a_like()
    _compare_runs(gpu, oracle, prob, "toplek", 8 * 301, 1.0, 3, workers=8, threads=os.cpu_count())


@pytest.mark.parametrize("comp", ["topk", "toplek", "randk", "randseqk", "natural", "identity"])
def test_run_vs_oracle_reference_order(gpu, oracle, comp):
    """The reference-order kernels against the oracle's reference-order restatement, bit for bit,
    on uneven clients with tail samples (n_i not multiples of 8) and d not a multiple of 8."""
    prob = datagen.binary_problem(25, 30, [37, 52, 29, 61, 44, 33], 0.15, 1e-3)
    U = 30 * 31 // 2
    k = {"topk": 120, "toplek": 150, "randk": 60, "randseqk": 30, "natural": U, "identity": U}[comp]
    alpha = {"randk": k / U, "randseqk": k / U, "natural": 8 / 9}.get(comp, 1.0)
    _compare_runs(gpu, oracle, prob, comp, k, alpha, 8, workers=4, order="reference")


def test_run_options_vs_oracle_reference_order(gpu, oracle):
    """FedNL-LS, tracked objective values and Option A in the reference's order; dense features;
    the w8a-like workload at full size."""
    prob = datagen.binary_problem(26, 30, [37, 52, 29, 61, 44, 33], 0.15, 1e-3)
    _compare_runs(gpu, oracle, prob, "topk", 120, 1.0, 10, workers=4, order="reference",
                  line_search=(0.5, 0.5, 5), track_f=True)
    _compare_runs(gpu, oracle, prob, "randk", 60, 60 / 465, 6, workers=4, order="reference", option_a=True)
    dense = datagen.dense_problem(27, 19, [31, 27, 40], 1e-2)
    _compare_runs(gpu, oracle, dense, "topk", 38, 1.0, 6, workers=2, order="reference")
    w8a = datagen.workload_w8a_like()
    _compare_runs(gpu, oracle, w8a, "toplek", 8 * 301, 1.0, 3, workers=16, threads=os.cpu_count(),
                  order="reference")


def test_run_is_deterministic(gpu):
    prob = datagen.binary_problem(23, 40, [50, 61, 47, 55], 0.2, 1e-3)
    xs = []
    for _ in range(2):
        fed = gpu.FedNL(prob, "toplek", 300, 1.0, workers=3)
        g = fed.run(6)
        xs.append((fed.x(), g))
        fed.close()
    assert xs[0][0].tobytes() == xs[1][0].tobytes()
    assert xs[0][1].tobytes() == xs[1][1].tobytes()


def test_run_converges_to_tolerance(gpu):
    """FedNL with TopK on the a9a-like workload reaches ||grad|| <= 1e-9."""
    prob = datagen.workload_a9a_like()
    fed = gpu.FedNL(prob, "topk", 8 * 124, 1.0, workers=8)
    g = fed.run(60)
    assert np.min(g) <= 1e-9, g[-5:]
    fed.close()


def test_edge_cases(gpu, oracle):
    # single-sample clients, k >= U for TopK/TopLEK, d = 1
    prob = datagen.binary_problem(24, 6, [1, 3, 1], 0.5, 1e-2)
    U = 21
    for comp, k in (("topk", U), ("toplek", U + 5), ("topk", 1), ("toplek", 1)):
        _compare_runs(gpu, oracle, prob, comp, k, 1.0, 3, workers=2)
    one = datagen.Problem(1, np.array([4, 2], dtype=np.int32), np.ones((6, 1)),
                          np.array([1.0, -1, 1, 1, -1, 1]), 1e-2)
    _compare_runs(gpu, oracle, one, "topk", 1, 1.0, 3, workers=1)
    for order in ("reference",):
        for comp, k in (("topk", U), ("toplek", U + 5), ("topk", 1), ("toplek", 1)):
            _compare_runs(gpu, oracle, prob, comp, k, 1.0, 3, workers=2, order=order)
        _compare_runs(gpu, oracle, one, "topk", 1, 1.0, 3, workers=1, order=order)


# ---- the remaining operator entries of the reference's worker and master ----------------------

def _sym_full(rng, n, d, lda):
    out = np.zeros((n, d, lda))
    for m in range(n):
        a = rng.standard_normal((d, d))
        out[m, :, :d] = np.triu(a) + np.triu(a, 1).T
    return out.reshape(n, -1)


@pytest.mark.parametrize("comp", ["topk", "randk"])
def test_shift_update_operator(gpu, oracle, comp):
    """fednl_gpu_shift_update against the worker's update written out in numpy
    (LocalWorkerForFedNL_TopK.h:103-129 / RandK.h:136-162), bit for bit, on TopK and RandK selections."""
    rng = np.random.default_rng(31)
    d, lda, n = 37, 40, 5
    U = d * (d + 1) // 2
    k = 3 * d
    diffs = _sym_full(rng, n, d, lda)
    shifts = _sym_full(rng, n, d, lda)
    if comp == "topk":
        idx = np.stack([oracle.topk(diffs[m], d, lda, k) for m in range(n)])
        mult = 1.0
    else:
        st = np.array([123], dtype=np.uint32)
        idx = np.stack([oracle.randk(st, d, lda, k) for _ in range(n)])
        mult = U / k
    counts = np.full(n, k, dtype=np.int32)
    counts[2] = k // 2                        # a shorter message (TopLEK keeps fewer than k)
    alpha = 0.75
    want = shifts.copy()
    got = gpu.shift_update(shifts.copy(), diffs, d, lda, idx, counts, alpha, mult)
    for m in range(n):
        for f in idx[m, :counts[m]]:
            f = int(f)
            j, i = divmod(f, lda)
            item = diffs[m, f] * mult if mult != 1.0 else diffs[m, f]
            upd = alpha * item
            want[m, f] = want[m, f] + upd
            if i != j:
                want[m, i * lda + j] = want[m, i * lda + j] + upd
    np.testing.assert_array_equal(got, want)
    bad = idx.copy()
    bad[0, 0] = 1                             # row 1 of column 0: below the diagonal
    with pytest.raises(gpu.FedNLError):
        gpu.shift_update(shifts, diffs, d, lda, bad, counts, alpha, mult)


def test_aggregate_operator(gpu):
    """fednl_gpu_aggregate against the master's merge in client order (TrainLoop.h:1100-1333), bit for
    bit: g and l as running sums times 1/n, H += each client's message in client order."""
    rng = np.random.default_rng(32)
    d, lda, nc, k = 29, 32, 9, 60
    U = d * (d + 1) // 2
    up = np.array([j * lda + i for j in range(d) for i in range(j + 1)], dtype=np.uint32)
    grads = rng.standard_normal((nc, d))
    lks = rng.random(nc)
    H = _sym_full(rng, 1, d, lda)[0]
    idx = np.stack([np.sort(rng.choice(up, k, replace=False)) for _ in range(nc)]).astype(np.uint32)
    vals = rng.standard_normal((nc, k)) * 1e-3
    counts = np.full(nc, k, dtype=np.int32)
    counts[4] = 17
    Hg, g, l = gpu.aggregate(grads, lks, d, lda, H, idx, vals, counts)
    gw = np.zeros(d)
    lw = 0.0
    Hw = H.copy()
    for c in range(nc):
        gw = gw + grads[c]
        lw = lw + lks[c]
        Hw[idx[c, :counts[c]].astype(np.int64)] += vals[c, :counts[c]]
    np.testing.assert_array_equal(g, gw * (1.0 / nc))
    assert l == lw * (1.0 / nc)
    np.testing.assert_array_equal(Hg, Hw)
    H0, g0, l0 = gpu.aggregate(grads, lks, d, lda, H)             # no Hessian messages
    np.testing.assert_array_equal(H0, H)
    np.testing.assert_array_equal(g0, g)
    dup = idx.copy()
    dup[1, 1] = dup[1, 0]
    with pytest.raises(gpu.FedNLError):
        gpu.aggregate(grads, lks, d, lda, H, dup, vals, counts)
    assert U > k


def test_compress_identity_operator(gpu, oracle):
    """fednl_gpu_compress_identity against LocalWorkerForFedNL_Identical.h:80-94 written out in numpy:
    message = upper entries times alpha/n in the upper-index order, shift += alpha diff on both
    triangles, bit for bit."""
    rng = np.random.default_rng(33)
    d, lda, n = 21, 24, 4
    diffs = _sym_full(rng, n, d, lda)
    shifts = _sym_full(rng, n, d, lda)
    alpha, pre = 1.0, 1.0 / 7.0
    idx, vals, sh = gpu.compress_identity(diffs, d, lda, alpha, pre, shifts)
    up = oracle.upper_indices(d, lda)
    for m in range(n):
        np.testing.assert_array_equal(idx[m], up)
        np.testing.assert_array_equal(vals[m], diffs[m][up.astype(np.int64)] * pre)
        want = shifts[m].copy()
        full = diffs[m].reshape(d, lda)
        for j in range(d):
            for i in range(d):
                v = full[max(i, j), min(i, j)]
                want[j * lda + i] = want[j * lda + i] + alpha * v
        np.testing.assert_array_equal(sh[m], want)
