"""Tensor-core (tcgen05) weighted Gram matrices of the mixed-precision form against an FP64 numpy
reference of the same sum.  TF32 keeps 10 mantissa bits of each input (relative rounding 2^-11)
and accumulates in FP32, so the bar is a Frobenius relative error below 2e-3 per client and no
entry off by more than 1e-2 of the largest magnitude."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from ufednl_gb300 import build, fednl
    build.build()
    fednl.load()
    return fednl


@pytest.mark.parametrize("d,ns", [(128, [37, 200, 64]), (256, [513, 96, 1000, 32]), (384, [700])])
def test_weighted_gram_tf32(gpu, d, ns):
    rng = np.random.default_rng(d + len(ns))
    S = sum(ns)
    X = rng.standard_normal((S, d)).astype(np.float32)
    w = rng.uniform(0.0, 0.25, S).astype(np.float32)
    lam = 1e-3
    out = gpu.weighted_gram_tf32(X, w, ns, lam)
    off = 0
    for c, n in enumerate(ns):
        Xc = X[off:off + n].astype(np.float64)
        ref = Xc.T @ (Xc * w[off:off + n, None].astype(np.float64)) + lam * np.eye(d)
        off += n
        got = out[c].astype(np.float64)
        iu = np.triu_indices(d)
        err = np.linalg.norm(got[iu] - ref[iu]) / np.linalg.norm(ref[iu])
        assert err < 2e-3, (c, err)
        assert np.max(np.abs(got[iu] - ref[iu])) < 1e-2 * np.max(np.abs(ref))


def test_mixed_round_tracks_fp64(gpu):
    """The mixed-precision round (TF32 tensor-core Hessians, FP32 shifts, float-float margins and
    gradients, FP64 master and solve) against the FP64 engine on the same data and the same
    RandK-Philox stream: the first gradient norm agrees to 1e-10 (it does not depend on Hessians),
    the ||g|| trajectories agree within 2% every round while ||g|| falls by more than 30x (RandK
    with alpha = k/U learns the Hessians slowly), and the iterates agree to 1e-2 relative."""
    from ufednl_gb300 import datagen
    prob = datagen.dense_problem_fp32(51, 256, [300, 180, 420, 260, 350, 200], 1e-3)
    d, k = 256, 4 * 256
    alpha = k / (d * (d + 1) // 2)
    mx = gpu.MixedFedNL(prob, k, alpha)
    g_mx = mx.run(30)
    x_mx = mx.x()
    mx.close()
    p64 = datagen.Problem(d, prob.n_samples, prob.features.astype(np.float64), prob.labels, prob.lam)
    f64 = gpu.FedNL(p64, "randk_philox", k, alpha, feature_format=2)
    g_64 = f64.run(30)
    x_64 = f64.x()
    f64.close()
    print("mixed", g_mx[[0, 5, 10, 20, 29]], "fp64", g_64[[0, 5, 10, 20, 29]])
    assert abs(g_mx[0] - g_64[0]) <= 1e-10 * g_64[0]
    assert g_mx[-1] < g_mx[0] / 30 and g_64[-1] < g_64[0] / 30
    rel = np.abs(g_mx - g_64) / g_64
    assert np.all(rel < 0.02), rel
    assert np.linalg.norm(x_mx - x_64) <= 1e-2 * np.linalg.norm(x_64)


def _topk_check(diff, sel, k):
    """sel is the k largest |diff| (FP32 magnitudes), ties at the threshold to the lower positions."""
    mag = np.abs(diff.astype(np.float32))
    assert len(sel) == min(k, len(diff))
    if len(sel) == len(diff):
        return
    order = np.lexsort((np.arange(len(diff)), -mag))        # magnitude descending, position ascending
    np.testing.assert_array_equal(np.sort(order[:k]), sel)


@pytest.mark.parametrize("d,comp", [(200, "topk"), (130, "topk"), (256, "topk"), (69, "topk")])
def test_mixed_topk_selects_the_k_largest(gpu, d, comp):
    """TopK on the FP32 differences (d padded to the tile grid): every client's selection is the
    exact top-k of that round's differences."""
    from ufednl_gb300 import datagen
    prob = datagen.dense_problem_fp32(61, d, [90, 150, 64, 200], 1e-3)
    k = 8 * d
    mx = gpu.MixedFedNL(prob, k, 1.0, compressor=comp)
    for r in range(3):
        mx.run(1)
        for c in range(prob.n_clients):
            _topk_check(mx.diff(c), mx.selection(c), k)
    mx.close()


def _packed_diag(U):
    d = int((np.sqrt(8 * U + 1) - 1) / 2)
    diag = np.zeros(U, dtype=bool)
    diag[[j * (j + 1) // 2 + j for j in range(d)]] = True
    return diag


@pytest.mark.parametrize("d", [130, 256])
def test_mixed_toplek_window_rule(gpu, d):
    """TopLEK on the FP32 differences: the kept set is a prefix of the top-k order (largest first),
    and its size is K-1-m* or K-m* where m* is the first removal (smallest first) at which the
    removed mass plus the mass outside the top-k passes (1 - k/U) F - F/10."""
    from ufednl_gb300 import datagen
    prob = datagen.dense_problem_fp32(62, d, [120, 80, 160], 1e-3)
    U = d * (d + 1) // 2
    k = 8 * d
    mx = gpu.MixedFedNL(prob, k, 1.0, compressor="toplek")
    diag = _packed_diag(U)
    seen = set()
    for r in range(4):
        mx.run(1)
        for c in range(prob.n_clients):
            diff = mx.diff(c).astype(np.float64)
            sel = mx.selection(c)
            mag = np.abs(diff)
            order = np.lexsort((np.arange(U), -np.abs(mx.diff(c))))
            top = order[:k]
            keep = len(sel)
            np.testing.assert_array_equal(np.sort(top[:keep]), sel)
            terms = np.where(diag, 1.0, 2.0) * mag * mag
            F = terms.sum()
            asc = top[::-1]                                    # smallest of the top-k first
            num0 = F - terms[top].sum()
            lo = (1 - k / U) * F - 0.1 * F
            if not ((1 - k / U) * F + 0.1 * F > num0):        # no window (e.g. all differences zero)
                assert keep == 0, (r, c, keep)
                continue
            nx = num0 + np.cumsum(terms[asc])
            mstar = int(np.argmax(nx > lo))
            ok = {k - 1 - mstar, k - mstar}
            near = {k - 1 - m for m in (mstar - 1, mstar + 1)} | {k - m for m in (mstar - 1, mstar + 1)}
            assert keep in ok or keep in near, (r, c, keep, mstar)
            seen.add(keep == k - mstar)
    mx.close()


@pytest.mark.parametrize("comp", ["topk", "toplek"])
def test_mixed_top_compressors_reach_tolerance_like_fp64(gpu, comp):
    """The w8a-like workload (d = 301 binary features padded to 384 on the tensor cores, 142
    clients with n_i in 200-600, k = 8d): the mixed-precision round with TopK / TopLEK reaches
    ||g|| <= 1e-9 at most three rounds after the FP64 engine does, and the first ||g|| agrees to
    1e-10 (it does not depend on the Hessians)."""
    from ufednl_gb300 import datagen
    prob = datagen.workload_w8a_like()
    k = 8 * prob.d
    mx = gpu.MixedFedNL(prob, k, 1.0, compressor=comp)
    g_mx = mx.run(30)
    mx.close()
    f64 = gpu.FedNL(prob, comp, k, 1.0, workers=16)
    g_64 = f64.run(30)
    f64.close()
    print(comp, "mixed", g_mx[:20], "fp64", g_64[:20])
    assert abs(g_mx[0] - g_64[0]) <= 1e-10 * g_64[0]
    assert np.any(g_64 <= 1e-9)
    r64 = int(np.argmax(g_64 <= 1e-9))
    assert np.any(g_mx[: r64 + 4] <= 1e-9)


def test_mixed_padded_randk_tracks_fp64(gpu):
    """RandK-Philox at d = 200 (padded to 256): the same stream as the FP64 engine, trajectories
    within 2%."""
    from ufednl_gb300 import datagen
    prob = datagen.dense_problem_fp32(64, 200, [300, 180, 420, 260], 1e-3)
    d, k = 200, 4 * 200
    alpha = k / (d * (d + 1) // 2)
    mx = gpu.MixedFedNL(prob, k, alpha)
    g_mx = mx.run(20)
    mx.close()
    p64 = datagen.Problem(d, prob.n_samples, prob.features.astype(np.float64), prob.labels, prob.lam)
    f64 = gpu.FedNL(p64, "randk_philox", k, alpha, feature_format=2)
    g_64 = f64.run(20)
    f64.close()
    assert abs(g_mx[0] - g_64[0]) <= 1e-10 * g_64[0]
    assert np.all(np.abs(g_mx - g_64) / g_64 < 0.02)


def _spd(rng, d, cond):
    q, _ = np.linalg.qr(rng.standard_normal((d, d)))
    ev = np.geomspace(1.0, 1.0 / cond, d)
    return (q * ev) @ q.T


@pytest.mark.parametrize("d", [1, 5, 31, 32, 33, 64, 65, 100, 257, 301, 304])
def test_mixed_solve_matches_fp64(gpu, d):
    """The mixed form's Newton solve (FP32 shared-memory Cholesky, one refinement step on a
    float-float residual): relative error against an FP64 solve below 2e-8 for condition numbers
    up to 1e3 and below 2e-4 at 1e5 (one refinement step squares the FP32 solve's error, about
    cond x 2^-24)."""
    rng = np.random.default_rng(d)
    for cond, tol in ((1e3, 2e-8), (1e5, 2e-4)):
        H = _spd(rng, d, cond)
        lda = d + 3
        Hc = np.zeros((d, lda))
        Hc[:, :d] = H.T                                   # column-major with leading dimension lda
        g = rng.standard_normal(d)
        l = 1e-3
        dx = gpu.cholesky_option_b_solve_mixed(Hc.ravel(), d, lda, l, g)
        ref = np.linalg.solve(H + l * np.eye(d), g)
        err = np.linalg.norm(dx - ref) / np.linalg.norm(ref)
        assert err < tol, (d, cond, err)


def test_mixed_solve_not_pd(gpu):
    H = np.array([[1.0, 2.0], [2.0, 1.0]])
    with pytest.raises(gpu.FedNLError) as e:
        gpu.cholesky_option_b_solve_mixed(H.ravel(), 2, 2, 0.0, np.ones(2))
    assert e.value.code == -4


@pytest.mark.parametrize("d", [1, 5, 31, 32, 33, 64, 65, 100, 257, 301, 640, 1024, 1312])
def test_mixed_coop32_solve_matches_fp64(gpu, d):
    """The FP32 Cholesky on a cooperative grid with FP64-residual refinement (to 2^-30, six steps at
    most): relative error against an FP64 solve below 5e-9 at condition 1e3; at 1e5 each step gains
    only a factor of about cond x 2^-24 x a growth factor in d, and the bar is 1e-3."""
    rng = np.random.default_rng(1000 + d)
    for cond, tol in ((1e3, 5e-9), (1e5, 1e-3)):
        H = _spd(rng, d, cond)
        lda = d + 3
        Hc = np.zeros((d, lda))
        Hc[:, :d] = H.T
        g = rng.standard_normal(d)
        l = 1e-3
        dx = gpu.cholesky_option_b_solve32(Hc.ravel(), d, lda, l, g)
        ref = np.linalg.solve(H + l * np.eye(d), g)
        err = np.linalg.norm(dx - ref) / np.linalg.norm(ref)
        assert err < tol, (d, cond, err)


def test_mixed_coop32_solve_same_for_every_grid(gpu):
    """Every element of the factor, the residual and the solves is computed by the same arithmetic
    whichever CTA owns it: the result is bit-identical across CTA counts and between the
    cooperative launch (grid barriers) and a single cluster (cluster barriers)."""
    rng = np.random.default_rng(7)
    d = 300
    H = _spd(rng, d, 1e4)
    g = rng.standard_normal(d)
    ref = gpu.cholesky_option_b_solve32(H, d, d, 1e-3, g, grid=1)
    for G in (2, 3, 7, 45, 64, -2, -8, -16):             # negative: one thread-block cluster
        np.testing.assert_array_equal(gpu.cholesky_option_b_solve32(H, d, d, 1e-3, g, grid=G), ref)
    exact = np.linalg.solve(H + 1e-3 * np.eye(d), g)
    e = [np.linalg.norm(gpu.cholesky_option_b_solve32(H, d, d, 1e-3, g, refine=r) - exact) / np.linalg.norm(exact)
         for r in (0, 1, 2, 6)]
    assert e[0] < 0.05 and e[3] < 1e-8 and e[3] <= e[2] <= e[1] <= e[0], e


def test_mixed_coop32_solve_hands_ill_conditioned_and_indefinite_systems_to_fp64(gpu):
    """A pivot that keeps fewer than six bits in FP32 (condition 1e9 here) sends the system to the
    FP64 cooperative solve in the same launch: the answer has FP64 accuracy.  A matrix that is not
    positive definite is reported by that solve (FEDNL_ENOTPD)."""
    rng = np.random.default_rng(11)
    d = 96
    H = _spd(rng, d, 1e9)
    g = rng.standard_normal(d)
    dx = gpu.cholesky_option_b_solve32(H, d, d, 0.0, g)
    ref = np.linalg.solve(H, g)
    assert np.linalg.norm(dx - ref) / np.linalg.norm(ref) < 1e-5
    with pytest.raises(gpu.FedNLError) as e:
        gpu.cholesky_option_b_solve32(np.array([[1.0, 2.0], [2.0, 1.0]]), 2, 2, 0.0, np.ones(2))
    assert e.value.code == -4


@pytest.mark.parametrize("comp", ["randk_philox", "toplek"])
def test_mixed_round_with_coop32_solve_tracks_fp64_solve(gpu, comp):
    """The mixed round solved by the FP32 cooperative Cholesky with two refinement steps: the ||g||
    trajectory agrees with the FP64-solve trajectory to 1e-8 relative while ||g|| falls by decades."""
    from ufednl_gb300 import datagen
    d = 200
    prob = datagen.dense_problem_fp32(71, d, [240, 300, 180, 260], 1e-3)
    k = 4 * d if comp == "randk_philox" else 8 * d
    alpha = k / (d * (d + 1) // 2) if comp == "randk_philox" else 1.0
    a = gpu.MixedFedNL(prob, k, alpha, compressor=comp)
    ga = a.run(15)
    a.close()
    b = gpu.MixedFedNL(prob, k, alpha, compressor=comp, solver="fp32_coop")
    gb = b.run(15)
    b.close()
    assert abs(ga[0] - gb[0]) <= 1e-14 * ga[0]
    n = int(np.sum(ga > 1e-8))
    assert n >= 4 and np.all(np.abs(ga[:n] - gb[:n]) <= 1e-8 * ga[:n]), (ga, gb)


@pytest.mark.parametrize("comp", ["randk_philox", "toplek"])
def test_mixed_round_with_refined_fp32_solve_tracks_fp64_solve(gpu, comp):
    """The same mixed round solved by the FP32 shared-memory Cholesky with one refinement step
    instead of the FP64 cooperative Cholesky: the ||g|| trajectories agree to 1e-6 relative while
    ||g|| falls by decades (the refined solve is accurate to about 1e-8 relative)."""
    from ufednl_gb300 import datagen
    d = 200
    prob = datagen.dense_problem_fp32(71, d, [240, 300, 180, 260], 1e-3)
    k = 4 * d if comp == "randk_philox" else 8 * d
    alpha = k / (d * (d + 1) // 2) if comp == "randk_philox" else 1.0
    a = gpu.MixedFedNL(prob, k, alpha, compressor=comp)
    ga = a.run(15)
    a.close()
    b = gpu.MixedFedNL(prob, k, alpha, compressor=comp, solver="fp32_refined")
    gb = b.run(15)
    b.close()
    assert abs(ga[0] - gb[0]) <= 1e-14 * ga[0]          # ||g|| summed in another order
    n = int(np.sum(ga > 1e-8))
    assert np.all(np.abs(ga[:n] - gb[:n]) <= 1e-6 * ga[:n]), (ga, gb)
