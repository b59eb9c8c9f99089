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
