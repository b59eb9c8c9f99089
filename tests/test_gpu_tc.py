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
