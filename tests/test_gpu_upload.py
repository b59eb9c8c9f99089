"""Client-data upload (fednl_gpu_upload_client_data): the host conversion of the dense FP64 rows into
the binary layout runs on host threads over client ranges; the format it picks and the first
non-binary entry it reports do not depend on how the clients are split."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from ufednl_gb300 import build, fednl
    build.build()
    fednl.load()
    return fednl


def _problem():
    from ufednl_gb300 import datagen
    return datagen.binary_problem(11, 40, [31, 18, 40, 27, 64, 5, 90, 33, 12, 70, 44], 0.2, 1e-3)


def test_binary_auto_and_dense_uploads_agree(gpu):
    """AUTO detects the 0/1 features and takes the binary kernels (the same iterates bit for bit as the
    explicit binary format); the dense layout agrees within 1e-12 relative."""
    prob = _problem()
    xs = []
    for fmt in (0, 1, 2):
        f = gpu.FedNL(prob, "topk", 3 * 40, 1.0, feature_format=fmt)
        g = f.run(4)
        xs.append((g, f.x()))
        f.close()
    np.testing.assert_array_equal(xs[1][0], xs[0][0])
    np.testing.assert_array_equal(xs[1][1], xs[0][1])
    np.testing.assert_allclose(xs[2][0], xs[0][0], rtol=1e-12, atol=0)
    assert np.linalg.norm(xs[2][1] - xs[0][1]) <= 1e-12 * np.linalg.norm(xs[0][1])


@pytest.mark.parametrize("pos", [(0, 0), (57, 3), (200, 39), (-1, 39)])
def test_binary_upload_reports_the_first_non_binary_entry(gpu, pos):
    """A value that is neither 0 nor 1 fails the explicit binary format with the position of the first
    such entry in sample order, whichever client range holds it; AUTO falls back to dense."""
    prob = _problem()
    S = prob.features.shape[0]
    s, i = pos[0] % S, pos[1]
    prob.features[s, i] = 0.5
    if s + 7 < S:
        prob.features[s + 7, 1] = 2.0          # a later entry must not be the one reported
    with pytest.raises(gpu.FedNLError, match=rf"feature \({s},{i}\) is not 0/1"):
        gpu.FedNL(prob, "topk", 3 * 40, 1.0, feature_format=1)
    f = gpu.FedNL(prob, "topk", 3 * 40, 1.0, feature_format=0)
    g0 = f.run(2)
    f.close()
    f = gpu.FedNL(prob, "topk", 3 * 40, 1.0, feature_format=2)
    g2 = f.run(2)
    f.close()
    np.testing.assert_array_equal(g0, g2)


@pytest.mark.parametrize("intercept", [True, False])
def test_csr_upload_packs_the_same_layout(gpu, intercept):
    """fednl_gpu_upload_client_csr (0/1 features as CSR columns, bit layout packed on the device) gives
    the same run bit for bit as the dense upload, with and without an intercept column."""
    from ufednl_gb300 import datagen
    prob = datagen.binary_problem(21, 33, [40, 75, 64, 129, 12], 0.15, 1e-3)
    if not intercept:
        prob = datagen.Problem(prob.d - 1, prob.n_samples, np.ascontiguousarray(prob.features[:, :-1]),
                               prob.labels, prob.lam)
    out = []
    for csr in (False, True):
        f = gpu.FedNL(prob, "toplek", 4 * prob.d, 1.0, workers=2, csr=csr)
        out.append((f.run(5), f.x(), f.hess_schedule()))
        f.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


def test_csr_upload_rejects_unsorted_columns(gpu):
    import ctypes as C
    from ufednl_gb300 import datagen
    prob = datagen.binary_problem(22, 9, [3, 4], 0.4, 1e-3)
    f = gpu.FedNL(prob, "topk", 9, 1.0)
    rp = np.arange(prob.total_samples + 1, dtype=np.int32) * 2
    ci = np.tile(np.array([5, 3], dtype=np.int32), prob.total_samples)      # descending within each row
    lab = np.ascontiguousarray(prob.labels)
    rc = gpu.load().fednl_gpu_upload_client_csr(f._h, rp.ctypes.data_as(C.POINTER(C.c_int32)),
                                               ci.ctypes.data_as(C.POINTER(C.c_int32)),
                                               lab.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc != 0 and "ascending" in gpu.load().fednl_gpu_last_error().decode()
    f.close()


def test_binary_upload_negative_zero_and_row_tail(gpu):
    """The scan skips four +0.0 values at a time by their bits: -0.0 (sign bit set) still counts as 0,
    and the values past the last multiple of four in a row (d = 41) are checked one by one."""
    from ufednl_gb300 import datagen
    prob = datagen.binary_problem(23, 41, [30, 50, 21, 64], 0.15, 1e-3)
    neg = datagen.Problem(prob.d, prob.n_samples, np.where(prob.features == 0.0, -0.0, prob.features),
                          prob.labels, prob.lam)
    assert np.signbit(neg.features).sum() > 0
    out = []
    for p in (prob, neg):
        f = gpu.FedNL(p, "topk", 3 * 41, 1.0, feature_format=1)
        out.append((f.run(3), f.x()))
        f.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    for s, i in [(17, 40), (100, 37), (0, 1)]:
        bad = datagen.Problem(prob.d, prob.n_samples, prob.features.copy(), prob.labels, prob.lam)
        bad.features[s, i] = 0.5
        with pytest.raises(gpu.FedNLError, match=rf"feature \({s},{i}\) is not 0/1"):
            gpu.FedNL(bad, "topk", 3 * 41, 1.0, feature_format=1)
