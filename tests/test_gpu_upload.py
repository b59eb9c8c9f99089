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
