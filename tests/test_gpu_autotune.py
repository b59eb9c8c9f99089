"""Autotuning of the round's Newton solve and of the binary Hessian's launch shape: the measurement
leaves the run's state untouched, the FP64 engine's results do not depend on the chosen CTA count or
shape, and the mixed engine's choice keeps its trajectory (the FP32 solver agrees with the FP64 one
to about 1e-6 relative)."""
import numpy as np
import pytest

from ufednl_gb300 import datagen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from ufednl_gb300 import build, fednl
    build.build()
    fednl.load()
    return fednl


def test_fp64_autotune_keeps_results(gpu):
    prob = datagen.binary_problem(91, 77, [60, 81, 49, 70], 0.2, 1e-3)
    a = gpu.FedNL(prob, "toplek", 8 * 77, 1.0, workers=2)
    b = gpu.FedNL(prob, "toplek", 8 * 77, 1.0, workers=2)
    ga = a.run(3)
    gb = b.run(3)
    x_before = b.x()
    t = b.autotune()
    assert 1 <= t["chol_ctas"] <= 152 and t["solve_ms"] > 0
    # the Hessian's launch shape, tuned per (d, n_i bucket): n_i up to 81 is bucket 7
    assert t["hess_threads"] in (128, 256, 512) and t["ni_bucket"] == 7 and t["hess_ms"] > 0
    np.testing.assert_array_equal(b.x(), x_before)            # tuning ran on scratch outputs
    ga = np.concatenate([ga, a.run(5)])
    gb = np.concatenate([gb, b.run(5)])
    np.testing.assert_array_equal(ga, gb)
    np.testing.assert_array_equal(a.x(), b.x())
    a.close()
    b.close()


@pytest.mark.parametrize("d", [128, 384])
def test_mixed_autotune_choice_tracks(gpu, d):
    prob = datagen.dense_problem_fp32(92, d, [200, 150, 260], 1e-3)
    k = 8 * d
    a = gpu.MixedFedNL(prob, k, 1.0, compressor="topk")
    b = gpu.MixedFedNL(prob, k, 1.0, compressor="topk")
    ga = a.run(2)
    gb = b.run(2)
    x_before = b.x()
    t = b.autotune()
    assert t["solver"] in ("fp64", "fp32_refined", "fp32_coop") and t["solve_ms"] > 0
    if d > 304:
        assert t["solver"] != "fp32_refined"
    np.testing.assert_array_equal(b.x(), x_before)
    ga = np.concatenate([ga, a.run(6)])
    gb = np.concatenate([gb, b.run(6)])
    n = int(np.sum(ga > 1e-8))
    assert np.all(np.abs(ga[:n] - gb[:n]) <= 1e-6 * ga[:n]), (ga, gb, t)
    a.close()
    b.close()
