"""The FP64 Cholesky's square root and reciprocal are computed from integer arithmetic (FP32
estimates, Newton steps with exact 64-bit residuals, an exact remainder test for the rounding); they
must equal the hardware's correctly rounded sqrt and 1.0 / x bit for bit, which keeps the factor
identical to the oracle's.  The same algorithms were checked on the host against IEEE sqrt and
division over 4e7 inputs."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from ufednl_gb300 import build, fednl
    build.build()
    fednl.load()
    return fednl


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_integer_sqrt_and_reciprocal_are_correctly_rounded(gpu, seed):
    s, r = gpu.selftest_rn(1 << 26, seed)
    assert (s, r) == (0, 0)
