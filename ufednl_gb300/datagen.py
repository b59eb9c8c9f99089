"""Seeded synthetic FedNL problems with the shapes of the u-FedNL benchmark workloads.

The reference measures on LIBSVM sets (a9a, w8a, phishing); these generators stand in for them
with the same dimension, sample counts and feature densities, drawn from fixed seeds:

* ``binary_problem`` -- {0,1} features drawn Bernoulli(p) plus an intercept column of ones
  (the reference appends the intercept as the last attribute,
  dopt/dopt/optimization_problems/include/ml/dataset_loader_fs.h:854-860), labels y = +-1 drawn
  as Bernoulli(sigma(a^T w*)) with a planted w* ~ N(0, I/d).
* ``dense_problem`` -- N(0,1) features (stored FP64 after an FP32 round trip), intercept last.

Features are returned row-major ``[sum n_i, d]`` FP64 with the clients concatenated in order,
labels ``[sum n_i]`` in {-1, +1}.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Problem:
    d: int
    n_samples: np.ndarray          # int32 [n_clients]
    features: np.ndarray           # float64 [S, d]
    labels: np.ndarray             # float64 [S]
    lam: float
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def n_clients(self) -> int:
        return int(self.n_samples.shape[0])

    @property
    def total_samples(self) -> int:
        return int(self.n_samples.sum())

    def client_slice(self, c: int) -> slice:
        off = int(self.n_samples[:c].sum())
        return slice(off, off + int(self.n_samples[c]))

    def is_binary(self) -> bool:
        f = self.features
        return bool(np.all((f == 0.0) | (f == 1.0)))


def _labels(rng: np.random.Generator, a: np.ndarray, d: int) -> np.ndarray:
    w = rng.normal(0.0, 1.0 / np.sqrt(d), size=d)
    p = 1.0 / (1.0 + np.exp(-(a @ w)))
    return np.where(rng.random(a.shape[0]) < p, 1.0, -1.0)


def binary_problem(seed: int, d: int, n_samples, density: float, lam: float, name: str = "") -> Problem:
    """Bernoulli(density) {0,1} features with d-1 attributes plus the intercept column."""
    rng = np.random.default_rng(seed)
    ns = np.asarray(n_samples, dtype=np.int32)
    s = int(ns.sum())
    a = (rng.random((s, d - 1)) < density).astype(np.float64)
    a = np.concatenate([a, np.ones((s, 1))], axis=1)
    y = _labels(rng, a, d)
    return Problem(d=d, n_samples=ns, features=np.ascontiguousarray(a), labels=y, lam=lam, name=name)


def dense_problem(seed: int, d: int, n_samples, lam: float, name: str = "") -> Problem:
    """N(0,1) features (FP32-representable) with d-1 attributes plus the intercept column."""
    rng = np.random.default_rng(seed)
    ns = np.asarray(n_samples, dtype=np.int32)
    s = int(ns.sum())
    a = rng.standard_normal((s, d - 1)).astype(np.float32).astype(np.float64)
    a = np.concatenate([a, np.ones((s, 1))], axis=1)
    y = _labels(rng, a, d)
    return Problem(d=d, n_samples=ns, features=np.ascontiguousarray(a), labels=y, lam=lam, name=name)


# ---- the benchmark workloads ---------------------------------------------------------------

def workload_a9a_like() -> Problem:
    """d=124 (123 Bernoulli(0.11) + intercept), 80 clients x 407 samples, lambda 1e-3, seed 0."""
    return binary_problem(0, 124, [407] * 80, 0.11, 1e-3, name="a9a-like d124 80x407")


def workload_w8a_like() -> Problem:
    """d=301 (300 Bernoulli(0.039) + intercept), 142 clients, n_i ~ U{200..600}, lambda 1e-3, seed 1."""
    rng = np.random.default_rng(1)
    ns = rng.integers(200, 601, size=142)
    p = binary_problem(1001, 301, ns, 0.039, 1e-3, name="w8a-like d301 142 clients n_i 200-600")
    return p


def workload_dense_1024() -> Problem:
    """d=1024 dense N(0,1) FP32 features, 256 clients, n_i ~ U{512..4096}, lambda 1e-4, seed 2."""
    rng = np.random.default_rng(2)
    ns = rng.integers(512, 4097, size=256)
    return dense_problem(1002, 1024, ns, 1e-4, name="dense d1024 256 clients n_i 512-4096")


def dense_problem_fp32(seed: int, d: int, n_samples, lam: float, name: str = "") -> Problem:
    """Dense N(0,1) features kept as FP32 (no intercept column), labels from a planted
    w* ~ N(0, I/d): the mixed-precision configuration.  features has dtype float32."""
    rng = np.random.default_rng(seed)
    ns = np.asarray(n_samples, dtype=np.int32)
    s = int(ns.sum())
    a = rng.standard_normal((s, d), dtype=np.float32)
    w = rng.normal(0.0, 1.0 / np.sqrt(d), size=d).astype(np.float32)
    z = a @ w
    p = 1.0 / (1.0 + np.exp(-z.astype(np.float64)))
    y = np.where(rng.random(s) < p, 1.0, -1.0)
    return Problem(d=d, n_samples=ns, features=a, labels=y, lam=lam, name=name)


def workload_dense_fp32_1024() -> Problem:
    """The mixed-precision workload: d=1024 dense N(0,1) FP32 features, 256 clients,
    n_i ~ U{512..4096} (seed 2), lambda 1e-4, planted labels."""
    rng = np.random.default_rng(2)
    ns = rng.integers(512, 4097, size=256)
    return dense_problem_fp32(1002, 1024, ns, 1e-4, name="dense FP32 d1024 256 clients n_i 512-4096")


def workload_phishing_pp() -> Problem:
    """d=69 (68 Bernoulli(0.45) + intercept), 2048 clients x 6 samples, lambda 1e-3, seed 3."""
    return binary_problem(3, 69, [6] * 2048, 0.45, 1e-3, name="phishing-like d69 2048x6")


def reference_lda(d: int) -> int:
    """LDA of the reference's AVX2 build: d rounded up to a multiple of 4
    (dopt/dopt/linalg_matrices/include/MatrixNMD.h:44-80)."""
    return (d + 3) // 4 * 4
