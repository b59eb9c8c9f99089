"""The binary Hessian's kernels give the same bits: the common-sample lists built at upload
(k_hess_hits) against the attribute masks intersected every round (k_hess_binary, masks in shared or
global memory), at every block size, over whole TopLEK / TopK / RandK runs and the initial shifts.
Covers clients with and without an intercept column, attributes common enough that upper positions
hold long lists, a problem dense enough that no lists are built, and FedNL-PP (its Hessian keeps H_i
for the Lk taken after the update)."""
import numpy as np
import pytest

from ufednl_gb300 import datagen

pytestmark = pytest.mark.gpu

SCHEDULES = [("lists", 128), ("lists", 256), ("lists", 512), ("masks_smem", 256), ("masks_global", 128),
             ("masks_global", 512)]


@pytest.fixture(scope="module")
def gpu():
    from ufednl_gb300 import build, fednl
    build.build()
    fednl.load()
    return fednl


def skewed_problem(seed, d, ns, intercept=True):
    """Bernoulli features whose first attributes are common (density 0.6) and the rest rare (0.06):
    upper positions among the common attributes hold dozens of common samples."""
    rng = np.random.default_rng(seed)
    s = int(np.sum(ns))
    dens = np.where(np.arange(d - 1) < 6, 0.6, 0.06)
    a = (rng.random((s, d - 1)) < dens).astype(np.float64)
    if intercept:
        a = np.concatenate([a, np.ones((s, 1))], axis=1)
    else:
        a = np.concatenate([a, (rng.random((s, 1)) < 0.3).astype(np.float64)], axis=1)
    w = rng.standard_normal(d) / np.sqrt(d)
    y = np.where(rng.random(s) < 1.0 / (1.0 + np.exp(-(a @ w))), 1.0, -1.0)
    return datagen.Problem(d=d, n_samples=np.asarray(ns, dtype=np.int32), features=np.ascontiguousarray(a),
                           labels=y, lam=1e-3)


def run_with(gpu, prob, comp, k, schedule, rounds=6):
    f = gpu.FedNL(prob, comp, k, 1.0, workers=3, hess_schedule=schedule)    # initial shifts too
    sch = f.hess_schedule()
    assert sch["lists_built"] and (sch["kernel"], sch["threads"]) == schedule
    g = f.run(rounds)
    x = f.x()
    f.close()
    return g, x


@pytest.mark.parametrize("intercept", [True, False])
@pytest.mark.parametrize("comp", ["toplek", "topk", "randk"])
def test_schedules_identical(gpu, comp, intercept):
    prob = skewed_problem(5 + intercept, 57, [70, 131, 64, 200, 97], intercept)
    k = 4 * prob.d
    ref_g, ref_x = run_with(gpu, prob, comp, k, SCHEDULES[0])
    for sch in SCHEDULES[1:]:
        g, x = run_with(gpu, prob, comp, k, sch)
        np.testing.assert_array_equal(g, ref_g, err_msg=str(sch))
        np.testing.assert_array_equal(x, ref_x, err_msg=str(sch))


def test_lists_default_and_dense_fallback(gpu):
    prob = datagen.binary_problem(11, 41, [50, 90, 64], 0.05, 1e-3)
    f = gpu.FedNL(prob, "topk", 4 * 41, 1.0)
    assert f.hess_schedule() == {"kernel": "lists", "threads": 256, "lists_built": True}
    f.close()
    dense = datagen.binary_problem(12, 31, [600, 500], 0.5, 1e-3)     # ~100 pairs per sample: no lists
    f = gpu.FedNL(dense, "topk", 4 * 31, 1.0)
    sch = f.hess_schedule()
    assert not sch["lists_built"] and sch["kernel"] == "masks_smem"
    with pytest.raises(RuntimeError):
        f.set_hess_schedule("lists", 256)
    f.close()


def test_pp_schedules_identical(gpu):
    prob = skewed_problem(21, 33, [6] * 64)
    out = []
    for sch in [("lists", 256), ("masks_global", 256)]:
        f = gpu.FedNL(prob, "randseqk", prob.d, 1.0, clients_per_round=16, hess_schedule=sch)
        out.append((f.run(8), f.x()))
        f.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
