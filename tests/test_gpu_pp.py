"""FedNL-PP (dopt/bin_fednl_local_pp) on the GPU, through the C ABI.

Bars: the sampled clients, compressor index sets and generator streams are bit-exact with the
reference's golden PP runs; against the CPU oracle every round's iterate, gradient estimate, l,
true gradient, sampled set, messages, Lk, directions and shifts are bit-identical (same IEEE
operations in the same order)."""
import glob
import os

import numpy as np
import pytest

from conftest import golden_path
from test_oracle_golden import check_pp_against_reference
from ufednl_gb300 import datagen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from ufednl_gb300 import build, fednl
    build.build()
    fednl.load()
    return fednl


def _problem(z):
    return datagen.Problem(int(z["d"]), z["n_samples"], z["features"], z["labels"], float(z["lam"]))


@pytest.mark.parametrize("path", sorted(glob.glob(golden_path("pp_*.npz"))), ids=os.path.basename)
def test_pp_golden(gpu, path):
    z = np.load(path)
    prob = _problem(z)
    fed = gpu.FedNL(prob, str(z["compressor"]), int(z["k"]), float(z["alpha"]), lda=int(z["lda"]), workers=1,
                    clients_per_round=int(z["tau"]), client_seed=int(z["sel_seed"]))
    check_pp_against_reference(fed, z, prob)
    fed.close()


def _compare_pp(gpu, oracle, prob, comp, k, alpha, tau, rounds, workers=1, check_every=1):
    orc = oracle.FedNL(prob, comp, k, alpha, workers=workers, threads=min(workers, os.cpu_count() or 1),
                       clients_per_round=tau)
    fed = gpu.FedNL(prob, comp, k, alpha, workers=workers, clients_per_round=tau)
    for r in range(rounds):
        go = orc.round()
        gg = fed.round()
        sel = orc.selected()
        np.testing.assert_array_equal(fed.selected(), sel, err_msg=f"round {r}: sampled clients")
        np.testing.assert_array_equal(fed.x(), orc.x(), err_msg=f"round {r}: iterate")
        np.testing.assert_array_equal(fed.grad(), orc.grad(), err_msg=f"round {r}: gradient estimate")
        np.testing.assert_array_equal(fed.true_grad(), orc.true_grad(), err_msg=f"round {r}: true gradient")
        assert fed.l() == orc.l(), f"round {r}: l"
        assert gg == go, f"round {r}: ||true gradient||"
        if r % check_every == 0:
            for c in sel[:: max(1, len(sel) // 6)]:
                c = int(c)
                io, vo = orc.message(c)
                ig, vg = fed.message(c)
                np.testing.assert_array_equal(ig, io, err_msg=f"round {r} client {c}: indices")
                np.testing.assert_array_equal(vg, vo, err_msg=f"round {r} client {c}: values")
                assert fed.lk(c) == orc.lk(c), f"round {r} client {c}: Lk"
                for a, b in zip(fed.dir(c), orc.dir(c)):
                    np.testing.assert_array_equal(a, b, err_msg=f"round {r} client {c}: direction")
    c0 = int(orc.selected()[0])
    np.testing.assert_array_equal(fed.shift(c0), orc.shift(c0))
    fed.close()
    orc.close()


@pytest.mark.parametrize("comp", ["randseqk", "randk", "natural", "identity", "topk", "toplek"])
def test_pp_vs_oracle_small(gpu, oracle, comp):
    prob = datagen.binary_problem(31, 30, [9, 14, 7, 11, 12, 8, 10, 13, 9, 6, 15, 10, 8, 12, 11, 9], 0.3, 1e-3)
    U = 30 * 31 // 2
    k = {"topk": 120, "toplek": 150, "randk": 60, "randseqk": 30, "natural": U, "identity": U}[comp]
    alpha = {"randk": k / U, "randseqk": k / U, "natural": 8 / 9}.get(comp, 1.0)
    _compare_pp(gpu, oracle, prob, comp, k, alpha, 5, 10, workers=3)


def test_pp_vs_oracle_dense(gpu, oracle):
    prob = datagen.dense_problem(32, 12, [8, 11, 6, 9, 10, 7, 12, 5], 1e-2)
    _compare_pp(gpu, oracle, prob, "randseqk", 12, 12 / 78, 3, 8)


@pytest.mark.parametrize("comp", ["randseqk", "natural"])
def test_pp_vs_oracle_phishing_like_full_size(gpu, oracle, comp):
    """The phishing-like FedNL-PP workload at its full size: d=69, 2048 clients x 6 samples,
    tau = 128 sampled clients per round."""
    prob = datagen.workload_phishing_pp()
    U = 69 * 70 // 2
    k, alpha = (69, 69 / U) if comp == "randseqk" else (U, 8 / 9)
    _compare_pp(gpu, oracle, prob, comp, k, alpha, 128, 6, check_every=2)


def test_pp_full_participation_and_rejects_bad_tau(gpu, oracle):
    prob = datagen.binary_problem(33, 10, [7, 9, 8, 6], 0.4, 1e-3)
    _compare_pp(gpu, oracle, prob, "natural", 55, 8 / 9, 4, 5)          # tau = n: every client
    with pytest.raises(gpu.FedNLError):
        gpu.FedNL(prob, "natural", 55, 8 / 9, clients_per_round=5)
