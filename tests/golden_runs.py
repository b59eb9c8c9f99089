"""Shared readers and contracts for the golden whole-run fixtures (tests/golden/run*.npz), used by
the oracle tests and the GPU parity tests.

A fixture holds the reference's own run (produced by tests/golden/make_golden.py through
oracle/ref_harness.cpp): per round the iterate, ||g||, l and, for the dumped rounds, every client's
message and Lk.  Small fixtures store their inputs and full messages; the workload-sized ones
(the a9a-like and w8a-like benchmark workloads) store the generator's name with a digest of its
output and 16-byte digests of the messages.
"""
from __future__ import annotations

import hashlib

import numpy as np

from ufednl_gb300 import datagen


def message_digest(idx, val, lk) -> np.ndarray:
    """16-byte digest of one client's round message: indices u32, values f64, Lk f64, little endian."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(idx, dtype="<u4").tobytes())
    h.update(np.ascontiguousarray(val, dtype="<f8").tobytes())
    h.update(np.array([lk], dtype="<f8").tobytes())
    return np.frombuffer(h.digest()[:16], dtype=np.uint8)


def problem_digest(prob) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(prob.n_samples, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(prob.features, dtype="<f8").tobytes())
    h.update(np.ascontiguousarray(prob.labels, dtype="<f8").tobytes())
    return h.hexdigest()


def problem_of(z) -> datagen.Problem:
    """The fixture's inputs: stored arrays, or the named workload regenerated and checked against
    the stored digest."""
    if "workload" in z:
        prob = getattr(datagen, str(z["workload"]))()
        assert problem_digest(prob) == str(z["inputs_sha256"]), "workload generator output changed"
        return prob
    return datagen.Problem(int(z["d"]), z["n_samples"], z["features"], z["labels"], float(z["lam"]))


def is_workload(z) -> bool:
    return "workload" in z


def run_kwargs(z) -> dict:
    """Option A / FedNL-LS / tracking switches of an extended golden run (runx_*.npz)."""
    if "f" not in z:
        return {}
    ls = (float(z["ls_c"]), float(z["ls_gamma"]), int(z["ls_max"])) if int(z["line_search"]) else None
    return dict(option_a=bool(int(z["option_a"])), line_search=ls, track_f=bool(int(z["track_f"])))


def exact_rounds(z) -> int:
    """Rounds that must be bit-identical in the reference-order mode: all of them, or those before
    the first round in which the reference's libm exp (its sigmoid's scalar tail) returned a value
    other than the correctly rounded one and that changed a sigmoid value."""
    mis = int(z["libm_first_misround"]) if "libm_first_misround" in z else -1
    return int(z["rounds"]) if mis < 0 else mis


def check_run_bitexact(fed, z, n_clients: int) -> int:
    """Contract of a reference-order run (fed: oracle or GPU engine with ref_order) against the
    reference's golden run.

    Rounds before exact_rounds(z): the iterate, ||g||, l, every dumped client message (indices and
    values) and Lk are bit-identical, and so is the number of line-search evaluations; the tracked
    objective f(x_k) agrees to 1e-12 (the reference's loss takes libm's log on its scalar tail).
    Later rounds: iterates agree within 1e-10 relative every round.  Returns the number of
    bit-identical rounds."""
    rounds, dump = int(z["rounds"]), int(z["dump_rounds"])
    exact = exact_rounds(z)
    digests = "msg_digest" in z
    pos = mi = 0
    for r in range(rounds):
        g = fed.round()
        x, xr = fed.x(), z["x"][r]
        if r < exact:
            assert np.array_equal(x, xr), f"round {r}: iterate differs (max rel {np.max(np.abs(x - xr)) / np.max(np.abs(xr)):.3e})"
            assert g == z["gnorm"][r], f"round {r}: ||g|| {g!r} vs {z['gnorm'][r]!r}"
            assert fed.l() == z["l"][r], f"round {r}: l {fed.l()!r} vs {z['l'][r]!r}"
            if "f" in z:
                assert abs(fed.f() - z["f"][r]) <= 1e-12 * abs(z["f"][r]), (r, fed.f(), z["f"][r])
                assert fed.ls_steps() == int(z["ls_steps"][r])
        else:
            np.testing.assert_allclose(x, xr, rtol=1e-10, atol=1e-10 * np.max(np.abs(xr)),
                                       err_msg=f"round {r}")
        if r < dump:
            for c in range(n_clients):
                cnt = int(z["msg_count"][mi])
                if r < exact:
                    idx, val = fed.message(c)
                    lk = fed.lk(c)
                    if digests:
                        assert np.array_equal(message_digest(idx, val, lk), z["msg_digest"][mi]), \
                            f"round {r} client {c}: message or Lk differs"
                    else:
                        np.testing.assert_array_equal(idx, z["msg_idx"][pos:pos + cnt], err_msg=f"round {r} client {c}")
                        np.testing.assert_array_equal(val, z["msg_val"][pos:pos + cnt], err_msg=f"round {r} client {c}")
                        assert lk == z["lk"][mi], f"round {r} client {c}: Lk differs"
                pos += cnt
                mi += 1
    return exact
