"""The reference's local driver on the engine: fednl_gpu_execute_local (doptExecuteLocal's command
line) and the LIBSVM loader it uses.

The loader is pinned bit for bit by fixtures made with the reference's own TextFileDataSetLoader
(tests/golden/make_golden.py, "libsvm"); argument handling returns the reference's
TrainReturnCodes before any device work, so it is tested without a GPU.  The GPU test runs a whole
command and compares the callback and the tracking records with the same run made through the
Python API."""
import glob
import os
import struct

import numpy as np
import pytest

from conftest import golden_path
from ufednl_gb300 import datagen

LIBSVM = sorted(glob.glob(golden_path("libsvm_*.npz")))


@pytest.fixture(scope="module")
def lib():
    from ufednl_gb300 import build, fednl
    build.build()
    return fednl


@pytest.mark.parametrize("path", LIBSVM, ids=os.path.basename)
def test_libsvm_loader_matches_reference(lib, path):
    z = np.load(path)
    txt = path.rsplit("_", 1)[0] + ".txt"
    x, y = lib.load_libsvm(txt, bool(int(z["add_intercept"])))
    np.testing.assert_array_equal(x, z["x"])
    np.testing.assert_array_equal(y, z["y"])


def test_libsvm_loader_errors(lib, tmp_path):
    with pytest.raises(lib.FedNLError):
        lib.load_libsvm(str(tmp_path / "missing.txt"))
    three = tmp_path / "three.txt"
    three.write_text("1 1:1\n2 1:1\n3 2:1\n")
    with pytest.raises(lib.FedNLError):
        lib.load_libsvm(str(three))
    bad = tmp_path / "bad.txt"
    bad.write_text("1 x:1\n-1 2:1\n")
    with pytest.raises(lib.FedNLError):
        lib.load_libsvm(str(bad))


def test_execute_local_argument_errors(lib, tmp_path):
    data = golden_path("libsvm_binary01.txt")
    base = (f"--train_dataset {data} --clients 2 --lambda 0.001 --rounds 3 --algorithm fednl1 "
            f"--k_compressor_as_d_mult 1 --alpha_step_size 1 --fednl-option-b --out {tmp_path}/t.bin")
    assert lib.execute_local("--lambda 0.1")[0] == -1                                   # no --out
    assert lib.execute_local(f"--out {tmp_path}/t.bin --train_dataset {tmp_path}/none.txt")[0] == -3
    assert lib.execute_local(base + " --compressor topk --debug forcesequpdate,bogus")[0] == -8
    assert lib.execute_local(base + " --compressor fancy")[0] == -2                     # unknown compressor
    assert lib.execute_local(base.replace("fednl1", "gd") + " --compressor topk")[0] == -2
    assert lib.execute_local(base.replace("--fednl-option-b", "") + " --compressor topk")[0] == -1
    assert lib.execute_local(base.replace("--rounds 3", "") + " --compressor topk")[0] == -1
    assert lib.execute_local(base.replace("--clients 2", "--clients 99") + " --compressor topk")[0] == -5
    assert lib.execute_local(base + " --compressor topk --gpu-arith-order sideways")[0] == -1


def test_reference_symbols_argument_errors(lib, tmp_path):
    """doptExecuteLocal / doptExecuteLocalPP under the reference's names: the same return codes as the
    reference's train() before any device work; the PP binary needs --clients-per-round in 1..clients."""
    data = golden_path("libsvm_binary01.txt")
    base = (f"--train_dataset {data} --clients 2 --lambda 0.001 --rounds 3 --algorithm fednl1 "
            f"--k_compressor_as_d_mult 1 --alpha_step_size 1 --fednl-option-b --compressor topk "
            f"--out {tmp_path}/t.bin")
    assert lib.dopt_execute_local("--lambda 0.1")[0] == -1
    assert lib.dopt_execute_local(base + " --debug bogus")[0] == -8
    assert lib.dopt_execute_local_pp(base)[0] == -1                                   # no --clients-per-round
    assert lib.dopt_execute_local_pp(base + " --clients-per-round 0")[0] == -1
    assert lib.dopt_execute_local_pp(base + " --clients-per-round 3")[0] == -1         # more than --clients
    assert lib.dopt_execute_local_pp(base + " --clients-per-round 1 --gpu-arith-order reference")[0] == -1
    assert lib.dopt_execute_local_pp(base.replace("topk", "fancy") + " --clients-per-round 1")[0] == -2


def _write_libsvm(path, prob):
    with open(path, "w") as f:
        for s in range(prob.total_samples):
            a = prob.features[s]
            items = " ".join(f"{i + 1}:{int(a[i])}" for i in range(prob.d) if a[i] != 0.0)
            f.write(f"{'+1' if prob.labels[s] > 0 else '-1'} {items}\n")


@pytest.mark.gpu
@pytest.mark.parametrize("extra,comp,k", [("--use_theoretical_alpha_option_2 --theoretical_alpha", "topk", 2),
                                          ("--alpha_step_size 1 --line_search --c_line_search 0.5 "
                                           "--gamma_line_search 0.5", "toplek", 2),
                                          ("--theoretical_alpha", "seqk", 1)])
def test_execute_local_matches_api_run(lib, tmp_path, extra, comp, k):
    """A whole bin_fednl_local command line: even split of the file's samples over 6 clients with
    the reference's reshuffle, intercept added by the loader, tracking file written; the callback
    and the tracked ||g|| / f must equal the same run made through the Python API."""
    prob = datagen.binary_problem(41, 16, [30] * 6, 0.3, 1e-3)       # last attribute = intercept
    body = datagen.Problem(prob.d - 1, prob.n_samples, prob.features[:, :-1], prob.labels, prob.lam)
    data = tmp_path / "data.txt"
    _write_libsvm(data, body)
    out = tmp_path / "track_{algorithm}_{dataset}.bin"
    cmd = (f"--train_dataset {data} --clients 6 --reshuffle_train --add_intercept --lambda 0.001 --rounds 12 "
           f"--workers 3 --algorithm fednl1 --compressor {comp} --k_compressor_as_d_mult {k} --fednl-option-b "
           f"--tracking --out {out} --debug forcesequpdate {extra}")
    rc, cbv = lib.execute_local(cmd)
    assert rc == 0 and cbv is not None
    # the same run through the Python API
    x, y = lib.load_libsvm(str(data), True)
    n = len(y)
    order = np.arange(n)
    st = np.uint32(123)
    nm = n - 1
    for i in range(n):                               # Shuffle.h:133-160 with RandomGenIntegerLinear
        st = np.uint32((int(st) * 214013 + 2531011) & 0xffffffff)
        u = float(st) * (1.0 / 4294967295.0)
        v = u * nm
        r = int(v) + (1 if v - int(v) > 0.5 else 0)
        if r:
            order[i], order[i + r] = order[i + r], order[i]
        nm -= 1
    per = n // 6
    sel = order[:per * 6]
    p2 = datagen.Problem(x.shape[1], np.full(6, per, dtype=np.int32), x[sel], y[sel], 1e-3)
    d = x.shape[1]
    U = d * (d + 1) // 2
    comp_api = {"topk": "topk", "toplek": "toplek", "seqk": "randseqk"}[comp]
    kk = int(k * d)
    alpha = 1.0 if comp != "seqk" else 1.0 / (U / kk - 1.0 + 1.0)
    opts = dict(track_f=True)
    if "line_search" in extra:
        opts["line_search"] = (0.5, 0.5, 5)
    fed = lib.FedNL(p2, comp_api, kk, alpha, workers=3, order="reference", **opts)
    gn, fs = [], []
    for _ in range(12):
        gn.append(fed.round())
        fs.append(fed.f())
    g = fed.grad()
    fed.close()
    g2 = float(np.dot(g, g))
    assert cbv[0] == d
    assert cbv[1] == pytest.approx(np.sqrt(g2), rel=1e-12, abs=1e-300)
    # the reference's own symbol gives the same callback values
    rc2, cbv2 = lib.dopt_execute_local(cmd)
    assert rc2 == 0 and cbv2 == cbv
    # tracking file: header then one record per round (TrainLoop.h:753-792, 1679-1691)
    raw = open(str(tmp_path / f"track_fednl1_data.bin"), "rb").read()
    parts = raw.split(b"\0", 3)
    assert parts[0] == b"data" and parts[1].startswith(b"FedNL") and parts[2] == comp.encode()
    rest = parts[3]
    hdr = struct.unpack("<6i4d", rest[:56])
    assert hdr[0] == per and hdr[2] == 12 and hdr[3] == 6 and hdr[4] == d and hdr[5] == kk
    recs = rest[56:]
    assert len(recs) == 12 * (4 + 6 * 8)
    for r in range(12):
        rec = struct.unpack("<i6d", recs[r * 52:(r + 1) * 52])
        assert rec[0] == r
        assert rec[1] == gn[r]
        assert rec[2] == fs[r]


@pytest.mark.gpu
def test_execute_local_pp_matches_api_run(lib, tmp_path):
    """doptExecuteLocalPP: bin_fednl_local_pp's command line (even split over 8 clients, 3 sampled per
    round by the reference's fixed-seed sampler, RandSeqK with the theoretical alpha); the callback
    receives the dimension and the tracked ||true gradient|| per round equals the same FedNL-PP run
    made through the Python API."""
    prob = datagen.binary_problem(43, 12, [20] * 8, 0.35, 1e-3)
    body = datagen.Problem(prob.d - 1, prob.n_samples, prob.features[:, :-1], prob.labels, prob.lam)
    data = tmp_path / "pp.txt"
    _write_libsvm(data, body)
    out = tmp_path / "pp_{algorithm}.bin"
    cmd = (f"--train_dataset {data} --clients 8 --clients-per-round 3 --add_intercept --lambda 0.001 "
           f"--rounds 10 --workers 2 --algorithm fednl1 --compressor seqk --k_compressor_as_d_mult 1 "
           f"--theoretical_alpha --fednl-option-b --tracking --out {out}")
    rc, d_cb = lib.dopt_execute_local_pp(cmd)
    assert rc == 0
    x, y = lib.load_libsvm(str(data), True)
    d = x.shape[1]
    assert d_cb == d
    n = len(y) // 8
    p2 = datagen.Problem(d, np.full(8, n, dtype=np.int32), x[:8 * n], y[:8 * n], 1e-3)
    U = d * (d + 1) // 2
    fed = lib.FedNL(p2, "randseqk", d, 1.0 / (U / d - 1.0 + 1.0), workers=2, clients_per_round=3)
    gn = [fed.round() for _ in range(10)]
    fed.close()
    raw = open(str(tmp_path / "pp_fednl1.bin"), "rb").read()
    parts = raw.split(b"\0", 3)
    assert parts[0] == b"pp" and parts[1].startswith(b"FedNL-PP") and parts[2] == b"seqk"
    recs = parts[3][56:]
    assert len(recs) == 10 * 52
    for r in range(10):
        rec = struct.unpack("<i6d", recs[r * 52:(r + 1) * 52])
        assert rec[0] == r and rec[1] == gn[r]


def _read_tracking(raw: bytes):
    """The tracking layout the engine writes (TrainLoop.h:753-792, 1679-1691): three NUL-terminated
    strings, six int32 and four doubles, then per round an int32 and six doubles."""
    parts = raw.split(b"\0", 3)
    rest = parts[3]
    ints = struct.unpack("<6i", rest[:24])
    dbl = struct.unpack("<4d", rest[24:56])
    recs = [struct.unpack("<i6d", rest[56 + 52 * r:56 + 52 * (r + 1)]) for r in range(ints[2])]
    return [p.decode() for p in parts[:3]], ints, dbl, recs


def test_tracking_file_read_by_reference_reader():
    """tests/golden/tracking_show.npz holds a tracking file written by the engine's driver and what the
    reference's own reader (experiments/show.py, run unchanged by make_tracking_golden.py) read from
    it: every header field and per-round value agrees with the engine's layout, bit for bit."""
    z = np.load(golden_path("tracking_show.npz"))
    strs, ints, dbl, recs = _read_tracking(z["raw"].tobytes())
    assert strs == [str(z["dataset"]), str(z["algorithm"]), str(z["compressor"])]
    assert list(ints) == list(z["ints"])
    np.testing.assert_array_equal(np.array(dbl), z["doubles"])
    n = len(recs)
    assert n == len(z["rounds"]) == ints[2]
    got = np.array([r[1:] for r in recs])
    np.testing.assert_array_equal([r[0] for r in recs], z["rounds"])
    np.testing.assert_array_equal(got[:, 0], z["grad_norm"])
    np.testing.assert_array_equal(got[:, 1], z["func_value"])          # show.py: f - f* with f* = 0
    np.testing.assert_array_equal(got[:, 2], z["x_norm"])
    nc = ints[3]
    np.testing.assert_array_equal((got[:, 3] * 8 / nc) + (got[:, 4] * 8 / nc), z["send_bits_total"])
    np.testing.assert_array_equal(got[:, 4] * 8 / nc, z["send_bits_indices"])
    np.testing.assert_array_equal(got[:, 5], z["elapsed"])


@pytest.mark.gpu
def test_tracking_file_matches_reference_reader_fixture(lib, tmp_path):
    """The driver run that made the fixture, again: the new file equals the fixture's bytes except the
    per-round wall-clock times, so the reference's reader reads the same values from it."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_tracking_golden", golden_path("make_tracking_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    data = tmp_path / "data.txt"
    mk.write_libsvm(data, mk.tracking_problem())
    out = tmp_path / "track_{algorithm}_{dataset}.bin"
    rc, _ = lib.execute_local(mk.COMMAND.format(data=data, out=out))
    assert rc == 0
    new = _read_tracking(open(tmp_path / "track_fednl1_data.bin", "rb").read())
    ref = _read_tracking(np.load(golden_path("tracking_show.npz"))["raw"].tobytes())
    assert new[0] == ref[0] and new[1] == ref[1] and new[2] == ref[2]
    for a, b in zip(new[3], ref[3]):
        assert a[:6] == b[:6]                    # all but the elapsed time
