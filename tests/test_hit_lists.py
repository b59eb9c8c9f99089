"""The common-sample lists that both client-data uploads build for the binary Hessian's list kernel
(host code of the library, reached without a device through fednl_gpu_hit_lists), against a numpy
restatement of their format: for every client and upper position p = b (b + 1) / 2 + a, the samples
holding both attributes, in sample order, coded as none / one sample / a record of the 512-position
segment, with the diagonal and an intercept column coded apart (their entries come from attribute
sums).  Covers several segments, clients with and without an intercept column, empty rows, one-sample
clients, the size limits and bad rows."""
import numpy as np
import pytest

from ufednl_gb300 import datagen


@pytest.fixture(scope="module")
def lib():
    from ufednl_gb300 import build, fednl
    build.build()
    return fednl


def to_csr(a):
    rows = [np.nonzero(r == 1.0)[0] for r in a]
    rp = np.zeros(len(rows) + 1, np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    ci = np.concatenate(rows).astype(np.int32) if rp[-1] else np.zeros(0, np.int32)
    return rp, ci


def expected_lists(a, ns):
    S, d = a.shape
    U = d * (d + 1) // 2
    ustr = (U + 31) // 32 * 32
    nseg = (U + 511) // 512
    pb = np.repeat(np.arange(d), np.arange(1, d + 1))                 # b of each upper position
    pa = np.concatenate([np.arange(b + 1) for b in range(d)])        # a of each upper position
    off = np.concatenate([[0], np.cumsum(ns)])
    codes, segs, rec, hits = [], [], [], []
    maxrec = 1
    for c in range(len(ns)):
        ac = a[off[c]:off[c + 1]] == 1.0
        icpt = bool(ac[:, d - 1].all())
        code = np.full(ustr, 0x7FFF, np.uint16)
        seg = np.zeros(nseg + 1, np.uint32)
        for g in range(nseg):
            seg[g] = len(rec)
            for p in range(g * 512, min(U, g * 512 + 512)):
                ai, bi = int(pa[p]), int(pb[p])
                if ai == bi:
                    code[p] = 0xC000 | ai
                    continue
                if icpt and bi == d - 1:
                    code[p] = 0xA000 | ai
                    continue
                common = np.nonzero(ac[:, ai] & ac[:, bi])[0]
                if len(common) == 1:
                    code[p] = common[0]
                elif len(common) > 1:
                    code[p] = 0x8000 | (len(rec) - seg[g])
                    rec.append(len(hits))
                    hits.extend(common.tolist())
            maxrec = max(maxrec, len(rec) - int(seg[g]))
        seg[nseg] = len(rec)
        codes.append(code)
        segs.append(seg)
    rec.append(len(hits))
    return {"code": np.stack(codes), "seg": np.stack(segs), "rec": np.asarray(rec, np.uint32),
            "hits": np.asarray(hits, np.uint16), "maxrec": maxrec}


def skewed(seed, d, ns, intercept):
    rng = np.random.default_rng(seed)
    s = int(np.sum(ns))
    dens = np.where(np.arange(d - 1) < 6, 0.6, 0.06)
    a = (rng.random((s, d - 1)) < dens).astype(np.float64)
    last = np.ones((s, 1)) if intercept else (rng.random((s, 1)) < 0.3).astype(np.float64)
    return np.concatenate([a, last], axis=1)


def check(lib, a, ns):
    rp, ci = to_csr(a)
    got = lib.hit_lists(a.shape[1], ns, rp, ci)
    want = expected_lists(a, ns)
    np.testing.assert_array_equal(got["code"], want["code"])
    np.testing.assert_array_equal(got["seg"], want["seg"])
    np.testing.assert_array_equal(got["rec"], want["rec"])
    np.testing.assert_array_equal(got["hits"], want["hits"])
    assert got["maxrec"] == want["maxrec"]
    return want


@pytest.mark.parametrize("intercept", [True, False])
def test_lists_match_the_restatement(lib, intercept):
    ns = [70, 131, 64, 200, 97]
    want = check(lib, skewed(5, 57, ns, intercept), ns)        # U = 1653: four segments
    assert len(want["rec"]) > 100 and want["maxrec"] > 10


def test_empty_rows_and_one_sample_clients(lib):
    ns = [1, 40, 1, 33]
    a = skewed(9, 23, ns, True)
    a[3:9, :] = 0.0                         # rows with no attribute set: client 1 loses its intercept
    a[0, :] = 0.0                           # the one-sample client 0: no intercept, no pairs
    check(lib, a, ns)


def test_intercept_only_in_some_clients(lib):
    prob = datagen.binary_problem(31, 41, [50, 90, 64], 0.05, 1e-3)
    a = prob.features.copy()
    a[60, 40] = 0.0                         # client 1 (samples 50-139) without the intercept
    check(lib, a, [50, 90, 64])


def test_limits_and_bad_rows(lib):
    dense = datagen.binary_problem(12, 31, [600, 500], 0.5, 1e-3)       # ~100 pairs per sample
    rp, ci = to_csr(dense.features)
    with pytest.raises(lib.FedNLError, match="not built"):
        lib.hit_lists(31, [600, 500], rp, ci)
    rp = np.array([0, 2, 3], np.int32)
    with pytest.raises(lib.FedNLError, match="ascending"):
        lib.hit_lists(9, [2], rp, np.array([5, 3, 1], np.int32))
    with pytest.raises(lib.FedNLError, match="ascending"):
        lib.hit_lists(4, [2], rp, np.array([1, 3, 4], np.int32))      # column d
    with pytest.raises(lib.FedNLError, match="decreases"):
        lib.hit_lists(4, [2], np.array([0, 2, 1], np.int32), np.array([1, 3], np.int32))


def test_concurrent_callers(lib):
    """Calls from several host threads at once (ctypes releases the GIL; the library's worker pool
    takes one job at a time) give the same lists as a single call."""
    from concurrent.futures import ThreadPoolExecutor
    ns = [70, 131, 64, 200, 97]
    a = skewed(5, 57, ns, True)
    rp, ci = to_csr(a)
    ref = lib.hit_lists(57, ns, rp, ci)
    with ThreadPoolExecutor(6) as ex:
        outs = list(ex.map(lambda _: lib.hit_lists(57, ns, rp, ci), range(24)))
    for o in outs:
        for key in ("code", "seg", "rec", "hits"):
            np.testing.assert_array_equal(o[key], ref[key])
        assert o["maxrec"] == ref["maxrec"]
