"""Host side of the serving loop, without a GPU: the request stream, admission footprints and the
native server's queue and argument handling (no device work is issued; with no device visible the
server admits nothing and its ticks are empty)."""
import numpy as np
import pytest

from ufednl_gb300 import datagen


@pytest.fixture(scope="module")
def serving():
    from ufednl_gb300 import build
    build.build()
    from ufednl_gb300 import serving as s
    return s


def test_stream_is_seeded_and_follows_its_distribution(serving):
    a = serving.draw_stream(2000, rate=200.0, seed=4)
    b = serving.draw_stream(2000, rate=200.0, seed=4)
    assert [(r.arrival_s, r.d, r.compressor) for r in a] == [(r.arrival_s, r.d, r.compressor) for r in b]
    t = np.array([r.arrival_s for r in a])
    assert np.all(np.diff(t) > 0)
    assert abs(np.mean(np.diff(t)) - 1 / 200) < 0.1 / 200           # Poisson process at 200/s
    assert {r.d for r in a} == {69, 124, 301, 1024}
    nc = np.array([r.n_clients for r in a])
    assert nc.min() >= 16 and nc.max() <= 512
    assert abs(np.median(np.log(nc)) - 0.5 * (np.log(16) + np.log(512))) < 0.2   # log-uniform
    ns = np.concatenate([r.n_samples for r in a[:50]])
    assert ns.min() >= 50 and ns.max() <= 2000
    assert {r.compressor for r in a} == {"topk", "randk", "toplek"}
    assert all(r.k == 8 * r.d for r in a)
    assert {r.lam for r in a} == {1e-3, 1e-4}
    assert {r.precision for r in a} == {serving.PRECISION_MIXED}


def test_make_data_shapes(serving):
    r = serving.Request(0, 0.0, 69, np.array([50, 60], dtype=np.int32), "bernoulli", 0.3, 1e-3, "topk", 552, 11,
                        engine=serving.PRECISION_FP64)
    f, y = serving.make_data(r)
    assert f.shape == (110, 69) and f.dtype == np.float64
    assert set(np.unique(f)) <= {0.0, 1.0} and np.all(f[:, -1] == 1.0)
    assert set(np.unique(y)) <= {-1.0, 1.0}
    r2 = serving.Request(1, 0.0, 128, np.array([50], dtype=np.int32), "normal", 0.3, 1e-3, "randk", 1024, 12)
    f2, _ = serving.make_data(r2)
    assert f2.shape == (50, 128) and f2.dtype == np.float32


def test_footprints(serving):
    reqs = serving.draw_stream(40, seed=4)
    for t, r in enumerate(reqs):
        r.engine = serving.PRECISION_FP64 if t % 2 else serving.PRECISION_MIXED
        b = serving.footprint(r)
        S, d = int(r.n_samples.sum()), r.d
        U = d * (d + 1) // 2
        if r.precision == serving.PRECISION_FP64:
            assert b >= 2 * r.n_clients * U * 8 + S * d * 8       # shifts + differences + data bound
        else:
            assert b >= r.n_clients * U * 4 + S * d * 4           # FP32 shifts + staged data
    small = serving.Request(0, 0.0, 69, np.array([50] * 16, dtype=np.int32), "bernoulli", 0.3, 1e-3, "topk", 552, 1)
    big = serving.Request(0, 0.0, 69, np.array([50] * 32, dtype=np.int32), "bernoulli", 0.3, 1e-3, "topk", 552, 1)
    assert serving.footprint(big) > serving.footprint(small)


def test_server_queue_and_argument_errors(serving):
    from ufednl_gb300 import fednl
    srv = serving.Server()
    prob = datagen.binary_problem(5, 12, [8, 9], 0.3, 1e-3)
    pid = srv.submit_problem(prob, "topk", 24, 1.0)
    st, x = srv.status(pid)
    assert st.state == serving.QUEUED and st.rounds == 0 and st.d == 12 and st.bytes > 0
    with pytest.raises(fednl.FedNLError):
        srv.submit_problem(prob, "topk", 24, 1.0, max_rounds=0)
    with pytest.raises(fednl.FedNLError):
        srv.submit_problem(prob, "topk", 24, 1.0, precision=7)
    with pytest.raises(fednl.FedNLError):         # the mixed engine runs TopK, TopLEK and RandK-Philox
        srv.submit_problem(prob, "natural", 78, 8 / 9, precision=serving.PRECISION_MIXED)
    pm = srv.submit_problem(prob, "toplek", 24, 1.0, precision=serving.PRECISION_MIXED)   # any d (padded)
    assert srv.status(pm)[0].state == serving.QUEUED
    assert len(srv.latencies()) == 0
    srv.close()
