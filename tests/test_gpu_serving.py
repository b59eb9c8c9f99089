"""The serving split of a round on the GPU: each problem's client phase on its own stream, then one
cooperative launch that solves the Option-B systems of all live problems (fednl_gpu_solve_batch).

Bar: every problem's iterates and ||g|| are the same bit for bit alone (fednl_gpu_run, its own
k_chol_coop launch with its own CTA count) and in the mix (any CTA share of the batched launch,
problems of different d, FP64 and mixed-precision handles together).  The Cholesky's arithmetic
is fixed per matrix entry (one FMA chain per entry, in column order), so the CTA count a problem
gets does not change its result."""
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


def _specs():
    """(kind, problem, compressor, k, alpha, options) of a mix of d and compressors."""
    out = []
    rng = np.random.default_rng(4)
    for t, (d, comp) in enumerate([(31, "topk"), (69, "toplek"), (124, "randk"), (301, "toplek"), (60, "natural"),
                                   (124, "topk"), (301, "randseqk"), (200, "identity")]):
        nc = int(rng.integers(3, 9))
        ns = [int(v) for v in rng.integers(20, 80, nc)]
        prob = datagen.binary_problem(100 + t, d, ns, 0.1 + 0.05 * t, 1e-3)
        U = d * (d + 1) // 2
        k = {"natural": U, "identity": U}.get(comp, 8 * d)
        alpha = {"randk": k / U, "randseqk": k / U, "natural": 8 / 9}.get(comp, 1.0)
        out.append(("fp64", prob, comp, k, alpha, {}))
    for t, (d, comp) in enumerate([(128, "randk_philox"), (256, "randk_philox"), (200, "topk"), (69, "toplek")]):
        prob = datagen.dense_problem_fp32(200 + t, d, [160, 96, 224], 1e-3)
        k = 4 * d if comp == "randk_philox" else 8 * d
        alpha = k / (d * (d + 1) // 2) if comp == "randk_philox" else 1.0
        out.append(("mixed", prob, comp, k, alpha, {}))
    return out


def _make(gpu, spec):
    kind, prob, comp, k, alpha, opts = spec
    if kind == "mixed":
        return gpu.MixedFedNL(prob, k, alpha, compressor=comp)
    return gpu.FedNL(prob, comp, k, alpha, workers=2, **opts)


def test_split_round_equals_round(gpu):
    prob = datagen.binary_problem(7, 69, [40, 55, 38, 61], 0.3, 1e-3)
    a = gpu.FedNL(prob, "toplek", 8 * 69, 1.0, workers=2)
    b = gpu.FedNL(prob, "toplek", 8 * 69, 1.0, workers=2)
    for r in range(8):
        ga = a.round()
        b.client_phase()
        gpu.solve_batch([b])
        gb = b.round_result()
        assert ga == gb, f"round {r}"
        np.testing.assert_array_equal(a.x(), b.x(), err_msg=f"round {r}")
    a.close()
    b.close()


def test_each_result_same_alone_and_in_the_mix(gpu):
    rounds = 6
    specs = _specs()
    alone = []
    for s in specs:
        p = _make(gpu, s)
        g = p.run(rounds)
        alone.append((g, p.x()))
        p.close()
    # the mix: eight copies of the d=301 problem as well, so that the batched launch has fewer CTAs
    # than the problems would take alone and every problem runs on a smaller share
    extra = [specs[3]] * 8
    live = [_make(gpu, s) for s in specs + extra]
    got = [[] for _ in live]
    for r in range(rounds):
        for p in live:
            p.client_phase()
        gpu.solve_batch(live)
        for i, p in enumerate(live):
            got[i].append(p.round_result())
    for i, p in enumerate(live):
        j = i if i < len(specs) else 3
        np.testing.assert_array_equal(np.array(got[i]), alone[j][0], err_msg=f"problem {i}: ||g||")
        np.testing.assert_array_equal(p.x(), alone[j][1], err_msg=f"problem {i}: x")
        p.close()


def test_more_problems_than_resident_ctas(gpu):
    """More live problems than the GPU holds CTAs: the batch is solved in successive launches."""
    prob = datagen.binary_problem(9, 12, [8, 10], 0.4, 1e-3)
    ref = gpu.FedNL(prob, "topk", 24, 1.0)
    g_ref = ref.run(3)
    x_ref = ref.x()
    ref.close()
    live = [gpu.FedNL(prob, "topk", 24, 1.0) for _ in range(170)]
    for r in range(3):
        for p in live:
            p.client_phase()
        gpu.solve_batch(live)
        for p in live:
            assert p.round_result() == g_ref[r]
    for p in live:
        np.testing.assert_array_equal(p.x(), x_ref)
        p.close()


def test_mem_info_and_split_round_argument_errors(gpu):
    free, total = gpu.mem_info()
    assert 0 < free <= total
    prob = datagen.binary_problem(3, 10, [7, 9, 8, 6], 0.4, 1e-3)
    pp = gpu.FedNL(prob, "natural", 55, 8 / 9, clients_per_round=2)
    with pytest.raises(gpu.FedNLError):
        pp.client_phase()
    pp.close()


def test_server_results_same_alone_and_in_the_mix(gpu):
    """The native serving loop (admission, client phases on per-problem streams, one batched solve
    per tick, retirement at the tolerance): every problem ends with the rounds, ||g|| and iterate it
    has alone, bit for bit, although problems join and leave the mix at different ticks."""
    from ufednl_gb300 import serving
    specs = _specs()
    tol, max_rounds = 1e-9, 12
    srv = serving.Server(reserve_bytes=1 << 30)
    ids = []
    for t, s in enumerate(specs):
        kind, prob, comp, k, alpha, opts = s
        prec = serving.PRECISION_MIXED if kind == "mixed" else serving.PRECISION_FP64
        ids.append((srv.submit_problem(prob, comp, k, alpha, precision=prec, tol=tol, max_rounds=max_rounds,
                                       seed_base=123), t))
        if t % 3 == 2:               # later arrivals join a running mix
            srv.tick()
    srv.run_until_idle()
    for pid, t in ids:
        st, x = srv.status(pid)
        assert st.state == serving.DONE, (t, st.state, st.error)
        kind, prob, comp, k, alpha, opts = specs[t]
        spec_w1 = (kind, prob, comp, k, alpha, {})
        rounds, g, x_alone = _alone_until_w1(gpu, spec_w1, tol, max_rounds)
        assert st.rounds == rounds, t
        assert st.grad_norm == g, t
        np.testing.assert_array_equal(x, x_alone, err_msg=f"problem {t}")
    lat = srv.latencies()
    assert len(lat) == sum(srv.status(pid)[0].rounds for pid, _ in ids)
    srv.close()


def _alone_until_w1(gpu, spec, tol, max_rounds):
    kind, prob, comp, k, alpha, opts = spec
    if kind == "mixed":
        p = gpu.MixedFedNL(prob, k, alpha, compressor=comp)
    else:
        p = gpu.FedNL(prob, comp, k, alpha, workers=1, feature_format=0)
    r = 0
    while True:
        g = p.run(1)[0]
        r += 1
        if g <= tol or r >= max_rounds:
            break
    x = p.x()
    p.close()
    return r, g, x


def test_server_refuses_what_never_fits(gpu):
    from ufednl_gb300 import serving
    prob = datagen.binary_problem(5, 40, [30, 25, 33], 0.3, 1e-3)
    srv = serving.Server(budget_bytes=1 << 16)          # 64 KB: smaller than any problem's state
    pid = srv.submit_problem(prob, "topk", 320, 1.0)
    s = srv.wait_settled(pid)                           # the admission thread refuses it
    st = srv.tick()
    assert st.live == 0 and st.pending == 0
    assert s.state == serving.FAILED and s.error == -2
    srv.close()
