"""The distributed client's wire format (fednl_gpu_encode_client_round) against the restatement in
oracle/pywire.py, whose framing is pinned to the reference's own dopt::MutableData
(tests/test_oracle_golden.py::test_wire_framing_matches_reference).  The per-client inputs (the
gradient, Lk, the differences, the selection) are the engine's, which the parity tests pin bit
for bit to the oracle; the bar here is byte equality of the whole round's packet stream."""
import numpy as np
import pytest

from oracle import pywire
from ufednl_gb300 import datagen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from ufednl_gb300 import build, fednl
    build.build()
    fednl.load()
    return fednl


CASES = [("topk", 723, 1.0), ("toplek", 723, 1.0), ("randk", 723, None), ("randseqk", 723, None),
         ("natural", None, 8 / 9), ("identity", None, 1.0)]


@pytest.mark.parametrize("comp,k,alpha", CASES, ids=[c[0] for c in CASES])
def test_client_round_bytes(gpu, comp, k, alpha):
    d = 40
    U = d * (d + 1) // 2
    prob = datagen.binary_problem(81, d, [50, 64, 41, 58, 47], 0.25, 1e-3)
    k = k or U
    alpha = alpha if alpha is not None else k / U
    fed = gpu.FedNL(prob, comp, k, alpha, workers=2, track_f=True)
    prescale = (1.0 / prob.n_clients) * alpha            # TrainLoop.h:717-719 of the distributed client
    for r in range(2):
        fed.round()
        for c in range(prob.n_clients):
            diff = fed.diff(c)
            idx, _ = fed.message(c)
            lda = fed.lda
            pos = [(int(t) // lda) * (int(t) // lda + 1) // 2 + int(t) % lda for t in idx]
            for flags in (0, pywire.WIRE_LK, pywire.WIRE_LK | pywire.WIRE_FINISH | pywire.WIRE_RANDK_INDICES):
                got = fed.encode_round(c, flags)
                want = pywire.encode_client_round(comp, fed.client_grad(c), fed.lk(c), 0.0, idx, diff[pos], diff,
                                                  prescale, U, k, flags)
                assert got == want, (comp, r, c, flags)
            # with f_i: the packet carries this client's objective; the master's f is their mean
            full = fed.encode_round(c, pywire.WIRE_LK | pywire.WIRE_FI)
            recs = pywire.decode(full)
            assert recs[-1][0] == pywire.SIG_FI and len(recs[-1][1]) == 8
    fis = [np.frombuffer(pywire.decode(fed.encode_round(c, pywire.WIRE_FI))[-1][1], "<f8")[0]
           for c in range(prob.n_clients)]
    assert np.isfinite(fis).all()
    fed.close()


def test_chunking_layout(gpu):
    """Chunk boundaries: 359 entries per chunk, the last chunk flagged, Natural's trailing pair."""
    d = 40
    U = d * (d + 1) // 2
    prob = datagen.binary_problem(82, d, [40, 52], 0.3, 1e-3)
    fed = gpu.FedNL(prob, "topk", 723, 1.0)
    fed.round()
    recs = pywire.decode(fed.encode_round(0, pywire.WIRE_LK))
    sigs = [s for s, _ in recs]
    assert sigs == [41, 47, 42, 44, 42, 44, 43, 45]
    assert [len(p) for s, p in recs if s in (42, 43)] == [359 * 4, 359 * 4, 5 * 4]
    assert [len(p) for s, p in recs if s in (44, 45)] == [359 * 8, 359 * 8, 5 * 8]
    fed.close()
    fed = gpu.FedNL(prob, "natural", U, 8 / 9)
    fed.round()
    recs = pywire.decode(fed.encode_round(1, 0))
    items = [p for s, p in recs if s in (44, 45)]
    assert [len(p) for p in items] == [537, 537, 3 * ((U - 2 * 358) // 2) + 3]
    fed.close()


def test_encoder_arguments(gpu):
    prob = datagen.binary_problem(83, 12, [20, 30], 0.3, 1e-3)
    fed = gpu.FedNL(prob, "topk", 24, 1.0)
    fed.round()
    with pytest.raises(gpu.FedNLError):
        fed.encode_round(0, pywire.WIRE_FI)          # no tracking: f_i is not formed
    with pytest.raises(gpu.FedNLError):
        fed.encode_round(0, 64)
    fed.close()
    fed = gpu.FedNL(prob, "randk_philox", 24, 24 / 78)
    fed.round()
    with pytest.raises(gpu.FedNLError):
        fed.encode_round(0, 0)                       # Philox positions must travel with the items
    assert len(fed.encode_round(0, pywire.WIRE_RANDK_INDICES)) > 0
    fed.close()
