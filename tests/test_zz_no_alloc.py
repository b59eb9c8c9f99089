"""The allocation-free Option-B solve, called through the C ABI with device buffers the caller owns.

Callers that cannot allocate device memory (a stream capture whose pool forbids new allocations,
latency-critical loops, hosts whose framework owns all device memory) use
fednl_gpu_optionb_solve_noalloc: its scratch is a fixed device array of the library.  Two calls in
a row must give exactly the result of the allocating entry point fednl_gpu_optionb_solve (same
kernel and operation order, so the tolerance is zero), the shared scratch must be reset between
calls, the device's free memory must not change during a call, and sizes beyond the array's
maximum (d = 512) must be rejected.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spd(rng, d, lda):
    a = rng.standard_normal((d, d + 7)) / np.sqrt(d)
    h = a @ a.T
    full = np.zeros((d, lda))
    full[:, :d] = h.T               # column-major d x lda (symmetric)
    return full.reshape(-1)


def test_optionb_solve_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from ufednl_gb300 import fednl
    L = fednl.load()
    rng = np.random.default_rng(31)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for d, lda, l in ((301, 304, 7.3e-2), (77, 80, 1e-3)):     # two calls in a row, different sizes
        H = _spd(rng, d, lda)
        g = rng.standard_normal(d)
        ref = fednl.cholesky_option_b_solve(H, d, lda, l, g)
        Hd = torch.tensor(H, device=dev, dtype=torch.float64)
        gd = torch.tensor(g, device=dev, dtype=torch.float64)
        dxd = torch.full((d,), float("nan"), device=dev, dtype=torch.float64)
        torch.cuda.synchronize(dev)
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc = L.fednl_gpu_optionb_solve_noalloc(C.c_void_p(Hd.data_ptr()), d, lda, l, C.c_void_p(gd.data_ptr()),
                                               C.c_void_p(dxd.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == 0, L.fednl_gpu_last_error().decode()
        free_after = torch.cuda.mem_get_info(dev)[0]
        np.testing.assert_array_equal(dxd.cpu().numpy(), ref)
        assert free_after == free_before


def test_optionb_solve_noalloc_rejects_oversize_and_not_pd():
    torch = pytest.importorskip("torch")
    from ufednl_gb300 import fednl
    L = fednl.load()
    dev = torch.device("cuda", 0)
    d = 513
    Hd = torch.zeros(d * d, device=dev, dtype=torch.float64)
    gd = torch.zeros(d, device=dev, dtype=torch.float64)
    dxd = torch.zeros(d, device=dev, dtype=torch.float64)
    rc = L.fednl_gpu_optionb_solve_noalloc(C.c_void_p(Hd.data_ptr()), d, d, 0.0, C.c_void_p(gd.data_ptr()),
                                           C.c_void_p(dxd.data_ptr()), None)
    assert rc == -1 and b"maximum" in L.fednl_gpu_last_error()
    bad = torch.tensor([1.0, 2.0, 2.0, 1.0], device=dev, dtype=torch.float64)
    g2 = torch.ones(2, device=dev, dtype=torch.float64)
    dx2 = torch.zeros(2, device=dev, dtype=torch.float64)
    rc = L.fednl_gpu_optionb_solve_noalloc(C.c_void_p(bad.data_ptr()), 2, 2, 0.0, C.c_void_p(g2.data_ptr()),
                                           C.c_void_p(dx2.data_ptr()), None)
    assert rc == -4
    # the scratch's status word is cleared by the next call: a positive-definite solve succeeds again
    rng = np.random.default_rng(5)
    H = _spd(rng, 9, 12)
    g = rng.standard_normal(9)
    Hd9 = torch.tensor(H, device=dev, dtype=torch.float64)
    gd9 = torch.tensor(g, device=dev, dtype=torch.float64)
    dx9 = torch.zeros(9, device=dev, dtype=torch.float64)
    rc = L.fednl_gpu_optionb_solve_noalloc(C.c_void_p(Hd9.data_ptr()), 9, 12, 0.5, C.c_void_p(gd9.data_ptr()),
                                           C.c_void_p(dx9.data_ptr()), None)
    assert rc == 0
    np.testing.assert_array_equal(dx9.cpu().numpy(), fednl.cholesky_option_b_solve(H, 9, 12, 0.5, g))
