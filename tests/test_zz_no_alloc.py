"""The allocation-free Option-B solve, called through the C ABI with device buffers the caller owns.

fednl_gpu_optionb_solve_noalloc serves callers that cannot allocate device memory: a host framework
that owns all device memory through its own allocator, a process under a fixed device-memory budget,
or a latency-critical loop in which cudaMalloc / cudaFree would synchronise the device.  Its scratch
is one fixed device array of the library, shared by every call.

Checked here: two calls in a row give exactly what the allocating entry point
fednl_gpu_optionb_solve gives (same kernel and operation order, so the tolerance is zero); the
device's free memory does not change during those calls; sizes above the array's maximum (d = 512)
are rejected with a clear error; a failed call's status does not leak into the next one.  The first
call on a device does a one-time set-up that can load the library's device code on that device and
so reserve the array; the checks therefore make one warm-up call before they measure free memory.
They run both in this test process (after the other tests, this file being collected last) and in a
fresh process of their own."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _spd(rng, d, lda):
    a = rng.standard_normal((d, d + 7)) / np.sqrt(d)
    h = a @ a.T
    full = np.zeros((d, lda))
    full[:, :d] = h.T               # column-major d x lda (symmetric)
    return full.reshape(-1)


def _noalloc(L, H, d, lda, l, g, dx, stream):
    return L.fednl_gpu_optionb_solve_noalloc(C.c_void_p(H.data_ptr()), d, lda, l, C.c_void_p(g.data_ptr()),
                                             C.c_void_p(dx.data_ptr()), C.c_void_p(stream))


def run_checks():
    """Warm-up call, then two calls in a row against the allocating entry point with the free device
    memory unchanged, then the size limit and the status reset.  Raises AssertionError on a failure."""
    import torch
    from ufednl_gb300 import fednl
    L = fednl.load()
    rng = np.random.default_rng(31)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    # one-time set-up of this device (address lookup, possibly the first load of the device code)
    Hw = torch.tensor(_spd(rng, 5, 8), device=dev, dtype=torch.float64)
    gw = torch.ones(5, device=dev, dtype=torch.float64)
    dxw = torch.zeros(5, device=dev, dtype=torch.float64)
    assert _noalloc(L, Hw, 5, 8, 0.1, gw, dxw, stream) == 0, L.fednl_gpu_last_error().decode()
    cases = [(301, 304, 7.3e-2), (77, 80, 1e-3)]           # two calls in a row, different sizes
    inputs = []
    for d, lda, l in cases:
        H = _spd(rng, d, lda)
        g = rng.standard_normal(d)
        ref = fednl.cholesky_option_b_solve(H, d, lda, l, g)   # allocating entry point, outside the window
        inputs.append((d, lda, l, ref, torch.tensor(H, device=dev, dtype=torch.float64),
                       torch.tensor(g, device=dev, dtype=torch.float64),
                       torch.full((d,), float("nan"), device=dev, dtype=torch.float64)))
    torch.cuda.synchronize(dev)
    for d, lda, l, ref, Hd, gd, dxd in inputs:
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc = _noalloc(L, Hd, d, lda, l, gd, dxd, stream)
        assert rc == 0, L.fednl_gpu_last_error().decode()
        free_after = torch.cuda.mem_get_info(dev)[0]
        assert free_after == free_before, (free_before, free_after)
        np.testing.assert_array_equal(dxd.cpu().numpy(), ref)
    # above the array's maximum: rejected before any device work
    d = 513
    Hd = torch.zeros(d * d, device=dev, dtype=torch.float64)
    gd = torch.zeros(d, device=dev, dtype=torch.float64)
    dxd = torch.zeros(d, device=dev, dtype=torch.float64)
    assert _noalloc(L, Hd, d, d, 0.0, gd, dxd, 0) == -1
    assert b"maximum" in L.fednl_gpu_last_error()
    # not positive definite, then a good system again: the shared status word was cleared
    bad = torch.tensor([1.0, 2.0, 2.0, 1.0], device=dev, dtype=torch.float64)
    assert _noalloc(L, bad, 2, 2, 0.0, torch.ones(2, device=dev, dtype=torch.float64),
                    torch.zeros(2, device=dev, dtype=torch.float64), 0) == -4
    H = _spd(rng, 9, 12)
    g = rng.standard_normal(9)
    dx9 = torch.zeros(9, device=dev, dtype=torch.float64)
    assert _noalloc(L, torch.tensor(H, device=dev, dtype=torch.float64), 9, 12, 0.5,
                    torch.tensor(g, device=dev, dtype=torch.float64), dx9, 0) == 0
    np.testing.assert_array_equal(dx9.cpu().numpy(), fednl.cholesky_option_b_solve(H, 9, 12, 0.5, g))


def test_optionb_solve_noalloc_in_this_process():
    pytest.importorskip("torch")
    run_checks()


def test_optionb_solve_noalloc_in_a_fresh_process():
    pytest.importorskip("torch")
    code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r); "
            "import test_zz_no_alloc as t; t.run_checks(); print('fresh process ok')" % (REPO, HERE))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "fresh process ok" in r.stdout, r.stdout[-2000:] + r.stderr[-4000:]
