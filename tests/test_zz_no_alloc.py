"""gev_sum_noalloc through the C-ABI against the allocating gev_field_sum.

gev_sum_noalloc is the field reduction for host codes that must not allocate
device memory while they run: their fields fill the GPU and its memory belongs
to their own pool (or to PyTorch's caching allocator), and a cudaMalloc /
cudaFree there can fail or synchronise the device in the middle of a queued time
step.  Its scratch is a static device array that every call shares, so the test
makes two calls in a row, the second over fewer values than the first: a call
that read partial sums the previous call left behind would be caught.

This file sorts last so that a run stopping at the first failure has run every
other test before it."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# same values, FP64 additions in a different order: agreement relative to sum |x|
TOL_SUM = 1e-13
MAX_N = 1 << 30  # GEV_SUM_NOALLOC_MAX_N


def _entry(gpu):
    f = gpu.lib().gev_sum_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_char_p, ctypes.c_size_t]
    return f


@pytest.mark.parametrize("prec", [0, 1])
def test_sum_noalloc_matches_field_sum_two_calls(gpu, prec):
    import torch

    entry = _entry(gpu)
    err = ctypes.create_string_buffer(256)
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda:0")
    rng = np.random.default_rng(11 + prec)
    # first call: one component of a 96^3 field (108 whole chunks of 8192 values); second: a
    # 48^3 field (14 chunks, the last one partial); third: a 24^3 field (2 chunks, one partial)
    for N, ncomp, comp in ((96, 3, 2), (48, 1, 0), (24, 1, 0)):
        ctx = gpu.Context(N, prec)
        x = 0.25 + rng.standard_normal((ncomp, N, N, N))
        f = ctx.real(ncomp).upload(x)
        want = f.sum(comp)
        ptr, nbytes = f.device_ptr()
        esize = 8 if prec == 0 else 4
        n = N ** 3
        assert nbytes == ncomp * n * esize
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = entry(0, ptr + comp * n * esize, prec, n, out.data_ptr(), ctx.stream(), err, len(err))
        assert rc == 0, err.value.decode()
        ctx.sync()
        got = out.item()
        scale = float(np.abs(x[comp]).sum())
        assert abs(got - want) <= TOL_SUM * scale, (N, got, want)
        # the stored values (FP32 in the mixed form) summed exactly in FP64 on the host
        stored = x[comp].astype(np.float32).astype(np.float64) if prec == 1 else x[comp]
        assert abs(got - float(np.sum(stored))) <= TOL_SUM * scale


def test_sum_noalloc_edges(gpu):
    import torch

    entry = _entry(gpu)
    err = ctypes.create_string_buffer(256)
    ctx = gpu.Context(16, 1)
    f = ctx.real(1).upload(np.ones((1, 16, 16, 16)))
    ptr, _ = f.device_ptr()
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    # n = 0 sums nothing and writes 0
    assert entry(0, None, 1, 0, out.data_ptr(), ctx.stream(), err, len(err)) == 0
    ctx.sync()
    assert out.item() == 0.0
    # one value past the limit is refused before any work is enqueued
    assert entry(0, ptr, 1, MAX_N + 1, out.data_ptr(), ctx.stream(), err, len(err)) == -1
    assert b"exceeds" in err.value
    # a partial chunk: 4096 ones plus the first 100 again
    assert entry(0, ptr, 1, 4096, out.data_ptr(), ctx.stream(), err, len(err)) == 0
    ctx.sync()
    assert out.item() == 4096.0
    assert entry(0, ptr, 1, 100, out.data_ptr(), ctx.stream(), err, len(err)) == 0
    ctx.sync()
    assert out.item() == 100.0
    # many chunks and a ragged last one: the first 96^3 - 777 values of a 96^3 field
    N = 96
    ctx2 = gpu.Context(N, 0)
    x = np.random.default_rng(5).standard_normal((1, N, N, N))
    f2 = ctx2.real(1).upload(x)
    ptr2, _ = f2.device_ptr()
    n = N ** 3 - 777
    assert entry(0, ptr2, 0, n, out.data_ptr(), ctx2.stream(), err, len(err)) == 0
    ctx2.sync()
    flat = x.reshape(-1)[:n]
    assert abs(out.item() - float(np.sum(flat))) <= TOL_SUM * float(np.abs(flat).sum())
