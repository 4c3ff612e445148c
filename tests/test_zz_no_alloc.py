"""qob_dot_noalloc, called through the C ABI.

qob_dot_noalloc is the inner product for callers that must not allocate device
memory while they run: a program whose memory pool already owns the GPU's
memory, or code issuing work while a stream is captured into a CUDA graph.  It
keeps its partial sums in a fixed 128 KiB device array inside the library and
writes the result to device memory the caller owns.

This file checks that it returns what qob_dot (which stages through a context
buffer and pinned host memory) returns, within the FP64 tolerance the parity
tests use, on two calls in a row with different sizes and element types; at
the edges of its range (n = 0 writes 0 without reading x or y; n = 16,777,216
fills every partial slot of the array); that device memory in use does not
change across calls once the entry point has been called on the device; and
that it rejects sizes beyond its limit.  It is collected last so that a run
stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12
LIMIT = 16_777_216


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _setup():
    import torch

    from qobgpu import _lib as L
    from qobgpu.device import get_context

    lib = L.lib()
    ctx = get_context(0)
    stream = C.c_void_p(torch.cuda.current_stream(0).cuda_stream)
    return torch, L, lib, ctx, stream


def _dot(lib, L, ctx, code, x, y, n, stream):
    ref = (C.c_double * 2)()
    assert lib.qob_dot(ctx.ptr, code, _ptr(x), _ptr(y), n, ref, stream) == L.QOB_OK
    return complex(ref[0], ref[1])


def test_dot_noalloc_matches_dot_on_two_calls():
    torch, L, lib, ctx, stream = _setup()
    rng = np.random.default_rng(2024)
    result = torch.zeros(2, dtype=torch.float64, device="cuda:0")  # caller-owned output
    cases = [(1_000_003, np.complex128, L.QOB_C128), (4096 * 7 + 5, np.complex64, L.QOB_C64)]
    for n, dt, code in cases:  # two calls in a row; the second is smaller than the first
        xh = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(dt)
        yh = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(dt)
        x = torch.as_tensor(xh, device="cuda:0")
        y = torch.as_tensor(yh, device="cuda:0")
        want = _dot(lib, L, ctx, code, x, y, n, stream)
        rc = lib.qob_dot_noalloc(ctx.ptr, code, _ptr(x), _ptr(y), n, _ptr(result), stream)
        assert rc == L.QOB_OK, lib.qob_last_error(ctx.ptr)
        torch.cuda.synchronize(0)
        got = complex(*result.cpu().numpy())
        assert abs(got - want) <= TOL * abs(want), (n, got, want)
        exact = np.vdot(xh.astype(np.complex128), yh.astype(np.complex128))
        assert abs(got - exact) <= TOL * abs(exact)


def test_dot_noalloc_edges_of_its_range():
    """n = 0 (no partials: the final kernel alone writes 0, over a NaN-filled
    result) and n = 16,777,216 in ComplexF64 and ComplexF32 (all 8192 partial
    slots, the last one included), each against qob_dot."""
    torch, L, lib, ctx, stream = _setup()
    result = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda:0")
    x0 = torch.zeros(1, dtype=torch.complex128, device="cuda:0")
    assert lib.qob_dot_noalloc(ctx.ptr, L.QOB_C128, _ptr(x0), _ptr(x0), 0, _ptr(result), stream) == L.QOB_OK
    torch.cuda.synchronize(0)
    assert complex(*result.cpu().numpy()) == 0j
    g = torch.Generator(device="cuda:0")
    g.manual_seed(11)
    for tdt, code in ((torch.complex64, L.QOB_C64), (torch.complex128, L.QOB_C128)):
        x = torch.randn(LIMIT, dtype=tdt, device="cuda:0", generator=g)
        y = torch.randn(LIMIT, dtype=tdt, device="cuda:0", generator=g)
        y[-1] = 1e6  # the last element (last partial slot) carries weight
        want = _dot(lib, L, ctx, code, x, y, LIMIT, stream)
        rc = lib.qob_dot_noalloc(ctx.ptr, code, _ptr(x), _ptr(y), LIMIT, _ptr(result), stream)
        assert rc == L.QOB_OK, lib.qob_last_error(ctx.ptr)
        torch.cuda.synchronize(0)
        got = complex(*result.cpu().numpy())
        assert abs(got - want) <= TOL * abs(want), (tdt, got, want)
        del x, y


def test_dot_noalloc_holds_device_memory_steady():
    """Once the entry point has run on the device (the module is loaded and the
    array's address looked up), further calls leave the device's free memory
    unchanged (cudaMemGetInfo before and after)."""
    torch, L, lib, ctx, stream = _setup()
    n = 3_000_001
    x = torch.randn(n, dtype=torch.complex128, device="cuda:0")
    y = torch.randn(n, dtype=torch.complex128, device="cuda:0")
    result = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    assert lib.qob_dot_noalloc(ctx.ptr, L.QOB_C128, _ptr(x), _ptr(y), n, _ptr(result), stream) == L.QOB_OK
    torch.cuda.synchronize(0)
    free0, _ = torch.cuda.mem_get_info(0)
    for k in range(5):
        m = n - 100_000 * k
        assert lib.qob_dot_noalloc(ctx.ptr, L.QOB_C128, _ptr(x), _ptr(y), m, _ptr(result), stream) == L.QOB_OK
    torch.cuda.synchronize(0)
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)


def test_dot_noalloc_rejects_sizes_beyond_limit():
    torch, L, lib, ctx, _ = _setup()
    n = LIMIT + 1
    x = torch.zeros(n, dtype=torch.complex64, device="cuda:0")
    result = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    rc = lib.qob_dot_noalloc(ctx.ptr, L.QOB_C64, _ptr(x), _ptr(x), n, _ptr(result), None)
    assert rc == L.QOB_ERR_ARG
    assert b"16777216" in lib.qob_last_error(ctx.ptr)
