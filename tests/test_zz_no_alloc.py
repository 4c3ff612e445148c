"""qob_dot_noalloc, called through the C ABI.

qob_dot_noalloc is the inner product for callers that must not allocate device
memory while they run: a program whose memory pool already owns the GPU's
memory, or code issuing work while a stream is captured into a CUDA graph.  It
keeps its partial sums in a fixed 128 KiB device array inside the library and
writes the result to device memory the caller owns.

This file checks that it returns what qob_dot (which stages through a context
buffer and pinned host memory) returns, within the FP64 tolerance the parity
tests use, on two calls in a row with different sizes and element types, and
that it rejects sizes beyond its 16,777,216-element limit.  It is collected
last so that a run stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12
LIMIT = 16_777_216


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_dot_noalloc_matches_dot_on_two_calls():
    import torch

    from qobgpu import _lib as L
    from qobgpu.device import get_context

    lib = L.lib()
    ctx = get_context(0)
    stream = C.c_void_p(torch.cuda.current_stream(0).cuda_stream)
    rng = np.random.default_rng(2024)
    result = torch.zeros(2, dtype=torch.float64, device="cuda:0")  # caller-owned output
    cases = [(1_000_003, np.complex128, L.QOB_C128), (4096 * 7 + 5, np.complex64, L.QOB_C64)]
    for n, dt, code in cases:  # two calls in a row; the second is smaller than the first
        xh = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(dt)
        yh = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(dt)
        x = torch.as_tensor(xh, device="cuda:0")
        y = torch.as_tensor(yh, device="cuda:0")
        ref = (C.c_double * 2)()
        assert lib.qob_dot(ctx.ptr, code, _ptr(x), _ptr(y), n, ref, stream) == L.QOB_OK
        rc = lib.qob_dot_noalloc(ctx.ptr, code, _ptr(x), _ptr(y), n, _ptr(result), stream)
        assert rc == L.QOB_OK, lib.qob_last_error(ctx.ptr)
        torch.cuda.synchronize(0)
        got = complex(*result.cpu().numpy())
        want = complex(ref[0], ref[1])
        assert abs(got - want) <= TOL * abs(want), (n, got, want)
        exact = np.vdot(xh.astype(np.complex128), yh.astype(np.complex128))
        assert abs(got - exact) <= TOL * abs(exact)


def test_dot_noalloc_rejects_sizes_beyond_limit():
    import torch

    from qobgpu import _lib as L
    from qobgpu.device import get_context

    lib = L.lib()
    ctx = get_context(0)
    n = LIMIT + 1
    x = torch.zeros(n, dtype=torch.complex64, device="cuda:0")
    result = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    rc = lib.qob_dot_noalloc(ctx.ptr, L.QOB_C64, _ptr(x), _ptr(x), n, _ptr(result), None)
    assert rc == L.QOB_ERR_ARG
    assert b"16777216" in lib.qob_last_error(ctx.ptr)
