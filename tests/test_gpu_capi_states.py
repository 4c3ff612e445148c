"""The C ABI's own device states (qob_state_*) and the one-shot batched apply
(qob_apply_batched), called directly through ctypes as a C caller would,
against the oracle.  Tolerance: relative l2 1e-12 (ComplexF64)."""
import ctypes as C

import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import rel_l2
from qobgpu import _lib as L
from qobgpu.device import get_context, handle, raise_for
from qobgpu.hamiltonians import heisenberg_chain, two_mode_cavity

pytestmark = pytest.mark.gpu

AL, BE = 0.7 - 0.2j, 0.3


def test_states_and_mul_without_torch_memory():
    lib = L.lib()
    ctx = get_context(0)
    H = heisenberg_chain(10, seed=41)
    h = handle(ctx, H)
    n, k = len(H.basis_l), 5
    rng = Q.Rng(800)
    x = np.asfortranarray(rng.complex_normal(n * k).reshape(n, k, order="F"))
    y = np.asfortranarray(rng.complex_normal(n * k).reshape(n, k, order="F"))
    dx, dy = C.c_void_p(), C.c_void_p()
    raise_for(lib.qob_state_alloc(ctx.ptr, L.QOB_C128, n, k, C.byref(dx)), ctx)
    raise_for(lib.qob_state_alloc(ctx.ptr, L.QOB_C128, n, k, C.byref(dy)), ctx)
    try:
        raise_for(lib.qob_state_upload(ctx.ptr, L.QOB_C128, dx, x.ctypes.data_as(C.c_void_p), n, k, None), ctx)
        raise_for(lib.qob_state_upload(ctx.ptr, L.QOB_C128, dy, y.ctypes.data_as(C.c_void_p), n, k, None), ctx)
        raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 0, h.ptr, L.QOB_C128, AL.real, AL.imag, dx, n, k, n, BE, 0.0, dy,
                              n, k, n, None), ctx)
        out = np.zeros((n, k), complex, order="F")
        raise_for(lib.qob_state_download(ctx.ptr, L.QOB_C128, dy, out.ctypes.data_as(C.c_void_p), n, k, None), ctx)
    finally:
        lib.qob_state_free(ctx.ptr, dx)
        lib.qob_state_free(ctx.ptr, dy)
    g = Q.GenericBasis(k)
    ref = OR.mul(Q.Operator(H.basis_l, g, y), H, Q.Operator(H.basis_r, g, x), AL, BE)
    assert rel_l2(out, ref) < 1e-12


def test_apply_batched_uneven_models():
    import torch

    lib = L.lib()
    ctx = get_context(0)
    rng = Q.Rng(801)
    models = [two_mode_cavity(int(a), int(b), seed=50 + i) for i, (a, b) in enumerate([(3, 5), (7, 2), (4, 4), (6, 6)])]
    xs, ys, refs, hs = [], [], [], []
    for H in models:
        n = len(H.basis_l)
        x, y = rng.ket_data(n), rng.ket_data(n)
        refs.append(OR.mul(Q.Ket(H.basis_l, y), H, Q.Ket(H.basis_r, x), AL, BE))
        xs.append(torch.as_tensor(x, device="cuda:0"))
        ys.append(torch.as_tensor(y, device="cuda:0"))
        hs.append(handle(ctx, H))
    m = len(models)
    ops = (C.c_void_p * m)(*[h.ptr for h in hs])
    xp = (C.c_void_p * m)(*[t.data_ptr() for t in xs])
    yp = (C.c_void_p * m)(*[t.data_ptr() for t in ys])
    al = (C.c_double * (2 * m))(*([AL.real, AL.imag] * m))
    be = (C.c_double * (2 * m))(*([BE, 0.0] * m))
    raise_for(lib.qob_apply_batched(ctx.ptr, L.QOB_C128, m, ops, xp, yp, al, be, None), ctx)
    for y, r in zip(ys, refs):
        assert rel_l2(y.cpu().numpy(), r) < 1e-12


def test_host_async_stream_of_batches():
    """A stream of host batches through qob_mul_host_async: kets from the left
    in chunks, a single ket, and bras from the right, more calls than staging
    sets and ticket slots in flight; pinned and pageable host memory; one wait
    on the last ticket covers every earlier call."""
    import torch

    lib = L.lib()
    ctx = get_context(0)
    H = heisenberg_chain(10, seed=43)
    h = handle(ctx, H)
    n = len(H.basis_l)
    rng = Q.Rng(802)
    calls = []
    for i in range(20):
        kind = ("kets", "kets", "ket", "bras")[i % 4]
        k = {"kets": 16 + i, "ket": 1, "bras": 3}[kind]
        shape = (n, k) if kind != "bras" else (k, n)
        pinned = i % 2 == 0

        def buf():
            a = rng.complex_normal(shape[0] * shape[1]).reshape(shape, order="F")
            if pinned:
                t = torch.empty(shape[1], shape[0], dtype=torch.complex128).pin_memory()
                v = t.numpy().T  # column-major view of page-locked memory
                v[...] = a
                return v, t
            return np.asfortranarray(a), None

        (x, kx), (y, ky) = buf(), buf()
        if kind == "bras":
            g = Q.GenericBasis(k)
            ref = OR.mul(Q.Operator(g, H.basis_r, y.copy()), Q.Operator(g, H.basis_l, x.copy()), H, AL, BE)
            side = L.QOB_RIGHT
        else:
            g = Q.GenericBasis(k)
            ref = OR.mul(Q.Operator(H.basis_l, g, y.copy()), H, Q.Operator(H.basis_r, g, x.copy()), AL, BE)
            side = L.QOB_LEFT
        t = C.c_uint64()
        raise_for(lib.qob_mul_host_async(ctx.ptr, side, int(kind == "ket"), h.ptr, L.QOB_C128, AL.real, AL.imag,
                                         x.ctypes.data_as(C.c_void_p), shape[0], shape[1], BE, 0.0,
                                         y.ctypes.data_as(C.c_void_p), shape[0], shape[1], C.byref(t)), ctx)
        calls.append((t.value, y, ref, kx, ky, x))
    tickets = [c[0] for c in calls]
    assert tickets == sorted(tickets) and len(set(tickets)) == len(tickets)
    raise_for(lib.qob_host_wait(ctx.ptr, tickets[-1]), ctx)
    for _, y, ref, *_ in calls:
        assert rel_l2(y, ref) < 1e-12
    # an early ticket whose event slot a later call recorded again still returns
    raise_for(lib.qob_host_wait(ctx.ptr, tickets[0]), ctx)
    raise_for(lib.qob_host_wait(ctx.ptr, 0), ctx)
    assert lib.qob_host_wait(ctx.ptr, tickets[-1] + 5) == L.QOB_ERR_ARG


def test_host_async_argument_errors_return_at_once():
    lib = L.lib()
    ctx = get_context(0)
    H = heisenberg_chain(6, seed=44)
    h = handle(ctx, H)
    n = len(H.basis_l)
    x = np.zeros((n + 1, 2), complex, order="F")
    y = np.zeros((n, 2), complex, order="F")
    t = C.c_uint64()
    rc = lib.qob_mul_host_async(ctx.ptr, L.QOB_LEFT, 0, h.ptr, L.QOB_C128, 1.0, 0.0, x.ctypes.data_as(C.c_void_p),
                                n + 1, 2, 0.0, 0.0, y.ctypes.data_as(C.c_void_p), n, 2, C.byref(t))
    assert rc == L.QOB_ERR_DIM
    z = np.zeros((n, 4), complex, order="F")
    rc = lib.qob_mul_host_async(ctx.ptr, L.QOB_LEFT, 0, h.ptr, L.QOB_C128, 1.0, 0.0, z.ctypes.data_as(C.c_void_p),
                                n, 2, 0.0, 0.0, z[:, 1:].ctypes.data_as(C.c_void_p), n, 2, C.byref(t))
    assert rc == L.QOB_ERR_ALIAS
