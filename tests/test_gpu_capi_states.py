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
