"""The staged-tile gather (k_gather_t) against the oracle, through the C ABI.

Compact plans -- every merged group one run of power-of-two subsystems with one
stored entry per row, as spin chains compile -- applied to kets from the left
can run with their input tiles copied into shared memory (qob_op_set_tile, or a
tile shape the autotuner picks).  Each tile shape is checked against the oracle
(the restated reference mul!) on a real-valued chain (the bench's Hamiltonian
family), a complex-valued chain (sigma_x sigma_y and sigma_y sigma_z bonds with
complex coefficients) and a lazy Liouvillian (real entries with per-group
factors of i and a complex diagonal), over 37 kets (a ragged last block), with
beta = 0.3 and with beta = 0 over a NaN-filled output, in ComplexF64 (1e-12),
ComplexF32 (1e-5) and double-float (1e-12) arithmetic.  On the bench's own
workload the tiled result agrees with the untiled kernel's to rounding.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import rel_l2
from qobgpu import operators as O
from qobgpu.hamiltonians import heisenberg_chain

pytestmark = pytest.mark.gpu

AL, BE = 0.7 - 0.2j, 0.3
FORMS = (("c128", 1e-12), ("c64", 1e-5), ("ff", 1e-12))


def complex_chain(nspins, seed):
    """sum_i c_i sigma_x^i sigma_y^(i+1) + d_i sigma_y^i sigma_z^(i+1) + h_i sigma_z^i, complex c_i, d_i."""
    rng = Q.Rng(seed)
    bs = Q.SpinBasis("1/2")
    b = Q.tensor_basis(*([bs] * nspins))
    sx, sy, sz = O.sigmax(bs), O.sigmay(bs), O.sigmaz(bs)
    factors, ops = [], []
    for i in range(1, nspins):
        c = rng.complex_normal(2)
        factors += [complex(c[0]), complex(c[1])]
        ops += [O.LazyTensor(b, b, (i, i + 1), (sx, sy)), O.LazyTensor(b, b, (i, i + 1), (sy, sz))]
    for i in range(1, nspins + 1):
        factors.append(float(rng.uniform(1, -1, 1)[0]))
        ops.append(O.LazyTensor(b, b, (i,), (sz,)))
    return O.LazySum(b, b, factors, tuple(ops))


def liouvillian_5(seed):
    from qobgpu import superoperators as S

    H = heisenberg_chain(5, seed=seed)
    bs = Q.SpinBasis("1/2")
    b = H.basis_l
    J = [O.LazyTensor(b, b, (i,), (O.sigmam(bs),)) for i in range(1, 6)]
    return S.lazy_liouvillian(H, J, rates=Q.Rng(seed + 1).uniform(5, 0.1, 1.0)).vectorised


def _apply(op, X, Y, form, alpha, beta, tile=None):
    """qob_mul of op on the columns of X (dim x k, column-major), tiled when
    tile = (bits, kets per thread, ket sets per warp); returns Y's result."""
    import torch

    from qobgpu import _lib as L
    from qobgpu.device import dtype_code, get_context, handle, raise_for

    lib = L.lib()
    ctx = get_context(0)
    hd = handle(ctx, op)
    code = dtype_code("ff" if form == "ff" else (np.complex64 if form == "c64" else np.complex128))
    if tile is None:
        raise_for(lib.qob_op_set_launch(ctx.ptr, hd.ptr, L.QOB_LEFT, code, 1, 256, 1), ctx)
    else:
        raise_for(lib.qob_op_set_tile(ctx.ptr, hd.ptr, L.QOB_LEFT, code, tile[1], tile[2], tile[0]), ctx)
    tdt = torch.complex64 if form == "c64" else torch.complex128
    n, k = X.shape
    xd = torch.as_tensor(np.ascontiguousarray(X.T), device="cuda:0").to(tdt).t()
    yd = torch.as_tensor(np.ascontiguousarray(Y.T), device="cuda:0").to(tdt).t()
    raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 0, hd.ptr, code, alpha.real, alpha.imag, C.c_void_p(xd.data_ptr()),
                          n, k, n, complex(beta).real, complex(beta).imag, C.c_void_p(yd.data_ptr()), n, k, n,
                          C.c_void_p(torch.cuda.current_stream(0).cuda_stream)), ctx)
    torch.cuda.synchronize(0)
    flags = C.c_uint()
    raise_for(lib.qob_device_status(ctx.ptr, None, C.byref(flags)), ctx)
    assert flags.value == 0
    return yd.cpu().numpy().astype(np.complex128)


def _oracle(op, X, Y, alpha, beta):
    ref = np.asfortranarray(Y.copy())
    OR.mul_kets_threaded(OR.build_node(op), alpha, np.asfortranarray(X), beta, ref, 8)
    return ref


@pytest.mark.parametrize("tile", [(6, 1, 1), (7, 2, 1), (8, 4, 1), (9, 1, 4), (7, 2, 16), (6, 1, 32), (8, 2, 8)])
@pytest.mark.parametrize("which", ["real_chain", "complex_chain", "liouvillian"])
def test_tile_shapes_against_oracle(tile, which):
    op = {"real_chain": lambda: heisenberg_chain(10, seed=6), "complex_chain": lambda: complex_chain(9, 31),
          "liouvillian": lambda: liouvillian_5(41)}[which]()
    n = len(op.basis_l)
    rng = Q.Rng(700 + tile[0])
    X = rng.kets_data(n, 37)
    Y = rng.kets_data(n, 37)
    for beta in (BE, 0.0):
        Yin = Y if beta != 0.0 else np.full_like(Y, np.nan)
        ref = _oracle(op, X, Yin if beta != 0.0 else np.zeros_like(Y), AL, beta)
        for form, tol in FORMS:
            got = _apply(op, X, Yin, form, AL, beta, tile)
            err = rel_l2(got, ref)
            assert err < tol, (which, tile, form, beta, err)


@pytest.mark.parametrize("form,close", [("c128", 1e-15), ("c64", 1e-7), ("ff", 1e-15)])
def test_tile_matches_untiled_on_bench_workload(form, close):
    """heisenberg_chain(14, seed=3) on 64 kets: every staged-tile shape the
    autotuner may pick agrees with the untiled kernel to rounding (both do the
    same operations in the same order; the compiler may contract a multiply
    and an add into one FMA in one kernel and not in the other), and with the
    oracle at the form's tolerance."""
    H = heisenberg_chain(14, seed=3)
    n = len(H.basis_l)
    rng = Q.Rng(711)
    X = rng.kets_data(n, 64)
    Y = rng.kets_data(n, 64)
    base = _apply(H, X, Y, form, AL, BE)
    ref = _oracle(H, X, Y, AL, BE)
    tol = dict(FORMS)[form]
    for tile in ((10, 1, 1), (10, 2, 1), (9, 4, 1), (11, 1, 1), (12, 1, 1), (9, 1, 4), (8, 1, 16), (8, 2, 8),
                 (7, 2, 16)):
        got = _apply(H, X, Y, form, AL, BE, tile)
        assert rel_l2(got, base) < close, (form, tile, rel_l2(got, base))
        assert rel_l2(got, ref) < tol


def test_tune_considers_tiles_and_result_stays_exact():
    """qob_op_tune_ex reports the staged-tile shapes' times for a compact plan
    (48 times) and writes no more than the length it is given; whatever the
    tuner picks matches the oracle."""
    from qobgpu import _lib as L
    from qobgpu.device import get_context, handle, raise_for

    H = heisenberg_chain(12, seed=8)
    lib = L.lib()
    ctx = get_context(0)
    hd = handle(ctx, H)
    times = (C.c_double * 48)()
    chosen = C.c_int()
    raise_for(lib.qob_op_tune_ex(ctx.ptr, hd.ptr, L.QOB_LEFT, L.QOB_C64, 32, times, 48, C.byref(chosen)), ctx)
    assert sum(1 for t in times[36:] if t > 0) >= 10
    short = (C.c_double * 37)()  # a shorter array gets only its own length
    short[36] = 12345.0
    raise_for(lib.qob_op_tune_ex(ctx.ptr, hd.ptr, L.QOB_LEFT, L.QOB_C64, 32, short, 36, C.byref(chosen)), ctx)
    assert short[36] == 12345.0
    n = len(H.basis_l)
    rng = Q.Rng(712)
    X, Y = rng.kets_data(n, 32), rng.kets_data(n, 32)
    import torch

    xd = torch.as_tensor(np.ascontiguousarray(X.T), device="cuda:0").to(torch.complex64).t()
    yd = torch.as_tensor(np.ascontiguousarray(Y.T), device="cuda:0").to(torch.complex64).t()
    raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 0, hd.ptr, L.QOB_C64, AL.real, AL.imag, C.c_void_p(xd.data_ptr()),
                          n, 32, n, BE, 0.0, C.c_void_p(yd.data_ptr()), n, 32, n, None), ctx)
    torch.cuda.synchronize(0)
    assert rel_l2(yd.cpu().numpy().astype(np.complex128), _oracle(H, X, Y, AL, BE)) < 1e-5


@pytest.mark.parametrize("tile", [None, (10, 2, 1)])
def test_pdl_keeps_chained_applications_ordered(tile):
    """QOB_OPT_PDL: each application's blocks may be scheduled while the previous
    kernel finishes, and wait for it before touching memory.  A chain
    y1 = H x, y2 = H y1, y3 = H y2 recorded into a CUDA graph and replayed (each
    step reading the one before) equals the oracle's chain, and is bitwise
    equal to the same chain without PDL."""
    import torch

    from qobgpu import _lib as L
    from qobgpu.device import dtype_code, get_context, handle, raise_for

    H = heisenberg_chain(12, seed=9)
    n, k = len(H.basis_l), 16
    rng = Q.Rng(720)
    X = rng.kets_data(n, k)
    lib = L.lib()
    ctx = get_context(0)
    hd = handle(ctx, H)
    code = dtype_code(np.complex128)
    if tile:
        raise_for(lib.qob_op_set_tile(ctx.ptr, hd.ptr, L.QOB_LEFT, code, tile[1], tile[2], tile[0]), ctx)
    else:
        raise_for(lib.qob_op_set_launch(ctx.ptr, hd.ptr, L.QOB_LEFT, code, 2, 128, 1), ctx)
    ref = [np.asfortranarray(X)]
    for _ in range(3):
        ref.append(_oracle(H, ref[-1], np.zeros_like(X), 1.0, 0.0))
    outs = {}
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    for pdl in (0, 1):
        raise_for(lib.qob_set_option(ctx.ptr, L.QOB_OPT_PDL, pdl), ctx)
        bufs = [torch.as_tensor(np.ascontiguousarray(X.T), device="cuda:0").t()]
        bufs += [torch.zeros(k, n, dtype=torch.complex128, device="cuda:0").t() for _ in range(3)]

        def chain():
            for i in range(3):
                raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 0, hd.ptr, code, 1.0, 0.0, C.c_void_p(bufs[i].data_ptr()),
                                      n, k, n, 0.0, 0.0, C.c_void_p(bufs[i + 1].data_ptr()), n, k, n, sp), ctx)

        torch.cuda.synchronize()
        chain()  # direct launches
        stream.synchronize()
        g = C.c_void_p()
        raise_for(lib.qob_graph_begin(ctx.ptr, sp), ctx)
        chain()
        raise_for(lib.qob_graph_end(ctx.ptr, sp, C.byref(g)), ctx)
        for b in bufs[1:]:
            b.zero_()
        torch.cuda.synchronize()
        for _ in range(3):
            raise_for(lib.qob_graph_launch(ctx.ptr, g, sp), ctx)
        stream.synchronize()
        lib.qob_graph_free(ctx.ptr, g)
        outs[pdl] = [b.cpu().numpy() for b in bufs[1:]]
    raise_for(lib.qob_set_option(ctx.ptr, L.QOB_OPT_PDL, 0), ctx)
    for i in range(3):
        assert rel_l2(outs[1][i], ref[i + 1]) < 1e-12
        assert np.array_equal(outs[1][i], outs[0][i])
