"""The index-pair gather (k_gather_j2: two consecutive output indices per
thread) against the oracle, through the C ABI.

Compact plans -- every merged group one run of power-of-two subsystems with one
stored entry per row, as spin chains compile -- applied in ComplexF64,
ComplexF32 or double-float to kets from the left can run with two output indices per thread
(qob_op_set_pairs, or a pair shape the autotuner picks): a group above bit 0
serves both indices with one slot lookup, the group on bit 0 index by index.
Each pair shape is checked against the oracle (the restated reference mul!) on
a real-valued chain (the bench's Hamiltonian family) and a lazy Liouvillian
(real entries with per-group factors of i and a complex diagonal), over 37 kets
(a ragged last ket set), with beta = 0.3 and with beta = 0 over a NaN-filled
output, at 1e-12 (ComplexF64 and double-float) and 1e-5 (ComplexF32).  Calls
the pair kernel cannot take run the one-index kernel: complex-valued plans,
ComplexF32 columns with an odd stride.  On the bench's own workload
the pair kernel agrees with the one-index kernel to rounding.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import rel_l2
from qobgpu.hamiltonians import heisenberg_chain
from test_gpu_tiles import complex_chain, liouvillian_5

pytestmark = pytest.mark.gpu

AL, BE = 0.7 - 0.2j, 0.3


def _apply(op, X, Y, form, alpha, beta, pairs=None, ld_pad=0):
    """qob_mul of op on the columns of X (dim x k, column-major, leading
    dimension dim + ld_pad); pairs = (kets per thread, threads, ket sets per
    warp) selects the pair kernel, None the one-index kernel (2 kets per
    thread, 256 threads)."""
    import torch

    from qobgpu import _lib as L
    from qobgpu.device import dtype_code, get_context, handle, raise_for

    lib = L.lib()
    ctx = get_context(0)
    hd = handle(ctx, op)
    code = dtype_code("ff" if form == "ff" else (np.complex64 if form == "c64" else np.complex128))
    if pairs is None:
        raise_for(lib.qob_op_set_launch(ctx.ptr, hd.ptr, L.QOB_LEFT, code, 2, 256, 1), ctx)
    else:
        raise_for(lib.qob_op_set_pairs(ctx.ptr, hd.ptr, L.QOB_LEFT, code, pairs[0], pairs[1], pairs[2]), ctx)
    tdt = torch.complex64 if form == "c64" else torch.complex128
    n, k = X.shape
    ld = n + ld_pad
    xd = torch.zeros(k, ld, dtype=tdt, device="cuda:0")
    yd = torch.zeros(k, ld, dtype=tdt, device="cuda:0")
    xd[:, :n] = torch.as_tensor(np.ascontiguousarray(X.T), device="cuda:0").to(tdt)
    yd[:, :n] = torch.as_tensor(np.ascontiguousarray(Y.T), device="cuda:0").to(tdt)
    raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 0, hd.ptr, code, alpha.real, alpha.imag, C.c_void_p(xd.data_ptr()),
                          n, k, ld, complex(beta).real, complex(beta).imag, C.c_void_p(yd.data_ptr()), n, k, ld,
                          C.c_void_p(torch.cuda.current_stream(0).cuda_stream)), ctx)
    torch.cuda.synchronize(0)
    flags = C.c_uint()
    raise_for(lib.qob_device_status(ctx.ptr, None, C.byref(flags)), ctx)
    assert flags.value == 0
    return yd[:, :n].t().cpu().numpy().astype(np.complex128)


def _oracle(op, X, Y, alpha, beta):
    ref = np.asfortranarray(Y.copy())
    OR.mul_kets_threaded(OR.build_node(op), alpha, np.asfortranarray(X), beta, ref, 8)
    return ref


@pytest.mark.parametrize("pairs", [(2, 256, 1), (4, 128, 1), (2, 256, 4), (4, 128, 8), (2, 128, 16)])
@pytest.mark.parametrize("which", ["real_chain", "liouvillian", "complex_chain"])
def test_pair_shapes_against_oracle(pairs, which):
    op = {"real_chain": lambda: heisenberg_chain(10, seed=6), "liouvillian": lambda: liouvillian_5(41),
          "complex_chain": lambda: complex_chain(9, 31)}[which]()
    n = len(op.basis_l)
    rng = Q.Rng(800 + pairs[0] * 16 + pairs[2])
    X = rng.kets_data(n, 37)
    Y = rng.kets_data(n, 37)
    for beta in (BE, 0.0):
        Yin = Y if beta != 0.0 else np.full_like(Y, np.nan)
        ref = _oracle(op, X, Yin if beta != 0.0 else np.zeros_like(Y), AL, beta)
        for form, tol in (("c128", 1e-12), ("c64", 1e-5), ("ff", 1e-12)):
            got = _apply(op, X, Yin, form, AL, beta, pairs)
            err = rel_l2(got, ref)
            assert err < tol, (which, pairs, form, beta, err)


def test_pairs_odd_stride_complexf32_runs_one_index_kernel():
    """ComplexF32 columns with an odd leading dimension are not 16-byte aligned
    pairwise: the call runs the one-index kernel, with the same result."""
    H = heisenberg_chain(9, seed=5)
    n = len(H.basis_l)
    rng = Q.Rng(830)
    X, Y = rng.kets_data(n, 12), rng.kets_data(n, 12)
    ref = _oracle(H, X, Y, AL, BE)
    for pad in (1, 2):
        got = _apply(H, X, Y, "c64", AL, BE, (2, 256, 1), ld_pad=pad)
        assert rel_l2(got, ref) < 1e-5, pad


@pytest.mark.parametrize("form,close", [("c128", 1e-15), ("c64", 1e-7), ("ff", 1e-15)])
def test_pairs_match_one_index_on_bench_workload(form, close):
    """heisenberg_chain(14, seed=3) on 64 kets: every pair shape the autotuner
    may pick agrees with the one-index kernel to rounding (the same operations
    in the same order per output; the compiler may contract a multiply and an
    add differently) and with the oracle at the form's tolerance."""
    H = heisenberg_chain(14, seed=3)
    n = len(H.basis_l)
    rng = Q.Rng(840)
    X = rng.kets_data(n, 64)
    Y = rng.kets_data(n, 64)
    base = _apply(H, X, Y, form, AL, BE)
    ref = _oracle(H, X, Y, AL, BE)
    tol = 1e-5 if form == "c64" else 1e-12
    for pairs in ((2, 256, 1), (4, 256, 1), (2, 128, 1), (4, 128, 1), (2, 256, 4), (4, 128, 4), (2, 128, 8),
                  (4, 128, 8), (2, 128, 16), (4, 128, 16)):
        got = _apply(H, X, Y, form, AL, BE, pairs)
        assert rel_l2(got, base) < close, (form, pairs, rel_l2(got, base))
        assert rel_l2(got, ref) < tol


def test_tune_reports_pair_shapes():
    """qob_op_tune_ex times the ten pair shapes for a compact plan on kets
    (times_ms[48:58]) and the chosen shape's result matches the oracle."""
    import torch

    from qobgpu import _lib as L
    from qobgpu.device import get_context, handle, raise_for

    H = heisenberg_chain(12, seed=8)
    lib = L.lib()
    ctx = get_context(0)
    hd = handle(ctx, H)
    times = (C.c_double * 58)()
    chosen = C.c_int()
    raise_for(lib.qob_op_tune_ex(ctx.ptr, hd.ptr, L.QOB_LEFT, L.QOB_C64, 64, times, 58, C.byref(chosen)), ctx)
    assert all(t > 0 for t in times[48:58])
    n = len(H.basis_l)
    rng = Q.Rng(850)
    X, Y = rng.kets_data(n, 64), rng.kets_data(n, 64)
    xd = torch.as_tensor(np.ascontiguousarray(X.T), device="cuda:0").to(torch.complex64).t()
    yd = torch.as_tensor(np.ascontiguousarray(Y.T), device="cuda:0").to(torch.complex64).t()
    raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 0, hd.ptr, L.QOB_C64, AL.real, AL.imag, C.c_void_p(xd.data_ptr()),
                          n, 64, n, BE, 0.0, C.c_void_p(yd.data_ptr()), n, 64, n, None), ctx)
    torch.cuda.synchronize(0)
    assert rel_l2(yd.cpu().numpy().astype(np.complex128), _oracle(H, X, Y, AL, BE)) < 1e-5
