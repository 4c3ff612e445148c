"""Full-size GPU checks at the benchmark configurations' sizes.

The bench's own workload (the 14-spin Heisenberg chain on 64 kets, through
qob_mul with the autotuned launch shape) is compared with the oracle on every
ket in ComplexF64 (1e-12), ComplexF32 (1e-5) and double-float (1e-12).  Beside
that, size-independent properties: linearity of the application, Hermiticity
of H (<a|H b> = conj(<b|H a>)), and conservation of the norm under RK4 time
evolution.  Tolerances are relative (l2) and written per assertion.
"""
import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import rel_l2
from qobgpu.hamiltonians import heisenberg_chain, jaynes_cummings, two_mode_cavity

pytestmark = pytest.mark.gpu


def test_heisenberg_16_spins_against_oracle():
    from qobgpu.mul import mul_, to_device

    H = heisenberg_chain(16, seed=9)  # dim 65536, 61 terms
    rng = Q.Rng(201)
    psi, out = Q.Ket(H.basis_r, rng.ket_data(len(H.basis_r))), Q.Ket(H.basis_l, rng.ket_data(len(H.basis_l)))
    ref = OR.mul(out, H, psi, 0.7 - 0.2j, 0.3)
    for dtype, tol in ((np.complex128, 1e-12), (np.complex64, 1e-5)):
        r = to_device(out, dtype=dtype)
        mul_(r, H, to_device(psi, dtype=dtype), 0.7 - 0.2j, 0.3)
        assert rel_l2(r.data.cpu().numpy().astype(np.complex128), ref) < tol


@pytest.mark.parametrize("form,tol", [("c128", 1e-12), ("c64", 1e-5), ("ff", 1e-12)])
def test_heisenberg_14_batch64_against_oracle(form, tol):
    """The bench step: mul!(Y, H, X, 0.7 - 0.2i, 0.3) with H =
    heisenberg_chain(14, seed=3) on 64 normalised complex-Gaussian kets, X and Y
    column-major 16384 x 64 with leading dimension 16384, the launch shape
    qob_op_tune picks for 64 kets, one qob_mul call; every ket against the
    oracle's mul! (src/operators_lazysum.jl:189-200), which gets the same
    ComplexF64 inputs."""
    import ctypes as C

    import torch

    from qobgpu import _lib as L
    from qobgpu.device import dtype_code, get_context, handle, raise_for

    H = heisenberg_chain(14, seed=3)
    dim, k = len(H.basis_l), 64
    rng = Q.Rng(2002)
    X = rng.kets_data(dim, k)
    X /= np.linalg.norm(X, axis=0, keepdims=True)
    Y = rng.kets_data(dim, k)
    alpha, beta = 0.7 - 0.2j, 0.3
    ref = np.asfortranarray(Y.copy())
    OR.mul_kets_threaded(OR.build_node(H), alpha, np.asfortranarray(X), beta, ref, 16)

    lib = L.lib()
    ctx = get_context(0)
    hd = handle(ctx, H)
    code = dtype_code("ff" if form == "ff" else (np.complex64 if form == "c64" else np.complex128))
    chosen = C.c_int()
    raise_for(lib.qob_op_tune(ctx.ptr, hd.ptr, L.QOB_LEFT, code, k, None, C.byref(chosen)), ctx)
    tdt = torch.complex64 if form == "c64" else torch.complex128
    # column-major dim x 64, ld = dim: the transpose of a contiguous 64 x dim tensor
    xd = torch.as_tensor(np.ascontiguousarray(X.T), device="cuda:0").to(tdt).t()
    yd = torch.as_tensor(np.ascontiguousarray(Y.T), device="cuda:0").to(tdt).t()
    stream = torch.cuda.current_stream(0)
    raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 0, hd.ptr, code, alpha.real, alpha.imag, C.c_void_p(xd.data_ptr()),
                          dim, k, dim, beta, 0.0, C.c_void_p(yd.data_ptr()), dim, k, dim,
                          C.c_void_p(stream.cuda_stream)), ctx)
    torch.cuda.synchronize(0)
    got = yd.cpu().numpy().astype(np.complex128)
    errs = [rel_l2(got[:, c], ref[:, c]) for c in range(k)]
    assert max(errs) < tol, (form, max(errs), chosen.value)
    assert rel_l2(got, ref) < tol


def test_heisenberg_14_batch64_linearity_and_hermiticity():
    import torch

    from qobgpu import operators as O
    from qobgpu.mul import mul_

    H = heisenberg_chain(14, seed=3)
    n, k = len(H.basis_l), 64
    g = torch.Generator(device="cuda:0")
    g.manual_seed(7)

    def cols():
        return torch.randn(k, n, dtype=torch.complex128, device="cuda:0", generator=g).t()

    a, b = 0.3 + 1.1j, -0.8 + 0.25j
    X1, X2 = cols(), cols()
    gb = Q.GenericBasis(k)

    def apply(X):
        Y = O.Operator(H.basis_l, gb, torch.zeros(k, n, dtype=torch.complex128, device="cuda:0").t())
        mul_(Y, H, O.Operator(H.basis_r, gb, X), 1.0, 0.0)
        return Y.data

    HX1, HX2 = apply(X1), apply(X2)
    Hcomb = apply((a * X1 + b * X2).t().contiguous().t())
    lin = torch.linalg.vector_norm(Hcomb - (a * HX1 + b * HX2)) / torch.linalg.vector_norm(Hcomb)
    assert lin.item() < 1e-13
    # <x1_c | H x2_c> == conj(<x2_c | H x1_c>) for every column c (H is Hermitian)
    lhs = (X1.conj() * HX2).sum(0)
    rhs = (X2.conj() * HX1).sum(0).conj()
    assert (torch.abs(lhs - rhs) / torch.abs(lhs)).max().item() < 1e-12


def test_all_256_cavities_in_one_batch():
    import torch

    from qobgpu.evolution import Batch

    rng = Q.Rng(40)
    b = Batch(np.complex128)
    refs, outs = [], []
    for k in range(256):
        n1, n2 = rng.integers(2, 8, 64)
        H = two_mode_cavity(int(n1), int(n2), seed=1000 + k)
        n = len(H.basis_l)
        x, y = rng.ket_data(n), rng.ket_data(n)
        refs.append(OR.mul(Q.Ket(H.basis_l, y), H, Q.Ket(H.basis_r, x), 0.7 - 0.2j, 0.3))
        yd = torch.as_tensor(y, device="cuda:0")
        b.add(H, torch.as_tensor(x, device="cuda:0"), yd, 0.7 - 0.2j, 0.3)
        outs.append(yd)
    b.run()
    torch.cuda.synchronize()
    assert b.info()["fused"] == 256
    worst = max(rel_l2(o.cpu().numpy(), r) for o, r in zip(outs, refs))
    assert worst < 1e-12


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-6)])
def test_rk4_renormalised_16_spins_and_jc8192(dtype, tol):
    """With renormalisation (FP64 norm, every step) the state stays on the unit
    sphere; RK4 alone loses norm as |R(i theta)|^2 = 1 - theta^6/72 + ..."""
    import torch

    from qobgpu.evolution import rk4

    for H in (heisenberg_chain(16, seed=12), jaynes_cummings(63, 63, seed=13)):
        psi = Q.Rng(14).ket_data(len(H.basis_l))
        d = torch.as_tensor(psi.astype(dtype), device="cuda:0")
        rk4(H, d, 1e-3, 100, renormalise=True)
        nrm = torch.linalg.vector_norm(d.to(torch.complex128)).item()
        assert abs(nrm - 1.0) < tol


def test_rk4_jc8192_against_host_rk4():
    import torch

    from qobgpu.evolution import rk4
    from test_gpu_evolution import rk4_host

    H = jaynes_cummings(63, 63, seed=13)
    psi = Q.Rng(15).ket_data(len(H.basis_l))
    d = torch.as_tensor(psi, device="cuda:0")
    rk4(H, d, 1e-3, 100)
    assert rel_l2(d.cpu().numpy(), rk4_host(H, psi, 1e-3, 100)) < 1e-12
