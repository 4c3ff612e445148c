"""FFTOperator on the GPU (csrc/fft.cu: radix-2 Stockham FFT for power-of-two
axes, direct DFT otherwise) against the oracle's restated mul!
(src/particle.jl:438-535), and the Gaussian known answers of
test/test_particle.jl.  Tolerances: relative l2 1e-12 (ComplexF64), 1e-5 (ComplexF32)."""
import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import rel_l2
from qobgpu import operators as O
from qobgpu.bases import MomentumBasis, PositionBasis
from qobgpu.particle import gaussianstate, momentum, potentialoperator, transform

pytestmark = pytest.mark.gpu

AL, BE = 0.7 - 0.2j, 0.3 + 0.1j


def gpu(result, a, b, alpha, beta, dtype=np.complex128):
    from qobgpu.mul import mul_, to_device

    r = to_device(result, dtype=dtype)
    if isinstance(b, (Q.Ket,)) or (isinstance(b, O.Operator) and isinstance(b.data, np.ndarray)):
        b = to_device(b, dtype=dtype)
    else:
        a = to_device(a, dtype=dtype)
    mul_(r, a, b, alpha, beta)
    d = r.data
    return d.cpu().numpy().astype(np.complex128) if d.ndim == 1 else d.t().contiguous().cpu().numpy().T.astype(np.complex128)


@pytest.mark.parametrize("n", [200, 256, 4096])
@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-5)])
def test_four_forms(n, dtype, tol):
    bx = PositionBasis(-32.5, 20.1, n)
    bp = MomentumBasis(bx)
    rng = Q.Rng(720 + n)
    for T in (transform(bp, bx), transform(bx, bp)):
        x, y = rng.complex_normal(n), rng.complex_normal(n)
        ket = Q.Ket(T.basis_l, y)
        ref = OR.mul(ket, T, Q.Ket(T.basis_r, x), AL, BE)
        assert rel_l2(gpu(ket, T, Q.Ket(T.basis_r, x), AL, BE, dtype), ref) < tol
        ref0 = OR.mul(ket, T, Q.Ket(T.basis_r, x), AL, 0.0)
        assert rel_l2(gpu(ket, T, Q.Ket(T.basis_r, x), AL, 0.0, dtype), ref0) < tol
        bra = Q.Bra(T.basis_r, y)
        ref = OR.mul(bra, Q.Bra(T.basis_l, x), T, AL, BE)
        assert rel_l2(gpu(bra, Q.Bra(T.basis_l, x), T, AL, BE, dtype), ref) < tol
        g = Q.GenericBasis(7)
        A = O.Operator(T.basis_r, g, np.asfortranarray(rng.complex_normal(n * 7).reshape(n, 7, order="F")))
        Y = O.Operator(T.basis_l, g, np.asfortranarray(rng.complex_normal(n * 7).reshape(n, 7, order="F")))
        ref = OR.mul(Y, T, A, AL, BE)
        assert rel_l2(gpu(Y, T, A, AL, BE, dtype), ref) < tol
        A2 = O.Operator(g, T.basis_l, np.asfortranarray(rng.complex_normal(7 * n).reshape(7, n, order="F")))
        Y2 = O.Operator(g, T.basis_r, np.asfortranarray(rng.complex_normal(7 * n).reshape(7, n, order="F")))
        ref = OR.mul(Y2, A2, T, AL, BE)
        assert rel_l2(gpu(Y2, A2, T, AL, BE, dtype), ref) < tol


def test_gaussian_known_answer_on_device():
    bx = PositionBasis(-32.5, 20.1, 200)
    bp = MomentumBasis(bx)
    px, pp = gaussianstate(bx, 5.1, -3.2, 1.0), gaussianstate(bp, 5.1, -3.2, 1.0)
    got = gpu(Q.Ket(bp, np.zeros(200, complex)), transform(bp, bx), px, 1.0, 0.0)
    assert np.linalg.norm(got - pp.data) < 1e-12
    got = gpu(Q.Ket(bx, np.zeros(200, complex)), transform(bx, bp), pp, 1.0, 0.0)
    assert np.linalg.norm(got - px.data) < 1e-12


@pytest.mark.parametrize("shape", [(21, 18), (32, 64)])
def test_two_dimensional_grid(shape):
    bxs = [PositionBasis(-3.0 - i, 4.0 + i, n) for i, n in enumerate(shape)]
    bps = [MomentumBasis(b) for b in bxs]
    bX, bP = Q.tensor_basis(*bxs), Q.tensor_basis(*bps)
    rng = Q.Rng(730)
    n = len(bX)
    for T in (transform(bX, bP), transform(bP, bX)):
        x, y = rng.complex_normal(n), rng.complex_normal(n)
        ref = OR.mul(Q.Ket(T.basis_l, y), T, Q.Ket(T.basis_r, x), AL, BE)
        assert rel_l2(gpu(Q.Ket(T.basis_l, y), T, Q.Ket(T.basis_r, x), AL, BE), ref) < 1e-12
        bra_ref = OR.mul(Q.Bra(T.basis_r, y), Q.Bra(T.basis_l, x), T, AL, BE)
        assert rel_l2(gpu(Q.Bra(T.basis_r, y), Q.Bra(T.basis_l, x), T, AL, BE), bra_ref) < 1e-12


def test_particle_hamiltonian_lazy():
    """H = Txp * p^2/2 * Tpx + V(x) as LazySum(LazyProduct(FFT, diag, FFT), diag): the
    split-operator form of a particle Hamiltonian, applied in one call."""
    bx = PositionBasis(-10.0, 10.0, 512)
    bp = MomentumBasis(bx)
    Txp, Tpx = transform(bx, bp), transform(bp, bx)
    p = momentum(bp)
    p2 = O.Operator(bp, bp, (p.data @ p.data).tocsc() * 0.5)
    kin = O.LazyProduct((Txp, p2, Tpx))
    V = potentialoperator(bx, lambda x: 0.5 * x * x)
    H = O.LazySum(bx, bx, [1.0, 1.0], (kin, V))
    psi = gaussianstate(bx, 0.5, 0.3, 1.0)
    out = Q.Ket(bx, Q.Rng(740).complex_normal(512))
    ref = OR.mul(out, H, psi, AL, BE)
    assert rel_l2(gpu(out, H, psi, AL, BE), ref) < 1e-12
