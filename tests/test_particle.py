"""FFTOperator on the CPU: the oracle's restated mul! (src/particle.jl:438-535,
with FFTW's transforms restated as direct DFT sums) pinned to the reference's
test/test_particle.jl known answers (a Gaussian wave packet transformed between
position and momentum grids) and checked against numpy's FFT and dense
materialisation."""
import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from qobgpu import operators as O
from qobgpu.bases import MomentumBasis, PositionBasis, samplepoints, spacing
from qobgpu.particle import dagger, gaussianstate, tensor, transform

N, XMIN, XMAX = 200, -32.5, 20.1
X0, P0, SIGMA = 5.1, -3.2, 1.0


def bases(n=N):
    bx = PositionBasis(XMIN, XMAX, n)
    return bx, MomentumBasis(bx)


def dense_fft(T):
    """after .* W .* before as a matrix (numpy FFT of the identity's columns)."""
    n = len(T.basis_r)
    eye = np.eye(n, dtype=complex)
    W = np.fft.fft(eye, axis=0) if T.sign < 0 else np.fft.ifft(eye, axis=0) * n
    return (T.mul_after[:, None] * W) * T.mul_before[None, :]


def test_bases():
    bx, bp = bases()
    b2 = PositionBasis(bp)
    assert abs((bx.xmax - bx.xmin) - (b2.xmax - b2.xmin)) < 1e-12 and b2.N == bx.N
    assert spacing(bx) == (XMAX - XMIN) / N
    assert samplepoints(bx)[3] == XMIN + 3 * spacing(bx)


def test_gaussian_packet_known_answer():
    """Tpx * psi_x == psi_p and Txp * psi_p == psi_x to 1e-12 (test/test_particle.jl:99-126)."""
    bx, bp = bases()
    px, pp = gaussianstate(bx, X0, P0, SIGMA), gaussianstate(bp, X0, P0, SIGMA)
    assert abs(np.linalg.norm(px.data) - 1) < 1e-12 and abs(np.linalg.norm(pp.data) - 1) < 1e-12
    Tpx, Txp = transform(bp, bx), transform(bx, bp)
    got = OR.mul(Q.Ket(bp, np.zeros(N, complex)), Tpx, px)
    assert np.linalg.norm(got - pp.data) < 1e-12
    got = OR.mul(Q.Ket(bx, np.zeros(N, complex)), Txp, pp)
    assert np.linalg.norm(got - px.data) < 1e-12
    # mul!(psi_, Tpx, psi0_bx, 1, 1) on psi_ == psi0_bp
    got = OR.mul(Q.Ket(bp, pp.data.copy()), Tpx, px, 1.0, 1.0)
    assert np.linalg.norm(got - 2 * pp.data) < 1e-12


@pytest.mark.parametrize("n", [200, 256])
def test_all_forms_against_numpy(n):
    bx, bp = bases(n)
    rng = Q.Rng(700 + n)
    a, b = 0.7 - 0.2j, 0.3 + 0.1j
    for T in (transform(bp, bx), transform(bx, bp)):
        D = dense_fft(T)
        x = rng.complex_normal(n)
        y = rng.complex_normal(n)
        got = OR.mul(Q.Ket(T.basis_l, y), T, Q.Ket(T.basis_r, x), a, b)
        assert np.linalg.norm(got - (a * D @ x + b * y)) < 1e-12 * np.linalg.norm(got)
        got = OR.mul(Q.Bra(T.basis_r, y), Q.Bra(T.basis_l, x), T, a, b)
        assert np.linalg.norm(got - (a * x @ D + b * y)) < 1e-12 * np.linalg.norm(got)
        A = rng.complex_normal(n * 5).reshape(n, 5, order="F")
        Y = rng.complex_normal(n * 5).reshape(n, 5, order="F")
        g = Q.GenericBasis(5)
        got = OR.mul(O.Operator(T.basis_l, g, np.asfortranarray(Y)), T, O.Operator(T.basis_r, g, np.asfortranarray(A)), a, b)
        assert np.linalg.norm(got - (a * D @ A + b * Y)) < 1e-12 * np.linalg.norm(got)
        got = OR.mul(O.Operator(g, T.basis_r, np.asfortranarray(Y.T)), O.Operator(g, T.basis_l, np.asfortranarray(A.T)),
                     T, a, b)
        assert np.linalg.norm(got - (a * A.T @ D + b * Y.T)) < 1e-12 * np.linalg.norm(got)


def test_composite_transform_is_kron_of_axes_and_errors():
    bxs = [PositionBasis(-3.0, 4.0, 21), PositionBasis(-2.0, 5.0, 18)]
    bps = [MomentumBasis(b) for b in bxs]
    Txp = transform(Q.tensor_basis(*bxs), Q.tensor_basis(*bps))
    subs = [transform(bxs[i], bps[i]) for i in range(2)]
    D = np.kron(dense_fft(subs[1]), dense_fft(subs[0]))
    assert np.allclose(Txp.mul_before, np.kron(subs[1].mul_before, subs[0].mul_before))
    rng = Q.Rng(711)
    x = rng.complex_normal(21 * 18)
    got = OR.mul(Q.Ket(Txp.basis_l, np.zeros(21 * 18, complex)), Txp, Q.Ket(Txp.basis_r, x))
    assert np.linalg.norm(got - D @ x) < 1e-12 * np.linalg.norm(got)
    t2 = tensor(subs[0], subs[1])
    assert t2.axes == Txp.axes and np.allclose(t2.mul_after, Txp.mul_after)
    assert dagger(Txp).basis_l == Txp.basis_r
    with pytest.raises(AssertionError):
        transform(Q.tensor_basis(*bxs), Q.tensor_basis(*bxs))
    with pytest.raises(O.IncompatibleBases):
        transform(Q.tensor_basis(Q.SpinBasis("1/2"), Q.SpinBasis("1/2")),
                  Q.tensor_basis(Q.SpinBasis("1/2"), Q.SpinBasis("1/2")))
