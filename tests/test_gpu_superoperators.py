"""Superoperator application on the GPU against the oracle.

The reference applies a superoperator as ``a.data * vec(rho)``
(src/superoperators.jl:82-85); the oracle restates that product (CSC gemv of
src/sparsematrix.jl) on the materialised Liouvillian.  The device applies both
the materialised form (sparse gather on vec(rho)) and the lazy doubled-basis
LazySum (fused gather).  Tolerances (relative l2): 1e-12 ComplexF64, 1e-5 ComplexF32.
"""
import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import rel_l2
from qobgpu import operators as O
from qobgpu import superoperators as S
from qobgpu.hamiltonians import heisenberg_chain, jaynes_cummings

pytestmark = pytest.mark.gpu

AL, BE = 0.7 - 0.2j, 0.3


def spin_model(nspins, seed):
    H = heisenberg_chain(nspins, seed=seed)
    bs = Q.SpinBasis("1/2")
    b = H.basis_l
    J = [O.LazyTensor(b, b, (i,), (O.sigmam(bs),)) for i in range(1, nspins + 1)]
    rates = Q.Rng(seed + 1).uniform(nspins, 0.1, 1.0)
    return H, J, rates


def oracle_apply(mat: S.SuperOperator, rho, out, alpha, beta):
    node = OR.build_node(mat.vectorised)
    return OR.mul_arrays(0, True, node, alpha, rho.reshape(-1, order="F"), beta, out.reshape(-1, order="F").copy())


def device_apply(s, rho, out, alpha, beta, dtype):
    import torch

    n = rho.shape[0]
    r = O.Operator(s.basis_r[0], s.basis_r[1], torch.as_tensor(rho.astype(dtype).T.copy(), device="cuda:0").t())
    y = O.Operator(s.basis_l[0], s.basis_l[1], torch.as_tensor(out.astype(dtype).T.copy(), device="cuda:0").t())
    S.mul_super(y, s, r, alpha, beta)
    return y.data.t().contiguous().cpu().numpy().T.reshape(-1, order="F").astype(np.complex128), n


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-5)])
@pytest.mark.parametrize("rates_kind", ["vector", "matrix"])
def test_lazy_and_materialised_liouvillian_heisenberg(dtype, tol, rates_kind):
    H, J, rates = spin_model(6, 501)
    if rates_kind == "matrix":
        R = np.diag(rates).astype(complex)
        R[0, 1], R[1, 0] = 0.1j, -0.1j
        rates = R
    lazy = S.lazy_liouvillian(H, J, rates=rates)
    mat = S.liouvillian(O.sparse(H), [O.sparse(j) for j in J], rates=rates)
    rng = Q.Rng(502)
    n = len(H.basis_l)
    rho = rng.complex_normal(n * n).reshape(n, n, order="F")
    out = rng.complex_normal(n * n).reshape(n, n, order="F")
    ref = oracle_apply(mat, rho, out, AL, BE)
    for s in (lazy, mat):
        got, _ = device_apply(s, rho, out, AL, BE, dtype)
        assert rel_l2(got, ref) < tol, type(s).__name__


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-5)])
def test_lazy_liouvillian_jaynes_cummings_cavity_decay(dtype, tol):
    Hj = jaynes_cummings(7, 7, seed=503)
    b = Hj.basis_l
    bf1, bs, bf2 = b.bases
    J = [O.LazyTensor(b, b, (1,), (O.destroy(bf1),)), O.LazyTensor(b, b, (3,), (O.destroy(bf2),)),
         O.LazyTensor(b, b, (2,), (O.sigmam(bs),))]
    lazy = S.lazy_liouvillian(Hj, J, rates=[0.3, 0.2, 0.1])
    mat = S.liouvillian(O.sparse(Hj), [O.sparse(j) for j in J], rates=[0.3, 0.2, 0.1])
    rng = Q.Rng(504)
    n = len(b)
    rho = rng.complex_normal(n * n).reshape(n, n, order="F")
    out = rng.complex_normal(n * n).reshape(n, n, order="F")
    ref = oracle_apply(mat, rho, out, 1.0, 0.0)
    got, _ = device_apply(lazy, rho, out, 1.0, 0.0, dtype)
    assert rel_l2(got, ref) < tol


def test_spre_spost_sprepost_on_device():
    rng = Q.Rng(505)
    b = Q.tensor_basis(Q.SpinBasis("1/2"), Q.FockBasis(3))
    n = len(b)
    a = O.Operator(b, b, np.asfortranarray(rng.complex_normal(n * n).reshape(n, n, order="F")))
    c = O.sparse(O.Operator(b, b, np.asfortranarray(rng.complex_normal(n * n).reshape(n, n, order="F"))))
    rho = rng.complex_normal(n * n).reshape(n, n, order="F")
    out = rng.complex_normal(n * n).reshape(n, n, order="F")
    for s in (S.spre(a), S.spost(a), S.sprepost(a, c), S.spre(c), S.spost(c)):
        ref = oracle_apply(s, rho, out, AL, BE)
        got, _ = device_apply(s, rho, out, AL, BE, np.complex128)
        assert rel_l2(got, ref) < 1e-12


def test_apply_allocating_with_host_data():
    """``S * rho`` with numpy data: copied to the device and back."""
    H, J, rates = spin_model(4, 506)
    lazy = S.lazy_liouvillian(H, J, rates=rates)
    mat = S.liouvillian(O.sparse(H), [O.sparse(j) for j in J], rates=rates)
    rng = Q.Rng(507)
    n = len(H.basis_l)
    rho = O.Operator(H.basis_l, H.basis_r, np.asfortranarray(rng.complex_normal(n * n).reshape(n, n, order="F")))
    ref = oracle_apply(mat, rho.data, np.zeros((n, n), complex), 1.0, 0.0)
    got = lazy * rho
    assert rel_l2(got.data.reshape(-1, order="F"), ref) < 1e-12
