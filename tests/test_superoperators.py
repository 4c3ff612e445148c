"""Superoperators on the CPU: the construction identities of the reference's
test/test_superoperators.jl:160-230 on seeded inputs (host logic), the lazy
Liouvillian against the materialised one, and the oracle (restated mul!) on
the doubled-basis LazySum against the materialised matrix-vector product
(the reference's ``*(::SuperOperator, ::Operator)``, src/superoperators.jl:82-85).
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle as OR
import qobgpu as Q
from helpers import rand_op, rel_l2
from qobgpu import operators as O
from qobgpu import superoperators as S
from qobgpu.hamiltonians import heisenberg_chain, jaynes_cummings


def vec(a):
    return np.asarray(a).reshape(-1, order="F")


def unvec(v, n, m):
    return np.asarray(v).reshape(n, m, order="F")


def host_apply(s, rho: np.ndarray) -> np.ndarray:
    """S * rho with numpy (test-side check of the construction only)."""
    d = s.data
    v = d @ vec(rho)
    return unvec(v, len(s.basis_l[0]), len(s.basis_l[1]))


def dense_data(op):
    return np.asarray(O.dense(op).data)


@pytest.fixture
def ops():
    rng = Q.Rng(401)
    b = Q.tensor_basis(Q.SpinBasis("1/2"), Q.FockBasis(2))
    return b, rand_op(rng, b, b), rand_op(rng, b, b)


def test_spre_spost_sprepost_identities(ops):
    b, op1, op2 = ops
    a1, a2 = dense_data(op1), dense_data(op2)
    for conv in (lambda o: o, O.sparse):
        o1 = conv(op1)
        assert rel_l2(host_apply(S.spre(o1), a2), a1 @ a2) < 1e-14
        assert rel_l2(host_apply(S.spost(o1), a2), a2 @ a1) < 1e-14
        assert rel_l2(host_apply(S.spre(conv(O.dagger(op1))), a2), a1.conj().T @ a2) < 1e-14
        assert rel_l2(host_apply(S.sprepost(o1, op1), a2), a1 @ a2 @ a1) < 1e-14
    # sprepost(A, B) == spre(A) * spost(B)
    lhs = S.sprepost(op1, op2).data
    rhs = (S.spre(op1) * S.spost(op2)).data
    assert np.abs(np.asarray(lhs) - np.asarray(rhs)).max() < 1e-13
    # data layouts: kron(I, A), kron(transpose(A), I)
    n = len(b)
    assert np.array_equal(S.spre(op1).data, np.kron(np.eye(n), a1))
    assert np.array_equal(S.spost(op1).data, np.kron(a1.T, np.eye(n)))


def test_sparse_results_stay_sparse_and_equal(ops):
    b, op1, op2 = ops
    s = S.spre(O.sparse(op1))
    assert sp.issparse(s.data)
    assert S.dense(s) == S.DenseSuperOperator(s.basis_l, s.basis_r, s.data.toarray())


def test_non_square_sprepost_and_errors():
    b1, b2 = Q.FockBasis(1), Q.FockBasis(5)
    # op = |0><0| from b2 to b1: fockstate(b1, 0) (x) dagger(fockstate(b2, 0))
    d = np.zeros((len(b1), len(b2)), complex)
    d[0, 0] = 1.0
    op = O.Operator(b1, b2, np.asfortranarray(d))
    rho1 = np.zeros((len(b1), len(b1)), complex)
    rho1[0, 0] = 1.0
    rho2 = np.zeros((len(b2), len(b2)), complex)
    rho2[0, 0] = 1.0
    got = host_apply(S.sprepost(O.dagger(op), op), rho1)
    assert np.array_equal(got, rho2)
    with pytest.raises(O.ArgumentError):
        S.spre(op)
    with pytest.raises(O.ArgumentError):
        S.spost(op)


def _lindblad_direct(H, J, rates, rho):
    Hd = dense_data(H)
    out = -1j * (Hd @ rho - rho @ Hd)
    for r, j in zip(rates, J):
        jd = dense_data(j)
        jdj = jd.conj().T @ jd
        out = out + r * (jd @ rho @ jd.conj().T - 0.5 * jdj @ rho - 0.5 * rho @ jdj)
    return out


def _spin_model(nspins, seed):
    H = heisenberg_chain(nspins, seed=seed)
    bs = Q.SpinBasis("1/2")
    b = H.basis_l
    J = [O.LazyTensor(b, b, (i,), (O.sigmam(bs),)) for i in range(1, nspins + 1)]
    rates = Q.Rng(seed + 1).uniform(nspins, 0.1, 1.0)
    return H, J, rates


def test_liouvillian_matches_master_equation_and_rate_forms():
    H, J, rates = _spin_model(3, 402)
    Hs, Js = O.sparse(H), [O.sparse(j) for j in J]
    L = S.liouvillian(Hs, Js, rates=rates)
    rng = Q.Rng(403)
    n = len(H.basis_l)
    rho = rng.complex_normal(n * n).reshape(n, n, order="F")
    assert rel_l2(host_apply(L, rho), _lindblad_direct(H, J, rates, rho)) < 1e-13
    # a diagonal rate matrix gives the same superoperator
    Lm = S.liouvillian(Hs, Js, rates=np.diag(rates))
    assert np.abs((Lm.data - L.data).toarray()).max() < 1e-15
    with pytest.raises(AssertionError):
        S.liouvillian(Hs, Js, rates=np.zeros((4, 4)))
    # scalar arithmetic
    assert L / 2.0 == 0.5 * L == L * 0.5
    assert (-L) == S.SparseSuperOperator(L.basis_l, L.basis_r, -L.data)


def test_lazy_liouvillian_materialises_to_liouvillian():
    H, J, rates = _spin_model(4, 404)
    lazy = S.lazy_liouvillian(H, J, rates=rates)
    mat = S.liouvillian(O.sparse(H), [O.sparse(j) for j in J], rates=rates)
    assert np.abs((S.sparse(lazy).data - mat.data).toarray()).max() < 1e-14
    # non-diagonal rate matrix (collective decay channels)
    R = np.array([[0.5, 0.1j, 0, 0], [-0.1j, 0.4, 0, 0], [0, 0, 0.3, 0.05], [0, 0, 0.05, 0.2]])
    lazy = S.lazy_liouvillian(H, J, rates=R)
    mat = S.liouvillian(O.sparse(H), [O.sparse(j) for j in J], rates=R)
    assert np.abs((S.sparse(lazy).data - mat.data).toarray()).max() < 1e-14
    # Jaynes-Cummings with cavity decay (LazySum jump: a1 + a3, cross terms)
    Hj = jaynes_cummings(3, 4, seed=5)
    b = Hj.basis_l
    bf1, bf2 = b.bases[0], b.bases[2]
    Jj = [O.LazySum(b, b, [1.0, 0.5], (O.LazyTensor(b, b, (1,), (O.destroy(bf1),)),
                                       O.LazyTensor(b, b, (3,), (O.destroy(bf2),))))]
    lazy = S.lazy_liouvillian(Hj, Jj, rates=[0.7])
    mat = S.liouvillian(O.sparse(Hj), [O.sparse(j) for j in Jj], rates=[0.7])
    assert np.abs((S.sparse(lazy).data - mat.data).toarray()).max() < 1e-13


def test_lazy_liouvillian_single_site_fallback():
    """A full-space operator on a composite basis keeps the doubled basis at two sites."""
    H, J, rates = _spin_model(3, 405)
    Hs = O.sparse(H)  # full-space operator: no site-wise form
    lazy = S.lazy_liouvillian(Hs, J, rates=rates)
    assert len(lazy.operator.basis_l.bases) == 2
    mat = S.liouvillian(Hs, [O.sparse(j) for j in J], rates=rates)
    assert np.abs((S.sparse(lazy).data - mat.data).toarray()).max() < 1e-14


def test_oracle_on_doubled_basis_equals_materialised_product():
    """The restated reference mul! on the lazy form vs the materialised matrix-vector product."""
    H, J, rates = _spin_model(4, 406)
    lazy = S.lazy_liouvillian(H, J, rates=rates)
    mat = S.liouvillian(O.sparse(H), [O.sparse(j) for j in J], rates=rates)
    rng = Q.Rng(407)
    n = len(H.basis_l)
    rho = rng.complex_normal(n * n)
    out = rng.complex_normal(n * n)
    alpha, beta = 0.7 - 0.2j, 0.3
    v = lazy.vectorised
    got = OR.mul(Q.Ket(v.basis_l, out), v, Q.Ket(v.basis_r, rho), alpha, beta)
    ref_node = OR.build_node(mat.vectorised)
    ref = OR.mul_arrays(0, True, ref_node, alpha, rho, beta, out.copy())
    assert rel_l2(got, ref) < 1e-13
    assert rel_l2(ref, alpha * (mat.data @ rho) + beta * out) < 1e-14
