"""CPU tests: the oracle (restated reference mul!) against dense materialisation.

These are the identities the reference's own tests check
(test/test_operators_lazytensor.jl:237-496, test/test_operators_lazysum.jl:255-347,
test/test_operators_sparse.jl:318-473, test/test_operators_lazyproduct.jl:170-245),
re-created on the project's seeded inputs: a lazy operator applied with mul!
equals its dense materialisation applied with numpy.
"""
import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import dense_of, rand_op, rand_state, rel_l2
from qobgpu import operators as O

A, B = 1.5 + 0j, 2.1 + 0j


def lazytensor_bases():
    b1a, b1b = Q.GenericBasis(2), Q.GenericBasis(3)
    b2a, b2b = Q.GenericBasis(1), Q.GenericBasis(4)
    b3a, b3b = Q.GenericBasis(6), Q.GenericBasis(5)
    return (b1a, b1b, b2a, b2b, b3a, b3b), Q.tensor_basis(b1a, b2a, b3a), Q.tensor_basis(b1b, b2b, b3b)


@pytest.mark.parametrize("sparse_factors", [False, True])
def test_lazytensor_gemv_mixed_precision_and_adjoints(sparse_factors):
    rng = Q.Rng(11)
    (b1a, b1b, b2a, b2b, b3a, b3b), bl, br = lazytensor_bases()
    s1 = rand_op(rng, b1a, b1b, np.complex64)
    s2 = O.dagger(rand_op(rng, b2b, b2a))
    s3 = O.dagger(rand_op(rng, b3b, b3a))
    facs = (s1, s2, s3)
    if sparse_factors:
        facs = tuple(O.sparse(f) for f in facs)
    op = O.LazyTensor(bl, br, (1, 2, 3), facs, 0.1)
    D = 0.1 * np.kron(np.kron(dense_of(s3), dense_of(s2)), dense_of(s1))
    psi = Q.Ket(br, rng.ket_data(len(br), np.complex64))
    out0 = rand_state(rng, bl)
    y = OR.mul(out0, op, psi, 1.0, 0.0)
    assert rel_l2(y, D @ psi.data) < 1e-6
    y = OR.mul(out0, op, psi, A, B)
    assert rel_l2(y, A * D @ psi.data + B * out0.data) < 1e-6
    # bra from the left
    bra = rand_state(rng, bl, Q.Bra)
    r0 = rand_state(rng, br, Q.Bra)
    y = OR.mul(r0, bra, op, A, B)
    assert rel_l2(y, A * bra.data @ D + B * r0.data) < 1e-13


@pytest.mark.parametrize("sparse_factors", [False, True])
def test_lazytensor_gemm_both_sides(sparse_factors):
    rng = Q.Rng(12)
    (b1a, b1b, b2a, b2b, b3a, b3b), bl, br = lazytensor_bases()
    facs = (rand_op(rng, b1a, b1b), rand_op(rng, b2a, b2b), O.sparse(rand_op(rng, b3a, b3b)))
    if sparse_factors:
        facs = tuple(O.sparse(f) for f in facs)
    op = O.LazyTensor(bl, br, (1, 2, 3), facs, 0.1)
    D = dense_of(op)
    b2 = Q.GenericBasis(13)
    st = rand_op(rng, br, b2)
    r0 = rand_op(rng, bl, b2)
    y = OR.mul(r0, op, st, A, B)
    assert rel_l2(y, A * D @ st.data + B * r0.data) < 1e-12
    bl2 = Q.GenericBasis(17)
    st = rand_op(rng, bl2, bl)
    r0 = rand_op(rng, bl2, br)
    y = OR.mul(r0, st, op, A, B)
    assert rel_l2(y, A * st.data @ D + B * r0.data) < 1e-12


def iso_bases():
    bl = Q.tensor_basis(Q.FockBasis(2), Q.GenericBasis(2), Q.SpinBasis("1/2"), Q.GenericBasis(1), Q.GenericBasis(2))
    br = Q.tensor_basis(Q.FockBasis(2), Q.GenericBasis(2), Q.SpinBasis("1/2"), Q.GenericBasis(2), Q.GenericBasis(1))
    return bl, br


def iso_ops():
    bl, br = iso_bases()
    iso = O.identityoperator(bl.bases[4], br.bases[4])
    n1 = O.LazyTensor(bl, br, (1, 3), (O.number(bl.bases[0]), O.sigmax(bl.bases[2])))
    n1_sp = O.LazyTensor(bl, br, (1, 2, 3, 5), (O.number(bl.bases[0]), O.identityoperator(bl.bases[1]),
                                                O.sigmax(bl.bases[2]), iso))
    n1_de = O.LazyTensor(bl, br, (1, 2, 3, 5), (O.dense(O.number(bl.bases[0])), O.identityoperator(bl.bases[1]),
                                                O.sigmax(bl.bases[2]), iso))
    return bl, br, n1, n1_sp, n1_de


def test_explicit_isometries():
    """test/test_operators_lazytensor.jl:446-496: pure-sparse, Eye-padded and
    dense-factor forms of the same isometry agree, incl. NaN-killing beta = 0."""
    rng = Q.Rng(13)
    bl, br, n1, n1_sp, n1_de = iso_ops()
    D = dense_of(n1)
    assert np.array_equal(D, dense_of(n1_sp)) and np.array_equal(D, dense_of(n1_de))
    state = rand_op(rng, br, br)
    out = rand_op(rng, bl, br)
    alpha, beta = rng.complex_normal(1)[0].real, rng.complex_normal(1)[0].real
    ref = alpha * D @ state.data + beta * out.data
    for op in (n1, n1_sp, n1_de):
        assert rel_l2(OR.mul(out, op, state, alpha, beta), ref) < 1e-12
    nan_out = O.Operator(bl, br, np.full(out.data.shape, np.nan + 0j, order="F"))
    for op in (n1, n1_sp, n1_de):
        y = OR.mul(nan_out, op, state, alpha, 0.0)
        assert rel_l2(y, alpha * D @ state.data) < 1e-12
        assert np.array_equal(OR.mul(out, op, state, 0.0, beta), beta * out.data)
        assert np.all(OR.mul(nan_out, op, state, 0.0, 0.0) == 0)
    state = rand_op(rng, bl, bl)
    for op in (n1, n1_sp, n1_de):
        assert rel_l2(OR.mul(out, state, op, alpha, beta), alpha * state.data @ D + beta * out.data) < 1e-12


def test_lazysum_gemv_gemm_and_empty():
    """test/test_operators_lazysum.jl:255-347."""
    rng = Q.Rng(14)
    (b1a, b1b, b2a, b2b, b3a, b3b), bl, br = lazytensor_bases()
    ops = tuple(rand_op(rng, bl, br) for _ in range(3))
    op = O.LazySum([0.1, 0.3, 1.2], ops)
    D = 0.1 * ops[0].data + 0.3 * ops[1].data + 1.2 * ops[2].data
    zero = O.LazySum(bl, br)
    psi = rand_state(rng, br)
    out = rand_state(rng, bl)
    assert rel_l2(OR.mul(out, op, psi, 1.0, 0.0), D @ psi.data) < 1e-13
    assert np.all(OR.mul(out, zero, psi, 1.0, 0.0) == 0)
    assert rel_l2(OR.mul(out, op, psi, A, B), A * D @ psi.data + B * out.data) < 1e-13
    assert rel_l2(OR.mul(out, zero, psi, A, B), B * out.data) < 1e-15
    st = rand_op(rng, br, br)
    res = O.Operator(bl, br, np.full((len(bl), len(br)), np.nan + 0j, order="F"))
    assert rel_l2(OR.mul(res, op, st, 1.0, 0.0), D @ st.data) < 1e-12


def sparse_case(rng, n, density):
    b = Q.GenericBasis(n)
    return b, O.sparse(rand_op(rng, b, b, density=density))


@pytest.mark.parametrize("n,density", [(20, 0.5), (60, 0.3)])  # nnz <= 550 and > 550 branches
def test_sparse_gemv_gemm(n, density):
    """test/test_operators_sparse.jl:318-437 (gemv, gemm small and big, adjoint)."""
    rng = Q.Rng(15)
    b, S = sparse_case(rng, n, density)
    D = dense_of(S)
    psi, out = rand_state(rng, b), rand_state(rng, b)
    assert rel_l2(OR.mul(out, S, psi, A, B), A * D @ psi.data + B * out.data) < 1e-13
    bra, rb = rand_state(rng, b, Q.Bra), rand_state(rng, b, Q.Bra)
    assert rel_l2(OR.mul(rb, bra, S, A, B), A * bra.data @ D + B * rb.data) < 1e-13
    st, ro = rand_op(rng, b, b), rand_op(rng, b, b)
    assert rel_l2(OR.mul(ro, S, st, A, B), A * D @ st.data + B * ro.data) < 1e-13
    assert rel_l2(OR.mul(ro, st, S, A, B), A * st.data @ D + B * ro.data) < 1e-13
    Sa = O.dagger(S)
    assert rel_l2(OR.mul(ro, Sa, st, A, B), A * D.conj().T @ st.data + B * ro.data) < 1e-13
    assert rel_l2(OR.mul(ro, st, Sa, A, B), A * st.data @ D.conj().T + B * ro.data) < 1e-13
    assert rel_l2(OR.mul(out, Sa, psi, A, B), A * D.conj().T @ psi.data + B * out.data) < 1e-13


@pytest.mark.parametrize("nops", [1, 2, 3])
def test_lazyproduct(nops):
    """test/test_operators_lazyproduct.jl:170-245."""
    rng = Q.Rng(16 + nops)
    bs = [Q.GenericBasis(k) for k in (3, 5, 4, 6)]
    ops = [rand_op(rng, bs[i], bs[i + 1]) for i in range(nops)]
    op = O.LazyProduct(tuple(ops), factor=0.5 - 0.1j)
    D = (0.5 - 0.1j) * np.linalg.multi_dot([o.data for o in ops] + [np.eye(len(bs[nops]))])
    psi, out = rand_state(rng, bs[nops]), rand_state(rng, bs[0])
    assert rel_l2(OR.mul(out, op, psi, A, B), A * D @ psi.data + B * out.data) < 1e-13
    bra, rb = rand_state(rng, bs[0], Q.Bra), rand_state(rng, bs[nops], Q.Bra)
    assert rel_l2(OR.mul(rb, bra, op, A, B), A * bra.data @ D + B * rb.data) < 1e-13
    assert np.array_equal(OR.mul(out, op, psi, 0.0, B), B * out.data)


def test_hamiltonians_against_dense():
    from qobgpu.hamiltonians import heisenberg_chain, jaynes_cummings, two_mode_cavity

    rng = Q.Rng(17)
    for H in (jaynes_cummings(15, 15), heisenberg_chain(8), two_mode_cavity(9, 12)):
        D = dense_of(H)
        psi, out = rand_state(rng, H.basis_r), rand_state(rng, H.basis_l)
        a, b = 0.7 - 0.2j, 0.3
        assert rel_l2(OR.mul(out, H, psi, a, b), a * D @ psi.data + b * out.data) < 1e-14
        rho = rand_op(rng, H.basis_r, H.basis_r)
        r0 = rand_op(rng, H.basis_l, H.basis_r)
        assert rel_l2(OR.mul(r0, H, rho, a, b), a * D @ rho.data + b * r0.data) < 1e-14
        assert rel_l2(OR.mul(r0, rho, H, a, b), a * rho.data @ D + b * r0.data) < 1e-14


def test_errors():
    rng = Q.Rng(18)
    b2, b3 = Q.GenericBasis(2), Q.GenericBasis(3)
    S = O.sparse(rand_op(rng, b2, b3))
    node = OR.build_node(S)
    with pytest.raises(OR.OracleError) as e:
        OR.mul_arrays(0, True, node, 1.0, np.zeros(2, complex), 0.0, np.zeros(2, complex))
    assert e.value.code == 1
    b = Q.tensor_basis(b2, b2)
    lt = O.LazyTensor(b, b, (1,), (O.sparse(rand_op(rng, b2, b2)),))
    n = OR.build_node(lt)
    x = np.ones(4, complex)
    rc = OR.lib().oref_mul(0, 1, n.ptr, 1.0, 0.0, OR._dp(x.view(np.float64)), 4, 1, 0.0, 0.0,
                           OR._dp(x.view(np.float64)), 4, 1)
    assert rc == 2  # aliasing ArgumentError (src/operators_lazytensor.jl:704-708)
