"""LazyKet on the CPU: the oracle's restated expect(op, ::LazyKet)
(src/states_lazyket.jl:64-125) against numpy dense materialisation, on the
cases of the reference's test/test_states.jl:215-270 (seeded inputs), and the
LazyKet container's host logic."""
import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import rand_op
from qobgpu import operators as O
from qobgpu.lazyket import LazyKet, tensor
from qobgpu.states import basisstate


def dense_expect(op, kets):
    psi = LazyKet(Q.tensor_basis(*[k.basis for k in kets]), kets).to_ket().data
    D = np.asarray(O.dense(op).data)
    return complex(np.vdot(psi, D @ psi))


def rand_ket(rng, b):
    return Q.Ket(b, rng.ket_data(len(b)))


@pytest.fixture
def model():
    rng = Q.Rng(601)
    b1, b2, b3 = Q.GenericBasis(4), Q.FockBasis(5), Q.SpinBasis("1/2")
    b = Q.tensor_basis(b1, b2, b3)
    kets = [rand_ket(rng, x) for x in (b1, b2, b3)]
    ops = [rand_op(rng, x, x) for x in (b1, b2, b3)]
    c = complex(*rng.uniform(2))
    op = O.LazyTensor(b, b, (1, 2, 3), tuple(ops), c)
    return b, kets, ops, op, rng


def test_spin_product_state_sigmaz():
    b1, b2 = Q.SpinBasis("1/2"), Q.SpinBasis(1)
    b = Q.tensor_basis(b1, b2)
    psi1, psi2 = basisstate(b1, 2), basisstate(b2, 1)  # spindown(b1), spinup(b2)
    sz = O.LazyTensor(b, b, (1, 2), (O.sigmaz(b1), O.sigmaz(b2)))
    got = OR.expect_lazyket(sz, [psi1, psi2])
    assert got == dense_expect(O.tensor(O.sigmaz(b1), O.sigmaz(b2)), [psi1, psi2])


def test_lazytensor_sum_product_nested_and_missing_indices(model):
    b, kets, ops, op, rng = model
    assert abs(OR.expect_lazyket(op, kets) - dense_expect(op, kets)) < 1e-12 * abs(dense_expect(op, kets))
    f = complex(*rng.uniform(2))
    s = O.LazySum(b, b, [f, f], (op, op))
    assert abs(OR.expect_lazyket(s, kets) - 2 * f * OR.expect_lazyket(op, kets)) < 1e-12 * abs(OR.expect_lazyket(s, kets))
    g = complex(*rng.uniform(2))
    p = O.LazyProduct((op, op), factor=g)
    ref = g * complex(np.vdot(LazyKet(b, kets).to_ket().data,
                              np.linalg.matrix_power(np.asarray(O.dense(op).data), 2) @ LazyKet(b, kets).to_ket().data))
    assert abs(OR.expect_lazyket(p, kets) - ref) < 1e-12 * abs(ref)
    nested = O.LazySum(b, b, [0.3 - 0.1j, 1.7], (p, op))
    ref_n = (0.3 - 0.1j) * ref + 1.7 * dense_expect(op, kets)
    assert abs(OR.expect_lazyket(nested, kets) - ref_n) < 1e-12 * abs(ref_n)
    missing = O.LazyTensor(b, b, (1, 3), (ops[0], ops[2]), 0.4 + 0.2j)
    assert abs(OR.expect_lazyket(missing, kets) - dense_expect(missing, kets)) < 1e-12 * abs(dense_expect(missing, kets))


def test_lazyket_container():
    b1, b2 = Q.SpinBasis("1/2"), Q.SpinBasis(1)
    b = Q.tensor_basis(b1, b2)
    psi1, psi2 = basisstate(b1, 2), basisstate(b2, 1)
    psi = LazyKet(b, (psi1, psi2))
    assert tensor(psi, psi) == LazyKet(Q.tensor_basis(b, b), (psi1, psi2, psi1, psi2))
    assert np.array_equal(psi.to_ket().data, Q.tensor_states(psi1, psi2).data)
    with pytest.raises(AssertionError):
        LazyKet(b, (psi2, psi1))  # wrong subsystem bases
    with pytest.raises(AssertionError):
        LazyKet(b, (psi1,))
