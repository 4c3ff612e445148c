"""LazyKet on the GPU (qob_expect_lazyket, site-wise mul!) against the oracle's
restated expect(op, ::LazyKet) (src/states_lazyket.jl:64-125).
Tolerances: relative 1e-12 (ComplexF64 states), 1e-5 (ComplexF32 states)."""
import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import rand_op
from qobgpu import operators as O
from qobgpu import lazyket as LK
from qobgpu.hamiltonians import heisenberg_chain
from qobgpu.states import basisstate

pytestmark = pytest.mark.gpu


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture
def model():
    rng = Q.Rng(611)
    b1, b2, b3 = Q.GenericBasis(4), Q.FockBasis(5), Q.SpinBasis("1/2")
    b = Q.tensor_basis(b1, b2, b3)
    kets = [Q.Ket(x, rng.ket_data(len(x))) for x in (b1, b2, b3)]
    ops = [rand_op(rng, x, x) for x in (b1, b2, b3)]
    op = O.LazyTensor(b, b, (1, 2, 3), tuple(ops), 0.6 + 0.3j)
    return b, kets, ops, op


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-5)])
def test_expect_forms(model, dtype, tol):
    b, kets, ops, op = model
    ks = [Q.Ket(k.basis, k.data.astype(dtype)) for k in kets]
    psi = LK.LazyKet(b, ks)
    forms = [
        op,
        O.LazySum(b, b, [0.2 + 0.1j, -1.3], (op, op)),
        O.LazyProduct((op, op), factor=0.7 - 0.4j),
        O.LazySum(b, b, [0.3 - 0.1j, 1.7], (O.LazyProduct((op, op), factor=0.5), op)),
        O.LazyTensor(b, b, (1, 3), (ops[0], O.sparse(ops[2])), 0.4 + 0.2j),
        O.LazyTensor(b, b, (2,), (O.dagger(ops[1]),)),
    ]
    oracle_kets = [Q.Ket(k.basis, k.data.astype(dtype).astype(np.complex128)) for k in kets]
    for f in forms:
        ref = OR.expect_lazyket(f, oracle_kets)
        assert rel(LK.expect(f, psi), ref) < tol, f


def test_expect_batch_many_product_states():
    """4096 product states of a 12-spin chain in one launch, against the oracle per state."""
    import torch

    H = heisenberg_chain(12, seed=31)
    b = H.basis_l
    rng = Q.Rng(612)
    n = 4096
    states = rng.complex_normal(n * 24).reshape(n, 24)
    res = LK.expect_batch(H, b, torch.as_tensor(states, device="cuda:0")).cpu().numpy()
    for s in range(0, n, 257):
        kets = [states[s, 2 * i:2 * i + 2] for i in range(12)]
        ref = OR.expect_lazyket(H, kets)
        assert rel(res[s], ref) < 1e-12


def test_norm_normalize_and_mul(model):
    b, kets, ops, op = model
    psi = LK.LazyKet(b, [Q.Ket(k.basis, k.data.copy()) for k in kets])
    assert rel(LK.norm(psi), np.prod([np.linalg.norm(k.data) for k in kets])) < 1e-14
    nrm = LK.normalize(psi)
    assert abs(LK.norm(nrm) - 1.0) < 1e-14
    # mul!(y::LazyKet, op::LazyTensor, x::LazyKet): Ket(y) == dense(op) * Ket(x)
    y = LK.LazyKet(b, [Q.Ket(k.basis, np.zeros(len(k.basis), complex)) for k in kets])
    LK.mul_(y, op, psi, 1.0 - 0.5j, 0.0)
    ref = (1.0 - 0.5j) * (np.asarray(O.dense(op).data) @ psi.to_ket().data)
    assert np.linalg.norm(y.to_ket().data - ref) / np.linalg.norm(ref) < 1e-12
    with pytest.raises(O.ArgumentError):
        LK.mul_(y, op, psi, 1.0, 0.5)


def test_spin_sigmaz_known_answer():
    b1, b2 = Q.SpinBasis("1/2"), Q.SpinBasis(1)
    b = Q.tensor_basis(b1, b2)
    psi = LK.LazyKet(b, (basisstate(b1, 2), basisstate(b2, 1)))  # spindown, spinup
    sz = O.LazyTensor(b, b, (1, 2), (O.sigmaz(b1), O.sigmaz(b2)))
    # sigmaz eigenvalues 2m: spin-1/2 down -> -1, spin-1 up -> +2
    assert LK.expect(sz, psi) == -2.0
