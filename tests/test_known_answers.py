"""Known-answer values of the reference's precompile scenarios
(benchmark/precompile/scenarios.jl), for the oracle (CPU) and, for fock() and
composite(), for the device path (GPU; the device forms of the other two are
covered by the particle and time-dependent GPU tests):

* fock() (:1-14): <alpha|a|alpha> = alpha for the coherent state alpha = 1.2 on
  FockBasis(20) (atol 1e-10), and tr(n dm(alpha)) = |alpha|^2 (atol 1e-9);
* particle() (:61-80): the Gaussian packet (x0 0.1, p0 0.3, sigma 1) on
  PositionBasis(-10, 10, 200) transformed to momentum space keeps norm 1 and
  has real(<p>) = 0.3 (atol 1e-12);
* time_dependent() (:153-166): TimeDependentSum((cos, sin), (sigmax, sigmaz)) at
  t = 0.25 on spinup equals (cos 0.25 sigmax + sin 0.25 sigmaz) spinup to 1e-12;
* composite() (:16-40): H = n (x) I + I (x) 2 sigma+ sigma- + a (x) sigma+ + a^dag (x) sigma-
  on FockBasis(20) (x) SpinBasis(1/2) applied to |1> (x) |down> gives
  |1, down> + |0, up> (the scenario checks the basis and a finite norm; the
  state itself follows from the ladder actions: n|1> = |1>, sigma- |down> = 0,
  a|1> = |0>, sigma+ |down> = |up>), norm sqrt(2).
"""
import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from qobgpu import operators as O

ALPHA = 1.2


def fock_case():
    b = Q.FockBasis(20)
    state = Q.coherentstate(b, ALPHA)
    return b, state


def composite_case():
    sb, fb = Q.SpinBasis("1/2"), Q.FockBasis(20)
    basis = Q.tensor_basis(fb, sb)
    atom = O.scale(O.multiply(O.sigmap(sb), O.sigmam(sb)), 2.0)
    lazy = O.LazySum(basis, basis, np.ones(4), (
        O.LazyTensor(basis, basis, (1,), (O.number(fb),)),
        O.LazyTensor(basis, basis, (2,), (atom,)),
        O.LazyTensor(basis, basis, (1, 2), (O.destroy(fb), O.sigmap(sb))),
        O.LazyTensor(basis, basis, (1, 2), (O.create(fb), O.sigmam(sb)))))
    # the scenario's own form: embedded and tensor-product sparse operators
    materialised = O.LazySum(basis, basis, np.ones(4), (
        O.embed(basis, basis, 1, O.number(fb)), O.embed(basis, basis, 2, atom),
        O.tensor(O.destroy(fb), O.sigmap(sb)), O.tensor(O.create(fb), O.sigmam(sb))))
    psi = Q.tensor_states(Q.fockstate(fb, 1), Q.spindown(sb))
    expected = Q.tensor_states(Q.fockstate(fb, 1), Q.spindown(sb)).data + \
        Q.tensor_states(Q.fockstate(fb, 0), Q.spinup(sb)).data
    return basis, (lazy, materialised), psi, expected


def oracle_apply(op, psi):
    return OR.mul(Q.Ket(op.basis_l, np.zeros(len(op.basis_l), np.complex128)), op, psi, 1.0, 0.0)


def test_oracle_fock_scenario():
    b, state = fock_case()
    a_state = oracle_apply(O.destroy(b), state)
    assert abs(np.vdot(state.data, a_state) - ALPHA) <= 1e-10
    rho = Q.dm(state)
    n_rho = OR.mul(O.Operator(b, b, np.zeros((len(b), len(b)), np.complex128, order="F")), O.number(b), rho,
                   1.0, 0.0)
    assert abs(np.trace(n_rho) - ALPHA ** 2) <= 1e-9
    assert abs(np.trace(rho.data) - 1.0) <= 1e-12


def test_oracle_composite_scenario():
    basis, ops, psi, expected = composite_case()
    for H in ops:
        got = oracle_apply(H, psi)
        assert np.array_equal(got, expected)
        assert np.linalg.norm(got) == np.sqrt(2.0)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,atol", [(np.complex128, 1e-10), (np.complex64, 1e-6)])
def test_device_fock_scenario(dtype, atol):
    from qobgpu.mul import expect, to_device

    b, state = fock_case()
    dstate = to_device(state, dtype=dtype)
    assert abs(expect(O.destroy(b), dstate) - ALPHA) <= atol
    drho = to_device(Q.dm(state), dtype=dtype)
    assert abs(expect(O.number(b), drho) - ALPHA ** 2) <= 10 * atol


@pytest.mark.gpu
@pytest.mark.parametrize("arith", [None, "ff"])
def test_device_composite_scenario(arith):
    from qobgpu.mul import mul_, norm, to_device

    basis, ops, psi, expected = composite_case()
    for H in ops:
        out = to_device(Q.Ket(basis, np.zeros(len(basis), np.complex128)))
        mul_(out, H, to_device(psi), 1.0, 0.0, arith=arith)
        got = out.data.cpu().numpy()
        assert np.array_equal(got, expected)
        assert abs(norm(out) - np.sqrt(2.0)) <= 1e-15


def test_oracle_particle_scenario():
    from qobgpu.bases import MomentumBasis, PositionBasis
    from qobgpu.particle import gaussianstate, momentum, transform

    bx = PositionBasis(-10, 10, 200)
    bp = MomentumBasis(bx)
    psi = gaussianstate(bx, 0.1, 0.3, 1.0)
    phi = oracle_apply(transform(bp, bx), psi)
    assert abs(np.linalg.norm(phi) - 1.0) <= 1e-12
    p_phi = oracle_apply(momentum(bp), Q.Ket(bp, phi))
    assert abs(np.vdot(phi, p_phi).real - 0.3) <= 1e-12


def test_oracle_time_dependent_scenario():
    b = Q.SpinBasis("1/2")
    sx, sz = O.sigmax(b), O.sigmaz(b)
    op = O.TimeDependentSum((np.cos, np.sin), (sx, sz))
    op.set_time(0.25)
    assert op.current_time == 0.25
    up = Q.spinup(b)
    got = oracle_apply(op.static_op, up)
    expected = (np.cos(0.25) * sx.data.toarray() + np.sin(0.25) * sz.data.toarray()) @ up.data
    assert np.linalg.norm(got - expected) < 1e-12
