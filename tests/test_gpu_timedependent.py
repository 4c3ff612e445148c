"""Time-dependent sums on the GPU: coefficient updates re-evaluated on the
device (set_factors between mul! calls, and inside RK4 steps) against the
oracle's mul! with the same coefficients (src/time_dependent_operator.jl:162-171,
279-290: set_time! rewrites the static LazySum's factors before each mul!).

Tolerances (relative l2): 1e-12 for ComplexF64, 1e-5 for ComplexF32.
"""
import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import rel_l2
from qobgpu import operators as O
from qobgpu.hamiltonians import heisenberg_chain, jaynes_cummings

pytestmark = pytest.mark.gpu

AL, BE = 0.7 - 0.2j, 0.3


def td_heisenberg(nspins, seed):
    """Chain whose sigma_x sigma_x couplings oscillate around the sigma_y sigma_y ones:
    where Jx(t) == Jy the aligned-spin entries of a bond cancel, elsewhere not."""
    H = heisenberg_chain(nspins, seed=seed)
    coefs = []
    for k, f in enumerate(H.factors):
        if k < 3 * (nspins - 1) and k % 3 == 0:
            coefs.append(lambda t, f=f: f * (1.0 + 0.5 * np.sin(3.0 * t)))
        elif k < 3 * (nspins - 1) and k % 3 == 2:
            coefs.append(lambda t, f=f: f * np.cos(t))
        else:
            coefs.append(complex(f))
    return O.TimeDependentSum(coefs, H.operators)


def td_driven_jc(n1, n2, seed):
    """Jaynes-Cummings with a rotating-frame drive: complex coefficients exp(+-i nu t)."""
    H = jaynes_cummings(n1, n2, seed=seed)
    nu = 1.7
    coefs = [complex(f) for f in H.factors]
    coefs[3] = lambda t, f=H.factors[3]: f * np.exp(1j * nu * t)
    coefs[4] = lambda t, f=H.factors[4]: f * np.exp(-1j * nu * t)
    return O.TimeDependentSum(coefs, H.operators)


def rk4_host_td(td, psi, dt, nsteps, t0=0.0):
    """Fixed-step RK4 with set_time! before every right-hand side and the oracle's mul!."""

    def f(t, v):
        td.set_time(t)
        node = OR.build_node(td)
        return OR.mul_arrays(0, True, node, -1j, v, 0.0, np.zeros_like(v))

    psi = np.array(psi, dtype=np.complex128)
    for s in range(nsteps):
        t = t0 + s * dt
        k1 = f(t, psi)
        k2 = f(t + dt / 2, psi + dt / 2 * k1)
        k3 = f(t + dt / 2, psi + dt / 2 * k2)
        k4 = f(t + dt, psi + dt * k3)
        psi = psi + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
    return psi


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-5)])
def test_set_factors_refresh_on_device_and_rebuild(dtype, tol):
    """A factor change that the stored pattern holds is re-evaluated on the device
    (two extra launches: values, merged diagonal); one that creates entries outside
    it, or complex values in a real-valued form, rebuilds the structure."""
    from qobgpu import _lib as L
    from qobgpu.mul import mul_, to_device

    H = heisenberg_chain(6, seed=21)
    nb = 5
    rng = Q.Rng(301)
    psi = Q.Ket(H.basis_r, rng.ket_data(len(H.basis_r)))
    out = Q.Ket(H.basis_l, rng.ket_data(len(H.basis_l)))
    base = np.array(H.factors, dtype=np.complex128)

    def factors(jx_scale, jy_scale, phase=1.0):
        f = base.copy()
        for b in range(nb):
            f[3 * b] *= jx_scale
            f[3 * b + 1] *= jy_scale
        f[3 * nb:] *= phase
        return f

    steps = [
        (factors(1.0, 1.0), None),        # first compile: aligned entries cancel, not stored
        (factors(2.0, 2.0), "device"),    # Jx == Jy still: the pattern holds
        (factors(2.0, 0.5), "rebuild"),   # aligned entries appear
        (factors(0.7, 0.7), "device"),    # zero values in stored slots are fine
        (factors(1.0, 1.0, 1j), "rebuild"),  # complex values in a real-valued form
        (factors(1.2, 1.2), "device"),    # complex storage holds real values
        (factors(1.5, 0.5), "rebuild"),   # aligned entries appear again
    ]
    d_psi = to_device(psi, dtype=dtype)
    for f, path in steps:
        H.set_factors(f)
        ref = OR.mul(out, H, psi, AL, BE)
        r = to_device(out, dtype=dtype)
        n0 = L.lib().qob_kernel_launches()
        mul_(r, H, d_psi, AL, BE)
        launches = L.lib().qob_kernel_launches() - n0
        got = r.data.cpu().numpy().astype(np.complex128)
        assert rel_l2(got, ref) < tol, (f, path)
        if path == "device":
            assert launches == 3  # values + merged diagonal + gather
        elif path == "rebuild":
            assert launches == 2  # merged diagonal (during the upload) + gather


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-5)])
@pytest.mark.parametrize("model", ["heisenberg8", "driven_jc"])
def test_rk4_time_dependent_against_host(model, dtype, tol):
    import torch

    from qobgpu.evolution import rk4

    td = td_heisenberg(8, seed=22) if model == "heisenberg8" else td_driven_jc(15, 15, seed=23)
    psi = Q.Rng(302).ket_data(len(td.basis_l))
    dt, nsteps, t0 = 2e-3, 60, 0.25
    ref = rk4_host_td(td, psi, dt, nsteps, t0)
    d = torch.as_tensor(psi.astype(dtype), device="cuda:0")
    rk4(td, d, dt, nsteps, t0=t0)
    assert rel_l2(d.cpu().numpy().astype(np.complex128), ref) < tol
    assert td.current_time == pytest.approx(t0 + nsteps * dt)


def test_mul_after_time_dependent_rk4_uses_current_factors():
    """After the steps the compiled values belong to the last stage; the next mul!
    re-evaluates them from the operator's own factors."""
    import torch

    from qobgpu.evolution import rk4
    from qobgpu.mul import mul_, to_device

    td = td_heisenberg(6, seed=24)
    rng = Q.Rng(303)
    psi = Q.Ket(td.basis_r, rng.ket_data(len(td.basis_r)))
    out = Q.Ket(td.basis_l, rng.ket_data(len(td.basis_l)))
    d = torch.as_tensor(rng.ket_data(len(td.basis_l)), device="cuda:0")
    rk4(td, d, 1e-2, 7, t0=0.0)
    td.set_time(2.9)
    ref = OR.mul(out, td, psi, AL, BE)
    r = to_device(out)
    mul_(r, td, to_device(psi), AL, BE)
    assert rel_l2(r.data.cpu().numpy(), ref) < 1e-12


def test_rk4_time_dependent_argument_checks():
    import ctypes as C

    import torch

    from qobgpu import _lib as L
    from qobgpu.device import get_context, handle

    td = td_heisenberg(4, seed=25)
    ctx = get_context(0)
    h = handle(ctx, td)
    d = torch.zeros(16, dtype=torch.complex128, device="cuda:0")
    rows = np.zeros((5, len(td.coefficients)), np.complex128)
    rc = L.lib().qob_rk4_td(ctx.ptr, h.ptr, L.QOB_C128, C.c_void_p(d.data_ptr()), 16, 1e-3, 3,
                            rows.ctypes.data_as(C.c_void_p), 5, 0, None)
    assert rc == L.QOB_ERR_ARG  # 3 steps need 7 rows
    static = heisenberg_chain(4, seed=25)
    hs = handle(ctx, O.LazyProduct((static, static)))
    rc = L.lib().qob_rk4_td(ctx.ptr, hs.ptr, L.QOB_C128, C.c_void_p(d.data_ptr()), 16, 1e-3, 2,
                            rows.ctypes.data_as(C.c_void_p), 5, 0, None)
    assert rc == L.QOB_ERR_ARG  # not a LazySum


@pytest.mark.parametrize("threaded", [False, True])
def test_server_time_dependent_requests_in_a_mix(threaded):
    """Time-dependent requests served beside a static one: each matches the
    host RK4 with set_time! per stage, and equals qob_rk4_td run alone bitwise."""
    import torch

    from qobgpu.evolution import Server, rk4

    static = heisenberg_chain(8, seed=31)
    tds = [td_heisenberg(8, seed=32), td_driven_jc(7, 7, seed=33)]
    rng = Q.Rng(304)
    psis = [rng.ket_data(len(H.basis_l)) for H in [static] + tds]
    dt, nsteps, t0 = 2e-3, 40, 0.1
    alone = []
    for H, p in zip(tds, psis[1:]):
        d = torch.as_tensor(p.copy(), device="cuda:0")
        rk4(H, d, dt, nsteps, t0=t0)
        alone.append(d.cpu().numpy())
    refs = [rk4_host_td(H, p, dt, nsteps, t0) for H, p in zip(tds, psis[1:])]
    S = Server(np.complex128)
    rid_static = S.submit(static, psis[0], nsteps + 7, dt)
    ids = [S.submit(H, p, nsteps, dt, t0=t0) for H, p in zip(tds, psis[1:])]
    if threaded:
        S.start()
        for i in ids + [rid_static]:
            S.wait(i, 120.0)
        S.stop()
    else:
        while S.step():
            pass
    for i, a, r in zip(ids, alone, refs):
        st, _, got = S.poll(i)
        assert st == 2
        assert rel_l2(got, r) < 1e-12
        assert np.array_equal(got, a), "served result differs from the same evolution run alone"
    assert S.poll(rid_static)[0] == 2
    S.close()


def test_server_time_dependent_request_that_cannot_compile_fails_alone():
    """A time-dependent request whose terms do not all fit the fused gather (a
    LazyProduct term) fails with -QOB_ERR_UNSUPPORTED at admission; the
    requests beside it complete."""
    from qobgpu import _lib as L
    from qobgpu.evolution import Server

    H = heisenberg_chain(6, seed=41)
    b = H.basis_l
    prod = O.LazyProduct((H.operators[0], H.operators[1]))
    bad = O.TimeDependentSum([1.0, lambda t: np.cos(t)], (H.operators[2], prod))
    good = td_heisenberg(6, seed=42)
    rng = Q.Rng(305)
    S = Server(np.complex128)
    r_bad = S.submit(bad, rng.ket_data(len(b)), 10, 1e-3)
    r_good = S.submit(good, rng.ket_data(len(b)), 10, 1e-3)
    while S.step():
        pass
    assert S.poll(r_bad)[0] == -L.QOB_ERR_UNSUPPORTED
    assert S.poll(r_good)[0] == 2
    S.close()
