"""ComplexF64 mul! in double-float arithmetic (QOB_C128X, ``arith="ff"``)
against the oracle.

The data stay ComplexF64; the fused LazySum part accumulates pairs of FP32
numbers (about 48 significant bits).  Tolerance: the ComplexF64 bar, relative
l2 1e-12, over every value mode (real, phased, complex groups), launch shape,
beta mode, side (kets, bras, operators from both sides), composite plan
(dense, mode-k, LazyProduct passes beside the gather) and the coefficient
refresh of a TimeDependentSum; the measured errors sit near 1e-15.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import host_copy, rand_op, rand_state, rel_l2
from qobgpu import operators as O
from qobgpu.hamiltonians import heisenberg_chain, jaynes_cummings, jaynes_cummings_sparse, two_mode_cavity

pytestmark = pytest.mark.gpu

TOL = 1e-12
AL, BE = 0.7 - 0.2j, 0.3


def ff_mul(result, a, b, alpha, beta):
    """mul_ with arith="ff" on device copies of the state operands; host result data."""
    from qobgpu.mul import mul_, to_device

    r = to_device(result)
    if isinstance(b, Q.states.StateVector) or (isinstance(b, O.Operator) and isinstance(b.data, np.ndarray)
                                               and not isinstance(a, Q.states.StateVector)):
        b = to_device(b)
    else:
        a = to_device(a)
    mul_(r, a, b, alpha, beta, arith="ff")
    return host_copy(r)


def check(result, a, b, alpha=AL, beta=BE, tol=TOL):
    ref = OR.mul(result, a, b, alpha, beta)
    err = rel_l2(ff_mul(result, a, b, alpha, beta), ref)
    assert err < tol, f"relative l2 error {err:.3e} >= {tol:g}"
    return err


def test_benchmark_hamiltonians_kets_and_batches():
    rng = Q.Rng(900)
    H = jaynes_cummings(15, 15, seed=1)
    psi, out = rand_state(rng, H.basis_r), rand_state(rng, H.basis_l)
    errs = [check(out, H, psi, AL, b) for b in (BE, 0.0, 1.0, 0.4 + 0.9j)]
    H = heisenberg_chain(14, seed=3)
    nb = 8
    X = O.Operator(H.basis_r, Q.GenericBasis(nb), rng.kets_data(len(H.basis_r), nb))
    Y = O.Operator(H.basis_l, Q.GenericBasis(nb), rng.kets_data(len(H.basis_l), nb))
    errs.append(check(Y, H, X))
    # far inside the FP64 bar: double-float keeps about 48 bits
    assert max(errs) < 1e-13, errs


@pytest.mark.parametrize("block,split", [(128, 1), (256, 1), (-256, 1), (256, 4), (128, 8), (128, 16), (256, 32), (-256, 16)])
@pytest.mark.parametrize("tc", [1, 2, 4, 8])
def test_every_launch_shape(tc, block, split):
    from qobgpu import _lib as L
    from qobgpu.device import get_context, handle, raise_for

    ctx = get_context(0)
    for H, seed in ((heisenberg_chain(10, seed=6), 901), (jaynes_cummings(7, 7, seed=2), 902)):
        rng = Q.Rng(seed)
        nb = 37
        X = O.Operator(H.basis_r, Q.GenericBasis(nb), rng.kets_data(len(H.basis_r), nb))
        Y = O.Operator(H.basis_l, Q.GenericBasis(nb), rng.kets_data(len(H.basis_l), nb))
        h = handle(ctx, H)
        raise_for(L.lib().qob_op_set_launch(ctx.ptr, h.ptr, L.QOB_LEFT, L.QOB_C128X, tc, block, split), ctx)
        check(Y, H, X)
        check(Y, H, X, AL, 0.0)


def test_operators_from_both_sides_and_bras():
    rng = Q.Rng(903)
    H = heisenberg_chain(8, seed=4)
    rho = rand_op(rng, H.basis_r, H.basis_r)
    r0 = rand_op(rng, H.basis_l, H.basis_r)
    check(r0, H, rho)
    check(r0, rho, H)  # strided vectors: the rows of rho
    bra, rb = rand_state(rng, H.basis_l, Q.Bra), rand_state(rng, H.basis_r, Q.Bra)
    check(rb, bra, H)


def test_sparse_operator_wide_rows():
    """A full-space SparseOperator: rows too wide for fixed slots (the CSR form)."""
    S = jaynes_cummings_sparse(31, 63, seed=1)
    rng = Q.Rng(904)
    n = len(S.basis_l)
    psi, out = rand_state(rng, S.basis_r), rand_state(rng, S.basis_l)
    check(out, S, psi)
    X = O.Operator(S.basis_r, Q.GenericBasis(24), np.asfortranarray(rng.complex_normal(n * 24).reshape(n, 24, order="F")))
    Y = O.Operator(S.basis_l, Q.GenericBasis(24), np.asfortranarray(rng.complex_normal(n * 24).reshape(n, 24, order="F")))
    check(Y, S, X)
    b = Q.GenericBasis(300)
    Sp = O.sparse(rand_op(rng, b, b, density=0.05))  # complex entries
    psi, out = rand_state(rng, b), rand_state(rng, b)
    check(out, O.dagger(Sp), psi)


def test_complex_coefficients_and_non_square():
    rng = Q.Rng(905)
    H = heisenberg_chain(9, seed=8)
    Hc = O.LazySum([0.3 + 0.2j * (k % 3) for k in range(len(H.operators))], H.operators)
    psi, out = rand_state(rng, Hc.basis_r), rand_state(rng, Hc.basis_l)
    check(out, Hc, psi)
    for k in range(3):
        n1, n2 = rng.integers(2, 8, 64)
        Hm = two_mode_cavity(int(n1), int(n2), seed=20 + k)
        psi, out = rand_state(rng, Hm.basis_r), rand_state(rng, Hm.basis_l)
        check(out, Hm, psi)
    # a LazyTensor between different bases (truncated identity outside the support)
    b1a, b1b, b2a, b2b = Q.GenericBasis(2), Q.GenericBasis(3), Q.GenericBasis(4), Q.GenericBasis(4)
    bl, br = Q.tensor_basis(b1a, b2a), Q.tensor_basis(b1b, b2b)
    op = O.LazyTensor(bl, br, (1,), (rand_op(rng, b1a, b1b),), 0.7)
    psi, out = rand_state(rng, br), rand_state(rng, bl)
    check(out, op, psi)


def test_composite_plans_dense_modek_product():
    rng = Q.Rng(906)
    b1, b2, b3 = Q.GenericBasis(200), Q.GenericBasis(3), Q.GenericBasis(200)
    b = Q.tensor_basis(b1, b2, b3)
    big = O.LazyTensor(b, b, (1, 3), (rand_op(rng, b1, b1), rand_op(rng, b3, b3)), 0.3)
    small = O.LazyTensor(b, b, (2,), (rand_op(rng, b2, b2),), 1.1)
    op = O.LazySum([1.0, 0.5], (big, small))  # mode-k chain beside a fused gather
    psi, out = rand_state(rng, b), rand_state(rng, b)
    check(out, op, psi)
    bs = [Q.GenericBasis(k) for k in (3, 5, 4, 6)]
    prod = O.LazyProduct(tuple(rand_op(rng, bs[i], bs[i + 1]) for i in range(3)), factor=0.5 - 0.1j)
    psi, out = rand_state(rng, bs[3]), rand_state(rng, bs[0])
    check(out, prod, psi)
    bra, rb = rand_state(rng, bs[0], Q.Bra), rand_state(rng, bs[3], Q.Bra)
    check(rb, bra, prod)


def test_lazy_liouvillian_phased_groups():
    """The doubled-basis Liouvillian stores real numbers per group with the
    factor i on the Hamiltonian parts (the phased value mode)."""
    import torch

    from qobgpu import superoperators as S
    from qobgpu.mul import mul_
    from qobgpu.states import Ket

    H = heisenberg_chain(5, seed=907)
    bs = Q.SpinBasis("1/2")
    b = H.basis_l
    J = [O.LazyTensor(b, b, (i,), (O.sigmam(bs),)) for i in range(1, 6)]
    lazy = S.lazy_liouvillian(H, J, rates=[0.1, 0.2, 0.3, 0.4, 0.5])
    mat = S.liouvillian(O.sparse(H), [O.sparse(j) for j in J], rates=[0.1, 0.2, 0.3, 0.4, 0.5])
    rng = Q.Rng(908)
    n = len(b)
    rho = rng.complex_normal(n * n)
    out = rng.complex_normal(n * n)
    ref = OR.mul_arrays(0, True, OR.build_node(mat.vectorised), AL, rho, BE, out.copy())
    v = lazy.vectorised
    x = torch.as_tensor(rho, device="cuda:0")
    y = torch.as_tensor(out, device="cuda:0")
    mul_(Ket(v.basis_l, y), v, Ket(v.basis_r, x), AL, BE, arith="ff")
    assert rel_l2(y.cpu().numpy(), ref) < TOL


def test_time_dependent_sum_refresh():
    """New coefficients re-evaluate the stored double-float values on the device."""
    H = heisenberg_chain(6, seed=7)
    td = O.TimeDependentSum([(lambda t, k=k: np.cos(t + k) + 0.5j * np.sin(2 * t - k)) for k in range(len(H.operators))],
                            H.operators)
    rng = Q.Rng(909)
    psi, out = rand_state(rng, H.basis_r), rand_state(rng, H.basis_l)
    for t in (0.0, 0.3, 1.1):
        td.set_time(t)
        ref = OR.mul(out, td.static_op, psi, AL, BE)
        assert rel_l2(ff_mul(out, td, psi, AL, BE), ref) < TOL


def test_host_buffers_and_tuning():
    from qobgpu import _lib as L
    from qobgpu.device import get_context, handle, raise_for
    from qobgpu.mul import mul_

    H = heisenberg_chain(9, seed=5)
    rng = Q.Rng(910)
    n = len(H.basis_l)
    ctx = get_context(0)
    h = handle(ctx, H)
    times = (C.c_double * 36)()
    chosen = C.c_int()
    raise_for(L.lib().qob_op_tune(ctx.ptr, h.ptr, L.QOB_LEFT, L.QOB_C128X, 16, times, C.byref(chosen)), ctx)
    assert chosen.value & 0xFFFF in (1, 2, 4, 8) and max(times) > 0
    for ncols in (1, 16):
        X = O.Operator(H.basis_r, Q.GenericBasis(ncols), rng.kets_data(n, ncols))
        Y = O.Operator(H.basis_l, Q.GenericBasis(ncols), rng.kets_data(n, ncols))
        ref = OR.mul(Y, H, X, AL, BE)
        got = O.Operator(Y.basis_l, Y.basis_r, np.array(Y.data, order="F", copy=True))
        mul_(got, H, X, AL, BE, arith="ff")
        assert rel_l2(got.data, ref) < TOL


def test_range_scaled_states_nan_and_overflow():
    """Elements scaled by 2^60 and 2^-60 keep the precision; NaN propagates;
    magnitudes of 2^128 and above become infinite (the documented range)."""
    H = jaynes_cummings(6, 6, seed=9)
    rng = Q.Rng(911)
    psi, out = rand_state(rng, H.basis_r), rand_state(rng, H.basis_l)
    for s in (2.0 ** 60, 2.0 ** -60):
        p = Q.Ket(H.basis_r, psi.data * s)
        o = Q.Ket(H.basis_l, out.data * s)
        check(o, H, p)
    from qobgpu.mul import mul_, to_device

    bad = psi.data.copy()
    bad[3] = np.nan
    got = ff_mul(out, H, Q.Ket(H.basis_r, bad), AL, 0.0)
    r64 = to_device(out)
    mul_(r64, H, to_device(Q.Ket(H.basis_r, bad)), AL, 0.0)  # the same plan structure in FP64
    ref = host_copy(r64)
    assert np.isnan(got).any() and np.array_equal(np.isnan(got), np.isnan(ref))
    big = psi.data.copy()
    big[0] = 1e300
    got = ff_mul(out, H, Q.Ket(H.basis_r, big), AL, 0.0)
    assert not np.all(np.isfinite(got))


def test_fp32_data_rejects_double_float():
    from qobgpu.mul import mul_, to_device

    H = jaynes_cummings(3, 3)
    rng = Q.Rng(912)
    psi = to_device(rand_state(rng, H.basis_r), dtype=np.complex64)
    out = to_device(rand_state(rng, H.basis_l), dtype=np.complex64)
    with pytest.raises(O.ArgumentError):
        mul_(out, H, psi, 1.0, 0.0, arith="ff")


@pytest.mark.parametrize("ncols", [1, 5])
def test_dense_operator_double_float(ncols):
    """A 700 x 500 DenseOperator (dense pass, split over column ranges) and its
    product with a 2-factor dense LazyTensor (mode products), both in
    double-float arithmetic."""
    rng = Q.Rng(913 + ncols)
    bl, br = Q.GenericBasis(700), Q.GenericBasis(500)
    D = rand_op(rng, bl, br)
    X = O.Operator(br, Q.GenericBasis(ncols), rng.kets_data(500, ncols))
    Y = O.Operator(bl, Q.GenericBasis(ncols), rng.kets_data(700, ncols))
    assert check(Y, D, X, AL, 0.4 - 0.9j) < 1e-13
    b1, b2 = Q.GenericBasis(40), Q.GenericBasis(30)
    b = Q.tensor_basis(b1, b2)
    lt = O.LazyTensor(b, b, (1, 2), (rand_op(rng, b1, b1), rand_op(rng, b2, b2)), 0.6)
    psi, out = rand_state(rng, b), rand_state(rng, b)
    assert check(out, lt, psi) < 1e-13


def test_rk4_and_server_double_float():
    """RK4 with the operator in double-float arithmetic (ComplexF64 states and
    stage arithmetic): time-dependent steps against the host RK4, a static chain
    against the FP64 device RK4, and both served in a mix, each request equal
    bitwise to the same evolution run alone."""
    import torch

    from qobgpu.evolution import Server, rk4
    from test_gpu_timedependent import rk4_host_td, td_heisenberg

    dt, nsteps, t0 = 2e-3, 40, 0.1
    td = td_heisenberg(8, seed=920)
    static = heisenberg_chain(8, seed=921)
    rng = Q.Rng(922)
    p_td, p_st = rng.ket_data(len(td.basis_l)), rng.ket_data(len(static.basis_l))
    ref_td = rk4_host_td(td, p_td, dt, nsteps, t0)
    d = torch.as_tensor(p_td.copy(), device="cuda:0")
    rk4(td, d, dt, nsteps, t0=t0, arith="ff")
    alone_td = d.cpu().numpy()
    assert rel_l2(alone_td, ref_td) < TOL
    d64 = torch.as_tensor(p_st.copy(), device="cuda:0")
    rk4(static, d64, dt, nsteps)
    dff = torch.as_tensor(p_st.copy(), device="cuda:0")
    rk4(static, dff, dt, nsteps, arith="ff")
    alone_st = dff.cpu().numpy()
    assert rel_l2(alone_st, d64.cpu().numpy()) < TOL
    S = Server(np.complex128, arith="ff")
    i_st = S.submit(static, p_st, nsteps, dt)
    i_td = S.submit(td, p_td, nsteps, dt, t0=t0)
    while S.step():
        pass
    for i, a in ((i_st, alone_st), (i_td, alone_td)):
        st, _, got = S.poll(i)
        assert st == 2
        assert np.array_equal(got, a), "served result differs from the same evolution run alone"
    S.close()


@pytest.mark.parametrize("n", [200, 256, 4096])
def test_fft_transforms_double_float(n):
    """FFTOperator passes in double-float arithmetic: direct DFT (200 points),
    radix-2 Stockham (256), the four-step form (4096 points, one ket), kets and
    bras, and a 2-D composite transform; plus the particle Hamiltonian
    Txp (p^2/2) Tpx + V (a LazySum holding a LazyProduct of FFT operators)."""
    from qobgpu.bases import MomentumBasis, PositionBasis
    from qobgpu.particle import momentum, potentialoperator, transform

    bx = PositionBasis(-32.5, 20.1, n)
    bp = MomentumBasis(bx)
    rng = Q.Rng(930 + n)
    al, be = 0.7 - 0.2j, 0.3 + 0.1j
    for T in (transform(bp, bx), transform(bx, bp)):
        x, y = rng.complex_normal(n), rng.complex_normal(n)
        assert check(Q.Ket(T.basis_l, y), T, Q.Ket(T.basis_r, x), al, be) < 1e-13
        assert check(Q.Bra(T.basis_r, y), Q.Bra(T.basis_l, x), T, al, be) < 1e-13
    Tpx, Txp = transform(bp, bx), transform(bx, bp)
    pd = np.asarray(momentum(bp).data.diagonal())
    K = O.Operator(bp, bp, O.spdiagm(n, n, {0: pd * pd / 2}))
    V = potentialoperator(bx, lambda q: 0.5 * q * q)
    H = O.LazySum(bx, bx, [1.0, 1.0], (O.LazyProduct((Txp, K, Tpx)), V))
    psi, out = rand_state(rng, bx), rand_state(rng, bx)
    check(out, H, psi)
    bxs = [PositionBasis(-3.0, 4.0, 32), PositionBasis(-4.0, 5.0, 21)]
    bX, bP = Q.tensor_basis(*bxs), Q.tensor_basis(*[MomentumBasis(b) for b in bxs])
    T2 = transform(bP, bX)
    m = len(bX)
    x, y = rng.complex_normal(m), rng.complex_normal(m)
    check(Q.Ket(T2.basis_l, y), T2, Q.Ket(T2.basis_r, x), al, be)


def test_uneven_batch_double_float():
    """Uneven two-mode cavities in one persistent launch (the fused batch kernel
    splitting each element as it loads), against the oracle."""
    import torch

    from qobgpu.evolution import Batch

    rng = Q.Rng(940)
    b = Batch(np.complex128, arith="ff")
    refs, ys = [], []
    for k in range(12):
        n1, n2 = rng.integers(2, 3, 20)
        H = two_mode_cavity(int(n1), int(n2), seed=941 + k)
        n = len(H.basis_l)
        x, y = rng.ket_data(n), rng.ket_data(n)
        refs.append(OR.mul(Q.Ket(H.basis_l, y), H, Q.Ket(H.basis_r, x), AL, BE))
        xt, yt = torch.as_tensor(x, device="cuda:0"), torch.as_tensor(y, device="cuda:0")
        b.add(H, xt, yt, AL, BE)
        ys.append(yt)
    assert b.info()["fused"] == 12
    b.run()
    torch.cuda.synchronize()
    for yt, r in zip(ys, refs):
        assert rel_l2(yt.cpu().numpy(), r) < 1e-13


def test_batch_double_float_complex_and_mixed_items():
    """A double-float batch holding complex-valued models (the fused kernel's
    complex form) and real ones (run apart, as in the other dtypes), against the
    oracle; the served engine uses the same tables."""
    import torch

    from qobgpu.evolution import Batch

    rng = Q.Rng(960)
    b = Batch(np.complex128, arith="ff")
    refs, ys = [], []
    for k in range(6):
        n1, n2 = rng.integers(2, 3, 12)
        H = two_mode_cavity(int(n1), int(n2), seed=961 + k)
        if k % 2 == 0:  # complex coefficients: drive with a phase
            H = O.LazySum(H.basis_l, H.basis_r, [0.7, 1.1, 0.3, 0.4 * np.exp(0.6j)], H.operators)
        n = len(H.basis_l)
        x, y = rng.ket_data(n), rng.ket_data(n)
        refs.append(OR.mul(Q.Ket(H.basis_l, y), H, Q.Ket(H.basis_r, x), AL, BE))
        xt, yt = torch.as_tensor(x, device="cuda:0"), torch.as_tensor(y, device="cuda:0")
        b.add(H, xt, yt, AL, BE)
        ys.append(yt)
    b.run()
    torch.cuda.synchronize()
    info = b.info()
    assert info["items"] == 6 and info["fused"] >= 3
    for yt, r in zip(ys, refs):
        assert rel_l2(yt.cpu().numpy(), r) < 1e-13
