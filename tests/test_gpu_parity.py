"""GPU parity: libqobgpu (through the C ABI via the qobgpu mirror) against the
oracle (restated reference mul!) on the same seeded inputs.

Tolerances (relative l2, stated per test): 1e-12 for ComplexF64, 1e-5 for the
ComplexF32 mode, as the plain form and the precision mode require.
"""
import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import host_copy, rand_op, rand_state, rel_l2
from qobgpu import operators as O
from qobgpu.hamiltonians import (heisenberg_chain, jaynes_cummings, jaynes_cummings_sparse,
                                 random_density_columns, two_mode_cavity)

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5
AL, BE = 0.7 - 0.2j, 0.3


def _is_state(x):
    return isinstance(x, Q.states.StateVector) or (isinstance(x, O.Operator) and isinstance(x.data, np.ndarray))


def gpu_mul(result, a, b, alpha=1.0, beta=0.0, dtype=np.complex128):
    """mul_ on device copies of the state operands; returns the host result data."""
    from qobgpu.mul import mul_, to_device

    r = to_device(result, dtype=dtype)
    if isinstance(b, Q.states.StateVector) or (_is_state(b) and not isinstance(a, Q.states.StateVector)):
        b = to_device(b, dtype=dtype)
    else:
        a = to_device(a, dtype=dtype)
    mul_(r, a, b, alpha, beta)
    return host_copy(r)


def check(result, a, b, alpha, beta, tol=TOL64, dtype=np.complex128):
    ref = OR.mul(result, a, b, alpha, beta)
    got = gpu_mul(result, a, b, alpha, beta, dtype)
    err = rel_l2(got, ref)
    assert err < tol, f"relative l2 error {err:.3e} >= {tol:g}"
    return err


# ---------------------------------------------------------------- benchmark Hamiltonians
def test_jaynes_cummings_ket_fp64_and_fp32():
    H = jaynes_cummings(15, 15, seed=1)
    rng = Q.Rng(100)
    psi, out = rand_state(rng, H.basis_r), rand_state(rng, H.basis_l)
    check(out, H, psi, AL, BE, TOL64)
    check(out, H, psi, AL, BE, TOL32, np.complex64)
    check(out, H, psi, AL, 0.0, TOL64)
    check(out, H, psi, AL, 1.0, TOL64)


def test_heisenberg_14_spins_batch():
    H = heisenberg_chain(14, seed=3)
    rng = Q.Rng(101)
    nb = 8
    X = O.Operator(H.basis_r, Q.GenericBasis(nb), rng.kets_data(len(H.basis_r), nb))
    Y = O.Operator(H.basis_l, Q.GenericBasis(nb), rng.kets_data(len(H.basis_l), nb))
    check(Y, H, X, AL, BE, TOL64)
    check(Y, H, X, AL, BE, TOL32, np.complex64)
    psi, out = rand_state(rng, H.basis_r), rand_state(rng, H.basis_l)
    check(out, H, psi, AL, BE, TOL64)


@pytest.mark.parametrize("block,split", [(128, 1), (256, 1), (-256, 1), (128, 4), (256, 2), (128, 8), (128, 16), (256, 32), (-256, 4), (-256, 16)])
@pytest.mark.parametrize("tc", [1, 2, 4, 8])
def test_every_launch_shape(tc, block, split):
    """Each vectors-per-thread tile and launch shape (-256: the persistent grid of
    SMs x resident blocks; split: vector sets per warp) on the 10-spin chain (a
    compact-form plan) and the Jaynes-Cummings model (generic groups), 37 kets
    (ragged last tiles)."""
    from qobgpu import _lib as L
    from qobgpu.device import dtype_code, get_context, handle, raise_for

    ctx = get_context(0)
    for H, seed in ((heisenberg_chain(10, seed=6), 120), (jaynes_cummings(7, 7, seed=2), 121)):
        rng = Q.Rng(seed)
        nb = 37
        X = O.Operator(H.basis_r, Q.GenericBasis(nb), rng.kets_data(len(H.basis_r), nb))
        Y = O.Operator(H.basis_l, Q.GenericBasis(nb), rng.kets_data(len(H.basis_l), nb))
        for dtype, tol in ((np.complex128, TOL64), (np.complex64, TOL32)):
            h = handle(ctx, H)
            raise_for(L.lib().qob_op_set_launch(ctx.ptr, h.ptr, L.QOB_LEFT, dtype_code(dtype), tc, block, split),
                      ctx)
            check(Y, H, X, AL, BE, tol, dtype)
            check(Y, H, X, AL, 0.0, tol, dtype)


def test_heisenberg_operator_both_sides_8_spins():
    H = heisenberg_chain(8, seed=4)
    rng = Q.Rng(102)
    rho = rand_op(rng, H.basis_r, H.basis_r)
    r0 = rand_op(rng, H.basis_l, H.basis_r)
    check(r0, H, rho, AL, BE, TOL64)
    check(r0, rho, H, AL, BE, TOL64)
    check(r0, rho, H, AL, BE, TOL32, np.complex64)
    bra, rb = rand_state(rng, H.basis_l, Q.Bra), rand_state(rng, H.basis_r, Q.Bra)
    check(rb, bra, H, AL, BE, TOL64)


@pytest.mark.parametrize("dtype,tol", [(np.complex128, TOL64), (np.complex64, TOL32)])
def test_sparse_operator_spmv_spmm(dtype, tol):
    S = jaynes_cummings_sparse(31, 63, seed=1)
    rng = Q.Rng(103)
    n = len(S.basis_l)
    psi, out = rand_state(rng, S.basis_r), rand_state(rng, S.basis_l)
    check(out, S, psi, AL, BE, tol, dtype)
    rho = O.Operator(S.basis_r, Q.GenericBasis(256), random_density_columns(n, 256, seed=5))
    r0 = O.Operator(S.basis_l, Q.GenericBasis(256), np.asfortranarray(rng.complex_normal(n * 256).reshape(n, 256, order="F")))
    check(r0, S, rho, AL, BE, tol, dtype)


def test_two_mode_cavities():
    rng = Q.Rng(104)
    for k in range(4):
        n1, n2 = rng.integers(2, 8, 64)
        H = two_mode_cavity(int(n1), int(n2), seed=10 + k)
        psi, out = rand_state(rng, H.basis_r), rand_state(rng, H.basis_l)
        check(out, H, psi, AL, BE, TOL64)
        check(out, H, psi, AL, BE, TOL32, np.complex64)


# ---------------------------------------------------------------- reference test identities
def lt_bases():
    b1a, b1b = Q.GenericBasis(2), Q.GenericBasis(3)
    b2a, b2b = Q.GenericBasis(1), Q.GenericBasis(4)
    b3a, b3b = Q.GenericBasis(6), Q.GenericBasis(5)
    return (b1a, b1b, b2a, b2b, b3a, b3b), Q.tensor_basis(b1a, b2a, b3a), Q.tensor_basis(b1b, b2b, b3b)


@pytest.mark.parametrize("sparse_factors", [False, True])
def test_lazytensor_mixed_precision_adjoint(sparse_factors):
    rng = Q.Rng(105)
    (b1a, b1b, b2a, b2b, b3a, b3b), bl, br = lt_bases()
    facs = (rand_op(rng, b1a, b1b, np.complex64), O.dagger(rand_op(rng, b2b, b2a)), O.dagger(rand_op(rng, b3b, b3a)))
    if sparse_factors:
        facs = tuple(O.sparse(f) for f in facs)
    op = O.LazyTensor(bl, br, (1, 2, 3), facs, 0.1)
    psi, out = rand_state(rng, br), rand_state(rng, bl)
    check(out, op, psi, 1.0, 0.0, TOL64)
    check(out, op, psi, 1.5, 2.1, TOL64)
    bra, rb = rand_state(rng, bl, Q.Bra), rand_state(rng, br, Q.Bra)
    check(rb, bra, op, 1.5, 2.1, TOL64)
    st, r0 = rand_op(rng, br, Q.GenericBasis(13)), rand_op(rng, bl, Q.GenericBasis(13))
    check(r0, op, st, 1.5, 2.1, TOL64)
    st, r0 = rand_op(rng, Q.GenericBasis(17), bl), rand_op(rng, Q.GenericBasis(17), br)
    check(r0, st, op, 1.5, 2.1, TOL64)


def test_explicit_isometries_nan_alpha_beta():
    from test_oracle import iso_ops

    rng = Q.Rng(106)
    bl, br, n1, n1_sp, n1_de = iso_ops()
    state, out = rand_op(rng, br, br), rand_op(rng, bl, br)
    nan_out = O.Operator(bl, br, np.full(out.data.shape, np.nan + 0j, order="F"))
    for op in (n1, n1_sp, n1_de):
        check(out, op, state, -0.8, 1.3, TOL64)
        got = gpu_mul(nan_out, op, state, -0.8, 0.0)
        assert np.all(np.isfinite(got))
        assert rel_l2(got, OR.mul(nan_out, op, state, -0.8, 0.0)) < TOL64
        assert np.array_equal(gpu_mul(out, op, state, 0.0, 1.3), OR.mul(out, op, state, 0.0, 1.3))
        assert np.all(gpu_mul(nan_out, op, state, 0.0, 0.0) == 0)
    st2 = rand_op(rng, bl, bl)
    for op in (n1, n1_sp, n1_de):
        check(out, st2, op, -0.8, 1.3, TOL64)


def test_lazysum_dense_terms_and_empty():
    rng = Q.Rng(107)
    _, bl, br = lt_bases()
    ops = tuple(rand_op(rng, bl, br) for _ in range(3))
    op = O.LazySum([0.1, 0.3, 1.2], ops)
    psi, out = rand_state(rng, br), rand_state(rng, bl)
    check(out, op, psi, 1.5, 2.1, TOL64)
    zero = O.LazySum(bl, br)
    assert rel_l2(gpu_mul(out, zero, psi, 1.5, 2.1), 2.1 * out.data) < 1e-15
    nan_out = Q.Ket(bl, np.full(len(bl), np.nan + 0j))
    assert np.all(gpu_mul(nan_out, zero, psi, 1.0, 0.0) == 0)
    st = rand_op(rng, br, br)
    res = O.Operator(bl, br, np.full((len(bl), len(br)), np.nan + 0j, order="F"))
    got = gpu_mul(res, op, st, 1.0, 0.0)
    assert rel_l2(got, OR.mul(res, op, st, 1.0, 0.0)) < TOL64


@pytest.mark.parametrize("nops", [1, 2, 3])
def test_lazyproduct(nops):
    rng = Q.Rng(108 + nops)
    bs = [Q.GenericBasis(k) for k in (3, 5, 4, 6)]
    ops = [rand_op(rng, bs[i], bs[i + 1]) for i in range(nops)]
    op = O.LazyProduct(tuple(ops), factor=0.5 - 0.1j)
    psi, out = rand_state(rng, bs[nops]), rand_state(rng, bs[0])
    check(out, op, psi, 1.5, 2.1, TOL64)
    bra, rb = rand_state(rng, bs[0], Q.Bra), rand_state(rng, bs[nops], Q.Bra)
    check(rb, bra, op, 1.5, 2.1, TOL64)


def test_sparse_adjoint_and_big_dense():
    rng = Q.Rng(110)
    b = Q.GenericBasis(300)
    S = O.sparse(rand_op(rng, b, b, density=0.05))
    psi, out = rand_state(rng, b), rand_state(rng, b)
    check(out, O.dagger(S), psi, 1.5, 2.1, TOL64)
    Dn = rand_op(rng, b, b)  # > 256: the dense pass
    check(out, Dn, psi, 1.5, 2.1, TOL64)
    check(out, O.dagger(Dn), psi, 1.5, 2.1, TOL64)


def test_large_dense_factor_mode_products():
    """LazyTensor with two 200x200 dense factors: too large to merge, runs as
    the mode-product chain of _tp_sum_matmul!."""
    rng = Q.Rng(111)
    b1, b2, b3 = Q.GenericBasis(200), Q.GenericBasis(3), Q.GenericBasis(200)
    b = Q.tensor_basis(b1, b2, b3)
    op = O.LazyTensor(b, b, (1, 3), (rand_op(rng, b1, b1), rand_op(rng, b3, b3)), 0.3)
    from qobgpu.device import prepare

    info = prepare(op)
    assert info["extra_passes"] == 1
    psi, out = rand_state(rng, b), rand_state(rng, b)
    check(out, op, psi, 1.5, 2.1, TOL64)


@pytest.mark.parametrize("ncols", [1, 3, 16, 37])
def test_host_buffers_through_qob_mul_host(ncols):
    """numpy (host) data goes through qob_mul_host: copies in, kernels, copy out
    (in four chunks over three streams for 8 or more columns)."""
    from qobgpu.mul import mul_

    H = heisenberg_chain(9, seed=5)
    rng = Q.Rng(115)
    n = len(H.basis_l)
    X = O.Operator(H.basis_r, Q.GenericBasis(ncols), rng.kets_data(n, ncols))
    Y = O.Operator(H.basis_l, Q.GenericBasis(ncols), rng.kets_data(n, ncols))
    ref = OR.mul(Y, H, X, AL, BE)
    got = O.Operator(Y.basis_l, Y.basis_r, np.array(Y.data, order="F", copy=True))
    mul_(got, H, X, AL, BE)
    assert rel_l2(got.data, ref) < TOL64


# ---------------------------------------------------------------- errors and state
def test_dimension_and_alias_errors():
    from qobgpu.mul import mul_, to_device

    H = jaynes_cummings(3, 3)
    rng = Q.Rng(112)
    psi = to_device(rand_state(rng, H.basis_r))
    with pytest.raises(O.ArgumentError):
        mul_(psi, H, psi, 1.0, 0.0)  # output aliased with input
    wrong = to_device(Q.Ket(Q.GenericBasis(len(H.basis_l)), np.zeros(len(H.basis_l), complex)))
    with pytest.raises(O.IncompatibleBases):
        mul_(wrong, H, psi)


def test_set_factors_time_dependent_sum():
    H = heisenberg_chain(6, seed=7)
    td = O.TimeDependentSum([(lambda t, k=k: np.cos(t + k)) for k in range(len(H.operators))], H.operators)
    rng = Q.Rng(113)
    psi, out = rand_state(rng, H.basis_r), rand_state(rng, H.basis_l)
    for t in (0.0, 0.3, 1.1):
        td.set_time(t)
        ref = OR.mul(out, td.static_op, psi, AL, BE)
        got = gpu_mul(out, td, psi, AL, BE)
        assert rel_l2(got, ref) < TOL64


def test_norm_dot_expect_fp64():
    from qobgpu.mul import dot, expect, norm, to_device

    H = jaynes_cummings(15, 15)
    rng = Q.Rng(114)
    a, b = rand_state(rng, H.basis_r), rand_state(rng, H.basis_r)
    da, db = to_device(a), to_device(b)
    assert abs(norm(da) - np.linalg.norm(a.data)) < 1e-14
    assert abs(dot(da, db) - np.vdot(a.data, b.data)) < 1e-14
    D = O.dense(H).data
    assert abs(expect(H, da) - np.vdot(a.data, D @ a.data)) < 1e-12 * abs(np.vdot(a.data, D @ a.data))
    f = to_device(a, dtype=np.complex64)
    assert abs(norm(f) - np.linalg.norm(a.data.astype(np.complex64).astype(np.complex128))) < 1e-12


@pytest.mark.parametrize("dtype,tol", [(np.complex128, TOL64), (np.complex64, TOL32)])
def test_variance_and_subsystem_expect(dtype, tol):
    """variance(op, psi) (src/operators.jl:139-142) of a Hermitian LazySum (real
    result) and of a non-Hermitian one (complex result), and expect(index, op,
    psi) (src/operators_sparse.jl:49-61), against the oracle's mul! followed by
    FP64 inner products on the host."""
    from qobgpu.mul import expect, to_device, variance

    H = jaynes_cummings(15, 15)
    b = H.basis_r
    rng = Q.Rng(141)
    psi = rand_state(rng, b)
    psi.data[:] /= np.linalg.norm(psi.data)
    A = O.LazySum(b, b, (1.0, 0.4j - 0.2), (H, O.LazyTensor(b, b, (1,), (O.destroy(b.bases[0]),))))
    dpsi = to_device(psi, dtype=dtype)
    v = psi.data.astype(dtype).astype(np.complex128)  # the state the device holds

    def ref_apply(op, u):
        return OR.mul(Q.Ket(b, np.zeros(len(b), np.complex128)), op, Q.Ket(b, u), 1.0, 0.0)

    for op in (H, A):
        x = ref_apply(op, v)
        z = ref_apply(op, x)
        ref = np.vdot(v, z) - np.vdot(v, x) ** 2
        got = variance(op, dpsi)
        # relative to the two terms of the difference (<op^2>, <op>^2)
        scale = abs(np.vdot(v, z)) + abs(np.vdot(v, x)) ** 2
        assert abs(got - ref) <= tol * scale, (op, got, ref)
    var_h = variance(H, dpsi)
    assert abs(var_h.imag) <= tol * abs(var_h.real)

    # errors relative to |op psi| (the state is normalised)
    for index, f in ((2, O.sigmaz(b.bases[1])), (3, O.number(b.bases[2]))):
        x = ref_apply(O.LazyTensor(b, b, (index,), (f,)), v)
        ref = np.vdot(v, x)
        assert abs(expect(index, f, dpsi) - ref) <= tol * np.linalg.norm(x), (index, ref)


@pytest.mark.parametrize("dtype,tol", [(np.complex128, TOL64), (np.complex64, TOL32)])
def test_expect_on_density_operators(dtype, tol):
    """expect(op, rho) = sum_ij op[i,j] rho[j,i] (src/operators_dense.jl:223-230,
    src/operators_sparse.jl:36-46) for a LazySum, its sparse form and a
    non-Hermitian dense operator, on a random density operator, also held with a
    leading dimension larger than its rows; against the oracle's mul! of the
    operator on rho's columns and the trace summed on the host."""
    import torch

    from qobgpu.mul import expect, to_device

    H = jaynes_cummings(7, 7)  # 128 x 128
    b = H.basis_r
    n = len(b)
    rho = random_density_columns(n, n, rank=16, seed=151)
    rng = Q.Rng(152)
    ops = (H, O.sparse(H), rand_op(rng, b, b))
    held = rho.astype(dtype).astype(np.complex128)  # what the device holds
    R = O.Operator(b, b, np.asfortranarray(held))
    drho = to_device(O.Operator(b, b, rho), dtype=dtype)
    # the same matrix inside a larger allocation: leading dimension n + 5
    tdt = torch.complex64 if dtype == np.complex64 else torch.complex128
    big = torch.zeros((n + 5) * n, dtype=tdt, device="cuda:0")
    view = big.as_strided((n, n), (1, n + 5))
    view.copy_(drho.data)
    dview = O.Operator(b, b, view)
    for op in ops:
        t = OR.mul(O.Operator(b, b, np.zeros((n, n), np.complex128, order="F")), op, R, 1.0, 0.0)
        ref = np.trace(t)
        scale = np.sum(np.abs(np.diag(t)))
        for state in (drho, dview):
            got = expect(op, state)
            assert abs(got - ref) <= tol * scale, (op, got, ref)
    # a Hermitian operator on a density operator: real
    got = expect(H, drho)
    assert abs(got.imag) <= tol * abs(got.real)


@pytest.mark.parametrize("dtype,tol", [(np.complex128, TOL64), (np.complex64, TOL32)])
def test_expect_on_a_density_operator_in_column_blocks(dtype, tol):
    """expect(op, rho) on dim 8192 (Jaynes-Cummings, FockBasis(63) x spin x
    FockBasis(63)): rho is larger than the 256 MiB workspace, so op is applied
    to 2 (ComplexF32) or 4 (ComplexF64) blocks of its columns.  rho = V V^dagger
    of rank 4 is formed on the device; the reference is sum_k <v_k|op v_k> with
    the oracle's mul! (tr(op V V^dagger) = sum_k v_k^dagger op v_k)."""
    import torch

    from qobgpu.mul import expect

    H = jaynes_cummings(63, 63, seed=3)
    b = H.basis_r
    n = len(b)
    rng = Q.Rng(171)
    V = rng.kets_data(n, 4) / 2.0
    tdt = torch.complex64 if dtype == np.complex64 else torch.complex128
    Vd = torch.as_tensor(V.astype(dtype), device="cuda:0")
    rho = (Vd @ Vd.conj().t()).t().contiguous().t()  # column-major n x n
    held = V.astype(dtype).astype(np.complex128)
    ref, scale = 0j, 0.0
    for k in range(4):
        v = np.ascontiguousarray(held[:, k])
        hv = OR.mul(Q.Ket(b, np.zeros(n, np.complex128)), H, Q.Ket(b, v), 1.0, 0.0)
        ref += np.vdot(v, hv)
        scale += np.linalg.norm(v) * np.linalg.norm(hv)
    got = expect(H, O.Operator(b, b, rho))
    assert rho.dtype == tdt
    assert abs(got - ref) <= tol * scale, (got, ref)


@pytest.mark.parametrize("dtype,tol", [(np.complex128, TOL64), (np.complex64, TOL32)])
def test_variance_on_density_operators(dtype, tol):
    """variance(op, rho) = tr(op op rho) - tr(op rho)^2 and variance(index, op,
    rho) on a composite basis (FockBasis(7) x SpinBasis(1/2) x FockBasis(7)):
    the device applies op to rho's columns into a column-major workspace X, then
    takes tr(op X) and tr(op rho); against the oracle's two mul! of op on rho's
    columns and the traces summed on the host."""
    from qobgpu.mul import to_device, variance

    H = jaynes_cummings(7, 7)
    b = H.basis_r
    n = len(b)
    rho = random_density_columns(n, n, rank=12, seed=161)
    held = rho.astype(dtype).astype(np.complex128)  # what the device holds
    R = O.Operator(b, b, np.asfortranarray(held))
    drho = to_device(O.Operator(b, b, rho), dtype=dtype)
    A = O.LazySum(b, b, (1.0, 0.3j - 0.5), (H, O.LazyTensor(b, b, (1,), (O.destroy(b.bases[0]),))))

    def ref_variance(op):
        zero = O.Operator(b, b, np.zeros((n, n), np.complex128, order="F"))
        X = OR.mul(zero, op, R, 1.0, 0.0)
        Z = OR.mul(zero, op, O.Operator(b, b, np.asfortranarray(X)), 1.0, 0.0)
        t1, t2 = np.trace(Z), np.trace(X)
        return t1 - t2 ** 2, abs(t1) + abs(t2) ** 2  # value, scale of the two terms

    for op in (H, A, O.sparse(H)):
        ref, scale = ref_variance(op)
        got = variance(op, drho)
        assert abs(got - ref) <= tol * scale, (op, got, ref)
    got = variance(H, drho)  # Hermitian op, density operator: real
    assert abs(got.imag) <= tol * abs(got.real)
    for index, f in ((2, O.sigmax(b.bases[1])), (3, O.number(b.bases[2]))):
        ref, scale = ref_variance(O.LazyTensor(b, b, (index,), (f,)))
        got = variance(index, f, drho)
        assert abs(got - ref) <= tol * scale, (index, got, ref)


@pytest.mark.parametrize("ncols", [1, 3, 13])
def test_dense_operator_split_columns(ncols):
    """A 700 x 500 DenseOperator (split over column ranges with an ordered
    reduction of the partial sums) on kets from the left and on rows of an
    operator from the right, complex beta."""
    rng = Q.Rng(130 + ncols)
    bl, br = Q.GenericBasis(700), Q.GenericBasis(500)
    D = rand_op(rng, bl, br)
    X = O.Operator(br, Q.GenericBasis(ncols), rng.kets_data(500, ncols))
    Y = O.Operator(bl, Q.GenericBasis(ncols), rng.kets_data(700, ncols))
    check(Y, D, X, AL, 0.4 - 0.9j, TOL64)
    check(Y, D, X, AL, 0.4 - 0.9j, TOL32, np.complex64)
    R = O.Operator(Q.GenericBasis(ncols), bl, np.asfortranarray(rng.complex_normal(ncols * 700).reshape(ncols, 700, order="F")))
    Z = O.Operator(Q.GenericBasis(ncols), br, np.asfortranarray(rng.complex_normal(ncols * 500).reshape(ncols, 500, order="F")))
    check(Z, R, D, AL, 0.4 - 0.9j, TOL64)
