"""CPU tests of the host side: the C-ABI library loads and exports every symbol
the header declares, the seeded generator is stable, and the magic-number
division used by the kernels' index arithmetic is exact."""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"^\s*(?:int|int64_t|const char\*|void)\s+(qob_\w+)\s*\(", txt, re.M))
    return names


def test_library_exports_every_declared_symbol():
    import ctypes

    import __graft_entry__ as g

    g.build()
    from qobgpu import _lib

    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 19
    for n in sorted(names):
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"
    assert set(_lib.SIGNATURES) == names


def test_library_without_gpu_reports_cuda_error_not_crash():
    import ctypes

    import torch
    from qobgpu import _lib

    if torch.cuda.is_available():
        return
    p = ctypes.c_void_p()
    assert _lib.lib().qob_create(ctypes.byref(p), 0, 0) == _lib.QOB_ERR_CUDA


def test_rng_is_stable():
    import qobgpu as Q

    r = Q.Rng(1)
    u = r.uniform(3)
    assert np.allclose(u, Q.Rng(1).uniform(3))
    assert 0 <= u.min() and u.max() < 1
    k = Q.Rng(5).ket_data(64)
    assert abs(np.linalg.norm(k) - 1) < 1e-14


def test_lemire_division_exact():
    """n / d and n % d via M = floor((2^64-1)/d) + 1 (Lemire, Kaser & Kurz 2019),
    as the kernels compute them, for 32-bit n and d > 1."""
    rng = np.random.default_rng(0)
    ds = list(range(2, 70)) + [2 ** k for k in range(1, 31)] + list(rng.integers(2, 2 ** 31, 200))
    ns = list(range(0, 300)) + [2 ** 31 - 1, 2 ** 32 - 1] + list(rng.integers(0, 2 ** 32, 300))
    for d in ds:
        d = int(d)
        M = (2 ** 64 - 1) // d + 1
        for n in ns:
            n = int(n)
            q = (M * n) >> 64
            low = (M * n) & (2 ** 64 - 1)
            r = (low * d) >> 64
            assert q == n // d and r == n % d, (n, d)


def test_dtype_codes_and_double_float_argument_checks():
    """The Python side maps numpy dtypes and the "ff" arithmetic to the C ABI's
    codes and refuses double-float arithmetic on ComplexF32 data before any
    library call."""
    import pytest

    from qobgpu import _lib as L
    from qobgpu import operators as O
    from qobgpu.device import dtype_code
    from qobgpu.mul import _code

    assert dtype_code(np.complex128) == L.QOB_C128 == 0
    assert dtype_code(np.complex64) == L.QOB_C64 == 1
    assert dtype_code("ff") == L.QOB_C128X == 2
    assert _code(np.complex128, None) == L.QOB_C128
    assert _code(np.complex128, "ff") == L.QOB_C128X
    assert _code(np.complex64, None) == L.QOB_C64
    with pytest.raises(O.ArgumentError):
        _code(np.complex64, "ff")
    with pytest.raises(O.ArgumentError):
        _code(np.complex128, "fp16")


def test_reference_flop_count_of_the_heisenberg_chain():
    """bench.py's count of the reference's term-by-term arithmetic: 53 Pauli
    product terms, each touching every one of the 2^14 rows once, 8 flops per
    complex multiply-add, plus the beta scaling: 8 * 54 * 16384."""
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from qobgpu.hamiltonians import heisenberg_chain

    H = heisenberg_chain(14, seed=3)
    assert len(H.operators) == 53
    assert bench.reference_flops(H) == 8 * 54 * 16384


def test_subsystem_expect_argument_checks():
    """expect(index, op, psi) refuses an index outside the composite basis, an
    operator on another subsystem's basis and a state on a simple basis before
    any device call (src/operators_sparse.jl:49-55)."""
    import pytest

    import qobgpu as Q
    from qobgpu import operators as O
    from qobgpu.mul import expect

    bf, bs = Q.FockBasis(3), Q.SpinBasis("1/2")
    b = Q.tensor_basis(bf, bs)
    psi = Q.Ket(b, np.zeros(len(b), np.complex128))
    with pytest.raises(AssertionError):
        expect(3, O.sigmaz(bs), psi)
    with pytest.raises(O.IncompatibleBases):
        expect(1, O.sigmaz(bs), psi)
    with pytest.raises(O.ArgumentError):
        expect(1, O.sigmaz(bs), Q.Ket(bs, np.zeros(2, np.complex128)))
    with pytest.raises(TypeError):
        expect(O.sigmaz(bs))


def test_density_expect_argument_checks():
    """expect(op, rho) refuses a density operator on other bases and host data
    before any device call."""
    import pytest

    import qobgpu as Q
    from qobgpu import operators as O
    from qobgpu.mul import expect

    b2, b3 = Q.GenericBasis(2), Q.GenericBasis(3)
    op = O.Operator(b2, b2, np.eye(2, dtype=np.complex128, order="F"))
    with pytest.raises(O.IncompatibleBases):
        expect(op, O.Operator(b3, b3, np.eye(3, dtype=np.complex128, order="F")))
    with pytest.raises(O.ArgumentError):
        expect(op, O.Operator(b2, b2, np.eye(2, dtype=np.complex128, order="F")))


def test_ket_expect_and_variance_argument_checks():
    """expect(op, psi) and variance(op, psi) take a Ket on the operator's basis;
    a Bra or another basis is refused before any device call."""
    import pytest

    import qobgpu as Q
    from qobgpu import operators as O
    from qobgpu.mul import expect, variance

    b2, b3 = Q.GenericBasis(2), Q.GenericBasis(3)
    op = O.Operator(b2, b2, np.eye(2, dtype=np.complex128, order="F"))
    for f in (expect, variance):
        with pytest.raises(O.ArgumentError):
            f(op, Q.Bra(b2, np.zeros(2, np.complex128)))
        with pytest.raises(O.IncompatibleBases):
            f(op, Q.Ket(b3, np.zeros(3, np.complex128)))


def test_expect_variance_forms_compose_as_the_reference(monkeypatch):
    """The host front end of expect / variance (test/test_operators.jl:52-60):
    subsystem forms equal the embedded operator's, lists of states give lists,
    and variance on a density operator is tr(op op rho) - tr(op rho)^2.  The
    device calls are replaced by numpy here (the GPU tests run the real ones)."""
    import torch

    import qobgpu as Q
    import qobgpu.mul as M
    from qobgpu import operators as O

    def dense(op):
        return np.asarray(O.dense(op).data)

    def host(d):
        return d.cpu().numpy() if hasattr(d, "cpu") else np.asarray(d)

    def reduce_op(name, op, psi):
        v = host(psi.data)
        x = dense(op) @ v
        if name == "qob_expect":
            return complex(np.vdot(v, x))
        return complex(np.vdot(v, dense(op) @ x) - np.vdot(v, x) ** 2)

    def expect_dm(op, rho):
        return complex(np.trace(dense(op) @ host(rho.data)))

    def mul(result, a, b, alpha=1.0, beta=0.0, **kw):
        result.data.copy_(torch.from_numpy(alpha * dense(a) @ host(b.data)))
        return result

    monkeypatch.setattr(M, "_reduce_op", reduce_op)
    monkeypatch.setattr(M, "_expect_dm", expect_dm)
    monkeypatch.setattr(M, "mul_", mul)

    rng = Q.Rng(77)
    b1, b2 = Q.FockBasis(3), Q.SpinBasis("1/2")
    b = Q.tensor_basis(b1, b2)
    n = len(b)
    op1 = O.Operator(b1, b1, np.asfortranarray(rng.complex_normal(16).reshape(4, 4)))
    emb = O.embed(b, b, 1, op1)
    psi = Q.Ket(b, rng.ket_data(n))
    A = rng.complex_normal(n * n).reshape(n, n)
    rho_np = A @ A.conj().T
    rho_np /= np.trace(rho_np)
    rho = O.Operator(b, b, torch.from_numpy(np.ascontiguousarray(rho_np.T)).t())  # column-major

    for f in (M.expect, M.variance):
        assert abs(f(1, op1, rho) - f(emb, rho)) < 1e-12
        assert abs(f(1, op1, psi) - f(emb, psi)) < 1e-12
        assert f(emb, [rho, rho]) == [f(emb, rho)] * 2
        assert f(1, op1, [rho, psi]) == [f(1, op1, rho), f(1, op1, psi)]
    # time-dependent operators at their current time (test/test_time_dependent_operators.jl:40-47)
    o = O.TimeDependentSum((lambda t: 2.0 * t,), (emb,), init_time=1.0)
    subo = O.TimeDependentSum((lambda t: 2.0,), (op1,))
    op1x2 = O.Operator(b1, b1, np.asfortranarray(2.0 * op1.data))
    emb2 = O.embed(b, b, 1, op1x2)
    for f in (M.expect, M.variance):
        for st in (psi, rho):
            assert abs(f(o, st) - f(emb2, st)) < 1e-12
            assert abs(f(1, subo, st) - f(1, op1x2, st)) < 1e-12
    D = dense(emb)
    want = np.trace(D @ D @ rho_np) - np.trace(D @ rho_np) ** 2
    assert abs(M.variance(emb, rho) - want) < 1e-12
    v = psi.data
    want = np.vdot(v, D @ D @ v) - np.vdot(v, D @ v) ** 2
    assert abs(M.variance(1, op1, psi) - want) < 1e-12
