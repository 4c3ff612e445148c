"""``mul_`` -- the reference's 5-argument ``mul!(result, a, b, alpha, beta)``.

Dispatch follows the reference:
* ``mul_(::Ket, op, ::Ket, α, β)``            op applied from the left to a ket
* ``mul_(::Bra, ::Bra, op, α, β)``            a bra times op
* ``mul_(::Operator, op, ::Operator, α, β)``  op times a dense operator (its columns)
* ``mul_(::Operator, ::Operator, op, α, β)``  a dense operator times op (its rows)

States whose data are CUDA ``torch`` tensors stay on the device (the path an
ODE right-hand side uses); numpy data are copied to the device and back
around the call.  Every call runs the CUDA kernels of libqobgpu.so; there is
no host arithmetic on this path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import operators as O
from .bases import CompositeBasis
from .device import dtype_code, get_context, handle, raise_for
from .states import Bra, Ket, StateVector


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _state_like(o) -> bool:
    return isinstance(o, O.Operator) and (isinstance(o.data, np.ndarray) or _is_torch(o.data))


def _np_dtype(a):
    if _is_torch(a):
        import torch

        return np.complex64 if a.dtype == torch.complex64 else np.complex128
    return np.complex64 if a.dtype == np.complex64 else np.complex128


def _stream_ptr(device: int):
    import torch

    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _matrix_view(a):
    """(rows, cols, ld) of a 1-D or column-major 2-D array/tensor."""
    if a.ndim == 1:
        return a.shape[0], 1, max(1, a.shape[0])
    r, c = a.shape
    if _is_torch(a):
        st = a.stride()
        if st[0] != 1 and r > 1:
            raise O.ArgumentError("device operator data must be column-major (stride (1, ld))")
        return r, c, max(1, st[1] if c > 1 else r)
    if not a.flags.f_contiguous:
        raise O.ArgumentError("host operator data must be Fortran-ordered")
    return r, c, max(1, r)


def _classify(result, a, b):
    """(side, is_vector, op, x, y)"""
    if isinstance(b, StateVector):
        if not isinstance(b, Ket) or not isinstance(result, Ket):
            raise O.ArgumentError("mul_(result::Ket, op, b::Ket) expected")
        if result.basis != a.basis_l or b.basis != a.basis_r:
            raise O.IncompatibleBases()
        return L.QOB_LEFT, True, a, b.data, result.data
    if isinstance(a, StateVector):
        if not isinstance(a, Bra) or not isinstance(result, Bra):
            raise O.ArgumentError("mul_(result::Bra, a::Bra, op) expected")
        if a.basis != b.basis_l or result.basis != b.basis_r:
            raise O.IncompatibleBases()
        return L.QOB_RIGHT, True, b, a.data, result.data
    if not isinstance(result, O.Operator) or not _state_like(result):
        raise O.ArgumentError("result must be an Operator with dense data")
    if a.basis_r != b.basis_l or result.basis_l != a.basis_l or result.basis_r != b.basis_r:
        raise O.IncompatibleBases()
    # the dense data operand is the state; the other one is applied to it
    if _state_like(b) or not _state_like(a):
        return L.QOB_LEFT, False, a, b.data, result.data
    return L.QOB_RIGHT, False, b, a.data, result.data


def _code(ydt, arith):
    if arith is None:
        return dtype_code(ydt)
    if arith != "ff" or ydt != np.complex128:
        raise O.ArgumentError('arith="ff" (double-float) applies to ComplexF64 data')
    return L.QOB_C128X


def mul_(result, a, b, alpha=1.0, beta=0.0, device: int | None = None, arith: str | None = None):
    """In place ``result = alpha * a * b + beta * result``; returns ``result``.
    ``arith="ff"``: ComplexF64 data, the fused LazySum part in double-float
    arithmetic on the FP32 pipes (about 1e-14 relative; QOB_C128X)."""
    side, is_vec, op, x, y = _classify(result, a, b)
    alpha, beta = complex(alpha), complex(beta)
    lib = L.lib()
    if _is_torch(y):
        import torch

        dev = y.device.index if device is None else device
        ctx = get_context(dev)
        h = handle(ctx, op)
        ydt = _np_dtype(y)
        if not _is_torch(x) or x.device != y.device or _np_dtype(x) != ydt:
            xt = torch.as_tensor(np.asarray(x) if not _is_torch(x) else x, device=y.device)
            x = xt.to(torch.complex64 if ydt == np.complex64 else torch.complex128)
            if x.ndim == 2 and x.stride(0) != 1 and x.shape[0] > 1:
                x = x.t().contiguous().t()
        xr, xc, xld = _matrix_view(x)
        yr, yc, yld = _matrix_view(y)
        if side == L.QOB_RIGHT and x.ndim == 1:
            xr, xc, xld = 1, x.shape[0], 1
            yr, yc, yld = 1, y.shape[0], 1
        rc = lib.qob_mul(ctx.ptr, side, int(is_vec), h.ptr, _code(ydt, arith), alpha.real, alpha.imag,
                         C.c_void_p(x.data_ptr()), xr, xc, xld, beta.real, beta.imag, C.c_void_p(y.data_ptr()),
                         yr, yc, yld, _stream_ptr(dev))
        raise_for(rc, ctx)
        return result
    # host arrays: copy in, apply on the device, copy back
    dev = 0 if device is None else device
    ctx = get_context(dev)
    h = handle(ctx, op)
    ydt = _np_dtype(y)
    xh = np.asfortranarray(np.asarray(x.detach().cpu().numpy() if _is_torch(x) else x), dtype=ydt)
    if not (isinstance(y, np.ndarray) and (y.flags.f_contiguous or y.ndim == 1)):
        raise O.ArgumentError("host result data must be a Fortran-ordered numpy array")
    if side == L.QOB_LEFT:
        xr, xc = (xh.shape[0], 1) if xh.ndim == 1 else xh.shape
        yr, yc = (y.shape[0], 1) if y.ndim == 1 else y.shape
    else:
        xr, xc = (1, xh.shape[0]) if xh.ndim == 1 else xh.shape
        yr, yc = (1, y.shape[0]) if y.ndim == 1 else y.shape
    rc = lib.qob_mul_host(ctx.ptr, side, int(is_vec), h.ptr, _code(ydt, arith), alpha.real, alpha.imag,
                          xh.ctypes.data_as(C.c_void_p), xr, xc, beta.real, beta.imag, y.ctypes.data_as(C.c_void_p),
                          yr, yc)
    raise_for(rc, ctx)
    return result


def apply_alloc(op, psi: Ket) -> Ket:
    """``op * psi`` (src/operators_dense.jl:111-115): allocate, then mul_."""
    if _is_torch(psi.data):
        import torch

        out = torch.zeros(len(op.basis_l), dtype=psi.data.dtype, device=psi.data.device)
    else:
        out = np.zeros(len(op.basis_l), dtype=_np_dtype(psi.data))
    return mul_(Ket(op.basis_l, out), op, psi)


def apply_alloc_bra(psi: Bra, op) -> Bra:
    if _is_torch(psi.data):
        import torch

        out = torch.zeros(len(op.basis_r), dtype=psi.data.dtype, device=psi.data.device)
    else:
        out = np.zeros(len(op.basis_r), dtype=_np_dtype(psi.data))
    return mul_(Bra(op.basis_r, out), psi, op)


def to_device(obj, device: int = 0, dtype=None):
    """Copy of a Ket/Bra/Operator(dense) with column-major CUDA tensor data."""
    import torch

    d = obj.data
    a = d.detach().cpu().numpy() if _is_torch(d) else O._to_dense_array(d) if isinstance(obj, O.Operator) else d
    if dtype is not None:
        a = a.astype(dtype)
    t = torch.as_tensor(np.ascontiguousarray(a.T) if a.ndim == 2 else np.ascontiguousarray(a),
                        device=f"cuda:{device}")
    if a.ndim == 2:
        t = t.t()  # column-major view of shape (m, n)
    if isinstance(obj, O.Operator):
        return O.Operator(obj.basis_l, obj.basis_r, t)
    return type(obj)(obj.basis, t)


def _vec_ptr(x):
    if _is_torch(x):
        if not x.is_contiguous():
            raise O.ArgumentError("device state must be contiguous")
        return C.c_void_p(x.data_ptr()), x.device.index
    raise O.ArgumentError("norm/dot/expect on the device need CUDA tensor data")


def norm(psi: StateVector) -> float:
    """FP64 norm (src/states.jl:89), accumulated in double even for ComplexF32 data."""
    p, dev = _vec_ptr(psi.data)
    ctx = get_context(dev)
    out = (C.c_double * 1)()
    raise_for(L.lib().qob_norm(ctx.ptr, dtype_code(_np_dtype(psi.data)), p, psi.data.shape[0], out,
                               _stream_ptr(dev)), ctx)
    return out[0]


def dot(x: StateVector, y: StateVector) -> complex:
    """sum(conj(x) .* y) in FP64."""
    px, dev = _vec_ptr(x.data)
    py, _ = _vec_ptr(y.data)
    ctx = get_context(dev)
    out = (C.c_double * 2)()
    raise_for(L.lib().qob_dot(ctx.ptr, dtype_code(_np_dtype(x.data)), px, py, x.data.shape[0], out,
                              _stream_ptr(dev)), ctx)
    return complex(out[0], out[1])


def _state_basis(state):
    """The composite basis a subsystem index refers to: a ket's basis, or a
    density operator's (left = right) basis."""
    if isinstance(state, O.Operator):
        if state.basis_l != state.basis_r:
            raise O.IncompatibleBases()
        return state.basis_l
    return state.basis


def _site_operator(index, op, state):
    """LazyTensor(basis, index, op) for the subsystem forms of expect and
    variance, with the reference's checks (src/operators_sparse.jl:49-55)."""
    b = _state_basis(state)
    if not isinstance(b, CompositeBasis):
        raise O.ArgumentError("a subsystem expectation value needs a state on a composite basis")
    if not 1 <= int(index) <= len(b.bases):  # check_indices, as LazyTensor's constructor
        raise AssertionError("index out of range")
    site = b.bases[int(index) - 1]
    if op.basis_l != site or op.basis_r != site:
        raise O.IncompatibleBases("the operator's bases differ from the subsystem's")
    if not isinstance(op, O.Operator):  # a lazy subsystem operator: its (small) sparse form
        op = O.sparse(op)
    return O.LazyTensor(b, b, (int(index),), (op,))


def _reduce_op(name, op, psi) -> complex:
    """qob_expect / qob_variance on a device ket."""
    if not isinstance(psi, Ket):  # the reference defines these for kets (a MethodError otherwise)
        raise O.ArgumentError("expect / variance of an operator take a Ket (or a density operator)")
    if not (op.basis_l == op.basis_r == psi.basis):
        raise O.IncompatibleBases()
    p, dev = _vec_ptr(psi.data)
    ctx = get_context(dev)
    h = handle(ctx, op)
    out = (C.c_double * 2)()
    fn = getattr(L.lib(), name)
    raise_for(fn(ctx.ptr, h.ptr, dtype_code(_np_dtype(psi.data)), p, psi.data.shape[0], out, _stream_ptr(dev)), ctx)
    return complex(out[0], out[1])


def _expect_dm(op, rho) -> complex:
    """tr(op rho) for a density operator with device data (src/operators_dense.jl:223-230)."""
    if not (op.basis_l == op.basis_r == rho.basis_l == rho.basis_r):
        raise O.IncompatibleBases()
    d = rho.data
    if not _is_torch(d):
        raise O.ArgumentError("expect(op, rho) on the device needs CUDA tensor data")
    r, c, ld = _matrix_view(d)
    if r != c:
        raise O.DimensionMismatch("a density operator is square")
    dev = d.device.index
    ctx = get_context(dev)
    h = handle(ctx, op)
    out = (C.c_double * 2)()
    raise_for(L.lib().qob_expect_dm(ctx.ptr, h.ptr, dtype_code(_np_dtype(d)), C.c_void_p(d.data_ptr()), r, ld, out,
                                    _stream_ptr(dev)), ctx)
    return complex(out[0], out[1])


def _variance_dm(op, rho) -> complex:
    """variance(op, rho) = expect(op * op, rho) - expect(op, rho)^2, the generic
    form for density operators (QuantumInterface, a dependency outside the
    reference tree): X = op rho on the device, then tr(op X) - tr(op rho)^2."""
    if not (op.basis_l == op.basis_r == rho.basis_l == rho.basis_r):
        raise O.IncompatibleBases()
    d = rho.data
    if not _is_torch(d):
        raise O.ArgumentError("variance(op, rho) on the device needs CUDA tensor data")
    n = d.shape[0]
    X = O.Operator(rho.basis_l, rho.basis_r, d.new_zeros((n, n)).t())  # column-major
    mul_(X, op, rho, 1.0, 0.0)
    return _expect_dm(op, X) - _expect_dm(op, rho) ** 2


def _split_args(name, args):
    """(index or None, op, state) of f(op, state) / f(index, op, state)."""
    if len(args) == 3:
        return args
    if len(args) == 2:
        return (None,) + tuple(args)
    raise TypeError(f"{name}(op, state) or {name}(index, op, state)")


def expect(*args):
    """``expect(op, psi) = <psi|op|psi>`` (src/operators.jl:119) in FP64;
    ``expect(op, rho) = tr(op rho)`` for a density operator (src/operators_dense.jl:223-230,
    src/operators_sparse.jl:36-46); ``expect(index, op, state)``: op on
    subsystem ``index`` of a composite state, applied as
    ``LazyTensor(basis, index, op)`` (src/operators_sparse.jl:49-61); a list of
    states gives the list of values (test/test_operators.jl:54-55)."""
    index, op, state = _split_args("expect", args)
    op = O.static_operator(op)  # a TimeDependentSum at its current time (src/time_dependent_operator.jl:76-81)
    if isinstance(state, (list, tuple)):
        return [expect(op, s) if index is None else expect(index, op, s) for s in state]
    if index is not None:
        op = _site_operator(index, op, state)
    if isinstance(state, O.Operator):
        return _expect_dm(op, state)
    return _reduce_op("qob_expect", op, state)


def variance(*args):
    """``variance(op, psi) = <psi|op (op psi)> - <psi|op psi>^2``
    (src/operators.jl:139-142): two applications of op on the device and two
    FP64 inner products; ``variance(op, rho)`` for a density operator;
    ``variance(index, op, state)`` with op on subsystem ``index``, equal to the
    variance of the embedded operator (test/test_operators.jl:57-58); a list of
    states gives the list of values (:59-60)."""
    index, op, state = _split_args("variance", args)
    op = O.static_operator(op)
    if isinstance(state, (list, tuple)):
        return [variance(op, s) if index is None else variance(index, op, s) for s in state]
    if index is not None:
        op = _site_operator(index, op, state)
    if isinstance(state, O.Operator):
        return _variance_dm(op, state)
    return _reduce_op("qob_variance", op, state)
