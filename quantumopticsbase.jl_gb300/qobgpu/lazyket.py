"""``LazyKet``: a tensor product of kets kept as its factors
(src/states_lazyket.jl), with expectation values of lazy operators computed on
the device -- for one state or for many product states in one launch
(``expect_batch``).

Arithmetic runs in libqobgpu's kernels: norms through ``qob_norm``, site
applications through ``qob_mul``, expectation values through
``qob_expect_lazyket``; host data are copied to the device for the call.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import operators as O
from .bases import CompositeBasis
from .device import dtype_code, get_context, handle, raise_for
from .states import Ket, tensor_states


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


class LazyKet:
    """``LazyKet(b, kets)`` (src/states_lazyket.jl:12-25): b a CompositeBasis,
    kets one Ket per subsystem (assertion errors as in the reference)."""

    def __init__(self, basis: CompositeBasis, kets):
        kets = tuple(kets)
        if not isinstance(basis, CompositeBasis):
            raise TypeError("LazyKet needs a CompositeBasis")
        if len(kets) != len(basis.bases):
            raise AssertionError("one ket per subsystem")
        for k, b in zip(kets, basis.bases):
            if not isinstance(k, Ket):
                raise AssertionError("LazyKet factors must be Kets")
            if k.basis != b:
                raise AssertionError("ket basis differs from the subsystem basis")
        self.basis = basis
        self.kets = kets

    @property
    def dtype(self):
        return np.result_type(*[_dt(k.data) for k in self.kets])

    def __eq__(self, other):
        if not isinstance(other, LazyKet) or self.basis != other.basis:
            return False
        return all(np.array_equal(_host(a.data), _host(b.data)) for a, b in zip(self.kets, other.kets))

    __hash__ = object.__hash__

    def to_ket(self) -> Ket:
        """``Ket(ket::LazyKet) = ⊗(ket.kets...)`` (:35)."""
        return tensor_states(*[Ket(k.basis, _host(k.data)) for k in self.kets])

    def __repr__(self):
        return f"LazyKet({self.basis!r}, {len(self.kets)} kets)"


def _dt(a):
    if _is_torch(a):
        import torch

        return np.complex64 if a.dtype == torch.complex64 else np.complex128
    return np.complex64 if a.dtype == np.complex64 else np.complex128


def _host(a):
    return a.detach().cpu().numpy() if _is_torch(a) else np.asarray(a)


def tensor(x, y) -> LazyKet:
    """tensor of LazyKets and Kets (:40-48)."""
    xs = x.kets if isinstance(x, LazyKet) else (x,)
    ys = y.kets if isinstance(y, LazyKet) else (y,)
    from .bases import tensor as tensor_bases

    return LazyKet(tensor_bases(x.basis, y.basis), xs + ys)


def _device_ket(k: Ket, device: int, dtype):
    import torch

    d = k.data
    if _is_torch(d):
        t = d.to(device=f"cuda:{device}")
    else:
        t = torch.as_tensor(np.ascontiguousarray(d), device=f"cuda:{device}")
    t = t.to(torch.complex64 if dtype == np.complex64 else torch.complex128).contiguous()
    return Ket(k.basis, t)


def norm(state: LazyKet, device: int = 0) -> float:
    """``norm(state) = prod(norm.(kets))`` (:51), each norm in FP64 on the device."""
    from .mul import norm as knorm

    out = 1.0
    for k in state.kets:
        out *= knorm(_device_ket(k, device, _dt(k.data)))
    return out


def normalize_(state: LazyKet, device: int = 0) -> LazyKet:
    """``normalize!`` (:52-57): every site ket scaled by 1/norm on the device."""
    from .mul import mul_, norm as knorm

    kets = []
    for k in state.kets:
        dk = _device_ket(k, device, _dt(k.data))
        n = knorm(dk)
        src = Ket(k.basis, dk.data.clone())
        mul_(dk, O.identityoperator(k.basis), src, 1.0 / n, 0.0)
        if _is_torch(k.data):
            k.data.copy_(dk.data)
        else:
            k.data[...] = dk.data.cpu().numpy()
        kets.append(k)
    return state


def normalize(state: LazyKet, device: int = 0) -> LazyKet:
    y = LazyKet(state.basis, [Ket(k.basis, k.data.clone() if _is_torch(k.data) else np.array(k.data))
                              for k in state.kets])
    return normalize_(y, device)


def mul_(y: LazyKet, op: O.LazyTensor, x: LazyKet, alpha=1.0, beta=0.0, device: int = 0) -> LazyKet:
    """``mul!(y::LazyKet, op::LazyTensor, x::LazyKet, alpha, beta)`` (:131-150): each
    site ket with a factor is that factor times x's site ket, the others are
    copies, and the first site is scaled by op.factor * alpha.  beta must be 0."""
    from .mul import mul_ as kmul

    if beta != 0:
        raise O.ArgumentError("cannot perform muladd operation on LazyKets since addition is not implemented")
    if not isinstance(op, O.LazyTensor):
        raise O.ArgumentError("mul! on LazyKets needs a LazyTensor")
    if len(y.basis.bases) != len(x.basis.bases):
        raise O.IncompatibleBases()
    square = op.basis_l == op.basis_r
    facs = dict(zip(op.indices, op.operators))
    for i, (yk, xk) in enumerate(zip(y.kets, x.kets), start=1):
        scale = complex(op.factor) * complex(alpha) if i == 1 else 1.0
        if i in facs:
            f = facs[i]
        else:
            if not square:
                raise O.ArgumentError("a missing index needs the same bases on both sides")
            f = O.identityoperator(xk.basis)
        dy = _device_ket(yk, device, _dt(yk.data))
        kmul(dy, f, _device_ket(xk, device, _dt(yk.data)), scale, 0.0)
        if _is_torch(yk.data):
            yk.data.copy_(dy.data)
        else:
            yk.data[...] = dy.data.cpu().numpy()
    return y


def expect_batch(op, basis: CompositeBasis, states, result=None):
    """Expectation values of ``op`` on many product states in one launch.

    ``states``: CUDA tensor of shape (nstates, sum of the site lengths), each
    row the concatenated site kets of one state; returns a complex128 CUDA
    tensor of nstates values (or fills ``result``)."""
    import torch

    dims = np.asarray(basis.shape, np.int64)
    if states.ndim != 2 or states.shape[1] != int(dims.sum()):
        raise O.DimensionMismatch("states must be (nstates, sum of site dimensions)")
    if not states.is_contiguous():
        raise O.ArgumentError("states must be contiguous")
    dev = states.device.index
    ctx = get_context(dev)
    h = handle(ctx, op)
    if result is None:
        result = torch.empty(states.shape[0], dtype=torch.complex128, device=states.device)
    dt = np.complex64 if states.dtype == torch.complex64 else np.complex128
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    raise_for(L.lib().qob_expect_lazyket(ctx.ptr, h.ptr, dtype_code(dt), len(dims), dims.ctypes.data_as(L.I64P),
                                         C.c_void_p(states.data_ptr()), states.shape[0],
                                         C.c_void_p(result.data_ptr()), s), ctx)
    return result


def expect(op, state: LazyKet, device: int = 0) -> complex:
    """``expect(op, state::LazyKet)`` (:64-125) for a LazyTensor, LazySum or LazyProduct."""
    import torch

    if getattr(op, "basis_l", None) != state.basis or getattr(op, "basis_r", None) != state.basis:
        raise O.IncompatibleBases()
    dt = state.dtype
    tdt = torch.complex64 if dt == np.complex64 else torch.complex128
    row = torch.cat([_device_ket(k, device, dt).data.to(tdt) for k in state.kets]).reshape(1, -1)
    return complex(expect_batch(op, state.basis, row).cpu().numpy()[0])


__all__ = ["LazyKet", "tensor", "norm", "normalize", "normalize_", "mul_", "expect", "expect_batch"]
