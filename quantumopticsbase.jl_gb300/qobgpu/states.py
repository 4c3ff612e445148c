"""Ket and Bra state vectors (src/states.jl:11-32).

``data`` is either a host numpy vector or a CUDA ``torch.Tensor`` (device
resident).  Device-resident states are what the GPU path keeps in HBM between
applications; host states are copied in and out around each call.
"""
from __future__ import annotations

import numbers

import numpy as np

from .bases import Basis
from .operators import DimensionMismatch


def _length(data) -> int:
    return int(data.shape[0]) if data.ndim == 1 else -1


class StateVector:
    def __init__(self, basis: Basis, data=None, dtype=np.complex128):
        if data is None:
            data = np.zeros(len(basis), dtype=dtype)
        if isinstance(data, (list, tuple)):
            data = np.asarray(data, dtype=dtype)
        if data.ndim != 1 or _length(data) != len(basis):
            raise DimensionMismatch(
                f"Tried to assign data of length {tuple(data.shape)} to Hilbert space of size {len(basis)}"
            )
        self.basis = basis
        self.data = data

    @property
    def on_device(self) -> bool:
        return not isinstance(self.data, np.ndarray)

    def copy(self):
        d = self.data.copy() if isinstance(self.data, np.ndarray) else self.data.clone()
        return type(self)(self.basis, d)

    def to_host(self) -> np.ndarray:
        return self.data if isinstance(self.data, np.ndarray) else self.data.cpu().numpy()

    def __len__(self):
        return len(self.basis)

    def __repr__(self):
        where = "device" if self.on_device else "host"
        return f"{type(self).__name__}({self.basis!r}, {where})"


class Ket(StateVector):
    """``Ket(b, data)``."""

    def __rmul__(self, other):
        if isinstance(other, numbers.Number):
            return Ket(self.basis, other * self.data)
        return NotImplemented


class Bra(StateVector):
    """``Bra(b, data)``."""

    def __mul__(self, other):
        from .operators import AbstractOperator

        if isinstance(other, AbstractOperator):
            from .mul import apply_alloc_bra

            return apply_alloc_bra(self, other)
        if isinstance(other, numbers.Number):
            return Bra(self.basis, other * self.data)
        return NotImplemented


def dagger_state(x: StateVector) -> StateVector:
    """``dagger(x::Ket) = Bra(x.basis, conj(x.data))`` (src/states.jl:94-95)."""
    d = x.data.conj()
    if not isinstance(d, np.ndarray):
        d = d.resolve_conj()
    return (Bra if isinstance(x, Ket) else Ket)(x.basis, d)


def tensor_states(*states: StateVector) -> StateVector:
    """``tensor(a::Ket, b::Ket) = Ket(a.basis ⊗ b.basis, kron(b.data, a.data))`` (src/states.jl:105)."""
    from .bases import tensor as tb

    data = states[-1].to_host()
    for s in reversed(states[:-1]):
        data = np.kron(data, s.to_host())
    return type(states[0])(tb(*[s.basis for s in states]), data)


def basisstate(b: Basis, indices, dtype=np.complex128) -> Ket:
    """``basisstate(b, indices)`` with 1-based per-subsystem indices
    (``_basisstate_index``, src/states.jl:137-165)."""
    if isinstance(indices, numbers.Integral):
        indices = (indices,)
    lin, stride = 0, 1
    for d, i in zip(b.shape, indices):
        if not (1 <= i <= d):
            raise IndexError("basis state index out of bounds")
        lin += (i - 1) * stride
        stride *= d
    data = np.zeros(len(b), dtype=dtype)
    data[lin] = 1
    return Ket(b, data)


def fockstate(b, n: int, dtype=np.complex128) -> Ket:
    """``fockstate(b, n)``: the Fock state |n> of a FockBasis (src/fock.jl:154-158)."""
    if not (b.offset <= n <= b.N):
        raise AssertionError("b.offset <= n <= b.N")
    return basisstate(b, n - b.offset + 1, dtype)


def coherentstate(b, alpha, dtype=np.complex128) -> Ket:
    """``coherentstate(b, alpha)`` (src/fock.jl:165-196): exp(-|alpha|^2 / 2)
    alpha^n / sqrt(n!) for n = offset ... N by the same recurrence, not
    renormalised after the truncation."""
    alpha = complex(alpha)
    c = np.exp(-abs(alpha) ** 2 / 2) + 0j
    for n in range(1, b.offset + 1):
        c *= alpha / np.sqrt(n)
    data = np.zeros(len(b), dtype=np.complex128)
    data[0] = c
    for n in range(1, b.N - b.offset + 1):
        data[n] = data[n - 1] * alpha / np.sqrt(n + b.offset)
    return Ket(b, data.astype(dtype))


def spinup(b, dtype=np.complex128) -> Ket:
    """``spinup(b) = basisstate(b, 1)`` (src/spin.jl:94)."""
    return basisstate(b, 1, dtype)


def spindown(b, dtype=np.complex128) -> Ket:
    """``spindown(b) = basisstate(b, b.shape[1])`` (src/spin.jl:101)."""
    return basisstate(b, len(b), dtype)


def dm(psi: Ket):
    """``dm(psi) = tensor(psi, dagger(psi))``: the dense density operator |psi><psi|
    (src/operators_dense.jl:291)."""
    from .operators import Operator

    d = psi.to_host()
    return Operator(psi.basis, psi.basis, np.asfortranarray(np.outer(d, d.conj())))
