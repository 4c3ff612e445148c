"""Bases: the shape metadata of QuantumOpticsBase.jl / QuantumInterface.

Only what the operator-application path needs: a basis knows its shape, and a
composite basis lists its sub-bases with the first subsystem fastest in the
linear index (``tensor(a::Ket, b::Ket) = kron(b.data, a.data)``,
src/states.jl:105; ``_comp_size``, src/operators_lazytensor.jl:517-518).
"""
from __future__ import annotations

from fractions import Fraction
from math import pi, prod


class Basis:
    """Abstract basis; ``shape`` is a tuple of subsystem lengths."""

    shape: tuple = ()

    def __len__(self) -> int:
        return int(prod(self.shape))

    @property
    def length(self) -> int:
        return len(self)

    def _key(self):
        return (type(self).__name__, self.shape)

    def __eq__(self, other) -> bool:
        return isinstance(other, Basis) and self._key() == other._key()

    def __hash__(self) -> int:
        return hash(self._key())

    def __repr__(self) -> str:
        return f"{type(self).__name__}{self.shape}"

    # b1 ⊗ b2 is written b1 @ b2 in Python (and tensor(b1, b2)).
    def __matmul__(self, other: "Basis") -> "CompositeBasis":
        return tensor(self, other)

    def __pow__(self, n: int) -> "CompositeBasis":
        return tensor(*([self] * n))


class GenericBasis(Basis):
    def __init__(self, N: int):
        self.N = int(N)
        self.shape = (self.N,)


class NLevelBasis(Basis):
    def __init__(self, N: int):
        self.N = int(N)
        self.shape = (self.N,)


class FockBasis(Basis):
    """Fock space truncated at photon number N, starting at ``offset``."""

    def __init__(self, N: int, offset: int = 0):
        if offset < 0 or N < offset:
            raise ValueError("FockBasis requires 0 <= offset <= N")
        self.N = int(N)
        self.offset = int(offset)
        self.shape = (self.N - self.offset + 1,)

    def _key(self):
        return ("FockBasis", self.N, self.offset)


class SpinBasis(Basis):
    """Spin-s basis with 2s+1 states, ordered m = s, s-1, ..., -s."""

    def __init__(self, spinnumber):
        s = Fraction(spinnumber)
        if s <= 0 or (2 * s).denominator != 1:
            raise ValueError("spin number must be a positive multiple of 1/2")
        self.spinnumber = s
        self.shape = (int(2 * s + 1),)

    def _key(self):
        return ("SpinBasis", self.spinnumber)


class PositionBasis(Basis):
    """Real-space grid of N points x_i = xmin + i (xmax - xmin) / N, i = 0 .. N-1
    (QuantumInterface's PositionBasis; spacing / samplepoints, src/particle.jl:70-96).
    ``PositionBasis(b::MomentumBasis)`` is the grid the FFT pairs with b."""

    def __init__(self, xmin, xmax=None, N=None):
        if isinstance(xmin, MomentumBasis):
            b = xmin
            dp = (b.pmax - b.pmin) / b.N
            xmin, xmax, N = -pi / dp, pi / dp, b.N
        self.xmin, self.xmax, self.N = float(xmin), float(xmax), int(N)
        self.shape = (self.N,)

    def _key(self):
        return ("PositionBasis", self.xmin, self.xmax, self.N)


class MomentumBasis(Basis):
    """Momentum grid of N points p_i = pmin + i (pmax - pmin) / N;
    ``MomentumBasis(b::PositionBasis)`` is the grid the FFT pairs with b."""

    def __init__(self, pmin, pmax=None, N=None):
        if isinstance(pmin, PositionBasis):
            b = pmin
            dx = (b.xmax - b.xmin) / b.N
            pmin, pmax, N = -pi / dx, pi / dx, b.N
        self.pmin, self.pmax, self.N = float(pmin), float(pmax), int(N)
        self.shape = (self.N,)

    def _key(self):
        return ("MomentumBasis", self.pmin, self.pmax, self.N)


def spacing(b) -> float:
    """(src/particle.jl:70-82)"""
    if isinstance(b, PositionBasis):
        return (b.xmax - b.xmin) / b.N
    if isinstance(b, MomentumBasis):
        return (b.pmax - b.pmin) / b.N
    raise TypeError("spacing of a PositionBasis or MomentumBasis")


def samplepoints(b):
    """(src/particle.jl:84-96): [min + i * spacing for i = 0 .. N-1]."""
    d = spacing(b)
    lo = b.xmin if isinstance(b, PositionBasis) else b.pmin
    return [lo + i * d for i in range(b.N)]


class CompositeBasis(Basis):
    def __init__(self, bases):
        self.bases = tuple(bases)
        self.shape = tuple(len(b) for b in self.bases)

    def _key(self):
        return ("CompositeBasis", tuple(b._key() for b in self.bases))

    def __repr__(self) -> str:
        return " ⊗ ".join(repr(b) for b in self.bases)


def tensor(*bases: Basis) -> CompositeBasis:
    """Composite basis; nested composites are flattened (QuantumInterface's tensor)."""
    out = []
    for b in bases:
        if isinstance(b, CompositeBasis):
            out.extend(b.bases)
        else:
            out.append(b)
    return CompositeBasis(out)


def comp_size(b: Basis) -> tuple:
    """``_comp_size`` (src/operators_lazytensor.jl:517-518)."""
    if isinstance(b, CompositeBasis):
        return tuple(len(x) for x in b.bases)
    return (len(b),)
