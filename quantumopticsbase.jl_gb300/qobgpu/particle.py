"""Particle bases and the FFT operator between them (src/particle.jl).

``transform(b1, b2)`` builds the operator that maps a state on a position grid
to the matching momentum grid (or back), exactly as the reference defines it:
a phase vector ``mul_before``, the unnormalised DFT over the transformed
subsystems (FFTW's ``fft!`` for position -> momentum, ``bfft!`` for momentum
-> position, as seen by a ket) and a phase vector ``mul_after`` that includes
1/sqrt(N).  Both phase arrays are Kronecker products of per-axis vectors; the
device keeps the per-axis vectors and runs one FFT pass per axis (csrc/fft.cu).
"""
from __future__ import annotations

import numpy as np

from . import operators as O
from .bases import CompositeBasis, MomentumBasis, PositionBasis, samplepoints, spacing
from .bases import tensor as tensor_bases
from .states import Ket


class FFTOperator(O.AbstractOperator):
    """``FFTOperators`` / ``FFTKets`` (src/particle.jl:196-240).

    axes: transformed subsystems (1-based); sign: the DFT sign a ket sees
    (-1: fft!, +1: bfft!); before / after: one phase vector per axis.
    ``ket_only`` marks the FFTKets variant, which applies to kets only."""

    def __init__(self, basis_l, basis_r, axes, sign, before, after, ket_only=False):
        self.basis_l = basis_l
        self.basis_r = basis_r
        self.axes = tuple(int(a) for a in axes)
        self.sign = -1 if sign < 0 else 1
        self.before = [np.asarray(v, np.complex128) for v in before]
        self.after = [np.asarray(v, np.complex128) for v in after]
        self.ket_only = bool(ket_only)

    @property
    def shape_sub(self):
        return self.basis_l.shape

    def _full(self, vecs):
        """Kronecker product over all subsystems (ones on untransformed ones),
        first subsystem fastest: the reference's mul_before / mul_after."""
        full = np.ones(1, np.complex128)
        per = dict(zip(self.axes, vecs))
        for i, n in enumerate(self.shape_sub, start=1):
            v = per.get(i, np.ones(n, np.complex128))
            full = np.kron(v, full)
        return full

    @property
    def mul_before(self):
        return self._full(self.before)

    @property
    def mul_after(self):
        return self._full(self.after)

    def __repr__(self):
        kind = "FFTKets" if self.ket_only else "FFTOperators"
        return f"{kind}({self.basis_l!r} <- {self.basis_r!r}, axes={self.axes})"


def _check_pair(bx: PositionBasis, bp: MomentumBasis):
    Lx = bx.xmax - bx.xmin
    dp = spacing(bp)
    if bx.N != bp.N or abs(2 * np.pi / dp - Lx) / Lx > 1e-12:
        raise O.IncompatibleBases()


def _px_vectors(bp: MomentumBasis, bx: PositionBasis):
    """momentum <- position (src/particle.jl:248-262): fft!."""
    x = np.asarray(samplepoints(bx))
    p = np.asarray(samplepoints(bp))
    before = np.exp(-1j * bp.pmin * (x - bx.xmin))
    after = np.exp(-1j * bx.xmin * p) / np.sqrt(bx.N)
    return before, after


def _xp_vectors(bx: PositionBasis, bp: MomentumBasis):
    """position <- momentum (:271-285): bfft!."""
    x = np.asarray(samplepoints(bx))
    p = np.asarray(samplepoints(bp))
    before = np.exp(1j * bx.xmin * (p - bp.pmin))
    after = np.exp(1j * bp.pmin * x) / np.sqrt(bp.N)
    return before, after


def transform(basis_l, basis_r, ket_only: bool = False, index=()):
    """``transform(b1, b2; ket_only, index)`` (src/particle.jl:242-420)."""
    if isinstance(basis_l, MomentumBasis) and isinstance(basis_r, PositionBasis):
        _check_pair(basis_r, basis_l)
        b, a = _px_vectors(basis_l, basis_r)
        return FFTOperator(basis_l, basis_r, (1,), -1, [b], [a], ket_only)
    if isinstance(basis_l, PositionBasis) and isinstance(basis_r, MomentumBasis):
        _check_pair(basis_l, basis_r)
        b, a = _xp_vectors(basis_l, basis_r)
        return FFTOperator(basis_l, basis_r, (1,), 1, [b], [a], ket_only)
    if isinstance(basis_l, CompositeBasis) and isinstance(basis_r, CompositeBasis):
        bl, br = basis_l.bases, basis_r.bases
        if len(bl) != len(br):
            raise AssertionError("composite bases of different lengths")
        index = tuple(index)
        if not index:
            pos = [isinstance(b, PositionBasis) for b in bl]
            mom = [isinstance(b, MomentumBasis) for b in bl]
            if any(pos) and not any(mom):
                index = tuple(i + 1 for i, v in enumerate(pos) if v)
            elif any(mom) and not any(pos):
                index = tuple(i + 1 for i, v in enumerate(mom) if v)
            else:
                raise O.IncompatibleBases()
        for i in range(len(bl)):
            if len(bl[i]) != len(br[i]):
                raise O.IncompatibleBases()
        if all(isinstance(bl[i - 1], PositionBasis) for i in index):
            if not all(isinstance(br[i - 1], MomentumBasis) for i in index):
                raise AssertionError("position axes need momentum counterparts")
            vecs = []
            for i in index:
                _check_pair(bl[i - 1], br[i - 1])
                vecs.append(_xp_vectors(bl[i - 1], br[i - 1]))
            sign = 1
        elif all(isinstance(bl[i - 1], MomentumBasis) for i in index):
            if not all(isinstance(br[i - 1], PositionBasis) for i in index):
                raise AssertionError("momentum axes need position counterparts")
            vecs = []
            for i in index:
                _check_pair(br[i - 1], bl[i - 1])
                vecs.append(_px_vectors(bl[i - 1], br[i - 1]))
            sign = -1
        else:
            raise O.IncompatibleBases()
        return FFTOperator(basis_l, basis_r, index, sign, [v[0] for v in vecs], [v[1] for v in vecs], ket_only)
    raise O.IncompatibleBases()


def dagger(op: FFTOperator) -> FFTOperator:
    """``dagger(op) = transform(op.basis_r, op.basis_l)`` (:422-423)."""
    if isinstance(op.basis_l, CompositeBasis):
        return transform(op.basis_r, op.basis_l, op.ket_only, op.axes)
    return transform(op.basis_r, op.basis_l, op.ket_only)


def tensor(a: FFTOperator, b: FFTOperator) -> FFTOperator:
    """(:425-426)"""
    return transform(tensor_bases(a.basis_l, b.basis_l), tensor_bases(a.basis_r, b.basis_r),
                     a.ket_only and b.ket_only)


def gaussianstate(b, x0, p0, sigma, dtype=np.complex128) -> Ket:
    """``gaussianstate(b, x0, p0, sigma)`` (src/particle.jl:45-68)."""
    if isinstance(b, PositionBasis):
        dx = spacing(b)
        alpha = 1.0 / (np.pi ** 0.25 * np.sqrt(sigma)) * np.sqrt(dx)
        x = np.asarray(samplepoints(b))
        data = alpha * np.exp(1j * p0 * (x - x0 / 2) - (x - x0) ** 2 / (2 * sigma ** 2))
    elif isinstance(b, MomentumBasis):
        dp = spacing(b)
        alpha = np.sqrt(sigma) / np.pi ** 0.25 * np.sqrt(dp)
        p = np.asarray(samplepoints(b))
        data = alpha * np.exp(-1j * x0 * (p - p0 / 2) - (p - p0) ** 2 / 2 * sigma ** 2)
    else:
        raise TypeError("gaussianstate needs a PositionBasis or MomentumBasis")
    return Ket(b, data.astype(dtype))


def position(b: PositionBasis, dtype=np.complex128) -> O.Operator:
    """Position operator in real space (src/particle.jl:104-107)."""
    if not isinstance(b, PositionBasis):
        raise TypeError("position in its own basis: PositionBasis")
    d = np.asarray(samplepoints(b), dtype)
    return O.Operator(b, b, O.spdiagm(b.N, b.N, {0: d}, dtype))


def momentum(b: MomentumBasis, dtype=np.complex128) -> O.Operator:
    """Momentum operator in momentum space (src/particle.jl:122-125)."""
    if not isinstance(b, MomentumBasis):
        raise TypeError("momentum in its own basis: MomentumBasis")
    d = np.asarray(samplepoints(b), dtype)
    return O.Operator(b, b, O.spdiagm(b.N, b.N, {0: d}, dtype))


def potentialoperator(b, V, dtype=np.complex128) -> O.Operator:
    """Diagonal potential V(x) on a position grid or a composite of position grids
    (src/particle.jl:143-199, position-space forms)."""
    if isinstance(b, PositionBasis):
        d = np.asarray([V(x) for x in samplepoints(b)], dtype)
        return O.Operator(b, b, O.spdiagm(b.N, b.N, {0: d}, dtype))
    if isinstance(b, CompositeBasis) and all(isinstance(x, PositionBasis) for x in b.bases):
        grids = np.meshgrid(*[np.asarray(samplepoints(x)) for x in b.bases], indexing="ij")
        vals = np.vectorize(V)(*grids).astype(dtype)
        d = vals.reshape(-1, order="F")
        n = len(b)
        return O.Operator(b, b, O.spdiagm(n, n, {0: d}, dtype))
    raise O.IncompatibleBases()


__all__ = ["FFTOperator", "transform", "dagger", "tensor", "gaussianstate", "position", "momentum",
           "potentialoperator"]
