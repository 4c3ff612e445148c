"""Superoperators: ``spre``, ``spost``, ``sprepost``, ``liouvillian``
(src/superoperators.jl:10-240) and their application to density operators.

A superoperator acts on vec(rho), the column-major vectorisation of an
N x N operator (row index fastest), so ``S * rho`` is one matrix-vector
product of length N^2 -- the same device path as ``mul!`` on a ket.

Two forms:

* ``SuperOperator`` holds the reference's materialised matrix
  (``spre(A).data == kron(I, A)``, ``spost(A).data == kron(transpose(A), I)``,
  ``sprepost(A, B).data == kron(transpose(B), A)``); the device applies it as
  a sparse (or dense) operator on vec(rho), as the reference's
  ``a.data * reshape(b.data, ...)`` (:82-85) does on the CPU.
* ``LazySuperOperator`` keeps the same map unmaterialised: a LazySum on the
  doubled composite basis (the subsystems of rho's rows, then those of its
  columns), where ``spre(T)`` is T on the row subsystems and ``spost(T)`` is
  transpose(T) on the column subsystems.  ``lazy_liouvillian(H, J)`` builds
  ``-i H rho + i rho H + sum_ij r_ij (J_i rho J_j^dag - 1/2 {J_j^dag J_i, rho})``
  this way from LazySum / LazyTensor Hamiltonians and jump operators, and the
  fused gather applies all of it in one pass over rho.
"""
from __future__ import annotations

import numbers

import numpy as np
import scipy.sparse as sp

from . import operators as O
from .bases import Basis, CompositeBasis, GenericBasis


class AbstractSuperOperator:
    basis_l: tuple
    basis_r: tuple


def _pair_len(bs) -> int:
    return len(bs[0]) * len(bs[1])


def _data_matrix(d):
    """Sparse (csc) or dense (Fortran) matrix of operator data (Eye, Adjoint resolved)."""
    if isinstance(d, O.Adjoint):
        p = d.parent
        if sp.issparse(p) or isinstance(p, O.Eye):
            return O._to_csc(d)
        return O._to_dense_array(d)
    if isinstance(d, O.Eye) or sp.issparse(d):
        return O._to_csc(d)
    return np.asfortranarray(np.asarray(d))


def _kron(a, b):
    if sp.issparse(a) and sp.issparse(b):
        return sp.kron(a, b, format="csc")
    return np.asfortranarray(np.kron(a.toarray() if sp.issparse(a) else a, b.toarray() if sp.issparse(b) else b))


def _transpose(a):
    return a.T.tocsc() if sp.issparse(a) else np.asfortranarray(a.T)


def _identity_like(a, n):
    return sp.identity(n, dtype=a.dtype if a.dtype == np.complex64 else np.complex128, format="csc")


class SuperOperator(AbstractSuperOperator):
    """``SuperOperator(basis_l, basis_r, data)`` (src/superoperators.jl:10-24):
    basis_l and basis_r are pairs (b1, b2); data maps vec of an operator on
    basis_r to vec of an operator on basis_l."""

    def __init__(self, basis_l, basis_r=None, data=None):
        if data is None:  # SuperOperator(b, data)
            basis_r, data = basis_l, basis_r
        basis_l, basis_r = tuple(basis_l), tuple(basis_r)
        if (len(basis_l) != 2 or len(basis_r) != 2 or _pair_len(basis_l) != data.shape[0]
                or _pair_len(basis_r) != data.shape[1]):
            raise O.DimensionMismatch(
                f"Tried to assign data of size {tuple(data.shape)} to Hilbert spaces of sizes "
                f"{tuple(len(b) for b in basis_l)}, {tuple(len(b) for b in basis_r)}")
        self.basis_l = basis_l
        self.basis_r = basis_r
        self.data = data.tocsc() if sp.issparse(data) else np.asfortranarray(np.asarray(data))
        self._vec = None

    @property
    def shape(self):
        return self.data.shape

    @property
    def vectorised(self) -> O.Operator:
        """The operator on vec(rho) the device applies (cached)."""
        if self._vec is None:
            self._vec = O.Operator(GenericBasis(self.data.shape[0]), GenericBasis(self.data.shape[1]), self.data)
        return self._vec

    def _same(self, other):
        if self.basis_l != other.basis_l or self.basis_r != other.basis_r:
            raise O.IncompatibleBases()

    def __mul__(self, other):
        if isinstance(other, numbers.Number):
            return SuperOperator(self.basis_l, self.basis_r, self.data * other)
        if isinstance(other, SuperOperator):
            if self.basis_r != other.basis_l:
                raise O.IncompatibleBases()
            d = self.data @ other.data
            return SuperOperator(self.basis_l, other.basis_r, d.tocsc() if sp.issparse(d) else d)
        if isinstance(other, O.Operator):
            return apply(self, other)
        return NotImplemented

    def __rmul__(self, other):
        if isinstance(other, numbers.Number):
            return self * other
        return NotImplemented

    def __truediv__(self, other):
        if isinstance(other, numbers.Number):
            return SuperOperator(self.basis_l, self.basis_r, self.data / other)
        return NotImplemented

    def __add__(self, other):
        self._same(other)
        d = self.data + other.data
        return SuperOperator(self.basis_l, self.basis_r, d.tocsc() if sp.issparse(d) else np.asarray(d))

    def __sub__(self, other):
        self._same(other)
        d = self.data - other.data
        return SuperOperator(self.basis_l, self.basis_r, d.tocsc() if sp.issparse(d) else np.asarray(d))

    def __neg__(self):
        return SuperOperator(self.basis_l, self.basis_r, -self.data)

    def __eq__(self, other):
        if not isinstance(other, SuperOperator):
            return NotImplemented
        if self.basis_l != other.basis_l or self.basis_r != other.basis_r:
            return False
        a = self.data.toarray() if sp.issparse(self.data) else self.data
        b = other.data.toarray() if sp.issparse(other.data) else other.data
        return bool(np.array_equal(a, b))

    __hash__ = object.__hash__


def DenseSuperOperator(basis_l, basis_r=None, data=None) -> SuperOperator:
    if basis_r is None:
        basis_r = basis_l
    if data is None:
        data = np.zeros((_pair_len(basis_l), _pair_len(basis_r)), np.complex128, order="F")
    return SuperOperator(basis_l, basis_r, np.asfortranarray(data.toarray() if sp.issparse(data) else data))


def SparseSuperOperator(basis_l, basis_r=None, data=None) -> SuperOperator:
    if basis_r is None:
        basis_r = basis_l
    if data is None:
        data = sp.csc_matrix((_pair_len(basis_l), _pair_len(basis_r)), dtype=np.complex128)
    return SuperOperator(basis_l, basis_r, sp.csc_matrix(data))


def dense(s) -> SuperOperator:
    if isinstance(s, LazySuperOperator):
        s = s.materialise()
    return DenseSuperOperator(s.basis_l, s.basis_r, s.data)


def sparse(s) -> SuperOperator:
    if isinstance(s, LazySuperOperator):
        return s.materialise()
    return SparseSuperOperator(s.basis_l, s.basis_r, s.data)


def identitysuperoperator(b: Basis) -> SuperOperator:
    """(src/superoperators.jl:104-105)"""
    n = len(b)
    return SuperOperator((b, b), (b, b), sp.identity(n * n, dtype=np.complex128, format="csc"))


def dagger(s: SuperOperator) -> SuperOperator:
    d = s.data.conj().T
    return SuperOperator(s.basis_r, s.basis_l, d.tocsc() if sp.issparse(d) else np.asfortranarray(d))


def _check_square(op):
    if op.basis_l != op.basis_r:
        raise O.ArgumentError("It's not clear what spre of a non-square operator should be. See issue #113")


def _materialised(op):
    if not isinstance(op, O.Operator):
        raise O.ArgumentError(f"spre/spost of {type(op).__name__}: use lazy_spre / lazy_spost / lazy_liouvillian")
    return _data_matrix(op.data)


def spre(op) -> SuperOperator:
    """``spre(A) * B == A * B``: data kron(I, A) (src/superoperators.jl:129-134)."""
    _check_square(op)
    a = _materialised(op)
    return SuperOperator((op.basis_l, op.basis_l), (op.basis_r, op.basis_r), _kron(_identity_like(a, a.shape[0]), a))


def spost(op) -> SuperOperator:
    """``spost(A) * B == B * A``: data kron(transpose(A), I) (:149-154)."""
    _check_square(op)
    a = _materialised(op)
    return SuperOperator((op.basis_r, op.basis_r), (op.basis_l, op.basis_l),
                         _kron(_transpose(a), _identity_like(a, a.shape[0])))


def sprepost(A, B) -> SuperOperator:
    """``sprepost(A, B) * C == A * C * B``: data kron(transpose(B), A) (:169)."""
    a, b = _materialised(A), _materialised(B)
    return SuperOperator((A.basis_l, B.basis_r), (A.basis_r, B.basis_l), _kron(_transpose(b), a))


def _check_input(H, J, Jdagger, rates):
    """(src/superoperators.jl:171-186); violations raise AssertionError as there."""
    for j in list(J) + list(Jdagger):
        if j.basis_l != H.basis_l or j.basis_r != H.basis_r:
            raise AssertionError("jump operators must act on the Hamiltonian's bases")
    if len(J) != len(Jdagger):
        raise AssertionError("J and Jdagger differ in length")
    r = np.asarray(rates)
    if r.ndim == 2 and not (r.shape[0] == r.shape[1] == len(J)):
        raise AssertionError("rates matrix must be length(J) x length(J)")
    if r.ndim == 1 and r.shape[0] != len(J):
        raise AssertionError("rates vector must have length(J) entries")


def liouvillian(H, J, rates=None, Jdagger=None) -> SuperOperator:
    """``liouvillian(H, J; rates, Jdagger)`` (src/superoperators.jl:205-225), materialised:
    ``S rho = -i[H, rho] + sum_i r_i (J_i rho J_i^dag - 1/2 J_i^dag J_i rho - 1/2 rho J_i^dag J_i)``."""
    J = list(J)
    rates = np.ones(len(J)) if rates is None else rates
    Jdagger = [O.dagger(j) for j in J] if Jdagger is None else list(Jdagger)
    _check_input(H, J, Jdagger, rates)
    L = spre(O.scale(H, -1j)) + spost(O.scale(H, 1j))
    r = np.asarray(rates)
    pairs = ([(i, j, r[i, j]) for i in range(len(J)) for j in range(len(J))] if r.ndim == 2
             else [(i, i, r[i]) for i in range(len(J))])
    for i, j, rij in pairs:
        jdj = O.scale(O.multiply(Jdagger[j], J[i]), rij / 2)
        L = L - (spre(jdj) + spost(jdj))
        L = L + spre(O.scale(J[i], rij)) * spost(Jdagger[j])
    return L


# ---------------------------------------------------------------------------
# lazy form: a LazySum on the doubled basis
# ---------------------------------------------------------------------------


class _Composite(Exception):
    """A term acts on the whole of a composite basis (not site by site)."""


def _csc(op):
    return O._to_csc(op.data if isinstance(op, O.Operator) else O.sparse(op).data)


def _site_terms(op, nsites):
    """op as a list of (coefficient, 0-based sorted sites, csc factors)."""
    op = O.static_operator(op)
    if isinstance(op, O.LazySum):
        out = []
        for f, t in zip(op.factors, op.operators):
            out += [(complex(f) * c, s, m) for c, s, m in _site_terms(t, nsites)]
        return out
    if isinstance(op, O.LazyTensor):
        sites, mats = [], []
        for i, o in sorted(zip(op.indices, op.operators), key=lambda p: p[0]):
            sites.append(i - 1)
            mats.append(_csc(o))
        return [(complex(op.factor), tuple(sites), tuple(mats))]
    if isinstance(op, O.Operator):
        if nsites != 1:
            raise _Composite()
        return [(1.0 + 0j, (0,), (_csc(op),))]
    if isinstance(op, O.LazyProduct):
        if nsites != 1:
            raise _Composite()
        return [(1.0 + 0j, (0,), (_csc(O.sparse(op)),))]
    raise O.ArgumentError(f"no lazy superoperator form for {type(op).__name__}")


def _product(a, b, dims):
    """Site-wise product of two site terms a * b (identity on the sites one lacks)."""
    ca, sa, ma = a
    cb, sb, mb = b
    da, db = dict(zip(sa, ma)), dict(zip(sb, mb))
    sites = tuple(sorted(set(sa) | set(sb)))
    mats = []
    for s in sites:
        x = da.get(s)
        y = db.get(s)
        if x is None:
            mats.append(y)
        elif y is None:
            mats.append(x)
        else:
            mats.append((x @ y).tocsc())
    return (ca * cb, sites, tuple(mats))


class LazySuperOperator(AbstractSuperOperator):
    """A superoperator kept as a LazySum on the doubled basis (rows, then columns)."""

    def __init__(self, basis: Basis, operator: O.LazySum):
        self.basis_l = (basis, basis)
        self.basis_r = (basis, basis)
        self.operator = operator

    @property
    def vectorised(self) -> O.LazySum:
        return self.operator

    @property
    def shape(self):
        n = len(self.basis_l[0]) ** 2
        return (n, n)

    def materialise(self) -> SuperOperator:
        return SuperOperator(self.basis_l, self.basis_r, O.sparse(self.operator).data)

    def __mul__(self, other):
        if isinstance(other, O.Operator):
            return apply(self, other)
        return NotImplemented


def _lazy_from_terms(b: Basis, nsites: int, site_bases, terms) -> LazySuperOperator:
    """LazySum on the doubled basis from (coefficient, doubled sites, csc factors) terms."""
    dbl = CompositeBasis(list(site_bases) * 2)
    factors, ops = [], []
    for c, sites, mats in terms:
        if c == 0:
            continue
        facs = tuple(O.Operator(site_bases[s % nsites], site_bases[s % nsites], m) for s, m in zip(sites, mats))
        ops.append(O.LazyTensor(dbl, dbl, tuple(s + 1 for s in sites), facs))
        factors.append(c)
    return LazySuperOperator(b, O.LazySum(dbl, dbl, np.asarray(factors, np.complex128), tuple(ops)))


def _split(b: Basis, ops):
    """Site bases and site terms of every operator; falls back to one site (the
    whole basis) when some operator is not site-wise."""
    if isinstance(b, CompositeBasis):
        try:
            sb = list(b.bases)
            return sb, [_site_terms(o, len(sb)) for o in ops]
        except _Composite:
            pass
    g = GenericBasis(len(b))
    return [g], [[(1.0 + 0j, (0,), (_csc(O.sparse(o) if not isinstance(o, O.Operator) else o),))] for o in ops]


def _shift(term, n, transpose=False):
    c, sites, mats = term
    return (c, tuple(s + n for s in sites), tuple(m.T.tocsc() for m in mats) if transpose else mats)


def _join(a, b):
    """Term a on the row sites times term b on the column sites (disjoint)."""
    return (a[0] * b[0], a[1] + b[1], a[2] + b[2])


def lazy_spre(op) -> LazySuperOperator:
    _check_square(op)
    sb, (t,) = _split(op.basis_l, [op])
    return _lazy_from_terms(op.basis_l, len(sb), sb, t)


def lazy_spost(op) -> LazySuperOperator:
    _check_square(op)
    sb, (t,) = _split(op.basis_l, [op])
    n = len(sb)
    return _lazy_from_terms(op.basis_l, n, sb, [_shift(x, n, True) for x in t])


def lazy_liouvillian(H, J, rates=None, Jdagger=None) -> LazySuperOperator:
    """The Liouvillian of ``liouvillian(H, J; rates, Jdagger)`` as a LazySum on the
    doubled basis: spre(-iH) + spost(iH) + sum_ij r_ij (spre(J_i) spost(Jdag_j)
    - 1/2 spre(Jdag_j J_i) - 1/2 spost(Jdag_j J_i)); every product is formed site
    by site, so the terms stay LazyTensors of local factors."""
    J = list(J)
    rates = np.ones(len(J)) if rates is None else rates
    Jdagger = [O.dagger(j) for j in J] if Jdagger is None else list(Jdagger)
    _check_input(H, J, Jdagger, rates)
    _check_square(H)
    b = H.basis_l
    sb, split = _split(b, [H] + J + Jdagger)
    n = len(sb)
    dims = [len(x) for x in sb]
    tH, tJ, tJd = split[0], split[1:1 + len(J)], split[1 + len(J):]
    terms = []
    for c, s, m in tH:
        terms.append((-1j * c, s, m))                       # spre(-iH)
        terms.append(_shift((1j * c, s, m), n, True))       # spost(iH)
    r = np.asarray(rates)
    pairs = ([(i, j, r[i, j]) for i in range(len(J)) for j in range(len(J))] if r.ndim == 2
             else [(i, i, r[i]) for i in range(len(J))])
    for i, j, rij in pairs:
        if rij == 0:
            continue
        for a in tJ[i]:
            for d in tJd[j]:
                terms.append(_join((rij * a[0], a[1], a[2]), _shift(d, n, True)))  # J_i rho Jdag_j
                jd = _product(d, a, dims)                                           # Jdag_j J_i
                terms.append((-0.5 * rij * jd[0], jd[1], jd[2]))
                terms.append(_shift((-0.5 * rij * jd[0], jd[1], jd[2]), n, True))
    return _lazy_from_terms(b, n, sb, terms)


# ---------------------------------------------------------------------------
# application
# ---------------------------------------------------------------------------


def _vec(a):
    """vec of column-major operator data (a view: numpy Fortran order or a torch (1, N) strided tensor)."""
    if type(a).__module__.startswith("torch"):
        if a.ndim == 2 and (a.stride(0) != 1 or (a.shape[1] > 1 and a.stride(1) != a.shape[0])):
            raise O.ArgumentError("device operator data must be contiguous column-major")
        return a.t().reshape(-1) if a.ndim == 2 else a
    if not a.flags.f_contiguous:
        raise O.ArgumentError("host operator data must be Fortran-ordered")
    return a.reshape(-1, order="F")


def mul_super(result: O.Operator, s, rho: O.Operator, alpha=1.0, beta=0.0):
    """In place vec(result) = alpha * S vec(rho) + beta * vec(result), on the device."""
    from .mul import mul_
    from .states import Ket

    if tuple(s.basis_r) != (rho.basis_l, rho.basis_r):
        raise O.IncompatibleBases()
    if tuple(s.basis_l) != (result.basis_l, result.basis_r):
        raise O.IncompatibleBases()
    v = s.vectorised
    x, y = _vec(rho.data), _vec(result.data)
    mul_(Ket(v.basis_l, y), v, Ket(v.basis_r, x), alpha, beta)
    return result


def apply(s, rho: O.Operator) -> O.Operator:
    """``S * rho`` (src/superoperators.jl:82-85): a new operator on basis_l."""
    d = rho.data
    if type(d).__module__.startswith("torch"):
        import torch

        out = torch.zeros((len(s.basis_l[1]), len(s.basis_l[0])), dtype=d.dtype, device=d.device).t()
    else:
        out = np.zeros((len(s.basis_l[0]), len(s.basis_l[1])), dtype=np.complex64 if d.dtype == np.complex64
                       else np.complex128, order="F")
    res = O.Operator(s.basis_l[0], s.basis_l[1], out)
    return mul_super(res, s, rho)


__all__ = [
    "AbstractSuperOperator", "SuperOperator", "DenseSuperOperator", "SparseSuperOperator", "LazySuperOperator",
    "spre", "spost", "sprepost", "liouvillian", "lazy_spre", "lazy_spost", "lazy_liouvillian",
    "identitysuperoperator", "dagger", "dense", "sparse", "mul_super", "apply",
]
