"""Operator types of QuantumOpticsBase.jl's operator-application path.

The Python mirror keeps the reference's names, fields and argument meaning:

* ``Operator(basis_l, basis_r, data)`` (src/operators_dense.jl:12-20) with data a
  dense column-major matrix (``DenseOperator``), a CSC sparse matrix
  (``SparseOperator``, src/operators_sparse.jl:5-7), an ``Eye`` (FillArrays,
  src/operators_sparse.jl:86-88) or an ``Adjoint`` of one of those.
* ``LazyTensor(basis_l, basis_r, indices, operators, factor)`` with 1-based,
  sorted ``indices`` (src/operators_lazytensor.jl:15-36).
* ``LazySum(basis_l, basis_r, factors, operators)`` (src/operators_lazysum.jl:41-71).
* ``LazyProduct(operators, factor)`` (src/operators_lazyproduct.jl:33-58).
* ``TimeDependentSum`` (src/time_dependent_operator.jl:103-146, 162-171).

Host data lives in numpy / scipy; the GPU library receives copies through its
C ABI when an operator is first applied on the device.
"""
from __future__ import annotations

import numbers
from math import prod

import numpy as np
import scipy.sparse as sp

from .bases import Basis, CompositeBasis, FockBasis, SpinBasis, comp_size
from .bases import tensor as tensor_bases


class DimensionMismatch(ValueError):
    """Julia's ``DimensionMismatch``."""


class IncompatibleBases(ValueError):
    """QuantumInterface's ``IncompatibleBases``."""


class ArgumentError(ValueError):
    """Julia's ``ArgumentError``."""


# ---------------------------------------------------------------------------
# data containers
# ---------------------------------------------------------------------------


class Eye:
    """FillArrays ``Eye{T}(m, n)``: ones on the main diagonal, truncated."""

    def __init__(self, m: int, n: int | None = None, dtype=np.complex128):
        self.m = int(m)
        self.n = int(m if n is None else n)
        self.dtype = np.dtype(dtype)

    @property
    def shape(self):
        return (self.m, self.n)

    def toarray(self) -> np.ndarray:
        return np.eye(self.m, self.n, dtype=self.dtype)


class Adjoint:
    """Lazy conjugate transpose of a dense, sparse or Eye matrix (Julia's ``Adjoint``)."""

    def __init__(self, parent):
        self.parent = parent

    @property
    def shape(self):
        m, n = self.parent.shape
        return (n, m)

    @property
    def dtype(self):
        return self.parent.dtype

    def toarray(self) -> np.ndarray:
        return np.conj(_to_dense_array(self.parent)).T.copy(order="F")


def _to_dense_array(d) -> np.ndarray:
    if isinstance(d, np.ndarray):
        return d
    if sp.issparse(d):
        return d.toarray(order="F")
    if isinstance(d, (Eye, Adjoint)):
        return d.toarray()
    if hasattr(d, "cpu"):  # torch tensor
        return d.cpu().numpy()
    raise TypeError(f"unsupported operator data {type(d)}")


def _to_csc(d) -> sp.csc_matrix:
    if sp.issparse(d):
        return d.tocsc()
    if isinstance(d, Eye):
        k = min(d.m, d.n)
        return sp.csc_matrix(
            (np.ones(k, d.dtype), np.arange(k, dtype=np.int64), np.r_[np.arange(k + 1), np.full(d.n - k, k)]),
            shape=(d.m, d.n),
        )
    if isinstance(d, Adjoint):
        return _to_csc(d.parent).conj().T.tocsc()
    return sp.csc_matrix(_to_dense_array(d))


def spdiagm(m: int, n: int, diags: dict, dtype=np.complex128) -> sp.csc_matrix:
    """``SparseArrays.spdiagm(k => v, ...)`` keeping every given entry as stored
    (numerical zeros included), CSC with rows ascending in each column."""
    rows, cols, vals = [], [], []
    for k, v in diags.items():
        v = np.asarray(v, dtype=dtype)
        i = np.arange(len(v))
        r, c = (i, i + k) if k >= 0 else (i - k, i)
        rows.append(r)
        cols.append(c)
        vals.append(v)
    rows = np.concatenate(rows) if rows else np.zeros(0, np.int64)
    cols = np.concatenate(cols) if cols else np.zeros(0, np.int64)
    vals = np.concatenate(vals) if vals else np.zeros(0, dtype)
    order = np.lexsort((rows, cols))
    rows, cols, vals = rows[order], cols[order], vals[order]
    indptr = np.zeros(n + 1, np.int64)
    np.add.at(indptr, cols + 1, 1)
    indptr = np.cumsum(indptr)
    return sp.csc_matrix((vals, rows.astype(np.int64), indptr), shape=(m, n))


# ---------------------------------------------------------------------------
# operator types
# ---------------------------------------------------------------------------


class AbstractOperator:
    basis_l: Basis
    basis_r: Basis

    @property
    def shape(self):
        return (len(self.basis_l), len(self.basis_r))

    def size(self):
        return self.shape

    # arithmetic shared by all operators
    def __mul__(self, other):
        from .states import Ket

        if isinstance(other, numbers.Number):
            return scale(self, other)
        if isinstance(other, Ket):
            from .mul import apply_alloc

            return apply_alloc(self, other)
        if isinstance(other, AbstractOperator):
            return multiply(self, other)
        return NotImplemented

    def __rmul__(self, other):
        if isinstance(other, numbers.Number):
            return scale(self, other)
        return NotImplemented

    def __truediv__(self, other):
        if isinstance(other, numbers.Number):
            return scale(self, 1.0 / other)
        return NotImplemented

    def __add__(self, other):
        return add(self, other)

    def __sub__(self, other):
        return add(self, scale(other, -1))

    def __neg__(self):
        return scale(self, -1)

    def dagger(self):
        return dagger(self)


class Operator(AbstractOperator):
    """``Operator{BL,BR,T}`` (src/operators_dense.jl:12-20)."""

    def __init__(self, basis_l: Basis, basis_r: Basis | None = None, data=None):
        if data is None:  # Operator(b, data)
            basis_r, data = basis_l, basis_r
        self.basis_l = basis_l
        self.basis_r = basis_r
        if isinstance(data, np.ndarray) and data.ndim == 2 and not data.flags.f_contiguous:
            data = np.asfortranarray(data)
        self.data = data
        if tuple(data.shape) != (len(basis_l), len(basis_r)):
            raise DimensionMismatch(
                f"Tried to assign data of size {tuple(data.shape)} to bases of length "
                f"{len(basis_l)} and {len(basis_r)}!"
            )

    @property
    def dtype(self):
        d = self.data
        if hasattr(d, "dtype"):
            dt = d.dtype
            return np.dtype(str(dt).replace("torch.", "")) if not isinstance(dt, np.dtype) else dt
        return np.dtype(np.complex128)

    @property
    def kind(self) -> str:
        """'dense' | 'sparse' | 'eye' | 'dense_adj' | 'sparse_adj' | 'eye_adj' | 'device'."""
        d = self.data
        if isinstance(d, Adjoint):
            p = d.parent
            if isinstance(p, Eye):
                return "eye_adj"
            return "sparse_adj" if sp.issparse(p) else "dense_adj"
        if isinstance(d, Eye):
            return "eye"
        if sp.issparse(d):
            return "sparse"
        if isinstance(d, np.ndarray):
            return "dense"
        return "device"

    def __repr__(self):
        return f"Operator({self.basis_l!r} -> {self.basis_r!r}, {self.kind})"


def DenseOperator(basis_l, basis_r=None, data=None) -> Operator:
    if data is None and basis_r is not None and not isinstance(basis_r, Basis):
        basis_r, data = basis_l, basis_r
    if basis_r is None:
        basis_r = basis_l
    if data is None:
        data = np.zeros((len(basis_l), len(basis_r)), np.complex128, order="F")
    if isinstance(data, AbstractOperator):
        return Operator(data.basis_l, data.basis_r, np.asfortranarray(dense(data).data))
    return Operator(basis_l, basis_r, np.asfortranarray(_to_dense_array(data)))


def SparseOperator(basis_l, basis_r=None, data=None) -> Operator:
    if isinstance(basis_l, AbstractOperator):
        return sparse(basis_l)
    if data is None and basis_r is not None and not isinstance(basis_r, Basis):
        basis_r, data = basis_l, basis_r
    if basis_r is None:
        basis_r = basis_l
    if data is None:
        data = sp.csc_matrix((len(basis_l), len(basis_r)), dtype=np.complex128)
    return Operator(basis_l, basis_r, _to_csc(data))


def identityoperator(b1: Basis, b2: Basis | None = None, dtype=np.complex128) -> Operator:
    """``identityoperator(T, b1, b2)`` -> Operator with Eye data (src/operators_sparse.jl:180-186)."""
    b2 = b1 if b2 is None else b2
    return Operator(b1, b2, Eye(len(b1), len(b2), dtype))


class LazyTensor(AbstractOperator):
    """``LazyTensor(basis_l, basis_r, indices, operators, factor)``.

    ``indices`` are 1-based subsystem numbers and must be sorted
    (src/operators_lazytensor.jl:15-36).
    """

    def __init__(self, basis_l, basis_r=None, indices=None, operators=None, factor=None):
        if not isinstance(basis_r, Basis):  # LazyTensor(basis, indices, operators[, factor])
            basis_l, basis_r, indices, operators, factor = basis_l, basis_l, basis_r, indices, operators
        if not isinstance(basis_l, CompositeBasis):
            basis_l = CompositeBasis([basis_l])
        if not isinstance(basis_r, CompositeBasis):
            basis_r = CompositeBasis([basis_r])
        if isinstance(indices, numbers.Integral):
            indices = (indices,)
        if isinstance(operators, AbstractOperator):
            operators = (operators,)
        indices = tuple(int(i) for i in indices)
        operators = tuple(operators)
        N = len(basis_l.bases)
        if N != len(basis_r.bases):
            raise AssertionError("basis_l and basis_r have different numbers of subsystems")
        if len(indices) != len(operators):
            raise AssertionError("indices and operators have different lengths")
        if list(indices) != sorted(indices) or len(set(indices)) != len(indices):
            raise AssertionError("indices must be sorted and unique")
        for i, op in zip(indices, operators):
            if not (1 <= i <= N):
                raise AssertionError("index out of range")
            if not isinstance(op, AbstractOperator):
                raise AssertionError("LazyTensor factors must be operators")
            if op.basis_l != basis_l.bases[i - 1] or op.basis_r != basis_r.bases[i - 1]:
                raise AssertionError("factor bases do not match the composite basis")
        self.basis_l = basis_l
        self.basis_r = basis_r
        self.indices = indices
        self.operators = operators
        self.factor = complex(1.0 if factor is None else factor)

    def __repr__(self):
        return f"LazyTensor(indices={self.indices}, factor={self.factor})"


class LazySum(AbstractOperator):
    """``LazySum([basis_l, basis_r,] [factors,] operators)`` (src/operators_lazysum.jl:41-71)."""

    def __init__(self, *args):
        if len(args) >= 2 and isinstance(args[0], Basis):
            basis_l, basis_r = args[0], args[1]
            if len(args) == 2:
                factors, ops = (), ()
            elif len(args) == 3:
                ops = tuple(args[2])
                factors = np.ones(len(ops))
            else:
                factors, ops = args[2], args[3]
        elif len(args) == 2 and not isinstance(args[0], AbstractOperator):
            factors, ops = args
            basis_l, basis_r = ops[0].basis_l, ops[0].basis_r
        else:
            ops = args[0] if len(args) == 1 and isinstance(args[0], (tuple, list)) else args
            if len(ops) == 0:
                raise ArgumentError("LazySum needs a basis, or at least one operator!")
            factors = np.ones(len(ops))
            basis_l, basis_r = ops[0].basis_l, ops[0].basis_r
        ops = tuple(ops)
        factors = np.asarray(factors, dtype=np.complex128).copy()
        if len(ops) != len(factors):
            raise ArgumentError("LazySum `operators` and `factors` have different lengths.")
        for o in ops:
            if o.basis_l != basis_l or o.basis_r != basis_r:
                raise IncompatibleBases()
        self.basis_l = basis_l
        self.basis_r = basis_r
        self.factors = factors
        self.operators = ops
        self._version = 0

    def set_factors(self, factors):
        """Rewrite the factors in place (what ``set_time!`` does to a TimeDependentSum)."""
        f = np.asarray(factors, dtype=np.complex128)
        if f.shape != self.factors.shape:
            raise ArgumentError("wrong number of factors")
        self.factors[:] = f
        self._version += 1

    def __repr__(self):
        return f"LazySum({len(self.operators)} terms)"


class LazyProduct(AbstractOperator):
    """``LazyProduct(operators, factor)`` (src/operators_lazyproduct.jl:33-58)."""

    def __init__(self, *ops, factor=1.0):
        if len(ops) == 1 and isinstance(ops[0], (tuple, list)):
            ops = tuple(ops[0])
        if len(ops) == 0:
            raise ArgumentError("LazyProduct needs at least one operator!")
        for a, b in zip(ops[:-1], ops[1:]):
            if a.basis_r != b.basis_l:
                raise IncompatibleBases()
        self.operators = tuple(ops)
        self.factor = complex(factor)
        self.basis_l = ops[0].basis_l
        self.basis_r = ops[-1].basis_r

    def __repr__(self):
        return f"LazyProduct({len(self.operators)} factors, factor={self.factor})"


class TimeDependentSum(AbstractOperator):
    """``TimeDependentSum(coefficients, operators)`` wrapping a LazySum
    (src/time_dependent_operator.jl:103-146).  ``set_time(t)`` rewrites the
    static operator's factors (``update_static_coefficients!``, :279-290)."""

    def __init__(self, coefficients, operators, init_time=0.0):
        self.coefficients = tuple(coefficients)
        self.static_op = LazySum(np.ones(len(operators)), tuple(operators))
        self.basis_l = self.static_op.basis_l
        self.basis_r = self.static_op.basis_r
        self.current_time = None
        self.set_time(init_time)

    def set_time(self, t: float):
        if t == self.current_time:
            return self
        self.current_time = t
        vals = [c(t) if callable(c) else c for c in self.coefficients]
        self.static_op.set_factors(vals)
        return self


def static_operator(op):
    return op.static_op if isinstance(op, TimeDependentSum) else op


# ---------------------------------------------------------------------------
# constructors (src/fock.jl:8-44, src/spin.jl:14-85)
# ---------------------------------------------------------------------------


def number(b: FockBasis, dtype=np.complex128) -> Operator:
    n = len(b)
    return Operator(b, b, spdiagm(n, n, {0: np.arange(b.offset, b.N + 1)}, dtype))


def destroy(b: FockBasis, dtype=np.complex128) -> Operator:
    n = len(b)
    ns = np.arange(b.offset + 1, b.N + 1, dtype=np.float64)
    return Operator(b, b, spdiagm(n, n, {1: np.sqrt(ns)}, dtype))


def create(b: FockBasis, dtype=np.complex128) -> Operator:
    n = len(b)
    ns = np.arange(b.offset + 1, b.N + 1, dtype=np.float64)
    return Operator(b, b, spdiagm(n, n, {-1: np.sqrt(ns)}, dtype))


def _spin_ladder(b: SpinBasis):
    s = float(b.spinnumber)
    N = len(b)
    a = np.arange(1, N, dtype=np.float64)
    return np.sqrt((s + 1) * 2 * a - a * (a + 1))


def sigmax(b: SpinBasis, dtype=np.complex128) -> Operator:
    N = len(b)
    d = _spin_ladder(b).astype(np.complex128)
    return Operator(b, b, spdiagm(N, N, {1: d, -1: d}, dtype))


def sigmay(b: SpinBasis, dtype=np.complex128) -> Operator:
    N = len(b)
    d = 1j * _spin_ladder(b)
    return Operator(b, b, spdiagm(N, N, {-1: d, 1: -d}, dtype))


def sigmaz(b: SpinBasis, dtype=np.complex128) -> Operator:
    N = len(b)
    s = b.spinnumber
    ms = [float(2 * (s - k)) for k in range(N)]
    return Operator(b, b, spdiagm(N, N, {0: ms}, dtype))


def sigmap(b: SpinBasis, dtype=np.complex128) -> Operator:
    N = len(b)
    s = b.spinnumber
    S = float((s + 1) * s)
    ms = [s - 1 - k for k in range(N - 1)]
    d = [np.sqrt(S - float(m * (m + 1))) for m in ms]
    return Operator(b, b, spdiagm(N, N, {1: d}, dtype))


def sigmam(b: SpinBasis, dtype=np.complex128) -> Operator:
    N = len(b)
    s = b.spinnumber
    S = float((s + 1) * s)
    ms = [s - k for k in range(N - 1)]
    d = [np.sqrt(S - float(m * (m - 1))) for m in ms]
    return Operator(b, b, spdiagm(N, N, {-1: d}, dtype))


# ---------------------------------------------------------------------------
# conversions and algebra (host side, used to build and to check operators)
# ---------------------------------------------------------------------------


def _embed_strides(dims):
    s, t = [], 1
    for d in dims:
        s.append(t)
        t *= d
    return s, t


def embed(basis_l: CompositeBasis, basis_r: CompositeBasis, indices, op: Operator) -> Operator:
    """Sparse ``embed`` (src/operators_sparse.jl:128-178): the operator on the
    subsystems ``indices`` (1-based) tensored with identities elsewhere, built as
    CSC with zeros dropped."""
    if isinstance(indices, numbers.Integral):
        indices = [indices]
    indices = [int(i) for i in indices]
    N = len(basis_l.bases)
    dl = list(basis_l.shape)
    dr = list(basis_r.shape)
    sl, total_l = _embed_strides(dl)
    sr, total_r = _embed_strides(dr)

    def offsets(dims, strides, idx):
        out = np.zeros(int(prod(dims)) if dims else 1, np.int64)
        for lin in range(len(out)):
            c, off = lin, 0
            for d, i in zip(dims, idx):
                c, digit = divmod(c, d)
                off += digit * strides[i - 1]
            out[lin] = off
        return out

    comp = [i for i in range(1, N + 1) if i not in indices]
    sel_rows = offsets([dl[i - 1] for i in indices], sl, indices)
    sel_cols = offsets([dr[i - 1] for i in indices], sr, indices)
    idd = [min(dl[i - 1], dr[i - 1]) for i in comp]
    id_rows = offsets(idd, sl, comp)
    id_cols = offsets(idd, sr, comp)
    data = _to_csc(op.data).tocoo()
    keep = data.data != 0
    r, c, v = data.row[keep], data.col[keep], data.data[keep]
    rows = (sel_rows[r][:, None] + id_rows[None, :]).ravel()
    cols = (sel_cols[c][:, None] + id_cols[None, :]).ravel()
    vals = np.repeat(v, len(id_rows))
    m = sp.csc_matrix((vals, (rows, cols)), shape=(total_l, total_r))
    m.sum_duplicates()
    m.sort_indices()
    return Operator(basis_l, basis_r, m)


def _kron_list(mats):
    """kron in the reference's reversed order: first subsystem fastest."""
    out = mats[-1]
    for m in reversed(mats[:-1]):
        out = np.kron(out, m) if isinstance(out, np.ndarray) else sp.kron(out, m, format="csc")
    return out


def dense(op) -> Operator:
    op = static_operator(op)
    if isinstance(op, Operator):
        return Operator(op.basis_l, op.basis_r, np.asfortranarray(_to_dense_array(op.data)))
    s = sparse(op)
    return Operator(s.basis_l, s.basis_r, np.asfortranarray(s.data.toarray()))


def sparse(op) -> Operator:
    """``sparse`` of any operator: LazyTensor -> factor * embed (src/operators_lazytensor.jl:91),
    LazySum -> sum of factors .* sparse.(operators) (src/operators_lazysum.jl:81)."""
    op = static_operator(op)
    if isinstance(op, Operator):
        return Operator(op.basis_l, op.basis_r, _to_csc(op.data))
    if isinstance(op, LazyTensor):
        N = len(op.basis_l.bases)
        if len(op.indices) == 0:
            mats = [_to_csc(Eye(op.basis_l.shape[i], op.basis_r.shape[i])) for i in range(N)]
        else:
            mats = []
            for i in range(1, N + 1):
                if i in op.indices:
                    mats.append(_to_csc(op.operators[op.indices.index(i)].data))
                else:
                    mats.append(_to_csc(Eye(op.basis_l.shape[i - 1], op.basis_r.shape[i - 1])))
        m = _kron_list(mats).tocsc() * op.factor
        m.eliminate_zeros()
        return Operator(op.basis_l, op.basis_r, m.tocsc())
    if isinstance(op, LazySum):
        m = sp.csc_matrix(op.shape, dtype=np.complex128)
        for f, o in zip(op.factors, op.operators):
            m = m + f * sparse(o).data
        return Operator(op.basis_l, op.basis_r, m.tocsc())
    if isinstance(op, LazyProduct):
        m = sparse(op.operators[0]).data
        for o in op.operators[1:]:
            m = m @ sparse(o).data
        return Operator(op.basis_l, op.basis_r, (op.factor * m).tocsc())
    raise TypeError(f"sparse() of {type(op)}")


def tensor(*ops):
    """Tensor product of operators; data as kron(b.data, a.data) (src/operators_dense.jl:134)."""
    from .states import Ket, Bra, tensor_states

    if all(isinstance(o, (Ket, Bra)) for o in ops):
        return tensor_states(*ops)
    if all(isinstance(o, Basis) for o in ops):
        return tensor_bases(*ops)
    bl = tensor_bases(*[o.basis_l for o in ops])
    br = tensor_bases(*[o.basis_r for o in ops])
    if all(isinstance(o, Operator) for o in ops):
        if any(o.kind in ("dense", "dense_adj") for o in ops):
            data = np.asfortranarray(_kron_list([_to_dense_array(o.data) for o in ops]))
        else:
            data = _kron_list([_to_csc(o.data) for o in ops]).tocsc()
        return Operator(bl, br, data)
    # lazy: a tensor of LazyTensors / data operators is a LazyTensor
    idx, facs, factor, off = [], [], 1.0 + 0j, 0
    for o in ops:
        n = len(o.basis_l.bases) if isinstance(o.basis_l, CompositeBasis) else 1
        if isinstance(o, LazyTensor):
            idx += [i + off for i in o.indices]
            facs += list(o.operators)
            factor *= o.factor
        elif isinstance(o, Operator) and n == 1:
            idx.append(off + 1)
            facs.append(o)
        else:
            raise ArgumentError("tensor of a lazy operator with a composite non-lazy operator")
        off += n
    return LazyTensor(bl, br, tuple(idx), tuple(facs), factor)


def dagger(op):
    if isinstance(op, Operator):
        d = op.data
        nd = d.parent if isinstance(d, Adjoint) else Adjoint(d)
        return Operator(op.basis_r, op.basis_l, nd)
    if isinstance(op, LazyTensor):
        return LazyTensor(op.basis_r, op.basis_l, op.indices, tuple(dagger(o) for o in op.operators),
                          np.conj(op.factor))
    if isinstance(op, LazySum):
        return LazySum(op.basis_r, op.basis_l, np.conj(op.factors), tuple(dagger(o) for o in op.operators))
    if isinstance(op, LazyProduct):
        return LazyProduct(tuple(dagger(o) for o in reversed(op.operators)), factor=np.conj(op.factor))
    raise TypeError(f"dagger of {type(op)}")


def scale(op, a):
    a = complex(a)
    if isinstance(op, Operator):
        d = op.data
        if isinstance(d, (Eye, Adjoint)):
            d = _to_csc(d) if isinstance(d, Eye) or sp.issparse(d.parent) else _to_dense_array(d)
        return Operator(op.basis_l, op.basis_r, a * d)
    if isinstance(op, LazyTensor):
        return LazyTensor(op.basis_l, op.basis_r, op.indices, op.operators, op.factor * a)
    if isinstance(op, LazySum):
        return LazySum(op.basis_l, op.basis_r, op.factors * a, op.operators)
    if isinstance(op, LazyProduct):
        return LazyProduct(op.operators, factor=op.factor * a)
    raise TypeError(f"cannot scale {type(op)}")


def _is_lazy(o):
    return isinstance(o, (LazyTensor, LazySum, LazyProduct, TimeDependentSum))


def add(a, b):
    """``+`` with the reference's merge of two single-factor LazyTensors on the
    same indices (src/operators_lazytensor.jl:100-114)."""
    if a.basis_l != b.basis_l or a.basis_r != b.basis_r:
        raise IncompatibleBases()
    if (isinstance(a, LazyTensor) and isinstance(b, LazyTensor) and len(a.operators) == 1
            and len(b.operators) == 1 and a.indices == b.indices
            and isinstance(a.operators[0], Operator) and isinstance(b.operators[0], Operator)):
        op = add(scale(a.operators[0], a.factor), scale(b.operators[0], b.factor))
        return LazyTensor(a.basis_l, a.basis_r, a.indices, (op,))
    if _is_lazy(a) or _is_lazy(b):
        la = a if isinstance(a, LazySum) else LazySum((a,))
        lb = b if isinstance(b, LazySum) else LazySum((b,))
        return LazySum(a.basis_l, a.basis_r, np.r_[la.factors, lb.factors], la.operators + lb.operators)
    if a.kind in ("sparse", "eye", "sparse_adj", "eye_adj") and b.kind in ("sparse", "eye", "sparse_adj", "eye_adj"):
        return Operator(a.basis_l, a.basis_r, (_to_csc(a.data) + _to_csc(b.data)).tocsc())
    return Operator(a.basis_l, a.basis_r, np.asfortranarray(_to_dense_array(a.data) + _to_dense_array(b.data)))


def multiply(a, b):
    """``a * b`` of operators: lazy operands give a LazyProduct, data operands a data product."""
    if a.basis_r != b.basis_l:
        raise IncompatibleBases()
    if _is_lazy(a) or _is_lazy(b):
        if isinstance(b, Operator) and b.kind in ("dense", "device") and not _is_lazy(b):
            from .mul import mul_

            out = Operator(a.basis_l, b.basis_r, np.zeros((len(a.basis_l), len(b.basis_r)), np.complex128, order="F"))
            return mul_(out, a, b)
        if isinstance(a, Operator) and a.kind in ("dense", "device") and not _is_lazy(a):
            from .mul import mul_

            out = Operator(a.basis_l, b.basis_r, np.zeros((len(a.basis_l), len(b.basis_r)), np.complex128, order="F"))
            return mul_(out, a, b)
        la = a.operators if isinstance(a, LazyProduct) else (a,)
        lb = b.operators if isinstance(b, LazyProduct) else (b,)
        fa = a.factor if isinstance(a, LazyProduct) else 1.0
        fb = b.factor if isinstance(b, LazyProduct) else 1.0
        return LazyProduct(la + lb, factor=fa * fb)
    if a.kind.startswith("dense") or b.kind.startswith("dense"):
        return Operator(a.basis_l, b.basis_r, np.asfortranarray(_to_dense_array(a.data) @ _to_dense_array(b.data)))
    return Operator(a.basis_l, b.basis_r, (_to_csc(a.data) @ _to_csc(b.data)).tocsc())


def eltype(op) -> np.dtype:
    """Promoted element type of an operator tree."""
    op = static_operator(op)
    if isinstance(op, Operator):
        return op.dtype
    if isinstance(op, LazyTensor):
        return np.result_type(np.complex64, *[eltype(o) for o in op.operators]) if op.operators else np.dtype(np.complex128)
    if isinstance(op, (LazySum, LazyProduct)):
        return np.result_type(*[eltype(o) for o in op.operators]) if op.operators else np.dtype(np.complex128)
    return np.dtype(np.complex128)


__all__ = [
    "DimensionMismatch", "IncompatibleBases", "ArgumentError", "Eye", "Adjoint", "spdiagm",
    "AbstractOperator", "Operator", "DenseOperator", "SparseOperator", "identityoperator",
    "LazyTensor", "LazySum", "LazyProduct", "TimeDependentSum", "static_operator", "number",
    "destroy", "create", "sigmax", "sigmay", "sigmaz", "sigmap", "sigmam", "embed", "dense",
    "sparse", "tensor", "dagger", "scale", "add", "multiply", "eltype", "comp_size",
]
