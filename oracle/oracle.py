"""ctypes front end of the CPU oracle (liboref.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU
legs of bench.py as the checker / CPU baseline, never by the product path.

``build_node(op)`` walks an operator tree of the Python mirror (qobgpu) and
builds the oracle's own copy of it; ``mul(result, a, b, alpha, beta)`` runs the
restated reference ``mul!`` on host numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboref.so")
_lib = None

D = C.POINTER(C.c_double)
I64 = C.POINTER(C.c_int64)
VP = C.c_void_p


def build(force: bool = False) -> str:
    """Compile liboref.so with the committed Makefile (gcc only)."""
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("qob_oracle.cpp", "qob_oracle.h")
    ):
        subprocess.run(["make", "-s", "-C", _HERE, "liboref.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.oref_sparse.argtypes = [C.c_int64, C.c_int64, I64, I64, D, C.c_int]
        L.oref_dense.argtypes = [C.c_int64, C.c_int64, D, C.c_int]
        L.oref_eye.argtypes = [C.c_int64, C.c_int64]
        L.oref_lazytensor.argtypes = [C.c_int, I64, I64, C.c_int, I64, C.POINTER(VP), C.c_double, C.c_double]
        L.oref_lazysum.argtypes = [C.c_int64, C.c_int64, C.c_int, D, C.POINTER(VP)]
        L.oref_lazyproduct.argtypes = [C.c_int, C.POINTER(VP), C.c_double, C.c_double]
        L.oref_lazysum_set_factors.argtypes = [VP, D]
        for f in ("oref_sparse", "oref_dense", "oref_eye", "oref_lazytensor", "oref_lazysum", "oref_lazyproduct"):
            getattr(L, f).restype = VP
        L.oref_free.argtypes = [VP]
        L.oref_mul.argtypes = [C.c_int, C.c_int, VP, C.c_double, C.c_double, D, C.c_int64, C.c_int64,
                               C.c_double, C.c_double, D, C.c_int64, C.c_int64]
        L.oref_mul.restype = C.c_int
        L.oref_mul_kets_threaded.argtypes = [VP, C.c_double, C.c_double, D, C.c_double, C.c_double, D,
                                             C.c_int64, C.c_int]
        L.oref_mul_kets_threaded.restype = C.c_int
        L.oref_fft.argtypes = [C.c_int, I64, C.c_int, I64, C.c_int, D, D]
        L.oref_fft.restype = VP
        L.oref_expect_lazyket.argtypes = [VP, C.c_int, I64, D, D]
        L.oref_expect_lazyket.restype = C.c_int
        L.oref_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(D)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(I64)


class Node:
    """Owns one oracle node and keeps its children alive."""

    def __init__(self, ptr, children=()):
        self.ptr = ptr
        self.children = list(children)

    def __del__(self):
        if self.ptr and _lib is not None:
            _lib.oref_free(self.ptr)
            self.ptr = None


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128)).view(np.float64)


def build_node(op) -> Node:
    """Oracle copy of a qobgpu operator tree."""
    import scipy.sparse as sp
    from qobgpu import operators as O

    L = lib()
    op = O.static_operator(op)
    if isinstance(op, O.Operator):
        d = op.data
        adj = 0
        if isinstance(d, O.Adjoint):
            d, adj = d.parent, 1
        if isinstance(d, O.Eye):
            if adj:
                return Node(L.oref_eye(d.n, d.m))
            return Node(L.oref_eye(d.m, d.n))
        if sp.issparse(d):
            c = d.tocsc()
            colptr = (c.indptr.astype(np.int64) + 1).copy()
            rowval = (c.indices.astype(np.int64) + 1).copy()
            nz = _c128(c.data)
            return Node(L.oref_sparse(c.shape[0], c.shape[1], _ip(colptr), _ip(rowval), _dp(nz), adj))
        a = np.asfortranarray(np.asarray(d if isinstance(d, np.ndarray) else d.cpu().numpy(), np.complex128))
        flat = np.ascontiguousarray(a.reshape(-1, order="F")).view(np.float64)
        return Node(L.oref_dense(a.shape[0], a.shape[1], _dp(flat), adj))
    if isinstance(op, O.LazyTensor):
        kids = [build_node(o) for o in op.operators]
        sl = np.asarray(op.basis_l.shape, np.int64)
        sr = np.asarray(op.basis_r.shape, np.int64)
        idx = np.asarray(op.indices, np.int64)
        arr = (VP * max(1, len(kids)))(*[k.ptr for k in kids])
        p = L.oref_lazytensor(len(sl), _ip(sl), _ip(sr), len(kids), _ip(idx), arr, op.factor.real, op.factor.imag)
        return Node(p, kids)
    if isinstance(op, O.LazySum):
        kids = [build_node(o) for o in op.operators]
        f = _c128(op.factors)
        arr = (VP * max(1, len(kids)))(*[k.ptr for k in kids])
        p = L.oref_lazysum(len(op.basis_l), len(op.basis_r), len(kids), _dp(f), arr)
        return Node(p, kids)
    if isinstance(op, O.LazyProduct):
        kids = [build_node(o) for o in op.operators]
        arr = (VP * len(kids))(*[k.ptr for k in kids])
        p = L.oref_lazyproduct(len(kids), arr, op.factor.real, op.factor.imag)
        return Node(p, kids)
    from qobgpu.particle import FFTOperator

    if isinstance(op, FFTOperator):
        shape = np.asarray(op.basis_l.shape, np.int64)
        axes = np.asarray(op.axes, np.int64)
        mb = _c128(op.mul_before)
        ma = _c128(op.mul_after)
        return Node(L.oref_fft(len(shape), _ip(shape), len(axes), _ip(axes), op.sign, _dp(mb), _dp(ma)))
    raise TypeError(f"oracle: unsupported operator {type(op)}")


class OracleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def mul_arrays(side: int, is_vector: bool, node: Node, alpha, x: np.ndarray, beta, y: np.ndarray) -> np.ndarray:
    """y <- alpha*op*x + beta*y (side 0) or alpha*x*op + beta*y (side 1), in place
    on a complex128 Fortran-ordered copy that is returned."""
    L = lib()
    x = np.asfortranarray(np.asarray(x, np.complex128))
    y = np.asfortranarray(np.array(y, np.complex128, copy=True))
    if x.ndim == 1:
        xr, xc = (x.shape[0], 1) if side == 0 else (1, x.shape[0])
    else:
        xr, xc = x.shape
    if y.ndim == 1:
        yr, yc = (y.shape[0], 1) if side == 0 else (1, y.shape[0])
    else:
        yr, yc = y.shape
    xf = x.reshape(-1, order="F").view(np.float64)
    yf = y.reshape(-1, order="F").view(np.float64)
    a, b = complex(alpha), complex(beta)
    rc = L.oref_mul(side, int(is_vector), node.ptr, a.real, a.imag, _dp(xf), xr, xc, b.real, b.imag, _dp(yf), yr, yc)
    if rc:
        raise OracleError(rc, L.oref_last_error().decode())
    return yf.view(np.complex128).reshape(y.shape, order="F")


def mul(result, a, b, alpha=1.0, beta=0.0):
    """Oracle ``mul!(result, a, b, alpha, beta)`` on qobgpu host objects; returns
    the new result data (the input objects are left untouched)."""
    from qobgpu import operators as O
    from qobgpu.states import Bra, Ket

    if isinstance(b, Ket):
        return mul_arrays(0, True, build_node(a), alpha, b.to_host(), beta, result.to_host())
    if isinstance(a, Bra):
        return mul_arrays(1, True, build_node(b), alpha, a.to_host(), beta, result.to_host())

    def state_like(o):
        return isinstance(o, O.Operator) and o.kind in ("dense", "device")

    if state_like(b) or not state_like(a):
        return mul_arrays(0, False, build_node(a), alpha, O._to_dense_array(b.data), beta,
                          O._to_dense_array(result.data))
    return mul_arrays(1, False, build_node(b), alpha, O._to_dense_array(a.data), beta,
                      O._to_dense_array(result.data))


def mul_kets_threaded(node: Node, alpha, X: np.ndarray, beta, Y: np.ndarray, nthreads: int) -> int:
    """Apply the operator to each column of X (one Ket per column) on nthreads threads."""
    L = lib()
    a, b = complex(alpha), complex(beta)
    xf = X.reshape(-1, order="F").view(np.float64)
    yf = Y.reshape(-1, order="F").view(np.float64)
    rc = L.oref_mul_kets_threaded(node.ptr, a.real, a.imag, _dp(xf), b.real, b.imag, _dp(yf), X.shape[1], nthreads)
    if rc:
        raise OracleError(rc, L.oref_last_error().decode())
    return rc


def expect_lazyket(op, kets) -> complex:
    """Oracle ``expect(op, LazyKet(basis, kets))`` (src/states_lazyket.jl:64-125);
    kets: the site kets (qobgpu Ket objects or arrays) in subsystem order."""
    L = lib()
    node = build_node(op)
    arrs = [np.asarray(k.to_host() if hasattr(k, "to_host") else k, np.complex128) for k in kets]
    dims = np.asarray([a.shape[0] for a in arrs], np.int64)
    flat = np.ascontiguousarray(np.concatenate(arrs)).view(np.float64)
    out = np.zeros(2)
    rc = L.oref_expect_lazyket(node.ptr, len(arrs), _ip(dims), _dp(flat), _dp(out))
    if rc:
        raise OracleError(rc, L.oref_last_error().decode())
    return complex(out[0], out[1])
