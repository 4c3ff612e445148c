"""Device contexts and operator handles over the C ABI.

A ``Context`` wraps one ``qob_ctx`` (one CUDA device).  ``handle(ctx, op)``
turns a Python operator tree into C-ABI handles the first time it is used on a
device and caches them on the Python objects; a LazySum whose factors changed
since is updated in place with ``qob_op_set_factors`` (what
``TimeDependentSum``'s ``set_time!`` does, src/time_dependent_operator.jl:162-171).
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np
import scipy.sparse as sp

from . import _lib as L
from . import operators as O


class QobError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"qobgpu error {code}: {msg}")
        self.code = code


def raise_for(code: int, ctx) -> None:
    if code == L.QOB_OK:
        return
    msg = L.lib().qob_last_error(ctx.ptr if ctx is not None else None)
    msg = msg.decode() if msg else ""
    if code == L.QOB_ERR_DIM:
        raise O.DimensionMismatch(msg)
    if code in (L.QOB_ERR_ALIAS, L.QOB_ERR_UNSUPPORTED):
        raise O.ArgumentError(msg)
    raise QobError(code, msg)


class Context:
    def __init__(self, device: int = 0):
        self.device = int(device)
        p = C.c_void_p()
        rc = L.lib().qob_create(C.byref(p), self.device, 0)
        if rc:
            raise QobError(rc, f"qob_create failed on device {device}")
        self.ptr = p
        self._finalizer = weakref.finalize(self, L.lib().qob_destroy, p)


_contexts: dict[int, Context] = {}


def get_context(device: int = 0) -> Context:
    if device not in _contexts:
        _contexts[device] = Context(device)
    return _contexts[device]


class Handle:
    """One qob_op*; freed when the Python object goes away."""

    def __init__(self, ctx: Context, ptr: C.c_void_p, children=()):
        self.ctx = ctx
        self.ptr = ptr
        self.children = list(children)
        self._finalizer = weakref.finalize(self, L.lib().qob_op_free, ctx.ptr, ptr)


def dtype_code(dt) -> int:
    """numpy complex128 / complex64, or "ff" for ComplexF64 data applied in
    double-float arithmetic (QOB_C128X)."""
    if isinstance(dt, str) and dt == "ff":
        return L.QOB_C128X
    return L.QOB_C64 if np.dtype(dt) == np.complex64 else L.QOB_C128


def _c_array(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def _new(fn, ctx, *args):
    out = C.c_void_p()
    raise_for(fn(ctx.ptr, *args, C.byref(out)), ctx)
    return out


def _leaf(ctx: Context, op: O.Operator) -> Handle:
    lib = L.lib()
    d = op.data
    adj = 0
    if isinstance(d, O.Adjoint):
        d, adj = d.parent, 1
    if isinstance(d, O.Eye):
        m, n = (d.n, d.m) if adj else (d.m, d.n)
        return Handle(ctx, _new(lib.qob_op_eye, ctx, m, n))
    if hasattr(d, "device") and not isinstance(d, np.ndarray) and not sp.issparse(d):
        d = d.detach().cpu().numpy()
    if sp.issparse(d):
        c = d.tocsc()
        dt = np.complex64 if c.dtype == np.complex64 else np.complex128
        colptr = np.ascontiguousarray(c.indptr, dtype=np.int64) + 1
        rowval = np.ascontiguousarray(c.indices, dtype=np.int64) + 1
        nz = np.ascontiguousarray(c.data, dtype=dt)
        h = _new(lib.qob_op_sparse, ctx, c.shape[0], c.shape[1], _c_array(colptr, C.c_int64),
                 _c_array(rowval, C.c_int64), nz.ctypes.data_as(C.c_void_p), dtype_code(dt), adj)
        return Handle(ctx, h)
    a = np.asarray(d)
    dt = np.complex64 if a.dtype == np.complex64 else np.complex128
    a = np.asfortranarray(a, dtype=dt)
    h = _new(lib.qob_op_dense, ctx, a.shape[0], a.shape[1], a.ctypes.data_as(C.c_void_p), max(1, a.shape[0]),
             dtype_code(dt), adj)
    return Handle(ctx, h)


def _build(ctx: Context, op) -> Handle:
    lib = L.lib()
    if isinstance(op, O.Operator):
        return _leaf(ctx, op)
    if isinstance(op, O.LazyTensor):
        kids = [handle(ctx, o) for o in op.operators]
        sl = np.asarray(op.basis_l.shape, np.int64)
        sr = np.asarray(op.basis_r.shape, np.int64)
        idx = np.asarray(op.indices if op.indices else [0], np.int64)
        arr = (C.c_void_p * max(1, len(kids)))(*[k.ptr for k in kids])
        h = _new(lib.qob_op_lazytensor, ctx, len(sl), _c_array(sl, C.c_int64), _c_array(sr, C.c_int64), len(kids),
                 _c_array(idx, C.c_int64), arr, op.factor.real, op.factor.imag)
        return Handle(ctx, h, kids)
    if isinstance(op, O.LazySum):
        kids = [handle(ctx, o) for o in op.operators]
        f = np.ascontiguousarray(op.factors, np.complex128).view(np.float64)
        arr = (C.c_void_p * max(1, len(kids)))(*[k.ptr for k in kids])
        h = _new(lib.qob_op_lazysum, ctx, len(op.basis_l), len(op.basis_r), len(kids), _c_array(f, C.c_double), arr)
        hd = Handle(ctx, h, kids)
        hd.factors_seen = op.factors.copy()
        return hd
    if isinstance(op, O.LazyProduct):
        kids = [handle(ctx, o) for o in op.operators]
        arr = (C.c_void_p * len(kids))(*[k.ptr for k in kids])
        h = _new(lib.qob_op_lazyproduct, ctx, len(kids), arr, op.factor.real, op.factor.imag)
        return Handle(ctx, h, kids)
    if isinstance(op, O.TimeDependentSum):
        return handle(ctx, op.static_op)
    from .particle import FFTOperator

    if isinstance(op, FFTOperator):
        shape = np.asarray(op.basis_l.shape, np.int64)
        axes = np.asarray(op.axes, np.int64)
        signs = (C.c_int * len(axes))(*([op.sign] * len(axes)))
        before = np.ascontiguousarray(np.concatenate(op.before)).view(np.float64)
        after = np.ascontiguousarray(np.concatenate(op.after)).view(np.float64)
        h = _new(lib.qob_op_fft, ctx, len(shape), _c_array(shape, C.c_int64), len(axes), _c_array(axes, C.c_int64),
                 signs, _c_array(before, C.c_double), _c_array(after, C.c_double))
        return Handle(ctx, h)
    raise O.ArgumentError(f"no device form for {type(op).__name__}")


def handle(ctx: Context, op) -> Handle:
    """Cached device handle of ``op`` on ``ctx`` (factor changes of LazySums are pushed)."""
    op = O.static_operator(op)
    cache = op.__dict__.setdefault("_qob_handles", {})
    h = cache.get(ctx.device)
    if h is None:
        h = _build(ctx, op)
        cache[ctx.device] = h
    else:
        _sync_factors(ctx, op, h)
    return h


def _sync_factors(ctx: Context, op, h: Handle) -> None:
    if isinstance(op, O.LazySum):
        if not np.array_equal(h.factors_seen, op.factors):
            f = np.ascontiguousarray(op.factors, np.complex128).view(np.float64)
            raise_for(L.lib().qob_op_set_factors(ctx.ptr, h.ptr, _c_array(f, C.c_double)), ctx)
            h.factors_seen = op.factors.copy()
        for o, k in zip(op.operators, h.children):
            _sync_factors(ctx, o, k)
    elif isinstance(op, (O.LazyProduct,)):
        for o, k in zip(op.operators, h.children):
            _sync_factors(ctx, o, k)


def prepare(op, side: int = L.QOB_LEFT, dtype=np.complex128, device: int = 0) -> dict:
    """Compile the device form ahead of time; returns its structure summary."""
    ctx = get_context(device)
    h = handle(ctx, op)
    info = (C.c_int64 * 4)()
    raise_for(L.lib().qob_op_prepare(ctx.ptr, h.ptr, side, dtype_code(dtype), info), ctx)
    return {"groups": info[0], "diagonal": bool(info[1]), "entries": info[2], "extra_passes": info[3]}
