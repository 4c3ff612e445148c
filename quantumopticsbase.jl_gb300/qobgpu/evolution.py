"""Batched application, RK4 time evolution and the request server (device side).

* ``Batch`` -- many (operator, x, y, alpha, beta) applications of uneven size
  run as one persistent launch (``qob_batch_*``).
* ``rk4(H, psi, dt, nsteps)`` -- fixed-step RK4 of dpsi/dt = -i H psi on a
  device state (``qob_rk4``).
* ``Server`` -- continuous-batching request loop for short time evolutions
  (``qob_server_*``): states and operators stay on the device, requests are
  admitted by free device memory, finished ones report their latency.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import operators as O
from .device import Context, dtype_code, get_context, handle, raise_for


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class Batch:
    """y_i = alpha_i * op_i * x_i + beta_i * y_i for many kets in one launch."""

    def __init__(self, dtype=np.complex128, device: int = 0, arith: str | None = None):
        """``arith="ff"``: ComplexF64 kets, operators applied in double-float
        arithmetic (QOB_C128X)."""
        self.ctx = get_context(device)
        self.dtype = np.dtype(dtype)
        code = dtype_code(self.dtype)
        if arith == "ff":
            if self.dtype != np.complex128:
                raise O.ArgumentError('arith="ff" (double-float) applies to ComplexF64 kets')
            code = L.QOB_C128X
        p = C.c_void_p()
        raise_for(L.lib().qob_batch_create(self.ctx.ptr, code, C.byref(p)), self.ctx)
        self.ptr = p
        self._keep = []

    def add(self, op, x, y, alpha=1.0, beta=0.0):
        """x, y: contiguous CUDA tensors of the batch's dtype (kept alive by the batch)."""
        h = handle(self.ctx, op)
        a, b = complex(alpha), complex(beta)
        raise_for(L.lib().qob_batch_add(self.ctx.ptr, self.ptr, h.ptr, a.real, a.imag, _ptr(x), _ptr(y), b.real,
                                        b.imag), self.ctx)
        self._keep.append((h, x, y))

    def run(self, stream=None):
        raise_for(L.lib().qob_batch_run(self.ctx.ptr, self.ptr, stream), self.ctx)

    def tune(self):
        t = (C.c_double * 4)()
        ch = C.c_int()
        raise_for(L.lib().qob_batch_tune(self.ctx.ptr, self.ptr, t, C.byref(ch)), self.ctx)
        return ch.value, list(t)

    def set_tile(self, tile: int):
        """Fix the tile length (128, 256, 512 or 1024) without timing."""
        raise_for(L.lib().qob_batch_set_tile(self.ctx.ptr, self.ptr, int(tile)), self.ctx)

    def info(self):
        v = (C.c_int64 * 5)()
        raise_for(L.lib().qob_batch_info(self.ctx.ptr, self.ptr, v), self.ctx)
        return {"items": v[0], "fused": v[1], "tiles": v[2], "tile": v[3], "grid": v[4]}

    def __del__(self):
        try:
            if self.ptr:
                L.lib().qob_batch_free(self.ctx.ptr, self.ptr)
        except Exception:
            pass


def factor_rows(H: O.TimeDependentSum, t0: float, dt: float, nsteps: int) -> np.ndarray:
    """The coefficients of ``H`` at t0 + r*dt/2, r = 0 .. 2*nsteps (the times at
    which an RK4 step evaluates its right-hand side), as (rows, nterms) complex."""
    times = t0 + 0.5 * dt * np.arange(2 * nsteps + 1)
    rows = np.empty((len(times), len(H.coefficients)), np.complex128)
    for k, c in enumerate(H.coefficients):
        rows[:, k] = [c(t) for t in times] if callable(c) else c
    return rows


def rk4(H, psi, dt: float, nsteps: int, renormalise: bool = False, t0: float = 0.0, arith: str | None = None):
    """In-place RK4 on a device Ket (or a contiguous CUDA tensor).

    A ``TimeDependentSum`` is evolved with its coefficients evaluated on the host
    at every stage time (as ``set_time!`` would, src/time_dependent_operator.jl:162-171)
    and applied on the device inside the steps; afterwards its current time is
    t0 + nsteps*dt.  ``arith="ff"``: ComplexF64 states with the operator applied
    in double-float arithmetic (QOB_C128X)."""
    data = psi.data if hasattr(psi, "data") and not hasattr(psi, "data_ptr") else psi
    ctx = get_context(data.device.index)
    import torch

    dt_code = L.QOB_C64 if data.dtype == torch.complex64 else L.QOB_C128
    if arith == "ff":
        if data.dtype != torch.complex128:
            raise O.ArgumentError('arith="ff" (double-float) applies to ComplexF64 states')
        dt_code = L.QOB_C128X
    s = C.c_void_p(torch.cuda.current_stream(data.device.index).cuda_stream)
    if isinstance(H, O.TimeDependentSum):
        h = handle(ctx, H)
        rows = np.ascontiguousarray(factor_rows(H, t0, dt, nsteps))
        raise_for(L.lib().qob_rk4_td(ctx.ptr, h.ptr, dt_code, _ptr(data), data.shape[0], float(dt), int(nsteps),
                                     rows.ctypes.data_as(C.c_void_p), rows.shape[0], int(renormalise), s), ctx)
        H.set_time(t0 + nsteps * dt)
        return psi
    h = handle(ctx, H)
    raise_for(L.lib().qob_rk4(ctx.ptr, h.ptr, dt_code, _ptr(data), data.shape[0], float(dt), int(nsteps),
                              int(renormalise), s), ctx)
    return psi


class Server:
    """Continuous-batching server of RK4 time-evolution requests."""

    def __init__(self, dtype=np.complex128, mem_budget: int = 8 << 30, max_active: int = 256,
                 renormalise: bool = False, device: int = 0, arith: str | None = None):
        """``arith="ff"``: ComplexF64 requests with the operators applied in
        double-float arithmetic (QOB_C128X)."""
        self.ctx: Context = get_context(device)
        self.dtype = np.dtype(dtype)
        code = dtype_code(self.dtype)
        if arith == "ff":
            if self.dtype != np.complex128:
                raise O.ArgumentError('arith="ff" (double-float) applies to ComplexF64 requests')
            code = L.QOB_C128X
        p = C.c_void_p()
        raise_for(L.lib().qob_server_create(self.ctx.ptr, code, int(mem_budget), int(max_active),
                                            int(renormalise), C.byref(p)), self.ctx)
        self.ptr = p
        self._ops = {}
        self._sizes = {}

    def submit(self, H, psi0: np.ndarray, nsteps: int, dt: float, t0: float = 0.0) -> int:
        """Queue nsteps RK4 steps of psi0 under H; a TimeDependentSum is evolved
        with its coefficients at every stage time from t0 (qob_server_submit_td)."""
        h = handle(self.ctx, H)
        self._ops[id(H)] = (H, h)
        a = np.ascontiguousarray(psi0, dtype=self.dtype)
        rid = C.c_int64()
        if isinstance(H, O.TimeDependentSum):
            rows = np.ascontiguousarray(factor_rows(H, t0, dt, nsteps))
            raise_for(L.lib().qob_server_submit_td(self.ptr, h.ptr, a.ctypes.data_as(C.c_void_p), a.shape[0],
                                                   int(nsteps), float(dt), rows.ctypes.data_as(C.c_void_p),
                                                   rows.shape[0], C.byref(rid)), self.ctx)
        else:
            raise_for(L.lib().qob_server_submit(self.ptr, h.ptr, a.ctypes.data_as(C.c_void_p), a.shape[0],
                                                int(nsteps), float(dt), C.byref(rid)), self.ctx)
        self._sizes[rid.value] = a.shape[0]
        return rid.value

    def step(self) -> int:
        n = C.c_int()
        raise_for(L.lib().qob_server_step(self.ptr, C.byref(n)), self.ctx)
        return n.value

    def start(self):
        raise_for(L.lib().qob_server_start(self.ptr), self.ctx)

    def stop(self):
        raise_for(L.lib().qob_server_stop(self.ptr), self.ctx)

    def poll(self, rid: int):
        """(status, times[submit, admit, done], result or None)."""
        out = np.empty(self._sizes[rid], dtype=self.dtype)
        t = (C.c_double * 3)()
        st = C.c_int()
        raise_for(L.lib().qob_server_poll(self.ptr, rid, out.ctypes.data_as(C.c_void_p), t, C.byref(st)), self.ctx)
        return st.value, list(t), (out if st.value == 2 else None)

    def wait(self, rid: int, timeout: float = 60.0) -> int:
        st = C.c_int()
        raise_for(L.lib().qob_server_wait(self.ptr, rid, float(timeout), C.byref(st)), self.ctx)
        return st.value

    def stats(self):
        v = (C.c_int64 * 8)()
        raise_for(L.lib().qob_server_stats(self.ptr, v), self.ctx)
        keys = ["queued", "active", "completed", "rejected", "request_steps", "iterations", "device_bytes",
                "last_error"]
        w = (C.c_int64 * 2)()
        raise_for(L.lib().qob_server_stats2(self.ptr, w), self.ctx)
        return dict(zip(keys, list(v)), cancelled=w[0], alloc_refusals=w[1])

    def cancel(self, rid: int) -> None:
        """Cancel a queued or running request (status -QOB_ERR_CANCELLED)."""
        raise_for(L.lib().qob_server_cancel(self.ptr, rid), self.ctx)

    def set_alloc_hook(self, hook) -> None:
        """``hook(nbytes) -> bool``: asked before each admission's device
        allocation; False refuses it as if the device were out of memory.  None
        removes the hook."""
        if hook is None:
            self._hook = None
            raise_for(L.lib().qob_server_set_alloc_hook(self.ptr, None, None), self.ctx)
            return
        self._hook = L.ALLOC_HOOK(lambda user, nbytes: 0 if hook(int(nbytes)) else 1)
        raise_for(L.lib().qob_server_set_alloc_hook(self.ptr, C.cast(self._hook, C.c_void_p), None), self.ctx)

    def close(self):
        if self.ptr:
            L.lib().qob_server_destroy(self.ptr)
            self.ptr = None
            self._hook = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
