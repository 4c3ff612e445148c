"""The bounds-checked build (QOB_DEBUG_BOUNDS) on the GPU.

In that build every slot index and every gathered input index of the fused
gather kernels is checked before it is used; an index out of range is skipped
and recorded in the context's device status word, which qob_device_status
turns into QOB_ERR_ARG with a message -- no trap, no fault.  The test moves the
input offset of one stored entry of a 6-spin chain's compiled plan past the end
of the vectors (qob_debug_shift_slot, present only in that build; the moved
offset points at most 64 elements past a vector, inside the same allocation,
so even an unchecked read would stay in mapped memory), applies it with the
untiled and the staged-tile kernels, and checks that the status reports the
bad index while an intact operator still matches the oracle with a clean
status.  It runs in a child process that loads libqobgpu_debug.so through
QOB_LIBRARY.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import ctypes as C, sys
import numpy as np
sys.path[:0] = [{root!r}, {root!r} + "/quantumopticsbase.jl_gb300", {root!r} + "/oracle", {root!r} + "/tests"]
import torch
import oracle as OR
import qobgpu as Q
from qobgpu import _lib as L
from qobgpu.device import get_context, handle, raise_for
from qobgpu.hamiltonians import heisenberg_chain
from helpers import rel_l2
lib = L.lib()
assert L.LIB_PATH.endswith("libqobgpu_debug.so"), L.LIB_PATH
lib.qob_debug_shift_slot.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
ctx = get_context(0)
AL, BE = 0.7 - 0.2j, 0.3
n, k = 64, 5

def run(H, tile):
    hd = handle(ctx, H)
    if tile:
        raise_for(lib.qob_op_set_tile(ctx.ptr, hd.ptr, L.QOB_LEFT, L.QOB_C128, 1, 1, 6), ctx)
    else:
        raise_for(lib.qob_op_set_launch(ctx.ptr, hd.ptr, L.QOB_LEFT, L.QOB_C128, 1, 256, 1), ctx)
    rng = Q.Rng(5)
    X, Y = rng.kets_data(n, k), rng.kets_data(n, k)
    xd = torch.as_tensor(np.ascontiguousarray(X.T), device="cuda:0").t()
    yd = torch.as_tensor(np.ascontiguousarray(Y.T), device="cuda:0").t()
    raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 0, hd.ptr, L.QOB_C128, AL.real, AL.imag, C.c_void_p(xd.data_ptr()),
                          n, k, n, BE, 0.0, C.c_void_p(yd.data_ptr()), n, k, n, None), ctx)
    torch.cuda.synchronize()
    flags = C.c_uint()
    rc = lib.qob_device_status(ctx.ptr, None, C.byref(flags))
    ref = np.asfortranarray(Y.copy())
    OR.mul_kets_threaded(OR.build_node(H), AL, np.asfortranarray(X), BE, ref, 4)
    return rc, flags.value, lib.qob_last_error(ctx.ptr), rel_l2(yd.cpu().numpy(), ref)

for tile in (False, True):
    good = heisenberg_chain(6, seed=2)
    rc, fl, msg, err = run(good, tile)
    assert rc == 0 and fl == 0 and err < 1e-12, (tile, rc, fl, err)
    bad = heisenberg_chain(6, seed=2)
    hd = handle(ctx, bad)
    z_in = torch.zeros(n, dtype=torch.complex128, device="cuda:0")
    z_out = torch.zeros(n, dtype=torch.complex128, device="cuda:0")
    raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 1, hd.ptr, L.QOB_C128, 1.0, 0.0, C.c_void_p(z_in.data_ptr()), n, 1, n,
                          0.0, 0.0, C.c_void_p(z_out.data_ptr()), n, 1, n, None), ctx)  # compiles the plan
    torch.cuda.synchronize()
    raise_for(lib.qob_debug_shift_slot(ctx.ptr, hd.ptr, L.QOB_LEFT, L.QOB_C128, n), ctx)
    rc, fl, msg, err = run(bad, tile)
    assert rc == L.QOB_ERR_ARG and fl == 2, (tile, rc, fl)
    assert b"out-of-range" in msg, msg
    assert err > 1e-6, err  # the skipped entries change the result
    rc, fl, msg, err = run(good, tile)
    assert rc == 0 and fl == 0 and err < 1e-12, (tile, rc, fl, err)
print("debug-bounds ok")
'''


def test_debug_bounds_build_reports_bad_index_without_fault():
    sys.path.insert(0, os.path.join(ROOT, "quantumopticsbase.jl_gb300"))
    import build as qob_build

    lib = qob_build.build(debug_bounds=True)
    env = dict(os.environ, QOB_LIBRARY=lib)
    r = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT)], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "debug-bounds ok" in r.stdout
