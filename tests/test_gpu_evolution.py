"""GPU tests of the batched, time-evolution and serving paths.

* uneven batches (two-mode cavities of different dimensions, one launch)
  against the oracle's mul! per model, FP64 and FP32, also replayed from a
  CUDA graph;
* RK4 against an RK4 on the host whose right-hand side is the oracle's mul!;
* the server: a request's result is bitwise the same alone and in a mix of
  other requests that arrive before and after it; requests larger than the
  memory budget are rejected while the rest are served.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as OR
import qobgpu as Q
from helpers import rel_l2
from qobgpu.hamiltonians import heisenberg_chain, jaynes_cummings, two_mode_cavity

pytestmark = pytest.mark.gpu


def rk4_host(H, psi, dt, nsteps):
    """Fixed-step RK4 of dpsi/dt = -i H psi with the oracle's mul! as right-hand side."""
    node = OR.build_node(H)

    def f(v):
        return OR.mul_arrays(0, True, node, -1j, v, 0.0, np.zeros_like(v))

    psi = np.array(psi, dtype=np.complex128)
    for _ in range(nsteps):
        k1 = f(psi)
        k2 = f(psi + dt / 2 * k1)
        k3 = f(psi + dt / 2 * k2)
        k4 = f(psi + dt * k3)
        psi = psi + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
    return psi


def cavity_models(count, seed):
    rng = Q.Rng(seed)
    out = []
    for k in range(count):
        n1, n2 = rng.integers(2, 8, 64)
        out.append(two_mode_cavity(int(n1), int(n2), seed=100 + k))
    return out


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-5)])
def test_uneven_batch_matches_oracle(dtype, tol):
    import torch

    from qobgpu.evolution import Batch

    models = cavity_models(24, seed=7)
    rng = Q.Rng(8)
    b = Batch(dtype)
    xs, ys, ref = [], [], []
    tdt = torch.complex64 if dtype == np.complex64 else torch.complex128
    for H in models:
        n = len(H.basis_l)
        x = rng.ket_data(n)
        y = rng.ket_data(n)
        a, be = 0.7 - 0.2j, 0.3
        ref.append(OR.mul(Q.Ket(H.basis_l, y), H, Q.Ket(H.basis_r, x), a, be))
        xd = torch.as_tensor(x.astype(dtype), device="cuda:0")
        yd = torch.as_tensor(y.astype(dtype), device="cuda:0")
        b.add(H, xd, yd, a, be)
        xs.append(xd)
        ys.append(yd)
    y0 = [t.clone() for t in ys]
    b.run()
    torch.cuda.synchronize()
    info = b.info()
    assert info["fused"] == len(models)
    for yd, r in zip(ys, ref):
        assert rel_l2(yd.cpu().numpy().astype(np.complex128), r) < tol
    # replay from a CUDA graph after restoring the outputs
    for yd, y in zip(ys, y0):
        yd.copy_(y)
    from qobgpu import _lib as L

    lib = L.lib()
    s = torch.cuda.Stream()
    sp = C.c_void_p(s.cuda_stream)
    g = C.c_void_p()
    assert lib.qob_graph_begin(b.ctx.ptr, sp) == 0
    assert lib.qob_batch_run(b.ctx.ptr, b.ptr, sp) == 0
    assert lib.qob_graph_end(b.ctx.ptr, sp, C.byref(g)) == 0
    assert lib.qob_graph_launch(b.ctx.ptr, g, sp) == 0
    s.synchronize()
    lib.qob_graph_free(b.ctx.ptr, g)
    for yd, r in zip(ys, ref):
        assert rel_l2(yd.cpu().numpy().astype(np.complex128), r) < tol
    # beta == 0 overwrites outputs that hold NaN (src/operators_lazysum.jl:179-186)
    b0 = Batch(dtype)
    outs, ref0 = [], []
    for H, xd in zip(models[:6], xs[:6]):
        yd = torch.full((len(H.basis_l),), complex("nan"), dtype=tdt, device="cuda:0")
        b0.add(H, xd, yd, 0.5, 0.0)
        outs.append(yd)
        x = xd.cpu().numpy().astype(np.complex128)
        ref0.append(OR.mul(Q.Ket(H.basis_l, np.zeros(len(H.basis_l), complex)), H, Q.Ket(H.basis_r, x), 0.5, 0.0))
    b0.run()
    torch.cuda.synchronize()
    for yd, r in zip(outs, ref0):
        got = yd.cpu().numpy().astype(np.complex128)
        assert np.all(np.isfinite(got)) and rel_l2(got, r) < tol


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-5)])
def test_batch_set_tile_every_length_matches_oracle(dtype, tol):
    """qob_batch_set_tile fixes the persistent launch's tile length without
    timing: every allowed length (128 .. 1024 output indices, so tiles that
    cover several items' ends and items longer than one tile) gives the oracle's
    result, qob_batch_info reports the length and tile count, and a length
    outside the four is refused with QOB_ERR_ARG."""
    import torch

    from qobgpu import _lib as L
    from qobgpu.evolution import Batch

    models = cavity_models(12, seed=17)
    rng = Q.Rng(18)
    data = []
    for H in models:
        n = len(H.basis_l)
        data.append((H, rng.ket_data(n), rng.ket_data(n)))
    ref = [OR.mul(Q.Ket(H.basis_l, y), H, Q.Ket(H.basis_r, x), 0.7 - 0.2j, 0.3) for H, x, y in data]
    for tile in (128, 256, 512, 1024):
        b = Batch(dtype)
        ys = []
        for H, x, y in data:
            yd = torch.as_tensor(y.astype(dtype), device="cuda:0")
            b.add(H, torch.as_tensor(x.astype(dtype), device="cuda:0"), yd, 0.7 - 0.2j, 0.3)
            ys.append(yd)
        b.set_tile(tile)
        info = b.info()
        assert info["tile"] == tile
        assert info["tiles"] == sum(-(-len(H.basis_l) // tile) for H, _, _ in data)
        b.run()
        torch.cuda.synchronize()
        for yd, r in zip(ys, ref):
            assert rel_l2(yd.cpu().numpy().astype(np.complex128), r) < tol, tile
    assert L.lib().qob_batch_set_tile(b.ctx.ptr, b.ptr, 300) == L.QOB_ERR_ARG


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 1e-5)])
def test_rk4_matches_host_rk4(dtype, tol):
    import torch

    from qobgpu.evolution import rk4

    H = heisenberg_chain(8, seed=11)
    psi0 = Q.Rng(12).ket_data(len(H.basis_l))
    ref = rk4_host(H, psi0, 1e-3, 20)
    d = torch.as_tensor(psi0.astype(dtype), device="cuda:0")
    rk4(H, d, 1e-3, 20)
    assert rel_l2(d.cpu().numpy().astype(np.complex128), ref) < tol


def test_server_result_same_alone_and_in_the_mix():
    from qobgpu.evolution import Server

    target = heisenberg_chain(10, seed=21)
    psi = Q.Rng(22).ket_data(len(target.basis_l))
    others = [jaynes_cummings(15, 15, seed=23), heisenberg_chain(12, seed=24), jaynes_cummings(31, 63, seed=25)]
    rng = Q.Rng(26)

    S = Server(np.complex128)
    rid = S.submit(target, psi, 30, 1e-3)
    while S.step():
        pass
    st, _, alone = S.poll(rid)
    assert st == 2
    S.close()

    S = Server(np.complex128)
    early = [S.submit(H, rng.ket_data(len(H.basis_l)), 40, 1e-3) for H in others[:2]]
    for _ in range(5):
        S.step()
    rid = S.submit(target, psi, 30, 1e-3)  # joins while others run
    S.step()
    late = S.submit(others[2], rng.ket_data(len(others[2].basis_l)), 10, 1e-3)
    while S.step():
        pass
    st, times, mixed = S.poll(rid)
    assert st == 2 and times[0] <= times[1] <= times[2]
    assert np.array_equal(alone, mixed), "result differs between alone and in the mix"
    for r in early + [late]:
        assert S.poll(r)[0] == 2
    assert rel_l2(mixed, rk4_host(target, psi, 1e-3, 30)) < 1e-12
    S.close()


def test_server_worker_thread_and_budget_rejection():
    from qobgpu.evolution import Server

    small = heisenberg_chain(8, seed=31)
    big = heisenberg_chain(14, seed=32)
    budget = 4 * len(small.basis_l) * 16 * 3  # room for three small requests, never for the big one
    S = Server(np.complex128, mem_budget=budget, max_active=8)
    S.start()
    rng = Q.Rng(33)
    ids = [S.submit(small, rng.ket_data(len(small.basis_l)), 25, 1e-3) for _ in range(6)]
    rbig = S.submit(big, rng.ket_data(len(big.basis_l)), 5, 1e-3)
    for i in ids:
        assert S.wait(i, 60.0) == 2
    st, _, _ = S.poll(rbig)
    assert st == -6  # QOB_ERR_OOM: larger than the budget, rejected at submission
    stats = S.stats()
    assert stats["completed"] == 6 and stats["rejected"] == 1 and stats["device_bytes"] == 0
    S.stop()
    S.close()


def test_server_cancel_queued_and_running():
    """qob_server_cancel: a queued request leaves at once, a running one before
    the engine's next iteration; both end with status -QOB_ERR_CANCELLED, their
    memory back, and the other requests' results are unchanged."""
    from qobgpu.evolution import Server

    H = heisenberg_chain(8, seed=41)
    rng = Q.Rng(42)
    psis = [rng.ket_data(len(H.basis_l)) for _ in range(3)]
    S = Server(np.complex128, max_active=1)  # one at a time: the second waits in the queue
    a = S.submit(H, psis[0], 40, 1e-3)
    b = S.submit(H, psis[1], 40, 1e-3)
    S.step()  # a runs, b is queued
    assert S.poll(b)[0] == 0
    S.cancel(b)
    assert S.poll(b)[0] == -9
    c = S.submit(H, psis[2], 400, 1e-3)
    while S.poll(a)[0] != 2:
        S.step()
    S.step()  # c is admitted and runs
    assert S.poll(c)[0] == 1
    S.cancel(c)
    S.step()  # retired before this iteration steps
    st = S.poll(c)[0]
    assert st == -9
    stats = S.stats()
    assert stats["cancelled"] == 2 and stats["active"] == 0 and stats["device_bytes"] == 0
    assert rel_l2(S.poll(a)[2], rk4_host(H, psis[0], 1e-3, 40)) < 1e-12
    d = S.submit(H, psis[1], 20, 1e-3)  # the server goes on
    while S.step():
        pass
    assert S.poll(d)[0] == 2
    assert rel_l2(S.poll(d)[2], rk4_host(H, psis[1], 1e-3, 20)) < 1e-12
    import pytest as _pytest

    from qobgpu.device import QobError

    with _pytest.raises(QobError):
        S.cancel(d)  # already finished: QOB_ERR_STATE
    S.close()


def test_server_alloc_hook_queues_then_rejects():
    """A host-side allocation hook that refuses memory: with other requests
    running the new one waits in the queue and runs once the hook allows it (same
    result as alone); with nothing running it is rejected with -QOB_ERR_OOM
    after three refusals; the server keeps serving afterwards."""
    from qobgpu.evolution import Server

    H = heisenberg_chain(8, seed=43)
    rng = Q.Rng(44)
    p0, p1, p2 = (rng.ket_data(len(H.basis_l)) for _ in range(3))
    S = Server(np.complex128)
    a = S.submit(H, p0, 30, 1e-3)
    S.step()  # a admitted
    allow = {"on": False}
    asked = []

    def hook(nbytes):
        asked.append(nbytes)
        return allow["on"]

    S.set_alloc_hook(hook)
    b = S.submit(H, p1, 30, 1e-3)
    for _ in range(3):
        S.step()
    assert S.poll(b)[0] == 0 and asked  # refused, still queued while a runs
    allow["on"] = True
    while S.step():
        pass
    assert S.poll(a)[0] == 2 and S.poll(b)[0] == 2
    assert rel_l2(S.poll(b)[2], rk4_host(H, p1, 1e-3, 30)) < 1e-12
    allow["on"] = False
    c = S.submit(H, p2, 10, 1e-3)
    for _ in range(4):
        S.step()
    assert S.poll(c)[0] == -6  # nothing else active: rejected after three refusals
    st = S.stats()
    assert st["alloc_refusals"] >= 4 and st["device_bytes"] == 0
    S.set_alloc_hook(None)
    d = S.submit(H, p2, 10, 1e-3)
    while S.step():
        pass
    assert S.poll(d)[0] == 2
    S.close()
