"""Secondary workloads of the benchmark (``python bench.py --suite``), and the
compact batched / served runs the headline line of ``bench.py`` carries.

One JSON line per workload, each timed with CUDA events on the launching
stream (device-resident data, CUDA-graph replay where the workload is a fixed
launch sequence) or, for the served stream, with the host clock around request
submission and completion:

* ``jc512``       Jaynes-Cummings LazySum, FockBasis(15) x Spin(1/2) x FockBasis(15),
                  mul!(out, H, psi, 0.7-0.2i, 0.3) on one ket and on 64 kets (ComplexF64,
                  ComplexF64 in double-float arithmetic, ComplexF32; also for ``lindblad``);
* ``sparse4096``  sparse(H) of the 32 x 2 x 64 Jaynes-Cummings model: SpMV on a ket
                  and SpMM on 256 columns of a density matrix, FP64 and FP32;
* ``rho_h8``      mul!(rho', rho, H) and mul!(rho', H, rho) with the 8-spin
                  Heisenberg chain on a 256 x 256 operator;
* ``lindblad``    Lindblad right-hand side S rho, lazy Liouvillian of 8 / 10 / 12-spin
                  chains with sigma_- decay (and the materialised one at 8 spins);
* ``particle``    split-operator particle Hamiltonian (FFT operators) on 4096 and 512 x 512 grids;
* ``modek``       LazyTensor mode products with dense factors too large to merge (120,000 and
                  65,536 states, 1 and 16 kets);
* ``dense``       DenseOperator mul! with n = 1024 and 4096 on one and several kets;
* ``cavities256`` 256 two-mode cavity models (dims 81 ... 4225) in one launch;
* ``served``      Poisson arrivals of 100-step RK4 requests (Heisenberg chains of
                  8 ... 16 spins, Jaynes-Cummings models of dim 512 ... 8192).
"""
from __future__ import annotations

import ctypes as C
import json
import time

import numpy as np

import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "quantumopticsbase.jl_gb300"))

from qobgpu import _lib as L  # noqa: E402
from qobgpu.device import dtype_code, get_context, handle, raise_for  # noqa: E402
from qobgpu.hamiltonians import (heisenberg_chain, jaynes_cummings, jaynes_cummings_sparse,  # noqa: E402
                                 random_density_columns, two_mode_cavity)
from qobgpu.rng import Rng  # noqa: E402


def _timed_graph(ctx, stream, record, reps=20):
    """ms per replay of a graph that `record()` issues on `stream`."""
    import torch

    lib = L.lib()
    sp = C.c_void_p(stream.cuda_stream)
    record(sp)  # warm-up: compiles plans, sizes workspaces
    stream.synchronize()
    g = C.c_void_p()
    raise_for(lib.qob_graph_begin(ctx.ptr, sp), ctx)
    record(sp)
    raise_for(lib.qob_graph_end(ctx.ptr, sp, C.byref(g)), ctx)
    for _ in range(3):
        lib.qob_graph_launch(ctx.ptr, g, sp)
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        lib.qob_graph_launch(ctx.ptr, g, sp)
    e1.record(stream)
    e1.synchronize()
    lib.qob_graph_free(ctx.ptr, g)
    return e0.elapsed_time(e1) / reps


def _modes(dmma=False, tc32=False):
    """(torch dtype, numpy dtype, dtype code, label): ComplexF64, ComplexF64 in
    double-float arithmetic (QOB_C128X), ComplexF32; with dmma, also ComplexF64
    on the FP64 tensor cores (QOB_OPT_FP64_TENSOR, "complex128 DMMA"); with
    tc32, also ComplexF32 on the tcgen05 tensor cores (QOB_OPT_FP32_TENSOR,
    "complex64 tcgen05")."""
    import torch

    out = [(torch.complex128, np.complex128, L.QOB_C128, "complex128"),
           (torch.complex128, np.complex128, L.QOB_C128X, "complex128 double-float"),
           (torch.complex64, np.complex64, L.QOB_C64, "complex64")]
    if dmma:
        out.insert(1, (torch.complex128, np.complex128, L.QOB_C128, "complex128 DMMA"))
    if tc32:
        out.append((torch.complex64, np.complex64, L.QOB_C64, "complex64 tcgen05"))
    return tuple(out)


class _Fp64Tensor:
    """The tensor-core option of a row: QOB_OPT_FP64_TENSOR for the rows
    labelled DMMA, QOB_OPT_FP32_TENSOR for those labelled tcgen05."""

    def __init__(self, ctx, label):
        self.ctx = ctx
        self.opt = (L.QOB_OPT_FP64_TENSOR if label.endswith("DMMA")
                    else L.QOB_OPT_FP32_TENSOR if label.endswith("tcgen05") else None)

    def __enter__(self):
        if self.opt:
            raise_for(L.lib().qob_set_option(self.ctx.ptr, self.opt, 1), self.ctx)

    def __exit__(self, *exc):
        if self.opt:
            raise_for(L.lib().qob_set_option(self.ctx.ptr, self.opt, 0), self.ctx)


def _cols(n, k, dt, seed):
    import torch

    g = torch.Generator(device="cuda:0")
    g.manual_seed(seed)
    t = torch.randn(k, n, dtype=dt, device="cuda:0", generator=g)
    return t.t()  # column-major n x k


def _mul_recorder(ctx, h, side, n_out, n_in, ncols, x, y, code, alpha=0.7 - 0.2j, beta=0.3, reps=1):
    lib = L.lib()

    def rec(sp):
        for _ in range(reps):
            if side == L.QOB_LEFT:
                rc = lib.qob_mul(ctx.ptr, L.QOB_LEFT, int(ncols == 1), h.ptr, code, alpha.real, alpha.imag,
                                 C.c_void_p(x.data_ptr()), n_in, ncols, n_in, beta, 0.0, C.c_void_p(y.data_ptr()),
                                 n_out, ncols, n_out, sp)
            else:
                rows = x.shape[0]
                rc = lib.qob_mul(ctx.ptr, L.QOB_RIGHT, 0, h.ptr, code, alpha.real, alpha.imag,
                                 C.c_void_p(x.data_ptr()), rows, n_in, rows, beta, 0.0, C.c_void_p(y.data_ptr()),
                                 rows, n_out, rows, sp)
            raise_for(rc, ctx)

    return rec


def jc512(ctx, stream):
    import torch

    H = jaynes_cummings(15, 15, seed=1)
    h = handle(ctx, H)
    out = []
    for tdt, npdt, code, label in _modes():
        for ncols in (1, 64):
            x = _cols(512, ncols, tdt, 1)
            y = _cols(512, ncols, tdt, 2)
            reps = 50
            ms = _timed_graph(ctx, stream, _mul_recorder(ctx, h, L.QOB_LEFT, 512, 512, ncols, x, y, code,
                                                         reps=reps))
            out.append({"dtype": label, "kets": ncols, "us_per_apply_call": ms * 1e3 / reps,
                        "applies_per_s": ncols * reps / (ms * 1e-3)})
    return {"workload": "jc512", "results": out}


def sparse4096(ctx, stream):
    import torch

    out = []
    for tdt, npdt in ((torch.complex128, np.complex128), (torch.complex64, np.complex64)):
        S = jaynes_cummings_sparse(31, 63, seed=1, dtype=npdt)
        h = handle(ctx, S)
        n = len(S.basis_l)
        nnz = S.data.nnz
        s = 16 if npdt == np.complex128 else 8
        for ncols in (1, 256):
            if ncols == 1:
                x = _cols(n, 1, tdt, 3).contiguous()
                y = _cols(n, 1, tdt, 4).contiguous()
            else:
                rho = random_density_columns(n, 256, seed=5, dtype=npdt)
                x = torch.as_tensor(np.ascontiguousarray(rho.T), device="cuda:0").t()
                y = _cols(n, 256, tdt, 6)
            reps = 20
            ms = _timed_graph(ctx, stream, _mul_recorder(ctx, h, L.QOB_LEFT, n, n, ncols, x, y, dtype_code(npdt), reps=reps))
            t = ms * 1e-3 / reps
            bytes_ = nnz * (s + 4) + (n + 1) * 4 + 3 * n * ncols * s
            out.append({"dtype": np.dtype(npdt).name, "columns": ncols, "nnz": int(nnz), "us_per_call": t * 1e6,
                        "algorithmic_GBps": bytes_ / t / 1e9})
    return {"workload": "sparse4096", "results": out}


def rho_h8(ctx, stream):
    import torch

    H = heisenberg_chain(8, seed=4)
    h = handle(ctx, H)
    out = []
    for tdt, npdt in ((torch.complex128, np.complex128), (torch.complex64, np.complex64)):
        x = _cols(256, 256, tdt, 7)
        y = _cols(256, 256, tdt, 8)
        for side in (L.QOB_LEFT, L.QOB_RIGHT):
            reps = 20
            ms = _timed_graph(ctx, stream, _mul_recorder(ctx, h, side, 256, 256, 256, x, y, dtype_code(npdt), reps=reps))
            out.append({"dtype": np.dtype(npdt).name, "form": "H*rho" if side == L.QOB_LEFT else "rho*H",
                        "us_per_call": ms * 1e3 / reps})
    return {"workload": "rho_h8", "results": out}


def cavities256(ctx, stream, tile=None):
    """256 uneven two-mode cavities in one persistent launch; the tile length
    tuned (qob_batch_tune), or fixed to `tile` (the tuned 256 under a
    profiler, whose replays would time the tuner's candidates differently)."""
    import torch

    from qobgpu.evolution import Batch

    rng = Rng(40)
    models = []
    for k in range(256):
        n1, n2 = rng.integers(2, 8, 64)
        models.append(two_mode_cavity(int(n1), int(n2), seed=1000 + k))
    dims = [len(m.basis_l) for m in models]
    out = []
    for tdt, npdt, code, label in _modes():
        b = Batch(npdt, arith="ff" if code == L.QOB_C128X else None)
        for k, H in enumerate(models):
            x = _cols(dims[k], 1, tdt, 10 + k).contiguous()
            y = _cols(dims[k], 1, tdt, 20 + k).contiguous()
            b.add(H, x, y, 0.7 - 0.2j, 0.3)
        if tile:
            b.set_tile(tile)
            chosen = tile
        else:
            chosen, times = b.tune()
        ms = _timed_graph(ctx, stream, lambda sp: raise_for(L.lib().qob_batch_run(ctx.ptr, b.ptr, sp), ctx), reps=50)
        s = 16 if npdt == np.complex128 else 8
        bytes_ = 3 * sum(dims) * s
        out.append({"dtype": label, "models": 256, "total_dim": int(sum(dims)), "tile": chosen,
                    "us_per_launch": ms * 1e3, "applies_per_s": 256 / (ms * 1e-3),
                    "algorithmic_GBps": bytes_ / (ms * 1e-3) / 1e9, "info": b.info()})
    return {"workload": "cavities256", "results": out}


def lindblad(ctx, stream):
    """Lindblad right-hand side S rho on an N x N density operator: the lazy
    Liouvillian (one fused gather over vec(rho)) for Heisenberg chains of 8, 10
    and 12 spins with sigma_- decay on every spin, and the materialised sparse
    Liouvillian (the reference's form) at 8 spins."""
    import torch

    from qobgpu import operators as O
    from qobgpu import superoperators as SO
    from qobgpu.bases import SpinBasis

    out = []
    for nspins in (8, 10, 12):
        H = heisenberg_chain(nspins, seed=80 + nspins)
        b = H.basis_l
        J = [O.LazyTensor(b, b, (i,), (O.sigmam(SpinBasis("1/2")),)) for i in range(1, nspins + 1)]
        rates = Rng(90 + nspins).uniform(nspins, 0.1, 1.0)
        forms = [("lazy", SO.lazy_liouvillian(H, J, rates=rates))]
        if nspins == 8:
            forms.append(("materialised", SO.liouvillian(O.sparse(H), [O.sparse(j) for j in J], rates=rates)))
        n2 = len(b) ** 2
        for form, L_ in forms:
            h = handle(ctx, L_.vectorised)
            for tdt, npdt, code, label in _modes():
                x = _cols(n2, 1, tdt, 30).contiguous()
                y = _cols(n2, 1, tdt, 31).contiguous()
                reps = 20
                ms = _timed_graph(ctx, stream, _mul_recorder(ctx, h, L.QOB_LEFT, n2, n2, 1, x, y, code,
                                                             alpha=1.0 + 0j, beta=0.0, reps=reps))
                t = ms * 1e-3 / reps
                s = 16 if npdt == np.complex128 else 8
                row = {"spins": nspins, "rho_dim": len(b), "form": form, "dtype": label,
                       "us_per_apply": t * 1e6, "algorithmic_GBps": 2 * n2 * s / t / 1e9}
                if form == "materialised":
                    row["nnz"] = int(L_.data.nnz)
                else:
                    info = (C.c_int64 * 4)()
                    raise_for(L.lib().qob_op_prepare(ctx.ptr, h.ptr, L.QOB_LEFT, code, info), ctx)
                    row["terms"] = len(L_.operator.operators)
                    row["groups"] = int(info[0])
                out.append(row)
            del h
    return {"workload": "lindblad", "results": out}


def particle(ctx, stream):
    """Split-operator particle Hamiltonian H = Txp (p^2/2) Tpx + V(x) (LazySum of a
    LazyProduct of FFT operators and diagonals, src/particle.jl) on a 1-D grid of
    4096 points (1 and 64 kets) and a 2-D grid of 512 x 512 points (1 ket), and
    the bare FFT transform Tpx on the same grids."""
    import torch

    from qobgpu import operators as O
    from qobgpu.bases import MomentumBasis, PositionBasis
    from qobgpu.bases import tensor as tensor_bases
    from qobgpu.particle import momentum, potentialoperator, transform

    out = []
    grids = [("1d_4096", [PositionBasis(-40.0, 40.0, 4096)]),
             ("2d_512x512", [PositionBasis(-20.0, 20.0, 512), PositionBasis(-20.0, 20.0, 512)])]
    for name, bxs in grids:
        bps = [MomentumBasis(b) for b in bxs]
        bX = bxs[0] if len(bxs) == 1 else tensor_bases(*bxs)
        bP = bps[0] if len(bps) == 1 else tensor_bases(*bps)
        Txp, Tpx = transform(bX, bP), transform(bP, bX)
        n = len(bX)
        # kinetic energy diagonal on the momentum grid, potential on the position grid
        kin = np.zeros(n)
        for i, b in enumerate(bps):
            p = np.asarray(momentum(b).data.diagonal()).real
            stride = int(np.prod([len(x) for x in bps[:i]]))
            kin += np.tile(np.repeat(p * p / 2, stride), n // (stride * len(b)))
        K = O.Operator(bP, bP, O.spdiagm(n, n, {0: kin.astype(complex)}))
        V = potentialoperator(bX, (lambda x: 0.5 * x * x) if len(bxs) == 1 else (lambda x, y: 0.5 * (x * x + y * y)))
        H = O.LazySum(bX, bX, [1.0, 1.0], (O.LazyProduct((Txp, K, Tpx)), V))
        for op_name, op in (("H", H), ("Tpx", Tpx)):
            h = handle(ctx, op)
            for tdt, npdt, code, label in _modes():
                for ncols in ((1, 64) if len(bxs) == 1 else (1,)):
                    x = _cols(n, ncols, tdt, 50).contiguous() if ncols == 1 else _cols(n, ncols, tdt, 50)
                    y = _cols(n, ncols, tdt, 51).contiguous() if ncols == 1 else _cols(n, ncols, tdt, 51)
                    reps = 20
                    ms = _timed_graph(ctx, stream, _mul_recorder(ctx, h, L.QOB_LEFT, n, n, ncols, x, y,
                                                                 code, reps=reps))
                    t = ms * 1e-3 / reps
                    out.append({"grid": name, "operator": op_name, "dtype": label, "kets": ncols,
                                "us_per_call": t * 1e6, "applies_per_s": ncols / t})
    return {"workload": "particle", "results": out}


def served(ctx, stream, nreq=192, rate=2000.0, seed=50):
    from qobgpu.evolution import Server

    rng = Rng(seed)
    pool = [heisenberg_chain(n, seed=60 + n) for n in (8, 10, 12, 14, 16)]
    pool += [jaynes_cummings(15, 15, seed=70), jaynes_cummings(31, 63, seed=71), jaynes_cummings(63, 63, seed=72)]
    picks = rng.integers(nreq, 0, len(pool) - 1)
    gaps = -np.log(1.0 - rng.uniform(nreq)) / rate
    psis = [rng.ket_data(len(pool[p].basis_l)) for p in picks]
    results = {}
    for npdt, arith, label in ((np.complex64, None, "complex64"), (np.complex128, None, "complex128"),
                               (np.complex128, "ff", "complex128 double-float")):
        S = Server(npdt, mem_budget=16 << 30, max_active=256, arith=arith)
        for H in pool:  # compile plans before the clock starts
            S.submit(H, np.zeros(len(H.basis_l)), 1, 1e-3)
        while S.step():
            pass
        S.start()
        ids = []
        t0 = time.perf_counter()
        for k in range(nreq):
            ids.append(S.submit(pool[picks[k]], psis[k], 100, 1e-3))
            time.sleep(gaps[k])
        for i in ids:
            S.wait(i, 600.0)
        wall = time.perf_counter() - t0
        lat, res = [], []
        for i in ids:
            st, tm, r = S.poll(i)
            lat.append(tm[2] - tm[0])
            res.append(r)
        stats = S.stats()
        S.stop()
        S.close()
        results[label] = {"p50_ms": float(np.percentile(lat, 50) * 1e3),
                                        "p99_ms": float(np.percentile(lat, 99) * 1e3),
                                        "requests_per_s": nreq / wall, "applies_per_s": nreq * 400 / wall,
                                        "wall_s": wall, "engine_iterations": stats["iterations"], "res": res}
    def errs(name):
        return [float(np.linalg.norm(a.astype(np.complex128) - b) / np.linalg.norm(b))
                for a, b in zip(results[name]["res"], results["complex128"]["res"])]

    e32, eff = errs("complex64"), errs("complex128 double-float")
    for v in results.values():
        v.pop("res")
    return {"workload": "served", "requests": nreq, "poisson_rate_per_s": rate, "steps_per_request": 100,
            "dt": 1e-3, "results": results, "fp32_rel_err_vs_fp64_max": max(e32),
            "fp32_rel_err_vs_fp64_median": float(np.median(e32)), "double_float_rel_err_vs_fp64_max": max(eff)}


def host_link(ctx, stream):
    """Pinned host <-> device copy bandwidth (explains the end-to-end numbers)."""
    import torch

    n = 64 * 16384  # one 64-ket ComplexF64 batch: 16 MiB
    h = torch.empty(n, dtype=torch.complex128).pin_memory()
    d = torch.empty(n, dtype=torch.complex128, device="cuda:0")
    out = {}
    for name, fn in (("h2d", lambda: d.copy_(h, non_blocking=True)), ("d2h", lambda: h.copy_(d, non_blocking=True))):
        with torch.cuda.stream(stream):
            for _ in range(3):
                fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(20):
                fn()
            e1.record(stream)
        e1.synchronize()
        out[name + "_GBps"] = 20 * n * 16 / (e0.elapsed_time(e1) * 1e-3) / 1e9
    return {"workload": "host_link", "bytes_per_copy": n * 16, "results": out}


def modek(ctx, stream):
    """Mode products of a LazyTensor whose dense factors are too large to merge
    (_tp_sum_matmul!'s path): two 200 x 200 dense factors on the outer sites of
    FockBasis(199) x Spin(1) x FockBasis(199) (120,000 states), one ket and 16
    kets; and one 64 x 64 dense factor with a 16 x 16 one on a 64 x 16 x 64 space."""
    import torch

    from qobgpu import operators as O
    from qobgpu.bases import GenericBasis
    from qobgpu.bases import tensor as tensor_basis

    rng = Rng(60)

    def dense(d):
        a = rng.complex_normal(d * d).reshape(d, d, order="F")
        return O.Operator(GenericBasis(d), GenericBasis(d), np.asfortranarray(a))

    out = []
    for dims, sites in (((200, 3, 200), (1, 3)), ((64, 16, 64), (1, 2))):
        bs = [GenericBasis(d) for d in dims]
        b = tensor_basis(*bs)
        facs = tuple(dense(dims[s - 1]) for s in sites)
        op = O.LazyTensor(b, b, sites, facs, 0.3)
        h = handle(ctx, op)
        n = len(b)
        for tdt, npdt, code, label in _modes(dmma=True, tc32=True):
            for ncols in (1, 16):
                x = _cols(n, ncols, tdt, 61)
                y = _cols(n, ncols, tdt, 62)
                reps = 5
                with _Fp64Tensor(ctx, label):
                    ms = _timed_graph(ctx, stream, _mul_recorder(ctx, h, L.QOB_LEFT, n, n, ncols, x, y, code,
                                                                 reps=reps))
                t = ms * 1e-3 / reps
                flops = 8.0 * n * ncols * sum(dims[s - 1] for s in sites)  # complex FMA = 8 flop per term
                out.append({"dims": list(dims), "dense_sites": list(sites), "dtype": label, "kets": ncols,
                            "us_per_call": t * 1e6, "tflops": flops / t / 1e12})
        del h
    return {"workload": "modek", "results": out}


def dense(ctx, stream):
    """DenseOperator mul! (gemv / gemm): n x n dense operators, n = 1024 and 4096,
    on 1 and 64 / 16 kets."""
    from qobgpu import operators as O
    from qobgpu.bases import GenericBasis

    rng = Rng(70)
    out = []
    for nd, kets in ((1024, (1, 64)), (4096, (1, 16))):
        b = GenericBasis(nd)
        op = O.Operator(b, b, np.asfortranarray(rng.complex_normal(nd * nd).reshape(nd, nd, order="F")))
        h = handle(ctx, op)
        for tdt, npdt, code, label in _modes(dmma=True, tc32=True):
            for ncols in kets:
                x = _cols(nd, ncols, tdt, 71)
                y = _cols(nd, ncols, tdt, 72)
                reps = 5
                with _Fp64Tensor(ctx, label):
                    ms = _timed_graph(ctx, stream, _mul_recorder(ctx, h, L.QOB_LEFT, nd, nd, ncols, x, y, code,
                                                                 reps=reps))
                t = ms * 1e-3 / reps
                s_ = 16 if npdt == np.complex128 else 8
                out.append({"n": nd, "dtype": label, "kets": ncols, "us_per_call": t * 1e6,
                            "tflops": 8.0 * nd * nd * ncols / t / 1e12,
                            "matrix_GBps": nd * nd * s_ / t / 1e9})
        del h
    return {"workload": "dense", "results": out}


WORKLOADS = ("jc512", "sparse4096", "rho_h8", "lindblad", "particle", "modek", "dense", "cavities256", "served",
             "host_link")


def run_suite(device: int = 0, only=None, pdl: int = 1, batch_tile=None):
    """Run the workloads (all, or the names in `only`), one JSON line each,
    with programmatic dependent launch on (pdl = 1, as the headline bench) or
    off; batch_tile fixes the persistent batch's tile length instead of
    tuning it."""
    import torch

    ctx = get_context(device)
    raise_for(L.lib().qob_set_option(ctx.ptr, L.QOB_OPT_PDL, int(pdl)), ctx)
    stream = torch.cuda.Stream(device)
    names = [w for w in WORKLOADS if not only or w in only]
    for fn in (globals()[w] for w in names):
        t0 = time.perf_counter()
        line = fn(ctx, stream, batch_tile) if fn is cavities256 and batch_tile else fn(ctx, stream)
        line["seconds"] = time.perf_counter() - t0
        line["pdl"] = bool(pdl)
        print(json.dumps(line), flush=True)
