#!/usr/bin/env python3
"""LazySum·ket applies/s on GB300 for QuantumOpticsBase.jl's mul! hot path.

Workload: the 14-spin open Heisenberg chain, H = Σ J(σxσx + σyσy + σzσz) +
Σ h_i σz_i (dim 16384, 53 LazyTensor terms, J = 1, h_i ~ U(-1, 1)), applied as
mul!(Y, H, X, α = 0.7 - 0.2i, β = 0.3) to batches of 64 normalised
complex-Gaussian kets.  One step = one application to one 64-ket batch.
Twenty distinct batches rotate (1280 kets, 640 MiB of input + output in
ComplexF64, more than twice the 129 MB L2), so every step streams its kets from
HBM.

`value` is the plain ComplexF64 form, device-resident, replayed from a CUDA
graph and timed with CUDA events on the launching stream.  `e2e` is the same
metric through the C ABI's host-buffer calls (qob_mul_host_async +
qob_host_wait; `sync_value`: qob_mul_host) with the kets copied from pinned host
memory and the results copied back every step.  The ComplexF32 and the
double-float modes are reported beside it, with their errors against the
ComplexF64 result.

`--impl reference` times the CPU restatement of the reference mul! (the
oracle port; Julia is not available) on all host threads, same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "quantumopticsbase.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "LazySum·ket applies/s (14-spin Heisenberg, batch 64)"
UNIT = "applies/s"
NSPINS, BATCH, ROTATE = 14, 64, 20
ALPHA, BETA = 0.7 - 0.2j, 0.3
# launch shapes of qob_op_tune, in its order (threads per block, P = persistent, sN = N ket sets per warp)
SHAPES = ("128", "256", "P256", "128s4", "256s4", "128s8", "256s8", "128s16", "256s16")
# staged-tile shapes of qob_op_tune, in its order: (tile bits, kets per thread, ket sets per warp)
TILE_SHAPES = ((10, 1, 1), (10, 2, 1), (9, 4, 1), (11, 1, 1), (11, 2, 1), (12, 1, 1), (9, 1, 4), (8, 1, 16),
               (8, 2, 8), (9, 2, 4), (10, 1, 4), (7, 2, 16))
# index-pair shapes of qob_op_tune_ex, in its order: (kets per thread, threads, ket sets per warp)
PAIR_SHAPES = ((2, 256, 1), (4, 256, 1), (2, 128, 1), (4, 128, 1), (2, 256, 4), (4, 128, 4), (2, 128, 8), (4, 128, 8),
               (2, 128, 16), (4, 128, 16))
NCANDS = 36 + len(TILE_SHAPES) + len(PAIR_SHAPES)
SEED_H = 3
ORACLE_BUILD = ("oracle/liboref.so, g++ -O3 -ffp-contract=off: every multiply and add rounded separately, as the "
                "reference's Julia code computes; portable flags (no -march=native), the same binary that checks "
                "parity")
# GB300's FP64 pipe: 2 DFMA lanes per SM clock (ncu's peak_sustained for
# sm__sass_thread_inst_executed_op_dfma_pred_on; the dense ComplexF64 product
# sustains 1.96 of them)
FP64_LANES_PER_SM_CLOCK = 2
L2_NOTE = "20 distinct 64-ket batches rotate: 640 MiB (c128) / 320 MiB (c64) of in+out per rotation, > 2x the 129 MB L2"


def config():
    return {
        "workload": "heisenberg14_lazysum_ket_batch64",
        "dim": 2 ** NSPINS,
        "terms": 3 * (NSPINS - 1) + NSPINS,
        "batch_kets": BATCH,
        "alpha": [ALPHA.real, ALPHA.imag],
        "beta": [BETA, 0.0],
        "l2": L2_NOTE,
        "parallelism": "replicas",
    }


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="own", choices=["own", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-graph", action="store_true", help="direct launches (used for ncu captures)")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--shape", default=None,
                   help="fixed launch shapes instead of tuning, e.g. c128=4x256s4,c64=4x128 (used for ncu captures)")
    p.add_argument("--suite", action="store_true", help="secondary workloads, one JSON line each")
    p.add_argument("--only", nargs="*", default=None, help="with --suite: these workloads only")
    p.add_argument("--probe", action="store_true", help="print the device's measured FP64 / FP32 FMA rates")
    p.add_argument("--pdl", type=int, default=1, choices=[0, 1],
                   help="programmatic dependent launch (QOB_OPT_PDL) for every timed form (default on: the steps "
                        "measured 1-3 %% faster with it); the other setting is timed beside it in the pdl sub-object")
    p.add_argument("--batch-tile", type=int, default=None, choices=[128, 256, 512, 1024],
                   help="with --suite: fix the uneven batch's tile length instead of tuning it (for profiling)")
    p.add_argument("--no-secondary", action="store_true",
                   help="leave out the batched and served sub-objects (used for ncu captures)")
    return p.parse_args()


def read_json(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples (SM clock, throttle reasons) tagged with host time."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.samples = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        if not self.samples:
            return None
        inside = [s for t, s in self.samples if t0 <= t <= t1 + 0.15]
        note = None
        if not inside:  # timed region shorter than the sampling period: nearest samples
            inside = [min(self.samples, key=lambda ts: abs(ts[0] - (t0 + t1) / 2))[1]]
            note = "timed region shorter than the 100 ms sampling period; nearest sample"
        mhz = [float(s[0]) for s in inside if s[0].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for s in inside for n, v in zip(names, s[3:7]) if v == "Active"})
        out = {"sm_mhz": statistics.median(mhz) if mhz else None,
               "sm_max_mhz": float(inside[0][1]) if inside[0][1].replace(".", "").isdigit() else None,
               "reasons": reasons, "samples": len(inside)}
        if note:
            out["note"] = note
        return out


# ---------------------------------------------------------------------------
def max_over_ranks(value: float, world: int, device=None) -> float:
    """The largest per-rank value (the slowest rank's time) on every rank; the
    process group's backend decides where the reduction runs (NCCL: the GPU)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    if device is None:
        device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units per second over all ranks for weak scaling (every rank does the
    same work; the slowest rank's time bounds the job)."""
    return units_per_rank * world / seconds


def reference_flops(H) -> int:
    """Flops of one term-by-term application as the reference evaluates a
    LazySum (src/operators_lazysum.jl:194-197): each LazyTensor term visits
    dim_rest x prod(nnz of its factors) entries (src/operators_lazytensor.jl:652-685),
    8 flops per complex multiply-add, plus 8 per element for the beta scaling."""
    import numpy as np
    import scipy.sparse as sp

    dim = len(H.basis_r)
    total = 0
    for t in H.operators:
        nnz, covered = 1, 1
        for op in t.operators:
            d = op.data
            nnz *= int(d.nnz) if sp.issparse(d) else int(np.count_nonzero(d))
            covered *= len(op.basis_r)
        total += (dim // covered) * nnz
    return 8 * total + 8 * dim


def cpu_baseline(H, seconds: float):
    """The oracle port (restated reference mul!) on this host: single thread,
    kets applied one at a time until `seconds` pass; then all threads."""
    import numpy as np

    import oracle as OR
    import qobgpu as Q

    node = OR.build_node(H)
    dim = len(H.basis_l)
    rng = Q.Rng(99)
    X = rng.kets_data(dim, 1)
    Y = rng.kets_data(dim, 1)
    n, t0 = 0, time.perf_counter()
    while True:
        OR.mul_kets_threaded(node, ALPHA, X, BETA, Y, 1)
        n += 1
        if time.perf_counter() - t0 >= seconds and n >= 4:
            break
    single = n / (time.perf_counter() - t0)
    threads = os.cpu_count() or 1
    Xa = np.asfortranarray(np.repeat(X, threads * 2, axis=1))
    Ya = np.asfortranarray(np.repeat(Y, threads * 2, axis=1))
    t0 = time.perf_counter()
    OR.mul_kets_threaded(node, ALPHA, Xa, BETA, Ya, threads)
    allc = Xa.shape[1] / (time.perf_counter() - t0)
    return {"value": single, "unit": UNIT, "cores": 1, "kind": "port", "build": ORACLE_BUILD,
            "sample": f"{n} kets of the 14-spin Heisenberg LazySum, mul!(y, H, x, α, β) one ket at a time on one "
                      f"thread (restated reference CPU path; Julia absent), {seconds:.0f} s bound",
            "all_cores": {"value": allc, "cores": threads, "sample": f"{Xa.shape[1]} kets over {threads} threads"}}


# ---------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return
    import numpy as np

    import oracle as OR
    import qobgpu as Q
    from qobgpu.hamiltonians import heisenberg_chain

    H = heisenberg_chain(NSPINS, seed=SEED_H)
    node = OR.build_node(H)
    threads = os.cpu_count() or 1
    dim = len(H.basis_l)
    rng = Q.Rng(98)
    X = rng.kets_data(dim, threads)
    Y = rng.kets_data(dim, threads)
    for _ in range(args.warmup):
        OR.mul_kets_threaded(node, ALPHA, X, BETA, Y, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        OR.mul_kets_threaded(node, ALPHA, X, BETA, Y, threads)
    dt = time.perf_counter() - t0
    value = threads * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded complex-Gaussian kets)", "config": config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "build": ORACLE_BUILD,
                         "sample": f"each step applies H to {threads} kets, one per host thread "
                                   "(restated reference CPU path; Julia absent)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_own(args, rank, world, local_rank):
    import ctypes as C

    import numpy as np
    import torch

    import qobgpu as Q
    from qobgpu import _lib as L
    from qobgpu.device import dtype_code, get_context, handle, prepare, raise_for
    from qobgpu.hamiltonians import heisenberg_chain

    dev = local_rank
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    lib = L.lib()
    H = heisenberg_chain(NSPINS, seed=SEED_H)
    ctx = get_context(dev)
    hd = handle(ctx, H)
    dim = len(H.basis_l)
    stream = torch.cuda.Stream(dev)
    sp = C.c_void_p(stream.cuda_stream)
    plan = prepare(H, L.QOB_LEFT, np.complex128, dev)
    sampler = ClockSampler(dev) if rank == 0 else None

    gen = torch.Generator(device=f"cuda:{dev}")
    gen.manual_seed(1234 + rank)

    def batches(tdt):
        xs, ys = [], []
        for _ in range(ROTATE):
            for lst in (xs, ys):
                t = torch.randn(BATCH, dim, dtype=tdt, device=f"cuda:{dev}", generator=gen)
                t /= torch.linalg.vector_norm(t, dim=1, keepdim=True)
                lst.append(t.t())  # column-major dim x 64, ld = dim
        return xs, ys

    def mul_args(x, y, code):
        return (ctx.ptr, L.QOB_LEFT, 0, hd.ptr, code, ALPHA.real, ALPHA.imag, C.c_void_p(x.data_ptr()), dim, BATCH,
                dim, BETA, 0.0, C.c_void_p(y.data_ptr()), dim, BATCH, dim, sp)

    def timed(tdt, code, steps, warmup):
        xs, ys = batches(tdt)
        argl = [mul_args(xs[b], ys[b], code) for b in range(ROTATE)]
        with torch.cuda.stream(stream):
            for i in range(warmup):
                raise_for(lib.qob_mul(*argl[i % ROTATE]), ctx)
        stream.synchronize()
        n0 = lib.qob_kernel_launches()
        graph = None
        if not args.no_graph:
            g = C.c_void_p()
            reps, per = (steps // ROTATE, ROTATE) if steps % ROTATE == 0 and steps >= ROTATE else (1, steps)
            raise_for(lib.qob_graph_begin(ctx.ptr, sp), ctx)
            for i in range(per):
                raise_for(lib.qob_mul(*argl[i % ROTATE]), ctx)
            raise_for(lib.qob_graph_end(ctx.ptr, sp, C.byref(g)), ctx)
            graph = g
            launches = (lib.qob_kernel_launches() - n0) * reps
            raise_for(lib.qob_graph_launch(ctx.ptr, graph, sp), ctx)  # one untimed replay
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t_host0 = time.time()
        e0.record(stream)
        if graph is not None:
            for _ in range(reps):
                raise_for(lib.qob_graph_launch(ctx.ptr, graph, sp), ctx)
        else:
            n1 = lib.qob_kernel_launches()
            for i in range(steps):
                raise_for(lib.qob_mul(*argl[i % ROTATE]), ctx)
            launches = lib.qob_kernel_launches() - n1
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize(dev)
        t_host1 = time.time()
        ms = max_over_ranks(e0.elapsed_time(e1), world, f"cuda:{dev}")
        if graph is not None:
            lib.qob_graph_free(ctx.ptr, graph)
        return ms, launches, (t_host0, t_host1), (xs, ys)

    def step_stats(tdt, code, n=200):
        """Per-step times (CUDA events around each single application):
        cold -- the batches rotate (inputs beyond L2); warm -- one batch again and
        again.  host_driven: each step issued as the previous one runs, so a step
        whose launch the host has not yet issued when the device gets to it
        counts the wait; device: the same steps queued behind 16 copies of a
        1 GiB buffer (about 5 ms of device work), so the host is far ahead and
        the events hold device time only (max_gap_ms: the largest device idle
        time between two steps, ~0 when the queue stayed full)."""
        xs, ys = batches(tdt)
        argl = [mul_args(xs[b], ys[b], code) for b in range(ROTATE)]
        blk = torch.empty(2, 1 << 26, dtype=torch.complex128, device=f"cuda:{dev}")  # 2 x 1 GiB
        out = {}
        for mode in ("host_driven", "device"):
            for name, pick in (("cold", lambda i: argl[i % ROTATE]), ("warm", lambda i: argl[0])):
                evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
                with torch.cuda.stream(stream):
                    for i in range(5):
                        raise_for(lib.qob_mul(*pick(i)), ctx)
                    stream.synchronize()
                    if mode == "device":
                        for _ in range(16):
                            blk[1].copy_(blk[0])
                    for i in range(n):
                        evs[i][0].record(stream)
                        raise_for(lib.qob_mul(*pick(i)), ctx)
                        evs[i][1].record(stream)
                stream.synchronize()
                raw = [a.elapsed_time(b) for a, b in evs]
                t = sorted(raw)
                key = f"{mode}_{name}"
                out[key + "_median_ms"] = t[n // 2]
                out[key + "_p99_ms"] = t[min(n - 1, int(0.99 * n))]
                out[key + "_max_ms"] = t[-1]
                if mode == "device":
                    out[key + "_max_gap_ms"] = max(evs[i][1].elapsed_time(evs[i + 1][0]) for i in range(n - 1))
        del blk
        return out

    def tune(dt):
        times = (C.c_double * NCANDS)()
        chosen = C.c_int()
        raise_for(lib.qob_op_tune_ex(ctx.ptr, hd.ptr, L.QOB_LEFT, dtype_code(dt), BATCH, times, NCANDS,
                                     C.byref(chosen)), ctx)
        v = chosen.value
        ms = {f"{1 << (k // 9)}x{SHAPES[k % 9]}": times[k] for k in range(36)}
        ms.update({f"T{b}:{tc}x256s{ls}": times[36 + i] for i, (b, tc, ls) in enumerate(TILE_SHAPES)})
        ms.update({f"{tc}x{blk}s{ls}p": times[36 + len(TILE_SHAPES) + i] for i, (tc, blk, ls) in enumerate(PAIR_SHAPES)})
        return {"kets_per_thread": v & 0x7F, "index_pairs": bool((v >> 7) & 1), "tile_bits": (v >> 8) & 0xFF,
                "threads_per_block": (v >> 16) & 0x3FF, "ket_sets_per_warp": 1 << ((v >> 26) & 0x7),
                "persistent": bool(v >> 30), "ms_by_shape": ms}

    def fix(dt, spec):
        """A launch shape given as <kets per thread>x<threads>[s<ket sets per warp>], P for persistent,
        T<tile bits>:<kets per thread>x256[s<ket sets per warp>] for staged tiles, or a trailing p
        for two consecutive indices per thread (<kets per thread>x<threads>[s<sets>]p)."""
        if spec.endswith("p"):
            kt, rest = spec[:-1].split("x")
            split = int(rest.split("s")[1]) if "s" in rest else 1
            block = int(rest.split("s")[0])
            raise_for(lib.qob_op_set_pairs(ctx.ptr, hd.ptr, L.QOB_LEFT, dtype_code(dt), int(kt), block, split), ctx)
            return {"kets_per_thread": int(kt), "index_pairs": True, "threads_per_block": block,
                    "ket_sets_per_warp": split, "persistent": False, "fixed": spec}
        if spec.startswith("T"):
            tb, rest = spec[1:].split(":")
            kt, rest = rest.split("x")
            split = int(rest.split("s")[1]) if "s" in rest else 1
            raise_for(lib.qob_op_set_tile(ctx.ptr, hd.ptr, L.QOB_LEFT, dtype_code(dt), int(kt), split, int(tb)), ctx)
            return {"kets_per_thread": int(kt), "tile_bits": int(tb), "threads_per_block": 256,
                    "ket_sets_per_warp": split, "persistent": False, "fixed": spec}
        kt, rest = spec.split("x")
        split = int(rest.split("s")[1]) if "s" in rest else 1
        blk = rest.split("s")[0]
        block = -int(blk[1:]) if blk.startswith("P") else int(blk)
        raise_for(lib.qob_op_set_launch(ctx.ptr, hd.ptr, L.QOB_LEFT, dtype_code(dt), int(kt), block, split), ctx)
        return {"kets_per_thread": int(kt), "threads_per_block": abs(block), "ket_sets_per_warp": split,
                "persistent": block < 0, "fixed": spec}

    prepare(H, L.QOB_LEFT, np.complex64, dev)
    prepare(H, L.QOB_LEFT, "ff", dev)
    if args.shape:
        spec = dict(kv.split("=") for kv in args.shape.split(","))
        tuning = {k: fix(dt, spec[k]) if k in spec else tune(dt)
                  for k, dt in (("c128", np.complex128), ("c64", np.complex64), ("c128x", "ff"))}
    else:
        tuning = {"c128": tune(np.complex128), "c64": tune(np.complex64), "c128x": tune("ff")}
    K, W = args.steps, max(3, args.warmup)
    raise_for(lib.qob_set_option(ctx.ptr, L.QOB_OPT_PDL, args.pdl), ctx)
    ms64, launches64, win64, _ = timed(torch.complex128, dtype_code(np.complex128), K, W)
    stats64 = step_stats(torch.complex128, dtype_code(np.complex128))
    value = whole_job_rate(BATCH * K, world, ms64 / 1e3)

    # ComplexF32 mode on the same workload, error against the oracle on one ket
    ms32, _, _, _ = timed(torch.complex64, dtype_code(np.complex64), K, W)
    value32 = whole_job_rate(BATCH * K, world, ms32 / 1e3)
    # ComplexF64 data in double-float arithmetic on the FP32 pipes (QOB_C128X)
    msff, launchesff, _, _ = timed(torch.complex128, L.QOB_C128X, K, W)
    valueff = whole_job_rate(BATCH * K, world, msff / 1e3)
    # the other launch setting, for comparison
    raise_for(lib.qob_set_option(ctx.ptr, L.QOB_OPT_PDL, 1 - args.pdl), ctx)
    pdl_other = {f"{k}_ms_per_step": timed(tdt, code, K, W)[0] / K
                 for k, tdt, code in (("c128", torch.complex128, dtype_code(np.complex128)),
                                      ("c64", torch.complex64, dtype_code(np.complex64)),
                                      ("c128x", torch.complex128, L.QOB_C128X))}
    raise_for(lib.qob_set_option(ctx.ptr, L.QOB_OPT_PDL, args.pdl), ctx)
    pdl_info = {"headline_pdl": bool(args.pdl), "other_setting": pdl_other,
                "note": "programmatic dependent launch (QOB_OPT_PDL): each step's blocks are scheduled while the "
                        "previous step finishes; other_setting = the same steps timed with the opposite setting"}
    errs = oracle_errors(lib, ctx, hd, H, dim, stream) if rank == 0 else None

    # end to end through the host-buffer C call with pinned host memory
    e2e = None
    if rank == 0 or world > 1:
        e2e = end_to_end(lib, ctx, hd, dim, K, dev, world)

    if sampler:
        sampler.stop()
    if rank != 0:
        return
    peaks_live = probe_peaks(dev)
    batched = served = None
    if not args.no_secondary:
        batched, served = secondary(dev, value)
    bytes_per_ket = (2 + (1 if BETA != 0 else 0)) * dim * 16
    bytes32 = bytes_per_ket // 2 * BATCH
    t_launch = ms64 / 1e3 / K
    achieved = bytes_per_ket * BATCH / t_launch / 1e9
    peaks = read_json(os.path.join(ROOT, "MEASURED_PEAKS.json"))
    peak, peak_src = (peaks["hbm_gbs"], "measured") if peaks and "hbm_gbs" in peaks else (6800.0, "fallback")
    prof = read_json(os.path.join(ROOT, "profiles", "gather_heisenberg14_batch64.json")) or {}
    fp64 = None
    clocks = sampler.summary(*win64) if sampler else None
    if prof.get("dfma_per_launch"):
        fp64_rate = 2.0 * prof["dfma_per_launch"] / t_launch / 1e12
        sm_mhz = (clocks or {}).get("sm_mhz") or peaks_live["fp64_probe_sm_mhz"]
        fp64_peak = fp64_pipe_tflops(peaks_live["sms"], sm_mhz)
        fp64 = {"bound": "fp64 FMA pipe", "achieved": fp64_rate, "peak": fp64_peak,
                "unit": "TFLOP/s (executed DFMA + DMUL thread instructions x 2, from the ncu capture)",
                "frac": fp64_rate / fp64_peak,
                "peak_source": (f"{FP64_LANES_PER_SM_CLOCK} FP64 lanes per SM clock x 2 flops x {peaks_live['sms']} SMs "
                                f"x the {sm_mhz:.0f} MHz SM clock sampled during the timed steps"),
                "probe": {"tflops": peaks_live["fp64_fma_tflops"],
                          "lanes_per_sm_clock": peaks_live["fp64_fma_lanes_per_sm_clock"],
                          "frac_of_probe": fp64_rate / peaks_live["fp64_fma_tflops"],
                          "note": "qob_probe_peak_ex: chains of FMAs reach 1.68 of the 2 lanes per clock; the "
                                  "dense ComplexF64 product reaches 1.96, so the pipe's 2 is the denominator"},
                "fp64_ops_per_launch": prof["dfma_per_launch"]}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms64 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128", "data": "synthetic (seeded complex-Gaussian kets, normalised)", "config": config(),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src, "traffic": prof.get("dram_bytes_per_launch"),
                     "algorithmic_bytes_per_launch": bytes_per_ket * BATCH,
                     "kernel": kernel_name("double", tuning["c128"]),
                     "ncu_kernel": prof.get("kernel"),
                     "binding": "fp64 FMA throughput (GB300 FP64 ~1.25 TFLOP/s), see fp64_compute"},
        "fp64_compute": fp64,
        "reference_arithmetic": {"flop_per_apply": reference_flops(H),
                                 "tflops": reference_flops(H) * value / 1e12,
                                 "note": "the reference's term-by-term arithmetic (8 flops per complex "
                                         "multiply-add over every term's entries) per apply x applies/s; "
                                         "the compiled kernel executes ~9x fewer FP64 operations"},
        "step_ms": dict(stats64, note="200 single applications timed one by one with CUDA events: cold = "
                                      "rotating batches (inputs from HBM), warm = one batch repeated (L2-resident); "
                                      "host_driven = issued one after another as they run (host launch latency "
                                      "included when the device waits for it), device = the same queued behind "
                                      "~5 ms of device work (device time only)"),
        "plan": plan,
        "tuning": tuning,
        "gpu_launches": launches64,
        "rel_l2_err_vs_oracle": errs["c128"],
        "fp32_mode": {"value": value32, "unit": UNIT, "ms_per_step": ms32 / K, "vs_fp64": value32 / value,
                      "rel_l2_err_vs_oracle": errs["c64"], "kernel": kernel_name("float", tuning["c64"]),
                      "roofline": {"bound": "hbm", "achieved": bytes32 / (ms32 / 1e3 / K) / 1e9, "peak": peak,
                                   "unit": "GB/s", "frac": bytes32 / (ms32 / 1e3 / K) / 1e9 / peak,
                                   "algorithmic_bytes_per_launch": bytes32}},
        "ff_mode": {"value": valueff, "unit": UNIT, "ms_per_step": msff / K, "vs_fp64": valueff / value,
                    "rel_l2_err_vs_oracle": errs["c128x"], "gpu_launches": launchesff,
                    "kernel": kernel_name("double-float", tuning["c128x"]),
                    "note": "ComplexF64 data, fused gather in double-float (FP32-pair) arithmetic, "
                            "one split launch + one gather launch per step (QOB_C128X)"},
        "oracle_check": "each form's result on one 64-ket batch of this workload (same qob_mul call, tuned "
                        "shape) against the oracle (restated reference mul!, host threads, ComplexF64 inputs)",
        "pdl": pdl_info,
        "batched": batched,
        "served": served,
        "peaks_live": peaks_live,
        "e2e": e2e,
        "clocks": clocks,
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(H, args.cpu_seconds)
    print(json.dumps(line), flush=True)


def kernel_name(scalar, t):
    """The gather kernel a tuned shape runs, as the launch list names it."""
    if t.get("tile_bits"):
        return (f"k_gather_t<{scalar}, real values, {t['kets_per_thread']} kets/thread, real beta> x 256 threads, "
                f"tiles of 2^{t['tile_bits']} indices, {t['ket_sets_per_warp']} ket sets/warp")
    if t.get("index_pairs"):
        return (f"k_gather_j2<{scalar}, real values, {t['kets_per_thread']} kets/thread, real beta> x "
                f"{t['threads_per_block']} threads, 2 indices/thread, {t['ket_sets_per_warp']} ket sets/warp")
    return "{}<{}, real values, square, {} kets/thread, real beta> x {} threads, {} ket sets/warp".format(
        "k_gather_p" if t["persistent"] else "k_gather_j", scalar, t["kets_per_thread"], t["threads_per_block"],
        t["ket_sets_per_warp"])


def probe_peaks(dev):
    """The device's FP64 and FP32 FMA rates (TFLOP/s) from the library's FMA-chain
    probe (qob_probe_peak), measured in this run."""
    import ctypes as C

    import torch
    from qobgpu import _lib as L
    from qobgpu.device import get_context, raise_for

    ctx = get_context(dev)
    out = {"sms": torch.cuda.get_device_properties(dev).multi_processor_count}
    for which, name in ((0, "fp64"), (1, "fp32")):
        r, lanes, mhz = C.c_double(), C.c_double(), C.c_double()
        raise_for(L.lib().qob_probe_peak_ex(ctx.ptr, which, C.byref(r), C.byref(lanes), C.byref(mhz)), ctx)
        out[name + "_fma_tflops"] = r.value
        out[name + "_fma_lanes_per_sm_clock"] = lanes.value
        out[name + "_probe_sm_mhz"] = mhz.value
    out["how"] = ("qob_probe_peak_ex: 16 independent FMA chains per thread, one full wave of 256-thread blocks, "
                  "one untimed launch, best of three timed (CUDA events); lanes per SM clock from each SM's "
                  "cycle counter over its blocks, and the SM clock of that launch")
    return out


def fp64_pipe_tflops(sms, sm_mhz):
    """The FP64 pipe's rate at the SM clock a kernel ran at: FMA lanes per SM
    clock x 2 flops x SMs x clock."""
    return FP64_LANES_PER_SM_CLOCK * 2 * sms * sm_mhz * 1e6 / 1e12


def oracle_errors(lib, ctx, hd, H, dim, stream):
    """Relative l2 error of each form against the oracle (the restated reference
    mul!) on one 64-ket batch of the bench's workload: the same call (qob_mul,
    column-major dim x 64, ld = dim, the tuned launch shape), the oracle run on the
    host's threads with the same ComplexF64 inputs.  Max over the kets, and over
    the whole batch."""
    import ctypes as C

    import numpy as np
    import torch

    import oracle as OR
    import qobgpu as Q
    from qobgpu import _lib as L
    from qobgpu.device import raise_for

    rng = Q.Rng(97)
    X = rng.kets_data(dim, BATCH)
    Y = rng.kets_data(dim, BATCH)
    ref = np.asfortranarray(Y.copy())
    OR.mul_kets_threaded(OR.build_node(H), ALPHA, X, BETA, ref, os.cpu_count() or 1)
    out = {}
    for name, code, tdt in (("c128", L.QOB_C128, torch.complex128), ("c64", L.QOB_C64, torch.complex64),
                            ("c128x", L.QOB_C128X, torch.complex128)):
        xd = torch.as_tensor(np.ascontiguousarray(X.T), device=stream.device).to(tdt).t()
        yd = torch.as_tensor(np.ascontiguousarray(Y.T), device=stream.device).to(tdt).t()
        raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 0, hd.ptr, code, ALPHA.real, ALPHA.imag,
                              C.c_void_p(xd.data_ptr()), dim, BATCH, dim, BETA, 0.0, C.c_void_p(yd.data_ptr()),
                              dim, BATCH, dim, C.c_void_p(stream.cuda_stream)), ctx)
        stream.synchronize()
        got = yd.cpu().numpy().astype(np.complex128)
        per = [float(np.linalg.norm(got[:, c] - ref[:, c]) / np.linalg.norm(ref[:, c])) for c in range(BATCH)]
        out[name] = {"max_over_kets": max(per),
                     "batch": float(np.linalg.norm(got - ref) / np.linalg.norm(ref))}
    return out


def secondary(dev, value64):
    """The batched and served forms of the metric, compact: 256 uneven two-mode
    cavity models in one persistent launch (CUDA-graph replay), and a served
    stream of RK4 requests (Poisson arrivals for the latencies; all requests at
    once for the sustained rate), in ComplexF64, double-float and ComplexF32.
    ``fp32_vs_plain_fp64`` divides by the headline plain ComplexF64 applies/s."""
    import torch

    import bench_suite as BS
    from qobgpu.device import get_context

    ctx = get_context(dev)
    stream = torch.cuda.Stream(dev)
    cav = BS.cavities256(ctx, stream)
    batched = {r["dtype"]: {"applies_per_s": r["applies_per_s"], "us_per_launch": r["us_per_launch"],
                            "algorithmic_GBps": r["algorithmic_GBps"], "tile": r["tile"]} for r in cav["results"]}
    batched["config"] = "256 two-mode cavities FockBasis(n1) x FockBasis(n2), n1, n2 ~ U{8..64}, dims 81-4225, one ket each"
    batched["fp32_vs_plain_fp64"] = batched["complex64"]["applies_per_s"] / value64
    batched["fp32_vs_batched_fp64"] = batched["complex64"]["applies_per_s"] / batched["complex128"]["applies_per_s"]
    lat = BS.served(ctx, stream, nreq=128, rate=2000.0)
    burst = BS.served(ctx, stream, nreq=128, rate=1e9, seed=51)
    served = {"config": "requests of 100 RK4 steps (dt 1e-3): Heisenberg chains of 8-16 spins, Jaynes-Cummings "
                        "models of dim 512-8192; 128 Poisson arrivals at 2000/s for the latencies, 128 at once for "
                        "the sustained rate",
              "fp32_rel_err_vs_fp64_max": lat["fp32_rel_err_vs_fp64_max"],
              "double_float_rel_err_vs_fp64_max": lat["double_float_rel_err_vs_fp64_max"]}
    for k, v in lat["results"].items():
        served[k] = {"p50_ms": v["p50_ms"], "p99_ms": v["p99_ms"],
                     "sustained_applies_per_s": burst["results"][k]["applies_per_s"],
                     "sustained_requests_per_s": burst["results"][k]["requests_per_s"]}
    served["fp32_vs_fp64_sustained"] = (served["complex64"]["sustained_applies_per_s"]
                                        / served["complex128"]["sustained_applies_per_s"])
    return batched, served


def end_to_end(lib, ctx, hd, dim, K, dev, world):
    """K steps through the host-buffer C calls, each step its own pair of
    page-locked host batches (x and y of 64 kets; 4 pairs in turn): x and y go
    in, y comes back, every step.  The headline form streams the steps through
    qob_mul_host_async (a step's copies in overlap the previous step's kernels
    and copy out; a pair is reused once its earlier call's ticket has been
    waited on); the synchronous qob_mul_host is timed beside it."""
    import ctypes as C

    import torch

    from qobgpu import _lib as L
    from qobgpu.device import raise_for

    R = 4
    gen = torch.Generator().manual_seed(4321)
    xh = [torch.randn(BATCH, dim, dtype=torch.complex128, generator=gen).pin_memory() for _ in range(R)]
    yh = [torch.randn(BATCH, dim, dtype=torch.complex128, generator=gen).pin_memory() for _ in range(R)]

    def args(b):
        return (ctx.ptr, L.QOB_LEFT, 0, hd.ptr, L.QOB_C128, ALPHA.real, ALPHA.imag, C.c_void_p(xh[b].data_ptr()), dim,
                BATCH, BETA, 0.0, C.c_void_p(yh[b].data_ptr()), dim, BATCH)

    argl = [args(b) for b in range(R)]

    def run_sync(steps):
        for i in range(steps):
            raise_for(lib.qob_mul_host(*argl[i % R]), ctx)

    def run_async(steps):
        tickets = [0] * R
        t = C.c_uint64()
        for i in range(steps):
            b = i % R
            raise_for(lib.qob_host_wait(ctx.ptr, tickets[b]), ctx)
            raise_for(lib.qob_mul_host_async(*argl[b], C.byref(t)), ctx)
            tickets[b] = t.value
        raise_for(lib.qob_host_wait(ctx.ptr, t.value), ctx)

    def timed(run):
        run(3)
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize(dev)
        n0 = lib.qob_kernel_launches()
        t0 = time.perf_counter()
        run(K)
        torch.cuda.synchronize(dev)
        dt = max_over_ranks(time.perf_counter() - t0, world, f"cuda:{dev}")
        return BATCH * K * world / dt, lib.qob_kernel_launches() - n0

    v_async, l_async = timed(run_async)
    v_sync, _ = timed(run_sync)
    nbytes = BATCH * dim * 16
    return {"value": v_async, "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes, "d2h_bytes_per_step": nbytes,
            "gpu_launches": l_async, "sync_value": v_sync,
            "api": "qob_mul_host_async + qob_host_wait (page-locked host batches, 4 pairs in turn; x and the "
                   "beta-scaled y copied in, y copied out every step); sync_value: qob_mul_host, one call at a time"}


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    import __graft_entry__ as g

    g.build()
    if args.suite:
        from bench_suite import run_suite

        return run_suite(local_rank, args.only, args.pdl, args.batch_tile)
    if args.probe:
        return print(json.dumps(probe_peaks(local_rank)), flush=True)
    run_own(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
