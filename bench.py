"""Benchmark of the batched Kronecker matrix-vector product on GB300.

Default workload: the plain FP64 forward at d=6, n=4 (N=4096), matrix_stride 8,
4096 output vectors x fan-in 9 = 36864 entries, seeded synthetic data
(factors U[-1,1], inputs N(0,1)).  One step = one kronmult_batched pass over the
whole batch.  Prints one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config c1|c2|c4|c5] [--dtype f64|f32] [--scaling strong|weak]

value       GFLOP/s (algorithmic 2*d*n*N flops per entry) over K device-timed steps,
            inputs resident in HBM (the 1.2 GB input set is 9x the 129 MB L2, so no
            flush is needed between steps)
e2e         the same metric through the public API with host (pinned) buffers:
            each step copies the inputs and factors in and the outputs back
            (api.forward_from_host: 16 pieces, the last 2 % of the output groups,
            copies overlapping the forward),
            host wall clock per step including the final synchronisation; beside
            it, e2e.mapped_inputs: the kernels read inputs and factors straight
            from pinned host memory (api.forward_from_host_mapped)
roofline    the forward kernel against the roof that binds it; for FP64 that is the
            FP64 FMA pipe, measured live (HBM fraction reported beside it)
cpu_baseline  the reference's own kronmult_omp (built from its sources into oracle/_ref,
            rebuilt for the host's architecture from the staged sources) on all host
            cores, same workload; the C restatement of it only where that build cannot
            be made, which the line then says
--impl reference  the same reference build timed on all host cores, on this arm's
            workload, metric and config (rank 0 alone under torchrun)
N > 1       one process per GPU; by default one seeded batch is cut into shards at
            output-group boundaries (sharding.shard_batch), so no collective is needed
            and `value` is the whole batch's flops over the slowest rank's time
            ("strong"); --scaling weak gives every rank a full-size batch of its own
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "c1": ("config1", "fwd_d3_n4_b8192"),
    "c2": ("config2", "fwd_d6_n4_b36864"),
    "c4": ("config4", "fwd_d4_n8_b32768"),
    "c5": ("config5", "fwdadj_d3_n6_b16384"),
}
METRIC = "kron-matvec GFLOP/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", choices=sorted(CONFIGS), default="c2")
    p.add_argument("--dtype", choices=["f64", "f32"], default="f64")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--suite", action="store_true",
                   help="measure every configuration, one JSON line each (diagnostic report)")
    p.add_argument("--only", default="",
                   help="with --suite: run only the items whose name starts with this prefix (c1, c2, c3, c4, c5)")
    p.add_argument("--scaling", choices=["strong", "weak"], default="strong",
                   help="N > 1: strong = one batch cut into output-group shards (default); "
                        "weak = a full-size batch per rank")
    p.add_argument("--scale", type=float, default=1.0,
                   help="shrink the number of outputs/entries (profiling runs only; not a bench value)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_batch(cfg: str, rank: int, scale: float = 1.0, world: int = 1, scaling: str = "strong"):
    """The rank's share of the workload.

    strong (default): one seeded batch, cut into `world` shards at output-group
    boundaries (sharding.shard_batch: entries sharing an output stay on one rank, so
    no data crosses ranks); every rank builds the same batch and keeps its shard.
    weak: every rank owns a full-size batch with its own seed."""
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.sharding import shard_batch

    fn, _ = CONFIGS[cfg]
    seed0 = getattr(W, fn).__defaults__[1]
    if scaling == "weak" or world == 1:
        b = getattr(W, fn)(scale=scale, seed=seed0 + (7919 * rank if scaling == "weak" else 0))
        return b, b
    full = getattr(W, fn)(scale=scale, seed=seed0)
    shard, _ = shard_batch(full, rank, world)
    return shard, full


def config_dict(cfg: str, b, world: int, scaling: str = "strong") -> dict:
    """The workload description (`b` = the whole job's batch), identical in both arms."""
    _, wname = CONFIGS[cfg]
    return {"workload": wname, "d": b.d, "n": b.n, "matrix_stride": b.stride, "nb_batch": b.nb,
            "outputs": b.n_out, "fan_in": b.nb // max(b.n_out, 1),
            "l2": "inputs (%.2f GB) larger than L2; no flush" % (b.inputs.nbytes / 1e9),
            "parallelism": f"output-group shards x{world} ({scaling} scaling)"}


def cpu_impl():
    """The CPU implementation of the reference's algorithm to time: its own kronmult_omp,
    built from its sources into oracle/_ref (rebuilt for this host's architecture from the
    staged sources when needed).  Returns (impl, note); impl is "port" (the C restatement)
    only when that build cannot be made here, and the note says why."""
    from oracle import oracle as O

    if not O.available("reference"):
        try:
            O.build(ref=True)
        except Exception as exc:  # reported in the JSON line and on stderr
            print(f"bench: building the reference kronmult_omp failed: {exc}", file=sys.stderr)
    if O.available("reference"):
        O.max_threads("reference")  # loads it: an unloadable build fails loudly here
        return "reference", "the reference's kronmult_omp built from its sources (oracle/_ref)"
    note = "reference kronmult_omp build missing on this host; timed the C restatement of it instead"
    print(f"bench: {note}", file=sys.stderr)
    return "port", note


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def host_threads() -> int:
    """Every host core this process may run on (a launcher may have set OMP_NUM_THREADS=1
    for its ranks; the CPU legs run on rank 0 alone and use them all)."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _prefix(b, count):
    from kronmult_gb300.workloads import Batch

    return Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs[:count], b.out_init,
                 b.fac_index[:count], b.out_index[:count])


def cpu_baseline(b, dtype, budget_s: float = 15.0):
    """Time the reference's CPU implementation (cpu_impl: its own kronmult_omp, OpenMP,
    all host threads) on the workload, or on a bounded prefix of its entries when the
    whole would take longer than ~budget_s."""
    from oracle import oracle as O

    impl, note = cpu_impl()
    threads = host_threads()
    probe = min(b.nb, 2048)
    t0 = time.perf_counter()
    O.forward(_prefix(b, probe), dtype=dtype, impl=impl, nthreads=threads)
    per_entry = (time.perf_counter() - t0) / probe
    count = int(min(b.nb, max(probe, budget_s / 3 / max(per_entry, 1e-12))))
    sub = _prefix(b, count)
    best = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        O.forward(sub, dtype=dtype, impl=impl, nthreads=threads)
        best = min(best, time.perf_counter() - t0)
    flops = 2.0 * b.d * b.n * b.N * count
    return {"value": flops / best / 1e9, "unit": "GFLOP/s", "cores": threads, "kind": impl,
            "sample": f"{count} of {b.nb} entries of the same batch, best of 3, {threads} OpenMP threads ({note})"}


def run_reference(args, rank, world):
    """--impl reference: the reference's own CPU implementation (kronmult_omp) on the host
    cores, on this arm's workload, metric and config; rank 0 alone."""
    if rank != 0:
        return
    _, b = make_batch(args.config, 0, args.scale, world, args.scaling)
    dt = np.float64 if args.dtype == "f64" else np.float32
    from oracle import oracle as O

    impl, note = cpu_impl()
    threads = host_threads()
    # bounded sample per step so that warmup+steps stay within a few minutes
    probe = min(b.nb, 1024)
    t0 = time.perf_counter()
    O.forward(_prefix(b, probe), dtype=dt, impl=impl, nthreads=threads)
    per_entry = (time.perf_counter() - t0) / probe
    total_steps = args.steps + args.warmup
    count = int(min(b.nb, max(64, 120.0 / total_steps / max(per_entry, 1e-12))))
    sub = _prefix(b, count)
    for _ in range(args.warmup):
        O.forward(sub, dtype=dt, impl=impl, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.forward(sub, dtype=dt, impl=impl, nthreads=threads)
    el = time.perf_counter() - t0
    flops = 2.0 * b.d * b.n * b.N * count * args.steps
    v = flops / el / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": args.scaling, "vs_baseline": None, "dtype": args.dtype,
        "data": "synthetic (seeded PCG64; factors U[-1,1], inputs N(0,1))",
        "config": config_dict(args.config, b, world, args.scaling),
        "cpu_baseline": {"value": v, "unit": "GFLOP/s", "cores": threads, "kind": impl,
                         "sample": f"{count} of {b.nb} entries per step, {threads} OpenMP threads ({note})"},
        "e2e": {"value": v, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _timed(fn, stream, reps: int, warmup: int = 3) -> float:
    """Mean milliseconds per call of fn (which enqueues on `stream`), CUDA events."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def reference_gpu_ms(db, reps: int = 3, dtype: str = "f64"):
    """Milliseconds per launch of the reference's own GPU kernel (built from the reference
    sources into oracle/_ref) on the same batch, or None where it is not available.
    The kernel overwrites its inputs, so each launch runs on a fresh copy made outside
    the event-timed window."""
    import torch

    from oracle import ref_gpu

    if not ref_gpu.available():
        return None
    x0 = db.inputs
    x = x0.clone()
    ws = torch.empty_like(x)
    out = torch.zeros_like(db.outputs)
    es = x.element_size()
    k = torch.arange(db.nb, device=x.device, dtype=torch.int64)
    in_ptrs = x.data_ptr() + k * (db.N * es)
    ws_ptrs = ws.data_ptr() + k * (db.N * es)
    out_ptrs = out.data_ptr() + db.out_index * (out.shape[1] * es)
    st = torch.cuda.current_stream()
    total = 0.0
    for rep in range(reps + 1):
        x.copy_(x0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        ref_gpu.launch(db.d, db.n, db.mat_ptrs.data_ptr(), db.stride, in_ptrs.data_ptr(), out_ptrs.data_ptr(),
                       ws_ptrs.data_ptr(), db.nb, dtype=dtype, stream=st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        if rep > 0:
            total += e0.elapsed_time(e1)
    return total / reps


def suite_large(args, emit, reps):
    """The reference's published 'large' case, on device-generated seeded data."""
    import torch

    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300.workloads import Batch

    d, n, stride, nb, distinct = 6, 8, 67, 3903, 5
    N = n ** d
    nb = max(8, int(nb * args.scale))
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(3903)
    idx = torch.arange(nb, device=dev, dtype=torch.int64)
    out_index = torch.where(idx < distinct, idx, (idx * distinct) // nb)  # tests/utils/utils_cpu.h:73-83
    for dt, name in ((torch.float64, "f64"), (torch.float32, "f32")):
        fac = (torch.rand((nb * d, n * stride), generator=g, device=dev, dtype=dt) * 2 - 1)
        x0 = torch.randn((nb, N), generator=g, device=dev, dtype=dt)
        outs = torch.zeros((distinct, N), device=dev, dtype=dt)
        db = DeviceBatch(d, n, stride, fac, x0.clone(), outs, idx, out_index, with_workspace=True)
        meta = Batch("large", d, n, stride, n * stride, np.zeros((1, 1)), np.zeros((nb, 0)), np.zeros((distinct, 0)),
                     np.zeros(1, dtype=np.int64), np.zeros(nb, dtype=np.int64))
        meta.inputs = np.empty((nb, 0))

        class _Shape:  # flops/bytes of the full shape for emit()
            def flops(self_):
                return 2.0 * d * n * N * nb

            def bytes(self_, i, o):
                return i * N * nb + i * n * n * d * nb + 2.0 * o * N * distinct

        st = torch.cuda.current_stream()
        total = 0.0
        for rep in range(reps + 1):
            db.inputs.copy_(x0)  # the global-memory path overwrites inputs, as the reference does
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            db.forward(stream=st)
            e1.record(st)
            torch.cuda.synchronize()
            if rep:
                total += e0.elapsed_time(e1)
        es = 8 if name == "f64" else 4
        emit(f"large_n8_d6_b{nb}_{name}", _Shape(), total / reps, es, es,
             {"published_v100_ms": 221 if name == "f64" else 100, "source": "tests/bench_results.txt:12,42"})
        if name == "f64":
            # FP64-accurate double-float emulation, two passes through the workspace
            from kronmult_gb300.api import forward_f64_emulated

            db.inputs.copy_(x0)
            db.outputs.zero_()
            db.forward(stream=st)
            native = db.outputs.clone()
            db.inputs.copy_(x0)
            db.outputs.zero_()
            forward_f64_emulated(db, stream=st)
            torch.cuda.synchronize()
            err = (torch.linalg.norm(db.outputs - native) / torch.linalg.norm(native)).item()
            ms = _timed(lambda: forward_f64_emulated(db, stream=st), st, max(1, reps))
            emit(f"large_n8_d6_b{nb}_f64_emulated", _Shape(), ms, 8, 8,
                 {"rel_l2_vs_native_fp64": err, "published_v100_ms": 221})
            db.inputs.copy_(x0)
            ref = reference_gpu_ms(db, reps=1)
            if ref is not None:
                emit(f"large_n8_d6_b{nb}_reference_gpu_kernel_f64", _Shape(), ref, 8, 8)
        del db, fac, x0, outs
        torch.cuda.empty_cache()


def suite(args):
    """Every configuration, one JSON line each (diagnostic report, not the headline)."""
    import ctypes

    import torch

    from kronmult_gb300 import DeviceBatch, _lib, adjoint, check_device_error, forward_f32_f64out
    from kronmult_gb300 import grouped as G
    from kronmult_gb300 import workloads as W
    from oracle import oracle as O

    lib = _lib.lib()
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(dev)
    g = ctypes.c_double(0)
    lib.kronmult_diag_fp64_fma_gflops(ctypes.byref(g))
    fp64_peak = g.value
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, ValueError, KeyError):
        hbm_peak = 6800.0
    reps = max(3, args.steps)
    sc = args.scale

    def want(prefix):
        return not args.only or prefix.startswith(args.only) or args.only.startswith(prefix)

    def emit(name, b, ms, in_size, out_size, extra=None, launches=1):
        fl = b.flops() if not isinstance(b, list) else sum(x.flops() for x in b)
        by = (b.bytes(in_size, out_size) if not isinstance(b, list)
              else sum(x.bytes(in_size, out_size) for x in b))
        line = {"suite": name, "ms": ms, "gflops": fl / ms / 1e6, "gbytes_per_s": by / ms / 1e6,
                "fp64_frac": fl / ms / 1e6 / fp64_peak, "hbm_frac": by / ms / 1e6 / hbm_peak,
                "fp64_peak_gflops": fp64_peak, "hbm_peak_gbs": hbm_peak, "launches": launches}
        line.update(extra or {})
        print(json.dumps(line), flush=True)

    # FP64 arithmetic on this GPU: FMA pipe, FP64 tensor cores (DMMA), INT8 tensor cores,
    # and the lower bound of an FP64 emulation by 8-bit integer slices (Ozaki scheme) on
    # the configuration-2 workload, against the double-float kernel measured below
    if args.only == "fp64":
        dm, i8 = ctypes.c_double(0), ctypes.c_double(0)
        _lib.check(lib.kronmult_diag_fp64_mma_gflops(ctypes.byref(dm)), "kronmult_diag_fp64_mma_gflops")
        _lib.check(lib.kronmult_diag_int8_mma_tops(ctypes.byref(i8)), "kronmult_diag_int8_mma_tops")
        b = W.config2(scale=sc)
        # two modes fused into one n^2 x n^2 contraction (K = 16): d/2 fused modes per entry
        fused_modes = b.d // 2
        elements = fused_modes * b.N * b.nb  # element-mode products, each split and recombined
        db = DeviceBatch.from_host(b, device=dev)
        from kronmult_gb300.api import forward_f64_emulated

        df_ms = _timed(lambda: forward_f64_emulated(db, stream=st), st, reps)
        native_ms = _timed(lambda: db.forward(stream=st), st, reps)
        del db
        torch.cuda.empty_cache()
        rows = []
        for slices in (6, 7, 8):
            ew = ctypes.c_double(0)
            _lib.check(lib.kronmult_diag_ozaki_elementwise_ms(elements, slices, ctypes.byref(ew)),
                       "kronmult_diag_ozaki_elementwise_ms")
            # triangular slice products (i + j < slices), each a K = n^2 int8 contraction
            int8_ops = slices * (slices + 1) / 2 * 2.0 * (b.n * b.n) * elements
            mma_ms = int8_ops / (i8.value * 1e12) * 1e3
            rows.append({"slices": slices, "bits": 8 * slices - 1, "elementwise_ms": ew.value,
                         "int8_mma_ms_at_measured_rate": mma_ms, "lower_bound_ms": ew.value + mma_ms})
        print(json.dumps({"suite": "fp64_arithmetic", "fp64_fma_gflops": fp64_peak, "fp64_mma_gflops": dm.value,
                          "int8_mma_tops": i8.value, "workload": "fwd_d6_n4_b36864",
                          "element_mode_products": elements, "native_fp64_ms": native_ms,
                          "double_float_ms": df_ms, "ozaki": rows}), flush=True)
        cnt = (ctypes.c_ulonglong * 3)()
        _lib.check(lib.kronmult_diag_fp64_mma_rounding(cnt), "kronmult_diag_fp64_mma_rounding")
        share = (ctypes.c_double * 3)()
        _lib.check(lib.kronmult_diag_fp64_pipe_share(share), "kronmult_diag_fp64_pipe_share")
        print(json.dumps({"suite": "fp64_tensor_semantics", "elements": cnt[2], "equal_ascending_fma_chain": cnt[0],
                          "equal_descending_fma_chain": cnt[1], "ms_all_dfma": share[0], "ms_all_dmma": share[1],
                          "ms_half_each": share[2], "ms_half_each_if_shared": (share[0] + share[1]) / 2,
                          "ms_half_each_if_separate": max(share[0], share[1]) / 2}), flush=True)
        # the forward on the FP64 tensor path (mma m8n8k4) against the FMA-pipe kernels,
        # same batches (bitwise the same outputs with one output per entry)
        for d, n, n_out, fan in ((2, 8, 14000, 8), (4, 8, 512, 8), (3, 7, 3000, 8), (2, 16, 2000, 8),
                                 (3, 16, 128, 8), (6, 8, 400, 1)):
            b = W.make_batch(d, n, n, max(1, int(round(n_out * sc))), fan, seed=77)
            db = DeviceBatch.from_host(b, device=dev, with_workspace=n ** d * 8 > 200000)
            row = {"suite": "fp64_tensor_path", "d": d, "n": n, "nb": b.nb}
            for name, t in (("fma_pipe", {"fp64_path": 1}), ("tensor_path", {"fp64_path": 2})):
                ms = _timed(lambda: db.forward(stream=st, tuning=t), st, reps)
                row[name] = {"ms": ms, "gflops": b.flops() / ms / 1e6}
            print(json.dumps(row), flush=True)
            del db
            torch.cuda.empty_cache()
        return

    # C1, C2: plain forward
    for cname, fn in (("c1", W.config1), ("c2", W.config2)):
        if not want(cname):
            continue
        b = fn(scale=sc)
        db = DeviceBatch.from_host(b, device=dev)
        for pf in (0, 1):
            tune = None if pf == 0 else {"prefetch": 1}
            ms = _timed(lambda: db.forward(stream=st, tuning=tune), st, reps)
            emit(f"{cname}_fwd_f64" + ("" if pf == 0 else "_single_slot"), b, ms, 8, 8)
        from kronmult_gb300.api import forward_f64_emulated

        ms = _timed(lambda: forward_f64_emulated(db, stream=st), st, reps)
        with torch.cuda.stream(st):  # checks on the launch stream: zeroing ordered before the kernels
            db.outputs.zero_()
            db.forward(stream=st)
            ref_out = db.outputs.clone()
            db.outputs.zero_()
            forward_f64_emulated(db, stream=st)
        torch.cuda.synchronize()
        err = (torch.linalg.norm(db.outputs - ref_out) / torch.linalg.norm(ref_out)).item()
        emit(f"{cname}_fwd_f64_emulated", b, ms, 8, 8, {"rel_l2_vs_native_fp64": err,
                                                         "fp64_roof_multiple": b.flops() / ms / 1e6 / fp64_peak})
        # indexed entry point: int32 maps in, pointer arrays expanded on the stream
        from kronmult_gb300.api import forward_indexed

        fidx = (db.fac_index[:, None] * b.d + torch.arange(b.d, device=dev)[None, :]).to(torch.int32)
        oidx = db.out_index.to(torch.int32)
        scratch = forward_indexed(b.d, b.n, b.stride, db.factors, fidx, db.inputs, db.outputs, oidx, stream=st)
        ms = _timed(lambda: forward_indexed(b.d, b.n, b.stride, db.factors, fidx, db.inputs, db.outputs, oidx,
                                            scratch=scratch, stream=st), st, reps)
        emit(f"{cname}_fwd_f64_indexed", b, ms, 8, 8, launches=2)
        ref = reference_gpu_ms(db, reps=3)
        if ref is not None:
            emit(f"{cname}_reference_gpu_kernel_f64", b, ref, 8, 8,
                 {"note": "kronmult_gpu/kronmult.cu built for sm_103a; inputs restored between launches, "
                          "outside the timed window"})
        if cname == "c2":
            ms = _timed(lambda: lib.kronmult_batched_f64_noalloc(b.d, b.n, db.mat_ptrs.data_ptr(), b.stride,
                                                                 db.in_ptrs.data_ptr(), db.out_ptrs.data_ptr(),
                                                                 b.nb, st.cuda_stream), st, reps)
            emit("c2_fwd_f64_noalloc", b, ms, 8, 8, launches=2)
            db32 = DeviceBatch.from_host(b, device=dev, dtype=torch.float32)
            ms = _timed(lambda: db32.forward(stream=st), st, reps)
            with torch.cuda.stream(st):
                db32.outputs.zero_()
                db32.forward(stream=st)
                db.outputs.zero_()
                db.forward(stream=st)
            torch.cuda.synchronize()
            err = (torch.linalg.norm(db32.outputs.double() - db.outputs) / torch.linalg.norm(db.outputs)).item()
            emit("c2_fwd_f32", b, ms, 4, 4, {"rel_l2_vs_fp64": err})
            del db32
        del db
        torch.cuda.empty_cache()

    # C3: grouped persistent launch, atomic and deterministic, replayed from a CUDA graph
    groups = W.config3(scale=sc) if want("c3") else []
    dbs = [DeviceBatch.from_host(x, device=dev) for x in groups]
    if groups:
        ms_sep = _timed(lambda: [d.forward(stream=st) for d in dbs], st, reps)
        emit("c3_separate_launches_f64", groups, ms_sep, 8, 8, launches=len(dbs))
    for mode in ("atomic", "deterministic") if groups else ():
        plan = G.GroupedPlan(dbs, mode=mode)
        with torch.cuda.stream(st):
            plan.run(stream=st)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=st):
            plan.run(stream=st)
        ms = _timed(lambda: graph.replay(), torch.cuda.current_stream(), reps)
        emit(f"c3_grouped_{mode}_graph_f64", groups, ms, 8, 8, {"plan": plan.info()})
        plan.close()
        # the same with per-group team sizes picked by timing the persistent kernel
        tunings = G.autotune_grouped(dbs, mode=mode, stream=st)
        plan = G.GroupedPlan(dbs, mode=mode, tunings=tunings)
        with torch.cuda.stream(st):
            plan.run(stream=st)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=st):
            plan.run(stream=st)
        ms = _timed(lambda: graph.replay(), torch.cuda.current_stream(), reps)
        emit(f"c3_grouped_{mode}_autotuned_graph_f64", groups, ms, 8, 8,
             {"plan": plan.info(), "team_sizes": [t.get("team_size", 0) for t in tunings]})
        plan.close()
        # FP64 data, mode products in double-float arithmetic on the FP32 pipe
        with torch.cuda.stream(st):
            for x in dbs:
                x.outputs.zero_()
            plan = G.GroupedPlan(dbs, mode=mode)
            plan.run(stream=st)
        torch.cuda.synchronize()
        native = [x.outputs.clone() for x in dbs]
        plan.close()
        plan = G.GroupedPlan(dbs, mode=mode, arithmetic="emulated")
        with torch.cuda.stream(st):
            for x in dbs:
                x.outputs.zero_()
            plan.run(stream=st)
        torch.cuda.synchronize()
        num = sum(float(torch.linalg.norm(x.outputs - y) ** 2) for x, y in zip(dbs, native))
        den = sum(float(torch.linalg.norm(y) ** 2) for y in native)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=st):
            plan.run(stream=st)
        ms = _timed(lambda: graph.replay(), torch.cuda.current_stream(), reps)
        emit(f"c3_grouped_{mode}_emulated_graph_f64", groups, ms, 8, 8,
             {"plan": plan.info(), "rel_l2_vs_native_fp64": (num / den) ** 0.5})
        plan.close()
    del dbs
    torch.cuda.empty_cache()

    # C4: FP32 storage, FP32 / TF32 / BF16 contraction, FP64 outputs
    modes4 = [(c, k) for c, k in (("fp32", _lib.KRONMULT_COMPUTE_FP32), ("tf32", _lib.KRONMULT_COMPUTE_TF32),
                                  ("bf16", _lib.KRONMULT_COMPUTE_BF16), ("bf16x3", _lib.KRONMULT_COMPUTE_BF16X3))
              if want(f"c4_fwd_{c}")]
    b = W.config4(scale=sc) if modes4 else None
    ref = O.forward(b) if modes4 else None
    db = DeviceBatch.from_host(b, device=dev, dtype=torch.float32, out_dtype=torch.float64) if modes4 else None
    for cname, code in modes4:
        ms = _timed(lambda: forward_f32_f64out(db, compute=code, stream=st), st, reps)
        with torch.cuda.stream(st):
            db.outputs.zero_()
            forward_f32_f64out(db, compute=code, stream=st)
        torch.cuda.synchronize()
        check_device_error()  # a tensor-core wait that ran out would leave incomplete outputs
        got = db.outputs.cpu().numpy()
        emit(f"c4_fwd_{cname}", b, ms, 4, 8, {"rel_l2_vs_fp64": O.rel_l2(got, ref), "max_err_vs_fp64": O.max_rel(got, ref)})
    del db
    torch.cuda.empty_cache()

    # the reference's own published benchmark shape ("large": n=8, d=6, N=262144, 3903
    # entries, matrix_stride 67, 5 distinct outputs reached through its aliasing pattern,
    # tests/bench_results.txt:4): vectors beyond shared memory, global-memory sweep
    if want("large"):
        suite_large(args, emit, reps)

    # C5: forward + adjoint; plain FP64 launches vs FP32 captured in one CUDA graph
    if not want("c5"):
        return
    b = W.config5(scale=sc)
    gout = np.random.Generator(np.random.PCG64(1105)).standard_normal((b.n_out, b.N))
    res = {}
    for dt, captured in ((torch.float64, False), (torch.float32, True)):
        db = DeviceBatch.from_host(b, device=dev, dtype=dt)
        gt = torch.from_numpy(gout).to(dev, dt)
        gin = torch.zeros_like(db.inputs)
        gfa = torch.zeros_like(db.factors)

        def step():
            db.forward(stream=st)
            adjoint(db, gt, gin, gfa, stream=st)

        if captured:
            with torch.cuda.stream(st):
                step()
            torch.cuda.synchronize()
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=st):
                step()
            ms = _timed(lambda: graph.replay(), torch.cuda.current_stream(), reps)
        else:
            ms = _timed(step, st, reps)
        with torch.cuda.stream(st):
            db.outputs.zero_()
            gin.zero_()
            gfa.zero_()
            step()
        torch.cuda.synchronize()
        res[dt] = (ms, db.outputs.double().cpu().numpy(), gin.double().cpu().numpy(), gfa.double().cpu().numpy())
    (m64, y64, gi64, ga64), (m32, y32, gi32, ga32) = res[torch.float64], res[torch.float32]

    class _FwdAdj:  # forward + grad_input + grad_A contractions: 3 x 2dnN per entry
        def flops(self_):
            return 3.0 * b.flops()

        def bytes(self_, i, o):
            # x and g read, grad_input written, factors read and grad_A written, outputs once
            return b.bytes(i, o) + i * b.N * b.nb * 2 + 2.0 * i * b.n * b.n * b.d * b.n_sets

    # the grouped form: one plan holding the forward group and the adjoint group, FP32,
    # replayed from one CUDA graph (forward and adjoint run as parallel branches)
    db = DeviceBatch.from_host(b, device=dev, dtype=torch.float32)
    gt = torch.from_numpy(gout).to(dev, torch.float32)
    gin = torch.zeros_like(db.inputs)
    gfa = torch.zeros_like(db.factors)
    plan = G.GroupedPlan([db], mode="atomic", adjoints=[(db, gt, gin, gfa)])
    with torch.cuda.stream(st):
        plan.run(stream=st)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=st):
        plan.run(stream=st)
    m32g = _timed(lambda: graph.replay(), torch.cuda.current_stream(), reps)
    for t in (db.outputs, gin, gfa):
        t.zero_()
    graph.replay()
    torch.cuda.synchronize()
    y32g, gi32g, ga32g = (t.double().cpu().numpy() for t in (db.outputs, gin, gfa))
    plan.close()

    fm = {"flops_model": "3 x 2dnN per entry (forward, grad_input, grad_A contractions; "
                         "the partial products grad_A needs are not counted)"}
    emit("c5_fwd_adj_f64_plain", _FwdAdj(), m64, 8, 8, fm, launches=2)
    emit("c5_fwd_adj_f32_graph", _FwdAdj(), m32, 4, 4, {**fm,
        "speedup_vs_plain_fp64": m64 / m32,
        "rel_l2_vs_fp64": {"output": O.rel_l2(y32, y64), "grad_input": O.rel_l2(gi32, gi64),
                           "grad_factors": O.rel_l2(ga32, ga64)}}, launches=2)
    emit("c5_fwd_adj_f32_grouped_graph", _FwdAdj(), m32g, 4, 4, {**fm,
        "speedup_vs_plain_fp64": m64 / m32g,
        "form": "one grouped plan (forward group + adjoint group as parallel branches), one graph replay",
        "rel_l2_vs_fp64": {"output": O.rel_l2(y32g, y64), "grad_input": O.rel_l2(gi32g, gi64),
                           "grad_factors": O.rel_l2(ga32g, ga64)}}, launches=2)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.suite:
        suite(args)
        return
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    from kronmult_gb300 import DeviceBatch, _lib

    lib = _lib.lib()
    b, full = make_batch(args.config, rank, args.scale, world, args.scaling)
    tdt = torch.float64 if args.dtype == "f64" else torch.float32
    esize = 8 if args.dtype == "f64" else 4
    db = DeviceBatch.from_host(b, device=dev, dtype=tdt)
    stream = torch.cuda.Stream(dev)
    flops_step = b.flops()  # this rank's shard
    bytes_step = b.bytes(in_size=esize, out_size=esize)
    # the whole job per step: every rank's shard (strong), or world full batches (weak)
    job_flops = full.flops() * (world if args.scaling == "weak" else 1)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            db.forward(stream=stream)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)  # let nvidia-smi start sampling before the timed region
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        db.forward(stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = t.item()
    per_launch_s = ms / 1e3 / args.steps
    value = job_flops / per_launch_s / 1e9

    # ---- end to end through the public API with pinned host buffers
    h_in = torch.from_numpy(b.inputs).to(tdt).pin_memory()
    h_fac = torch.from_numpy(b.factors).to(tdt).pin_memory()
    h_out = torch.empty(db.outputs.shape, dtype=tdt).pin_memory()
    h2d = h_in.numel() * esize + h_fac.numel() * esize
    d2h = h_out.numel() * esize

    from kronmult_gb300.api import forward_from_host, forward_from_host_mapped

    pipe_streams = (torch.cuda.Stream(dev), torch.cuda.Stream(dev), torch.cuda.Stream(dev))

    def e2e_step():
        # copies in, forward, copy out: pipelined in 16 pieces over three streams, the last
        # piece 2 % of the output groups (12 equal pieces: 7.17 ms; this: 6.97 ms)
        forward_from_host(db, h_in, h_fac, h_out, chunks=16, streams=pipe_streams, last_share=0.02)

    def e2e_mapped_step():
        # kernels read inputs and factors from pinned host memory; outputs copied back in 2 pieces (9:1)
        forward_from_host_mapped(db, h_in, h_fac, h_out, chunks=2, streams=pipe_streams)

    def time_host_steps(step):
        step()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            step()
            torch.cuda.synchronize()  # the host result is complete at the end of every step
        ms = (time.perf_counter() - t0) * 1e3 / args.e2e_steps
        if world > 1:
            t = torch.tensor([ms], device=dev, dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = t.item()
        return ms

    e2e_ms = time_host_steps(e2e_step)
    e2e_value = job_flops / (e2e_ms / 1e3) / 1e9
    e2e_mapped_ms = None
    if tdt == torch.float64 and h_in.shape == db.inputs.shape and h_fac.shape == db.factors.shape:
        e2e_mapped_ms = time_host_steps(e2e_mapped_step)

    # ---- live roofline denominators
    fp64_peak = None
    if args.dtype == "f64":
        import ctypes

        g = ctypes.c_double(0)
        if lib.kronmult_diag_fp64_fma_gflops(ctypes.byref(g)) == 0:
            fp64_peak = g.value
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    hbm_src = "of measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks else "of fallback"
    achieved_gbs = bytes_step / per_launch_s / 1e9
    achieved_gflops = flops_step / per_launch_s / 1e9
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        traffic = tr.get(f"{args.config}_{args.dtype}")
    except (OSError, ValueError):
        pass
    if args.dtype == "f64" and fp64_peak:
        roofline = {"bound": "fp64", "achieved": achieved_gflops, "peak": fp64_peak, "unit": "GFLOP/s",
                    "frac": achieved_gflops / fp64_peak, "traffic": traffic,
                    "peak_source": "of measured (FP64 FMA probe kernel run by this benchmark)",
                    "hbm": {"achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                            "frac": achieved_gbs / hbm_peak, "peak_source": hbm_src}}
    else:
        roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved_gbs / hbm_peak, "traffic": traffic, "peak_source": hbm_src}

    ref_gpu_line = None
    if args.dtype == "f64":
        try:
            ref_ms = reference_gpu_ms(db, reps=3)
        except Exception as exc:  # the comparator is optional; report why it is missing
            ref_ms, ref_gpu_line = None, {"unavailable": str(exc)[:200]}
        if ref_ms:
            ref_gpu_line = {"value": flops_step / (ref_ms / 1e3) / 1e9, "unit": "GFLOP/s", "ms_per_launch": ref_ms,
                            "speedup_of_ours": ref_ms / (per_launch_s * 1e3),
                            "kernel": "kronmult_gpu/kronmult.cu cuda_kronmult_batchelement<double>, built for "
                                      "sm_103a from the reference sources, same workload and GPU"}
        elif ref_gpu_line is None:
            ref_gpu_line = {"unavailable": "reference cubin not built (needs the reference sources)"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(b, np.float64 if args.dtype == "f64" else np.float32)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": args.scaling, "vs_baseline": None, "dtype": args.dtype,
            "data": "synthetic (seeded PCG64; factors U[-1,1], inputs N(0,1))",
            "config": config_dict(args.config, full, world, args.scaling),
            "gbytes_per_s": achieved_gbs,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "reference_gpu_kernel": ref_gpu_line,
            "e2e": {"value": e2e_value, "unit": "GFLOP/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
                    "path": "api.forward_from_host: staging copies from pinned host memory, 16 pieces "
                            "(the last 2 % of the output groups)",
                    "mapped_inputs": None if e2e_mapped_ms is None else {
                        "ms_per_step": e2e_mapped_ms, "value": job_flops / (e2e_mapped_ms / 1e3) / 1e9,
                        "path": "api.forward_from_host_mapped: kernels read inputs and factors from pinned "
                                "host memory over the CPU-GPU link, outputs copied back"}},
            "gpu_launches": args.steps,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
