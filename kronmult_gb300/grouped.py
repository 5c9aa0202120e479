"""Grouped persistent forward (and adjoint) and the autotuner, over the C ABI.

`GroupedPlan([batch, ...], mode)` builds one plan for several DeviceBatch groups
of different (d, n, fan-in); `plan.run(stream)` enqueues, per group, a persistent
kernel compiled for its n that pulls work from the group's device queue -- in
parallel graph branches forked from `stream` in the atomic mode, one after another
in the deterministic mode (graph-capturable either way).  mode "atomic" adds with
atomics; "deterministic" orders the entries by output pointer on the device at
plan creation and sums every output's entries in entry order with a segmented
reduction (units of consecutive sorted entries, then the pieces of outputs that
span units in order), so the result is bitwise reproducible for a given plan.  `adjoints=[(batch, grad_out,
grad_in, grad_factors), ...]` adds adjoint groups (api.adjoint's arguments) to the
same run, as further parallel branches: one replay then runs a forward and its
backward.

`autotune_forward(d, n, dtype)` times the forward's launch shapes on the GPU and
stores the fastest in the library's tuning cache, which the planners consult.
`autotune_grouped(batches, mode)` picks a team size per group for the persistent
kernel itself and returns the tunings to pass to GroupedPlan.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .api import DeviceBatch, _stream_handle

MODES = {"atomic": _lib.KRONMULT_MODE_ATOMIC, "deterministic": _lib.KRONMULT_MODE_DETERMINISTIC}
DTYPES = {torch.float64: _lib.KRONMULT_DTYPE_F64, torch.float32: _lib.KRONMULT_DTYPE_F32}


class GroupedPlan:
    def __init__(self, batches: list[DeviceBatch], mode: str = "atomic", tunings: list[dict] | None = None,
                 adjoints: list | None = None, arithmetic: str = "native"):
        """arithmetic "emulated" (float64 groups, n <= 8): the forward groups' mode products
        in double-float arithmetic on the FP32 pipe (KRONMULT_DTYPE_F64_EMULATED; relative
        error ~1e-14 instead of the native FMA chains' bits); adjoint groups stay native."""
        adjoints = list(adjoints or [])
        if arithmetic not in ("native", "emulated"):
            raise ValueError("arithmetic must be 'native' or 'emulated'")
        if not batches and not adjoints:
            raise ValueError("at least one group is needed")
        dt = (batches[0] if batches else adjoints[0][0]).inputs.dtype
        for b in list(batches) + [a[0] for a in adjoints]:
            if b.inputs.dtype != dt or b.factors.dtype != dt:
                raise TypeError("all groups must share one dtype (float64 or float32)")
        for b in batches:
            if b.outputs.dtype != dt:
                raise TypeError("all groups must share one dtype (float64 or float32)")
        if dt not in DTYPES:
            raise TypeError("grouped forward is defined for float64 and float32")
        code = DTYPES[dt]
        if arithmetic == "emulated":
            if dt != torch.float64:
                raise TypeError("emulated arithmetic is defined for float64 groups")
            code = _lib.KRONMULT_DTYPE_F64_EMULATED
        self.batches = list(batches)  # keeps the pointer tables alive
        self.mode = mode
        groups = (_lib.Group * max(1, len(batches)))()
        for g, b in zip(groups, batches):
            g.matrix_count, g.matrix_size, g.matrix_stride, g.nb_batch = b.d, b.n, b.stride, b.nb
            g.matrix_list_batched = b.mat_ptrs.data_ptr()
            g.input_batched = b.in_ptrs.data_ptr()
            g.output_batched = b.out_ptrs.data_ptr()
        adj = (_lib.AdjointGroup * max(1, len(adjoints)))()
        self._adj_tables = []
        for a, (b, gout, gin, gfac) in zip(adj, adjoints):
            tables = _adjoint_tables(b, gout, gin, gfac)
            self._adj_tables.append((b, gout, gin, gfac) + tables)
            a.matrix_count, a.matrix_size, a.matrix_stride, a.nb_batch = b.d, b.n, b.stride, b.nb
            a.matrix_list_batched = b.mat_ptrs.data_ptr()
            a.input_batched = b.in_ptrs.data_ptr()
            a.grad_output_batched = tables[0].data_ptr()
            a.grad_input_batched = None if tables[1] is None else tables[1].data_ptr()
            a.grad_matrix_list_batched = None if tables[2] is None else tables[2].data_ptr()
            a.grad_matrix_stride = b.stride
        tp = None
        if tunings is not None:
            arr = (_lib.Tuning * len(batches))()
            for a, t in zip(arr, tunings):
                t = t or {}
                a.team_size = int(t.get("team_size", 0))
                a.ctas_per_sm = int(t.get("ctas_per_sm", 0))
                a.entries_per_team = int(t.get("entries_per_team", 0))
                a.prefetch = int(t.get("prefetch", 0))
                a.fp64_path = int(t.get("fp64_path", 0))
            tp = arr
        self._h = ctypes.c_void_p()
        st = _lib.lib().kronmult_grouped_plan_create_with_adjoint(ctypes.byref(self._h), groups, len(batches), adj,
                                                                 len(adjoints), code, MODES[mode], tp)
        _lib.check(st, "kronmult_grouped_plan_create")

    def regroup(self, stream=None) -> None:
        """Re-run the deterministic mode's device-side ordering (after an output pointer
        table changed in place); graph-capturable."""
        _lib.check(_lib.lib().kronmult_grouped_regroup(self._h, _stream_handle(stream)), "kronmult_grouped_regroup")

    def run(self, stream=None) -> None:
        _lib.check(_lib.lib().kronmult_grouped_run(self._h, _stream_handle(stream)), "kronmult_grouped_run")

    def info(self) -> dict:
        """grid (largest), block, smem (largest), items (work units of all groups), kernels
        (per run), sorted (entries ordered on the device, deterministic mode)."""
        v = (ctypes.c_longlong * 6)()
        _lib.check(_lib.lib().kronmult_grouped_plan_info(self._h, v, 6), "kronmult_grouped_plan_info")
        return dict(zip(("grid", "block", "smem", "items", "kernels", "sorted"), list(v)))

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _lib.lib().kronmult_grouped_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _adjoint_tables(b: DeviceBatch, grad_out: torch.Tensor, grad_in, grad_fac):
    """Device pointer tables of an adjoint group (as api.adjoint builds them)."""
    dev = b.inputs.device
    es = b.inputs.element_size()
    N = b.N
    if grad_out.dtype != b.inputs.dtype or grad_out.shape[1] != N or not grad_out.is_contiguous():
        raise ValueError("grad_out must be a contiguous (n_out, N) tensor of the batch dtype")
    gout = grad_out.data_ptr() + b.out_index * (N * es)
    gin = None
    if grad_in is not None:
        if grad_in.shape != b.inputs.shape or grad_in.dtype != b.inputs.dtype or not grad_in.is_contiguous():
            raise ValueError("grad_in must match the inputs' shape and dtype")
        k = torch.arange(b.nb, device=dev, dtype=torch.int64)
        gin = grad_in.data_ptr() + k * (N * es)
    gmat = None
    if grad_fac is not None:
        if grad_fac.shape != b.factors.shape or grad_fac.dtype != b.factors.dtype or not grad_fac.is_contiguous():
            raise ValueError("grad_factors must match the factors' shape and dtype")
        i = torch.arange(b.d, device=dev, dtype=torch.int64)
        gmat = (grad_fac.data_ptr() + (b.fac_index[:, None] * b.d + i[None, :]) * (b.factors.shape[1] * es)).reshape(-1)
    return gout, gin, gmat


def autotune_forward(d: int, n: int, dtype: int = _lib.KRONMULT_DTYPE_F64, nb_sample: int = 0):
    """Time the forward's launch shapes for (d, n, dtype); return (tuning dict, best ms)."""
    t = _lib.Tuning()
    ms = ctypes.c_float(0)
    _lib.check(_lib.lib().kronmult_autotune_forward(d, n, dtype, nb_sample, ctypes.byref(t), ctypes.byref(ms)),
               "kronmult_autotune_forward")
    return _as_dict(t), ms.value


def autotune_grouped(batches: list[DeviceBatch], mode: str = "atomic",
                     team_sizes=(0, 8, 16, 32, 64, 128, 256), reps: int = 5, stream=None) -> list[dict]:
    """Per-group tunings for GroupedPlan: for every group, a one-group plan of the
    persistent kernel is timed (CUDA events, `reps` launches after one warm-up) with
    each candidate team size (0 = the planner's own choice), and the fastest is kept.
    The groups' outputs are restored afterwards.  Returns one tuning dict per group."""
    st = stream or torch.cuda.current_stream()
    tunings = []
    for b in batches:
        saved = b.outputs.clone()
        best, best_ms, seen = {}, float("inf"), set()
        # FP64: both FMA-pipe mappings (whole fibres, one element per thread) for each size
        maps = (0, 3, 4) if b.inputs.dtype == torch.float64 and b.n <= 8 else (0,)
        for ts, fmap in ((t, m) for t in team_sizes for m in maps):
            t = {"team_size": int(ts)} if ts else {}
            if fmap:
                t["fp64_path"] = fmap
            try:
                plan = GroupedPlan([b], mode=mode, tunings=[t])
            except _lib.KronmultError:
                continue
            info = plan.info()
            shape = (info["block"], info["smem"], info["items"], info["grid"])
            if shape in seen:  # a forced size the planner grew into an already timed shape
                plan.close()
                continue
            seen.add(shape)
            plan.run(stream=st)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(reps):
                plan.run(stream=st)
            e1.record(st)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / reps
            plan.close()
            if ms < best_ms:
                best, best_ms = t, ms
        b.outputs.copy_(saved)
        tunings.append(best)
    torch.cuda.synchronize()
    return tunings


def tuning_cache_get(d: int, n: int, dtype: int = _lib.KRONMULT_DTYPE_F64):
    t = _lib.Tuning()
    if _lib.lib().kronmult_tuning_cache_get(d, n, dtype, ctypes.byref(t)) != 0:
        return None
    return _as_dict(t)


def _as_dict(t) -> dict:
    return {"team_size": t.team_size, "ctas_per_sm": t.ctas_per_sm, "entries_per_team": t.entries_per_team,
            "prefetch": t.prefetch, "fp64_path": t.fp64_path}


def tuning_cache_set(d: int, n: int, dtype: int, tuning: dict) -> None:
    t = _lib.Tuning(int(tuning.get("team_size", 0)), int(tuning.get("ctas_per_sm", 0)),
                    int(tuning.get("entries_per_team", 0)), int(tuning.get("prefetch", 0)),
                    int(tuning.get("fp64_path", 0)))
    _lib.check(_lib.lib().kronmult_tuning_cache_set(d, n, dtype, ctypes.byref(t)), "kronmult_tuning_cache_set")


def tuning_cache_clear() -> None:
    _lib.lib().kronmult_tuning_cache_clear()


def tuning_cache_save(path: str) -> None:
    _lib.check(_lib.lib().kronmult_tuning_cache_save(path.encode()), "kronmult_tuning_cache_save")


def tuning_cache_load(path: str) -> None:
    _lib.check(_lib.lib().kronmult_tuning_cache_load(path.encode()), "kronmult_tuning_cache_load")
