"""Python host mirror of the reference's `kronmult_batched` interface.

`kronmult_batched(...)` has the reference's argument list and meaning
(kronmult_gpu/kronmult.cuh:28-32): device-resident pointer arrays for the
factors, inputs, outputs and workspaces, and it adds kron(A_k) . x_k into
output k for every entry.  It is synchronous and raises `KronmultError` where the
reference would return a failing cudaError.  Pointer arrays may be given as
int64 CUDA tensors of device addresses or as raw device addresses (ints).

`DeviceBatch` owns a structured batch in device memory (dense factor, input and
output tensors plus index maps) and builds the pointer arrays from it; it is
how the tests, the benchmark and the autograd wrapper drive the C ABI.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .workloads import Batch

_FN = {torch.float64: "kronmult_batched_f64", torch.float32: "kronmult_batched_f32"}


def _addr(x) -> int | None:
    if x is None:
        return None
    if isinstance(x, torch.Tensor):
        if x.numel() > 0 and not x.is_cuda:
            raise ValueError("pointer arrays must be device-resident (CUDA tensors)")
        return x.data_ptr()
    return int(x)


def _stream_handle(stream) -> int | None:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    return int(stream)


def kronmult_batched(matrix_count: int, matrix_size: int, matrix_list_batched, matrix_stride: int,
                     input_batched, output_batched, workspace_batched, nb_batch: int,
                     dtype: torch.dtype = torch.float64) -> None:
    """Mirror of kronmult_batched<T>: synchronous, reference semantics (see module doc)."""
    if dtype not in _FN:
        raise TypeError("kronmult_batched is defined for float64 and float32 only")
    fn = getattr(_lib.lib(), _FN[dtype])
    st = fn(int(matrix_count), int(matrix_size), _addr(matrix_list_batched), int(matrix_stride),
            _addr(input_batched), _addr(output_batched), _addr(workspace_batched), int(nb_batch))
    _lib.check(st, _FN[dtype])


def kronmult_batched_async(matrix_count: int, matrix_size: int, matrix_list_batched, matrix_stride: int,
                           input_batched, output_batched, workspace_batched, nb_batch: int,
                           dtype: torch.dtype = torch.float64, stream=None, tuning=None) -> None:
    """Enqueue the forward on `stream` (default: torch's current stream); no synchronisation."""
    if dtype not in _FN:
        raise TypeError("kronmult_batched is defined for float64 and float32 only")
    name = _FN[dtype] + "_async"
    fn = getattr(_lib.lib(), name)
    st = fn(int(matrix_count), int(matrix_size), _addr(matrix_list_batched), int(matrix_stride),
            _addr(input_batched), _addr(output_batched), _addr(workspace_batched), int(nb_batch),
            _stream_handle(stream), _lib.tuning_ptr(tuning))
    _lib.check(st, name)


class DeviceBatch:
    """A batch in device memory with the pointer arrays the C ABI consumes.

    factors   (S*d, block)   row s*d+i holds factor i of set s (col-major, ld = stride)
    inputs    (B, N)
    outputs   (E, N)         accumulated into
    fac_index, out_index     (B,) int64 maps entry -> factor set / output vector
    """

    def __init__(self, d: int, n: int, stride: int, factors: torch.Tensor, inputs: torch.Tensor,
                 outputs: torch.Tensor, fac_index: torch.Tensor, out_index: torch.Tensor,
                 with_workspace: bool = False):
        self.d, self.n, self.stride = int(d), int(n), int(stride)
        self.factors, self.inputs, self.outputs = factors, inputs, outputs
        self.fac_index = fac_index.to(device=inputs.device, dtype=torch.int64)
        self.out_index = out_index.to(device=inputs.device, dtype=torch.int64)
        self.workspace = torch.empty_like(inputs) if with_workspace else None
        self.build_pointers()

    @classmethod
    def from_host(cls, b: Batch, device="cuda", dtype=torch.float64, out_dtype=None,
                  with_workspace: bool = False) -> "DeviceBatch":
        out_dtype = out_dtype or dtype
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(device=device, dtype=dt)
        return cls(b.d, b.n, b.stride, t(b.factors, dtype), t(b.inputs, dtype), t(b.out_init, out_dtype),
                   torch.from_numpy(b.fac_index), torch.from_numpy(b.out_index), with_workspace)

    @property
    def nb(self) -> int:
        return int(self.inputs.shape[0])

    @property
    def N(self) -> int:
        return self.n ** self.d

    def build_pointers(self) -> None:
        """(Re)build the device pointer arrays from the current tensors."""
        dev = self.inputs.device
        fes = self.factors.element_size()
        ies = self.inputs.element_size()
        oes = self.outputs.element_size()
        blk = self.factors.shape[1] if self.factors.dim() == 2 else 0
        B, d = self.nb, self.d
        i = torch.arange(d, device=dev, dtype=torch.int64)
        self.mat_ptrs = (self.factors.data_ptr()
                         + ((self.fac_index[:, None] * d + i[None, :]) * (blk * fes))).reshape(-1).contiguous()
        k = torch.arange(B, device=dev, dtype=torch.int64)
        self.in_ptrs = (self.inputs.data_ptr() + k * (self.inputs.shape[1] * ies)).contiguous()
        self.out_ptrs = (self.outputs.data_ptr() + self.out_index * (self.outputs.shape[1] * oes)).contiguous()
        self.ws_ptrs = None
        if self.workspace is not None:
            self.ws_ptrs = (self.workspace.data_ptr() + k * (self.workspace.shape[1] * ies)).contiguous()

    def forward(self, stream=None, tuning=None, sync: bool = False) -> None:
        """outputs[out_index[k]] += kron(factors of set fac_index[k]) . inputs[k] for all k."""
        dt = self.inputs.dtype
        if self.outputs.dtype == dt:
            if sync:
                kronmult_batched(self.d, self.n, self.mat_ptrs, self.stride, self.in_ptrs, self.out_ptrs,
                                 self.ws_ptrs, self.nb, dtype=dt)
            else:
                kronmult_batched_async(self.d, self.n, self.mat_ptrs, self.stride, self.in_ptrs, self.out_ptrs,
                                       self.ws_ptrs, self.nb, dtype=dt, stream=stream, tuning=tuning)
        elif dt == torch.float32 and self.outputs.dtype == torch.float64:
            forward_f32_f64out(self, compute=_lib.KRONMULT_COMPUTE_FP32, stream=stream, tuning=tuning, sync=sync)
        else:
            raise TypeError(f"unsupported storage/output dtypes {dt}/{self.outputs.dtype}")


def adjoint(b: DeviceBatch, grad_outputs: torch.Tensor, grad_inputs: torch.Tensor | None = None,
            grad_factors: torch.Tensor | None = None, stream=None, tuning=None) -> None:
    """Adjoint of DeviceBatch.forward on the same batch:
        grad_inputs[k]                  += kron(A_k)^T . grad_outputs[out_index[k]]
        grad_factors[fac_index[k]*d + i] += dL/dA_{k,i}   (summed over entries sharing the set)
    `grad_factors` has the factors' shape (same leading dimension).  Either may be None."""
    dt = b.inputs.dtype
    name = {torch.float64: "kronmult_batched_adjoint_f64_async",
            torch.float32: "kronmult_batched_adjoint_f32_async"}.get(dt)
    if name is None or b.factors.dtype != dt:
        raise TypeError("adjoint is defined for float64 and float32 batches")
    dev = b.inputs.device
    es = b.inputs.element_size()
    N = b.N
    gout = grad_outputs.contiguous()
    if gout.dtype != dt or gout.shape[1] != N:
        raise ValueError("grad_outputs must be (n_out, N) of the batch dtype")
    key = (gout.data_ptr(), None if grad_inputs is None else grad_inputs.data_ptr(),
           None if grad_factors is None else grad_factors.data_ptr())
    cached = getattr(b, "_adj_tables", None)
    if cached is not None and cached[0] == key:
        _, gout_ptrs, gin_ptrs, gmat_ptrs = cached
        fn = getattr(_lib.lib(), name)
        st = fn(b.d, b.n, b.mat_ptrs.data_ptr(), b.stride, b.in_ptrs.data_ptr(), gout_ptrs.data_ptr(),
                None if gin_ptrs is None else gin_ptrs.data_ptr(),
                None if gmat_ptrs is None else gmat_ptrs.data_ptr(), b.stride, b.nb, _stream_handle(stream),
                _lib.tuning_ptr(tuning))
        _lib.check(st, name)
        return
    gout_ptrs = gout.data_ptr() + b.out_index * (N * es)
    gin_ptrs = None
    if grad_inputs is not None:
        if grad_inputs.shape != b.inputs.shape or grad_inputs.dtype != dt or not grad_inputs.is_contiguous():
            raise ValueError("grad_inputs must match the inputs' shape and dtype")
        k = torch.arange(b.nb, device=dev, dtype=torch.int64)
        gin_ptrs = grad_inputs.data_ptr() + k * (N * es)
    gmat_ptrs = None
    if grad_factors is not None:
        if grad_factors.shape != b.factors.shape or grad_factors.dtype != dt or not grad_factors.is_contiguous():
            raise ValueError("grad_factors must match the factors' shape and dtype")
        i = torch.arange(b.d, device=dev, dtype=torch.int64)
        blk = b.factors.shape[1]
        gmat_ptrs = (grad_factors.data_ptr() + (b.fac_index[:, None] * b.d + i[None, :]) * (blk * es)).reshape(-1)
    fn = getattr(_lib.lib(), name)
    st = fn(b.d, b.n, b.mat_ptrs.data_ptr(), b.stride, b.in_ptrs.data_ptr(), gout_ptrs.data_ptr(),
            None if gin_ptrs is None else gin_ptrs.data_ptr(), None if gmat_ptrs is None else gmat_ptrs.data_ptr(),
            b.stride, b.nb, _stream_handle(stream), _lib.tuning_ptr(tuning))
    _lib.check(st, name)
    # keep the pointer tables referenced by the batch (reused while the same gradient
    # tensors are passed) so that their memory stays valid for the enqueued kernel
    b._adj_tables = (key, gout_ptrs, gin_ptrs, gmat_ptrs)
    b._adj_keep = gout


def check_device_error(clear: bool = True) -> None:
    """Raise KronmultError when a tensor-core kernel recorded a device-side failure (a
    bounded mbarrier wait that ran out: the kernel left early and its outputs are
    incomplete).  Reads the library's device error word (kronmult_device_error), which
    waits for the work already enqueued; with `clear` the word is reset."""
    code = ctypes.c_int(0)
    _lib.check(_lib.lib().kronmult_device_error(ctypes.byref(code), int(clear)), "kronmult_device_error")
    if code.value:
        raise _lib.KronmultError(code.value, "a tensor-core kernel",
                                 "device error word set: a bounded mbarrier wait timed out and the kernel "
                                 "left early, so its outputs are incomplete")


def forward_f32_f64out(b: DeviceBatch, compute: int = _lib.KRONMULT_COMPUTE_FP32, stream=None,
                       tuning=None, sync: bool = False) -> None:
    """FP32 factors/inputs, FP32 (or TF32/BF16 tensor-core) contraction, FP64 output accumulation.
    Enqueues only, unless `sync`: then it waits for the stream and, for the tensor-core
    modes, raises if the kernel recorded a device-side failure (check_device_error)."""
    fn = _lib.lib().kronmult_batched_f32_f64out_async
    st = fn(b.d, b.n, b.mat_ptrs.data_ptr(), b.stride, b.in_ptrs.data_ptr(), b.out_ptrs.data_ptr(),
            None if b.ws_ptrs is None else b.ws_ptrs.data_ptr(), b.nb, int(compute), _stream_handle(stream),
            _lib.tuning_ptr(tuning))
    _lib.check(st, "kronmult_batched_f32_f64out_async")
    if sync:
        torch.cuda.synchronize()
        if compute != _lib.KRONMULT_COMPUTE_FP32:
            check_device_error()


def forward_from_host(b: DeviceBatch, h_inputs: torch.Tensor, h_factors: torch.Tensor, h_outputs: torch.Tensor,
                      chunks: int = 8, streams=None, last_share: float | None = None) -> None:
    """End-to-end forward for a batch whose data lives in (pinned) host memory.

    Copies factors and inputs into the batch's device tensors, runs the forward and
    copies the outputs back into `h_outputs`, pipelined in `chunks` pieces cut at
    output-group boundaries: the host-to-device copy of piece i+1 and the
    device-to-host copy of piece i-1 overlap the forward of piece i.  When the
    factor sets or the outputs are not used in increasing order, the factors are
    copied before and the outputs after the whole batch instead.  With `last_share`
    the last piece holds that share of the output groups and the others split the
    rest evenly: the forward and the copy back of the last piece are the part of the
    step that nothing overlaps.  Enqueues only; synchronise with
    torch.cuda.synchronize()."""
    dev = b.inputs.device
    s_in, s_cmp, s_out = streams or (torch.cuda.Stream(dev), torch.cuda.Stream(dev), torch.cuda.Stream(dev))
    plan = _host_pipeline_plan(b, chunks, last_share)
    cuts, fac_rows, out_rows, monotone, out_monotone = plan
    nchunks = len(cuts) - 1
    d = b.d
    if not monotone:
        with torch.cuda.stream(s_in):
            b.factors.copy_(h_factors, non_blocking=True)
    ev_in = [torch.cuda.Event() for _ in range(nchunks)]
    ev_cmp = [torch.cuda.Event() for _ in range(nchunks)]
    es_p = b.mat_ptrs.element_size()
    fn = getattr(_lib.lib(), _FN[b.inputs.dtype] + "_async")
    for c in range(nchunks):
        lo, hi = cuts[c], cuts[c + 1]
        if hi <= lo:
            continue
        with torch.cuda.stream(s_in):
            b.inputs[lo:hi].copy_(h_inputs[lo:hi], non_blocking=True)
            if monotone:
                f0, f1 = fac_rows[c]
                b.factors[f0:f1].copy_(h_factors[f0:f1], non_blocking=True)
            ev_in[c].record(s_in)
        s_cmp.wait_event(ev_in[c])
        st = fn(b.d, b.n, b.mat_ptrs.data_ptr() + lo * d * es_p, b.stride, b.in_ptrs.data_ptr() + lo * es_p,
                b.out_ptrs.data_ptr() + lo * es_p, None, hi - lo, s_cmp.cuda_stream, None)
        _lib.check(st, "kronmult_batched_async")
        ev_cmp[c].record(s_cmp)
        if out_monotone:
            s_out.wait_event(ev_cmp[c])
            o0, o1 = out_rows[c]
            with torch.cuda.stream(s_out):
                h_outputs[o0:o1].copy_(b.outputs[o0:o1], non_blocking=True)
    if not out_monotone:
        s_out.wait_stream(s_cmp)
        with torch.cuda.stream(s_out):
            h_outputs.copy_(b.outputs, non_blocking=True)
    return s_in, s_cmp, s_out


def host_device_pointer(t: torch.Tensor) -> int:
    """Device address of a page-locked host tensor (kronmult_host_device_pointer)."""
    if t.device.type != "cpu" or not t.is_pinned():
        raise ValueError("host_device_pointer needs a page-locked (pinned) CPU tensor")
    dp = ctypes.c_void_p()
    _lib.check(_lib.lib().kronmult_host_device_pointer(t.data_ptr(), ctypes.byref(dp)),
               "kronmult_host_device_pointer")
    return int(dp.value)


def forward_from_host_mapped(b: DeviceBatch, h_inputs: torch.Tensor, h_factors: torch.Tensor,
                             h_outputs: torch.Tensor, chunks: int = 2, streams=None, last_share: float = 0.1):
    """End-to-end forward whose kernels read the inputs and factors straight from pinned
    host memory over the CPU-GPU link (no staging copy); the outputs are accumulated in
    device memory and copied back piecewise, the copy of piece i overlapping the
    forward of piece i+1.  On GB300 the CPU-GPU link moves about 0.21 TB/s
    host-to-device, by the copy engines or by loads from the SMs alike, and the FP64
    forward consumes its inputs at about that rate, so reading them over the link
    slows it by under 2 % and no copy-in precedes it.  Only the last piece's
    copy back is exposed, so the last piece takes `last_share` of the output groups
    (the others share the rest evenly): on the 36864-entry FP64 batch two pieces split
    9:1 measured 6.74 ms against 6.89 ms for an even split.  `h_inputs` and
    `h_factors` must be contiguous pinned tensors shaped like the batch's inputs and
    factors.  Enqueues only; synchronise with torch.cuda.synchronize()."""
    for h, t in ((h_inputs, b.inputs), (h_factors, b.factors)):
        if h.shape != t.shape or h.dtype != t.dtype or not h.is_contiguous():
            raise ValueError("h_inputs / h_factors must be contiguous pinned tensors shaped like the batch's")
    dev = b.inputs.device
    s_cmp, s_out = (streams or (torch.cuda.Stream(dev), torch.cuda.Stream(dev)))[-2:]
    cache = b.__dict__.setdefault("_mapped_ptrs", {})
    key = (h_inputs.data_ptr(), h_factors.data_ptr())
    if key not in cache:
        base_in = host_device_pointer(h_inputs)
        base_fac = host_device_pointer(h_factors)
        k = torch.arange(b.nb, device=dev, dtype=torch.int64)
        i = torch.arange(b.d, device=dev, dtype=torch.int64)
        in_ptrs = (base_in + k * (h_inputs.shape[1] * h_inputs.element_size())).contiguous()
        mat_ptrs = (base_fac + ((b.fac_index[:, None] * b.d + i[None, :])
                                * (h_factors.shape[1] * h_factors.element_size()))).reshape(-1).contiguous()
        cache.clear()
        cache[key] = (in_ptrs, mat_ptrs)
    in_ptrs, mat_ptrs = cache[key]
    cuts, _, out_rows, _, out_monotone = _host_pipeline_plan(b, chunks, last_share)
    nchunks = len(cuts) - 1
    es_p = 8
    fn = getattr(_lib.lib(), _FN[b.inputs.dtype] + "_async")
    for c in range(nchunks):
        lo, hi = cuts[c], cuts[c + 1]
        if hi <= lo:
            continue
        st = fn(b.d, b.n, mat_ptrs.data_ptr() + lo * b.d * es_p, b.stride, in_ptrs.data_ptr() + lo * es_p,
                b.out_ptrs.data_ptr() + lo * es_p, None, hi - lo, s_cmp.cuda_stream, None)
        _lib.check(st, "kronmult_batched_async")
        if out_monotone:
            ev = torch.cuda.Event()
            ev.record(s_cmp)
            s_out.wait_event(ev)
            o0, o1 = out_rows[c]
            with torch.cuda.stream(s_out):
                h_outputs[o0:o1].copy_(b.outputs[o0:o1], non_blocking=True)
    if not out_monotone:
        s_out.wait_stream(s_cmp)
        with torch.cuda.stream(s_out):
            h_outputs.copy_(b.outputs, non_blocking=True)
    return s_cmp, s_out


def _host_pipeline_plan(b: DeviceBatch, chunks: int, last_share: float | None = None):
    """Piece boundaries of forward_from_host (cut at output-group starts), the factor
    rows and output rows each piece touches, and whether factor sets and outputs are
    used in increasing order.  Pieces hold equal numbers of output groups, or, with
    `last_share` in (0, 1) and more than one piece, the last piece holds that share of
    the groups and the others split the rest evenly.  Computed once per batch and
    piece layout from host copies of the index maps, so repeated calls make no
    device-to-host transfer."""
    if last_share is not None and not 0.0 < last_share < 1.0:
        raise ValueError("last_share must lie in (0, 1)")
    key = (chunks, last_share)
    cache = b.__dict__.setdefault("_host_plans", {})
    if key in cache:
        return cache[key]
    nb = b.nb
    oi = b.out_index.cpu()
    fi = b.fac_index.cpu()
    starts = torch.nonzero(torch.cat([torch.tensor([True]), oi[1:] != oi[:-1]])).flatten().tolist() + [nb]
    ngroups = len(starts) - 1
    chunks = max(1, min(chunks, ngroups))
    if last_share is None or chunks == 1:
        cuts = [starts[(ngroups * c) // chunks] for c in range(chunks)] + [nb]
    else:
        head = min(ngroups - 1, max(chunks - 1, int(round(ngroups * (1.0 - last_share)))))
        cuts = [starts[(head * c) // (chunks - 1)] for c in range(chunks - 1)] + [starts[head], nb]
    monotone = bool(torch.all(fi[1:] >= fi[:-1])) if nb > 1 else True
    out_monotone = bool(torch.all(oi[1:] >= oi[:-1])) if nb > 1 else True
    fac_rows, out_rows = [], []
    for c in range(chunks):
        lo, hi = cuts[c], cuts[c + 1]
        if hi > lo:
            fac_rows.append((int(fi[lo]) * b.d, (int(fi[hi - 1]) + 1) * b.d))
            out_rows.append((int(oi[lo]), int(oi[hi - 1]) + 1))
        else:
            fac_rows.append((0, 0))
            out_rows.append((0, 0))
    plan = (cuts, fac_rows, out_rows, monotone, out_monotone)
    cache[key] = plan
    return plan


def forward_f64_emulated(b: DeviceBatch, stream=None) -> None:
    """FP64 batch forward computed in double-float arithmetic on the FP32 pipe
    (kronmult_batched_f64_emulated_async): FP64-accurate (relative error ~1e-14)."""
    if b.inputs.dtype != torch.float64 or b.outputs.dtype != torch.float64:
        raise TypeError("the emulated FP64 forward needs float64 factors, inputs and outputs")
    ws = b.ws_ptrs.data_ptr() if b.ws_ptrs is not None else None
    st = _lib.lib().kronmult_batched_f64_emulated_async(b.d, b.n, b.mat_ptrs.data_ptr(), b.stride,
                                                         b.in_ptrs.data_ptr(), b.out_ptrs.data_ptr(), ws, b.nb,
                                                         _stream_handle(stream))
    _lib.check(st, "kronmult_batched_f64_emulated_async")


def forward_indexed(d: int, n: int, stride: int, factors: torch.Tensor, factor_index: torch.Tensor,
                    inputs: torch.Tensor, outputs: torch.Tensor, output_index: torch.Tensor,
                    input_index: torch.Tensor | None = None, scratch: torch.Tensor | None = None,
                    stream=None) -> torch.Tensor:
    """Indexed forward (kronmult_indexed_*): factors (M, pitch) rows of factor storage,
    factor_index (B, d) int32, inputs (B or I, N), outputs (E, N), output_index (B,) int32.
    Returns the scratch tensor that holds the pointer tables (keep it alive until the
    launch has run, or pass one in to reuse it)."""
    dt = inputs.dtype
    name = {torch.float64: "kronmult_indexed_f64_async", torch.float32: "kronmult_indexed_f32_async"}.get(dt)
    if name is None:
        raise TypeError("indexed forward is defined for float64 and float32")
    nb = int(output_index.shape[0])
    need = int(_lib.lib().kronmult_indexed_scratch_bytes(d, nb))
    if scratch is None or scratch.numel() * scratch.element_size() < need:
        scratch = torch.empty(max(need, 8), dtype=torch.uint8, device=inputs.device)
    fi = factor_index.to(torch.int32).contiguous()
    oi = output_index.to(torch.int32).contiguous()
    ii = None if input_index is None else input_index.to(torch.int32).contiguous()
    st = getattr(_lib.lib(), name)(d, n, stride, factors.data_ptr(), factors.shape[1], fi.data_ptr(),
                                   inputs.data_ptr(), inputs.shape[1], None if ii is None else ii.data_ptr(),
                                   outputs.data_ptr(), outputs.shape[1], oi.data_ptr(), nb, scratch.data_ptr(),
                                   scratch.numel() * scratch.element_size(), _stream_handle(stream))
    _lib.check(st, name)
    scratch._kronmult_keep = (fi, oi, ii)
    return scratch
