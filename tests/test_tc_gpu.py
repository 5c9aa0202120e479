"""Tensor-core (tcgen05) reduced-precision forward for n = 8: TF32, BF16 and split-BF16
(BF16X3: v = hi + lo, three MMAs per product) mode products with FP32 accumulation and
FP64 output accumulation, against the FP64 oracle.  Errors are stated against FP64
(relative L2):
  FP32 CUDA-core <= 1e-6   TF32 <= 2e-3   BF16 <= 2e-2   BF16X3 <= 1e-4
(TF32 keeps 10 mantissa bits, BF16 7, the split pair about 16; each of the d roundings
of the vector and of the factors contributes about 2^-11, 2^-8 resp. 2^-17 relative
error, the dropped lo.lo term about 2^-16.)"""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-6, "tf32": 2e-3, "bf16": 2e-2, "bf16x3": 1e-4}


def code_of(compute):
    from kronmult_gb300 import _lib

    return {"fp32": _lib.KRONMULT_COMPUTE_FP32, "tf32": _lib.KRONMULT_COMPUTE_TF32,
            "bf16": _lib.KRONMULT_COMPUTE_BF16, "bf16x3": _lib.KRONMULT_COMPUTE_BF16X3}[compute]


def run_mode(b, cuda, compute):
    from kronmult_gb300 import DeviceBatch, _lib, forward_f32_f64out

    db = DeviceBatch.from_host(b, device=cuda, dtype=torch.float32, out_dtype=torch.float64)
    forward_f32_f64out(db, compute=code_of(compute))
    torch.cuda.synchronize()
    err = ctypes_device_error()
    assert err == 0, f"device error word {err}"
    return db.outputs.cpu().numpy()


def ctypes_device_error():
    import ctypes

    from kronmult_gb300 import _lib

    c = ctypes.c_int(0)
    _lib.check(_lib.lib().kronmult_device_error(ctypes.byref(c), 1), "kronmult_device_error")
    return c.value


@pytest.mark.parametrize("compute", ["tf32", "bf16", "bf16x3"])
@pytest.mark.parametrize("d", [1, 2, 3, 4])
def test_tc_shapes(cuda, compute, d):
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, 8, 8, 5, 3, seed=40 + d, factor_scale=1 / 8)
    got = run_mode(b, cuda, compute)
    assert O.rel_l2(got, O.forward(b)) <= TOL[compute]


@pytest.mark.parametrize("compute", ["fp32", "tf32", "bf16", "bf16x3"])
def test_config4_sample(cuda, compute):
    from kronmult_gb300 import workloads as W

    b = W.config4(scale=32 / 4096)
    got = run_mode(b, cuda, compute)
    err = O.rel_l2(got, O.forward(b))
    assert err <= TOL[compute]


def test_tc_matches_tf32_rounded_oracle(cuda):
    """The TF32 path equals an FP32 sweep whose operands are rounded to TF32 before
    every mode (round-to-nearest-even at 10 mantissa bits), up to FP32 summation order."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(2, 8, 8, 3, 2, seed=77, factor_scale=1 / 8)
    got = run_mode(b, cuda, "tf32")

    def tf32(a):
        a = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
        r = ((a + 0x1000) & ~np.uint64(0x1FFF)).astype(np.uint32)
        return r.view(np.float32).astype(np.float64)

    out = b.out_init.copy()
    for k in range(b.nb):
        x = tf32(b.inputs[k].astype(np.float32))
        for i in range(b.d - 1, -1, -1):
            A = b.factors[b.fac_index[k] * b.d + i]
            M = tf32(np.array([[A[r + c * b.stride] for c in range(8)] for r in range(8)], dtype=np.float32))
            F = x.size // 8
            y = (M @ x.reshape(F, 8).T).astype(np.float32)  # y[r, c]
            x = y.reshape(-1).astype(np.float64)
            if i > 0:
                x = tf32(x)
        out[b.out_index[k]] += x
    assert O.rel_l2(got, out) <= 1e-5


def test_tc_rejects_unsupported_shape(cuda):
    import kronmult_gb300 as K
    from kronmult_gb300 import workloads as W

    b = W.make_batch(2, 4, 4, 2, 2, seed=1)
    with pytest.raises(K.KronmultError):
        run_mode(b, cuda, "tf32")


def test_bounded_wait_runs_out_into_an_error_status(cuda):
    """A wait on an mbarrier that nothing arrives on ends in the device error word
    (code 1) instead of a hang; afterwards the context still runs the tensor-core
    forward correctly and the error word is clear."""
    import ctypes

    from kronmult_gb300 import _lib

    lib = _lib.lib()
    code = ctypes.c_int(-1)
    assert lib.kronmult_diag_wait_selftest(ctypes.byref(code)) == 0
    assert code.value == 1
    assert lib.kronmult_device_error(ctypes.byref(code), 0) == 0 and code.value == 0
    from kronmult_gb300 import workloads as W

    b = W.make_batch(3, 8, 8, 16, 4, seed=4242, factor_scale=1 / 8)
    assert O.rel_l2(run_mode(b, cuda, "tf32"), O.forward(b)) <= TOL["tf32"]


@pytest.mark.parametrize("compute", ["tf32", "bf16", "bf16x3"])
def test_tc_unaligned_inputs(cuda, compute):
    """Input vectors that do not start on a 16-byte boundary take the element-wise
    staging path (no bulk copy); results as with aligned inputs."""
    import ctypes

    from kronmult_gb300 import DeviceBatch, _lib
    from kronmult_gb300 import workloads as W

    b = W.make_batch(3, 8, 8, 6, 3, seed=4343, factor_scale=1 / 8)
    db = DeviceBatch.from_host(b, device=cuda, dtype=torch.float32, out_dtype=torch.float64)
    shifted = torch.zeros((b.nb, b.N + 1), dtype=torch.float32, device=cuda)
    shifted[:, 1:] = db.inputs
    k = torch.arange(b.nb, device=cuda, dtype=torch.int64)
    in_ptrs = (shifted.data_ptr() + 4 + k * ((b.N + 1) * 4)).contiguous()
    code = code_of(compute)
    st = _lib.lib().kronmult_batched_f32_f64out_async(b.d, b.n, db.mat_ptrs.data_ptr(), b.stride, in_ptrs.data_ptr(),
                                                      db.out_ptrs.data_ptr(), None, b.nb, code, None, None)
    assert st == 0
    torch.cuda.synchronize()
    assert ctypes_device_error() == 0
    assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= TOL[compute]


@pytest.mark.parametrize("compute", ["tf32", "bf16", "bf16x3"])
@pytest.mark.parametrize("tuning", [{"ctas_per_sm": 3}, {"ctas_per_sm": 5, "entries_per_team": 3},
                                    {"entries_per_team": 1}])
def test_tc_launch_shapes(cuda, compute, tuning):
    """Fewer resident CTAs per SM (the shared-memory reservation grows): the same values
    as the default launch up to FP64 summation order.  Other run lengths per CTA change
    which consecutive entries are summed in FP32 in tensor memory before the FP64
    atomics: equal up to FP32 rounding of those sums."""
    from kronmult_gb300 import DeviceBatch, _lib, forward_f32_f64out
    from kronmult_gb300 import workloads as W

    code = code_of(compute)
    b = W.config4(scale=24 / 4096)
    outs = []
    for t in (None, tuning):
        db = DeviceBatch.from_host(b, device=cuda, dtype=torch.float32, out_dtype=torch.float64)
        forward_f32_f64out(db, compute=code, tuning=t)
        torch.cuda.synchronize()
        assert ctypes_device_error() == 0
        outs.append(db.outputs.cpu().numpy())
    assert O.rel_l2(outs[1], outs[0]) <= (1e-6 if "entries_per_team" in tuning else 1e-12)
    assert O.rel_l2(outs[0], O.forward(b)) <= TOL[compute]


def test_split_bf16_accuracy_between_fp32_and_tf32(cuda):
    """The split-BF16 products keep about 16 significand bits: on the same batch the
    error against FP64 is far below TF32's and BF16's and above the FP32 sweep's."""
    from kronmult_gb300 import workloads as W

    b = W.config4(scale=48 / 4096)
    ref = O.forward(b)
    err = {c: O.rel_l2(run_mode(b, cuda, c), ref) for c in ("fp32", "tf32", "bf16", "bf16x3")}
    assert err["bf16x3"] < err["tf32"] / 10
    assert err["bf16x3"] < err["bf16"] / 100
    assert err["fp32"] < err["bf16x3"]

