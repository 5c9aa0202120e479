"""Parity of the CUDA forward with the reference's outputs (golden fixtures) and
with the C oracle on seeded batches of every configuration's shape; full-size
checks through size-independent properties.  Tolerances: relative L2 <= 1e-13
for FP64 (atomic summation order is the only permitted difference), 1e-5 for
FP32 against the FP64 result."""
import functools

import numpy as np
import pytest
import torch

from conftest import golden_names, load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-13
TOL32 = 1e-5


def run(b, cuda, dtype=torch.float64, out_dtype=None, tuning=None, sync=False, ws=False):
    from kronmult_gb300 import DeviceBatch

    db = DeviceBatch.from_host(b, device=cuda, dtype=dtype, out_dtype=out_dtype, with_workspace=ws)
    db.forward(tuning=tuning, sync=sync)
    torch.cuda.synchronize()
    return db.outputs.cpu().numpy(), db


@pytest.mark.parametrize("name", golden_names())
def test_golden_f64(cuda, name):
    b, z = load_golden(name)
    got, _ = run(b, cuda, sync=True)
    assert O.rel_l2(got, z["expected_f64"]) <= TOL64


@pytest.mark.parametrize("name", golden_names())
def test_golden_f32(cuda, name):
    b, z = load_golden(name)
    got, _ = run(b, cuda, dtype=torch.float32, sync=True)
    # FP32 against the reference's own FP32 result and against FP64
    assert O.rel_l2(got, z["expected_f32"]) <= TOL32
    assert O.rel_l2(got, z["expected_f64"]) <= TOL32


def test_config1_full_f64(cuda):
    from kronmult_gb300 import workloads as W

    b = W.config1()
    got, _ = run(b, cuda)
    assert O.rel_l2(got, O.forward(b)) <= TOL64


def test_config2_sample_f64(cuda):
    from kronmult_gb300 import workloads as W

    b = W.config2(scale=64 / 4096)
    got, _ = run(b, cuda)
    assert O.rel_l2(got, O.forward(b)) <= TOL64


@pytest.mark.parametrize("gi", range(4))
def test_config3_groups_f64(cuda, gi):
    from kronmult_gb300 import workloads as W

    b = W.config3(scale=0.02)[gi]
    got, _ = run(b, cuda)
    assert O.rel_l2(got, O.forward(b)) <= TOL64


def test_config4_fp32_f64out(cuda):
    from kronmult_gb300 import workloads as W

    b = W.config4(scale=16 / 4096)
    got, _ = run(b, cuda, dtype=torch.float32, out_dtype=torch.float64)
    ref32 = O.forward(b, dtype=np.float32, out_dtype=np.float64)
    ref64 = O.forward(b)
    assert O.rel_l2(got, ref32) <= 1e-6
    assert O.rel_l2(got, ref64) <= TOL32


def test_config5_shared_factors(cuda):
    from kronmult_gb300 import workloads as W

    b = W.config5(scale=32 / 2048)
    got, _ = run(b, cuda)
    assert O.rel_l2(got, O.forward(b)) <= TOL64
    got32, _ = run(b, cuda, dtype=torch.float32)
    assert O.rel_l2(got32, O.forward(b)) <= TOL32


@pytest.mark.parametrize("prefetch", [1, 2])
@pytest.mark.parametrize("team_size", [8, 16, 32, 64, 128, 256, 512])
def test_team_sizes_agree(cuda, team_size, prefetch):
    """Every launch shape the autotuner may pick gives the oracle's result."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(5, 4, 5, 7, 6, seed=99)
    got, _ = run(b, cuda, tuning={"team_size": team_size, "entries_per_team": 3, "prefetch": prefetch})
    assert O.rel_l2(got, O.forward(b)) <= TOL64


@pytest.mark.parametrize("ept", [1, 2, 8])
@pytest.mark.parametrize("team_size", [8, 32, 128, 256])
def test_single_entry_and_run_kernels(cuda, team_size, ept):
    """entries_per_team = 1 selects the single-entry kernel, larger values the
    run-accumulating one; both dtypes, all agree with the oracle."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(4, 4, 6, 9, 5, seed=300 + team_size)
    t = {"team_size": team_size, "entries_per_team": ept}
    got, _ = run(b, cuda, tuning=t)
    assert O.rel_l2(got, O.forward(b)) <= TOL64
    got32, _ = run(b, cuda, dtype=torch.float32, tuning=t)
    assert O.rel_l2(got32, O.forward(b)) <= TOL32


@pytest.mark.parametrize("n", [2, 3, 5, 6, 7, 8])
def test_prefetch_odd_sizes(cuda, n):
    """Unaligned vector lengths take the element-wise asynchronous copy."""
    from kronmult_gb300 import workloads as W

    d = 3 if n <= 6 else 2
    b = W.make_batch(d, n, n + 2, 4, 5, seed=200 + n)
    for pf in (1, 2):
        got, _ = run(b, cuda, tuning={"prefetch": pf, "entries_per_team": 4})
        assert O.rel_l2(got, O.forward(b)) <= TOL64
        got32, _ = run(b, cuda, dtype=torch.float32, tuning={"prefetch": pf, "entries_per_team": 4})
        assert O.rel_l2(got32, O.forward(b)) <= TOL32


def test_inputs_not_modified(cuda):
    from kronmult_gb300 import workloads as W

    b = W.config1(scale=4 / 1024)
    _, db = run(b, cuda)
    assert np.array_equal(db.inputs.cpu().numpy(), b.inputs)


def test_aliased_inputs(cuda):
    """Several entries reading one input vector (the reference cannot do this, it
    overwrites its inputs)."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W

    b = W.make_batch(3, 4, 4, 3, 4, seed=5)
    db = DeviceBatch.from_host(b, device=cuda)
    db.in_ptrs = torch.full_like(db.in_ptrs, db.inputs.data_ptr())
    db.forward(sync=True)
    b2 = W.Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, np.repeat(b.inputs[:1], b.nb, 0), b.out_init,
                 b.fac_index, b.out_index)
    assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b2)) <= TOL64


def test_large_vector_two_pass(cuda):
    """n^d beyond shared memory: two passes through the workspace; the input is only read."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W

    b = W.make_batch(5, 8, 8, 1, 2, seed=31)  # N = 32768: 128 KiB in FP32
    ref = O.forward(b)
    db = DeviceBatch.from_host(b, device=cuda, dtype=torch.float32, with_workspace=True)
    x0 = db.inputs.clone()
    db.forward(sync=True)
    assert O.rel_l2(db.outputs.double().cpu().numpy(), ref) <= TOL32
    assert torch.equal(db.inputs, x0)


def test_large_vector_global_sweep_f64(cuda):
    """FP64 vectors beyond shared memory: every mode through input/workspace."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(5, 8, 8, 1, 2, seed=31)  # N = 32768 doubles = 256 KiB
    got, _ = run(b, cuda, ws=True)
    assert O.rel_l2(got, O.forward(b)) <= TOL64


@pytest.mark.parametrize("d,n,dtype", [(10, 3, torch.float32), (7, 5, torch.float32), (8, 4, torch.float32),
                                       (16, 2, torch.float32), (5, 7, torch.float32), (7, 6, torch.float32),
                                       (10, 3, torch.float64), (8, 4, torch.float64)])
def test_large_vector_two_pass_shapes(cuda, d, n, dtype):
    """FP32 two-pass path with partial pass-2 tiles (n = 3, 5, 7) and every n; FP64
    shapes of the same sizes take the global sweep."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, n + 1, 3, 2, seed=700 + 10 * d + n)
    got, _ = run(b, cuda, dtype=dtype, ws=True)
    tol = TOL64 if dtype == torch.float64 else TOL32
    assert O.rel_l2(got, O.forward(b)) <= tol


def test_large_vector_global_fallback(cuda):
    """Beyond the two-pass limits (n = 2, d = 25: 2^12 slow positions would remain for
    pass 2) every mode goes through input/workspace in global memory."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(25, 2, 2, 1, 1, seed=32)  # N = 33554432
    got, _ = run(b, cuda, dtype=torch.float32, ws=True)
    assert O.rel_l2(got, O.forward(b)) <= TOL32


def test_reference_signature_mirror(cuda):
    """The Python mirror of kronmult_batched<double> with raw device pointer arrays."""
    import kronmult_gb300 as K
    from kronmult_gb300 import workloads as W

    b = W.config1(scale=8 / 1024)
    db = K.DeviceBatch.from_host(b, device=cuda)
    K.kronmult_batched(b.d, b.n, db.mat_ptrs, b.stride, db.in_ptrs, db.out_ptrs, None, b.nb)
    assert O.rel_l2(db.outputs.cpu().numpy(), O.forward(b)) <= TOL64


def test_full_config2_checksum(cuda):
    """Full-size configuration 2 (36864 entries, N = 4096): the sum of every output
    vector equals sum_k kron(colsum(A_k,0), ..., colsum(A_k,5)) . x_k, computed on the
    host from the inputs alone."""
    from kronmult_gb300 import workloads as W

    b = W.config2()
    got, db = run(b, cuda)
    n, d = b.n, b.d
    cs = np.empty((b.nb, d, n))
    for i in range(d):
        F = b.factors[b.fac_index * d + i][:, :b.stride * n].reshape(b.nb, n, b.stride)[:, :, :n]
        cs[:, i, :] = F.sum(axis=2)  # F[k, col, row]: column sums over rows
    x = b.inputs.reshape((b.nb,) + (n,) * d)
    s = x
    for i in range(d - 1, -1, -1):
        s = np.einsum("k...j,kj->k...", s, cs[:, i, :])
    want = np.zeros(b.n_out)
    np.add.at(want, b.out_index, s)
    have = got.sum(axis=1)
    assert np.linalg.norm(have - want) / np.linalg.norm(want) <= 1e-12


def test_linearity_full_config4_f32(cuda):
    """Full-size configuration 4 in FP32 storage with FP64 outputs: F(2x) = 2 F(x)
    exactly (scaling by two is exact in binary floating point)."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W

    b = W.config4()
    db = DeviceBatch.from_host(b, device=cuda, dtype=torch.float32, out_dtype=torch.float64)
    db.forward()
    y1 = db.outputs.clone()
    db.outputs.zero_()
    db.inputs.mul_(2)
    db.forward()
    torch.cuda.synchronize()
    # the atomic order may differ between the runs; compare normwise
    assert (torch.linalg.norm(db.outputs - 2 * y1) / torch.linalg.norm(2 * y1)).item() <= 1e-14


def test_cpp_drop_in_runs(cuda, tmp_path):
    """The reference-style C++ caller, linked against the library, passes its own check."""
    import subprocess

    from test_capi import build_drop_in

    exe = build_drop_in(tmp_path)
    p = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr


@pytest.mark.parametrize("n,d", [(2, 2), (2, 3), (2, 9), (4, 2), (4, 3), (4, 5), (4, 6), (8, 3), (8, 4)])
def test_fp32_two_modes_per_pass(cuda, n, d):
    """FP32 n = 2, 4 and 8 (d = 3, 4) runs two modes per shared-memory pass (odd d: one
    single step first); same result as the oracle's FP32 sweep up to FP32 rounding."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, n + 3, 6, 7, seed=400 + 10 * n + d)
    ref32 = O.forward(b, dtype=np.float32)
    got, _ = run(b, cuda, dtype=torch.float32)
    assert O.rel_l2(got, ref32) <= 1e-6
    assert O.rel_l2(got, O.forward(b)) <= TOL32
    got64o, _ = run(b, cuda, dtype=torch.float32, out_dtype=torch.float64)
    assert O.rel_l2(got64o, O.forward(b)) <= TOL32


def test_fp32_three_modes_per_pass_bitwise(cuda):
    """FP32 n = 4, d = 6 runs three modes per shared-memory pass (a lane pair per
    64-value tri-fibre).  With one output per entry its results equal, bit for bit, the
    one-mode-per-step kernel's (a forced team size selects that one): both are the same
    k-ascending FMA chains."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(6, 4, 7, 50, 1, seed=4646)
    plain, _ = run(b, cuda, dtype=torch.float32, tuning={"team_size": 128})
    for tuning in (None, {"entries_per_team": 3}):  # one wave; a grid of 3 entries per CTA
        got, _ = run(b, cuda, dtype=torch.float32, tuning=tuning)
        assert np.array_equal(got, plain)
    assert O.rel_l2(plain, O.forward(b)) <= TOL32


@pytest.mark.parametrize("tuning", [None, {"entries_per_team": 1}, {"entries_per_team": 5},
                                    {"entries_per_team": 64}, {"ctas_per_sm": 1}, {"ctas_per_sm": 7}])
def test_fp32_three_modes_per_pass_runs(cuda, tuning):
    """Ragged runs of entries into shared outputs (runs cut by the CTAs' shares of the
    entries), into FP32 and FP64 outputs: the oracle's FP32 sweep up to FP32 rounding."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(6, 4, 4, 9, [1, 7, 3, 12, 1, 2, 9, 4, 6], seed=4747, out_init="normal")
    ref32 = O.forward(b, dtype=np.float32)
    got, _ = run(b, cuda, dtype=torch.float32, tuning=tuning)
    assert O.rel_l2(got, ref32) <= 1e-6
    got64o, _ = run(b, cuda, dtype=torch.float32, out_dtype=torch.float64, tuning=tuning)
    assert O.rel_l2(got64o, O.forward(b)) <= TOL32


def test_fp32_three_modes_per_pass_unaligned_inputs(cuda):
    """Input vectors that do not start on a 16-byte boundary are staged value by value:
    the same bits as the aligned inputs."""
    from kronmult_gb300 import DeviceBatch, _lib
    from kronmult_gb300 import workloads as W

    b = W.make_batch(6, 4, 5, 6, 3, seed=4848)
    want, _ = run(b, cuda, dtype=torch.float32)
    db = DeviceBatch.from_host(b, device=cuda, dtype=torch.float32)
    shifted = torch.zeros((b.nb, b.N + 1), dtype=torch.float32, device=cuda)
    shifted[:, 1:] = db.inputs
    k = torch.arange(b.nb, device=cuda, dtype=torch.int64)
    in_ptrs = (shifted.data_ptr() + 4 + k * ((b.N + 1) * 4)).contiguous()
    st = _lib.lib().kronmult_batched_f32(b.d, b.n, db.mat_ptrs.data_ptr(), b.stride, in_ptrs.data_ptr(),
                                         db.out_ptrs.data_ptr(), None, b.nb)
    assert st == 0
    torch.cuda.synchronize()
    assert O.rel_l2(db.outputs.cpu().numpy(), want) <= 1e-6


@pytest.mark.parametrize("d,n", [(3, 6), (2, 6), (6, 3), (3, 5), (2, 7), (4, 3)])
def test_fp64_element_mapping(cuda, d, n):
    """FP64 shapes whose fibre count leaves lanes idle take the element-mapped kernel."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, n + 1, 6, 5, seed=500 + 10 * d + n)
    got, _ = run(b, cuda)
    assert O.rel_l2(got, O.forward(b)) <= TOL64


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_large_published_shape(cuda, dtype):
    """The reference's published 'large' shape (n = 8, d = 6, N = 262144, stride 67,
    its aliasing pattern onto 5 outputs) on 12 entries, through the global-memory path."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(6, 8, 67, 12, 1, seed=3903)
    idx = np.arange(b.nb)
    b = W.Batch(b.name, b.d, b.n, b.stride, b.block, b.factors, b.inputs, b.out_init[:5],
                b.fac_index, np.where(idx < 5, idx, (idx * 5) // b.nb))
    got, _ = run(b, cuda, dtype=dtype, ws=True)
    tol = TOL64 if dtype == torch.float64 else TOL32
    assert O.rel_l2(got, O.forward(b)) <= tol


@pytest.mark.parametrize("chunks", [1, 2, 5])
def test_forward_from_host_pipelines(cuda, chunks):
    """The end-to-end host pipelines (staging copies, and kernels reading pinned host
    memory directly) against the device-resident forward and the oracle."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.api import forward_from_host, forward_from_host_mapped

    b = W.config2(scale=24 / 4096)
    ref = O.forward(b)
    db = DeviceBatch.from_host(b, device=cuda)
    h_in = torch.from_numpy(b.inputs).pin_memory()
    h_fac = torch.from_numpy(b.factors).pin_memory()
    small_last = functools.partial(forward_from_host, last_share=0.05)
    for fn in (forward_from_host, forward_from_host_mapped, small_last):
        db.outputs.zero_()
        h_out = torch.full(db.outputs.shape, float("nan"), dtype=torch.float64).pin_memory()
        torch.cuda.synchronize()
        fn(db, h_in, h_fac, h_out, chunks=chunks)
        torch.cuda.synchronize()
        assert O.rel_l2(h_out.numpy(), ref) <= TOL64


@pytest.mark.parametrize("d,n", [(0, 3), (1, 1), (3, 1), (1, 2), (1, 8), (2, 9), (2, 12), (3, 10), (2, 16)])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_edge_shapes(cuda, d, n, dtype):
    """d = 0 (the empty product: output += input), n = 1, single factors, and n > 8
    (the generic kernel) against the oracle."""
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, n + 2, 5, 3, seed=900 + 10 * d + n, out_init="normal")
    got, _ = run(b, cuda, dtype=dtype)
    tol = TOL64 if dtype == torch.float64 else TOL32
    assert O.rel_l2(got, O.forward(b)) <= tol


@pytest.mark.parametrize("d,n", [(3, 6), (3, 3), (2, 4), (3, 5), (5, 3), (3, 7), (4, 4), (2, 6), (4, 5)])
def test_fp64_element_and_fibre_mappings_agree_bitwise(cuda, d, n):
    """FP64 maps output elements to threads where whole fibres would idle lanes
    (d = 3, n = 6; d = 2, n = 4; ...) and whole fibres elsewhere; both run the same
    k-ascending FMA chain per element, so with one entry per output the default
    launch and a launch forced onto fibres (a fixed team size) agree bit for bit."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W

    b = W.make_batch(d, n, n, 300, 1, seed=4000 + 10 * d + n)
    outs = []
    for tuning in (None, {"team_size": 16}):
        db = DeviceBatch.from_host(b, device=cuda, dtype=torch.float64)
        db.forward(tuning=tuning, sync=True)
        outs.append(db.outputs.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    assert O.rel_l2(outs[0], O.forward(b)) <= TOL64
