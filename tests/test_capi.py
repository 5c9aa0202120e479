"""The C ABI library: it loads, exports every symbol include/*.h declares, and its
host-side argument checks reject bad calls before touching a GPU.  No GPU needed."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT

CUDA_ERROR_INVALID_VALUE = 1


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(kronmult_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from kronmult_gb300 import _build, _lib

    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    return _lib.lib()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "kronmult_batched_f64" in names and "kronmult_batched_f32" in names


def test_every_declared_symbol_is_exported(lib):
    from kronmult_gb300 import _lib

    for name in declared_symbols():
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature in kronmult_gb300/_lib.py"


def test_pow_int_and_version(lib):
    assert lib.kronmult_pow_int(4, 6) == 4096
    assert lib.kronmult_pow_int(3, 0) == 1
    assert lib.kronmult_pow_int(2, 40) > 2**31 - 1  # saturates above the int range
    assert lib.kronmult_abi_version() >= 1


@pytest.mark.parametrize("args", [
    dict(d=-1, n=4, stride=4, nb=1),     # negative factor count
    dict(d=2, n=-4, stride=4, nb=1),     # negative size
    dict(d=2, n=4, stride=3, nb=1),      # stride below the matrix size
    dict(d=2, n=4, stride=4, nb=-5),     # negative batch
    dict(d=40, n=4, stride=4, nb=1),     # n^d beyond the 32-bit vector length
])
def test_invalid_arguments_rejected_on_host(lib, args):
    dummy = ctypes.c_void_p(16)
    for fn in (lib.kronmult_batched_f64_async, lib.kronmult_batched_f32_async):
        rc = fn(args["d"], args["n"], dummy, args["stride"], dummy, dummy, dummy, args["nb"], None, None)
        assert rc == CUDA_ERROR_INVALID_VALUE


def test_null_tables_rejected(lib):
    rc = lib.kronmult_batched_f64_async(2, 4, None, 4, None, None, None, 3, None, None)
    assert rc == CUDA_ERROR_INVALID_VALUE


def test_empty_batch_is_success_without_launch(lib):
    assert lib.kronmult_batched_f64_async(3, 4, None, 4, None, None, None, 0, None, None) == 0
    assert lib.kronmult_batched_f32_async(3, 0, None, 4, None, None, None, 7, None, None) == 0


def test_error_string(lib):
    from kronmult_gb300 import _lib

    assert "invalid argument" in _lib.error_string(1).lower()


def test_python_mirror_raises(lib):
    import kronmult_gb300 as K

    with pytest.raises(K.KronmultError) as e:
        K.kronmult_batched(2, 4, 8, 3, 8, 8, None, 1)
    assert e.value.status == CUDA_ERROR_INVALID_VALUE
    with pytest.raises(TypeError):
        import torch

        K.kronmult_batched(2, 4, 8, 4, 8, 8, None, 1, dtype=torch.float16)


def test_grouped_plan_rejects_bad_mode_and_dtype(lib):
    import ctypes

    from kronmult_gb300 import _lib

    h = ctypes.c_void_p()
    g = (_lib.Group * 1)()
    assert lib.kronmult_grouped_plan_create(ctypes.byref(h), g, 1, 7, 0, None) == CUDA_ERROR_INVALID_VALUE
    assert lib.kronmult_grouped_plan_create(ctypes.byref(h), g, 1, 0, 9, None) == CUDA_ERROR_INVALID_VALUE
    assert lib.kronmult_grouped_plan_create(None, g, 1, 0, 0, None) == CUDA_ERROR_INVALID_VALUE
    assert lib.kronmult_grouped_run(None, None) == CUDA_ERROR_INVALID_VALUE
    assert lib.kronmult_grouped_plan_destroy(None) == 0


def test_tuning_cache_roundtrip_on_host(lib, tmp_path):
    from kronmult_gb300 import grouped as G

    G.tuning_cache_clear()
    G.tuning_cache_set(5, 3, 0, {"team_size": 64, "entries_per_team": 4, "fp64_path": 4})
    assert G.tuning_cache_get(5, 3, 0) == {"team_size": 64, "ctas_per_sm": 0, "entries_per_team": 4, "prefetch": 0,
                                           "fp64_path": 4}
    path = str(tmp_path / "t.txt")
    G.tuning_cache_save(path)
    G.tuning_cache_clear()
    assert G.tuning_cache_get(5, 3, 0) is None
    G.tuning_cache_load(path)
    assert G.tuning_cache_get(5, 3, 0)["team_size"] == 64
    assert G.tuning_cache_get(5, 3, 0)["fp64_path"] == 4
    # a cache written before fp64_path existed (8 fields per line) loads with the automatic path
    lines = [ln.split() for ln in open(path) if not ln.startswith("#")]
    assert len(lines) == 1 and len(lines[0]) == 9
    with open(path, "w") as f:
        f.write("# v2\n" + " ".join(lines[0][:8]) + "\n")
    G.tuning_cache_clear()
    G.tuning_cache_load(path)
    assert G.tuning_cache_get(5, 3, 0)["fp64_path"] == 0
    G.tuning_cache_clear()
    with pytest.raises(Exception):
        G.tuning_cache_set(5, 3, 0, {"fp64_path": 5})
    G.tuning_cache_clear()


def build_drop_in(tmp_dir):
    """Compile tests/cpp/drop_in.cpp, a caller written against the reference's
    kronmult.cuh interface, against include/kronmult.cuh and the library."""
    import shutil
    import subprocess

    from kronmult_gb300 import _lib

    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = os.path.join(str(tmp_dir), "drop_in")
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda_home, "include"),
           os.path.join(ROOT, "tests", "cpp", "drop_in.cpp"), "-o", exe, "-L", libdir, "-lkronmult_gb300",
           "-L", os.path.join(cuda_home, "lib64"), "-lcudart", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_drop_in_compiles(lib, tmp_path):
    assert os.path.exists(build_drop_in(tmp_path))


def test_host_pipeline_piece_plan():
    """Host pipelines cut their pieces at output-group starts: even pieces, or a last
    piece holding `last_share` of the groups; every piece non-empty, cuts increasing."""
    from kronmult_gb300 import DeviceBatch
    from kronmult_gb300 import workloads as W
    from kronmult_gb300.api import _host_pipeline_plan

    b = W.config2(scale=24 / 4096)  # 24 output groups of 9 entries
    db = DeviceBatch.from_host(b, device="cpu")
    assert _host_pipeline_plan(db, 2)[0] == [0, 108, 216]
    assert _host_pipeline_plan(db, 2, 0.1)[0] == [0, 198, 216]
    assert _host_pipeline_plan(db, 3, 0.1)[0] == [0, 99, 198, 216]
    for chunks in (1, 2, 3, 7, 24, 40):
        for share in (None, 0.01, 0.1, 0.5, 0.99):
            cuts, _, out_rows, _, _ = _host_pipeline_plan(db, chunks, share)
            assert cuts[0] == 0 and cuts[-1] == b.nb
            assert all(lo < hi and lo % 9 == 0 for lo, hi in zip(cuts, cuts[1:]))
            assert len(cuts) - 1 == min(chunks, 24)
            assert out_rows[0][0] == 0 and out_rows[-1][1] == 24
    with pytest.raises(ValueError):
        _host_pipeline_plan(db, 2, 1.0)
