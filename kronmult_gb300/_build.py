"""Builds libkronmult_gb300.so in-tree with nvcc for sm_103a.

Every translation unit under csrc/ is compiled in parallel to an object file
under _build/, then linked into kronmult_gb300/libkronmult_gb300.so.  No cmake,
no torch extension machinery: the library has a plain C ABI
(include/kronmult_gb300.h) and links only the CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libkronmult_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-cudart", "shared", "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build kronmult_gb300")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    paths.append(os.path.join(ROOT, "include", "kronmult_gb300.h"))
    return max(os.path.getmtime(p) for p in paths)


def _compile(nvcc: str, src: str, obj: str) -> tuple[str, int, str]:
    cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    return src, p.returncode, p.stdout + p.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library if any source is newer than it; return its path."""
    srcs = sources()
    newest = max([_headers_mtime()] + [os.path.getmtime(s) for s in srcs])
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]
    jobs = max(1, min(len(srcs), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda so: _compile(nvcc, *so), zip(srcs, objs)))
    failed = [(s, log) for s, rc, log in results if rc != 0]
    for s, rc, log in results:
        if verbose and log.strip():
            print(f"--- {os.path.basename(s)}\n{log}", file=sys.stderr)
    if failed:
        msg = "\n".join(f"--- {os.path.basename(s)}\n{log}" for s, log in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stdout}{p.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
