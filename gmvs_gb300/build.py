"""Build the in-tree C-ABI library libgmvs_gb300.so for sm_103a.

Every translation unit is compiled in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a``) and linked into
``gmvs_gb300/_lib/libgmvs_gb300.so``.  Device code is compiled with
``-fmad=false`` and host code with ``-ffp-contract=off``: every fused
multiply-add is explicit, so results are reproducible bit for bit by a host
implementation of the same arithmetic.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(OUT_DIR, "libgmvs_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: only explicit fused multiply-adds are fused, so device code
# rounds exactly like the host restatement of the same arithmetic;
# -ffp-contract=off does the same for host code on aarch64 and x86-64.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-fvisibility=hidden", "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-I" + INCLUDE]

SOURCES = {
    "pm_f32.cu": [],
    "pm_qf32.cu": [],
    "pm_qf16.cu": [],
    "pm_tex.cu": [],
    "runtime.cu": [],
    "fusion.cu": [],
    "fuse_fixed.cu": [],
    "segments.cu": [],
    "gather.cu": [],
    "views.cu": [],
    "superpixel.cu": [],
    "job.cu": [],
    "prior.cpp": [],
    "felzenszwalb.cpp": [],
}


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gmvs_gb300")
    return cand


def _inputs() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "gmvs_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def is_stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(f) > t for f in _inputs())


def _compile(src: str, extra: list[str], verbose: bool, out_dir: str = OUT_DIR) -> str:
    obj = os.path.join(out_dir, "obj", src + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cpp"):
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, "-c", path, "-o", obj]
    else:
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, defines: tuple = (), out_dir: str = OUT_DIR) -> str:
    """Compile and link the library if any input changed; return its path.
    `defines` (e.g. ("GMVS_MIN_BLOCKS=3",)) and `out_dir` build a variant
    library elsewhere, for tuning experiments."""
    lib_path = os.path.join(out_dir, "libgmvs_gb300.so")
    if not force and not defines and out_dir == OUT_DIR and not is_stale():
        return LIB_PATH
    os.makedirs(os.path.join(out_dir, "obj"), exist_ok=True)
    extra_d = ["-D" + d for d in defines]
    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1] + extra_d, verbose, out_dir), SOURCES.items()))
    tmp = lib_path + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking libgmvs_gb300.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
