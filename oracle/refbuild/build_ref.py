"""Compile the reference's own GPU kernels to cubins for sm_103a, written to
oracle/_ref/.  Test and measurement infrastructure only: the cubins are
launched by oracle/refbuild/ref_harness.py to produce golden vectors and to
time the reference's plain per-view GPU path.

  ref_patch_match.cubin  gmvs/src/patch_match.cu      (module B, geometric pass)
  ref_fusion.cubin       gmvs/src/fusion.cu           (module B, fusion)
  ref_planar.cubin       gmvs/lib/src/patch_match_kernel.cu
                                                      (module A, random and
                                                       planar-prior passes)
  ref_planar_ieee.cubin, ref_patch_match_ieee.cubin, ref_fusion_ieee.cubin
                         the same sources without fast math and without
                         fused multiply-adds (-fmad=false): the reference's
                         own operation chains in IEEE fp32, against which
                         the oracle's restatements of those chains are pinned

The sources are read where they lie in the reference checkout: the folder
named by GMVS_REFERENCE, or else a `reference` folder beside this
repository's root.  The flags are the reference's own: module B as torch's
CUDAExtension builds it (no fast math), module A as its CMakeLists.txt
(-O3 --use_fast_math --maxrregcount=128), retargeted to sm_103a.

Two include shims stand in for headers this toolchain lacks
(oracle/refbuild/shim): cuda_texture_types.h, which CUDA 13 no longer ships,
and a declaration-only set of opencv2 headers.  Module A's header declares
cv::Mat, cv::Point, cv::Rect, cv::Mat_ and cv::Vec3b in PlanarInit's members
and signatures, but neither the kernels nor the launcher in
patch_match_kernel.cu touch an OpenCV object, so empty types suffice and no
OpenCV code is compiled.
"""

import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("GMVS_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference")

# (cubin name, source under the checkout, include folders under the checkout, extra flags)
UNITS = [
    ("patch_match", "gmvs/src/patch_match.cu", ["gmvs/include"],
     ["-DTORCH_EXTENSION_NAME=gmvs_src_ref", "-D__CUDA_NO_HALF_OPERATORS__"]),
    ("fusion", "gmvs/src/fusion.cu", ["gmvs/include"],
     ["-DTORCH_EXTENSION_NAME=gmvs_src_ref", "-D__CUDA_NO_HALF_OPERATORS__"]),
    ("planar", "gmvs/lib/src/patch_match_kernel.cu", ["gmvs/lib/include"],
     ["--use_fast_math", "--maxrregcount=128"]),
    ("planar_ieee", "gmvs/lib/src/patch_match_kernel.cu", ["gmvs/lib/include"],
     ["--maxrregcount=128", "-fmad=false", "-prec-div=true", "-prec-sqrt=true"]),
    ("patch_match_ieee", "gmvs/src/patch_match.cu", ["gmvs/include"],
     ["-DTORCH_EXTENSION_NAME=gmvs_src_ref", "-D__CUDA_NO_HALF_OPERATORS__", "-fmad=false"]),
    ("fusion_ieee", "gmvs/src/fusion.cu", ["gmvs/include"],
     ["-DTORCH_EXTENSION_NAME=gmvs_src_ref", "-D__CUDA_NO_HALF_OPERATORS__", "-fmad=false"]),
]


def available() -> bool:
    """True where the reference sources are present (not on the GPU machine)."""
    return all(os.path.isfile(os.path.join(REF, src)) for _, src, _, _ in UNITS)


def cubin(name: str) -> str:
    return os.path.join(OUT, f"ref_{name}.cubin")


def _torch_includes() -> list:
    import torch.utils.cpp_extension as ce

    return ce.include_paths() + [sysconfig.get_paths()["include"]]


def build(force: bool = False) -> list:
    if not available():
        raise RuntimeError(f"reference sources not found under {REF} (set GMVS_REFERENCE)")
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for name, src, incs, flags in UNITS:
        path = os.path.join(REF, src)
        out = cubin(name)
        if not force and os.path.exists(out) and os.path.getmtime(out) > os.path.getmtime(path):
            continue
        inc = [os.path.join(HERE, "shim")] + [os.path.join(REF, i) for i in incs]
        if not name.startswith("planar"):
            inc += _torch_includes()
        cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", *flags,
               "-diag-suppress", "550,177", *[f"-I{i}" for i in inc], path, "-o", out]
        jobs.append((name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)))
    for name, proc in jobs:
        _, err = proc.communicate()
        if proc.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{err[-4000:]}")
    return [cubin(n) for n, _, _, _ in UNITS]


if __name__ == "__main__":
    print("\n".join(build(force="--force" in sys.argv)))
    sys.exit(0)
