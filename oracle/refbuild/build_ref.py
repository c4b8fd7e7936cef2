"""Compile the reference's own module-B kernels (gmvs/src/patch_match.cu and
gmvs/src/fusion.cu, read where they lie under /root/reference) to cubins for
sm_103a, written to oracle/_ref/.  Test infrastructure only: the cubins are
launched by oracle/refbuild/ref_harness.py to produce golden vectors.

The only change to the reference build is an include shim for
cuda_texture_types.h, which CUDA 13 no longer ships.  Module A
(gmvs/lib/src/*) needs OpenCV and is not buildable here.
"""

import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
REF = os.environ.get("GMVS_REFERENCE", "/root/reference")


def available() -> bool:
    """True where the reference sources are present (not on the GPU machine)."""
    return os.path.isdir(os.path.join(REF, "gmvs", "src"))


def build(force: bool = False) -> list:
    import torch.utils.cpp_extension as ce

    if not available():
        raise RuntimeError(f"reference sources not found under {REF}")
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(REF, "gmvs", "src", f"{n}.cu") for n in ("patch_match", "fusion")]
    outs = [os.path.join(OUT, f"ref_{n}.cubin") for n in ("patch_match", "fusion")]
    if not force and all(os.path.exists(o) for o in outs) and \
            min(os.path.getmtime(o) for o in outs) > max(os.path.getmtime(s) for s in srcs):
        return outs
    incs = [os.path.join(HERE, "shim"), os.path.join(REF, "gmvs", "include")] + ce.include_paths() + \
        [sysconfig.get_paths()["include"]]
    outs = []
    for name in ("patch_match", "fusion"):
        out = os.path.join(OUT, f"ref_{name}.cubin")
        cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
               "-DTORCH_EXTENSION_NAME=gmvs_src_ref", "-D__CUDA_NO_HALF_OPERATORS__",
               *[f"-I{i}" for i in incs], os.path.join(REF, "gmvs", "src", f"{name}.cu"), "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}.cu:\n{r.stderr[-4000:]}")
        outs.append(out)
    return outs


if __name__ == "__main__":
    print("\n".join(build()))
    sys.exit(0)
