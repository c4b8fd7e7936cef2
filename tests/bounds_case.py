"""Runs a fixed set of passes with whichever library GMVS_GB300_LIB names and
saves their outputs (and the library's bounds-check violation bits) to the
.npz given as argv[1].  Used by test_bounds_check.py to run the
bounds-checked build in a process of its own."""

import sys

import numpy as np
import torch

from gmvs_gb300 import _abi, engine, synthetic
from scenes import gpu_view


def cases(cuda):
    out = {}
    for name, (H, W, seed) in {"std": (96, 128, 0), "ragged": (67, 93, 1)}.items():
        sc = synthetic.small_scene(seed, H=H, W=W)
        ref, src = sc.problems[0]
        ids = [ref] + list(src)
        rng = np.random.default_rng(seed)
        d = (sc.depths * (1.0 + rng.normal(0, 0.005, sc.depths.shape))).astype(np.float32)
        n = sc.normals + rng.normal(0, 0.02, sc.normals.shape)
        n = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
        runs = {
            "tex": dict(sampler=_abi.SAMPLER_TEX, max_iterations=2),
            "tex_split": dict(sampler=_abi.SAMPLER_TEX, max_iterations=2, split_sweep=1),
            "tex_split3": dict(sampler=_abi.SAMPLER_TEX, max_iterations=2, split_sweep=2),
            "f32": dict(sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_F32, max_iterations=2),
            "generic": dict(sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_QUAD_F16, patch_size=7,
                            radius_increment=1, max_iterations=1),
            "geom_split": dict(sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_QUAD_F16,
                               init_kind=_abi.INIT_DEPTH_NORMAL, sweep_kind=_abi.SWEEP_GEOM, max_iterations=2,
                               pass_index=2, split_sweep=1),
            "geom_split3": dict(sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_QUAD_F16,
                                init_kind=_abi.INIT_DEPTH_NORMAL, sweep_kind=_abi.SWEEP_GEOM, max_iterations=2,
                                pass_index=2, split_sweep=2),
        }
        for key, kw in runs.items():
            extra = {}
            if kw.get("sweep_kind") == _abi.SWEEP_GEOM:
                extra = dict(depths=[torch.from_numpy(d[i]).to(cuda) for i in ids],
                             ref_normal=torch.from_numpy(n[ref]).to(cuda))
            v = gpu_view(sc, ids, cuda, 0.3, 6.0, **extra)
            v.allocate_outputs(with_planes=True)
            engine.run_passes([v], engine.params_struct(**kw), engine.Workspace())
            out[f"{name}_{key}_depth"] = v.out_depth.cpu().numpy()
            out[f"{name}_{key}_cost"] = v.out_cost.cpu().numpy()
    return out


if __name__ == "__main__":
    cuda = torch.device("cuda", 0)
    res = cases(cuda)
    torch.cuda.synchronize()
    res["violations"] = np.array(_abi.lib().gmvs_bounds_violations(1))
    np.savez(sys.argv[1], **res)
