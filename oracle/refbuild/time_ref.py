"""Time the reference's own module-B geometric pass (the plain per-view GPU
path of gmvs/src/patch_match.cu, compiled from the reference sources by
build_ref.py) on the room scene used by bench.py, next to gmvs_gb300's
geometric pass on the same inputs.  Measurement infrastructure only.

    python oracle/refbuild/time_ref.py [views]   (needs a GPU and the cubins)
"""

import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def main(nviews: int = 4) -> None:
    import torch

    from gmvs_gb300 import _abi, engine, synthetic
    from oracle.refbuild import ref_harness as rh

    dev = torch.device("cuda")
    sc = synthetic.room_scene(0, H=1200, W=1600, num_views=20, device=dev)
    rng = np.random.default_rng(5)
    d_in = (sc.depths * (1.0 + rng.normal(0, 0.005, sc.depths.shape))).astype(np.float32)
    n = sc.normals + rng.normal(0, 0.02, sc.normals.shape)
    n_in = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    imgs = sc.images.astype(np.float32)
    cams = [rh.camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]
    drv = rh.Driver()
    ref_t = {}
    problems = sc.problems[:nviews]
    rh.run_patch_match(drv, cams, problems[0][0], problems[0][1], imgs, d_in, n_in, 2)  # warm-up
    t0 = time.perf_counter()
    for ref, src in problems:
        rh.run_patch_match(drv, cams, ref, src, imgs, d_in, n_in, 2, timings=ref_t)
    ref_s = time.perf_counter() - t0
    # gmvs_gb300: the same geometric pass through the C ABI, one view per call
    # (plain) and all views in one launch chain (batched)
    gi = torch.from_numpy(imgs).to(dev)
    gd = torch.from_numpy(d_in).to(dev)
    gn = torch.from_numpy(n_in).to(dev)
    gcams = [engine.make_camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]

    def views():
        out = []
        for ref, src in problems:
            ids = [ref] + list(src)
            dmin, dmax = sc.depth_range[0] * 0.6, sc.depth_range[1] * 1.2
            v = engine.ViewInputs(cams=[gcams[i] for i in ids], images=[gi[i] for i in ids], depth_min=dmin,
                                  depth_max=dmax, stream_id=ref, depths=[gd[i] for i in ids], ref_normal=gn[ref])
            v.allocate_outputs()
            out.append(v)
        return out

    p = engine.params_struct(init_kind=_abi.INIT_DEPTH_NORMAL, sweep_kind=_abi.SWEEP_GEOM,
                             sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_AUTO, max_iterations=2, pass_index=2)
    ws = engine.Workspace()
    plain = {}
    for split in (0, 1):
        p.split_sweep = split
        engine.run_passes(views()[:1], p, ws)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for v in views():
            engine.run_passes([v], p, ws)
        torch.cuda.synchronize()
        plain[split] = time.perf_counter() - t0
    batched = {}
    for split in (0, 1):
        p.split_sweep = split
        vs = views()
        plan = engine.Plan(vs, p, engine.Workspace())
        plan.launch()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plan.launch()
        plan.check()
        batched[split] = time.perf_counter() - t0
        plan.close()
    print(json.dumps({"views": len(problems), "size": "1600x1200", "num_src": len(problems[0][1]),
                      "reference_module_b_ms_per_view": 1000 * ref_s / len(problems),
                      "reference_breakdown_ms_per_view": {k: 1000 * v / len(problems) for k, v in ref_t.items()},
                      "gmvs_plain_ms_per_view": 1000 * plain[0] / len(problems),
                      "gmvs_plain_split_ms_per_view": 1000 * plain[1] / len(problems),
                      "gmvs_batched_ms_per_view": 1000 * batched[0] / len(problems),
                      "gmvs_batched_split_ms_per_view": 1000 * batched[1] / len(problems)}))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 4)
