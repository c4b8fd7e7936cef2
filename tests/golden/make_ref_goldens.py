"""Generate the reference golden vectors in tests/golden/ref_goldens.npz.

Runs the reference's own module-B kernels (compiled from the reference
sources by oracle/refbuild/build_ref.py into oracle/_ref/*.cubin, launched by
oracle/refbuild/ref_harness.py) on a GPU, on the seeded small scene at
160x128:

  ncc_view{j}   cost of PatchMatcher::run_patch_match with one source view j
                and max_iterations = 0: the bilateral NCC of the given
                hypotheses (initialization, patch_match.cu:1046-1082)
  ncc_all       the same with all four sources: the initial top-k cost
  geom_*        depth/normal/cost of a 2-iteration geometric pass from noisy
                ground-truth inputs (statistical comparison: curand stream)
  fuse_*        Fuser::run_fusion over the five views in order (gc = 3) from
                noisy ground-truth maps: per-view outputs and final masks

Usage (on a machine with a GPU and the cubins):
    python tests/golden/make_ref_goldens.py OUT.npz
The inputs are regenerated from the seeds, so only outputs are stored.
"""

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

H, W = 128, 160


def golden_inputs():
    """Scene, hypotheses and noisy maps shared by the generator and the tests."""
    from gmvs_gb300 import synthetic
    from scenes import gt_planes, random_planes

    sc = synthetic.small_scene(0, H=H, W=W)
    rng = np.random.default_rng(11)
    ref = 0
    gt = gt_planes(sc, ref)
    rp = random_planes(sc, ref, rng, 0.3, 6.0)
    pick = rng.random((H, W))[..., None] < 0.5
    planes = np.where(pick, gt, rp).astype(np.float32)
    # the same hypotheses as module B's (depth, world normal) inputs
    K, R = sc.K[ref], sc.R[ref]
    ys, xs = np.mgrid[0:H, 0:W]
    n_c = planes[..., :3].astype(np.float64)
    denom = (xs - K[0, 2]) / K[0, 0] * n_c[..., 0] + (ys - K[1, 2]) / K[1, 1] * n_c[..., 1] + n_c[..., 2]
    depth = (-planes[..., 3] / denom).astype(np.float32)
    n_w = (n_c @ R).astype(np.float32)
    hyp_depths = sc.depths.copy()
    hyp_normals = sc.normals.copy()
    hyp_depths[ref] = depth
    hyp_normals[ref] = n_w
    rng2 = np.random.default_rng(12)
    noisy_d = (sc.depths * (1.0 + rng2.normal(0, 0.005, sc.depths.shape))).astype(np.float32)
    nn = sc.normals + rng2.normal(0, 0.02, sc.normals.shape)
    noisy_n = (nn / np.linalg.norm(nn, axis=-1, keepdims=True)).astype(np.float32)
    return sc, hyp_depths, hyp_normals, noisy_d, noisy_n


def main(out_path: str) -> None:
    from gmvs_gb300 import synthetic
    from oracle.refbuild import ref_harness as rh

    sc, hyp_d, hyp_n, noisy_d, noisy_n = golden_inputs()
    cams = [rh.camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]
    imgs = sc.images.astype(np.float32)
    drv = rh.Driver()
    out = {}
    for j in (1, 2, 3, 4):
        _, _, c = rh.run_patch_match(drv, cams, 0, [j], imgs, hyp_d, hyp_n, 0)
        out[f"ncc_view{j}"] = c
    d, n, c = rh.run_patch_match(drv, cams, 0, [1, 2, 3, 4], imgs, hyp_d, hyp_n, 0)
    out["ncc_all"] = c
    d, n, c = rh.run_patch_match(drv, cams, 0, [1, 2, 3, 4], imgs, noisy_d, noisy_n, 2)
    out["geom_depth"], out["geom_normal"], out["geom_cost"] = d, n, c
    outs, masks = rh.run_fusion(drv, cams, sc.problems, noisy_d, noisy_n, 3)
    for k, (fd, fn) in enumerate(outs):
        out[f"fuse_depth{k}"] = fd
        out[f"fuse_normal{k}"] = fn
    out["fuse_masks"] = masks
    np.savez_compressed(out_path, **out)
    print(f"wrote {out_path}: " + ", ".join(f"{k}{list(v.shape)}" for k, v in out.items()))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(__file__), "ref_goldens.npz"))
