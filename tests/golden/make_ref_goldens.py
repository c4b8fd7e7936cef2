"""Generate the reference golden vectors under tests/golden/.

Runs the reference's own kernels (compiled from the reference sources by
oracle/refbuild/build_ref.py into oracle/_ref/*.cubin, launched by
oracle/refbuild/ref_harness.py) on a GPU.  Inputs are regenerated from seeds
by the tests, so only outputs (and the prior that the reference's second
module-A pass was given) are stored.

ref_goldens.npz (module B, seeded small scene at 160x128, 4 sources):
  ncc_view{j}   cost of PatchMatcher::run_patch_match with one source view j
                and max_iterations = 0: the bilateral NCC of the given
                hypotheses (initialization, patch_match.cu:1046-1082)
  ncc_all       the same with all four sources: the initial top-k cost
  geom_*        depth/normal/cost of a 2-iteration geometric pass from noisy
                ground-truth inputs (statistical comparison: curand stream)
  fuse_*        Fuser::run_fusion over the five views in order (gc = 3) from
                noisy ground-truth maps: per-view outputs and final masks

  geom_rerun_*  the same geometric pass run again (float16): the reference
                is not reproducible run to run (it reads same-colour
                neighbours while they are rewritten), so this is its own
                agreement ceiling

ref_goldens_planar.npz (module A, PlanarInit's kernels, the 160x128 scene
"s" and the 320x256 scene "c1" of the plain small configuration):
  {s}_ncc_view{j}, {s}_ncc_all, {s}_ncc_all_views
                the texture-path NCC of given hypotheses: RandomInitialization's
                planar-prior branch with every plane mask 0 re-evaluates the
                multi-view initial cost of the planes it is given
                (patch_match_kernel.cu:1545-1558), max_iterations = 0
  {s}_ieee_ncc_view{j}, {s}_ieee_ncc_all
                the same from the module built without fast math and without
                fused multiply-adds (ref_planar_ieee.cubin)
  {s}_rand_planes, {s}_rand_cost
                the random pass (init, 3 iterations, depth/normal, filter):
                exported (world normal, depth) and cost
  {s}_rand_rerun_planes
                the random pass run again (float16): the reference's own
                run-to-run agreement
  {s}_prior_table, {s}_prior_mask
                the prior given to the second pass: the oracle's triangulation
                of the reference's first-pass depth and cost (planes per
                triangle, triangle id + 1 per pixel)
  {s}_prior_planes, {s}_prior_cost
                the planar-prior pass that follows on the device-resident state
                (float16 for c1)

ref_goldens_cfg1.npz (module B on the 320x256 scene): c1_ncc_all,
  c1_geom_{depth,normal,cost}, c1_fuse_depth{k}, c1_fuse_masks; and the
  same NCC and fusion from module B built without fused multiply-adds
  (ref_patch_match_ieee / ref_fusion_ieee): c1_ieee_ncc_all,
  c1_ieee_fuse_depth{k}, c1_ieee_fuse_masks.

ref_goldens_room.npz (reference view 0 of the 20-view 1600x1200 room scene
with its 10 sources; per-pixel arrays as 8 crops of 96x96, see ROOM_CROPS):
  room_a_ncc_all, room_b_ncc_all   NCC of given hypotheses (modules A and B)
  room_b_geom_*                    2-iteration geometric pass (float16 crops)
  room_a_rand_*                    module-A random pass (float16 crops)
  room_*_acc                       whole-view fraction of pixels within 0.5 %
                                   of the ground-truth depth
  room_fuse_*                      fusion of view 0 from noisy maps: crops of
                                   the fused depth, the fused-pixel count and
                                   SHA-256 digests of the fused-pixel map and
                                   of the source masks
  room_ieee_fuse_*                 the same from module B's fusion built
                                   without fused multiply-adds
  room_images_sha                  digest of the rendered images (input check)

Usage (on a machine with a GPU and the cubins):
    python tests/golden/make_ref_goldens.py [small|planar|cfg1|room|all] [OUTDIR]
"""

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

H, W = 128, 160
ROOM_CROPS = [(y, x) for y in (96, 552, 1008) for x in (160, 760, 1360)][:8]
CROP = 96


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def crops(a: np.ndarray) -> np.ndarray:
    """The ROOM_CROPS tiles of a [H, W, ...] array, stacked [8, 96, 96, ...]."""
    return np.stack([a[y:y + CROP, x:x + CROP] for y, x in ROOM_CROPS])


def mixed_hypotheses(sc, ref: int, seed: int):
    """Half ground-truth, half random camera-frame planes of view `ref`, plus
    the same hypotheses as (depth, camera-frame normal) and (depth, world
    normal) maps."""
    from scenes import gt_planes, random_planes

    Hs, Ws = sc.hw
    rng = np.random.default_rng(seed)
    gt = gt_planes(sc, ref)
    rp = random_planes(sc, ref, rng, 0.3, max(6.0, sc.depth_range[1]))
    pick = rng.random((Hs, Ws))[..., None] < 0.5
    planes = np.where(pick, gt, rp).astype(np.float32)
    K, R = sc.K[ref], sc.R[ref]
    ys, xs = np.mgrid[0:Hs, 0:Ws]
    n_c = planes[..., :3].astype(np.float64)
    denom = (xs - K[0, 2]) / K[0, 0] * n_c[..., 0] + (ys - K[1, 2]) / K[1, 1] * n_c[..., 1] + n_c[..., 2]
    depth = (-planes[..., 3] / denom).astype(np.float32)
    n_w = (n_c @ R).astype(np.float32)
    return planes, depth, planes[..., :3].copy(), n_w


def noisy_maps(sc, seed: int):
    """Ground-truth depth and normal maps with 0.5 % depth noise and 0.02 normal noise."""
    rng2 = np.random.default_rng(seed)
    noisy_d = (sc.depths * (1.0 + rng2.normal(0, 0.005, sc.depths.shape))).astype(np.float32)
    nn = sc.normals + rng2.normal(0, 0.02, sc.normals.shape)
    noisy_n = (nn / np.linalg.norm(nn, axis=-1, keepdims=True)).astype(np.float32)
    return noisy_d, noisy_n


def golden_inputs():
    """Scene, hypotheses and noisy maps of ref_goldens.npz."""
    from gmvs_gb300 import synthetic

    sc = synthetic.small_scene(0, H=H, W=W)
    _, depth, _, n_w = mixed_hypotheses(sc, 0, 11)
    hyp_depths = sc.depths.copy()
    hyp_normals = sc.normals.copy()
    hyp_depths[0] = depth
    hyp_normals[0] = n_w
    noisy_d, noisy_n = noisy_maps(sc, 12)
    return sc, hyp_depths, hyp_normals, noisy_d, noisy_n


def planar_scenes():
    """(tag, scene) of the module-A goldens: 160x128 and the 320x256 plain small configuration."""
    from gmvs_gb300 import synthetic

    return [("s", synthetic.small_scene(0, H=H, W=W)), ("c1", synthetic.small_scene(0))]


def prior_from(cam_arg, depth, cost, superpixel, dmin, dmax):
    """The oracle's triangulation prior as (table [T, 4], mask uint16 [H, W])."""
    import oracle

    planes, masks, _ = oracle.build_prior(cam_arg, depth, cost, superpixel, True, dmin, dmax)
    T = int(masks.max())
    table = np.zeros((T, 4), np.float32)
    ys, xs = np.nonzero(masks)
    table[masks[ys, xs] - 1] = planes[ys, xs]
    assert T < 65536
    return table, masks.astype(np.uint16)


def prior_planes(table: np.ndarray, mask: np.ndarray) -> np.ndarray:
    out = np.zeros(mask.shape + (4,), np.float32)
    m = mask > 0
    out[m] = table[mask[m].astype(np.int64) - 1]
    return out


def _planar_cams(rh, sc, ids):
    from gmvs_gb300 import synthetic

    return [rh.camera(*synthetic.camera_args(sc, i)) for i in ids]


def planar_ncc(drv, rh, sc, ids, depth, n_c, module="planar"):
    """Module A's initial cost of given (camera-frame normal, depth) hypotheses."""
    imgs = sc.images[ids].astype(np.float32)
    run = rh.PlanarInitRef(drv, _planar_cams(rh, sc, ids), imgs, module)
    try:
        run.set_state(np.concatenate([n_c, depth[..., None]], -1), np.zeros(depth.shape, np.float32))
        run.run_patch_match(max_iterations=0, planar_prior=True)
        return run.costs.copy(), run.selected_views()
    finally:
        run.close()


def planar_passes(drv, rh, sc, ids):
    """Random pass, the oracle's prior of its result, then the prior pass."""
    from gmvs_gb300 import synthetic

    imgs = sc.images[ids].astype(np.float32)
    run = rh.PlanarInitRef(drv, _planar_cams(rh, sc, ids), imgs)
    try:
        run.run_patch_match(3, planar_prior=False)
        rand_planes, rand_cost = run.planes.copy(), run.costs.copy()
        table, mask = prior_from(synthetic.camera_args(sc, ids[0]), rand_planes[..., 3], rand_cost,
                                 sc.superpixels[ids[0]], run.params.depth_min, run.params.depth_max)
        run.planar_prior_init(prior_planes(table, mask), mask.astype(np.uint32))
        run.run_patch_match(3, planar_prior=True)
        return rand_planes, rand_cost, table, mask, run.planes.copy(), run.costs.copy()
    finally:
        run.close()


def make_small(drv, rh, out_dir):
    from gmvs_gb300 import synthetic

    sc, hyp_d, hyp_n, noisy_d, noisy_n = golden_inputs()
    cams = [rh.camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]
    imgs = sc.images.astype(np.float32)
    out = {}
    for j in (1, 2, 3, 4):
        _, _, c = rh.run_patch_match(drv, cams, 0, [j], imgs, hyp_d, hyp_n, 0)
        out[f"ncc_view{j}"] = c
    d, n, c = rh.run_patch_match(drv, cams, 0, [1, 2, 3, 4], imgs, hyp_d, hyp_n, 0)
    out["ncc_all"] = c
    d, n, c = rh.run_patch_match(drv, cams, 0, [1, 2, 3, 4], imgs, noisy_d, noisy_n, 2)
    out["geom_depth"], out["geom_normal"], out["geom_cost"] = d, n, c
    d, n, _ = rh.run_patch_match(drv, cams, 0, [1, 2, 3, 4], imgs, noisy_d, noisy_n, 2)
    out["geom_rerun_depth"], out["geom_rerun_normal"] = d.astype(np.float16), n.astype(np.float16)
    outs, masks = rh.run_fusion(drv, cams, sc.problems, noisy_d, noisy_n, 3)
    for k, (fd, fn) in enumerate(outs):
        out[f"fuse_depth{k}"] = fd
        out[f"fuse_normal{k}"] = fn
    out["fuse_masks"] = masks
    return os.path.join(out_dir, "ref_goldens.npz"), out


def make_planar(drv, rh, out_dir):
    out = {}
    for tag, sc in planar_scenes():
        ids = [0, 1, 2, 3, 4]
        _, depth, n_c, _ = mixed_hypotheses(sc, 0, 11)
        for j in (1, 2, 3, 4):
            out[f"{tag}_ncc_view{j}"], _ = planar_ncc(drv, rh, sc, [0, j], depth, n_c)
            out[f"{tag}_ieee_ncc_view{j}"], _ = planar_ncc(drv, rh, sc, [0, j], depth, n_c, "planar_ieee")
        out[f"{tag}_ncc_all"], out[f"{tag}_ncc_all_views"] = planar_ncc(drv, rh, sc, ids, depth, n_c)
        out[f"{tag}_ieee_ncc_all"], _ = planar_ncc(drv, rh, sc, ids, depth, n_c, "planar_ieee")
        rp, rc, table, mask, pp, pc = planar_passes(drv, rh, sc, ids)
        out[f"{tag}_rand_planes"], out[f"{tag}_rand_cost"] = rp, rc
        out[f"{tag}_rand_rerun_planes"] = planar_passes(drv, rh, sc, ids)[0].astype(np.float16)
        out[f"{tag}_prior_table"], out[f"{tag}_prior_mask"] = table, mask
        if tag == "c1":
            pp, pc = pp.astype(np.float16), pc.astype(np.float16)
        out[f"{tag}_prior_planes"], out[f"{tag}_prior_cost"] = pp, pc
    return os.path.join(out_dir, "ref_goldens_planar.npz"), out


def cfg1_inputs():
    from gmvs_gb300 import synthetic

    sc = synthetic.small_scene(0)
    _, depth, _, n_w = mixed_hypotheses(sc, 0, 21)
    hyp_d, hyp_n = sc.depths.copy(), sc.normals.copy()
    hyp_d[0], hyp_n[0] = depth, n_w
    noisy_d, noisy_n = noisy_maps(sc, 22)
    return sc, hyp_d, hyp_n, noisy_d, noisy_n


def make_cfg1(drv, rh, out_dir):
    from gmvs_gb300 import synthetic

    sc, hyp_d, hyp_n, noisy_d, noisy_n = cfg1_inputs()
    cams = [rh.camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]
    imgs = sc.images.astype(np.float32)
    out = {}
    _, _, out["c1_ncc_all"] = rh.run_patch_match(drv, cams, 0, [1, 2, 3, 4], imgs, hyp_d, hyp_n, 0)
    d, n, c = rh.run_patch_match(drv, cams, 0, [1, 2, 3, 4], imgs, noisy_d, noisy_n, 2)
    out["c1_geom_depth"], out["c1_geom_normal"], out["c1_geom_cost"] = d, n, c
    outs, masks = rh.run_fusion(drv, cams, sc.problems, noisy_d, noisy_n, 3)
    for k, (fd, _) in enumerate(outs):
        out[f"c1_fuse_depth{k}"] = fd
    out["c1_fuse_masks"] = masks
    _, _, out["c1_ieee_ncc_all"] = rh.run_patch_match(drv, cams, 0, [1, 2, 3, 4], imgs, hyp_d, hyp_n, 0,
                                                      module="patch_match_ieee")
    outs, masks = rh.run_fusion(drv, cams, sc.problems, noisy_d, noisy_n, 3, module="fusion_ieee")
    for k, (fd, _) in enumerate(outs):
        out[f"c1_ieee_fuse_depth{k}"] = fd
    out["c1_ieee_fuse_masks"] = masks
    return os.path.join(out_dir, "ref_goldens_cfg1.npz"), out


def room_inputs(device=None):
    """The 20-view 1600x1200 room scene, reference view 0 and its sources,
    mixed hypotheses and noisy maps."""
    from gmvs_gb300 import synthetic

    sc = synthetic.room_scene(0, H=1200, W=1600, num_views=20, device=device)
    ref, src = sc.problems[0]
    _, depth, n_c, n_w = mixed_hypotheses(sc, ref, 31)
    noisy_d, noisy_n = noisy_maps(sc, 32)
    return sc, ref, list(src), depth, n_c, n_w, noisy_d, noisy_n


def depth_accuracy(d: np.ndarray, gt: np.ndarray) -> float:
    ok = gt > 0
    return float(np.mean(np.abs(d[ok] - gt[ok]) <= 0.005 * gt[ok]))


def make_room(drv, rh, out_dir):
    import torch

    from gmvs_gb300 import synthetic

    sc, ref, src, depth, n_c, n_w, noisy_d, noisy_n = room_inputs(torch.device("cuda"))
    ids = [ref] + src
    out = {"room_images_sha": sha(sc.images)}
    cams = [rh.camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]
    imgs = sc.images.astype(np.float32)
    hyp_d, hyp_n = sc.depths.copy(), sc.normals.copy()
    hyp_d[ref], hyp_n[ref] = depth, n_w
    _, _, c = rh.run_patch_match(drv, cams, ref, src, imgs, hyp_d, hyp_n, 0)
    out["room_b_ncc_all"] = crops(c)
    c, _ = planar_ncc(drv, rh, sc, ids, depth, n_c)
    out["room_a_ncc_all"] = crops(c)
    gt = sc.depths[ref]
    d, n, c = rh.run_patch_match(drv, cams, ref, src, imgs, noisy_d, noisy_n, 2)
    out["room_b_geom_depth"], out["room_b_geom_normal"] = crops(d).astype(np.float16), crops(n).astype(np.float16)
    out["room_b_geom_acc"] = np.float64(depth_accuracy(d, gt))
    run = rh.PlanarInitRef(drv, _planar_cams(rh, sc, ids), imgs[ids])
    try:
        run.run_patch_match(3, planar_prior=False)
        d, n, c = run.export_plane()
    finally:
        run.close()
    out["room_a_rand_depth"], out["room_a_rand_normal"] = crops(d).astype(np.float16), crops(n).astype(np.float16)
    out["room_a_rand_acc"] = np.float64(depth_accuracy(d, gt))
    outs, masks = rh.run_fusion(drv, cams, [(ref, src)], noisy_d, noisy_n, 3)
    fd = outs[0][0]
    out["room_fuse_depth"] = crops(fd)
    out["room_fuse_count"] = np.int64((fd > 0).sum())
    out["room_fuse_sha"] = sha(fd > 0)
    out["room_fuse_masks_sha"] = sha(masks[ids].astype(bool))
    out["room_fuse_masks_count"] = masks[ids].reshape(len(ids), -1).sum(1).astype(np.int64)
    outs, masks = rh.run_fusion(drv, cams, [(ref, src)], noisy_d, noisy_n, 3, module="fusion_ieee")
    fd = outs[0][0]
    out["room_ieee_fuse_count"] = np.int64((fd > 0).sum())
    out["room_ieee_fuse_sha"] = sha(fd > 0)
    out["room_ieee_fuse_masks_sha"] = sha(masks[ids].astype(bool))
    out["room_ieee_fuse_depth"] = crops(fd)
    return os.path.join(out_dir, "ref_goldens_room.npz"), out


def main(which: str, out_dir: str) -> None:
    from oracle.refbuild import ref_harness as rh

    drv = rh.Driver()
    makers = {"small": make_small, "planar": make_planar, "cfg1": make_cfg1, "room": make_room}
    for name in (makers if which == "all" else [which]):
        path, out = makers[name](drv, rh, out_dir)
        np.savez_compressed(path, **out)
        print(f"wrote {path}: " + ", ".join(f"{k}{list(np.shape(v))}" for k, v in out.items()))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "all",
         sys.argv[2] if len(sys.argv) > 2 else os.path.dirname(os.path.abspath(__file__)))
