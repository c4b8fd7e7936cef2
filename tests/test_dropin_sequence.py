"""The drop-in modules driven by the reference's own call sequences, on the
reference's file layout: planar_init.initialization's default branch
(gmvs/planar_init.py:113-190) on gmvs_gb300.planar_initer.PlanarInit,
consistency.run_patch_match for two geometric iterations
(gmvs/consistency.py:27-138, launch.py:157-164) and consistency.run_fusion
(consistency.py:141-211) on gmvs_gb300.src — each step through the files the
reference writes and reads.  The fused maps equal ScenePipeline's (run with
the mirrors' random streams) bit for bit; the normals up to the
renormalisation's summation order (numpy here, torch there)."""

import os

import numpy as np
import pytest

from gmvs_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _read_camera(path):
    # the camera file layout of colmap2mvs.py:531-549, read as consistency.py:13-24 reads it
    tok = open(path).read().split()
    E = np.array([float(x) for x in tok[1:17]]).reshape(4, 4)
    return [float(x) for x in tok[18:27]], E[:3, :3].reshape(9).tolist(), E[:3, 3].tolist(), \
        (float(tok[27]), float(tok[30]))


def _initialization(root, out, ref, src, verbose=False):
    """planar_init.initialization, default branch (planar_init.py:113-190)."""
    from gmvs_gb300.planar_initer import PlanarInit

    save_dir = os.path.join(out, f"{ref:04}")
    os.makedirs(save_dir, exist_ok=True)
    initer = PlanarInit(verbose)
    initer.add_image(os.path.join(root, "images", f"{ref:04}.jpg"))
    height, width = initer.get_image(0).shape
    K, R, t, (dmin, dmax) = _read_camera(os.path.join(root, "cams", f"{ref:04}_cam.txt"))
    initer.add_camera(K, R, t, height, width, dmin, dmax)
    for s in src:
        initer.add_image(os.path.join(root, "images", f"{s:04}.jpg"))
        K, R, t, (dmin, dmax) = _read_camera(os.path.join(root, "cams", f"{s:04}_cam.txt"))
        initer.add_camera(K, R, t, height, width, dmin, dmax)
    initer.add_superpixel(np.load(os.path.join(root, "superpixels", f"{ref:04d}.npy")))
    initer.params.depth_min = initer.get_camera(0).depth_min * 0.6
    initer.params.depth_max = initer.get_camera(0).depth_max * 1.2
    initer.params.num_images = initer.get_num_images()
    initer.cuda_space_init()
    initer.run_patch_match()
    depth = np.zeros([height, width], dtype=np.float32)
    normal = np.zeros([height, width, 3], dtype=np.float32)
    cost = np.zeros([height, width], dtype=np.float32)
    initer.export_plane(depth, normal, cost)
    first = (depth.copy(), normal.copy(), cost.copy())
    initer.params.planar_prior = True
    initer.params.superpixel_filter = True
    tri_path = os.path.join(save_dir, "triangulation.png")
    initer.triangulation(depth, tri_path)
    initer.cuda_planar_prior_init()
    initer.run_patch_match()
    initer.export_plane(depth, normal, cost)  # in place, into the same arrays
    initer.jump_patch_match()
    np.save(os.path.join(save_dir, "depth.npy"), depth)
    np.save(os.path.join(save_dir, "normal.npy"), normal)
    np.save(os.path.join(save_dir, "cost.npy"), cost)
    return initer, first, tri_path


def _geometric(root, out, problems, first_stage, rng):
    """consistency.run_patch_match (consistency.py:27-138)."""
    import torch

    from gmvs_gb300 import imageio
    from gmvs_gb300 import src as _C

    cpp_problems, cameras, grays, depths, normals, costs = [], [], [], [], [], []
    suffix = "" if first_stage else "_geom"
    for ref, src in problems:
        d = os.path.join(out, f"{ref:04}")
        grays.append(torch.from_numpy(imageio.imread_gray(os.path.join(root, "images", f"{ref:04}.jpg"))).float())
        depth = torch.from_numpy(np.load(os.path.join(d, f"depth{suffix}.npy")))
        depths.append(depth)
        normals.append(torch.from_numpy(np.load(os.path.join(d, f"normal{suffix}.npy"))))
        costs.append(torch.from_numpy(np.load(os.path.join(d, f"cost{suffix}.npy"))))
        height, width = depth.shape
        K, R, t, (dmin, dmax) = _read_camera(os.path.join(root, "cams", f"{ref:04}_cam.txt"))
        cameras.append(_C.load_camera(K, R, t, height, width, dmin, dmax))
        cpp_problems.append(_C.load_problem(ref, src))
    pm = _C.PatchMatcher()
    pm.params.geom_consistency = True
    pm.params.max_iterations = 2
    depths, normals, costs = torch.stack(depths), torch.stack(normals), torch.stack(costs)
    pm.add_samples(cpp_problems, cameras, torch.stack(grays), depths, normals, costs)
    out_d, out_n = torch.zeros_like(depths), torch.zeros_like(normals)
    order = np.arange(len(problems))
    rng.shuffle(order)
    for i in order:
        depth, normal, cost = pm.run_patch_match(int(i), False)
        d = os.path.join(out, f"{problems[i][0]:04}")
        np.save(os.path.join(d, "depth_geom.npy"), depth.cpu().numpy())
        np.save(os.path.join(d, "normal_geom.npy"), normal.cpu().numpy())
        np.save(os.path.join(d, "cost_geom.npy"), cost.cpu().numpy())
        out_d[i], out_n[i] = depth, normal
    return out_d, out_n


def _fusion(root, depths, normals, problems, gc, out_dir):
    """consistency.run_fusion (consistency.py:141-211)."""
    import torch

    from gmvs_gb300 import src as _C

    num, height, width = depths.shape
    cpp_problems, cameras = [], []
    for ref, src in problems:
        K, R, t, (dmin, dmax) = _read_camera(os.path.join(root, "cams", f"{ref:04}_cam.txt"))
        cameras.append(_C.load_camera(K, R, t, height, width, dmin, dmax))
        cpp_problems.append(_C.load_problem(ref, src))
    masks = torch.zeros([num, height, width]).bool().cuda()
    fuser = _C.Fuser()
    fuser.load_samples(cpp_problems, cameras, depths, normals, masks)
    os.makedirs(out_dir, exist_ok=True)
    fused = []
    for i in range(num):
        proj_depth, proj_normal = fuser.run_fusion(i, gc)
        depth = proj_depth.cpu().numpy()
        normal = proj_normal.cpu().numpy()
        nn = np.linalg.norm(normal, axis=-1, ord=2, keepdims=True)
        normal /= np.where(nn > 0.5, nn, 1.0)
        dn = np.concatenate([depth[..., None], normal], axis=-1).astype(np.float32)
        np.save(os.path.join(out_dir, f"{problems[i][0]:04d}.npy"), dn)
        fused.append(dn)
    return np.stack(fused), masks.cpu().numpy()


def test_reference_call_sequences_equal_pipeline(gmvs_lib, tmp_path, cuda):
    import torch

    from gmvs_gb300.pipeline import ScenePipeline, scene_inputs_from_synthetic

    sc = synthetic.small_scene(0)  # the plain small configuration: 5 views at 320x256
    root, out = str(tmp_path / "scene"), str(tmp_path / "mvs")
    synthetic.write_scene(sc, root)
    problems = [(r, list(s)) for r, s in sc.problems]
    assert [r for r, _ in problems] == list(range(sc.num_views))

    firsts = {}
    for ref, src in problems:
        initer, first, tri = _initialization(root, out, ref, src)
        firsts[ref] = first
        assert os.path.getsize(tri) > 0
    # every public method of the module-A mirror was exercised above, plus these
    assert initer.get_num_images() == 5 and initer.get_camera(0).width == 320
    saved = np.load(os.path.join(out, f"{problems[-1][0]:04}", "cost.npy")).reshape(-1)
    for i in (7, 4000, 81919):  # NaN where no source view was sampled, as in the reference
        assert np.array_equal(np.float32(initer.get_cost(i)), saved[i], equal_nan=True)
    rng = np.random.default_rng(0)
    _geometric(root, out, problems, True, rng)
    depths, normals = _geometric(root, out, problems, False, rng)
    fused, masks = _fusion(root, depths, normals, problems, 3, os.path.join(out, "depth_normal"))

    pipe = ScenePipeline(scene_inputs_from_synthetic(sc, cuda), geom_iters=2, geom_consistent=3, mode="batched",
                         mirror_streams=True)
    fd, fn = pipe.run()
    torch.cuda.synchronize()
    assert np.array_equal(fused[..., 0], fd.cpu().numpy())
    assert np.abs(fused[..., 1:] - fn.cpu().numpy()).max() <= 1e-6
    assert np.array_equal(masks, pipe.masks.cpu().numpy())
    assert (fused[..., 0] > 0).mean() > 0.1
    # the intermediate files: the first (random) pass and the prior pass of every view
    first = ScenePipeline(scene_inputs_from_synthetic(sc, cuda), mode="batched", mirror_streams=True)
    first.random_pass()
    torch.cuda.synchronize()
    for ref, (d, n, c) in firsts.items():
        assert np.array_equal(d, first.depth[0][ref].cpu().numpy())
        assert np.array_equal(n, first.normal[0][ref].cpu().numpy())
        assert np.array_equal(c, first.cost[0][ref].cpu().numpy(), equal_nan=True)  # NaN: no view sampled
    first._prior(0)
    first.prior_pass()
    torch.cuda.synchronize()
    for ref, _ in problems:
        assert np.array_equal(np.load(os.path.join(out, f"{ref:04}", "depth.npy")), first.depth[1][ref].cpu().numpy())
