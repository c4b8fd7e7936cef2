"""Drop-in replacement for the reference's pybind module
``gmvs.lib.build.planar_initer`` (gmvs/lib/src/bindings.cpp:12-66): the
random-initialisation and planar-prior PatchMatch passes of one reference
view, the prior construction, and the three CPU segmentation helpers.

Observable differences, all deliberate:
  * images are read with a lossless PNG reader (OpenCV when present);
  * the random stream is Philox4x32-10;
  * cv::Subdiv2D is replaced by an exact-predicate Delaunay triangulation;
  * ``export_plane`` raises on arrays it cannot write in place (the
    reference silently writes into a converted copy);
  * ``params.geom_consistency`` raises: the reference never creates the
    depth textures that branch reads (planar_initer.cu:119-193 vs
    patch_match_kernel.cu:1757).
"""

from __future__ import annotations

import ctypes
from typing import List, Sequence

import numpy as np
import torch

from . import _abi, imageio
from ._abi import check, lib
from .engine import ViewInputs, Workspace, make_camera, make_problem, params_struct, run_passes
from .src import PatchMatchParams

Camera = _abi.gmvs_camera
Problem = _abi.gmvs_problem


def load_camera(K, R, t, height, width, depth_min, depth_max) -> Camera:
    return make_camera(K, R, t, height, width, depth_min, depth_max)


def load_problem(ref_image_id: int, src_image_ids: Sequence[int]) -> Problem:
    return make_problem(ref_image_id, src_image_ids)


def _as_c(a: np.ndarray, dtype, shape, name: str) -> np.ndarray:
    a = np.asarray(a)
    if a.shape != shape:
        raise ValueError(f"{name} has shape {a.shape}, expected {shape}")
    return np.ascontiguousarray(a, dtype=dtype)


def _on_device(a) -> bool:
    return getattr(a, "is_cuda", False) is True


def fusion_planar_mask(seg_ids: np.ndarray, planar_mask: np.ndarray, normals: np.ndarray, rows: int, cols: int,
                       thresh: int = 100, nonplanar_percent: float = 0.75, cos_sim_thresh: float = 0.8,
                       match_ratio_thresh: float = 0.9) -> np.ndarray:
    """fusion_planar_mask (planar_initer.cu:537-632).  numpy arrays run the
    host routine; CUDA tensors run the device kernels and return a CUDA
    tensor (same values)."""
    if _on_device(seg_ids):
        from . import engine

        return engine.fusion_planar_mask(seg_ids, planar_mask, normals, thresh, nonplanar_percent, cos_sim_thresh,
                                         match_ratio_thresh)
    s = _as_c(seg_ids, np.int32, (rows, cols), "seg_ids")
    m = _as_c(planar_mask, np.int32, (rows, cols), "planar_mask")
    n = _as_c(normals, np.float32, (rows, cols, 3), "normals")
    out = np.zeros((rows, cols), np.int32)
    check(lib().gmvs_fusion_planar_mask(s.ctypes.data, m.ctypes.data, n.ctypes.data, rows, cols, thresh,
                                        nonplanar_percent, cos_sim_thresh, match_ratio_thresh, out.ctypes.data))
    return out


def filter_by_var_map(var_map: np.ndarray, segment_ids_map: np.ndarray, var_thresh: float) -> np.ndarray:
    """filter_by_var_map (planar_initer.cu:634-684); CUDA tensors run on the
    device."""
    if _on_device(var_map):
        from . import engine

        return engine.filter_by_var_map(var_map, segment_ids_map, var_thresh)
    v = np.ascontiguousarray(var_map, dtype=np.float32)
    rows, cols = v.shape
    s = _as_c(segment_ids_map, np.int32, (rows, cols), "segment_ids_map")
    out = np.zeros((rows, cols), np.int32)
    check(lib().gmvs_filter_by_var_map(v.ctypes.data, s.ctypes.data, rows, cols, var_thresh, out.ctypes.data))
    return out


def sliding_window_normal(planar_region: np.ndarray, normal: np.ndarray, window_size: int) -> np.ndarray:
    """sliding_window_normal (planar_initer.cu:471-535); CUDA tensors run on
    the device."""
    if _on_device(normal):
        from . import engine

        return engine.sliding_window_normal(planar_region, normal, window_size)
    n = np.ascontiguousarray(normal, dtype=np.float32)
    rows, cols = n.shape[:2]
    r = _as_c(planar_region, np.int32, (rows, cols), "planar_region")
    out = np.zeros((rows, cols, 3), np.float32)
    check(lib().gmvs_sliding_window_normal(r.ctypes.data, n.ctypes.data, rows, cols, window_size, out.ctypes.data))
    return out


def build_planar_prior(camera: Camera, depth: np.ndarray, cost: np.ndarray, superpixel, superpixel_filter: bool,
                       depth_min: float, depth_max: float):
    """Prior planes [H, W, 4] (camera frame), masks [H, W] uint32 and the
    retained triangles [T, 3, 2] (x, y) — PlanarInit::triangulation."""
    d = np.ascontiguousarray(depth, dtype=np.float32)
    H, W = d.shape
    c = _as_c(cost, np.float32, (H, W), "cost")
    sp = None
    if superpixel_filter:
        if superpixel is None:
            raise ValueError("superpixel_filter is set but no superpixel map was added")
        sp = _as_c(superpixel, np.uint8, (H, W), "superpixel")
    planes = np.zeros((H, W, 4), np.float32)
    masks = np.zeros((H, W), np.uint32)
    max_tris = 2 * ((W + 4) // 5) * ((H + 4) // 5) + 16
    tris = np.zeros((max_tris, 3, 2), np.int32)
    count = ctypes.c_int32(0)
    cam = camera
    check(lib().gmvs_build_planar_prior(ctypes.byref(cam), H, W, d.ctypes.data, c.ctypes.data,
                                        None if sp is None else sp.ctypes.data, int(bool(superpixel_filter)),
                                        float(depth_min), float(depth_max), planes.ctypes.data, masks.ctypes.data,
                                        ctypes.byref(count), tris.ctypes.data, max_tris))
    return planes, masks, tris[:min(count.value, max_tris)]


def _draw_triangles(gray: np.ndarray, tris: np.ndarray) -> np.ndarray:
    """vis_triangulation (planar_initer.cu:258-279): red triangle edges."""
    img = np.repeat(np.clip(gray, 0, 255).astype(np.uint8)[..., None], 3, axis=2)
    H, W = gray.shape
    for t in tris:
        for a, b in ((0, 1), (0, 2), (1, 2)):
            x0, y0 = t[a]
            x1, y1 = t[b]
            n = int(max(abs(x1 - x0), abs(y1 - y0))) + 1
            xs = np.rint(np.linspace(x0, x1, n)).astype(int)
            ys = np.rint(np.linspace(y0, y1, n)).astype(int)
            ok = (xs >= 0) & (xs < W) & (ys >= 0) & (ys < H)
            img[ys[ok], xs[ok]] = (255, 0, 0)
    return img


class PlanarInit:
    """PlanarInit (gmvs/lib/include/planar_initer.cuh:74-134)."""

    def __init__(self, verbose: bool = False):
        self.verbose = bool(verbose)
        self.params = PatchMatchParams()
        self._images: List[np.ndarray] = []
        self._cameras: List[Camera] = []
        self._superpixel = None
        self._dev = None
        self._ws = None
        self._last = None       # ViewInputs of the last pass (device outputs)
        self._prior = None      # (planes, masks) host
        self._prior_dev = None
        self._pass = 0

    # images / cameras ------------------------------------------------------
    def add_image(self, image_path: str) -> None:
        self._images.append(imageio.imread_gray(image_path).astype(np.float32))

    def add_superpixel(self, superpixel: np.ndarray) -> None:
        self._superpixel = np.ascontiguousarray(superpixel, dtype=np.uint8)

    def get_image(self, index: int) -> np.ndarray:
        return self._images[index]

    def get_num_images(self) -> int:
        return len(self._images)

    def add_camera(self, K, R, t, height, width, depth_min, depth_max) -> None:
        self._cameras.append(make_camera(K, R, t, height, width, depth_min, depth_max))

    def get_camera(self, index: int) -> Camera:
        return self._cameras[index]

    # device ----------------------------------------------------------------
    def cuda_space_init(self) -> None:
        if len(self._images) < 2:
            raise RuntimeError("PlanarInit needs a reference image and at least one source image")
        H, W = self._images[0].shape
        for i, im in enumerate(self._images):
            if im.shape != (H, W):
                raise RuntimeError(f"image {i} is {im.shape}, the reference image is {(H, W)}")
        self._dev = torch.from_numpy(np.stack(self._images)).cuda()
        self._ws = Workspace()

    def cuda_planar_prior_init(self) -> None:
        if self._prior is None:
            raise RuntimeError("call triangulation() before cuda_planar_prior_init()")
        planes, masks = self._prior
        self._prior_dev = (torch.from_numpy(planes).cuda(), torch.from_numpy(masks.view(np.int32)).cuda())

    def run_patch_match(self) -> None:
        if self._dev is None:
            raise RuntimeError("call cuda_space_init() before run_patch_match()")
        if self.params.geom_consistency:
            raise RuntimeError("PlanarInit does not support geom_consistency (the reference never builds its "
                               "depth textures); use gmvs_gb300.src.PatchMatcher for the geometric pass")
        n = len(self._images)
        v = ViewInputs(cams=self._cameras[:n], images=[self._dev[i] for i in range(n)],
                       depth_min=self.params.depth_min, depth_max=self.params.depth_max, stream_id=0)
        if self.params.planar_prior:
            if self._prior_dev is None or self._last is None:
                raise RuntimeError("the planar-prior pass needs a previous pass and cuda_planar_prior_init()")
            v.prior_planes, v.prior_masks = self._prior_dev
            v.init_planes = self._last.out_planes
            v.init_costs = self._last.out_cost
            kinds = dict(init_kind=_abi.INIT_PRIOR, sweep_kind=_abi.SWEEP_PRIOR)
        else:
            kinds = dict(init_kind=_abi.INIT_RANDOM, sweep_kind=_abi.SWEEP_PHOTO)
        v.allocate_outputs(with_planes=True)
        p = params_struct(self.params, sampler=_abi.SAMPLER_TEX, run_filter=1, pass_index=self._pass, **kinds)
        run_passes([v], p, self._ws)
        self._pass += 1
        self._last = v
        if self.verbose:
            for i in range(self.params.max_iterations):
                print(f"iteration: {i}")

    def jump_patch_match(self) -> None:
        torch.cuda.synchronize()

    # outputs -----------------------------------------------------------------
    def export_plane(self, depth: np.ndarray, normal: np.ndarray, cost: np.ndarray) -> None:
        """Write depth [H, W], world normal [H, W, 3] and cost [H, W] in place."""
        if self._last is None:
            raise RuntimeError("run_patch_match() has not run")
        H, W = self._images[0].shape
        for a, shape, name in ((depth, (H, W), "depth"), (normal, (H, W, 3), "normal"), (cost, (H, W), "cost")):
            if not isinstance(a, np.ndarray) or a.dtype != np.float32 or a.shape != shape or \
                    not a.flags.c_contiguous or not a.flags.writeable:
                raise ValueError(f"{name} must be a writable C-contiguous float32 array of shape {shape}")
        depth[...] = self._last.out_depth.cpu().numpy()
        normal[...] = self._last.out_normal.cpu().numpy()
        cost[...] = self._last.out_cost.cpu().numpy()

    def get_cost(self, index: int) -> float:
        return float(self._last.out_cost.view(-1)[index])

    def triangulation(self, depth: np.ndarray, triangulation_path: str = " ") -> None:
        if self._last is None:
            raise RuntimeError("run_patch_match() has not run")
        cost = self._last.out_cost.cpu().numpy()
        planes, masks, tris = build_planar_prior(self._cameras[0], depth, cost, self._superpixel,
                                                 bool(self.params.superpixel_filter), self.params.depth_min,
                                                 self.params.depth_max)
        self._prior = (planes, masks)
        if triangulation_path.endswith(".png"):
            if self.verbose:
                print(f"save triangulation as {triangulation_path}")
            imageio.write_png(triangulation_path, _draw_triangles(self._images[0], tris))
