"""Drop-in replacement for the reference's torch extension ``gmvs.src``
(gmvs/src/bindings.cpp:8-54): ``load_camera``, ``load_problem``,
``PatchMatchParams``, ``Problem``, ``Camera``, ``PatchMatcher`` and ``Fuser``
with the same names, arguments, return types and error behaviour.

Differences that a caller can observe, all deliberate:
  * images, depths and normals are uploaded to the device once and kept
    resident (re-uploaded only when a host tensor is modified in place),
    instead of being copied for every problem;
  * the random stream is Philox4x32-10 keyed by (seed, pixel, reference id);
  * fusion collisions resolve deterministically (highest reference pixel).
"""

from __future__ import annotations

from typing import List, Sequence

import torch

from . import _abi
from .engine import ViewInputs, Workspace, fuse, make_camera, make_problem, params_struct, run_passes

Camera = _abi.gmvs_camera
Problem = _abi.gmvs_problem


def load_camera(K: Sequence[float], R: Sequence[float], t: Sequence[float], height: int, width: int,
                depth_min: float, depth_max: float) -> Camera:
    return make_camera(K, R, t, height, width, depth_min, depth_max)


def load_problem(ref_image_id: int, src_image_ids: Sequence[int]) -> Problem:
    return make_problem(ref_image_id, src_image_ids)


class PatchMatchParams:
    """PatchMatchParams (gmvs/include/data_structure.hpp:20-37) plus the
    extensions of gmvs_params (defaults keep reference behaviour)."""

    def __init__(self):
        self.max_iterations = 3
        self.patch_size = 11
        self.num_images = 5
        self.max_image_size = 3200
        self.radius_increment = 2
        self.sigma_spatial = 5.0
        self.sigma_color = 3.0
        self.top_k = 4
        self.baseline = 0.54
        self.depth_min = 0.0
        self.depth_max = 1.0
        self.disparity_min = 0.0
        self.disparity_max = 1.0
        self.geom_consistency = False
        self.multi_geometry = False
        self.planar_prior = False
        self.superpixel_filter = False
        # extensions
        self.seed = 3407
        self.staging = _abi.STAGE_AUTO
        self.tile_h = 0

    def __repr__(self) -> str:
        return "PatchMatchParams(" + ", ".join(f"{k}={v!r}" for k, v in vars(self).items()) + ")"


def _check_cpu(t: torch.Tensor, name: str) -> None:
    # CHECK_CPU_INPUT (gmvs/include/cuda_utils.cuh:3-11)
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if t.is_cuda:
        raise RuntimeError(f"{name} must be a CPU tensor")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")


def _check_cuda(t: torch.Tensor, name: str) -> None:
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")


class _Resident:
    """Device copy of a host tensor, refreshed when the host tensor changes."""

    def __init__(self):
        self.src = None
        self.version = None
        self.dev = None

    def get(self, host: torch.Tensor) -> torch.Tensor:
        if self.src is not host or self.version != host._version or self.dev is None:
            self.dev = host.to(device="cuda", dtype=torch.float32, non_blocking=False).contiguous()
            self.src = host
            self.version = host._version
        return self.dev


class PatchMatcher:
    """Geometric-consistency PatchMatch (PatchMatcher, gmvs/src/patch_match.cu:1315-1518)."""

    def __init__(self):
        self.params = PatchMatchParams()
        self.num_images = 0
        self._ws = None
        self._img = _Resident()
        self._dep = _Resident()
        self._nrm = _Resident()

    def add_samples(self, problems: List[Problem], cameras: List[Camera], images: torch.Tensor,
                    depths: torch.Tensor, normals: torch.Tensor, costs: torch.Tensor) -> None:
        for t, n in ((images, "images"), (depths, "depths"), (normals, "normals"), (costs, "costs")):
            _check_cpu(t, n)
        self.num_images = len(problems)
        self.cameras_host = list(cameras)
        self.problems_host = list(problems)
        self.height = int(cameras[0].height)
        self.width = int(cameras[0].width)
        self.images_host = images
        self.depths_host = depths
        self.normals_host = normals
        self.costs_host = costs

    def run_patch_match(self, problem_idx: int, verbose: bool = False):
        pb = self.problems_host[problem_idx]
        ref = int(pb.ref_image_id)
        src = [int(pb.src_image_ids[i]) for i in range(pb.num_ngb)]
        # patch_match.cu:1376-1380
        self.params.num_images = pb.num_ngb + 1
        self.params.depth_min = self.cameras_host[ref].depth_min * 0.6
        self.params.depth_max = self.cameras_host[ref].depth_max * 1.2
        imgs = self._img.get(self.images_host)
        deps = self._dep.get(self.depths_host)
        nrms = self._nrm.get(self.normals_host)
        ids = [ref] + src
        v = ViewInputs(
            cams=[self.cameras_host[i] for i in ids], images=[imgs[i] for i in ids],
            depth_min=self.params.depth_min, depth_max=self.params.depth_max, stream_id=ref,
            depths=[deps[i] for i in ids], ref_normal=nrms[ref])
        # the geometric half-sweeps run as three kernels unless the caller's
        # parameters say otherwise (same results, faster on the GB300)
        p = params_struct(self.params, init_kind=_abi.INIT_DEPTH_NORMAL, sweep_kind=_abi.SWEEP_GEOM,
                          sampler=_abi.SAMPLER_CLAMP, run_filter=1, pass_index=2,
                          split_sweep=int(getattr(self.params, "split_sweep", 2)))
        if self._ws is None:
            self._ws = Workspace()
        run_passes([v], p, self._ws)
        if verbose:
            for i in range(self.params.max_iterations):
                print(f"iteration: {i}")
        return v.out_depth, v.out_normal, v.out_cost


class Fuser:
    """Geometric-consistency fusion (Fuser, gmvs/src/fusion.cu:186-275)."""

    def __init__(self):
        self.depths_host = None
        self.normals_host = None
        self.masks_cuda = None
        self._scratch = None
        self._dep = _Resident()
        self._nrm = _Resident()

    def load_samples(self, problems: List[Problem], cameras: List[Camera], depths: torch.Tensor,
                     normals: torch.Tensor, masks: torch.Tensor) -> None:
        _check_cpu(depths, "depths")
        _check_cpu(normals, "normals")
        _check_cuda(masks, "masks")
        self.cameras_host = list(cameras)
        self.problems_host = list(problems)
        self.masks_cuda = masks
        self.height = int(cameras[0].height)
        self.width = int(cameras[0].width)
        self.depths_host = depths
        self.normals_host = normals

    def run_fusion(self, problem_idx: int, geom_consistent: int):
        pb = self.problems_host[problem_idx]
        ref = int(pb.ref_image_id)
        ids = [ref] + [int(pb.src_image_ids[i]) for i in range(pb.num_ngb)]
        deps = self._dep.get(self.depths_host)
        nrms = self._nrm.get(self.normals_host)
        if self._scratch is None:
            self._scratch = Workspace()
        return fuse(pb, [self.cameras_host[i] for i in ids], [deps[i] for i in ids], [nrms[i] for i in ids],
                    self.masks_cuda, geom_consistent, self._scratch)
