"""Thin host layer over the C ABI: builds gmvs_view_pass / gmvs_fuse_view
descriptors from torch CUDA tensors and runs passes, NCC evaluations and
fusion.  torch provides device memory and streams only; all compute is in
libgmvs_gb300.so.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Optional, Sequence, Tuple

import torch

from . import _abi
from ._abi import check, gmvs_camera, gmvs_fuse_view, gmvs_params, gmvs_problem, gmvs_view_pass, lib


def make_camera(K: Sequence[float], R: Sequence[float], t: Sequence[float], height: int, width: int,
                depth_min: float, depth_max: float) -> gmvs_camera:
    """load_camera (gmvs/src/data_structure.cpp:4-29)."""
    if len(K) != 9 or len(R) != 9 or len(t) != 3:
        raise ValueError("K and R need 9 values and t needs 3")
    c = gmvs_camera()
    for i in range(9):
        c.K[i] = float(K[i])
        c.R[i] = float(R[i])
    for i in range(3):
        c.t[i] = float(t[i])
    c.height = int(height)
    c.width = int(width)
    c.depth_min = float(depth_min)
    c.depth_max = float(depth_max)
    return c


def make_problem(ref_id: int, src_ids: Sequence[int]) -> gmvs_problem:
    """load_problem (gmvs/src/data_structure.cpp:31-39)."""
    if len(src_ids) > _abi.MAX_NGB:
        raise ValueError(f"at most {_abi.MAX_NGB} source views")
    p = gmvs_problem()
    p.ref_image_id = int(ref_id)
    p.num_ngb = len(src_ids)
    for i, s in enumerate(src_ids):
        p.src_image_ids[i] = int(s)
    return p


class Workspace:
    """Grow-only device byte buffer handed to the library as its workspace."""

    def __init__(self, device: Optional[torch.device] = None):
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.buf: Optional[torch.Tensor] = None

    def get(self, nbytes: int) -> tuple[int, int]:
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = None
            self.buf = torch.empty(max(nbytes, 1 << 20), dtype=torch.uint8, device=self.device)
        return self.buf.data_ptr(), self.buf.numel()


def _need_cuda_f32(t: torch.Tensor, name: str, shape: tuple) -> None:
    if not t.is_cuda or t.dtype != torch.float32 or not t.is_contiguous():
        raise ValueError(f"{name} must be a contiguous float32 CUDA tensor")
    if tuple(t.shape) != shape:
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {shape}")


@dataclass
class ViewInputs:
    """One reference view of a pass (device tensors, ref first)."""

    cams: list
    images: list
    depth_min: float
    depth_max: float
    stream_id: int = 0
    depths: Optional[list] = None
    ref_normal: Optional[torch.Tensor] = None
    prior_planes: Optional[torch.Tensor] = None
    prior_masks: Optional[torch.Tensor] = None
    init_planes: Optional[torch.Tensor] = None
    init_costs: Optional[torch.Tensor] = None
    out_depth: Optional[torch.Tensor] = None
    out_normal: Optional[torch.Tensor] = None
    out_cost: Optional[torch.Tensor] = None
    out_planes: Optional[torch.Tensor] = None
    keep: list = field(default_factory=list)

    @property
    def height(self) -> int:
        return int(self.images[0].shape[0])

    @property
    def width(self) -> int:
        return int(self.images[0].shape[1])

    def allocate_outputs(self, with_planes: bool = False) -> None:
        H, W = self.height, self.width
        dev = self.images[0].device
        if self.out_depth is None:
            self.out_depth = torch.empty((H, W), dtype=torch.float32, device=dev)
        if self.out_normal is None:
            self.out_normal = torch.empty((H, W, 3), dtype=torch.float32, device=dev)
        if self.out_cost is None:
            self.out_cost = torch.empty((H, W), dtype=torch.float32, device=dev)
        if with_planes and self.out_planes is None:
            self.out_planes = torch.empty((H, W, 4), dtype=torch.float32, device=dev)

    def to_struct(self) -> gmvs_view_pass:
        n = len(self.images) - 1
        if n < 1 or n > _abi.MAX_NGB:
            raise ValueError(f"need 1..{_abi.MAX_NGB} source views, got {n}")
        if len(self.cams) != n + 1:
            raise ValueError("one camera per image is required")
        H, W = self.height, self.width
        v = gmvs_view_pass()
        v.height, v.width, v.num_src, v.stream_id = H, W, n, int(self.stream_id)
        v.depth_min, v.depth_max = float(self.depth_min), float(self.depth_max)
        for i in range(n + 1):
            _need_cuda_f32(self.images[i], f"images[{i}]", (H, W))
            v.cams[i] = self.cams[i]
            v.images[i] = self.images[i].data_ptr()
            if self.depths is not None:
                _need_cuda_f32(self.depths[i], f"depths[{i}]", (H, W))
                v.depths[i] = self.depths[i].data_ptr()
        if self.ref_normal is not None:
            _need_cuda_f32(self.ref_normal, "ref_normal", (H, W, 3))
        v.ref_normal = _abi.ptr(self.ref_normal)
        if self.prior_planes is not None:
            _need_cuda_f32(self.prior_planes, "prior_planes", (H, W, 4))
        v.prior_planes = _abi.ptr(self.prior_planes)
        if self.prior_masks is not None:
            if not self.prior_masks.is_cuda or self.prior_masks.dtype != torch.int32 or \
                    tuple(self.prior_masks.shape) != (H, W) or not self.prior_masks.is_contiguous():
                raise ValueError("prior_masks must be a contiguous int32 CUDA tensor [H, W]")
        v.prior_masks = _abi.ptr(self.prior_masks)
        if self.init_planes is not None:
            _need_cuda_f32(self.init_planes, "init_planes", (H, W, 4))
        v.init_planes = _abi.ptr(self.init_planes)
        if self.init_costs is not None:
            _need_cuda_f32(self.init_costs, "init_costs", (H, W))
        v.init_costs = _abi.ptr(self.init_costs)
        self.allocate_outputs()
        v.out_depth = self.out_depth.data_ptr()
        v.out_normal = self.out_normal.data_ptr()
        v.out_cost = self.out_cost.data_ptr()
        v.out_planes = _abi.ptr(self.out_planes)
        return v


def params_struct(params=None, **overrides) -> gmvs_params:
    """gmvs_params from defaults, a PatchMatchParams-like object and overrides."""
    p = _abi.default_params()
    if params is not None:
        for name, _ in gmvs_params._fields_:
            if hasattr(params, name):
                val = getattr(params, name)
                setattr(p, name, int(val) if isinstance(val, bool) else val)
    for k, val in overrides.items():
        setattr(p, k, int(val) if isinstance(val, bool) else val)
    return p


def _views_array(views: Sequence[ViewInputs]):
    arr = (gmvs_view_pass * len(views))()
    for i, v in enumerate(views):
        arr[i] = v.to_struct()
    return arr


class Plan:
    """A compiled pass over a batch of views (gmvs_plan_*); launchable many
    times, including under CUDA graph capture."""

    def __init__(self, views: Sequence[ViewInputs], params: gmvs_params, workspace: Workspace,
                 stream: Optional[torch.cuda.Stream] = None):
        self.views = list(views)
        self.params = params
        self._arr = _views_array(self.views)
        need = lib().gmvs_plan_workspace_bytes(self._arr, len(self.views), ctypes.byref(params))
        if need == 0:
            raise _abi.GmvsError(_abi.ERR_INVALID, lib().gmvs_last_error().decode())
        ptr, size = workspace.get(need)
        self._ws = workspace.buf  # keep alive
        handle = ctypes.c_void_p()
        check(lib().gmvs_plan_create(self._arr, len(self.views), ctypes.byref(params), ptr, size,
                                     _abi.stream_ptr(stream), ctypes.byref(handle)))
        self.handle = handle

    @property
    def num_stages(self) -> int:
        return lib().gmvs_plan_num_stages(self.handle)

    def launch(self, stream: Optional[torch.cuda.Stream] = None) -> None:
        check(lib().gmvs_plan_launch(self.handle, _abi.stream_ptr(stream)))

    def launch_stage(self, stage: int, stream: Optional[torch.cuda.Stream] = None) -> None:
        check(lib().gmvs_plan_launch_stage(self.handle, stage, _abi.stream_ptr(stream)))

    def check(self, stream: Optional[torch.cuda.Stream] = None) -> None:
        check(lib().gmvs_plan_check(self.handle, _abi.stream_ptr(stream)))

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().gmvs_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_passes(views: Sequence[ViewInputs], params: gmvs_params, workspace: Workspace,
               stream: Optional[torch.cuda.Stream] = None) -> None:
    """One PatchMatch pass over every view of `views` (one launch per stage)."""
    plan = Plan(views, params, workspace, stream)
    try:
        plan.launch(stream)
        plan.check(stream)
    finally:
        plan.close()


def ncc_costs(view: ViewInputs, params: gmvs_params, planes: torch.Tensor, workspace: Workspace,
              want_costs: bool = True, stream: Optional[torch.cuda.Stream] = None):
    """Per-source NCC costs [N, H, W] of camera-frame planes [H, W, 4], plus
    the initial multi-view cost [H, W] and selected-view bits [H, W]."""
    H, W = view.height, view.width
    _need_cuda_f32(planes, "planes", (H, W, 4))
    n = len(view.images) - 1
    v = view.to_struct()
    need = lib().gmvs_ncc_workspace_bytes(ctypes.byref(v), ctypes.byref(params))
    ptr, size = workspace.get(need)
    dev = planes.device
    costs = torch.empty((n, H, W), dtype=torch.float32, device=dev) if want_costs else None
    init_cost = torch.empty((H, W), dtype=torch.float32, device=dev)
    init_views = torch.empty((H, W), dtype=torch.int32, device=dev)
    check(lib().gmvs_ncc_costs(ctypes.byref(v), ctypes.byref(params), planes.data_ptr(), _abi.ptr(costs),
                               init_cost.data_ptr(), init_views.data_ptr(), ptr, size, _abi.stream_ptr(stream)))
    return costs, init_cost, init_views


def fuse(problem: gmvs_problem, cams: Sequence[gmvs_camera], depths: Sequence[torch.Tensor],
         normals: Sequence[torch.Tensor], masks: torch.Tensor, geom_consistent: int, scratch: Workspace,
         out_count: Optional[torch.Tensor] = None, stream: Optional[torch.cuda.Stream] = None):
    """Fusion of one reference view; returns (depth [H, W], normal [H, W, 3])."""
    H, W = int(depths[0].shape[0]), int(depths[0].shape[1])
    n = problem.num_ngb
    if len(cams) != n + 1 or len(depths) != n + 1 or len(normals) != n + 1:
        raise ValueError("ref + one entry per source view is required")
    if not masks.is_cuda or masks.dtype != torch.bool or not masks.is_contiguous() or masks.dim() != 3 or \
            tuple(masks.shape[1:]) != (H, W):
        raise ValueError("masks must be a contiguous bool CUDA tensor [V, H, W]")
    a = gmvs_fuse_view()
    a.height, a.width, a.num_views = H, W, int(masks.shape[0])
    a.problem = problem
    for j in range(n + 1):
        _need_cuda_f32(depths[j], f"depths[{j}]", (H, W))
        _need_cuda_f32(normals[j], f"normals[{j}]", (H, W, 3))
        a.cams[j] = cams[j]
        a.depths[j] = depths[j].data_ptr()
        a.normals[j] = normals[j].data_ptr()
    a.masks = masks.data_ptr()
    a.geom_consistent = int(geom_consistent)
    out_depth = torch.empty((H, W), dtype=torch.float32, device=masks.device)
    out_normal = torch.empty((H, W, 3), dtype=torch.float32, device=masks.device)
    a.out_depth = out_depth.data_ptr()
    a.out_normal = out_normal.data_ptr()
    a.out_count = _abi.ptr(out_count)
    need = lib().gmvs_fuse_scratch_bytes(H, W)
    ptr, size = scratch.get(need)
    check(lib().gmvs_fuse(ctypes.byref(a), ptr, size, _abi.stream_ptr(stream)))
    return out_depth, out_normal


# ------------------------------------------------ segment statistics (device)
def _need_cuda(t: torch.Tensor, dtype, shape: tuple, name: str) -> None:
    if not t.is_cuda or t.dtype != dtype or not t.is_contiguous() or tuple(t.shape) != shape:
        raise ValueError(f"{name} must be a contiguous {dtype} CUDA tensor of shape {shape}")


def _seg_workspace(rows: int, cols: int, max_seg: int, workspace: Optional[Workspace], dev) -> Tuple[int, int]:
    need = lib().gmvs_segments_workspace_bytes(rows, cols, max_seg)
    ws = workspace or Workspace(dev)
    return ws.get(need) + (ws,)


def fusion_planar_mask(seg_ids: torch.Tensor, planar_mask: torch.Tensor, normals: torch.Tensor, thresh: int = 100,
                       nonplanar_percent: float = 0.75, cos_sim_thresh: float = 0.8, match_ratio_thresh: float = 0.9,
                       max_seg_id: Optional[int] = None, workspace: Optional[Workspace] = None,
                       stream: Optional[torch.cuda.Stream] = None) -> torch.Tensor:
    """Device fusion_planar_mask: int32 [H, W] CUDA tensors in and out."""
    rows, cols = int(seg_ids.shape[0]), int(seg_ids.shape[1])
    _need_cuda(seg_ids, torch.int32, (rows, cols), "seg_ids")
    _need_cuda(planar_mask, torch.int32, (rows, cols), "planar_mask")
    _need_cuda(normals, torch.float32, (rows, cols, 3), "normals")
    ms = int(seg_ids.max().item()) if max_seg_id is None else int(max_seg_id)
    out = torch.empty((rows, cols), dtype=torch.int32, device=seg_ids.device)
    ptr, size, _ws = _seg_workspace(rows, cols, max(ms, 0), workspace, seg_ids.device)
    check(lib().gmvs_fusion_planar_mask_device(seg_ids.data_ptr(), planar_mask.data_ptr(), normals.data_ptr(), rows,
                                               cols, max(ms, 0), int(thresh), float(nonplanar_percent),
                                               float(cos_sim_thresh), float(match_ratio_thresh), out.data_ptr(), ptr,
                                               size, _abi.stream_ptr(stream)))
    return out


def filter_by_var_map(var_map: torch.Tensor, seg_ids: torch.Tensor, var_thresh: float,
                      max_seg_id: Optional[int] = None, workspace: Optional[Workspace] = None,
                      stream: Optional[torch.cuda.Stream] = None) -> torch.Tensor:
    """Device filter_by_var_map: float32 / int32 [H, W] CUDA tensors."""
    rows, cols = int(var_map.shape[0]), int(var_map.shape[1])
    _need_cuda(var_map, torch.float32, (rows, cols), "var_map")
    _need_cuda(seg_ids, torch.int32, (rows, cols), "seg_ids")
    ms = int(seg_ids.max().item()) if max_seg_id is None else int(max_seg_id)
    out = torch.empty((rows, cols), dtype=torch.int32, device=seg_ids.device)
    ptr, size, _ws = _seg_workspace(rows, cols, max(ms, 0), workspace, seg_ids.device)
    check(lib().gmvs_filter_by_var_map_device(var_map.data_ptr(), seg_ids.data_ptr(), rows, cols, max(ms, 0),
                                              float(var_thresh), out.data_ptr(), ptr, size, _abi.stream_ptr(stream)))
    return out


def sliding_window_normal(planar_region: torch.Tensor, normals: torch.Tensor, window_size: int,
                          stream: Optional[torch.cuda.Stream] = None) -> torch.Tensor:
    """Device sliding_window_normal: int32 [H, W] and float32 [H, W, 3] CUDA tensors."""
    rows, cols = int(normals.shape[0]), int(normals.shape[1])
    _need_cuda(planar_region, torch.int32, (rows, cols), "planar_region")
    _need_cuda(normals, torch.float32, (rows, cols, 3), "normals")
    out = torch.empty((rows, cols, 3), dtype=torch.float32, device=normals.device)
    check(lib().gmvs_sliding_window_normal_device(planar_region.data_ptr(), normals.data_ptr(), rows, cols,
                                                  int(window_size), out.data_ptr(), _abi.stream_ptr(stream)))
    return out


def gather_points(depth: torch.Tensor, normal: torch.Tensor, K, pose, cos_thresh: float,
                  workspace: Optional[Workspace] = None, stream: Optional[torch.cuda.Stream] = None):
    """World points of one view's fused maps (depth [H, W], normal [H, W, 3]
    CUDA tensors; K 3x3, pose 4x4 camera-to-world).  Returns (points [M, 6],
    facing points [M', 6], filtered depth [H, W], filtered normal [H, W, 3])."""
    import numpy as np

    H, W = int(depth.shape[0]), int(depth.shape[1])
    _need_cuda(depth, torch.float32, (H, W), "depth")
    _need_cuda(normal, torch.float32, (H, W, 3), "normal")
    Kh = np.ascontiguousarray(np.asarray(K, np.float32).reshape(3, 3))
    Ph = np.ascontiguousarray(np.asarray(pose, np.float32).reshape(4, 4))
    dev = depth.device
    pts = torch.empty((H * W, 6), dtype=torch.float32, device=dev)
    fac = torch.empty((H * W, 6), dtype=torch.float32, device=dev)
    od = torch.empty((H, W), dtype=torch.float32, device=dev)
    on = torch.empty((H, W, 3), dtype=torch.float32, device=dev)
    counts = (ctypes.c_int64 * 2)()
    ws = workspace or Workspace(dev)
    ptr, size = ws.get(lib().gmvs_gather_workspace_bytes(H, W))
    check(lib().gmvs_gather_points(depth.data_ptr(), normal.data_ptr(), H, W, Kh.ctypes.data, Ph.ctypes.data,
                                   float(cos_thresh), pts.data_ptr(), fac.data_ptr(), od.data_ptr(), on.data_ptr(),
                                   ctypes.cast(counts, ctypes.c_void_p), ptr, size, _abi.stream_ptr(stream)))
    return pts[: counts[0]], fac[: counts[1]], od, on
