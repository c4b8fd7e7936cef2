"""The whole reconstruction of one scene, device-resident:

  1. random-initialisation pass of every reference view (module A,
     PlanarInit::run_patch_match, planar_init.py:113-172);
  2. planar prior of every view from its depth/cost map (host C++,
     PlanarInit::triangulation, planar_init.py:173-181);
  3. planar-prior pass of every view (planar_init.py:181-190);
  4. ``geom_iters`` geometric-consistency passes (module B,
     consistency.run_patch_match, launch.py:157-164);
  5. fusion of every view in order (consistency.run_fusion, launch.py:166-173).

``mode="batched"`` runs every stage of a pass as one launch over all views
(fp16 texel quads where lossless); ``mode="plain"`` is the per-view launch
chain with a synchronisation after every kernel, like the reference.
"""

from __future__ import annotations

import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _abi
from .engine import Plan, ViewInputs, Workspace, fuse, make_camera, make_problem, params_struct
from .planar_initer import build_planar_prior


@dataclass
class SceneInputs:
    images: torch.Tensor                     # float32 [V, H, W] on the device
    cams: List[_abi.gmvs_camera]             # per view
    problems: List[Tuple[int, List[int]]]    # (ref, src ids)
    superpixels: Optional[np.ndarray] = None  # uint8 [V, H, W] host


@dataclass
class StageTimes:
    seconds: Dict[str, float] = field(default_factory=dict)

    def add(self, k: str, v: float) -> None:
        self.seconds[k] = self.seconds.get(k, 0.0) + v


def _range(cam) -> Tuple[float, float]:
    # planar_init.py:149-150, gmvs/src/patch_match.cu:1379-1380
    return float(cam.depth_min) * 0.6, float(cam.depth_max) * 1.2


class ScenePipeline:
    """Runs the five stages for one scene; buffers are kept for reuse."""

    def __init__(self, scene: SceneInputs, geom_iters: int = 2, geom_consistent: int = 3, mode: str = "batched",
                 staging: int = _abi.STAGE_AUTO, tile_h: int = 0, prior_threads: int = 8, params=None):
        if mode not in ("batched", "plain"):
            raise ValueError("mode is 'batched' or 'plain'")
        self.sc = scene
        self.geom_iters = geom_iters
        self.gc = geom_consistent
        self.mode = mode
        self.staging = staging if mode == "batched" else _abi.STAGE_F32
        self.tile_h = tile_h
        self.prior_threads = prior_threads
        self.base = params
        self.ws: Dict[str, Workspace] = {}
        self.scratch = Workspace()
        V, H, W = scene.images.shape
        dev = scene.images.device
        self.V, self.H, self.W = V, H, W
        f32 = dict(dtype=torch.float32, device=dev)
        # stage outputs (double-buffered between consecutive passes)
        self.depth = [torch.empty((V, H, W), **f32) for _ in range(2)]
        self.normal = [torch.empty((V, H, W, 3), **f32) for _ in range(2)]
        self.cost = [torch.empty((V, H, W), **f32) for _ in range(2)]
        self.planes = [torch.empty((V, H, W, 4), **f32) for _ in range(2)]
        self.prior_planes = torch.empty((V, H, W, 4), **f32)
        self.prior_masks = torch.empty((V, H, W), dtype=torch.int32, device=dev)
        self.fused_depth = torch.empty((V, H, W), **f32)
        self.fused_normal = torch.empty((V, H, W, 3), **f32)
        self.masks = torch.zeros((V, H, W), dtype=torch.bool, device=dev)
        self.times = StageTimes()
        self.plans: Dict[str, List[Plan]] = {}

    # ------------------------------------------------------------ passes --
    def _views(self, kind: str, out: int, src_buf: Optional[int] = None) -> List[ViewInputs]:
        sc = self.sc
        views = []
        for ref, src in sc.problems:
            ids = [ref] + list(src)
            dmin, dmax = _range(sc.cams[ref])
            v = ViewInputs(cams=[sc.cams[i] for i in ids], images=[sc.images[i] for i in ids], depth_min=dmin,
                           depth_max=dmax, stream_id=ref)
            if kind == "prior":
                v.prior_planes = self.prior_planes[ref]
                v.prior_masks = self.prior_masks[ref]
                v.init_planes = self.planes[src_buf][ref]
                v.init_costs = self.cost[src_buf][ref]
            elif kind == "geom":
                v.depths = [self.depth[src_buf][i] for i in ids]
                v.ref_normal = self.normal[src_buf][ref]
            v.out_depth = self.depth[out][ref]
            v.out_normal = self.normal[out][ref]
            v.out_cost = self.cost[out][ref]
            v.out_planes = self.planes[out][ref]
            views.append(v)
        return views

    def _params(self, kind: str, pass_index: int) -> _abi.gmvs_params:
        kinds = {
            "random": dict(init_kind=_abi.INIT_RANDOM, sweep_kind=_abi.SWEEP_PHOTO, sampler=_abi.SAMPLER_TEX),
            "prior": dict(init_kind=_abi.INIT_PRIOR, sweep_kind=_abi.SWEEP_PRIOR, sampler=_abi.SAMPLER_TEX),
            "geom": dict(init_kind=_abi.INIT_DEPTH_NORMAL, sweep_kind=_abi.SWEEP_GEOM, sampler=_abi.SAMPLER_CLAMP,
                         max_iterations=2),
        }[kind]
        p = params_struct(self.base, staging=self.staging, tile_h=self.tile_h, pass_index=pass_index, run_filter=1,
                          **kinds)
        if self.base is not None and kind == "geom" and hasattr(self.base, "geom_max_iterations"):
            p.max_iterations = self.base.geom_max_iterations
        return p

    def _run(self, key: str, kind: str, out: int, src_buf: Optional[int], pass_index: int,
             stream: Optional[torch.cuda.Stream]) -> None:
        p = self._params(kind, pass_index)
        views = self._views(kind, out, src_buf)
        ws = self.ws.setdefault(key, Workspace())
        if self.mode == "batched":
            if key not in self.plans:
                self.plans[key] = [Plan(views, p, ws, stream)]
            for pl in self.plans[key]:
                pl.launch(stream)
        else:
            if key not in self.plans:
                # one workspace region per view keeps plans valid together
                self.plans[key] = []
            for k, v in enumerate(views):
                plan = Plan([v], p, ws, stream)
                for s in range(plan.num_stages):
                    plan.launch_stage(s, stream)
                    torch.cuda.synchronize()
                plan.close()

    def _prior(self, buf: int) -> None:
        """Host triangulation of every view (parallel over views)."""
        sc = self.sc
        depth = self.depth[buf].cpu().numpy()
        cost = self.cost[buf].cpu().numpy()
        planes = np.empty((self.V, self.H, self.W, 4), np.float32)
        masks = np.empty((self.V, self.H, self.W), np.uint32)
        spf = sc.superpixels is not None

        def one(ref: int) -> None:
            dmin, dmax = _range(sc.cams[ref])
            pl, mk, _ = build_planar_prior(sc.cams[ref], depth[ref], cost[ref],
                                           sc.superpixels[ref] if spf else None, spf, dmin, dmax)
            planes[ref], masks[ref] = pl, mk

        refs = [r for r, _ in sc.problems]
        with ThreadPoolExecutor(self.prior_threads) as ex:
            list(ex.map(one, refs))
        self.prior_planes.copy_(torch.from_numpy(planes))
        self.prior_masks.copy_(torch.from_numpy(masks.view(np.int32)))

    def _fuse(self, buf: int, stream: Optional[torch.cuda.Stream]) -> None:
        sc = self.sc
        self.masks.zero_()
        for ref, src in sc.problems:
            ids = [ref] + list(src)
            d, n = fuse(make_problem(ref, src), [sc.cams[i] for i in ids], [self.depth[buf][i] for i in ids],
                        [self.normal[buf][i] for i in ids], self.masks, self.gc, self.scratch, stream=stream)
            self.fused_depth[ref].copy_(d)
            self.fused_normal[ref].copy_(n)
        # normal renormalisation of consistency.py:193-197
        nn = torch.linalg.vector_norm(self.fused_normal, dim=-1, keepdim=True)
        self.fused_normal /= torch.where(nn > 0.5, nn, torch.ones_like(nn))

    def run(self, stream: Optional[torch.cuda.Stream] = None, timed: bool = False):
        def mark(name, t0):
            if timed:
                torch.cuda.synchronize()
                self.times.add(name, time.perf_counter() - t0)
            return time.perf_counter()

        t = time.perf_counter()
        self._run("random", "random", 0, None, 0, stream)
        t = mark("random_pass", t)
        self._prior(0)
        t = mark("triangulation", t)
        self._run("prior", "prior", 1, 0, 1, stream)
        t = mark("prior_pass", t)
        buf = 1
        for g in range(self.geom_iters):
            self._run(f"geom{g}", "geom", 1 - buf, buf, 2 + g, stream)
            buf = 1 - buf
        t = mark("geom_passes", t)
        if self.geom_iters > 0:
            self._fuse(buf, stream)
        mark("fusion", t)
        return self.fused_depth, self.fused_normal

    def close(self) -> None:
        for plans in self.plans.values():
            for p in plans:
                p.close()
        self.plans.clear()


def scene_inputs_from_synthetic(sc, device=None) -> SceneInputs:
    from . import synthetic

    dev = device or torch.device("cuda")
    cams = [make_camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]
    return SceneInputs(images=torch.from_numpy(sc.images.astype(np.float32)).to(dev), cams=cams,
                       problems=[(r, list(s)) for r, s in sc.problems], superpixels=sc.superpixels)
