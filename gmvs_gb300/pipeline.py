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
                 staging: int = _abi.STAGE_AUTO, tile_h: int = 0, prior_threads: int = 8, params=None,
                 graphs: bool = False, autotuner=None, overlap: bool = True, mirror_streams: bool = False):
        if mode not in ("batched", "plain"):
            raise ValueError("mode is 'batched' or 'plain'")
        if graphs and mode != "batched":
            raise ValueError("CUDA graphs replay the batched launch chains")
        self.graphs = graphs
        # mirror_streams: the random streams that the module mirrors
        # (planar_initer.PlanarInit, src.PatchMatcher) use, so that the
        # reference's own call sequence over them gives this pipeline's maps:
        # one stream shared by every view in the random and prior passes (the
        # reference seeds every view alike, curand_init(3407, y, x),
        # patch_match_kernel.cu:1491) and one pass index for every geometric
        # pass.  By default each view and pass draws its own stream.
        self.mirror_streams = mirror_streams
        self._graphs: Dict[str, torch.cuda.CUDAGraph] = {}
        if autotuner is not None and mode != "batched":
            raise ValueError("the autotuner picks launch shapes of the batched launch chains")
        self.autotuner = autotuner
        self.tuned: Dict[str, object] = {}
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
        # zero for views that are no problem's reference (fusion writes the others)
        self.fused_depth = torch.zeros((V, H, W), **f32)
        self.fused_normal = torch.zeros((V, H, W, 3), **f32)
        self.masks = torch.zeros((V, H, W), dtype=torch.bool, device=dev)
        self.times = StageTimes()
        self.plans: Dict[str, List[Plan]] = {}
        # Batched runs split the random and prior passes into two view groups
        # so that one group's host triangulation overlaps the other's device
        # work (results do not depend on the grouping).
        n = len(scene.problems)
        self.groups: List[List[int]] = [list(range(n))]
        if mode == "batched" and overlap and n >= 2:
            self.groups = [list(range(n // 2)), list(range(n // 2, n))]
        self._pinned: Optional[Dict[str, torch.Tensor]] = None
        self._copy_stream: Optional[torch.cuda.Stream] = None

    # ------------------------------------------------------------ passes --
    def _views(self, kind: str, out: int, src_buf: Optional[int] = None,
               group: Optional[List[int]] = None) -> List[ViewInputs]:
        sc = self.sc
        views = []
        problems = sc.problems if group is None else [sc.problems[k] for k in group]
        for ref, src in problems:
            ids = [ref] + list(src)
            dmin, dmax = _range(sc.cams[ref])
            sid = 0 if self.mirror_streams and kind != "geom" else ref
            v = ViewInputs(cams=[sc.cams[i] for i in ids], images=[sc.images[i] for i in ids], depth_min=dmin,
                           depth_max=dmax, stream_id=sid)
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
        if kind == "geom" and self.mode == "batched" and not hasattr(self.base, "split_sweep"):
            # the fp16-quad geometric half-sweeps are faster as three kernels
            # (same results); the autotuner, when given, decides instead
            p.split_sweep = 2
        return p

    def _passes(self):
        """(key, kind, output buffer, input buffer, pass index, view group) of
        every pass: the random and prior passes per view group, then the
        geometric passes over all views."""
        multi = len(self.groups) > 1
        out = [(f"random{g}" if multi else "random", "random", 0, None, 0, grp) for g, grp in enumerate(self.groups)]
        out += [(f"prior{g}" if multi else "prior", "prior", 1, 0, 1, grp) for g, grp in enumerate(self.groups)]
        buf = 1
        for g in range(self.geom_iters):
            out.append((f"geom{g}", "geom", 1 - buf, buf, 2 if self.mirror_streams else 2 + g, None))
            buf = 1 - buf
        return out

    def prepare(self, stream: Optional[torch.cuda.Stream] = None) -> None:
        """Create every pass's plan now (batched mode; plan creation
        synchronises `stream`) and, with ``graphs``, capture each pass's
        launch chain into a CUDA graph.  Needs the images in place.  With an
        autotuner, a pass whose launch shape is not tuned yet is prepared at
        its first launch instead, when its inputs exist to tune on."""
        if self.mode != "batched":
            return
        for key, kind, out, src_buf, pass_index, group in self._passes():
            if self.autotuner is not None:
                from .autotune import tune_key

                if tune_key(self._views(kind, out, src_buf, group), self._params(kind, pass_index)) \
                        not in self.autotuner.cache:
                    continue
            self._ensure(key, kind, out, src_buf, pass_index, group, stream)

    def _ensure(self, key: str, kind: str, out: int, src_buf: Optional[int], pass_index: int,
                group: Optional[List[int]], stream: Optional[torch.cuda.Stream]) -> None:
        if key not in self.plans:
            views = self._views(kind, out, src_buf, group)
            p = self._params(kind, pass_index)
            if self.autotuner is not None:
                res = self.autotuner.tune(views, p, stream)
                self.tuned[key] = res
                p = res.apply(p)
            ws = self.ws.setdefault(key, Workspace(self.sc.images.device))
            self.plans[key] = [Plan(views, p, ws, stream)]
        if self.graphs and key not in self._graphs:
            g = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream(device=self.sc.images.device)
            side.wait_stream(torch.cuda.current_stream() if stream is None else stream)
            with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
                for pl in self.plans[key]:
                    pl.launch(side)
            self._graphs[key] = g

    def _run(self, key: str, kind: str, out: int, src_buf: Optional[int], pass_index: int,
             group: Optional[List[int]], stream: Optional[torch.cuda.Stream]) -> None:
        if self.mode == "batched":
            self._ensure(key, kind, out, src_buf, pass_index, group, stream)
            if self.graphs:
                with torch.cuda.stream(stream or torch.cuda.current_stream()):
                    self._graphs[key].replay()
            else:
                for pl in self.plans[key]:
                    pl.launch(stream)
            return
        # plain: one plan per view, a synchronisation after every kernel
        p = self._params(kind, pass_index)
        ws = self.ws.setdefault(key, Workspace())
        for v in self._views(kind, out, src_buf, group):
            plan = Plan([v], p, ws, stream)
            for s in range(plan.num_stages):
                plan.launch_stage(s, stream)
                torch.cuda.synchronize()
            plan.close()

    def _prior(self, buf: int) -> None:
        """Host triangulation of every view (parallel over views)."""
        planes, masks = self.triangulate(self.depth[buf].cpu().numpy(), self.cost[buf].cpu().numpy())
        self.upload_prior(planes, masks)

    def upload_prior(self, planes: np.ndarray, masks: np.ndarray,
                     stream: Optional[torch.cuda.Stream] = None) -> None:
        with torch.cuda.stream(stream or torch.cuda.current_stream()):
            self.prior_planes.copy_(torch.from_numpy(planes), non_blocking=stream is not None)
            self.prior_masks.copy_(torch.from_numpy(masks.view(np.int32)), non_blocking=stream is not None)

    def triangulate(self, depth: np.ndarray, cost: np.ndarray):
        """Planar priors of every reference view from host depth/cost maps
        [V, H, W]; returns (planes float32 [V, H, W, 4], masks uint32 [V, H, W])."""
        sc = self.sc
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
        return planes, masks

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

        nvtx = torch.cuda.nvtx  # host ranges for profilers (nsys / ncu --nvtx)
        t = time.perf_counter()
        if len(self.groups) > 1 and not timed:
            nvtx.range_push("random+triangulation+prior (overlapped)")
            self._random_prior_overlapped(stream)
            nvtx.range_pop()
        else:
            nvtx.range_push("random_pass")
            self.random_pass(stream)
            nvtx.range_pop()
            t = mark("random_pass", t)
            nvtx.range_push("triangulation")
            self._prior(0)
            nvtx.range_pop()
            t = mark("triangulation", t)
            nvtx.range_push("prior_pass")
            self.prior_pass(stream)
            nvtx.range_pop()
            t = mark("prior_pass", t)
        nvtx.range_push("geom_passes")
        buf = self.geom_passes(stream)
        nvtx.range_pop()
        t = mark("geom_passes", t)
        nvtx.range_push("fusion")
        self.fusion(buf, stream)
        nvtx.range_pop()
        mark("fusion", t)
        return self.fused_depth, self.fused_normal

    def _random_prior_overlapped(self, stream: Optional[torch.cuda.Stream]) -> None:
        """Random passes of both view groups back to back; each group's
        depth/cost maps go to pinned host memory on a copy stream as soon as
        its pass ends and are triangulated on the host while the device
        works on the other group; each group's prior pass is enqueued as
        soon as its priors are uploaded."""
        st = stream or torch.cuda.current_stream()
        if self._pinned is None:
            V, H, W = self.V, self.H, self.W
            pin = lambda *shape, dt=torch.float32: torch.empty(shape, dtype=dt, pin_memory=True)
            self._pinned = {"depth": pin(V, H, W), "cost": pin(V, H, W), "planes": pin(V, H, W, 4),
                            "masks": pin(V, H, W, dt=torch.int32)}
            self._copy_stream = torch.cuda.Stream(device=self.sc.images.device)
        hp, cs = self._pinned, self._copy_stream
        passes = self._passes()
        ng = len(self.groups)
        done = []
        for g in range(ng):
            self._run(*passes[g], stream)
            ev = torch.cuda.Event()
            ev.record(st)
            done.append(ev)
        with ThreadPoolExecutor(1) as ex:
            futs = []
            for g, grp in enumerate(self.groups):
                refs = [self.sc.problems[k][0] for k in grp]
                cs.wait_event(done[g])
                with torch.cuda.stream(cs):
                    for r in refs:
                        hp["depth"][r].copy_(self.depth[0][r], non_blocking=True)
                        hp["cost"][r].copy_(self.cost[0][r], non_blocking=True)
                cs.synchronize()
                futs.append(ex.submit(self._triangulate_into, refs))
            for g, grp in enumerate(self.groups):
                futs[g].result()
                with torch.cuda.stream(st):
                    for k in grp:
                        r = self.sc.problems[k][0]
                        self.prior_planes[r].copy_(hp["planes"][r], non_blocking=True)
                        self.prior_masks[r].copy_(hp["masks"][r], non_blocking=True)
                self._run(*passes[ng + g], stream)

    def _triangulate_into(self, refs: List[int]) -> None:
        """Planar priors of `refs` from the pinned depth/cost maps into the
        pinned plane/mask buffers."""
        sc, hp = self.sc, self._pinned
        depth, cost = hp["depth"].numpy(), hp["cost"].numpy()
        planes, masks = hp["planes"].numpy(), hp["masks"].numpy().view(np.uint32)
        spf = sc.superpixels is not None

        def one(ref: int) -> None:
            dmin, dmax = _range(sc.cams[ref])
            pl, mk, _ = build_planar_prior(sc.cams[ref], depth[ref], cost[ref],
                                           sc.superpixels[ref] if spf else None, spf, dmin, dmax)
            planes[ref], masks[ref] = pl, mk

        with ThreadPoolExecutor(self.prior_threads) as ex:
            list(ex.map(one, refs))

    # the stages one at a time (for schedulers that interleave scenes)
    def random_pass(self, stream: Optional[torch.cuda.Stream] = None) -> None:
        for args in self._passes()[:len(self.groups)]:
            self._run(*args, stream)

    def prior_pass(self, stream: Optional[torch.cuda.Stream] = None) -> None:
        ng = len(self.groups)
        for args in self._passes()[ng:2 * ng]:
            self._run(*args, stream)

    def geom_passes(self, stream: Optional[torch.cuda.Stream] = None) -> int:
        """Enqueue the geometric passes; returns the buffer holding the result."""
        buf = 1
        for args in self._passes()[2 * len(self.groups):]:
            self._run(*args, stream)
            buf = args[2]
        return buf

    def fusion(self, buf: int, stream: Optional[torch.cuda.Stream] = None) -> None:
        if self.geom_iters > 0:
            with torch.cuda.stream(stream or torch.cuda.current_stream()):
                self._fuse(buf, stream)

    def close(self) -> None:
        self._graphs.clear()
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
