"""Launch-shape autotuner for the PatchMatch kernels.

The knobs that change speed but not results are the tile shape (a tile is
16 pixel columns by 2 * tile_h rows, tile_h thread rows of one warp each per
CTA, so tile_h = 8 is a 16 x 16 pixel tile and 4 a 16 x 8 tile; tile_w = 32
orders the work as 32-pixel-wide blocks of two such tiles, so the shapes
tried are 16 x 8, 16 x 16, 32 x 8 and 32 x 16 pixels), the resident CTAs per
SM (fewer CTAs leave more of the 256 KB of L1/shared memory to the sample
cache, more CTAs hide more latency) and whether each half-sweep runs as one
kernel or as two (neighbour hypotheses, then view selection and refinement:
fewer live registers per kernel, at the price of a per-pixel scratch in the
workspace).  The window stride (radius_increment) is a parameter of the
method -- stride 1 and 2 give different costs -- so it is not tuned: each
stride is tuned on its own and keyed separately.

A tuning run times whole plan launches (init, every half-sweep, filter) of a
representative subset of the batch's views with CUDA events and keeps the
fastest candidate.  Results are cached per key (sampler, staging, sweep
kind, largest source count, window, image-size class) in memory and,
optionally, in a JSON file.
"""

from __future__ import annotations

import ctypes
import json
import math
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _abi
from .engine import Plan, ViewInputs, Workspace

# (tile_w, tile_h) -> 16 x 8, 16 x 16, 32 x 8 and 32 x 16 pixel tiles
TILE_SHAPES = ((16, 4), (16, 8), (32, 4), (32, 8))
CTAS_PER_SM = (0,)
SPLIT = (0, 1, 2)  # half-sweeps as one, two or three kernels
# (tile_h, ctas_per_sm, split_sweep, tile_w); 2-row tiles and 1-3 CTAs per
# SM never won a sweep on the room scene (fewer resident warps) and are left
# out of the default list
CANDIDATES: Tuple[Tuple[int, ...], ...] = tuple(
    (th, c, sp, tw) for tw, th in TILE_SHAPES for c in CTAS_PER_SM for sp in SPLIT)


# Candidates timed within this fraction of the fastest are ties (run-to-run
# noise on a sample of the views).
TIE = 0.005


def pick(ms: Dict[str, float]) -> str:
    """The fastest candidate; among ties the taller tile (fewer tiles and
    queue claims), then the 16-pixel width, then fewer kernels per
    half-sweep.  Tuned on a few views the tile shapes tie, while on the whole
    64-view batching mix 16 x 16 tiles ran 4 % faster than 16 x 8."""
    fastest = min(ms.values())
    near = [k for k, v in ms.items() if v <= fastest * (1.0 + TIE)]

    def rank(k: str):
        c = [int(x) for x in k.split(",")]
        th, sp = c[0], c[2] if len(c) > 2 else 0
        tw = (c[3] if len(c) > 3 else 0) or 16
        return (th, -tw, -sp, -ms[k])

    return max(near, key=rank)


def _copy_params(p: _abi.gmvs_params) -> _abi.gmvs_params:
    q = _abi.gmvs_params()
    ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(p))
    return q


def tune_key(views: Sequence[ViewInputs], params: _abi.gmvs_params) -> str:
    nmax = max(len(v.images) - 1 for v in views)
    px = max(v.height * v.width for v in views)
    size_class = int(round(math.log2(max(px, 1))))
    return (f"s{params.sampler}-st{params.staging}-sw{params.sweep_kind}-i{params.init_kind}-n{nmax}"
            f"-p{params.patch_size}-r{params.radius_increment}-px{size_class}")


@dataclass
class TuneResult:
    key: str
    best: Tuple[int, ...]
    ms: Dict[str, float] = field(default_factory=dict)  # "tile_h,ctas,split" -> ms per plan launch

    def apply(self, params: _abi.gmvs_params) -> _abi.gmvs_params:
        q = _copy_params(params)
        q.tile_h, q.ctas_per_sm = self.best[0], self.best[1]
        q.split_sweep = self.best[2] if len(self.best) > 2 else 0
        q.tile_w = self.best[3] if len(self.best) > 3 else 0
        return q


class Autotuner:
    def __init__(self, cache_path: Optional[str] = None, candidates: Sequence[Tuple[int, ...]] = CANDIDATES,
                 reps: int = 2, max_views: int = 2):
        self.cache_path = cache_path
        self.candidates = tuple(candidates)
        self.reps = reps
        self.max_views = max_views
        self.cache: Dict[str, TuneResult] = {}
        if cache_path and os.path.exists(cache_path):
            with open(cache_path) as f:
                for k, v in json.load(f).items():
                    self.cache[k] = TuneResult(k, tuple(v["best"]), v.get("ms", {}))

    def _save(self) -> None:
        if not self.cache_path:
            return
        data = {k: {"best": list(r.best), "ms": r.ms} for k, r in self.cache.items()}
        tmp = self.cache_path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.cache_path)

    def tune(self, views: Sequence[ViewInputs], params: _abi.gmvs_params,
             stream: Optional[torch.cuda.Stream] = None) -> TuneResult:
        """Best (tile_h, ctas_per_sm, split_sweep, tile_w) for this kind of batch (cached)."""
        key = tune_key(views, params)
        if key in self.cache:
            return self.cache[key]
        sample = list(views)[: self.max_views]
        dev = sample[0].images[0].device
        st = stream or torch.cuda.current_stream(dev)
        ws = Workspace(dev)
        ms: Dict[str, float] = {}
        for cand in self.candidates:
            th, c = cand[0], cand[1]
            sp = cand[2] if len(cand) > 2 else 0
            tw = cand[3] if len(cand) > 3 else 0
            p = _copy_params(params)
            p.tile_h, p.ctas_per_sm, p.split_sweep, p.tile_w = th, c, sp, tw
            plan = Plan(sample, p, ws, st)
            try:
                plan.launch(st)  # warm-up (module load, first-touch)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                for _ in range(self.reps):
                    plan.launch(st)
                e1.record(st)
                plan.check(st)
                ms[",".join(str(x) for x in (th, c, sp, tw)[:max(3, len(cand))])] = e0.elapsed_time(e1) / self.reps
            finally:
                plan.close()
        best = pick(ms)
        res = TuneResult(key, tuple(int(x) for x in best.split(",")), ms)
        self.cache[key] = res
        self._save()
        return res
