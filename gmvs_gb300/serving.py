"""Continuous-batching reconstruction server (one GPU, one process).

Jobs are whole scenes (the inputs of ``launch.py``: images, cameras,
problems, superpixels).  The server admits queued jobs in arrival order as
soon as their device footprint fits in the memory budget and an active slot
is free, keeps every admitted job's images, plane fields, costs and maps
resident on the device, and advances all active jobs together: each job runs
its passes on its own CUDA stream, so the kernels of different jobs overlap
on the device (the tile-queue kernels of one job fill the SMs the previous
kernel of another job leaves idle at its tail), while the host triangulation
of one job overlaps the device work of the others.  A job that finishes
returns its memory and the next queued job is admitted at once.

Per-view latency is the time from a job's arrival to the moment its fused
maps are on the host, counted once for each of its reference views.  Results
do not depend on the mix: every job's kernels read only that job's buffers
and draw random numbers from counters keyed by (pixel, reference view,
pass), so a job returns the same maps alone and next to others.
"""

from __future__ import annotations

import heapq
import threading
import time
from concurrent.futures import Future, ThreadPoolExecutor
from dataclasses import dataclass, field
from types import SimpleNamespace
from typing import Dict, List, Optional

import numpy as np
import torch

from .pipeline import SceneInputs, ScenePipeline

# Bytes per pixel of one view that ScenePipeline keeps on the device
# (batched mode, worst-case staging):
#   images fp32 4 (+ 1 for the 8-bit upload); depth/normal/cost/planes
#   double-buffered 72; prior planes and masks 20; fused depth/normal 16;
#   masks 1; texture staging of the random and prior passes, each run as
#   two view-group plans that may both read every image, 2 x 2 x 4; quad
#   staging of each geometric pass 16.
_PER_VIEW_BYTES = 4 + 1 + 72 + 20 + 16 + 1 + 16
_PER_GEOM_PASS_VIEW_BYTES = 16
# per reference view and pass: plane/cost/view-mask ping-pong + converted planes
_PER_REF_PASS_BYTES = 64
# per pass: the neighbour-cost scratch of every warp that can be resident
# (at most 64 per SM), 16 pixels x 8 neighbours x num_src floats each
_CA_BYTES_PER_WARP_SRC = 16 * 8 * 4
_FIXED_BYTES = 64 << 20  # descriptors, tile lists, fusion scratch, allocator slack


def _num_sms() -> int:
    if torch.cuda.is_available():
        return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    return 152  # GB300


def footprint_bytes(num_views: int, height: int, width: int, num_refs: int, geom_iters: int = 2,
                    max_src: int = 32, sms: Optional[int] = None, split_geom: bool = True) -> int:
    """Upper bound of the device memory one job holds while it is active.
    `split_geom`: the geometric passes run their half-sweeps as three
    kernels, which pass each pixel's neighbour costs and refinement state
    through a scratch as large as all reference views of the pass; the
    random and prior passes of a served job run single kernels."""
    px = height * width
    per_view = _PER_VIEW_BYTES + geom_iters * _PER_GEOM_PASS_VIEW_BYTES
    passes = 2 + geom_iters
    plans = 4 + geom_iters  # random and prior passes in two view groups each
    pitch_slack = 4 * num_views * height * 256  # texture rows padded to 256 bytes
    ca = plans * (sms or _num_sms()) * 64 * _CA_BYTES_PER_WARP_SRC * max_src
    # split half-sweeps: per geometric pass and reference view,
    # (9 * max_src + 10 + 28) words for every pixel of one colour (cost
    # matrix, neighbour positions, refinement state), tiles rounded up
    split = (geom_iters * num_refs * (width + 16) * (height + 16) // 2 * (9 * max_src + 38) * 4) if split_geom else 0
    total = px * (num_views * per_view + num_refs * passes * _PER_REF_PASS_BYTES + 4) + pitch_slack + ca + split
    # the caching allocator's rounding and fragmentation: 5 % on top
    return total + total // 20 + _FIXED_BYTES


@dataclass
class Job:
    """A reconstruction request.  ``images`` are host uint8 or float32
    [V, H, W]; the result (fused depth [V, H, W], normal [V, H, W, 3]) lands
    in ``result`` as host arrays."""

    job_id: int
    images: np.ndarray
    cams: list
    problems: list
    superpixels: Optional[np.ndarray] = None
    arrival: float = 0.0          # seconds on the server clock
    output_dir: Optional[str] = None  # write {ref:04d}.npy [H, W, 4] (depth, normal) there, as consistency.py
    admitted: float = -1.0
    finished: float = -1.0
    result: Optional[tuple] = None
    error: Optional[BaseException] = None
    written: Optional[Future] = None  # the output files, when output_dir is set

    @property
    def num_views(self) -> int:
        return int(self.images.shape[0])

    @property
    def num_refs(self) -> int:
        return len(self.problems)

    def validate(self) -> None:
        """Reject malformed requests before they take a slot."""
        if self.images.ndim != 3 or min(self.images.shape) < 1:
            raise ValueError(f"job {self.job_id}: images must be [V, H, W]")
        V = self.images.shape[0]
        if len(self.cams) != V:
            raise ValueError(f"job {self.job_id}: {len(self.cams)} cameras for {V} images")
        if not self.problems:
            raise ValueError(f"job {self.job_id}: no reference views")
        for ref, src in self.problems:
            ids = [ref] + list(src)
            if not src or len(src) > 32 or min(ids) < 0 or max(ids) >= V or ref in src:
                raise ValueError(f"job {self.job_id}: bad problem {ref} <- {list(src)}")
        if self.superpixels is not None and tuple(self.superpixels.shape) != tuple(self.images.shape):
            raise ValueError(f"job {self.job_id}: superpixels do not match the images")

    def footprint(self, geom_iters: int, split_geom: bool = True) -> int:
        V, H, W = self.images.shape
        max_src = max((len(s) for _, s in self.problems), default=1)
        return footprint_bytes(V, H, W, len(self.problems), geom_iters, max_src, split_geom=split_geom)


class Cancelled(RuntimeError):
    """The job was cancelled before it finished."""


@dataclass
class _Active:
    job: Job
    pipe: ScenePipeline
    stream: torch.cuda.Stream
    bytes: int
    step: int = 0
    event: Optional[torch.cuda.Event] = None
    host: Optional[Future] = None
    pinned: Dict[str, torch.Tensor] = field(default_factory=dict)
    cancel: bool = False


class ReconstructionServer:
    """See the module docstring.  ``memory_budget`` bounds the summed
    footprints of the active jobs (default: 90 % of the free device memory
    when the server starts); ``max_active`` bounds the number of jobs in
    flight."""

    def __init__(self, device: Optional[torch.device] = None, memory_budget: Optional[int] = None,
                 max_active: int = 4, geom_iters: int = 2, prior_threads: int = 8, graphs: bool = False):
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        if memory_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            memory_budget = int(free * 0.9)
        self.budget = int(memory_budget)
        self.max_active = max_active
        self.geom_iters = geom_iters
        self.graphs = graphs
        self.queue: List[tuple] = []       # (arrival, job_id, job)
        self.active: List[_Active] = []
        self.done: List[Job] = []
        self.in_use = 0
        self.pool = ThreadPoolExecutor(max(1, prior_threads))
        # one stream per slot, reused by the jobs that take the slot (the
        # caching allocator reuses a stream's freed blocks for that stream)
        self._free_streams: List[torch.cuda.Stream] = []
        self.prior_threads = prior_threads
        self.t0 = time.perf_counter()
        self._lock = threading.Lock()

    # ------------------------------------------------------------- clock --
    def now(self) -> float:
        return time.perf_counter() - self.t0

    # ----------------------------------------------------------- requests --
    def split_geom(self, job: Job) -> bool:
        """Whether the job's geometric half-sweeps run as three kernels (faster,
        but their scratch grows with all the job's reference pixels): yes
        while that footprint takes at most half the budget, so that a large
        job does not shut every other job out; single kernels otherwise."""
        return job.footprint(self.geom_iters, True) <= self.budget // 2

    def _need(self, job: Job) -> int:
        return job.footprint(self.geom_iters, self.split_geom(job))

    def submit(self, job: Job) -> Job:
        """Queue a job; it is admitted once it has arrived and fits."""
        job.validate()
        if self._need(job) > self.budget:
            raise ValueError(f"job {job.job_id} needs {self._need(job)} bytes, more than the "
                             f"server's whole budget of {self.budget}")
        with self._lock:
            heapq.heappush(self.queue, (job.arrival, job.job_id, job))
        return job

    def _admit(self) -> None:
        now = self.now()
        while self.queue and len(self.active) < self.max_active:
            arrival, _, job = self.queue[0]
            if arrival > now:
                return
            need = self._need(job)
            if self.in_use + need > self.budget:
                return  # admission in arrival order: wait for memory
            if self._start(job, need) is False:
                return  # the device is fuller than the accounting says: wait for a job to finish
            heapq.heappop(self.queue)

    def cancel(self, job_id: int) -> bool:
        """Cancel a queued or active job; an active one stops at its next
        step boundary and returns its memory.  True if the job was found."""
        with self._lock:
            for k, (_, jid, job) in enumerate(self.queue):
                if jid == job_id:
                    self.queue.pop(k)
                    heapq.heapify(self.queue)
                    job.error = Cancelled(f"job {job_id} cancelled while queued")
                    job.finished = self.now()
                    self.done.append(job)
                    return True
        for a in self.active:
            if a.job.job_id == job_id:
                a.cancel = True
                return True
        return False

    def _start(self, job: Job, need: int) -> bool:
        """Allocate the job's device state and plans; False (nothing kept)
        when the device runs out of memory while other jobs are resident —
        the caller retries once one of them has finished.  The job is then
        accounted at the larger of its footprint bound and what it really
        took."""
        st = self._free_streams.pop() if self._free_streams else torch.cuda.Stream(device=self.device)
        before = torch.cuda.memory_allocated(self.device)
        pipe = None
        try:
            with torch.cuda.stream(st):
                host = torch.from_numpy(np.ascontiguousarray(job.images))
                imgs = host.pin_memory().to(self.device, non_blocking=True).to(torch.float32)
                scene = SceneInputs(images=imgs, cams=list(job.cams),
                                    problems=[(r, list(s)) for r, s in job.problems], superpixels=job.superpixels)
                params = None if self.split_geom(job) else SimpleNamespace(split_sweep=0)
                pipe = ScenePipeline(scene, geom_iters=self.geom_iters, mode="batched",
                                     prior_threads=self.prior_threads, graphs=self.graphs, params=params)
            st.synchronize()
            pipe.prepare(st)
        except torch.OutOfMemoryError:
            if pipe is not None:
                pipe.close()
            pipe = scene = imgs = None
            self._free_streams.append(st)
            torch.cuda.empty_cache()
            if not self.active:
                raise
            return False
        job.admitted = self.now()
        need = max(need, torch.cuda.memory_allocated(self.device) - before)
        self.in_use += need
        self.active.append(_Active(job=job, pipe=pipe, stream=st, bytes=need))
        return True

    # ------------------------------------------------------------ stepping --
    def _record(self, a: _Active) -> None:
        a.event = torch.cuda.Event()
        a.event.record(a.stream)

    def _advance(self, a: _Active) -> bool:
        """Move one job forward if its pending work is done; True when finished."""
        if a.event is not None and not a.event.query():
            return False
        if a.host is not None and not a.host.done():
            return False
        if a.cancel:  # nothing of the job is in flight now
            a.job.error = Cancelled(f"job {a.job.job_id} cancelled")
            a.job.finished = self.now()
            return True
        p, st = a.pipe, a.stream
        if a.step == 0:  # random pass, then the depth/cost maps to the host
            p.random_pass(st)
            with torch.cuda.stream(st):
                a.pinned["depth"] = torch.empty(p.depth[0].shape, dtype=torch.float32, pin_memory=True)
                a.pinned["cost"] = torch.empty(p.cost[0].shape, dtype=torch.float32, pin_memory=True)
                a.pinned["depth"].copy_(p.depth[0], non_blocking=True)
                a.pinned["cost"].copy_(p.cost[0], non_blocking=True)
            self._record(a)
        elif a.step == 1:  # host triangulation
            a.event = None
            a.host = self.pool.submit(p.triangulate, a.pinned["depth"].numpy(), a.pinned["cost"].numpy())
        elif a.step == 2:  # prior pass, geometric passes, fusion, results to the host
            planes, masks = a.host.result()
            a.host = None
            p.upload_prior(planes, masks, st)
            p.prior_pass(st)
            buf = p.geom_passes(st)
            p.fusion(buf, st)
            with torch.cuda.stream(st):
                a.pinned["fd"] = torch.empty(p.fused_depth.shape, dtype=torch.float32, pin_memory=True)
                a.pinned["fn"] = torch.empty(p.fused_normal.shape, dtype=torch.float32, pin_memory=True)
                a.pinned["fd"].copy_(p.fused_depth, non_blocking=True)
                a.pinned["fn"].copy_(p.fused_normal, non_blocking=True)
                a.pinned["planes"] = torch.from_numpy(planes)  # kept alive until the copy is done
            self._record(a)
        else:
            a.job.result = (a.pinned["fd"].numpy().copy(), a.pinned["fn"].numpy().copy())
            a.job.finished = self.now()
            if a.job.output_dir:
                a.job.written = self.pool.submit(write_depth_normal, a.job)
            return True
        a.step += 1
        return False

    def _retire(self, a: _Active) -> None:
        a.pipe.close()
        self._free_streams.append(a.stream)
        self.in_use -= a.bytes
        self.active.remove(a)
        self.done.append(a.job)

    def poll(self) -> int:
        """Admit what fits and advance every active job once; returns the
        number of jobs still queued or active."""
        self._admit()
        for a in list(self.active):
            try:
                finished = self._advance(a)
            except BaseException as e:  # a failing job does not take the others down
                a.job.error = e
                a.job.finished = self.now()
                finished = True
            if finished:
                self._retire(a)
                self._admit()
        return len(self.queue) + len(self.active)

    def run(self, idle_sleep: float = 0.0005) -> List[Job]:
        """Serve until the queue is empty and every job has finished."""
        while self.poll():
            time.sleep(idle_sleep)
        return self.done

    def close(self) -> None:
        for a in list(self.active):
            a.pipe.close()
        self.active.clear()
        self.pool.shutdown(wait=True)


def write_depth_normal(job: Job) -> List[str]:
    """The fused maps of every reference view as {ref:04d}.npy [H, W, 4]
    float32 (depth, normal) in job.output_dir, the layout consistency.py
    writes (gmvs/consistency.py:199-210)."""
    import os

    os.makedirs(job.output_dir, exist_ok=True)
    fd, fn = job.result
    paths = []
    for ref, _ in job.problems:
        path = os.path.join(job.output_dir, f"{int(ref):04d}.npy")
        np.save(path, np.concatenate([fd[ref][..., None], fn[ref]], -1).astype(np.float32))
        paths.append(path)
    return paths


def latency_stats(jobs: List[Job]) -> dict:
    """p50/p99 per-view latency (ms) and sustained ref-views/s of served jobs."""
    per_view = []
    for j in jobs:
        if j.error is None and j.finished >= 0:
            per_view += [(j.finished - j.arrival) * 1000.0] * j.num_refs
    if not per_view:
        return {"views": 0}
    span = max(j.finished for j in jobs) - min(j.arrival for j in jobs)
    return {"views": len(per_view), "p50_ms": float(np.percentile(per_view, 50)),
            "p99_ms": float(np.percentile(per_view, 99)), "ref_views_per_s": len(per_view) / span if span > 0 else None}


def synthetic_job(job_id: int, seed: int, num_views: int, height: int, width: int, num_src: int,
                  arrival: float = 0.0, device=None) -> Job:
    """A room-scene job (seeded, rendered on `device`) with host images."""
    from . import synthetic
    from .engine import make_camera

    sc = synthetic.room_scene(seed, H=height, W=width, num_views=num_views, num_src=num_src, device=device)
    cams = [make_camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]
    problems = [(r, list(s)) for r, s in sc.problems if len(s) > 0]
    return Job(job_id=job_id, images=sc.images, cams=cams, problems=problems, superpixels=sc.superpixels,
               arrival=arrival)


def poisson_stream(num_jobs: int, rate: float, seed: int, sizes=((480, 640), (960, 1280), (1200, 1600)),
                   views=(8, 16), src=(4, 10), device=None) -> List[Job]:
    """Jobs with Poisson arrivals at `rate` jobs/s, uneven sizes and view
    counts drawn from numpy.random.default_rng(seed)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for i in range(num_jobs):
        t += float(rng.exponential(1.0 / rate))
        H, W = sizes[int(rng.integers(len(sizes)))]
        V = int(rng.integers(views[0], views[1] + 1))
        N = int(min(rng.integers(src[0], src[1] + 1), V - 1))
        jobs.append(synthetic_job(i, int(rng.integers(1 << 30)), V, H, W, N, arrival=t, device=device))
    return jobs
