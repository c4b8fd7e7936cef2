"""Serving form: admission by device-memory footprint and arrival order (CPU,
with the device work stood in for), and on the GPU the same fused maps for
a job served alone, served in a mix of concurrent jobs, and run directly
through ScenePipeline."""

import numpy as np
import pytest
import torch

from gmvs_gb300 import serving


class _StandIn(serving.ReconstructionServer):
    """The scheduler of ReconstructionServer with the device work replaced
    by a job that takes `steps` polls to finish."""

    steps = 3

    def __init__(self, **kw):
        super().__init__(device=torch.device("cpu"), **kw)
        self.peak = 0
        self.order = []

    def _start(self, job, need):
        job.admitted = self.now()
        self.in_use += need
        self.peak = max(self.peak, self.in_use)
        self.order.append(job.job_id)
        self.active.append(serving._Active(job=job, pipe=None, stream=None, bytes=need))

    def _advance(self, a):
        if a.cancel:
            a.job.error = serving.Cancelled("cancelled")
            a.job.finished = self.now()
            return True
        a.step += 1
        if a.step >= self.steps:
            a.job.finished = self.now()
            return True
        return False

    def _retire(self, a):
        self.in_use -= a.bytes
        self.active.remove(a)
        self.done.append(a.job)


def _job(i, V=5, H=64, W=80, arrival=0.0):
    return serving.Job(job_id=i, images=np.zeros((V, H, W), np.uint8), cams=[None] * V,
                       problems=[(0, [1, 2])] * V, arrival=arrival)


def test_malformed_jobs_are_rejected_at_submission():
    srv = _StandIn(memory_budget=1 << 40)
    bad = [
        serving.Job(0, np.zeros((5, 8), np.uint8), [None] * 5, [(0, [1])]),          # not [V, H, W]
        serving.Job(1, np.zeros((5, 8, 8), np.uint8), [None] * 4, [(0, [1])]),       # a camera missing
        serving.Job(2, np.zeros((5, 8, 8), np.uint8), [None] * 5, []),               # no reference view
        serving.Job(3, np.zeros((5, 8, 8), np.uint8), [None] * 5, [(0, [5])]),       # source out of range
        serving.Job(4, np.zeros((5, 8, 8), np.uint8), [None] * 5, [(0, [0, 1])]),    # reference among sources
        serving.Job(5, np.zeros((5, 8, 8), np.uint8), [None] * 5, [(0, [])]),        # no source view
        serving.Job(6, np.zeros((5, 8, 8), np.uint8), [None] * 5, [(0, [1])],
                    superpixels=np.zeros((5, 4, 4), np.uint8)),                      # superpixels of another size
    ]
    for job in bad:
        with pytest.raises(ValueError):
            srv.submit(job)
    assert not srv.queue
    srv.close()


def test_cancel_queued_and_active_jobs():
    srv = _StandIn(memory_budget=1 << 40, max_active=1)
    srv.steps = 4
    for i in range(3):
        srv.submit(_job(i))
    srv.poll()                       # job 0 admitted and stepping
    assert srv.cancel(2) and srv.cancel(0) and not srv.cancel(99)
    done = srv.run(idle_sleep=0)
    by_id = {j.job_id: j for j in done}
    assert isinstance(by_id[0].error, serving.Cancelled) and isinstance(by_id[2].error, serving.Cancelled)
    assert by_id[1].error is None and by_id[1].finished >= 0
    assert srv.in_use == 0 and srv.order == [0, 1]
    srv.close()


def test_admission_by_footprint_and_arrival_order():
    one = _job(0).footprint(2)
    srv = _StandIn(memory_budget=int(2.5 * one), max_active=8)
    for i in range(6):
        srv.submit(_job(i))
    done = srv.run(idle_sleep=0)
    assert [j.job_id for j in done] == list(range(6))
    assert srv.order == list(range(6))
    assert srv.peak <= srv.budget and srv.peak == 2 * one  # two fit, the third waits for memory
    assert srv.in_use == 0
    srv.close()


def test_slots_and_future_arrivals():
    srv = _StandIn(memory_budget=1 << 40, max_active=2)
    srv.submit(_job(0))
    srv.submit(_job(1, arrival=0.05))
    srv.submit(_job(2))
    done = srv.run(idle_sleep=0.001)
    assert srv.order == [0, 2, 1]  # job 1 has not arrived when 0 and 2 are admitted
    assert all(j.admitted >= j.arrival for j in done)
    srv.close()


def test_large_jobs_run_single_kernel_geometric_half_sweeps():
    """The split geometric half-sweeps' scratch grows with all of a job's
    reference pixels; a job whose split footprint would take more than half
    the budget runs single kernels and is admitted with the smaller footprint."""
    job = _job(0)
    split, single = job.footprint(2, True), job.footprint(2, False)
    assert single < split
    small = _StandIn(memory_budget=int(1.5 * split))
    assert not small.split_geom(job) and small._need(job) == single
    big = _StandIn(memory_budget=4 * split)
    assert big.split_geom(job) and big._need(job) == split
    small.close()
    big.close()


def test_oversized_job_is_refused():
    srv = _StandIn(memory_budget=1 << 20)
    with pytest.raises(ValueError):
        srv.submit(_job(0))
    srv.close()


def test_footprint_formula():
    # linear in the views and the reference views, positive fixed part
    a = serving.footprint_bytes(10, 100, 100, 10, max_src=4, sms=152)
    b = serving.footprint_bytes(20, 100, 100, 20, max_src=4, sms=152)
    c = serving.footprint_bytes(0, 100, 100, 0, max_src=4, sms=152)
    assert c > 0 and b - a == a - c
    assert serving.footprint_bytes(10, 100, 100, 10, max_src=8, sms=152) > a


def _scene_job(job_id, seed, H, W, arrival=0.0):
    from gmvs_gb300 import engine, synthetic

    sc = synthetic.small_scene(seed, H=H, W=W)
    cams = [engine.make_camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]
    return serving.Job(job_id=job_id, images=sc.images, cams=cams, problems=[(r, list(s)) for r, s in sc.problems],
                       superpixels=sc.superpixels, arrival=arrival)


@pytest.mark.gpu
def test_same_result_alone_in_mix_and_direct(gmvs_lib, cuda, tmp_path):
    from gmvs_gb300.pipeline import SceneInputs, ScenePipeline

    a = _scene_job(0, 0, 256, 320)
    a.output_dir = str(tmp_path / "depth_normal")
    srv = serving.ReconstructionServer(device=cuda, max_active=1, prior_threads=4)
    srv.submit(a)
    srv.run()
    srv.close()
    assert a.error is None, a.error
    alone = a.result
    # the reference's file layout: {ref:04d}.npy [H, W, 4] = (depth, normal)
    paths = a.written.result()
    assert len(paths) == a.num_refs
    ref0 = a.problems[0][0]
    saved = np.load(paths[0])
    assert saved.shape == (256, 320, 4) and np.array_equal(saved[..., 0], alone[0][ref0])

    a2 = _scene_job(0, 0, 256, 320)
    mix = [a2, _scene_job(1, 1, 192, 256), _scene_job(2, 2, 256, 320, arrival=0.01)]
    srv = serving.ReconstructionServer(device=cuda, max_active=3, prior_threads=4)
    for j in mix:
        srv.submit(j)
    srv.run()
    srv.close()
    assert all(j.error is None for j in mix), [j.error for j in mix]
    for k in range(2):
        assert np.array_equal(a2.result[k], alone[k], equal_nan=True)
    stats = serving.latency_stats(mix)
    assert stats["views"] == sum(j.num_refs for j in mix) and stats["p99_ms"] >= stats["p50_ms"] > 0

    scene = SceneInputs(images=torch.from_numpy(a.images.astype(np.float32)).to(cuda), cams=a.cams,
                        problems=a.problems, superpixels=a.superpixels)
    pipe = ScenePipeline(scene, prior_threads=4)
    fd, fn = pipe.run()
    torch.cuda.synchronize()
    assert np.array_equal(fd.cpu().numpy(), alone[0], equal_nan=True)
    assert np.array_equal(fn.cpu().numpy(), alone[1], equal_nan=True)
    pipe.close()

    # the footprint bound covers what a job really holds
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    base = torch.cuda.memory_allocated(cuda)
    torch.cuda.reset_peak_memory_stats(cuda)
    b = _scene_job(3, 0, 256, 320)
    srv = serving.ReconstructionServer(device=cuda, max_active=1, prior_threads=4)
    srv.submit(b)
    srv.run()
    srv.close()
    used = torch.cuda.max_memory_allocated(cuda) - base
    assert used <= b.footprint(2), (used, b.footprint(2))


@pytest.mark.gpu
def test_graph_replay_matches_direct_launches(gmvs_lib, cuda):
    from gmvs_gb300 import engine, synthetic
    from gmvs_gb300.pipeline import ScenePipeline, scene_inputs_from_synthetic

    sc = synthetic.small_scene(0)
    outs = []
    for graphs in (False, True):
        pipe = ScenePipeline(scene_inputs_from_synthetic(sc, cuda), prior_threads=4, graphs=graphs)
        pipe.run()
        pipe.run()  # a second replay of the same graphs
        torch.cuda.synchronize()
        outs.append((pipe.fused_depth.cpu().numpy(), pipe.fused_normal.cpu().numpy()))
        pipe.close()
    for k in range(2):
        assert np.array_equal(outs[0][k], outs[1][k], equal_nan=True)
