"""Autotuner: the launch-shape knobs it turns leave results unchanged bit for
bit (GPU), and its cache round-trips through the JSON file (CPU)."""

import json

import numpy as np
import pytest

from gmvs_gb300 import _abi, autotune


def test_candidates_cover_tile_shapes_and_split():
    # 16x8, 16x16, 32x8 and 32x16 pixel tiles, half-sweeps as one, two or three kernels
    assert {(c[3], 2 * c[0]) for c in autotune.CANDIDATES} == {(16, 8), (16, 16), (32, 8), (32, 16)}
    assert {c[2] for c in autotune.CANDIDATES} == {0, 1, 2}
    p = autotune.TuneResult("k", (4, 0, 1, 32)).apply(_abi.default_params())
    assert (p.tile_h, p.ctas_per_sm, p.split_sweep, p.tile_w) == (4, 0, 1, 32)


def test_cache_file_round_trip(tmp_path, gmvs_lib):
    path = str(tmp_path / "tune.json")
    t = autotune.Autotuner(cache_path=path)
    t.cache["k"] = autotune.TuneResult("k", (8, 3, 1), {"8,3,1": 1.0, "4,0,0": 2.0})
    t._save()
    t2 = autotune.Autotuner(cache_path=path)
    assert t2.cache["k"].best == (8, 3, 1) and t2.cache["k"].ms["4,0,0"] == 2.0
    p = t2.cache["k"].apply(_abi.default_params())
    assert (p.tile_h, p.ctas_per_sm, p.split_sweep) == (8, 3, 1)
    assert json.load(open(path))["k"]["best"] == [8, 3, 1]


@pytest.mark.gpu
def test_launch_shape_does_not_change_results(gmvs_lib, small, cuda):
    from gmvs_gb300 import engine
    from scenes import gpu_view

    ref, src = small.problems[0]
    ids = [ref] + list(src)
    outs = {}
    for sampler, staging in ((_abi.SAMPLER_TEX, _abi.STAGE_AUTO), (_abi.SAMPLER_CLAMP, _abi.STAGE_QUAD_F16)):
        for th, c, tw in ((4, 0, 0), (2, 3, 0), (8, 2, 0), (1, 1, 0), (4, 0, 32), (8, 0, 32)):
            v = gpu_view(small, ids, cuda, 0.3, 6.0)
            v.allocate_outputs(with_planes=True)
            p = engine.params_struct(sampler=sampler, staging=staging, tile_h=th, ctas_per_sm=c,
                                     split_sweep=int(th == 8), tile_w=tw)
            engine.run_passes([v], p, engine.Workspace())
            outs[(sampler, th, c, tw)] = (v.out_depth.cpu().numpy(), v.out_cost.cpu().numpy(),
                                          v.out_planes.cpu().numpy())
        base = outs[(sampler, 4, 0, 0)]
        for (s, th, c, tw), o in outs.items():
            if s != sampler:
                continue
            for a, b in zip(o, base):
                assert np.array_equal(a, b, equal_nan=True), (sampler, th, c, tw)


@pytest.mark.gpu
def test_tuner_picks_a_candidate(gmvs_lib, small, cuda):
    from scenes import gpu_view
    from gmvs_gb300 import engine

    ref, src = small.problems[0]
    v = gpu_view(small, [ref] + list(src), cuda, 0.3, 6.0)
    v.allocate_outputs()
    t = autotune.Autotuner(candidates=((4, 0, 0), (8, 0, 1), (2, 3, 0)), reps=1)
    r = t.tune([v], engine.params_struct())
    assert r.best in ((4, 0, 0), (8, 0, 1), (2, 3, 0)) and len(r.ms) == 3 and all(ms > 0 for ms in r.ms.values())
    assert t.tune([v], engine.params_struct()) is r  # cached


def test_pick_breaks_ties_toward_taller_narrower_tiles():
    ms = {"4,0,0,16": 947.3, "4,0,1,16": 985.7, "8,0,0,16": 948.0, "4,0,0,32": 948.6, "8,0,0,32": 948.2}
    assert autotune.pick(ms) == "8,0,0,16"  # all four single-kernel shapes tie within 0.5 %
    assert autotune.pick({"4,0,2,16": 800.0, "8,0,2,16": 812.0, "8,0,0,16": 1160.0}) == "4,0,2,16"  # no tie
    assert autotune.pick({"8,0,1,16": 100.0, "8,0,2,16": 100.2}) == "8,0,1,16"  # tie: fewer kernels
