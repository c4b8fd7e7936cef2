"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes binding of the CPU restatement of the reference PatchMatch MVS path
(oracle.cpp, oracle_prior.cpp).  Only tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg use it, as the checker; the gmvs_gb300 package
never imports it.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")

_f, _i, _p = ctypes.c_float, ctypes.c_int32, ctypes.c_void_p


class oracle_params(ctypes.Structure):
    _fields_ = [("max_iterations", _i), ("patch_size", _i), ("radius_increment", _i), ("sigma_spatial", _f),
                ("sigma_color", _f), ("top_k", _i), ("depth_min", _f), ("depth_max", _f), ("init_kind", _i),
                ("sweep_kind", _i), ("sampler", _i), ("run_filter", _i), ("seed", ctypes.c_uint64),
                ("pass_index", _i), ("stream_id", _i), ("fp64", _i), ("max_half_sweeps", _i)]


class OCamera(ctypes.Structure):
    _fields_ = [("K", _f * 9), ("R", _f * 9), ("t", _f * 3), ("height", _i), ("width", _i), ("depth_min", _f),
                ("depth_max", _f)]


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("oracle.cpp", "oracle_prior.cpp", "Makefile")]
    if force or not os.path.exists(LIB_PATH) or any(os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in srcs):
        r = subprocess.run(["make", "-C", HERE, "-B" if force else "-s"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"building the oracle failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(oracle_params)
        sigs = {
            "oracle_philox4x32_10": (None, [_p, _p, _p]),
            "oracle_u01": (_f, [ctypes.c_uint32]),
            "oracle_ncc_costs": (_i, [_p, _i, _i, _i, _p, P, _p, _p, _p, _p, _i, _i]),
            "oracle_run_pass": (_i, [_p, _i, _i, _i, _p, _p, _p, _p, _p, _p, _p, P, _p, _p, _p, _p, _i]),
            "oracle_fuse": (_i, [_p, _i, _i, _p, _i, _i, _p, _p, _p, _i, _f, _p, _p, _p, _p]),
            "oracle_build_prior": (_i, [_p, _i, _i, _p, _p, _p, _i, _f, _f, _p, _p, ctypes.POINTER(_i), _p, _i]),
            "oracle_delaunay": (_i, [_p, _i, _i, _p, _i]),
            "oracle_fusion_planar_mask": (_i, [_p, _p, _p, _i, _i, _i, _f, _f, _f, _p]),
            "oracle_filter_by_var_map": (_i, [_p, _p, _i, _i, _f, _p]),
            "oracle_sliding_window_normal": (_i, [_p, _p, _i, _i, _i, _p]),
            "oracle_pm_expf": (_f, [_f]),
            "oracle_pm_sinf": (_f, [_f]),
            "oracle_pm_cosf": (_f, [_f]),
            "oracle_pm_acosf": (_f, [_f]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _np_ptr(a):
    return None if a is None else a.ctypes.data


def cameras(cam_args) -> ctypes.Array:
    """cam_args: list of (K[9], R[9], t[3], h, w, dmin, dmax)."""
    arr = (OCamera * len(cam_args))()
    for i, (K, R, t, h, w, dmin, dmax) in enumerate(cam_args):
        for k in range(9):
            arr[i].K[k] = K[k]
            arr[i].R[k] = R[k]
        for k in range(3):
            arr[i].t[k] = t[k]
        arr[i].height, arr[i].width = h, w
        arr[i].depth_min, arr[i].depth_max = dmin, dmax
    return arr


def make_params(**kw) -> oracle_params:
    p = oracle_params()
    p.max_iterations, p.patch_size, p.radius_increment = 3, 11, 2
    p.sigma_spatial, p.sigma_color, p.top_k = 5.0, 3.0, 4
    p.depth_min, p.depth_max = 0.0, 1.0
    p.init_kind, p.sweep_kind, p.sampler, p.run_filter = 0, 0, 0, 1
    p.seed, p.pass_index, p.stream_id = 3407, 0, 0
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def philox4x32_10(ctr, key) -> np.ndarray:
    c = (ctypes.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    k = (ctypes.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (ctypes.c_uint32 * 4)()
    lib().oracle_philox4x32_10(c, k, o)
    return np.array(list(o), dtype=np.uint32)


def pm(name: str, xs) -> np.ndarray:
    """The shared elementary function `name` (expf, sinf, cosf, acosf) on xs."""
    fn = getattr(lib(), f"oracle_pm_{name}")
    return np.array([fn(float(x)) for x in np.asarray(xs, np.float32)], np.float32)


def u01(x: int) -> float:
    return float(lib().oracle_u01(int(x) & 0xFFFFFFFF))


def ncc_costs(cam_args, images: np.ndarray, planes: np.ndarray, params: oracle_params, fp64: bool = False,
              nthreads: int = 0, ref_chain: bool = False):
    """images: float32 [1+N, H, W]; planes: float32 [H, W, 4] camera frame.
    fp64: the FP64 oracle; ref_chain: the reference's own fp32 operation
    chain instead of the shared formulation.
    Returns (costs [N, H, W], init_cost [H, W], init_views [H, W] uint32)."""
    imgs = np.ascontiguousarray(images, np.float32)
    n1, H, W = imgs.shape
    pl = np.ascontiguousarray(planes, np.float32)
    costs = np.zeros((n1 - 1, H, W), np.float32)
    ic = np.zeros((H, W), np.float32)
    iv = np.zeros((H, W), np.uint32)
    cams = cameras(cam_args)
    rc = lib().oracle_ncc_costs(cams, n1 - 1, H, W, _np_ptr(imgs), ctypes.byref(params), _np_ptr(pl),
                                _np_ptr(costs), _np_ptr(ic), _np_ptr(iv), 2 if ref_chain else int(fp64), nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle_ncc_costs failed ({rc})")
    return costs, ic, iv


def run_pass(cam_args, images: np.ndarray, params: oracle_params, depths=None, ref_normal=None, prior_planes=None,
             prior_masks=None, init_planes=None, init_costs=None, nthreads: int = 0):
    """One full pass; returns (depth, normal, cost, planes)."""
    imgs = np.ascontiguousarray(images, np.float32)
    n1, H, W = imgs.shape
    c32 = lambda a: None if a is None else np.ascontiguousarray(a, np.float32)
    dep, rn, pp, ip, icst = c32(depths), c32(ref_normal), c32(prior_planes), c32(init_planes), c32(init_costs)
    pm = None if prior_masks is None else np.ascontiguousarray(prior_masks, np.uint32)
    od = np.zeros((H, W), np.float32)
    on = np.zeros((H, W, 3), np.float32)
    oc = np.zeros((H, W), np.float32)
    op = np.zeros((H, W, 4), np.float32)
    cams = cameras(cam_args)
    rc = lib().oracle_run_pass(cams, n1 - 1, H, W, _np_ptr(imgs), _np_ptr(dep), _np_ptr(rn), _np_ptr(pp),
                               _np_ptr(pm), _np_ptr(ip), _np_ptr(icst), ctypes.byref(params), _np_ptr(od),
                               _np_ptr(on), _np_ptr(oc), _np_ptr(op), nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle_run_pass failed ({rc})")
    return od, on, oc, op


def cos_threshold() -> float:
    """Largest float32 c with acos(c) >= float32(0.174533) (see oracle_fuse)."""
    T = float(np.float32(0.174533))
    c = np.float32(np.cos(T))
    while np.arccos(np.float64(c)) < T:
        c = np.nextafter(c, np.float32(-2))
    while np.arccos(np.float64(np.nextafter(c, np.float32(2)))) >= T:
        c = np.nextafter(c, np.float32(2))
    return float(c)


def fuse(cam_args, ref_id: int, src_ids, depths: np.ndarray, normals: np.ndarray, masks: np.ndarray,
         geom_consistent: int, with_hits: bool = False):
    """Fusion of one reference view.  depths [1+N, H, W], normals [1+N, H, W, 3]
    (ref, then sources), masks uint8 [V, H, W] updated in place.
    Returns (depth, normal, count); with_hits=True adds the number of
    reference pixels written to each output pixel (> 1: a collision)."""
    d = np.ascontiguousarray(depths, np.float32)
    n = np.ascontiguousarray(normals, np.float32)
    assert masks.dtype == np.uint8 and masks.flags.c_contiguous
    n1, H, W = d.shape
    ids = np.ascontiguousarray(src_ids, np.int32)
    od = np.zeros((H, W), np.float32)
    on = np.zeros((H, W, 3), np.float32)
    cnt = np.zeros((H, W), np.int32)
    hits = np.zeros((H, W), np.int32)
    cams = cameras(cam_args)
    rc = lib().oracle_fuse(cams, n1 - 1, int(ref_id), _np_ptr(ids), H, W, _np_ptr(d), _np_ptr(n), _np_ptr(masks),
                           int(geom_consistent), ctypes.c_float(cos_threshold()), _np_ptr(od), _np_ptr(on),
                           _np_ptr(cnt), _np_ptr(hits))
    if rc != 0:
        raise RuntimeError(f"oracle_fuse failed ({rc})")
    return (od, on, cnt, hits) if with_hits else (od, on, cnt)


def build_prior(cam_arg, depth: np.ndarray, cost: np.ndarray, superpixel, superpixel_filter: bool,
                depth_min: float, depth_max: float):
    d = np.ascontiguousarray(depth, np.float32)
    H, W = d.shape
    c = np.ascontiguousarray(cost, np.float32)
    sp = None if superpixel is None else np.ascontiguousarray(superpixel, np.uint8)
    planes = np.zeros((H, W, 4), np.float32)
    masks = np.zeros((H, W), np.uint32)
    max_tris = 2 * ((W + 4) // 5) * ((H + 4) // 5) + 16
    tris = np.zeros((max_tris, 3, 2), np.int32)
    count = ctypes.c_int32(0)
    cams = cameras([cam_arg])
    rc = lib().oracle_build_prior(cams, H, W, _np_ptr(d), _np_ptr(c), _np_ptr(sp), int(bool(superpixel_filter)),
                                  ctypes.c_float(depth_min), ctypes.c_float(depth_max), _np_ptr(planes),
                                  _np_ptr(masks), ctypes.byref(count), _np_ptr(tris), max_tris)
    if rc != 0:
        raise RuntimeError(f"oracle_build_prior failed ({rc})")
    return planes, masks, tris[:count.value]


def delaunay(xy: np.ndarray, extent: int) -> np.ndarray:
    pts = np.ascontiguousarray(xy, np.int32)
    n = pts.shape[0]
    out = np.zeros((2 * n + 16, 3), np.int32)
    k = lib().oracle_delaunay(_np_ptr(pts), n, int(extent), _np_ptr(out), out.shape[0])
    return out[:k]


def fusion_planar_mask(seg, planar, normals, rows, cols, thresh=100, nonplanar_percent=0.75, cos_sim_thresh=0.8,
                       match_ratio_thresh=0.9):
    s = np.ascontiguousarray(seg, np.int32)
    m = np.ascontiguousarray(planar, np.int32)
    n = np.ascontiguousarray(normals, np.float32)
    out = np.zeros((rows, cols), np.int32)
    lib().oracle_fusion_planar_mask(_np_ptr(s), _np_ptr(m), _np_ptr(n), rows, cols, thresh,
                                    ctypes.c_float(nonplanar_percent), ctypes.c_float(cos_sim_thresh),
                                    ctypes.c_float(match_ratio_thresh), _np_ptr(out))
    return out


def filter_by_var_map(var_map, seg, var_thresh):
    v = np.ascontiguousarray(var_map, np.float32)
    s = np.ascontiguousarray(seg, np.int32)
    rows, cols = v.shape
    out = np.zeros((rows, cols), np.int32)
    lib().oracle_filter_by_var_map(_np_ptr(v), _np_ptr(s), rows, cols, ctypes.c_float(var_thresh), _np_ptr(out))
    return out


def sliding_window_normal(region, normals, win):
    r = np.ascontiguousarray(region, np.int32)
    n = np.ascontiguousarray(normals, np.float32)
    rows, cols = r.shape
    out = np.zeros((rows, cols, 3), np.float32)
    lib().oracle_sliding_window_normal(_np_ptr(r), _np_ptr(n), rows, cols, int(win), _np_ptr(out))
    return out
