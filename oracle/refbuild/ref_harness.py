"""Launch the reference's own module-B kernels (cubins built by build_ref.py
from gmvs/src/patch_match.cu and gmvs/src/fusion.cu) through the CUDA
driver API, with the launch sequence, shapes and buffers of
PatchMatcher::run_patch_match (gmvs/src/patch_match.cu:1353-1518) and
Fuser::run_fusion (gmvs/src/fusion.cu:211-275).  Test infrastructure only:
it produces golden vectors; nothing in the product uses it.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(os.path.dirname(HERE), "_ref")

_f, _i, _p = ctypes.c_float, ctypes.c_int32, ctypes.c_void_p


class Camera(ctypes.Structure):  # mvs::Camera (gmvs/include/data_structure.hpp:39-47)
    _fields_ = [("K", _f * 9), ("R", _f * 9), ("t", _f * 3), ("height", _i), ("width", _i), ("depth_min", _f),
                ("depth_max", _f)]


class Problem(ctypes.Structure):  # mvs::Problem (data_structure.hpp:33-37)
    _fields_ = [("num_ngb", _i), ("ref_image_id", _i), ("src_image_ids", _i * 32)]


class Params(ctypes.Structure):  # mvs::PatchMatchParams (data_structure.hpp:20-37)
    _fields_ = [("max_iterations", _i), ("patch_size", _i), ("num_images", _i), ("max_image_size", _i),
                ("radius_increment", _i), ("sigma_spatial", _f), ("sigma_color", _f), ("top_k", _i),
                ("baseline", _f), ("depth_min", _f), ("depth_max", _f), ("disparity_min", _f),
                ("disparity_max", _f), ("geom_consistency", ctypes.c_bool), ("multi_geometry", ctypes.c_bool),
                ("planar_prior", ctypes.c_bool)]


def default_params() -> Params:
    p = Params()
    p.max_iterations, p.patch_size, p.num_images, p.max_image_size, p.radius_increment = 3, 11, 5, 3200, 2
    p.sigma_spatial, p.sigma_color, p.top_k = 5.0, 3.0, 4
    p.baseline, p.depth_min, p.depth_max, p.disparity_min, p.disparity_max = 0.54, 0.0, 1.0, 0.0, 1.0
    return p


class Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._ck(self.cu.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self._ck(self.cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
        self.ctx = ctypes.c_void_p()
        self._ck(self.cu.cuDevicePrimaryCtxRetain(ctypes.byref(self.ctx), dev), "cuDevicePrimaryCtxRetain")
        self._ck(self.cu.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")
        self.cu.cuMemAlloc_v2.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_size_t]
        self.cu.cuMemcpyHtoD_v2.argtypes = [ctypes.c_uint64, _p, ctypes.c_size_t]
        self.cu.cuMemcpyDtoH_v2.argtypes = [_p, ctypes.c_uint64, ctypes.c_size_t]
        self.cu.cuMemsetD8_v2.argtypes = [ctypes.c_uint64, ctypes.c_ubyte, ctypes.c_size_t]
        self.cu.cuMemFree_v2.argtypes = [ctypes.c_uint64]
        self.cu.cuLaunchKernel.argtypes = [_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                           ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, _p,
                                           ctypes.POINTER(ctypes.c_void_p), _p]
        self.allocs = []
        self.funcs = {}
        for name in ("patch_match", "fusion"):
            self._load(os.path.join(REF_DIR, f"ref_{name}.cubin"))

    def _ck(self, rc, what):
        if rc != 0:
            msg = ctypes.c_char_p()
            self.cu.cuGetErrorString(rc, ctypes.byref(msg))
            raise RuntimeError(f"{what} failed: {rc} {msg.value}")

    def _load(self, path):
        mod = ctypes.c_void_p()
        self._ck(self.cu.cuModuleLoad(ctypes.byref(mod), path.encode()), f"cuModuleLoad {path}")
        n = ctypes.c_uint()
        self._ck(self.cu.cuModuleGetFunctionCount(ctypes.byref(n), mod), "cuModuleGetFunctionCount")
        fns = (ctypes.c_void_p * n.value)()
        self._ck(self.cu.cuModuleEnumerateFunctions(fns, n, mod), "cuModuleEnumerateFunctions")
        for f in fns:
            nm = ctypes.c_char_p()
            self._ck(self.cu.cuFuncGetName(ctypes.byref(nm), ctypes.c_void_p(f)), "cuFuncGetName")
            self.funcs[nm.value.decode()] = ctypes.c_void_p(f)

    def func(self, stem: str):
        key = f"{len(stem)}{stem}"
        hits = [k for k in self.funcs if key in k]
        if len(hits) != 1:
            raise RuntimeError(f"kernel {stem}: {hits}")
        return self.funcs[hits[0]]

    def alloc(self, nbytes: int) -> int:
        d = ctypes.c_uint64()
        self._ck(self.cu.cuMemAlloc_v2(ctypes.byref(d), max(int(nbytes), 4)), "cuMemAlloc")
        self.allocs.append(d.value)
        return d.value

    def put(self, arr: np.ndarray) -> int:
        a = np.ascontiguousarray(arr)
        d = self.alloc(a.nbytes)
        self._ck(self.cu.cuMemcpyHtoD_v2(d, a.ctypes.data, a.nbytes), "HtoD")
        return d

    def put_struct(self, s) -> int:
        d = self.alloc(ctypes.sizeof(s))
        self._ck(self.cu.cuMemcpyHtoD_v2(d, ctypes.addressof(s), ctypes.sizeof(s)), "HtoD")
        return d

    def get(self, d: int, shape, dtype) -> np.ndarray:
        out = np.empty(shape, dtype)
        self._ck(self.cu.cuMemcpyDtoH_v2(out.ctypes.data, d, out.nbytes), "DtoH")
        return out

    def launch(self, stem, grid, block, args):
        holders = []
        ptrs = (ctypes.c_void_p * len(args))()
        for k, a in enumerate(args):
            if isinstance(a, ctypes.Structure):
                h = a
            elif isinstance(a, bool):
                h = ctypes.c_bool(a)
            elif isinstance(a, (ctypes.c_int32, ctypes.c_bool, ctypes.c_uint64)):
                h = a
            else:
                h = ctypes.c_uint64(int(a))
            holders.append(h)
            ptrs[k] = ctypes.cast(ctypes.pointer(h), ctypes.c_void_p)
        g = tuple(grid) + (1,) * (3 - len(grid))
        b = tuple(block) + (1,) * (3 - len(block))
        self._ck(self.cu.cuLaunchKernel(self.func(stem), g[0], g[1], g[2], b[0], b[1], b[2], 0, None, ptrs, None),
                 f"launch {stem}")
        self._ck(self.cu.cuCtxSynchronize(), f"sync after {stem}")

    def free_all(self):
        for d in self.allocs:
            self.cu.cuMemFree_v2(d)
        self.allocs.clear()


def camera(K, R, t, h, w, dmin, dmax) -> Camera:
    c = Camera()
    for k in range(9):
        c.K[k], c.R[k] = K[k], R[k]
    for k in range(3):
        c.t[k] = t[k]
    c.height, c.width, c.depth_min, c.depth_max = h, w, dmin, dmax
    return c


def run_patch_match(drv: Driver, cams, ref: int, src, images, depths, normals, max_iterations: int,
                    timings: dict = None):
    """PatchMatcher::run_patch_match for one problem (patch_match.cu:1353-1518);
    images/depths [V, H, W] and normals [V, H, W, 3] are indexed by view id.
    `timings` (optional) receives the seconds spent in uploads, kernels
    (each followed by the reference's cudaDeviceSynchronize) and downloads."""
    import time

    t0 = time.perf_counter()
    V, H, W = images.shape
    p = default_params()
    p.max_iterations = max_iterations
    p.geom_consistency = True
    p.num_images = len(src) + 1
    p.depth_min = cams[ref].depth_min * 0.6
    p.depth_max = cams[ref].depth_max * 1.2
    ids = [ref] + list(src)
    d_img = drv.put(images[ids].astype(np.float32))
    d_dep = drv.put(depths[ids].astype(np.float32))
    d_nrm = drv.put(normals[ids].astype(np.float32))
    cam_arr = (Camera * len(ids))(*[cams[i] for i in ids])
    d_cam = drv.alloc(ctypes.sizeof(cam_arr))
    drv._ck(drv.cu.cuMemcpyHtoD_v2(d_cam, ctypes.addressof(cam_arr), ctypes.sizeof(cam_arr)), "HtoD")
    d_plane = drv.alloc(16 * H * W)
    d_rand = drv.alloc(64 * H * W)
    d_sel = drv.alloc(4 * H * W)
    d_cost = drv.alloc(4 * H * W)
    g16 = ((W + 15) // 16, (H + 15) // 16)
    gcb = ((W + 15) // 16, ((H // 2) + 15) // 16)
    drv._ck(drv.cu.cuCtxSynchronize(), "sync")
    t1 = time.perf_counter()
    drv.launch("initialization", g16, (16, 16), [d_img, d_dep, d_nrm, d_cam, d_plane, d_cost, d_rand, d_sel, p])
    for i in range(max_iterations):
        for black in (True, False):
            drv.launch("black_red_pixel_update", gcb, (16, 16),
                       [d_img, d_dep, d_cam, d_plane, d_cost, d_rand, d_sel, p, ctypes.c_int32(i), bool(black)])
    drv.launch("get_depth_and_normal", g16, (16, 16), [d_cam, d_plane, p])
    drv.launch("black_red_pixel_filter", gcb, (16, 16), [d_cam, d_plane, d_cost, True])
    drv.launch("black_red_pixel_filter", gcb, (16, 16), [d_cam, d_plane, d_cost, False])
    od, on, oc = drv.alloc(4 * H * W), drv.alloc(12 * H * W), drv.alloc(4 * H * W)
    drv.launch("export_plane_hypotheses_cost", (((H * W) - 1) // 256 + 1,), (256,),
               [d_plane, d_cost, ctypes.c_int32(H), ctypes.c_int32(W), od, on, oc])
    t2 = time.perf_counter()
    out = (drv.get(od, (H, W), np.float32), drv.get(on, (H, W, 3), np.float32), drv.get(oc, (H, W), np.float32))
    drv.free_all()
    if timings is not None:
        timings["upload_s"] = timings.get("upload_s", 0.0) + (t1 - t0)
        timings["kernels_s"] = timings.get("kernels_s", 0.0) + (t2 - t1)
        timings["download_s"] = timings.get("download_s", 0.0) + (time.perf_counter() - t2)
    return out


def run_fusion(drv: Driver, cams, problems, depths, normals, geom_consistent: int):
    """Fuser::run_fusion for every problem in order (fusion.cu:211-275) with a
    shared mask buffer; returns per-view (depth, normal) and the final masks."""
    V, H, W = depths.shape
    d_masks = drv.alloc(V * H * W)
    drv._ck(drv.cu.cuMemsetD8_v2(d_masks, 0, V * H * W), "memset")
    outs = []
    for ref, src in problems:
        ids = [ref] + list(src)
        d_dep = drv.put(depths[ids].astype(np.float32))
        d_nrm = drv.put(normals[ids].astype(np.float32))
        cam_arr = (Camera * len(ids))(*[cams[i] for i in ids])
        d_cam = drv.alloc(ctypes.sizeof(cam_arr))
        drv._ck(drv.cu.cuMemcpyHtoD_v2(d_cam, ctypes.addressof(cam_arr), ctypes.sizeof(cam_arr)), "HtoD")
        pb = Problem()
        pb.num_ngb, pb.ref_image_id = len(src), ref
        for k, s in enumerate(src):
            pb.src_image_ids[k] = s
        d_pb = drv.put_struct(pb)
        od, on = drv.alloc(4 * H * W), drv.alloc(12 * H * W)
        drv._ck(drv.cu.cuMemsetD8_v2(od, 0, 4 * H * W), "memset")
        drv._ck(drv.cu.cuMemsetD8_v2(on, 0, 12 * H * W), "memset")
        drv.launch("batch_fusion_kernel", (((H * W) - 1) // 256 + 1,), (256,),
                   [d_dep, d_nrm, d_masks, d_cam, d_pb, ctypes.c_int32(geom_consistent), ctypes.c_int32(H),
                    ctypes.c_int32(W), od, on])
        outs.append((drv.get(od, (H, W), np.float32), drv.get(on, (H, W, 3), np.float32)))
    masks = drv.get(d_masks, (V, H, W), np.uint8)
    drv.free_all()
    return outs, masks
