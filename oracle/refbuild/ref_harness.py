"""Launch the reference's own kernels through the CUDA driver API, from
cubins that build_ref.py compiles out of the reference sources:

  module B (gmvs/src/patch_match.cu, gmvs/src/fusion.cu) with the launch
  sequence, shapes and buffers of PatchMatcher::run_patch_match
  (gmvs/src/patch_match.cu:1353-1518) and Fuser::run_fusion
  (gmvs/src/fusion.cu:211-275);

  module A (gmvs/lib/src/patch_match_kernel.cu) with PlanarInit's device
  state (cuda_space_init, gmvs/lib/src/planar_initer.cu:119-193: one float
  CUDA array per image behind a texture object with Wrap addressing, linear
  filtering and unnormalised coordinates; cuda_planar_prior_init, :195-223)
  and launcher (PlanarInit::run_patch_match, patch_match_kernel.cu:1711-1809).

Test and measurement infrastructure only: it produces golden vectors and
times the reference's plain per-view GPU path; nothing in the product uses it.
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


class ParamsA(ctypes.Structure):  # module A's PatchMatchParams (gmvs/lib/include/planar_initer.hpp:13-31)
    _fields_ = Params._fields_ + [("superpixel_filter", ctypes.c_bool)]


class ArrayDesc(ctypes.Structure):  # CUDA_ARRAY_DESCRIPTOR (cuda.h)
    _fields_ = [("Width", ctypes.c_size_t), ("Height", ctypes.c_size_t), ("Format", ctypes.c_int),
                ("NumChannels", ctypes.c_uint)]


class Memcpy2D(ctypes.Structure):  # CUDA_MEMCPY2D (cuda.h)
    _fields_ = [("srcXInBytes", ctypes.c_size_t), ("srcY", ctypes.c_size_t), ("srcMemoryType", ctypes.c_int),
                ("srcHost", _p), ("srcDevice", ctypes.c_uint64), ("srcArray", _p), ("srcPitch", ctypes.c_size_t),
                ("dstXInBytes", ctypes.c_size_t), ("dstY", ctypes.c_size_t), ("dstMemoryType", ctypes.c_int),
                ("dstHost", _p), ("dstDevice", ctypes.c_uint64), ("dstArray", _p), ("dstPitch", ctypes.c_size_t),
                ("WidthInBytes", ctypes.c_size_t), ("Height", ctypes.c_size_t)]


class ResourceDesc(ctypes.Structure):  # CUDA_RESOURCE_DESC (cuda.h): type, 128-byte union, flags
    _fields_ = [("resType", ctypes.c_int), ("res", ctypes.c_uint64 * 16), ("flags", ctypes.c_uint)]


class TextureDesc(ctypes.Structure):  # CUDA_TEXTURE_DESC (cuda.h)
    _fields_ = [("addressMode", ctypes.c_int * 3), ("filterMode", ctypes.c_int), ("flags", ctypes.c_uint),
                ("maxAnisotropy", ctypes.c_uint), ("mipmapFilterMode", ctypes.c_int),
                ("mipmapLevelBias", ctypes.c_float), ("minMipmapLevelClamp", ctypes.c_float),
                ("maxMipmapLevelClamp", ctypes.c_float), ("borderColor", ctypes.c_float * 4),
                ("reserved", ctypes.c_int * 12)]


CU_AD_FORMAT_FLOAT, CU_MEMORYTYPE_HOST, CU_MEMORYTYPE_ARRAY = 0x20, 1, 3
CU_RESOURCE_TYPE_ARRAY, CU_TR_ADDRESS_MODE_WRAP, CU_TR_FILTER_MODE_LINEAR = 0, 0, 1
MAX_IMAGES = 1024  # cudaTextureObjects (gmvs/lib/include/planar_initer.cuh:36-38)


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
        self.cu.cuArrayCreate_v2.argtypes = [ctypes.POINTER(_p), ctypes.POINTER(ArrayDesc)]
        self.cu.cuArrayDestroy.argtypes = [_p]
        self.cu.cuMemcpy2D_v2.argtypes = [ctypes.POINTER(Memcpy2D)]
        self.cu.cuTexObjectCreate.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ResourceDesc),
                                              ctypes.POINTER(TextureDesc), _p]
        self.cu.cuTexObjectDestroy.argtypes = [ctypes.c_uint64]
        self.allocs = []
        self.funcs = {}  # module name -> {mangled kernel name: function}
        for name in ("patch_match", "fusion", "planar", "planar_ieee", "patch_match_ieee", "fusion_ieee"):
            path = os.path.join(REF_DIR, f"ref_{name}.cubin")
            if name in ("patch_match", "fusion") or os.path.exists(path):
                self._load(name, path)

    def _ck(self, rc, what):
        if rc != 0:
            msg = ctypes.c_char_p()
            self.cu.cuGetErrorString(rc, ctypes.byref(msg))
            raise RuntimeError(f"{what} failed: {rc} {msg.value}")

    def _load(self, module, path):
        mod = ctypes.c_void_p()
        self._ck(self.cu.cuModuleLoad(ctypes.byref(mod), path.encode()), f"cuModuleLoad {path}")
        n = ctypes.c_uint()
        self._ck(self.cu.cuModuleGetFunctionCount(ctypes.byref(n), mod), "cuModuleGetFunctionCount")
        fns = (ctypes.c_void_p * n.value)()
        self._ck(self.cu.cuModuleEnumerateFunctions(fns, n, mod), "cuModuleEnumerateFunctions")
        for f in fns:
            nm = ctypes.c_char_p()
            self._ck(self.cu.cuFuncGetName(ctypes.byref(nm), ctypes.c_void_p(f)), "cuFuncGetName")
            self.funcs.setdefault(module, {})[nm.value.decode()] = ctypes.c_void_p(f)

    def func(self, stem: str, module: str = None):
        key = f"{len(stem)}{stem}"
        hits = [fns[k] for m, fns in self.funcs.items() if module in (None, m) for k in fns if key in k]
        if len(hits) != 1:
            raise RuntimeError(f"kernel {stem} in {module or 'any module'}: {len(hits)} matches")
        return hits[0]

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

    def launch(self, stem, grid, block, args, module: str = None):
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
        self._ck(self.cu.cuLaunchKernel(self.func(stem, module), g[0], g[1], g[2], b[0], b[1], b[2], 0, None, ptrs, None),
                 f"launch {stem}")
        self._ck(self.cu.cuCtxSynchronize(), f"sync after {stem}")

    def free_all(self):
        for d in self.allocs:
            self.cu.cuMemFree_v2(d)
        self.allocs.clear()

    def texture(self, img: np.ndarray):
        """One float CUDA array with a texture object over it, as
        PlanarInit::cuda_space_init makes them (planar_initer.cu:125-159).
        Returns (texture object, array)."""
        a = np.ascontiguousarray(img, np.float32)
        H, W = a.shape
        arr = _p()
        self._ck(self.cu.cuArrayCreate_v2(ctypes.byref(arr), ctypes.byref(ArrayDesc(W, H, CU_AD_FORMAT_FLOAT, 1))),
                 "cuArrayCreate")
        cp = Memcpy2D()
        cp.srcMemoryType, cp.srcHost, cp.srcPitch = CU_MEMORYTYPE_HOST, a.ctypes.data, W * 4
        cp.dstMemoryType, cp.dstArray = CU_MEMORYTYPE_ARRAY, arr
        cp.WidthInBytes, cp.Height = W * 4, H
        self._ck(self.cu.cuMemcpy2D_v2(ctypes.byref(cp)), "cuMemcpy2D")
        rd = ResourceDesc()
        rd.resType = CU_RESOURCE_TYPE_ARRAY
        rd.res[0] = arr.value
        td = TextureDesc()
        td.addressMode[0] = td.addressMode[1] = CU_TR_ADDRESS_MODE_WRAP
        td.filterMode = CU_TR_FILTER_MODE_LINEAR
        td.flags = 0  # element-type reads, unnormalised coordinates
        tex = ctypes.c_uint64()
        self._ck(self.cu.cuTexObjectCreate(ctypes.byref(tex), ctypes.byref(rd), ctypes.byref(td), None),
                 "cuTexObjectCreate")
        return tex.value, arr

    def free_texture(self, tex: int, arr) -> None:
        self.cu.cuTexObjectDestroy(tex)
        self.cu.cuArrayDestroy(arr)


def camera(K, R, t, h, w, dmin, dmax) -> Camera:
    c = Camera()
    for k in range(9):
        c.K[k], c.R[k] = K[k], R[k]
    for k in range(3):
        c.t[k] = t[k]
    c.height, c.width, c.depth_min, c.depth_max = h, w, dmin, dmax
    return c


def run_patch_match(drv: Driver, cams, ref: int, src, images, depths, normals, max_iterations: int,
                    timings: dict = None, module: str = "patch_match"):
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
    drv.launch("initialization", g16, (16, 16), [d_img, d_dep, d_nrm, d_cam, d_plane, d_cost, d_rand, d_sel, p],
               module)
    for i in range(max_iterations):
        for black in (True, False):
            drv.launch("black_red_pixel_update", gcb, (16, 16),
                       [d_img, d_dep, d_cam, d_plane, d_cost, d_rand, d_sel, p, ctypes.c_int32(i), bool(black)],
                       module)
    drv.launch("get_depth_and_normal", g16, (16, 16), [d_cam, d_plane, p], module)
    drv.launch("black_red_pixel_filter", gcb, (16, 16), [d_cam, d_plane, d_cost, True], module)
    drv.launch("black_red_pixel_filter", gcb, (16, 16), [d_cam, d_plane, d_cost, False], module)
    od, on, oc = drv.alloc(4 * H * W), drv.alloc(12 * H * W), drv.alloc(4 * H * W)
    drv.launch("export_plane_hypotheses_cost", (((H * W) - 1) // 256 + 1,), (256,),
               [d_plane, d_cost, ctypes.c_int32(H), ctypes.c_int32(W), od, on, oc], module)
    t2 = time.perf_counter()
    out = (drv.get(od, (H, W), np.float32), drv.get(on, (H, W, 3), np.float32), drv.get(oc, (H, W), np.float32))
    drv.free_all()
    if timings is not None:
        timings["upload_s"] = timings.get("upload_s", 0.0) + (t1 - t0)
        timings["kernels_s"] = timings.get("kernels_s", 0.0) + (t2 - t1)
        timings["download_s"] = timings.get("download_s", 0.0) + (time.perf_counter() - t2)
    return out


def run_fusion(drv: Driver, cams, problems, depths, normals, geom_consistent: int, module: str = "fusion"):
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
                    ctypes.c_int32(W), od, on], module)
        outs.append((drv.get(od, (H, W), np.float32), drv.get(on, (H, W, 3), np.float32)))
    masks = drv.get(d_masks, (V, H, W), np.uint8)
    drv.free_all()
    return outs, masks


class PlanarInitRef:
    """Module A's PlanarInit for one reference view, on the reference's own
    kernels: the device state of cuda_space_init / cuda_planar_prior_init
    (planar_initer.cu:119-223), the launch sequence of run_patch_match
    (patch_match_kernel.cu:1711-1809, every launch followed by a device
    synchronisation) and export_plane (planar_initer.cu:104-117).

    cams: Camera structs, reference first; images: float32 [1+N, H, W]
    (the grey levels cv::imread + convertTo(CV_32F) give).  Pass-to-pass state
    (planes, costs) stays on the device as in the reference."""

    def __init__(self, drv: Driver, cams, images: np.ndarray, module: str = "planar"):
        import time

        t0 = time.perf_counter()
        self.drv = drv
        self.module = module
        n1, H, W = images.shape
        self.H, self.W, self.n1 = H, W, n1
        self.params = ParamsA()
        for name, _ in Params._fields_:
            setattr(self.params, name, getattr(default_params(), name))
        self.params.num_images = n1
        self.params.depth_min = cams[0].depth_min * 0.6  # planar_init.py:149-150
        self.params.depth_max = cams[0].depth_max * 1.2
        self.textures = [drv.texture(images[k]) for k in range(n1)]
        objs = np.zeros(MAX_IMAGES, np.uint64)
        objs[:n1] = [t for t, _ in self.textures]
        self.d_tex = drv.put(objs)
        cam_arr = (Camera * n1)(*cams)
        self.d_cam = drv.alloc(ctypes.sizeof(cam_arr))
        drv._ck(drv.cu.cuMemcpyHtoD_v2(self.d_cam, ctypes.addressof(cam_arr), ctypes.sizeof(cam_arr)), "HtoD")
        self.d_plane = drv.alloc(16 * H * W)
        self.d_cost = drv.alloc(4 * H * W)
        self.d_rand = drv.alloc(64 * H * W)
        self.d_sel = drv.alloc(4 * H * W)
        # the prior buffers exist from the start (the reference allocates them
        # in cuda_planar_prior_init; before that no kernel reads them)
        self.d_prior = drv.alloc(16 * H * W)
        self.d_mask = drv.alloc(4 * H * W)
        drv._ck(drv.cu.cuMemsetD8_v2(self.d_prior, 0, 16 * H * W), "memset")
        drv._ck(drv.cu.cuMemsetD8_v2(self.d_mask, 0, 4 * H * W), "memset")
        self.planes = np.zeros((H, W, 4), np.float32)
        self.costs = np.zeros((H, W), np.float32)
        self.upload_s = time.perf_counter() - t0

    def set_state(self, planes: np.ndarray, costs: np.ndarray) -> None:
        """Overwrite the device planes and costs (the state a previous pass leaves)."""
        self.drv._ck(self.drv.cu.cuMemcpyHtoD_v2(self.d_plane, np.ascontiguousarray(planes, np.float32).ctypes.data,
                                                 16 * self.H * self.W), "HtoD")
        self.drv._ck(self.drv.cu.cuMemcpyHtoD_v2(self.d_cost, np.ascontiguousarray(costs, np.float32).ctypes.data,
                                                 4 * self.H * self.W), "HtoD")

    def planar_prior_init(self, prior_planes: np.ndarray, masks: np.ndarray) -> None:
        """cuda_planar_prior_init (planar_initer.cu:195-223): prior planes
        (camera-frame normal, distance) and triangle ids + 1 (0: none)."""
        H, W = self.H, self.W
        self.drv._ck(self.drv.cu.cuMemcpyHtoD_v2(
            self.d_prior, np.ascontiguousarray(prior_planes, np.float32).ctypes.data, 16 * H * W), "HtoD")
        self.drv._ck(self.drv.cu.cuMemcpyHtoD_v2(
            self.d_mask, np.ascontiguousarray(masks, np.uint32).ctypes.data, 4 * H * W), "HtoD")

    def run_patch_match(self, max_iterations: int = 3, planar_prior: bool = False) -> None:
        """PlanarInit::run_patch_match (patch_match_kernel.cu:1711-1809)."""
        drv, H, W, p = self.drv, self.H, self.W, self.params
        p.max_iterations = max_iterations
        p.planar_prior = planar_prior
        g16 = ((W + 15) // 16, (H + 15) // 16)
        gcb = ((W + 31) // 32, ((H // 2) + 15) // 16)
        drv.launch("RandomInitialization", g16, (16, 16),
                   [self.d_tex, self.d_cam, self.d_plane, self.d_cost, self.d_rand, self.d_sel, self.d_prior,
                    self.d_mask, p], self.module)
        for i in range(max_iterations):
            for stem in ("BlackPixelUpdate", "RedPixelUpdate"):
                # texture_depths: only read with geom_consistency, which this path never sets
                drv.launch(stem, gcb, (32, 16),
                           [self.d_tex, self.d_tex, self.d_cam, self.d_plane, self.d_cost, self.d_rand, self.d_sel,
                            self.d_prior, self.d_mask, p, ctypes.c_int32(i)], self.module)
        drv.launch("GetDepthandNormal", g16, (16, 16), [self.d_cam, self.d_plane, p], self.module)
        drv.launch("BlackPixelFilter", gcb, (32, 16), [self.d_cam, self.d_plane, self.d_cost], self.module)
        drv.launch("RedPixelFilter", gcb, (32, 16), [self.d_cam, self.d_plane, self.d_cost], self.module)
        self.planes = drv.get(self.d_plane, (H, W, 4), np.float32)
        self.costs = drv.get(self.d_cost, (H, W), np.float32)

    def selected_views(self) -> np.ndarray:
        return self.drv.get(self.d_sel, (self.H, self.W), np.uint32)

    def export_plane(self):
        """export_plane (planar_initer.cu:104-117): depth = w, normal = xyz, cost."""
        return self.planes[..., 3].copy(), self.planes[..., :3].copy(), self.costs.copy()

    def close(self) -> None:
        for t, a in self.textures:
            self.drv.free_texture(t, a)
        self.textures = []
        self.drv.free_all()
