"""ctypes mirror of include/gmvs_gb300.h and the loader of libgmvs_gb300.so.

The library is built in-tree by ``gmvs_gb300.build.build()``.  There is no
fallback: every entry point of this package calls into the CUDA library, and
importing a function that needs it raises when the library is missing.
"""

from __future__ import annotations

import ctypes
import os
import threading

MAX_NGB = 32
OK = 0
ERR_INVALID = 1
ERR_CUDA = 2
ERR_WORKSPACE = 3
ERR_DEVICE = 4

INIT_RANDOM, INIT_PRIOR, INIT_DEPTH_NORMAL = 0, 1, 2
SWEEP_PHOTO, SWEEP_PRIOR, SWEEP_GEOM = 0, 1, 2
SAMPLER_CLAMP, SAMPLER_TEX = 0, 1
STAGE_F32, STAGE_QUAD_F32, STAGE_QUAD_F16, STAGE_AUTO = 0, 1, 2, 3
FUSE_FIXED_MAX_PIXELS = 1 << 22

_f = ctypes.c_float
_i = ctypes.c_int32
_p = ctypes.c_void_p


class gmvs_camera(ctypes.Structure):
    _fields_ = [("K", _f * 9), ("R", _f * 9), ("t", _f * 3), ("height", _i), ("width", _i),
                ("depth_min", _f), ("depth_max", _f)]


class gmvs_problem(ctypes.Structure):
    _fields_ = [("num_ngb", _i), ("ref_image_id", _i), ("src_image_ids", _i * MAX_NGB)]


class gmvs_params(ctypes.Structure):
    _fields_ = [("max_iterations", _i), ("patch_size", _i), ("num_images", _i), ("max_image_size", _i),
                ("radius_increment", _i), ("sigma_spatial", _f), ("sigma_color", _f), ("top_k", _i),
                ("baseline", _f), ("depth_min", _f), ("depth_max", _f), ("disparity_min", _f),
                ("disparity_max", _f), ("geom_consistency", _i), ("multi_geometry", _i), ("planar_prior", _i),
                ("superpixel_filter", _i), ("seed", ctypes.c_uint64), ("init_kind", _i), ("sweep_kind", _i),
                ("sampler", _i), ("staging", _i), ("pass_index", _i), ("tile_w", _i), ("tile_h", _i),
                ("run_filter", _i), ("ctas_per_sm", _i), ("split_sweep", _i),
                ("tex_storage", _i)]


class gmvs_view_pass(ctypes.Structure):
    _fields_ = [("height", _i), ("width", _i), ("num_src", _i), ("stream_id", _i), ("depth_min", _f),
                ("depth_max", _f), ("cams", gmvs_camera * (1 + MAX_NGB)), ("images", _p * (1 + MAX_NGB)),
                ("depths", _p * (1 + MAX_NGB)), ("ref_normal", _p), ("prior_planes", _p), ("prior_masks", _p),
                ("init_planes", _p), ("init_costs", _p), ("out_depth", _p), ("out_normal", _p),
                ("out_cost", _p), ("out_planes", _p)]


class gmvs_fuse_view(ctypes.Structure):
    _fields_ = [("height", _i), ("width", _i), ("num_views", _i), ("problem", gmvs_problem),
                ("cams", gmvs_camera * (1 + MAX_NGB)), ("depths", _p * (1 + MAX_NGB)),
                ("normals", _p * (1 + MAX_NGB)), ("masks", _p), ("geom_consistent", _i), ("out_depth", _p),
                ("out_normal", _p), ("out_count", _p)]


class gmvs_superpixel_params(ctypes.Structure):
    _fields_ = [("seg_rows", _i), ("seg_cols", _i), ("scale", ctypes.c_double), ("sigma", ctypes.c_double),
                ("min_size", _i), ("close_size", _i), ("var_windlen", _i), ("var_thresh", _f)]


_SIGS = {
    "gmvs_version": (_i, []),
    "gmvs_last_error": (ctypes.c_char_p, []),
    "gmvs_bounds_violations": (_i, [_i]),
    "gmvs_default_params": (None, [ctypes.POINTER(gmvs_params)]),
    "gmvs_plan_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(gmvs_view_pass), _i,
                                                    ctypes.POINTER(gmvs_params)]),
    "gmvs_plan_create": (_i, [ctypes.POINTER(gmvs_view_pass), _i, ctypes.POINTER(gmvs_params), _p,
                              ctypes.c_size_t, _p, ctypes.POINTER(_p)]),
    "gmvs_plan_launch": (_i, [_p, _p]),
    "gmvs_plan_num_stages": (_i, [_p]),
    "gmvs_plan_launch_stage": (_i, [_p, _i, _p]),
    "gmvs_plan_check": (_i, [_p, _p]),
    "gmvs_plan_destroy": (None, [_p]),
    "gmvs_run_passes": (_i, [ctypes.POINTER(gmvs_view_pass), _i, ctypes.POINTER(gmvs_params), _p,
                             ctypes.c_size_t, _p]),
    "gmvs_ncc_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(gmvs_view_pass), ctypes.POINTER(gmvs_params)]),
    "gmvs_ncc_costs": (_i, [ctypes.POINTER(gmvs_view_pass), ctypes.POINTER(gmvs_params), _p, _p, _p, _p, _p,
                            ctypes.c_size_t, _p]),
    "gmvs_fuse_scratch_bytes": (ctypes.c_size_t, [_i, _i]),
    "gmvs_fuse": (_i, [ctypes.POINTER(gmvs_fuse_view), _p, ctypes.c_size_t, _p]),
    "gmvs_fuse_fixed_scratch": (_i, [ctypes.POINTER(gmvs_fuse_view), _p]),
    "gmvs_build_planar_prior": (_i, [ctypes.POINTER(gmvs_camera), _i, _i, _p, _p, _p, _i, _f, _f, _p, _p,
                                     ctypes.POINTER(_i), _p, _i]),
    "gmvs_fusion_planar_mask": (_i, [_p, _p, _p, _i, _i, _i, _f, _f, _f, _p]),
    "gmvs_filter_by_var_map": (_i, [_p, _p, _i, _i, _f, _p]),
    "gmvs_sliding_window_normal": (_i, [_p, _p, _i, _i, _i, _p]),
    "gmvs_segments_workspace_bytes": (ctypes.c_size_t, [_i, _i, _i]),
    "gmvs_fusion_planar_mask_device": (_i, [_p, _p, _p, _i, _i, _i, _i, _f, _f, _f, _p, _p, ctypes.c_size_t, _p]),
    "gmvs_filter_by_var_map_device": (_i, [_p, _p, _i, _i, _i, _f, _p, _p, ctypes.c_size_t, _p]),
    "gmvs_sliding_window_normal_device": (_i, [_p, _p, _i, _i, _i, _p, _p]),
    "gmvs_gather_workspace_bytes": (ctypes.c_size_t, [_i, _i]),
    "gmvs_gather_points": (_i, [_p, _p, _i, _i, _p, _p, _f, _p, _p, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "gmvs_view_scores": (_i, [_p, _p, _i, _p, _i, _p, _p, _p]),
    "gmvs_ctx_create": (_i, [_i, ctypes.POINTER(_p)]),
    "gmvs_ctx_destroy": (None, [_p]),
    "gmvs_ctx_last_error": (_i, [_p, ctypes.c_char_p, ctypes.c_size_t]),
    "gmvs_job_create": (_i, [_p, ctypes.POINTER(gmvs_camera), _i, _i, _i, _p, _p, ctypes.POINTER(gmvs_problem), _i,
                             ctypes.POINTER(_p)]),
    "gmvs_job_destroy": (None, [_p]),
    "gmvs_pass_random_prior": (_i, [_p, _p, _i, ctypes.POINTER(gmvs_params), _p]),
    "gmvs_pass_geom": (_i, [_p, _p, _i, ctypes.POINTER(gmvs_params), _p, _p, _p]),
    "gmvs_job_fuse": (_i, [_p, _p, _i, _i, _p, _p]),
    "gmvs_export": (_i, [_p, _i, _i, _p, _p, _p, _p]),
    "gmvs_superpixel_default_params": (None, [ctypes.POINTER(gmvs_superpixel_params)]),
    "gmvs_superpixel_workspace_bytes": (ctypes.c_size_t, [_i, _i, ctypes.POINTER(gmvs_superpixel_params)]),
    "gmvs_superpixel_labels_host": (_i, [_i, _i, _p, ctypes.c_double, _i, _p, _p]),
    "gmvs_superpixels": (_i, [_p, _p, _p, _i, _i, ctypes.POINTER(gmvs_superpixel_params), _p, _p, _p, _p, _p, _p,
                              ctypes.c_size_t, _p]),
}

EXPORTED = tuple(_SIGS)

_lock = threading.Lock()
_lib = None


def library_path() -> str:
    """The in-tree library, or the variant named by GMVS_GB300_LIB."""
    from .build import LIB_PATH

    return os.environ.get("GMVS_GB300_LIB", LIB_PATH)


def lib() -> ctypes.CDLL:
    """The loaded C-ABI library (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = library_path()
            if not os.path.exists(path):
                raise RuntimeError(
                    f"{path} is missing: build the CUDA library with gmvs_gb300.build.build() "
                    "(this package has no CPU fallback)")
            L = ctypes.CDLL(path)
            for name, (res, args) in _SIGS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


class GmvsError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"gmvs error {code}: {msg}")
        self.code = code


def check(rc: int) -> None:
    if rc != OK:
        raise GmvsError(rc, lib().gmvs_last_error().decode(errors="replace"))


def default_params() -> gmvs_params:
    p = gmvs_params()
    lib().gmvs_default_params(ctypes.byref(p))
    return p


def ptr(t) -> int | None:
    """data_ptr of a torch tensor (None for None)."""
    return None if t is None else t.data_ptr()


def stream_ptr(stream=None) -> int | None:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream or None
