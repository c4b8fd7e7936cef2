/*
 * gmvs_gb300 — C ABI of the GB300-native ACMP-style PatchMatch MVS hot path.
 *
 * Every entry point takes plain pointers and sizes, returns an int32 status
 * (GMVS_OK == 0) and never throws.  Device pointers are CUDA device
 * addresses on the current device; `stream` is a cudaStream_t passed as
 * void* (NULL = legacy default stream).  gmvs_last_error() returns the
 * message of the last failing call on the calling thread.
 *
 * The structs below are layout-compatible with the reference's PODs so the
 * Python mirrors of `gmvs.src` and `gmvs.lib.build.planar_initer` can fill
 * them field by field.
 */
#ifndef GMVS_GB300_H
#define GMVS_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GMVS_API __attribute__((visibility("default")))
#else
#define GMVS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GMVS_MAX_NGB 32
#define GMVS_OK 0
#define GMVS_ERR_INVALID 1    /* bad argument (size, pointer, enum) */
#define GMVS_ERR_CUDA 2       /* a CUDA runtime call failed */
#define GMVS_ERR_WORKSPACE 3  /* workspace / scratch too small */
#define GMVS_ERR_DEVICE 4     /* a kernel reported an error status */

/* Pinhole camera, world->camera X_c = R X_w + t.
 * Same layout as mvs::Camera (gmvs/include/data_structure.hpp:39-47) and
 * Camera (gmvs/lib/include/planar_initer.hpp:39-47). 100 bytes. */
typedef struct gmvs_camera {
    float K[9];
    float R[9];
    float t[3];
    int32_t height;
    int32_t width;
    float depth_min;
    float depth_max;
} gmvs_camera;

/* One reference view and its source views.
 * Same layout as mvs::Problem (gmvs/include/data_structure.hpp:33-37). */
typedef struct gmvs_problem {
    int32_t num_ngb;
    int32_t ref_image_id;
    int32_t src_image_ids[GMVS_MAX_NGB];
} gmvs_problem;

/* How the hypothesis field is initialised before the sweeps. */
enum gmvs_init_kind {
    GMVS_INIT_RANDOM = 0,       /* RandomInitialization random branch (patch_match_kernel.cu:1560-1576) */
    GMVS_INIT_PRIOR = 1,        /* planar-prior branch (patch_match_kernel.cu:1513-1559) */
    GMVS_INIT_DEPTH_NORMAL = 2  /* module B initialization (gmvs/src/patch_match.cu:1046-1082) */
};

/* Which cost the checkerboard sweeps minimise. */
enum gmvs_sweep_kind {
    GMVS_SWEEP_PHOTO = 0,  /* module A, photometric only (patch_match_kernel.cu:813-1351, geom off) */
    GMVS_SWEEP_PRIOR = 1,  /* module A with the planar-prior restricted cost (patch_match_kernel.cu:1245-1319) */
    GMVS_SWEEP_GEOM = 2    /* module B, photometric + 0.1*geometric (gmvs/src/patch_match.cu:678-1041) */
};

/* How source images are sampled.
 *  TEX: hardware texture, linear filter, unnormalised coordinates at +0.5
 *       (module A, planar_initer.cu:150-158, patch_match_kernel.cu:443-464);
 *  CLAMP: fp32 bilinear with the reference's truncate-then-clamp indexing
 *       (module B, gmvs/src/patch_match.cu:10-33). */
enum gmvs_sampler { GMVS_SAMPLER_CLAMP = 0, GMVS_SAMPLER_TEX = 1 };

/* Device staging of the images for the CLAMP sampler. */
enum gmvs_staging {
    GMVS_STAGE_F32 = 0,       /* plain fp32 rows, four scalar loads per sample */
    GMVS_STAGE_QUAD_F32 = 1,  /* fp32 texel quads, one 16-byte load per sample */
    GMVS_STAGE_QUAD_F16 = 2,  /* fp16 texel quads, one 8-byte load per sample */
    GMVS_STAGE_AUTO = 3       /* library picks (quad f16 when lossless, else quad f32) */
};

/* PatchMatch parameters: the 17 fields of PatchMatchParams
 * (gmvs/lib/include/planar_initer.hpp:13-31) in order, then extensions that
 * default to reference behaviour. */
typedef struct gmvs_params {
    int32_t max_iterations;   /* 3 */
    int32_t patch_size;       /* 11 */
    int32_t num_images;       /* 5 (set per view from num_src + 1) */
    int32_t max_image_size;   /* 3200 (unused, as in the reference) */
    int32_t radius_increment; /* 2 */
    float sigma_spatial;      /* 5 */
    float sigma_color;        /* 3 */
    int32_t top_k;            /* 4 */
    float baseline;           /* 0.54 (unused) */
    float depth_min;          /* per-view values come from gmvs_view_pass */
    float depth_max;
    float disparity_min;      /* unused */
    float disparity_max;      /* unused */
    int32_t geom_consistency;
    int32_t multi_geometry;   /* unused */
    int32_t planar_prior;
    int32_t superpixel_filter;
    /* extensions */
    uint64_t seed;            /* Philox key, default 3407 (RANDOM_SEED, patch_match_kernel.cu:3) */
    int32_t init_kind;        /* gmvs_init_kind */
    int32_t sweep_kind;       /* gmvs_sweep_kind */
    int32_t sampler;          /* gmvs_sampler */
    int32_t staging;          /* gmvs_staging */
    int32_t pass_index;       /* decorrelates the Philox streams of successive passes */
    int32_t tile_w;           /* sweep tile width in pixels: 0 or 16 (one lane pair per pixel), or 32:
                                 the warps in flight take 32-pixel-wide blocks of two 16-column tiles,
                                 row by row (same results; another memory-access order) */
    int32_t tile_h;           /* sweep tile height in thread rows, 1..8 (0 = 4); a tile is 16 x 2*tile_h pixels */
    int32_t run_filter;       /* 1 = depth/normal conversion + checkerboard median filter */
    int32_t ctas_per_sm;      /* PatchMatch kernels: resident CTAs per SM (0 = as many as fit); fewer CTAs
                                 leave more of the SM's L1 to the texture/sample cache */
    int32_t split_sweep;      /* 1 = each half-sweep as two kernels (neighbour hypotheses, then view
                                 selection and refinement) through a per-pixel scratch in the workspace;
                                 2 = as three (neighbour hypotheses and the current plane, then view
                                 selection and the refinement planes, then the refinement); same
                                 results */
    int32_t tex_storage;      /* TEX sampler: 0 = pitched rows in the workspace; 1 = CUDA arrays (the
                                 block-linear layout module A uses), allocated by gmvs_plan_create and
                                 freed by gmvs_plan_destroy -- the one case where the library allocates
                                 device memory; same results */
} gmvs_params;

/* One reference view of one pass.  All pointers are device pointers except
 * `cams`, which is a host array copied by value.  Views in one call may have
 * different sizes and source counts. */
typedef struct gmvs_view_pass {
    int32_t height;
    int32_t width;
    int32_t num_src;                             /* N <= GMVS_MAX_NGB */
    int32_t stream_id;                           /* Philox stream (reference image id) */
    float depth_min;                             /* search range of this view */
    float depth_max;
    gmvs_camera cams[1 + GMVS_MAX_NGB];          /* ref, then src */
    const float* images[1 + GMVS_MAX_NGB];       /* fp32 [H][W] gray images (row pitch = width) */
    const float* depths[1 + GMVS_MAX_NGB];       /* GEOM: input depths [H][W] (ref, then src) */
    const float* ref_normal;                     /* DEPTH_NORMAL init: world normals [H][W][3] */
    const float* prior_planes;                   /* PRIOR: float4 [H][W] (camera-frame n, d) */
    const uint32_t* prior_masks;                 /* PRIOR: [H][W] triangle id + 1, 0 = none */
    const float* init_planes;                    /* PRIOR init: previous pass planes float4 [H][W] */
    const float* init_costs;                     /* PRIOR init: previous pass costs [H][W] */
    float* out_depth;                            /* [H][W] */
    float* out_normal;                           /* [H][W][3] world frame */
    float* out_cost;                             /* [H][W] */
    float* out_planes;                           /* optional float4 [H][W]: exported plane field */
} gmvs_view_pass;

/* Fusion of one reference view (gmvs/src/fusion.cu:61-182, 211-275). */
typedef struct gmvs_fuse_view {
    int32_t height;
    int32_t width;
    int32_t num_views;                           /* V, extent of `masks` */
    gmvs_problem problem;
    gmvs_camera cams[1 + GMVS_MAX_NGB];          /* ref, then src in problem order */
    const float* depths[1 + GMVS_MAX_NGB];       /* device [H][W] (ref, then src) */
    const float* normals[1 + GMVS_MAX_NGB];      /* device [H][W][3] */
    uint8_t* masks;                              /* device bool [V][H][W], read and written */
    int32_t geom_consistent;
    float* out_depth;                            /* device [H][W], zero-filled by the call */
    float* out_normal;                           /* device [H][W][3], zero-filled by the call */
    int32_t* out_count;                          /* optional device [H][W]: consistent-view count, -1 = skipped */
} gmvs_fuse_view;

GMVS_API int32_t gmvs_version(void);
/* Bounds-checked builds (-DGMVS_BOUNDS_CHECK): the OR of the violation bits
 * the PatchMatch kernels raised since the last reset (1 image tap, 2 depth
 * tap, 4 neighbour cost or plane, 8 scratch; 0 = none); -1 in normal
 * builds.  No counterpart in the reference (it has no checks). */
GMVS_API int32_t gmvs_bounds_violations(int32_t reset);
GMVS_API const char* gmvs_last_error(void);

/* Fill `p` with the reference defaults (PatchMatchParams(), data_structure.hpp:20-37). */
GMVS_API void gmvs_default_params(gmvs_params* p);

/* ---------------------------------------------------------------- passes --
 * A plan owns one PatchMatch pass over `n_views` reference views (one view =
 * the plain per-view path of PlanarInit::run_patch_match,
 * patch_match_kernel.cu:1711-1809, and PatchMatcher::run_patch_match,
 * gmvs/src/patch_match.cu:1353-1518; many views = one launch per stage for
 * the whole batch).  The caller provides the device workspace; the library
 * allocates no device memory.  Creating a plan uploads descriptors and
 * stages images on `stream`; gmvs_plan_launch only enqueues kernels (it can
 * be captured into a CUDA graph). */
typedef struct gmvs_plan gmvs_plan;

GMVS_API size_t gmvs_plan_workspace_bytes(const gmvs_view_pass* views, int32_t n_views,
                                 const gmvs_params* params);
GMVS_API int32_t gmvs_plan_create(const gmvs_view_pass* views, int32_t n_views,
                         const gmvs_params* params, void* workspace,
                         size_t workspace_bytes, void* stream, gmvs_plan** out);
/* Enqueue the whole chain: init, 2*max_iterations half-sweeps, filter, export. */
GMVS_API int32_t gmvs_plan_launch(gmvs_plan* plan, void* stream);
/* Number of stages and one stage at a time (for schedulers interleaving plans). */
GMVS_API int32_t gmvs_plan_num_stages(const gmvs_plan* plan);
GMVS_API int32_t gmvs_plan_launch_stage(gmvs_plan* plan, int32_t stage, void* stream);
/* Device error word of the plan's kernels (0 = ok); synchronises `stream`. */
GMVS_API int32_t gmvs_plan_check(gmvs_plan* plan, void* stream);
GMVS_API void gmvs_plan_destroy(gmvs_plan* plan);

/* Convenience: create, launch, check and destroy in one call. */
GMVS_API int32_t gmvs_run_passes(const gmvs_view_pass* views, int32_t n_views,
                        const gmvs_params* params, void* workspace,
                        size_t workspace_bytes, void* stream);

/* Per-view NCC costs of given hypotheses: for every pixel of view 0 of
 * `view`, the bilateral NCC against each source view for the camera-frame
 * plane planes[y][x] (float4 n, d).  costs: device [num_src][H][W].
 * Also writes the initial multi-view cost and selected-view mask
 * (ComputeMultiViewInitialCostandSelectedViews, patch_match_kernel.cu:518-569)
 * into init_cost / init_views when those are non-NULL. */
GMVS_API size_t gmvs_ncc_workspace_bytes(const gmvs_view_pass* view, const gmvs_params* params);
GMVS_API int32_t gmvs_ncc_costs(const gmvs_view_pass* view, const gmvs_params* params,
                       const float* planes, float* costs, float* init_cost,
                       uint32_t* init_views, void* workspace, size_t workspace_bytes,
                       void* stream);

/* ---------------------------------------------------------------- fusion --
 * Deterministic geometric-consistency fusion of one reference view.  Output
 * pixels hit by several reference pixels take the value of the highest
 * reference pixel index (the last writer of a sequential scan). */
GMVS_API size_t gmvs_fuse_scratch_bytes(int32_t height, int32_t width);
GMVS_API int32_t gmvs_fuse(const gmvs_fuse_view* args, void* scratch, size_t scratch_bytes,
                  void* stream);

/* gmvs_fuse without any device allocation.  No counterpart in the reference
 * (Fuser::run_fusion, gmvs/src/fusion.cu:211-275, allocates per call).
 * For callers that have no device allocator at hand and may not allocate at
 * the point of the call: a plain C / FFI caller that would otherwise need a
 * cudaMalloc per call for gmvs_fuse's scratch, or a job running under a
 * fixed device-memory budget, where an allocation in the middle of the job
 * could fail.  Same inputs, outputs and results as gmvs_fuse; the per-pixel
 * scratch is a library-owned device array of GMVS_FUSE_FIXED_MAX_PIXELS
 * int32 entries (16 MiB), and views with height * width above that are
 * rejected with GMVS_ERR_INVALID.  The first call in each CUDA context
 * (normally: on each device, in the device's primary context) looks the
 * array up, which may load a module: make that first call before any stream
 * capture.  A new context on the device (after cudaDeviceReset, or another
 * context made current through the driver API) is looked up afresh.  Every call re-initialises
 * the part of the array it uses on `stream`, so nothing has to be cleared
 * beforehand; but all calls on a device share the one array, so calls whose
 * work can overlap on the device (different streams, several host threads)
 * race and must be serialised by the caller. */
#define GMVS_FUSE_FIXED_MAX_PIXELS (1 << 22)
GMVS_API int32_t gmvs_fuse_fixed_scratch(const gmvs_fuse_view* args, void* stream);

/* -------------------------------------------------- host (CPU) routines --
 * Planar prior from a depth/cost map: support points, Delaunay
 * triangulation, superpixel filter, rasterisation and plane fit
 * (PlanarInit::triangulation, planar_initer.cu:225-420, 700-745).
 * out_planes: host float4 [H][W]; out_masks: host uint32 [H][W];
 * out_tri_count receives the number of retained triangles. */
GMVS_API int32_t gmvs_build_planar_prior(const gmvs_camera* ref_cam, int32_t height, int32_t width,
                                const float* depth, const float* cost,
                                const uint8_t* superpixel, int32_t superpixel_filter,
                                float depth_min, float depth_max,
                                float* out_planes, uint32_t* out_masks,
                                int32_t* out_tri_count, int32_t* out_tris, int32_t max_tris);

/* planar_initer.cu:537-632 */
GMVS_API int32_t gmvs_fusion_planar_mask(const int32_t* seg_ids, const int32_t* planar_mask,
                                const float* normals, int32_t rows, int32_t cols,
                                int32_t thresh, float nonplanar_percent,
                                float cos_sim_thresh, float match_ratio_thresh,
                                int32_t* out_mask);
/* planar_initer.cu:634-684 */
GMVS_API int32_t gmvs_filter_by_var_map(const float* var_map, const int32_t* seg_ids,
                               int32_t rows, int32_t cols, float var_thresh,
                               int32_t* out_ids);
/* planar_initer.cu:471-535 (host loop) */
GMVS_API int32_t gmvs_sliding_window_normal(const int32_t* planar_region, const float* normals,
                                   int32_t rows, int32_t cols, int32_t window_size,
                                   float* out_normals);

/* ------------------------------------------- device segment statistics --
 * The three routines above on device arrays, with the same results bit for
 * bit (every float sum in the reference's raster order).  Segment ids must
 * lie in [0, max_seg_id] (the caller knows or computes the largest id);
 * an id outside it is reported as GMVS_ERR_INVALID.  The two per-segment
 * routines take a 256-byte aligned device workspace of
 * gmvs_segments_workspace_bytes(rows, cols, max_seg_id) bytes and
 * synchronise `stream` before returning (to read their error word). */
GMVS_API size_t gmvs_segments_workspace_bytes(int32_t rows, int32_t cols, int32_t max_seg_id);
/* planar_initer.cu:537-632 */
GMVS_API int32_t gmvs_fusion_planar_mask_device(const int32_t* seg_ids, const int32_t* planar_mask,
                                       const float* normals, int32_t rows, int32_t cols,
                                       int32_t max_seg_id, int32_t thresh, float nonplanar_percent,
                                       float cos_sim_thresh, float match_ratio_thresh,
                                       int32_t* out_mask, void* workspace, size_t workspace_bytes,
                                       void* stream);
/* planar_initer.cu:634-684 */
GMVS_API int32_t gmvs_filter_by_var_map_device(const float* var_map, const int32_t* seg_ids,
                                      int32_t rows, int32_t cols, int32_t max_seg_id,
                                      float var_thresh, int32_t* out_ids, void* workspace,
                                      size_t workspace_bytes, void* stream);
/* planar_initer.cu:471-535 */
GMVS_API int32_t gmvs_sliding_window_normal_device(const int32_t* planar_region, const float* normals,
                                          int32_t rows, int32_t cols, int32_t window_size,
                                          float* out_normals, void* stream);

/* ------------------------------------------------------------ point gather --
 * The fusion scripts' gather of one view's fused depth/normal map into
 * world points (gmvs/scripts/mvs_fusion_segmentaion.py:195-236), one device
 * pass: for every pixel with depth > 0, p = o + depth * R d with
 * d = ((x - cx) / fx, (y - cy) / fy, 1) and (R, o) the camera-to-world pose,
 * written with its normal as 6 floats to out_points in raster order; the
 * points with dot(-R d, n) > cos_thresh (normal facing the camera) also go
 * to out_facing (optional), and out_depth / out_normal (optional) receive
 * the maps with only those pixels kept.  depth [H][W], normal [H][W][3] and
 * the outputs are device arrays; out_points and out_facing hold up to H * W
 * points.  intrinsics: host 3x3 row-major K; pose: host 4x4 row-major.
 * out_counts (host, 2 entries) receives the two point counts; the call
 * synchronises `stream`.  No counterpart in the reference's C++ (it is
 * torch code in the script). */
GMVS_API size_t gmvs_gather_workspace_bytes(int32_t height, int32_t width);
GMVS_API int32_t gmvs_gather_points(const float* depth, const float* normal, int32_t height, int32_t width,
                           const float* intrinsics, const float* pose, float cos_thresh,
                           float* out_points, float* out_facing, float* out_depth, float* out_normal,
                           int64_t* out_counts, void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------- view selection --
 * calc_score of the COLMAP conversion (gmvs/scripts/colmap2mvs.py:324-357)
 * for every pair of num_images images, into the symmetric device matrix
 * scores [V][V] (zero diagonal).  point_ids: device int32, image i's point
 * ids sorted ascending without -1 entries at [offsets[i], offsets[i+1])
 * (offsets: device, V + 1 entries); xyz: device FP64 [num_points][3] indexed
 * by point id (ids outside it are ignored); centers: device FP64 [V][3]
 * camera centres.  No counterpart in the reference's C++ (it is a Python
 * loop over a process pool). */
GMVS_API int32_t gmvs_view_scores(const long long* offsets, const int32_t* point_ids, int32_t num_images,
                         const double* xyz, int32_t num_points, const double* centers, float* scores,
                         void* stream);

/* ------------------------------------------------------------ scene jobs --
 * The reference's whole reconstruction of one scene (launch.py:143-173) for
 * hosts that are not Python: a job holds the scene's cameras, problems and
 * images and owns the device state of its passes (it allocates, like
 * PlanarInit, planar_initer.cu:21-62; the plan API above does not);
 * gmvs_pass_random_prior runs the random pass, the host triangulation and
 * the planar-prior pass of planar_init.py:113-190 (PlanarInit::
 * run_patch_match, triangulation, cuda_planar_prior_init), gmvs_pass_geom
 * one geometric pass of consistency.py (PatchMatcher::run_patch_match,
 * gmvs/src/patch_match.cu:1353-1518), gmvs_job_fuse the fusion of every
 * problem in order (Fuser::run_fusion, gmvs/src/fusion.cu:211-275) with the
 * normal renormalisation of consistency.py:193-197, and gmvs_export copies
 * one view's maps out (PlanarInit::export_plane, planar_initer.cu:104-117).
 * The pass parameters come from the caller's gmvs_params (init / sweep kind,
 * sampler and pass index are set per pass; the reference's geometric passes
 * use max_iterations = 2).  Problem sets are indices into `problems`
 * (NULL = all).  Every call enqueues on `stream`; the prior pass and plan
 * creation synchronise it.  A context must outlive its jobs. */
typedef struct gmvs_ctx gmvs_ctx;
typedef struct gmvs_job gmvs_job;

GMVS_API int32_t gmvs_ctx_create(int32_t device, gmvs_ctx** out);
GMVS_API void gmvs_ctx_destroy(gmvs_ctx* ctx);
/* The message of the last failing job call of this context. */
GMVS_API int32_t gmvs_ctx_last_error(const gmvs_ctx* ctx, char* buf, size_t len);
/* cams: host [num_images], every one height x width; images: device fp32
 * [num_images][height][width], caller-owned, kept for the job's life;
 * superpixels: host uint8 [num_images][height][width] (copied) or NULL =
 * no superpixel filter in the triangulation; problems: host [num_problems]. */
GMVS_API int32_t gmvs_job_create(gmvs_ctx* ctx, const gmvs_camera* cams, int32_t num_images, int32_t height,
                        int32_t width, const float* images, const uint8_t* superpixels,
                        const gmvs_problem* problems, int32_t num_problems, gmvs_job** out);
GMVS_API void gmvs_job_destroy(gmvs_job* job);
GMVS_API int32_t gmvs_pass_random_prior(gmvs_job* job, const int32_t* problem_ids, int32_t n,
                               const gmvs_params* params, void* stream);
/* depth_in [V][H][W] / normal_in [V][H][W][3] (device): the maps the pass
 * starts from, or both NULL = the job's last pass. */
GMVS_API int32_t gmvs_pass_geom(gmvs_job* job, const int32_t* problem_ids, int32_t n, const gmvs_params* params,
                       const float* depth_in, const float* normal_in, void* stream);
/* masks: device bool [V][H][W] the fusion marks (zeroed first), or NULL =
 * the job's own. */
GMVS_API int32_t gmvs_job_fuse(gmvs_job* job, const int32_t* order, int32_t n, int32_t geom_consistent,
                      uint8_t* masks, void* stream);
/* which: 0 = the last pass (depth, normal, cost), 1 = fused (depth, normal;
 * cost must be NULL).  Outputs are device or host arrays of one view
 * ([H][W], [H][W][3], [H][W]); any may be NULL. */
GMVS_API int32_t gmvs_export(gmvs_job* job, int32_t view, int32_t which, float* depth, float* normal, float* cost,
                    void* stream);

/* -------------------------------------------------------------- superpixels --
 * The segmentation preprocessing of gmvs/scripts/extract_superpixel.py:
 * extract_superpixel (lines 55-74: resize to seg_cols x seg_rows,
 * Felzenszwalb segmentation, segments of at most seg_rows * seg_cols / 128
 * pixels dropped, nearest resize back) and seg_func's segment-id map
 * (lines 77-113: a close_size x close_size morphological close, an
 * optional mask with its small-segment filter, and the variance filter
 * where(winVar(gray / 255, var_windlen) / max < var_thresh, ids, 0)).
 * No counterpart in the reference's C++ (it is a Python script over OpenCV
 * and scikit-image). */
typedef struct gmvs_superpixel_params {
    int32_t seg_rows;    /* working size of the segmentation (288) */
    int32_t seg_cols;    /* (384) */
    double scale;        /* Felzenszwalb scale (100) */
    double sigma;        /* Gaussian pre-smoothing (0.5; <= 0: none) */
    int32_t min_size;    /* minimum component size of the second merge pass (5) */
    int32_t close_size;  /* odd box of the morphological close (11) */
    int32_t var_windlen; /* box of the variance map (15); <= 1 turns the variance filter off */
    float var_thresh;    /* (0.2); <= 0 turns the variance filter off */
} gmvs_superpixel_params;

GMVS_API void gmvs_superpixel_default_params(gmvs_superpixel_params* out);
GMVS_API size_t gmvs_superpixel_workspace_bytes(int32_t rows, int32_t cols, const gmvs_superpixel_params* params);
/* image: device uint8 [rows][cols][3] (channel order as read, BGR from
 * OpenCV); gray: device uint8 [rows][cols], needed when the variance filter
 * is on and out_ids_map or out_var_map is given; mask: device uint8
 * [rows][cols], nonzero = keep, or NULL.  Outputs (device, each optional):
 * out_segment int32 [rows][cols] = extract_superpixel's labels;
 * out_ids uint8 = segment ids after the close (and mask);
 * out_ids_map int32 = the variance-filtered ids (the ids themselves when
 * the filter is off); out_var_map float = the normalised variance map.
 * out_num_segments (host, optional) = segments kept by the size filter.
 * The Felzenszwalb merge runs on the calling thread between the device
 * stages, so the call synchronises `stream` once and returns with the
 * remaining kernels queued on it. */
/* The host half alone, on host arrays: weights of the right, down,
 * down-right and up-right edges of a rows x cols grid, each group in raster
 * order ((rows * (cols - 1) + (rows - 1) * cols + 2 (rows - 1)(cols - 1))
 * non-negative values); writes labels [rows][cols] after the merge and the
 * size filter (0 = dropped or the first segment). */
GMVS_API int32_t gmvs_superpixel_labels_host(int32_t rows, int32_t cols, const double* weights, double scale,
                                    int32_t min_size, int32_t* labels, int32_t* out_num_segments);
GMVS_API int32_t gmvs_superpixels(const uint8_t* image, const uint8_t* gray, const uint8_t* mask, int32_t rows,
                         int32_t cols, const gmvs_superpixel_params* params, int32_t* out_segment,
                         uint8_t* out_ids, int32_t* out_ids_map, float* out_var_map,
                         int32_t* out_num_segments, void* workspace, size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GMVS_GB300_H */
