// Host runtime of the C ABI: plans (workspace layout, descriptor upload,
// image staging, launch sequencing) and the per-view NCC entry point.
// The library allocates no device memory: every buffer lives in the
// caller's workspace.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "errors.h"
#include "kernels.h"
#include "pm_device.cuh"
#include "pmath.h"

using namespace gmvs;

// ------------------------------------------------------------- errors --
namespace gmvs {
thread_local std::string g_last_error;
int32_t fail(int32_t code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
int32_t fail_cuda(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return GMVS_ERR_CUDA;
}
}  // namespace gmvs

extern "C" int32_t gmvs_version(void) { return 1; }

extern "C" int32_t gmvs_bounds_violations(int32_t reset) {
    const unsigned v[4] = {gmvs::oob_read_f32(reset != 0), gmvs::oob_read_qf32(reset != 0),
                           gmvs::oob_read_qf16(reset != 0), gmvs::oob_read_tex(reset != 0)};
    unsigned all = 0;
    for (unsigned x : v) {
        if (x == ~0u) return -1;
        all |= x;
    }
    return (int32_t)all;
}
extern "C" const char* gmvs_last_error(void) { return g_last_error.c_str(); }

extern "C" void gmvs_default_params(gmvs_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->max_iterations = 3;
    p->patch_size = 11;
    p->num_images = 5;
    p->max_image_size = 3200;
    p->radius_increment = 2;
    p->sigma_spatial = 5.0f;
    p->sigma_color = 3.0f;
    p->top_k = 4;
    p->baseline = 0.54f;
    p->depth_min = 0.0f;
    p->depth_max = 1.0f;
    p->disparity_min = 0.0f;
    p->disparity_max = 1.0f;
    p->seed = 3407;
    p->init_kind = GMVS_INIT_RANDOM;
    p->sweep_kind = GMVS_SWEEP_PHOTO;
    p->sampler = GMVS_SAMPLER_TEX;
    p->staging = GMVS_STAGE_AUTO;
    p->run_filter = 1;
}

// -------------------------------------------------- finalisation kernels --
namespace gmvs {
namespace {

__global__ void k_convert(const DevView* __restrict__ views, const Tile* __restrict__ tiles,
                          const int* __restrict__ ntiles, int final_buf) {
    const int nt = *ntiles;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const Tile T = tiles[t];
        const DevView& V = views[T.view];
        const int px = T.x0 + threadIdx.x;
        for (int dy = 0; dy < 2; ++dy) {
            const int py = 2 * (T.yh0 + (int)threadIdx.y) + dy;
            if (px < V.W && py < V.H) convert_pixel(V, final_buf, px, py);
        }
    }
}

__global__ void k_filter(const DevView* __restrict__ views, const Tile* __restrict__ tiles,
                         const int* __restrict__ ntiles, int final_buf, int colour, int run_filter) {
    const int nt = *ntiles;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const Tile T = tiles[t];
        const DevView& V = views[T.view];
        const int px = T.x0 + threadIdx.x;
        const int py = 2 * (T.yh0 + (int)threadIdx.y) + ((px & 1) ^ colour);
        if (px < V.W && py < V.H) filter_export_pixel(V, final_buf, run_filter != 0, px, py);
    }
}

// texel quads for the CLAMP sampler (see SampQuadF32): (a, b - a, c, d - c)
// for the texels a b / c d at (x, y), (x+1, y), (x, y+1), (x+1, y+1), the
// differences rounded to fp32 as the sampler's interpolation forms them
__global__ void k_stage_quad_f32(const float* __restrict__ img, float4* __restrict__ out, int H, int W) {
    const int n = H * W;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int y = i / W, x = i - y * W;
        const int xu = min(x + 1, W - 1), yu = min(y + 1, H - 1);
        const float a = img[y * W + x], b = img[y * W + xu], c = img[yu * W + x], d = img[yu * W + xu];
        out[i] = make_float4(a, b - a, c, d - c);
    }
}
// fp16 quads are staged only for integer images in [0, 2048], whose values
// and differences are exact in fp16
__global__ void k_stage_quad_f16(const float* __restrict__ img, uint2* __restrict__ out, int H, int W) {
    const int n = H * W;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int y = i / W, x = i - y * W;
        const int xu = min(x + 1, W - 1), yu = min(y + 1, H - 1);
        const float a = img[y * W + x], b = img[y * W + xu], c = img[yu * W + x], d = img[yu * W + xu];
        __half2 t = __floats2half2_rn(a, b - a);
        __half2 u = __floats2half2_rn(c, d - c);
        out[i] = make_uint2(*reinterpret_cast<uint32_t*>(&t), *reinterpret_cast<uint32_t*>(&u));
    }
}
// 1 when every pixel is an integer in [0, 2048] (exact in fp16), else 0
__global__ void k_check_f16_exact(const float* __restrict__ img, int n, int* __restrict__ flag) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float v = img[i];
        if (!(v >= 0.0f && v <= 2048.0f && v == rintf(v))) atomicAnd(flag, 0);
    }
}

}  // namespace

cudaError_t launch_convert(const LaunchShape& ls, const DevView* v, const Tile* t, const int* nt, int fb,
                           cudaStream_t st) {
    k_convert<<<ls.grid, ls.block, 0, st>>>(v, t, nt, fb);
    return cudaGetLastError();
}
cudaError_t launch_filter(const LaunchShape& ls, const DevView* v, const Tile* t, const int* nt, int fb, int colour,
                          int run_filter, cudaStream_t st) {
    k_filter<<<ls.grid, ls.block, 0, st>>>(v, t, nt, fb, colour, run_filter);
    return cudaGetLastError();
}

}  // namespace gmvs

// ------------------------------------------------------------------ plans --
namespace {

constexpr size_t kAlign = 512;  // >= textureAlignment
inline size_t align_up(size_t v, size_t a = kAlign) { return (v + a - 1) / a * a; }

struct ImageSlot {
    const float* src;
    int H, W;
    size_t offset;   // staged copy in the workspace (quad / pitched), or ~0 when used in place
    size_t pitch;    // bytes (texture copies)
};

struct Layout {
    size_t header = 0;     // error word + tile queue
    size_t views = 0;
    size_t tiles = 0;
    size_t images = 0;
    size_t state = 0;
    size_t ca = 0;         // neighbour-cost scratch of the resident warps
    size_t nbc = 0, nbi = 0;  // split half-sweeps: per-unit neighbour costs and positions
    size_t rfs = 0;           // three-kernel half-sweeps: per-unit refinement state
    int ca_ctas = 0;       // resident CTAs per SM it holds
    size_t total = 0;
    int ntiles = 0;
    std::vector<ImageSlot> slots;
    std::vector<int> ref_slot;               // per view: slot of each image (1 + N entries)
    std::vector<std::vector<int>> view_slots;
    std::vector<size_t> view_state;          // per view: offset of its state block
};

int variant_of(const gmvs_params* p, int staging_resolved) {
    if (p->sampler == GMVS_SAMPLER_TEX) return kVarTex;
    switch (staging_resolved) {
        case GMVS_STAGE_F32: return kVarF32;
        case GMVS_STAGE_QUAD_F32: return kVarQuadF32;
        default: return kVarQuadF16;
    }
}

size_t bytes_per_pixel(int variant, const gmvs_params* p) {
    if (variant == kVarTex && p->tex_storage == 1) return 0;  // CUDA arrays, outside the workspace
    switch (variant) {
        case kVarQuadF32: return 16;
        case kVarQuadF16: return 8;
        case kVarTex: return 4;
        default: return 0;
    }
}

// a tile is 16 pixel columns (one lane pair per pixel in the PatchMatch kernels);
// tile_w = 32 orders the work as 32-pixel-wide blocks of two such tiles
int tile_w_of(const gmvs_params*) { return 16; }
bool wide_tiles(const gmvs_params* p) { return p->tile_w == 32; }
// 16-column tiles per tile row of a view (an even count for wide tiles: the
// right tile of the last pair may lie past the image and holds no pixel)
int tiles_across(int width, const gmvs_params* p) {
    const int n = (width + 15) / 16;
    return wide_tiles(p) ? (n + 1) / 2 * 2 : n;
}
int tile_h_of(const gmvs_params* p) { return p->tile_h > 0 ? p->tile_h : 4; }

int num_offsets(const gmvs_params* p) {
    const int r = p->patch_size / 2;
    return (2 * r) / p->radius_increment + 1;
}

int32_t validate(const gmvs_view_pass* views, int32_t n, const gmvs_params* p) {
    if (!views || n < 1) return fail(GMVS_ERR_INVALID, "no views");
    if (!p) return fail(GMVS_ERR_INVALID, "params is NULL");
    if (p->max_iterations < 0 || p->max_iterations > kMaxIters)
        return fail(GMVS_ERR_INVALID, "max_iterations must be in [0, 32]");
    if (p->patch_size < 1 || p->radius_increment < 1) return fail(GMVS_ERR_INVALID, "bad patch_size / radius_increment");
    if (p->sampler != GMVS_SAMPLER_CLAMP && p->sampler != GMVS_SAMPLER_TEX)
        return fail(GMVS_ERR_INVALID, "unknown sampler");
    if (p->staging < GMVS_STAGE_F32 || p->staging > GMVS_STAGE_AUTO) return fail(GMVS_ERR_INVALID, "unknown staging");
    if (p->init_kind < 0 || p->init_kind > 2 || p->sweep_kind < 0 || p->sweep_kind > 2)
        return fail(GMVS_ERR_INVALID, "unknown init_kind / sweep_kind");
    if (p->tile_h < 0 || p->tile_h > 8) return fail(GMVS_ERR_INVALID, "tile_h must be in [0, 8]");
    if (p->tile_w != 0 && p->tile_w != 16 && p->tile_w != 32)
        return fail(GMVS_ERR_INVALID, "tile_w must be 0, 16 or 32");
    if (p->ctas_per_sm < 0 || p->ctas_per_sm > 32) return fail(GMVS_ERR_INVALID, "ctas_per_sm must be in [0, 32]");
    if (p->split_sweep < 0 || p->split_sweep > 2) return fail(GMVS_ERR_INVALID, "split_sweep must be 0, 1 or 2");
    if (p->tex_storage != 0 && p->tex_storage != 1) return fail(GMVS_ERR_INVALID, "tex_storage must be 0 or 1");
    for (int v = 0; v < n; ++v) {
        const gmvs_view_pass& V = views[v];
        if (V.height < 1 || V.width < 1) return fail(GMVS_ERR_INVALID, "view " + std::to_string(v) + ": empty image");
        if ((long long)V.height * V.width * 4 > 0x7fffffffLL)
            return fail(GMVS_ERR_INVALID, "view " + std::to_string(v) + ": image too large");
        if (V.num_src < 1 || V.num_src > GMVS_MAX_NGB)
            return fail(GMVS_ERR_INVALID, "view " + std::to_string(v) + ": num_src must be in [1, 32]");
        for (int i = 0; i <= V.num_src; ++i)
            if (!V.images[i]) return fail(GMVS_ERR_INVALID, "view " + std::to_string(v) + ": image pointer is NULL");
        const bool need_dep = p->sweep_kind == GMVS_SWEEP_GEOM || p->init_kind == GMVS_INIT_DEPTH_NORMAL;
        if (need_dep)
            for (int i = 0; i <= V.num_src; ++i)
                if (!V.depths[i]) return fail(GMVS_ERR_INVALID, "view " + std::to_string(v) + ": depth map is NULL");
        if (p->init_kind == GMVS_INIT_DEPTH_NORMAL && !V.ref_normal)
            return fail(GMVS_ERR_INVALID, "view " + std::to_string(v) + ": ref_normal is NULL");
        if ((p->init_kind == GMVS_INIT_PRIOR || p->sweep_kind == GMVS_SWEEP_PRIOR) &&
            (!V.prior_planes || !V.prior_masks))
            return fail(GMVS_ERR_INVALID, "view " + std::to_string(v) + ": planar prior is NULL");
        if (p->init_kind == GMVS_INIT_PRIOR && (!V.init_planes || !V.init_costs))
            return fail(GMVS_ERR_INVALID, "view " + std::to_string(v) + ": previous pass planes/costs are NULL");
        if (!V.out_depth || !V.out_normal || !V.out_cost)
            return fail(GMVS_ERR_INVALID, "view " + std::to_string(v) + ": output pointer is NULL");
        for (int i = 0; i <= V.num_src; ++i)
            if (V.cams[i].K[0] == 0.0f || V.cams[i].K[4] == 0.0f)
                return fail(GMVS_ERR_INVALID, "view " + std::to_string(v) + ": camera focal length is zero");
    }
    return GMVS_OK;
}


int num_sms();

// Block and dynamic shared memory of a plan's half-sweep kernel.
LaunchShape sweep_shape(const gmvs_params* p, int nmax) {
    const int TW = tile_w_of(p), TH = tile_h_of(p);
    const size_t patch_bytes = (size_t)18 * (2 * TW * TH) * 8;  // kPatchSlots float2 per thread
    return LaunchShape{1, dim3(2 * TW, TH), (size_t)(nmax + 28) * TW * TH * 4 + patch_bytes, num_sms(),
                       p->ctas_per_sm, 0};
}

// Most resident CTAs per SM of that kernel (the neighbour-cost scratch is
// sized for them); 64 warps per SM when the query fails.
int sweep_max_ctas(int variant, const gmvs_params* p, int nmax) {
    const LaunchShape ls = sweep_shape(p, nmax);
    const bool generic = num_offsets(p) != 6;
    int c = 0;
    switch (variant) {
        case kVarF32: c = sweep_ctas_per_sm_f32(ls, generic); break;
        case kVarQuadF32: c = sweep_ctas_per_sm_qf32(ls, generic); break;
        case kVarQuadF16: c = sweep_ctas_per_sm_qf16(ls, generic); break;
        default: c = sweep_ctas_per_sm_tex(ls, generic); break;
    }
    return c > 0 ? c : 64 / tile_h_of(p);
}

Layout make_layout(const gmvs_view_pass* views, int32_t n, const gmvs_params* p, int variant, bool with_state) {
    Layout L;
    L.header = 256;
    L.views = align_up(L.header);
    size_t off = align_up(L.views + sizeof(DevView) * (size_t)n);
    const int TW = tile_w_of(p), TH = tile_h_of(p);
    int ntiles = 0;
    for (int v = 0; v < n; ++v) {
        const int hh = (views[v].height + 1) / 2;
        ntiles += tiles_across(views[v].width, p) * ((hh + TH - 1) / TH);
    }
    L.ntiles = ntiles;
    L.tiles = off;
    off = align_up(off + sizeof(Tile) * (size_t)ntiles);
    // unique images
    std::map<const float*, int> idx;
    L.view_slots.resize(n);
    const size_t bpp = bytes_per_pixel(variant, p);
    L.images = off;
    for (int v = 0; v < n; ++v) {
        for (int i = 0; i <= views[v].num_src; ++i) {
            const float* ptr = views[v].images[i];
            auto it = idx.find(ptr);
            int s;
            if (it == idx.end()) {
                ImageSlot sl{ptr, views[v].height, views[v].width, ~(size_t)0, 0};
                if (bpp) {
                    sl.pitch = variant == kVarTex ? align_up((size_t)sl.W * 4, 256) : (size_t)sl.W * bpp;
                    sl.offset = off;
                    off = align_up(off + sl.pitch * (size_t)sl.H);
                }
                s = (int)L.slots.size();
                L.slots.push_back(sl);
                idx[ptr] = s;
            } else {
                s = it->second;
            }
            L.view_slots[v].push_back(s);
        }
    }
    L.state = off;
    if (with_state) {
        for (int v = 0; v < n; ++v) {
            const size_t px = (size_t)views[v].height * views[v].width;
            L.view_state.push_back(off);
            off = align_up(off + px * 16 * 2);  // planes
            off = align_up(off + px * 4 * 2);   // costs
            off = align_up(off + px * 4 * 2);   // selected views
            off = align_up(off + px * 16);      // converted planes
        }
        int nmax = 1;
        for (int v = 0; v < n; ++v) nmax = std::max(nmax, views[v].num_src);
        L.ca = off;
        L.ca_ctas = sweep_max_ctas(variant, p, nmax);
        const size_t warps = (size_t)num_sms() * L.ca_ctas * tile_h_of(p);
        off = align_up(off + warps * 16 * 8 * nmax * sizeof(float));
        if (p->split_sweep) {
            // the three-kernel form keeps a ninth row (the current plane's
            // costs) and the refinement state
            const size_t units = (size_t)ntiles * tile_h_of(p);
            const size_t rows = p->split_sweep == 2 ? 9 : 8;
            L.nbc = off;
            off = align_up(off + units * 16 * rows * nmax * sizeof(float));
            L.nbi = off;
            off = align_up(off + units * 16 * 10 * sizeof(int));
            if (p->split_sweep == 2) {
                L.rfs = off;
                off = align_up(off + units * 16 * kRefineWords * sizeof(float));
            }
        }
    }
    L.total = off;
    return L;
}

void fill_view(DevView& D, const gmvs_view_pass& V, const gmvs_params* p) {
    std::memset(&D, 0, sizeof(D));
    D.init_kind = p->init_kind;
    D.sweep_kind = p->sweep_kind;
    D.pass_index = p->pass_index;
    D.H = V.height;
    D.W = V.width;
    D.N = V.num_src;
    D.stream_id = V.stream_id;
    D.depth_min = V.depth_min;
    D.depth_max = V.depth_max;
    for (int i = 0; i <= V.num_src; ++i) {
        std::memcpy(D.cam[i].K, V.cams[i].K, sizeof(float) * 9);
        std::memcpy(D.cam[i].R, V.cams[i].R, sizeof(float) * 9);
        std::memcpy(D.cam[i].t, V.cams[i].t, sizeof(float) * 3);
        D.dep[i] = V.depths[i];
    }
    // homography constants in FP64 (ComputeHomography, patch_match_kernel.cu:262-360)
    const gmvs_camera& r = V.cams[0];
    double Cr[3];
    for (int a = 0; a < 3; ++a)
        Cr[a] = -((double)r.R[0 * 3 + a] * r.t[0] + (double)r.R[1 * 3 + a] * r.t[1] + (double)r.R[2 * 3 + a] * r.t[2]);
    const double fx = r.K[0], fy = r.K[4], cx = r.K[2], cy = r.K[5];
    const double Kinv[9] = {1.0 / fx, 0.0, -cx / fx, 0.0, 1.0 / fy, -cy / fy, 0.0, 0.0, 1.0};
    for (int j = 0; j < V.num_src; ++j) {
        const gmvs_camera& s = V.cams[j + 1];
        double Cs[3], Rr[9], tr[3];
        for (int a = 0; a < 3; ++a)
            Cs[a] = -((double)s.R[0 * 3 + a] * s.t[0] + (double)s.R[1 * 3 + a] * s.t[1] +
                      (double)s.R[2 * 3 + a] * s.t[2]);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                Rr[a * 3 + b] = (double)s.R[a * 3 + 0] * r.R[b * 3 + 0] + (double)s.R[a * 3 + 1] * r.R[b * 3 + 1] +
                                (double)s.R[a * 3 + 2] * r.R[b * 3 + 2];
        for (int a = 0; a < 3; ++a)
            tr[a] = (double)s.R[a * 3 + 0] * (Cr[0] - Cs[0]) + (double)s.R[a * 3 + 1] * (Cr[1] - Cs[1]) +
                    (double)s.R[a * 3 + 2] * (Cr[2] - Cs[2]);
        const double Ks[9] = {s.K[0], 0.0, s.K[2], 0.0, s.K[4], s.K[5], 0.0, 0.0, s.K[8]};
        double KR[9];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                KR[a * 3 + b] = Ks[a * 3 + 0] * Rr[0 * 3 + b] + Ks[a * 3 + 1] * Rr[1 * 3 + b] + Ks[a * 3 + 2] * Rr[2 * 3 + b];
        float A[9], bv[3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                A[a * 3 + b] = (float)(KR[a * 3 + 0] * Kinv[0 * 3 + b] + KR[a * 3 + 1] * Kinv[1 * 3 + b] +
                                       KR[a * 3 + 2] * Kinv[2 * 3 + b]);
        for (int a = 0; a < 3; ++a)
            bv[a] = (float)(Ks[a * 3 + 0] * tr[0] + Ks[a * 3 + 1] * tr[1] + Ks[a * 3 + 2] * tr[2]);
        D.hs[j][0] = make_float4(A[0], A[1], A[2], A[3]);
        D.hs[j][1] = make_float4(A[4], A[5], A[6], A[7]);
        D.hs[j][2] = make_float4(A[8], bv[0], bv[1], bv[2]);
        D.hs[j][3] = make_float4((float)s.width, (float)s.height, 0.0f, 0.0f);
    }
    D.ref_normal = V.ref_normal;
    D.prior_planes = (const float4*)V.prior_planes;
    D.prior_masks = V.prior_masks;
    D.init_planes = (const float4*)V.init_planes;
    D.init_costs = V.init_costs;
    D.out_depth = V.out_depth;
    D.out_normal = V.out_normal;
    D.out_cost = V.out_cost;
    D.out_planes = (float4*)V.out_planes;
}

void fill_params(DevParams& P, const gmvs_params* p, int nmax) {
    std::memset(&P, 0, sizeof(P));
    P.patch_size = p->patch_size;
    P.radius_increment = p->radius_increment;
    P.top_k = p->top_k;
    P.sigma_spatial = p->sigma_spatial;
    P.sigma_color = p->sigma_color;
    P.init_kind = p->init_kind;
    P.sweep_kind = p->sweep_kind;
    P.sampler = p->sampler;
    P.staging = p->staging;
    P.seed_lo = (uint32_t)p->seed;
    P.seed_hi = (uint32_t)(p->seed >> 32);
    P.pass_index = p->pass_index;
    P.max_iterations = p->max_iterations;
    P.nmax = nmax;
    // cost_threshold = 0.8 * expf(iter*iter / -90) (patch_match_kernel.cu:1143)
    for (int it = 0; it < kMaxIters; ++it)
        P.cost_thr[it] = (float)(0.8 * (double)pmath::expf_((float)(it * it) / (-90.0f)));
}

int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

}  // namespace

struct gmvs_plan {
    int n_views = 0;
    gmvs_params params;
    DevParams dprm;
    int variant = 0;
    bool generic = false;
    int split = 0;        // half-sweeps as one, two or three kernels (gmvs_params.split_sweep)
    char* ws = nullptr;
    int* d_err = nullptr;
    int* d_ntiles = nullptr;  // tile queue: count, next unit, warps done
    DevView* d_views = nullptr;
    Tile* d_tiles = nullptr;
    int ntiles = 0;
    std::vector<cudaTextureObject_t> texs;
    std::vector<cudaArray_t> arrays;  // tex_storage == 1: one CUDA array per image slot
    std::vector<ImageSlot> slots;
    LaunchShape init_ls, sweep_ls, fin_ls;
    int num_stages = 0;
    int final_buf = 0;
};

namespace {

// Texture objects over the workspace copies (created once per plan).
int32_t create_textures(gmvs_plan* P, const Layout& L) {
    if (P->variant != kVarTex) return GMVS_OK;
    const bool arrays = P->params.tex_storage == 1;
    for (const ImageSlot& s : L.slots) {
        cudaResourceDesc rd;
        std::memset(&rd, 0, sizeof(rd));
        if (arrays) {  // the block-linear layout of module A's cudaMallocArray (planar_initer.cu:150-158)
            const cudaChannelFormatDesc cd = cudaCreateChannelDesc<float>();
            cudaArray_t a = nullptr;
            cudaError_t e = cudaMallocArray(&a, &cd, s.W, s.H);
            if (e != cudaSuccess) return fail_cuda(e, "allocating texture arrays");
            P->arrays.push_back(a);
            rd.resType = cudaResourceTypeArray;
            rd.res.array.array = a;
        } else {
            rd.resType = cudaResourceTypePitch2D;
            rd.res.pitch2D.devPtr = P->ws + s.offset;
            rd.res.pitch2D.desc = cudaCreateChannelDesc<float>();
            rd.res.pitch2D.width = s.W;
            rd.res.pitch2D.height = s.H;
            rd.res.pitch2D.pitchInBytes = s.pitch;
        }
        cudaTextureDesc td;  // the reference's descriptor (planar_initer.cu:150-158)
        std::memset(&td, 0, sizeof(td));
        td.addressMode[0] = cudaAddressModeWrap;
        td.addressMode[1] = cudaAddressModeWrap;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        cudaTextureObject_t tex = 0;
        cudaError_t e = cudaCreateTextureObject(&tex, &rd, &td, nullptr);
        if (e != cudaSuccess) return fail_cuda(e, "creating texture objects");
        P->texs.push_back(tex);
    }
    return GMVS_OK;
}

// Refresh the staged copies of the caller's images (every launch, so new
// image contents are always seen; capturable in a CUDA graph).
int32_t restage(const gmvs_plan* P, cudaStream_t st) {
    for (size_t k = 0; k < P->arrays.size(); ++k) {
        const ImageSlot& s = P->slots[k];
        cudaError_t e = cudaMemcpy2DToArrayAsync(P->arrays[k], 0, 0, s.src, (size_t)s.W * 4, (size_t)s.W * 4, s.H,
                                                 cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return fail_cuda(e, "staging texture arrays");
    }
    for (const ImageSlot& s : P->slots) {
        if (s.offset == ~(size_t)0) continue;
        void* dst = P->ws + s.offset;
        cudaError_t e = cudaSuccess;
        const int n = s.H * s.W;
        const int blocks = std::min((n + 255) / 256, num_sms() * 8);
        if (P->variant == kVarQuadF32) {
            k_stage_quad_f32<<<blocks, 256, 0, st>>>(s.src, (float4*)dst, s.H, s.W);
            e = cudaGetLastError();
        } else if (P->variant == kVarQuadF16) {
            k_stage_quad_f16<<<blocks, 256, 0, st>>>(s.src, (uint2*)dst, s.H, s.W);
            e = cudaGetLastError();
        } else if (P->variant == kVarTex) {
            e = cudaMemcpy2DAsync(dst, s.pitch, s.src, (size_t)s.W * 4, (size_t)s.W * 4, s.H, cudaMemcpyDeviceToDevice,
                                  st);
        }
        if (e != cudaSuccess) return fail_cuda(e, "staging images");
    }
    return GMVS_OK;
}

// Build descriptors + tiles for a plan over `views` and upload them.
int32_t build_plan(gmvs_plan* P, const gmvs_view_pass* views, int32_t n, const gmvs_params* p, void* workspace,
                   size_t ws_bytes, cudaStream_t st, bool with_state, int staging) {
    P->n_views = n;
    P->params = *p;
    P->variant = variant_of(p, staging);
    P->generic = num_offsets(p) != 6;
    const Layout L = make_layout(views, n, p, P->variant, with_state);
    if (!workspace || ws_bytes < L.total)
        return fail(GMVS_ERR_WORKSPACE, "workspace too small: need " + std::to_string(L.total) + " bytes, got " +
                                            std::to_string(ws_bytes));
    if (((uintptr_t)workspace) % 256 != 0) return fail(GMVS_ERR_INVALID, "workspace must be 256-byte aligned");
    P->ws = (char*)workspace;
    P->d_err = (int*)P->ws;
    P->d_ntiles = (int*)(P->ws + 4);
    P->d_views = (DevView*)(P->ws + L.views);
    P->d_tiles = (Tile*)(P->ws + L.tiles);
    P->ntiles = L.ntiles;
    int nmax = 1;
    for (int v = 0; v < n; ++v) nmax = std::max(nmax, views[v].num_src);
    fill_params(P->dprm, p, nmax);
    P->dprm.wide = wide_tiles(p) ? 1 : 0;
    if (with_state) {
        P->dprm.ca = (float*)(P->ws + L.ca);
        P->dprm.ca_slots = num_sms() * L.ca_ctas * tile_h_of(p);
        P->dprm.nb_units = p->split_sweep ? L.ntiles * tile_h_of(p) : 0;
        if (p->split_sweep) {
            P->dprm.nbc = (float*)(P->ws + L.nbc);
            P->dprm.nbi = (int*)(P->ws + L.nbi);
            if (p->split_sweep == 2) P->dprm.rfs = (float*)(P->ws + L.rfs);
        }
    }
    P->split = with_state ? p->split_sweep : 0;
    P->slots = L.slots;
    int32_t rc = create_textures(P, L);
    if (rc != GMVS_OK) return rc;
    std::vector<DevView> hv(n);
    std::vector<Tile> ht;
    ht.reserve(L.ntiles);
    const int TW = tile_w_of(p), TH = tile_h_of(p);
    size_t tex_i = 0;
    std::map<int, cudaTextureObject_t> slot_tex;
    for (size_t s = 0; s < L.slots.size(); ++s)
        if (P->variant == kVarTex) slot_tex[(int)s] = P->texs[tex_i++];
    for (int v = 0; v < n; ++v) {
        fill_view(hv[v], views[v], p);
        for (int i = 0; i <= views[v].num_src; ++i) {
            const ImageSlot& s = L.slots[L.view_slots[v][i]];
            hv[v].img[i] = s.offset == ~(size_t)0 ? (const void*)s.src : (const void*)(P->ws + s.offset);
            if (P->variant == kVarTex) hv[v].tex[i] = slot_tex[L.view_slots[v][i]];
        }
        if (with_state) {
            const size_t px = (size_t)views[v].height * views[v].width;
            char* b = P->ws + L.view_state[v];
            hv[v].plane[0] = (float4*)b;
            hv[v].plane[1] = (float4*)(b + px * 16);
            b = (char*)align_up((uintptr_t)(b + px * 32));
            hv[v].cost[0] = (float*)b;
            hv[v].cost[1] = (float*)(b + px * 4);
            b = (char*)align_up((uintptr_t)(b + px * 8));
            hv[v].sel[0] = (uint32_t*)b;
            hv[v].sel[1] = (uint32_t*)(b + px * 4);
            b = (char*)align_up((uintptr_t)(b + px * 8));
            hv[v].fin = (float4*)b;
        }
        const int hh = (views[v].height + 1) / 2;
        const int across = tiles_across(views[v].width, p);
        for (int y = 0; y < hh; y += TH)
            for (int k = 0; k < across; ++k) ht.push_back(Tile{v, k * TW, y, -1});
    }
    int hdr[4] = {0, L.ntiles, 0, 0};  // error word, tile queue (count, next unit, warps done)
    cudaError_t e = cudaMemcpyAsync(P->ws, hdr, sizeof(hdr), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(P->d_views, hv.data(), sizeof(DevView) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !ht.empty())
        e = cudaMemcpyAsync(P->d_tiles, ht.data(), sizeof(Tile) * ht.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // host vectors die at return
    if (e != cudaSuccess) return fail_cuda(e, "uploading plan descriptors");
    const int npix = TW * TH;
    const int grid = std::max(1, std::min(L.ntiles, num_sms() * 16));
    const size_t patch_bytes = (size_t)18 * (2 * TW * TH) * 8;  // kPatchSlots float2 per thread
    const int sms = num_sms();
    const int ctas = p->ctas_per_sm;
    P->init_ls = LaunchShape{grid, dim3(2 * TW, TH), (size_t)2 * nmax * npix * 4 + patch_bytes, sms, ctas};
    P->sweep_ls = sweep_shape(p, nmax);
    P->sweep_ls.grid = grid;
    P->sweep_ls.max_ctas = with_state ? L.ca_ctas : 0;
    P->fin_ls = LaunchShape{grid, dim3(TW, TH), 0, sms, 0};
    P->num_stages = 2 * p->max_iterations + 4;
    P->final_buf = p->max_iterations & 1;
    return GMVS_OK;
}

// AUTO staging: quad fp16 when every image is exactly representable.
int32_t resolve_auto(const gmvs_view_pass* views, int32_t n, const gmvs_params* p, void* ws, cudaStream_t st,
                     int* staging) {
    *staging = p->staging;
    if (p->sampler == GMVS_SAMPLER_TEX || p->staging != GMVS_STAGE_AUTO) return GMVS_OK;
    int* flag = (int*)ws;  // header scratch; rewritten by build_plan
    int one = 1;
    cudaError_t e = cudaMemcpyAsync(flag, &one, 4, cudaMemcpyHostToDevice, st);
    std::map<const float*, int> seen;
    for (int v = 0; v < n && e == cudaSuccess; ++v)
        for (int i = 0; i <= views[v].num_src; ++i) {
            if (seen.count(views[v].images[i])) continue;
            seen[views[v].images[i]] = 1;
            const int cnt = views[v].height * views[v].width;
            k_check_f16_exact<<<std::min((cnt + 255) / 256, num_sms() * 8), 256, 0, st>>>(views[v].images[i], cnt,
                                                                                          flag);
            e = cudaGetLastError();
            if (e != cudaSuccess) break;
        }
    int host = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&host, flag, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda(e, "checking images for fp16 staging");
    *staging = host ? GMVS_STAGE_QUAD_F16 : GMVS_STAGE_QUAD_F32;
    return GMVS_OK;
}

int32_t launch_stage(gmvs_plan* P, int stage, cudaStream_t st) {
    const int I = P->params.max_iterations;
    cudaError_t e = cudaSuccess;
    const DevView* dv = P->d_views;
    const Tile* dt = P->d_tiles;
    int* nt = P->d_ntiles;
    if (stage == 0) {
        int32_t rc = restage(P, st);
        if (rc != GMVS_OK) return rc;
        // the queue kernels reset it when they finish; clear it here too so a
        // chain that was interrupted by an error starts clean
        e = cudaMemsetAsync(nt + 1, 0, 2 * sizeof(int), st);
        if (e != cudaSuccess) return fail_cuda(e, "resetting the tile queue");
        switch (P->variant) {
            case kVarF32: e = launch_init_f32(P->init_ls, dv, P->dprm, dt, nt, P->d_err, P->generic, st); break;
            case kVarQuadF32: e = launch_init_qf32(P->init_ls, dv, P->dprm, dt, nt, P->d_err, P->generic, st); break;
            case kVarQuadF16: e = launch_init_qf16(P->init_ls, dv, P->dprm, dt, nt, P->d_err, P->generic, st); break;
            default: e = launch_init_tex(P->init_ls, dv, P->dprm, dt, nt, P->d_err, P->generic, st); break;
        }
    } else if (stage <= 2 * I) {
        const int s = stage - 1;
        switch (P->variant) {
            case kVarF32:
                e = launch_sweep_f32(P->sweep_ls, dv, P->dprm, dt, nt, s, P->d_err, P->generic, P->split, st);
                break;
            case kVarQuadF32:
                e = launch_sweep_qf32(P->sweep_ls, dv, P->dprm, dt, nt, s, P->d_err, P->generic, P->split, st);
                break;
            case kVarQuadF16:
                e = launch_sweep_qf16(P->sweep_ls, dv, P->dprm, dt, nt, s, P->d_err, P->generic, P->split, st);
                break;
            default:
                e = launch_sweep_tex(P->sweep_ls, dv, P->dprm, dt, nt, s, P->d_err, P->generic, P->split, st);
                break;
        }
    } else if (stage == 2 * I + 1) {
        e = launch_convert(P->fin_ls, dv, dt, nt, P->final_buf, st);
    } else if (stage == 2 * I + 2 || stage == 2 * I + 3) {
        e = launch_filter(P->fin_ls, dv, dt, nt, P->final_buf, stage - (2 * I + 2), P->params.run_filter, st);
    } else {
        return fail(GMVS_ERR_INVALID, "stage out of range");
    }
    if (e != cudaSuccess) return fail_cuda(e, ("launching stage " + std::to_string(stage)).c_str());
    return GMVS_OK;
}

}  // namespace

extern "C" size_t gmvs_plan_workspace_bytes(const gmvs_view_pass* views, int32_t n_views, const gmvs_params* params) {
    if (validate(views, n_views, params) != GMVS_OK) return 0;
    // AUTO may pick quad f32, the larger staging: size for it
    int staging = params->staging == GMVS_STAGE_AUTO ? GMVS_STAGE_QUAD_F32 : params->staging;
    return make_layout(views, n_views, params, variant_of(params, staging), true).total;
}

extern "C" int32_t gmvs_plan_create(const gmvs_view_pass* views, int32_t n_views, const gmvs_params* params,
                                    void* workspace, size_t workspace_bytes, void* stream, gmvs_plan** out) {
    if (!out) return fail(GMVS_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int32_t rc = validate(views, n_views, params);
    if (rc != GMVS_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (!workspace || workspace_bytes < 256) return fail(GMVS_ERR_WORKSPACE, "workspace too small");
    int staging = GMVS_STAGE_F32;
    rc = resolve_auto(views, n_views, params, workspace, st, &staging);
    if (rc != GMVS_OK) return rc;
    gmvs_plan* P = new gmvs_plan();
    rc = build_plan(P, views, n_views, params, workspace, workspace_bytes, st, true, staging);
    if (rc != GMVS_OK) {
        gmvs_plan_destroy(P);
        return rc;
    }
    *out = P;
    return GMVS_OK;
}

extern "C" int32_t gmvs_plan_num_stages(const gmvs_plan* plan) { return plan ? plan->num_stages : 0; }

extern "C" int32_t gmvs_plan_launch_stage(gmvs_plan* plan, int32_t stage, void* stream) {
    if (!plan) return fail(GMVS_ERR_INVALID, "plan is NULL");
    return launch_stage(plan, stage, (cudaStream_t)stream);
}

extern "C" int32_t gmvs_plan_launch(gmvs_plan* plan, void* stream) {
    if (!plan) return fail(GMVS_ERR_INVALID, "plan is NULL");
    for (int s = 0; s < plan->num_stages; ++s) {
        int32_t rc = launch_stage(plan, s, (cudaStream_t)stream);
        if (rc != GMVS_OK) return rc;
    }
    return GMVS_OK;
}

extern "C" int32_t gmvs_plan_check(gmvs_plan* plan, void* stream) {
    if (!plan) return fail(GMVS_ERR_INVALID, "plan is NULL");
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, plan->d_err, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return fail_cuda(e, "plan execution");
    if (err) return fail(GMVS_ERR_DEVICE, "kernel error status " + std::to_string(err));
    return GMVS_OK;
}

extern "C" void gmvs_plan_destroy(gmvs_plan* plan) {
    if (!plan) return;
    for (cudaTextureObject_t t : plan->texs) cudaDestroyTextureObject(t);
    for (cudaArray_t a : plan->arrays) cudaFreeArray(a);
    delete plan;
}

extern "C" int32_t gmvs_run_passes(const gmvs_view_pass* views, int32_t n_views, const gmvs_params* params,
                                   void* workspace, size_t workspace_bytes, void* stream) {
    gmvs_plan* P = nullptr;
    int32_t rc = gmvs_plan_create(views, n_views, params, workspace, workspace_bytes, stream, &P);
    if (rc != GMVS_OK) return rc;
    rc = gmvs_plan_launch(P, stream);
    if (rc == GMVS_OK) rc = gmvs_plan_check(P, stream);
    gmvs_plan_destroy(P);
    return rc;
}

// ------------------------------------------------------------------ NCC --
extern "C" size_t gmvs_ncc_workspace_bytes(const gmvs_view_pass* view, const gmvs_params* params) {
    if (!view || !params) return 0;
    int staging = params->staging == GMVS_STAGE_AUTO ? GMVS_STAGE_QUAD_F32 : params->staging;
    return make_layout(view, 1, params, variant_of(params, staging), false).total;
}

extern "C" int32_t gmvs_ncc_costs(const gmvs_view_pass* view, const gmvs_params* params, const float* planes,
                                  float* costs, float* init_cost, uint32_t* init_views, void* workspace,
                                  size_t workspace_bytes, void* stream) {
    if (!view || !params) return fail(GMVS_ERR_INVALID, "view/params is NULL");
    if (!planes) return fail(GMVS_ERR_INVALID, "planes is NULL");
    if (view->num_src < 1 || view->num_src > GMVS_MAX_NGB) return fail(GMVS_ERR_INVALID, "num_src must be in [1, 32]");
    if (view->height < 1 || view->width < 1) return fail(GMVS_ERR_INVALID, "empty image");
    for (int i = 0; i <= view->num_src; ++i)
        if (!view->images[i]) return fail(GMVS_ERR_INVALID, "image pointer is NULL");
    if (params->patch_size < 1 || params->radius_increment < 1)
        return fail(GMVS_ERR_INVALID, "bad patch_size / radius_increment");
    cudaStream_t st = (cudaStream_t)stream;
    if (!workspace || workspace_bytes < 256) return fail(GMVS_ERR_WORKSPACE, "workspace too small");
    int staging = GMVS_STAGE_F32;
    int32_t rc = resolve_auto(view, 1, params, workspace, st, &staging);
    if (rc != GMVS_OK) return rc;
    gmvs_plan P;
    rc = build_plan(&P, view, 1, params, workspace, workspace_bytes, st, false, staging);
    if (rc == GMVS_OK) rc = restage(&P, st);
    if (rc == GMVS_OK) {
        cudaError_t e;
        const float4* pl = (const float4*)planes;
        switch (P.variant) {
            case kVarF32:
                e = launch_ncc_f32(P.init_ls, P.d_views, P.dprm, P.d_tiles, P.d_ntiles, pl, costs, init_cost,
                                   init_views, P.generic, st);
                break;
            case kVarQuadF32:
                e = launch_ncc_qf32(P.init_ls, P.d_views, P.dprm, P.d_tiles, P.d_ntiles, pl, costs, init_cost,
                                    init_views, P.generic, st);
                break;
            case kVarQuadF16:
                e = launch_ncc_qf16(P.init_ls, P.d_views, P.dprm, P.d_tiles, P.d_ntiles, pl, costs, init_cost,
                                    init_views, P.generic, st);
                break;
            default:
                e = launch_ncc_tex(P.init_ls, P.d_views, P.dprm, P.d_tiles, P.d_ntiles, pl, costs, init_cost,
                                   init_views, P.generic, st);
                break;
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = fail_cuda(e, "NCC kernel");
    }
    for (cudaTextureObject_t t : P.texs) cudaDestroyTextureObject(t);
    P.texs.clear();
    for (cudaArray_t a : P.arrays) cudaFreeArray(a);
    P.arrays.clear();
    return rc;
}
