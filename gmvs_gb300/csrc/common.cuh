// Device-side data layout and helpers shared by the PatchMatch and fusion
// kernels.  Host code fills DevView/DevParams/Tile (see runtime.cu); kernels
// only read them.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gmvs_gb300.h"

namespace gmvs {

constexpr int kMaxNgb = GMVS_MAX_NGB;
constexpr int kMaxIters = 32;

// Error bits a kernel may raise in the plan's device error word.
enum : int { kErrBadView = 1, kErrBadStage = 2 };

struct DevCam {  // world -> camera, as gmvs_camera without the extents
    float K[9];
    float R[9];
    float t[3];
};

// One reference view of a pass.  Homography of plane (n, w) in the ref
// camera frame towards source j is H = A_j - b_j g^T with
//   A_j = K_s R_rel K_r^-1,  b_j = K_s t_rel,
//   g   = (n_x / fx, n_y / fy, n_z - n_x cx / fx - n_y cy / fy) / w,
// which is ComputeHomography (patch_match_kernel.cu:262-360) re-associated;
// A_j and b_j are formed once per view pair in FP64 and rounded once.
// Per source view j, hs[j] packs A_j, b_j and the centre-test extents into
// four 16-byte words (one vector load each):
//   hs[j][0] = A0 A1 A2 A3,  hs[j][1] = A4 A5 A6 A7,  hs[j][2] = A8 b0 b1 b2,
//   hs[j][3] = src width, src height, 0, 0.
struct DevView {
    int H, W, N, stream_id;
    int init_kind, sweep_kind, pass_index;  // per view, so one launch can mix passes
    float depth_min, depth_max;
    int pad_[3];
    float4 hs[kMaxNgb][4];
    DevCam cam[1 + kMaxNgb];  // ref, then sources (geometric term, conversions)
    const void* img[1 + kMaxNgb];           // CLAMP sampler: staged planes
    unsigned long long tex[1 + kMaxNgb];    // TEX sampler: texture objects
    const float* dep[1 + kMaxNgb];          // GEOM: input depth maps
    const float* ref_normal;                // DEPTH_NORMAL init
    const float4* prior_planes;
    const uint32_t* prior_masks;
    const float4* init_planes;
    const float* init_costs;
    float4* plane[2];   // ping-pong state
    float* cost[2];
    uint32_t* sel[2];
    float4* fin;        // converted (world normal, depth) planes for the filter
    float* out_depth;
    float* out_normal;
    float* out_cost;
    float4* out_planes;
};

struct DevParams {
    int patch_size, radius_increment, top_k;
    float sigma_spatial, sigma_color;
    int init_kind, sweep_kind, sampler, staging;
    uint32_t seed_lo, seed_hi;
    int pass_index, max_iterations;
    int nmax;  // largest N of the plan (shared-memory stride)
    float cost_thr[kMaxIters];
    // The 8 x nmax neighbour-cost matrix of every pixel in flight lives in
    // global memory (L2-resident), one block of 8 * nmax * 16 floats per
    // resident warp: block (blockIdx.x * blockDim.y + threadIdx.y), element
    // (k * nmax + i) * 16 + pixel-in-warp.  Keeping it out of shared memory
    // lets more warps be resident.
    float* ca;
    // Split half-sweeps (two kernels): the neighbour-cost matrix and the
    // neighbour positions of every pixel of a launch, per work unit u (one
    // thread row of a tile): nbc + u * 8 * nmax * 16, nbi + u * 10 * 16.
    float* nbc;
    int* nbi;
    // Three-kernel half-sweeps: nbc holds a ninth row (the current plane's
    // costs) and rfs + u * kRefineWords * 16 the refinement state.
    float* rfs;
    int ca_slots;  // warp blocks in `ca`
    int nb_units;  // unit blocks in `nbc` / `nbi`
    int wide;      // 32-pixel-wide tiles: the tile list pairs 16-column tiles (see unit_tile)
};

// A tile is TW columns x TH thread rows of one view; thread row r covers
// image rows 2*(yh0 + r) and 2*(yh0 + r) + 1 (zig-zag by column parity, the
// reference's red/black launch mapping, patch_match_kernel.cu:1592-1599).
// stage < 0: use the launch's stage argument.
struct Tile {
    int view, x0, yh0, stage;
};

// ---------------------------------------------------------------- Philox --
// Philox4x32-10 (Salmon et al., SC'11).  Key = seed; counter = (pixel,
// stream, phase, block), phase = pass_index << 8 | step (0 init, 1 + 2*iter +
// colour for the sweeps).  Uniforms are ((x >> 8) + 1) * 2^-24 in (0, 1].
__device__ __forceinline__ uint4 philox10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k.x += 0x9E3779B9u;
            k.y += 0xBB67AE85u;
        }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

struct DevRng {
    uint2 key;
    uint4 ctr;
    uint4 buf;
    int left;
    __device__ __forceinline__ DevRng(uint32_t seed_lo, uint32_t seed_hi, uint32_t pixel, uint32_t stream,
                                      uint32_t phase) {
        key = make_uint2(seed_lo, seed_hi);
        ctr = make_uint4(pixel, stream, phase, 0u);
        left = 0;
    }
    __device__ __forceinline__ float uniform() {
        if (left == 0) {
            buf = philox10(ctr, key);
            ctr.w += 1u;
            left = 4;
        }
        const uint32_t x = buf.x;
        buf.x = buf.y;
        buf.y = buf.z;
        buf.z = buf.w;
        --left;
        return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f);
    }
};

__device__ __forceinline__ uint32_t phase_of(int pass_index, int step) {
    return ((uint32_t)pass_index << 8) | (uint32_t)step;
}

// ------------------------------------------------------------ tile queue --
// q[0] = tiles in the list, q[1] = next unit to claim, q[2] = warps done.
// A unit is one thread row of one tile (16 pixel columns of one row pair).
// Warps claim units in list order, so the units in flight at any moment are
// one compact run of the list -- a band of rows of one view -- whose source
// footprint stays in L2; a static stride over the list lets the resident
// CTAs drift apart across the whole batch and thrash L2 at full size.  The
// last warp to finish resets the queue for the next launch on the stream.
// Work unit u (one thread row of one 16-column tile) -> (tile, thread row).
// Plain order: all TH rows of tile t, then tile t + 1.  Wide (32-pixel) tiles:
// the tile list holds 16-column tiles in left/right pairs, and consecutive
// units alternate between the two halves of one row, so the warps in flight
// cover a 32 x 2*TH pixel block.
__device__ __forceinline__ void unit_tile(int u, int TH, int wide, int& t, int& row) {
    if (!wide) {
        t = u / TH;
        row = u - t * TH;
        return;
    }
    const int s = u / (2 * TH), r = u - s * 2 * TH;
    row = r >> 1;
    t = 2 * s + (r & 1);
}
// Drops a warp-private scratch block whose contents are dead from L2 without
// writing it back to DRAM (PTX `discard.global.L2`, a weak write of an
// indeterminate value to each 128-byte line).  `base` is 128-byte aligned and
// `bytes` a multiple of 128.  The warp barriers order every lane's last reads
// of the block before the discards and the discards before the next writes.
__device__ __forceinline__ void discard_l2_block(const void* base, int bytes, unsigned lane) {
    __syncwarp();
    const size_t g = __cvta_generic_to_global(base);
    for (int off = (int)lane * 128; off < bytes; off += 32 * 128)
        asm volatile("discard.global.L2 [%0], 128;" ::"l"(g + (size_t)off) : "memory");
    __syncwarp();
}
__device__ __forceinline__ int claim_unit(int* q, unsigned lane) {
    int u = 0;
    if (lane == 0) u = atomicAdd(q + 1, 1);
    return __shfl_sync(0xffffffffu, u, 0);
}
__device__ __forceinline__ void release_queue(int* q, unsigned lane) {
    if (lane == 0) {
        __threadfence();
        const int warps = (int)(gridDim.x * blockDim.y);
        if (atomicAdd(q + 2, 1) == warps - 1) {
            q[1] = 0;
            q[2] = 0;
        }
    }
}

// ---------------------------------------------------- bounds-checked build --
// Built with -DGMVS_BOUNDS_CHECK, every gathered index (image taps, depth
// taps, neighbour costs and planes, per-warp and per-pixel scratch) is
// tested against its array: an index outside it raises a bit in this
// module's violation word (read by gmvs_bounds_violations) and the access
// reads element 0 instead.  Compute-sanitizer's stand-in; the normal build
// compiles the checks away.
#ifdef GMVS_BOUNDS_CHECK
static __device__ unsigned int g_oob;
__device__ __forceinline__ long long checked_index(long long i, long long n, unsigned bit) {
    if (i < 0 || i >= n) {
        atomicOr(&g_oob, bit);
        return 0;
    }
    return i;
}
#define GMVS_IDX(i, n, bit) ((int)gmvs::checked_index((long long)(i), (long long)(n), (bit)))
#else
#define GMVS_IDX(i, n, bit) (i)
#endif
// violation bits
enum : unsigned { kOobImage = 1, kOobDepth = 2, kOobNeighbour = 4, kOobScratch = 8 };

// --------------------------------------------------------------- helpers --
__device__ __forceinline__ float lerpf(float a, float b, float w) { return fmaf(w, b - a, a); }

// module B bilinear_interpolate (gmvs/src/patch_match.cu:10-33)
__device__ __forceinline__ float bilinear_clamp(const float* __restrict__ img, float u, float v, int H, int W) {
    const int hl = min(max(__float2int_rz(v), 0), H - 1);
    const int wl = min(max(__float2int_rz(u), 0), W - 1);
    const float hd = v - (float)hl;
    const float wd = u - (float)wl;
    const int hu = (hl == H - 1) ? hl : hl + 1;
    const int wu = (wl == W - 1) ? wl : wl + 1;
    [[maybe_unused]] const int n = H * W;  // read by the bounds-checked build
    const float v0 = __ldg(img + GMVS_IDX(hl * W + wl, n, kOobDepth));
    const float v1 = __ldg(img + GMVS_IDX(hl * W + wu, n, kOobDepth));
    const float v2 = __ldg(img + GMVS_IDX(hu * W + wl, n, kOobDepth));
    const float v3 = __ldg(img + GMVS_IDX(hu * W + wu, n, kOobDepth));
    return lerpf(lerpf(v0, v1, wd), lerpf(v2, v3, wd), hd);
}

// Get3DPointonWorld_cu (patch_match_kernel.cu:590-620)
__device__ __forceinline__ void point_on_world(float x, float y, float depth, const DevCam& c, float out[3]) {
    const float px = depth * (x - c.K[2]) / c.K[0];
    const float py = depth * (y - c.K[5]) / c.K[4];
    const float pz = depth;
    const float tx = c.R[0] * px + c.R[3] * py + c.R[6] * pz;
    const float ty = c.R[1] * px + c.R[4] * py + c.R[7] * pz;
    const float tz = c.R[2] * px + c.R[5] * py + c.R[8] * pz;
    const float Cx = -(c.R[0] * c.t[0] + c.R[3] * c.t[1] + c.R[6] * c.t[2]);
    const float Cy = -(c.R[1] * c.t[0] + c.R[4] * c.t[1] + c.R[7] * c.t[2]);
    const float Cz = -(c.R[2] * c.t[0] + c.R[5] * c.t[1] + c.R[8] * c.t[2]);
    out[0] = tx + Cx;
    out[1] = ty + Cy;
    out[2] = tz + Cz;
}

// ProjectonCamera_cu (patch_match_kernel.cu:622-648)
__device__ __forceinline__ void project_on_camera(const float X[3], const DevCam& c, float& u, float& v,
                                                  float& depth) {
    const float tx = c.R[0] * X[0] + c.R[1] * X[1] + c.R[2] * X[2] + c.t[0];
    const float ty = c.R[3] * X[0] + c.R[4] * X[1] + c.R[5] * X[2] + c.t[1];
    const float tz = c.R[6] * X[0] + c.R[7] * X[1] + c.R[8] * X[2] + c.t[2];
    depth = c.K[6] * tx + c.K[7] * ty + c.K[8] * tz;
    u = (c.K[0] * tx + c.K[1] * ty + c.K[2] * tz) / depth;
    v = (c.K[3] * tx + c.K[4] * ty + c.K[5] * tz) / depth;
}

}  // namespace gmvs
