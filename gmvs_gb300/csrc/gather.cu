// Point gather of the fusion scripts (mvs_fusion_segmentaion.py:195-236) as
// one device pass per view: for every pixel with depth > 0 the world point
//   p = o + depth * R d,   d = ((x - cx) / fx, (y - cy) / fy, 1),
// (R, o = rotation and centre of the camera-to-world pose) with its normal,
// in raster order; the points whose normal faces the camera,
// dot(-R d, n) > cos_thresh, go to a second list, and the depth/normal maps
// keep only those pixels.  Raster order is kept by an ordered compaction:
// per-block counts, one scan over the blocks, then each block writes at its
// offset with a block-local scan.
#include <algorithm>
#include <cstdint>
#include <string>

#include "common.cuh"
#include "errors.h"

namespace gmvs {
namespace {

constexpr int kGatherBlock = 256;

struct GatherArgs {
    const float* depth;   // [H][W]
    const float* normal;  // [H][W][3]
    int H, W;
    float fx, fy, cx, cy;
    float R[9];  // camera-to-world rotation, row-major
    float o[3];  // camera centre
    float cos_thresh;
};

struct PixelPoint {
    bool valid, facing;
    float p[3], n[3];
};

__device__ __forceinline__ PixelPoint eval_pixel(const GatherArgs& a, int k) {
    PixelPoint r;
    const float d = a.depth[k];
    r.valid = d > 0.0f;
    r.facing = false;
    if (!r.valid) return r;
    const int y = k / a.W, x = k - y * a.W;
    const float dx = ((float)x - a.cx) / a.fx, dy = ((float)y - a.cy) / a.fy;
    float dir[3];
    for (int i = 0; i < 3; ++i) dir[i] = a.R[3 * i] * dx + a.R[3 * i + 1] * dy + a.R[3 * i + 2];
    for (int i = 0; i < 3; ++i) {
        r.p[i] = a.o[i] + d * dir[i];
        r.n[i] = a.normal[(size_t)k * 3 + i];
    }
    const float dot = -dir[0] * r.n[0] + -dir[1] * r.n[1] + -dir[2] * r.n[2];
    r.facing = dot > a.cos_thresh;
    return r;
}

// block-wide exclusive scan of two flags; returns the block totals
__device__ __forceinline__ int2 block_scan2(int f0, int f1, int& e0, int& e1) {
    __shared__ int s0[kGatherBlock / 32], s1[kGatherBlock / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned b0 = __ballot_sync(0xffffffffu, f0), b1 = __ballot_sync(0xffffffffu, f1);
    const unsigned below = (1u << lane) - 1u;
    e0 = __popc(b0 & below);
    e1 = __popc(b1 & below);
    if (lane == 0) {
        s0[w] = __popc(b0);
        s1[w] = __popc(b1);
    }
    __syncthreads();
    int t0 = 0, t1 = 0, p0 = 0, p1 = 0;
    for (int i = 0; i < kGatherBlock / 32; ++i) {
        if (i == w) {
            p0 = t0;
            p1 = t1;
        }
        t0 += s0[i];
        t1 += s1[i];
    }
    e0 += p0;
    e1 += p1;
    __syncthreads();
    return make_int2(t0, t1);
}

__global__ void k_gather_count(GatherArgs a, int2* __restrict__ block_counts) {
    const int k = blockIdx.x * kGatherBlock + threadIdx.x;
    int f0 = 0, f1 = 0;
    if (k < a.H * a.W) {
        const PixelPoint r = eval_pixel(a, k);
        f0 = r.valid;
        f1 = r.valid && r.facing;
    }
    int e0, e1;
    const int2 t = block_scan2(f0, f1, e0, e1);
    if (threadIdx.x == 0) block_counts[blockIdx.x] = t;
}

// exclusive scan over the blocks (one CTA); totals into totals[0..1]
__global__ void k_gather_scan(int2* __restrict__ block_counts, int nblocks, long long* __restrict__ totals) {
    __shared__ int2 part[1024];
    const int t = threadIdx.x, T = blockDim.x;
    const int per = (nblocks + T - 1) / T;
    const int b = t * per, e = min(nblocks, b + per);
    int2 sum = make_int2(0, 0);
    for (int i = b; i < e; ++i) {
        sum.x += block_counts[i].x;
        sum.y += block_counts[i].y;
    }
    part[t] = sum;
    __syncthreads();
    if (t == 0) {
        int2 run = make_int2(0, 0);
        for (int i = 0; i < T; ++i) {
            const int2 v = part[i];
            part[i] = run;
            run.x += v.x;
            run.y += v.y;
        }
        totals[0] = run.x;
        totals[1] = run.y;
    }
    __syncthreads();
    int2 run = part[t];
    for (int i = b; i < e; ++i) {
        const int2 v = block_counts[i];
        block_counts[i] = run;
        run.x += v.x;
        run.y += v.y;
    }
}

__global__ void k_gather_write(GatherArgs a, const int2* __restrict__ block_offsets, float* __restrict__ all_pts,
                               float* __restrict__ facing_pts, float* __restrict__ out_depth,
                               float* __restrict__ out_normal) {
    const int k = blockIdx.x * kGatherBlock + threadIdx.x;
    const bool in = k < a.H * a.W;
    PixelPoint r;
    r.valid = r.facing = false;
    if (in) r = eval_pixel(a, k);
    const int f0 = r.valid, f1 = r.valid && r.facing;
    int e0, e1;
    block_scan2(f0, f1, e0, e1);
    if (!in) return;
    const int2 base = block_offsets[blockIdx.x];
    if (f0) {
        float* q = all_pts + (size_t)(base.x + e0) * 6;
        q[0] = r.p[0], q[1] = r.p[1], q[2] = r.p[2], q[3] = r.n[0], q[4] = r.n[1], q[5] = r.n[2];
    }
    if (f1 && facing_pts) {
        float* q = facing_pts + (size_t)(base.y + e1) * 6;
        q[0] = r.p[0], q[1] = r.p[1], q[2] = r.p[2], q[3] = r.n[0], q[4] = r.n[1], q[5] = r.n[2];
    }
    if (out_depth) out_depth[k] = f1 ? a.depth[k] : 0.0f;
    if (out_normal)
        for (int i = 0; i < 3; ++i) out_normal[(size_t)k * 3 + i] = f1 ? a.normal[(size_t)k * 3 + i] : 0.0f;
}

}  // namespace
}  // namespace gmvs

extern "C" size_t gmvs_gather_workspace_bytes(int32_t height, int32_t width) {
    if (height < 1 || width < 1) return 0;
    const size_t blocks = ((size_t)height * width + gmvs::kGatherBlock - 1) / gmvs::kGatherBlock;
    return 256 + ((blocks * sizeof(int2) + 255) & ~(size_t)255);
}

extern "C" int32_t gmvs_gather_points(const float* depth, const float* normal, int32_t height, int32_t width,
                                      const float* intrinsics, const float* pose, float cos_thresh,
                                      float* out_points, float* out_facing, float* out_depth, float* out_normal,
                                      int64_t* out_counts, void* workspace, size_t workspace_bytes, void* stream) {
    using namespace gmvs;
    if (!depth || !normal || !intrinsics || !pose || !out_points || !out_counts)
        return fail(GMVS_ERR_INVALID, "gmvs_gather_points: NULL argument");
    if (height < 1 || width < 1 || (long long)height * width > 0x7fffffffLL)
        return fail(GMVS_ERR_INVALID, "gmvs_gather_points: bad image size");
    const size_t need = gmvs_gather_workspace_bytes(height, width);
    if (!workspace || workspace_bytes < need || (uintptr_t)workspace % 256)
        return fail(GMVS_ERR_WORKSPACE,
                    "gmvs_gather_points: workspace must be 256-byte aligned and hold " + std::to_string(need));
    GatherArgs a;
    a.depth = depth;
    a.normal = normal;
    a.H = height;
    a.W = width;
    a.fx = intrinsics[0];
    a.fy = intrinsics[4];
    a.cx = intrinsics[2];
    a.cy = intrinsics[5];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) a.R[3 * i + j] = pose[4 * i + j];
        a.o[i] = pose[4 * i + 3];
    }
    a.cos_thresh = cos_thresh;
    if (a.fx == 0.0f || a.fy == 0.0f) return fail(GMVS_ERR_INVALID, "gmvs_gather_points: zero focal length");
    cudaStream_t st = (cudaStream_t)stream;
    long long* totals = (long long*)workspace;
    int2* blocks = (int2*)((char*)workspace + 256);
    const int nb = (int)(((size_t)height * width + kGatherBlock - 1) / kGatherBlock);
    k_gather_count<<<nb, kGatherBlock, 0, st>>>(a, blocks);
    k_gather_scan<<<1, 1024, 0, st>>>(blocks, nb, totals);
    k_gather_write<<<nb, kGatherBlock, 0, st>>>(a, blocks, out_points, out_facing, out_depth, out_normal);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_counts, totals, 2 * sizeof(long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda(e, "gmvs_gather_points");
    return GMVS_OK;
}
