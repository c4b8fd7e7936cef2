// View-selection scores of the COLMAP conversion (calc_score,
// gmvs/scripts/colmap2mvs.py:324-357) for every image pair at once: one warp
// per pair.  The shared points are found by binary search of image i's
// points in image j's sorted list; each contributes one to the score and
// its triangulation angle, in degrees and FP64 as the script computes it, is
// tested against 1 degree.  The script zeroes a score whose 75th-percentile
// angle, sorted(angles)[int(0.75 * n)], is below 1 degree; that element is
// below 1 exactly when more than int(0.75 * n) of the angles are, so no sort
// is needed.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>

#include "common.cuh"
#include "errors.h"

namespace gmvs {
namespace {

__device__ __forceinline__ bool contains(const int32_t* __restrict__ a, long long n, int32_t key) {
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (a[mid] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo < n && a[lo] == key;
}

// pairs (i, j), i < j, in row-major order of the upper triangle; ids
// outside [0, num_points) are not read (the wrapper rejects them first)
__global__ void k_view_scores(const long long* __restrict__ off, const int32_t* __restrict__ ids, int V,
                              int num_points, const double* __restrict__ xyz, const double* __restrict__ centers,
                              float* __restrict__ scores, long long npairs) {
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long p = warp; p < npairs; p += nwarps) {
        // decode p -> (i, j): row i holds V - 1 - i pairs and starts at
        // p_i = i (2V - 1 - i) / 2; estimate i from the quadratic, then fix
        const double tv = 2.0 * V - 1.0;
        int i = (int)((tv - sqrt(tv * tv - 8.0 * (double)p)) * 0.5);
        i = max(0, min(i, V - 2));
        auto row_start = [V](long long r) { return r * (2LL * V - 1 - r) / 2; };
        while (i > 0 && row_start(i) > p) --i;
        while (i < V - 2 && row_start(i + 1) <= p) ++i;
        const int j = i + 1 + (int)(p - row_start(i));
        const int32_t* a = ids + off[i];
        const long long na = off[i + 1] - off[i];
        const int32_t* b = ids + off[j];
        const long long nb = off[j + 1] - off[j];
        const double cix = centers[3 * i], ciy = centers[3 * i + 1], ciz = centers[3 * i + 2];
        const double cjx = centers[3 * j], cjy = centers[3 * j + 1], cjz = centers[3 * j + 2];
        long long n = 0, below = 0;
        for (long long k = lane; k < na; k += 32) {
            const int32_t id = a[k];
            if (id < 0 || id >= num_points || !contains(b, nb, id)) continue;
            const double px = xyz[3 * (size_t)id], py = xyz[3 * (size_t)id + 1], pz = xyz[3 * (size_t)id + 2];
            const double ax = cix - px, ay = ciy - py, az = ciz - pz;
            const double bx = cjx - px, by = cjy - py, bz = cjz - pz;
            const double dot = ax * bx + ay * by + az * bz;
            const double la = sqrt(ax * ax + ay * ay + az * az), lb = sqrt(bx * bx + by * by + bz * bz);
            const double theta = (180.0 / 3.14159265358979323846) * acos(dot / la / lb);
            ++n;
            below += theta < 1.0;
        }
        for (int o = 16; o > 0; o >>= 1) {
            n += __shfl_xor_sync(0xffffffffu, n, o);
            below += __shfl_xor_sync(0xffffffffu, below, o);
        }
        if (lane == 0) {
            const long long k75 = (long long)((double)n * 0.75);
            const float s = (n > 0 && below > k75) ? 0.0f : (float)n;
            scores[(size_t)i * V + j] = s;
            scores[(size_t)j * V + i] = s;
        }
    }
}

}  // namespace
}  // namespace gmvs

extern "C" int32_t gmvs_view_scores(const long long* offsets, const int32_t* point_ids, int32_t num_images,
                                    const double* xyz, int32_t num_points, const double* centers, float* scores,
                                    void* stream) {
    using namespace gmvs;
    if (!offsets || !point_ids || !xyz || !centers || !scores)
        return fail(GMVS_ERR_INVALID, "gmvs_view_scores: NULL argument");
    if (num_images < 1) return fail(GMVS_ERR_INVALID, "gmvs_view_scores: no images");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t V = (size_t)num_images;
    cudaError_t e = cudaMemsetAsync(scores, 0, sizeof(float) * V * V, st);
    if (e != cudaSuccess) return fail_cuda(e, "gmvs_view_scores");
    const long long npairs = (long long)V * (long long)(V - 1) / 2;
    if (npairs > 0) {
        const long long warps = std::min<long long>(npairs, 152LL * 64);
        const int blocks = (int)((warps * 32 + 255) / 256);
        k_view_scores<<<blocks, 256, 0, st>>>(offsets, point_ids, num_images, num_points, xyz, centers, scores,
                                              npairs);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail_cuda(e, "gmvs_view_scores");
    }
    return GMVS_OK;
}
