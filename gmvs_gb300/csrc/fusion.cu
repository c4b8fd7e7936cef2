// Geometric-consistency fusion of one reference view (batch_fusion_kernel,
// gmvs/src/fusion.cu:61-182).  Built with -fmad=false: every add, multiply,
// divide and square root rounds exactly as the IEEE host arithmetic of a
// sequential scan, so consistency counts and masks are reproducible bit for
// bit.  Deterministic where the reference races: an output pixel hit by
// several reference pixels takes the highest reference pixel index (the last
// writer of a sequential scan), resolved with an atomicMax on a per-pixel
// winner word, after which the winner's result is recomputed.
#include <cmath>
#include <cstring>
#include <string>

#include "common.cuh"
#include "errors.h"
#include "kernels.h"

namespace gmvs {
namespace {

struct DevFuse {
    int H, W, N, ref_id, gc;
    float cos_thresh;
    uint8_t* masks;
    int src_ids[kMaxNgb];
    DevCam cam[1 + kMaxNgb];
    const float* dep[1 + kMaxNgb];
    const float* nrm[1 + kMaxNgb];
};

// One source view of the consistency test (fusion.cu:104-143).
__device__ __forceinline__ bool check_view(const DevFuse& F, int j, const float rp[3], const float rn[3], float rd,
                                           int c, int r, float sp[3], float sn[3], int& sidx) {
    const DevCam& sc = F.cam[j + 1];
    float u, v, pd;
    project_on_camera(rp, sc, u, v, pd);
    const int sr = __float2int_rz(v + 0.5f), scc = __float2int_rz(u + 0.5f);
    if (!(scc >= 0 && scc < F.W && sr >= 0 && sr < F.H)) return false;
    sidx = sr * F.W + scc;
    const float sd = F.dep[j + 1][sidx];
    sn[0] = F.nrm[j + 1][sidx * 3 + 0];
    sn[1] = F.nrm[j + 1][sidx * 3 + 1];
    sn[2] = F.nrm[j + 1][sidx * 3 + 2];
    if (sd <= 0.0f) return false;
    point_on_world((float)scc, (float)sr, sd, sc, sp);
    float tu, tv;
    project_on_camera(sp, F.cam[0], tu, tv, pd);
    const float dx = (float)c - tu, dy = (float)r - tv;
    const float reproj = sqrtf(dx * dx + dy * dy);
    const float rel = fabsf(pd - rd) / rd;
    const float dot = rn[0] * sn[0] + rn[1] * sn[1] + rn[2] * sn[2];
    // acosf(dot) < 0.174533f, NaN counted as 0 (get_angle_cu, fusion.cu:50-59)
    const bool angle_ok = !(dot >= -1.0f && dot <= 1.0f) || dot > F.cos_thresh;
    return reproj < 2.0f && rel < 0.01f && angle_ok;
}

// Consistency of reference pixel ri: returns the count (-1 when skipped),
// the averaged point/normal and the projected output pixel (-1 if none).
__device__ int fuse_eval(const DevFuse& F, int ri, float cn[3], int& proj, float& pdepth) {
    proj = -1;
    const size_t HW = (size_t)F.H * F.W;
    if (F.masks[(size_t)F.ref_id * HW + ri]) return -1;
    const float rd = F.dep[0][ri];
    const float rn[3] = {F.nrm[0][ri * 3 + 0], F.nrm[0][ri * 3 + 1], F.nrm[0][ri * 3 + 2]};
    if (rd <= 0) return -1;
    const int r = ri / F.W, c = ri - r * F.W;
    float rp[3];
    point_on_world((float)c, (float)r, rd, F.cam[0], rp);
    float cp[3] = {rp[0], rp[1], rp[2]};
    cn[0] = rn[0];
    cn[1] = rn[1];
    cn[2] = rn[2];
    int num = 0;
    for (int j = 0; j < F.N; ++j) {
        float sp[3], sn[3];
        int sidx;
        if (check_view(F, j, rp, rn, rd, c, r, sp, sn, sidx)) {
            cp[0] += sp[0];
            cp[1] += sp[1];
            cp[2] += sp[2];
            cn[0] += sn[0];
            cn[1] += sn[1];
            cn[2] += sn[2];
            ++num;
        }
    }
    if (num >= F.gc) {
        const float den = (float)num + 1.0f;
        for (int k = 0; k < 3; ++k) {
            cp[k] /= den;
            cn[k] /= den;
        }
        float pu, pv;
        project_on_camera(cp, F.cam[0], pu, pv, pdepth);
        const int pr = __float2int_rz(pv + 0.5f), pc = __float2int_rz(pu + 0.5f);
        if (pc >= 0 && pc < F.W && pr >= 0 && pr < F.H && pdepth > 0.001f) proj = pr * F.W + pc;
    }
    return num;
}

__global__ void k_fuse_scan(const __grid_constant__ DevFuse F, int* __restrict__ winner, int32_t* __restrict__ count) {
    const int n = F.H * F.W;
    for (int ri = blockIdx.x * blockDim.x + threadIdx.x; ri < n; ri += gridDim.x * blockDim.x) {
        float cn[3], pdepth;
        int proj;
        const int num = fuse_eval(F, ri, cn, proj, pdepth);
        if (count) count[ri] = num;
        if (num < F.gc) continue;
        if (proj >= 0) atomicMax(&winner[proj], ri);
        // mark the source pixels that took part (fusion.cu:172-179)
        const size_t HW = (size_t)n;
        const float rd = F.dep[0][ri];
        const float rn[3] = {F.nrm[0][ri * 3 + 0], F.nrm[0][ri * 3 + 1], F.nrm[0][ri * 3 + 2]};
        const int r = ri / F.W, c = ri - r * F.W;
        float rp[3];
        point_on_world((float)c, (float)r, rd, F.cam[0], rp);
        for (int j = 0; j < F.N; ++j) {
            float sp[3], sn[3];
            int sidx;
            if (check_view(F, j, rp, rn, rd, c, r, sp, sn, sidx)) F.masks[(size_t)F.src_ids[j] * HW + sidx] = 1;
        }
    }
}

__global__ void k_fuse_write(const __grid_constant__ DevFuse F, const int* __restrict__ winner,
                             float* __restrict__ out_depth, float* __restrict__ out_normal) {
    const int n = F.H * F.W;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int w = winner[p];
        if (w < 0) continue;
        float cn[3], pdepth;
        int proj;
        fuse_eval(F, w, cn, proj, pdepth);
        out_depth[p] = pdepth;
        out_normal[p * 3 + 0] = cn[0];
        out_normal[p * 3 + 1] = cn[1];
        out_normal[p * 3 + 2] = cn[2];
    }
}

// Largest float c with acos(c) >= 0.174533f, so that for any float d in
// [-1, 1]: d > c  <=>  acos(d) < 0.174533f in exact arithmetic.
float cos_threshold() {
    const double T = (double)0.174533f;
    float c = (float)std::cos(T);
    while (std::acos((double)c) < T) c = std::nextafter(c, -2.0f);
    while (std::acos((double)std::nextafter(c, 2.0f)) >= T) c = std::nextafter(c, 2.0f);
    return c;
}

int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace

// Shared by gmvs_fuse and gmvs_fuse_fixed_scratch (fuse_fixed.cu).
int32_t fuse_run(const gmvs_fuse_view* a, int* winner, cudaStream_t st) {
    if (!a) return fail(GMVS_ERR_INVALID, "args is NULL");
    const gmvs_problem& pb = a->problem;
    if (a->height < 1 || a->width < 1) return fail(GMVS_ERR_INVALID, "empty image");
    if (pb.num_ngb < 0 || pb.num_ngb > GMVS_MAX_NGB) return fail(GMVS_ERR_INVALID, "num_ngb must be in [0, 32]");
    if (!a->masks || !a->out_depth || !a->out_normal) return fail(GMVS_ERR_INVALID, "NULL masks/output");
    if (pb.ref_image_id < 0 || pb.ref_image_id >= a->num_views) return fail(GMVS_ERR_INVALID, "ref id out of range");
    for (int j = 0; j <= pb.num_ngb; ++j)
        if (!a->depths[j] || !a->normals[j]) return fail(GMVS_ERR_INVALID, "NULL depth/normal map");
    for (int j = 0; j < pb.num_ngb; ++j) {
        if (pb.src_image_ids[j] < 0 || pb.src_image_ids[j] >= a->num_views)
            return fail(GMVS_ERR_INVALID, "src id out of range");
        if (pb.src_image_ids[j] == pb.ref_image_id)
            return fail(GMVS_ERR_INVALID, "a source view equals the reference view");
    }
    DevFuse F;
    std::memset(&F, 0, sizeof(F));
    F.H = a->height;
    F.W = a->width;
    F.N = pb.num_ngb;
    F.ref_id = pb.ref_image_id;
    F.gc = a->geom_consistent;
    F.cos_thresh = cos_threshold();
    F.masks = a->masks;
    for (int j = 0; j < F.N; ++j) F.src_ids[j] = pb.src_image_ids[j];
    for (int j = 0; j <= F.N; ++j) {
        std::memcpy(F.cam[j].K, a->cams[j].K, sizeof(float) * 9);
        std::memcpy(F.cam[j].R, a->cams[j].R, sizeof(float) * 9);
        std::memcpy(F.cam[j].t, a->cams[j].t, sizeof(float) * 3);
        F.dep[j] = a->depths[j];
        F.nrm[j] = a->normals[j];
    }
    const size_t n = (size_t)F.H * F.W;
    cudaError_t e = cudaMemsetAsync(winner, 0xFF, n * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->out_depth, 0, n * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->out_normal, 0, n * 3 * sizeof(float), st);
    if (e != cudaSuccess) return fail_cuda(e, "fusion memset");
    const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)sm_count() * 8);
    k_fuse_scan<<<blocks, 256, 0, st>>>(F, winner, a->out_count);
    k_fuse_write<<<blocks, 256, 0, st>>>(F, winner, a->out_depth, a->out_normal);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "fusion kernels");
    return GMVS_OK;
}

}  // namespace gmvs

extern "C" size_t gmvs_fuse_scratch_bytes(int32_t height, int32_t width) {
    if (height < 1 || width < 1) return 0;
    return (size_t)height * width * sizeof(int);
}

extern "C" int32_t gmvs_fuse(const gmvs_fuse_view* args, void* scratch, size_t scratch_bytes, void* stream) {
    if (!args) return gmvs::fail(GMVS_ERR_INVALID, "args is NULL");
    const size_t need = gmvs_fuse_scratch_bytes(args->height, args->width);
    if (!scratch || scratch_bytes < need)
        return gmvs::fail(GMVS_ERR_WORKSPACE, "fusion scratch too small: need " + std::to_string(need) + " bytes");
    return gmvs::fuse_run(args, (int*)scratch, (cudaStream_t)stream);
}
