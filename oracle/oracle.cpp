// SPDX-License-Identifier: MIT
//
// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of Gorilla-Lab-SCUT/gmvs's ACMP-style PatchMatch MVS hot
// path, used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline
// leg as the checker.  Nothing in the gmvs_gb300 package may load it.
//
// Every routine cites the reference function it restates (paths relative to
// the reference project).  Two sampling semantics are restated:
//   * module B (gmvs/src/patch_match.cu): fp32 bilinear on global memory with
//     truncate-then-clamp indexing;
//   * module A (gmvs/lib/src/patch_match_kernel.cu): tex2D with linear
//     filtering (8-bit fractional weights, clamped addressing).
// Arithmetic.  The fp32 restatement uses one documented formulation, shared
// with the CUDA kernels so both round identically: the homography is
// H = A - b g^T with A = K_s R_rel K_r^-1 and b = K_s t_rel formed in FP64
// and rounded once, projected coordinates are X * (1 / Z) with a correctly
// rounded reciprocal, every fused multiply-add is explicit (std::fma), each
// window moment is (left half of the columns) + (right half), and
// exp / sin / cos / acos come
// from gmvs_gb300/csrc/pmath.h.  The reference chains the same algebra in
// fp32 (ComputeHomography, patch_match_kernel.cu:262-360); the fp64 path
// below restates that chain in double and serves as the FP64 oracle.
// Deliberate, documented differences from the reference GPU code:
//   * the RNG is Philox4x32-10 (Salmon et al., SC'11) instead of curand
//     XORWOW; draws are consumed in the reference's order;
//   * within one half-sweep every read sees the state at the start of that
//     half-sweep (the reference reads same-colour "V" neighbours while they
//     are being rewritten, patch_match_kernel.cu:999-1098);
//   * rejection loops are bounded at 64 rounds;
//   * fusion output collisions resolve to the highest reference pixel index.
//
// Built with -ffp-contract=off so that x86-64 and aarch64 hosts round alike.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../gmvs_gb300/csrc/pmath.h"
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int kMaxNgb = 32;

struct Cam {  // == mvs::Camera (gmvs/include/data_structure.hpp:39-47)
    float K[9];
    float R[9];
    float t[3];
    int32_t height;
    int32_t width;
    float depth_min;
    float depth_max;
};
static_assert(sizeof(Cam) == 100, "camera layout");

struct F4 {
    float x, y, z, w;
};

}  // namespace

extern "C" {

// Oracle parameters (a subset of PatchMatchParams plus pass selection).
struct oracle_params {
    int32_t max_iterations;
    int32_t patch_size;
    int32_t radius_increment;
    float sigma_spatial;
    float sigma_color;
    int32_t top_k;
    float depth_min;
    float depth_max;
    int32_t init_kind;   // 0 random, 1 prior, 2 depth/normal
    int32_t sweep_kind;  // 0 photo (A), 1 prior (A), 2 geom (B)
    int32_t sampler;     // 0 clamp (B), 1 texture (A)
    int32_t run_filter;
    uint64_t seed;
    int32_t pass_index;
    int32_t stream_id;
    int32_t fp64;             // 1: every NCC of the pass in double precision (the FP64 CPU baseline)
    int32_t max_half_sweeps;  // > 0: stop after this many half-sweeps (0: 2 * max_iterations)
};

}  // extern "C"

namespace {

// ------------------------------------------------------------------ Philox --
// Philox4x32-10, Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11: multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key
// increments 0x9E3779B9 / 0xBB67AE85, ten rounds.
inline void philox10(const uint32_t in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// Uniform in (0, 1] from the top 24 bits: ((x >> 8) + 1) * 2^-24.  Plays the
// role of curand_uniform (patch_match_kernel.cu:147-151 and every other draw).
inline float u01(uint32_t x) { return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f); }

// Counter-based per-pixel stream: key = seed, counter = (pixel, stream,
// phase, block).  phase = pass_index << 8 | step, step 0 = init and
// 1 + 2*iter + colour for the sweeps.
struct Rng {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    int idx;
    Rng(uint64_t seed, uint32_t pixel, uint32_t stream, uint32_t phase) {
        key[0] = (uint32_t)seed;
        key[1] = (uint32_t)(seed >> 32);
        ctr[0] = pixel;
        ctr[1] = stream;
        ctr[2] = phase;
        ctr[3] = 0;
        idx = 4;
    }
    float uniform() {
        if (idx == 4) {
            philox10(ctr, key, buf);
            ctr[3] += 1;
            idx = 0;
        }
        return u01(buf[idx++]);
    }
};

// ---------------------------------------------------------- small helpers --
// sort_small: insertion sort (patch_match_kernel.cu:5-13, patch_match.cu:35-42)
inline void sort_small(float* d, int n) {
    int j;
    for (int i = 1; i < n; i++) {
        float tmp = d[i];
        for (j = i; j >= 1 && tmp < d[j - 1]; j--) d[j] = d[j - 1];
        d[j] = tmp;
    }
}
// FindMinCostIndex: ties pick the last index (patch_match_kernel.cu:15-25)
inline int find_min_idx(const float* c, int n) {
    float m = c[0];
    int mi = 0;
    for (int i = 1; i < n; ++i)
        if (c[i] <= m) {
            m = c[i];
            mi = i;
        }
    return mi;
}
// FindMaxCostIndex: ties pick the last index (patch_match_kernel.cu:27-37)
inline int find_max_idx(const float* c, int n) {
    float m = c[0];
    int mi = 0;
    for (int i = 1; i < n; ++i)
        if (c[i] >= m) {
            m = c[i];
            mi = i;
        }
    return mi;
}
inline void set_bit(uint32_t& v, int n) { v |= (uint32_t)(1u << n); }
inline int is_set(uint32_t v, int n) { return (v >> n) & 1; }

// float -> int32 the way sm_* cvt.rzi.s32.f32 does it: truncation toward
// zero, saturation, NaN -> 0.
inline int32_t f2i_rz(float v) {
    if (v != v) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}
template <class T>
inline T clampv(T v, T lo, T hi) {
    return v < lo ? lo : (v > hi ? hi : v);
}

// NormalizeVec3 (patch_match_kernel.cu:61-68): v * rsqrt(|v|^2)
inline void normalize3(F4& v) {
    const float n2 = v.x * v.x + v.y * v.y + v.z * v.z;
    const float inv = 1.0f / std::sqrt(n2);
    v.x *= inv;
    v.y *= inv;
    v.z *= inv;
}

// TransformPDFToCDF (patch_match_kernel.cu:70-83)
inline void pdf_to_cdf(float* probs, int n) {
    float sum = 0.0f;
    for (int i = 0; i < n; ++i) sum += probs[i];
    const float inv = 1.0f / sum;
    float cum = 0.0f;
    for (int i = 0; i < n; ++i) {
        const float p = probs[i] * inv;
        cum += p;
        probs[i] = cum;
    }
}

// ------------------------------------------------------------ camera math --
// Get3DPoint / GetViewDirection / GetDistance2Origin
// (patch_match_kernel.cu:86-124; patch_match.cu:97-134)
inline void get_3d_point(const Cam& c, int px, int py, float depth, float X[3]) {
    X[0] = depth * ((float)px - c.K[2]) / c.K[0];
    X[1] = depth * ((float)py - c.K[5]) / c.K[4];
    X[2] = depth;
}
inline F4 view_direction(const Cam& c, int px, int py, float depth) {
    float X[3];
    get_3d_point(c, px, py, depth, X);
    const float norm = std::sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
    return F4{X[0] / norm, X[1] / norm, X[2] / norm, 0.0f};
}
inline float distance_to_origin(const Cam& c, int px, int py, float depth, const F4& n) {
    float X[3];
    get_3d_point(c, px, py, depth, X);
    return -(n.x * X[0] + n.y * X[1] + n.z * X[2]);
}
// ComputeDepthfromPlaneHypothesis (patch_match_kernel.cu:126-135)
inline float depth_from_plane(const Cam& c, const F4& pl, int px, int py) {
    return -pl.w * c.K[0] /
           (((float)px - c.K[2]) * pl.x + (c.K[0] / c.K[4]) * ((float)py - c.K[5]) * pl.y +
            c.K[0] * pl.z);
}
// TransformNormal: camera -> world, R^T n (patch_match_kernel.cu:372-382)
inline F4 normal_to_world(const Cam& c, const F4& p) {
    return F4{c.R[0] * p.x + c.R[3] * p.y + c.R[6] * p.z, c.R[1] * p.x + c.R[4] * p.y + c.R[7] * p.z,
              c.R[2] * p.x + c.R[5] * p.y + c.R[8] * p.z, p.w};
}
// TransformNormal2RefCam: world -> camera, R n (patch_match_kernel.cu:384-395)
inline F4 normal_to_cam(const Cam& c, const F4& p) {
    return F4{c.R[0] * p.x + c.R[1] * p.y + c.R[2] * p.z, c.R[3] * p.x + c.R[4] * p.y + c.R[5] * p.z,
              c.R[6] * p.x + c.R[7] * p.y + c.R[8] * p.z, p.w};
}
// Get3DPointonWorld_cu (patch_match_kernel.cu:590-620; patch_match.cu:524-548;
// fusion.cu:6-33)
inline void point_on_world(float x, float y, float depth, const Cam& c, float out[3]) {
    float px = depth * (x - c.K[2]) / c.K[0];
    float py = depth * (y - c.K[5]) / c.K[4];
    float pz = depth;
    float tx = c.R[0] * px + c.R[3] * py + c.R[6] * pz;
    float ty = c.R[1] * px + c.R[4] * py + c.R[7] * pz;
    float tz = c.R[2] * px + c.R[5] * py + c.R[8] * pz;
    float Cx = -(c.R[0] * c.t[0] + c.R[3] * c.t[1] + c.R[6] * c.t[2]);
    float Cy = -(c.R[1] * c.t[0] + c.R[4] * c.t[1] + c.R[7] * c.t[2]);
    float Cz = -(c.R[2] * c.t[0] + c.R[5] * c.t[1] + c.R[8] * c.t[2]);
    out[0] = tx + Cx;
    out[1] = ty + Cy;
    out[2] = tz + Cz;
}
// ProjectonCamera_cu (patch_match_kernel.cu:622-648; patch_match.cu:550-560;
// fusion.cu:35-48)
inline void project_on_camera(const float X[3], const Cam& c, float& u, float& v, float& depth) {
    float tx = c.R[0] * X[0] + c.R[1] * X[1] + c.R[2] * X[2] + c.t[0];
    float ty = c.R[3] * X[0] + c.R[4] * X[1] + c.R[5] * X[2] + c.t[1];
    float tz = c.R[6] * X[0] + c.R[7] * X[1] + c.R[8] * X[2] + c.t[2];
    depth = c.K[6] * tx + c.K[7] * ty + c.K[8] * tz;
    u = (c.K[0] * tx + c.K[1] * ty + c.K[2] * tz) / depth;
    v = (c.K[3] * tx + c.K[4] * ty + c.K[5] * tz) / depth;
}

// ComputeHomography (patch_match_kernel.cu:262-360; patch_match.cu:211-299),
// in T = float (the reference) or T = double (the FP64 oracle).
template <class T>
void homography(const Cam& r, const Cam& s, const F4& pl, T H[9]) {
    T rC[3], sC[3];
    rC[0] = -((T)r.R[0] * r.t[0] + (T)r.R[3] * r.t[1] + (T)r.R[6] * r.t[2]);
    rC[1] = -((T)r.R[1] * r.t[0] + (T)r.R[4] * r.t[1] + (T)r.R[7] * r.t[2]);
    rC[2] = -((T)r.R[2] * r.t[0] + (T)r.R[5] * r.t[1] + (T)r.R[8] * r.t[2]);
    sC[0] = -((T)s.R[0] * s.t[0] + (T)s.R[3] * s.t[1] + (T)s.R[6] * s.t[2]);
    sC[1] = -((T)s.R[1] * s.t[0] + (T)s.R[4] * s.t[1] + (T)s.R[7] * s.t[2]);
    sC[2] = -((T)s.R[2] * s.t[0] + (T)s.R[5] * s.t[1] + (T)s.R[8] * s.t[2]);
    T Rr[9], Cr[3], tr[3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            Rr[a * 3 + b] = (T)s.R[a * 3 + 0] * r.R[b * 3 + 0] + (T)s.R[a * 3 + 1] * r.R[b * 3 + 1] +
                            (T)s.R[a * 3 + 2] * r.R[b * 3 + 2];
    for (int a = 0; a < 3; ++a) Cr[a] = rC[a] - sC[a];
    for (int a = 0; a < 3; ++a)
        tr[a] = (T)s.R[a * 3 + 0] * Cr[0] + (T)s.R[a * 3 + 1] * Cr[1] + (T)s.R[a * 3 + 2] * Cr[2];
    const T n[3] = {(T)pl.x, (T)pl.y, (T)pl.z};
    const T w = (T)pl.w;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) H[a * 3 + b] = Rr[a * 3 + b] - tr[a] * n[b] / w;
    T tmp[9];
    const T K0 = r.K[0], K2 = r.K[2], K4 = r.K[4], K5 = r.K[5];
    for (int a = 0; a < 3; ++a) {
        tmp[a * 3 + 0] = H[a * 3 + 0] / K0;
        tmp[a * 3 + 1] = H[a * 3 + 1] / K4;
        tmp[a * 3 + 2] = -H[a * 3 + 0] * K2 / K0 - H[a * 3 + 1] * K5 / K4 + H[a * 3 + 2];
    }
    const T S0 = s.K[0], S2 = s.K[2], S4 = s.K[4], S5 = s.K[5], S8 = s.K[8];
    H[0] = S0 * tmp[0] + S2 * tmp[6];
    H[1] = S0 * tmp[1] + S2 * tmp[7];
    H[2] = S0 * tmp[2] + S2 * tmp[8];
    H[3] = S4 * tmp[3] + S5 * tmp[6];
    H[4] = S4 * tmp[4] + S5 * tmp[7];
    H[5] = S4 * tmp[5] + S5 * tmp[8];
    H[6] = S8 * tmp[6];
    H[7] = S8 * tmp[7];
    H[8] = S8 * tmp[8];
}
// ComputeCorrespondingPoint (patch_match_kernel.cu:362-368)
template <class T>
inline void corresponding_point(const T H[9], T px, T py, T& u, T& v) {
    const T x = H[0] * px + H[1] * py + H[2];
    const T y = H[3] * px + H[4] * py + H[5];
    const T z = H[6] * px + H[7] * py + H[8];
    u = x / z;
    v = y / z;
}

// -------------------------------------------------------------- sampling --
// Module B bilinear_interpolate (patch_match.cu:10-33): truncate, clamp,
// lerp(a, b, w) = fma(w, b - a, a) (cuda_utils.cuh:35-40).
template <class T>
inline T lerp_t(T a, T b, T w) {
    return w * (b - a) + a;
}
template <>
inline float lerp_t<float>(float a, float b, float w) {
    return std::fmaf(w, b - a, a);
}
template <class T>
inline T bilinear_clamp(const float* img, T u, T v, int H, int W) {
    const int hl = clampv(f2i_rz((float)v), 0, H - 1);
    const int wl = clampv(f2i_rz((float)u), 0, W - 1);
    const T hd = v - (T)hl;
    const T wd = u - (T)wl;
    const int hu = (hl == H - 1) ? hl : hl + 1;
    const int wu = (wl == W - 1) ? wl : wl + 1;
    const T v0 = img[hl * W + wl], v1 = img[hl * W + wu];
    const T v2 = img[hu * W + wl], v3 = img[hu * W + wu];
    return lerp_t<T>(lerp_t<T>(v0, v1, wd), lerp_t<T>(v2, v3, wd), hd);
}
// Module A tex2D<float>(tex, x, y) on a float32 texture with
// cudaFilterModeLinear, unnormalised coordinates (planar_initer.cu:150-158):
// x_B = x - 0.5, i = floor(x_B); the fractions a, b are held with 8
// fractional bits, rounded half up; the corner weight w11 = a*b is rounded
// half up to 8 fractional bits and the other weights follow from it
// (a - w11, b - w11, 1 - a - b + w11); out-of-range texel indices are
// clamped to the edge (cudaAddressModeWrap acts as clamp with unnormalised
// coordinates).  Pinned on a GB300 against 42,600 hardware fetches
// (fraction sweeps, ties, random full-precision coordinates inside and
// outside the texture): all equal bit for bit.  The fp64 path is the ideal
// (unquantised) bilinear interpolation.
template <class T>
inline T tex2d_linear(const float* img, float x, float y, int H, int W) {
    const float xb = x - 0.5f, yb = y - 0.5f;
    const float fx = std::floor(xb), fy = std::floor(yb);
    if (!(fx == fx) || !(fy == fy)) return (T)NAN;
    double a, b, w00, w10, w01, w11;
    a = (double)xb - (double)fx;
    b = (double)yb - (double)fy;
    if (!std::is_same<T, double>::value) {
        a = std::floor(a * 256.0 + 0.5) / 256.0;
        b = std::floor(b * 256.0 + 0.5) / 256.0;
        w11 = std::floor(a * b * 256.0 + 0.5) / 256.0;
    } else {
        w11 = a * b;
    }
    w10 = a - w11;
    w01 = b - w11;
    w00 = 1.0 - a - b + w11;
    const double ix = clampv((double)fx, -1.0, (double)W), iy = clampv((double)fy, -1.0, (double)H);
    const int i0 = clampv((int)ix, 0, W - 1), i1 = clampv((int)ix + 1, 0, W - 1);
    const int j0 = clampv((int)iy, 0, H - 1), j1 = clampv((int)iy + 1, 0, H - 1);
    const double v = w00 * img[j0 * W + i0] + w10 * img[j0 * W + i1] + w01 * img[j1 * W + i0] + w11 * img[j1 * W + i1];
    return (T)v;
}

// ----------------------------------------------------------------- views --
struct ViewConst {  // A = K_s R_rel K_r^-1, b = K_s t_rel (rounded from FP64)
    float A[9];
    float b[3];
};

// The FP64 formation of the per-view-pair homography constants.
inline ViewConst view_consts(const Cam& r, const Cam& s) {
    ViewConst vc;
    double Cr[3];
    for (int a = 0; a < 3; ++a)
        Cr[a] = -((double)r.R[0 * 3 + a] * r.t[0] + (double)r.R[1 * 3 + a] * r.t[1] + (double)r.R[2 * 3 + a] * r.t[2]);
    const double fx = r.K[0], fy = r.K[4], cx = r.K[2], cy = r.K[5];
    const double Kinv[9] = {1.0 / fx, 0.0, -cx / fx, 0.0, 1.0 / fy, -cy / fy, 0.0, 0.0, 1.0};
    double Cs[3], Rr[9], tr[3];
    for (int a = 0; a < 3; ++a)
        Cs[a] = -((double)s.R[0 * 3 + a] * s.t[0] + (double)s.R[1 * 3 + a] * s.t[1] + (double)s.R[2 * 3 + a] * s.t[2]);
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
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            vc.A[a * 3 + b] = (float)(KR[a * 3 + 0] * Kinv[0 * 3 + b] + KR[a * 3 + 1] * Kinv[1 * 3 + b] +
                                      KR[a * 3 + 2] * Kinv[2 * 3 + b]);
    for (int a = 0; a < 3; ++a) vc.b[a] = (float)(Ks[a * 3 + 0] * tr[0] + Ks[a * 3 + 1] * tr[1] + Ks[a * 3 + 2] * tr[2]);
    return vc;
}

struct ViewSet {
    int H, W, N;  // N = number of source views
    const Cam* cams;       // [1 + N]
    const float* images;   // [(1 + N) * H * W]
    const float* depths;   // [(1 + N) * H * W] or null
    int sampler;           // 0 clamp (B), 1 texture (A)
    int patch_size, radius_increment;
    float sigma_spatial, sigma_color;
    int top_k;
    std::vector<ViewConst> vc;  // per source view
    int fp64 = 0;               // NCCs in double precision (bilateral_ncc<double>)
    void init_consts() {
        vc.clear();
        for (int j = 1; j <= N; ++j) vc.push_back(view_consts(cams[0], cams[j]));
    }
    const float* img(int i) const { return images + (size_t)i * H * W; }
    const float* dep(int i) const { return depths + (size_t)i * H * W; }
};

// ComputeBilateralWeight (patch_match_kernel.cu:397-410): un-squared distances.
template <class T>
inline T bilateral_weight(T xd, T yd, T pix, T center, T ss, T sc) {
    const T sd = std::sqrt(xd * xd + yd * yd);
    const T cd = std::fabs(pix - center);
    return std::exp(-sd / ((T)2 * ss * ss) - cd / ((T)2 * sc * sc));
}
template <>
inline float bilateral_weight<float>(float xd, float yd, float pix, float center, float ss, float sc) {
    const float sd = std::sqrt(xd * xd + yd * yd);
    const float cd = std::fabs(pix - center);
    return pmath::expf_(-sd / (2.0f * ss * ss) - cd / (2.0f * sc * sc));
}

// ComputeBilateralNCC: module A (patch_match_kernel.cu:412-516) or module B
// (patch_match.cu:347-445) semantics, evaluated in T.
template <class T>
T bilateral_ncc(const ViewSet& vs, int src, int px, int py, const F4& pl) {
    const T cost_max = 2;
    const int radius = vs.patch_size / 2;
    const Cam& rc = vs.cams[0];
    const Cam& sc = vs.cams[src];
    T H[9];
    homography<T>(rc, sc, pl, H);
    T cu, cv;
    corresponding_point<T>(H, (T)px, (T)py, cu, cv);
    if (cu >= (T)sc.width || cu < (T)0 || cv >= (T)sc.height || cv < (T)0) return cost_max;
    const int Hh = vs.H, Ww = vs.W;
    const float* ref = vs.img(0);
    const float* sim = vs.img(src);
    const T ss = vs.sigma_spatial, scol = vs.sigma_color;
    T s_r = 0, s_rr = 0, s_s = 0, s_ss = 0, s_rs = 0, s_w = 0;
    if (vs.sampler == 0) {
        const T center = ref[py * Ww + px];
        for (int i = -radius; i < radius + 1; i += vs.radius_increment) {
            for (int j = -radius; j < radius + 1; j += vs.radius_increment) {
                const int qx = clampv(px + i, 0, Ww - 1), qy = clampv(py + j, 0, Hh - 1);
                const T r = ref[qy * Ww + qx];
                T u, v;
                corresponding_point<T>(H, (T)qx, (T)qy, u, v);
                const T s = bilinear_clamp<T>(sim, u, v, Hh, Ww);
                const T w = bilateral_weight<T>((T)i, (T)j, r, center, ss, scol);
                s_r += w * r;
                s_rr += w * r * r;
                s_s += w * s;
                s_ss += w * s * s;
                s_rs += w * r * s;
                s_w += w;
            }
        }
    } else {
        const T center = tex2d_linear<T>(ref, (float)px + 0.5f, (float)py + 0.5f, Hh, Ww);
        for (int i = -radius; i < radius + 1; i += vs.radius_increment) {
            T r_r = 0, r_s = 0, r_rr = 0, r_ss = 0, r_rs = 0, r_w = 0;
            for (int j = -radius; j < radius + 1; j += vs.radius_increment) {
                const int qx = px + i, qy = py + j;
                const T r = tex2d_linear<T>(ref, (float)qx + 0.5f, (float)qy + 0.5f, Hh, Ww);
                T u, v;
                corresponding_point<T>(H, (T)qx, (T)qy, u, v);
                const T s = tex2d_linear<T>(sim, (float)u + 0.5f, (float)v + 0.5f, Hh, Ww);
                const T w = bilateral_weight<T>((T)i, (T)j, r, center, ss, scol);
                r_r += w * r;
                r_rr += w * r * r;
                r_s += w * s;
                r_ss += w * s * s;
                r_rs += w * r * s;
                r_w += w;
            }
            s_r += r_r;
            s_rr += r_rr;
            s_s += r_s;
            s_ss += r_ss;
            s_rs += r_rs;
            s_w += r_w;
        }
    }
    const T inv = (T)1 / s_w;
    s_r *= inv;
    s_rr *= inv;
    s_s *= inv;
    s_ss *= inv;
    s_rs *= inv;
    const T var_r = s_rr - s_r * s_r;
    const T var_s = s_ss - s_s * s_s;
    const T kMinVar = (T)1e-5f;
    if (var_r < kMinVar || var_s < kMinVar) return cost_max;
    const T cov = s_rs - s_r * s_s;
    const T vrs = std::sqrt(var_r * var_s);
    return std::fmax((T)0, std::fmin(cost_max, (T)1 - cov / vrs));
}

// ComputeBilateralNCC in the shared fp32 formulation (see the file header):
// module A (patch_match_kernel.cu:412-516) or module B (patch_match.cu:
// 347-445) sampling, H = A - b g^T, X * (1 / Z), explicit fused
// multiply-adds; each window sum is accumulated over the left half of the
// window columns and over the right half in (x offset, y offset) order, and
// the two halves are added.
inline float ncc_f32(const ViewSet& vs, int src, int px, int py, const F4& pl) {
    const Cam& rc = vs.cams[0];
    const Cam& sc = vs.cams[src];
    const ViewConst& C = vs.vc[src - 1];
    const float fx = rc.K[0], fy = rc.K[4], cx = rc.K[2], cy = rc.K[5];
    const float iw = 1.0f / pl.w;
    const float g[3] = {pl.x / fx * iw, pl.y / fy * iw, (pl.z - pl.x * cx / fx - pl.y * cy / fy) * iw};
    float m[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) m[r * 3 + c] = std::fma(-C.b[r], g[c], C.A[r * 3 + c]);
    const float fpx = (float)px, fpy = (float)py;
    const float cz = m[6] * fpx + m[7] * fpy + m[8];
    const float cu = (m[0] * fpx + m[1] * fpy + m[2]) / cz;
    const float cv = (m[3] * fpx + m[4] * fpy + m[5]) / cz;
    if (cu >= (float)sc.width || cu < 0.0f || cv >= (float)sc.height || cv < 0.0f) return 2.0f;
    const int radius = vs.patch_size / 2;
    const int Hh = vs.H, Ww = vs.W;
    const float* ref = vs.img(0);
    const float* sim = vs.img(src);
    const bool tex = vs.sampler == 1;
    const float center = tex ? tex2d_linear<float>(ref, fpx + 0.5f, fpy + 0.5f, Hh, Ww) : ref[py * Ww + px];
    // window sums: left half of the columns (x offsets) + right half
    const int ncol = (2 * radius) / vs.radius_increment + 1;
    const int half = (ncol + 1) / 2;
    float acc[2][6] = {{0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}};
    for (int ci = 0; ci < ncol; ++ci) {
        const int i = -radius + ci * vs.radius_increment;
        float* A = acc[ci < half ? 0 : 1];  // s_w, s_r, s_rr, ss, sss, srs
        for (int j = -radius; j < radius + 1; j += vs.radius_increment) {
            int qx = px + i, qy = py + j;
            if (!tex) {
                qx = clampv(qx, 0, Ww - 1);
                qy = clampv(qy, 0, Hh - 1);
            }
            const float r = tex ? tex2d_linear<float>(ref, (float)qx + 0.5f, (float)qy + 0.5f, Hh, Ww)
                                : ref[qy * Ww + qx];
            const float w = bilateral_weight<float>((float)i, (float)j, r, center, vs.sigma_spatial, vs.sigma_color);
            const float wr = w * r;
            A[1] += wr;
            A[2] = std::fma(wr, r, A[2]);
            A[0] += w;
            const float fqx = (float)qx, fqy = (float)qy;
            const float bx = std::fma(m[0], fqx, m[2]), by = std::fma(m[3], fqx, m[5]), bz = std::fma(m[6], fqx, m[8]);
            const float rz = 1.0f / std::fma(m[7], fqy, bz);
            const float u = std::fma(m[1], fqy, bx) * rz;
            const float v = std::fma(m[4], fqy, by) * rz;
            const float s = tex ? tex2d_linear<float>(sim, u + 0.5f, v + 0.5f, Hh, Ww)
                                : bilinear_clamp<float>(sim, u, v, Hh, Ww);
            const float ws = w * s;
            A[3] += ws;
            A[4] = std::fma(ws, s, A[4]);
            A[5] = std::fma(wr, s, A[5]);
        }
    }
    const float s_w = acc[0][0] + acc[1][0], s_r = acc[0][1] + acc[1][1], s_rr = acc[0][2] + acc[1][2];
    const float ss = acc[0][3] + acc[1][3], sss = acc[0][4] + acc[1][4], srs = acc[0][5] + acc[1][5];
    const float inv = 1.0f / s_w;
    const float mean_r = s_r * inv;
    const float var_r = s_rr * inv - mean_r * mean_r;
    const float sm = ss * inv;
    const float sq = sss * inv;
    const float sr = srs * inv;
    const float var_s = sq - sm * sm;
    if (var_r < 1e-5f || var_s < 1e-5f) return 2.0f;
    const float cov = sr - mean_r * sm;
    const float vrs = std::sqrt(var_r * var_s);
    return std::fmax(0.0f, std::fmin(2.0f, 1.0f - cov / vrs));
}

// One NCC of a pass: the shared fp32 formulation, or FP64 for the baseline.
inline float ncc_eval(const ViewSet& vs, int src, int px, int py, const F4& pl) {
    return vs.fp64 ? (float)bilateral_ncc<double>(vs, src, px, py, pl) : ncc_f32(vs, src, px, py, pl);
}

// ComputeMultiViewCostVector (patch_match_kernel.cu:571-588)
inline void cost_vector(const ViewSet& vs, int px, int py, const F4& pl, float* out) {
    for (int i = 1; i <= vs.N; ++i) out[i - 1] = ncc_eval(vs, i, px, py, pl);
}

// ComputeMultiViewInitialCostandSelectedViews (patch_match_kernel.cu:518-569)
inline float initial_cost(const float* cv, int N, int top_k_param, uint32_t* sel) {
    float sorted[kMaxNgb];
    int valid = 0;
    for (int i = 0; i < N; ++i) {
        sorted[i] = cv[i];
        if (cv[i] < 2.0f) valid++;
    }
    sort_small(sorted, N);
    *sel = 0;
    const int top_k = std::min(valid, top_k_param);
    if (top_k > 0) {
        float c = 0.0f;
        for (int i = 0; i < top_k; ++i) c += sorted[i];
        const float thr = sorted[top_k - 1];
        for (int i = 0; i < N; ++i)
            if (cv[i] <= thr) set_bit(*sel, i);
        return c / (float)top_k;
    }
    return 2.0f;
}

// compute_geom_consistency_cost (patch_match.cu:562-593): bilinear clamp.
inline float geom_cost(const ViewSet& vs, int src, const F4& pl, int px, int py) {
    const Cam& rc = vs.cams[0];
    const Cam& sc = vs.cams[src];
    const float depth = depth_from_plane(rc, pl, px, py);
    float X[3];
    point_on_world((float)px, (float)py, depth, rc, X);
    float su, sv, sd;
    project_on_camera(X, sc, su, sv, sd);
    const float src_depth = bilinear_clamp<float>(vs.dep(src), su, sv, vs.H, vs.W);
    if (src_depth == 0.0f) return 5.0f;
    float Y[3];
    point_on_world(su, sv, src_depth, sc, Y);
    float bu, bv, bd;
    project_on_camera(Y, rc, bu, bv, bd);
    const float dc = (float)px - bu, dr = (float)py - bv;
    return std::fmin(5.0f, std::sqrt(dc * dc + dr * dr));
}

// GenerateRandomNormal (patch_match_kernel.cu:137-172), rejection bounded.
inline F4 random_normal(const Cam& c, int px, int py, Rng& rng, float depth) {
    float q1 = 1.0f, q2 = 1.0f, s = 2.0f;
    for (int it = 0; it < 64 && s >= 1.0f; ++it) {
        q1 = 2.0f * rng.uniform() - 1.0f;
        q2 = 2.0f * rng.uniform() - 1.0f;
        s = q1 * q1 + q2 * q2;
    }
    if (s >= 1.0f) {  // 64 rejections: probability < 1e-42
        q1 = 0.0f;
        q2 = 0.0f;
        s = 0.0f;
    }
    const float sq = std::sqrt(1.0f - s);
    F4 n{2.0f * q1 * sq, 2.0f * q2 * sq, 1.0f - 2.0f * s, 0.0f};
    const F4 vd = view_direction(c, px, py, depth);
    if (n.x * vd.x + n.y * vd.y + n.z * vd.z > 0.0f) {
        n.x = -n.x;
        n.y = -n.y;
        n.z = -n.z;
    }
    normalize3(n);
    return n;
}

// GeneratePerturbedNormal (patch_match_kernel.cu:174-213)
inline F4 perturbed_normal(const Cam& c, int px, int py, const F4& n, Rng& rng, float pert) {
    const F4 vd = view_direction(c, px, py, 1.0f);
    const float a1 = (rng.uniform() - 0.5f) * pert;
    const float a2 = (rng.uniform() - 0.5f) * pert;
    const float a3 = (rng.uniform() - 0.5f) * pert;
    const float s1 = pmath::sinf_(a1), s2 = pmath::sinf_(a2), s3 = pmath::sinf_(a3);
    const float c1 = pmath::cosf_(a1), c2 = pmath::cosf_(a2), c3 = pmath::cosf_(a3);
    float R[9];
    R[0] = c2 * c3;
    R[1] = c3 * s1 * s2 - c1 * s3;
    R[2] = s1 * s3 + c1 * c3 * s2;
    R[3] = c2 * s3;
    R[4] = c1 * c3 + s1 * s2 * s3;
    R[5] = c1 * s2 * s3 - c3 * s1;
    R[6] = -s2;
    R[7] = c2 * s1;
    R[8] = c1 * c2;
    F4 np{R[0] * n.x + R[1] * n.y + R[2] * n.z, R[3] * n.x + R[4] * n.y + R[5] * n.z,
          R[6] * n.x + R[7] * n.y + R[8] * n.z, 0.0f};
    if (np.x * vd.x + np.y * vd.y + np.z * vd.z >= 0.0f) np = n;
    normalize3(np);
    return np;
}

// ------------------------------------------------------------------ state --
struct State {
    std::vector<F4> plane;
    std::vector<float> cost;
    std::vector<uint32_t> sel;
    explicit State(size_t n) : plane(n), cost(n), sel(n) {}
};

struct PassCtx {
    ViewSet vs;
    oracle_params prm;
    const F4* prior_planes;
    const uint32_t* prior_masks;
};

inline uint32_t phase_of(const oracle_params& p, int step) {
    return ((uint32_t)p.pass_index << 8) | (uint32_t)step;
}

// One pixel of RandomInitialization (patch_match_kernel.cu:1467-1577) or
// module B initialization (patch_match.cu:1046-1082).
void init_pixel(const PassCtx& ctx, int px, int py, const float* ref_depth, const float* ref_normal,
                const F4* init_planes, const float* init_costs, State& st) {
    const ViewSet& vs = ctx.vs;
    const oracle_params& p = ctx.prm;
    const Cam& rc = vs.cams[0];
    const int W = vs.W;
    const int c = py * W + px;
    Rng rng(p.seed, (uint32_t)c, (uint32_t)p.stream_id, phase_of(p, 0));
    F4 pl;
    if (p.init_kind == 2) {
        // compute_plane_hypothesis_from_normal_depth (patch_match.cu:329-339)
        pl = F4{ref_normal[c * 3 + 0], ref_normal[c * 3 + 1], ref_normal[c * 3 + 2], ref_depth[c]};
        pl = normal_to_cam(rc, pl);
        const float depth = pl.w;
        pl.w = distance_to_origin(rc, px, py, depth, pl);
    } else if (p.init_kind == 1) {
        // planar-prior branch (patch_match_kernel.cu:1513-1559)
        if (ctx.prior_masks[c] > 0 && init_costs[c] >= 0.1f) {
            const float pert = 0.02f;
            F4 pp = ctx.prior_planes[c];
            float d = pp.w;
            const float dmin = (1 - 3 * pert) * d;
            const float dmax = (1 + 3 * pert) * d;
            d = rng.uniform() * (dmax - dmin) + dmin;
            F4 np = perturbed_normal(rc, px, py, pp, rng, (float)(3 * pert * M_PI));
            np.w = d;
            pl = np;
        } else {
            pl = init_planes[c];
            const float depth = pl.w;
            pl.w = distance_to_origin(rc, px, py, depth, pl);
        }
    } else {
        // GenerateRandomPlaneHypothesis (patch_match_kernel.cu:215-230)
        const float depth = rng.uniform() * (p.depth_max - p.depth_min) + p.depth_min;
        pl = random_normal(rc, px, py, rng, depth);
        pl.w = distance_to_origin(rc, px, py, depth, pl);
    }
    st.plane[c] = pl;
    float cv[kMaxNgb];
    cost_vector(vs, px, py, pl, cv);
    st.cost[c] = initial_cost(cv, vs.N, vs.top_k, &st.sel[c]);
}

// The prior term: exp(-c^2/beta) * (gamma + exp(-dd^2/2sd^2) exp(-da^2/2sa^2))
// (patch_match_kernel.cu:1256-1290, 784-801)
struct PriorConsts {
    float gamma, two_depth_sigma_sq, two_angle_sigma_sq, beta, depth_sigma, angle_sigma;
};
inline PriorConsts prior_consts(const oracle_params& p) {
    PriorConsts k;
    k.gamma = 0.5f;
    k.depth_sigma = (p.depth_max - p.depth_min) / 64.0f;
    k.two_depth_sigma_sq = 2 * k.depth_sigma * k.depth_sigma;
    k.angle_sigma = (float)(M_PI * (5.0f / 180.0f));
    k.two_angle_sigma_sq = 2 * k.angle_sigma * k.angle_sigma;
    k.beta = 0.18f;
    return k;
}
inline float restricted(const PriorConsts& k, float cost, float depth_diff, float angle_cos) {
    const float angle_diff = pmath::acosf_(angle_cos);
    const float prior = k.gamma + pmath::expf_(-depth_diff * depth_diff / k.two_depth_sigma_sq) *
                                      pmath::expf_(-angle_diff * angle_diff / k.two_angle_sigma_sq);
    return pmath::expf_(-cost * cost / k.beta) * prior;
}

// One pixel of a half-sweep: CheckerboardPropagation (patch_match_kernel.cu:
// 813-1351; patch_match.cu:678-1041) followed by PlaneHypothesisRefinement
// (patch_match_kernel.cu:684-811; patch_match.cu:595-676).  Reads `in`
// (snapshot), writes pixel (px, py) of `out`.
void sweep_pixel(const PassCtx& ctx, int px, int py, int iter, int colour, float cost_threshold,
                 const State& in, State& out) {
    const ViewSet& vs = ctx.vs;
    const oracle_params& prm = ctx.prm;
    const Cam& rc = vs.cams[0];
    const int W = vs.W, H = vs.H, N = vs.N;
    const bool geom = prm.sweep_kind == 2;
    const bool prior_mode = prm.sweep_kind == 1;
    const int center = py * W + px;
    Rng rng(prm.seed, (uint32_t)center, (uint32_t)prm.stream_id, phase_of(prm, 1 + 2 * iter + colour));

    int left_near = center - 1, left_far = center - 3, right_near = center + 1, right_far = center + 3;
    int up_near = center - W, up_far = center - 3 * W, down_near = center + W, down_far = center + 3 * W;

    // float cost_array[8][32] = {2.0f}: only [0][0] is 2, the rest 0.
    float cost_array[8][kMaxNgb];
    std::memset(cost_array, 0, sizeof(cost_array));
    cost_array[0][0] = 2.0f;
    bool flag[8] = {false, false, false, false, false, false, false, false};
    const std::vector<float>& costs = in.cost;
    float cmin;
    int cminp;

    if (py > 2) {  // up_far
        flag[1] = true;
        cmin = costs[up_far];
        cminp = up_far;
        for (int i = 1; i < 11; ++i)
            if (py > 2 + 2 * i) {
                int t = up_far - 2 * i * W;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
        up_far = cminp;
        cost_vector(vs, px, py, in.plane[up_far], cost_array[1]);
    }
    if (py < H - 3) {  // down_far
        flag[3] = true;
        cmin = costs[down_far];
        cminp = down_far;
        for (int i = 1; i < 11; ++i)
            if (py < H - 3 - 2 * i) {
                int t = down_far + 2 * i * W;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
        down_far = cminp;
        cost_vector(vs, px, py, in.plane[down_far], cost_array[3]);
    }
    if (px > 2) {  // left_far
        flag[5] = true;
        cmin = costs[left_far];
        cminp = left_far;
        for (int i = 1; i < 11; ++i)
            if (px > 2 + 2 * i) {
                int t = left_far - 2 * i;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
        left_far = cminp;
        cost_vector(vs, px, py, in.plane[left_far], cost_array[5]);
    }
    if (px < W - 3) {  // right_far: keeps the MAXIMUM (patch_match_kernel.cu:954)
        flag[7] = true;
        cmin = costs[right_far];
        cminp = right_far;
        for (int i = 1; i < 11; ++i)
            if (px < W - 3 - 2 * i) {
                int t = right_far + 2 * i;
                if (cmin < costs[t]) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
        right_far = cminp;
        cost_vector(vs, px, py, in.plane[right_far], cost_array[7]);
    }
    if (py > 0) {  // up_near, V shape
        flag[0] = true;
        cmin = costs[up_near];
        cminp = up_near;
        for (int i = 0; i < 3; ++i) {
            if (py > 1 + i && px > i) {
                int t = up_near - (1 + i) * W - i;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
            if (py > 1 + i && px < W - 1 - i) {
                int t = up_near - (1 + i) * W + i;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
        }
        up_near = cminp;
        cost_vector(vs, px, py, in.plane[up_near], cost_array[0]);
    }
    if (py < H - 1) {  // down_near
        flag[2] = true;
        cmin = costs[down_near];
        cminp = down_near;
        for (int i = 0; i < 3; ++i) {
            if (py < H - 2 - i && px > i) {
                int t = down_near + (1 + i) * W - i;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
            if (py < H - 2 - i && px < W - 1 - i) {
                int t = down_near + (1 + i) * W + i;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
        }
        down_near = cminp;
        cost_vector(vs, px, py, in.plane[down_near], cost_array[2]);
    }
    if (px > 0) {  // left_near
        flag[4] = true;
        cmin = costs[left_near];
        cminp = left_near;
        for (int i = 0; i < 3; ++i) {
            if (px > 1 + i && py > i) {
                int t = left_near - (1 + i) - i * W;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
            if (px > 1 + i && py < H - 1 - i) {
                int t = left_near - (1 + i) + i * W;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
        }
        left_near = cminp;
        cost_vector(vs, px, py, in.plane[left_near], cost_array[4]);
    }
    if (px < W - 1) {  // right_near
        flag[6] = true;
        cmin = costs[right_near];
        cminp = right_near;
        for (int i = 0; i < 3; ++i) {
            if (px < W - 2 - i && py > i) {
                int t = right_near + (1 + i) - i * W;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
            if (px < W - 2 - i && py < H - 1 - i) {
                int t = right_near + (1 + i) + i * W;
                if (costs[t] < cmin) {
                    cmin = costs[t];
                    cminp = t;
                }
            }
        }
        right_near = cminp;
        cost_vector(vs, px, py, in.plane[right_near], cost_array[6]);
    }
    const int positions[8] = {up_near, up_far, down_near, down_far, left_near, left_far, right_near, right_far};

    // Multi-hypothesis joint view selection (patch_match_kernel.cu:1114-1176)
    float view_weights[kMaxNgb] = {0};
    float priors[kMaxNgb] = {0};
    const int nbr[4] = {center - W, center + W, center - 1, center + 1};
    for (int i = 0; i < 4; ++i)
        if (flag[2 * i])
            for (int j = 0; j < N; ++j) priors[j] += is_set(in.sel[nbr[i]], j) == 1 ? 0.9f : 0.1f;
    float probs[kMaxNgb] = {0};
    for (int i = 0; i < N; ++i) {
        float count = 0;
        int count_false = 0;
        float tmpw = 0;
        for (int j = 0; j < 8; ++j) {
            if (cost_array[j][i] < cost_threshold) {
                tmpw += pmath::expf_(cost_array[j][i] * cost_array[j][i] / (-0.18f));
                count++;
            }
            if (cost_array[j][i] > 1.2f) count_false++;
        }
        if (count > 2 && count_false < 3)
            probs[i] = tmpw / count;
        else if (count_false < 3)
            probs[i] = pmath::expf_(cost_threshold * cost_threshold / (-0.32f));
        probs[i] = probs[i] * priors[i];
    }
    pdf_to_cdf(probs, N);
    for (int s = 0; s < 15; ++s) {
        const float rp = rng.uniform() - 1.1920928955078125e-07f;  // FLT_EPSILON
        for (int v = 0; v < N; ++v)
            if (probs[v] > rp) {
                view_weights[v] += 1.0f;
                break;
            }
    }
    uint32_t temp_sel = 0;
    float weight_norm = 0;
    for (int i = 0; i < N; ++i)
        if (view_weights[i] > 0) {
            set_bit(temp_sel, i);
            weight_norm += view_weights[i];
        }

    // final costs of the 8 candidates (patch_match_kernel.cu:1178-1211;
    // patch_match.cu:920-946)
    float final_costs[8] = {0};
    for (int i = 0; i < 8; ++i) {
        for (int j = 0; j < N; ++j) {
            if (view_weights[j] > 0) {
                if (geom && flag[i])
                    final_costs[i] += view_weights[j] *
                                      (cost_array[i][j] + 0.1f * geom_cost(vs, j + 1, in.plane[positions[i]], px, py));
                else
                    final_costs[i] += view_weights[j] * cost_array[i][j];
            }
        }
        final_costs[i] /= weight_norm;
    }
    const int min_idx = find_min_idx(final_costs, 8);

    // current pixel (patch_match_kernel.cu:1216-1241; patch_match.cu:951-968)
    F4 cur_plane = in.plane[center];
    float cvn[kMaxNgb];
    cost_vector(vs, px, py, cur_plane, cvn);
    float cost_now = 0.0f;
    for (int i = 0; i < N; ++i) {
        if (geom)
            cost_now += view_weights[i] * (cvn[i] + 0.1f * geom_cost(vs, i + 1, cur_plane, px, py));
        else
            cost_now += view_weights[i] * cvn[i];
    }
    cost_now /= weight_norm;
    float cur_cost = cost_now;
    uint32_t cur_sel = in.sel[center];
    float depth_now = depth_from_plane(rc, cur_plane, px, py);
    float restricted_cost = 0.0f;
    const PriorConsts pk = prior_consts(prm);
    const uint32_t mask = prior_mode ? ctx.prior_masks[center] : 0u;
    F4 prior_plane{0, 0, 0, 0};
    float depth_prior = 0.0f;

    if (prior_mode) {
        prior_plane = ctx.prior_planes[center];
        depth_prior = depth_from_plane(rc, prior_plane, px, py);
        if (mask > 0) {  // patch_match_kernel.cu:1256-1305
            float rfc[8] = {0};
            for (int i = 0; i < 8; ++i) {
                if (flag[i]) {
                    const F4& q = in.plane[positions[i]];
                    const float dn = depth_from_plane(rc, q, px, py);
                    const float ac = prior_plane.x * q.x + prior_plane.y * q.y + prior_plane.z * q.z;
                    rfc[i] = restricted(pk, final_costs[i], dn - depth_prior, ac);
                }
            }
            const int max_idx = find_max_idx(rfc, 8);
            const float dn = depth_from_plane(rc, cur_plane, px, py);
            const float ac = prior_plane.x * cur_plane.x + prior_plane.y * cur_plane.y + prior_plane.z * cur_plane.z;
            const float rcn = restricted(pk, cost_now, dn - depth_prior, ac);
            if (flag[max_idx]) {
                const F4& q = in.plane[positions[max_idx]];
                const float db = depth_from_plane(rc, q, px, py);
                if (db >= prm.depth_min && db <= prm.depth_max && rfc[max_idx] > rcn) {
                    depth_now = db;
                    cur_plane = q;
                    cur_cost = final_costs[max_idx];
                    restricted_cost = rfc[max_idx];
                    cur_sel = temp_sel;
                }
            }
        } else if (flag[min_idx]) {  // selected views are NOT updated here (1306-1318)
            const F4& q = in.plane[positions[min_idx]];
            const float db = depth_from_plane(rc, q, px, py);
            if (db >= prm.depth_min && db <= prm.depth_max && final_costs[min_idx] < cost_now) {
                depth_now = db;
                cur_plane = q;
                cur_cost = final_costs[min_idx];
            }
        }
    } else if (flag[min_idx]) {  // patch_match_kernel.cu:1321-1335; patch_match.cu:975-990
        const F4& q = in.plane[positions[min_idx]];
        const float db = depth_from_plane(rc, q, px, py);
        if (db >= prm.depth_min && db <= prm.depth_max && final_costs[min_idx] < cost_now) {
            depth_now = db;
            cur_plane = q;
            cur_cost = final_costs[min_idx];
            cur_sel = temp_sel;
        }
    }

    // PlaneHypothesisRefinement (patch_match_kernel.cu:684-811)
    {
        const float pert = 0.02f;
        float depth_rand;
        F4 n_rand;
        const bool use_prior = prior_mode && mask > 0;
        if (use_prior) {
            depth_rand = rng.uniform() * 6 * pk.depth_sigma + (depth_prior - 3 * pk.depth_sigma);
            n_rand = perturbed_normal(rc, px, py, prior_plane, rng, pk.angle_sigma);
        } else {
            depth_rand = rng.uniform() * (prm.depth_max - prm.depth_min) + prm.depth_min;
            n_rand = random_normal(rc, px, py, rng, depth_now);
        }
        // do { ... } while (d < min && d > max): runs exactly once (quirk).
        const float dmin_p = (1 - pert) * depth_now;
        const float dmax_p = (1 + pert) * depth_now;
        const float depth_pert = rng.uniform() * (dmax_p - dmin_p) + dmin_p;
        const F4 n_pert = perturbed_normal(rc, px, py, cur_plane, rng, (float)(pert * M_PI));
        const float depths[5] = {depth_rand, depth_now, depth_rand, depth_now, depth_pert};
        const F4 normals[5] = {cur_plane, n_rand, n_rand, n_pert, cur_plane};
        for (int k = 0; k < 5; ++k) {
            F4 cand = normals[k];
            cand.w = distance_to_origin(rc, px, py, depths[k], cand);
            float cvk[kMaxNgb];
            for (int j = 0; j < N; ++j) cvk[j] = 0.0f;
            for (int j = 0; j < N; ++j)
                if (view_weights[j] > 0) cvk[j] = ncc_eval(vs, j + 1, px, py, cand);
            float tc = 0.0f;
            for (int j = 0; j < N; ++j) {
                if (view_weights[j] > 0) {
                    if (geom)
                        tc += view_weights[j] * (cvk[j] + 0.1f * geom_cost(vs, j + 1, cand, px, py));
                    else
                        tc += view_weights[j] * cvk[j];
                }
            }
            tc /= weight_norm;
            const float db = depth_from_plane(rc, cand, px, py);
            if (use_prior) {
                const float ac = prior_plane.x * cand.x + prior_plane.y * cand.y + prior_plane.z * cand.z;
                const float rtc = restricted(pk, tc, depths[k] - depth_prior, ac);
                if (db >= prm.depth_min && db <= prm.depth_max && rtc > restricted_cost) {
                    depth_now = db;
                    cur_plane = cand;
                    cur_cost = tc;
                    restricted_cost = rtc;
                }
            } else if (db >= prm.depth_min && db <= prm.depth_max && tc < cur_cost) {
                depth_now = db;
                cur_plane = cand;
                cur_cost = tc;
            }
        }
    }
    out.plane[center] = cur_plane;
    out.cost[center] = cur_cost;
    out.sel[center] = cur_sel;
}

// CheckerboardFilter (patch_match_kernel.cu:1355-1463; patch_match.cu:1165-1281)
// on the .w (= depth) channel, in place (reads only the other colour).
void filter_pixel(const int W, const int H, int px, int py, std::vector<F4>& pl, const std::vector<float>& costs) {
    const int center = py * W + px;
    float f[21];
    int n = 0;
    f[n++] = pl[center].w;
    const int left = center - 1, leftleft = center - 3, up = center - W, upup = center - 3 * W;
    const int down = center + W, downdown = center + 3 * W, right = center + 1, rightright = center + 3;
    if (costs[center] < 0.001f) return;
    if (py > 0) f[n++] = pl[up].w;
    if (py > 2) f[n++] = pl[upup].w;
    if (py > 4) f[n++] = pl[upup - W * 2].w;
    if (py < H - 1) f[n++] = pl[down].w;
    if (py < H - 3) f[n++] = pl[downdown].w;
    if (py < H - 5) f[n++] = pl[downdown + W * 2].w;
    if (px > 0) f[n++] = pl[left].w;
    if (px > 2) f[n++] = pl[leftleft].w;
    if (px > 4) f[n++] = pl[leftleft - 2].w;
    if (px < W - 1) f[n++] = pl[right].w;
    if (px < W - 3) f[n++] = pl[rightright].w;
    if (px < W - 5) f[n++] = pl[rightright + 2].w;
    if (py > 0 && px < W - 2) f[n++] = pl[up + 2].w;
    if (py < H - 1 && px < W - 2) f[n++] = pl[down + 2].w;
    if (py > 0 && px > 1) f[n++] = pl[up - 2].w;
    if (py < H - 1 && px > 1) f[n++] = pl[down - 2].w;
    if (px > 0 && py > 2) f[n++] = pl[left - W * 2].w;
    if (px < W - 1 && py > 2) f[n++] = pl[right - W * 2].w;
    if (px > 0 && py < H - 2) f[n++] = pl[left + W * 2].w;
    if (px < W - 1 && py < H - 2) f[n++] = pl[right + W * 2].w;
    sort_small(f, n);
    const int m = n / 2;
    pl[center].w = (n % 2 == 0) ? (f[m - 1] + f[m]) / 2 : f[m];
}

inline int nthreads_or_default(int n) {
#ifdef _OPENMP
    return n > 0 ? n : omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

}  // namespace

extern "C" {

int oracle_version(void) { return 1; }

void oracle_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { philox10(ctr, key, out); }

float oracle_u01(uint32_t x) { return u01(x); }

// The shared elementary functions, for their accuracy tests.
float oracle_pm_expf(float x) { return pmath::expf_(x); }
float oracle_pm_sinf(float x) { return pmath::sinf_(x); }
float oracle_pm_cosf(float x) { return pmath::cosf_(x); }
float oracle_pm_acosf(float x) { return pmath::acosf_(x); }

// Per-view NCC costs of given camera-frame planes (float4 per pixel) and the
// initial multi-view cost / selected views.  fp64 = 1 evaluates the NCC in
// double precision (the FP64 oracle); fp64 = 2 in the reference's own fp32
// chain (ComputeHomography / ComputeCorrespondingPoint / ComputeBilateralNCC
// in float, in the reference's operation order, without fused multiply-adds
// and with IEEE exp, division and square root).
int oracle_ncc_costs(const Cam* cams, int num_src, int H, int W, const float* images, const oracle_params* prm,
                     const float* planes, float* costs, float* init_cost, uint32_t* init_views, int fp64,
                     int nthreads) {
    if (num_src < 1 || num_src > kMaxNgb || H < 1 || W < 1) return 1;
    ViewSet vs{H, W, num_src, cams, images, nullptr, prm->sampler, prm->patch_size, prm->radius_increment,
               prm->sigma_spatial, prm->sigma_color, prm->top_k, {}};
    vs.init_consts();
    const F4* pl = reinterpret_cast<const F4*>(planes);
    const int nt = nthreads_or_default(nthreads);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            const int c = y * W + x;
            float cv[kMaxNgb];
            for (int s = 1; s <= num_src; ++s) {
                if (fp64 == 1)
                    cv[s - 1] = (float)bilateral_ncc<double>(vs, s, x, y, pl[c]);
                else if (fp64 == 2)
                    cv[s - 1] = bilateral_ncc<float>(vs, s, x, y, pl[c]);
                else
                    cv[s - 1] = ncc_f32(vs, s, x, y, pl[c]);
                if (costs) costs[(size_t)(s - 1) * H * W + c] = cv[s - 1];
            }
            uint32_t sel = 0;
            const float ic = initial_cost(cv, num_src, prm->top_k, &sel);
            if (init_cost) init_cost[c] = ic;
            if (init_views) init_views[c] = sel;
        }
    }
    return 0;
}

// One full PatchMatch pass over one reference view: init, 2*I half-sweeps,
// GetDepthandNormal, black then red filter, export
// (PlanarInit::run_patch_match, patch_match_kernel.cu:1711-1809;
// PatchMatcher::run_patch_match, patch_match.cu:1353-1518).
// images/depths: (1 + N) planes of H*W (ref first).  Outputs: depth [H*W],
// normal [H*W*3] (world), cost [H*W], planes [H*W*4] (optional).
int oracle_run_pass(const Cam* cams, int num_src, int H, int W, const float* images, const float* depths,
                    const float* ref_normal, const float* prior_planes, const uint32_t* prior_masks,
                    const float* init_planes, const float* init_costs, const oracle_params* prm, float* out_depth,
                    float* out_normal, float* out_cost, float* out_planes, int nthreads) {
    if (num_src < 1 || num_src > kMaxNgb || H < 1 || W < 1) return 1;
    if (prm->init_kind == 2 && (!depths || !ref_normal)) return 1;
    if (prm->sweep_kind == 2 && !depths) return 1;
    if ((prm->init_kind == 1 || prm->sweep_kind == 1) && (!prior_planes || !prior_masks)) return 1;
    if (prm->init_kind == 1 && (!init_planes || !init_costs)) return 1;
    PassCtx ctx;
    ctx.vs = ViewSet{H, W, num_src, cams, images, depths, prm->sampler, prm->patch_size, prm->radius_increment,
                     prm->sigma_spatial, prm->sigma_color, prm->top_k, {}};
    ctx.vs.init_consts();
    ctx.vs.fp64 = prm->fp64;
    ctx.prm = *prm;
    ctx.prior_planes = reinterpret_cast<const F4*>(prior_planes);
    ctx.prior_masks = prior_masks;
    const size_t n = (size_t)H * W;
    State a(n), b(n);
    const int nt = nthreads_or_default(nthreads);
    const F4* ip = reinterpret_cast<const F4*>(init_planes);
#pragma omp parallel for schedule(dynamic, 2) num_threads(nt)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) init_pixel(ctx, x, y, depths, ref_normal, ip, init_costs, a);

    int half_sweeps = 0;
    for (int it = 0; it < prm->max_iterations; ++it) {
        // cost_threshold = 0.8 * expf(iter*iter / -90) (patch_match_kernel.cu:1143)
        const float thr = (float)(0.8 * (double)pmath::expf_((float)(it * it) / (-90.0f)));
        for (int colour = 0; colour < 2; ++colour) {
            if (prm->max_half_sweeps > 0 && half_sweeps++ >= prm->max_half_sweeps) break;
            b = a;
#pragma omp parallel for schedule(dynamic, 2) num_threads(nt)
            for (int y = 0; y < H; ++y)
                for (int x = 0; x < W; ++x)
                    if (((x + y) & 1) == colour) sweep_pixel(ctx, x, y, it, colour, thr, a, b);
            std::swap(a, b);
        }
    }
    // GetDepthandNormal (patch_match_kernel.cu:1655-1674)
    const Cam& rc = cams[0];
    if (prm->run_filter) {
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                F4& p = a.plane[y * W + x];
                p.w = depth_from_plane(rc, p, x, y);
                p = normal_to_world(rc, p);
            }
        for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static) num_threads(nt)
            for (int y = 0; y < H; ++y)
                for (int x = 0; x < W; ++x)
                    if (((x + y) & 1) == colour) filter_pixel(W, H, x, y, a.plane, a.cost);
        }
    }
    // export_plane_hypotheses_cost (patch_match.cu:1284-1313)
    for (size_t i = 0; i < n; ++i) {
        if (out_depth) out_depth[i] = a.plane[i].w;
        if (out_normal) {
            out_normal[i * 3 + 0] = a.plane[i].x;
            out_normal[i * 3 + 1] = a.plane[i].y;
            out_normal[i * 3 + 2] = a.plane[i].z;
        }
        if (out_cost) out_cost[i] = a.cost[i];
        if (out_planes) {
            out_planes[i * 4 + 0] = a.plane[i].x;
            out_planes[i * 4 + 1] = a.plane[i].y;
            out_planes[i * 4 + 2] = a.plane[i].z;
            out_planes[i * 4 + 3] = a.plane[i].w;
        }
    }
    return 0;
}

// batch_fusion_kernel for one reference view, sequential over reference
// pixels (fusion.cu:61-182).  depths/normals: (1 + N) planes (ref, then src in
// problem order).  masks: uint8 [V][H][W], updated in place.  Output pixels
// written by several reference pixels keep the last (highest index) writer.
// Angle test: acosf(d) < 0.174533 is evaluated as "d outside [-1, 1] or NaN,
// or d > cos_thresh" with cos_thresh supplied by the caller.
int oracle_fuse(const Cam* cams, int num_src, int ref_id, const int32_t* src_ids, int H, int W, const float* depths,
                const float* normals, uint8_t* masks, int geom_consistent, float cos_thresh, float* out_depth,
                float* out_normal, int32_t* out_count, int32_t* out_hits) {
    const size_t HW = (size_t)H * W;
    std::memset(out_depth, 0, HW * sizeof(float));
    std::memset(out_normal, 0, HW * 3 * sizeof(float));
    if (out_hits) std::memset(out_hits, 0, HW * sizeof(int32_t));
    const Cam& rc = cams[0];
    std::vector<uint8_t> pending;  // masks are applied after the scan: the
                                   // kernel reads only masks[ref] and writes
                                   // only masks[src] (src != ref)
    std::vector<size_t> set_list;
    for (int r = 0; r < H; ++r) {
        for (int c = 0; c < W; ++c) {
            const int ri = r * W + c;
            if (out_count) out_count[ri] = -1;
            if (masks[(size_t)ref_id * HW + ri]) continue;
            const float rd = depths[ri];
            const float rn[3] = {normals[ri * 3 + 0], normals[ri * 3 + 1], normals[ri * 3 + 2]};
            if (rd <= 0) continue;
            float rp[3];
            point_on_world((float)c, (float)r, rd, rc, rp);
            float cp[3] = {rp[0], rp[1], rp[2]};
            float cn[3] = {rn[0], rn[1], rn[2]};
            int used_x[kMaxNgb], used_y[kMaxNgb];
            int num = 0;
            for (int j = 0; j < num_src; ++j) {
                used_x[j] = -1;
                used_y[j] = -1;
            }
            for (int j = 0; j < num_src; ++j) {
                const Cam& sc = cams[j + 1];
                float u, v, pd;
                project_on_camera(rp, sc, u, v, pd);
                const int sr = f2i_rz(v + 0.5f), scc = f2i_rz(u + 0.5f);
                if (scc >= 0 && scc < W && sr >= 0 && sr < H) {
                    const size_t si = (size_t)(j + 1) * HW + (size_t)sr * W + scc;
                    const float sd = depths[si];
                    const float sn[3] = {normals[si * 3 + 0], normals[si * 3 + 1], normals[si * 3 + 2]};
                    if (sd <= 0.0f) continue;
                    float sp[3];
                    point_on_world((float)scc, (float)sr, sd, sc, sp);
                    float tu, tv;
                    project_on_camera(sp, rc, tu, tv, pd);
                    const float dx = (float)c - tu, dy = (float)r - tv;
                    const float reproj = std::sqrt(dx * dx + dy * dy);
                    const float rel = std::fabs(pd - rd) / rd;
                    const float dot = rn[0] * sn[0] + rn[1] * sn[1] + rn[2] * sn[2];
                    const bool angle_ok = !(dot >= -1.0f && dot <= 1.0f) || dot > cos_thresh;
                    if (reproj < 2.0f && rel < 0.01f && angle_ok) {
                        cp[0] += sp[0];
                        cp[1] += sp[1];
                        cp[2] += sp[2];
                        cn[0] += sn[0];
                        cn[1] += sn[1];
                        cn[2] += sn[2];
                        used_x[j] = scc;
                        used_y[j] = sr;
                        ++num;
                    }
                }
            }
            if (out_count) out_count[ri] = num;
            if (num >= geom_consistent) {
                const float den = (float)num + 1.0f;
                for (int k = 0; k < 3; ++k) {
                    cp[k] /= den;
                    cn[k] /= den;
                }
                float pu, pv, pdd;
                project_on_camera(cp, rc, pu, pv, pdd);
                const int pr = f2i_rz(pv + 0.5f), pc = f2i_rz(pu + 0.5f);
                if (pc >= 0 && pc < W && pr >= 0 && pr < H && pdd > 0.001f) {
                    const size_t pi = (size_t)pr * W + pc;
                    if (out_hits) out_hits[pi] += 1;
                    out_depth[pi] = pdd;
                    out_normal[pi * 3 + 0] = cn[0];
                    out_normal[pi * 3 + 1] = cn[1];
                    out_normal[pi * 3 + 2] = cn[2];
                }
                for (int j = 0; j < num_src; ++j) {
                    if (used_x[j] == -1) continue;
                    set_list.push_back((size_t)src_ids[j] * HW + (size_t)used_y[j] * W + used_x[j]);
                }
            }
        }
    }
    for (size_t k : set_list) masks[k] = 1;
    return 0;
}

}  // extern "C"
