// PatchMatch device code: samplers, the reference-side patch, the bilateral
// NCC, initialisation, one checkerboard half-sweep (propagation + joint view
// selection + refinement), depth/normal conversion and the median filter.
// Included by one .cu file per sampler so the instantiations compile in
// parallel.
#pragma once

#include "common.cuh"
#include "pmath.h"

namespace gmvs {

// --------------------------------------------------------------- samplers --
// All samplers reproduce module B's truncate-then-clamp bilinear
// (gmvs/src/patch_match.cu:10-33) except SampTex, which is module A's
// hardware tex2D (patch_match_kernel.cu:443-464).
struct SampF32 {  // plain fp32 rows, four loads per sample
    const float* __restrict__ p;
    int H, W;
    __device__ __forceinline__ SampF32(const DevView& V, int img) : p((const float*)V.img[img]), H(V.H), W(V.W) {}
    __device__ __forceinline__ float at(int x, int y) const { return __ldg(p + GMVS_IDX(y * W + x, H * W, kOobImage)); }
    __device__ __forceinline__ float sample(float u, float v) const { return bilinear_clamp(p, u, v, H, W); }
    static constexpr bool kTex = false;
};

// Texel quads: quad[y][x] = (a, b - a, c, d - c) for the four taps the
// reference reads for a sample whose clamped integer corner is (x, y):
// a = I[y][x], b = I[y][xu], c = I[yu][x], d = I[yu][xu] with
// xu = min(x+1, W-1), yu = min(y+1, H-1).  The differences are the ones the
// interpolation fma(w, b - a, a) forms, rounded the same way at staging, so
// the sample is unchanged and costs two subtractions less.
// hl = clamp(trunc(v), 0, H - 1) exactly as the reference, without int/float
// conversions: clamping first makes trunc == floor, and adding 2^23 with
// round-down leaves floor(v) in the low mantissa bits.  NaN -> 0 and +-inf
// clamp to the edges like the saturating conversion.
__device__ __forceinline__ void clamp_corner(float u, float v, int H, int W, int& idx, float& wd, float& hd) {
    const float vc = fminf(fmaxf(v, 0.0f), (float)(H - 1));
    const float uc = fminf(fmaxf(u, 0.0f), (float)(W - 1));
    const float tv = __fadd_rd(vc, 8388608.0f), tu = __fadd_rd(uc, 8388608.0f);
    const int hl = __float_as_int(tv) - 0x4B000000, wl = __float_as_int(tu) - 0x4B000000;
    hd = v - (tv - 8388608.0f);
    wd = u - (tu - 8388608.0f);
    idx = hl * W + wl;
}

struct SampQuadF32 {
    const float4* __restrict__ p;
    int H, W;
    __device__ __forceinline__ SampQuadF32(const DevView& V, int img)
        : p((const float4*)V.img[img]), H(V.H), W(V.W) {}
    __device__ __forceinline__ float at(int x, int y) const {
        return __ldg(&p[GMVS_IDX(y * W + x, H * W, kOobImage)]).x;
    }
    __device__ __forceinline__ float sample(float u, float v) const {
        int idx;
        float wd, hd;
        clamp_corner(u, v, H, W, idx, wd, hd);
        const float4 q = __ldg(&p[GMVS_IDX(idx, H * W, kOobImage)]);
        return lerpf(fmaf(wd, q.y, q.x), fmaf(wd, q.w, q.z), hd);
    }
    static constexpr bool kTex = false;
};

struct SampQuadF16 {
    const uint2* __restrict__ p;
    int H, W;
    __device__ __forceinline__ SampQuadF16(const DevView& V, int img)
        : p((const uint2*)V.img[img]), H(V.H), W(V.W) {}
    __device__ __forceinline__ static float2 h2f(uint32_t u) {
        __half2 h = *reinterpret_cast<__half2*>(&u);
        return __half22float2(h);
    }
    __device__ __forceinline__ float at(int x, int y) const {
        return h2f(__ldg(&p[GMVS_IDX(y * W + x, H * W, kOobImage)]).x).x;
    }
    __device__ __forceinline__ float sample(float u, float v) const {
        int idx;
        float wd, hd;
        clamp_corner(u, v, H, W, idx, wd, hd);
        const uint2 q = __ldg(&p[GMVS_IDX(idx, H * W, kOobImage)]);
        const float2 t = h2f(q.x), b = h2f(q.y);
        return lerpf(fmaf(wd, t.y, t.x), fmaf(wd, b.y, b.x), hd);
    }
    static constexpr bool kTex = false;
};

struct SampTex {
    cudaTextureObject_t t;
    __device__ __forceinline__ SampTex(const DevView& V, int img) : t((cudaTextureObject_t)V.tex[img]) {}
    __device__ __forceinline__ float at(int x, int y) const {
        return tex2D<float>(t, (float)x + 0.5f, (float)y + 0.5f);
    }
    __device__ __forceinline__ float sample(float u, float v) const { return tex2D<float>(t, u + 0.5f, v + 0.5f); }
    static constexpr bool kTex = true;
};

// Correctly rounded reciprocal: the hardware approximation refined by one
// Newton step with fused multiply-adds.  Checked on a GB300 against the IEEE
// round-to-nearest reciprocal for every significand at 30 binary exponents
// between 2^-125 and 2^125 of both signs: identical.  Outside that range
// (and for 0, inf, NaN) the IEEE reciprocal is used.
constexpr float kRcpLo = 2.35098870e-38f, kRcpHi = 4.25352959e+37f;  // 2^-125, 2^125
// the refined approximation alone: callers guarantee kRcpLo <= |x| <= kRcpHi
__device__ __forceinline__ float rcp_in_range(float x) {
    float y;
    asm("rcp.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    const float e = __fmaf_rn(-x, y, 1.0f);
    return __fmaf_rn(y, e, y);
}
__device__ __forceinline__ float rcp_rn(float x) {
    const float ax = fabsf(x);
    if (!(ax >= kRcpLo && ax <= kRcpHi)) return __frcp_rn(x);
    return rcp_in_range(x);
}

// -------------------------------------------------------- reference patch --
// A pixel is evaluated by two adjacent lanes of a warp.  Lane half h = 0
// takes the left half of the window columns (x offsets), h = 1 the right
// half; every window sum is (left half) + (right half), combined with one
// shuffle.  The bilateral weights, the reference samples and the reference
// moments do not depend on the hypothesis (ComputeBilateralWeight depends
// only on the window offset and |I_ref - I_ref(centre)|,
// patch_match_kernel.cu:397-410), so they are formed once per pixel and
// launch.  NS = samples per axis (6 for the default 11x11 window with
// stride 2); NS = 0 is the generic path that recomputes them per sample.
struct Pair {
    int h;          // which half of the window columns
    unsigned mask;  // the two lanes of the pixel
};
__device__ __forceinline__ Pair make_pair(unsigned lane) { return Pair{(int)(lane & 1u), 3u << (lane & 30u)}; }
// left + right: lane 0 adds (l, r), lane 1 adds (r, l); IEEE addition commutes
__device__ __forceinline__ float pair_sum(const Pair& q, float v) { return v + __shfl_xor_sync(q.mask, v, 1); }

// The per-lane window weights (w, w * I_ref) live in shared memory: slot
// k of this lane at pw[k * pstride], k = column-in-half * NS + row.
template <int NS>
struct Patch {
    static constexpr int NC = NS / 2;  // columns per lane (NS even)
    float2* pw;
    int pstride;
    float inv, mean_r, var_r;
};
template <>
struct Patch<0> {
    float center, inv, mean_r, var_r;
    int c0, c1;  // this lane's window columns
};

__device__ __forceinline__ float bilateral_weight(float xd, float yd, float pix, float center, float ss, float sc) {
    const float sd = sqrtf(xd * xd + yd * yd);
    const float cd = fabsf(pix - center);
    return pmath::expf_(-sd / (2.0f * ss * ss) - cd / (2.0f * sc * sc));
}

template <class S>
__device__ __forceinline__ int window_coord(int p, int off, int n) {
    if constexpr (S::kTex) return p + off;
    else return min(max(p + off, 0), n - 1);
}

template <class S, int NS>
__device__ __forceinline__ void make_patch(Patch<NS>& P, const S& ref, const DevView& V, const DevParams& prm, int px,
                                           int py, const Pair& q) {
    const int radius = prm.patch_size / 2;
    const int inc = prm.radius_increment;
    float s_w = 0.f, s_r = 0.f, s_rr = 0.f;
    if constexpr (NS > 0) {
        constexpr int NC = NS / 2;
        const float center = ref.at(px, py);
#pragma unroll 1
        for (int al = 0; al < NC; ++al) {
            const int qx = window_coord<S>(px, -radius + (q.h * NC + al) * inc, V.W);
#pragma unroll
            for (int b = 0; b < NS; ++b) {
                const float r = ref.at(qx, window_coord<S>(py, -radius + b * inc, V.H));
                const float w = bilateral_weight((float)(-radius + (q.h * NC + al) * inc), (float)(-radius + b * inc),
                                                 r, center, prm.sigma_spatial, prm.sigma_color);
                const float wr = w * r;
                P.pw[(al * NS + b) * P.pstride] = make_float2(w, wr);
                s_r += wr;
                s_rr = fmaf(wr, r, s_rr);
                s_w += w;
            }
        }
    } else {
        const int n = (2 * radius) / inc + 1;
        const int half = (n + 1) / 2;
        P.c0 = q.h ? half : 0;
        P.c1 = q.h ? n : half;
        P.center = ref.at(px, py);
        for (int a = P.c0; a < P.c1; ++a) {
            const int i = -radius + a * inc;
            for (int b = 0; b < n; ++b) {
                const int j = -radius + b * inc;
                const float r = ref.at(window_coord<S>(px, i, V.W), window_coord<S>(py, j, V.H));
                const float w = bilateral_weight((float)i, (float)j, r, P.center, prm.sigma_spatial, prm.sigma_color);
                const float wr = w * r;
                s_r += wr;
                s_rr = fmaf(wr, r, s_rr);
                s_w += w;
            }
        }
    }
    s_w = pair_sum(q, s_w);
    s_r = pair_sum(q, s_r);
    s_rr = pair_sum(q, s_rr);
    P.inv = 1.0f / s_w;
    P.mean_r = s_r * P.inv;
    P.var_r = s_rr * P.inv - P.mean_r * P.mean_r;
}

// Hypothesis-dependent row of the homography: g = K_r^-T n / w.
struct Hyp {
    float g0, g1, g2;
};
__device__ __forceinline__ Hyp make_hyp(const DevCam& rc, float4 pl) {
    const float fx = rc.K[0], fy = rc.K[4], cx = rc.K[2], cy = rc.K[5];
    const float iw = 1.0f / pl.w;
    Hyp h;
    h.g0 = pl.x / fx * iw;
    h.g1 = pl.y / fy * iw;
    h.g2 = (pl.z - pl.x * cx / fx - pl.y * cy / fy) * iw;
    return h;
}

// Bilateral NCC of one hypothesis against source j (0-based): ComputeBilateralNCC
// (patch_match_kernel.cu:412-516; gmvs/src/patch_match.cu:347-445).  Both
// lanes of the pair return the same value.
template <class S, int NS>
__device__ __forceinline__ float ncc_cost(const DevView& V, const DevParams& prm, int j, const Hyp& h,
                                          const Patch<NS>& P, int px, int py, const Pair& q) {
    const float4 h0 = V.hs[j][0], h1 = V.hs[j][1], h2 = V.hs[j][2], h3 = V.hs[j][3];
    const float A[9] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w, h2.x};
    const float b[3] = {h2.y, h2.z, h2.w};
    const float m0 = fmaf(-b[0], h.g0, A[0]), m1 = fmaf(-b[0], h.g1, A[1]), m2 = fmaf(-b[0], h.g2, A[2]);
    const float m3 = fmaf(-b[1], h.g0, A[3]), m4 = fmaf(-b[1], h.g1, A[4]), m5 = fmaf(-b[1], h.g2, A[5]);
    const float m6 = fmaf(-b[2], h.g0, A[6]), m7 = fmaf(-b[2], h.g1, A[7]), m8 = fmaf(-b[2], h.g2, A[8]);
    const float fpx = (float)px, fpy = (float)py;
    const float cz = m6 * fpx + m7 * fpy + m8;
    const float cu = (m0 * fpx + m1 * fpy + m2) / cz;
    const float cv = (m3 * fpx + m4 * fpy + m5) / cz;
    if (cu >= h3.x || cu < 0.0f || cv >= h3.y || cv < 0.0f) return 2.0f;
    const S src(V, j + 1);
    float ss = 0.f, sss = 0.f, srs = 0.f;
    if constexpr (NS > 0) {
        constexpr int NC = NS / 2;
        const int radius = prm.patch_size / 2;
        const int inc = prm.radius_increment;
        float qys[NS];
#pragma unroll
        for (int bb = 0; bb < NS; ++bb) qys[bb] = (float)window_coord<S>(py, -radius + bb * inc, V.H);
        const float qx0 = (float)window_coord<S>(px, -radius + (q.h * NC) * inc, V.W);
        const float qx1 = (float)window_coord<S>(px, -radius + (q.h * NC + NC - 1) * inc, V.W);
        // The projective depth z = fma(m7, qy, fma(m6, qx, m8)) is monotone in
        // qx and in qy (a rounded fma is monotone in its addend, and in its
        // multiplicand for a fixed multiplier), so over this lane's part of
        // the window it is extreme at the four corners.  When the corners lie
        // on one side of zero inside the range where the refined reciprocal
        // is exact, every sample does, and the per-sample range test drops.
        const float bz0 = fmaf(m6, qx0, m8), bz1 = fmaf(m6, qx1, m8);
        const float za = fmaf(m7, qys[0], bz0), zb = fmaf(m7, qys[NS - 1], bz0);
        const float zc = fmaf(m7, qys[0], bz1), zd = fmaf(m7, qys[NS - 1], bz1);
        const float zlo = fminf(fminf(za, zb), fminf(zc, zd)), zhi = fmaxf(fmaxf(za, zb), fmaxf(zc, zd));
        const bool in_range = (zlo >= kRcpLo && zhi <= kRcpHi) || (zhi <= -kRcpLo && zlo >= -kRcpHi);
        // QY(bb): the window row's coordinate, from the table where the row
        // loop is unrolled; computed in place where it is not, so that the
        // table is never indexed at run time (that would put it in local
        // memory for every evaluation)
#define GMVS_QY_TABLE(bb) qys[bb]
#define GMVS_QY_DIRECT(bb) ((float)window_coord<S>(py, -radius + (bb) * inc, V.H))
#define GMVS_SAMPLE_COLUMN(RCP, ROWS, QY)                                                          \
    {                                                                                              \
        const float qx = (float)window_coord<S>(px, -radius + (q.h * NC + al) * inc, V.W);        \
        const float bx = fmaf(m0, qx, m2), by = fmaf(m3, qx, m5), bz = fmaf(m6, qx, m8);           \
        _Pragma(ROWS) for (int bb = 0; bb < NS; ++bb) {                                            \
            const float qy = QY(bb);                                                               \
            const float rz = RCP(fmaf(m7, qy, bz));                                                \
            const float u = fmaf(m1, qy, bx) * rz;                                                 \
            const float v = fmaf(m4, qy, by) * rz;                                                 \
            const float s = src.sample(u, v);                                                      \
            const float2 wt = P.pw[(al * NS + bb) * P.pstride];                                    \
            const float ws = wt.x * s;                                                             \
            ss += ws;                                                                              \
            sss = fmaf(ws, s, sss);                                                                \
            srs = fmaf(wt.y, s, srs);                                                              \
        }                                                                                          \
    }
        if (in_range) {
            if constexpr (S::kTex) {
                // one instruction per sample, one column's fetches in flight
                // at a time: with every column unrolled the extra live
                // registers spill at the 80-register budget (measured 2.5 %
                // slower on the random pass, 10 % on the prior pass)
#pragma unroll 1
                for (int al = 0; al < NC; ++al) GMVS_SAMPLE_COLUMN(rcp_in_range, "unroll", GMVS_QY_TABLE)
            } else {
                // software-interpolated samples: keep the code compact
#pragma unroll 1
                for (int al = 0; al < NC; ++al) GMVS_SAMPLE_COLUMN(rcp_in_range, "unroll", GMVS_QY_TABLE)
            }
        } else if constexpr (S::kTex) {
#pragma unroll 1
            for (int al = 0; al < NC; ++al) GMVS_SAMPLE_COLUMN(rcp_rn, "unroll 1", GMVS_QY_DIRECT)
        } else {
            // the software samplers keep the table in local memory (measured
            // faster at their 128-register budget than holding it in registers
            // across the rolled column loop)
#pragma unroll 1
            for (int al = 0; al < NC; ++al) GMVS_SAMPLE_COLUMN(rcp_rn, "unroll 1", GMVS_QY_TABLE)
        }
#undef GMVS_SAMPLE_COLUMN
#undef GMVS_QY_TABLE
#undef GMVS_QY_DIRECT
    } else {
        const int radius = prm.patch_size / 2;
        const int inc = prm.radius_increment;
        const int n = (2 * radius) / inc + 1;
        const S ref(V, 0);
        for (int a = P.c0; a < P.c1; ++a) {
            const int i = -radius + a * inc;
            const float fqx = (float)window_coord<S>(px, i, V.W);
            const float bx = fmaf(m0, fqx, m2), by = fmaf(m3, fqx, m5), bz = fmaf(m6, fqx, m8);
            for (int bb = 0; bb < n; ++bb) {
                const int jj = -radius + bb * inc;
                const int qy = window_coord<S>(py, jj, V.H);
                const float r = ref.at((int)fqx, qy);
                const float w =
                    bilateral_weight((float)i, (float)jj, r, P.center, prm.sigma_spatial, prm.sigma_color);
                const float fqy = (float)qy;
                const float rz = rcp_rn(fmaf(m7, fqy, bz));
                const float u = fmaf(m1, fqy, bx) * rz;
                const float v = fmaf(m4, fqy, by) * rz;
                const float s = src.sample(u, v);
                const float ws = w * s;
                ss += ws;
                sss = fmaf(ws, s, sss);
                srs = fmaf(w * r, s, srs);
            }
        }
    }
    ss = pair_sum(q, ss);
    sss = pair_sum(q, sss);
    srs = pair_sum(q, srs);
    const float sm = ss * P.inv;
    const float sq = sss * P.inv;
    const float sr = srs * P.inv;
    const float var_s = sq - sm * sm;
    if (P.var_r < 1e-5f || var_s < 1e-5f) return 2.0f;
    const float cov = sr - P.mean_r * sm;
    const float vrs = sqrtf(P.var_r * var_s);
    return fmaxf(0.0f, fminf(2.0f, 1.0f - cov / vrs));
}

// ----------------------------------------------------------- camera math --
__device__ __forceinline__ float depth_from_plane(const DevCam& c, float4 pl, int px, int py) {
    return -pl.w * c.K[0] /
           (((float)px - c.K[2]) * pl.x + (c.K[0] / c.K[4]) * ((float)py - c.K[5]) * pl.y + c.K[0] * pl.z);
}
__device__ __forceinline__ void get_3d_point(const DevCam& c, int px, int py, float depth, float X[3]) {
    X[0] = depth * ((float)px - c.K[2]) / c.K[0];
    X[1] = depth * ((float)py - c.K[5]) / c.K[4];
    X[2] = depth;
}
__device__ __forceinline__ float distance_to_origin(const DevCam& c, int px, int py, float depth, float4 n) {
    float X[3];
    get_3d_point(c, px, py, depth, X);
    return -(n.x * X[0] + n.y * X[1] + n.z * X[2]);
}
__device__ __forceinline__ float4 view_direction(const DevCam& c, int px, int py, float depth) {
    float X[3];
    get_3d_point(c, px, py, depth, X);
    const float norm = sqrtf(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
    return make_float4(X[0] / norm, X[1] / norm, X[2] / norm, 0.0f);
}
__device__ __forceinline__ void normalize3(float4& v) {
    const float inv = 1.0f / sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    v.x *= inv;
    v.y *= inv;
    v.z *= inv;
}
__device__ __forceinline__ float4 normal_to_world(const DevCam& c, float4 p) {
    return make_float4(c.R[0] * p.x + c.R[3] * p.y + c.R[6] * p.z, c.R[1] * p.x + c.R[4] * p.y + c.R[7] * p.z,
                       c.R[2] * p.x + c.R[5] * p.y + c.R[8] * p.z, p.w);
}
__device__ __forceinline__ float4 normal_to_cam(const DevCam& c, float4 p) {
    return make_float4(c.R[0] * p.x + c.R[1] * p.y + c.R[2] * p.z, c.R[3] * p.x + c.R[4] * p.y + c.R[5] * p.z,
                       c.R[6] * p.x + c.R[7] * p.y + c.R[8] * p.z, p.w);
}

// GenerateRandomNormal (patch_match_kernel.cu:137-172); rejection bounded at 64.
static __device__ __noinline__ float4 random_normal(const DevCam& c, int px, int py, DevRng& rng, float depth) {
    float q1 = 1.0f, q2 = 1.0f, s = 2.0f;
    for (int it = 0; it < 64 && s >= 1.0f; ++it) {
        q1 = 2.0f * rng.uniform() - 1.0f;
        q2 = 2.0f * rng.uniform() - 1.0f;
        s = q1 * q1 + q2 * q2;
    }
    if (s >= 1.0f) {
        q1 = 0.0f;
        q2 = 0.0f;
        s = 0.0f;
    }
    const float sq = sqrtf(1.0f - s);
    float4 n = make_float4(2.0f * q1 * sq, 2.0f * q2 * sq, 1.0f - 2.0f * s, 0.0f);
    const float4 vd = view_direction(c, px, py, depth);
    if (n.x * vd.x + n.y * vd.y + n.z * vd.z > 0.0f) {
        n.x = -n.x;
        n.y = -n.y;
        n.z = -n.z;
    }
    normalize3(n);
    return n;
}

// GeneratePerturbedNormal (patch_match_kernel.cu:174-213)
static __device__ __noinline__ float4 perturbed_normal(const DevCam& c, int px, int py, float4 n, DevRng& rng, float pert) {
    const float4 vd = view_direction(c, px, py, 1.0f);
    const float a1 = (rng.uniform() - 0.5f) * pert;
    const float a2 = (rng.uniform() - 0.5f) * pert;
    const float a3 = (rng.uniform() - 0.5f) * pert;
    const float s1 = pmath::sinf_(a1), s2 = pmath::sinf_(a2), s3 = pmath::sinf_(a3);
    const float c1 = pmath::cosf_(a1), c2 = pmath::cosf_(a2), c3 = pmath::cosf_(a3);
    const float R0 = c2 * c3, R1 = c3 * s1 * s2 - c1 * s3, R2 = s1 * s3 + c1 * c3 * s2;
    const float R3 = c2 * s3, R4 = c1 * c3 + s1 * s2 * s3, R5 = c1 * s2 * s3 - c3 * s1;
    const float R6 = -s2, R7 = c2 * s1, R8 = c1 * c2;
    float4 np = make_float4(R0 * n.x + R1 * n.y + R2 * n.z, R3 * n.x + R4 * n.y + R5 * n.z,
                            R6 * n.x + R7 * n.y + R8 * n.z, 0.0f);
    if (np.x * vd.x + np.y * vd.y + np.z * vd.z >= 0.0f) np = n;
    normalize3(np);
    return np;
}

// compute_geom_consistency_cost (gmvs/src/patch_match.cu:562-593), in two
// parts: the world point of the reference pixel at the plane's depth depends
// only on the plane, so callers that test one plane against several source
// views form it once (geom_point) and evaluate each view from it (geom_cost).
struct GeomPoint {
    float X[3];
};
__device__ __forceinline__ GeomPoint geom_point(const DevView& V, float4 pl, int px, int py) {
    const DevCam& rc = V.cam[0];
    GeomPoint g;
    point_on_world((float)px, (float)py, depth_from_plane(rc, pl, px, py), rc, g.X);
    return g;
}
static __device__ __noinline__ float geom_cost(const DevView& V, int j, const GeomPoint& g, int px, int py) {
    const DevCam& rc = V.cam[0];
    const DevCam& sc = V.cam[j + 1];
    float su, sv, sd;
    project_on_camera(g.X, sc, su, sv, sd);
    const float src_depth = bilinear_clamp(V.dep[j + 1], su, sv, V.H, V.W);
    if (src_depth == 0.0f) return 5.0f;
    float Y[3];
    point_on_world(su, sv, src_depth, sc, Y);
    float bu, bv, bd;
    project_on_camera(Y, rc, bu, bv, bd);
    const float dc = (float)px - bu, dr = (float)py - bv;
    return fminf(5.0f, sqrtf(dc * dc + dr * dr));
}

// planar-prior restricted cost (patch_match_kernel.cu:1256-1290, 784-801)
struct PriorK {
    float gamma, two_dsq, two_asq, beta, depth_sigma, angle_sigma;
};
__device__ __forceinline__ PriorK prior_k(const DevView& V) {
    PriorK k;
    k.gamma = 0.5f;
    k.depth_sigma = (V.depth_max - V.depth_min) / 64.0f;
    k.two_dsq = 2 * k.depth_sigma * k.depth_sigma;
    k.angle_sigma = (float)(3.14159265358979323846 * (5.0f / 180.0f));
    k.two_asq = 2 * k.angle_sigma * k.angle_sigma;
    k.beta = 0.18f;
    return k;
}
static __device__ __noinline__ float restricted(const PriorK& k, float cost, float dd, float ac) {
    const float ad = pmath::acosf_(ac);
    const float pr = k.gamma + pmath::expf_(-dd * dd / k.two_dsq) * pmath::expf_(-ad * ad / k.two_asq);
    return pmath::expf_(-cost * cost / k.beta) * pr;
}

// insertion sort, FindMinCostIndex / FindMaxCostIndex (patch_match_kernel.cu:5-37)
__device__ __forceinline__ int find_min_idx8(const float* c) {
    float m = c[0];
    int mi = 0;
#pragma unroll
    for (int i = 1; i < 8; ++i)
        if (c[i] <= m) {
            m = c[i];
            mi = i;
        }
    return mi;
}
__device__ __forceinline__ int find_max_idx8(const float* c) {
    float m = c[0];
    int mi = 0;
#pragma unroll
    for (int i = 1; i < 8; ++i)
        if (c[i] >= m) {
            m = c[i];
            mi = i;
        }
    return mi;
}

// ------------------------------------------------------------------ init --
// One pixel of RandomInitialization (patch_match_kernel.cu:1467-1577) or of
// module B's initialization (gmvs/src/patch_match.cu:1046-1082), evaluated by
// a lane pair.  `cv` is the pixel's shared-memory slot (stride npix),
// 2 * nmax floats; both lanes write the same values.
template <class S, int NS>
__device__ void init_pixel(const DevView& V, const DevParams& prm, int px, int py, float* cv, int npix,
                           const Pair& q, float2* pw, int pstride) {
    const int W = V.W, N = V.N;
    const int c = py * W + px;
    const DevCam& rc = V.cam[0];
    DevRng rng(prm.seed_lo, prm.seed_hi, (uint32_t)c, (uint32_t)V.stream_id, phase_of(V.pass_index, 0));
    float4 pl;
    if (V.init_kind == GMVS_INIT_DEPTH_NORMAL) {
        // compute_plane_hypothesis_from_normal_depth (gmvs/src/patch_match.cu:329-339)
        pl = make_float4(V.ref_normal[c * 3 + 0], V.ref_normal[c * 3 + 1], V.ref_normal[c * 3 + 2], V.dep[0][c]);
        pl = normal_to_cam(rc, pl);
        const float depth = pl.w;
        pl.w = distance_to_origin(rc, px, py, depth, pl);
    } else if (V.init_kind == GMVS_INIT_PRIOR) {
        if (V.prior_masks[c] > 0 && V.init_costs[c] >= 0.1f) {
            const float pert = 0.02f;
            const float4 pp = V.prior_planes[c];
            float d = pp.w;
            const float dmin = (1 - 3 * pert) * d;
            const float dmax = (1 + 3 * pert) * d;
            d = rng.uniform() * (dmax - dmin) + dmin;
            float4 np = perturbed_normal(rc, px, py, pp, rng, (float)(3 * pert * 3.14159265358979323846));
            np.w = d;
            pl = np;
        } else {
            pl = V.init_planes[c];
            const float depth = pl.w;
            pl.w = distance_to_origin(rc, px, py, depth, pl);
        }
    } else {
        const float depth = rng.uniform() * (V.depth_max - V.depth_min) + V.depth_min;
        pl = random_normal(rc, px, py, rng, depth);
        pl.w = distance_to_origin(rc, px, py, depth, pl);
    }
    Patch<NS> P;
    if constexpr (NS > 0) {
        P.pw = pw;
        P.pstride = pstride;
    }
    make_patch<S, NS>(P, S(V, 0), V, prm, px, py, q);
    const Hyp h = make_hyp(rc, pl);
    int valid = 0;
    for (int i = 0; i < N; ++i) {
        const float v = ncc_cost<S, NS>(V, prm, i, h, P, px, py, q);
        cv[i * npix] = v;
        cv[(prm.nmax + i) * npix] = v;
        if (v < 2.0f) valid++;
    }
    // ComputeMultiViewInitialCostandSelectedViews (patch_match_kernel.cu:518-569)
    float* srt = cv + prm.nmax * npix;
    if (q.h == 0) {
        for (int i = 1; i < N; i++) {
            const float tmp = srt[i * npix];
            int j = i;
            for (; j >= 1 && tmp < srt[(j - 1) * npix]; j--) srt[j * npix] = srt[(j - 1) * npix];
            srt[j * npix] = tmp;
        }
        uint32_t sel = 0;
        float cost = 2.0f;
        const int top_k = min(valid, prm.top_k);
        if (top_k > 0) {
            float acc = 0.0f;
            for (int i = 0; i < top_k; ++i) acc += srt[i * npix];
            const float thr = srt[(top_k - 1) * npix];
            for (int i = 0; i < N; ++i)
                if (cv[i * npix] <= thr) sel |= 1u << i;
            cost = acc / (float)top_k;
        }
        V.plane[0][c] = pl;
        V.cost[0][c] = cost;
        V.sel[0][c] = sel;
    }
}

// The geometric terms of source views ja and jb (jb < 0: none) for the
// pixel of lane pair q: each lane evaluates one and a shuffle hands both
// lanes both, instead of both lanes evaluating both.  Both lanes of the pair
// call this with the same arguments, so the shuffle always has its partner.
__device__ __forceinline__ void pair_geom(const DevView& V, int ja, int jb, const GeomPoint& g, int px, int py,
                                          const Pair& q, float& ga, float& gb) {
    const int jm = q.h ? jb : ja;
    const float gm = jm >= 0 ? geom_cost(V, jm, g, px, py) : 0.0f;
    const float go = __shfl_xor_sync(q.mask, gm, 1);
    ga = q.h ? go : gm;
    gb = q.h ? gm : go;
}

// The source views a weighted sum visits, as a bit set walked in ascending
// order (the accumulation order of the reference).  With the software
// samplers each lane pair walks only its own selected views, so at step k
// every pair of the warp evaluates its k-th selected view on the same
// instructions instead of the warp stepping through every view with the
// unselected pairs idle (geometric pass 6-9 % faster, results unchanged).
// A texture fetch whose texture differs across the warp costs more than the
// idle lanes save (random pass 5.5 % slower), so the texture sampler walks
// every view and skips the unselected ones.
__device__ __forceinline__ uint32_t all_view_bits(int N) { return N >= 32 ? 0xffffffffu : ((1u << N) - 1u); }
template <class S>
__device__ __forceinline__ uint32_t sel_views(uint32_t sel, int N) {
    if constexpr (S::kTex) return all_view_bits(N);
    else return sel;
}

// --------------------------------------------------------------- sweep --
// Per-pixel words the three-kernel half-sweep passes from its selection
// kernel to its refinement kernel: current plane (4), its cost and depth,
// selected views, the view-selection draw counters (4), the three
// refinement planes (12), the random and perturbed depths, the depth before
// refinement and the restricted cost; one spare.
constexpr int kRefineWords = 28;

// One pixel of a half-sweep: CheckerboardPropagation (patch_match_kernel.cu:
// 813-1351; gmvs/src/patch_match.cu:678-1041) then PlaneHypothesisRefinement
// (patch_match_kernel.cu:684-811; gmvs/src/patch_match.cu:595-676), by a lane
// pair.  Reads the state at the start of the half-sweep (buffer `same` for
// this colour, `opp` for the other) and writes the pixel to buffer `outb`.
// `my` is the pixel's shared-memory slot (stride npix): nmax view weights,
// then the cold per-pixel state (neighbour positions, candidate final costs,
// refinement planes); the 8 x nmax cost matrix (9 x nmax in the three-kernel
// form) is `ca`, global scratch at stride 16.  All 14 hypotheses
// (8 neighbours, the current plane, 5 refinement candidates) go through one
// NCC loop.
// PH selects the part of the half-sweep: 0 = all of it; 1 = the neighbour
// hypotheses only (their cost matrix and positions go to per-pixel scratch);
// 2 = the rest, from that scratch.  1 then 2 compute exactly what 0 does, as
// two kernels with fewer live registers each.  Three kernels: 3 = the
// neighbour hypotheses and the current plane against every source view
// (cost matrix rows 0-7 and row 8), 4 = view selection, the candidates' final
// costs, the current plane's cost from row 8, the best candidate and the
// refinement planes, with no NCC (state to `rf`), 5 = the five refinement
// hypotheses, from `rf`.  3, 4, 5 compute exactly what 0 does.  `nb`
// (PH 1-4): this pixel's 10 scratch words (flags, same-colour bits, 8
// positions) at stride 16; `rf` (PH 4, 5): its kRefineWords state words at
// stride 16.
template <class S, int NS, int PH>
__device__ void sweep_pixel(const DevView& V, const DevParams& prm, int px, int py, int iter, int colour, float* my,
                            int npix, const Pair& q, float2* pw, int pstride, float* __restrict__ ca,
                            int* __restrict__ nb, float* __restrict__ rf) {
    const int W = V.W, H = V.H, N = V.N, nmax = prm.nmax;
    const int center = py * W + px;
    const int same = iter & 1;
    const int opp = colour == 0 ? (iter & 1) : ((iter + 1) & 1);
    const int outb = (iter + 1) & 1;
    const float* __restrict__ cs = V.cost[same];
    const float* __restrict__ co = V.cost[opp];
    const DevCam& rc = V.cam[0];
    const bool geom = V.sweep_kind == GMVS_SWEEP_GEOM;
    const bool prior_mode = V.sweep_kind == GMVS_SWEEP_PRIOR;
#define CA(k, i) ca[((k) * nmax + (i)) * 16]
#define VW(i) my[(i) * npix]
#define POS(k) (*reinterpret_cast<int*>(&my[(nmax + (k)) * npix]))
#define FC(k) my[(nmax + 8 + (k)) * npix]
#define PL4(slot, c) my[(nmax + 16 + 4 * (slot) + (c)) * npix]

    DevRng rng(prm.seed_lo, prm.seed_hi, (uint32_t)center, (uint32_t)V.stream_id,
               phase_of(V.pass_index, 1 + 2 * iter + colour));
    Patch<NS> P;
    if constexpr (NS > 0) {
        P.pw = pw;
        P.pstride = pstride;
    }
    if constexpr (PH != 4) make_patch<S, NS>(P, S(V, 0), V, prm, px, py, q);  // PH 4 runs no NCC

    // Adaptive checkerboard sampling.  pos = linear index; the buffer of a
    // candidate follows from its offset parity (odd = other colour).
    unsigned flags = 0u, fromsame = 0u;
    if constexpr (PH == 5) {
        // the refinement needs no neighbour positions
    } else if constexpr (PH == 2 || PH == 4) {
        flags = (unsigned)nb[0];
        fromsame = (unsigned)nb[16];
        for (int k = 0; k < 8; ++k)
            if ((flags >> k) & 1u) POS(k) = nb[(2 + k) * 16];
    } else {
        int pos[8];
        {
            float cmin;
            int cminp;
            bool csame;
            if (py > 2) {  // up_far (odd offsets only)
                flags |= 1u << 1;
                cminp = center - 3 * W;
                cmin = co[GMVS_IDX(cminp, H * W, kOobNeighbour)];
                for (int i = 1; i < 11; ++i)
                    if (py > 2 + 2 * i) {
                        const int t = center - 3 * W - 2 * i * W;
                        const float v = co[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                        }
                    }
                pos[1] = cminp;
            }
            if (py < H - 3) {  // down_far
                flags |= 1u << 3;
                cminp = center + 3 * W;
                cmin = co[GMVS_IDX(cminp, H * W, kOobNeighbour)];
                for (int i = 1; i < 11; ++i)
                    if (py < H - 3 - 2 * i) {
                        const int t = center + 3 * W + 2 * i * W;
                        const float v = co[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                        }
                    }
                pos[3] = cminp;
            }
            if (px > 2) {  // left_far
                flags |= 1u << 5;
                cminp = center - 3;
                cmin = co[GMVS_IDX(cminp, H * W, kOobNeighbour)];
                for (int i = 1; i < 11; ++i)
                    if (px > 2 + 2 * i) {
                        const int t = center - 3 - 2 * i;
                        const float v = co[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                        }
                    }
                pos[5] = cminp;
            }
            if (px < W - 3) {  // right_far keeps the maximum (patch_match_kernel.cu:954)
                flags |= 1u << 7;
                cminp = center + 3;
                cmin = co[GMVS_IDX(cminp, H * W, kOobNeighbour)];
                for (int i = 1; i < 11; ++i)
                    if (px < W - 3 - 2 * i) {
                        const int t = center + 3 + 2 * i;
                        const float v = co[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (cmin < v) {
                            cmin = v;
                            cminp = t;
                        }
                    }
                pos[7] = cminp;
            }
            // near neighbours: the first candidate (offset 1) has the other
            // colour, the V-shaped ones (offset parity even) this colour.
            if (py > 0) {  // up_near
                flags |= 1u << 0;
                cminp = center - W;
                cmin = co[GMVS_IDX(cminp, H * W, kOobNeighbour)];
                csame = false;
                for (int i = 0; i < 3; ++i) {
                    if (py > 1 + i && px > i) {
                        const int t = center - W - (1 + i) * W - i;
                        const float v = cs[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                            csame = true;
                        }
                    }
                    if (py > 1 + i && px < W - 1 - i) {
                        const int t = center - W - (1 + i) * W + i;
                        const float v = cs[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                            csame = true;
                        }
                    }
                }
                pos[0] = cminp;
                if (csame) fromsame |= 1u << 0;
            }
            if (py < H - 1) {  // down_near
                flags |= 1u << 2;
                cminp = center + W;
                cmin = co[GMVS_IDX(cminp, H * W, kOobNeighbour)];
                csame = false;
                for (int i = 0; i < 3; ++i) {
                    if (py < H - 2 - i && px > i) {
                        const int t = center + W + (1 + i) * W - i;
                        const float v = cs[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                            csame = true;
                        }
                    }
                    if (py < H - 2 - i && px < W - 1 - i) {
                        const int t = center + W + (1 + i) * W + i;
                        const float v = cs[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                            csame = true;
                        }
                    }
                }
                pos[2] = cminp;
                if (csame) fromsame |= 1u << 2;
            }
            if (px > 0) {  // left_near
                flags |= 1u << 4;
                cminp = center - 1;
                cmin = co[GMVS_IDX(cminp, H * W, kOobNeighbour)];
                csame = false;
                for (int i = 0; i < 3; ++i) {
                    if (px > 1 + i && py > i) {
                        const int t = center - 1 - (1 + i) - i * W;
                        const float v = cs[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                            csame = true;
                        }
                    }
                    if (px > 1 + i && py < H - 1 - i) {
                        const int t = center - 1 - (1 + i) + i * W;
                        const float v = cs[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                            csame = true;
                        }
                    }
                }
                pos[4] = cminp;
                if (csame) fromsame |= 1u << 4;
            }
            if (px < W - 1) {  // right_near
                flags |= 1u << 6;
                cminp = center + 1;
                cmin = co[GMVS_IDX(cminp, H * W, kOobNeighbour)];
                csame = false;
                for (int i = 0; i < 3; ++i) {
                    if (px < W - 2 - i && py > i) {
                        const int t = center + 1 + (1 + i) - i * W;
                        const float v = cs[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                            csame = true;
                        }
                    }
                    if (px < W - 2 - i && py < H - 1 - i) {
                        const int t = center + 1 + (1 + i) + i * W;
                        const float v = cs[GMVS_IDX(t, H * W, kOobNeighbour)];
                        if (v < cmin) {
                            cmin = v;
                            cminp = t;
                            csame = true;
                        }
                    }
                }
                pos[6] = cminp;
                if (csame) fromsame |= 1u << 6;
            }
        }
        for (int k = 0; k < 8; ++k)
            if ((flags >> k) & 1u) POS(k) = pos[k];
        if constexpr (PH == 1 || PH == 3) {
            if (q.h == 0) {
                nb[0] = (int)flags;
                nb[16] = (int)fromsame;
                for (int k = 0; k < 8; ++k) nb[(2 + k) * 16] = (flags >> k) & 1u ? pos[k] : 0;
            }
        }
    }
#define NPL(k) (V.plane[((fromsame >> (k)) & 1u) ? same : opp][GMVS_IDX(POS(k), H * W, kOobNeighbour)])

    // state carried between the phases of the hypothesis loop
    float weight_norm = 0.0f, cost_now = 0.0f, cur_cost = 0.0f, depth_now = 0.0f, restricted_cost = 0.0f;
    float depth_prior = 0.0f, depth_rand = 0.0f, dnow = 0.0f, depth_pert = 0.0f;
    uint32_t temp_sel = 0u, cur_sel = V.sel[same][center];
    float4 cur = V.plane[same][center];
    float4 ppl = make_float4(0.f, 0.f, 0.f, 0.f);
    const PriorK pk = prior_k(V);
    const uint32_t mask = prior_mode ? V.prior_masks[center] : 0u;
    const bool use_prior = prior_mode && mask > 0;
    int min_idx = 0;

    if constexpr (PH == 5) {
        // the state the selection kernel left (layout: kRefineWords)
        cur = make_float4(rf[0], rf[16], rf[32], rf[48]);
        cur_cost = rf[4 * 16];
        depth_now = rf[5 * 16];
        cur_sel = __float_as_uint(rf[6 * 16]);
        const unsigned long long cnt_lo = (unsigned long long)__float_as_uint(rf[7 * 16]) |
                                          ((unsigned long long)__float_as_uint(rf[8 * 16]) << 32);
        const unsigned long long cnt_hi = (unsigned long long)__float_as_uint(rf[9 * 16]) |
                                          ((unsigned long long)__float_as_uint(rf[10 * 16]) << 32);
        for (int i = 0; i < N; ++i) {  // the selection kernel's weights, in its order
            const float w = (float)((((i < 16) ? cnt_lo : cnt_hi) >> ((i & 15) * 4)) & 15ull);
            VW(i) = w;
            if (w > 0) {
                temp_sel |= 1u << i;
                weight_norm += w;
            }
        }
        for (int c = 0; c < 12; ++c) PL4(c >> 2, c & 3) = rf[(11 + c) * 16];
        depth_rand = rf[23 * 16];
        depth_pert = rf[24 * 16];
        dnow = rf[25 * 16];
        restricted_cost = rf[26 * 16];
        if (prior_mode) {
            ppl = V.prior_planes[center];
            depth_prior = depth_from_plane(rc, ppl, px, py);
        }
    }
    constexpr int s_begin = (PH == 2 || PH == 4) ? 8 : (PH == 5 ? 9 : 0);
    constexpr int s_end = PH == 1 ? 8 : (PH == 3 ? 9 : (PH == 4 ? 10 : 14));
    for (int s = s_begin; s < s_end; ++s) {
        float4 pl;
        const bool all_views = s < 8 || PH == 3;
        if (s < 8) {
            if (!((flags >> s) & 1u)) {
                // the reference's `float cost_array[8][32] = {2.0f}` (2 at [0][0], else 0)
                for (int i = 0; i < N; ++i) CA(s, i) = (s == 0 && i == 0) ? 2.0f : 0.0f;
                continue;
            }
            pl = NPL(s);
        } else if (PH == 3) {
            pl = cur;  // its costs against every view: row 8 of the matrix
        } else if (s == 8) {
            // multi-hypothesis joint view selection (patch_match_kernel.cu:1114-1176)
            const uint32_t* so = V.sel[opp];
            [[maybe_unused]] const int HW = H * W;  // read by the bounds-checked build
            const uint32_t nb_sel[4] = {(flags & 1u) ? so[GMVS_IDX(center - W, HW, kOobNeighbour)] : 0u,
                                        (flags & 4u) ? so[GMVS_IDX(center + W, HW, kOobNeighbour)] : 0u,
                                        (flags & 16u) ? so[GMVS_IDX(center - 1, HW, kOobNeighbour)] : 0u,
                                        (flags & 64u) ? so[GMVS_IDX(center + 1, HW, kOobNeighbour)] : 0u};
            const float thr = prm.cost_thr[iter];
            const float fallback = pmath::expf_(thr * thr / (-0.32f));
            float prob_sum = 0.0f;
            for (int i = 0; i < N; ++i) {
                float pri = 0.0f;
                for (int k = 0; k < 4; ++k)
                    if (flags & (1u << (2 * k))) pri += ((nb_sel[k] >> i) & 1u) ? 0.9f : 0.1f;
                float count = 0.0f, tmpw = 0.0f;
                int count_false = 0;
                for (int k = 0; k < 8; ++k) {
                    const float c = CA(k, i);
                    if (c < thr) {
                        tmpw += pmath::expf_(c * c / (-0.18f));
                        count++;
                    }
                    if (c > 1.2f) count_false++;
                }
                float prob = 0.0f;
                if (count > 2 && count_false < 3)
                    prob = tmpw / count;
                else if (count_false < 3)
                    prob = fallback;
                prob = prob * pri;
                VW(i) = prob;  // the PDF lives in the weight slots until the draws
                prob_sum += prob;
            }
            {  // TransformPDFToCDF (patch_match_kernel.cu:70-83)
                const float inv = 1.0f / prob_sum;
                float cum = 0.0f;
                for (int i = 0; i < N; ++i) {
                    cum += VW(i) * inv;
                    VW(i) = cum;
                }
            }
            // 15 draws; hits per view (at most 15) counted in 4-bit fields
            // (two scalars, not an array: a run-time index would put it in local memory)
            unsigned long long cnt_lo = 0ull, cnt_hi = 0ull;  // views 0-15, 16-31
            for (int d = 0; d < 15; ++d) {
                const float rp = rng.uniform() - 1.1920928955078125e-07f;  // curand_uniform - FLT_EPSILON
                for (int v = 0; v < N; ++v)
                    if (VW(v) > rp) {
                        if (v < 16)
                            cnt_lo += 1ull << (v * 4);
                        else
                            cnt_hi += 1ull << ((v - 16) * 4);
                        break;
                    }
            }
            for (int i = 0; i < N; ++i) {
                const float w = (float)((((i < 16) ? cnt_lo : cnt_hi) >> ((i & 15) * 4)) & 15ull);
                VW(i) = w;
                if (w > 0) {
                    temp_sel |= 1u << i;
                    weight_norm += w;
                }
            }
            if constexpr (PH == 4) {
                if (q.h == 0) {
                    rf[7 * 16] = __uint_as_float((uint32_t)cnt_lo);
                    rf[8 * 16] = __uint_as_float((uint32_t)(cnt_lo >> 32));
                    rf[9 * 16] = __uint_as_float((uint32_t)cnt_hi);
                    rf[10 * 16] = __uint_as_float((uint32_t)(cnt_hi >> 32));
                }
            }
            // final costs of the 8 candidates (patch_match_kernel.cu:1178-1211;
            // gmvs/src/patch_match.cu:920-946)
            for (int k = 0; k < 8; ++k) {
                float acc = 0.0f;
                const bool fk = (flags >> k) & 1u;
                GeomPoint gk;
                if (geom && fk) gk = geom_point(V, NPL(k), px, py);
                // the views with a nonzero weight, ascending (see the hypothesis loop)
                if (geom && fk) {
                    // two views a step, the geometric term of one on each lane of the pair
                    for (uint32_t todo = temp_sel; todo;) {
                        const int ja = __ffs(todo) - 1;
                        todo &= todo - 1u;
                        const int jb = todo ? __ffs(todo) - 1 : -1;
                        if (jb >= 0) todo &= todo - 1u;
                        float ga, gb;
                        pair_geom(V, ja, jb, gk, px, py, q, ga, gb);
                        acc += VW(ja) * (CA(k, ja) + 0.1f * ga);
                        if (jb >= 0) acc += VW(jb) * (CA(k, jb) + 0.1f * gb);
                    }
                } else {
                    for (uint32_t todo = sel_views<S>(temp_sel, N); todo; todo &= todo - 1u) {
                        const int j = __ffs(todo) - 1;
                        const float w = VW(j);
                        if (w > 0) acc += w * CA(k, j);
                    }
                }
                FC(k) = acc / weight_norm;
            }
            {  // FindMinCostIndex: ties pick the last index
                float m = FC(0);
                for (int k = 1; k < 8; ++k)
                    if (FC(k) <= m) {
                        m = FC(k);
                        min_idx = k;
                    }
            }
            pl = cur;
        } else {
            if (s == 9 && PH != 5) {
                cur_cost = cost_now;
                depth_now = depth_from_plane(rc, cur, px, py);
                if (prior_mode) {
                    ppl = V.prior_planes[center];
                    depth_prior = depth_from_plane(rc, ppl, px, py);
                    if (mask > 0) {  // patch_match_kernel.cu:1256-1305
                        // FindMaxCostIndex over the restricted costs (0 for
                        // absent neighbours; ties pick the last index).  The
                        // texture kernels keep a running maximum (an array
                        // indexed at run time would sit in local memory); the
                        // software samplers keep the array, measured faster
                        // in their single-kernel form.
                        float rfc_max = 0.0f;
                        int max_idx = 0;
                        if constexpr (S::kTex) {
#pragma unroll 1
                            for (int k = 0; k < 8; ++k) {
                                float r = 0.0f;
                                if ((flags >> k) & 1u) {
                                    const float4 qp = NPL(k);
                                    const float dn = depth_from_plane(rc, qp, px, py);
                                    const float ac = ppl.x * qp.x + ppl.y * qp.y + ppl.z * qp.z;
                                    r = restricted(pk, FC(k), dn - depth_prior, ac);
                                }
                                if (k == 0 || r >= rfc_max) {
                                    rfc_max = r;
                                    max_idx = k;
                                }
                            }
                        } else {
                            float rfc[8];
                            for (int k = 0; k < 8; ++k) {
                                rfc[k] = 0.0f;
                                if ((flags >> k) & 1u) {
                                    const float4 qp = NPL(k);
                                    const float dn = depth_from_plane(rc, qp, px, py);
                                    const float ac = ppl.x * qp.x + ppl.y * qp.y + ppl.z * qp.z;
                                    rfc[k] = restricted(pk, FC(k), dn - depth_prior, ac);
                                }
                            }
                            max_idx = find_max_idx8(rfc);
                            rfc_max = rfc[max_idx];
                        }
                        const float dn = depth_from_plane(rc, cur, px, py);
                        const float ac = ppl.x * cur.x + ppl.y * cur.y + ppl.z * cur.z;
                        const float rcn = restricted(pk, cost_now, dn - depth_prior, ac);
                        if ((flags >> max_idx) & 1u) {
                            const float4 qp = NPL(max_idx);
                            const float db = depth_from_plane(rc, qp, px, py);
                            if (db >= V.depth_min && db <= V.depth_max && rfc_max > rcn) {
                                depth_now = db;
                                cur = qp;
                                cur_cost = FC(max_idx);
                                restricted_cost = rfc_max;
                                cur_sel = temp_sel;
                            }
                        }
                    } else if ((flags >> min_idx) & 1u) {  // no selected-view update (1306-1318)
                        const float4 qp = NPL(min_idx);
                        const float db = depth_from_plane(rc, qp, px, py);
                        if (db >= V.depth_min && db <= V.depth_max && FC(min_idx) < cost_now) {
                            depth_now = db;
                            cur = qp;
                            cur_cost = FC(min_idx);
                        }
                    }
                } else if ((flags >> min_idx) & 1u) {
                    const float4 qp = NPL(min_idx);
                    const float db = depth_from_plane(rc, qp, px, py);
                    if (db >= V.depth_min && db <= V.depth_max && FC(min_idx) < cost_now) {
                        depth_now = db;
                        cur = qp;
                        cur_cost = FC(min_idx);
                        cur_sel = temp_sel;
                    }
                }
                // refinement candidates (patch_match_kernel.cu:684-760)
                const float pert = 0.02f;
                float4 n_rand;
                if (use_prior) {
                    depth_rand = rng.uniform() * 6 * pk.depth_sigma + (depth_prior - 3 * pk.depth_sigma);
                    n_rand = perturbed_normal(rc, px, py, ppl, rng, pk.angle_sigma);
                } else {
                    depth_rand = rng.uniform() * (V.depth_max - V.depth_min) + V.depth_min;
                    n_rand = random_normal(rc, px, py, rng, depth_now);
                }
                const float dmin_p = (1 - pert) * depth_now;
                const float dmax_p = (1 + pert) * depth_now;
                depth_pert = rng.uniform() * (dmax_p - dmin_p) + dmin_p;  // do/while runs once (quirk)
                const float4 n_pert = perturbed_normal(rc, px, py, cur, rng, (float)(pert * 3.14159265358979323846));
                // slots: 0 = base plane (after propagation), 1 = random normal, 2 = perturbed normal
                PL4(0, 0) = cur.x, PL4(0, 1) = cur.y, PL4(0, 2) = cur.z, PL4(0, 3) = cur.w;
                PL4(1, 0) = n_rand.x, PL4(1, 1) = n_rand.y, PL4(1, 2) = n_rand.z, PL4(1, 3) = n_rand.w;
                PL4(2, 0) = n_pert.x, PL4(2, 1) = n_pert.y, PL4(2, 2) = n_pert.z, PL4(2, 3) = n_pert.w;
                dnow = depth_now;
                if constexpr (PH == 4) {
                    if (q.h == 0) {
                        rf[0] = cur.x, rf[16] = cur.y, rf[32] = cur.z, rf[48] = cur.w;
                        rf[4 * 16] = cur_cost;
                        rf[5 * 16] = depth_now;
                        rf[6 * 16] = __uint_as_float(cur_sel);
                        for (int c = 0; c < 12; ++c) rf[(11 + c) * 16] = PL4(c >> 2, c & 3);
                        rf[23 * 16] = depth_rand;
                        rf[24 * 16] = depth_pert;
                        rf[25 * 16] = dnow;
                        rf[26 * 16] = restricted_cost;
                    }
                    return;
                }
            }
            // candidates (depth, normal): (rand, base), (now, rand), (rand, rand), (now, pert), (pert, base)
            const int k = s - 9;
            const int slot = (k == 1 || k == 2) ? 1 : (k == 3 ? 2 : 0);
            const float dk = (k == 0 || k == 2) ? depth_rand : (k == 4 ? depth_pert : dnow);
            pl = make_float4(PL4(slot, 0), PL4(slot, 1), PL4(slot, 2), PL4(slot, 3));
            pl.w = distance_to_origin(rc, px, py, dk, pl);
        }

        // the hypothesis against every source view (neighbours) or the
        // sampled ones (current plane, refinement)
        Hyp hy{};
        if constexpr (PH != 4) hy = make_hyp(rc, pl);
        if (geom && !all_views) {
            // the geometric terms of the selected views, split across the
            // lane pair, parked in row 0 of the neighbour-cost matrix (no
            // longer read once the eight final costs are formed at s == 8)
            const GeomPoint gp = geom_point(V, pl, px, py);
            for (uint32_t todo = temp_sel; todo;) {
                const int ja = __ffs(todo) - 1;
                todo &= todo - 1u;
                const int jb = todo ? __ffs(todo) - 1 : -1;
                if (jb >= 0) todo &= todo - 1u;
                float ga, gb;
                pair_geom(V, ja, jb, gp, px, py, q, ga, gb);
                CA(0, ja) = ga;
                if (jb >= 0) CA(0, jb) = gb;
            }
        }
        float acc = 0.0f;
        for (uint32_t todo = all_views ? all_view_bits(N) : sel_views<S>(temp_sel, N); todo; todo &= todo - 1u) {
            const int j = __ffs(todo) - 1;
            float w = 0.0f;
            if (!all_views) {
                w = VW(j);
                if (!(w > 0)) continue;
            }
            float c;
            if constexpr (PH == 4)
                c = CA(8, j);  // the current plane's cost, from the first kernel
            else
                c = ncc_cost<S, NS>(V, prm, j, hy, P, px, py, q);
            if (all_views)
                CA(s, j) = c;
            else if (geom)
                acc += w * (c + 0.1f * CA(0, j));
            else
                acc += w * c;
        }
        if (s == 8) {
            if constexpr (PH != 3) cost_now = acc / weight_norm;
        } else if (s > 8) {
            const float tc = acc / weight_norm;
            const float db = depth_from_plane(rc, pl, px, py);
            const float dk = (s == 9 || s == 11) ? depth_rand : ((s == 13) ? depth_pert : dnow);
            if (use_prior) {
                const float ac = ppl.x * pl.x + ppl.y * pl.y + ppl.z * pl.z;
                const float rtc = restricted(pk, tc, dk - depth_prior, ac);
                if (db >= V.depth_min && db <= V.depth_max && rtc > restricted_cost) {
                    depth_now = db;
                    cur = pl;
                    cur_cost = tc;
                    restricted_cost = rtc;
                }
            } else if (db >= V.depth_min && db <= V.depth_max && tc < cur_cost) {
                depth_now = db;
                cur = pl;
                cur_cost = tc;
            }
        }
    }
    if ((PH == 0 || PH == 2 || PH == 5) && q.h == 0) {
        V.plane[outb][center] = cur;
        V.cost[outb][center] = cur_cost;
        V.sel[outb][center] = cur_sel;
    }
#undef NPL
#undef PL4
#undef FC
#undef POS
#undef CA
#undef VW
}

// ---------------------------------------------------------- finalisation --
// GetDepthandNormal (patch_match_kernel.cu:1655-1674): depth first, then the
// normal is rotated to the world frame.
__device__ __forceinline__ void convert_pixel(const DevView& V, int final_buf, int px, int py) {
    const int c = py * V.W + px;
    float4 p = V.plane[final_buf][c];
    p.w = depth_from_plane(V.cam[0], p, px, py);
    V.fin[c] = normal_to_world(V.cam[0], p);
}

// CheckerboardFilter (patch_match_kernel.cu:1355-1463) on fin[].w, in place
// (only the other colour is read), then the export of this pixel
// (export_plane_hypotheses_cost, gmvs/src/patch_match.cu:1284-1313).
__device__ __forceinline__ void filter_export_pixel(const DevView& V, int final_buf, bool run_filter, int px, int py) {
    const int W = V.W, H = V.H;
    const int center = py * W + px;
    float4* __restrict__ pl = V.fin;
    const float cost = V.cost[final_buf][center];
    float4 me = pl[center];
    if (run_filter && !(cost < 0.001f)) {
        float f[21];
        int n = 0;
        f[n++] = me.w;
        const int left = center - 1, leftleft = center - 3, up = center - W, upup = center - 3 * W;
        const int down = center + W, downdown = center + 3 * W, right = center + 1, rightright = center + 3;
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
        for (int i = 1; i < n; i++) {
            const float tmp = f[i];
            int j = i;
            for (; j >= 1 && tmp < f[j - 1]; j--) f[j] = f[j - 1];
            f[j] = tmp;
        }
        const int m = n / 2;
        me.w = (n % 2 == 0) ? (f[m - 1] + f[m]) / 2 : f[m];
        pl[center].w = me.w;
    }
    V.out_depth[center] = me.w;
    V.out_normal[center * 3 + 0] = me.x;
    V.out_normal[center * 3 + 1] = me.y;
    V.out_normal[center * 3 + 2] = me.z;
    V.out_cost[center] = cost;
    if (V.out_planes) V.out_planes[center] = me;
}

}  // namespace gmvs
