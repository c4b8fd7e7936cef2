// Superpixel extraction of the segmentation preprocessing
// (gmvs/scripts/extract_superpixel.py): extract_superpixel (lines 55-74)
// and seg_func's segment-id map (lines 77-113), on the device except for
// the Felzenszwalb merge, which is a sequential scan and runs on the host
// (felzenszwalb.cpp) between the two device halves:
//
//   image [rows][cols][3] u8 --k_resize--> small [seg_rows][seg_cols][3] u8
//     --k_gauss_rows, k_gauss_cols--> smoothed FP64 (of x * (1 / 255))
//     --k_edge_weights--> 4 edge groups of FP64 weights --k_sort_* (stable
//     radix sort), k_sorted_ends--> edges in visiting order --D2H-->
//   host: two merge passes, labels, size filter --H2D-->
//     labels [seg_rows][seg_cols] --k_nearest_tables, k_up_dilate_rows
//     (nearest resize fused with the row maximum), k_box_extreme (column
//     maximum, row minimum), k_erode_cols_ids (column minimum)--> closed
//     ids u8 [rows][cols] (mask and its
//     per-id histogram fused), k_mask_filter
//   gray u8 --k_box_rows, k_box_cols_var--> sqrt|E[g^2] - E[g]^2| and its
//     maximum --k_var_apply--> var map f32, where(var < thresh, ids, 0).
//
// Every FP64 value is formed in the order of the CPU restatement, so the
// outputs equal it bit for bit; the integer stages are exact.  The
// arithmetic each stage restates (OpenCV's resize, close and box filter,
// scikit-image's Felzenszwalb) is described where it is computed.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "common.cuh"
#include "errors.h"
#include "superpixel.h"

namespace gmvs {
namespace {

constexpr int kMaxGaussRadius = 16;
struct GaussTaps {
    int r;
    double w[2 * kMaxGaussRadius + 1];
};

// reflect border with the edge pixel repeated: fedcba|abcdefgh|hgfedcb
// (OpenCV BORDER_REFLECT, SciPy mode "reflect")
__host__ __device__ inline int reflect_index(int i, int n) {
    if (n == 1) return 0;
    while (i < 0 || i >= n) i = i < 0 ? -i - 1 : 2 * n - 1 - i;
    return i;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr int kSortChunk = 2048;  // edges per block and radix pass (8 tiles of 256)

struct SpLayout {
    size_t small, gtmp, smooth, weights, keys2, vals, vals2, counts, ends_a, ends_b, sort_err, labels, sxs, sys, a, b,
        ids, s1, s2, var, vmax, hist, total;
    int64_t ne;
    int sort_blocks;
};

SpLayout sp_layout(int rows, int cols, const gmvs_superpixel_params& p) {
    const size_t ns = (size_t)p.seg_rows * p.seg_cols, n = (size_t)rows * cols;
    SpLayout L;
    L.ne = (int64_t)p.seg_rows * (p.seg_cols - 1) + (int64_t)(p.seg_rows - 1) * p.seg_cols +
           2LL * (p.seg_rows - 1) * (p.seg_cols - 1);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off = align256(off + bytes);
        return at;
    };
    L.small = take(ns * 3);
    L.gtmp = take(ns * 3 * sizeof(double));
    L.smooth = take(ns * 3 * sizeof(double));
    const size_t ne1 = (size_t)std::max<int64_t>(L.ne, 1);
    L.sort_blocks = (int)((ne1 + kSortChunk - 1) / kSortChunk);
    L.weights = take(ne1 * sizeof(double));  // sorted in place: the weights in visiting order
    L.keys2 = take(ne1 * sizeof(double));
    L.vals = take(ne1 * sizeof(uint32_t));
    L.vals2 = take(ne1 * sizeof(uint32_t));
    L.counts = take((size_t)256 * L.sort_blocks * sizeof(int32_t));
    L.ends_a = take(ne1 * sizeof(int32_t));
    L.ends_b = take(ne1 * sizeof(int32_t));
    L.sort_err = take(sizeof(int32_t));
    L.labels = take(ns * sizeof(int32_t));
    L.sxs = take((size_t)cols * sizeof(int32_t));
    L.sys = take((size_t)rows * sizeof(int32_t));
    L.a = take(n * sizeof(int32_t));
    L.b = take(n * sizeof(int32_t));
    L.ids = take(n);
    L.s1 = take(n * sizeof(double));
    L.s2 = take(n * sizeof(double));
    L.var = take(n * sizeof(double));
    L.vmax = take(sizeof(unsigned long long));
    L.hist = take(257 * sizeof(int32_t));  // 256 bins + the smallest present id
    L.total = off;
    return L;
}

// ------------------------------------------------------------- resize ---
// Bilinear resampling with pixel-centre alignment (OpenCV INTER_LINEAR for
// 8-bit images): src = (dst + 0.5) * (src_size / dst_size) - 0.5 in FP64,
// rounded to fp32, clamped at the edges; 11-bit fixed-point weights
// rounded to nearest (ties to even); the two-pass integer sum is rounded by
// a 22-bit shift.  An exact 2x reduction on both axes averages 2 x 2
// blocks with rounding (OpenCV takes INTER_AREA there).
struct Tap {
    int s0, s1, a0, a1;
};

__device__ inline Tap linear_tap(int d, int src, double scale) {
    float f = __double2float_rn((d + 0.5) * scale - 0.5);
    const float fl = floorf(f);
    int s = (int)fl;
    f = f - fl;
    if (s < 0) f = 0.0f, s = 0;
    if (s >= src - 1) f = 0.0f, s = src - 1;
    Tap t;
    t.s0 = s;
    t.s1 = min(s + 1, src - 1);
    t.a0 = __float2int_rn((1.0f - f) * 2048.0f);
    t.a1 = __float2int_rn(f * 2048.0f);
    return t;
}

__global__ void k_resize(const uint8_t* __restrict__ src, int H, int W, uint8_t* __restrict__ dst, int oh, int ow,
                         double scale_x, double scale_y, int area2) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= ow || y >= oh) return;
    uint8_t* o = dst + ((size_t)y * ow + x) * 3;
    if (area2) {
        const uint8_t* p0 = src + ((size_t)(2 * y) * W + 2 * x) * 3;
        const uint8_t* p1 = p0 + (size_t)W * 3;
        for (int c = 0; c < 3; ++c) o[c] = (uint8_t)((p0[c] + p0[3 + c] + p1[c] + p1[3 + c] + 2) >> 2);
        return;
    }
    const Tap tx = linear_tap(x, W, scale_x), ty = linear_tap(y, H, scale_y);
    const uint8_t* r0 = src + (size_t)ty.s0 * W * 3;
    const uint8_t* r1 = src + (size_t)ty.s1 * W * 3;
    for (int c = 0; c < 3; ++c) {
        const long long h0 = (long long)r0[tx.s0 * 3 + c] * tx.a0 + (long long)r0[tx.s1 * 3 + c] * tx.a1;
        const long long h1 = (long long)r1[tx.s0 * 3 + c] * tx.a0 + (long long)r1[tx.s1 * 3 + c] * tx.a1;
        const long long v = (h0 * ty.a0 + h1 * ty.a1 + (1LL << 21)) >> 22;
        o[c] = (uint8_t)min(max(v, 0LL), 255LL);
    }
}

// ------------------------------------------------------------ smoothing ---
// Gaussian pre-smoothing of each channel of x / 255 (scikit-image scales
// 8-bit input by 1/255 and smooths with SciPy's gaussian_filter: weights
// exp(-0.5 / sigma^2 * k^2) / sum over |k| <= int(4 sigma + 0.5), reflect
// borders, rows then columns).  Per output: the centre tap times its
// weight, then the tap pairs from the outermost inwards, each pair summed
// before it is weighted.
__global__ void k_gauss_rows(const uint8_t* __restrict__ small, int h, int w, GaussTaps g,
                             double* __restrict__ out) {
    const size_t n = (size_t)h * w * 3;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % 3), x = (int)((i / 3) % w), y = (int)(i / (3 * (size_t)w));
        auto at = [&](int yy) { return (double)small[((size_t)reflect_index(yy, h) * w + x) * 3 + c] * (1.0 / 255.0); };
        double s = at(y) * g.w[g.r];
        for (int k = -g.r; k < 0; ++k) s = s + (at(y + k) + at(y - k)) * g.w[g.r + k];
        out[i] = s;
    }
}

__global__ void k_gauss_cols(const double* __restrict__ in, int h, int w, GaussTaps g, double* __restrict__ out) {
    const size_t n = (size_t)h * w * 3;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % 3), x = (int)((i / 3) % w), y = (int)(i / (3 * (size_t)w));
        const double* row = in + (size_t)y * w * 3 + c;
        auto at = [&](int xx) { return row[(size_t)reflect_index(xx, w) * 3]; };
        double s = at(x) * g.w[g.r];
        for (int k = -g.r; k < 0; ++k) s = s + (at(x + k) + at(x - k)) * g.w[g.r + k];
        out[i] = s;
    }
}

// Euclidean colour distance of each edge's two smoothed pixels, channels
// summed in storage order; the groups and their order are those the host
// merge decodes (right, down, down-right, up-right; raster order each).
__global__ void k_edge_weights(const double* __restrict__ sm, int h, int w, double* __restrict__ wt, long long ne) {
    const long long nr = (long long)h * (w - 1), nd = (long long)(h - 1) * w, ng = (long long)(h - 1) * (w - 1);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ne;
         i += (long long)gridDim.x * blockDim.x) {
        long long e = i, a, b;
        if (e < nr) {
            const long long y = e / (w - 1), x = e % (w - 1);
            a = y * w + x, b = a + 1;
        } else if ((e -= nr) < nd) {
            a = e, b = e + w;
        } else {
            e -= nd;
            const bool up = e >= ng;
            if (up) e -= ng;
            const long long y = e / (w - 1), x = e % (w - 1), p = y * w + x;
            if (up)
                a = p + 1, b = p + w;
            else
                a = p, b = p + w + 1;
        }
        const double* pa = sm + a * 3;
        const double* pb = sm + b * 3;
        const double d0 = pb[0] - pa[0], d1 = pb[1] - pa[1], d2 = pb[2] - pa[2];
        double s = d0 * d0;
        s = s + d1 * d1;
        s = s + d2 * d2;
        wt[i] = sqrt(s);
    }
}

// ------------------------------------------------------------ edge order --
// The merge visits the edges by ascending weight, equal weights in edge
// order: a stable LSD radix sort of the weights' IEEE bit patterns (which
// order non-negative doubles like their values), 8 passes of 8-bit digits,
// carrying the edge index.  Each pass: per-block digit counts over a chunk
// of kSortChunk edges, one exclusive scan over (digit, block), then a
// scatter that ranks equal digits within a warp (match + popc), across the
// warps of a 256-edge tile and across tiles in order, so the chunk keeps
// its order within each digit.
__global__ void k_sort_init(uint32_t* __restrict__ vals, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        vals[i] = (uint32_t)i;
}

__global__ void __launch_bounds__(256) k_sort_count(const unsigned long long* __restrict__ keys, long long n, int shift,
                                                    int32_t* __restrict__ counts, int nblocks) {
    __shared__ int32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kSortChunk;
    for (int i = threadIdx.x; i < kSortChunk; i += 256) {
        const long long e = base + i;
        if (e < n) atomicAdd(&h[(keys[e] >> shift) & 255], 1);
    }
    __syncthreads();
    counts[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// exclusive scan of counts[0, total) in place (total a multiple of 4); one
// block of 1024 threads walking the array in coalesced rounds of 4096 (four
// counts per thread, warp scans, a scan of the warp totals, a carry between
// rounds), the next round's counts loaded while this round is scanned
__global__ void __launch_bounds__(1024) k_sort_scan(int32_t* __restrict__ counts, int total) {
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t carry;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int4* c4 = reinterpret_cast<int4*>(counts);
    const int n4 = total / 4;
    if (t == 0) carry = 0;
    __syncthreads();
    int4 next = t < n4 ? c4[t] : make_int4(0, 0, 0, 0);
    for (int base = 0; base < n4; base += 1024) {
        const int i = base + t;
        const int4 v = next;
        if (i + 1024 < n4) next = c4[i + 1024];
        const int32_t s = v.x + v.y + v.z + v.w;
        int32_t x = s;  // inclusive scan of the thread sums within the warp
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            int32_t z = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t y = __shfl_up_sync(0xffffffffu, z, o);
                if (lane >= o) z += y;
            }
            warp_tot[lane] = z;
        }
        __syncthreads();
        const int32_t excl = carry + (w ? warp_tot[w - 1] : 0) + (x - s);
        if (i < n4) c4[i] = make_int4(excl, excl + v.x, excl + v.x + v.y, excl + v.x + v.y + v.z);
        __syncthreads();
        if (t == 1023) carry = excl + s;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_sort_scatter(const unsigned long long* __restrict__ kin,
                                                      const uint32_t* __restrict__ vin,
                                                      unsigned long long* __restrict__ kout,
                                                      uint32_t* __restrict__ vout, long long n, int shift,
                                                      const int32_t* __restrict__ offsets, int nblocks, int* err) {
    __shared__ int32_t run[256];         // next slot of each digit for this chunk
    __shared__ int32_t wcount[8][256];   // per-warp digit counts of the current tile
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    run[t] = offsets[t * nblocks + blockIdx.x];
    for (int w = 0; w < 8; ++w) wcount[w][t] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kSortChunk;
    for (int tile = 0; tile < kSortChunk; tile += 256) {
        const long long e = base + tile + t;
        const bool valid = e < n;
        unsigned long long k = 0;
        uint32_t v = 0;
        int d = 256;  // past the end: a digit of its own, never written
        if (valid) {
            k = kin[e];
            v = vin[e];
            d = (int)((k >> shift) & 255);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == __ffs(peers) - 1) wcount[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            long long pos = (long long)run[d] + rank;
            for (int w = 0; w < warp; ++w) pos += wcount[w][d];
            if (pos >= 0 && pos < n) {
                kout[pos] = k;
                vout[pos] = v;
            } else {
                atomicOr(err, 1);
            }
        }
        __syncthreads();
        int32_t add = 0;
        for (int w = 0; w < 8; ++w) {
            add += wcount[w][t];
            wcount[w][t] = 0;
        }
        run[t] += add;
        __syncthreads();
    }
}

// endpoints of the sorted edges (the groups of k_edge_weights)
__global__ void k_sorted_ends(const uint32_t* __restrict__ order, long long ne, int h, int w, int32_t* __restrict__ sa,
                              int32_t* __restrict__ sb) {
    const long long nr = (long long)h * (w - 1), nd = (long long)(h - 1) * w, ng = (long long)(h - 1) * (w - 1);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ne;
         i += (long long)gridDim.x * blockDim.x) {
        long long e = order[i], a, b;
        if (e >= ne) {  // not a permutation: the sort's own check reports it
            sa[i] = sb[i] = 0;
            continue;
        }
        if (e < nr) {
            const long long y = e / (w - 1), x = e % (w - 1);
            a = y * w + x, b = a + 1;
        } else if ((e -= nr) < nd) {
            a = e, b = e + w;
        } else {
            e -= nd;
            const bool up = e >= ng;
            if (up) e -= ng;
            const long long y = e / (w - 1), x = e % (w - 1), p = y * w + x;
            if (up)
                a = p + 1, b = p + w;
            else
                a = p, b = p + w + 1;
        }
        sa[i] = (int32_t)a;
        sb[i] = (int32_t)b;
    }
}

// -------------------------------------------------- nearest resize + close --
// Nearest resize back to full size (OpenCV INTER_NEAREST:
// src = min(floor(dst * (1 / (dst_size / src_size))), src_size - 1)), one
// table entry per full-size column and row.
__global__ void k_nearest_tables(int W, int H, int sw, int sh, double ifx, double ify, int32_t* __restrict__ sxs,
                                 int32_t* __restrict__ sys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < W) sxs[i] = min((int)floor((double)i * ifx), sw - 1);
    if (i < H) sys[i] = min((int)floor((double)i * ify), sh - 1);
}

// The resize fused with the first pass of the close: a box maximum along the
// row over the pixels inside the image (the close's dilation, then erosion,
// with a close_size box; the border takes no part).
__global__ void k_up_dilate_rows(const int32_t* __restrict__ lbl, int sw, int H, int W,
                                 const int32_t* __restrict__ sxs, const int32_t* __restrict__ sys, int lo, int hi,
                                 int32_t* __restrict__ seg_out, int32_t* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const int32_t* row = lbl + (size_t)sys[y] * sw;
    int m = INT_MIN;
    for (int k = max(lo, -x); k <= min(hi, W - 1 - x); ++k) m = max(m, row[sxs[x + k]]);
    const size_t p = (size_t)y * W + x;
    out[p] = m;
    if (seg_out) seg_out[p] = row[sxs[x]];
}

template <bool kMax, bool kAlongRow>
__global__ void k_box_extreme(const int32_t* __restrict__ in, int H, int W, int lo, int hi,
                              int32_t* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    int m = kMax ? INT_MIN : INT_MAX;
    for (int k = lo; k <= hi; ++k) {
        const int xx = kAlongRow ? x + k : x, yy = kAlongRow ? y : y + k;
        if (xx < 0 || xx >= W || yy < 0 || yy >= H) continue;
        const int v = in[(size_t)yy * W + xx];
        m = kMax ? max(m, v) : min(m, v);
    }
    out[(size_t)y * W + x] = m;
}

// last pass of the close (column minimum), the cast to 8 bits (label & 255),
// the optional mask and the per-id histogram the mask's filter needs
__global__ void k_erode_cols_ids(const int32_t* __restrict__ in, int H, int W, int lo, int hi,
                                 const uint8_t* __restrict__ mask, uint8_t* __restrict__ ids, int32_t* hist) {
    __shared__ int32_t sh[256];
    const int t = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    if (hist)
        for (int i = t; i < 256; i += nt) sh[i] = 0;
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x < W && y < H) {
        int m = INT_MAX;
        for (int k = lo; k <= hi; ++k) {
            const int yy = y + k;
            if (yy < 0 || yy >= H) continue;
            m = min(m, in[(size_t)yy * W + x]);
        }
        const size_t p = (size_t)y * W + x;
        uint8_t u = (uint8_t)(m & 255);
        if (mask && !mask[p]) u = 0;
        ids[p] = u;
        if (hist) atomicAdd(&sh[u], 1);
    }
    __syncthreads();
    if (hist)
        for (int i = t; i < 256; i += nt)
            if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// seg_func's mask filter (extract_superpixel.py:90-94): every id present
// except the smallest present one is cleared when it covers fewer than
// rows * cols / 128 pixels.  hist[256] receives the smallest present id.
__global__ void k_first_present(int32_t* hist) {
    if (threadIdx.x != 0) return;
    int f = 256;
    for (int i = 0; i < 256; ++i)
        if (hist[i] > 0) {
            f = i;
            break;
        }
    hist[256] = f;
}

__global__ void k_mask_filter(uint8_t* __restrict__ ids, size_t n, const int32_t* __restrict__ hist) {
    const int first = hist[256];
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
        const int u = ids[p];
        if (u != first && (long long)hist[u] * 128 < (long long)n) ids[p] = 0;
    }
}

// ---------------------------------------------------------- variance map --
// winVar (extract_superpixel.py:47-52) of g = gray / 255: box means of g
// and g^2 over var_windlen x var_windlen with reflect borders (the window's
// row sums in order, then the row sums in order, times 1 / area), then
// sqrt(|E[g^2] - E[g]^2|) and its maximum.
__global__ void k_box_rows(const uint8_t* __restrict__ gray, int H, int W, int lo, int hi, double* __restrict__ s1,
                           double* __restrict__ s2) {
    __shared__ double level[256];  // g / 255 for every gray level: one FP64 division each
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    for (int i = t; i < 256; i += blockDim.x * blockDim.y) level[i] = (double)i / 255.0;
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const uint8_t* row = gray + (size_t)y * W;
    double a = 0.0, b = 0.0;
    for (int k = lo; k <= hi; ++k) {
        const double v = level[row[reflect_index(x + k, W)]];
        a = a + v;
        b = b + v * v;
    }
    s1[(size_t)y * W + x] = a;
    s2[(size_t)y * W + x] = b;
}

__global__ void k_box_cols_var(const double* __restrict__ s1, const double* __restrict__ s2, int H, int W, int lo,
                               int hi, double inv_area, double* __restrict__ var, unsigned long long* vmax) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    double v = 0.0;
    if (x < W && y < H) {
        double a = 0.0, b = 0.0;
        for (int k = lo; k <= hi; ++k) {
            const size_t q = (size_t)reflect_index(y + k, H) * W + x;
            a = a + s1[q];
            b = b + s2[q];
        }
        const double m1 = a * inv_area, m2 = b * inv_area;
        v = sqrt(fabs(m2 - m1 * m1));
        var[(size_t)y * W + x] = v;
    }
    // non-negative doubles order like their bit patterns
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    for (int o = 16; o > 0; o >>= 1) u = max(u, __shfl_xor_sync(0xffffffffu, u, o));
    if ((threadIdx.x & 31) == 0) atomicMax(vmax, u);
}

__global__ void k_var_apply(const double* __restrict__ var, const unsigned long long* __restrict__ vmax,
                            const uint8_t* __restrict__ ids, size_t n, float thresh, float* __restrict__ out_var,
                            int32_t* __restrict__ out_map) {
    const double mx = __longlong_as_double((long long)*vmax);
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
        const float vm = __double2float_rn(var[p] / mx);  // 0 / 0 = NaN: nothing passes, as in numpy
        if (out_var) out_var[p] = vm;
        if (out_map) out_map[p] = vm < thresh ? (int32_t)ids[p] : 0;
    }
}

__global__ void k_ids_to_int(const uint8_t* __restrict__ ids, size_t n, int32_t* __restrict__ out) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x)
        out[p] = ids[p];
}

int grid_1d(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

int32_t check_params(int rows, int cols, const gmvs_superpixel_params* p, const char* who) {
    if (!p) return fail(GMVS_ERR_INVALID, std::string(who) + ": NULL params");
    if (rows < 1 || cols < 1 || (long long)rows * cols > (1LL << 30))
        return fail(GMVS_ERR_INVALID, std::string(who) + ": image size out of range");
    if (p->seg_rows < 1 || p->seg_cols < 1 || (long long)p->seg_rows * p->seg_cols > (1LL << 26))
        return fail(GMVS_ERR_INVALID, std::string(who) + ": seg_rows / seg_cols out of range");
    if (!(p->sigma <= 3.8) || !(p->scale >= 0.0) || p->min_size < 0)
        return fail(GMVS_ERR_INVALID, std::string(who) + ": sigma must be <= 3.8, scale >= 0, min_size >= 0");
    if (p->close_size < 1 || p->close_size > 255 || p->close_size % 2 == 0)
        return fail(GMVS_ERR_INVALID, std::string(who) + ": close_size must be odd, 1..255");
    if (p->var_windlen > 1023) return fail(GMVS_ERR_INVALID, std::string(who) + ": var_windlen must be <= 1023");
    return GMVS_OK;
}

}  // namespace
}  // namespace gmvs

extern "C" void gmvs_superpixel_default_params(gmvs_superpixel_params* out) {
    if (!out) return;
    out->seg_rows = 288;
    out->seg_cols = 384;
    out->scale = 100.0;
    out->sigma = 0.5;
    out->min_size = 5;
    out->close_size = 11;
    out->var_windlen = 15;
    out->var_thresh = 0.2f;
}

extern "C" size_t gmvs_superpixel_workspace_bytes(int32_t rows, int32_t cols, const gmvs_superpixel_params* params) {
    using namespace gmvs;
    if (check_params(rows, cols, params, "gmvs_superpixel_workspace_bytes") != GMVS_OK) return 0;
    return sp_layout(rows, cols, *params).total + 256;
}

extern "C" int32_t gmvs_superpixels(const uint8_t* image, const uint8_t* gray, const uint8_t* mask, int32_t rows,
                                    int32_t cols, const gmvs_superpixel_params* params, int32_t* out_segment,
                                    uint8_t* out_ids, int32_t* out_ids_map, float* out_var_map,
                                    int32_t* out_num_segments, void* workspace, size_t workspace_bytes,
                                    void* stream) {
    using namespace gmvs;
    const char* who = "gmvs_superpixels";
    int32_t rc = check_params(rows, cols, params, who);
    if (rc != GMVS_OK) return rc;
    const gmvs_superpixel_params& P = *params;
    const bool var_on = P.var_thresh > 0.0f && P.var_windlen > 1;
    if (!image) return fail(GMVS_ERR_INVALID, std::string(who) + ": NULL image");
    if (var_on && (out_ids_map || out_var_map) && !gray)
        return fail(GMVS_ERR_INVALID, std::string(who) + ": the variance filter needs the gray image");
    const SpLayout L = sp_layout(rows, cols, P);
    char* ws = (char*)(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    if (!workspace || workspace_bytes < L.total + 256)
        return fail(GMVS_ERR_INVALID, std::string(who) + ": workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    const int sh = P.seg_rows, sw = P.seg_cols;

    // device half 1: resize, smoothing, edge weights
    const dim3 b2(32, 8);
    {
        const bool area2 = rows == 2 * sh && cols == 2 * sw;
        k_resize<<<dim3((sw + 31) / 32, (sh + 7) / 8), b2, 0, st>>>(image, rows, cols, (uint8_t*)(ws + L.small), sh,
                                                                    sw, 1.0 / ((double)sw / cols),
                                                                    1.0 / ((double)sh / rows), area2 ? 1 : 0);
        GaussTaps g{};
        if (P.sigma > 0.0) {
            g.r = (int)(4.0 * P.sigma + 0.5);
            double phi[2 * kMaxGaussRadius + 1], total = 0.0;
            for (int k = -g.r; k <= g.r; ++k) phi[k + g.r] = std::exp(-0.5 / (P.sigma * P.sigma) * (double)(k * k));
            for (int k = 0; k <= 2 * g.r; ++k) total += phi[k];
            for (int k = 0; k <= 2 * g.r; ++k) g.w[k] = phi[k] / total;
        } else {
            g.r = 0;
            g.w[0] = 1.0;
        }
        const size_t n3 = (size_t)sh * sw * 3;
        k_gauss_rows<<<grid_1d(n3), 256, 0, st>>>((const uint8_t*)(ws + L.small), sh, sw, g, (double*)(ws + L.gtmp));
        k_gauss_cols<<<grid_1d(n3), 256, 0, st>>>((const double*)(ws + L.gtmp), sh, sw, g, (double*)(ws + L.smooth));
        if (L.ne > 0)
            k_edge_weights<<<grid_1d((size_t)L.ne), 256, 0, st>>>((const double*)(ws + L.smooth), sh, sw,
                                                                  (double*)(ws + L.weights), L.ne);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, who);

    // the visiting order on the device; endpoints and weights to the host
    const size_t ne1 = (size_t)std::max<int64_t>(L.ne, 1);
    std::vector<double> sorted_w(ne1);
    std::vector<int32_t> ends_a(ne1), ends_b(ne1), labels((size_t)sh * sw);
    int32_t sort_err = 0;
    if (L.ne > 0) {
        unsigned long long* ka = (unsigned long long*)(ws + L.weights);
        unsigned long long* kb = (unsigned long long*)(ws + L.keys2);
        uint32_t* va = (uint32_t*)(ws + L.vals);
        uint32_t* vb = (uint32_t*)(ws + L.vals2);
        int32_t* counts = (int32_t*)(ws + L.counts);
        int* err = (int*)(ws + L.sort_err);
        e = cudaMemsetAsync(err, 0, sizeof(int), st);
        if (e != cudaSuccess) return fail_cuda(e, who);
        k_sort_init<<<grid_1d((size_t)L.ne), 256, 0, st>>>(va, L.ne);
        for (int pass = 0; pass < 8; ++pass) {  // even: the result ends in ka / va
            k_sort_count<<<L.sort_blocks, 256, 0, st>>>(ka, L.ne, 8 * pass, counts, L.sort_blocks);
            k_sort_scan<<<1, 1024, 0, st>>>(counts, 256 * L.sort_blocks);
            k_sort_scatter<<<L.sort_blocks, 256, 0, st>>>(ka, va, kb, vb, L.ne, 8 * pass, counts, L.sort_blocks, err);
            std::swap(ka, kb);
            std::swap(va, vb);
        }
        k_sorted_ends<<<grid_1d((size_t)L.ne), 256, 0, st>>>(va, L.ne, sh, sw, (int32_t*)(ws + L.ends_a),
                                                             (int32_t*)(ws + L.ends_b));
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sorted_w.data(), ka, sizeof(double) * L.ne, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ends_a.data(), ws + L.ends_a, sizeof(int32_t) * L.ne, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ends_b.data(), ws + L.ends_b, sizeof(int32_t) * L.ne, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&sort_err, err, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return fail_cuda(e, who);
    }
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda(e, who);
    if (sort_err) return fail(GMVS_ERR_DEVICE, std::string(who) + ": edge sort produced an out-of-range slot");
    // host: the merge
    const int32_t kept = superpixel_merge_sorted(sh, sw, L.ne, ends_a.data(), ends_b.data(), sorted_w.data(),
                                                 P.scale / 255.0, P.min_size, labels.data());
    if (out_num_segments) *out_num_segments = kept;
    // pageable source: the call returns once the labels are staged
    e = cudaMemcpyAsync(ws + L.labels, labels.data(), sizeof(int32_t) * labels.size(), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return fail_cuda(e, who);

    // device half 2: full-size labels, close, mask, variance filter
    const size_t n = (size_t)rows * cols;
    const dim3 g2((cols + 31) / 32, (rows + 7) / 8);
    const double ifx = 1.0 / ((double)cols / sw), ify = 1.0 / ((double)rows / sh);
    const bool need_ids = out_ids || out_ids_map;
    int32_t* sxs = (int32_t*)(ws + L.sxs);
    int32_t* sys = (int32_t*)(ws + L.sys);
    if (need_ids || out_segment) {
        const int m = std::max(rows, cols);
        k_nearest_tables<<<(m + 255) / 256, 256, 0, st>>>(cols, rows, sw, sh, ifx, ify, sxs, sys);
    }
    int32_t* a = (int32_t*)(ws + L.a);
    int32_t* b = (int32_t*)(ws + L.b);
    uint8_t* ids = out_ids ? out_ids : (uint8_t*)(ws + L.ids);
    const int lo = -(P.close_size / 2), hi = P.close_size - 1 - P.close_size / 2;
    if (need_ids) {
        k_up_dilate_rows<<<g2, b2, 0, st>>>((const int32_t*)(ws + L.labels), sw, rows, cols, sxs, sys, lo, hi,
                                            out_segment, a);
        k_box_extreme<true, false><<<g2, b2, 0, st>>>(a, rows, cols, lo, hi, b);
        k_box_extreme<false, true><<<g2, b2, 0, st>>>(b, rows, cols, lo, hi, a);
        int32_t* hist = mask ? (int32_t*)(ws + L.hist) : nullptr;
        if (hist) {
            e = cudaMemsetAsync(hist, 0, 257 * sizeof(int32_t), st);
            if (e != cudaSuccess) return fail_cuda(e, who);
        }
        k_erode_cols_ids<<<g2, b2, 0, st>>>(a, rows, cols, lo, hi, mask, ids, hist);
        if (hist) {
            k_first_present<<<1, 32, 0, st>>>(hist);
            k_mask_filter<<<grid_1d(n), 256, 0, st>>>(ids, n, hist);
        }
    } else if (out_segment) {
        k_up_dilate_rows<<<g2, b2, 0, st>>>((const int32_t*)(ws + L.labels), sw, rows, cols, sxs, sys, 0, 0,
                                            out_segment, a);
    }
    if (var_on && (out_ids_map || out_var_map)) {
        unsigned long long* vmax = (unsigned long long*)(ws + L.vmax);
        e = cudaMemsetAsync(vmax, 0, sizeof(unsigned long long), st);
        if (e != cudaSuccess) return fail_cuda(e, who);
        const int vlo = -(P.var_windlen / 2), vhi = P.var_windlen - 1 - P.var_windlen / 2;
        k_box_rows<<<g2, b2, 0, st>>>(gray, rows, cols, vlo, vhi, (double*)(ws + L.s1), (double*)(ws + L.s2));
        k_box_cols_var<<<g2, b2, 0, st>>>((const double*)(ws + L.s1), (const double*)(ws + L.s2), rows, cols, vlo,
                                          vhi, 1.0 / (double)(P.var_windlen * P.var_windlen), (double*)(ws + L.var),
                                          vmax);
        k_var_apply<<<grid_1d(n), 256, 0, st>>>((const double*)(ws + L.var), vmax, ids, n, P.var_thresh, out_var_map,
                                                out_ids_map);
    } else if (out_ids_map) {
        k_ids_to_int<<<grid_1d(n), 256, 0, st>>>(ids, n, out_ids_map);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, who);
    return GMVS_OK;
}
