// Device versions of the superpixel statistics the fusion scripts call
// through module A (fusion_planar_mask, filter_by_var_map,
// sliding_window_normal; gmvs/lib/src/planar_initer.cu:471-684).  They give
// the results of the host routines in prior.cpp bit for bit: every float sum
// runs in the reference's order.  For the per-segment sums that order is the
// raster order of the segment's pixels, so the pixels are first put in a
// stable order by segment (a counting sort whose per-row histograms are
// scanned down each segment's column), and one thread then accumulates each
// segment sequentially.
#include <algorithm>
#include <cstdint>
#include <string>

#include "common.cuh"
#include "errors.h"

namespace gmvs {
namespace {

// Workspace layout for rows x cols pixels and segment ids 0..max_seg.
struct SegLayout {
    size_t hist, count, start, order, kind, total;
};
size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
SegLayout seg_layout(int rows, int cols, int max_seg) {
    const size_t ns = (size_t)max_seg + 1;
    SegLayout L;
    size_t off = 0;
    L.hist = off;   // int32 [rows][ns]: per-row counts, then per-row start offsets
    off = align256(off + sizeof(int32_t) * (size_t)rows * ns);
    L.count = off;  // int32 [ns]
    off = align256(off + sizeof(int32_t) * ns);
    L.start = off;  // int32 [ns + 1]: first slot of each segment in `order`
    off = align256(off + sizeof(int32_t) * (ns + 1));
    L.order = off;  // int32 [rows * cols]: pixels sorted by segment, raster order inside
    off = align256(off + sizeof(int32_t) * (size_t)rows * cols);
    L.kind = off;   // int32 [ns]: per-segment decision / label
    off = align256(off + sizeof(int32_t) * ns);
    L.total = off;
    return L;
}

// --------------------------------------------------------- stable order --
// error bit 1: a segment id outside [0, max_seg]
__global__ void k_row_hist(const int32_t* __restrict__ seg, int rows, int cols, int max_seg,
                           int32_t* __restrict__ hist, int* __restrict__ err) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int32_t* h = hist + (size_t)r * (max_seg + 1);
    const int32_t* s = seg + (size_t)r * cols;
    int32_t cur = -1, run = 0;  // superpixels come in runs along a row
    for (int c = 0; c < cols; ++c) {
        const int32_t id = s[c];
        if (id < 0 || id > max_seg) {
            atomicOr(err, 1);
            continue;
        }
        if (id == cur) {
            ++run;
        } else {
            if (cur >= 0) h[cur] += run;
            cur = id;
            run = 1;
        }
    }
    if (cur >= 0) h[cur] += run;
}

// down each segment's column: per-row counts -> per-row offsets, totals
__global__ void k_col_scan(int32_t* __restrict__ hist, int rows, int max_seg, int32_t* __restrict__ count) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > max_seg) return;
    int32_t run = 0;
    for (int r = 0; r < rows; ++r) {
        int32_t* p = hist + (size_t)r * (max_seg + 1) + s;
        const int32_t t = *p;
        *p = run;
        run += t;
    }
    count[s] = run;
}

// exclusive scan of the segment sizes (one block)
__global__ void k_seg_scan(const int32_t* __restrict__ count, int ns, int32_t* __restrict__ start) {
    __shared__ int32_t part[1024];
    const int t = threadIdx.x, T = blockDim.x;
    const int per = (ns + T - 1) / T;
    const int b = t * per, e = min(ns, b + per);
    int32_t sum = 0;
    for (int i = b; i < e; ++i) sum += count[i];
    part[t] = sum;
    __syncthreads();
    if (t == 0) {
        int32_t run = 0;
        for (int i = 0; i < T; ++i) {
            const int32_t v = part[i];
            part[i] = run;
            run += v;
        }
        start[ns] = run;
    }
    __syncthreads();
    int32_t run = part[t];
    for (int i = b; i < e; ++i) {
        start[i] = run;
        run += count[i];
    }
}

__global__ void k_row_scatter(const int32_t* __restrict__ seg, int rows, int cols, int max_seg,
                              int32_t* __restrict__ hist, const int32_t* __restrict__ start,
                              int32_t* __restrict__ order) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int32_t* h = hist + (size_t)r * (max_seg + 1);
    const int32_t* s = seg + (size_t)r * cols;
    int32_t cur = -1, slot = 0;  // next slot of the current run's segment
    for (int c = 0; c < cols; ++c) {
        const int32_t id = s[c];
        if (id < 0 || id > max_seg) continue;
        if (id != cur) {
            if (cur >= 0) h[cur] = slot - start[cur];
            cur = id;
            slot = start[id] + h[id];
        }
        order[slot++] = r * cols + c;
    }
    if (cur >= 0) h[cur] = slot - start[cur];
}

// ----------------------------------------------------- filter_by_var_map --
__global__ void k_var_keep(const float* __restrict__ var, const int32_t* __restrict__ start,
                           const int32_t* __restrict__ order, int max_seg, float thresh, int32_t* __restrict__ keep) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > max_seg) return;
    if (s == 0) {
        keep[0] = 0;
        return;
    }
    float acc = 0.0f, cnt = 0.0f;
    for (int q = start[s]; q < start[s + 1]; ++q) {
        cnt += 1.0f;
        acc += var[order[q]];
    }
    keep[s] = (acc / cnt) <= thresh ? 1 : 0;
}

__global__ void k_var_paint(const int32_t* __restrict__ seg, size_t n, int max_seg, const int32_t* __restrict__ keep,
                            int32_t* __restrict__ out) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int32_t id = seg[k];
        out[k] = (id > 0 && id <= max_seg && keep[id]) ? id : 0;
    }
}

// ---------------------------------------------------- fusion_planar_mask --
// kind: 0 = left unlabelled, 1 = object (300), 2 = textureless (301 + rank),
// 3 = planar superpixel (its own id)
__global__ void k_planar_kind(const int32_t* __restrict__ planar, const float* __restrict__ normals,
                              const int32_t* __restrict__ start, const int32_t* __restrict__ order, int max_seg,
                              int thresh, float nonplanar_percent, float cos_sim_thresh, float match_ratio_thresh,
                              int32_t* __restrict__ kind) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > max_seg) return;
    if (s == 0) {
        kind[0] = 0;
        return;
    }
    const int b = start[s], e = start[s + 1];
    int npi = 0, pli = 0;
    for (int q = b; q < e; ++q) {
        if (planar[order[q]] == 0)
            ++npi;
        else
            ++pli;
    }
    const float np = (float)npi, pl = (float)pli;
    const float amount = np + pl;
    int k = 0;
    if (amount <= (float)thresh) {
        k = 0;
    } else if (np / amount >= nonplanar_percent) {
        float avg0 = 0.0f, avg1 = 0.0f, avg2 = 0.0f;
        for (int q = b; q < e; ++q) {
            const int i = order[q];
            if (planar[i] != 0) continue;
            avg0 += normals[(size_t)i * 3];
            avg1 += normals[(size_t)i * 3 + 1];
            avg2 += normals[(size_t)i * 3 + 2];
        }
        avg0 /= np;
        avg1 /= np;
        avg2 /= np;
        int valid = 0;
        for (int q = b; q < e; ++q) {
            const int i = order[q];
            if (planar[i] != 0) continue;
            const float cs =
                avg0 * normals[(size_t)i * 3] + avg1 * normals[(size_t)i * 3 + 1] + avg2 * normals[(size_t)i * 3 + 2];
            valid += cs > cos_sim_thresh ? 1 : 0;
        }
        k = ((float)valid / np > match_ratio_thresh) ? 3 : 1;
    } else if (np / amount < 0.25f) {
        k = 2;
    } else {
        k = 3;
    }
    kind[s] = k;
}

// labels in segment order: textureless segments count up from 301
__global__ void k_planar_labels(int32_t* __restrict__ kind, int ns) {
    __shared__ int32_t part[1024];
    const int t = threadIdx.x, T = blockDim.x;
    const int per = (ns + T - 1) / T;
    const int b = t * per, e = min(ns, b + per);
    int32_t c = 0;
    for (int i = b; i < e; ++i) c += kind[i] == 2;
    part[t] = c;
    __syncthreads();
    if (t == 0) {
        int32_t run = 0;
        for (int i = 0; i < T; ++i) {
            const int32_t v = part[i];
            part[i] = run;
            run += v;
        }
    }
    __syncthreads();
    int32_t vps = 301 + part[t];
    for (int i = b; i < e; ++i) {
        const int32_t k = kind[i];
        kind[i] = k == 1 ? 300 : (k == 2 ? vps++ : (k == 3 ? i : 0));
    }
}

__global__ void k_label_paint(const int32_t* __restrict__ seg, size_t n, int max_seg,
                              const int32_t* __restrict__ label, int32_t* __restrict__ out) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int32_t id = seg[k];
        out[k] = (id > 0 && id <= max_seg) ? label[id] : 0;
    }
}

// ------------------------------------------------- sliding_window_normal --
__global__ void k_window_normal(const int32_t* __restrict__ region, const float* __restrict__ normals, int rows,
                                int cols, int half, float* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (r >= rows || c >= cols) return;
    const size_t k = (size_t)r * cols + c;
    if (region[k] == 1) {
        out[k * 3] = out[k * 3 + 1] = out[k * 3 + 2] = 0.0f;
        return;
    }
    int valid = 0;
    float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
    for (int rr = max(0, r - half); rr < min(rows, r + half + 1); ++rr)
        for (int cc = max(0, c - half); cc < min(cols, c + half + 1); ++cc) {
            const size_t q = (size_t)rr * cols + cc;
            if (region[q] == 1) continue;
            ++valid;
            n0 += normals[q * 3];
            n1 += normals[q * 3 + 1];
            n2 += normals[q * 3 + 2];
        }
    const float v = (float)valid;
    out[k * 3] = n0 / v;
    out[k * 3 + 1] = n1 / v;
    out[k * 3 + 2] = n2 / v;
}

int32_t check_args(int rows, int cols, int max_seg, void* ws, size_t ws_bytes, const char* who) {
    if (rows < 1 || cols < 1) return fail(GMVS_ERR_INVALID, std::string(who) + ": empty image");
    if (max_seg < 0) return fail(GMVS_ERR_INVALID, std::string(who) + ": max_seg_id must be >= 0");
    const size_t need = seg_layout(rows, cols, max_seg).total + 256;
    if (!ws || ws_bytes < need)
        return fail(GMVS_ERR_WORKSPACE, std::string(who) + ": workspace too small: need " + std::to_string(need));
    if ((uintptr_t)ws % 256) return fail(GMVS_ERR_INVALID, std::string(who) + ": workspace must be 256-byte aligned");
    return GMVS_OK;
}

// Stable order of the pixels by segment; the error word lives in the last
// 256 bytes of the workspace.
int32_t build_order(const int32_t* seg, int rows, int cols, int max_seg, char* ws, const SegLayout& L,
                    cudaStream_t st) {
    int32_t* hist = (int32_t*)(ws + L.hist);
    int* err = (int*)(ws + L.total);
    const int ns = max_seg + 1;
    cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(int32_t) * (size_t)rows * ns, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), st);
    if (e != cudaSuccess) return fail_cuda(e, "segment workspace reset");
    k_row_hist<<<(rows + 127) / 128, 128, 0, st>>>(seg, rows, cols, max_seg, hist, err);
    k_col_scan<<<(ns + 127) / 128, 128, 0, st>>>(hist, rows, max_seg, (int32_t*)(ws + L.count));
    k_seg_scan<<<1, 1024, 0, st>>>((const int32_t*)(ws + L.count), ns, (int32_t*)(ws + L.start));
    k_row_scatter<<<(rows + 127) / 128, 128, 0, st>>>(seg, rows, cols, max_seg, hist, (const int32_t*)(ws + L.start),
                                                       (int32_t*)(ws + L.order));
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "segment order kernels");
    return GMVS_OK;
}

// read the error word (synchronises the stream)
int32_t seg_check(char* ws, const SegLayout& L, cudaStream_t st, const char* who) {
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, ws + L.total, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda(e, who);
    if (err) return fail(GMVS_ERR_INVALID, std::string(who) + ": a segment id is outside [0, max_seg_id]");
    return GMVS_OK;
}

int blocks_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 4096); }

}  // namespace
}  // namespace gmvs

extern "C" size_t gmvs_segments_workspace_bytes(int32_t rows, int32_t cols, int32_t max_seg_id) {
    if (rows < 1 || cols < 1 || max_seg_id < 0) return 0;
    return gmvs::seg_layout(rows, cols, max_seg_id).total + 256;
}

extern "C" int32_t gmvs_fusion_planar_mask_device(const int32_t* seg_ids, const int32_t* planar_mask,
                                                  const float* normals, int32_t rows, int32_t cols,
                                                  int32_t max_seg_id, int32_t thresh, float nonplanar_percent,
                                                  float cos_sim_thresh, float match_ratio_thresh, int32_t* out_mask,
                                                  void* workspace, size_t workspace_bytes, void* stream) {
    using namespace gmvs;
    const char* who = "gmvs_fusion_planar_mask_device";
    if (!seg_ids || !planar_mask || !normals || !out_mask) return fail(GMVS_ERR_INVALID, std::string(who) + ": NULL");
    int32_t rc = check_args(rows, cols, max_seg_id, workspace, workspace_bytes, who);
    if (rc != GMVS_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    char* ws = (char*)workspace;
    const SegLayout L = seg_layout(rows, cols, max_seg_id);
    rc = build_order(seg_ids, rows, cols, max_seg_id, ws, L, st);
    if (rc != GMVS_OK) return rc;
    const int ns = max_seg_id + 1;
    int32_t* kind = (int32_t*)(ws + L.kind);
    k_planar_kind<<<(ns + 127) / 128, 128, 0, st>>>(planar_mask, normals, (const int32_t*)(ws + L.start),
                                                     (const int32_t*)(ws + L.order), max_seg_id, thresh,
                                                     nonplanar_percent, cos_sim_thresh, match_ratio_thresh, kind);
    k_planar_labels<<<1, 1024, 0, st>>>(kind, ns);
    const size_t n = (size_t)rows * cols;
    k_label_paint<<<blocks_for(n), 256, 0, st>>>(seg_ids, n, max_seg_id, kind, out_mask);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, who);
    return seg_check(ws, L, st, who);
}

extern "C" int32_t gmvs_filter_by_var_map_device(const float* var_map, const int32_t* seg_ids, int32_t rows,
                                                 int32_t cols, int32_t max_seg_id, float var_thresh,
                                                 int32_t* out_ids, void* workspace, size_t workspace_bytes,
                                                 void* stream) {
    using namespace gmvs;
    const char* who = "gmvs_filter_by_var_map_device";
    if (!var_map || !seg_ids || !out_ids) return fail(GMVS_ERR_INVALID, std::string(who) + ": NULL");
    int32_t rc = check_args(rows, cols, max_seg_id, workspace, workspace_bytes, who);
    if (rc != GMVS_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    char* ws = (char*)workspace;
    const SegLayout L = seg_layout(rows, cols, max_seg_id);
    rc = build_order(seg_ids, rows, cols, max_seg_id, ws, L, st);
    if (rc != GMVS_OK) return rc;
    const int ns = max_seg_id + 1;
    int32_t* keep = (int32_t*)(ws + L.kind);
    k_var_keep<<<(ns + 127) / 128, 128, 0, st>>>(var_map, (const int32_t*)(ws + L.start),
                                                  (const int32_t*)(ws + L.order), max_seg_id, var_thresh, keep);
    const size_t n = (size_t)rows * cols;
    k_var_paint<<<blocks_for(n), 256, 0, st>>>(seg_ids, n, max_seg_id, keep, out_ids);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, who);
    return seg_check(ws, L, st, who);
}

extern "C" int32_t gmvs_sliding_window_normal_device(const int32_t* planar_region, const float* normals,
                                                     int32_t rows, int32_t cols, int32_t window_size,
                                                     float* out_normals, void* stream) {
    using namespace gmvs;
    if (!planar_region || !normals || !out_normals || rows < 1 || cols < 1)
        return fail(GMVS_ERR_INVALID, "gmvs_sliding_window_normal_device: NULL argument or empty image");
    if (window_size < 1) return fail(GMVS_ERR_INVALID, "gmvs_sliding_window_normal_device: window_size must be >= 1");
    const dim3 block(32, 8), grid((cols + 31) / 32, (rows + 7) / 8);
    k_window_normal<<<grid, block, 0, (cudaStream_t)stream>>>(planar_region, normals, rows, cols, window_size / 2,
                                                               out_normals);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "gmvs_sliding_window_normal_device");
    return GMVS_OK;
}
