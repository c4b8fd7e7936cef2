// Host half of the superpixel extraction: the Felzenszwalb-Huttenlocher
// merge (IJCV 2004) as scikit-image's segmentation.felzenszwalb
// parameterises it, which extract_superpixel.py:62 calls, followed by the
// script's size filter (extract_superpixel.py:64-71).  The merge is a
// sequential scan of the edges in ascending weight (each decision depends
// on every earlier one), so it runs here on one core between the device
// stages that form the edge weights and paint the full-size labels.
//
// Edges of the 8-connected rows x cols grid, in the order of the weights
// the device writes: right (p, p+1), down (p, p+cols), down-right
// (p, p+cols+1), up-right (p+1, p+cols), each group in raster order of p.
// Edges are visited by ascending weight; equal weights keep that order (a
// stable LSD radix sort on the IEEE bit patterns, which order non-negative
// doubles like their values).  A component is rooted at its smallest pixel
// index, so the final numbering by root is the numbering by each
// component's first pixel in raster order.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gmvs_gb300.h"
#include "superpixel.h"

namespace gmvs {

int32_t fail(int32_t code, const std::string& msg);

namespace {

void edge_ends(int rows, int cols, int64_t e, int32_t& a, int32_t& b) {
    const int64_t nr = (int64_t)rows * (cols - 1), nd = (int64_t)(rows - 1) * cols,
                  ng = (int64_t)(rows - 1) * (cols - 1);
    if (e < nr) {
        const int64_t y = e / (cols - 1), x = e % (cols - 1), p = y * cols + x;
        a = (int32_t)p, b = (int32_t)(p + 1);
        return;
    }
    e -= nr;
    if (e < nd) {
        a = (int32_t)e, b = (int32_t)(e + cols);
        return;
    }
    e -= nd;
    const bool up = e >= ng;
    if (up) e -= ng;
    const int64_t y = e / (cols - 1), x = e % (cols - 1), p = y * cols + x;
    if (!up)
        a = (int32_t)p, b = (int32_t)(p + cols + 1);
    else
        a = (int32_t)(p + 1), b = (int32_t)(p + cols);
}

// stable ascending order of non-negative doubles: 4 passes of 16-bit digits
std::vector<uint32_t> sort_edges(const double* w, int64_t n) {
    std::vector<uint64_t> key(n), key2(n);
    std::vector<uint32_t> idx(n), idx2(n);
    for (int64_t i = 0; i < n; ++i) {
        std::memcpy(&key[i], &w[i], 8);
        idx[i] = (uint32_t)i;
    }
    std::vector<int64_t> count(65537);
    for (int pass = 0; pass < 4; ++pass) {
        const int sh = 16 * pass;
        std::fill(count.begin(), count.end(), 0);
        for (int64_t i = 0; i < n; ++i) ++count[((key[i] >> sh) & 0xffff) + 1];
        bool trivial = false;
        for (int d = 1; d <= 65536; ++d) {
            if (count[d] == n) trivial = true;
            count[d] += count[d - 1];
        }
        if (trivial) continue;  // every key has the same digit: the order stands
        for (int64_t i = 0; i < n; ++i) {
            const int64_t at = count[(key[i] >> sh) & 0xffff]++;
            key2[at] = key[i];
            idx2[at] = idx[i];
        }
        key.swap(key2);
        idx.swap(idx2);
    }
    return idx;
}

struct Forest {
    std::vector<int32_t> parent, size;
    std::vector<double> inner;
    explicit Forest(int32_t n) : parent(n), size(n, 1), inner(n, 0.0) {
        for (int32_t i = 0; i < n; ++i) parent[i] = i;
    }
    int32_t find(int32_t a) {
        int32_t r = a;
        while (parent[r] != r) r = parent[r];
        while (parent[a] != r) {
            const int32_t nx = parent[a];
            parent[a] = r;
            a = nx;
        }
        return r;
    }
    int32_t join(int32_t a, int32_t b) {
        const int32_t r = std::min(a, b);
        const int32_t s = size[a] + size[b];
        parent[a] = parent[b] = r;
        size[r] = s;
        return r;
    }
};

}  // namespace

int32_t superpixel_labels(int rows, int cols, const double* weights, double k, int min_size, int32_t* labels) {
    const int32_t n = rows * cols;
    const int64_t ne = (int64_t)rows * (cols - 1) + (int64_t)(rows - 1) * cols + 2LL * (rows - 1) * (cols - 1);
    const std::vector<uint32_t> order = sort_edges(weights, ne);
    Forest f(n);
    for (int64_t i = 0; i < ne; ++i) {
        int32_t a, b;
        edge_ends(rows, cols, order[i], a, b);
        a = f.find(a), b = f.find(b);
        if (a == b) continue;
        const double w = weights[order[i]];
        const double ta = f.inner[a] + k / (double)f.size[a];
        const double tb = f.inner[b] + k / (double)f.size[b];
        if (w < std::min(ta, tb)) f.inner[f.join(a, b)] = w;
    }
    for (int64_t i = 0; i < ne; ++i) {
        int32_t a, b;
        edge_ends(rows, cols, order[i], a, b);
        a = f.find(a), b = f.find(b);
        if (a == b) continue;
        if (f.size[a] < min_size || f.size[b] < min_size) f.join(a, b);
    }
    // labels by root order, then the size filter: label 0 stays 0, every
    // other label with more than rows * cols / 128 pixels is renumbered
    // 1, 2, ... in label order, the rest become 0
    std::vector<int32_t> rank(n, -1);
    int32_t nl = 0;
    for (int32_t i = 0; i < n; ++i)
        if (f.find(i) == i) rank[i] = nl++;
    std::vector<int64_t> count(nl, 0);
    for (int32_t i = 0; i < n; ++i) {
        labels[i] = rank[f.find(i)];
        ++count[labels[i]];
    }
    std::vector<int32_t> keep(nl, 0);
    int32_t kept = 0;
    for (int32_t l = 1; l < nl; ++l)
        if (count[l] * 128 > (int64_t)n) keep[l] = ++kept;
    for (int32_t i = 0; i < n; ++i) labels[i] = keep[labels[i]];
    return kept;
}

}  // namespace gmvs

extern "C" int32_t gmvs_superpixel_labels_host(int32_t rows, int32_t cols, const double* weights, double scale,
                                               int32_t min_size, int32_t* labels, int32_t* out_num_segments) {
    if (!weights || !labels || rows < 1 || cols < 1 || (int64_t)rows * cols > (1LL << 26))
        return gmvs::fail(GMVS_ERR_INVALID, "gmvs_superpixel_labels_host: NULL argument or size out of range");
    if (!(scale >= 0.0) || min_size < 0)
        return gmvs::fail(GMVS_ERR_INVALID, "gmvs_superpixel_labels_host: scale and min_size must be >= 0");
    const int64_t ne = (int64_t)rows * (cols - 1) + (int64_t)(rows - 1) * cols + 2LL * (rows - 1) * (cols - 1);
    for (int64_t i = 0; i < ne; ++i)
        if (!(weights[i] >= 0.0))
            return gmvs::fail(GMVS_ERR_INVALID, "gmvs_superpixel_labels_host: weights must be >= 0 and not NaN");
    const int32_t kept = gmvs::superpixel_labels(rows, cols, weights, scale / 255.0, min_size, labels);
    if (out_num_segments) *out_num_segments = kept;
    return GMVS_OK;
}
