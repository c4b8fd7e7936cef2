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

// endpoints of every edge, in edge order (no divisions in the merge loops)
void edge_ends(int rows, int cols, std::vector<int32_t>& ea, std::vector<int32_t>& eb) {
    int64_t e = 0;
    for (int y = 0; y < rows; ++y)  // right
        for (int x = 0; x + 1 < cols; ++x, ++e) ea[e] = y * cols + x, eb[e] = y * cols + x + 1;
    for (int y = 0; y + 1 < rows; ++y)  // down
        for (int x = 0; x < cols; ++x, ++e) ea[e] = y * cols + x, eb[e] = (y + 1) * cols + x;
    for (int y = 0; y + 1 < rows; ++y)  // down-right
        for (int x = 0; x + 1 < cols; ++x, ++e) ea[e] = y * cols + x, eb[e] = (y + 1) * cols + x + 1;
    for (int y = 0; y + 1 < rows; ++y)  // up-right
        for (int x = 0; x + 1 < cols; ++x, ++e) ea[e] = y * cols + x + 1, eb[e] = (y + 1) * cols + x;
}

// stable ascending order of non-negative doubles: LSD radix sort with 8-bit
// digits (256 buckets keep the scatter cache-friendly); a pass whose digit
// is the same for every key is skipped
std::vector<uint32_t> sort_edges(const double* w, int64_t n) {
    std::vector<uint64_t> key(n), key2(n);
    std::vector<uint32_t> idx(n), idx2(n);
    for (int64_t i = 0; i < n; ++i) {
        std::memcpy(&key[i], &w[i], 8);
        idx[i] = (uint32_t)i;
    }
    int64_t count[8][257] = {};
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 8; ++d) ++count[d][((key[i] >> (8 * d)) & 0xff) + 1];
    for (int d = 0; d < 8; ++d) {
        int64_t* c = count[d];
        bool trivial = false;
        for (int k = 1; k <= 256; ++k) {
            if (c[k] == n) trivial = true;
            c[k] += c[k - 1];
        }
        if (trivial) continue;  // every key has the same digit: the order stands
        const int sh = 8 * d;
        for (int64_t i = 0; i < n; ++i) {
            const int64_t at = c[(key[i] >> sh) & 0xff]++;
            key2[at] = key[i];
            idx2[at] = idx[i];
        }
        key.swap(key2);
        idx.swap(idx2);
    }
    return idx;
}

// one 16-byte node per pixel: a find and the size / inner-cost test that
// follows touch one cache line
struct Node {
    int32_t parent, size;
    double inner;
};

struct Forest {
    std::vector<Node> node;
    explicit Forest(int32_t n) : node(n) {
        for (int32_t i = 0; i < n; ++i) node[i] = Node{i, 1, 0.0};
    }
    int32_t find(int32_t a) {
        int32_t r = a;
        while (node[r].parent != r) r = node[r].parent;
        while (node[a].parent != r) {
            const int32_t nx = node[a].parent;
            node[a].parent = r;
            a = nx;
        }
        return r;
    }
    int32_t join(int32_t a, int32_t b) {
        const int32_t r = std::min(a, b);
        const int32_t s = node[a].size + node[b].size;
        node[a].parent = node[b].parent = r;
        node[r].size = s;
        return r;
    }
};

}  // namespace

int32_t superpixel_merge_sorted(int rows, int cols, int64_t ne, const int32_t* sa, const int32_t* sb,
                                const double* sw, double k, int min_size, int32_t* labels) {
    const int32_t n = rows * cols;
    Forest f(n);
    for (int64_t i = 0; i < ne; ++i) {
        const int32_t a = f.find(sa[i]), b = f.find(sb[i]);
        if (a == b) continue;
        const double ta = f.node[a].inner + k / (double)f.node[a].size;
        const double tb = f.node[b].inner + k / (double)f.node[b].size;
        if (sw[i] < std::min(ta, tb)) f.node[f.join(a, b)].inner = sw[i];
    }
    for (int64_t i = 0; i < ne; ++i) {
        const int32_t a = f.find(sa[i]), b = f.find(sb[i]);
        if (a == b) continue;
        if (f.node[a].size < min_size || f.node[b].size < min_size) f.join(a, b);
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

int32_t superpixel_labels(int rows, int cols, const double* weights, double k, int min_size, int32_t* labels) {
    const int64_t ne = (int64_t)rows * (cols - 1) + (int64_t)(rows - 1) * cols + 2LL * (rows - 1) * (cols - 1);
    const std::vector<uint32_t> order = sort_edges(weights, ne);
    // endpoints and weights in visiting order: both passes stream them
    std::vector<int32_t> ea(ne), eb(ne), sa(ne), sb(ne);
    std::vector<double> sw(ne);
    edge_ends(rows, cols, ea, eb);
    for (int64_t i = 0; i < ne; ++i) {
        const uint32_t e = order[i];
        sa[i] = ea[e], sb[i] = eb[e], sw[i] = weights[e];
    }
    return superpixel_merge_sorted(rows, cols, ne, sa.data(), sb.data(), sw.data(), k, min_size, labels);
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
