// SPDX-License-Identifier: MIT
//
// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the planar-prior construction of module A
// (gmvs/lib/src/planar_initer.cu) and of its three CPU segmentation helpers.
//
// cv::Subdiv2D (planar_initer.cu:356-361) is replaced by a brute-force
// Bowyer-Watson Delaunay triangulation with exact integer predicates,
// inserting the support points in their generation order inside a fixed
// integer super-triangle; a triangle is discarded when it uses a
// super-triangle vertex.  Retained triangles are listed in a canonical order
// (vertex indices rotated so the smallest comes first, then sorted), which
// fixes the triangle ids written into the mask.  Delaunay triangulations of
// co-circular support points are not unique, so the triangles (and with them
// the prior) can differ from OpenCV's; the prior pass is compared with the
// reference statistically, and exactly against this restatement.
// The plane through three points is the normalised cross product, which is
// the null vector cv::SVD::solveZ returns up to sign (planar_initer.cu:700-745);
// the sign is then fixed exactly as the reference does.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Cam {
    float K[9];
    float R[9];
    float t[3];
    int32_t height;
    int32_t width;
    float depth_min;
    float depth_max;
};

typedef __int128 i128;

struct Pt {
    int64_t x, y;
};

// orientation of (a, b, c): > 0 counter-clockwise (y down image coords are
// treated as plain Cartesian coordinates).
inline int64_t orient(const Pt& a, const Pt& b, const Pt& c) {
    return (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
}

// > 0 when d lies strictly inside the circumcircle of the counter-clockwise
// triangle (a, b, c).
inline bool in_circle(const Pt& a, const Pt& b, const Pt& c, const Pt& d) {
    const i128 adx = a.x - d.x, ady = a.y - d.y;
    const i128 bdx = b.x - d.x, bdy = b.y - d.y;
    const i128 cdx = c.x - d.x, cdy = c.y - d.y;
    const i128 ad = adx * adx + ady * ady;
    const i128 bd = bdx * bdx + bdy * bdy;
    const i128 cd = cdx * cdx + cdy * cdy;
    const i128 det = adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx);
    return det > 0;
}

struct Tri {
    int v[3];
    bool alive;
};

// Brute-force Bowyer-Watson.  pts[0..n) are the input points; three super
// vertices are appended.  Returns triangles over input points only, in
// canonical order.
std::vector<std::array<int, 3>> delaunay_bw(const std::vector<Pt>& in, int64_t extent) {
    std::vector<Pt> pts = in;
    const int n = (int)in.size();
    const int64_t M = std::max<int64_t>(extent, 16) * 8;
    pts.push_back(Pt{-M, -M});
    pts.push_back(Pt{3 * M, -M});
    pts.push_back(Pt{-M, 3 * M});
    std::vector<Tri> tris;
    tris.push_back(Tri{{n, n + 1, n + 2}, true});
    if (orient(pts[n], pts[n + 1], pts[n + 2]) < 0) std::swap(tris[0].v[1], tris[0].v[2]);
    for (int p = 0; p < n; ++p) {
        std::vector<std::array<int, 2>> edges;
        for (auto& t : tris) {
            if (!t.alive) continue;
            if (in_circle(pts[t.v[0]], pts[t.v[1]], pts[t.v[2]], pts[p])) {
                t.alive = false;
                for (int e = 0; e < 3; ++e) edges.push_back({t.v[e], t.v[(e + 1) % 3]});
            }
        }
        // boundary edges = edges not shared (in opposite direction) by two bad triangles
        for (size_t i = 0; i < edges.size(); ++i) {
            bool shared = false;
            for (size_t j = 0; j < edges.size(); ++j)
                if (i != j && edges[i][0] == edges[j][1] && edges[i][1] == edges[j][0]) {
                    shared = true;
                    break;
                }
            if (!shared) {
                Tri t{{edges[i][0], edges[i][1], p}, true};
                if (orient(pts[t.v[0]], pts[t.v[1]], pts[t.v[2]]) == 0) continue;  // degenerate sliver
                tris.push_back(t);
            }
        }
        // compact occasionally
        if (tris.size() > 4 * (size_t)(p + 8)) {
            std::vector<Tri> keep;
            for (auto& t : tris)
                if (t.alive) keep.push_back(t);
            tris.swap(keep);
        }
    }
    std::vector<std::array<int, 3>> out;
    for (auto& t : tris) {
        if (!t.alive) continue;
        if (t.v[0] >= n || t.v[1] >= n || t.v[2] >= n) continue;
        int r = 0;
        if (t.v[1] < t.v[r]) r = 1;
        if (t.v[2] < t.v[r]) r = 2;
        out.push_back({t.v[r], t.v[(r + 1) % 3], t.v[(r + 2) % 3]});
    }
    std::sort(out.begin(), out.end());
    return out;
}

// PlanarInit::get_support_points (planar_initer.cu:225-256)
std::vector<Pt> support_points(int rows, int cols, const float* cost) {
    std::vector<Pt> sp;
    const int step = 5;
    for (int col = 0; col < cols; col += step) {
        for (int row = 0; row < rows; row += step) {
            float min_cost = 2.0f;
            int tx = 0, ty = 0;
            const int cb = std::min(cols, col + step), rb = std::min(rows, row + step);
            for (int c = col; c < cb; ++c)
                for (int r = row; r < rb; ++r) {
                    const float v = cost[r * cols + c];
                    if (v < 2.0f && min_cost > v) {
                        tx = c;
                        ty = r;
                        min_cost = v;
                    }
                }
            if (min_cost < 0.1f) sp.push_back(Pt{tx, ty});
        }
    }
    return sp;
}

// PlanarInit::get_3D_point_on_ref_cam (planar_initer.cu:686-698)
inline void ref_point(int x, int y, float depth, const Cam& c, double X[3]) {
    X[0] = (double)(depth * ((float)x - c.K[2]) / c.K[0]);
    X[1] = (double)(depth * ((float)y - c.K[5]) / c.K[4]);
    X[2] = (double)depth;
}

// get_prior_plane_params (planar_initer.cu:700-745): plane through three
// back-projected vertices, |n| = 1, w >= 0.
void prior_plane(const Pt tri[3], const float* depth, int cols, const Cam& c, float out[4]) {
    double X[3][3];
    for (int k = 0; k < 3; ++k)
        ref_point((int)tri[k].x, (int)tri[k].y, depth[tri[k].y * cols + tri[k].x], c, X[k]);
    const double e1[3] = {X[1][0] - X[0][0], X[1][1] - X[0][1], X[1][2] - X[0][2]};
    const double e2[3] = {X[2][0] - X[0][0], X[2][1] - X[0][1], X[2][2] - X[0][2]};
    double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    double d = -(n[0] * X[0][0] + n[1] * X[0][1] + n[2] * X[0][2]);
    double norm = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (d < 0) norm = -norm;
    out[0] = (float)(n[0] / norm);
    out[1] = (float)(n[1] / norm);
    out[2] = (float)(n[2] / norm);
    out[3] = (float)(d / norm);
}

// PlanarInit::get_depth_from_plane_param (planar_initer.cu:279-286)
inline float depth_from_prior(const float* pl, int x, int y, const Cam& c) {
    return -pl[3] / (((float)x - c.K[2]) * pl[0] / c.K[0] + ((float)y - c.K[5]) * pl[1] / c.K[4] + pl[2]);
}

// barycentric stepping shared by the superpixel filter and process_mask
// (planar_initer.cu:310-327 and 377-401); visit(x, y) returns false to stop.
template <class F>
void raster_triangle(const Pt& a, const Pt& b, const Pt& c, F visit) {
    const float L01 = (float)std::sqrt(std::pow((double)(a.x - b.x), 2) + std::pow((double)(a.y - b.y), 2));
    const float L02 = (float)std::sqrt(std::pow((double)(a.x - c.x), 2) + std::pow((double)(a.y - c.y), 2));
    const float L12 = (float)std::sqrt(std::pow((double)(b.x - c.x), 2) + std::pow((double)(b.y - c.y), 2));
    const float mel = std::max(L01, std::max(L02, L12));
    const float step = (float)(1.0 / mel);
    for (float p = 0; p < 1.0; p += step) {
        for (float q = 0; q < 1.0 - p; q += step) {
            const int x = (int)(p * a.x + q * b.x + (1.0 - p - q) * c.x);
            const int y = (int)(p * a.y + q * b.y + (1.0 - p - q) * c.y);
            if (!visit(x, y)) return;
        }
    }
}

}  // namespace

extern "C" {

// PlanarInit::triangulation + process_mask + cuda_planar_prior_init
// (planar_initer.cu:347-420, 288-345, 195-223).  out_planes: float4 [H][W]
// (0 where mask == 0), out_masks: [H][W] triangle id + 1.  out_tris (3 ints
// per retained triangle, up to max_tris) lists the retained triangles as
// vertex coordinates x0 y0 x1 y1 x2 y2 when non-null (6 ints each).
int oracle_build_prior(const Cam* cam, int rows, int cols, const float* depth, const float* cost,
                       const uint8_t* superpixel, int superpixel_filter, float depth_min, float depth_max,
                       float* out_planes, uint32_t* out_masks, int32_t* out_tri_count, int32_t* out_tris,
                       int32_t max_tris) {
    const std::vector<Pt> sp = support_points(rows, cols, cost);
    std::vector<std::array<int, 3>> tl = delaunay_bw(sp, std::max(rows, cols));
    std::vector<std::array<Pt, 3>> kept;
    const float zero_ratio_thresh = 0.1f;
    for (const auto& t : tl) {
        const Pt a = sp[t[0]], b = sp[t[1]], c = sp[t[2]];
        bool retain = true;
        if (superpixel_filter) {
            float count = 0.0f, zero_count = 0.0f;
            uint8_t seg = 0;
            raster_triangle(a, b, c, [&](int x, int y) {
                const uint8_t s = superpixel[y * cols + x];
                count += 1.0f;
                if (s == 0) zero_count += 1.0f;
                if (seg == 0)
                    seg = s;
                else if (s == 0)
                    return true;
                else if (s != seg) {
                    retain = false;
                    return false;
                }
                return true;
            });
            if (zero_count / count > zero_ratio_thresh) retain = false;
        }
        if (retain) kept.push_back({a, b, c});
    }
    // process_mask: later triangles overwrite earlier ones
    std::vector<float> mask((size_t)rows * cols, 0.0f);
    std::vector<std::array<float, 4>> planes;
    uint32_t idx = 0;
    for (const auto& t : kept) {
        raster_triangle(t[0], t[1], t[2], [&](int x, int y) {
            mask[(size_t)y * cols + x] = (float)(idx + 1.0);
            return true;
        });
        std::array<float, 4> pl;
        prior_plane(t.data(), depth, cols, *cam, pl.data());
        planes.push_back(pl);
        idx++;
    }
    for (int i = 0; i < cols; ++i)
        for (int j = 0; j < rows; ++j) {
            const size_t k = (size_t)j * cols + i;
            if (mask[k] > 0) {
                const float d = depth_from_prior(planes[(size_t)mask[k] - 1].data(), i, j, *cam);
                if (!(d <= depth_max && d >= depth_min)) mask[k] = 0;
            }
        }
    for (size_t k = 0; k < (size_t)rows * cols; ++k) {
        out_masks[k] = (uint32_t)mask[k];
        for (int e = 0; e < 4; ++e) out_planes[k * 4 + e] = mask[k] > 0 ? planes[(size_t)mask[k] - 1][e] : 0.0f;
    }
    if (out_tri_count) *out_tri_count = (int32_t)kept.size();
    if (out_tris)
        for (int32_t i = 0; i < (int32_t)kept.size() && i < max_tris; ++i)
            for (int e = 0; e < 3; ++e) {
                out_tris[i * 6 + e * 2 + 0] = (int32_t)kept[i][e].x;
                out_tris[i * 6 + e * 2 + 1] = (int32_t)kept[i][e].y;
            }
    return 0;
}

// Delaunay triangles (canonical order) of integer points, for the
// triangulation tests.  Returns the number of triangles (writes up to
// max_tris triples of point indices).
int oracle_delaunay(const int32_t* xy, int n, int extent, int32_t* out, int max_tris) {
    std::vector<Pt> pts(n);
    for (int i = 0; i < n; ++i) pts[i] = Pt{xy[2 * i], xy[2 * i + 1]};
    auto t = delaunay_bw(pts, extent);
    for (int i = 0; i < (int)t.size() && i < max_tris; ++i)
        for (int e = 0; e < 3; ++e) out[i * 3 + e] = t[i][e];
    return (int)t.size();
}

// fusion_planar_mask (planar_initer.cu:537-632)
int oracle_fusion_planar_mask(const int32_t* seg_ids, const int32_t* planar_mask, const float* normals, int rows,
                              int cols, int thresh, float nonplanar_percent, float cos_sim_thresh,
                              float match_ratio_thresh, int32_t* out) {
    int32_t max_val = seg_ids[0];
    for (int i = 1; i < rows * cols; ++i) max_val = std::max(max_val, seg_ids[i]);
    const uint32_t nseg = (uint32_t)max_val + 1;
    std::vector<std::vector<std::array<float, 3>>> seg_normals(nseg);
    std::vector<std::vector<int>> seg_map(nseg);
    std::vector<std::array<int, 2>> cnt(nseg, {0, 0});
    for (int r = 0; r < rows; ++r)
        for (int c = 0; c < cols; ++c) {
            const int k = r * cols + c;
            const int s = seg_ids[k];
            seg_map[s].push_back(k);
            if (planar_mask[k] == 0) {
                ++cnt[s][0];
                seg_normals[s].push_back({normals[k * 3], normals[k * 3 + 1], normals[k * 3 + 2]});
            } else {
                ++cnt[s][1];
            }
        }
    std::memset(out, 0, sizeof(int32_t) * rows * cols);
    uint32_t vps = 301;
    for (int s = 1; s < (int)nseg; ++s) {
        const float nonplanar = (float)cnt[s][0];
        const float planar = (float)cnt[s][1];
        const float amount = nonplanar + planar;
        if (amount <= thresh) continue;
        bool skip = false;
        if (nonplanar / amount >= nonplanar_percent) {
            skip = true;
            float avg[3] = {0, 0, 0};
            for (auto& n : seg_normals[s])
                for (int e = 0; e < 3; ++e) avg[e] += n[e];
            for (int e = 0; e < 3; ++e) avg[e] /= nonplanar;
            int valid = 0;
            for (auto& n : seg_normals[s]) {
                const float cs = avg[0] * n[0] + avg[1] * n[1] + avg[2] * n[2];
                valid += cs > cos_sim_thresh ? 1 : 0;
            }
            const float ratio = (float)valid / nonplanar;
            if (ratio > match_ratio_thresh)
                skip = false;
            else
                for (int k : seg_map[s]) out[k] = 300;
        } else if (nonplanar / amount < 0.25f) {
            for (int k : seg_map[s]) out[k] = (int32_t)vps;
            vps += 1;
            skip = true;
        }
        if (skip) continue;
        for (int k : seg_map[s]) out[k] = s;
    }
    return 0;
}

// filter_by_var_map (planar_initer.cu:634-684)
int oracle_filter_by_var_map(const float* var_map, const int32_t* seg, int rows, int cols, float var_thresh,
                             int32_t* out) {
    int32_t max_val = seg[0];
    for (int i = 1; i < rows * cols; ++i) max_val = std::max(max_val, seg[i]);
    std::vector<float> acc(max_val + 1, 0.0f), count(max_val + 1, 0.0f);
    std::vector<char> keep(max_val + 1, 0);
    for (int k = 0; k < rows * cols; ++k) {
        if (seg[k] == 0) continue;
        ++count[seg[k]];
        acc[seg[k]] += var_map[k];
    }
    for (int s = 1; s < max_val + 1; ++s) keep[s] = (acc[s] / count[s]) <= var_thresh;
    for (int k = 0; k < rows * cols; ++k) out[k] = keep[seg[k]] ? seg[k] : 0;
    return 0;
}

// sliding_window_normal host loop (planar_initer.cu:471-535)
int oracle_sliding_window_normal(const int32_t* region, const float* normals, int rows, int cols, int win,
                                 float* out) {
    const int h = win / 2;
    for (int r = 0; r < rows; ++r)
        for (int c = 0; c < cols; ++c) {
            const int k = r * cols + c;
            if (region[k] == 1) {
                out[k * 3] = out[k * 3 + 1] = out[k * 3 + 2] = 0.0f;
                continue;
            }
            int valid = 0;
            float n[3] = {0, 0, 0};
            for (int rr = r - h; rr < r + h + 1; ++rr)
                for (int cc = c - h; cc < c + h + 1; ++cc) {
                    if (rr < 0 || rr >= rows || cc < 0 || cc >= cols) continue;
                    if (region[rr * cols + cc] == 1) continue;
                    ++valid;
                    for (int e = 0; e < 3; ++e) n[e] += normals[(rr * cols + cc) * 3 + e];
                }
            for (int e = 0; e < 3; ++e) out[k * 3 + e] = n[e] / (float)valid;
        }
    return 0;
}

}  // extern "C"
