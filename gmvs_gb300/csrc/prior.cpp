// Host (CPU) part of module A: the planar prior built from a depth/cost map
// (PlanarInit::triangulation / process_mask / get_prior_plane_params /
// cuda_planar_prior_init, planar_initer.cu:195-420, 686-745) and the three
// CPU segmentation helpers (planar_initer.cu:471-684).
//
// cv::Subdiv2D is replaced by an incremental Delaunay triangulation
// (Bowyer-Watson with a visibility walk for point location and a
// breadth-first conflict region) using exact integer predicates.  Points are
// inserted in support-point order inside a fixed integer super-triangle and
// a point strictly inside a circumcircle conflicts, so the triangulation is
// fully determined by the input: co-circular support points (frequent on the
// 5-pixel support grid) are resolved by insertion order.  Triangles are
// reported with their smallest vertex index first, sorted.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gmvs_gb300.h"

namespace gmvs {
int32_t fail(int32_t code, const std::string& msg);
}

namespace {

typedef __int128 i128;

struct P2 {
    int64_t x, y;
};

inline int64_t orient2(const P2& a, const P2& b, const P2& c) {
    return (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
}

inline bool incircle(const P2& a, const P2& b, const P2& c, const P2& d) {
    const i128 adx = a.x - d.x, ady = a.y - d.y;
    const i128 bdx = b.x - d.x, bdy = b.y - d.y;
    const i128 cdx = c.x - d.x, cdy = c.y - d.y;
    const i128 ad = adx * adx + ady * ady;
    const i128 bd = bdx * bdx + bdy * bdy;
    const i128 cd = cdx * cdx + cdy * cdy;
    return adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx) > 0;
}

class Delaunay {
   public:
    // v[i]: counter-clockwise vertices; nb[i]: triangle across the edge
    // opposite v[i] (v[(i+1)%3] -> v[(i+2)%3]), -1 on the hull.
    struct Tri {
        int v[3];
        int nb[3];
        bool alive;
    };

    Delaunay(const std::vector<P2>& in, int64_t extent) : pts_(in), n_((int)in.size()) {
        const int64_t M = std::max<int64_t>(extent, 16) * 8;
        pts_.push_back(P2{-M, -M});
        pts_.push_back(P2{3 * M, -M});
        pts_.push_back(P2{-M, 3 * M});
        Tri t{{n_, n_ + 1, n_ + 2}, {-1, -1, -1}, true};
        if (orient2(pts_[n_], pts_[n_ + 1], pts_[n_ + 2]) < 0) std::swap(t.v[1], t.v[2]);
        tris_.push_back(t);
        mark_.push_back(0);
        for (int p = 0; p < n_; ++p) insert(p);
    }

    std::vector<std::array<int, 3>> triangles() const {
        std::vector<std::array<int, 3>> out;
        for (const Tri& t : tris_) {
            if (!t.alive || t.v[0] >= n_ || t.v[1] >= n_ || t.v[2] >= n_) continue;
            int r = 0;
            if (t.v[1] < t.v[r]) r = 1;
            if (t.v[2] < t.v[r]) r = 2;
            out.push_back({t.v[r], t.v[(r + 1) % 3], t.v[(r + 2) % 3]});
        }
        std::sort(out.begin(), out.end());
        return out;
    }

   private:
    std::vector<P2> pts_;
    int n_;
    std::vector<Tri> tris_;
    std::vector<int> mark_;
    int stamp_ = 0;
    int last_ = 0;
    std::vector<int> free_;

    int locate(const P2& p) {
        int t = last_;
        if (!tris_[t].alive) {
            for (t = (int)tris_.size() - 1; t >= 0 && !tris_[t].alive; --t) {
            }
        }
        for (size_t guard = 0; guard < 4 * tris_.size() + 16; ++guard) {
            const Tri& T = tris_[t];
            int next = -1;
            for (int i = 0; i < 3; ++i) {
                if (orient2(pts_[T.v[(i + 1) % 3]], pts_[T.v[(i + 2) % 3]], p) < 0) {
                    next = T.nb[i];
                    break;
                }
            }
            if (next < 0) return t;
            t = next;
        }
        // fall back to a scan (walks terminate on Delaunay meshes)
        for (int k = 0; k < (int)tris_.size(); ++k) {
            const Tri& T = tris_[k];
            if (!T.alive) continue;
            bool in = true;
            for (int i = 0; i < 3; ++i)
                if (orient2(pts_[T.v[(i + 1) % 3]], pts_[T.v[(i + 2) % 3]], p) < 0) in = false;
            if (in) return k;
        }
        return t;
    }

    void insert(int p) {
        const P2& P = pts_[p];
        const int t0 = locate(P);
        ++stamp_;
        std::vector<int> cav{t0}, stack{t0};
        mark_[t0] = stamp_;
        while (!stack.empty()) {
            const int t = stack.back();
            stack.pop_back();
            for (int i = 0; i < 3; ++i) {
                const int nb = tris_[t].nb[i];
                if (nb < 0 || mark_[nb] == stamp_) continue;
                const Tri& N = tris_[nb];
                if (incircle(pts_[N.v[0]], pts_[N.v[1]], pts_[N.v[2]], P)) {
                    mark_[nb] = stamp_;
                    cav.push_back(nb);
                    stack.push_back(nb);
                }
            }
        }
        // boundary edges (a -> b) with the outside neighbour
        struct Edge {
            int a, b, out;
        };
        std::vector<Edge> bnd;
        for (int t : cav) {
            const Tri& T = tris_[t];
            for (int i = 0; i < 3; ++i) {
                const int nb = T.nb[i];
                if (nb >= 0 && mark_[nb] == stamp_) continue;
                bnd.push_back(Edge{T.v[(i + 1) % 3], T.v[(i + 2) % 3], nb});
            }
        }
        for (int t : cav) {
            tris_[t].alive = false;
            free_.push_back(t);
        }
        // new fan (a, b, p); link across (a, b) to the outside neighbour
        std::vector<int> made(bnd.size());
        std::vector<std::pair<int, int>> by_a;  // vertex a -> new triangle
        for (size_t k = 0; k < bnd.size(); ++k) {
            const Edge& E = bnd[k];
            Tri t{{E.a, E.b, p}, {-1, -1, E.out}, true};
            int id;
            if (!free_.empty()) {
                id = free_.back();
                free_.pop_back();
                tris_[id] = t;
            } else {
                id = (int)tris_.size();
                tris_.push_back(t);
                mark_.push_back(0);
            }
            made[k] = id;
            if (E.out >= 0) {
                Tri& O = tris_[E.out];
                for (int i = 0; i < 3; ++i)
                    if (O.v[(i + 1) % 3] == E.b && O.v[(i + 2) % 3] == E.a) O.nb[i] = id;
            }
            by_a.push_back({E.a, id});
        }
        std::sort(by_a.begin(), by_a.end());
        auto find_a = [&](int a) {
            auto it = std::lower_bound(by_a.begin(), by_a.end(), std::make_pair(a, -1));
            return (it != by_a.end() && it->first == a) ? it->second : -1;
        };
        for (size_t k = 0; k < bnd.size(); ++k) {
            Tri& T = tris_[made[k]];
            // edge opposite v[0]=a is (b, p): neighbour is the new triangle starting at b
            T.nb[0] = find_a(T.v[1]);
            // edge opposite v[1]=b is (p, a): neighbour is the new triangle ending at a
        }
        for (size_t k = 0; k < bnd.size(); ++k) {
            Tri& T = tris_[made[k]];
            const int nb = T.nb[0];
            if (nb >= 0) tris_[nb].nb[1] = made[k];
        }
        last_ = made.empty() ? last_ : made[0];
    }
};

std::vector<P2> support_points(int rows, int cols, const float* cost) {
    std::vector<P2> sp;
    const int step = 5;
    for (int col = 0; col < cols; col += step)
        for (int row = 0; row < rows; row += step) {
            float min_cost = 2.0f;
            int tx = 0, ty = 0;
            const int cb = std::min(cols, col + step), rb = std::min(rows, row + step);
            for (int c = col; c < cb; ++c)
                for (int r = row; r < rb; ++r) {
                    const float v = cost[(size_t)r * cols + c];
                    if (v < 2.0f && min_cost > v) {
                        tx = c;
                        ty = r;
                        min_cost = v;
                    }
                }
            if (min_cost < 0.1f) sp.push_back(P2{tx, ty});
        }
    return sp;
}

template <class F>
void raster(const P2& a, const P2& b, const P2& c, F visit) {
    const float L01 = (float)std::sqrt(std::pow((double)(a.x - b.x), 2) + std::pow((double)(a.y - b.y), 2));
    const float L02 = (float)std::sqrt(std::pow((double)(a.x - c.x), 2) + std::pow((double)(a.y - c.y), 2));
    const float L12 = (float)std::sqrt(std::pow((double)(b.x - c.x), 2) + std::pow((double)(b.y - c.y), 2));
    const float mel = std::max(L01, std::max(L02, L12));
    const float step = (float)(1.0 / mel);
    for (float p = 0; p < 1.0; p += step)
        for (float q = 0; q < 1.0 - p; q += step) {
            const int x = (int)(p * a.x + q * b.x + (1.0 - p - q) * c.x);
            const int y = (int)(p * a.y + q * b.y + (1.0 - p - q) * c.y);
            if (!visit(x, y)) return;
        }
}

void plane_of(const P2 t[3], const float* depth, int cols, const gmvs_camera& c, float out[4]) {
    double X[3][3];
    for (int k = 0; k < 3; ++k) {
        const float d = depth[t[k].y * cols + t[k].x];
        X[k][0] = (double)(d * ((float)t[k].x - c.K[2]) / c.K[0]);
        X[k][1] = (double)(d * ((float)t[k].y - c.K[5]) / c.K[4]);
        X[k][2] = (double)d;
    }
    const double e1[3] = {X[1][0] - X[0][0], X[1][1] - X[0][1], X[1][2] - X[0][2]};
    const double e2[3] = {X[2][0] - X[0][0], X[2][1] - X[0][1], X[2][2] - X[0][2]};
    const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const double d = -(n[0] * X[0][0] + n[1] * X[0][1] + n[2] * X[0][2]);
    double norm = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (d < 0) norm = -norm;
    for (int k = 0; k < 3; ++k) out[k] = (float)(n[k] / norm);
    out[3] = (float)(d / norm);
}

}  // namespace

extern "C" int32_t gmvs_build_planar_prior(const gmvs_camera* cam, int32_t rows, int32_t cols, const float* depth,
                                           const float* cost, const uint8_t* superpixel, int32_t superpixel_filter,
                                           float depth_min, float depth_max, float* out_planes, uint32_t* out_masks,
                                           int32_t* out_tri_count, int32_t* out_tris, int32_t max_tris) {
    if (!cam || !depth || !cost || !out_planes || !out_masks || rows < 1 || cols < 1)
        return gmvs::fail(GMVS_ERR_INVALID, "gmvs_build_planar_prior: NULL argument or empty image");
    if (superpixel_filter && !superpixel)
        return gmvs::fail(GMVS_ERR_INVALID, "gmvs_build_planar_prior: superpixel filter without superpixels");
    const std::vector<P2> sp = support_points(rows, cols, cost);
    const Delaunay dt(sp, std::max(rows, cols));
    const auto tl = dt.triangles();
    std::vector<std::array<P2, 3>> kept;
    kept.reserve(tl.size());
    for (const auto& t : tl) {
        const P2 a = sp[t[0]], b = sp[t[1]], c = sp[t[2]];
        bool retain = true;
        if (superpixel_filter) {  // planar_initer.cu:370-406
            float count = 0.0f, zero = 0.0f;
            uint8_t seg = 0;
            raster(a, b, c, [&](int x, int y) {
                const uint8_t s = superpixel[(size_t)y * cols + x];
                count += 1.0f;
                if (s == 0) zero += 1.0f;
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
            if (zero / count > 0.1f) retain = false;
        }
        if (retain) kept.push_back({a, b, c});
    }
    // process_mask (planar_initer.cu:288-345): later triangles overwrite
    std::vector<uint32_t> mask((size_t)rows * cols, 0u);
    std::vector<std::array<float, 4>> planes(kept.size());
    for (size_t i = 0; i < kept.size(); ++i) {
        const uint32_t id = (uint32_t)i + 1;
        raster(kept[i][0], kept[i][1], kept[i][2], [&](int x, int y) {
            mask[(size_t)y * cols + x] = id;
            return true;
        });
        plane_of(kept[i].data(), depth, cols, *cam, planes[i].data());
    }
    for (size_t k = 0; k < (size_t)rows * cols; ++k) {
        float* o = out_planes + k * 4;
        if (mask[k] > 0) {
            const int i = (int)(k % cols), j = (int)(k / cols);
            const float* pl = planes[mask[k] - 1].data();
            // get_depth_from_plane_param (planar_initer.cu:279-286)
            const float d = -pl[3] / (((float)i - cam->K[2]) * pl[0] / cam->K[0] +
                                      ((float)j - cam->K[5]) * pl[1] / cam->K[4] + pl[2]);
            if (!(d <= depth_max && d >= depth_min)) mask[k] = 0;
        }
        out_masks[k] = mask[k];
        if (mask[k] > 0)
            std::memcpy(o, planes[mask[k] - 1].data(), 16);
        else
            std::memset(o, 0, 16);
    }
    if (out_tri_count) *out_tri_count = (int32_t)kept.size();
    if (out_tris)
        for (int32_t i = 0; i < (int32_t)kept.size() && i < max_tris; ++i)
            for (int e = 0; e < 3; ++e) {
                out_tris[i * 6 + e * 2 + 0] = (int32_t)kept[i][e].x;
                out_tris[i * 6 + e * 2 + 1] = (int32_t)kept[i][e].y;
            }
    return GMVS_OK;
}

extern "C" int32_t gmvs_fusion_planar_mask(const int32_t* seg_ids, const int32_t* planar_mask, const float* normals,
                                           int32_t rows, int32_t cols, int32_t thresh, float nonplanar_percent,
                                           float cos_sim_thresh, float match_ratio_thresh, int32_t* out) {
    if (!seg_ids || !planar_mask || !normals || !out || rows < 1 || cols < 1)
        return gmvs::fail(GMVS_ERR_INVALID, "gmvs_fusion_planar_mask: NULL argument or empty image");
    const size_t n = (size_t)rows * cols;
    int32_t max_val = seg_ids[0];
    for (size_t i = 1; i < n; ++i) max_val = std::max(max_val, seg_ids[i]);
    for (size_t i = 0; i < n; ++i)
        if (seg_ids[i] < 0) return gmvs::fail(GMVS_ERR_INVALID, "gmvs_fusion_planar_mask: negative segment id");
    const size_t nseg = (size_t)max_val + 1;
    // counting sort of pixels by segment keeps each segment's pixels in scan order
    std::vector<int64_t> start(nseg + 1, 0);
    std::vector<int32_t> nonplanar(nseg, 0), planar(nseg, 0);
    for (size_t k = 0; k < n; ++k) {
        start[seg_ids[k] + 1]++;
        if (planar_mask[k] == 0)
            nonplanar[seg_ids[k]]++;
        else
            planar[seg_ids[k]]++;
    }
    for (size_t s = 0; s < nseg; ++s) start[s + 1] += start[s];
    std::vector<int64_t> fillp(start.begin(), start.end() - 1);
    std::vector<int32_t> order(n);
    for (size_t k = 0; k < n; ++k) order[fillp[seg_ids[k]]++] = (int32_t)k;
    std::memset(out, 0, sizeof(int32_t) * n);
    uint32_t vps = 301;
    for (size_t s = 1; s < nseg; ++s) {
        const float np = (float)nonplanar[s], pl = (float)planar[s];
        const float amount = np + pl;
        if (amount <= thresh) continue;
        bool skip = false;
        if (np / amount >= nonplanar_percent) {
            skip = true;
            float avg[3] = {0, 0, 0};
            for (int64_t q = start[s]; q < start[s + 1]; ++q) {
                const int32_t k = order[q];
                if (planar_mask[k] != 0) continue;
                for (int e = 0; e < 3; ++e) avg[e] += normals[(size_t)k * 3 + e];
            }
            for (int e = 0; e < 3; ++e) avg[e] /= np;
            int valid = 0;
            for (int64_t q = start[s]; q < start[s + 1]; ++q) {
                const int32_t k = order[q];
                if (planar_mask[k] != 0) continue;
                const float cs = avg[0] * normals[(size_t)k * 3] + avg[1] * normals[(size_t)k * 3 + 1] +
                                 avg[2] * normals[(size_t)k * 3 + 2];
                valid += cs > cos_sim_thresh ? 1 : 0;
            }
            if ((float)valid / np > match_ratio_thresh)
                skip = false;
            else
                for (int64_t q = start[s]; q < start[s + 1]; ++q) out[order[q]] = 300;
        } else if (np / amount < 0.25f) {
            for (int64_t q = start[s]; q < start[s + 1]; ++q) out[order[q]] = (int32_t)vps;
            vps += 1;
            skip = true;
        }
        if (skip) continue;
        for (int64_t q = start[s]; q < start[s + 1]; ++q) out[order[q]] = (int32_t)s;
    }
    return GMVS_OK;
}

extern "C" int32_t gmvs_filter_by_var_map(const float* var_map, const int32_t* seg, int32_t rows, int32_t cols,
                                          float var_thresh, int32_t* out) {
    if (!var_map || !seg || !out || rows < 1 || cols < 1)
        return gmvs::fail(GMVS_ERR_INVALID, "gmvs_filter_by_var_map: NULL argument or empty image");
    const size_t n = (size_t)rows * cols;
    int32_t max_val = seg[0];
    for (size_t i = 1; i < n; ++i) max_val = std::max(max_val, seg[i]);
    if (max_val < 0) max_val = 0;
    std::vector<float> acc(max_val + 1, 0.0f), cnt(max_val + 1, 0.0f);
    std::vector<char> keep(max_val + 1, 0);
    for (size_t k = 0; k < n; ++k) {
        if (seg[k] <= 0) continue;
        ++cnt[seg[k]];
        acc[seg[k]] += var_map[k];
    }
    for (int s = 1; s <= max_val; ++s) keep[s] = (acc[s] / cnt[s]) <= var_thresh;
    for (size_t k = 0; k < n; ++k) out[k] = (seg[k] > 0 && keep[seg[k]]) ? seg[k] : 0;
    return GMVS_OK;
}

extern "C" int32_t gmvs_sliding_window_normal(const int32_t* region, const float* normals, int32_t rows, int32_t cols,
                                              int32_t win, float* out) {
    if (!region || !normals || !out || rows < 1 || cols < 1)
        return gmvs::fail(GMVS_ERR_INVALID, "gmvs_sliding_window_normal: NULL argument or empty image");
    const int h = win / 2;
    for (int r = 0; r < rows; ++r)
        for (int c = 0; c < cols; ++c) {
            const size_t k = (size_t)r * cols + c;
            if (region[k] == 1) {
                out[k * 3] = out[k * 3 + 1] = out[k * 3 + 2] = 0.0f;
                continue;
            }
            // float accumulation in window scan order, as the reference
            int valid = 0;
            float n[3] = {0, 0, 0};
            for (int rr = std::max(0, r - h); rr < std::min(rows, r + h + 1); ++rr)
                for (int cc = std::max(0, c - h); cc < std::min(cols, c + h + 1); ++cc) {
                    const size_t q = (size_t)rr * cols + cc;
                    if (region[q] == 1) continue;
                    ++valid;
                    for (int e = 0; e < 3; ++e) n[e] += normals[q * 3 + e];
                }
            for (int e = 0; e < 3; ++e) out[k * 3 + e] = n[e] / (float)valid;
        }
    return GMVS_OK;
}
