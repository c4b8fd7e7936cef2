// Scene-level C API: a context and a job that own the device state of one
// scene and run the reference's reconstruction sequence (launch.py:143-173:
// the random pass, triangulation and planar-prior pass of planar_init.py,
// the geometric passes and the fusion of consistency.py) through the plan
// API, for hosts that are not Python (a C or C++ replacement of launch.py
// binds these and nothing else).  The Python pipeline (pipeline.py) runs
// the same passes with the same parameters, so both give the same maps.
//
// Unlike the plan API, a job allocates its device buffers itself (like the
// reference's PlanarInit, planar_initer.cu:21-62): per view the depth,
// normal, cost and plane maps of two passes (double-buffered between
// passes), the prior planes and masks, the fused maps and the fusion masks.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "errors.h"

struct gmvs_ctx {
    int device = 0;
    std::string last_error;
};

struct gmvs_job {
    gmvs_ctx* ctx = nullptr;
    int V = 0, H = 0, W = 0;
    std::vector<gmvs_camera> cams;
    std::vector<gmvs_problem> problems;
    const float* images = nullptr;  // caller-owned device [V][H][W]
    std::vector<uint8_t> superpixels;  // host [V][H][W] or empty
    char* block = nullptr;             // one device allocation for every map below
    float* depth[2] = {};
    float* normal[2] = {};
    float* cost[2] = {};
    float* planes[2] = {};
    float* prior_planes = nullptr;
    uint32_t* prior_masks = nullptr;
    float* fused_depth = nullptr;
    float* fused_normal = nullptr;
    uint8_t* masks = nullptr;
    int latest = -1;  // buffer of the last pass (-1: none yet)
    int geom_count = 0;
    void* ws = nullptr;  // plan workspace, grown on demand
    size_t ws_bytes = 0;
    void* ws2 = nullptr;  // the second view group's, for the random + prior pass
    size_t ws2_bytes = 0;
    void* fuse_scratch = nullptr;
    size_t fuse_bytes = 0;
};

namespace gmvs {
namespace {

// the calling thread's current device is restored on return
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int32_t job_fail(gmvs_job* job, int32_t rc) {
    if (rc != GMVS_OK && job && job->ctx) job->ctx->last_error = g_last_error;
    return rc;
}

int32_t grow(void** p, size_t* have, size_t need, cudaStream_t st, const char* who) {
    if (*have >= need) return GMVS_OK;
    cudaError_t e = cudaStreamSynchronize(st);  // nothing queued may still use the old buffer
    if (e == cudaSuccess && *p) e = cudaFree(*p);
    *p = nullptr;
    *have = 0;
    if (e == cudaSuccess) e = cudaMalloc(p, need);
    if (e != cudaSuccess) return fail_cuda(e, who);
    *have = need;
    return GMVS_OK;
}

// search range of a reference view (planar_init.py:149-150,
// gmvs/src/patch_match.cu:1379-1380), formed in FP64 and rounded once like
// the Python callers' float(depth_min) * 0.6
void view_range(const gmvs_camera& c, float& dmin, float& dmax) {
    dmin = (float)((double)c.depth_min * 0.6);
    dmax = (float)((double)c.depth_max * 1.2);
}

int32_t problem_set(const gmvs_job* job, const int32_t* ids, int32_t n, std::vector<int>& out, const char* who) {
    out.clear();
    if (!ids) {
        for (int k = 0; k < (int)job->problems.size(); ++k) out.push_back(k);
        return GMVS_OK;
    }
    if (n < 1) return fail(GMVS_ERR_INVALID, std::string(who) + ": empty problem set");
    std::vector<char> seen(job->problems.size(), 0);
    for (int32_t i = 0; i < n; ++i) {
        if (ids[i] < 0 || ids[i] >= (int32_t)job->problems.size())
            return fail(GMVS_ERR_INVALID, std::string(who) + ": problem index out of range");
        if (seen[ids[i]]++)  // one launch may not write a view's maps twice
            return fail(GMVS_ERR_INVALID, std::string(who) + ": problem listed twice");
        out.push_back(ids[i]);
    }
    return GMVS_OK;
}

gmvs_view_pass base_view(const gmvs_job* job, const gmvs_problem& pr, int out) {
    gmvs_view_pass v;
    std::memset(&v, 0, sizeof(v));
    const size_t hw = (size_t)job->H * job->W;
    const int ref = pr.ref_image_id;
    v.height = job->H;
    v.width = job->W;
    v.num_src = pr.num_ngb;
    v.stream_id = ref;
    view_range(job->cams[ref], v.depth_min, v.depth_max);
    for (int j = 0; j <= pr.num_ngb; ++j) {
        const int id = j == 0 ? ref : pr.src_image_ids[j - 1];
        v.cams[j] = job->cams[id];
        v.images[j] = job->images + id * hw;
    }
    v.out_depth = job->depth[out] + ref * hw;
    v.out_normal = job->normal[out] + ref * hw * 3;
    v.out_cost = job->cost[out] + ref * hw;
    v.out_planes = job->planes[out] + ref * hw * 4;
    return v;
}

int32_t run_views(gmvs_job* job, const std::vector<gmvs_view_pass>& views, const gmvs_params& p, cudaStream_t st,
                  const char* who) {
    const size_t need = gmvs_plan_workspace_bytes(views.data(), (int32_t)views.size(), &p);
    if (need == 0) return GMVS_ERR_INVALID;  // the message is set
    int32_t rc = grow(&job->ws, &job->ws_bytes, need, st, who);
    if (rc != GMVS_OK) return rc;
    return gmvs_run_passes(views.data(), (int32_t)views.size(), &p, job->ws, job->ws_bytes, st);
}

// consistency.py:193-197: n / |n| where |n| > 0.5
__global__ void k_renormalise(float* __restrict__ n, size_t count) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        float* v = n + 3 * i;
        const float x = v[0], y = v[1], z = v[2];
        const float len = sqrtf(x * x + y * y + z * z);
        if (len > 0.5f) {
            v[0] = x / len;
            v[1] = y / len;
            v[2] = z / len;
        }
    }
}

}  // namespace
}  // namespace gmvs

using namespace gmvs;

extern "C" int32_t gmvs_ctx_create(int32_t device, gmvs_ctx** out) {
    if (!out) return fail(GMVS_ERR_INVALID, "gmvs_ctx_create: NULL out");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return fail_cuda(e, "gmvs_ctx_create");
    if (device < 0 || device >= count) return fail(GMVS_ERR_INVALID, "gmvs_ctx_create: no such device");
    gmvs_ctx* c = new gmvs_ctx;
    c->device = device;
    *out = c;
    return GMVS_OK;
}

extern "C" void gmvs_ctx_destroy(gmvs_ctx* ctx) { delete ctx; }

extern "C" int32_t gmvs_ctx_last_error(const gmvs_ctx* ctx, char* buf, size_t len) {
    if (!ctx || !buf || len == 0) return GMVS_ERR_INVALID;
    const size_t n = std::min(len - 1, ctx->last_error.size());
    std::memcpy(buf, ctx->last_error.data(), n);
    buf[n] = 0;
    return GMVS_OK;
}

extern "C" int32_t gmvs_job_create(gmvs_ctx* ctx, const gmvs_camera* cams, int32_t num_images, int32_t height,
                                   int32_t width, const float* images, const uint8_t* superpixels,
                                   const gmvs_problem* problems, int32_t num_problems, gmvs_job** out) {
    const char* who = "gmvs_job_create";
    if (!ctx || !cams || !images || !problems || !out) return fail(GMVS_ERR_INVALID, std::string(who) + ": NULL");
    *out = nullptr;
    if (num_images < 1 || height < 1 || width < 1 || num_problems < 1)
        return fail(GMVS_ERR_INVALID, std::string(who) + ": empty scene");
    for (int32_t k = 0; k < num_problems; ++k) {
        const gmvs_problem& p = problems[k];
        bool ok = p.ref_image_id >= 0 && p.ref_image_id < num_images && p.num_ngb >= 1 && p.num_ngb <= GMVS_MAX_NGB;
        for (int j = 0; ok && j < p.num_ngb; ++j) ok = p.src_image_ids[j] >= 0 && p.src_image_ids[j] < num_images;
        if (!ok) {
            ctx->last_error = std::string(who) + ": problem " + std::to_string(k) + " is out of range";
            return fail(GMVS_ERR_INVALID, ctx->last_error);
        }
        // caught here rather than by the fusion after every pass has run
        for (int j = 0; j < p.num_ngb; ++j) {
            std::string why;
            if (p.src_image_ids[j] == p.ref_image_id) why = "a source view equals the reference view";
            for (int i = 0; why.empty() && i < j; ++i)
                if (p.src_image_ids[i] == p.src_image_ids[j])
                    why = "source view " + std::to_string(p.src_image_ids[j]) + " is listed twice";
            if (!why.empty()) {
                ctx->last_error = std::string(who) + ": problem " + std::to_string(k) + ": " + why;
                return fail(GMVS_ERR_INVALID, ctx->last_error);
            }
        }
    }
    std::vector<char> is_ref(num_images, 0);
    for (int32_t k = 0; k < num_problems; ++k)
        if (is_ref[problems[k].ref_image_id]++) {
            ctx->last_error = std::string(who) + ": two problems share reference view " +
                              std::to_string(problems[k].ref_image_id);
            return fail(GMVS_ERR_INVALID, ctx->last_error);
        }
    for (int32_t i = 0; i < num_images; ++i)
        if (cams[i].height != height || cams[i].width != width) {
            ctx->last_error = std::string(who) + ": every camera must be height x width";
            return fail(GMVS_ERR_INVALID, ctx->last_error);
        }
    DeviceGuard dg(ctx->device);
    gmvs_job* j = new gmvs_job;
    j->ctx = ctx;
    j->V = num_images, j->H = height, j->W = width;
    j->cams.assign(cams, cams + num_images);
    j->problems.assign(problems, problems + num_problems);
    j->images = images;
    const size_t hw = (size_t)height * width, v = (size_t)num_images;
    if (superpixels) j->superpixels.assign(superpixels, superpixels + v * hw);
    // one allocation: 2 x (depth 1 + normal 3 + cost 1 + planes 4) + prior 4 + masks 1 + fused 4 floats, masks bytes
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t f = v * hw * sizeof(float);
    size_t off = 0;
    std::vector<size_t> at;
    for (size_t words : {1, 3, 1, 4, 1, 3, 1, 4, 4, 1, 1, 3}) {
        at.push_back(off);
        off = al(off + words * f);
    }
    const size_t masks_at = off;
    off = al(off + v * hw);
    cudaError_t e = cudaMalloc((void**)&j->block, off);
    if (e != cudaSuccess) {
        delete j;
        ctx->last_error = std::string(who) + ": device allocation of " + std::to_string(off) + " bytes failed";
        return fail(GMVS_ERR_CUDA, ctx->last_error);
    }
    for (int b = 0; b < 2; ++b) {
        j->depth[b] = (float*)(j->block + at[4 * b + 0]);
        j->normal[b] = (float*)(j->block + at[4 * b + 1]);
        j->cost[b] = (float*)(j->block + at[4 * b + 2]);
        j->planes[b] = (float*)(j->block + at[4 * b + 3]);
    }
    j->prior_planes = (float*)(j->block + at[8]);
    j->prior_masks = (uint32_t*)(j->block + at[9]);
    j->fused_depth = (float*)(j->block + at[10]);
    j->fused_normal = (float*)(j->block + at[11]);
    j->masks = (uint8_t*)(j->block + masks_at);
    // views that are no problem's reference keep zero fused maps
    e = cudaMemset(j->block, 0, off);
    if (e != cudaSuccess) {
        cudaFree(j->block);
        delete j;
        return fail_cuda(e, who);
    }
    *out = j;
    return GMVS_OK;
}

extern "C" void gmvs_job_destroy(gmvs_job* job) {
    if (!job) return;
    DeviceGuard dg(job->ctx->device);
    cudaDeviceSynchronize();
    if (job->ws) cudaFree(job->ws);
    if (job->ws2) cudaFree(job->ws2);
    if (job->fuse_scratch) cudaFree(job->fuse_scratch);
    if (job->block) cudaFree(job->block);
    delete job;
}

namespace gmvs {
namespace {

// The planar prior of the given problems' reference views from their
// first-pass depth and cost (host, all cores; planar_init.py:173-181).
int32_t triangulate(const gmvs_job* job, const std::vector<int>& ids, const std::vector<float>& depth,
                    const std::vector<float>& cost, std::vector<float>& planes, std::vector<uint32_t>& masks) {
    const size_t hw = (size_t)job->H * job->W;
    const bool spf = !job->superpixels.empty();
    std::vector<int32_t> rcs(ids.size(), GMVS_OK);
    std::vector<std::string> errs(ids.size());
    const size_t nthreads =
        std::max<size_t>(1, std::min<size_t>(ids.size(), std::max(1u, std::thread::hardware_concurrency())));
    std::vector<std::thread> pool;
    for (size_t t = 0; t < nthreads; ++t)
        pool.emplace_back([&, t]() {
            for (size_t i = t; i < ids.size(); i += nthreads) {
                const int ref = job->problems[ids[i]].ref_image_id;
                float dmin, dmax;
                view_range(job->cams[ref], dmin, dmax);
                rcs[i] = gmvs_build_planar_prior(&job->cams[ref], job->H, job->W, depth.data() + i * hw,
                                                 cost.data() + i * hw,
                                                 spf ? job->superpixels.data() + ref * hw : nullptr, spf ? 1 : 0,
                                                 dmin, dmax, planes.data() + i * hw * 4, masks.data() + i * hw,
                                                 nullptr, nullptr, 0);
                if (rcs[i] != GMVS_OK) errs[i] = g_last_error;  // thread-local: copy it out
            }
        });
    for (auto& th : pool) th.join();
    for (size_t i = 0; i < ids.size(); ++i)
        if (rcs[i] != GMVS_OK) return fail(rcs[i], errs[i]);
    return GMVS_OK;
}

}  // namespace
}  // namespace gmvs

// The problems run in two view groups so that the host triangulation of one
// overlaps device work of the other: random pass of group 0, random pass of
// group 1 (triangulation of group 0 meanwhile), prior pass of group 0
// (triangulation of group 1 meanwhile), prior pass of group 1 -- the order
// the Python pipeline uses.  A view's results do not depend on the grouping
// (its random stream is keyed by its own id).  Each group's plans live in
// their own workspace; plan descriptors are uploaded on a side stream so
// that creating a plan does not wait for the other group's kernels.
extern "C" int32_t gmvs_pass_random_prior(gmvs_job* job, const int32_t* problem_ids, int32_t n,
                                          const gmvs_params* params, void* stream) {
    const char* who = "gmvs_pass_random_prior";
    if (!job || !params) return fail(GMVS_ERR_INVALID, std::string(who) + ": NULL");
    DeviceGuard dg(job->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<int> set;
    int32_t rc = problem_set(job, problem_ids, n, set, who);
    if (rc != GMVS_OK) return job_fail(job, rc);
    const size_t hw = (size_t)job->H * job->W;
    // the random-initialisation pass (planar_init.py:113-172) into buffer 0,
    // the planar-prior pass (planar_init.py:181-190) from buffer 0 into 1
    gmvs_params pr = *params;
    pr.init_kind = GMVS_INIT_RANDOM;
    pr.sweep_kind = GMVS_SWEEP_PHOTO;
    pr.sampler = GMVS_SAMPLER_TEX;
    pr.pass_index = 0;
    pr.run_filter = 1;
    gmvs_params pp = pr;
    pp.init_kind = GMVS_INIT_PRIOR;
    pp.sweep_kind = GMVS_SWEEP_PRIOR;
    pp.pass_index = 1;
    const size_t G = set.size() >= 2 ? 2 : 1;
    std::vector<int> grp[2];
    for (size_t i = 0; i < set.size(); ++i) grp[i * G / set.size()].push_back(set[i]);
    std::vector<gmvs_view_pass> rv[2], pv[2];
    void** ws[2] = {&job->ws, &job->ws2};
    size_t* ws_bytes[2] = {&job->ws_bytes, &job->ws2_bytes};
    for (size_t g = 0; g < G; ++g) {
        for (int k : grp[g]) {
            rv[g].push_back(base_view(job, job->problems[k], 0));
            gmvs_view_pass v = base_view(job, job->problems[k], 1);
            const int ref = job->problems[k].ref_image_id;
            v.prior_planes = job->prior_planes + ref * hw * 4;
            v.prior_masks = job->prior_masks + ref * hw;
            v.init_planes = job->planes[0] + ref * hw * 4;
            v.init_costs = job->cost[0] + ref * hw;
            pv[g].push_back(v);
        }
        const size_t nr = gmvs_plan_workspace_bytes(rv[g].data(), (int32_t)rv[g].size(), &pr);
        const size_t np = gmvs_plan_workspace_bytes(pv[g].data(), (int32_t)pv[g].size(), &pp);
        if (nr == 0 || np == 0) return job_fail(job, GMVS_ERR_INVALID);  // the message is set
        rc = grow(ws[g], ws_bytes[g], std::max(nr, np), st, who);
        if (rc != GMVS_OK) return job_fail(job, rc);
    }
    cudaStream_t side = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    gmvs_plan* plan[2] = {nullptr, nullptr};
    // on every exit: nothing of this call may still run when its plans,
    // events, stream and host buffers go
    auto finish = [&](int32_t code) {
        cudaStreamSynchronize(st);
        if (side) cudaStreamSynchronize(side);
        for (size_t g = 0; g < 2; ++g) {
            if (plan[g]) gmvs_plan_destroy(plan[g]);
            if (ev[g]) cudaEventDestroy(ev[g]);
        }
        if (side) cudaStreamDestroy(side);
        return job_fail(job, code);
    };
    cudaError_t e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    for (size_t g = 0; g < G && e == cudaSuccess; ++g) e = cudaEventCreateWithFlags(&ev[g], cudaEventDisableTiming);
    if (e != cudaSuccess) return finish(fail_cuda(e, who));
    // 1. both groups' random passes
    for (size_t g = 0; g < G; ++g) {
        rc = gmvs_plan_create(rv[g].data(), (int32_t)rv[g].size(), &pr, *ws[g], *ws_bytes[g], side, &plan[g]);
        if (rc == GMVS_OK) rc = gmvs_plan_launch(plan[g], st);
        if (rc != GMVS_OK) return finish(rc);
        e = cudaEventRecord(ev[g], st);
        if (e != cudaSuccess) return finish(fail_cuda(e, who));
    }
    for (size_t g = 0; g < G; ++g) {
        // 2. group g's first-pass depth and cost to the host once its random
        // pass is done, its triangulation there while the device runs on
        const size_t m = grp[g].size();
        std::vector<float> depth(m * hw), cost(m * hw), planes(m * hw * 4);
        std::vector<uint32_t> masks(m * hw);
        e = cudaStreamWaitEvent(side, ev[g], 0);
        for (size_t i = 0; i < m && e == cudaSuccess; ++i) {
            const int ref = job->problems[grp[g][i]].ref_image_id;
            e = cudaMemcpyAsync(depth.data() + i * hw, job->depth[0] + ref * hw, hw * 4, cudaMemcpyDeviceToHost,
                                side);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(cost.data() + i * hw, job->cost[0] + ref * hw, hw * 4, cudaMemcpyDeviceToHost,
                                    side);
        }
        if (e != cudaSuccess) return finish(fail_cuda(e, who));
        rc = gmvs_plan_check(plan[g], side);  // synchronises the side stream
        if (rc != GMVS_OK) return finish(rc);
        gmvs_plan_destroy(plan[g]);
        plan[g] = nullptr;
        rc = triangulate(job, grp[g], depth, cost, planes, masks);
        if (rc != GMVS_OK) return finish(rc);
        for (size_t i = 0; i < m && e == cudaSuccess; ++i) {
            const int ref = job->problems[grp[g][i]].ref_image_id;
            e = cudaMemcpyAsync(job->prior_planes + ref * hw * 4, planes.data() + i * hw * 4, hw * 16,
                                cudaMemcpyHostToDevice, side);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(job->prior_masks + ref * hw, masks.data() + i * hw, hw * 4,
                                    cudaMemcpyHostToDevice, side);
        }
        if (e != cudaSuccess) return finish(fail_cuda(e, who));
        // 3. group g's prior pass; creating its plan synchronises the side
        // stream, so the uploads above are done before it is queued
        rc = gmvs_plan_create(pv[g].data(), (int32_t)pv[g].size(), &pp, *ws[g], *ws_bytes[g], side, &plan[g]);
        if (rc == GMVS_OK) rc = gmvs_plan_launch(plan[g], st);
        if (rc != GMVS_OK) return finish(rc);
    }
    for (size_t g = 0; g < G; ++g) {
        rc = gmvs_plan_check(plan[g], st);
        if (rc != GMVS_OK) return finish(rc);
    }
    rc = finish(GMVS_OK);
    if (rc == GMVS_OK) job->latest = 1;
    return rc;
}

extern "C" int32_t gmvs_pass_geom(gmvs_job* job, const int32_t* problem_ids, int32_t n, const gmvs_params* params,
                                  const float* depth_in, const float* normal_in, void* stream) {
    const char* who = "gmvs_pass_geom";
    if (!job || !params) return fail(GMVS_ERR_INVALID, std::string(who) + ": NULL");
    if ((depth_in == nullptr) != (normal_in == nullptr))
        return job_fail(job, fail(GMVS_ERR_INVALID, std::string(who) + ": give both input maps or neither"));
    if (!depth_in && job->latest < 0)
        return job_fail(job, fail(GMVS_ERR_INVALID, std::string(who) + ": no previous pass to start from"));
    DeviceGuard dg(job->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<int> set;
    int32_t rc = problem_set(job, problem_ids, n, set, who);
    if (rc != GMVS_OK) return job_fail(job, rc);
    const size_t hw = (size_t)job->H * job->W;
    const float* din = depth_in ? depth_in : job->depth[job->latest];
    const float* nin = normal_in ? normal_in : job->normal[job->latest];
    const int out = job->latest < 0 ? 0 : 1 - job->latest;
    // consistency.run_patch_match (launch.py:157-164): module B from the previous maps
    gmvs_params p = *params;
    p.init_kind = GMVS_INIT_DEPTH_NORMAL;
    p.sweep_kind = GMVS_SWEEP_GEOM;
    p.sampler = GMVS_SAMPLER_CLAMP;
    p.pass_index = 2 + job->geom_count;
    p.run_filter = 1;
    std::vector<gmvs_view_pass> views;
    for (int k : set) {
        const gmvs_problem& pr = job->problems[k];
        gmvs_view_pass v = base_view(job, pr, out);
        for (int j = 0; j <= pr.num_ngb; ++j) {
            const int id = j == 0 ? pr.ref_image_id : pr.src_image_ids[j - 1];
            v.depths[j] = din + id * hw;
        }
        v.ref_normal = nin + pr.ref_image_id * hw * 3;
        views.push_back(v);
    }
    rc = run_views(job, views, p, st, who);
    if (rc != GMVS_OK) return job_fail(job, rc);
    job->latest = out;
    ++job->geom_count;
    return GMVS_OK;
}

extern "C" int32_t gmvs_job_fuse(gmvs_job* job, const int32_t* order, int32_t n, int32_t geom_consistent,
                                 uint8_t* masks, void* stream) {
    const char* who = "gmvs_job_fuse";
    if (!job) return fail(GMVS_ERR_INVALID, std::string(who) + ": NULL");
    if (job->latest < 0) return job_fail(job, fail(GMVS_ERR_INVALID, std::string(who) + ": no pass to fuse"));
    DeviceGuard dg(job->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<int> set;
    int32_t rc = problem_set(job, order, n, set, who);
    if (rc != GMVS_OK) return job_fail(job, rc);
    const size_t hw = (size_t)job->H * job->W;
    uint8_t* mk = masks ? masks : job->masks;
    cudaError_t e = cudaMemsetAsync(mk, 0, (size_t)job->V * hw, st);
    if (e != cudaSuccess) return job_fail(job, fail_cuda(e, who));
    rc = grow(&job->fuse_scratch, &job->fuse_bytes, gmvs_fuse_scratch_bytes(job->H, job->W), st, who);
    if (rc != GMVS_OK) return job_fail(job, rc);
    const int b = job->latest;
    // consistency.run_fusion over the problems in order (launch.py:166-173)
    for (int k : set) {
        const gmvs_problem& pr = job->problems[k];
        gmvs_fuse_view a;
        std::memset(&a, 0, sizeof(a));
        a.height = job->H;
        a.width = job->W;
        a.num_views = job->V;
        a.problem = pr;
        for (int j = 0; j <= pr.num_ngb; ++j) {
            const int id = j == 0 ? pr.ref_image_id : pr.src_image_ids[j - 1];
            a.cams[j] = job->cams[id];
            a.depths[j] = job->depth[b] + id * hw;
            a.normals[j] = job->normal[b] + id * hw * 3;
        }
        a.masks = mk;
        a.geom_consistent = geom_consistent;
        a.out_depth = job->fused_depth + pr.ref_image_id * hw;
        a.out_normal = job->fused_normal + pr.ref_image_id * hw * 3;
        rc = gmvs_fuse(&a, job->fuse_scratch, job->fuse_bytes, st);
        if (rc != GMVS_OK) return job_fail(job, rc);
    }
    const size_t cnt = (size_t)job->V * hw;
    k_renormalise<<<(int)std::min<size_t>((cnt + 255) / 256, 152 * 16), 256, 0, st>>>(job->fused_normal, cnt);
    e = cudaGetLastError();
    if (e != cudaSuccess) return job_fail(job, fail_cuda(e, who));
    return GMVS_OK;
}

extern "C" int32_t gmvs_export(gmvs_job* job, int32_t view, int32_t which, float* depth, float* normal, float* cost,
                               void* stream) {
    const char* who = "gmvs_export";
    if (!job) return fail(GMVS_ERR_INVALID, std::string(who) + ": NULL");
    if (view < 0 || view >= job->V) return job_fail(job, fail(GMVS_ERR_INVALID, std::string(who) + ": no such view"));
    if (which != 0 && which != 1)
        return job_fail(job, fail(GMVS_ERR_INVALID, std::string(who) + ": which is 0 (last pass) or 1 (fused)"));
    if (which == 0 && job->latest < 0)
        return job_fail(job, fail(GMVS_ERR_INVALID, std::string(who) + ": no pass has run"));
    if (which == 1 && cost) return job_fail(job, fail(GMVS_ERR_INVALID, std::string(who) + ": fused maps have no cost"));
    DeviceGuard dg(job->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    const size_t hw = (size_t)job->H * job->W;
    const float* sd = which ? job->fused_depth : job->depth[job->latest];
    const float* sn = which ? job->fused_normal : job->normal[job->latest];
    cudaError_t e = cudaSuccess;
    if (depth) e = cudaMemcpyAsync(depth, sd + view * hw, hw * 4, cudaMemcpyDefault, st);
    if (e == cudaSuccess && normal) e = cudaMemcpyAsync(normal, sn + view * hw * 3, hw * 12, cudaMemcpyDefault, st);
    if (e == cudaSuccess && cost)
        e = cudaMemcpyAsync(cost, job->cost[job->latest] + view * hw, hw * 4, cudaMemcpyDefault, st);
    if (e != cudaSuccess) return job_fail(job, fail_cuda(e, who));
    return GMVS_OK;
}
