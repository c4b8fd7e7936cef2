// gmvs_fuse_fixed_scratch: fusion of one reference view that allocates no
// device memory.  The per-pixel winner scratch that gmvs_fuse takes from the
// caller is here a file-scope device array of GMVS_FUSE_FIXED_MAX_PIXELS
// ints, looked up once per CUDA context with cudaGetSymbolAddress and passed
// to the same fusion kernels (fuse_run, fusion.cu).  The array lives in this
// translation unit's own module: under CUDA's lazy module loading (the
// default, CUDA_MODULE_LOADING=LAZY) its 16 MiB are only taken on a device
// once this entry point runs there; with CUDA_MODULE_LOADING=EAGER every
// process that loads the library reserves them on every device it uses.
#include <cuda.h>

#include <mutex>
#include <string>

#include "common.cuh"
#include "errors.h"
#include "kernels.h"

namespace gmvs {
namespace {

constexpr size_t kFixedPixels = (size_t)GMVS_FUSE_FIXED_MAX_PIXELS;
constexpr int kMaxContexts = 64;

// Shared by every call on a device; each call re-initialises the first
// height * width entries on its stream before the kernels read them.
static __device__ __align__(256) int g_fuse_winner[kFixedPixels];

std::mutex g_setup_mu;

// The symbol's address belongs to the CUDA context that loaded the module: a
// cudaDeviceReset, or a driver-API caller that makes another context current
// on the same device, gives the array a new address.  So the cache is keyed
// on the current context's process-unique id (cuCtxGetId; ids are never
// reused, unlike context handles), reached through the runtime's driver entry
// points so the library does not link libcuda itself.
struct ScratchEntry {
    unsigned long long ctx_id;
    int* ptr;
};
ScratchEntry g_entries[kMaxContexts] = {};
int g_num_entries = 0;
int g_next_evict = 0;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// *id = 0 when no context is current on this thread yet.
int32_t current_context_id(unsigned long long* id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        if (e != cudaSuccess) return fail_cuda(e, "cudaGetDriverEntryPointByVersion(cuCtxGetCurrent)");
        e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess) return fail_cuda(e, "cudaGetDriverEntryPointByVersion(cuCtxGetId)");
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return fail(GMVS_ERR_CUDA, "the driver does not provide cuCtxGetCurrent / cuCtxGetId");
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext ctx = nullptr;
    *id = 0;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return fail(GMVS_ERR_CUDA, "cuCtxGetCurrent failed");
    if (ctx && g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return fail(GMVS_ERR_CUDA, "cuCtxGetId failed");
    return GMVS_OK;
}

// Address of g_fuse_winner in the current context, looked up on the first
// call in each context (that lookup may load this module).
int32_t winner_scratch(int** out) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    unsigned long long id = 0;
    int32_t rc = current_context_id(&id);
    if (rc != GMVS_OK) return rc;
    for (int i = 0; id != 0 && i < g_num_entries; ++i)
        if (g_entries[i].ctx_id == id) {
            *out = g_entries[i].ptr;
            return GMVS_OK;
        }
    // first call in this context (or no context yet: the runtime then makes
    // the current device's primary context current while it looks the symbol up)
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_fuse_winner);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGetSymbolAddress(fixed fusion scratch)");
    if (id == 0) {
        rc = current_context_id(&id);
        if (rc != GMVS_OK) return rc;
        if (id == 0) return fail(GMVS_ERR_CUDA, "no current CUDA context after the symbol lookup");
    }
    int slot = g_num_entries < kMaxContexts ? g_num_entries++ : (g_next_evict++ % kMaxContexts);
    g_entries[slot] = ScratchEntry{id, static_cast<int*>(p)};
    *out = static_cast<int*>(p);
    return GMVS_OK;
}

}  // namespace
}  // namespace gmvs

extern "C" int32_t gmvs_fuse_fixed_scratch(const gmvs_fuse_view* args, void* stream) {
    if (!args) return gmvs::fail(GMVS_ERR_INVALID, "args is NULL");
    if (args->height < 1 || args->width < 1) return gmvs::fail(GMVS_ERR_INVALID, "empty image");
    const size_t n = (size_t)args->height * (size_t)args->width;
    if (n > gmvs::kFixedPixels)
        return gmvs::fail(GMVS_ERR_INVALID,
                          "gmvs_fuse_fixed_scratch: " + std::to_string(args->height) + "x" +
                              std::to_string(args->width) + " = " + std::to_string(n) +
                              " pixels exceeds the fixed scratch of " + std::to_string(gmvs::kFixedPixels) +
                              " pixels; use gmvs_fuse with caller-provided scratch");
    int* winner = nullptr;
    const int32_t rc = gmvs::winner_scratch(&winner);
    if (rc != GMVS_OK) return rc;
    return gmvs::fuse_run(args, winner, (cudaStream_t)stream);
}
