// gmvs_fuse_fixed_scratch: fusion of one reference view that allocates no
// device memory.  The per-pixel winner scratch that gmvs_fuse takes from the
// caller is here a file-scope device array of GMVS_FUSE_FIXED_MAX_PIXELS
// ints, looked up once per device with cudaGetSymbolAddress and passed to
// the same fusion kernels (fuse_run, fusion.cu).  The array lives in this
// translation unit's own module, so it is only loaded (and its 16 MiB only
// taken) by processes that call this entry point.
#include <mutex>
#include <string>

#include "common.cuh"
#include "errors.h"
#include "kernels.h"

namespace gmvs {
namespace {

constexpr size_t kFixedPixels = (size_t)GMVS_FUSE_FIXED_MAX_PIXELS;
constexpr int kMaxDevices = 64;

// Shared by every call on a device; each call re-initialises the first
// height * width entries on its stream before the kernels read them.
static __device__ __align__(256) int g_fuse_winner[kFixedPixels];

std::mutex g_setup_mu;
int* g_winner_ptr[kMaxDevices] = {};

// Address of g_fuse_winner on the current device, looked up on the first
// call per device (that lookup may load this module).
int32_t winner_scratch(int** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return fail(GMVS_ERR_DEVICE, "device ordinal " + std::to_string(dev) + " beyond the fixed-scratch table");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_winner_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_fuse_winner);
        if (e != cudaSuccess) return fail_cuda(e, "cudaGetSymbolAddress(fixed fusion scratch)");
        g_winner_ptr[dev] = static_cast<int*>(p);
    }
    *out = g_winner_ptr[dev];
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
