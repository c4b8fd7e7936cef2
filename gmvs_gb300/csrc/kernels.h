// Host-side launchers of the device kernels (internal to the library).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace gmvs {

// Sampler/staging variants of the PatchMatch kernels.
enum SamplerVariant : int { kVarF32 = 0, kVarQuadF32 = 1, kVarQuadF16 = 2, kVarTex = 3, kNumVariants = 4 };

struct LaunchShape {
    int grid;      // CTAs (persistent: each loops over tiles)
    dim3 block;    // (tile width, tile thread rows)
    size_t smem;   // dynamic shared memory bytes
    int sms = 1;   // SMs of the device (queue kernels: grid = resident CTAs)
    int ctas = 0;  // resident CTAs per SM wanted (0 = as many as fit)
    int max_ctas = 0;  // resident CTAs per SM the plan's per-warp scratch holds (0 = no limit)
};

// One entry per variant, defined in pm_<variant>.cu.
cudaError_t launch_init_f32(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*, int*,
                            bool generic, cudaStream_t);
cudaError_t launch_sweep_f32(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*, int,
                             int*, bool generic, int split, cudaStream_t);
cudaError_t launch_init_qf32(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*, int*,
                             bool generic, cudaStream_t);
cudaError_t launch_sweep_qf32(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*, int,
                              int*, bool generic, int split, cudaStream_t);
cudaError_t launch_init_qf16(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*, int*,
                             bool generic, cudaStream_t);
cudaError_t launch_sweep_qf16(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*, int,
                              int*, bool generic, int split, cudaStream_t);
cudaError_t launch_init_tex(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*, int*,
                            bool generic, cudaStream_t);
cudaError_t launch_sweep_tex(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*, int, int*,
                             bool generic, int split, cudaStream_t);
// Per-pixel NCC cost matrix of given hypotheses (gmvs_ncc_costs).
cudaError_t launch_ncc_f32(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*,
                           const float4*, float*, float*, uint32_t*, bool generic, cudaStream_t);
cudaError_t launch_ncc_qf32(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*,
                            const float4*, float*, float*, uint32_t*, bool generic, cudaStream_t);
cudaError_t launch_ncc_qf16(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*,
                            const float4*, float*, float*, uint32_t*, bool generic, cudaStream_t);
cudaError_t launch_ncc_tex(const LaunchShape&, const DevView*, const DevParams&, const Tile*, int*,
                           const float4*, float*, float*, uint32_t*, bool generic, cudaStream_t);

// Bounds-check violation bits of each variant's kernels (~0u: not a checked build).
unsigned oob_read_f32(bool reset);
unsigned oob_read_qf32(bool reset);
unsigned oob_read_qf16(bool reset);
unsigned oob_read_tex(bool reset);

// Most CTAs of k_sweep that can be resident on one SM with this shape (0 on error).
int sweep_ctas_per_sm_f32(const LaunchShape&, bool generic);
int sweep_ctas_per_sm_qf32(const LaunchShape&, bool generic);
int sweep_ctas_per_sm_qf16(const LaunchShape&, bool generic);
int sweep_ctas_per_sm_tex(const LaunchShape&, bool generic);

// Finalisation (runtime.cu): conversion, filter + export of one colour.
cudaError_t launch_convert(const LaunchShape&, const DevView*, const Tile*, const int*, int final_buf, cudaStream_t);
cudaError_t launch_filter(const LaunchShape&, const DevView*, const Tile*, const int*, int final_buf, int colour,
                          int run_filter, cudaStream_t);

// Fusion of one view (fusion.cu) with a given per-pixel winner scratch of
// height * width ints; the call re-initialises the scratch on `st`.
int32_t fuse_run(const gmvs_fuse_view* a, int* winner, cudaStream_t st);

}  // namespace gmvs
