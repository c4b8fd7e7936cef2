// PatchMatch kernels for the SampTex sampler.
#define GMVS_SAMPLER SampTex
#define GMVS_SUFFIX tex
// One texture instruction per sample leaves these kernels waiting on the
// texture path; a register budget for 4 x 256 threads per SM (64 registers,
// 32 warps instead of 16) hides more of that latency than its spills cost
// (on the 1600x1200 room scene, against 3 x 256: random pass 1.5 %, prior
// pass 7 % faster; against 2 x 256 more still).  The software-interpolated
// samplers keep 2 x 256.
#ifndef GMVS_MIN_BLOCKS
#define GMVS_MIN_BLOCKS 4
#endif
#include "pm_kernels.inc"
