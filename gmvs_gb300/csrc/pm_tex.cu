// PatchMatch kernels for the SampTex sampler.
#define GMVS_SAMPLER SampTex
#define GMVS_SUFFIX tex
// One texture instruction per sample leaves these kernels waiting on the
// texture path; a register budget for 3 x 256 threads per SM (24 warps
// instead of 16) hides more of that latency than its spills cost (random
// pass 11 % faster on the 1600x1200 room scene).  The software-interpolated
// samplers keep 2 x 256.
#ifndef GMVS_MIN_BLOCKS
#define GMVS_MIN_BLOCKS 3
#endif
#include "pm_kernels.inc"
