// PatchMatch kernels for the SampF32 sampler.
#define GMVS_SAMPLER SampF32
#define GMVS_SUFFIX f32
#include "pm_kernels.inc"
