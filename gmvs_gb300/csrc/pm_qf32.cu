// PatchMatch kernels for the SampQuadF32 sampler.
#define GMVS_SAMPLER SampQuadF32
#define GMVS_SUFFIX qf32
#include "pm_kernels.inc"
