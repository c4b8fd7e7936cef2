// PatchMatch kernels for the SampQuadF16 sampler.
#define GMVS_SAMPLER SampQuadF16
#define GMVS_SUFFIX qf16
#include "pm_kernels.inc"
