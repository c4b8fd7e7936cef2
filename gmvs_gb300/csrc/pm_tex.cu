// PatchMatch kernels for the SampTex sampler.
#define GMVS_SAMPLER SampTex
#define GMVS_SUFFIX tex
#include "pm_kernels.inc"
