// Host half of the superpixel extraction (felzenszwalb.cpp), shared with
// the device half (superpixel.cu).
#pragma once

#include <stdint.h>

namespace gmvs {

// Felzenszwalb merge and size filter of a rows x cols working image:
// weights of the right, down, down-right and up-right edges in raster order
// per group, k = scale / 255; writes the filtered labels (0 = dropped) and
// returns how many segments were kept.
int32_t superpixel_labels(int rows, int cols, const double* weights, double k, int min_size, int32_t* labels);

// The same from the ne edges already in visiting order (ascending weight,
// ties in edge order): endpoints sa, sb and weights sw.
int32_t superpixel_merge_sorted(int rows, int cols, int64_t ne, const int32_t* sa, const int32_t* sb,
                                const double* sw, double k, int min_size, int32_t* labels);

}  // namespace gmvs
