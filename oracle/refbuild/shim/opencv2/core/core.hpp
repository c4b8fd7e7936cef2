/* Declaration-only stand-in for the OpenCV types that the reference's module-A
 * header (gmvs/lib/include/planar_initer.cuh) names in class members and
 * function signatures.  It holds no OpenCV code: compiling
 * gmvs/lib/src/patch_match_kernel.cu needs only complete types for the
 * PlanarInit members, and none of that file's kernels or its launcher touch an
 * OpenCV object.  Test infrastructure only (reference goldens). */
#pragma once

// standard headers the real OpenCV core header brings in transitively
#include <cfloat>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

namespace cv {
struct Point {
    int x = 0, y = 0;
};
struct Rect {
    int x = 0, y = 0, width = 0, height = 0;
};
struct Vec3b {
    unsigned char val[3];
};
class Mat {
  public:
    int rows = 0, cols = 0;
};
template <typename T>
class Mat_ : public Mat {};
}  // namespace cv
