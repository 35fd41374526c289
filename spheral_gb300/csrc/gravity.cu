// Octree gravity (TreeGravity walk) -- placeholder until the device octree lands.
#include "kernels.cuh"
#include "../../include/sphgpu.h"
#include <cstdio>

namespace sph {
struct GravityWork { int unused; };
GravityWork* gravityCreate() { return new GravityWork{0}; }
void gravityDestroy(GravityWork* w) { delete w; }
int gravityEvaluate(GravityWork*, Fields, long, double, double, double, double*, cudaStream_t, LaunchCounter*,
                    char* err, int errlen) {
  std::snprintf(err, errlen, "device octree gravity is not built in this library");
  return SPHGPU_E_UNSUPPORTED;
}
}  // namespace sph
