// Shared device-side definitions of libsphgpu (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "convert.cuh"

namespace sph {

// Neighbour entries: 26-bit sorted node index + 6-bit image code (2 bits per axis).
constexpr int kIndexBits = 26;
constexpr uint32_t kIndexMask = (1u << kIndexBits) - 1u;
constexpr long kMaxNodes = (1L << kIndexBits);
constexpr int kMaxNodeLists = 8;
constexpr int kMaxTable = 1536;   // 3*(N1+1) coefficients; N1+1 <= 512

// Axis boundary kinds for the implicit ghost images.
enum AxisKind { AXIS_OPEN = 0, AXIS_PERIODIC = 1, AXIS_REFLECT = 2 };

struct Grid {
  double lo[3];        // grid origin per axis
  double hi[3];        // periodic / wall extents (hi of the domain)
  double cell[3];      // cell edge per axis
  double inv2[3];      // 2 / cell edge (half-cells per unit length; set on the host)
  int nc[3];           // cells per axis
  int kindLo[3];       // AxisKind of the low side
  int kindHi[3];       // AxisKind of the high side
  double wallLo[3];    // reflecting wall coordinates / periodic planes
  double wallHi[3];
  float cellf[3];      // cell edges rounded to FP32 (set on the host: no device conversions)
  float ext2f;         // kernel extent squared, FP32
  int subShift;        // 3: sort keys carry one sub-cell Morton level below the cell key; 0: none
};

struct NodeListParams {
  double nPerh, hmin, hmax, rhoMin, rhoMax, gamma, minP, maxP;
  double hminInv, hmaxInv;   // 1/hmin, 1/hmax (computed on the host)
  double hminratio;          // NodeList::hminratio (ASPH eigenvalue floor)
  double gm1, ggm1;          // gamma - 1 and gamma (gamma - 1) (computed on the host)
};

struct HydroParams {
  int compatible, gradh, xsph, correctVelGrad, sumAllLists, densityUpdate;
  int linearInExpansion, quadraticInExpansion, useVelMagDt;
  double epsTensile, nTensile, Cl, Cq, eps2, cfl;
  double W0;          // kernel value at eta = 0 (Hdet = 1)
  double WnPerh;      // W(1/nPerh of the first NodeList, 1)
  int numLists;
  int tableN1;        // N1 of the quadratic table
  double tableXstep;  // interval of the quadratic table
  double extent;      // kernel extent
  int hermN;          // Hermite knots of the nperh lookup
  double hermXmin, hermXmax, hermXstep;
  const NodeListParams* lists;   // device table of the NodeLists (kMaxNodeLists entries)
  int limitedQ;                  // LimitedMonaghanGingoldViscosity instead of MonaghanGingoldViscosity
  double etaCrit, etaFold;       // its full-Q distance and fold width in eta
  int asph;                      // an ASPH smoothing scale: tensor H throughout
  int asphEnd;                   // ASPHSmoothingScale: H integrated in the step, reset at its end
  int fixShape;                  // ASPH fixShape: Hideal keeps the shape of H
  int hUpdate;                   // HEvolutionType: 0 IdealH, 1 IntegrateH, 2 FixedH
  int totalEnergy;               // evolveTotalEnergy: DepsDt is the total-energy rate
  int radialOnly;                // ASPH radialOnly
  int crk;                       // CRKSPH (LinearOrder reproducing kernels) instead of SPH
  int rkVolume;                  // RKVolumeType: 0 m/rho, 1 RKSumVolume, 4 HVolume
  int plainSums;                 // FP32 sweeps add plainly instead of compensated (FP32_PLAIN mode)
  // Domain decomposition: caller index of every (sorted) node and the count
  // of owned nodes; caller indices >= nOwn are halo copies of another
  // domain's nodes and take no part in the time-step vote.  Null without a
  // decomposition.  Set by the host just before the dt launches.
  const int* ghostOrig;
  long nOwn;
};
__device__ __forceinline__ bool isGhost(const HydroParams& hp, long i) {
  return hp.ghostOrig != nullptr && hp.ghostOrig[i] >= hp.nOwn;
}

// safeInvVar (src/Utilities/safeInv.hh): sgn(x) / max(fuzz, |x|), fuzz 1e-30
__device__ __forceinline__ double safeInvVarD(double x) { return (x < 0.0 ? -1.0 : 1.0) / fmax(1.0e-30, fabs(x)); }

// Image of coordinate p under the per-axis code (reference ghost mapping,
// PlanarBoundary::mapPosition -> mapPositionThroughPlanes, with
// closestPointOnPlane = p + ((origin - p).n) n).  Written with explicit
// round-to-nearest adds so no multiply-add contraction changes the bits.
__device__ __forceinline__ double imageCoord(double p, int code, int kindLo, int kindHi, double lo, double hi) {
  if (code == 0) return p;
  if (code == 1) {
    if (kindLo == AXIS_PERIODIC) return __dsub_rn(__dadd_rn(p, __dsub_rn(lo, p)), __dsub_rn(hi, p));   // low image
    return __dsub_rn(__dadd_rn(p, __dsub_rn(lo, p)), __dsub_rn(p, lo));                                 // mirror at lo
  }
  if (kindHi == AXIS_PERIODIC) return __dadd_rn(__dadd_rn(p, __dsub_rn(hi, p)), __dsub_rn(p, lo));      // high image
  return __dadd_rn(__dadd_rn(p, __dsub_rn(hi, p)), __dsub_rn(hi, p));                                    // mirror at hi
}
__device__ __forceinline__ bool mirrored(int code, int kindLo, int kindHi) {
  return (code == 1 && kindLo == AXIS_REFLECT) || (code == 2 && kindHi == AXIS_REFLECT);
}

// |(a x, a y, a z)|^2 exactly as GeomVector::magnitude2 of H*r for H = a I
// (left-to-right sum, no contraction).
__device__ __forceinline__ double eta2Exact(double a, double rx, double ry, double rz) {
  const double ex = __dmul_rn(a, rx), ey = __dmul_rn(a, ry), ez = __dmul_rn(a, rz);
  return __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
}

__host__ __device__ __forceinline__ uint32_t spreadBits10(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
__host__ __device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  return spreadBits10(x) | (spreadBits10(y) << 1) | (spreadBits10(z) << 2);
}

}  // namespace sph
