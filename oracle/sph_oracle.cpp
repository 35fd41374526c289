// =============================================================================
// CPU ORACLE -- test infrastructure only.
//
// A plain C++17 / OpenMP FP64 restatement of the reference's ideal-gas SPH
// hydro step, written to check the GPU product path.  Nothing in the product
// (spheral_gb300/, include/) links or calls this file; only the tests, the
// smoke check and the CPU-baseline leg of bench.py load it.
//
// It follows the reference's own formulation literally:
//   * ghost nodes are explicit extra nodes created boundary by boundary
//     (PlanarBoundary / PeriodicBoundary / ReflectingBoundary), and
//   * every sweep walks the UNORDERED pair list (internal-internal pairs once,
//     internal-ghost pairs once) with thread-private accumulators that are
//     summed at the end (FieldList::threadCopy / threadReduce),
// so that it can also serve as the timed "reference CPU path".
//
// Reference files restated (paths inside the llnl/spheral source tree):
//   src/Kernel/BSplineKernelInline.hh:28-93            cubic B-spline
//   src/Kernel/TableKernel.cc:23-66,169-209            table + nperh lookups
//   src/Utilities/QuadraticInterpolator.cc:60-100      quadratic table fit
//   src/Utilities/QuadraticInterpolatorViewInline.hh   lookups
//   src/Utilities/CubicHermiteInterpolator.cc:95-180   Hermite knots, monotonic
//   src/Utilities/CubicHermiteInterpolatorViewInline.hh
//   src/Utilities/bisectRoot.hh:20-74
//   src/Neighbor/ConnectivityMap.cc:747-1029           pair criterion / pairs
//   src/Neighbor/ConnectivityMapInline.hh:296-309
//   src/Boundary/PlanarBoundary.cc:102-334, PeriodicBoundary.cc:77-128,
//   src/Boundary/findNodesTouchingThroughPlanes.cc:13-76,
//   src/Boundary/mapPositionThroughPlanes.hh:17-27, Utilities/pointDistances.hh:69-74
//   src/SPH/computeSPHSumMassDensity.cc:15-87
//   src/SPH/computeSPHOmegaGradhCorrection.cc:15-116
//   src/SPH/SPH.cc:166-555                             pair loop + finalize
//   src/ArtificialViscosity/MonaghanGingoldViscosity.cc:41-101
//   src/SmoothingScale/SPHSmoothingScale.cc:101-275
//   src/Physics/GenericHydro.cc:113-381                dt
//   src/Hydro/SpecificThermalEnergyPolicy.cc:47-174    compatible energy
//   src/Integrator/CheapSynchronousRK2.cc:40-132, Integrator.cc:67-169
//   src/DataBase/State.cc:222-340 (+ Increment/Replace bounded policies)
//   src/Material/GammaLawGas.cc:185-243
//   src/Geometry/GeomSymmetricTensorInline.hh:1650-1747,2230-2260
//   src/Geometry/GeomTensorInline.hh:1885-1972
//   src/Gravity/TreeGravity.cc:55-82,146-480,819-932, TreeGravityInline.hh:38-165
//   CRKSPH: src/CRKSPH/CRKSPH.cc:143-380, CRKSPHBase.cc:190-225,
//   src/CRKSPH/computeCRKSPHSumMassDensity.cc:15-110, src/RK/RKCorrections.cc:300-420,
//   src/RK/RKUtilities.cc:66-80,181-206,250-491, RKUtilitiesInline.hh:155-163,345-351,
//   src/RK/computeRKVolumes.cc:20-70, computeRKSumVolume.cc:30-110, computeHVolumes.cc:25-60,
//   src/RK/ContinuityVolumePolicy.cc:40-75, src/Boundary/ReflectingBoundary.cc:402-432
//
// Third-party arithmetic: the reference fits each quadratic table interval
// with Eigen's 3x3 inverse and solves the Hermite knot system with Eigen's
// SparseLU (Eigen 5.0.0, not vendored).  Here the 3x3 inverse is the cofactor
// formula and the tridiagonal system is solved with the Thomas algorithm: the
// coefficients agree with the reference to rounding, bit parity is unpinned.
// =============================================================================
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

using std::vector;
static const double kTiny30 = 1.0e-30;
static const double kDblEps = std::numeric_limits<double>::epsilon();

//------------------------------------------------------------------------------
// Small geometry types (component orders as in GeomVector / GeomTensor /
// GeomSymmetricTensor of the reference).
//------------------------------------------------------------------------------
struct V3 { double x = 0, y = 0, z = 0; };
struct ST { double xx = 0, xy = 0, xz = 0, yy = 0, yz = 0, zz = 0; };   // symmetric
struct T9 { double xx = 0, xy = 0, xz = 0, yx = 0, yy = 0, yz = 0, zx = 0, zy = 0, zz = 0; };

static inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 add(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 mul(const V3& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 mul(double s, const V3& a) { return {s * a.x, s * a.y, s * a.z}; }
static inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double mag2(const V3& a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline double mag(const V3& a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline V3 unitVector(const V3& a) {            // GeomVectorInline.hh:998
  const double m = mag(a);
  return m > 1.0e-50 ? V3{a.x / m, a.y / m, a.z / m} : V3{1.0, 0.0, 0.0};
}
static inline V3 dotSV(const ST& H, const V3& r) {    // GeomSymmetricTensorInline.hh:1773
  return {H.xx * r.x + H.xy * r.y + H.xz * r.z,
          H.xy * r.x + H.yy * r.y + H.yz * r.z,
          H.xz * r.x + H.yz * r.y + H.zz * r.z};
}
static inline ST scaleS(const ST& H, double s) {
  return {H.xx * s, H.xy * s, H.xz * s, H.yy * s, H.yz * s, H.zz * s};
}
static inline ST scaleS(double s, const ST& H) {
  return {s * H.xx, s * H.xy, s * H.xz, s * H.yy, s * H.yz, s * H.zz};
}
static inline double detS(const ST& H) {               // GeomSymmetricTensorInline.hh:1740
  return (H.xx * H.yy * H.zz + H.xy * H.yz * H.xz + H.xz * H.xy * H.yz -
          H.xx * H.yz * H.yz - H.xy * H.xy * H.zz - H.xz * H.yy * H.xz);
}
static inline double maxAbsS(const ST& H) {
  return std::max(std::fabs(H.xx), std::max(std::fabs(H.xy), std::max(std::fabs(H.xz),
         std::max(std::fabs(H.yy), std::max(std::fabs(H.yz), std::fabs(H.zz))))));
}
// Eberly closed-form eigenvalues, GeomSymmetricTensorInline.hh:2230-2260.
static inline V3 eigenValuesS(const ST& H) {
  const double onethird = 1.0 / 3.0;
  const double sqrt3 = std::sqrt(3.0);
  const double fscale = std::max(10.0 * kDblEps, maxAbsS(H));
  const double fscalei = 1.0 / fscale;
  const double a00 = H.xx * fscalei, a01 = H.xy * fscalei, a02 = H.xz * fscalei;
  const double a11 = H.yy * fscalei, a12 = H.yz * fscalei, a22 = H.zz * fscalei;
  const double c0 = a00 * a11 * a22 + 2.0 * a01 * a02 * a12 - a00 * a12 * a12 - a11 * a02 * a02 - a22 * a01 * a01;
  const double c1 = a00 * a11 - a01 * a01 + a00 * a22 - a02 * a02 + a11 * a22 - a12 * a12;
  const double c2 = a00 + a11 + a22;
  const double c2Div3 = c2 * onethird;
  const double aDiv3 = std::min(0.0, onethird * (c1 - c2 * c2Div3));
  const double mbDiv2 = 0.5 * (c0 + c2Div3 * (2.0 * c2Div3 * c2Div3 - c1));
  const double q = std::min(0.0, mbDiv2 * mbDiv2 + aDiv3 * aDiv3 * aDiv3);
  const double magv = std::sqrt(-aDiv3);
  const double angle = std::atan2(std::sqrt(-q), mbDiv2) * onethird;
  const double cs = std::cos(angle), sn = std::sin(angle);
  return {fscale * (c2Div3 + 2.0 * magv * cs),
          fscale * (c2Div3 - magv * (cs + sqrt3 * sn)),
          fscale * (c2Div3 - magv * (cs - sqrt3 * sn))};
}
static inline double maxElem(const V3& v) { return std::max(v.x, std::max(v.y, v.z)); }
static inline double minElem(const V3& v) { return std::min(v.x, std::min(v.y, v.z)); }
static inline bool isIsotropic(const ST& H) {
  return H.xy == 0.0 && H.xz == 0.0 && H.yz == 0.0 && H.xx == H.yy && H.xx == H.zz;
}
static inline T9 dyad(const V3& a, const V3& b) {     // GeomVectorInline.hh:946
  return {a.x * b.x, a.x * b.y, a.x * b.z, a.y * b.x, a.y * b.y, a.y * b.z, a.z * b.x, a.z * b.y, a.z * b.z};
}
static inline void addT(T9& a, const T9& b) {
  a.xx += b.xx; a.xy += b.xy; a.xz += b.xz; a.yx += b.yx; a.yy += b.yy; a.yz += b.yz; a.zx += b.zx; a.zy += b.zy; a.zz += b.zz;
}
static inline void subT(T9& a, const T9& b) {
  a.xx -= b.xx; a.xy -= b.xy; a.xz -= b.xz; a.yx -= b.yx; a.yy -= b.yy; a.yz -= b.yz; a.zx -= b.zx; a.zy -= b.zy; a.zz -= b.zz;
}
static inline T9 scaleT(double s, const T9& a) {
  return {s * a.xx, s * a.xy, s * a.xz, s * a.yx, s * a.yy, s * a.yz, s * a.zx, s * a.zy, s * a.zz};
}
static inline double traceT(const T9& a) { return a.xx + a.yy + a.zz; }
static inline double detT(const T9& a) {               // GeomTensorInline.hh:1969
  return (a.xx * a.yy * a.zz + a.xy * a.yz * a.zx + a.xz * a.yx * a.zy -
          a.xx * a.yz * a.zy - a.xy * a.yx * a.zz - a.xz * a.yy * a.zx);
}
static inline T9 inverseT(const T9& a) {               // GeomTensorInline.hh:1885
  const double d = detT(a);
  return {(a.yy * a.zz - a.yz * a.zy) / d, (a.xz * a.zy - a.xy * a.zz) / d, (a.xy * a.yz - a.xz * a.yy) / d,
          (a.yz * a.zx - a.yx * a.zz) / d, (a.xx * a.zz - a.xz * a.zx) / d, (a.xz * a.yx - a.xx * a.yz) / d,
          (a.yx * a.zy - a.yy * a.zx) / d, (a.xy * a.zx - a.xx * a.zy) / d, (a.xx * a.yy - a.xy * a.yx) / d};
}
static inline T9 dotTT(const T9& a, const T9& b) {    // GeomTensorInline.hh:2031
  return {a.xx * b.xx + a.xy * b.yx + a.xz * b.zx, a.xx * b.xy + a.xy * b.yy + a.xz * b.zy, a.xx * b.xz + a.xy * b.yz + a.xz * b.zz,
          a.yx * b.xx + a.yy * b.yx + a.yz * b.zx, a.yx * b.xy + a.yy * b.yy + a.yz * b.zy, a.yx * b.xz + a.yy * b.yz + a.yz * b.zz,
          a.zx * b.xx + a.zy * b.yx + a.zz * b.zx, a.zx * b.xy + a.zy * b.yy + a.zz * b.zy, a.zx * b.xz + a.zy * b.yz + a.zz * b.zz};
}
static inline double sgn(double x) { return x < 0.0 ? -1.0 : 1.0; }
static inline double safeInv(double x, double fuzz = kTiny30) { return x / (x * x + fuzz); }
static inline double safeInvVar(double x, double fuzz = kTiny30) { return sgn(x) / std::max(fuzz, std::fabs(x)); }
static inline bool fuzzyEqual(double a, double b, double fuzz = 1.0e-15) {
  return std::fabs(a - b) <= fuzz * std::max(1.0, std::fabs(a) + std::fabs(b));
}
static inline double pow4(double x) { return x * x * x * x; }
static inline double rootnu3(double x) { return sgn(x) * std::pow(std::fabs(x), 0.3333333333333333); }

//------------------------------------------------------------------------------
// Symmetric-tensor functions of the ASPH smoothing scale.
//------------------------------------------------------------------------------
static inline ST divS(const ST& H, double s) { return {H.xx / s, H.xy / s, H.xz / s, H.yy / s, H.yz / s, H.zz / s}; }
static inline ST identityS() { return {1.0, 0.0, 0.0, 1.0, 0.0, 1.0}; }
static inline void addS(ST& a, const ST& b) { a.xx += b.xx; a.xy += b.xy; a.xz += b.xz; a.yy += b.yy; a.yz += b.yz; a.zz += b.zz; }
// GeomSymmetricTensor<3>::Inverse (GeomSymmetricTensorInline.hh:1650-1661)
static inline ST inverseS(const ST& a) {
  const double d = detS(a);
  return {(a.yy * a.zz - a.yz * a.yz) / d, (a.yz * a.xz - a.xy * a.zz) / d, (a.xy * a.yz - a.yy * a.xz) / d,
          (a.xx * a.zz - a.xz * a.xz) / d, (a.xy * a.xz - a.xx * a.yz) / d, (a.xx * a.yy - a.xy * a.xy) / d};
}
// Eigen-pairs of a symmetric tensor (GeomSymmetricTensor<3>::eigenVectors,
// GeomSymmetricTensorInline.hh:2309-2345): the tensor is scaled by its largest
// element and elements below 1e-20 are zeroed, as there; the reference then
// calls Eigen's SelfAdjointEigenSolver (Eigen 5.0.0, not vendored).  This
// restatement diagonalises with cyclic Jacobi rotations, which converge to the
// same eigen-pairs to rounding; every use below is a function of the tensor
// (V f(lambda) V^T), so neither the order nor the signs of the pairs matter.
// vec[r][k]: component r of eigenvector k.
struct EigS { double val[3]; double vec[3][3]; };
static EigS eigenVectorsS(const ST& H) {
  const double fscale = std::max(10.0 * kDblEps, maxAbsS(H));
  const double fi = 1.0 / fscale;
  auto z = [](double x) { return std::fabs(x) < 1.0e-20 ? 0.0 : x; };
  double a[3][3] = {{z(H.xx * fi), z(H.xy * fi), z(H.xz * fi)},
                    {z(H.xy * fi), z(H.yy * fi), z(H.yz * fi)},
                    {z(H.xz * fi), z(H.yz * fi), z(H.zz * fi)}};
  double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  static const int P[3] = {0, 0, 1}, Q[3] = {1, 2, 2};
  for (int sweep = 0; sweep < 32; ++sweep) {
    const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    if (off <= 1.0e-40) break;
    for (int r = 0; r < 3; ++r) {
      const int p = P[r], q = Q[r];
      const double apq = a[p][q];
      if (apq == 0.0) continue;
      const double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
      const double t = sgn(theta) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
      const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
      a[p][p] -= t * apq;
      a[q][q] += t * apq;
      a[p][q] = a[q][p] = 0.0;
      const int o = 3 - p - q;   // the third index
      const double aop = a[o][p], aoq = a[o][q];
      a[o][p] = a[p][o] = c * aop - s * aoq;
      a[o][q] = a[q][o] = s * aop + c * aoq;
      for (int k = 0; k < 3; ++k) {
        const double vp = v[k][p], vq = v[k][q];
        v[k][p] = c * vp - s * vq;
        v[k][q] = s * vp + c * vq;
      }
    }
  }
  EigS e;
  for (int k = 0; k < 3; ++k) {
    e.val[k] = a[k][k] * fscale;
    const double nrm = 1.0 / std::sqrt(v[0][k] * v[0][k] + v[1][k] * v[1][k] + v[2][k] * v[2][k]);
    for (int r = 0; r < 3; ++r) e.vec[r][k] = v[r][k] * nrm;
  }
  return e;
}
// diag(d) rotated back to the frame of the eigenvectors (rotationalTransform).
static ST fromEigen(const double d[3], const double V[3][3]) {
  ST r;
  auto el = [&](int i, int j) { return V[i][0] * d[0] * V[j][0] + V[i][1] * d[1] * V[j][1] + V[i][2] * d[2] * V[j][2]; };
  r.xx = el(0, 0); r.xy = el(0, 1); r.xz = el(0, 2); r.yy = el(1, 1); r.yz = el(1, 2); r.zz = el(2, 2);
  return r;
}
// enforceMinEigenValue / enforceMaxEigenValue (GeomSymmetricTensorInline.hh:2578-2640):
// the tensor is returned unchanged when no eigenvalue needs the bound.
static ST enforceMinEig(const ST& H, double x) {
  const EigS e = eigenVectorsS(H);
  if (std::min(e.val[0], std::min(e.val[1], e.val[2])) >= x) return H;
  const double d[3] = {std::max(e.val[0], x), std::max(e.val[1], x), std::max(e.val[2], x)};
  return fromEigen(d, e.vec);
}
static ST enforceMaxEig(const ST& H, double x) {
  const EigS e = eigenVectorsS(H);
  if (std::max(e.val[0], std::max(e.val[1], e.val[2])) <= x) return H;
  const double d[3] = {std::min(e.val[0], x), std::min(e.val[1], x), std::min(e.val[2], x)};
  return fromEigen(d, e.vec);
}
// GeomSymmetricTensor::sqrt (GeomSymmetricTensorInline.hh:2497-2510)
static ST sqrtS(const ST& H) {
  const EigS e = eigenVectorsS(H);
  const double d[3] = {std::sqrt(std::max(0.0, e.val[0])), std::sqrt(std::max(0.0, e.val[1])),
                       std::sqrt(std::max(0.0, e.val[2]))};
  return fromEigen(d, e.vec);
}
// rotationMatrix (src/Utilities/rotationMatrix.hh:42-61): rows are the new
// axes, the first along runit.
static T9 rotationMatrix3(const V3& u) {
  const double rxy = std::sqrt(u.x * u.x + u.y * u.y);
  if (fuzzyEqual(rxy, 0.0)) return {0.0, 0.0, u.z, 0.0, 1.0, 0.0, -u.z, 0.0, 0.0};
  return {u.x, u.y, u.z, -u.y / rxy, u.x / rxy, 0.0, -u.x * u.z / rxy, -u.y * u.z / rxy, rxy};
}
// R A R^T of a symmetric tensor (GeomSymmetricTensor::rotationalTransform).
static ST rotateS(const ST& A, const T9& R) {
  const double a[3][3] = {{A.xx, A.xy, A.xz}, {A.xy, A.yy, A.yz}, {A.xz, A.yz, A.zz}};
  const double r[3][3] = {{R.xx, R.xy, R.xz}, {R.yx, R.yy, R.yz}, {R.zx, R.zy, R.zz}};
  double m[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) s += r[i][k] * a[k][l] * r[j][l];
      m[i][j] = s;
    }
  return {m[0][0], m[0][1], m[0][2], m[1][1], m[1][2], m[2][2]};
}
static T9 transposeT(const T9& t) { return {t.xx, t.yx, t.zx, t.xy, t.yy, t.zy, t.xz, t.yz, t.zz}; }
// radialEvolution for Dim<3> (SmoothingScaleUtilities.hh): H in the frame
// whose first axis is nhat, the radial extent scaled by 1/s, the transverse
// block by r0/r1 -- (1,2) and (2,1) address the same element of a
// SymTensor, so yz is divided twice -- and back to the lab frame.
static ST radialEvolution3(const ST& Hi, const V3& nhat, double s, double r0, double r1) {
  const T9 Tp = rotationMatrix3(nhat);
  ST h = rotateS(Hi, Tp);
  const double fr = r1 * safeInvVar(r0);
  h.xx /= s;
  h.yy /= fr;
  h.yz /= fr;
  h.yz /= fr;
  h.zz /= fr;
  return rotateS(h, transposeT(Tp));
}

// Tensor DH/Dt of ASPH (SmoothingScaleUtilities.hh, smoothingScaleDerivative
// for Dim<3>): the rate of H under the velocity gradient with the rotation of
// the frame taken out.
static ST smoothingScaleDerivative3(const ST& H, const T9& D) {
  const double AA = H.xx * D.xy - H.xy * (D.xx - D.yy) + H.xz * D.zy - H.yy * D.yx - H.yz * D.zx;
  const double BB = H.xx * D.xz + H.xy * D.yz - H.xz * (D.xx - D.zz) - H.yz * D.yx - H.zz * D.zx;
  const double CC = H.xy * D.xz + H.yy * D.yz - H.yz * (D.yy - D.zz) - H.xz * D.xy - H.zz * D.zy;
  const double thpt = H.yy + H.zz;
  const double Ga = (H.xx + H.yy) * thpt - H.xz * H.xz;
  const double Gb = (H.yy + H.zz) * H.yz + H.xy * H.xz;
  const double Gc = (H.xx + H.zz) * thpt - H.xy * H.xy;
  const double Gd = thpt * AA + H.xz * CC;
  const double Ge = thpt * BB - H.xy * CC;
  const double ack = 1.0 / (Ga * Gc - Gb * Gb);
  const double Gdot = (Gc * Gd - Gb * Ge) * ack;
  const double Tdot = (Gb * Gd - Ga * Ge) * ack;
  const double Phidot = (H.xz * Gdot + H.xy * Tdot + CC) / thpt;
  ST r;
  r.xx = -H.xx * D.xx + H.xy * (Gdot - D.yx) - H.xz * (Tdot + D.zx);
  r.xy = H.yy * Gdot - H.yz * Tdot - H.xx * D.xy - H.xy * D.yy - H.xz * D.zy;
  r.xz = H.yz * Gdot - H.zz * Tdot - H.xx * D.xz - H.xy * D.yz - H.xz * D.zz;
  r.yy = H.yz * (Phidot - D.zy) - H.xy * (Gdot + D.xy) - H.yy * D.yy;
  r.yz = H.xy * Tdot - H.yy * Phidot - H.xz * D.xy - H.yz * D.yy - H.zz * D.zy;
  r.zz = H.xz * (Tdot - D.xz) - H.yz * (Phidot + D.yz) - H.zz * D.zz;
  return r;
}

//------------------------------------------------------------------------------
// Cubic B-spline (3-D), BSplineKernelInline.hh:28-93.
//------------------------------------------------------------------------------
struct BSpline3 {
  double A = 1.0 / M_PI;
  double extent = 2.0;
  double value(double eta, double Hdet) const {
    if (eta < 1.0) { const double eta2 = eta * eta; return A * Hdet * (1.0 - 1.5 * eta2 + 0.75 * eta2 * eta); }
    if (eta < 2.0) { const double d = 2.0 - eta; return A * Hdet * 0.25 * (d * d * d); }
    return 0.0;
  }
  double grad(double eta, double Hdet) const {
    if (eta < 1.0) return -A * Hdet * (3.0 - 2.25 * eta) * eta;
    if (eta < 2.0) { const double d = 2.0 - eta; return -A * Hdet * 0.75 * (d * d); }
    return 0.0;
  }
  double grad2(double eta, double Hdet) const {
    if (eta < 1.0) return -A * Hdet * (3 - 4.5 * eta);
    if (eta < 2.0) return A * Hdet * 1.5 * (2 - eta);
    return 0.0;
  }
};

//------------------------------------------------------------------------------
// QuadraticInterpolator (QuadraticInterpolator.cc:60-100 + Inline.hh).
//------------------------------------------------------------------------------
struct QuadInterp {
  size_t N1 = 0;
  double xmin = 0, xmax = 0, xstep = 0;
  vector<double> c;
  template <class F>
  void initialize(double x0_, double x1_, size_t n, const F& f) {
    if (n % 2 == 0) ++n;
    const double st = (x1_ - x0_) / (n - 1u);
    vector<double> y(n);
    for (size_t i = 0; i < n; ++i) y[i] = f(x0_ + i * st);
    N1 = (n - 1u) / 2u - 1u;
    xmin = x0_; xmax = x1_;
    xstep = (x1_ - x0_) / (N1 + 1u);
    c.assign(3 * (N1 + 1u), 0.0);
    for (size_t i0 = 0; i0 <= N1; ++i0) {
      const double a0 = xmin + i0 * xstep, a1 = a0 + 0.5 * xstep, a2 = a0 + xstep;
      // A = [[1,a0,a0^2],[1,a1,a1^2],[1,a2,a2^2]] ; X = A^{-1} B (cofactor inverse)
      const double m00 = 1.0, m01 = a0, m02 = a0 * a0;
      const double m10 = 1.0, m11 = a1, m12 = a1 * a1;
      const double m20 = 1.0, m21 = a2, m22 = a2 * a2;
      const double C00 = m11 * m22 - m12 * m21, C01 = m12 * m20 - m10 * m22, C02 = m10 * m21 - m11 * m20;
      const double det = m00 * C00 + m01 * C01 + m02 * C02;
      const double inv[3][3] = {
          {C00 / det, (m02 * m21 - m01 * m22) / det, (m01 * m12 - m02 * m11) / det},
          {C01 / det, (m00 * m22 - m02 * m20) / det, (m02 * m10 - m00 * m12) / det},
          {C02 / det, (m01 * m20 - m00 * m21) / det, (m00 * m11 - m01 * m10) / det}};
      const double B0 = y[2 * i0], B1 = y[2 * i0 + 1], B2 = y[2 * i0 + 2];
      for (int r = 0; r < 3; ++r) c[3 * i0 + r] = inv[r][0] * B0 + inv[r][1] * B1 + inv[r][2] * B2;
    }
  }
  size_t lowerBound(double x) const {
    return 3u * std::min(N1, size_t(std::max(0.0, x - xmin) / xstep));
  }
  double operator()(double x) const { const size_t i0 = lowerBound(x); return c[i0] + (c[i0 + 1] + c[i0 + 2] * x) * x; }
  double at(double x, size_t i0) const { return c[i0] + (c[i0 + 1] + c[i0 + 2] * x) * x; }
};

//------------------------------------------------------------------------------
// CubicHermiteInterpolator (CubicHermiteInterpolator.cc, ViewInline.hh).
//------------------------------------------------------------------------------
struct HermiteInterp {
  size_t N = 0;
  double xmin = 0, xmax = 0, xstep = 0;
  vector<double> v;   // [0,N): values, [N,2N): gradients
  template <class F>
  void initialize(double x0_, double x1_, size_t n, const F& f) {
    const double st = (x1_ - x0_) / (n - 1u);
    vector<double> y(n);
    for (size_t i = 0; i < n; ++i) y[i] = f(x0_ + i * st);
    N = n; xmin = x0_; xmax = x1_;
    xstep = (x1_ - x0_) / (N - 1u);
    v.assign(2 * N, 0.0);
    for (size_t i = 0; i < N; ++i) v[i] = y[i];
    gradientKnots();
  }
  // Tridiagonal system of CubicHermiteInterpolator::initializeGradientKnots,
  // solved with the Thomas algorithm.
  void gradientKnots() {
    vector<double> a(N, 0.0), b(N, 4.0), cc(N, 0.0), d(N, 0.0);
    cc[0] = -1.0; a[N - 1] = -1.0;
    d[0] = 3.0 * (v[1] - v[0]) / xstep;
    d[N - 1] = 3.0 * (v[N - 1] - v[N - 2]) / xstep;
    for (size_t k = 1; k + 1 < N; ++k) { a[k] = -0.5; cc[k] = -0.5; d[k] = 1.5 * (v[k + 1] - v[k - 1]) / xstep; }
    vector<double> cp(N), dp(N);
    cp[0] = cc[0] / b[0]; dp[0] = d[0] / b[0];
    for (size_t k = 1; k < N; ++k) {
      const double m = b[k] - a[k] * cp[k - 1];
      cp[k] = cc[k] / m;
      dp[k] = (d[k] - a[k] * dp[k - 1]) / m;
    }
    v[N + N - 1] = dp[N - 1];
    for (size_t k = N - 1; k-- > 0;) v[N + k] = dp[k] - cp[k] * v[N + k + 1];
  }
  void makeMonotonic() {
    vector<double> cg(N - 1);
    const double dxInv = 1.0 / xstep;
    for (size_t k = 0; k + 1 < N; ++k) cg[k] = (v[k + 1] - v[k]) * dxInv;
    auto g = [&](size_t i) -> double& { return v[N + i]; };
    for (size_t k = 1; k + 1 < N; ++k) {
      if (cg[k - 1] * cg[k] <= 0.0) g(k) = 0.0;
      if (cg[k] == 0.0) { g(k) = 0.0; g(k + 1) = 0.0; }
    }
    bool done = false;
    while (!done) {
      done = true;
      for (size_t k = 0; k + 1 < N; ++k) {
        double alpha = g(k) / cg[k], beta = g(k + 1) / cg[k];
        if (alpha < 0.0) { g(k) = 0.0; alpha = 0.0; done = false; }
        if (beta < 0.0) { g(k + 1) = 0.0; beta = 0.0; done = false; }
        const double tau = 3.0 / std::sqrt(alpha * alpha + beta * beta);
        if (tau < 1.0) { g(k) = 0.99 * tau * alpha * cg[k]; g(k + 1) = 0.99 * tau * beta * cg[k]; done = false; }
      }
    }
  }
  size_t lowerBound(double x) const { return std::min(N - 2u, size_t(std::max(0.0, x - xmin) / xstep)); }
  double eval(double x, size_t i0) const {
    const double t = std::max(0.0, std::min(1.0, (x - xmin - i0 * xstep) / xstep));
    const double t2 = t * t, t3 = t * t2;
    return ((2.0 * t3 - 3.0 * t2 + 1.0) * v[i0] + (-2.0 * t3 + 3.0 * t2) * v[i0 + 1u] +
            xstep * ((t3 - 2.0 * t2 + t) * v[N + i0] + (t3 - t2) * v[N + i0 + 1u]));
  }
  double operator()(double x) const {
    if (x < xmin) return v[0] + v[N] * (x - xmin);
    if (x > xmax) return v[N - 1u] + v[2u * N - 1u] * (x - xmin);
    return eval(x, lowerBound(x));
  }
};

template <class F>
static double bisectRoot(const F& f, double xmin, double xmax, double xacc = 1.0e-15, double yacc = 1.0e-10,
                         unsigned maxIter = 100u) {
  const double fxmin = f(xmin), fxmax = f(xmax);
  if (fuzzyEqual(fxmin, 0.0, yacc)) return xmin;
  if (fuzzyEqual(fxmax, 0.0, yacc)) return xmax;
  double x0, x1;
  if (fxmin < 0.0) { x0 = xmin; x1 = xmax; } else { x0 = xmax; x1 = xmin; }
  unsigned iter = 0;
  while (iter++ < maxIter) {
    const double dx = 0.5 * (x1 - x0);
    const double r = x0 + dx;
    if (std::fabs(dx) <= xacc) return r;
    const double fr = f(r);
    if (fuzzyEqual(fr, 0.0, yacc)) return r;
    if (fr < 0.0) x0 = r; else x1 = r;
  }
  return 0.0;
}

//------------------------------------------------------------------------------
// NBSplineKernel<Dim<3>> (src/Kernel/NBSplineKernel.cc:20-118,
// NBSplineKernelInline.hh:40-99): the centred cardinal B-spline of the given
// order, sum_i (-1)^i C(k, i) (eta - i + k/2)_+^(k-1) / (k-1)! with
// k = order + 1, extent (order + 1) / 2 (integer division) and the volume
// normalisation from Simpson's rule (10,000 bins) of 4 pi r^2 W(r)
// (VolumeIntegrationFunctions.cc, simpsonsIntegration.hh:19-50).
//------------------------------------------------------------------------------
struct NBSpline3 {
  int order = 3;
  double A = 1.0;
  double extent = 2.0;
  static int factorial(int n) {
    if (n < 0) return std::numeric_limits<int>::max();
    int r = 1;
    for (int i = 1; i < n + 1; ++i) r *= i;
    return r;
  }
  static int binomial(int n, int m) { return factorial(n) / (factorial(n - m) * factorial(m)); }
  static double oneSided(double x, int e) { return x >= 0.0 ? std::pow(x, e) : 0.0; }
  double series(double eta, int e) const {
    const int k = order + 1;
    const double halfk = 0.5 * k;
    double r = 0.0;
    for (int i = 0; i <= k; ++i) r += std::pow(-1.0, i) * binomial(k, i) * oneSided(eta - i + halfk, e);
    return r;
  }
  explicit NBSpline3(int o) : order(o) {
    extent = (double)((order + 1) / 2);
    A = 1.0;
    const int nb = 10000;
    const double dx = (extent - 0.0) / nb;
    double sum = 0.0;
    for (int i = 0; i < nb + 1; ++i) {
      const double r = 0.0 + i * dx;
      const double f = 4.0 * M_PI * r * r * value(r, 1.0);
      if (i == 0 || i == nb) sum += f;
      else if (i % 2 == 0) sum += 2.0 * f;
      else sum += 4.0 * f;
    }
    sum *= dx / 3.0;
    A = 1.0 / sum;
  }
  double value(double eta, double Hdet) const {
    if (eta >= extent) return 0.0;
    const int k1 = std::max(0, order);
    return series(eta, k1) * (A * Hdet / factorial(k1));
  }
  double grad(double eta, double Hdet) const {
    if (eta >= extent) return 0.0;
    const int k2 = std::max(-1, order - 1);
    return series(eta, k2) * (A * Hdet / factorial(k2));
  }
  double grad2(double eta, double Hdet) const {
    if (eta >= extent) return 0.0;
    const int k3 = std::max(-2, order - 2);
    return series(eta, k3) * (A * Hdet / factorial(k3));
  }
};

//------------------------------------------------------------------------------
// WendlandC2Kernel / WendlandC4Kernel, 3-D forms
// (src/Kernel/WendlandC2KernelInline.hh:40-90, WendlandC4KernelInline.hh:28-90).
//------------------------------------------------------------------------------
struct WendlandC2_3 {
  double A = 21.0 / (2.0 * M_PI), extent = 1.0;
  double value(double e, double Hdet) const { return A * Hdet * (std::pow(1.0 - e, 4) * (1.0 + 4.0 * e)) * (e < 1.0 ? 1.0 : 0.0); }
  double grad(double e, double Hdet) const { return A * Hdet * (20.0 * std::pow(e - 1.0, 3) * e) * (e < 1.0 ? 1.0 : 0.0); }
  double grad2(double e, double Hdet) const { return A * Hdet * (20.0 * std::pow(e - 1.0, 2) * (4.0 * e - 1.0)) * (e < 1.0 ? 1.0 : 0.0); }
};
struct WendlandC4_3 {
  double A = 495.0 / (32.0 * M_PI), extent = 1.0;
  double value(double e, double Hdet) const {
    return A * Hdet * (std::pow(1.0 - e, 6) * (1.0 + 6.0 * e + (35.0 / 3.0) * (e * e))) * (e < 1.0 ? 1.0 : 0.0);
  }
  double grad(double e, double Hdet) const {
    return A * Hdet * ((56.0 / 3.0) * std::pow(e - 1.0, 5) * e * (5.0 * e + 1.0)) * (e < 1.0 ? 1.0 : 0.0);
  }
  double grad2(double e, double Hdet) const {
    return A * Hdet * ((56.0 / 3.0) * std::pow(e - 1.0, 4) * (35.0 * (e * e) - 4.0 * e - 1.0)) * (e < 1.0 ? 1.0 : 0.0);
  }
};

//------------------------------------------------------------------------------
// TableKernel<Dim<3>> (TableKernel.cc:169-209).
//------------------------------------------------------------------------------
struct TableKernel {
  QuadInterp W, gW, g2W;
  HermiteInterp nperhLookup, wsumLookup;
  double extent = 2.0, minNperh = 0, maxNperh = 0;
  int numPoints = 0;
  double kernelValueSPH(double eta) const { return eta < extent ? std::fabs(gW(eta)) : 0.0; }
  double kernelValue(double eta, double Hdet) const { return eta < extent ? Hdet * W(eta) : 0.0; }
  double gradValue(double eta, double Hdet) const { return eta < extent ? Hdet * gW(eta) : 0.0; }
  void kernelAndGradValue(double eta, double Hdet, double& w, double& g) const {
    if (eta < extent) { const size_t i0 = W.lowerBound(eta); w = Hdet * W.at(eta, i0); g = Hdet * gW.at(eta, i0); }
    else { w = 0.0; g = 0.0; }
  }
  double sumKernelValues(double nPerh) const {          // TableKernel.cc:53-66
    const double deta = 1.0 / nPerh;
    double result = 0.0, etar = deta;
    while (etar < extent) {
      const double q = etar / deta;
      result += 4.0 * M_PI * (q * q) * kernelValueSPH(etar);
      etar += deta;
    }
    return std::pow(result, 1.0 / 3.0);
  }
  void build(int nPoints, double minNperh_ = 0.25, double maxNperh_ = 64.0) {
    buildFrom(BSpline3(), nPoints, minNperh_, maxNperh_);
  }
  template <class K>
  void buildFrom(const K& k, int nPoints, double minNperh_ = 0.25, double maxNperh_ = 64.0) {
    numPoints = nPoints;
    extent = k.extent;
    W.initialize(0.0, k.extent, nPoints, [&](double x) { return k.value(x, 1.0); });
    gW.initialize(0.0, k.extent, nPoints, [&](double x) { return k.grad(x, 1.0); });
    g2W.initialize(0.0, k.extent, nPoints, [&](double x) { return k.grad2(x, 1.0); });
    maxNperh = maxNperh_;
    minNperh = std::max(minNperh_, 1.1 / k.extent);
    if (maxNperh <= minNperh) maxNperh = 4.0 * minNperh;
    wsumLookup.initialize(minNperh, maxNperh, nPoints, [&](double x) { return sumKernelValues(x); });
    nperhLookup.initialize(wsumLookup(minNperh), wsumLookup(maxNperh), nPoints, [&](double Wsum) {
      return bisectRoot([&](double nperh) { return wsumLookup(nperh) - Wsum; }, minNperh, maxNperh);
    });
    wsumLookup.makeMonotonic();
    nperhLookup.makeMonotonic();
  }
  double equivalentNodesPerSmoothingScale(double Wsum) const { return std::max(0.0, nperhLookup(Wsum)); }
  double equivalentWsum(double nPerh) const { return std::max(0.0, wsumLookup(nPerh)); }
};

//------------------------------------------------------------------------------
// Problem description.
//------------------------------------------------------------------------------
struct NodeListParams {
  double nPerh = 1.51, hmin = 1e-20, hmax = 1e20, rhoMin = 1e-10, rhoMax = 1e10, gamma = 5.0 / 3.0;
  double hminratio = 0.1;   // NodeList::hminratio (FluidNodeList default 0.1)
  double minP = -std::numeric_limits<double>::max(), maxP = std::numeric_limits<double>::max();
};

// One plane pair (periodic) or one plane (reflecting), axis-aligned.
struct Boundary {
  int type = 0;         // 0 periodic, 1 reflecting
  int axis = 0;
  double lo = 0, hi = 0;   // periodic: the two planes; reflecting: wall at lo (normal +) or hi (normal -)
  int wallHigh = 0;        // reflecting: 0 -> wall at lo with normal +axis, 1 -> wall at hi with normal -axis
  // ghost bookkeeping: parallel lists, per sub-boundary
  vector<int> control[2], ghost[2];
};

struct Config {
  int numTablePoints = 1000;
  double cfl = 0.25;
  int useVelocityMagnitudeForDt = 0;
  int compatibleEnergy = 1;
  int gradhCorrection = 1;
  int XSPH = 0;
  int correctVelocityGradient = 1;
  int sumMassDensityOverAllNodeLists = 1;
  int densityUpdate = 0;     // 0 RigorousSumDensity, 1 IntegrateDensity
  double epsTensile = 0.0, nTensile = 4.0;
  double Cl = 1.0, Cq = 1.0, eps2 = 1.0e-2;
  int linearInExpansion = 0, quadraticInExpansion = 0;
  // 0 MonaghanGingoldViscosity, 1 LimitedMonaghanGingoldViscosity
  int viscosity = 0;
  double etaCritFrac = 1.0, etaFoldFrac = 0.2;
  // 0 SPHSmoothingScale, 1 ASPHClassicSmoothingScale (SPHHydros.py:130-138, ASPH="CLASSIC")
  int smoothingScale = 0;
  int fixShape = 0;          // ASPHClassicSmoothingScale fixShape
  int radialOnly = 0;        // ASPHClassicSmoothingScale radialOnly (ASPHRadialFunctor defaults: about the origin)
  int hUpdate = 0;           // HEvolutionType: 0 IdealH, 1 IntegrateH, 2 FixedH (SmoothingScaleBase.cc:53-82)
  int evolveTotalEnergy = 0; // SPH evolveTotalEnergy (SPH.cc:105-108, 541)
  int hydro = 0;             // 0 SPH, 1 CRKSPH (CRKSPHHydros.py:9-110, LinearOrder)
  int kernel = 0;            // base kernel of the TableKernel: 0 BSplineKernel, 1 NBSplineKernel(kernelOrder),
                             // 2 WendlandC2Kernel, 3 WendlandC4Kernel
  int kernelOrder = 3;
  int rkVolume = 1;          // RKVolumeType: 0 RKMassOverDensity, 1 RKSumVolume, 4 HVolume
  double dtMin = 0.0, dtMax = std::numeric_limits<double>::max(), dtGrowth = 2.0;
  int gravity = 0;
  double G = 1.0, softening = 0.01, opening = 0.5, ftimestep = 0.1;
};

static inline double& comp(V3& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
static inline double compc(const V3& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// mapPositionThroughPlanes (mapPositionThroughPlanes.hh:17-27) for an
// axis-aligned plane pair; only the axis coordinate changes.  enter/exit
// planes are (coordinate w, normal sign s).
static inline double mapCoord(double p, double wEnter, double sEnter, double wExit, double sExit) {
  // closestPointOnPlane: p + ((origin - p).n) n  (pointDistances.hh:69-74)
  const double dotv = (wExit - p) * sExit;
  const double p0 = p + dotv * sExit;
  const double s = (p - wEnter) * sEnter;          // enterPlane.signedDistance
  return p0 - s * sExit;
}

struct Problem {
  Config cfg;
  TableKernel W;
  vector<NodeListParams> lists;
  vector<Boundary> bcs;
  int nInt = 0, nTot = 0;
  double time = 0.0, lastDt = 1.0e-5;
  int cycle = 0;
  double dtMultiplier = 1.0;

  // state (size nTot)
  vector<V3> pos, vel;
  vector<double> mass, rho, eps, P, cs, omega;
  vector<ST> H;
  // CRKSPH: the RK volume and the LinearOrder corrections (C_0..3, then
  // dC/dx, dC/dy, dC/dz, 4 each: RKUtilities offsetGradC)
  typedef std::array<double, 16> RKC;
  vector<double> vol;
  vector<RKC> rkc;
  vector<int> list;
  // ghost transform bookkeeping: for each ghost: control index and per-axis code
  vector<int> ctrl;      // flat control index (ultimately an internal node)
  vector<int> image;     // per-axis 2-bit codes: 0 none, 1 low image / lo mirror, 2 high image / hi mirror

  // connectivity
  vector<std::pair<int, int>> pairs;
  vector<int> numNeighbors;   // per internal node
  vector<vector<int>> neighbors;  // per internal node: flat neighbor indices (for the numNeighbors contract / tests)

  // derivatives (size nTot)
  vector<double> rhoSum, normalization, DrhoDt, DepsDt, maxQ, effQ, XSPHWeightSum, massZeroth, DepsDtCompat;
  vector<V3> DxDt, DvDt, gradRho, XSPHDeltaV, massFirst, DvDtGrav;
  vector<T9> DvDx, localDvDx, M, localM;
  vector<ST> DHDt, Hideal, massSecond;
  vector<double> radius0;   // radialOnly: |x| at preStepInitialize (SmoothingScaleBase.cc:104-121)
  // ArtificialViscosityVelocityGradient: the Q's copy of DvDx, a state field
  // (ArtificialViscosityHandle.cc:52,78-79; zero until the first copy)
  vector<T9> DvDxQ;
  vector<V3> pairAccel;   // per pair
  vector<double> potential;
  double extraEnergy = 0.0, dtMinAcc = std::numeric_limits<double>::max();
  std::string dtReason;

  void resizeAll(int n) {
    pos.resize(n); vel.resize(n); mass.resize(n); rho.resize(n); eps.resize(n); P.resize(n); cs.resize(n);
    omega.resize(n, 1.0); H.resize(n); list.resize(n); vol.resize(n, 0.0); rkc.resize(n, RKC{});
  }
  void resizeDerivs() {
    const int n = nTot;
    auto z = [&](vector<double>& v) { v.assign(n, 0.0); };
    auto zv = [&](vector<V3>& v) { v.assign(n, V3{}); };
    auto zt = [&](vector<T9>& v) { v.assign(n, T9{}); };
    auto zs = [&](vector<ST>& v) { v.assign(n, ST{}); };
    if ((int)rhoSum.size() != nInt) {
      z(rhoSum); z(normalization); z(DrhoDt); z(DepsDt); z(maxQ); z(effQ); z(XSPHWeightSum); z(massZeroth); z(DepsDtCompat);
      zv(DxDt); zv(DvDt); zv(gradRho); zv(XSPHDeltaV); zv(massFirst); zv(DvDtGrav);
      zt(DvDx); zt(localDvDx); zt(M); zt(localM); zs(DHDt); zs(Hideal); zs(massSecond); z(potential);
    }
  }
  // Resize derivative arrays to nTot, preserving internal values (ghost
  // entries are scratch).
  template <class T> static void keepResize(vector<T>& v, int nInt_, int nTot_) { v.resize(nTot_); (void)nInt_; }
  void derivsToTotal() {
    keepResize(rhoSum, nInt, nTot); keepResize(normalization, nInt, nTot); keepResize(DrhoDt, nInt, nTot);
    keepResize(DepsDt, nInt, nTot); keepResize(maxQ, nInt, nTot); keepResize(effQ, nInt, nTot);
    keepResize(XSPHWeightSum, nInt, nTot); keepResize(massZeroth, nInt, nTot); keepResize(DepsDtCompat, nInt, nTot);
    keepResize(DxDt, nInt, nTot); keepResize(DvDt, nInt, nTot); keepResize(gradRho, nInt, nTot);
    keepResize(XSPHDeltaV, nInt, nTot); keepResize(massFirst, nInt, nTot); keepResize(DvDtGrav, nInt, nTot);
    keepResize(DvDx, nInt, nTot); keepResize(localDvDx, nInt, nTot); keepResize(M, nInt, nTot); keepResize(localM, nInt, nTot);
    keepResize(DHDt, nInt, nTot); keepResize(Hideal, nInt, nTot); keepResize(massSecond, nInt, nTot);
    keepResize(potential, nInt, nTot);
    if ((int)DvDxQ.size() < nInt) DvDxQ.assign(nInt, T9{});
    DvDxQ.resize(nTot);
  }
  // ArtificialViscosityHandle::postStateUpdate (ArtificialViscosityHandle.cc:167-183):
  // without a rigorous gradient the Q copies the hydro's DvDx; its ghost
  // values follow at the next applyGhostBoundaries (tensors reflect as R T R).
  void copyQVelocityGradient() {
    if (cfg.viscosity != 1) return;
    for (int i = 0; i < nInt; ++i) DvDxQ[i] = DvDx[i];
    applyGhostQGradient();
  }
  // ArtificialViscosityHandle::applyGhostBoundaries (ArtificialViscosityHandle.cc:96-110)
  void applyGhostQGradient() {
    if (cfg.viscosity != 1 || (int)DvDxQ.size() < nTot) return;
    applyGhostField(DvDxQ, [](T9& t, int a) {
      if (a == 0) { t.xy = -t.xy; t.xz = -t.xz; t.yx = -t.yx; t.zx = -t.zx; }
      else if (a == 1) { t.xy = -t.xy; t.yx = -t.yx; t.yz = -t.yz; t.zy = -t.zy; }
      else { t.xz = -t.xz; t.zx = -t.zx; t.yz = -t.yz; t.zy = -t.zy; }
    });
  }

  double hmaxOf(const ST& Hi) const { return 1.0 / minElem(eigenValuesS(Hi)); }

  //----------------------------------------------------------------------------
  // Ghost nodes: Integrator::setGhostNodes -> Boundary::setAllGhostNodes ->
  // PlanarBoundary::setGhostNodes (findNodesTouchingThroughPlanes).
  //----------------------------------------------------------------------------
  void planeSpec(const Boundary& b, int sub, double& wEnter, double& sEnter, double& wExit, double& sExit) const {
    if (b.type == 0) {
      if (sub == 0) { wEnter = b.lo; sEnter = 1.0; wExit = b.hi; sExit = -1.0; }   // mPlane1Boundary(plane1, plane2)
      else          { wEnter = b.hi; sEnter = -1.0; wExit = b.lo; sExit = 1.0; }   // mPlane2Boundary(plane2, plane1)
    } else {
      const double w = b.wallHigh ? b.hi : b.lo, s = b.wallHigh ? -1.0 : 1.0;
      wEnter = wExit = w; sEnter = sExit = s;
    }
  }
  void setGhostNodes() {
    nTot = nInt;
    resizeAll(nInt);
    ctrl.assign(nInt, -1);
    image.assign(nInt, 0);
    const double ext = W.extent;
    const int nLists = (int)lists.size();
    for (auto& b : bcs) {
      const int nsub = b.type == 0 ? 2 : 1;
      for (int sub = 0; sub < nsub; ++sub) {
        b.control[sub].clear(); b.ghost[sub].clear();
        double wEn, sEn, wEx, sEx;
        planeSpec(b, sub, wEn, sEn, wEx, sEx);
        for (int L = 0; L < nLists; ++L) {
          const int n = nTot;
          double hmax = 0.0;
          for (int i = 0; i < n; ++i) {
            if (list[i] != L) continue;
            const double p = compc(pos[i], b.axis);
            const double hmaxi = hmaxOf(H[i]);
            const double dEx = std::fabs((p - wEx) * sEx), dEn = std::fabs((p - wEn) * sEn);
            if (hmaxi > hmax && std::min(dEx, dEn) < ext * hmaxi) hmax = hmaxi;
          }
          vector<int> controls;
          if (hmax > 0.0) {
            for (int i = 0; i < n; ++i) {
              if (list[i] != L) continue;
              const double disti = ((compc(pos[i], b.axis) - wEx) * sEx) / hmax;
              if (disti >= 0.0 && disti <= ext) controls.push_back(i);
            }
          }
          // append ghosts
          for (int c : controls) {
            const int g = nTot++;
            pos.push_back(pos[c]); vel.push_back(vel[c]); mass.push_back(mass[c]); rho.push_back(rho[c]);
            eps.push_back(eps[c]); P.push_back(P[c]); cs.push_back(cs[c]); omega.push_back(omega[c]);
            H.push_back(H[c]); list.push_back(list[c]); vol.push_back(vol[c]); rkc.push_back(rkc[c]);
            const int root = ctrl[c] < 0 ? c : ctrl[c];
            ctrl.push_back(root);
            const int code = (b.type == 0 ? (sub == 0 ? 1 : 2) : (b.wallHigh ? 2 : 1));
            int im = image[c];
            im &= ~(3 << (2 * b.axis));
            im |= code << (2 * b.axis);
            image.push_back(im);
            // position: mapPosition(pos(control), mExitPlane, mEnterPlane);
            // H: applyGhostBoundary(Hfield) (PlanarBoundary::updateGhostNodes,
            // PlanarBoundary.cc:291-327), reflected through a wall
            comp(pos[g], b.axis) = mapCoord(compc(pos[c], b.axis), wEx, sEx, wEn, sEn);
            if (b.type == 1) {
              ST& h = H[g];
              if (b.axis == 0) { h.xy = -h.xy; h.xz = -h.xz; }
              else if (b.axis == 1) { h.xy = -h.xy; h.yz = -h.yz; }
              else { h.xz = -h.xz; h.yz = -h.yz; }
            }
            b.control[sub].push_back(c);
            b.ghost[sub].push_back(g);
          }
        }
      }
    }
    derivsToTotal();
  }
  // applyGhostBoundaries for the state fields (boundary by boundary).
  void applyGhostState() {
    for (auto& b : bcs) {
      const int nsub = b.type == 0 ? 2 : 1;
      for (int sub = 0; sub < nsub; ++sub) {
        double wEn, sEn, wEx, sEx;
        planeSpec(b, sub, wEn, sEn, wEx, sEx);
        for (size_t k = 0; k < b.control[sub].size(); ++k) {
          const int c = b.control[sub][k], g = b.ghost[sub][k];
          pos[g] = pos[c];
          comp(pos[g], b.axis) = mapCoord(compc(pos[c], b.axis), wEx, sEx, wEn, sEn);
          H[g] = H[c]; mass[g] = mass[c]; rho[g] = rho[c]; eps[g] = eps[c]; P[g] = P[c]; cs[g] = cs[c];
          omega[g] = omega[c]; vel[g] = vel[c];
          if (cfg.hydro == 1) vol[g] = vol[c];
          if (b.type == 1) {
            comp(vel[g], b.axis) = -compc(vel[c], b.axis);
            // (R H R).Symmetric(): flips the off-diagonal terms that touch the axis
            ST h = H[c];
            if (b.axis == 0) { h.xy = -h.xy; h.xz = -h.xz; }
            else if (b.axis == 1) { h.xy = -h.xy; h.yz = -h.yz; }
            else { h.xz = -h.xz; h.yz = -h.yz; }
            H[g] = h;
          }
        }
      }
    }
    applyGhostQGradient();
  }
  template <class T, class Fn>
  void applyGhostField(vector<T>& f, Fn reflect) {
    for (auto& b : bcs) {
      const int nsub = b.type == 0 ? 2 : 1;
      for (int sub = 0; sub < nsub; ++sub)
        for (size_t k = 0; k < b.control[sub].size(); ++k) {
          const int c = b.control[sub][k], g = b.ghost[sub][k];
          f[g] = f[c];
          if (b.type == 1) reflect(f[g], b.axis);
        }
    }
  }
  void applyGhostScalar(vector<double>& f) { applyGhostField(f, [](double&, int) {}); }
  void applyGhostVector(vector<V3>& f) { applyGhostField(f, [](V3& v, int a) { comp(v, a) = -comp(v, a); }); }

  //----------------------------------------------------------------------------
  // ConnectivityMap::computeConnectivity (pair criterion and pair list).
  //----------------------------------------------------------------------------
  void computeConnectivity() {
    const double ext = W.extent, ext2 = ext * ext;
    double hmaxAll = 0.0;
    V3 lo{1e300, 1e300, 1e300}, hi{-1e300, -1e300, -1e300};
    for (int i = 0; i < nTot; ++i) {
      hmaxAll = std::max(hmaxAll, hmaxOf(H[i]));
      lo.x = std::min(lo.x, pos[i].x); lo.y = std::min(lo.y, pos[i].y); lo.z = std::min(lo.z, pos[i].z);
      hi.x = std::max(hi.x, pos[i].x); hi.y = std::max(hi.y, pos[i].y); hi.z = std::max(hi.z, pos[i].z);
    }
    double cell = std::max(ext * hmaxAll * 1.0001, 1e-300);
    int nc[3];
    double L[3] = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
    for (int a = 0; a < 3; ++a) nc[a] = std::max(1, (int)std::floor(L[a] / cell) + 1);
    while ((double)nc[0] * nc[1] * nc[2] > 8.0e7) { cell *= 1.26; for (int a = 0; a < 3; ++a) nc[a] = std::max(1, (int)std::floor(L[a] / cell) + 1); }
    auto cidx = [&](const V3& p, int c[3]) {
      const double q[3] = {p.x - lo.x, p.y - lo.y, p.z - lo.z};
      for (int a = 0; a < 3; ++a) c[a] = std::min(nc[a] - 1, std::max(0, (int)std::floor(q[a] / cell)));
    };
    const size_t ncell = (size_t)nc[0] * nc[1] * nc[2];
    vector<int> head(ncell + 1, 0), order(nTot);
    vector<int> cellOf(nTot);
    for (int i = 0; i < nTot; ++i) { int c[3]; cidx(pos[i], c); cellOf[i] = (c[2] * nc[1] + c[1]) * nc[0] + c[0]; head[cellOf[i] + 1]++; }
    for (size_t k = 0; k < ncell; ++k) head[k + 1] += head[k];
    { vector<int> fill(head.begin(), head.end() - 1); for (int i = 0; i < nTot; ++i) order[fill[cellOf[i]]++] = i; }
    neighbors.assign(nInt, {});
    numNeighbors.assign(nInt, 0);
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = omp_get_max_threads();
#endif
    vector<vector<std::pair<int, int>>> tp(nthreads);
#pragma omp parallel
    {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      auto& mine = tp[tid];
#pragma omp for schedule(dynamic, 256)
      for (int i = 0; i < nInt; ++i) {
        int c[3]; cidx(pos[i], c);
        const V3 ri = pos[i]; const ST Hi = H[i];
        auto& nb = neighbors[i];
        for (int dz = -1; dz <= 1; ++dz) for (int dy = -1; dy <= 1; ++dy) for (int dx = -1; dx <= 1; ++dx) {
          const int x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
          if (x < 0 || y < 0 || z < 0 || x >= nc[0] || y >= nc[1] || z >= nc[2]) continue;
          const int cc = (z * nc[1] + y) * nc[0] + x;
          for (int k = head[cc]; k < head[cc + 1]; ++k) {
            const int j = order[k];
            if (j == i) continue;
            const V3 rij = sub(ri, pos[j]);
            const double eta2i = mag2(dotSV(Hi, rij));
            const double eta2j = mag2(dotSV(H[j], rij));
            if (eta2i <= ext2 || eta2j <= ext2) {
              nb.push_back(j);
              if (j > i) mine.push_back({i, j});   // calculatePairInteraction (one NodeList ordering)
            }
          }
        }
        std::sort(nb.begin(), nb.end());
        numNeighbors[i] = (int)nb.size();
      }
    }
    pairs.clear();
    for (auto& v : tp) pairs.insert(pairs.end(), v.begin(), v.end());
    std::sort(pairs.begin(), pairs.end());
    pairAccel.assign(pairs.size(), V3{});
  }

  //----------------------------------------------------------------------------
  // Equation of state (GammaLawGas) -- PressurePolicy / SoundSpeedPolicy.
  //----------------------------------------------------------------------------
  double pressure(int i) const {
    const auto& L = lists[list[i]];
    double p = (L.gamma - 1.0) * rho[i] * eps[i];
    return p < L.minP ? L.minP : (p > L.maxP ? L.maxP : p);
  }
  double soundSpeed(int i) const {
    const auto& L = lists[list[i]];
    return std::sqrt(std::max(0.0, L.gamma * (L.gamma - 1.0) * eps[i]));
  }
  void updateEOS(int n) {
    for (int i = 0; i < n; ++i) { P[i] = pressure(i); cs[i] = soundSpeed(i); }
  }

  //----------------------------------------------------------------------------
  // Thread-private accumulation helper (FieldList::threadCopy/threadReduce).
  //----------------------------------------------------------------------------
  template <class T, class Body>
  static void pairSweep(size_t npairs, vector<T>& out, int n, Body body) {
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = omp_get_max_threads();
#endif
    vector<vector<T>> priv(nthreads, vector<T>(n));
#pragma omp parallel
    {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      auto& p = priv[tid];
#pragma omp for schedule(static)
      for (long kk = 0; kk < (long)npairs; ++kk) body(kk, p);
    }
    for (int t = 0; t < nthreads; ++t)
      for (int i = 0; i < n; ++i) out[i] += priv[t][i];
  }

  //----------------------------------------------------------------------------
  // computeSPHSumMassDensity (computeSPHSumMassDensity.cc:15-87).
  //----------------------------------------------------------------------------
  void sumMassDensity() {
    vector<double> rhoNew(nTot, 0.0);
    for (int i = 0; i < nInt; ++i) {
      const double Hdet = detS(H[i]);
      const V3 etaii = dotSV(H[i], pos[i]);
      rhoNew[i] = mass[i] * W.kernelValue(mag(sub(etaii, etaii)), Hdet);
    }
    vector<double> acc(nTot, 0.0);
    pairSweep(pairs.size(), acc, nTot, [&](long k, vector<double>& p) {
      const int i = pairs[k].first, j = pairs[k].second;
      const double Hdeti = detS(H[i]), Hdetj = detS(H[j]);
      const double Wi = W.kernelValue(mag(sub(dotSV(H[i], pos[i]), dotSV(H[i], pos[j]))), Hdeti);
      const double Wj = W.kernelValue(mag(sub(dotSV(H[j], pos[i]), dotSV(H[j], pos[j]))), Hdetj);
      const bool same = list[i] == list[j];
      p[i] += (same ? mass[j] : mass[i]) * Wj;
      p[j] += (same ? mass[i] : mass[j]) * Wi;
    });
    for (int i = 0; i < nInt; ++i) rho[i] = rhoNew[i] + acc[i];
    applyGhostScalar(rho);
  }

  //----------------------------------------------------------------------------
  // computeSPHOmegaGradhCorrection (computeSPHOmegaGradhCorrection.cc:15-116).
  //----------------------------------------------------------------------------
  void omegaGradh() {
    const double W0 = W.kernelValue(0.0, 1.0);
    struct Acc { double w = 0, g = 0; Acc& operator+=(const Acc& o) { w += o.w; g += o.g; return *this; } };
    vector<Acc> acc(nTot);
    pairSweep(pairs.size(), acc, nTot, [&](long k, vector<Acc>& p) {
      const int i = pairs[k].first, j = pairs[k].second;
      const V3 rij = sub(pos[i], pos[j]);
      const double etai = mag(dotSV(H[i], rij)), etaj = mag(dotSV(H[j], rij));
      double Wi, gWi, Wj, gWj;
      W.kernelAndGradValue(etai, detS(H[i]), Wi, gWi);
      W.kernelAndGradValue(etaj, detS(H[j]), Wj, gWj);
      p[i].w += Wi; p[j].w += Wj;
      p[i].g += etai * gWi; p[j].g += etaj * gWj;
    });
    for (int i = 0; i < nInt; ++i) {
      if (numNeighbors[i] == 0) { omega[i] = 1.0; continue; }
      double o = acc[i].w;
      o += detS(H[i]) * W0;
      omega[i] = std::max(1.0e-30, -acc[i].g / (3 * o));
    }
    applyGhostScalar(omega);
  }

  //----------------------------------------------------------------------------
  // SPH::evaluateDerivativesImpl (SPH.cc:166-555) for a Scalar Q
  // (MonaghanGingoldViscosity::QPiij), followed by
  // SPHSmoothingScale::evaluateDerivatives (SPHSmoothingScale.cc:101-275).
  //----------------------------------------------------------------------------
  struct PairAcc {
    double rhoSum = 0, norm = 0, DepsDt = 0, maxQ = 0, effQ = 0, xsphW = 0, m0 = 0;
    V3 DvDt, gradRho, xsphDV, m1;
    T9 DvDx, localDvDx, M, localM;
    ST m2;
    PairAcc& operator+=(const PairAcc& o) {
      rhoSum += o.rhoSum; norm += o.norm; DepsDt += o.DepsDt; maxQ = std::max(maxQ, o.maxQ); effQ += o.effQ;
      xsphW += o.xsphW; m0 += o.m0; addS(m2, o.m2);
      DvDt = add(DvDt, o.DvDt); gradRho = add(gradRho, o.gradRho); xsphDV = add(xsphDV, o.xsphDV); m1 = add(m1, o.m1);
      addT(DvDx, o.DvDx); addT(localDvDx, o.localDvDx); addT(M, o.M); addT(localM, o.localM);
      return *this;
    }
  };
  static V3 dotTV(const T9& t, const V3& v) {            // GeomTensorInline.hh: Tensor.dot(Vector)
    return {t.xx * v.x + t.xy * v.y + t.xz * v.z, t.yx * v.x + t.yy * v.y + t.yz * v.z,
            t.zx * v.x + t.zy * v.y + t.zz * v.z};
  }
  static double limiterVL(double x) {                    // LimitedMonaghanGingoldViscosity.cc:26-32 (van Leer)
    return x > 0.0 ? 2.0 / (1.0 + x) * 2.0 * x / (1.0 + x) : 0.0;
  }
  // MonaghanGingoldViscosity::QPiij (MonaghanGingoldViscosity.cc:41-101) and,
  // with cfg.viscosity == 1, LimitedMonaghanGingoldViscosity::QPiij
  // (LimitedMonaghanGingoldViscosity.cc:113-213): the velocities are first
  // corrected along the pair by the van Leer limited DvDx of the Q.
  void QPiij(double& QPiij_, double& QPiji_, double& Qij, double& Qji, const V3& xi, const V3& etai, const V3& vi,
             double rhoi, double csi, const V3& xj, const V3& etaj, const V3& vj, double rhoj, double csj,
             const T9& DvDxi, const T9& DvDxj) const {
    const double fCli = 1.0, fCqi = 1.0, fClj = 1.0, fCqj = 1.0, fshear = 1.0;
    const double Clij = 0.5 * (fCli + fClj) * fshear * cfg.Cl;
    const double Cqij = 0.5 * (fCqi + fCqj) * fshear * cfg.Cq;
    V3 vij = sub(vi, vj);
    if (cfg.viscosity == 1) {
      const double nPerh = lists[0].nPerh;
      const double etaCrit = cfg.etaCritFrac / nPerh, etaFold = cfg.etaFoldFrac / nPerh;
      const V3 xij = mul(0.5, sub(xi, xj));
      const double gradi = dot(dotTV(DvDxi, xij), xij);
      const double gradj = dot(dotTV(DvDxj, xij), xij);
      const double ri = gradi / (sgn(gradj) * std::max(1.0e-30, std::fabs(gradj)));
      const double rj = gradj / (sgn(gradi) * std::max(1.0e-30, std::fabs(gradi)));
      double phi = limiterVL(std::min(ri, rj));
      const double etaij = std::min(mag(etai), mag(etaj));
      if (etaij < etaCrit) {
        const double z = (etaij - etaCrit) / etaFold;
        phi *= std::exp(-(z * z));
      }
      const V3 vi1 = sub(vi, mul(phi, dotTV(DvDxi, xij)));
      const V3 vj1 = add(vj, mul(phi, dotTV(DvDxj, xij)));
      vij = sub(vi1, vj1);
    }
    const double mui = dot(vij, etai) / (mag2(etai) + cfg.eps2);
    const double muj = dot(vij, etaj) / (mag2(etaj) + cfg.eps2);
    const double li = cfg.linearInExpansion ? mui : std::min(0.0, mui);
    const double lj = cfg.linearInExpansion ? muj : std::min(0.0, muj);
    const double qi = cfg.quadraticInExpansion ? -sgn(mui) * mui * mui : std::min(0.0, mui) * std::min(0.0, mui);
    const double qj = cfg.quadraticInExpansion ? -sgn(muj) * muj * muj : std::min(0.0, muj) * std::min(0.0, muj);
    const double ei = -Clij * csi * li + Cqij * qi;
    const double ej = -Clij * csj * lj + Cqij * qj;
    QPiij_ = ei / rhoi; QPiji_ = ej / rhoj;
    Qij = rhoi * ei; Qji = rhoj * ej;
  }
  void evaluateDerivatives() {
    const double W0 = W.kernelValue(0.0, 1.0);
    const double tiny = 1.0e-30;
    const double epsTensile = cfg.epsTensile;
    const bool compatible = cfg.compatibleEnergy != 0, XSPH = cfg.XSPH != 0;
    vector<PairAcc> acc(nTot);
    pairAccel.assign(pairs.size(), V3{});
    pairSweep(pairs.size(), acc, nTot, [&](long kk, vector<PairAcc>& p) {
      const int i = pairs[kk].first, j = pairs[kk].second;
      const V3 ri = pos[i], vi = vel[i]; const double mi = mass[i], rhoi = rho[i], Pi = P[i], ci = cs[i];
      const ST Hi = H[i]; const double safeOmegai = safeInv(omega[i], tiny), Hdeti = detS(Hi);
      const V3 rj = pos[j], vj = vel[j]; const double mj = mass[j], rhoj = rho[j], Pj = P[j], cj = cs[j];
      const ST Hj = H[j]; const double safeOmegaj = safeInv(omega[j], tiny), Hdetj = detS(Hj);
      // SPH.cc:264-266: the tensile scale uses the first NodeList's nPerh
      const double WnPerhi = W.kernelValue(1.0 / lists[0].nPerh, 1.0);
      const double WnPerhj = WnPerhi;
      auto& ai = p[i]; auto& aj = p[j];

      const V3 rij = sub(ri, rj);
      const V3 etai = dotSV(Hi, rij), etaj = dotSV(Hj, rij);
      const double etaMagi = mag(etai), etaMagj = mag(etaj);
      const V3 etaiUnit = mul(etai, safeInvVar(etaMagi)), etajUnit = mul(etaj, safeInvVar(etaMagj));
      double Wi, gWi, Wj, gWj;
      W.kernelAndGradValue(etaMagi, Hdeti, Wi, gWi);
      W.kernelAndGradValue(etaMagj, Hdetj, Wj, gWj);
      const V3 gradWi = dotSV(scaleS(gWi, Hi), etaiUnit), gradWj = dotSV(scaleS(gWj, Hj), etajUnit);
      const double WQi = Wi, WQj = Wj; const V3 gradWQi = gradWi, gradWQj = gradWj;
      if (list[i] == list[j]) {
        ai.rhoSum += mj * Wi; aj.rhoSum += mi * Wj;
        ai.norm += mi / rhoi * Wi; aj.norm += mj / rhoj * Wj;
      }
      const V3 vij = sub(vi, vj);
      double QPi_ij, QPi_ji, Qi, Qj;
      QPiij(QPi_ij, QPi_ji, Qi, Qj, ri, etai, vi, rhoi, ci, rj, etaj, vj, rhoj, cj, DvDxQ[i], DvDxQ[j]);
      const V3 Qacci = mul(0.5, mul(QPi_ij, gradWQi)), Qaccj = mul(0.5, mul(QPi_ji, gradWQj));
      const double workQi = dot(vij, Qacci), workQj = dot(vij, Qaccj);
      ai.maxQ = std::max(ai.maxQ, Qi); aj.maxQ = std::max(aj.maxQ, Qj);
      ai.effQ += mj * Qi * WQi / rhoj; aj.effQ += mi * Qj * WQj / rhoi;
      const double Ri = epsTensile * pow4(Wi / (Hdeti * WnPerhi)) * (Pi < 0.0 ? -Pi : 0.0);
      const double Rj = epsTensile * pow4(Wj / (Hdetj * WnPerhj)) * (Pj < 0.0 ? -Pj : 0.0);
      const double Peffi = Pi + Ri, Peffj = Pj + Rj;
      const double Prhoi = safeOmegai * Peffi / (rhoi * rhoi), Prhoj = safeOmegaj * Peffj / (rhoj * rhoj);
      const V3 deltaDvDt = add(add(add(mul(Prhoi, gradWi), mul(Prhoj, gradWj)), Qacci), Qaccj);
      ai.DvDt = sub(ai.DvDt, mul(mj, deltaDvDt));
      aj.DvDt = add(aj.DvDt, mul(mi, deltaDvDt));
      if (compatible) pairAccel[kk] = mul(-mj, deltaDvDt);
      ai.DepsDt += mj * (Prhoi * dot(vij, gradWi) + workQi);
      aj.DepsDt += mi * (Prhoj * dot(vij, gradWj) + workQj);
      const T9 dDvDxi = scaleT(mj, dyad(vij, gradWi)), dDvDxj = scaleT(mi, dyad(vij, gradWj));
      subT(ai.DvDx, dDvDxi); subT(aj.DvDx, dDvDxj);
      subT(ai.localDvDx, dDvDxi); subT(aj.localDvDx, dDvDxj);
      if (XSPH) {
        const double w = 0.5 * (mi / rhoi * Wi + mj / rhoj * Wj);
        ai.xsphW += w; aj.xsphW += w;
        ai.xsphDV = sub(ai.xsphDV, mul(w, vij)); aj.xsphDV = add(aj.xsphDV, mul(w, vij));
      }
      ai.gradRho = add(ai.gradRho, mul(mj * (rhoj - rhoi), gradWi));
      aj.gradRho = add(aj.gradRho, mul(mi * (rhoj - rhoi), gradWj));
      subT(ai.M, scaleT(mj, dyad(rij, gradWi))); subT(aj.M, scaleT(mi, dyad(rij, gradWj)));
      subT(ai.localM, scaleT(mj, dyad(rij, gradWi))); subT(aj.localM, scaleT(mi, dyad(rij, gradWj)));
      // SPHSmoothingScale moments (fweightij for distinct NodeLists).
      const double fweightij = (list[i] != list[j]) ? mj * rhoi / (mi * rhoj) : 1.0;
      const double WSPHi = W.kernelValueSPH(etaMagi), WSPHj = W.kernelValueSPH(etaMagj);
      ai.m0 += fweightij * WSPHi; aj.m0 += 1.0 / fweightij * WSPHj;
      ai.m1 = sub(ai.m1, mul(fweightij * WSPHi, etai)); aj.m1 = add(aj.m1, mul(1.0 / fweightij * WSPHj, etaj));
      if (cfg.smoothingScale == 1) {
        // ASPHClassicSmoothingScale second moment (ASPHClassicSmoothingScale.cc:167-176):
        // xij xij / |xij|^5 weighted by WSPH^2
        const double rm = mag(rij);
        const double f5 = safeInvVar(rm * rm * rm * rm * rm);
        const ST xd{rij.x * rij.x * f5, rij.x * rij.y * f5, rij.x * rij.z * f5,
                    rij.y * rij.y * f5, rij.y * rij.z * f5, rij.z * rij.z * f5};
        addS(ai.m2, scaleS(fweightij * WSPHi * WSPHi, xd));
        addS(aj.m2, scaleS(1.0 / fweightij * WSPHj * WSPHj, xd));
      }
    });
    // SPH finalize, SPH.cc:480-552
    for (int i = 0; i < nInt; ++i) {
      auto& a = acc[i];
      const double mi = mass[i], rhoi = rho[i]; const V3 vi = vel[i]; const double Hdeti = detS(H[i]);
      rhoSum[i] = a.rhoSum + mi * W0 * Hdeti;
      normalization[i] = a.norm + mi / rhoi * W0 * Hdeti;
      T9 Mi = a.M, lMi = a.localM, DvDxi = a.DvDx, lDvDxi = a.localDvDx;
      if (cfg.correctVelocityGradient && std::fabs(detT(Mi)) > 1.0e-10 && numNeighbors[i] > 8) {
        Mi = inverseT(Mi); DvDxi = dotTT(DvDxi, Mi);
      } else {
        DvDxi.xx /= rhoi; DvDxi.xy /= rhoi; DvDxi.xz /= rhoi; DvDxi.yx /= rhoi; DvDxi.yy /= rhoi;
        DvDxi.yz /= rhoi; DvDxi.zx /= rhoi; DvDxi.zy /= rhoi; DvDxi.zz /= rhoi;
      }
      if (cfg.correctVelocityGradient && std::fabs(detT(lMi)) > 1.0e-10 && numNeighbors[i] > 8) {
        lMi = inverseT(lMi); lDvDxi = dotTT(lDvDxi, lMi);
      } else {
        lDvDxi.xx /= rhoi; lDvDxi.xy /= rhoi; lDvDxi.xz /= rhoi; lDvDxi.yx /= rhoi; lDvDxi.yy /= rhoi;
        lDvDxi.yz /= rhoi; lDvDxi.zx /= rhoi; lDvDxi.zy /= rhoi; lDvDxi.zz /= rhoi;
      }
      M[i] = Mi; localM[i] = lMi; DvDx[i] = DvDxi; localDvDx[i] = lDvDxi;
      gradRho[i] = {a.gradRho.x / rhoi, a.gradRho.y / rhoi, a.gradRho.z / rhoi};
      DrhoDt[i] = -rhoi * traceT(DvDxi);
      DvDt[i] = a.DvDt;
      // evolveTotalEnergy: the total-energy rate (SPH.cc:541)
      DepsDt[i] = cfg.evolveTotalEnergy ? mi * (dot(vi, a.DvDt) + a.DepsDt) : a.DepsDt;
      maxQ[i] = a.maxQ; effQ[i] = a.effQ;
      XSPHWeightSum[i] = a.xsphW; XSPHDeltaV[i] = a.xsphDV;
      if (XSPH) {
        XSPHWeightSum[i] += Hdeti * mi / rhoi * W0;
        const double ws = std::max(tiny, XSPHWeightSum[i]);
        DxDt[i] = add(vi, V3{XSPHDeltaV[i].x / ws, XSPHDeltaV[i].y / ws, XSPHDeltaV[i].z / ws});
      } else {
        DxDt[i] = vi;
      }
      if (cfg.smoothingScale == 1) { asphClassicFinalize(i, a, DvDxi); continue; }
      if (cfg.smoothingScale == 2) {
        // ASPHSmoothingScale::evaluateDerivatives (ASPHSmoothingScale.cc:105-149):
        // only the tensor rate; the ideal H comes at the end of the step
        DHDt[i] = smoothingScaleDerivative3(H[i], DvDxi);
        continue;
      }
      // SPHSmoothingScale finalize
      const auto& L = lists[list[i]];
      double m0 = rootnu3(std::max(0.0, a.m0));
      massZeroth[i] = m0; massFirst[i] = a.m1;
      const double tr = traceT(DvDxi);
      const ST mH{-H[i].xx, -H[i].xy, -H[i].xz, -H[i].yy, -H[i].yz, -H[i].zz};
      DHDt[i] = scaleS(ST{mH.xx / 3, mH.xy / 3, mH.xz / 3, mH.yy / 3, mH.yz / 3, mH.zz / 3}, tr);
      const double cur = fuzzyEqual(m0, 0.0) ? 0.5 * L.nPerh : W.equivalentNodesPerSmoothingScale(m0);
      const double s = std::min(4.0, std::max(0.25, L.nPerh / (cur + 1.0e-30)));
      const double aa = s < 1.0 ? 0.4 * (1.0 + s * s) : 0.4 * (1.0 + 1.0 / (s * s * s));
      const double hi0 = 1.0 / H[i].xx;
      const double hi1 = std::min(L.hmax, std::max(L.hmin, hi0 * (1.0 - aa + aa * s)));
      const double hinv = 1.0 / hi1;
      Hideal[i] = ST{hinv * 1.0, hinv * 0.0, hinv * 0.0, hinv * 1.0, hinv * 0.0, hinv * 1.0};
    }
  }

  // ASPHClassicSmoothingScale::evaluateDerivatives, the node part
  // (ASPHClassicSmoothingScale.cc:180-291): DHDt from the tensor rate; the
  // shape of Hideal from the normalised second moment of the neighbour
  // distribution (eigenvalues floored at hminratio of the largest), its size
  // from the zeroth moment as in the SPH IdealH, then the eigenvalues bounded
  // by 1/hmax and min(1/hmin, max(1/hmax, smallest)/hminratio).
  void asphClassicFinalize(int i, const PairAcc& a, const T9& DvDxi) {
    const auto& L = lists[list[i]];
    const double tiny = 1.0e-50;
    const ST Hi = H[i];
    DHDt[i] = smoothingScaleDerivative3(Hi, DvDxi);
    const double m0 = rootnu3(std::max(0.0, a.m0));
    massZeroth[i] = m0; massFirst[i] = a.m1; massSecond[i] = a.m2;
    const double cur = fuzzyEqual(m0, 0.0) ? 0.5 * L.nPerh : W.equivalentNodesPerSmoothingScale(m0);
    const double s = std::min(4.0, std::max(0.25, L.nPerh / cur));
    const double psiweight = std::max(0.0, std::min(1.0, 2.0 / s - 1.0));
    const ST& M2 = a.m2;
    ST Hid;
    if (psiweight > 0.0 && detS(M2) > 0.0 && minElem(eigenValuesS(M2)) > 0.0) {
      ST psi = divS(M2, maxAbsS(M2));
      if (detS(psi) > 1.0e-10) psi = divS(psi, rootnu3(std::fabs(detS(psi)) + tiny));
      else psi = identityS();
      EigS pe = eigenVectorsS(psi);
      for (int k = 0; k < 3; ++k) pe.val[k] = 1.0 / std::sqrt(pe.val[k]);
      const double psimin = std::max(pe.val[0], std::max(pe.val[1], pe.val[2])) * L.hminratio;
      const double d[3] = {std::max(psimin, pe.val[0]), std::max(psimin, pe.val[1]), std::max(psimin, pe.val[2])};
      psi = fromEigen(d, pe.vec);
      psi = divS(psi, rootnu3(detS(psi) + tiny));
      Hid = inverseS(sqrtS(psi));
    } else {
      Hid = identityS();
    }
    const double aa = s < 1.0 ? 0.4 * (1.0 + s * s) : 0.4 * (1.0 + 1.0 / (s * s * s + tiny));
    if (cfg.fixShape) Hid = divS(Hi, 1.0 - aa + aa * s);
    else if (cfg.radialOnly) Hid = radialEvolution3(Hi, unitVector(pos[i]), 1.0 - aa + aa * s,
                                                    i < (int)radius0.size() ? radius0[i] : 0.0, mag(pos[i]));
    else Hid = scaleS(Hid, rootnu3(detS(Hi)) / (1.0 - aa + aa * s));
    const EigS he = eigenVectorsS(Hid);
    const double hminInv = safeInvVar(L.hmin), hmaxInv = safeInvVar(L.hmax);
    const double hminEffInv = std::min(hminInv, std::max(hmaxInv, std::min(he.val[0], std::min(he.val[1], he.val[2]))) / L.hminratio);
    double d[3];
    for (int k = 0; k < 3; ++k) d[k] = std::max(hmaxInv, std::min(hminEffInv, he.val[k]));
    Hideal[i] = fromEigen(d, he.vec);
  }

  //============================================================================
  // CRKSPH with LinearOrder reproducing kernels.
  //============================================================================
  // ReflectingBoundary::applyGhostBoundary for RKCoefficients
  // (ReflectingBoundary.cc:402-432) with the reflection operator of
  // RKUtilities::getTransformationMatrix: for a wall normal to axis a an entry
  // changes sign once per index equal to a (C_{1+a}; dC_a[0]; dC_a[1+k] and
  // dC_k[1+a] for k != a; dC_a[1+a] keeps its sign).
  static void reflectRKC(RKC& c, int a) {
    c[1 + a] = -c[1 + a];
    for (int d = 0; d < 3; ++d)
      for (int k = 0; k < 4; ++k) {
        const int flips = (d == a ? 1 : 0) + ((k >= 1 && k - 1 == a) ? 1 : 0);
        if (flips == 1) c[4 + 4 * d + k] = -c[4 + 4 * d + k];
      }
  }
  void applyGhostRKC() { applyGhostField(rkc, [](RKC& c, int a) { reflectRKC(c, a); }); }

  // computeRKVolumes (computeRKVolumes.cc:20-70) for the volume types that
  // need no tessellation: RKMassOverDensity, RKSumVolume
  // (computeRKSumVolume.cc:30-110), HVolume (computeHVolumes.cc:25-60, with
  // the first NodeList's nPerh).
  void computeRKVolumes() {
    vol.resize(nTot);
    if (cfg.rkVolume == 0) {
      for (int i = 0; i < nInt; ++i) vol[i] = mass[i] / rho[i];
    } else if (cfg.rkVolume == 4) {
      const double nPerh = lists[0].nPerh;
      for (int i = 0; i < nInt; ++i) vol[i] = 0.125 * 4.0 / 3.0 * M_PI / detS(scaleS(nPerh, H[i]));
    } else {
      const double etaVolMax = std::pow(0.5 * W.extent, 3) * (4.0 / 3.0 * M_PI);
      const double W0 = W.kernelValue(0.0, 1.0);
      vector<double> acc(nTot, 0.0);
      pairSweep(pairs.size(), acc, nTot, [&](long kk, vector<double>& p) {
        const int i = pairs[kk].first, j = pairs[kk].second;
        const V3 rij = sub(pos[i], pos[j]);
        p[i] += W.kernelValue(mag(dotSV(H[i], rij)), detS(H[i]));
        p[j] += W.kernelValue(mag(dotSV(H[j], rij)), detS(H[j]));
      });
      for (int i = 0; i < nInt; ++i) {
        const double Hdeti = detS(H[i]);
        const double v = acc[i] + Hdeti * W0;
        vol[i] = std::min(etaVolMax / Hdeti, 1.0 / v);
      }
    }
    applyGhostScalar(vol);
  }

  // computeCRKSPHSumMassDensity (computeCRKSPHSumMassDensity.cc:15-110):
  // pairs of the same NodeList, plain kernel of each side's own H.
  void crkSumMassDensity() {
    struct Acc { double wsum = 0, rho = 0, vol1 = 0;
                 Acc& operator+=(const Acc& o) { wsum += o.wsum; rho += o.rho; vol1 += o.vol1; return *this; } };
    vector<Acc> acc(nTot);
    pairSweep(pairs.size(), acc, nTot, [&](long kk, vector<Acc>& p) {
      const int i = pairs[kk].first, j = pairs[kk].second;
      if (list[i] != list[j]) return;
      const V3 rij = sub(pos[i], pos[j]);
      const double Wi = W.kernelValue(mag(dotSV(H[i], rij)), detS(H[i]));
      const double Wj = W.kernelValue(mag(dotSV(H[j], rij)), detS(H[j]));
      const double Vi = vol[i], Vj = vol[j];
      p[i].wsum += Vj * Wj; p[j].wsum += Vi * Wi;
      p[i].rho += mass[j] * Vj * Wj; p[j].rho += mass[i] * Vi * Wi;
      p[i].vol1 += Vj * Vj * Wj; p[j].vol1 += Vi * Vi * Wi;
    });
    const double W0 = W.kernelValue(0.0, 1.0);
    for (int i = 0; i < nInt; ++i) {
      const auto& L = lists[list[i]];
      const double mi = mass[i], Vi = vol[i], Hdeti = detS(H[i]);
      const double wsum = acc[i].wsum + Vi * Hdeti * W0;
      const double vol1 = (acc[i].vol1 + Vi * Vi * Hdeti * W0) / wsum;
      rho[i] = std::max(std::max(L.rhoMin, 0.1 * mi * Hdeti),
                        std::min(L.rhoMax, (acc[i].rho + mi * Vi * Hdeti * W0) / (wsum * vol1)));
    }
    applyGhostScalar(rho);
  }

  // RKUtilities::evaluateBaseKernelAndGradient (RKUtilities.cc:66-80)
  void rkBase(const V3& x, const ST& Hm, double& w, V3& dw) const {
    const V3 eta = dotSV(Hm, x);
    const double etaMag = mag(eta);
    const V3 etaUnit = unitVector(eta);
    const double Hdet = detS(Hm);
    w = W.kernelValue(etaMag, Hdet);
    const double dk = W.gradValue(etaMag, Hdet);
    dw = mul(dotSV(Hm, etaUnit), dk);
  }
  // RKUtilities::evaluateKernelAndGradient (RKUtilities.cc:181-206), LinearOrder:
  // P = (1, x, y, z), dP/dx_d = e_{1+d}; inner products summed from index 0.
  void rkKernelAndGradient(const V3& x, const ST& Hm, const RKC& c, double& WR, V3& gradWR) const {
    double w; V3 dw;
    rkBase(x, Hm, w, dw);
    const double P[4] = {1.0, x.x, x.y, x.z};
    double CP = 0.0;
    for (int k = 0; k < 4; ++k) CP += c[k] * P[k];
    double g[3];
    for (int d = 0; d < 3; ++d) {
      const double CdP = c[1 + d];
      double dCP = 0.0;
      for (int k = 0; k < 4; ++k) dCP += c[4 + 4 * d + k] * P[k];
      g[d] = (CdP + dCP) * w + CP * compc(dw, d);
    }
    WR = CP * w;
    gradWR = {g[0], g[1], g[2]};
  }
  // 4x4 solve by Gaussian elimination with partial pivoting (the reference
  // uses Eigen's colPivHouseholderQr; any accurate solver gives the same
  // corrections to rounding).  A is overwritten by its LU factors; piv
  // records the row order.
  static void lu4(double A[4][4], int piv[4]) {
    for (int k = 0; k < 4; ++k) piv[k] = k;
    for (int k = 0; k < 4; ++k) {
      int p = k;
      for (int r = k + 1; r < 4; ++r) if (std::fabs(A[r][k]) > std::fabs(A[p][k])) p = r;
      if (p != k) { for (int c = 0; c < 4; ++c) std::swap(A[k][c], A[p][c]); std::swap(piv[k], piv[p]); }
      const double inv = 1.0 / A[k][k];
      for (int r = k + 1; r < 4; ++r) {
        const double f = A[r][k] * inv;
        A[r][k] = f;
        for (int c = k + 1; c < 4; ++c) A[r][c] -= f * A[k][c];
      }
    }
  }
  static void solve4(const double LU[4][4], const int piv[4], const double b[4], double x[4]) {
    double y[4];
    for (int r = 0; r < 4; ++r) {
      double v = b[piv[r]];
      for (int c = 0; c < r; ++c) v -= LU[r][c] * y[c];
      y[r] = v;
    }
    for (int r = 3; r >= 0; --r) {
      double v = y[r];
      for (int c = r + 1; c < 4; ++c) v -= LU[r][c] * x[c];
      x[r] = v / LU[r][r];
    }
  }
  // RKUtilities::computeCorrections (RKUtilities.cc:250-491), LinearOrder, no
  // Hessian: moments over the neighbours of i and i itself with the
  // scatter kernel W(x_ij, H_j), then C = M^-1 e_0, dC_d = -M^-1 (dM_d C);
  // ghost values follow (RKCorrections::initialize returns true, so the
  // integrator applies the ghost boundaries after it).
  void computeRKCorrections() {
    rkc.resize(nTot);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nInt; ++i) {
      double M[4][4] = {}, dM[3][4][4] = {};
      auto addTo = [&](int j) {
        const V3 xij = sub(pos[i], pos[j]);
        double w; V3 dw;
        rkBase(xij, H[j], w, dw);
        const double vj = vol[j];
        const double p[4] = {1.0, xij.x, xij.y, xij.z};
        for (int k = 0; k < 4; ++k)
          for (int l = k; l < 4; ++l) M[k][l] += vj * p[k] * p[l] * w;
        for (int d = 0; d < 3; ++d)
          for (int k = 0; k < 4; ++k)
            for (int l = k; l < 4; ++l) {
              const double dpk = (k == 1 + d) ? 1.0 : 0.0, dpl = (l == 1 + d) ? 1.0 : 0.0;
              dM[d][k][l] += vj * ((dpk * p[l] + p[k] * dpl) * w + p[k] * p[l] * compc(dw, d));
            }
      };
      for (int j : neighbors[i]) addTo(j);
      addTo(i);
      for (int k = 0; k < 4; ++k)
        for (int l = 0; l < k; ++l) {
          M[k][l] = M[l][k];
          for (int d = 0; d < 3; ++d) dM[d][k][l] = dM[d][l][k];
        }
      int piv[4];
      lu4(M, piv);
      const double e0[4] = {1.0, 0.0, 0.0, 0.0};
      double C[4];
      solve4(M, piv, e0, C);
      RKC out{};
      for (int k = 0; k < 4; ++k) out[k] = C[k];
      for (int d = 0; d < 3; ++d) {
        double rhs[4], dC[4];
        for (int k = 0; k < 4; ++k) {
          double v = 0.0;
          for (int l = 0; l < 4; ++l) v += dM[d][k][l] * C[l];
          rhs[k] = -v;
        }
        solve4(M, piv, rhs, dC);
        for (int k = 0; k < 4; ++k) out[4 + 4 * d + k] = dC[k];
      }
      rkc[i] = out;
    }
    applyGhostRKC();
  }

  // CRKSPH::evaluateDerivativesImpl (CRKSPH.cc:180-380) with the
  // SPHSmoothingScale moments (SPHSmoothingScale.cc:150-275).
  struct CrkAcc {
    double DepsDt = 0, maxQ = 0, effQ = 0, m0 = 0;
    V3 DvDt, xsphDV, m1;
    T9 DvDx, localDvDx;
    CrkAcc& operator+=(const CrkAcc& o) {
      DepsDt += o.DepsDt; maxQ = std::max(maxQ, o.maxQ); effQ += o.effQ; m0 += o.m0;
      DvDt = add(DvDt, o.DvDt); xsphDV = add(xsphDV, o.xsphDV); m1 = add(m1, o.m1);
      addT(DvDx, o.DvDx); addT(localDvDx, o.localDvDx);
      return *this;
    }
  };
  void evaluateDerivativesCRK() {
    const bool compatible = cfg.compatibleEnergy != 0, XSPH = cfg.XSPH != 0;
    vector<CrkAcc> acc(nTot);
    pairAccel.assign(pairs.size(), V3{});
    pairSweep(pairs.size(), acc, nTot, [&](long kk, vector<CrkAcc>& p) {
      const int i = pairs[kk].first, j = pairs[kk].second;
      const V3 ri = pos[i], vi = vel[i]; const double mi = mass[i], rhoi = rho[i], Pi = P[i], ci = cs[i];
      const V3 rj = pos[j], vj = vel[j]; const double mj = mass[j], rhoj = rho[j], Pj = P[j], cj = cs[j];
      const ST Hi = H[i], Hj = H[j];
      const double weighti = vol[i], weightj = vol[j];
      auto& ai = p[i]; auto& aj = p[j];
      const V3 rij = sub(ri, rj), vij = sub(vi, vj);
      const V3 etai = dotSV(Hi, rij), etaj = dotSV(Hj, rij);
      double Wi, Wj; V3 gradWi, gradWj;
      rkKernelAndGradient(rij, Hj, rkc[i], Wj, gradWj);
      rkKernelAndGradient(mul(-1.0, rij), Hi, rkc[j], Wi, gradWi);
      const V3 deltagrad = sub(gradWj, gradWi);
      double QPiij_, QPiji_, Qi, Qj;
      QPiij(QPiij_, QPiji_, Qi, Qj, ri, etai, vi, rhoi, ci, rj, etaj, vj, rhoj, cj, DvDxQ[i], DvDxQ[j]);
      const V3 Qaccij = mul(rhoi * rhoi * QPiij_ + rhoj * rhoj * QPiji_, deltagrad);
      const double workQi = dot(mul(rhoj * rhoj * QPiji_, vij), deltagrad);
      const double workQj = dot(mul(rhoi * rhoi * QPiij_, vij), deltagrad);
      ai.maxQ = std::max(ai.maxQ, 4.0 * Qi); aj.maxQ = std::max(aj.maxQ, 4.0 * Qj);
      ai.effQ += weightj * Qi * Wj; aj.effQ += weighti * Qj * Wi;
      const T9 dDi = scaleT(weightj, dyad(vij, gradWj)), dDj = scaleT(weighti, dyad(vij, gradWi));
      subT(ai.DvDx, dDi); addT(aj.DvDx, dDj);
      if (list[i] == list[j]) { subT(ai.localDvDx, dDi); addT(aj.localDvDx, dDj); }
      const V3 force = mul(0.5 * weighti * weightj, add(mul(Pi + Pj, deltagrad), Qaccij));
      ai.DvDt = sub(ai.DvDt, mul(force, 1.0 / mi));
      aj.DvDt = add(aj.DvDt, mul(force, 1.0 / mj));
      if (compatible) pairAccel[kk] = mul(force, -1.0 / mi);
      ai.DepsDt += 0.5 * weighti * weightj * (Pj * dot(vij, deltagrad) + workQi) / mi;
      aj.DepsDt += 0.5 * weighti * weightj * (Pi * dot(vij, deltagrad) + workQj) / mj;
      if (XSPH && list[i] == list[j]) {
        ai.xsphDV = sub(ai.xsphDV, mul(weightj * Wj, vij));
        aj.xsphDV = add(aj.xsphDV, mul(weighti * Wi, vij));
      }
      // SPHSmoothingScale moments
      const double fweightij = (list[i] != list[j]) ? mj * rhoi / (mi * rhoj) : 1.0;
      const double WSPHi = W.kernelValueSPH(mag(etai)), WSPHj = W.kernelValueSPH(mag(etaj));
      ai.m0 += fweightij * WSPHi; aj.m0 += 1.0 / fweightij * WSPHj;
      ai.m1 = sub(ai.m1, mul(fweightij * WSPHi, etai)); aj.m1 = add(aj.m1, mul(1.0 / fweightij * WSPHj, etaj));
    });
    for (int i = 0; i < nInt; ++i) {
      auto& a = acc[i];
      const double mi = mass[i], rhoi = rho[i]; const V3 vi = vel[i];
      DvDx[i] = a.DvDx; localDvDx[i] = a.localDvDx;
      M[i] = T9{}; localM[i] = T9{}; gradRho[i] = V3{}; rhoSum[i] = 0.0; normalization[i] = 0.0;
      XSPHWeightSum[i] = 0.0;
      XSPHDeltaV[i] = a.xsphDV;
      DxDt[i] = XSPH ? add(vi, a.xsphDV) : vi;
      DrhoDt[i] = -rhoi * traceT(a.DvDx);
      DvDt[i] = a.DvDt;
      DepsDt[i] = cfg.evolveTotalEnergy ? mi * (dot(vi, a.DvDt) + a.DepsDt) : a.DepsDt;
      maxQ[i] = a.maxQ; effQ[i] = a.effQ;
      // SPHSmoothingScale finalize (SPHSmoothingScale.cc:232-272)
      const auto& L = lists[list[i]];
      const double m0 = rootnu3(std::max(0.0, a.m0));
      massZeroth[i] = m0; massFirst[i] = a.m1;
      const double tr = traceT(a.DvDx);
      DHDt[i] = ST{-H[i].xx / 3 * tr, -H[i].xy / 3 * tr, -H[i].xz / 3 * tr, -H[i].yy / 3 * tr, -H[i].yz / 3 * tr,
                   -H[i].zz / 3 * tr};
      const double cur = fuzzyEqual(m0, 0.0) ? 0.5 * L.nPerh : W.equivalentNodesPerSmoothingScale(m0);
      const double s = std::min(4.0, std::max(0.25, L.nPerh / (cur + 1.0e-30)));
      const double aa = s < 1.0 ? 0.4 * (1.0 + s * s) : 0.4 * (1.0 + 1.0 / (s * s * s));
      const double hi0 = 1.0 / H[i].xx;
      const double hi1 = std::min(L.hmax, std::max(L.hmin, hi0 * (1.0 - aa + aa * s)));
      const double hinv = 1.0 / hi1;
      Hideal[i] = ST{hinv, 0.0, 0.0, hinv, 0.0, hinv};
    }
  }

  // ContinuityVolumePolicy::update (ContinuityVolumePolicy.cc:40-75): fires
  // after the mass density (its dependency), so it sees the updated rho and H.
  void volumeUpdate(double multiplier) {
    for (int i = 0; i < nInt; ++i) {
      const double volMin = 0.5 * mass[i] * safeInvVar(rho[i]);
      const double volMax = 4.0 * M_PI / (3.0 * detS(H[i]));
      const double dVdt = -mass[i] * safeInvVar(rho[i] * rho[i]) * DrhoDt[i];
      vol[i] = std::max(volMin, std::min(volMax, vol[i] + multiplier * dVdt));
    }
  }

  // SPHBase::finalizeDerivatives: ghost values of DvDt and DepsDt.
  void finalizeDerivatives() {
    if (cfg.compatibleEnergy) { applyGhostVector(DvDt); applyGhostScalar(DepsDt); }
  }

  //----------------------------------------------------------------------------
  // GenericHydro::dt (GenericHydro.cc:113-381).
  //----------------------------------------------------------------------------
  double hydroDt() {
    const double tiny = kDblEps;
    double minDt = std::numeric_limits<double>::max();
    std::string reason;
    for (int L = 0; L < (int)lists.size(); ++L) {
      const double nPerh = lists[L].nPerh;
      for (int i = 0; i < nInt; ++i) {
        if (list[i] != L) continue;
        const double nodeScalei = 1.0 / maxElem(eigenValuesS(H[i])) / nPerh;
        const double csDt = nodeScalei / (cs[i] + tiny);
        if (csDt < minDt) { minDt = csDt; reason = "sound speed"; }
        const double csq = std::sqrt(maxQ[i] / rho[i]);
        const double csqDt = nodeScalei / (csq + tiny);
        if (csqDt < minDt) { minDt = csqDt; reason = "artificial viscosity"; }
        const double divv = traceT(DvDx[i]);
        const double divvDt = 1.0 / (std::fabs(divv) + tiny);
        if (divvDt < minDt) { minDt = divvDt; reason = "velocity divergence"; }
        const double vmagi = mag(vel[i]);
        const double dtAcc = 0.1 * std::max(nodeScalei / (vmagi + tiny), vmagi / (mag(DvDt[i]) + tiny));
        if (dtAcc < minDt) { minDt = dtAcc; reason = "acceleration"; }
        if (cfg.useVelocityMagnitudeForDt) {
          const double velDt = nodeScalei / (mag(vel[i]) + 1.0e-10);
          if (velDt < minDt) { minDt = velDt; reason = "velocity magnitude"; }
        }
      }
      for (size_t k = 0; k < pairs.size(); ++k) {
        const int i = pairs[k].first, j = pairs[k].second;
        const double nsi = 1.0 / maxElem(eigenValuesS(H[i])) / nPerh;
        const double nsj = 1.0 / maxElem(eigenValuesS(H[j])) / nPerh;
        const double dtv = std::min(nsi, nsj) * safeInvVar(mag(sub(vel[i], vel[j])), tiny);
        if (dtv < minDt) { minDt = dtv; reason = "pairwise velocity difference"; }
      }
    }
    dtReason = reason;
    return minDt * cfg.cfl;
  }
  double gravityDt() const {
    return cfg.ftimestep * dtMinAcc;   // TreeGravity::dt, AccelerationRatio
  }
  double selectDt(double dtMin, double dtMax) {
    double dt = dtMax;
    const double hv = hydroDt();
    if (hv > 0.0 && hv < dt) dt = hv;
    if (cfg.gravity) { const double gv = gravityDt(); if (gv > 0.0 && gv < dt) dt = gv; }
    dt *= dtMultiplier;
    dt = std::min(dt, cfg.dtGrowth * lastDt);
    dt = std::min(dtMax, std::max(dtMin, dt));
    return dt;
  }

  //----------------------------------------------------------------------------
  // SpecificThermalEnergyPolicy::update (SpecificThermalEnergyPolicy.cc:47-174).
  //----------------------------------------------------------------------------
  void compatibleEnergyUpdate(double multiplier) {
    const double hdt = 0.5 * multiplier;
    vector<double> acc(nTot, 0.0);
    pairSweep(pairs.size(), acc, nTot, [&](long kk, vector<double>& p) {
      const int i = pairs[kk].first, j = pairs[kk].second;
      const double mi = mass[i], mj = mass[j];
      const V3 vi12 = add(vel[i], mul(DvDt[i], hdt)), vj12 = add(vel[j], mul(DvDt[j], hdt));
      const V3 vji12 = sub(vj12, vi12);
      const double duij = dot(vji12, pairAccel[kk]);
      const double weighti = std::max(kDblEps, DepsDt[i] * sgn(duij));
      const double weightj = std::max(kDblEps, DepsDt[j] * sgn(duij));
      const double wi = weighti / (weighti + weightj);
      p[i] += wi * duij;
      p[j] += (1.0 - wi) * duij * mi / mj;
    });
    for (int i = 0; i < nInt; ++i) { DepsDtCompat[i] = acc[i]; eps[i] += acc[i] * multiplier; }
  }

  //----------------------------------------------------------------------------
  // State::update for this package set.  midStep: timeAdvanceOnly update with
  // the previous derivatives (CheapSynchronousRK2.cc:75-80); otherwise the full
  // update from state0 (CheapSynchronousRK2.cc:105-110).
  //----------------------------------------------------------------------------
  // The eigenvalue limits of the ASPH smoothing scales: every eigenvalue of
  // H within [1/hmax, min(1/hmin, max(1/hmax, smallest)/hminratio)]
  // (constructSymTensorWithBoundedDiagonal + rotationalTransform,
  // IncrementASPHHtensor.cc:88-92, ASPHSmoothingScale.cc:355-359).
  static ST limitASPH(const ST& h, const NodeListParams& L) {
    const EigS he = eigenVectorsS(h);
    const double hminInv = 1.0 / L.hmin, hmaxInv = 1.0 / L.hmax;
    const double hminEffInv =
        std::min(hminInv, std::max(hmaxInv, std::min(he.val[0], std::min(he.val[1], he.val[2]))) / L.hminratio);
    double d[3];
    for (int k = 0; k < 3; ++k) d[k] = std::max(hmaxInv, std::min(hminEffInv, he.val[k]));
    return fromEigen(d, he.vec);
  }
  // IncrementASPHHtensor::update (src/SmoothingScale/IncrementASPHHtensor.cc:37-100):
  // fixShape scales H by the cube root of the determinant ratio of the plain
  // increment; radialOnly increments only the radial diagonal element in the
  // frame whose first axis is the radial direction (about the origin, at the
  // position before this update); otherwise H += m DH/Dt; then the limits.
  ST incrementASPHHtensor(const ST& Hi, const ST& D, double m, const V3& xi, const NodeListParams& L) const {
    ST h = Hi;
    if (cfg.fixShape) {
      const ST hp{Hi.xx + m * D.xx, Hi.xy + m * D.xy, Hi.xz + m * D.xz, Hi.yy + m * D.yy, Hi.yz + m * D.yz,
                  Hi.zz + m * D.zz};
      h = scaleS(Hi, rootnu3(detS(hp) / detS(Hi)));
    } else if (cfg.radialOnly) {
      const T9 T = rotationMatrix3(unitVector(xi));
      h = rotateS(Hi, T);
      const ST d = rotateS(D, T);
      h.xx += m * d.xx;
      h = rotateS(h, transposeT(T));
    } else {
      h = ST{Hi.xx + m * D.xx, Hi.xy + m * D.xy, Hi.xz + m * D.xz, Hi.yy + m * D.yy, Hi.yz + m * D.yz,
             Hi.zz + m * D.zz};
    }
    return limitASPH(h, L);
  }
  // ASPHSmoothingScale::finalize (ASPHSmoothingScale.cc:157-380) in its
  // fixShape and radialOnly forms (no Voronoi second moment): the zeroth
  // moment of the end-of-step state over the step's pairs, the IdealH size
  // ratio, H scaled (fixShape) or reshaped radially (radialOnly), the limits.
  // With IntegrateH or FixedH only the limits are applied.
  void asphFinalize() {
    if (cfg.hUpdate != 0) {
      for (int i = 0; i < nInt; ++i) H[i] = limitASPH(H[i], lists[list[i]]);
      return;
    }
    vector<double> m0(nTot, 0.0);
    pairSweep(pairs.size(), m0, nTot, [&](long kk, vector<double>& p) {
      const int i = pairs[kk].first, j = pairs[kk].second;
      const V3 rij = sub(pos[i], pos[j]);
      const double WSPHi = W.kernelValueSPH(mag(dotSV(H[i], rij))), WSPHj = W.kernelValueSPH(mag(dotSV(H[j], rij)));
      const double fweightij = (list[i] != list[j]) ? mass[j] * rho[i] / (mass[i] * rho[j]) : 1.0;
      p[i] += fweightij * WSPHi;
      p[j] += 1.0 / fweightij * WSPHj;
    });
    for (int i = 0; i < nInt; ++i) {
      const auto& L = lists[list[i]];
      const double mz = rootnu3(std::max(0.0, m0[i]));
      massZeroth[i] = mz;
      const double cur = fuzzyEqual(mz, 0.0) ? 0.5 * L.nPerh : W.equivalentNodesPerSmoothingScale(mz);
      const double s = std::min(4.0, std::max(0.25, L.nPerh / (cur + 1.0e-30)));
      const double aa = s < 1.0 ? 0.4 * (1.0 + s * s) : 0.4 * (1.0 + 1.0 / (s * s * s));
      ST Hid;
      if (cfg.fixShape) Hid = divS(H[i], 1.0 - aa + aa * s);
      else Hid = radialEvolution3(H[i], unitVector(pos[i]), 1.0 - aa + aa * s,
                                  i < (int)radius0.size() ? radius0[i] : 0.0, mag(pos[i]));
      Hid = limitASPH(Hid, L);
      Hideal[i] = Hid;
      H[i] = Hid;
    }
  }

  static ST clampH(const ST& h, double minv, double maxv) {
    // min(maxv, max(minv, H)): SymTensor min/max with a scalar bound the
    // eigenvalues (GeomSymmetricTensorInline.hh:2745-2772); the isotropic
    // case in closed form.
    if (isIsotropic(h)) {
      double a = h.xx;
      if (a < minv) a = minv;
      if (a > maxv) a = maxv;
      return ST{a, 0.0, 0.0, a, 0.0, a};
    }
    return enforceMaxEig(enforceMinEig(h, minv), maxv);
  }
  void stateUpdate(double multiplier, bool midStep) {
    // specific thermal energy
    if (midStep || !cfg.compatibleEnergy) {
      if (cfg.evolveTotalEnergy) {
        // SpecificFromTotalThermalEnergyPolicy::update (SpecificFromTotalThermalEnergyPolicy.cc:40-70);
        // it fires before the velocity update (no dependencies, key order)
        for (int i = 0; i < nInt; ++i) {
          const double E0 = mass[i] * (0.5 * mag2(vel[i]) + eps[i]);
          const double E1 = E0 + multiplier * DepsDt[i];
          eps[i] = E1 / mass[i] - 0.5 * mag2(add(vel[i], mul(multiplier, DvDt[i])));
        }
      } else {
        for (int i = 0; i < nInt; ++i) eps[i] += multiplier * DepsDt[i];
      }
    } else {
      compatibleEnergyUpdate(multiplier);
    }
    for (int i = 0; i < nInt; ++i) {
      const auto& L = lists[list[i]];
      const V3 pos0i = pos[i];   // State::update applies the "H" policy before "position" (key order)
      pos[i] = add(pos[i], mul(multiplier, DxDt[i]));
      vel[i] = add(vel[i], mul(multiplier, DvDt[i]));
      if (cfg.gravity) vel[i] = add(vel[i], mul(multiplier, DvDtGrav[i]));
      rho[i] = std::min(L.rhoMax, std::max(L.rhoMin, rho[i] + multiplier * DrhoDt[i]));
      // H: ReplaceBoundedState (IdealH; its timeAdvanceOnly update is the
      // increment), IncrementBoundedState (IntegrateH), no policy (FixedH);
      // ASPHSmoothingScale: IncrementASPHHtensor for IdealH and IntegrateH
      if (cfg.smoothingScale == 2) {
        if (cfg.hUpdate != 2) H[i] = incrementASPHHtensor(H[i], DHDt[i], multiplier, pos0i, L);
      } else if (cfg.hUpdate == 2) {
      } else if (midStep || cfg.hUpdate == 1) {
        ST hn{H[i].xx + multiplier * DHDt[i].xx, H[i].xy + multiplier * DHDt[i].xy, H[i].xz + multiplier * DHDt[i].xz,
              H[i].yy + multiplier * DHDt[i].yy, H[i].yz + multiplier * DHDt[i].yz, H[i].zz + multiplier * DHDt[i].zz};
        H[i] = clampH(hn, 1.0 / L.hmax, 1.0 / L.hmin);
      } else {
        H[i] = clampH(Hideal[i], 1.0 / L.hmax, 1.0 / L.hmin);
      }
    }
    if (cfg.hydro == 1) volumeUpdate(multiplier);
    updateEOS(nInt);
  }

  // Boundary::setAllViolationNodes + enforceBoundary (PlanarBoundary.cc:153-190,
  // ReflectingBoundary.cc:465-500): map positions of internal nodes that left
  // through a plane and reflect their vectors.
  void enforceBoundaries() {
    for (auto& b : bcs) {
      const int nsub = b.type == 0 ? 2 : 1;
      for (int sub = 0; sub < nsub; ++sub) {
        double wEn, sEn, wEx, sEx;
        planeSpec(b, sub, wEn, sEn, wEx, sEx);
        for (int i = 0; i < nInt; ++i) {
          const double p = compc(pos[i], b.axis);
          const double sd = (p - wEn) * sEn;            // vec < plane: compare() == 1
          if (sd < 0.0 && !orc::fuzzyEqual(sd, 0.0)) {
            comp(pos[i], b.axis) = mapCoord(p, wEn, sEn, wEx, sEx);
            if (b.type == 1) {
              comp(vel[i], b.axis) = -compc(vel[i], b.axis);
              // PlanarBoundary::updateViolationNodes: H -> (R H R).Symmetric()
              ST& h = H[i];
              if (b.axis == 0) { h.xy = -h.xy; h.xz = -h.xz; }
              else if (b.axis == 1) { h.xy = -h.xy; h.yz = -h.yz; }
              else { h.xz = -h.xz; h.yz = -h.yz; }
            }
          }
        }
      }
    }
  }

  //----------------------------------------------------------------------------
  // TreeGravity (TreeGravity.cc:146-480, 819-932; TreeGravityInline.hh:38-165).
  //----------------------------------------------------------------------------
  struct Cell {
    double M = 0, Mglobal = 0; V3 xcm, vcm; double rcm2cc2 = 0; uint64_t key = 0;
    vector<uint64_t> daughters; vector<Cell*> daughterPtrs;
    vector<double> masses; vector<V3> positions, velocities;
  };
  static const int num1dbits = 21;
  vector<std::unordered_map<uint64_t, Cell>> tree;
  V3 gxmin, gxmax; double boxLength = 0;
  void buildCellKey(int ilevel, const V3& xi, uint64_t& key, uint64_t& ix, uint64_t& iy, uint64_t& iz) const {
    const uint64_t ncell = (1ULL << ilevel), maxcell = ncell - 1ULL, max1dKey = (1ULL << num1dbits) - 1ULL;
    ix = std::min(maxcell, (uint64_t)((xi.x - gxmin.x) / boxLength * ncell));
    iy = std::min(maxcell, (uint64_t)((xi.y - gxmin.y) / boxLength * ncell));
    iz = std::min(maxcell, (uint64_t)((xi.z - gxmin.z) / boxLength * ncell));
    key = (std::min(max1dKey, iz) << 2 * num1dbits) + (std::min(max1dKey, iy) << num1dbits) + std::min(max1dKey, ix);
  }
  void addNodeToTree(double mi, const V3& xi, const V3& vi) {
    int ilevel = 0; bool terminated = false;
    uint64_t key = 0, parentKey = 0, otherKey, ix, iy, iz;
    while (ilevel < num1dbits && !terminated) {
      if (ilevel == (int)tree.size()) tree.emplace_back();
      buildCellKey(ilevel, xi, key, ix, iy, iz);
      auto itr = tree[ilevel].find(key);
      if (itr == tree[ilevel].end()) {
        terminated = true;
        Cell c; c.M = mi; c.Mglobal = mi; c.xcm = xi; c.vcm = vi; c.key = key;
        c.masses = {mi}; c.positions = {xi}; c.velocities = {vi};
        tree[ilevel][key] = c;
      } else {
        Cell& cell = itr->second;
        if (!cell.masses.empty()) {
          if (ilevel < num1dbits - 1) {
            const int il1 = ilevel + 1;
            if (il1 == (int)tree.size()) tree.emplace_back();   // capacity reserved: no reallocation
            buildCellKey(il1, cell.xcm, otherKey, ix, iy, iz);
            Cell d; d.M = cell.M; d.Mglobal = cell.M; d.xcm = cell.xcm; d.vcm = cell.vcm; d.key = otherKey;
            d.masses = {cell.M}; d.positions = {cell.xcm}; d.velocities = {cell.vcm};
            tree[il1][otherKey] = d;
            cell.daughters = {otherKey};
            cell.masses.clear(); cell.positions.clear(); cell.velocities.clear();
          } else {
            cell.masses.push_back(mi); cell.positions.push_back(xi); cell.velocities.push_back(vi);
          }
        }
        const double Mn = cell.M + mi;
        const V3 xs = add(mul(cell.M, cell.xcm), mul(mi, xi));
        const V3 vs = add(mul(cell.M, cell.vcm), mul(mi, vi));
        cell.xcm = V3{xs.x / Mn, xs.y / Mn, xs.z / Mn};
        cell.vcm = V3{vs.x / Mn, vs.y / Mn, vs.z / Mn};
        cell.M += mi;
        cell.Mglobal = cell.M;
      }
      if (ilevel > 0) {
        auto& par = tree[ilevel - 1][parentKey];
        if (std::find(par.daughters.begin(), par.daughters.end(), key) == par.daughters.end()) par.daughters.push_back(key);
      }
      parentKey = key;
      ++ilevel;
    }
  }
  void buildTree() {
    tree.clear();
    tree.reserve(num1dbits);
    if (nInt == 0) return;
    gxmin = pos[0]; gxmax = pos[0];
    for (int i = 0; i < nInt; ++i) {
      gxmin.x = std::min(gxmin.x, pos[i].x); gxmin.y = std::min(gxmin.y, pos[i].y); gxmin.z = std::min(gxmin.z, pos[i].z);
      gxmax.x = std::max(gxmax.x, pos[i].x); gxmax.y = std::max(gxmax.y, pos[i].y); gxmax.z = std::max(gxmax.z, pos[i].z);
    }
    boxLength = std::max(gxmax.x - gxmin.x, std::max(gxmax.y - gxmin.y, gxmax.z - gxmin.z));
    for (int i = 0; i < nInt; ++i) addNodeToTree(mass[i], pos[i], vel[i]);
    for (size_t l = 0; l + 1 < tree.size(); ++l)
      for (auto& kv : tree[l]) {
        kv.second.daughterPtrs.clear();
        for (auto dk : kv.second.daughters) kv.second.daughterPtrs.push_back(&tree[l + 1][dk]);
      }
    for (size_t l = 0; l < tree.size(); ++l) {
      const double cellsize = boxLength / (1U << l);
      for (auto& kv : tree[l]) {
        const uint64_t k = kv.first;
        const uint64_t mask = (1ULL << num1dbits) - 1ULL;
        const uint64_t ix = k & mask, iy = (k >> num1dbits) & mask, iz = (k >> 2 * num1dbits) & mask;
        const V3 cc{gxmin.x + (ix + 0.5) * cellsize, gxmin.y + (iy + 0.5) * cellsize, gxmin.z + (iz + 0.5) * cellsize};
        kv.second.rcm2cc2 = mag2(sub(kv.second.xcm, cc));
      }
    }
  }
  // applyTreeForces for one tree (single process: no remote trees, so the
  // cellsCompleted sets never filter a cell).
  void applyTreeForces() {
    const double boxLength2 = boxLength * boxLength;
    const double soft2 = cfg.softening * cfg.softening;
    const double opening2 = cfg.opening * cfg.opening;
    DvDtGrav.assign(nTot, V3{});
    potential.assign(nTot, 0.0);
    double result = std::numeric_limits<double>::max();
    const int numLevels = (int)tree.size();
    if (numLevels >= 1) {
      const Cell& root = tree[0].begin()->second;
#pragma omp parallel for schedule(dynamic, 64) reduction(min : result)
      for (int i = 0; i < nInt; ++i) {
        const V3 xi = pos[i];
        V3 a{}; double phi = 0.0;
        int ilevel = 0;
        vector<Cell*> remaining = root.daughterPtrs, next;
        while (!remaining.empty() && ++ilevel < numLevels) {
          next.clear();
          // 64-bit shift: the 32-bit form in the reference is only defined below level 16
          const double cellsize2 = boxLength2 / (double)(1ULL << (2 * ilevel));
          for (Cell* cp : remaining) {
            const Cell& cell = *cp;
            V3 xji = sub(cell.xcm, xi);
            double rji2 = mag2(xji);
            if (rji2 > cellsize2 / opening2 + cell.rcm2cc2) {
              const V3 nhat = unitVector(xji);
              rji2 += soft2;
              a = add(a, mul(cell.Mglobal * (1.0 / rji2), nhat));
              phi -= cell.Mglobal * (1.0 / std::sqrt(rji2));
            } else if (cell.daughterPtrs.empty()) {
              for (size_t j = 0; j < cell.masses.size(); ++j) {
                const double mj = cell.masses[j];
                V3 x2 = sub(cell.positions[j], xi);
                double r2 = mag2(x2);
                if (r2 / soft2 > 1.0e-10) {
                  const V3 nhat = unitVector(x2);
                  r2 += soft2;
                  a = add(a, mul(mj * (1.0 / r2), nhat));
                  phi -= mj * (1.0 / std::sqrt(r2));
                }
              }
            } else {
              next.insert(next.end(), cell.daughterPtrs.begin(), cell.daughterPtrs.end());
            }
          }
          remaining.swap(next);
        }
        DvDtGrav[i] = a; potential[i] = phi;
        const double amag = mag(a);
        if (amag > 0.0) result = std::min(result, std::sqrt(cfg.softening / amag));
      }
    }
    dtMinAcc = result / std::sqrt(cfg.G);
    extraEnergy = 0.0;
    for (int i = 0; i < nInt; ++i) {
      DvDtGrav[i] = mul(DvDtGrav[i], cfg.G);
      potential[i] *= cfg.G;
      extraEnergy += 0.5 * mass[i] * potential[i];
    }
  }

  //----------------------------------------------------------------------------
  // Problem start-up (SPHBase::initializeProblemStartupDependencies): ghosts,
  // connectivity, pressure, sound speed and the grad-h correction.
  //----------------------------------------------------------------------------
  void initialize() {
    resizeDerivs();
    setGhostNodes();
    computeConnectivity();
    applyGhostState();
    updateEOS(nTot);
    applyGhostState();
    if (cfg.hydro == 1) {
      // RKCorrections::initializeProblemStartupDependencies (RKCorrections.cc:85-150)
      computeRKVolumes();
      computeRKCorrections();
      return;
    }
    if (cfg.gradhCorrection) omegaGradh();
  }

  //----------------------------------------------------------------------------
  // One Integrator::step -> CheapSynchronousRK2::step (no dt-check retry:
  // allowDtCheck defaults to false).
  //----------------------------------------------------------------------------
  double step(double maxTime) {
    setGhostNodes();
    applyGhostState();
    computeConnectivity();
    const double t = time;
    // preStepInitialize: RigorousSumDensity
    if (cfg.radialOnly) {   // SmoothingScaleBase::preStepInitialize
      radius0.assign(nInt, 0.0);
      for (int i = 0; i < nInt; ++i) radius0[i] = mag(pos[i]);
    }
    if (cfg.hydro == 1) {
      // RKCorrections::preStepInitialize (volumes), then
      // CRKSPHBase::preStepInitialize (CRKSPHBase.cc:190-225, the CRK sum).
      // The corrections RKCorrections::initialize computes at t are
      // recomputed at t + dt/2 before anything reads them.
      computeRKVolumes();
      if (cfg.densityUpdate == 0) crkSumMassDensity();
    } else if (cfg.densityUpdate == 0) {
      sumMassDensity();
    }
    // initializeDerivatives(t, 0): TreeGravity::initialize builds the tree
    if (cfg.gravity) buildTree();
    const double dt = selectDt(std::min(cfg.dtMin, maxTime - t), std::min(cfg.dtMax, maxTime - t));
    const double hdt = 0.5 * dt;
    // state0 copy (internal + ghost values)
    const auto pos0 = pos; const auto vel0 = vel; const auto rho0 = rho; const auto eps0 = eps;
    const auto H0 = H; const auto P0 = P; const auto cs0 = cs; const auto omega0 = omega; const auto vol0 = vol;
    // mid-step: timeAdvanceOnly update with the previous derivatives
    stateUpdate(hdt, true);
    time = t + hdt;
    applyGhostState();
    copyQVelocityGradient();
    if (cfg.gradhCorrection) { omegaGradh(); applyGhostState(); }
    // derivatives at the midpoint
    if (cfg.gravity) buildTree();
    if (cfg.hydro == 1) {
      computeRKCorrections();   // RKCorrections::initialize(t + dt/2)
      evaluateDerivativesCRK();
    } else {
      evaluateDerivatives();
    }
    if (cfg.gravity) applyTreeForces();
    finalizeDerivatives();
    // full step from state0
    pos = pos0; vel = vel0; rho = rho0; eps = eps0; H = H0; P = P0; cs = cs0; omega = omega0; vol = vol0;
    stateUpdate(dt, false);
    time = t + dt;
    applyGhostState();
    copyQVelocityGradient();
    if (cfg.gradhCorrection) { omegaGradh(); applyGhostState(); }
    // postStepFinalize: the ASPHSmoothingScale end-of-step H
    if (cfg.smoothingScale == 2) asphFinalize();
    enforceBoundaries();
    ++cycle;
    lastDt = dt;
    return dt;
  }

  // Conserved totals (SpheralConservation.py:54-150): mass, momentum(3),
  // kinetic, thermal, package (gravity) energy, total energy.
  void conservation(double out[8]) const {
    double m = 0, px = 0, py = 0, pz = 0, ke = 0, te = 0;
    for (int i = 0; i < nInt; ++i) {
      m += mass[i]; px += mass[i] * vel[i].x; py += mass[i] * vel[i].y; pz += mass[i] * vel[i].z;
      ke += 0.5 * mass[i] * mag2(vel[i]); te += mass[i] * eps[i];
    }
    out[0] = m; out[1] = px; out[2] = py; out[3] = pz; out[4] = ke; out[5] = te;
    out[6] = cfg.gravity ? extraEnergy : 0.0; out[7] = ke + te + out[6];
  }
};

}  // namespace orc

//==============================================================================
// C ABI for the test harness (ctypes).
//==============================================================================
using orc::Problem;

extern "C" {

struct orc_config {
  int num_table_points;
  double cfl;
  int use_velocity_magnitude_for_dt, compatible_energy, gradh_correction, xsph, correct_velocity_gradient,
      sum_mass_density_over_all_nodelists, density_update;
  double eps_tensile, n_tensile, Cl, Cq, eps2;
  int linear_in_expansion, quadratic_in_expansion;
  double dt_min, dt_max, dt_growth, last_dt, time;
  int gravity;
  double G, softening, opening, ftimestep;
  int viscosity;
  double eta_crit_frac, eta_fold_frac;
  int smoothing_scale, fix_shape, h_update, evolve_total_energy, radial_only;
  int hydro, rk_volume;
  int kernel, kernel_order;
};

void* orc_create(const orc_config* c) {
  auto* p = new Problem();
  auto& g = p->cfg;
  g.numTablePoints = c->num_table_points; g.cfl = c->cfl; g.useVelocityMagnitudeForDt = c->use_velocity_magnitude_for_dt;
  g.compatibleEnergy = c->compatible_energy; g.gradhCorrection = c->gradh_correction; g.XSPH = c->xsph;
  g.correctVelocityGradient = c->correct_velocity_gradient; g.sumMassDensityOverAllNodeLists = c->sum_mass_density_over_all_nodelists;
  g.densityUpdate = c->density_update; g.epsTensile = c->eps_tensile; g.nTensile = c->n_tensile;
  g.Cl = c->Cl; g.Cq = c->Cq; g.eps2 = c->eps2; g.linearInExpansion = c->linear_in_expansion;
  g.quadraticInExpansion = c->quadratic_in_expansion; g.dtMin = c->dt_min; g.dtMax = c->dt_max; g.dtGrowth = c->dt_growth;
  g.gravity = c->gravity; g.G = c->G; g.softening = c->softening; g.opening = c->opening; g.ftimestep = c->ftimestep;
  g.viscosity = c->viscosity; g.etaCritFrac = c->eta_crit_frac; g.etaFoldFrac = c->eta_fold_frac;
  g.smoothingScale = c->smoothing_scale; g.fixShape = c->fix_shape; g.hUpdate = c->h_update;
  g.evolveTotalEnergy = c->evolve_total_energy; g.radialOnly = c->radial_only;
  g.hydro = c->hydro; g.rkVolume = c->rk_volume;
  g.kernel = c->kernel; g.kernelOrder = c->kernel_order;
  p->lastDt = c->last_dt; p->time = c->time;
  if (g.kernel == 1) p->W.buildFrom(orc::NBSpline3(g.kernelOrder), c->num_table_points);
  else if (g.kernel == 2) p->W.buildFrom(orc::WendlandC2_3(), c->num_table_points);
  else if (g.kernel == 3) p->W.buildFrom(orc::WendlandC4_3(), c->num_table_points);
  else p->W.build(c->num_table_points);
  return p;
}
void orc_destroy(void* h) { delete static_cast<Problem*>(h); }

int orc_set_nodelist(void* h, int L, double nPerh, double hmin, double hmax, double rhoMin, double rhoMax, double gamma) {
  auto* p = static_cast<Problem*>(h);
  if (L < 0) return 1;
  if ((int)p->lists.size() <= L) p->lists.resize(L + 1);
  auto& n = p->lists[L];
  n.nPerh = nPerh; n.hmin = hmin; n.hmax = hmax; n.rhoMin = rhoMin; n.rhoMax = rhoMax; n.gamma = gamma;
  return 0;
}
int orc_set_nodelist_hminratio(void* h, int L, double hminratio) {
  auto* p = static_cast<Problem*>(h);
  if (L < 0) return 1;
  if ((int)p->lists.size() <= L) p->lists.resize(L + 1);
  p->lists[L].hminratio = hminratio;
  return 0;
}
// Eigen-pairs of a symmetric tensor (xx, xy, xz, yy, yz, zz): vals[3],
// vecs[9] row-major with eigenvector k in column k.
int orc_sym_eigen(const double* a, double* vals, double* vecs) {
  const orc::ST t{a[0], a[1], a[2], a[3], a[4], a[5]};
  const orc::EigS e = orc::eigenVectorsS(t);
  for (int k = 0; k < 3; ++k) vals[k] = e.val[k];
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) vecs[3 * r + k] = e.vec[r][k];
  return 0;
}
// radialEvolution of one H (xx xy xz yy yz zz) at position x with scale s
// and start-of-step radius r0.
int orc_radial_evolution(const double* h, const double* x, double s, double r0, double* out) {
  const orc::ST H{h[0], h[1], h[2], h[3], h[4], h[5]};
  const orc::V3 X{x[0], x[1], x[2]};
  const orc::ST r = orc::radialEvolution3(H, orc::unitVector(X), s, r0, orc::mag(X));
  out[0] = r.xx; out[1] = r.xy; out[2] = r.xz; out[3] = r.yy; out[4] = r.yz; out[5] = r.zz;
  return 0;
}
// The ASPH tensor DH/Dt for one (H, DvDx).
int orc_smoothing_scale_derivative(const double* h, const double* d, double* out) {
  const orc::ST H{h[0], h[1], h[2], h[3], h[4], h[5]};
  const orc::T9 D{d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8]};
  const orc::ST r = orc::smoothingScaleDerivative3(H, D);
  out[0] = r.xx; out[1] = r.xy; out[2] = r.xz; out[3] = r.yy; out[4] = r.yz; out[5] = r.zz;
  return 0;
}
// type 0 periodic (lo, hi); type 1 reflecting wall at lo (wall_high=0) or hi (wall_high=1)
int orc_add_boundary(void* h, int type, int axis, double lo, double hi, int wall_high) {
  auto* p = static_cast<Problem*>(h);
  orc::Boundary b; b.type = type; b.axis = axis; b.lo = lo; b.hi = hi; b.wallHigh = wall_high;
  p->bcs.push_back(b);
  return 0;
}
// H given as 6 components per node (xx, xy, xz, yy, yz, zz).
int orc_set_particles(void* h, int n, const double* pos, const double* vel, const double* mass, const double* rho,
                      const double* eps, const double* H, const int* list) {
  auto* p = static_cast<Problem*>(h);
  p->nInt = p->nTot = n;
  p->resizeAll(n);
  p->ctrl.assign(n, -1); p->image.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    p->pos[i] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    p->vel[i] = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
    p->mass[i] = mass[i]; p->rho[i] = rho[i]; p->eps[i] = eps[i];
    p->H[i] = {H[6 * i], H[6 * i + 1], H[6 * i + 2], H[6 * i + 3], H[6 * i + 4], H[6 * i + 5]};
    p->list[i] = list ? list[i] : 0;
    p->omega[i] = 1.0;
  }
  if (p->lists.empty()) p->lists.resize(1);
  p->rhoSum.clear();
  p->resizeDerivs();
  return 0;
}
int orc_initialize(void* h) { static_cast<Problem*>(h)->initialize(); return 0; }
// Ghosts + connectivity + ghost state on the current positions.
int orc_connectivity(void* h) {
  auto* p = static_cast<Problem*>(h);
  p->setGhostNodes(); p->applyGhostState(); p->computeConnectivity();
  return 0;
}
int orc_update_eos(void* h) { auto* p = static_cast<Problem*>(h); p->updateEOS(p->nTot); return 0; }
int orc_sum_density(void* h) {
  auto* p = static_cast<Problem*>(h);
  if (p->cfg.hydro == 1) p->crkSumMassDensity(); else p->sumMassDensity();
  return 0;
}
// CRKSPH: the RK volumes (RKCorrections::preStepInitialize) and the
// corrections (RKCorrections::initialize) of the current state
int orc_rk_volumes(void* h) { static_cast<Problem*>(h)->computeRKVolumes(); return 0; }
int orc_rk_corrections(void* h) { static_cast<Problem*>(h)->computeRKCorrections(); return 0; }
int orc_gradh(void* h) { auto* p = static_cast<Problem*>(h); p->omegaGradh(); return 0; }
int orc_apply_ghosts(void* h) { static_cast<Problem*>(h)->applyGhostState(); return 0; }
int orc_eval_derivs(void* h) {
  auto* p = static_cast<Problem*>(h);
  if (p->cfg.hydro == 1) p->evaluateDerivativesCRK(); else p->evaluateDerivatives();
  p->finalizeDerivatives();
  return 0;
}
double orc_hydro_dt(void* h) { return static_cast<Problem*>(h)->hydroDt(); }
double orc_step(void* h, double maxTime) { return static_cast<Problem*>(h)->step(maxTime); }
int orc_gravity(void* h) {
  auto* p = static_cast<Problem*>(h);
  p->buildTree(); p->applyTreeForces();
  return 0;
}
int orc_num_internal(void* h) { return static_cast<Problem*>(h)->nInt; }
int orc_num_total(void* h) { return static_cast<Problem*>(h)->nTot; }
long orc_num_pairs(void* h) { return (long)static_cast<Problem*>(h)->pairs.size(); }
double orc_time(void* h) { return static_cast<Problem*>(h)->time; }
// Pair list as flat (i, j) with j possibly a ghost; ghosts resolved through
// ctrl/image so the caller can compare against (control index, image code).
int orc_get_pairs(void* h, int* i_out, int* jctrl_out, int* image_out) {
  auto* p = static_cast<Problem*>(h);
  for (size_t k = 0; k < p->pairs.size(); ++k) {
    const int i = p->pairs[k].first, j = p->pairs[k].second;
    i_out[k] = i;
    jctrl_out[k] = j < p->nInt ? j : p->ctrl[j];
    image_out[k] = j < p->nInt ? 0 : p->image[j];
  }
  return 0;
}
int orc_get_num_neighbors(void* h, int* out) {
  auto* p = static_cast<Problem*>(h);
  for (int i = 0; i < p->nInt; ++i) out[i] = p->numNeighbors[i];
  return 0;
}
void orc_conservation(void* h, double* out) { static_cast<Problem*>(h)->conservation(out); }
double orc_extra_energy(void* h) { return static_cast<Problem*>(h)->extraEnergy; }
double orc_dt_min_acc(void* h) { return static_cast<Problem*>(h)->dtMinAcc; }

// Field access by name (internal nodes only).  Returns number of components or -1.
int orc_get_field(void* h, const char* name, double* out) {
  auto* p = static_cast<Problem*>(h);
  const std::string s(name);
  const int n = p->nInt;
  auto sc = [&](const std::vector<double>& f) { for (int i = 0; i < n; ++i) out[i] = f[i]; return 1; };
  auto v3 = [&](const std::vector<orc::V3>& f) {
    for (int i = 0; i < n; ++i) { out[3 * i] = f[i].x; out[3 * i + 1] = f[i].y; out[3 * i + 2] = f[i].z; }
    return 3;
  };
  auto t9 = [&](const std::vector<orc::T9>& f) {
    for (int i = 0; i < n; ++i) {
      const auto& t = f[i]; double* o = out + 9 * i;
      o[0] = t.xx; o[1] = t.xy; o[2] = t.xz; o[3] = t.yx; o[4] = t.yy; o[5] = t.yz; o[6] = t.zx; o[7] = t.zy; o[8] = t.zz;
    }
    return 9;
  };
  auto s6 = [&](const std::vector<orc::ST>& f) {
    for (int i = 0; i < n; ++i) {
      const auto& t = f[i]; double* o = out + 6 * i;
      o[0] = t.xx; o[1] = t.xy; o[2] = t.xz; o[3] = t.yy; o[4] = t.yz; o[5] = t.zz;
    }
    return 6;
  };
  if (s == "position") return v3(p->pos);
  if (s == "velocity") return v3(p->vel);
  if (s == "mass") return sc(p->mass);
  if (s == "massDensity") return sc(p->rho);
  if (s == "specificThermalEnergy") return sc(p->eps);
  if (s == "H") return s6(p->H);
  if (s == "pressure") return sc(p->P);
  if (s == "soundSpeed") return sc(p->cs);
  if (s == "omegaGradh") return sc(p->omega);
  if (s == "massDensitySum") return sc(p->rhoSum);
  if (s == "normalization") return sc(p->normalization);
  if (s == "DxDt") return v3(p->DxDt);
  if (s == "DvDt") return v3(p->DvDt);
  if (s == "DrhoDt") return sc(p->DrhoDt);
  if (s == "DepsDt") return sc(p->DepsDt);
  if (s == "DvDx") return t9(p->DvDx);
  if (s == "ArtificialViscosityVelocityGradient") return t9(p->DvDxQ);
  if (s == "internalDvDx") return t9(p->localDvDx);
  if (s == "gradRho") return v3(p->gradRho);
  if (s == "M") return t9(p->M);
  if (s == "localM") return t9(p->localM);
  if (s == "maxViscousPressure") return sc(p->maxQ);
  if (s == "effViscousPressure") return sc(p->effQ);
  if (s == "XSPHWeightSum") return sc(p->XSPHWeightSum);
  if (s == "XSPHDeltaV") return v3(p->XSPHDeltaV);
  if (s == "DHDt") return s6(p->DHDt);
  if (s == "Hideal") return s6(p->Hideal);
  if (s == "massSecondMoment") return s6(p->massSecond);
  if (s == "massZerothMoment") return sc(p->massZeroth);
  if (s == "massFirstMoment") return v3(p->massFirst);
  if (s == "DvDtGravity") return v3(p->DvDtGrav);
  if (s == "potential") return sc(p->potential);
  if (s == "DepsDtCompatible") return sc(p->DepsDtCompat);
  if (s == "volume") return sc(p->vol);
  if (s == "rkCorrections") {
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 16; ++k) out[16 * i + k] = p->rkc[i][k];
    return 16;
  }
  return -1;
}
// Overwrite a state field (internal nodes) by name.
int orc_set_field(void* h, const char* name, const double* in) {
  auto* p = static_cast<Problem*>(h);
  const std::string s(name);
  const int n = p->nInt;
  if (s == "pressure") { for (int i = 0; i < n; ++i) p->P[i] = in[i]; return 0; }
  if (s == "soundSpeed") { for (int i = 0; i < n; ++i) p->cs[i] = in[i]; return 0; }
  if (s == "omegaGradh") { for (int i = 0; i < n; ++i) p->omega[i] = in[i]; return 0; }
  if (s == "massDensity") { for (int i = 0; i < n; ++i) p->rho[i] = in[i]; return 0; }
  if (s == "specificThermalEnergy") { for (int i = 0; i < n; ++i) p->eps[i] = in[i]; return 0; }
  return -1;
}
// Kernel table export: W, gradW, grad2W coefficient arrays (3*(N1+1) each),
// and the Hermite nperh/Wsum lookups (2*n each).  meta: [N1, xstep, nH,
// nperh_xmin, nperh_xmax, wsum_xmin, wsum_xmax, minNperh, maxNperh].
int orc_table(void* h, double* w, double* g, double* g2, double* nperh, double* wsum, double* meta) {
  auto* p = static_cast<Problem*>(h);
  const auto& W = p->W;
  for (size_t k = 0; k < W.W.c.size(); ++k) { w[k] = W.W.c[k]; g[k] = W.gW.c[k]; g2[k] = W.g2W.c[k]; }
  for (size_t k = 0; k < W.nperhLookup.v.size(); ++k) { nperh[k] = W.nperhLookup.v[k]; wsum[k] = W.wsumLookup.v[k]; }
  meta[0] = (double)W.W.N1; meta[1] = W.W.xstep; meta[2] = (double)W.nperhLookup.N;
  meta[3] = W.nperhLookup.xmin; meta[4] = W.nperhLookup.xmax; meta[5] = W.wsumLookup.xmin; meta[6] = W.wsumLookup.xmax;
  meta[7] = W.minNperh; meta[8] = W.maxNperh; meta[9] = W.extent;
  return 0;
}
static const orc::NBSpline3& nbsplineOf(int order) {   // one normalised kernel per order (orders 1..15)
  static orc::NBSpline3* cache[16] = {nullptr};
  const int o = std::min(15, std::max(1, order));
  if (!cache[o]) cache[o] = new orc::NBSpline3(o);
  return *cache[o];
}
double orc_nbspline_value(int order, double eta) { return nbsplineOf(order).value(eta, 1.0); }
double orc_nbspline_grad(int order, double eta) { return nbsplineOf(order).grad(eta, 1.0); }
double orc_kernel_value(void* h, double eta, double Hdet) { return static_cast<Problem*>(h)->W.kernelValue(eta, Hdet); }
double orc_grad_value(void* h, double eta, double Hdet) {
  double w, g; static_cast<Problem*>(h)->W.kernelAndGradValue(eta, Hdet, w, g); return g;
}
double orc_nperh_lookup(void* h, double wsum) { return static_cast<Problem*>(h)->W.equivalentNodesPerSmoothingScale(wsum); }
double orc_wsum_lookup(void* h, double nperh) { return static_cast<Problem*>(h)->W.equivalentWsum(nperh); }
double orc_bspline_value(double eta) { return orc::BSpline3().value(eta, 1.0); }
double orc_bspline_grad(double eta) { return orc::BSpline3().grad(eta, 1.0); }
// Thread count of the OpenMP loops that follow (the CPU baseline times the
// same sample on all host threads and on one).
int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n >= 1) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
}  // extern "C"
