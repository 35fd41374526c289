// Symmetric 3x3 tensors of the ASPH path (tensor H) on the device: loads
// and stores in the field bank, images through reflecting walls, the
// closed-form eigenvalues used by the reference for H's extent, a Jacobi
// eigen-decomposition for the tensor functions (bounds, square root), the
// ASPH tensor DH/Dt and the ASPHClassicSmoothingScale shape of Hideal.  The
// tensor functions are templated on the arithmetic type: FP64 for the FP64
// mode, FP32 for the per-node tail of the mixed mode.
#pragma once
#include <cfloat>
#include "fields.cuh"

namespace sph {
namespace dev {

template <class T>
struct SymT {
  T xx, xy, xz, yy, yz, zz;
};
using Sym = SymT<double>;

template <class T> struct TensorEps;
template <> struct TensorEps<double> {
  static constexpr double eps = DBL_EPSILON;
  static constexpr double offStop = 1.0e-40;   // squared off-diagonal norm ending the Jacobi sweeps
};
template <> struct TensorEps<float> {
  static constexpr float eps = FLT_EPSILON;
  static constexpr float offStop = 1.0e-14f;
};

__device__ __forceinline__ Sym loadSym(const Fields& F, int first, long i) {
  return Sym{F.f[first][i], F.f[first + 1][i], F.f[first + 2][i], F.f[first + 3][i], F.f[first + 4][i],
             F.f[first + 5][i]};
}
template <class T>
__device__ __forceinline__ void storeSym(Fields& F, int first, long i, const SymT<T>& h) {
  F.f[first][i] = h.xx;
  F.f[first + 1][i] = h.xy;
  F.f[first + 2][i] = h.xz;
  F.f[first + 3][i] = h.yy;
  F.f[first + 4][i] = h.yz;
  F.f[first + 5][i] = h.zz;
}

// (R H R).Symmetric() for the mirrors of image code `code`: the off-diagonal
// terms with exactly one index on a mirrored axis change sign.
__device__ __forceinline__ void imageSym(const Grid& g, int code, Sym& h) {
  if (code) {
    const double sx = mirrored(code & 3, g.kindLo[0], g.kindHi[0]) ? -1.0 : 1.0;
    const double sy = mirrored((code >> 2) & 3, g.kindLo[1], g.kindHi[1]) ? -1.0 : 1.0;
    const double sz = mirrored((code >> 4) & 3, g.kindLo[2], g.kindHi[2]) ? -1.0 : 1.0;
    h.xy *= sx * sy;
    h.xz *= sx * sz;
    h.yz *= sy * sz;
  }
}

// H * r (GeomSymmetricTensor * GeomVector), row by row.
__device__ __forceinline__ void symDot(const Sym& h, double x, double y, double z, double& ox, double& oy,
                                       double& oz) {
  ox = h.xx * x + h.xy * y + h.xz * z;
  oy = h.xy * x + h.yy * y + h.yz * z;
  oz = h.xz * x + h.yz * y + h.zz * z;
}
// |H r|^2 with the reference's operation order and no contraction (the
// neighbour criterion of ConnectivityMap must match bit for bit).
__device__ __forceinline__ double eta2ExactSym(const Sym& h, double x, double y, double z) {
  const double ex = __dadd_rn(__dadd_rn(__dmul_rn(h.xx, x), __dmul_rn(h.xy, y)), __dmul_rn(h.xz, z));
  const double ey = __dadd_rn(__dadd_rn(__dmul_rn(h.xy, x), __dmul_rn(h.yy, y)), __dmul_rn(h.yz, z));
  const double ez = __dadd_rn(__dadd_rn(__dmul_rn(h.xz, x), __dmul_rn(h.yz, y)), __dmul_rn(h.zz, z));
  return __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
}
// GeomSymmetricTensor<3>::Determinant (GeomSymmetricTensorInline.hh:1740-1747)
template <class T>
__device__ __forceinline__ T symDet(const SymT<T>& h) {
  return (h.xx * h.yy * h.zz + h.xy * h.yz * h.xz + h.xz * h.xy * h.yz - h.xx * h.yz * h.yz - h.xy * h.xy * h.zz -
          h.xz * h.yy * h.xz);
}
template <class T>
__device__ __forceinline__ T symMaxAbs(const SymT<T>& h) {
  return fmax(fabs(h.xx), fmax(fabs(h.xy), fmax(fabs(h.xz), fmax(fabs(h.yy), fmax(fabs(h.yz), fabs(h.zz))))));
}
template <class T>
__device__ __forceinline__ SymT<T> symScale(const SymT<T>& h, T s) {
  return SymT<T>{h.xx * s, h.xy * s, h.xz * s, h.yy * s, h.yz * s, h.zz * s};
}
template <class T>
__device__ __forceinline__ SymT<T> symDiv(const SymT<T>& h, T s) {
  return SymT<T>{h.xx / s, h.xy / s, h.xz / s, h.yy / s, h.yz / s, h.zz / s};
}
// GeomSymmetricTensor<3>::Inverse (GeomSymmetricTensorInline.hh:1650-1661)
template <class T>
__device__ __forceinline__ SymT<T> symInverse(const SymT<T>& a) {
  const T d = symDet(a);
  return SymT<T>{(a.yy * a.zz - a.yz * a.yz) / d, (a.yz * a.xz - a.xy * a.zz) / d, (a.xy * a.yz - a.yy * a.xz) / d,
                 (a.xx * a.zz - a.xz * a.xz) / d, (a.xy * a.xz - a.xx * a.yz) / d, (a.xx * a.yy - a.xy * a.xy) / d};
}

// Closed-form eigenvalues (GeomSymmetricTensor<3>::eigenValues,
// GeomSymmetricTensorInline.hh:2230-2260, after D. Eberly): the reference's
// measure of a node's extent (cell size, dt node scale).
__device__ __forceinline__ void symEigenValues(const Sym& h, double ev[3]) {
  const double onethird = 1.0 / 3.0;
  const double sqrt3 = 1.7320508075688772;
  const double fscale = fmax(10.0 * DBL_EPSILON, symMaxAbs(h));
  const double fi = 1.0 / fscale;
  const double a00 = h.xx * fi, a01 = h.xy * fi, a02 = h.xz * fi, a11 = h.yy * fi, a12 = h.yz * fi, a22 = h.zz * fi;
  const double c0 = a00 * a11 * a22 + 2.0 * a01 * a02 * a12 - a00 * a12 * a12 - a11 * a02 * a02 - a22 * a01 * a01;
  const double c1 = a00 * a11 - a01 * a01 + a00 * a22 - a02 * a02 + a11 * a22 - a12 * a12;
  const double c2 = a00 + a11 + a22;
  const double c2Div3 = c2 * onethird;
  const double aDiv3 = fmin(0.0, onethird * (c1 - c2 * c2Div3));
  const double mbDiv2 = 0.5 * (c0 + c2Div3 * (2.0 * c2Div3 * c2Div3 - c1));
  const double q = fmin(0.0, mbDiv2 * mbDiv2 + aDiv3 * aDiv3 * aDiv3);
  const double mag = sqrt(-aDiv3);
  const double angle = atan2(sqrt(-q), mbDiv2) * onethird;
  double sn, cs;
  sincos(angle, &sn, &cs);
  ev[0] = fscale * (c2Div3 + 2.0 * mag * cs);
  ev[1] = fscale * (c2Div3 - mag * (cs + sqrt3 * sn));
  ev[2] = fscale * (c2Div3 - mag * (cs - sqrt3 * sn));
}

// Eigen-pairs for the tensor functions (GeomSymmetricTensor<3>::eigenVectors,
// GeomSymmetricTensorInline.hh:2309-2345: scale by the largest element, zero
// elements below 1e-20, then a self-adjoint eigensolver).  Cyclic Jacobi
// rotations; V[r][k] is component r of eigenvector k.  Every caller applies a
// function to the eigenvalues and rotates back (V f(lambda) V^T), which does
// not depend on the order or signs of the pairs.
template <class T>
__device__ __forceinline__ void symEigen(const SymT<T>& h, T val[3], T V[3][3]) {
  const T fscale = fmax(T(10) * TensorEps<T>::eps, symMaxAbs(h));
  const T fi = T(1) / fscale;
  auto z = [](T x) { return fabs(x) < T(1.0e-20) ? T(0) : x; };
  T a00 = z(h.xx * fi), a01 = z(h.xy * fi), a02 = z(h.xz * fi);
  T a11 = z(h.yy * fi), a12 = z(h.yz * fi), a22 = z(h.zz * fi);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) V[r][k] = r == k ? T(1) : T(0);
  // one rotation in the (p, q) plane; o is the third index
  auto rot = [&](T& app, T& aqq, T& apq, T& aop, T& aoq, int p, int q) {
    if (apq == T(0)) return;
    const T theta = (aqq - app) / (T(2) * apq);
    const T t = (theta < T(0) ? T(-1) : T(1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
    const T c = T(1) / sqrt(t * t + T(1)), s = t * c;
    app -= t * apq;
    aqq += t * apq;
    apq = T(0);
    const T op = aop, oq = aoq;
    aop = c * op - s * oq;
    aoq = s * op + c * oq;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const T vp = V[k][p], vq = V[k][q];
      V[k][p] = c * vp - s * vq;
      V[k][q] = s * vp + c * vq;
    }
  };
  for (int sweep = 0; sweep < 32; ++sweep) {
    if (a01 * a01 + a02 * a02 + a12 * a12 <= TensorEps<T>::offStop) break;
    rot(a00, a11, a01, a02, a12, 0, 1);   // plane (0,1); third index 2: a20, a21
    rot(a00, a22, a02, a01, a12, 0, 2);   // plane (0,2); third index 1: a10, a12
    rot(a11, a22, a12, a01, a02, 1, 2);   // plane (1,2); third index 0: a01, a02
  }
  val[0] = a00 * fscale;
  val[1] = a11 * fscale;
  val[2] = a22 * fscale;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const T nrm = T(1) / sqrt(V[0][k] * V[0][k] + V[1][k] * V[1][k] + V[2][k] * V[2][k]);
#pragma unroll
    for (int r = 0; r < 3; ++r) V[r][k] *= nrm;
  }
}

// diag(d) in the frame of the eigenvectors (rotationalTransform).
template <class T>
__device__ __forceinline__ SymT<T> symFromEigen(const T d[3], const T V[3][3]) {
  auto el = [&](int i, int j) { return V[i][0] * d[0] * V[j][0] + V[i][1] * d[1] * V[j][1] + V[i][2] * d[2] * V[j][2]; };
  return SymT<T>{el(0, 0), el(0, 1), el(0, 2), el(1, 1), el(1, 2), el(2, 2)};
}

// min(maxv, max(minv, H)) for a SymTensor and scalar bounds: enforceMinEigenValue
// then enforceMaxEigenValue (GeomSymmetricTensorInline.hh:2578-2640, 2745-2772),
// each returning H unchanged when no eigenvalue needs the bound.  Gershgorin
// discs settle the common case where every eigenvalue is safely inside.
__device__ __forceinline__ Sym symBound(const Sym& h, double minv, double maxv) {
  const double r0 = fabs(h.xy) + fabs(h.xz), r1 = fabs(h.xy) + fabs(h.yz), r2 = fabs(h.xz) + fabs(h.yz);
  const double lo = fmin(h.xx - r0, fmin(h.yy - r1, h.zz - r2));
  const double hi = fmax(h.xx + r0, fmax(h.yy + r1, h.zz + r2));
  if (lo > minv && hi < maxv) return h;
  double val[3], V[3][3];
  Sym r = h;
  symEigen(r, val, V);
  if (fmin(val[0], fmin(val[1], val[2])) < minv) {
    const double d[3] = {fmax(val[0], minv), fmax(val[1], minv), fmax(val[2], minv)};
    r = symFromEigen(d, V);
    symEigen(r, val, V);
  }
  if (fmax(val[0], fmax(val[1], val[2])) > maxv) {
    const double d[3] = {fmin(val[0], maxv), fmin(val[1], maxv), fmin(val[2], maxv)};
    r = symFromEigen(d, V);
  }
  return r;
}

// ASPH tensor DH/Dt for Dim<3> (SmoothingScaleUtilities.hh,
// smoothingScaleDerivative): the rate of H under DvDx (row-major 9) with the
// frame rotation removed.
template <class T>
__device__ __forceinline__ SymT<T> smoothingScaleDerivative(const SymT<T>& H, const T* D) {
  const T Dxx = D[0], Dxy = D[1], Dxz = D[2], Dyx = D[3], Dyy = D[4], Dyz = D[5], Dzx = D[6], Dzy = D[7], Dzz = D[8];
  const T AA = H.xx * Dxy - H.xy * (Dxx - Dyy) + H.xz * Dzy - H.yy * Dyx - H.yz * Dzx;
  const T BB = H.xx * Dxz + H.xy * Dyz - H.xz * (Dxx - Dzz) - H.yz * Dyx - H.zz * Dzx;
  const T CC = H.xy * Dxz + H.yy * Dyz - H.yz * (Dyy - Dzz) - H.xz * Dxy - H.zz * Dzy;
  const T thpt = H.yy + H.zz;
  const T Ga = (H.xx + H.yy) * thpt - H.xz * H.xz;
  const T Gb = (H.yy + H.zz) * H.yz + H.xy * H.xz;
  const T Gc = (H.xx + H.zz) * thpt - H.xy * H.xy;
  const T Gd = thpt * AA + H.xz * CC;
  const T Ge = thpt * BB - H.xy * CC;
  const T ack = T(1) / (Ga * Gc - Gb * Gb);
  const T Gdot = (Gc * Gd - Gb * Ge) * ack;
  const T Tdot = (Gb * Gd - Ga * Ge) * ack;
  const T Phidot = (H.xz * Gdot + H.xy * Tdot + CC) / thpt;
  return SymT<T>{-H.xx * Dxx + H.xy * (Gdot - Dyx) - H.xz * (Tdot + Dzx),
                 H.yy * Gdot - H.yz * Tdot - H.xx * Dxy - H.xy * Dyy - H.xz * Dzy,
                 H.yz * Gdot - H.zz * Tdot - H.xx * Dxz - H.xy * Dyz - H.xz * Dzz,
                 H.yz * (Phidot - Dzy) - H.xy * (Gdot + Dxy) - H.yy * Dyy,
                 H.xy * Tdot - H.yy * Phidot - H.xz * Dxy - H.yz * Dyy - H.zz * Dzy,
                 H.xz * (Tdot - Dxz) - H.yz * (Phidot + Dyz) - H.zz * Dzz};
}

template <class T> __device__ __forceinline__ T rootnu3T(T x) { return (x < T(0) ? T(-1) : T(1)) * pow(fabs(x), T(1) / T(3)); }
template <> __device__ __forceinline__ double rootnu3T<double>(double x) {
  return (x < 0.0 ? -1.0 : 1.0) * pow(fabs(x), 0.3333333333333333);
}

// rotationMatrix (src/Utilities/rotationMatrix.hh:42-61) of the unit vector
// (ux, uy, uz): rows are the new axes, the first along u.
template <class T>
__device__ __forceinline__ void rotationMatrix3(T ux, T uy, T uz, T R[3][3]) {
  const T rxy = sqrt(ux * ux + uy * uy);
  if (fabs(rxy - T(0)) <= T(1.0e-15) * fmax(T(1), fabs(rxy))) {
    R[0][0] = 0; R[0][1] = 0; R[0][2] = uz;
    R[1][0] = 0; R[1][1] = 1; R[1][2] = 0;
    R[2][0] = -uz; R[2][1] = 0; R[2][2] = 0;
  } else {
    R[0][0] = ux; R[0][1] = uy; R[0][2] = uz;
    R[1][0] = -uy / rxy; R[1][1] = ux / rxy; R[1][2] = 0;
    R[2][0] = -ux * uz / rxy; R[2][1] = -uy * uz / rxy; R[2][2] = rxy;
  }
}
// R A R^T (transpose = false) or R^T A R (true) of a symmetric tensor.
template <class T>
__device__ __forceinline__ SymT<T> symRotate(const SymT<T>& A, const T R[3][3], bool transpose) {
  const T a[3][3] = {{A.xx, A.xy, A.xz}, {A.xy, A.yy, A.yz}, {A.xz, A.yz, A.zz}};
  T m[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int l = 0; l < 3; ++l)
          s += (transpose ? R[k][i] : R[i][k]) * a[k][l] * (transpose ? R[l][j] : R[j][l]);
      m[i][j] = s;
    }
  return SymT<T>{m[0][0], m[0][1], m[0][2], m[1][1], m[1][2], m[2][2]};
}
// radialEvolution for Dim<3> (SmoothingScaleUtilities.hh): H in the frame
// whose first axis is the radial direction, the radial extent scaled by 1/s,
// the transverse block by r0/r1 -- (1,2) and (2,1) address one element of a
// SymTensor there, so yz is divided twice -- and back to the lab frame.
template <class T>
__device__ __forceinline__ SymT<T> radialEvolution(const SymT<T>& Hi, T x, T y, T z, T s, T r0) {
  const T r1 = sqrt(x * x + y * y + z * z);
  T ux = T(1), uy = T(0), uz = T(0);   // GeomVector::unitVector
  if (r1 > T(sizeof(T) == 8 ? 1.0e-50 : 0.0)) { ux = x / r1; uy = y / r1; uz = z / r1; }   // 1e-50 is 0 in FP32
  T R[3][3];
  rotationMatrix3(ux, uy, uz, R);
  SymT<T> h = symRotate(Hi, R, false);
  const T fr = r1 * ((r0 < T(0) ? T(-1) : T(1)) / fmax(T(1.0e-30), fabs(r0)));
  h.xx /= s;
  h.yy /= fr;
  h.yz /= fr;
  h.yz /= fr;
  h.zz /= fr;
  return symRotate(h, R, true);
}

// Hideal of ASPHClassicSmoothingScale (ASPHClassicSmoothingScale.cc:205-288)
// from the second moment M2 of the neighbour distribution, H, the ratio s of
// the target to the current nodes per smoothing scale and the NodeList
// limits: the shape from the normalised M2 (eigenvalues of psi^-1/2 floored
// at hminratio of the largest; identity when M2 is not positive definite or
// psiweight is zero), the size as in the SPH IdealH (or H rescaled, with
// fixShape), then the eigenvalues bounded by 1/hmax and
// min(1/hmin, max(1/hmax, smallest) / hminratio).
// radialOnly: H reshaped along the radial direction of x about the origin
// (radialEvolution, the default ASPHRadialFunctor) with r0 its start-of-step
// radius.
template <class T>
__device__ __forceinline__ SymT<T> asphClassicHideal(const SymT<T>& M2, bool m2Positive, const SymT<T>& Hi, T s,
                                                     bool fixShape, T hminInv, T hmaxInv, T hminratio,
                                                     bool radialOnly = false, T x = T(0), T y = T(0), T z = T(0),
                                                     T r0 = T(0)) {
  const T tiny = T(sizeof(T) == 8 ? 1.0e-50 : 0.0);   // 1e-50 is 0 in FP32
  const T psiweight = fmax(T(0), fmin(T(1), T(2) / s - T(1)));
  SymT<T> Hid{T(1), T(0), T(0), T(1), T(0), T(1)};
  T ev[3], V[3][3], d[3];
  if (psiweight > T(0) && symDet(M2) > T(0) && m2Positive) {
    SymT<T> psi = symDiv(M2, symMaxAbs(M2));
    const T dp = symDet(psi);
    if (dp > T(1.0e-10)) psi = symDiv(psi, rootnu3T(fabs(dp) + tiny));
    else psi = SymT<T>{T(1), T(0), T(0), T(1), T(0), T(1)};
    symEigen(psi, ev, V);
#pragma unroll
    for (int k = 0; k < 3; ++k) ev[k] = T(1) / sqrt(ev[k]);
    const T psimin = fmax(ev[0], fmax(ev[1], ev[2])) * hminratio;
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = fmax(psimin, ev[k]);
    psi = symFromEigen(d, V);
    psi = symDiv(psi, rootnu3T(symDet(psi) + tiny));
    symEigen(psi, ev, V);   // psi^(1/2), then its inverse
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = sqrt(fmax(T(0), ev[k]));
    Hid = symInverse(symFromEigen(d, V));
  }
  const T aa = s < T(1) ? T(0.4) * (T(1) + s * s) : T(0.4) * (T(1) + T(1) / (s * s * s + tiny));
  if (fixShape) Hid = symDiv(Hi, T(1) - aa + aa * s);
  else if (radialOnly) Hid = radialEvolution(Hi, x, y, z, T(1) - aa + aa * s, r0);
  else Hid = symScale(Hid, rootnu3T(symDet(Hi)) / (T(1) - aa + aa * s));
  symEigen(Hid, ev, V);
  const T hminEffInv = fmin(hminInv, fmax(hmaxInv, fmin(ev[0], fmin(ev[1], ev[2]))) / hminratio);
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = fmax(hmaxInv, fmin(hminEffInv, ev[k]));
  return symFromEigen(d, V);
}

// The eigenvalue limits of the ASPH smoothing scales: every eigenvalue of H
// within [1/hmax, min(1/hmin, max(1/hmax, smallest)/hminratio)]
// (constructSymTensorWithBoundedDiagonal + rotationalTransform,
// IncrementASPHHtensor.cc:88-92, ASPHSmoothingScale.cc:355-359).
__device__ __forceinline__ Sym limitASPH(const Sym& h, double hminInv, double hmaxInv, double hminratio) {
  double ev[3], V[3][3], d[3];
  symEigen(h, ev, V);
  const double hminEffInv = fmin(hminInv, fmax(hmaxInv, fmin(ev[0], fmin(ev[1], ev[2]))) / hminratio);
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = fmax(hmaxInv, fmin(hminEffInv, ev[k]));
  return symFromEigen(d, V);
}
// IncrementASPHHtensor::update (src/SmoothingScale/IncrementASPHHtensor.cc:37-100)
// for one node: fixShape scales H by the cube root of the determinant ratio
// of the plain increment; radialOnly increments only the radial diagonal
// element in the frame whose first axis is the radial direction of the
// position (x, y, z) before this update; otherwise H += m DH/Dt; then the
// limits.
__device__ __forceinline__ Sym incrementASPHHtensor(const Sym& H, const Sym& D, double m, double x, double y,
                                                    double z, bool fixShape, bool radialOnly, double hminInv,
                                                    double hmaxInv, double hminratio) {
  Sym h;
  if (fixShape) {
    const Sym hp{H.xx + m * D.xx, H.xy + m * D.xy, H.xz + m * D.xz, H.yy + m * D.yy, H.yz + m * D.yz,
                 H.zz + m * D.zz};
    h = symScale(H, rootnu3T(symDet(hp) / symDet(H)));
  } else if (radialOnly) {
    const double r = sqrt(x * x + y * y + z * z);
    double ux = 1.0, uy = 0.0, uz = 0.0;   // GeomVector::unitVector
    if (r > 1.0e-50) { ux = x / r; uy = y / r; uz = z / r; }
    double R[3][3];
    rotationMatrix3(ux, uy, uz, R);
    h = symRotate(H, R, false);
    const Sym dr = symRotate(D, R, false);
    h.xx += m * dr.xx;
    h = symRotate(h, R, true);
  } else {
    h = Sym{H.xx + m * D.xx, H.xy + m * D.xy, H.xz + m * D.xz, H.yy + m * D.yy, H.yz + m * D.yz, H.zz + m * D.zz};
  }
  return limitASPH(h, hminInv, hmaxInv, hminratio);
}

// FP32 mirror of tensor H for the FP32 sweeps and the neighbour pre-filter:
// (xx xy xz yy) (yz zz det(H) lambda_max).
__device__ __forceinline__ void writeTensorMirror(const Fields& F, const Fields32& P, long i) {
  const Sym h = loadSym(F, F_HT_XX, i);
  P.hten[2 * i] = make_float4((float)h.xx, (float)h.xy, (float)h.xz, (float)h.yy);
  P.hten[2 * i + 1] = make_float4((float)h.yz, (float)h.zz, (float)symDet(h), (float)F.f[F_HLMAX][i]);
}
// H_j of a neighbour entry from the mirror, seen through the mirror-axis bits
// mir (dcode layout) of the entry.
__device__ __forceinline__ void loadTensor32(const Fields32& P, int j, uint32_t mir, float4& a, float4& b) {
  a = P.hten[2 * j];
  b = P.hten[2 * j + 1];
  if (mir) {
    const float sx = (mir & 3u) ? -1.f : 1.f, sy = (mir & 12u) ? -1.f : 1.f, sz = (mir & 48u) ? -1.f : 1.f;
    a.y *= sx * sy;
    a.z *= sx * sz;
    b.x *= sy * sz;
  }
}
// H r in FP32 from the mirror (a = xx xy xz yy, b = yz zz . .), fixed order.
__device__ __forceinline__ void symDot32(const float4& a, const float4& b, float x, float y, float z, float& ox,
                                         float& oy, float& oz) {
  ox = __fmaf_rn(a.z, z, __fmaf_rn(a.y, y, __fmul_rn(a.x, x)));
  oy = __fmaf_rn(b.x, z, __fmaf_rn(a.w, y, __fmul_rn(a.y, x)));
  oz = __fmaf_rn(b.y, z, __fmaf_rn(b.x, y, __fmul_rn(a.z, x)));
}
__device__ __forceinline__ float eta2Sym32(const float4& a, const float4& b, float x, float y, float z) {
  float ex, ey, ez;
  symDot32(a, b, x, y, z, ex, ey, ez);
  return __fmaf_rn(ez, ez, __fmaf_rn(ey, ey, __fmul_rn(ex, ex)));
}

// Derived extent of a tensor H: smallest and largest eigenvalue.
__device__ __forceinline__ void symExtent(const Sym& h, double& lmin, double& lmax) {
  double ev[3];
  symEigenValues(h, ev);
  lmin = fmin(ev[0], fmin(ev[1], ev[2]));
  lmax = fmax(ev[0], fmax(ev[1], ev[2]));
}

}  // namespace dev
}  // namespace sph
