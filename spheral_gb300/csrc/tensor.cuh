// Symmetric 3x3 tensors of the ASPH path (tensor H) on the device: loads
// and stores in the field bank, images through reflecting walls, the
// closed-form eigenvalues used by the reference for H's extent, a Jacobi
// eigen-decomposition for the tensor functions (bounds, square root) and the
// ASPH tensor DH/Dt.
#pragma once
#include "fields.cuh"

namespace sph {
namespace dev {

struct Sym {
  double xx, xy, xz, yy, yz, zz;
};

__device__ __forceinline__ Sym loadSym(const Fields& F, int first, long i) {
  return Sym{F.f[first][i], F.f[first + 1][i], F.f[first + 2][i], F.f[first + 3][i], F.f[first + 4][i],
             F.f[first + 5][i]};
}
__device__ __forceinline__ void storeSym(Fields& F, int first, long i, const Sym& h) {
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
__device__ __forceinline__ double symDet(const Sym& h) {
  return (h.xx * h.yy * h.zz + h.xy * h.yz * h.xz + h.xz * h.xy * h.yz - h.xx * h.yz * h.yz - h.xy * h.xy * h.zz -
          h.xz * h.yy * h.xz);
}
__device__ __forceinline__ double symMaxAbs(const Sym& h) {
  return fmax(fabs(h.xx), fmax(fabs(h.xy), fmax(fabs(h.xz), fmax(fabs(h.yy), fmax(fabs(h.yz), fabs(h.zz))))));
}
__device__ __forceinline__ Sym symScale(const Sym& h, double s) {
  return Sym{h.xx * s, h.xy * s, h.xz * s, h.yy * s, h.yz * s, h.zz * s};
}
__device__ __forceinline__ Sym symDiv(const Sym& h, double s) {
  return Sym{h.xx / s, h.xy / s, h.xz / s, h.yy / s, h.yz / s, h.zz / s};
}
// GeomSymmetricTensor<3>::Inverse (GeomSymmetricTensorInline.hh:1650-1661)
__device__ __forceinline__ Sym symInverse(const Sym& a) {
  const double d = symDet(a);
  return Sym{(a.yy * a.zz - a.yz * a.yz) / d, (a.yz * a.xz - a.xy * a.zz) / d, (a.xy * a.yz - a.yy * a.xz) / d,
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
__device__ __forceinline__ void symEigen(const Sym& h, double val[3], double V[3][3]) {
  const double fscale = fmax(10.0 * DBL_EPSILON, symMaxAbs(h));
  const double fi = 1.0 / fscale;
  auto z = [](double x) { return fabs(x) < 1.0e-20 ? 0.0 : x; };
  double a00 = z(h.xx * fi), a01 = z(h.xy * fi), a02 = z(h.xz * fi);
  double a11 = z(h.yy * fi), a12 = z(h.yz * fi), a22 = z(h.zz * fi);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) V[r][k] = r == k ? 1.0 : 0.0;
  // one rotation in the (p, q) plane; o is the third index
  auto rot = [&](double& app, double& aqq, double& apq, double& aop, double& aoq, int p, int q) {
    if (apq == 0.0) return;
    const double theta = (aqq - app) / (2.0 * apq);
    const double t = (theta < 0.0 ? -1.0 : 1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
    const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
    app -= t * apq;
    aqq += t * apq;
    apq = 0.0;
    const double op = aop, oq = aoq;
    aop = c * op - s * oq;
    aoq = s * op + c * oq;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double vp = V[k][p], vq = V[k][q];
      V[k][p] = c * vp - s * vq;
      V[k][q] = s * vp + c * vq;
    }
  };
  for (int sweep = 0; sweep < 32; ++sweep) {
    if (a01 * a01 + a02 * a02 + a12 * a12 <= 1.0e-40) break;
    rot(a00, a11, a01, a02, a12, 0, 1);   // plane (0,1); third index 2: a20, a21
    rot(a00, a22, a02, a01, a12, 0, 2);   // plane (0,2); third index 1: a10, a12
    rot(a11, a22, a12, a01, a02, 1, 2);   // plane (1,2); third index 0: a01, a02
  }
  val[0] = a00 * fscale;
  val[1] = a11 * fscale;
  val[2] = a22 * fscale;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double nrm = 1.0 / sqrt(V[0][k] * V[0][k] + V[1][k] * V[1][k] + V[2][k] * V[2][k]);
#pragma unroll
    for (int r = 0; r < 3; ++r) V[r][k] *= nrm;
  }
}

// diag(d) in the frame of the eigenvectors (rotationalTransform).
__device__ __forceinline__ Sym symFromEigen(const double d[3], const double V[3][3]) {
  auto el = [&](int i, int j) { return V[i][0] * d[0] * V[j][0] + V[i][1] * d[1] * V[j][1] + V[i][2] * d[2] * V[j][2]; };
  return Sym{el(0, 0), el(0, 1), el(0, 2), el(1, 1), el(1, 2), el(2, 2)};
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
__device__ __forceinline__ Sym smoothingScaleDerivative(const Sym& H, const double* D) {
  const double Dxx = D[0], Dxy = D[1], Dxz = D[2], Dyx = D[3], Dyy = D[4], Dyz = D[5], Dzx = D[6], Dzy = D[7],
               Dzz = D[8];
  const double AA = H.xx * Dxy - H.xy * (Dxx - Dyy) + H.xz * Dzy - H.yy * Dyx - H.yz * Dzx;
  const double BB = H.xx * Dxz + H.xy * Dyz - H.xz * (Dxx - Dzz) - H.yz * Dyx - H.zz * Dzx;
  const double CC = H.xy * Dxz + H.yy * Dyz - H.yz * (Dyy - Dzz) - H.xz * Dxy - H.zz * Dzy;
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
  return Sym{-H.xx * Dxx + H.xy * (Gdot - Dyx) - H.xz * (Tdot + Dzx),
             H.yy * Gdot - H.yz * Tdot - H.xx * Dxy - H.xy * Dyy - H.xz * Dzy,
             H.yz * Gdot - H.zz * Tdot - H.xx * Dxz - H.xy * Dyz - H.xz * Dzz,
             H.yz * (Phidot - Dzy) - H.xy * (Gdot + Dxy) - H.yy * Dyy,
             H.xy * Tdot - H.yy * Phidot - H.xz * Dxy - H.yz * Dyy - H.zz * Dzy,
             H.xz * (Tdot - Dxz) - H.yz * (Phidot + Dyz) - H.zz * Dzz};
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
