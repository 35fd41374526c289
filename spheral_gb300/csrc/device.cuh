// Device helpers shared by the FP64 (hydro.cu) and FP32 (hydro32.cu) sweeps.
#pragma once
#include "kernels.cuh"
#include <cfloat>
#include "tensor.cuh"

namespace sph {
namespace dev {

constexpr double kTiny30 = 1.0e-30;

// Kahan-compensated FP32 accumulation (explicit round-to-nearest so the
// compensation survives contraction); the pair leaves as the FP64 value s - c.
__device__ __forceinline__ void kahanAdd(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}
__device__ __forceinline__ double kahanValue(float s, float c) { return (double)s - (double)c; }
// The same accumulation, or a plain FP32 sum when `plain` (uniform per launch).
__device__ __forceinline__ void sumAdd(float& s, float& c, float x, int plain) {
  if (plain) s = __fadd_rn(s, x);
  else kahanAdd(s, c, x);
}

// eta from eta^2 in the FP32 sweeps: eta^2 times its reciprocal square root
// (the hardware approximation; eta^2 = 0 gives 0), as the pair kernel forms
// its eta_i and eta_j; the density/dt and grad-h sweeps use it too.
__device__ __forceinline__ float etaFromSq(float e2) { return __fmul_rn(e2, rsqrtf(fmaxf(e2, 1.0e-30f))); }

// Velocity of a mirror image: the components along the mirrored axes flip
// (mir: per-axis bits of the entry's cell-offset code that cross a wall).
__device__ __forceinline__ void mirrorVel(uint32_t mir, float& vx, float& vy, float& vz) {
  if (mir) {
    if (mir & 3u) vx = -vx;
    if (mir & 12u) vy = -vy;
    if (mir & 48u) vz = -vz;
  }
}

// Warp-interleaved neighbour storage: slot q of node i lives at
// ((i / 32) * cap + q) * 32 + i % 32, so a warp reading slot q of its 32 nodes
// touches one contiguous 128-byte line.
__device__ __forceinline__ long long nbSlot(long i, int q, int cap) {
  return ((long long)(i >> 5) * cap + q) * 32 + (i & 31);
}

__device__ __forceinline__ void unpackCell(uint32_t cc, int c[3]) {
  c[0] = (int)(cc & 1023u);
  c[1] = (int)((cc >> 10) & 1023u);
  c[2] = (int)((cc >> 20) & 1023u);
}

// Walk the 27 cells around packed cell cc, resolving periodic wrap and
// reflecting mirrors; fn(k, dcode) for every candidate slot k in cell order.
// dcode packs the cell offset per axis (2 bits: 0 -> 0, 1 -> -1, 2 -> +1);
// together with the home cell it identifies the image (imageCode).
template <class Fn>
__device__ __forceinline__ void forEachCandidate(const Grid& g, uint32_t cc, const int* __restrict__ cellStart,
                                                 const int* __restrict__ cellEnd, Fn fn) {
  int c[3];
  unpackCell(cc, c);
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int d[3] = {dx, dy, dz};
        int cell[3];
        int dcode = 0;
        bool ok = true;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          int nn = c[a] + d[a];
          if (d[a] != 0) dcode |= (d[a] < 0 ? 1 : 2) << (2 * a);
          if (nn < 0) {
            if (g.kindLo[a] == AXIS_PERIODIC) nn = g.nc[a] - 1;
            else if (g.kindLo[a] == AXIS_REFLECT) nn = 0;
            else ok = false;
          } else if (nn >= g.nc[a]) {
            if (g.kindHi[a] == AXIS_PERIODIC) nn = 0;
            else if (g.kindHi[a] == AXIS_REFLECT) nn = g.nc[a] - 1;
            else ok = false;
          }
          cell[a] = nn;
        }
        if (!ok) continue;
        const uint32_t key = morton3((uint32_t)cell[0], (uint32_t)cell[1], (uint32_t)cell[2]);
        const int s = cellStart[key], e = cellEnd[key];
        for (int k = s; k < e; ++k) fn(k, dcode);
      }
}

// Image code (2 bits per axis: 0 none, 1 low side, 2 high side) of a
// neighbour entry with cell-offset code dcode seen from home cell c.
__device__ __forceinline__ int imageCode(const Grid& g, const int c[3], int dcode) {
  int code = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int d = (dcode >> (2 * a)) & 3;
    if (d == 1 && c[a] == 0) code |= 1 << (2 * a);
    else if (d == 2 && c[a] == g.nc[a] - 1) code |= 2 << (2 * a);
  }
  return code;
}

// Per-axis bits (dcode layout) of the offsets that cross a reflecting wall
// from home cell c: those neighbour entries are mirror images.
__device__ __forceinline__ uint32_t mirrorMask(const Grid& g, const int c[3]) {
  uint32_t m = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (c[a] == 0 && g.kindLo[a] == AXIS_REFLECT) m |= 1u << (2 * a);
    if (c[a] == g.nc[a] - 1 && g.kindHi[a] == AXIS_REFLECT) m |= 2u << (2 * a);
  }
  return m;
}

// FP32 separation r_i - r_j' on cell-relative coordinates: r = (x_i - x_j')
// - d cell per axis, with x_j' = cell - x_j for a mirror image.  Periodic
// images need no box arithmetic: the cell offset d carries the wrap.
__device__ __forceinline__ void relSep(const float4& pi, const float4& pj, int dcode, uint32_t mm, float cx,
                                       float cy, float cz, float& rx, float& ry, float& rz) {
  float xj = pj.x, yj = pj.y, zj = pj.z;
  const uint32_t mir = (uint32_t)dcode & mm;
  if (mir) {
    if (mir & 3u) xj = cx - xj;
    if (mir & 12u) yj = cy - yj;
    if (mir & 48u) zj = cz - zj;
  }
  const int d0 = dcode & 3, d1 = (dcode >> 2) & 3, d2 = (dcode >> 4) & 3;
  const float ox = d0 == 1 ? cx : (d0 == 2 ? -cx : 0.0f);
  const float oy = d1 == 1 ? cy : (d1 == 2 ? -cy : 0.0f);
  const float oz = d2 == 1 ? cz : (d2 == 2 ? -cz : 0.0f);
  rx = __fadd_rn(__fsub_rn(pi.x, xj), ox);
  ry = __fadd_rn(__fsub_rn(pi.y, yj), oy);
  rz = __fadd_rn(__fsub_rn(pi.z, zj), oz);
}

// The cell offset (ox, oy, oz) of each of the 64 cell-offset codes of a
// neighbour entry, staged once per block: relSepTab then reads it with one
// shared load instead of decoding the code per pair.
__device__ __forceinline__ void fillCellOffsets(float4* sOff, float cx, float cy, float cz) {
  for (int t = threadIdx.x; t < 64; t += blockDim.x) {
    const int d0 = t & 3, d1 = (t >> 2) & 3, d2 = (t >> 4) & 3;
    sOff[t] = make_float4(d0 == 1 ? cx : (d0 == 2 ? -cx : 0.0f), d1 == 1 ? cy : (d1 == 2 ? -cy : 0.0f),
                          d2 == 1 ? cz : (d2 == 2 ? -cz : 0.0f), 0.0f);
  }
}
// relSep with the offsets from the staged table (bitwise the same result).
__device__ __forceinline__ void relSepTab(const float4& pi, const float4& pj, int dcode, uint32_t mm, float cx,
                                          float cy, float cz, const float4* __restrict__ sOff, float& rx, float& ry,
                                          float& rz) {
  float xj = pj.x, yj = pj.y, zj = pj.z;
  const uint32_t mir = (uint32_t)dcode & mm;
  if (mir) {
    if (mir & 3u) xj = cx - xj;
    if (mir & 12u) yj = cy - yj;
    if (mir & 48u) zj = cz - zj;
  }
  const float4 o = sOff[dcode];
  rx = __fadd_rn(__fsub_rn(pi.x, xj), o.x);
  ry = __fadd_rn(__fsub_rn(pi.y, yj), o.y);
  rz = __fadd_rn(__fsub_rn(pi.z, zj), o.z);
}

__device__ __forceinline__ void imagePos(const Grid& g, int code, double& x, double& y, double& z) {
  if (code) {
    x = imageCoord(x, code & 3, g.kindLo[0], g.kindHi[0], g.wallLo[0], g.wallHi[0]);
    y = imageCoord(y, (code >> 2) & 3, g.kindLo[1], g.kindHi[1], g.wallLo[1], g.wallHi[1]);
    z = imageCoord(z, (code >> 4) & 3, g.kindLo[2], g.kindHi[2], g.wallLo[2], g.wallHi[2]);
  }
}
__device__ __forceinline__ void imageVec(const Grid& g, int code, double& x, double& y, double& z) {
  if (code) {
    if (mirrored(code & 3, g.kindLo[0], g.kindHi[0])) x = -x;
    if (mirrored((code >> 2) & 3, g.kindLo[1], g.kindHi[1])) y = -y;
    if (mirrored((code >> 4) & 3, g.kindLo[2], g.kindHi[2])) z = -z;
  }
}

// Tensor seen through the image: a mirror along axis a is R = I - 2 e_a e_a,
// and R T R flips every component with exactly one index on a mirrored axis.
__device__ __forceinline__ void imageTensor(const Grid& g, int code, double* T) {
  if (code) {
    const double s[3] = {mirrored(code & 3, g.kindLo[0], g.kindHi[0]) ? -1.0 : 1.0,
                         mirrored((code >> 2) & 3, g.kindLo[1], g.kindHi[1]) ? -1.0 : 1.0,
                         mirrored((code >> 4) & 3, g.kindLo[2], g.kindHi[2]) ? -1.0 : 1.0};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) T[3 * r + c] *= s[r] * s[c];
  }
}

// QuadraticInterpolatorView lookup shared by W and dW/deta
// (src/Utilities/QuadraticInterpolatorViewInline.hh:17-21,71-77).
__device__ __forceinline__ int tableIndex(double eta, int N1, double xstep) {
  const long k = (long)(fmax(0.0, eta) / xstep);
  return 3 * (int)min((long)N1, k);
}
__device__ __forceinline__ double tableEval(const double* c, int i0, double x) {
  return c[i0] + (c[i0 + 1] + c[i0 + 2] * x) * x;
}

__device__ __forceinline__ double blockMin(double v, double* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sm[lane] : DBL_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  __syncthreads();
  return v;
}
__device__ __forceinline__ double blockMax(double v, double* sm) { return -blockMin(-v, sm); }
__device__ __forceinline__ double blockSum(double v, double* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}


__device__ __forceinline__ double hermiteLookup(const double* __restrict__ v, const HydroParams& hp, double x) {
  // CubicHermiteInterpolatorView::operator() (CubicHermiteInterpolatorViewInline.hh:10-36)
  const int N = hp.hermN;
  if (x < hp.hermXmin) return v[0] + v[N] * (x - hp.hermXmin);
  if (x > hp.hermXmax) return v[N - 1] + v[2 * N - 1] * (x - hp.hermXmin);
  long k = (long)(fmax(0.0, x - hp.hermXmin) / hp.hermXstep);
  const int i0 = (int)min((long)(N - 2), k);
  const double t = fmax(0.0, fmin(1.0, (x - hp.hermXmin - i0 * hp.hermXstep) / hp.hermXstep));
  const double t2 = t * t, t3 = t * t2;
  return ((2.0 * t3 - 3.0 * t2 + 1.0) * v[i0] + (-2.0 * t3 + 3.0 * t2) * v[i0 + 1] +
          hp.hermXstep * ((t3 - 2.0 * t2 + t) * v[N + i0] + (t3 - t2) * v[N + i0 + 1]));
}

// Per-node completion shared by the FP64 and FP32 pair kernels: self terms,
// corrected velocity gradient, continuity, XSPH, and the IdealH update.
struct NodeAcc {
  double rhoSum, norm, dvx, dvy, dvz, deps, gx, gy, gz, maxQ, effQ, xw, xdx, xdy, xdz, m0, m1x, m1y, m1z;
  double D[9], M[9];
  double m2[6];   // ASPH second moment (xx xy xz yy yz zz)
};

// SPH finalize (SPH.cc:480-552): self terms, the corrected velocity gradient,
// continuity and XSPH; D returns the final DvDx.
__device__ __forceinline__ void finalizeHydro(Fields& F, long i, const NodeAcc& a, double mi, double rhoi,
                                              double vxi, double vyi, double vzi, double Hdeti, int numNb,
                                              const HydroParams& hp, double* D) {
  F.f[F_RHOSUM][i] = a.rhoSum + mi * hp.W0 * Hdeti;
  F.f[F_NORM][i] = a.norm + mi / rhoi * hp.W0 * Hdeti;
  double Mm[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) { D[k] = a.D[k]; Mm[k] = a.M[k]; }
  const double detM = (Mm[0] * Mm[4] * Mm[8] + Mm[1] * Mm[5] * Mm[6] + Mm[2] * Mm[3] * Mm[7] -
                       Mm[0] * Mm[5] * Mm[7] - Mm[1] * Mm[3] * Mm[8] - Mm[2] * Mm[4] * Mm[6]);
  if (hp.correctVelGrad && fabs(detM) > 1.0e-10 && numNb > 8) {
    // GeomTensor<3>::Inverse (src/Geometry/GeomTensorInline.hh:1885-1890)
    const double inv[9] = {(Mm[4] * Mm[8] - Mm[5] * Mm[7]) / detM, (Mm[2] * Mm[7] - Mm[1] * Mm[8]) / detM,
                           (Mm[1] * Mm[5] - Mm[2] * Mm[4]) / detM, (Mm[5] * Mm[6] - Mm[3] * Mm[8]) / detM,
                           (Mm[0] * Mm[8] - Mm[2] * Mm[6]) / detM, (Mm[2] * Mm[3] - Mm[0] * Mm[5]) / detM,
                           (Mm[3] * Mm[7] - Mm[4] * Mm[6]) / detM, (Mm[1] * Mm[6] - Mm[0] * Mm[7]) / detM,
                           (Mm[0] * Mm[4] - Mm[1] * Mm[3]) / detM};
    double R[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        R[3 * r + c] = D[3 * r] * inv[c] + D[3 * r + 1] * inv[3 + c] + D[3 * r + 2] * inv[6 + c];
#pragma unroll
    for (int k = 0; k < 9; ++k) { D[k] = R[k]; Mm[k] = inv[k]; }
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k) D[k] /= rhoi;
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) { F.f[F_DVDX_XX + k][i] = D[k]; F.f[F_M_XX + k][i] = Mm[k]; }
  F.f[F_GRADRHO_X][i] = a.gx / rhoi;
  F.f[F_GRADRHO_Y][i] = a.gy / rhoi;
  F.f[F_GRADRHO_Z][i] = a.gz / rhoi;
  const double trace = D[0] + D[4] + D[8];
  F.f[F_DRHODT][i] = -rhoi * trace;
  F.f[F_DVDT_X][i] = a.dvx;
  F.f[F_DVDT_Y][i] = a.dvy;
  F.f[F_DVDT_Z][i] = a.dvz;
  // evolveTotalEnergy: the total-energy rate m (v . DvDt + DepsDt) (SPH.cc:541)
  F.f[F_DEPSDT][i] = hp.totalEnergy ? mi * ((vxi * a.dvx + vyi * a.dvy + vzi * a.dvz) + a.deps) : a.deps;
  F.f[F_MAXQ][i] = a.maxQ;
  F.f[F_EFFQ][i] = a.effQ;
  double xw = a.xw;
  if (hp.xsph) {
    xw += Hdeti * mi / rhoi * hp.W0;
    const double ws = fmax(kTiny30, xw);
    F.f[F_DXDT_X][i] = vxi + a.xdx / ws;
    F.f[F_DXDT_Y][i] = vyi + a.xdy / ws;
    F.f[F_DXDT_Z][i] = vzi + a.xdz / ws;
  } else {
    F.f[F_DXDT_X][i] = vxi;
    F.f[F_DXDT_Y][i] = vyi;
    F.f[F_DXDT_Z][i] = vzi;
  }
  F.f[F_XSPHW][i] = xw;
  F.f[F_XSPHDV_X][i] = a.xdx;
  F.f[F_XSPHDV_Y][i] = a.xdy;
  F.f[F_XSPHDV_Z][i] = a.xdz;
}

__device__ __forceinline__ void finalizeNode(Fields& F, long i, int li, const NodeAcc& a, double mi, double rhoi,
                                             double vxi, double vyi, double vzi, double ai, int numNb,
                                             const HydroParams& hp, const double* __restrict__ herm) {
  double D[9];
  finalizeHydro(F, i, a, mi, rhoi, vxi, vyi, vzi, (ai * ai) * ai, numNb, hp, D);
  const double trace = D[0] + D[4] + D[8];
  // SPHSmoothingScale finalize (SPHSmoothingScale.cc:235-270)
  const NodeListParams L = hp.lists[li];
  const double m0s = fmax(0.0, a.m0);
  const double m0 = m0s < 0.0 ? -pow(-m0s, 0.3333333333333333) : pow(m0s, 0.3333333333333333);
  F.f[F_M0][i] = m0;
  F.f[F_M1_X][i] = a.m1x;
  F.f[F_M1_Y][i] = a.m1y;
  F.f[F_M1_Z][i] = a.m1z;
  F.f[F_DHDT][i] = ((-ai) / 3.0) * trace;
  const bool iso = fabs(m0 - 0.0) <= 1.0e-15 * fmax(1.0, fabs(m0));
  const double cur = iso ? 0.5 * L.nPerh : fmax(0.0, hermiteLookup(herm, hp, m0));
  const double s = fmin(4.0, fmax(0.25, L.nPerh / (cur + 1.0e-30)));
  const double aa = s < 1.0 ? 0.4 * (1.0 + s * s) : 0.4 * (1.0 + 1.0 / (s * s * s));
  const double hi0 = 1.0 / ai;
  const double hi1 = fmin(L.hmax, fmax(L.hmin, hi0 * (1.0 - aa + aa * s)));
  F.f[F_HIDEAL][i] = 1.0 / hi1;
}


// ASPHClassicSmoothingScale node part (ASPHClassicSmoothingScale.cc:180-291):
// tensor DH/Dt and Hideal (asphClassicHideal) from the moments.
__device__ __forceinline__ void finalizeNodeASPH(Fields& F, long i, int li, const NodeAcc& a, const Sym& Hi,
                                                 double mi, double rhoi, double vxi, double vyi, double vzi,
                                                 int numNb, const HydroParams& hp, const double* __restrict__ herm) {
  double D[9];
  finalizeHydro(F, i, a, mi, rhoi, vxi, vyi, vzi, symDet(Hi), numNb, hp, D);
  const NodeListParams L = hp.lists[li];
  storeSym(F, F_DHDTT_XX, i, smoothingScaleDerivative(Hi, D));
  if (hp.asphEnd) return;   // ASPHSmoothingScale: the ideal H comes at the end of the step
  const double m0 = rootnu3T(fmax(0.0, a.m0));
  F.f[F_M0][i] = m0;
  F.f[F_M1_X][i] = a.m1x;
  F.f[F_M1_Y][i] = a.m1y;
  F.f[F_M1_Z][i] = a.m1z;
  const Sym M2{a.m2[0], a.m2[1], a.m2[2], a.m2[3], a.m2[4], a.m2[5]};
  storeSym(F, F_M2_XX, i, M2);
  const bool isolated = fabs(m0) <= 1.0e-15 * fmax(1.0, fabs(m0));
  const double cur = isolated ? 0.5 * L.nPerh : fmax(0.0, hermiteLookup(herm, hp, m0));
  const double s = fmin(4.0, fmax(0.25, L.nPerh / cur));
  double ev[3];
  symEigenValues(M2, ev);
  storeSym(F, F_HIDEALT_XX, i,
           asphClassicHideal(M2, fmin(ev[0], fmin(ev[1], ev[2])) > 0.0, Hi, s, hp.fixShape != 0, L.hminInv,
                             L.hmaxInv, L.hminratio, hp.radialOnly != 0, F.f[F_X][i], F.f[F_Y][i], F.f[F_Z][i],
                             F.f[F_RAD0][i]));
}

// FP32 variant of finalizeNode for the mixed mode: the per-node completion
// (3x3 inverse, corrected gradient, IdealH lookup) in FP32, results stored in
// the FP64 fields.  GB300 runs FP64 at a small fraction of the FP32 rate, so
// per-node FP64 work is visible even next to a ~100-neighbour pair loop.
__device__ __forceinline__ float hermiteLookup32(const double* __restrict__ v, const HydroParams& hp, float x) {
  const int N = hp.hermN;
  const float xmin = (float)hp.hermXmin, xmax = (float)hp.hermXmax, st = (float)hp.hermXstep;
  if (x < xmin) return (float)v[0] + (float)v[N] * (x - xmin);
  if (x > xmax) return (float)v[N - 1] + (float)v[2 * N - 1] * (x - xmin);
  const int i0 = min(N - 2, (int)(fmaxf(0.0f, x - xmin) / st));
  const float t = fmaxf(0.0f, fminf(1.0f, (x - xmin - i0 * st) / st));
  const float t2 = t * t, t3 = t * t2;
  return ((2.0f * t3 - 3.0f * t2 + 1.0f) * (float)v[i0] + (-2.0f * t3 + 3.0f * t2) * (float)v[i0 + 1] +
          st * ((t3 - 2.0f * t2 + t) * (float)v[N + i0] + (t3 - t2) * (float)v[N + i0 + 1]));
}

struct NodeAcc32 {
  float rhoSum, norm, gx, gy, gz, maxQ, effQ, xw, xdx, xdy, xdz, m0, m1x, m1y, m1z;
  double dvx, dvy, dvz, deps;
  float D[9], M[9];
  float m2[6];      // TENSOR: ASPH second moment
  float4 h0, h1;    // TENSOR: the node's H mirror
};

// TENSOR: ASPHClassicSmoothingScale in FP32 (tensor DH/Dt, asphClassicHideal).
template <bool TENSOR>
__device__ __forceinline__ void finalizeNode32(Fields& F, long i, int li, const NodeAcc32& a, int numNb,
                                               const HydroParams& hp, const double* __restrict__ herm) {
  const float mi = (float)F.f[F_MASS][i], rhoi = (float)F.f[F_RHO][i], ai = (float)F.f[F_HINV][i];
  const float Hdeti = TENSOR ? a.h1.z : (ai * ai) * ai;
  const float W0 = (float)hp.W0;
  F.f[F_RHOSUM][i] = a.rhoSum + mi * W0 * Hdeti;
  F.f[F_NORM][i] = a.norm + mi / rhoi * W0 * Hdeti;
  float D[9], Mm[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) { D[k] = a.D[k]; Mm[k] = a.M[k]; }
  const float detM = (Mm[0] * Mm[4] * Mm[8] + Mm[1] * Mm[5] * Mm[6] + Mm[2] * Mm[3] * Mm[7] -
                      Mm[0] * Mm[5] * Mm[7] - Mm[1] * Mm[3] * Mm[8] - Mm[2] * Mm[4] * Mm[6]);
  const float irho = 1.0f / rhoi;
  if (hp.correctVelGrad && fabsf(detM) > 1.0e-10f && numNb > 8) {
    const float id = 1.0f / detM;
    const float inv[9] = {(Mm[4] * Mm[8] - Mm[5] * Mm[7]) * id, (Mm[2] * Mm[7] - Mm[1] * Mm[8]) * id,
                          (Mm[1] * Mm[5] - Mm[2] * Mm[4]) * id, (Mm[5] * Mm[6] - Mm[3] * Mm[8]) * id,
                          (Mm[0] * Mm[8] - Mm[2] * Mm[6]) * id, (Mm[2] * Mm[3] - Mm[0] * Mm[5]) * id,
                          (Mm[3] * Mm[7] - Mm[4] * Mm[6]) * id, (Mm[1] * Mm[6] - Mm[0] * Mm[7]) * id,
                          (Mm[0] * Mm[4] - Mm[1] * Mm[3]) * id};
    float R[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        R[3 * r + c] = D[3 * r] * inv[c] + D[3 * r + 1] * inv[3 + c] + D[3 * r + 2] * inv[6 + c];
#pragma unroll
    for (int k = 0; k < 9; ++k) { D[k] = R[k]; Mm[k] = inv[k]; }
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k) D[k] *= irho;
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) { F.f[F_DVDX_XX + k][i] = D[k]; F.f[F_M_XX + k][i] = Mm[k]; }
  F.f[F_GRADRHO_X][i] = a.gx * irho;
  F.f[F_GRADRHO_Y][i] = a.gy * irho;
  F.f[F_GRADRHO_Z][i] = a.gz * irho;
  const float trace = D[0] + D[4] + D[8];
  F.f[F_DRHODT][i] = -(double)rhoi * trace;
  F.f[F_DVDT_X][i] = a.dvx;
  F.f[F_DVDT_Y][i] = a.dvy;
  F.f[F_DVDT_Z][i] = a.dvz;
  F.f[F_DEPSDT][i] = hp.totalEnergy
                         ? (double)mi * ((F.f[F_VX][i] * a.dvx + F.f[F_VY][i] * a.dvy + F.f[F_VZ][i] * a.dvz) + a.deps)
                         : a.deps;
  F.f[F_MAXQ][i] = a.maxQ;
  F.f[F_EFFQ][i] = a.effQ;
  float xw = a.xw;
  const double vxi = F.f[F_VX][i], vyi = F.f[F_VY][i], vzi = F.f[F_VZ][i];
  if (hp.xsph) {
    xw += Hdeti * mi * irho * W0;
    const float ws = fmaxf(1.0e-30f, xw);
    F.f[F_DXDT_X][i] = vxi + a.xdx / ws;
    F.f[F_DXDT_Y][i] = vyi + a.xdy / ws;
    F.f[F_DXDT_Z][i] = vzi + a.xdz / ws;
  } else {
    F.f[F_DXDT_X][i] = vxi;
    F.f[F_DXDT_Y][i] = vyi;
    F.f[F_DXDT_Z][i] = vzi;
  }
  F.f[F_XSPHW][i] = xw;
  F.f[F_XSPHDV_X][i] = a.xdx;
  F.f[F_XSPHDV_Y][i] = a.xdy;
  F.f[F_XSPHDV_Z][i] = a.xdz;
  const NodeListParams L = hp.lists[li];
  const float m0 = cbrtf(fmaxf(0.0f, a.m0));
  if (!(TENSOR && hp.asphEnd)) {
    F.f[F_M0][i] = m0;
    F.f[F_M1_X][i] = a.m1x;
    F.f[F_M1_Y][i] = a.m1y;
    F.f[F_M1_Z][i] = a.m1z;
  }
  if (TENSOR) {
    const SymT<float> Hi{a.h0.x, a.h0.y, a.h0.z, a.h0.w, a.h1.x, a.h1.y};
    storeSym(F, F_DHDTT_XX, i, smoothingScaleDerivative(Hi, D));
    if (hp.asphEnd) return;   // ASPHSmoothingScale: the ideal H comes at the end of the step
    const SymT<float> M2{a.m2[0], a.m2[1], a.m2[2], a.m2[3], a.m2[4], a.m2[5]};
    storeSym(F, F_M2_XX, i, M2);
    const float nPerh = (float)L.nPerh;
    const bool isolated = fabsf(m0) <= 1.0e-15f * fmaxf(1.0f, fabsf(m0));
    const float cur = isolated ? 0.5f * nPerh : fmaxf(0.0f, hermiteLookup32(herm, hp, m0));
    const float s = fminf(4.0f, fmaxf(0.25f, nPerh / cur));
    // positive definite (Sylvester): every eigenvalue of M2 positive
    const bool pd = M2.xx > 0.0f && M2.xx * M2.yy - M2.xy * M2.xy > 0.0f && symDet(M2) > 0.0f;
    storeSym(F, F_HIDEALT_XX, i,
             asphClassicHideal(M2, pd, Hi, s, hp.fixShape != 0, (float)L.hminInv, (float)L.hmaxInv,
                               (float)L.hminratio, hp.radialOnly != 0, (float)F.f[F_X][i], (float)F.f[F_Y][i],
                               (float)F.f[F_Z][i], (float)F.f[F_RAD0][i]));
    return;
  }
  // FP32 forms of DHDt = -(H/3) tr(DvDx) and of the IdealH clamp
  // 1/clamp(h0 f, hmin, hmax) = clamp(H0 / f, 1/hmax, 1/hmin): no FP64 divide.
  F.f[F_DHDT][i] = (double)(-(ai * (1.0f / 3.0f)) * trace);
  const float nPerh = (float)L.nPerh;
  const bool iso = fabsf(m0) <= 1.0e-15f * fmaxf(1.0f, fabsf(m0));
  const float cur = iso ? 0.5f * nPerh : fmaxf(0.0f, hermiteLookup32(herm, hp, m0));
  const float s = fminf(4.0f, fmaxf(0.25f, nPerh / (cur + 1.0e-30f)));
  const float aa = s < 1.0f ? 0.4f * (1.0f + s * s) : 0.4f * (1.0f + 1.0f / (s * s * s));
  const double hid = (double)(ai / (1.0f - aa + aa * s));
  F.f[F_HIDEAL][i] = fmin(L.hminInv, fmax(L.hmaxInv, hid));
}

}  // namespace dev
}  // namespace sph
