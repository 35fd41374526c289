// Mixed-precision CRKSPH sweeps (LinearOrder): the RK sum volume, the CRK
// mass density, the correction moments and the pair loop in FP32 on the
// cell-relative mirror, the per-node completions (volume caps, the 4x4
// correction solve, the node finalize) and every stored field in FP64.
//
// Precision design, as the mixed SPH path:
//  * separations are formed from cell-relative FP32 positions;
//  * the corrected kernels and the pair force are evaluated with explicit
//    round-to-nearest intrinsics in one fixed order, so W^R(-r_ij, H_i, C_j)
//    computed on i's side is bitwise the W^R(r_ji, H_i, C_j) that j's side
//    computes, and the force f_ij = V_i V_j / 2 (P_i + P_j + rho_i e_i +
//    rho_j e_j) (gradW_j - gradW_i) is bitwise antisymmetric;
//  * acceleration and energy-rate sums are Kahan compensated;
//  * the correction moments are accumulated in the eta units of node i
//    (P~ = (1, a_i x)), where the moment matrix is O(1) and well
//    conditioned; C and dC/dx are recovered in FP64 (C_k = s_k C~_k,
//    dC_d = a_i s dC~_d with s = (1, a_i, a_i, a_i)).
#include "device.cuh"

namespace sph {
namespace {
using namespace dev;

inline unsigned gridFor(long n, int b) { return (unsigned)((n + b - 1) / b); }


// Packed table lookup: W and dW/deta at eta (zero beyond the extent).
__device__ __forceinline__ void lookup(const float4* __restrict__ ta, const float2* __restrict__ tb, int N1,
                                       float invStep, float eta, float extent, float& w, float& gr) {
  if (eta < extent) {
    const int k = min(N1, (int)(eta * invStep));
    const float4 A = ta[k];
    const float2 B = tb[k];
    w = __fmaf_rn(__fmaf_rn(A.z, eta, A.y), eta, A.x);
    gr = __fmaf_rn(__fmaf_rn(B.y, eta, B.x), eta, A.w);
  } else {
    w = 0.0f;
    gr = 0.0f;
  }
}

struct Tab32 {
  const float4* ta;
  const float2* tb;
  int N1;
  float invStep, extent;
};

__device__ __forceinline__ Tab32 loadTab32(float4* ta, float2* tb, const TableDev& t, const HydroParams& hp) {
  const int nint = hp.tableN1 + 1;
  for (int k = threadIdx.x; k < nint; k += blockDim.x) { ta[k] = t.p32a[k]; tb[k] = t.p32b[k]; }
  __syncthreads();
  return Tab32{ta, tb, hp.tableN1, (float)(1.0 / hp.tableXstep), (float)hp.extent};
}

// |eta| from eta (MUFU reciprocal square root, deterministic).
__device__ __forceinline__ float etaMag(float ex, float ey, float ez, float& e2, float& re) {
  e2 = __fmaf_rn(ez, ez, __fmaf_rn(ey, ey, __fmul_rn(ex, ex)));
  re = rsqrtf(fmaxf(e2, 1.0e-30f));
  return __fmul_rn(e2, re);
}

// Base kernel of H = a I at eta = a x: w = a^3 W(|eta|), dW = a^3 W'(|eta|) a eta^.
// G returns the bare W'(|eta|) (the SPH moment weight is |G|).
__device__ __forceinline__ void base32(const Tab32& T, float a, float ex, float ey, float ez, float em, float re,
                                       float& w, float& dwx, float& dwy, float& dwz, float& G) {
  float W;
  lookup(T.ta, T.tb, T.N1, T.invStep, em, T.extent, W, G);
  const float Hdet = __fmul_rn(__fmul_rn(a, a), a);
  w = __fmul_rn(Hdet, W);
  const float f = __fmul_rn(__fmul_rn(__fmul_rn(Hdet, G), a), re);
  dwx = __fmul_rn(f, ex);
  dwy = __fmul_rn(f, ey);
  dwz = __fmul_rn(f, ez);
}

// Corrected kernel W^R = (C.P) W and its gradient (C_{1+d} + dC_d.P) W + (C.P) dW_d.
__device__ __forceinline__ void rkEval32(const float* __restrict__ C, float x, float y, float z, float w, float dwx,
                                         float dwy, float dwz, float& WR, float& gx, float& gy, float& gz) {
  const float CP = __fmaf_rn(C[3], z, __fmaf_rn(C[2], y, __fmaf_rn(C[1], x, C[0])));
  const float d0 = __fmaf_rn(C[7], z, __fmaf_rn(C[6], y, __fmaf_rn(C[5], x, C[4])));
  const float d1 = __fmaf_rn(C[11], z, __fmaf_rn(C[10], y, __fmaf_rn(C[9], x, C[8])));
  const float d2 = __fmaf_rn(C[15], z, __fmaf_rn(C[14], y, __fmaf_rn(C[13], x, C[12])));
  gx = __fmaf_rn(CP, dwx, __fmul_rn(__fadd_rn(C[1], d0), w));
  gy = __fmaf_rn(CP, dwy, __fmul_rn(__fadd_rn(C[2], d1), w));
  gz = __fmaf_rn(CP, dwz, __fmul_rn(__fadd_rn(C[3], d2), w));
  WR = __fmul_rn(CP, w);
}

// Coefficients of a mirror image (the reflection operator of the LinearOrder
// coefficients: an entry flips once per index along the wall normal).
__device__ __forceinline__ void mirrorRKC(uint32_t mir, float* C) {
  if (!mir) return;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (!(mir & (3u << (2 * a)))) continue;
    C[1 + a] = -C[1 + a];
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int flips = (d == a ? 1 : 0) + ((k >= 1 && k - 1 == a) ? 1 : 0);
        if (flips == 1) C[4 + 4 * d + k] = -C[4 + 4 * d + k];
      }
  }
}

__device__ __forceinline__ void loadRKC(const float4* __restrict__ rkc, long j, float* C) {
  const float4 a = rkc[4 * j], b = rkc[4 * j + 1], c = rkc[4 * j + 2], d = rkc[4 * j + 3];
  C[0] = a.x; C[1] = a.y; C[2] = a.z; C[3] = a.w;
  C[4] = b.x; C[5] = b.y; C[6] = b.z; C[7] = b.w;
  C[8] = c.x; C[9] = c.y; C[10] = c.z; C[11] = c.w;
  C[12] = d.x; C[13] = d.y; C[14] = d.z; C[15] = d.w;
}

//------------------------------------------------------------------------------
// RKSumVolume: V_i = min(etaVolMax / Hdet_i, 1 / (sum_j W(|H_i r_ij|) + Hdet_i W0)).
//------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) rkSumVolume32(Fields F, Fields32 P, long n, Grid g, NeighborLists nl,
                                                     TableDev t, HydroParams hp) {
  __shared__ float4 ta[kMaxTable / 3];
  __shared__ float2 tb[kMaxTable / 3];
  __shared__ float4 sOff[64];
  const Tab32 T = loadTab32(ta, tb, t, hp);
  fillCellOffsets(sOff, g.cellf[0], g.cellf[1], g.cellf[2]);
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int ci[3];
  unpackCell(P.cell[i], ci);
  const uint32_t mm = mirrorMask(g, ci);
  const float cx = g.cellf[0], cy = g.cellf[1], cz = g.cellf[2];
  const float4 pi = P.posh[i];
  const float ai = pi.w;
  float s = 0.f, c = 0.f;
  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const uint32_t ent = nl.nbr[nbSlot(i, q, nl.cap)];
    const int j = (int)(ent & kIndexMask), dcode = (int)(ent >> kIndexBits);
    float rx, ry, rz;
    relSepTab(pi, P.posh[j], dcode, mm, cx, cy, cz, sOff, rx, ry, rz);
    float e2, re;
    const float em = etaMag(ai * rx, ai * ry, ai * rz, e2, re);
    float W, G;
    lookup(T.ta, T.tb, T.N1, T.invStep, em, T.extent, W, G);
    kahanAdd(s, c, W);
  }
  const double a = F.f[F_HINV][i];
  const double Hdet = (a * a) * a;
  const double halfExt = 0.5 * hp.extent;
  const double etaVolMax = ((halfExt * halfExt) * halfExt) * (4.0 / 3.0 * 3.141592653589793);
  const double V = fmin(etaVolMax / Hdet, 1.0 / (Hdet * kahanValue(s, c) + Hdet * hp.W0));
  F.f[F_VOL][i] = V;
  P.vol[i] = (float)V;
}

//------------------------------------------------------------------------------
// CRK mass density, FP32 sums over the same-NodeList neighbours.
//------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) crkDensity32(Fields F, Fields32 P, const int* __restrict__ list, long n,
                                                    Grid g, NeighborLists nl, TableDev t, HydroParams hp) {
  __shared__ float4 ta[kMaxTable / 3];
  __shared__ float2 tb[kMaxTable / 3];
  __shared__ float4 sOff[64];
  const Tab32 T = loadTab32(ta, tb, t, hp);
  fillCellOffsets(sOff, g.cellf[0], g.cellf[1], g.cellf[2]);
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int ci[3];
  unpackCell(P.cell[i], ci);
  const uint32_t mm = mirrorMask(g, ci);
  const float cx = g.cellf[0], cy = g.cellf[1], cz = g.cellf[2];
  const float4 pi = P.posh[i];
  const bool multi = hp.numLists > 1;
  const int li = list[i];
  float sw = 0.f, cw = 0.f, sr = 0.f, cr = 0.f, sv = 0.f, cv = 0.f;
  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const uint32_t ent = nl.nbr[nbSlot(i, q, nl.cap)];
    const int j = (int)(ent & kIndexMask), dcode = (int)(ent >> kIndexBits);
    if (multi && list[j] != li) continue;
    const float4 pj = P.posh[j];
    float rx, ry, rz;
    relSepTab(pi, pj, dcode, mm, cx, cy, cz, sOff, rx, ry, rz);
    const float aj = pj.w;
    float e2, re;
    const float em = etaMag(aj * rx, aj * ry, aj * rz, e2, re);
    float W, G;
    lookup(T.ta, T.tb, T.N1, T.invStep, em, T.extent, W, G);
    const float Wj = __fmul_rn(__fmul_rn(__fmul_rn(aj, aj), aj), W);
    const float Vj = P.vol[j];
    const float VW = __fmul_rn(Vj, Wj);
    kahanAdd(sw, cw, VW);
    kahanAdd(sr, cr, __fmul_rn(P.velm[j].w, VW));
    kahanAdd(sv, cv, __fmul_rn(Vj, VW));
  }
  const NodeListParams L = hp.lists[li];
  const double ai = F.f[F_HINV][i], mi = F.f[F_MASS][i], Vi = F.f[F_VOL][i];
  const double Hdeti = (ai * ai) * ai;
  const double wsum = kahanValue(sw, cw) + Vi * Hdeti * hp.W0;
  const double vol1 = (kahanValue(sv, cv) + Vi * Vi * Hdeti * hp.W0) / wsum;
  const double rho = fmax(fmax(L.rhoMin, 0.1 * mi * Hdeti),
                          fmin(L.rhoMax, (kahanValue(sr, cr) + mi * Vi * Hdeti * hp.W0) / (wsum * vol1)));
  F.f[F_RHO][i] = rho;
  P.thermo[i].x = (float)rho;
}

//------------------------------------------------------------------------------
// LinearOrder corrections: moments in the eta units of node i (FP32, the
// matrix itself Kahan compensated), the 4x4 solve and the unscaling in FP64.
//------------------------------------------------------------------------------
__device__ __forceinline__ int symIdx(int k, int l) {
  return k <= l ? (k * 4 - (k * (k - 1)) / 2 + (l - k)) : (l * 4 - (l * (l - 1)) / 2 + (k - l));
}

__global__ void __launch_bounds__(128) rkCorrections32(Fields F, Fields32 P, long n, Grid g, NeighborLists nl,
                                                       TableDev t, HydroParams hp) {
  __shared__ float4 ta[kMaxTable / 3];
  __shared__ float2 tb[kMaxTable / 3];
  __shared__ float4 sOff[64];
  const Tab32 T = loadTab32(ta, tb, t, hp);
  fillCellOffsets(sOff, g.cellf[0], g.cellf[1], g.cellf[2]);
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int ci[3];
  unpackCell(P.cell[i], ci);
  const uint32_t mm = mirrorMask(g, ci);
  const float cx = g.cellf[0], cy = g.cellf[1], cz = g.cellf[2];
  const float4 pi = P.posh[i];
  const float ai = pi.w, iai = 1.0f / ai;
  float Ms[10], Mc[10], dM[3][10];
#pragma unroll
  for (int k = 0; k < 10; ++k) { Ms[k] = 0.f; Mc[k] = 0.f; dM[0][k] = 0.f; dM[1][k] = 0.f; dM[2][k] = 0.f; }
  auto add = [&](float vj, float x, float y, float z, float w, float dwx, float dwy, float dwz) {
    // P~ = (1, a_i x); dM^_d = sum V ((e_{1+d} P~ + P~ e_{1+d}) W + P~ P~ dW_d / a_i)
    const float p[4] = {1.0f, ai * x, ai * y, ai * z};
    const float vw = vj * w;
    const float vd[3] = {vj * dwx * iai, vj * dwy * iai, vj * dwz * iai};
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int l = k; l < 4; ++l) {
        const float pp = p[k] * p[l];
        kahanAdd(Ms[symIdx(k, l)], Mc[symIdx(k, l)], vw * pp);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          float tt = vd[d] * pp;
          if (k == 1 + d) tt += vw * p[l];
          if (l == 1 + d) tt += vw * p[k];
          dM[d][symIdx(k, l)] += tt;
        }
      }
  };
  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const uint32_t ent = nl.nbr[nbSlot(i, q, nl.cap)];
    const int j = (int)(ent & kIndexMask), dcode = (int)(ent >> kIndexBits);
    const float4 pj = P.posh[j];
    float rx, ry, rz;
    relSepTab(pi, pj, dcode, mm, cx, cy, cz, sOff, rx, ry, rz);
    const float aj = pj.w;
    const float ex = aj * rx, ey = aj * ry, ez = aj * rz;
    float e2, re;
    const float em = etaMag(ex, ey, ez, e2, re);
    float w, dwx, dwy, dwz, G;
    base32(T, aj, ex, ey, ez, em, re, w, dwx, dwy, dwz, G);
    add(P.vol[j], rx, ry, rz, w, dwx, dwy, dwz);
  }
  {   // self: x = 0, the gradient along the unit vector (1, 0, 0) of a zero eta
    float W, G;
    lookup(T.ta, T.tb, T.N1, T.invStep, 0.0f, T.extent, W, G);
    const float Hdet = ai * ai * ai;
    add(P.vol[i], 0.f, 0.f, 0.f, Hdet * W, Hdet * G * ai, 0.f, 0.f);
  }
  // FP64 solve of M~ C~ = e_0, dC~_d = -M~^-1 (dM^_d C~) (LU, partial pivoting)
  double A[4][4];
  int piv[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    piv[r] = r;
#pragma unroll
    for (int c2 = 0; c2 < 4; ++c2) A[r][c2] = kahanValue(Ms[symIdx(r, c2)], Mc[symIdx(r, c2)]);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    int p = k;
#pragma unroll
    for (int r = k + 1; r < 4; ++r)
      if (fabs(A[r][k]) > fabs(A[p][k])) p = r;
    if (p != k) {
#pragma unroll
      for (int c2 = 0; c2 < 4; ++c2) { const double tmp = A[k][c2]; A[k][c2] = A[p][c2]; A[p][c2] = tmp; }
      const int tp = piv[k]; piv[k] = piv[p]; piv[p] = tp;
    }
    const double inv = 1.0 / A[k][k];
#pragma unroll
    for (int r = k + 1; r < 4; ++r) {
      const double f = A[r][k] * inv;
      A[r][k] = f;
#pragma unroll
      for (int c2 = k + 1; c2 < 4; ++c2) A[r][c2] -= f * A[k][c2];
    }
  }
  auto solve = [&](const double* b, double* x) {
    double yv[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      double v = b[piv[r]];
#pragma unroll
      for (int c2 = 0; c2 < r; ++c2) v -= A[r][c2] * yv[c2];
      yv[r] = v;
    }
#pragma unroll
    for (int r = 3; r >= 0; --r) {
      double v = yv[r];
#pragma unroll
      for (int c2 = r + 1; c2 < 4; ++c2) v -= A[r][c2] * x[c2];
      x[r] = v / A[r][r];
    }
  };
  const double a = (double)ai;
  const double e0[4] = {1.0, 0.0, 0.0, 0.0};
  double Ct[4];
  solve(e0, Ct);
  double C[16];
  C[0] = Ct[0]; C[1] = a * Ct[1]; C[2] = a * Ct[2]; C[3] = a * Ct[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double rhs[4], dC[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      double v = 0.0;
#pragma unroll
      for (int l = 0; l < 4; ++l) v += (double)dM[d][symIdx(k, l)] * Ct[l];
      rhs[k] = -v;
    }
    solve(rhs, dC);
    C[4 + 4 * d] = a * dC[0];
#pragma unroll
    for (int k = 1; k < 4; ++k) C[4 + 4 * d + k] = (a * a) * dC[k];
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) F.f[F_RKC_0 + k][i] = C[k];
#pragma unroll
  for (int k = 0; k < 4; ++k)
    P.rkc[4 * i + k] = make_float4((float)C[4 * k], (float)C[4 * k + 1], (float)C[4 * k + 2], (float)C[4 * k + 3]);
}

//------------------------------------------------------------------------------
// CRKSPH pair loop, FP32.
//------------------------------------------------------------------------------
// U: neighbour slots per loop iteration (1, or 2 with both slots' gathers
// issued together); the slots are evaluated in list order either way, so
// both give the same bits.
template <bool XSPH, bool COMPAT, bool LIMQ, int U = 1>
__global__ void __launch_bounds__(128) pairKernelCRK32(Fields F, Fields32 P, const int* __restrict__ list, long n,
                                                       Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                                                       float* __restrict__ pacc) {
  __shared__ float4 ta[kMaxTable / 3];
  __shared__ float2 tb[kMaxTable / 3];
  __shared__ float4 sOff[64];
  const Tab32 T = loadTab32(ta, tb, t, hp);
  fillCellOffsets(sOff, g.cellf[0], g.cellf[1], g.cellf[2]);
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int ci[3];
  unpackCell(P.cell[i], ci);
  const uint32_t mm = mirrorMask(g, ci);
  const float cx = g.cellf[0], cy = g.cellf[1], cz = g.cellf[2];
  const float4 pi = P.posh[i], vi = P.velm[i], thi = P.thermo[i];
  const bool multi = hp.numLists > 1;
  const int li = list[i];
  const float ai = pi.w, mi = vi.w, rhoi = thi.x, Pi = thi.y, csi = thi.z, Vi = P.vol[i];
  const float invMi = __frcp_rn(mi);
  float Ci[16];
  loadRKC(P.rkc, i, Ci);
  const float Cl = (float)hp.Cl, Cq = (float)hp.Cq, eps2 = (float)hp.eps2;
  const float mClci = __fmul_rn(-Cl, csi);
  const float etaCrit = (float)hp.etaCrit, etaFold = (float)hp.etaFold;
  float DQi[9];
  if (LIMQ) {
    const float4 d0 = P.dvq[3 * i], d1 = P.dvq[3 * i + 1], d2 = P.dvq[3 * i + 2];
    DQi[0] = d0.x; DQi[1] = d0.y; DQi[2] = d0.z; DQi[3] = d0.w;
    DQi[4] = d1.x; DQi[5] = d1.y; DQi[6] = d1.z; DQi[7] = d1.w; DQi[8] = d2.x;
  }
  float sdx = 0.f, cdx = 0.f, sdy = 0.f, cdy = 0.f, sdz = 0.f, cdz = 0.f, se = 0.f, ce = 0.f;
  float maxQ = 0.f, effQ = 0.f, xdx = 0.f, xdy = 0.f, xdz = 0.f, m0 = 0.f, m1x = 0.f, m1y = 0.f, m1z = 0.f;
  float D[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) D[k] = 0.f;

  const int cnt = nl.count[i];
  // One neighbour slot (list slot `slot`, entry `ent`, node j's mirrors and
  // corrections already gathered): its contributions to node i's sums.
  auto pairSlot = [&](long long slot, uint32_t ent, const float4& pj, const float4& vj4, const float4& thj,
                      float Vj, float* Cj) {
    const int j = (int)(ent & kIndexMask), dcode = (int)(ent >> kIndexBits);
    const uint32_t mq = (uint32_t)dcode & mm;
    float rx, ry, rz;
    relSepTab(pi, pj, dcode, mm, cx, cy, cz, sOff, rx, ry, rz);
    float vxj = vj4.x, vyj = vj4.y, vzj = vj4.z;
    mirrorVel(mq, vxj, vyj, vzj);
    const float aj = pj.w, mj = vj4.w, rhoj = thj.x, Pj = thj.y, csj = thj.z;
    const bool same = multi ? (list[j] == li) : true;
    mirrorRKC(mq, Cj);

    const float eix = ai * rx, eiy = ai * ry, eiz = ai * rz;
    const float ejx = aj * rx, ejy = aj * ry, ejz = aj * rz;
    float e2i, e2j, rei, rej;
    const float etai = etaMag(eix, eiy, eiz, e2i, rei);
    const float etaj = etaMag(ejx, ejy, ejz, e2j, rej);
    // W_j = W^R(r_ij, H_j, C_i); W_i = W^R(-r_ij, H_i, C_j)
    float w, dwx, dwy, dwz, G, Wj, gjx, gjy, gjz, Wi, gix, giy, giz, Gi;
    base32(T, aj, ejx, ejy, ejz, etaj, rej, w, dwx, dwy, dwz, G);
    rkEval32(Ci, rx, ry, rz, w, dwx, dwy, dwz, Wj, gjx, gjy, gjz);
    base32(T, ai, -eix, -eiy, -eiz, etai, rei, w, dwx, dwy, dwz, Gi);
    rkEval32(Cj, -rx, -ry, -rz, w, dwx, dwy, dwz, Wi, gix, giy, giz);
    const float dgx = __fsub_rn(gjx, gix), dgy = __fsub_rn(gjy, giy), dgz = __fsub_rn(gjz, giz);

    // Q (the mixed SPH sweep's form; the limited Q symmetric in i and j)
    const float vx = vi.x - vxj, vy = vi.y - vyj, vz = vi.z - vzj;
    float vqx = vx, vqy = vy, vqz = vz;
    if (LIMQ) {
      const float4 d0 = P.dvq[3 * (long)j], d1 = P.dvq[3 * (long)j + 1], d2 = P.dvq[3 * (long)j + 2];
      float Dj[9] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w, d2.x};
      if (mq) {
        const float sg[3] = {(mq & 3u) ? -1.f : 1.f, (mq & 12u) ? -1.f : 1.f, (mq & 48u) ? -1.f : 1.f};
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) Dj[3 * r + cc] *= sg[r] * sg[cc];
      }
      const float hx = 0.5f * rx, hy = 0.5f * ry, hz = 0.5f * rz;
      const float aix = __fmaf_rn(DQi[2], hz, __fmaf_rn(DQi[1], hy, __fmul_rn(DQi[0], hx)));
      const float aiy = __fmaf_rn(DQi[5], hz, __fmaf_rn(DQi[4], hy, __fmul_rn(DQi[3], hx)));
      const float aiz = __fmaf_rn(DQi[8], hz, __fmaf_rn(DQi[7], hy, __fmul_rn(DQi[6], hx)));
      const float ajx = __fmaf_rn(Dj[2], hz, __fmaf_rn(Dj[1], hy, __fmul_rn(Dj[0], hx)));
      const float ajy = __fmaf_rn(Dj[5], hz, __fmaf_rn(Dj[4], hy, __fmul_rn(Dj[3], hx)));
      const float ajz = __fmaf_rn(Dj[8], hz, __fmaf_rn(Dj[7], hy, __fmul_rn(Dj[6], hx)));
      const float gri = __fmaf_rn(aiz, hz, __fmaf_rn(aiy, hy, __fmul_rn(aix, hx)));
      const float grj = __fmaf_rn(ajz, hz, __fmaf_rn(ajy, hy, __fmul_rn(ajx, hx)));
      const float rri = __fdiv_rn(gri, (grj < 0.f ? -1.f : 1.f) * fmaxf(1.0e-30f, fabsf(grj)));
      const float rrj = __fdiv_rn(grj, (gri < 0.f ? -1.f : 1.f) * fmaxf(1.0e-30f, fabsf(gri)));
      const float xl = fminf(rri, rrj);
      float phi = xl > 0.f ? __fdiv_rn(4.0f * xl, __fmul_rn(1.0f + xl, 1.0f + xl)) : 0.f;   // van Leer
      const float etaij = fminf(etai, etaj);
      if (etaij < etaCrit) {
        const float z = __fdiv_rn(etaij - etaCrit, etaFold);
        phi *= expf(-(z * z));
      }
      vqx = __fsub_rn(vx, __fmul_rn(phi, __fadd_rn(aix, ajx)));
      vqy = __fsub_rn(vy, __fmul_rn(phi, __fadd_rn(aiy, ajy)));
      vqz = __fsub_rn(vz, __fmul_rn(phi, __fadd_rn(aiz, ajz)));
    }
    const float mui = __fdividef(__fmaf_rn(vqz, eiz, __fmaf_rn(vqy, eiy, __fmul_rn(vqx, eix))), __fadd_rn(e2i, eps2));
    const float muj = __fdividef(__fmaf_rn(vqz, ejz, __fmaf_rn(vqy, ejy, __fmul_rn(vqx, ejx))), __fadd_rn(e2j, eps2));
    const float mni = fminf(0.f, mui), mnj = fminf(0.f, muj);
    const float li_ = hp.linearInExpansion ? mui : mni;
    const float lj_ = hp.linearInExpansion ? muj : mnj;
    const float qi_ = hp.quadraticInExpansion ? -(mui < 0.f ? -1.f : 1.f) * mui * mui : mni * mni;
    const float qj_ = hp.quadraticInExpansion ? -(muj < 0.f ? -1.f : 1.f) * muj * muj : mnj * mnj;
    const float ei = __fmaf_rn(Cq, qi_, __fmul_rn(mClci, li_));
    const float ej = __fmaf_rn(Cq, qj_, __fmul_rn(__fmul_rn(-Cl, csj), lj_));
    // rho^2 QPi = rho e
    const float Qi = __fmul_rn(rhoi, ei), qj = __fmul_rn(rhoj, ej);
    maxQ = fmaxf(maxQ, 4.0f * Qi);
    effQ += Vj * Qi * Wj;
    // f_ij = V_i V_j / 2 (P_i + P_j + rho_i e_i + rho_j e_j) (gradW_j - gradW_i)
    const float f = __fmul_rn(0.5f, __fmul_rn(Vi, Vj));
    const float s = __fmul_rn(f, __fadd_rn(__fadd_rn(Pi, Pj), __fadd_rn(Qi, qj)));
    const float fx = __fmul_rn(s, dgx), fy = __fmul_rn(s, dgy), fz = __fmul_rn(s, dgz);
    const float ax = __fmul_rn(fx, invMi), ay = __fmul_rn(fy, invMi), az = __fmul_rn(fz, invMi);
    kahanAdd(sdx, cdx, -ax);
    kahanAdd(sdy, cdy, -ay);
    kahanAdd(sdz, cdz, -az);
    if (COMPAT) {
      pacc[3 * slot] = -ax;
      pacc[3 * slot + 1] = -ay;
      pacc[3 * slot + 2] = -az;
    }
    // DepsDt_i += V_i V_j / 2 (P_j + rho_j e_j) v_ij . (gradW_j - gradW_i) / m_i
    const float vdg = __fmaf_rn(vz, dgz, __fmaf_rn(vy, dgy, __fmul_rn(vx, dgx)));
    kahanAdd(se, ce, __fmul_rn(__fmul_rn(__fmul_rn(f, __fadd_rn(Pj, qj)), vdg), invMi));
    const float vvx = Vj * vx, vvy = Vj * vy, vvz = Vj * vz;
    D[0] -= vvx * gjx; D[1] -= vvx * gjy; D[2] -= vvx * gjz;
    D[3] -= vvy * gjx; D[4] -= vvy * gjy; D[5] -= vvy * gjz;
    D[6] -= vvz * gjx; D[7] -= vvz * gjy; D[8] -= vvz * gjz;
    if (XSPH && same) {
      const float xw = Vj * Wj;
      xdx -= xw * vx; xdy -= xw * vy; xdz -= xw * vz;
    }
    // SPHSmoothingScale moments: |W'(|eta_i|)| weights
    const float fw = same ? 1.0f : mj * rhoi / (mi * rhoj);
    const float fwW = fw * fabsf(Gi);
    m0 += fwW;
    m1x -= fwW * eix; m1y -= fwW * eiy; m1z -= fwW * eiz;
  };
  int q = 0;
  if (U == 2) {
    for (; q + 1 < cnt; q += 2) {
      const long long s0 = nbSlot(i, q, nl.cap), s1 = s0 + 32;
      const uint32_t e0 = nl.nbr[s0], e1 = nl.nbr[s1];
      const int j0 = (int)(e0 & kIndexMask), j1 = (int)(e1 & kIndexMask);
      const float4 p0 = P.posh[j0], v0 = P.velm[j0], t0 = P.thermo[j0];
      const float4 p1 = P.posh[j1], v1 = P.velm[j1], t1 = P.thermo[j1];
      const float V0 = P.vol[j0], V1 = P.vol[j1];
      float C0[16], C1[16];
      loadRKC(P.rkc, j0, C0);
      loadRKC(P.rkc, j1, C1);
      pairSlot(s0, e0, p0, v0, t0, V0, C0);
      pairSlot(s1, e1, p1, v1, t1, V1, C1);
    }
  }
  for (; q < cnt; ++q) {
    const long long slot = nbSlot(i, q, nl.cap);
    const uint32_t ent = nl.nbr[slot];
    const int j = (int)(ent & kIndexMask);
    float Cj[16];
    loadRKC(P.rkc, j, Cj);
    pairSlot(slot, ent, P.posh[j], P.velm[j], P.thermo[j], P.vol[j], Cj);
  }
  // node finalize: the sums leave as FP64 values, the per-node arithmetic is
  // FP32 (GB300's FP64 rate would make it visible next to the pair loop)
  const float trace = D[0] + D[4] + D[8];
#pragma unroll
  for (int k = 0; k < 9; ++k) { F.f[F_DVDX_XX + k][i] = D[k]; F.f[F_M_XX + k][i] = 0.0; }
  const double dvx = kahanValue(sdx, cdx), dvy = kahanValue(sdy, cdy), dvz = kahanValue(sdz, cdz);
  const double deps = kahanValue(se, ce);
  F.f[F_DRHODT][i] = (double)(-rhoi * trace);
  F.f[F_DVDT_X][i] = dvx;
  F.f[F_DVDT_Y][i] = dvy;
  F.f[F_DVDT_Z][i] = dvz;
  if (hp.totalEnergy) {
    const double vxd = F.f[F_VX][i], vyd = F.f[F_VY][i], vzd = F.f[F_VZ][i];
    F.f[F_DEPSDT][i] = F.f[F_MASS][i] * ((vxd * dvx + vyd * dvy + vzd * dvz) + deps);
  } else {
    F.f[F_DEPSDT][i] = deps;
  }
  F.f[F_MAXQ][i] = maxQ;
  F.f[F_EFFQ][i] = effQ;
  F.f[F_RHOSUM][i] = 0.0;
  F.f[F_NORM][i] = 0.0;
  F.f[F_GRADRHO_X][i] = 0.0; F.f[F_GRADRHO_Y][i] = 0.0; F.f[F_GRADRHO_Z][i] = 0.0;
  F.f[F_XSPHW][i] = 0.0;
  F.f[F_XSPHDV_X][i] = xdx;
  F.f[F_XSPHDV_Y][i] = xdy;
  F.f[F_XSPHDV_Z][i] = xdz;
  if (XSPH) {
    F.f[F_DXDT_X][i] = F.f[F_VX][i] + xdx;
    F.f[F_DXDT_Y][i] = F.f[F_VY][i] + xdy;
    F.f[F_DXDT_Z][i] = F.f[F_VZ][i] + xdz;
  } else {
    F.f[F_DXDT_X][i] = F.f[F_VX][i];
    F.f[F_DXDT_Y][i] = F.f[F_VY][i];
    F.f[F_DXDT_Z][i] = F.f[F_VZ][i];
  }
  // SPHSmoothingScale finalize in FP32: DHDt = -(H/3) tr(DvDx), Hideal =
  // clamp(H / f, 1/hmax, 1/hmin)
  const NodeListParams L = hp.lists[li];
  const float m0r = cbrtf(fmaxf(0.0f, m0));
  F.f[F_M0][i] = m0r;
  F.f[F_M1_X][i] = m1x;
  F.f[F_M1_Y][i] = m1y;
  F.f[F_M1_Z][i] = m1z;
  F.f[F_DHDT][i] = (double)(-(ai * (1.0f / 3.0f)) * trace);
  const float nPerh = (float)L.nPerh;
  const bool isolated = fabsf(m0r) <= 1.0e-15f * fmaxf(1.0f, fabsf(m0r));
  const float cur = isolated ? 0.5f * nPerh : fmaxf(0.0f, hermiteLookup32(t.herm, hp, m0r));
  const float sr = fminf(4.0f, fmaxf(0.25f, nPerh / (cur + 1.0e-30f)));
  const float aa = sr < 1.0f ? 0.4f * (1.0f + sr * sr) : 0.4f * (1.0f + 1.0f / (sr * sr * sr));
  F.f[F_HIDEAL][i] = fmin(L.hminInv, fmax(L.hmaxInv, (double)(ai / (1.0f - aa + aa * sr))));
}

__global__ void volumeMirrorKernel(Fields F, Fields32 P, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) P.vol[i] = (float)F.f[F_VOL][i];
}

}  // namespace

void launchRKVolumesFP32(Fields F, Fields32 P, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                         cudaStream_t s, LaunchCounter* lc) {
  if (hp.rkVolume == 1) {
    rkSumVolume32<<<gridFor(n, 128), 128, 0, s>>>(F, P, n, g, nl, t, hp);
    lc->add(1);
  } else {   // the per-node volume types in FP64, then the mirror
    launchRKVolumes(F, n, g, nl, t, hp, s, lc);
    volumeMirrorKernel<<<gridFor(n, 256), 256, 0, s>>>(F, P, n);
    lc->add(1);
  }
}
void launchVolumeMirror(Fields F, Fields32 P, long n, cudaStream_t s, LaunchCounter* lc) {
  volumeMirrorKernel<<<gridFor(n, 256), 256, 0, s>>>(F, P, n);
  lc->add(1);
}
void launchCRKDensityFP32(Fields F, Fields32 P, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                          HydroParams hp, cudaStream_t s, LaunchCounter* lc) {
  crkDensity32<<<gridFor(n, 128), 128, 0, s>>>(F, P, list, n, g, nl, t, hp);
  lc->add(1);
}
void launchRKCorrectionsFP32(Fields F, Fields32 P, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                             cudaStream_t s, LaunchCounter* lc) {
  rkCorrections32<<<gridFor(n, 128), 128, 0, s>>>(F, P, n, g, nl, t, hp);
  lc->add(1);
}
void launchPairCRKFP32(Fields F, Fields32 P, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                       HydroParams hp, float* pacc, int variant, cudaStream_t s, LaunchCounter* lc) {
  const unsigned gb = gridFor(n, 128);
#define SPH_CRK32(X, C, Q) pairKernelCRK32<X, C, Q><<<gb, 128, 0, s>>>(F, P, list, n, g, nl, t, hp, pacc)
  // variant 1: two slots per iteration (compatible energy, no XSPH)
  if (variant == 1 && !hp.xsph && hp.compatible) {
    if (hp.limitedQ) pairKernelCRK32<false, true, true, 2><<<gb, 128, 0, s>>>(F, P, list, n, g, nl, t, hp, pacc);
    else pairKernelCRK32<false, true, false, 2><<<gb, 128, 0, s>>>(F, P, list, n, g, nl, t, hp, pacc);
    lc->add(1);
    return;
  }
  if (hp.limitedQ) {
    if (hp.xsph) { if (hp.compatible) SPH_CRK32(true, true, true); else SPH_CRK32(true, false, true); }
    else { if (hp.compatible) SPH_CRK32(false, true, true); else SPH_CRK32(false, false, true); }
  } else {
    if (hp.xsph) { if (hp.compatible) SPH_CRK32(true, true, false); else SPH_CRK32(true, false, false); }
    else { if (hp.compatible) SPH_CRK32(false, true, false); else SPH_CRK32(false, false, false); }
  }
#undef SPH_CRK32
  lc->add(1);
}

}  // namespace sph
