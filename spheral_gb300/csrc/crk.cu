// CRKSPH with LinearOrder reproducing kernels, FP64 gather sweeps over the
// neighbour lists of the SPH path:
//   * RK volumes           src/RK/computeRKVolumes.cc:20-70 (RKMassOverDensity,
//                          RKSumVolume: computeRKSumVolume.cc:30-110, HVolume:
//                          computeHVolumes.cc:25-60)
//   * CRK mass density     src/CRKSPH/computeCRKSPHSumMassDensity.cc:15-110
//   * RK corrections       src/RK/RKUtilities.cc:250-491 (LinearOrder, no Hessian)
//   * CRKSPH pair loop     src/CRKSPH/CRKSPH.cc:180-380, with the
//                          SPHSmoothingScale moments (SPHSmoothingScale.cc:150-272)
// Isotropic H (a = 1/h): eta = a x, Hdet = a^3.
#include "device.cuh"
#include "kernels.cuh"

namespace sph {

namespace {

using namespace dev;

inline unsigned gridFor(long n, int b) { return (unsigned)((n + b - 1) / b); }

// RKUtilities::evaluateBaseKernelAndGradient (RKUtilities.cc:66-80) for H = a I:
// eta = a x, w = Hdet W(|eta|), grad = (H eta^) Hdet dW(|eta|); a zero eta
// takes the unit vector (1, 0, 0) (GeomVector::unitVector).
__device__ __forceinline__ void rkBaseEta(const double* __restrict__ tw, const double* __restrict__ tg,
                                          const HydroParams& hp, double a, double ex, double ey, double ez, double em,
                                          double& w, double& dwx, double& dwy, double& dwz) {
  double ux = 1.0, uy = 0.0, uz = 0.0;
  if (em > 1.0e-50) {
    const double ie = 1.0 / em;
    ux = ex * ie; uy = ey * ie; uz = ez * ie;
  }
  const double Hdet = (a * a) * a;
  double k = 0.0, dk = 0.0;
  if (em < hp.extent) {
    const int i0 = tableIndex(em, hp.tableN1, hp.tableXstep);
    k = Hdet * tableEval(tw, i0, em);
    dk = Hdet * tableEval(tg, i0, em);
  }
  w = k;
  dwx = (a * ux) * dk;
  dwy = (a * uy) * dk;
  dwz = (a * uz) * dk;
}
__device__ __forceinline__ void rkBase(const double* __restrict__ tw, const double* __restrict__ tg,
                                       const HydroParams& hp, double a, double x, double y, double z, double& w,
                                       double& dwx, double& dwy, double& dwz) {
  const double ex = a * x, ey = a * y, ez = a * z;
  rkBaseEta(tw, tg, hp, a, ex, ey, ez, sqrt(ex * ex + ey * ey + ez * ez), w, dwx, dwy, dwz);
}

// RKUtilities::evaluateKernelAndGradient (RKUtilities.cc:181-206), LinearOrder:
// W^R = (C.P) W, dW^R/dx_d = (C_{1+d} + dC_d.P) W + (C.P) dW/dx_d with
// P = (1, x, y, z).
__device__ __forceinline__ void rkEval(const double* __restrict__ C, double x, double y, double z, double w,
                                       double dwx, double dwy, double dwz, double& WR, double& gx, double& gy,
                                       double& gz) {
  const double CP = ((C[0] + C[1] * x) + C[2] * y) + C[3] * z;
  const double d0 = ((C[4] + C[5] * x) + C[6] * y) + C[7] * z;
  const double d1 = ((C[8] + C[9] * x) + C[10] * y) + C[11] * z;
  const double d2 = ((C[12] + C[13] * x) + C[14] * y) + C[15] * z;
  gx = (C[1] + d0) * w + CP * dwx;
  gy = (C[2] + d1) * w + CP * dwy;
  gz = (C[3] + d2) * w + CP * dwz;
  WR = CP * w;
}

// The corrections of a mirror image: ReflectingBoundary::applyGhostBoundary
// for RKCoefficients (ReflectingBoundary.cc:402-432) applies the reflection
// operator of RKUtilities::getTransformationMatrix; for a wall normal to axis
// a an entry flips once per index equal to a.  Periodic images keep them.
__device__ __forceinline__ void imageRKC(const Grid& g, int code, double* C) {
  if (!code) return;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int side = (code >> (2 * a)) & 3;
    if (!mirrored(side, g.kindLo[a], g.kindHi[a])) continue;
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

__device__ __forceinline__ void loadTables(double* smem, const TableDev& t, const HydroParams& hp) {
  const int ntab = 3 * (hp.tableN1 + 1);
  for (int k = threadIdx.x; k < ntab; k += blockDim.x) { smem[k] = t.w[k]; smem[ntab + k] = t.g[k]; }
  __syncthreads();
}

//------------------------------------------------------------------------------
// RK volumes.
//------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) rkVolumeKernel(Fields F, long n, Grid g, NeighborLists nl, TableDev t,
                                                      HydroParams hp) {
  extern __shared__ double smem[];
  if (hp.rkVolume == 1) loadTables(smem, t, hp);
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double ai = F.f[F_HINV][i];
  const double Hdeti = (ai * ai) * ai;
  if (hp.rkVolume == 0) {          // RKMassOverDensity
    F.f[F_VOL][i] = F.f[F_MASS][i] / F.f[F_RHO][i];
    return;
  }
  if (hp.rkVolume == 4) {          // HVolume with the first NodeList's nPerh
    const double b = hp.lists[0].nPerh * ai;
    F.f[F_VOL][i] = 0.125 * 4.0 / 3.0 * 3.141592653589793 / ((b * b) * b);
    return;
  }
  // RKSumVolume: 1 / sum_j W(|H_i r_ij|, Hdet_i) over the neighbours and i
  // itself, capped at the eta-space volume of the kernel
  int hc[3];
  unpackCell(nl.cell[i], hc);
  const double xi = F.f[F_X][i], yi = F.f[F_Y][i], zi = F.f[F_Z][i];
  const double* __restrict__ tw = smem;
  double sum = 0.0;
  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const uint32_t ent = nl.nbr[nbSlot(i, q, nl.cap)];
    const int j = (int)(ent & kIndexMask), code = imageCode(g, hc, (int)(ent >> kIndexBits));
    double xj = F.f[F_X][j], yj = F.f[F_Y][j], zj = F.f[F_Z][j];
    imagePos(g, code, xj, yj, zj);
    const double ex = ai * (xi - xj), ey = ai * (yi - yj), ez = ai * (zi - zj);
    const double em = sqrt(ex * ex + ey * ey + ez * ez);
    if (em < hp.extent) sum += Hdeti * tableEval(tw, tableIndex(em, hp.tableN1, hp.tableXstep), em);
  }
  const double halfExt = 0.5 * hp.extent;
  const double etaVolMax = ((halfExt * halfExt) * halfExt) * (4.0 / 3.0 * 3.141592653589793);
  const double v = sum + Hdeti * hp.W0;
  F.f[F_VOL][i] = fmin(etaVolMax / Hdeti, 1.0 / v);
}

//------------------------------------------------------------------------------
// CRK mass density: neighbours of the same NodeList, each with its own kernel.
//------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) crkDensityKernel(Fields F, const int* __restrict__ list, long n, Grid g,
                                                        NeighborLists nl, TableDev t, HydroParams hp) {
  extern __shared__ double smem[];
  loadTables(smem, t, hp);
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int hc[3];
  unpackCell(nl.cell[i], hc);
  const double* __restrict__ tw = smem;
  const double xi = F.f[F_X][i], yi = F.f[F_Y][i], zi = F.f[F_Z][i];
  const double ai = F.f[F_HINV][i], mi = F.f[F_MASS][i], Vi = F.f[F_VOL][i];
  const int li = list[i];
  double wsum = 0.0, rho = 0.0, vol1 = 0.0;
  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const uint32_t ent = nl.nbr[nbSlot(i, q, nl.cap)];
    const int j = (int)(ent & kIndexMask);
    if (list[j] != li) continue;
    const int code = imageCode(g, hc, (int)(ent >> kIndexBits));
    double xj = F.f[F_X][j], yj = F.f[F_Y][j], zj = F.f[F_Z][j];
    imagePos(g, code, xj, yj, zj);
    const double aj = F.f[F_HINV][j];
    const double ex = aj * (xi - xj), ey = aj * (yi - yj), ez = aj * (zi - zj);
    const double em = sqrt(ex * ex + ey * ey + ez * ez);
    if (em >= hp.extent) continue;
    const double Wj = ((aj * aj) * aj) * tableEval(tw, tableIndex(em, hp.tableN1, hp.tableXstep), em);
    const double Vj = F.f[F_VOL][j];
    wsum += Vj * Wj;
    rho += F.f[F_MASS][j] * Vj * Wj;
    vol1 += Vj * Vj * Wj;
  }
  const NodeListParams L = hp.lists[li];
  const double Hdeti = (ai * ai) * ai;
  wsum += Vi * Hdeti * hp.W0;
  vol1 = (vol1 + Vi * Vi * Hdeti * hp.W0) / wsum;
  F.f[F_RHO][i] = fmax(fmax(L.rhoMin, 0.1 * mi * Hdeti),
                       fmin(L.rhoMax, (rho + mi * Vi * Hdeti * hp.W0) / (wsum * vol1)));
}

//------------------------------------------------------------------------------
// LinearOrder corrections: moments M (4x4, symmetric) and dM/dx_d over the
// neighbours and i itself with the scatter kernel W(x_ij, H_j), then
// C = M^-1 e_0 and dC_d = -M^-1 (dM_d C) by one LU factorisation with
// partial pivoting (the reference solves with Eigen's colPivHouseholderQr:
// the corrections agree to rounding).
//------------------------------------------------------------------------------
__device__ __forceinline__ int symIdx(int k, int l) {   // upper triangle of 4x4, row-major
  return k <= l ? (k * 4 - (k * (k - 1)) / 2 + (l - k)) : (l * 4 - (l * (l - 1)) / 2 + (k - l));
}

__device__ __forceinline__ void addMoments(double* M, double (*dM)[10], double vj, double x, double y, double z,
                                           double w, double dwx, double dwy, double dwz) {
  // M_kl += V_j p_k p_l W; dM_d,kl += V_j ((dp_dk p_l + p_k dp_dl) W + p_k p_l dW_d)
  // with dp_dk = [k == 1 + d]: the products p_k p_l and V_j W, V_j dW_d are shared
  const double p[4] = {1.0, x, y, z};
  const double vw = vj * w;
  const double vd[3] = {vj * dwx, vj * dwy, vj * dwz};
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int l = k; l < 4; ++l) {
      const double pp = p[k] * p[l];
      M[symIdx(k, l)] += vw * pp;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        double t = vd[d] * pp;
        if (k == 1 + d) t += vw * p[l];
        if (l == 1 + d) t += vw * p[k];
        dM[d][symIdx(k, l)] += t;
      }
    }
}

__global__ void __launch_bounds__(128) rkCorrectionsKernel(Fields F, long n, Grid g, NeighborLists nl, TableDev t,
                                                           HydroParams hp) {
  extern __shared__ double smem[];
  loadTables(smem, t, hp);
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ntab = 3 * (hp.tableN1 + 1);
  const double* __restrict__ tw = smem;
  const double* __restrict__ tg = smem + ntab;
  int hc[3];
  unpackCell(nl.cell[i], hc);
  const double xi = F.f[F_X][i], yi = F.f[F_Y][i], zi = F.f[F_Z][i];
  double M[10], dM[3][10];
#pragma unroll
  for (int k = 0; k < 10; ++k) { M[k] = 0.0; dM[0][k] = 0.0; dM[1][k] = 0.0; dM[2][k] = 0.0; }
  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const uint32_t ent = nl.nbr[nbSlot(i, q, nl.cap)];
    const int j = (int)(ent & kIndexMask), code = imageCode(g, hc, (int)(ent >> kIndexBits));
    double xj = F.f[F_X][j], yj = F.f[F_Y][j], zj = F.f[F_Z][j];
    imagePos(g, code, xj, yj, zj);
    const double x = xi - xj, y = yi - yj, z = zi - zj;
    double w, dwx, dwy, dwz;
    rkBase(tw, tg, hp, F.f[F_HINV][j], x, y, z, w, dwx, dwy, dwz);
    addMoments(M, dM, F.f[F_VOL][j], x, y, z, w, dwx, dwy, dwz);
  }
  {   // self contribution
    double w, dwx, dwy, dwz;
    rkBase(tw, tg, hp, F.f[F_HINV][i], 0.0, 0.0, 0.0, w, dwx, dwy, dwz);
    addMoments(M, dM, F.f[F_VOL][i], 0.0, 0.0, 0.0, w, dwx, dwy, dwz);
  }
  // LU with partial pivoting of the full 4x4 M
  double A[4][4];
  int piv[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    piv[r] = r;
#pragma unroll
    for (int c = 0; c < 4; ++c) A[r][c] = M[symIdx(r, c)];
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    int p = k;
#pragma unroll
    for (int r = k + 1; r < 4; ++r)
      if (fabs(A[r][k]) > fabs(A[p][k])) p = r;
    if (p != k) {
#pragma unroll
      for (int c = 0; c < 4; ++c) { const double tmp = A[k][c]; A[k][c] = A[p][c]; A[p][c] = tmp; }
      const int tp = piv[k]; piv[k] = piv[p]; piv[p] = tp;
    }
    const double inv = 1.0 / A[k][k];
#pragma unroll
    for (int r = k + 1; r < 4; ++r) {
      const double f = A[r][k] * inv;
      A[r][k] = f;
#pragma unroll
      for (int c = k + 1; c < 4; ++c) A[r][c] -= f * A[k][c];
    }
  }
  auto solve = [&](const double* b, double* x) {
    double yv[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      double v = b[piv[r]];
#pragma unroll
      for (int c = 0; c < r; ++c) v -= A[r][c] * yv[c];
      yv[r] = v;
    }
#pragma unroll
    for (int r = 3; r >= 0; --r) {
      double v = yv[r];
#pragma unroll
      for (int c = r + 1; c < 4; ++c) v -= A[r][c] * x[c];
      x[r] = v / A[r][r];
    }
  };
  const double e0[4] = {1.0, 0.0, 0.0, 0.0};
  double C[4];
  solve(e0, C);
#pragma unroll
  for (int k = 0; k < 4; ++k) F.f[F_RKC_0 + k][i] = C[k];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double rhs[4], dC[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      double v = 0.0;
#pragma unroll
      for (int l = 0; l < 4; ++l) v += dM[d][symIdx(k, l)] * C[l];
      rhs[k] = -v;
    }
    solve(rhs, dC);
#pragma unroll
    for (int k = 0; k < 4; ++k) F.f[F_RKC_4 + 4 * d + k][i] = dC[k];
  }
}

//------------------------------------------------------------------------------
// CRKSPH pair loop, gathered from i's side: for each neighbour j,
//   (W_j, gradW_j) = W^R(r_ij, H_j, C_i),  (W_i, gradW_i) = W^R(-r_ij, H_i, C_j),
//   f_ij = V_i V_j / 2 ((P_i + P_j)(gradW_j - gradW_i) + Q_acc),
// which the same evaluation from j's side reproduces with the opposite sign.
//------------------------------------------------------------------------------
template <bool XSPH, bool COMPAT>
__global__ void __launch_bounds__(128) pairKernelCRK(Fields F, const int* __restrict__ list, long n, Grid g,
                                                     NeighborLists nl, TableDev t, HydroParams hp,
                                                     double* __restrict__ pacc) {
  extern __shared__ double smem[];
  loadTables(smem, t, hp);
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ntab = 3 * (hp.tableN1 + 1);
  const double* __restrict__ tw = smem;
  const double* __restrict__ tg = smem + ntab;
  int hc[3];
  unpackCell(nl.cell[i], hc);
  const double xi = F.f[F_X][i], yi = F.f[F_Y][i], zi = F.f[F_Z][i];
  const double vxi = F.f[F_VX][i], vyi = F.f[F_VY][i], vzi = F.f[F_VZ][i];
  const double mi = F.f[F_MASS][i], rhoi = F.f[F_RHO][i], Pi = F.f[F_P][i], ci = F.f[F_CS][i];
  const double ai = F.f[F_HINV][i], Vi = F.f[F_VOL][i];
  const double invMi = 1.0 / mi;   // the reference forms force / m_i as force * (1 / m_i)
  const int li = list[i];
  double Ci[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) Ci[k] = F.f[F_RKC_0 + k][i];
  const double Clij = 0.5 * (1.0 + 1.0) * 1.0 * hp.Cl;
  const double Cqij = 0.5 * (1.0 + 1.0) * 1.0 * hp.Cq;
  double DQi[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) DQi[k] = hp.limitedQ ? F.f[F_DVDXQ_XX + k][i] : 0.0;

  double dvx = 0.0, dvy = 0.0, dvz = 0.0, deps = 0.0, maxQ = 0.0, effQ = 0.0;
  double xdx = 0.0, xdy = 0.0, xdz = 0.0, m0 = 0.0, m1x = 0.0, m1y = 0.0, m1z = 0.0;
  double D[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) D[k] = 0.0;

  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const long long slot = nbSlot(i, q, nl.cap);
    const uint32_t ent = nl.nbr[slot];
    const int j = (int)(ent & kIndexMask), code = imageCode(g, hc, (int)(ent >> kIndexBits));
    double xj = F.f[F_X][j], yj = F.f[F_Y][j], zj = F.f[F_Z][j];
    double vxj = F.f[F_VX][j], vyj = F.f[F_VY][j], vzj = F.f[F_VZ][j];
    imagePos(g, code, xj, yj, zj);
    imageVec(g, code, vxj, vyj, vzj);
    const double mj = F.f[F_MASS][j], rhoj = F.f[F_RHO][j], Pj = F.f[F_P][j], cj = F.f[F_CS][j];
    const double aj = F.f[F_HINV][j], Vj = F.f[F_VOL][j];
    const int lj = list[j];
    double Cj[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) Cj[k] = F.f[F_RKC_0 + k][j];
    imageRKC(g, code, Cj);

    const double rx = xi - xj, ry = yi - yj, rz = zi - zj;
    const double vijx = vxi - vxj, vijy = vyi - vyj, vijz = vzi - vzj;
    // eta_i = H_i r_ij, eta_j = H_j r_ij (the base kernel of W_i at -r_ij sees -eta_i)
    const double eix = ai * rx, eiy = ai * ry, eiz = ai * rz;
    const double ejx = aj * rx, ejy = aj * ry, ejz = aj * rz;
    const double etaMag2i = eix * eix + eiy * eiy + eiz * eiz;
    const double etaMag2j = ejx * ejx + ejy * ejy + ejz * ejz;
    const double etaMagi = sqrt(etaMag2i), etaMagj = sqrt(etaMag2j);
    // corrected kernels: W_j with H_j and C_i, W_i with H_i and C_j at -r_ij
    double w, dwx, dwy, dwz, Wj, gjx, gjy, gjz, Wi, gix, giy, giz;
    rkBaseEta(tw, tg, hp, aj, ejx, ejy, ejz, etaMagj, w, dwx, dwy, dwz);
    rkEval(Ci, rx, ry, rz, w, dwx, dwy, dwz, Wj, gjx, gjy, gjz);
    rkBaseEta(tw, tg, hp, ai, -eix, -eiy, -eiz, etaMagi, w, dwx, dwy, dwz);
    rkEval(Cj, -rx, -ry, -rz, w, dwx, dwy, dwz, Wi, gix, giy, giz);
    const double dgx = gjx - gix, dgy = gjy - giy, dgz = gjz - giz;

    // Monaghan-Gingold Q (the limited form first corrects the two velocities
    // along the pair with the Q's DvDx)
    double vqx = vijx, vqy = vijy, vqz = vijz;
    if (hp.limitedQ) {
      double Dj[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) Dj[k] = F.f[F_DVDXQ_XX + k][j];
      imageTensor(g, code, Dj);
      const double hx = 0.5 * rx, hy = 0.5 * ry, hz = 0.5 * rz;
      const double aix = DQi[0] * hx + DQi[1] * hy + DQi[2] * hz;
      const double aiy = DQi[3] * hx + DQi[4] * hy + DQi[5] * hz;
      const double aiz = DQi[6] * hx + DQi[7] * hy + DQi[8] * hz;
      const double ajx = Dj[0] * hx + Dj[1] * hy + Dj[2] * hz;
      const double ajy = Dj[3] * hx + Dj[4] * hy + Dj[5] * hz;
      const double ajz = Dj[6] * hx + Dj[7] * hy + Dj[8] * hz;
      const double gri = aix * hx + aiy * hy + aiz * hz;
      const double grj = ajx * hx + ajy * hy + ajz * hz;
      const double rri = gri / ((grj < 0.0 ? -1.0 : 1.0) * fmax(1.0e-30, fabs(grj)));
      const double rrj = grj / ((gri < 0.0 ? -1.0 : 1.0) * fmax(1.0e-30, fabs(gri)));
      const double xl = fmin(rri, rrj);
      double phi = xl > 0.0 ? 2.0 / (1.0 + xl) * 2.0 * xl / (1.0 + xl) : 0.0;   // van Leer
      const double etaij = fmin(etaMagi, etaMagj);
      if (etaij < hp.etaCrit) {
        const double zz = (etaij - hp.etaCrit) / hp.etaFold;
        phi *= exp(-(zz * zz));
      }
      vqx = (vxi - phi * aix) - (vxj + phi * ajx);
      vqy = (vyi - phi * aiy) - (vyj + phi * ajy);
      vqz = (vzi - phi * aiz) - (vzj + phi * ajz);
    }
    const double mui = (vqx * eix + vqy * eiy + vqz * eiz) / (etaMag2i + hp.eps2);
    const double muj = (vqx * ejx + vqy * ejy + vqz * ejz) / (etaMag2j + hp.eps2);
    const double lmi = hp.linearInExpansion ? mui : fmin(0.0, mui);
    const double lmj = hp.linearInExpansion ? muj : fmin(0.0, muj);
    const double qmi = hp.quadraticInExpansion ? -(mui < 0.0 ? -1.0 : 1.0) * mui * mui : fmin(0.0, mui) * fmin(0.0, mui);
    const double qmj = hp.quadraticInExpansion ? -(muj < 0.0 ? -1.0 : 1.0) * muj * muj : fmin(0.0, muj) * fmin(0.0, muj);
    const double ei = -Clij * ci * lmi + Cqij * qmi;
    const double ej = -Clij * cj * lmj + Cqij * qmj;
    // rho^2 QPi = rho e (QPi_ij = e_i / rho_i): no division
    const double Qi = rhoi * ei;
    const double qj = rhoj * ej;
    const double qs = Qi + qj;
    const double Qax = qs * dgx, Qay = qs * dgy, Qaz = qs * dgz;
    const double workQi = (qj * vijx) * dgx + (qj * vijy) * dgy + (qj * vijz) * dgz;
    maxQ = fmax(maxQ, 4.0 * Qi);
    effQ += Vj * Qi * Wj;
    // velocity gradient
    const double vvx = Vj * vijx, vvy = Vj * vijy, vvz = Vj * vijz;
    D[0] -= vvx * gjx; D[1] -= vvx * gjy; D[2] -= vvx * gjz;
    D[3] -= vvy * gjx; D[4] -= vvy * gjy; D[5] -= vvy * gjz;
    D[6] -= vvz * gjx; D[7] -= vvz * gjy; D[8] -= vvz * gjz;
    // momentum and energy (type III CRK interpoint force); V_i V_j is formed
    // symmetrically so that j's side rounds the same force
    const double f = 0.5 * (Vi * Vj);
    const double PP = Pi + Pj;
    const double fx = f * (PP * dgx + Qax), fy = f * (PP * dgy + Qay), fz = f * (PP * dgz + Qaz);
    const double ax = fx * invMi, ay = fy * invMi, az = fz * invMi;
    dvx -= ax;
    dvy -= ay;
    dvz -= az;
    if (COMPAT) {
      pacc[3 * slot] = -ax;
      pacc[3 * slot + 1] = -ay;
      pacc[3 * slot + 2] = -az;
    }
    deps += f * (Pj * (vijx * dgx + vijy * dgy + vijz * dgz) + workQi) * invMi;
    if (XSPH && lj == li) {
      const double xw = Vj * Wj;
      xdx -= xw * vijx; xdy -= xw * vijy; xdz -= xw * vijz;
    }
    // SPHSmoothingScale zeroth / first moments
    double WSPHi = 0.0;
    if (etaMagi < hp.extent) WSPHi = fabs(tableEval(tg, tableIndex(etaMagi, hp.tableN1, hp.tableXstep), etaMagi));
    const double fw = (lj != li) ? mj * rhoi / (mi * rhoj) : 1.0;
    m0 += fw * WSPHi;
    const double fwW = fw * WSPHi;
    m1x -= fwW * eix; m1y -= fwW * eiy; m1z -= fwW * eiz;
  }
  // CRKSPH::evaluateDerivativesImpl finalize (CRKSPH.cc:385-420)
#pragma unroll
  for (int k = 0; k < 9; ++k) { F.f[F_DVDX_XX + k][i] = D[k]; F.f[F_M_XX + k][i] = 0.0; }
  const double trace = D[0] + D[4] + D[8];
  F.f[F_DRHODT][i] = -rhoi * trace;
  F.f[F_DVDT_X][i] = dvx;
  F.f[F_DVDT_Y][i] = dvy;
  F.f[F_DVDT_Z][i] = dvz;
  F.f[F_DEPSDT][i] = hp.totalEnergy ? mi * ((vxi * dvx + vyi * dvy + vzi * dvz) + deps) : deps;
  F.f[F_MAXQ][i] = maxQ;
  F.f[F_EFFQ][i] = effQ;
  F.f[F_RHOSUM][i] = 0.0;
  F.f[F_NORM][i] = 0.0;
  F.f[F_GRADRHO_X][i] = 0.0; F.f[F_GRADRHO_Y][i] = 0.0; F.f[F_GRADRHO_Z][i] = 0.0;
  F.f[F_XSPHW][i] = 0.0;
  F.f[F_XSPHDV_X][i] = xdx;
  F.f[F_XSPHDV_Y][i] = xdy;
  F.f[F_XSPHDV_Z][i] = xdz;
  F.f[F_DXDT_X][i] = XSPH ? vxi + xdx : vxi;
  F.f[F_DXDT_Y][i] = XSPH ? vyi + xdy : vyi;
  F.f[F_DXDT_Z][i] = XSPH ? vzi + xdz : vzi;
  // SPHSmoothingScale finalize (SPHSmoothingScale.cc:232-272)
  const NodeListParams L = hp.lists[li];
  const double m0s = fmax(0.0, m0);
  const double m0r = pow(m0s, 0.3333333333333333);
  F.f[F_M0][i] = m0r;
  F.f[F_M1_X][i] = m1x;
  F.f[F_M1_Y][i] = m1y;
  F.f[F_M1_Z][i] = m1z;
  F.f[F_DHDT][i] = ((-ai) / 3.0) * trace;
  const bool isolated = fabs(m0r - 0.0) <= 1.0e-15 * fmax(1.0, fabs(m0r));
  const double cur = isolated ? 0.5 * L.nPerh : fmax(0.0, hermiteLookup(t.herm, hp, m0r));
  const double s = fmin(4.0, fmax(0.25, L.nPerh / (cur + 1.0e-30)));
  const double aa = s < 1.0 ? 0.4 * (1.0 + s * s) : 0.4 * (1.0 + 1.0 / (s * s * s));
  const double hi0 = 1.0 / ai;
  const double hi1 = fmin(L.hmax, fmax(L.hmin, hi0 * (1.0 - aa + aa * s)));
  F.f[F_HIDEAL][i] = 1.0 / hi1;
}

size_t tableSmem(const HydroParams& hp) { return 2 * 3 * (size_t)(hp.tableN1 + 1) * sizeof(double); }

}  // namespace

void launchRKVolumes(Fields F, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp, cudaStream_t s,
                     LaunchCounter* lc) {
  rkVolumeKernel<<<gridFor(n, 128), 128, tableSmem(hp), s>>>(F, n, g, nl, t, hp);
  lc->add(1);
}
void launchCRKDensity(Fields F, const int* list, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                      cudaStream_t s, LaunchCounter* lc) {
  crkDensityKernel<<<gridFor(n, 128), 128, tableSmem(hp), s>>>(F, list, n, g, nl, t, hp);
  lc->add(1);
}
void launchRKCorrections(Fields F, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp, cudaStream_t s,
                         LaunchCounter* lc) {
  rkCorrectionsKernel<<<gridFor(n, 128), 128, tableSmem(hp), s>>>(F, n, g, nl, t, hp);
  lc->add(1);
}
void launchPairCRK(Fields F, const int* list, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                   double* pacc, cudaStream_t s, LaunchCounter* lc) {
  const size_t sm = tableSmem(hp);
  if (hp.xsph) {
    if (hp.compatible) pairKernelCRK<true, true><<<gridFor(n, 128), 128, sm, s>>>(F, list, n, g, nl, t, hp, pacc);
    else pairKernelCRK<true, false><<<gridFor(n, 128), 128, sm, s>>>(F, list, n, g, nl, t, hp, pacc);
  } else {
    if (hp.compatible) pairKernelCRK<false, true><<<gridFor(n, 128), 128, sm, s>>>(F, list, n, g, nl, t, hp, pacc);
    else pairKernelCRK<false, false><<<gridFor(n, 128), 128, sm, s>>>(F, list, n, g, nl, t, hp, pacc);
  }
  lc->add(1);
}

}  // namespace sph
