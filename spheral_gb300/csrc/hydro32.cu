// Mixed-precision sweeps of libsphgpu (sm_103a): the SPH pair loop, density
// sum, grad-h correction and pairwise dt limit in FP32 on cell-relative
// positions.  Time integration, the compatible-energy update, the per-node
// finalisation and all conserved tallies stay in FP64.
//
// Precision design.
//  * Positions are stored relative to the origin of each node's cell
//    (|x_rel| < one cell), so a pair separation is
//    (x_i,rel - x_j,rel) - d cell with d in {-1, 0, 1}: it keeps FP32 digits
//    relative to h instead of relative to the box size.
//  * The pair force Delta_ij is evaluated in a symmetric order,
//    (Prho_i gradW_i + Qacc_i) + (Prho_j gradW_j + Qacc_j), so the two ordered
//    slots (i, j) and (j, i) hold bitwise opposite values: momentum and the
//    compatible-energy split stay exactly antisymmetric despite FP32.
//  * The acceleration and energy-rate sums are Kahan compensated and leave
//    the kernel as the FP64 value s - c of the compensated pair (s, c).
#include "device.cuh"

namespace sph {
namespace {
using namespace dev;


__global__ void prepareKernel(Fields F, Fields32 P, long n, Grid g) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  // the same mirror values as the update kernel writes, by the same
  // integer-pipe conversions (the FP64 pipe bounds this kernel otherwise)
  int c[3];
  unpackCell(P.cell[i], c);
  const double ox = g.lo[0] + smallIntToDouble(c[0]) * g.cell[0];
  const double oy = g.lo[1] + smallIntToDouble(c[1]) * g.cell[1];
  const double oz = g.lo[2] + smallIntToDouble(c[2]) * g.cell[2];
  P.posh[i] = make_float4(toFloatRN(F.f[F_X][i] - ox), toFloatRN(F.f[F_Y][i] - oy), toFloatRN(F.f[F_Z][i] - oz),
                          toFloatRN(F.f[F_HINV][i]));
  P.velm[i] = make_float4(toFloatRN(F.f[F_VX][i]), toFloatRN(F.f[F_VY][i]), toFloatRN(F.f[F_VZ][i]),
                          toFloatRN(F.f[F_MASS][i]));
  // omega / (omega^2 + 1e-30) in FP32: an FP64 division here would cost
  // more on the narrow FP64 pipe than the rest of the kernel
  const float om = toFloatRN(F.f[F_OMEGA][i]);
  P.thermo[i] = make_float4(toFloatRN(F.f[F_RHO][i]), toFloatRN(F.f[F_P][i]), toFloatRN(F.f[F_CS][i]),
                            om / (om * om + 1.0e-30f));
  if (P.hten) writeTensorMirror(F, P, i);
  if (P.vol) P.vol[i] = toFloatRN(F.f[F_VOL][i]);
}

//------------------------------------------------------------------------------
// SPH pair loop (src/SPH/SPH.cc:294-470) + SPHSmoothingScale moments, FP32.
// Every operation that enters the pair force is deterministic and appears in
// the same order from both sides of the pair (explicit fma / rn intrinsics,
// MUFU reciprocal square root and fast division), so slot (j, i) holds the
// bitwise negation of slot (i, j).
//------------------------------------------------------------------------------
__device__ __forceinline__ void lookupPacked(const float4* __restrict__ ta, const float2* __restrict__ tb, int N1,
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

// TENSOR (ASPH): H_i, H_j from the FP32 tensor mirror (eta = H r,
// grad W = gW H eta^, both in a fixed order so the pair force stays bitwise
// antisymmetric), the second moment of ASPHClassicSmoothingScale and its
// FP32 finalize.
//
// PF selects the neighbour loop: 0 one slot per iteration, 1 software-
// pipelined (entry two slots ahead, node data one slot ahead), 2 or 4 that
// many slots per iteration (their gathers issued together, the next
// iteration's entries loaded ahead).  Every form evaluates the slots in list
// order, so all give the same bits.  LEAN (1: compensated sums, 2: plain
// FP32 sums): the sum type, no tensile correction and the standard Q
// expansion fixed at compile time (no run-time flag in the loop); 0 reads
// them from hp.
template <bool XSPH, bool COMPAT, bool MULTI, int MINB, int PF, bool LIMQ, bool TENSOR, int LEAN = 0>
__global__ void __launch_bounds__(128, MINB) pairKernelFP32(Fields F, Fields32 P, const int* __restrict__ list, long n,
                                                      Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                                                      float* __restrict__ pacc) {
  __shared__ float4 ta[kMaxTable / 3];
  __shared__ float2 tb[kMaxTable / 3];
  __shared__ float4 sOff[64];
  const int nint = hp.tableN1 + 1;
  for (int k = threadIdx.x; k < nint; k += blockDim.x) { ta[k] = t.p32a[k]; tb[k] = t.p32b[k]; }
  fillCellOffsets(sOff, g.cellf[0], g.cellf[1], g.cellf[2]);
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int ci[3];
  unpackCell(P.cell[i], ci);
  const uint32_t mm = mirrorMask(g, ci);
  const float cx = g.cellf[0], cy = g.cellf[1], cz = g.cellf[2];
  const float4 pi = P.posh[i], vi = P.velm[i], thi = P.thermo[i];
  const int li = MULTI ? list[i] : 0;
  const float ai = pi.w, mi = vi.w, rhoi = thi.x, Pi = thi.y, csi = thi.z, sOi = thi.w;
  float4 hi0 = make_float4(0.f, 0.f, 0.f, 0.f), hi1 = hi0;
  if (TENSOR) { hi0 = P.hten[2 * i]; hi1 = P.hten[2 * i + 1]; }
  const float Hdeti = TENSOR ? hi1.z : ai * ai * ai;
  const float extent = (float)hp.extent, invStep = (float)(1.0 / hp.tableXstep);
  const int N1 = hp.tableN1;
  const float Cl = (float)hp.Cl, Cq = (float)hp.Cq, eps2 = (float)hp.eps2;
  const float epsT = (float)hp.epsTensile, WnPerh = (float)hp.WnPerh;
  float DQi[9];   // the limited Q's DvDx of node i
  if (LIMQ) {
    const float4 d0 = P.dvq[3 * i], d1 = P.dvq[3 * i + 1], d2 = P.dvq[3 * i + 2];
    DQi[0] = d0.x; DQi[1] = d0.y; DQi[2] = d0.z; DQi[3] = d0.w;
    DQi[4] = d1.x; DQi[5] = d1.y; DQi[6] = d1.z; DQi[7] = d1.w; DQi[8] = d2.x;
  }
  const float etaCrit = (float)hp.etaCrit, etaFold = (float)hp.etaFold;
  const float iri = __frcp_rn(rhoi);
  const float mrhoi = mi * iri;
  const float Prhoi0 = __fmul_rn(__fmul_rn(__fmul_rn(sOi, Pi), iri), iri);
  const float mClci = __fmul_rn(-Cl, csi);

  float rhoSum = 0.f, norm = 0.f, maxQ = 0.f, effQ = 0.f, xw = 0.f, xdx = 0.f, xdy = 0.f, xdz = 0.f;
  float sdx = 0.f, cdx = 0.f, sdy = 0.f, cdy = 0.f, sdz = 0.f, cdz = 0.f, se = 0.f, ce = 0.f;
  float gx = 0.f, gy = 0.f, gz = 0.f, m0 = 0.f, m1x = 0.f, m1y = 0.f, m1z = 0.f;
  float D[9], M[9], m2[6];
#pragma unroll
  for (int k = 0; k < 9; ++k) { D[k] = 0.f; M[k] = 0.f; }
#pragma unroll
  for (int k = 0; k < 6; ++k) m2[k] = 0.f;

  const int cnt = nl.count[i];
  // One neighbour slot: the pair's contributions to node i's sums (and the
  // pair acceleration of the compatible-energy sweep at list slot k).
  auto slot = [&](uint32_t ent, const float4& pj, const float4& vj4, const float4& thj, float4 hj0, float4 hj1,
                  long long k) {
    const int j = (int)(ent & kIndexMask), dcode = (int)(ent >> kIndexBits);
    float rx, ry, rz;
    relSepTab(pi, pj, dcode, mm, cx, cy, cz, sOff, rx, ry, rz);
    float vxj = vj4.x, vyj = vj4.y, vzj = vj4.z;
    mirrorVel((uint32_t)dcode & mm, vxj, vyj, vzj);
    const float aj = pj.w, mj = vj4.w, rhoj = thj.x, Pj = thj.y, csj = thj.z, sOj = thj.w;
    const bool same = MULTI ? (list[j] == li) : true;
    if (TENSOR) {   // H_j through the mirrors of the entry
      const uint32_t mq = (uint32_t)dcode & mm;
      if (mq) {
        const float sx = (mq & 3u) ? -1.f : 1.f, sy = (mq & 12u) ? -1.f : 1.f, sz = (mq & 48u) ? -1.f : 1.f;
        hj0.y *= sx * sy;
        hj0.z *= sx * sz;
        hj1.x *= sy * sz;
      }
    }
    const float Hdetj = TENSOR ? hj1.z : aj * aj * aj;
    const float irj = __frcp_rn(rhoj);

    float eix, eiy, eiz, ejx, ejy, ejz;
    if (TENSOR) {
      symDot32(hi0, hi1, rx, ry, rz, eix, eiy, eiz);
      symDot32(hj0, hj1, rx, ry, rz, ejx, ejy, ejz);
    } else {
      eix = ai * rx; eiy = ai * ry; eiz = ai * rz;
      ejx = aj * rx; ejy = aj * ry; ejz = aj * rz;
    }
    const float e2i = __fmaf_rn(eiz, eiz, __fmaf_rn(eiy, eiy, __fmul_rn(eix, eix)));
    const float e2j = __fmaf_rn(ejz, ejz, __fmaf_rn(ejy, ejy, __fmul_rn(ejx, ejx)));
    const float ri = rsqrtf(fmaxf(e2i, 1.0e-30f)), rj = rsqrtf(fmaxf(e2j, 1.0e-30f));
    const float etai = __fmul_rn(e2i, ri), etaj = __fmul_rn(e2j, rj);
    float Wi, gi, Wj, gj;
    lookupPacked(ta, tb, N1, invStep, etai, extent, Wi, gi);
    lookupPacked(ta, tb, N1, invStep, etaj, extent, Wj, gj);
    const float WSPHi = fabsf(gi);
    Wi *= Hdeti;
    Wj *= Hdetj;
    // gradW = gW H eta/|eta|
    float gwix, gwiy, gwiz, gwjx, gwjy, gwjz;
    if (TENSOR) {
      const float fi = __fmul_rn(__fmul_rn(Hdeti, gi), ri);
      const float fj = __fmul_rn(__fmul_rn(Hdetj, gj), rj);
      float hx, hy, hz;
      symDot32(hi0, hi1, eix, eiy, eiz, hx, hy, hz);
      gwix = __fmul_rn(fi, hx); gwiy = __fmul_rn(fi, hy); gwiz = __fmul_rn(fi, hz);
      symDot32(hj0, hj1, ejx, ejy, ejz, hx, hy, hz);
      gwjx = __fmul_rn(fj, hx); gwjy = __fmul_rn(fj, hy); gwjz = __fmul_rn(fj, hz);
    } else {
      const float fi = __fmul_rn(__fmul_rn(__fmul_rn(Hdeti, gi), ai), ri);
      const float fj = __fmul_rn(__fmul_rn(__fmul_rn(Hdetj, gj), aj), rj);
      gwix = fi * eix; gwiy = fi * eiy; gwiz = fi * eiz;
      gwjx = fj * ejx; gwjy = fj * ejy; gwjz = fj * ejz;
    }

    if (same) {
      rhoSum += mj * Wi;
      norm += mrhoi * Wi;
    }
    const float vx = vi.x - vxj, vy = vi.y - vyj, vz = vi.z - vzj;
    float vqx = vx, vqy = vy, vqz = vz;
    if (LIMQ) {
      // LimitedMonaghanGingoldViscosity.cc:171-200 in a form symmetric in
      // (i, j): v_q = v_ij - phi (DvDx_i + DvDx_j) x_ij with x_ij = r/2, so
      // the pair force stays bitwise antisymmetric.
      const float4 d0 = P.dvq[3 * (long)j], d1 = P.dvq[3 * (long)j + 1], d2 = P.dvq[3 * (long)j + 2];
      float Dj[9] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w, d2.x};
      const uint32_t mq = (uint32_t)dcode & mm;
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
    const float li_ = (!LEAN && hp.linearInExpansion) ? mui : mni;
    const float lj_ = (!LEAN && hp.linearInExpansion) ? muj : mnj;
    const float qi_ = (!LEAN && hp.quadraticInExpansion) ? -(mui < 0.f ? -1.f : 1.f) * mui * mui : mni * mni;
    const float qj_ = (!LEAN && hp.quadraticInExpansion) ? -(muj < 0.f ? -1.f : 1.f) * muj * muj : mnj * mnj;
    const float ei = __fmaf_rn(Cq, qi_, __fmul_rn(mClci, li_));
    const float ej = __fmaf_rn(Cq, qj_, __fmul_rn(__fmul_rn(-Cl, csj), lj_));
    const float qai = __fmul_rn(0.5f, __fmul_rn(ei, iri)), qaj = __fmul_rn(0.5f, __fmul_rn(ej, irj));
    const float Qi = rhoi * ei;
    maxQ = fmaxf(maxQ, Qi);
    effQ += mj * Qi * Wi * irj;
    float Prhoi = Prhoi0, Prhoj = __fmul_rn(__fmul_rn(__fmul_rn(sOj, Pj), irj), irj);
    if (!LEAN && epsT != 0.f) {
      const float ti = Wi / (Hdeti * WnPerh), tj = Wj / (Hdetj * WnPerh);
      Prhoi = __fmul_rn(__fmul_rn(__fmul_rn(sOi, Pi + epsT * (ti * ti * ti * ti) * (Pi < 0.f ? -Pi : 0.f)), iri), iri);
      Prhoj = __fmul_rn(__fmul_rn(__fmul_rn(sOj, Pj + epsT * (tj * tj * tj * tj) * (Pj < 0.f ? -Pj : 0.f)), irj), irj);
    }
    // symmetric-order pair force: (Prho_i + Q_i/2) gradW_i + (Prho_j + Q_j/2) gradW_j
    const float ci_ = __fadd_rn(Prhoi, qai), cj_ = __fadd_rn(Prhoj, qaj);
    const float ddx = __fadd_rn(__fmul_rn(ci_, gwix), __fmul_rn(cj_, gwjx));
    const float ddy = __fadd_rn(__fmul_rn(ci_, gwiy), __fmul_rn(cj_, gwjy));
    const float ddz = __fadd_rn(__fmul_rn(ci_, gwiz), __fmul_rn(cj_, gwjz));
    const float pax = __fmul_rn(-mj, ddx), pay = __fmul_rn(-mj, ddy), paz = __fmul_rn(-mj, ddz);
    sumAdd(sdx, cdx, pax, LEAN == 2 ? 1 : (LEAN == 1 ? 0 : hp.plainSums));
    sumAdd(sdy, cdy, pay, LEAN == 2 ? 1 : (LEAN == 1 ? 0 : hp.plainSums));
    sumAdd(sdz, cdz, paz, LEAN == 2 ? 1 : (LEAN == 1 ? 0 : hp.plainSums));
    if (COMPAT) {
      pacc[3 * k] = pax;
      pacc[3 * k + 1] = pay;
      pacc[3 * k + 2] = paz;
    }
    const float vg = vx * gwix + vy * gwiy + vz * gwiz;
    sumAdd(se, ce, mj * (Prhoi + qai) * vg, LEAN == 2 ? 1 : (LEAN == 1 ? 0 : hp.plainSums));
    const float mvx = mj * vx, mvy = mj * vy, mvz = mj * vz;
    D[0] -= mvx * gwix; D[1] -= mvx * gwiy; D[2] -= mvx * gwiz;
    D[3] -= mvy * gwix; D[4] -= mvy * gwiy; D[5] -= mvy * gwiz;
    D[6] -= mvz * gwix; D[7] -= mvz * gwiy; D[8] -= mvz * gwiz;
    if (XSPH) {
      const float wx = 0.5f * (mrhoi * Wi + mj * irj * Wj);
      xw += wx;
      xdx -= wx * vx; xdy -= wx * vy; xdz -= wx * vz;
    }
    const float gr = mj * (rhoj - rhoi);
    gx += gr * gwix; gy += gr * gwiy; gz += gr * gwiz;
    const float mrx = mj * rx, mry = mj * ry, mrz = mj * rz;
    M[0] -= mrx * gwix; M[1] -= mrx * gwiy; M[2] -= mrx * gwiz;
    M[3] -= mry * gwix; M[4] -= mry * gwiy; M[5] -= mry * gwiz;
    M[6] -= mrz * gwix; M[7] -= mrz * gwiy; M[8] -= mrz * gwiz;
    const float fw = same ? 1.0f : mj * rhoi / (mi * rhoj);
    const float fwW = fw * WSPHi;
    m0 += fwW;
    m1x -= fwW * eix; m1y -= fwW * eiy; m1z -= fwW * eiz;
    if (TENSOR) {   // ASPHClassicSmoothingScale second moment: WSPH^2 r r / |r|^5
      const float ir = rsqrtf(fmaxf(rx * rx + ry * ry + rz * rz, 1.0e-30f));
      const float ir2 = ir * ir;
      const float w = fwW * WSPHi * (ir2 * ir2 * ir);
      m2[0] += w * (rx * rx); m2[1] += w * (rx * ry); m2[2] += w * (rx * rz);
      m2[3] += w * (ry * ry); m2[4] += w * (ry * rz); m2[5] += w * (rz * rz);
    }
  };
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (PF == 1) {
    // software pipeline over the neighbour list: the entry two slots ahead
    // and the node data one slot ahead are loaded while the current pair is
    // evaluated, so the gathers overlap the arithmetic
    uint32_t entA = 0u, entB = 0u;
    float4 pjA = zero4, vjA = zero4, thA = zero4, hA0 = zero4, hA1 = zero4;
    if (cnt > 0) {
      entA = nl.nbr[nbSlot(i, 0, nl.cap)];
      const int j0 = (int)(entA & kIndexMask);
      pjA = P.posh[j0]; vjA = P.velm[j0]; thA = P.thermo[j0];
      if (TENSOR) { hA0 = P.hten[2 * j0]; hA1 = P.hten[2 * j0 + 1]; }
    }
    if (cnt > 1) entB = nl.nbr[nbSlot(i, 1, nl.cap)];
    for (int q = 0; q < cnt; ++q) {
      const uint32_t ent = entA;
      const float4 pj = pjA, vj4 = vjA, thj = thA;
      const float4 hj0 = hA0, hj1 = hA1;
      if (q + 1 < cnt) {
        const int jn = (int)(entB & kIndexMask);
        pjA = P.posh[jn]; vjA = P.velm[jn]; thA = P.thermo[jn];
        if (TENSOR) { hA0 = P.hten[2 * jn]; hA1 = P.hten[2 * jn + 1]; }
        entA = entB;
      }
      if (q + 2 < cnt) entB = nl.nbr[nbSlot(i, q + 2, nl.cap)];
      slot(ent, pj, vj4, thj, hj0, hj1, nbSlot(i, q, nl.cap));
    }
  } else if (PF >= 2) {
    // PF slots per iteration (slot q + 1 sits 32 entries after slot q): their
    // gathers are issued together, the next iteration's entries meanwhile
    constexpr int U = PF >= 2 ? PF : 2;
    uint32_t nx[U];
    if (U <= cnt) {
#pragma unroll
      for (int u = 0; u < U; ++u) nx[u] = nl.nbr[nbSlot(i, u, nl.cap)];
    }
    int q = 0;
    for (; q + U <= cnt; q += U) {
      const long long k0 = nbSlot(i, q, nl.cap);
      uint32_t e[U];
#pragma unroll
      for (int u = 0; u < U; ++u) e[u] = nx[u];
      if (q + 2 * U <= cnt) {
#pragma unroll
        for (int u = 0; u < U; ++u) nx[u] = nl.nbr[k0 + 32 * (U + u)];
      }
      float4 pp[U], vv[U], tt[U], aa[U], bb[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int jj = (int)(e[u] & kIndexMask);
        pp[u] = P.posh[jj]; vv[u] = P.velm[jj]; tt[u] = P.thermo[jj];
        aa[u] = zero4; bb[u] = zero4;
        if (TENSOR) { aa[u] = P.hten[2 * jj]; bb[u] = P.hten[2 * jj + 1]; }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) slot(e[u], pp[u], vv[u], tt[u], aa[u], bb[u], k0 + 32 * u);
    }
    for (; q < cnt; ++q) {
      const long long k = nbSlot(i, q, nl.cap);
      const uint32_t ent = nl.nbr[k];
      const int jj = (int)(ent & kIndexMask);
      slot(ent, P.posh[jj], P.velm[jj], P.thermo[jj], TENSOR ? P.hten[2 * jj] : zero4,
           TENSOR ? P.hten[2 * jj + 1] : zero4, k);
    }
  } else {
    for (int q = 0; q < cnt; ++q) {
      const long long k = nbSlot(i, q, nl.cap);
      const uint32_t ent = nl.nbr[k];
      const int jj = (int)(ent & kIndexMask);
      slot(ent, P.posh[jj], P.velm[jj], P.thermo[jj], TENSOR ? P.hten[2 * jj] : zero4,
           TENSOR ? P.hten[2 * jj + 1] : zero4, k);
    }
  }
  NodeAcc32 a;
  a.rhoSum = rhoSum; a.norm = norm;
  a.dvx = kahanValue(sdx, cdx); a.dvy = kahanValue(sdy, cdy); a.dvz = kahanValue(sdz, cdz);
  a.deps = kahanValue(se, ce);
  a.gx = gx; a.gy = gy; a.gz = gz; a.maxQ = maxQ; a.effQ = effQ;
  a.xw = xw; a.xdx = xdx; a.xdy = xdy; a.xdz = xdz;
  a.m0 = m0; a.m1x = m1x; a.m1y = m1y; a.m1z = m1z;
#pragma unroll
  for (int k = 0; k < 9; ++k) { a.D[k] = D[k]; a.M[k] = M[k]; }
#pragma unroll
  for (int k = 0; k < 6; ++k) a.m2[k] = m2[k];
  a.h0 = hi0;
  a.h1 = hi1;
  finalizeNode32<TENSOR>(F, i, MULTI ? li : list[i], a, cnt, hp, t.herm);
}

//------------------------------------------------------------------------------
// Density sum, FP32 (computeSPHSumMassDensity.cc:15-87, gathered).
//------------------------------------------------------------------------------
template <bool TENSOR>
__global__ void __launch_bounds__(128) sumDensityKernel32(Fields F, Fields32 P, const int* __restrict__ list, long n,
                                                          Grid g, NeighborLists nl, TableDev t, HydroParams hp) {
  __shared__ float tw[kMaxTable];
  const int ntab = 3 * (hp.tableN1 + 1);
  for (int k = threadIdx.x; k < ntab; k += blockDim.x) tw[k] = t.w32[k];
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int ci[3];
  unpackCell(P.cell[i], ci);
  const uint32_t mm = mirrorMask(g, ci);
  const float cx = g.cellf[0], cy = g.cellf[1], cz = g.cellf[2];
  const float4 pi = P.posh[i];
  const float mi = P.velm[i].w;
  const bool multi = hp.numLists > 1;
  const int li = multi ? list[i] : 0;
  const float extent = (float)hp.extent, invStep = (float)(1.0 / hp.tableXstep);
  const int N1 = hp.tableN1;
  float s = 0.f, c = 0.f;
  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const long long k = nbSlot(i, q, nl.cap);
    const uint32_t ent = nl.nbr[k];
    const int j = (int)(ent & kIndexMask), dcode = (int)(ent >> kIndexBits);
    const float4 pj = P.posh[j];
    float rx, ry, rz;
    relSep(pi, pj, dcode, mm, cx, cy, cz, rx, ry, rz);
    float eta, Hdj;
    if (TENSOR) {   // |H_j r| with H_j through the mirrors
      float4 h0, h1;
      loadTensor32(P, j, (uint32_t)dcode & mm, h0, h1);
      eta = sqrtf(eta2Sym32(h0, h1, rx, ry, rz));
      Hdj = h1.z;
    } else {
      const float aj = pj.w;
      eta = aj * sqrtf(rx * rx + ry * ry + rz * rz);
      Hdj = aj * aj * aj;
    }
    if (eta < extent) {
      const int i0 = 3 * min(N1, (int)(eta * invStep));
      const float w = Hdj * (tw[i0] + (tw[i0 + 1] + tw[i0 + 2] * eta) * eta);
      sumAdd(s, c, ((multi ? list[j] == li : true) ? P.velm[j].w : mi) * w, hp.plainSums);
    }
  }
  const double a = F.f[F_HINV][i];
  const double Hdeti = TENSOR ? symDet(loadSym(F, F_HT_XX, i)) : (a * a) * a;
  const double self = F.f[F_MASS][i] * (Hdeti * hp.W0);
  const double rho = self + kahanValue(s, c);
  F.f[F_RHO][i] = rho;
  P.thermo[i].x = (float)rho;
}

//------------------------------------------------------------------------------
// Fused start-of-step sweep of the mixed mode: the density sum
// (computeSPHSumMassDensity.cc:15-87) and the time-step vote
// (GenericHydro.cc:113-381, pairwise velocity limit on the same neighbour
// data, node limits with the new density) in one pass over the lists.
//------------------------------------------------------------------------------
template <bool TENSOR, bool LEAN>
__global__ void __launch_bounds__(128) densityDtKernel32(Fields F, Fields32 P, const int* __restrict__ list, long n,
                                                         Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                                                         double maxNperh, double* __restrict__ part) {
  __shared__ float tw[kMaxTable];
  __shared__ double sv[128];
  __shared__ int sr[128];
  const int ntab = 3 * (hp.tableN1 + 1);
  for (int k = threadIdx.x; k < ntab; k += blockDim.x) tw[k] = t.w32[k];
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  double best = DBL_MAX;
  int reason = -1;
  if (i < n) {
    int ci[3];
    unpackCell(P.cell[i], ci);
    const uint32_t mm = mirrorMask(g, ci);
    const float cx = g.cellf[0], cy = g.cellf[1], cz = g.cellf[2];
    const float4 pi = P.posh[i], vi = P.velm[i];
    const float mi = vi.w;
    const bool multi = !LEAN && hp.numLists > 1;
    const int li = multi ? list[i] : 0;
    const float extent = (float)hp.extent, invStep = (float)(1.0 / hp.tableXstep);
    const int N1 = hp.tableN1;
    float s = 0.f, c = 0.f, worstPair = 0.0f;
    // the node scale of GenericHydro::dt: 1/h, the largest eigenvalue of H
    const float lmaxi = TENSOR ? P.hten[2 * i + 1].w : pi.w;
    const int cnt = nl.count[i];
    // software pipeline: entry two slots ahead, node data one slot ahead
    uint32_t entA = 0u, entB = 0u;
    float4 pjA = make_float4(0.f, 0.f, 0.f, 0.f), vjA = pjA, hA0 = pjA, hA1 = pjA;
    if (cnt > 0) {
      entA = nl.nbr[nbSlot(i, 0, nl.cap)];
      const int j0 = (int)(entA & kIndexMask);
      pjA = P.posh[j0]; vjA = P.velm[j0];
      if (TENSOR) { hA0 = P.hten[2 * j0]; hA1 = P.hten[2 * j0 + 1]; }
    }
    if (cnt > 1) entB = nl.nbr[nbSlot(i, 1, nl.cap)];
    for (int q = 0; q < cnt; ++q) {
      const uint32_t ent = entA;
      const float4 pj = pjA, vj = vjA;
      float4 h0 = hA0, h1 = hA1;
      if (q + 1 < cnt) {
        const int jn = (int)(entB & kIndexMask);
        pjA = P.posh[jn]; vjA = P.velm[jn];
        if (TENSOR) { hA0 = P.hten[2 * jn]; hA1 = P.hten[2 * jn + 1]; }
        entA = entB;
      }
      if (q + 2 < cnt) entB = nl.nbr[nbSlot(i, q + 2, nl.cap)];
      const int j = (int)(ent & kIndexMask), dcode = (int)(ent >> kIndexBits);
      float rx, ry, rz;
      relSep(pi, pj, dcode, mm, cx, cy, cz, rx, ry, rz);
      float eta, Hdj, lmaxj;
      if (TENSOR) {   // |H_j r| with H_j through the mirrors
        const uint32_t mq = (uint32_t)dcode & mm;
        if (mq) {
          const float sx = (mq & 3u) ? -1.f : 1.f, sy = (mq & 12u) ? -1.f : 1.f, sz = (mq & 48u) ? -1.f : 1.f;
          h0.y *= sx * sy;
          h0.z *= sx * sz;
          h1.x *= sy * sz;
        }
        eta = etaFromSq(eta2Sym32(h0, h1, rx, ry, rz));
        Hdj = h1.z;
        lmaxj = h1.w;
      } else {
        const float aj = pj.w;
        eta = aj * etaFromSq(rx * rx + ry * ry + rz * rz);
        Hdj = aj * aj * aj;
        lmaxj = aj;
      }
      if (eta < extent) {
        const int i0 = 3 * min(N1, (int)(eta * invStep));
        const float w = Hdj * (tw[i0] + (tw[i0 + 1] + tw[i0 + 2] * eta) * eta);
        sumAdd(s, c, ((multi ? list[j] == li : true) ? vj.w : mi) * w, LEAN ? 0 : hp.plainSums);
      }
      float vxj = vj.x, vyj = vj.y, vzj = vj.z;
      mirrorVel((uint32_t)dcode & mm, vxj, vyj, vzj);
      const float dx = vi.x - vxj, dy = vi.y - vyj, dz = vi.z - vzj;
      // min over pairs of min(h_i, h_j)/|v_ij| = 1/sqrt(max over pairs of
      // (max(a_i, a_j) |v_ij|)^2): no division or root per pair
      const float am = fmaxf(lmaxi, lmaxj);
      worstPair = fmaxf(worstPair, (am * am) * (dx * dx + dy * dy + dz * dz));
    }
    const float bestPair = worstPair > 0.0f ? rsqrtf(worstPair) : 3.0e38f;
    const double a = F.f[F_HINV][i];
    const double Hdeti = TENSOR ? symDet(loadSym(F, F_HT_XX, i)) : (a * a) * a;
    const double rho = F.f[F_MASS][i] * (Hdeti * hp.W0) + kahanValue(s, c);
    F.f[F_RHO][i] = rho;
    P.thermo[i].x = (float)rho;
    // Node limits of GenericHydro::dt in FP32 (the vote only picks the
    // minimum; GB300's FP64 divide and square root sequences would dominate
    // the sweep otherwise).
    const float tiny = (float)DBL_EPSILON;
    const NodeListParams L = hp.lists[multi ? li : list[i]];
    const float nodeScalei = 1.0f / (lmaxi * (float)L.nPerh);
    float bestf = 3.0e38f;
    const float csDt = nodeScalei / (P.thermo[i].z + tiny);
    if (csDt < bestf) { bestf = csDt; reason = 0; }
    const float csqDt = nodeScalei / (sqrtf((float)F.f[F_MAXQ][i] / (float)rho) + tiny);
    if (csqDt < bestf) { bestf = csqDt; reason = 1; }
    const float divv = (float)(F.f[F_DVDX_XX][i] + F.f[F_DVDX_YY][i] + F.f[F_DVDX_ZZ][i]);
    const float divvDt = 1.0f / (fabsf(divv) + tiny);
    if (divvDt < bestf) { bestf = divvDt; reason = 2; }
    const float vmag = sqrtf(vi.x * vi.x + vi.y * vi.y + vi.z * vi.z);
    const float ax = (float)F.f[F_DVDT_X][i], ay = (float)F.f[F_DVDT_Y][i], az = (float)F.f[F_DVDT_Z][i];
    const float dtAcc = 0.1f * fmaxf(nodeScalei / (vmag + tiny), vmag / (sqrtf(ax * ax + ay * ay + az * az) + tiny));
    if (dtAcc < bestf) { bestf = dtAcc; reason = 3; }
    if (hp.useVelMagDt) {
      const float velDt = nodeScalei / (vmag + 1.0e-10f);
      if (velDt < bestf) { bestf = velDt; reason = 4; }
    }
    const float pairDt = bestPair / (float)maxNperh;
    if (pairDt < bestf) { bestf = pairDt; reason = 5; }
    best = isGhost(hp, i) ? DBL_MAX : (double)bestf;   // halo copies do not vote
    if (isGhost(hp, i)) reason = -1;
  }
  sv[threadIdx.x] = best;
  sr[threadIdx.x] = reason;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o && sv[threadIdx.x + o] < sv[threadIdx.x]) {
      sv[threadIdx.x] = sv[threadIdx.x + o];
      sr[threadIdx.x] = sr[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = sv[0]; part[2 * blockIdx.x + 1] = (double)sr[0]; }
}

//------------------------------------------------------------------------------
// Grad-h correction, FP32 sums (computeSPHOmegaGradhCorrection.cc:15-116).
//------------------------------------------------------------------------------
// LEAN: compensated sums fixed at compile time.
template <bool TENSOR, bool LEAN>
__global__ void __launch_bounds__(128) gradhKernel32(Fields F, Fields32 P, long n, Grid g, NeighborLists nl,
                                                     TableDev t, HydroParams hp) {
  __shared__ float4 ta[kMaxTable / 3];
  __shared__ float2 tb[kMaxTable / 3];
  __shared__ float4 sOff[64];
  const int nint = hp.tableN1 + 1;
  for (int k = threadIdx.x; k < nint; k += blockDim.x) { ta[k] = t.p32a[k]; tb[k] = t.p32b[k]; }
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
  float4 hi0 = make_float4(0.f, 0.f, 0.f, 0.f), hi1 = hi0;
  if (TENSOR) { hi0 = P.hten[2 * i]; hi1 = P.hten[2 * i + 1]; }
  const float extent = (float)hp.extent, invStep = (float)(1.0 / hp.tableXstep);
  const int N1 = hp.tableN1;
  float ws = 0.f, wc = 0.f, gs = 0.f, gc = 0.f;
  const int cnt = nl.count[i];
  // software pipeline: entry two slots ahead, node position one slot ahead
  uint32_t entA = 0u, entB = 0u;
  float4 pjA = make_float4(0.f, 0.f, 0.f, 0.f);
  if (cnt > 0) {
    entA = nl.nbr[nbSlot(i, 0, nl.cap)];
    pjA = P.posh[(int)(entA & kIndexMask)];
  }
  if (cnt > 1) entB = nl.nbr[nbSlot(i, 1, nl.cap)];
  for (int q = 0; q < cnt; ++q) {
    const uint32_t ent = entA;
    const float4 pj = pjA;
    if (q + 1 < cnt) {
      pjA = P.posh[(int)(entB & kIndexMask)];
      entA = entB;
    }
    if (q + 2 < cnt) entB = nl.nbr[nbSlot(i, q + 2, nl.cap)];
    const int dcode = (int)(ent >> kIndexBits);
    float rx, ry, rz;
    relSepTab(pi, pj, dcode, mm, cx, cy, cz, sOff, rx, ry, rz);
    float eta;
    if (TENSOR) {
      eta = etaFromSq(eta2Sym32(hi0, hi1, rx, ry, rz));
    } else {
      const float ex = ai * rx, ey = ai * ry, ez = ai * rz;
      eta = etaFromSq(__fmaf_rn(ez, ez, __fmaf_rn(ey, ey, __fmul_rn(ex, ex))));
    }
    float w, gr;
    lookupPacked(ta, tb, N1, invStep, eta, extent, w, gr);
    sumAdd(ws, wc, w, LEAN ? 0 : hp.plainSums);
    sumAdd(gs, gc, eta * gr, LEAN ? 0 : hp.plainSums);
  }
  // Omega = -sum eta dW/deta / (3 (sum W + W0)) (Hdet cancels), in FP32 from
  // the compensated sums
  float omega = 1.0f;
  if (cnt > 0) omega = fmaxf(1.0e-30f, -(gs - gc) / (3.0f * ((ws - wc) + (float)hp.W0)));
  F.f[F_OMEGA][i] = (double)omega;
  P.thermo[i].w = omega / (omega * omega + 1.0e-30f);
}

//------------------------------------------------------------------------------
// GenericHydro::dt with the pairwise velocity limit in FP32.
//------------------------------------------------------------------------------
template <bool TENSOR>
__global__ void __launch_bounds__(128) dtKernel32(Fields F, Fields32 P, const int* __restrict__ list, long n, Grid g,
                                                  NeighborLists nl, HydroParams hp, double maxNperh,
                                                  double* __restrict__ part) {
  __shared__ double sv[128];
  __shared__ int sr[128];
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const double tiny = DBL_EPSILON;
  double best = DBL_MAX;
  int reason = -1;
  if (i < n && !isGhost(hp, i)) {
    int ci[3];
    unpackCell(P.cell[i], ci);
    const uint32_t mm = mirrorMask(g, ci);
    const NodeListParams L = hp.lists[list[i]];
    const double ai = F.f[TENSOR ? F_HLMAX : F_HINV][i];   // largest eigenvalue of H
    const double nodeScalei = 1.0 / ai / L.nPerh;
    const double vxi = F.f[F_VX][i], vyi = F.f[F_VY][i], vzi = F.f[F_VZ][i];
    const double rhoi = F.f[F_RHO][i];
    const double csDt = nodeScalei / (F.f[F_CS][i] + tiny);
    if (csDt < best) { best = csDt; reason = 0; }
    const double csqDt = nodeScalei / (sqrt(F.f[F_MAXQ][i] / rhoi) + tiny);
    if (csqDt < best) { best = csqDt; reason = 1; }
    const double divvDt = 1.0 / (fabs(F.f[F_DVDX_XX][i] + F.f[F_DVDX_YY][i] + F.f[F_DVDX_ZZ][i]) + tiny);
    if (divvDt < best) { best = divvDt; reason = 2; }
    const double vmag = sqrt(vxi * vxi + vyi * vyi + vzi * vzi);
    const double ax = F.f[F_DVDT_X][i], ay = F.f[F_DVDT_Y][i], az = F.f[F_DVDT_Z][i];
    const double dtAcc = 0.1 * fmax(nodeScalei / (vmag + tiny), vmag / (sqrt(ax * ax + ay * ay + az * az) + tiny));
    if (dtAcc < best) { best = dtAcc; reason = 3; }
    if (hp.useVelMagDt) {
      const double velDt = nodeScalei / (vmag + 1.0e-10);
      if (velDt < best) { best = velDt; reason = 4; }
    }
    const float4 vi = P.velm[i];
    const float hi = 1.0f / (TENSOR ? P.hten[2 * i + 1].w : P.posh[i].w);
    float bestPair = 3.0e38f;
    const int cnt = nl.count[i];
    for (int q = 0; q < cnt; ++q) {
      const long long k = nbSlot(i, q, nl.cap);
      const uint32_t ent = nl.nbr[k];
      const int j = (int)(ent & kIndexMask), dcode = (int)(ent >> kIndexBits);
      const float4 vj = P.velm[j];
      float vxj = vj.x, vyj = vj.y, vzj = vj.z;
      mirrorVel((uint32_t)dcode & mm, vxj, vyj, vzj);
      const float dx = vi.x - vxj, dy = vi.y - vyj, dz = vi.z - vzj;
      const float hmin = fminf(hi, 1.0f / (TENSOR ? P.hten[2 * j + 1].w : P.posh[j].w));
      const float dtv = hmin / fmaxf(1.0e-30f, sqrtf(dx * dx + dy * dy + dz * dz));
      bestPair = fminf(bestPair, dtv);
    }
    const double pairDt = (double)bestPair / maxNperh;
    if (pairDt < best) { best = pairDt; reason = 5; }
  }
  sv[threadIdx.x] = best;
  sr[threadIdx.x] = reason;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o && sv[threadIdx.x + o] < sv[threadIdx.x]) {
      sv[threadIdx.x] = sv[threadIdx.x + o];
      sr[threadIdx.x] = sr[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = sv[0]; part[2 * blockIdx.x + 1] = (double)sr[0]; }
}
__global__ void dtFinalKernel32(const double* __restrict__ part, int nb, double* __restrict__ out) {
  __shared__ double sv[256];
  __shared__ double sr[256];
  double best = DBL_MAX, reason = -1.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    if (part[2 * b] < best) { best = part[2 * b]; reason = part[2 * b + 1]; }
  sv[threadIdx.x] = best;
  sr[threadIdx.x] = reason;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o && sv[threadIdx.x + o] < sv[threadIdx.x]) {
      sv[threadIdx.x] = sv[threadIdx.x + o];
      sr[threadIdx.x] = sr[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { out[0] = sv[0]; out[1] = sr[0]; }
}

//------------------------------------------------------------------------------
// Compatible-energy sweep of the mixed mode (SpecificThermalEnergyPolicy.cc:110-173).
// v12 = v + a dt/2 is formed once per node in FP64; the per-pair work
// du_ij = (v12_j - v12_i) . pacc_ij uses the FP64 velocity difference rounded
// to FP32 and the FP32 pair acceleration; the weighted shares are summed and
// applied to the specific energy in FP64.
//------------------------------------------------------------------------------
__global__ void halfStepVelocityKernel(Fields F, long n, double hdt, float4* __restrict__ vhi,
                                       float4* __restrict__ vlo) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  // v12 = v + a dt/2 in FP64, stored as an unevaluated float pair hi + lo
  const double x = F.f[F_VX][i] + F.f[F_DVDT_X][i] * hdt;
  const double y = F.f[F_VY][i] + F.f[F_DVDT_Y][i] * hdt;
  const double z = F.f[F_VZ][i] + F.f[F_DVDT_Z][i] * hdt;
  const float hx = (float)x, hy = (float)y, hz = (float)z;
  vhi[i] = make_float4(hx, hy, hz, (float)F.f[F_DEPSDT][i]);
  vlo[i] = make_float4((float)(x - hx), (float)(y - hy), (float)(z - hz), 0.0f);
}

// B: slots per batch (the gathers and pair-acceleration reads in flight per
// thread); every B adds in the same slot order, so the result is the same.
template <int B>
__global__ void __launch_bounds__(128) energyKernel32(Fields F, long n, Grid g, NeighborLists nl,
                                                      const float4* __restrict__ vhi, const float4* __restrict__ vlo,
                                                      const float* __restrict__ pacc, double dt) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int ci[3];
  unpackCell(nl.cell[i], ci);
  const uint32_t mm = mirrorMask(g, ci);
  const float4 hi = vhi[i], lo = vlo[i];
  const float d0i = hi.w;
  const float feps = (float)DBL_EPSILON;
  float s = 0.0f, c = 0.0f;
  const int cnt = nl.count[i];
  // One slot: du = (v_j - v_i) . pacc_ij with the half-step velocities as
  // hi + lo float pairs, split by the DepsDt0 weights.
  auto slot = [&](uint32_t ent, float4 hj, float4 lj, float p0, float p1, float p2) {
    const int dcode = (int)(ent >> kIndexBits);
    float hx = hj.x, hy = hj.y, hz = hj.z, lx = lj.x, ly = lj.y, lz = lj.z;
    const uint32_t mir = (uint32_t)dcode & mm;
    if (mir) {
      if (mir & 3u) { hx = -hx; lx = -lx; }
      if (mir & 12u) { hy = -hy; ly = -ly; }
      if (mir & 48u) { hz = -hz; lz = -lz; }
    }
    // (hi_j - hi_i) + (lo_j - lo_i): the FP64 difference to FP32 rounding
    const float wx = __fadd_rn(__fsub_rn(hx, hi.x), __fsub_rn(lx, lo.x));
    const float wy = __fadd_rn(__fsub_rn(hy, hi.y), __fsub_rn(ly, lo.y));
    const float wz = __fadd_rn(__fsub_rn(hz, hi.z), __fsub_rn(lz, lo.z));
    const float du = __fmaf_rn(wz, p2, __fmaf_rn(wy, p1, __fmul_rn(wx, p0)));
    const float sg = du < 0.0f ? -1.0f : 1.0f;
    const float weighti = fmaxf(feps, d0i * sg);
    const float weightj = fmaxf(feps, hj.w * sg);
    // The split of du between i and j: both sides divide by the same sum with
    // IEEE rounding, so the two shares add up to du with unbiased rounding
    // errors.  (An approximate reciprocal here leaves a one-signed error on
    // every pair, which accumulates into a steady energy drift.)
    kahanAdd(s, c, __fmul_rn(__fdiv_rn(weighti, __fadd_rn(weighti, weightj)), du));
  };
  // Batches of B slots: all their loads are issued before any is used, so B
  // gathers and pair-acceleration reads are in flight together.  The entries
  // of the next batch are loaded while this batch's gathers are in flight.
  int q = 0;
  uint32_t en[B];
  if (B <= cnt) {
#pragma unroll
    for (int u = 0; u < B; ++u) en[u] = nl.nbr[nbSlot(i, u, nl.cap)];
  }
  for (; q + B <= cnt; q += B) {
    uint32_t e[B];
    float4 H[B], L[B];
    float p[B][3];
#pragma unroll
    for (int u = 0; u < B; ++u) e[u] = en[u];
    if (q + 2 * B <= cnt) {
#pragma unroll
      for (int u = 0; u < B; ++u) en[u] = nl.nbr[nbSlot(i, q + B + u, nl.cap)];
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const long long k = nbSlot(i, q + u, nl.cap);
      const int j = (int)(e[u] & kIndexMask);
      H[u] = vhi[j];
      L[u] = vlo[j];
      p[u][0] = pacc[3 * k]; p[u][1] = pacc[3 * k + 1]; p[u][2] = pacc[3 * k + 2];
    }
#pragma unroll
    for (int u = 0; u < B; ++u) slot(e[u], H[u], L[u], p[u][0], p[u][1], p[u][2]);
  }
  for (; q < cnt; ++q) {
    const long long k = nbSlot(i, q, nl.cap);
    const uint32_t ent = nl.nbr[k];
    const int j = (int)(ent & kIndexMask);
    slot(ent, vhi[j], vlo[j], pacc[3 * k], pacc[3 * k + 1], pacc[3 * k + 2]);
  }
  const double sum = kahanValue(s, c);
  F.f[F_DEPS_COMPAT][i] = sum;
  F.f[F_EPS][i] += sum * dt;
}

inline unsigned gridFor(long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

void launchPrepareFP32(Fields F, Fields32 F32, long n, Grid g, cudaStream_t s, LaunchCounter* lc) {
  prepareKernel<<<gridFor(n, 256), 256, 0, s>>>(F, F32, n, g);
  lc->add(1);
}

// variant (compatible energy, no XSPH, one NodeList): 0 the software-
// pipelined loop at 4 blocks per SM (<= 128 registers), 1 the same at 5
// (<= 102 registers), 2 two slots per iteration at 4, 3 four slots per
// iteration at 3 (<= 168 registers); with the limited Q, 0-1 the pipelined
// loop and 2-3 two slots per iteration.  Lean forms where the configuration
// allows.  Chosen at run time by the autotuner (kPairVariants); every
// variant gives the same bits.
void launchPairFP32(Fields F, Fields32 F32, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                    HydroParams hp, float* pacc, int variant, cudaStream_t s,
                    LaunchCounter* lc) {
  const int b = 128;
  const unsigned gb = gridFor(n, b);
  const bool multi = hp.numLists > 1;
  // lean forms (no run-time flag in the loop) when the configuration allows:
  // 1 with compensated sums, 2 with plain ones
  const int lean = (hp.epsTensile == 0.0 && !hp.linearInExpansion && !hp.quadraticInExpansion) ? (hp.plainSums ? 2 : 1) : 0;
#define SPH_PAIR32(X, C, M, MB, PF, LQ) \
  pairKernelFP32<X, C, M, MB, PF, LQ, false><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc)
#define SPH_PAIR32T(X, C, LQ)                                                                     \
  do {                                                                                            \
    if (variant & 1) pairKernelFP32<X, C, true, 4, true, LQ, true><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc); \
    else pairKernelFP32<X, C, true, 3, true, LQ, true><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc);             \
  } while (0)
  // ASPH (tensor H): NodeList test at run time; odd variants cap the
  // registers at 128 (4 blocks per SM), even ones at 168 (3); variants 0-1
  // the pipelined loop, 2-3 (compatible energy, no XSPH, standard Q) two
  // slots per iteration
  if (hp.asph) {
    if (!hp.xsph && hp.compatible && !hp.limitedQ && variant >= 2) {
      if (lean == 1) {
        if (variant & 1) pairKernelFP32<false, true, true, 4, 2, false, true, 1><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc);
        else pairKernelFP32<false, true, true, 3, 2, false, true, 1><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc);
      } else {
        if (variant & 1) pairKernelFP32<false, true, true, 4, 2, false, true, 0><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc);
        else pairKernelFP32<false, true, true, 3, 2, false, true, 0><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc);
      }
    } else if (hp.xsph) {
      if (hp.compatible) { if (hp.limitedQ) SPH_PAIR32T(true, true, true); else SPH_PAIR32T(true, true, false); }
      else { if (hp.limitedQ) SPH_PAIR32T(true, false, true); else SPH_PAIR32T(true, false, false); }
    } else {
      if (hp.compatible) { if (hp.limitedQ) SPH_PAIR32T(false, true, true); else SPH_PAIR32T(false, true, false); }
      else { if (hp.limitedQ) SPH_PAIR32T(false, false, true); else SPH_PAIR32T(false, false, false); }
    }
  } else if (hp.limitedQ) {   // LimitedMonaghanGingoldViscosity
    if (!hp.xsph && hp.compatible && !multi) {
      if (lean == 1) {
        if (variant >= 2) pairKernelFP32<false, true, false, 4, 2, true, false, 1><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc);
        else pairKernelFP32<false, true, false, 4, 1, true, false, 1><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc);
      } else {
        if (variant >= 2) pairKernelFP32<false, true, false, 4, 2, true, false, 0><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc);
        else pairKernelFP32<false, true, false, 4, 1, true, false, 0><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc);
      }
    } else if (hp.xsph) {
      if (hp.compatible) SPH_PAIR32(true, true, true, 4, false, true);
      else SPH_PAIR32(true, false, true, 4, false, true);
    } else {
      if (hp.compatible) SPH_PAIR32(false, true, true, 4, false, true);
      else SPH_PAIR32(false, false, true, 4, false, true);
    }
  } else if (!hp.xsph && hp.compatible && !multi) {
#define SPH_PAIR32V(MB, PF) \
  do {                                                                                                            \
    if (lean == 1) pairKernelFP32<false, true, false, MB, PF, false, false, 1><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc); \
    else if (lean == 2) pairKernelFP32<false, true, false, MB, PF, false, false, 2><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc); \
    else pairKernelFP32<false, true, false, MB, PF, false, false, 0><<<gb, b, 0, s>>>(F, F32, list, n, g, nl, t, hp, pacc); \
  } while (0)
    switch (variant) {
      case 1: SPH_PAIR32V(5, 1); break;
      case 2: SPH_PAIR32V(4, 2); break;
      case 3: SPH_PAIR32V(3, 4); break;
      default: SPH_PAIR32V(4, 1); break;
    }
#undef SPH_PAIR32V
  } else if (hp.xsph) {
    if (hp.compatible) {
      if (multi) SPH_PAIR32(true, true, true, 5, false, false); else SPH_PAIR32(true, true, false, 5, false, false);
    } else {
      if (multi) SPH_PAIR32(true, false, true, 5, false, false); else SPH_PAIR32(true, false, false, 5, false, false);
    }
  } else {
    if (hp.compatible) SPH_PAIR32(false, true, true, 5, false, false);
    else { if (multi) SPH_PAIR32(false, false, true, 5, false, false); else SPH_PAIR32(false, false, false, 5, false, false); }
  }
#undef SPH_PAIR32
#undef SPH_PAIR32T
  lc->add(1);
}

void launchSumDensityFP32(Fields F, Fields32 F32, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                          HydroParams hp, cudaStream_t s, LaunchCounter* lc) {
  if (hp.asph) sumDensityKernel32<true><<<gridFor(n, 128), 128, 0, s>>>(F, F32, list, n, g, nl, t, hp);
  else sumDensityKernel32<false><<<gridFor(n, 128), 128, 0, s>>>(F, F32, list, n, g, nl, t, hp);
  lc->add(1);
}

void launchGradhFP32(Fields F, Fields32 F32, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                     cudaStream_t s, LaunchCounter* lc) {
  if (hp.asph) {
    if (hp.plainSums) gradhKernel32<true, false><<<gridFor(n, 128), 128, 0, s>>>(F, F32, n, g, nl, t, hp);
    else gradhKernel32<true, true><<<gridFor(n, 128), 128, 0, s>>>(F, F32, n, g, nl, t, hp);
  } else {
    if (hp.plainSums) gradhKernel32<false, false><<<gridFor(n, 128), 128, 0, s>>>(F, F32, n, g, nl, t, hp);
    else gradhKernel32<false, true><<<gridFor(n, 128), 128, 0, s>>>(F, F32, n, g, nl, t, hp);
  }
  lc->add(1);
}

void launchDtFP32(Fields F, Fields32 F32, const int* list, long n, Grid g, NeighborLists nl, HydroParams hp,
                  double maxNperh, double* dScratch, int nScratch, double* dOut,
                  cudaStream_t s, LaunchCounter* lc) {
  (void)nScratch;
  const int nb = (int)gridFor(n, 128);
  if (hp.asph) dtKernel32<true><<<nb, 128, 0, s>>>(F, F32, list, n, g, nl, hp, maxNperh, dScratch);
  else dtKernel32<false><<<nb, 128, 0, s>>>(F, F32, list, n, g, nl, hp, maxNperh, dScratch);
  dtFinalKernel32<<<1, 256, 0, s>>>(dScratch, nb, dOut);
  lc->add(2);
}

void launchCompatibleEnergyFP32(Fields F, long n, Grid g, NeighborLists nl, const float* pacc, float4* vhi,
                                float4* vlo, double dt, int variant, cudaStream_t s, LaunchCounter* lc) {
  halfStepVelocityKernel<<<gridFor(n, 256), 256, 0, s>>>(F, n, 0.5 * dt, vhi, vlo);
  if (variant == 1) energyKernel32<8><<<gridFor(n, 128), 128, 0, s>>>(F, n, g, nl, vhi, vlo, pacc, dt);
  else if (variant == 2) energyKernel32<2><<<gridFor(n, 128), 128, 0, s>>>(F, n, g, nl, vhi, vlo, pacc, dt);
  else energyKernel32<4><<<gridFor(n, 128), 128, 0, s>>>(F, n, g, nl, vhi, vlo, pacc, dt);
  lc->add(2);
}

void launchDensityDtFP32(Fields F, Fields32 F32, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                         HydroParams hp, double maxNperh, double* dScratch,
                         double* dOut, cudaStream_t s, LaunchCounter* lc) {
  const int nb = (int)gridFor(n, 128);
  // lean: one NodeList and compensated sums fixed at compile time
  const bool lean = hp.numLists == 1 && !hp.plainSums;
  if (hp.asph) {
    if (lean) densityDtKernel32<true, true><<<nb, 128, 0, s>>>(F, F32, list, n, g, nl, t, hp, maxNperh, dScratch);
    else densityDtKernel32<true, false><<<nb, 128, 0, s>>>(F, F32, list, n, g, nl, t, hp, maxNperh, dScratch);
  } else if (lean) densityDtKernel32<false, true><<<nb, 128, 0, s>>>(F, F32, list, n, g, nl, t, hp, maxNperh, dScratch);
  else densityDtKernel32<false, false><<<nb, 128, 0, s>>>(F, F32, list, n, g, nl, t, hp, maxNperh, dScratch);
  dtFinalKernel32<<<1, 256, 0, s>>>(dScratch, nb, dOut);
  lc->add(2);
}

}  // namespace sph
