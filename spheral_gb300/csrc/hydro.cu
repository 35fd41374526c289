// SPH hydro kernels of libsphgpu (sm_103a): cell-list neighbour build,
// density sum, grad-h correction, the FP64 pair loop with its per-node
// finalisation and smoothing-scale update, the time-step vote, the
// compatible-energy sweep and the CheapSynchronousRK2 state updates.
//
// Formulation.  The reference walks an unordered pair list and scatters into
// both nodes through thread-private copies of 13 FieldLists
// (src/SPH/SPH.cc:271-475).  Here every kernel is a gather: one thread owns
// node i and walks i's neighbour list, so each unordered pair is evaluated
// twice (once per side) with no atomics and a fixed summation order.  Ghost
// nodes of periodic and reflecting boundaries are implicit: a neighbour
// entry carries a 6-bit image code and the neighbour's coordinates are mapped
// with the reference's own plane formula (imageCoord).
#include "device.cuh"

namespace sph {
namespace {
using namespace dev;

//------------------------------------------------------------------------------
// Bounds: min hinv, bounding box (for open axes) and, for tensor H, the
// largest half-width per axis of the unit ellipsoids {r : |H r| <= 1}, i.e.
// sqrt((H^-2)_aa) = |row a of H^-1| (the cell edge per axis).
//------------------------------------------------------------------------------
__global__ void boundsKernel(Fields F, long n, int tensor, double* __restrict__ part) {
  __shared__ double sm[32];
  double ah = DBL_MAX, mnx = DBL_MAX, mny = DBL_MAX, mnz = DBL_MAX, mxx = -DBL_MAX, mxy = -DBL_MAX, mxz = -DBL_MAX;
  double ex = 0.0, ey = 0.0, ez = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    ah = fmin(ah, F.f[F_HINV][i]);
    const double x = F.f[F_X][i], y = F.f[F_Y][i], z = F.f[F_Z][i];
    mnx = fmin(mnx, x); mny = fmin(mny, y); mnz = fmin(mnz, z);
    mxx = fmax(mxx, x); mxy = fmax(mxy, y); mxz = fmax(mxz, z);
    if (tensor) {
      const Sym w = symInverse(loadSym(F, F_HT_XX, i));
      ex = fmax(ex, sqrt(w.xx * w.xx + w.xy * w.xy + w.xz * w.xz));
      ey = fmax(ey, sqrt(w.xy * w.xy + w.yy * w.yy + w.yz * w.yz));
      ez = fmax(ez, sqrt(w.xz * w.xz + w.yz * w.yz + w.zz * w.zz));
    }
  }
  const double r[kBoundsVals] = {blockMin(ah, sm), blockMin(mnx, sm), blockMin(mny, sm), blockMin(mnz, sm),
                                 blockMax(mxx, sm), blockMax(mxy, sm), blockMax(mxz, sm),
                                 blockMax(ex, sm), blockMax(ey, sm), blockMax(ez, sm)};
  if (threadIdx.x == 0)
    for (int k = 0; k < kBoundsVals; ++k) part[blockIdx.x * kBoundsVals + k] = r[k];
}
__global__ void boundsFinalKernel(const double* __restrict__ part, int nb, double* __restrict__ out) {
  __shared__ double sm[32];
  double v[kBoundsVals];
  for (int k = 0; k < kBoundsVals; ++k) v[k] = k < 4 ? DBL_MAX : -DBL_MAX;
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int k = 0; k < kBoundsVals; ++k)
      v[k] = k < 4 ? fmin(v[k], part[b * kBoundsVals + k]) : fmax(v[k], part[b * kBoundsVals + k]);
  for (int k = 0; k < kBoundsVals; ++k) {
    const double r = k < 4 ? blockMin(v[k], sm) : blockMax(v[k], sm);
    if (threadIdx.x == 0) out[k] = r;
  }
}

//------------------------------------------------------------------------------
// Neighbour build.
//------------------------------------------------------------------------------
__global__ void cellKeyKernel(Fields F, long n, Grid g, uint32_t* __restrict__ keys, int* __restrict__ vals,
                              uint32_t* __restrict__ cellc) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double p[3] = {F.f[F_X][i], F.f[F_Y][i], F.f[F_Z][i]};
  uint32_t c[3], f[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    // position in half-cells, rounded down by the conversion itself: three
    // FP64-pipe instructions per axis (no division; the FP64 pipe is the
    // narrow one).  A node within rounding of a cell face may land in either
    // cell: the cells exceed the kernel support by a relative 1e-9, far
    // above that rounding.  NaN converts to the most negative value and is
    // clamped into cell 0.
    const long long hc = __double2ll_rd(__dmul_rn(__dsub_rn(p[a], g.lo[a]), g.inv2[a]));
    long long ci = hc >> 1;
    const bool clamped = ci < 0 || ci >= g.nc[a];
    ci = ci < 0 ? 0 : (ci >= g.nc[a] ? g.nc[a] - 1 : ci);
    c[a] = (uint32_t)ci;
    // the half of the cell the node is in (order within the cell only)
    f[a] = 2u * c[a] + ((!clamped && (hc & 1)) ? 1u : 0u);
  }
  // With a sub-cell level the key is the Morton key of the half-cells, whose
  // top bits are the cell's Morton key: nodes stay grouped by cell and within
  // a cell they are ordered by octant, so consecutive nodes of a cell (a work
  // chunk or a candidate batch of the neighbour search) sit close together.
  keys[i] = g.subShift ? morton3(f[0], f[1], f[2]) : morton3(c[0], c[1], c[2]);
  vals[i] = (int)i;
  cellc[i] = c[0] | (c[1] << 10) | (c[2] << 20);
}

__global__ void permuteKernel(Fields Fin, Fields Fout, const int* __restrict__ perm, const int* __restrict__ origIn,
                              int* __restrict__ origOut, const int* __restrict__ listIn, int* __restrict__ listOut,
                              const uint32_t* __restrict__ cellIn, uint32_t* __restrict__ cellOut, long n,
                              FieldRanges sel) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int p = perm[k];
  for (int r = 0; r < sel.n; ++r)
#pragma unroll 4
    for (int f = sel.first[r]; f < sel.last[r]; ++f) Fout.f[f][k] = Fin.f[f][p];
  origOut[k] = origIn[p];
  listOut[k] = listIn[p];
  cellOut[k] = cellIn[p];
}

__global__ void cellRangeKernel(const uint32_t* __restrict__ keys, long n, int shift, int* __restrict__ cellStart,
                                int* __restrict__ cellEnd) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t key = keys[k] >> shift;
  if (k == 0 || (keys[k - 1] >> shift) != key) cellStart[key] = (int)k;
  if (k == n - 1 || (keys[k + 1] >> shift) != key) cellEnd[key] = (int)(k + 1);
}

// Pair criterion of ConnectivityMap::computeConnectivity
// (src/Neighbor/ConnectivityMap.cc:917-929): (Hi rij)^2 <= ext^2 or
// (Hj rij)^2 <= ext^2, self excluded.  An FP32 test on cell-relative
// positions settles every candidate outside a narrow band around the
// threshold; candidates inside the band get the exact FP64 test with the
// reference's operation order, so the neighbour sets are exact.
//
// The search is group-cooperative.  A group of W lanes (W = 8, 16 or 32,
// chosen from the mean cell occupancy so few lanes idle) owns a chunk of up
// to W consecutive nodes of one cell (an "item"), so the 27 candidate cells,
// their offset codes and mirror flags are uniform across the group.  Each
// candidate cell is read in coalesced batches of W nodes staged in shared
// memory; every lane tests its own node against the batch.  Candidate cells
// are visited in a fixed order (dz, dy, dx from -1 to 1) and nodes within a
// cell in sorted order, so every list has a reproducible order.
// WRITE false: count only; true: count and write the warp-interleaved lists
// (slots beyond cap are counted, not written).
// Relative half-width of the FP32 band around |H r|^2 = ext^2 for a node with
// eigenvalues in [lmin, lmax].  Each FP32 separation component carries at
// most ~10 u C of rounding (C the largest cell edge, u = 2^-24), and the
// products and sums of H r add ~4 u |H| |r| per component; near the threshold
// (|H r| ~ ext, |r| <= ext / lmin) |H r| is then off by at most
// 30 u C lmax + 12 u ext lmax / lmin and its square by
// ext^2 u (60 C lmax / ext + 24 lmax / lmin + 3).  The band is four times that.
__device__ __forceinline__ float tensorBand(float lmax, float lmin, const Grid& g) {
  const float u = 5.9604645e-8f;
  const float C = fmaxf(g.cellf[0], fmaxf(g.cellf[1], g.cellf[2]));
  return 4.0f * u * (60.0f * C * lmax / sqrtf(g.ext2f) + 24.0f * lmax / lmin + 3.0f);
}

// The exact FP64 tensor criterion |H_i r|^2 <= ext^2 or |H_j r|^2 <= ext^2
// (H_j through the image).  Out of line: it runs for few candidates, and
// inlined its FP64 tensors would set the register count of the whole search.
__device__ __noinline__ bool exactTensorCriterion(const Fields& F, const Grid& g, long i, int j, int code, double qx,
                                                  double qy, double qz, double ext2) {
  Sym Hj = loadSym(F, F_HT_XX, j);
  imageSym(g, code, Hj);
  return eta2ExactSym(loadSym(F, F_HT_XX, i), qx, qy, qz) <= ext2 || eta2ExactSym(Hj, qx, qy, qz) <= ext2;
}

// TENSOR (ASPH): h^-1 in the FP32 mirror is the smallest eigenvalue of H, so
// the scalar pre-filter bounds |H r| from below and rejects the far
// candidates; the rest take |H_i r|^2 and |H_j r|^2 in FP32 from the tensor
// mirror with a per-node band (tensorBand), and only those inside a band
// take the exact FP64 tensor test.
//
// Batch culling: every chunk of up to W consecutive nodes of a cell has a
// bounding box (itemBoxKernel); a candidate batch whose box is farther from
// the group's own box than the largest FP32 band edge of the group allows,
// at the smaller of the two boxes' smallest h^-1, holds no neighbour of any
// of the group's nodes and is skipped whole (a group-uniform decision).
// With the sub-cell key order the chunks are compact, so the boxes are
// small and the far batches of the 27 cells drop out.
template <bool WRITE, int W, bool TENSOR>
__global__ void __launch_bounds__(128) neighborWarpKernel(Fields F, Fields32 P, long n, const int* __restrict__ items,
                                                          int nItems, Grid g, const int* __restrict__ cellStart,
                                                          const int* __restrict__ cellEnd, int* __restrict__ counts,
                                                          uint32_t* __restrict__ nbr, double ext2, float bandA,
                                                          float bandB, int cap, int* __restrict__ maxCount,
                                                          const long long* __restrict__ dItems,
                                                          const float4* __restrict__ box,
                                                          const int* __restrict__ chunkOf) {
  constexpr int G = 128 / W;             // groups per 128-thread block
  __shared__ float4 stage[G][W];         // one candidate batch per group
  constexpr int HW = TENSOR ? 2 * W : 1;
  __shared__ float4 stageH[G][HW];       // TENSOR: the batch's H (xx xy xz yy | yz zz band .)
  __shared__ int4 cinfo[G][27];          // the 27 candidate cells: node range, first work chunk, cell-offset code
  __shared__ float4 coff[G][27];         // the cell offset (ox, oy, oz) of each
  // Isotropic H: each batch's culling box is loaded a batch ahead (in lanes
  // 0 and 1) and passed through shared memory; the tensor path, heavier in
  // registers already, loads it when its batch comes up.
  constexpr bool BOXAHEAD = !TENSOR;
  __shared__ float4 sbox[G][2];          // the current batch's box (lo, hi)
  const int item = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) / W);
  const int lane = threadIdx.x % W, wib = threadIdx.x / W;
  // lanes of this group within the warp
  const unsigned gmask = (W == 32) ? 0xffffffffu : (((1u << W) - 1u) << ((threadIdx.x & 31) / W * W));
  // the grid is sized for an upper bound; the item count itself is on the device
  if (item >= min((long long)nItems, *dItems)) return;   // group-uniform
  const int k0 = items[item];
  const uint32_t cc = P.cell[k0];
  int hc[3];
  unpackCell(cc, hc);
  // The 27 cell ranges are independent loads: fetch them lane-parallel so
  // their latencies overlap, with each cell's first work chunk (its batches'
  // boxes follow consecutively) and its offset code and offset.  Cell t is
  // (dx, dy, dz) = (t%3, t/3%3, t/9) - 1.
  for (int t = lane; t < 27; t += W) {
    const int d[3] = {t % 3 - 1, (t / 3) % 3 - 1, t / 9 - 1};
    int cell[3];
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      int nn = hc[a] + d[a];
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
    const int d0 = t % 3, d1 = (t / 3) % 3, d2 = t / 9;   // 0, 1, 2 for -1, 0, +1
    const int dcode = (d0 == 0 ? 1 : (d0 == 2 ? 2 : 0)) | ((d1 == 0 ? 1 : (d1 == 2 ? 2 : 0)) << 2) |
                      ((d2 == 0 ? 1 : (d2 == 2 ? 2 : 0)) << 4);
    int4 r = make_int4(0, 0, 0, dcode);
    if (ok) {
      const uint32_t key = morton3((uint32_t)cell[0], (uint32_t)cell[1], (uint32_t)cell[2]);
      r.x = cellStart[key];
      r.y = cellEnd[key];
      if (r.x < r.y) r.z = chunkOf[r.x];
    }
    cinfo[wib][t] = r;
    coff[wib][t] = make_float4(d0 == 0 ? g.cellf[0] : (d0 == 2 ? -g.cellf[0] : 0.0f),
                               d1 == 0 ? g.cellf[1] : (d1 == 2 ? -g.cellf[1] : 0.0f),
                               d2 == 0 ? g.cellf[2] : (d2 == 2 ? -g.cellf[2] : 0.0f), 0.0f);
  }
  __syncwarp(gmask);
  const int k1 = min(k0 + W, cinfo[wib][13].y);   // cell 13 is the home cell
  const long i = k0 + lane;
  const bool active = i < k1;
  const float4 pi = active ? P.posh[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float ai2 = pi.w * pi.w;
  const float del = __fmaf_rn(bandA, pi.w, bandB);   // per-node band half-width (relative)
  const float e2t = g.ext2f;
  const float bandLo = del < 0.5f ? e2t * (1.0f - del) : -1.0f;
  const float bandHi = del < 0.5f ? e2t * (1.0f + del) : FLT_MAX;
  const uint32_t mm = mirrorMask(g, hc);
  const float cx = g.cellf[0], cy = g.cellf[1], cz = g.cellf[2];
  float4 hi0 = make_float4(0.f, 0.f, 0.f, 0.f), hi1 = hi0;
  float tLo = 0.f, tHi = 0.f;
  if (TENSOR && active) {
    hi0 = P.hten[2 * i];
    hi1 = P.hten[2 * i + 1];
    const float dI = tensorBand(hi1.w, pi.w, g);
    tLo = dI < 0.5f ? e2t * (1.0f - dI) : -1.0f;
    tHi = dI < 0.5f ? e2t * (1.0f + dI) : FLT_MAX;
  }
  int cnt = 0;
  // the group's box and the culling threshold on gap^2 min(a)^2: the largest
  // band edge of the group's nodes, widened against FP32 rounding; no
  // culling where a band is wide open
  const float4 gLo = box[2 * item], gHi = box[2 * item + 1];
  const float delMax = __fmaf_rn(bandA, gHi.w, bandB);
  const bool cull = delMax < 0.5f;
  const float cullThr = e2t * (1.0f + delMax) * 1.0001f;
  // slot 0 of node i in the warp-interleaved lists; slot q is 32 entries further per q
  uint32_t* out = WRITE ? nbr + nbSlot(i, 0, cap) : nullptr;
  // first batch of the first non-empty cell (and its box), loaded ahead of use
  int tn = 0;
  while (tn < 27 && cinfo[wib][tn].x >= cinfo[wib][tn].y) ++tn;
  float4 qn = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 hn0 = qn, hn1 = qn, nbox = qn;
  if (tn < 27) {
    const int4 c0 = cinfo[wib][tn];
    if (c0.x + lane < c0.y) {
      qn = P.posh[c0.x + lane];
      if (TENSOR) { hn0 = P.hten[2 * (c0.x + lane)]; hn1 = P.hten[2 * (c0.x + lane) + 1]; }
    }
    if (BOXAHEAD && cull && lane < 2) nbox = box[2 * c0.z + lane];
  }
  while (tn < 27) {
    const int t = tn;
    const int4 ct = cinfo[wib][t];
    const int s = ct.x, e = ct.y, dcode = ct.w;
    const float4 off = coff[wib][t];
    const uint32_t mir = (uint32_t)dcode & mm;
    const float ox = off.x, oy = off.y, oz = off.z;
    // next non-empty cell
    ++tn;
    while (tn < 27 && cinfo[wib][tn].x >= cinfo[wib][tn].y) ++tn;
    for (int base = s, cb = ct.z; base < e; base += W, ++cb) {
      float4 q = qn;
      float4 qh0 = hn0, qh1 = hn1;
      if (BOXAHEAD && cull) {
        if (lane < 2) sbox[wib][lane] = nbox;
        __syncwarp(gmask);
      }
      // prefetch the next batch's candidates (and box: that of chunk cb + 1,
      // or of the next cell's first chunk)
      if (base + W < e) {            // another batch of this cell follows
        const bool ok = base + W + lane < e;
        qn = ok ? P.posh[base + W + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (TENSOR && ok) { hn0 = P.hten[2 * (base + W + lane)]; hn1 = P.hten[2 * (base + W + lane) + 1]; }
        if (BOXAHEAD && cull && lane < 2) nbox = box[2 * (cb + 1) + lane];
      } else if (tn < 27) {          // last batch: prefetch the next cell's first batch
        const int4 cn = cinfo[wib][tn];
        const bool ok = cn.x + lane < cn.y;
        qn = ok ? P.posh[cn.x + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (TENSOR && ok) { hn0 = P.hten[2 * (cn.x + lane)]; hn1 = P.hten[2 * (cn.x + lane) + 1]; }
        if (BOXAHEAD && cull && lane < 2) nbox = box[2 * cn.z + lane];
      }
      if (cull) {
        float4 bLo, bHi;
        if (BOXAHEAD) { bLo = sbox[wib][0]; bHi = sbox[wib][1]; }
        else { bLo = box[2 * cb]; bHi = box[2 * cb + 1]; }
        // the batch's box in the frame of the group's cell: a candidate at q
        // (mirrored where the entry crosses a wall) sits at q - o there
        float lx = bLo.x, hx = bHi.x, ly = bLo.y, hy = bHi.y, lz = bLo.z, hz = bHi.z;
        if (mir & 3u) { lx = cx - bHi.x; hx = cx - bLo.x; }
        if (mir & 12u) { ly = cy - bHi.y; hy = cy - bLo.y; }
        if (mir & 48u) { lz = cz - bHi.z; hz = cz - bLo.z; }
        const float gx = fmaxf(0.0f, fmaxf((lx - ox) - gHi.x, gLo.x - (hx - ox)));
        const float gy = fmaxf(0.0f, fmaxf((ly - oy) - gHi.y, gLo.y - (hy - oy)));
        const float gz = fmaxf(0.0f, fmaxf((lz - oz) - gHi.z, gLo.z - (hz - oz)));
        const float am = fminf(gLo.w, bLo.w);
        if ((am * am) * (gx * gx + gy * gy + gz * gz) > cullThr) continue;   // group-uniform
      }
      if (TENSOR) {   // band of node j, then H_j seen through the mirrors
        qh1.z = tensorBand(qh1.w, q.w, g);
        const float sx = (mir & 3u) ? -1.f : 1.f, sy = (mir & 12u) ? -1.f : 1.f, sz = (mir & 48u) ? -1.f : 1.f;
        qh0.y *= sx * sy;   // xy
        qh0.z *= sx * sz;   // xz
        qh1.x *= sy * sz;   // yz
        stageH[wib][2 * lane] = qh0;
        stageH[wib][2 * lane + 1] = qh1;
      }
      if (mir) {
        if (mir & 3u) q.x = cx - q.x;
        if (mir & 12u) q.y = cy - q.y;
        if (mir & 48u) q.z = cz - q.z;
      }
      q.w = q.w * q.w;   // (h_j^-1)^2
      // Stage the batch in shared memory: each lane then reads every
      // candidate with one broadcast load.
      stage[wib][lane] = q;
      __syncwarp(gmask);
      const int nval = min(W, e - base);
      // the home cell's own batch contains node i itself
      const int self = (dcode == 0 && i >= base && i < base + nval) ? (int)(i - base) : -1;
      if (!TENSOR && active) {
        // Isotropic H.  The common path takes no branch per candidate: every
        // candidate up to the top of the band is stored, and the largest
        // stored e2 tells whether one of them sits inside the band; the
        // (rare) batches that hold one are written again in candidate order
        // with the exact FP64 criterion for the band candidates, so a list
        // is the same for every group width (and so is the rounding of its
        // sums).  The capacity is
        // checked once per batch unless the batch could overflow it, and
        // the self test runs only in the group's own batch of the home cell.
        const uint32_t ebase = (uint32_t)base | ((uint32_t)dcode << kIndexBits);
        const float px = __fadd_rn(pi.x, ox), py = __fadd_rn(pi.y, oy), pz = __fadd_rn(pi.z, oz);
        const bool own = dcode == 0 && base == k0;   // group-uniform: here candidate `lane` is node i
        const int cnt0 = cnt;
        bool amb = false;
        if (!WRITE || cnt + nval <= cap) {
          uint32_t* o = WRITE ? out + (size_t)cnt * 32 : nullptr;
          int c = 0;
          float mx = -1.0f;   // largest e2 stored
          if (!own) {
#pragma unroll 4
            for (int u = 0; u < nval; ++u) {
              const float4 cq = stage[wib][u];
              const float rx = __fsub_rn(px, cq.x), ry = __fsub_rn(py, cq.y), rz = __fsub_rn(pz, cq.z);
              const float e2 = fminf(ai2, cq.w) * (rx * rx + ry * ry + rz * rz);
              if (e2 <= bandHi) {
                if (WRITE) o[(size_t)c * 32] = ebase + (uint32_t)u;
                ++c;
                mx = fmaxf(mx, e2);
              }
            }
          } else {
#pragma unroll 4
            for (int u = 0; u < nval; ++u) {
              const float4 cq = stage[wib][u];
              const float rx = __fsub_rn(px, cq.x), ry = __fsub_rn(py, cq.y), rz = __fsub_rn(pz, cq.z);
              const float e2 = fminf(ai2, cq.w) * (rx * rx + ry * ry + rz * rz);
              if ((e2 <= bandHi) & (u != lane)) {
                if (WRITE) o[(size_t)c * 32] = ebase + (uint32_t)u;
                ++c;
                mx = fmaxf(mx, e2);
              }
            }
          }
          amb = mx >= bandLo;
          cnt += c;
        } else {   // this batch may reach the capacity: count past it, store below it
          for (int u = 0; u < nval; ++u) {
            const float4 cq = stage[wib][u];
            const float rx = __fsub_rn(px, cq.x), ry = __fsub_rn(py, cq.y), rz = __fsub_rn(pz, cq.z);
            const float e2 = fminf(ai2, cq.w) * (rx * rx + ry * ry + rz * rz);
            amb |= (e2 >= bandLo) & (e2 <= bandHi);
            if ((e2 < bandLo) & (u != self)) {
              if (WRITE && cnt < cap) out[(size_t)cnt * 32] = ebase + (uint32_t)u;
              ++cnt;
            }
          }
        }
        if (amb) {   // guard band: the batch again, band candidates by the exact FP64 criterion
          cnt = cnt0;
          for (int u = 0; u < nval; ++u) {
            const float4 cq = stage[wib][u];
            const float rx = __fsub_rn(px, cq.x), ry = __fsub_rn(py, cq.y), rz = __fsub_rn(pz, cq.z);
            const float e2 = fminf(ai2, cq.w) * (rx * rx + ry * ry + rz * rz);
            if (e2 > bandHi || u == self) continue;
            bool in = e2 < bandLo;
            if (!in) {
              const int j = base + u;
              double xjd = F.f[F_X][j], yjd = F.f[F_Y][j], zjd = F.f[F_Z][j];
              imagePos(g, imageCode(g, hc, dcode), xjd, yjd, zjd);
              const double qx = __dsub_rn(F.f[F_X][i], xjd), qy = __dsub_rn(F.f[F_Y][i], yjd),
                           qz = __dsub_rn(F.f[F_Z][i], zjd);
              in = eta2Exact(F.f[F_HINV][i], qx, qy, qz) <= ext2 || eta2Exact(F.f[F_HINV][j], qx, qy, qz) <= ext2;
            }
            if (in) {
              if (WRITE && cnt < cap) out[(size_t)cnt * 32] = ebase + (uint32_t)u;
              ++cnt;
            }
          }
        }
      }
      if (TENSOR && active) {
        // Tensor H: the scalar pre-filter (h^-1 the smallest eigenvalue)
        // rejects the far candidates, the rest take the FP32 tensor test on
        // each side with its own band; candidates inside a band only raise a
        // flag, and flagged batches are written again in candidate order with
        // the exact FP64 tensor criterion for the flagged candidates.
        const uint32_t ebase = (uint32_t)base | ((uint32_t)dcode << kIndexBits);
        // this node shifted by the cell offset: r = (x_i + o) - x_j
        const float px = __fadd_rn(pi.x, ox), py = __fadd_rn(pi.y, oy), pz = __fadd_rn(pi.z, oz);
        const int cnt0 = cnt;
        bool amb = false;
#pragma unroll 4
        for (int u = 0; u < nval; ++u) {
          const float4 cq = stage[wib][u];
          const float rx = __fsub_rn(px, cq.x), ry = __fsub_rn(py, cq.y), rz = __fsub_rn(pz, cq.z);
          const float e2 = fminf(ai2, cq.w) * (rx * rx + ry * ry + rz * rz);
          if (e2 <= bandHi) {
            const float4 h0 = stageH[wib][2 * u], h1 = stageH[wib][2 * u + 1];
            const float e2i = eta2Sym32(hi0, hi1, rx, ry, rz);
            const float e2j = eta2Sym32(h0, h1, rx, ry, rz);
            const float jLo = h1.z < 0.5f ? e2t * (1.0f - h1.z) : -1.0f;
            const float jHi = h1.z < 0.5f ? e2t * (1.0f + h1.z) : FLT_MAX;
            const bool in = (e2i <= tLo) | (e2j <= jLo);
            amb |= !in & !((e2i >= tHi) & (e2j >= jHi));
            if (in & (u != self)) {
              if (WRITE && cnt < cap) out[(size_t)cnt * 32] = ebase + (uint32_t)u;
              ++cnt;
            }
          }
        }
        if (amb) {   // guard band: the batch again, flagged candidates by the exact FP64 tensor criterion
          const int code = imageCode(g, hc, dcode);
          cnt = cnt0;
          for (int u = 0; u < nval; ++u) {
            const float4 cq = stage[wib][u];
            const float rx = __fsub_rn(px, cq.x), ry = __fsub_rn(py, cq.y), rz = __fsub_rn(pz, cq.z);
            const float e2 = fminf(ai2, cq.w) * (rx * rx + ry * ry + rz * rz);
            if (e2 > bandHi || u == self) continue;
            const float4 h0 = stageH[wib][2 * u], h1 = stageH[wib][2 * u + 1];
            const float e2i = eta2Sym32(hi0, hi1, rx, ry, rz);
            const float e2j = eta2Sym32(h0, h1, rx, ry, rz);
            const float jLo = h1.z < 0.5f ? e2t * (1.0f - h1.z) : -1.0f;
            const float jHi = h1.z < 0.5f ? e2t * (1.0f + h1.z) : FLT_MAX;
            bool in = (e2i <= tLo) | (e2j <= jLo);
            if (!in && !((e2i >= tHi) & (e2j >= jHi))) {
              const int j = base + u;
              double xjd = F.f[F_X][j], yjd = F.f[F_Y][j], zjd = F.f[F_Z][j];
              imagePos(g, code, xjd, yjd, zjd);
              const double qx = __dsub_rn(F.f[F_X][i], xjd), qy = __dsub_rn(F.f[F_Y][i], yjd),
                           qz = __dsub_rn(F.f[F_Z][i], zjd);
              in = exactTensorCriterion(F, g, i, j, code, qx, qy, qz, ext2);
            }
            if (in) {
              if (WRITE && cnt < cap) out[(size_t)cnt * 32] = ebase + (uint32_t)u;
              ++cnt;
            }
          }
        }
      }
      __syncwarp(gmask);
    }
  }
  // The stored count never exceeds the capacity: sweeps that run before an
  // overflow is noticed read only written slots.  The true maximum goes to
  // maxCount (the overflow signal).
  if (active) counts[i] = WRITE ? min(cnt, cap) : cnt;
  // one atomic per group: a per-node atomic on a single address serialises
  const int gmax = __reduce_max_sync(gmask, active ? cnt : 0);
  if (lane == 0) atomicMax(maxCount, gmax);
}

// Items of the warp search: the first node of every chunk of up to 32 nodes
// of a cell.  flag pass + scan + fill.
__global__ void itemFlagKernel(const uint32_t* __restrict__ keys, long n, int shift,
                               const int* __restrict__ cellStart, int width, int* __restrict__ flag) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  flag[k] = ((k - cellStart[keys[k] >> shift]) % width == 0) ? 1 : 0;
}
// Bounding box of every work chunk (up to `width` consecutive nodes of one
// cell) in its cell's FP32 coordinates, with the smallest and largest h^-1:
// box[2k] = (min x, min y, min z, min a), box[2k+1] = (max x, max y, max z,
// max a).  chunkOf[first node of the chunk] = k.
__global__ void itemBoxKernel(const int* __restrict__ items, const long long* __restrict__ dItems, long n,
                              int width, Fields32 P, float4* __restrict__ box, int* __restrict__ chunkOf) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= *dItems) return;
  const int s = items[k];
  const uint32_t cell = P.cell[s];
  float4 lo = P.posh[s], hi = lo;
  for (int j = s + 1; j < s + width && j < n && P.cell[j] == cell; ++j) {
    const float4 q = P.posh[j];
    lo = make_float4(fminf(lo.x, q.x), fminf(lo.y, q.y), fminf(lo.z, q.z), fminf(lo.w, q.w));
    hi = make_float4(fmaxf(hi.x, q.x), fmaxf(hi.y, q.y), fmaxf(hi.z, q.z), fmaxf(hi.w, q.w));
  }
  box[2 * k] = lo;
  box[2 * k + 1] = hi;
  chunkOf[s] = (int)k;
}
__global__ void itemFillKernel(const int* __restrict__ flag, const long long* __restrict__ pos, long n,
                               int* __restrict__ items) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  if (flag[k]) items[pos[k]] = (int)k;
}

//------------------------------------------------------------------------------
// computeSPHSumMassDensity (src/SPH/computeSPHSumMassDensity.cc:15-87),
// gathered: rho_i = m_i W(0) Hdet_i + sum_j m W(|Hj ri - Hj rj|, Hdet_j) with
// m = m_j for the same NodeList and m_i otherwise.  TENSOR: H_j a symmetric
// tensor (ASPH), seen through the image of the entry.
//------------------------------------------------------------------------------
template <bool TENSOR>
__global__ void __launch_bounds__(128) sumDensityKernel(Fields F, const int* __restrict__ list, long n, Grid g,
                                                        NeighborLists nl, TableDev t, HydroParams hp) {
  extern __shared__ double smem[];
  const int ntab = 3 * (hp.tableN1 + 1);
  for (int k = threadIdx.x; k < ntab; k += blockDim.x) smem[k] = t.w[k];
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int hc[3];
  unpackCell(nl.cell[i], hc);
  const double* __restrict__ X = F.f[F_X];
  const double* __restrict__ Y = F.f[F_Y];
  const double* __restrict__ Z = F.f[F_Z];
  const double* __restrict__ A = F.f[F_HINV];
  const double* __restrict__ Ms = F.f[F_MASS];
  const double xi = X[i], yi = Y[i], zi = Z[i], ai = A[i], mi = Ms[i];
  const int li = list[i];
  const double Hdeti = TENSOR ? symDet(loadSym(F, F_HT_XX, i)) : (ai * ai) * ai;
  const double self = mi * (Hdeti * smem[0]);
  double sum = 0.0;
  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const long long k = nbSlot(i, q, nl.cap);
    const uint32_t ent = nl.nbr[k];
    const int j = (int)(ent & kIndexMask), code = imageCode(g, hc, (int)(ent >> kIndexBits));
    double xj = X[j], yj = Y[j], zj = Z[j];
    imagePos(g, code, xj, yj, zj);
    double dx, dy, dz, Hdetj;
    if (TENSOR) {   // |Hj ri - Hj rj|
      Sym Hj = loadSym(F, F_HT_XX, j);
      imageSym(g, code, Hj);
      double ax, ay, az, bx, by, bz;
      symDot(Hj, xi, yi, zi, ax, ay, az);
      symDot(Hj, xj, yj, zj, bx, by, bz);
      dx = ax - bx; dy = ay - by; dz = az - bz;
      Hdetj = symDet(Hj);
    } else {
      const double aj = A[j];
      dx = __dsub_rn(__dmul_rn(aj, xi), __dmul_rn(aj, xj));
      dy = __dsub_rn(__dmul_rn(aj, yi), __dmul_rn(aj, yj));
      dz = __dsub_rn(__dmul_rn(aj, zi), __dmul_rn(aj, zj));
      Hdetj = (aj * aj) * aj;
    }
    const double eta = sqrt(dx * dx + dy * dy + dz * dz);
    if (eta < hp.extent) {
      const int i0 = tableIndex(eta, hp.tableN1, hp.tableXstep);
      const double Wj = Hdetj * tableEval(smem, i0, eta);
      sum += (list[j] == li ? Ms[j] : mi) * Wj;
    }
  }
  F.f[F_RHO][i] = self + sum;
}

//------------------------------------------------------------------------------
// computeSPHOmegaGradhCorrection (src/SPH/computeSPHOmegaGradhCorrection.cc:15-116).
//------------------------------------------------------------------------------
template <bool TENSOR>
__global__ void __launch_bounds__(128) gradhKernel(Fields F, long n, Grid g, NeighborLists nl, TableDev t,
                                                   HydroParams hp) {
  extern __shared__ double smem[];
  const int ntab = 3 * (hp.tableN1 + 1);
  for (int k = threadIdx.x; k < ntab; k += blockDim.x) { smem[k] = t.w[k]; smem[ntab + k] = t.g[k]; }
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int hc[3];
  unpackCell(nl.cell[i], hc);
  const double* __restrict__ X = F.f[F_X];
  const double* __restrict__ Y = F.f[F_Y];
  const double* __restrict__ Z = F.f[F_Z];
  const double xi = X[i], yi = Y[i], zi = Z[i], ai = F.f[F_HINV][i];
  Sym Hi{};
  if (TENSOR) Hi = loadSym(F, F_HT_XX, i);
  const double Hdeti = TENSOR ? symDet(Hi) : (ai * ai) * ai;
  double wsum = 0.0, gsum = 0.0;
  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const long long k = nbSlot(i, q, nl.cap);
    const uint32_t ent = nl.nbr[k];
    const int j = (int)(ent & kIndexMask), code = imageCode(g, hc, (int)(ent >> kIndexBits));
    double xj = X[j], yj = Y[j], zj = Z[j];
    imagePos(g, code, xj, yj, zj);
    const double rx = xi - xj, ry = yi - yj, rz = zi - zj;
    double ex, ey, ez;
    if (TENSOR) symDot(Hi, rx, ry, rz, ex, ey, ez);
    else { ex = ai * rx; ey = ai * ry; ez = ai * rz; }
    const double eta = sqrt(ex * ex + ey * ey + ez * ez);
    if (eta < hp.extent) {
      const int i0 = tableIndex(eta, hp.tableN1, hp.tableXstep);
      wsum += Hdeti * tableEval(smem, i0, eta);
      gsum += eta * (Hdeti * tableEval(smem + ntab, i0, eta));
    }
  }
  double omega;
  if (cnt == 0) omega = 1.0;
  else omega = fmax(1.0e-30, -gsum / (3.0 * (wsum + Hdeti * hp.W0)));
  F.f[F_OMEGA][i] = omega;
}

//------------------------------------------------------------------------------
// SPH::evaluateDerivativesImpl (src/SPH/SPH.cc:294-552) with
// MonaghanGingoldViscosity::QPiij (MonaghanGingoldViscosity.cc:41-101) and the
// SPHSmoothingScale moments + IdealH (SPHSmoothingScale.cc:154-272), FP64.
//------------------------------------------------------------------------------
// TENSOR: ASPH -- symmetric-tensor H_i, H_j (eta = H r, grad W = gW H eta^),
// the ASPHClassicSmoothingScale second moment and its finalize.
template <bool XSPH, bool COMPAT, bool TENSOR>
__global__ void __launch_bounds__(128) pairKernelFP64(Fields F, const int* __restrict__ list, long n, Grid g,
                                                      NeighborLists nl, TableDev t, HydroParams hp,
                                                      double* __restrict__ pacc) {
  extern __shared__ double smem[];
  const int ntab = 3 * (hp.tableN1 + 1);
  for (int k = threadIdx.x; k < ntab; k += blockDim.x) { smem[k] = t.w[k]; smem[ntab + k] = t.g[k]; }
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int hc[3];
  unpackCell(nl.cell[i], hc);
  const double* __restrict__ X = F.f[F_X];
  const double* __restrict__ Y = F.f[F_Y];
  const double* __restrict__ Z = F.f[F_Z];
  const double* __restrict__ VX = F.f[F_VX];
  const double* __restrict__ VY = F.f[F_VY];
  const double* __restrict__ VZ = F.f[F_VZ];
  const double* __restrict__ Ms = F.f[F_MASS];
  const double* __restrict__ RHO = F.f[F_RHO];
  const double* __restrict__ PP = F.f[F_P];
  const double* __restrict__ CS = F.f[F_CS];
  const double* __restrict__ OM = F.f[F_OMEGA];
  const double* __restrict__ A = F.f[F_HINV];
  const double* __restrict__ tw = smem;
  const double* __restrict__ tg = smem + ntab;

  const double xi = X[i], yi = Y[i], zi = Z[i], vxi = VX[i], vyi = VY[i], vzi = VZ[i];
  const double mi = Ms[i], rhoi = RHO[i], Pi = PP[i], ci = CS[i], omi = OM[i], ai = A[i];
  const int li = list[i];
  Sym Hi{};
  if (TENSOR) Hi = loadSym(F, F_HT_XX, i);
  const double Hdeti = TENSOR ? symDet(Hi) : (ai * ai) * ai;
  const double safeOmegai = omi / (omi * omi + kTiny30);
  const double tiny = kTiny30;
  const double Clij = 0.5 * (1.0 + 1.0) * 1.0 * hp.Cl;
  const double Cqij = 0.5 * (1.0 + 1.0) * 1.0 * hp.Cq;
  double DQi[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) DQi[k] = hp.limitedQ ? F.f[F_DVDXQ_XX + k][i] : 0.0;

  NodeAcc a;
  a.rhoSum = a.norm = a.dvx = a.dvy = a.dvz = a.deps = a.gx = a.gy = a.gz = 0.0;
  a.maxQ = 0.0; a.effQ = a.xw = a.xdx = a.xdy = a.xdz = a.m0 = a.m1x = a.m1y = a.m1z = 0.0;
#pragma unroll
  for (int k = 0; k < 9; ++k) { a.D[k] = 0.0; a.M[k] = 0.0; }
#pragma unroll
  for (int k = 0; k < 6; ++k) a.m2[k] = 0.0;

  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const long long k = nbSlot(i, q, nl.cap);
    const uint32_t ent = nl.nbr[k];
    const int j = (int)(ent & kIndexMask), code = imageCode(g, hc, (int)(ent >> kIndexBits));
    double xj = X[j], yj = Y[j], zj = Z[j], vxj = VX[j], vyj = VY[j], vzj = VZ[j];
    imagePos(g, code, xj, yj, zj);
    imageVec(g, code, vxj, vyj, vzj);
    const double mj = Ms[j], rhoj = RHO[j], Pj = PP[j], cj = CS[j], omj = OM[j], aj = A[j];
    const int lj = list[j];
    Sym Hj{};
    if (TENSOR) {
      Hj = loadSym(F, F_HT_XX, j);
      imageSym(g, code, Hj);
    }
    const double Hdetj = TENSOR ? symDet(Hj) : (aj * aj) * aj;
    const double safeOmegaj = omj / (omj * omj + kTiny30);

    const double rx = xi - xj, ry = yi - yj, rz = zi - zj;
    double eix, eiy, eiz, ejx, ejy, ejz;
    if (TENSOR) {
      symDot(Hi, rx, ry, rz, eix, eiy, eiz);
      symDot(Hj, rx, ry, rz, ejx, ejy, ejz);
    } else {
      eix = ai * rx; eiy = ai * ry; eiz = ai * rz;
      ejx = aj * rx; ejy = aj * ry; ejz = aj * rz;
    }
    const double etaMag2i = eix * eix + eiy * eiy + eiz * eiz;
    const double etaMag2j = ejx * ejx + ejy * ejy + ejz * ejz;
    const double etaMagi = sqrt(etaMag2i), etaMagj = sqrt(etaMag2j);
    const double sIi = 1.0 / fmax(tiny, etaMagi), sIj = 1.0 / fmax(tiny, etaMagj);
    const double uix = eix * sIi, uiy = eiy * sIi, uiz = eiz * sIi;
    const double ujx = ejx * sIj, ujy = ejy * sIj, ujz = ejz * sIj;
    double Wi = 0.0, gi = 0.0, Wj = 0.0, gj = 0.0;
    if (etaMagi < hp.extent) {
      const int i0 = tableIndex(etaMagi, hp.tableN1, hp.tableXstep);
      Wi = tableEval(tw, i0, etaMagi);
      gi = tableEval(tg, i0, etaMagi);
    }
    if (etaMagj < hp.extent) {
      const int i0 = tableIndex(etaMagj, hp.tableN1, hp.tableXstep);
      Wj = tableEval(tw, i0, etaMagj);
      gj = tableEval(tg, i0, etaMagj);
    }
    const double WSPHi = fabs(gi);
    Wi *= Hdeti; Wj *= Hdetj;
    const double gWi = Hdeti * gi, gWj = Hdetj * gj;
    double gwix, gwiy, gwiz, gwjx, gwjy, gwjz;
    if (TENSOR) {   // gW H eta^
      double hx, hy, hz;
      symDot(Hi, uix, uiy, uiz, hx, hy, hz);
      gwix = gWi * hx; gwiy = gWi * hy; gwiz = gWi * hz;
      symDot(Hj, ujx, ujy, ujz, hx, hy, hz);
      gwjx = gWj * hx; gwjy = gWj * hy; gwjz = gWj * hz;
    } else {
      const double gHi = gWi * ai, gHj = gWj * aj;
      gwix = gHi * uix; gwiy = gHi * uiy; gwiz = gHi * uiz;
      gwjx = gHj * ujx; gwjy = gHj * ujy; gwjz = gHj * ujz;
    }

    if (lj == li) {
      a.rhoSum += mj * Wi;
      a.norm += mi / rhoi * Wi;
    }
    const double vijx = vxi - vxj, vijy = vyi - vyj, vijz = vzi - vzj;
    // Monaghan-Gingold Q; the limited form first corrects the two velocities
    // along the pair with the Q's DvDx (LimitedMonaghanGingoldViscosity.cc:171-200)
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
        const double z = (etaij - hp.etaCrit) / hp.etaFold;
        phi *= exp(-(z * z));
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
    const double QPiij = ei / rhoi, QPiji = ej / rhoj;
    const double Qi = rhoi * ei;
    const double qai = 0.5 * QPiij, qaj = 0.5 * QPiji;
    const double Qaix = qai * gwix, Qaiy = qai * gwiy, Qaiz = qai * gwiz;
    const double Qajx = qaj * gwjx, Qajy = qaj * gwjy, Qajz = qaj * gwjz;
    const double workQi = vijx * Qaix + vijy * Qaiy + vijz * Qaiz;
    a.maxQ = fmax(a.maxQ, Qi);
    a.effQ += mj * Qi * Wi / rhoj;
    double Peffi = Pi, Peffj = Pj;
    if (hp.epsTensile != 0.0) {
      const double ri = Wi / (Hdeti * hp.WnPerh), rj = Wj / (Hdetj * hp.WnPerh);
      Peffi += hp.epsTensile * (ri * ri * ri * ri) * (Pi < 0.0 ? -Pi : 0.0);
      Peffj += hp.epsTensile * (rj * rj * rj * rj) * (Pj < 0.0 ? -Pj : 0.0);
    }
    const double Prhoi = safeOmegai * Peffi / (rhoi * rhoi);
    const double Prhoj = safeOmegaj * Peffj / (rhoj * rhoj);
    const double ddx = Prhoi * gwix + Prhoj * gwjx + Qaix + Qajx;
    const double ddy = Prhoi * gwiy + Prhoj * gwjy + Qaiy + Qajy;
    const double ddz = Prhoi * gwiz + Prhoj * gwjz + Qaiz + Qajz;
    a.dvx -= mj * ddx;
    a.dvy -= mj * ddy;
    a.dvz -= mj * ddz;
    if (COMPAT) {
      pacc[3 * k] = -mj * ddx;
      pacc[3 * k + 1] = -mj * ddy;
      pacc[3 * k + 2] = -mj * ddz;
    }
    a.deps += mj * (Prhoi * (vijx * gwix + vijy * gwiy + vijz * gwiz) + workQi);
    const double mvx = mj * vijx, mvy = mj * vijy, mvz = mj * vijz;
    a.D[0] -= mvx * gwix; a.D[1] -= mvx * gwiy; a.D[2] -= mvx * gwiz;
    a.D[3] -= mvy * gwix; a.D[4] -= mvy * gwiy; a.D[5] -= mvy * gwiz;
    a.D[6] -= mvz * gwix; a.D[7] -= mvz * gwiy; a.D[8] -= mvz * gwiz;
    if (XSPH) {
      const double wx = 0.5 * (mi / rhoi * Wi + mj / rhoj * Wj);
      a.xw += wx;
      a.xdx -= wx * vijx; a.xdy -= wx * vijy; a.xdz -= wx * vijz;
    }
    const double gr = mj * (rhoj - rhoi);
    a.gx += gr * gwix; a.gy += gr * gwiy; a.gz += gr * gwiz;
    const double mrx = mj * rx, mry = mj * ry, mrz = mj * rz;
    a.M[0] -= mrx * gwix; a.M[1] -= mrx * gwiy; a.M[2] -= mrx * gwiz;
    a.M[3] -= mry * gwix; a.M[4] -= mry * gwiy; a.M[5] -= mry * gwiz;
    a.M[6] -= mrz * gwix; a.M[7] -= mrz * gwiy; a.M[8] -= mrz * gwiz;
    // SPHSmoothingScale zeroth / first moments
    const double fw = (lj != li) ? mj * rhoi / (mi * rhoj) : 1.0;
    a.m0 += fw * WSPHi;
    const double fwW = fw * WSPHi;
    a.m1x -= fwW * eix; a.m1y -= fwW * eiy; a.m1z -= fwW * eiz;
    if (TENSOR) {   // ASPHClassicSmoothingScale second moment: WSPH^2 r r / |r|^5
      const double rm = sqrt(rx * rx + ry * ry + rz * rz);
      const double f5 = 1.0 / fmax(kTiny30, rm * rm * rm * rm * rm);
      const double w2 = fwW * WSPHi;
      a.m2[0] += w2 * (rx * rx * f5); a.m2[1] += w2 * (rx * ry * f5); a.m2[2] += w2 * (rx * rz * f5);
      a.m2[3] += w2 * (ry * ry * f5); a.m2[4] += w2 * (ry * rz * f5); a.m2[5] += w2 * (rz * rz * f5);
    }
  }
  if (TENSOR) finalizeNodeASPH(F, i, li, a, Hi, mi, rhoi, vxi, vyi, vzi, cnt, hp, t.herm);
  else finalizeNode(F, i, li, a, mi, rhoi, vxi, vyi, vzi, ai, cnt, hp, t.herm);
}

//------------------------------------------------------------------------------
// GenericHydro::dt (src/Physics/GenericHydro.cc:113-381): node limits and the
// pairwise velocity-difference limit, min-reduced.  The reason code travels
// with the value (value, reason) through both reduction stages.
//------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) dtKernel(Fields F, const int* __restrict__ list, long n, Grid g,
                                                NeighborLists nl, HydroParams hp, double maxNperh,
                                                double* __restrict__ part) {
  __shared__ double sv[128];
  __shared__ int sr[128];
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const double tiny = DBL_EPSILON;
  double best = DBL_MAX;
  int reason = -1;
  if (i < n && !isGhost(hp, i)) {
    int hc[3];
    unpackCell(nl.cell[i], hc);
    const NodeListParams L = hp.lists[list[i]];
    // max eigenvalue of H: h^-1 when isotropic, the stored extent for tensor H
    const double* __restrict__ HX = F.f[hp.asph ? F_HLMAX : F_HINV];
    const double ai = HX[i];
    const double nodeScalei = 1.0 / ai / L.nPerh;
    const double vxi = F.f[F_VX][i], vyi = F.f[F_VY][i], vzi = F.f[F_VZ][i];
    const double rhoi = F.f[F_RHO][i];
    const double csDt = nodeScalei / (F.f[F_CS][i] + tiny);
    if (csDt < best) { best = csDt; reason = 0; }
    const double csq = sqrt(F.f[F_MAXQ][i] / rhoi);
    const double csqDt = nodeScalei / (csq + tiny);
    if (csqDt < best) { best = csqDt; reason = 1; }
    const double divv = F.f[F_DVDX_XX][i] + F.f[F_DVDX_YY][i] + F.f[F_DVDX_ZZ][i];
    const double divvDt = 1.0 / (fabs(divv) + tiny);
    if (divvDt < best) { best = divvDt; reason = 2; }
    const double vmag = sqrt(vxi * vxi + vyi * vyi + vzi * vzi);
    const double ax = F.f[F_DVDT_X][i], ay = F.f[F_DVDT_Y][i], az = F.f[F_DVDT_Z][i];
    const double amag = sqrt(ax * ax + ay * ay + az * az);
    const double dtAcc = 0.1 * fmax(nodeScalei / (vmag + tiny), vmag / (amag + tiny));
    if (dtAcc < best) { best = dtAcc; reason = 3; }
    if (hp.useVelMagDt) {
      const double velDt = nodeScalei / (vmag + 1.0e-10);
      if (velDt < best) { best = velDt; reason = 4; }
    }
    const double nsi = 1.0 / ai / maxNperh;
    const int cnt = nl.count[i];
    for (int q = 0; q < cnt; ++q) {
      const long long k = nbSlot(i, q, nl.cap);
      const uint32_t ent = nl.nbr[k];
      const int j = (int)(ent & kIndexMask), code = imageCode(g, hc, (int)(ent >> kIndexBits));
      double vxj = F.f[F_VX][j], vyj = F.f[F_VY][j], vzj = F.f[F_VZ][j];
      imageVec(g, code, vxj, vyj, vzj);
      const double nsj = 1.0 / HX[j] / maxNperh;
      const double dvx = vxi - vxj, dvy = vyi - vyj, dvz = vzi - vzj;
      const double vm = sqrt(dvx * dvx + dvy * dvy + dvz * dvz);
      const double dtv = fmin(nsi, nsj) * (1.0 / fmax(tiny, vm));
      if (dtv < best) { best = dtv; reason = 5; }
    }
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
__global__ void dtFinalKernel(const double* __restrict__ part, int nb, double* __restrict__ out) {
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
// SpecificThermalEnergyPolicy::update (src/Hydro/SpecificThermalEnergyPolicy.cc:110-173),
// gathered: node i takes its own share w_i du_ij of every pair, with the pair
// acceleration stored per ordered slot by the pair loop.
//------------------------------------------------------------------------------
template <bool F32PACC>
__global__ void __launch_bounds__(128) energyKernel(Fields F, long n, Grid g, NeighborLists nl,
                                                    const double* __restrict__ pacc, const float* __restrict__ pacc32,
                                                    double dt) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int hc[3];
  unpackCell(nl.cell[i], hc);
  const double hdt = 0.5 * dt;
  const double* __restrict__ VX = F.f[F_VX];
  const double* __restrict__ VY = F.f[F_VY];
  const double* __restrict__ VZ = F.f[F_VZ];
  const double* __restrict__ AX = F.f[F_DVDT_X];
  const double* __restrict__ AY = F.f[F_DVDT_Y];
  const double* __restrict__ AZ = F.f[F_DVDT_Z];
  const double* __restrict__ D0 = F.f[F_DEPSDT];
  const double vxi = VX[i] + AX[i] * hdt, vyi = VY[i] + AY[i] * hdt, vzi = VZ[i] + AZ[i] * hdt;
  const double d0i = D0[i];
  double sum = 0.0;
  const int cnt = nl.count[i];
  for (int q = 0; q < cnt; ++q) {
    const long long k = nbSlot(i, q, nl.cap);
    const uint32_t ent = nl.nbr[k];
    const int j = (int)(ent & kIndexMask), code = imageCode(g, hc, (int)(ent >> kIndexBits));
    double vxj = VX[j], vyj = VY[j], vzj = VZ[j], axj = AX[j], ayj = AY[j], azj = AZ[j];
    imageVec(g, code, vxj, vyj, vzj);
    imageVec(g, code, axj, ayj, azj);
    const double wx = vxj + axj * hdt - vxi, wy = vyj + ayj * hdt - vyi, wz = vzj + azj * hdt - vzi;
    double px, py, pz;
    if (F32PACC) { px = pacc32[3 * k]; py = pacc32[3 * k + 1]; pz = pacc32[3 * k + 2]; }
    else { px = pacc[3 * k]; py = pacc[3 * k + 1]; pz = pacc[3 * k + 2]; }
    const double du = wx * px + wy * py + wz * pz;
    const double sg = du < 0.0 ? -1.0 : 1.0;
    const double weighti = fmax(DBL_EPSILON, d0i * sg);
    const double weightj = fmax(DBL_EPSILON, D0[j] * sg);
    const double wi = weighti / (weighti + weightj);
    sum += wi * du;
  }
  F.f[F_DEPS_COMPAT][i] = sum;
  F.f[F_EPS][i] += sum * dt;
}

//------------------------------------------------------------------------------
// State updates (State::update with IncrementState / IncrementBoundedState /
// ReplaceBoundedState, PressurePolicy, SoundSpeedPolicy) and GammaLawGas.
//------------------------------------------------------------------------------
__device__ __forceinline__ void eosNode(Fields& F, long i, const NodeListParams& L) {
  const double rho = F.f[F_RHO][i], eps = F.f[F_EPS][i];
  double p = (L.gamma - 1.0) * rho * eps;
  p = p < L.minP ? L.minP : (p > L.maxP ? L.maxP : p);
  F.f[F_P][i] = p;
  F.f[F_CS][i] = sqrt(fmax(0.0, L.gamma * (L.gamma - 1.0) * eps));
}

__global__ void restoreState0Kernel(Fields F, long n, int tensor, int crk) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  F.f[F_X][i] = F.f[F_X0][i]; F.f[F_Y][i] = F.f[F_Y0][i]; F.f[F_Z][i] = F.f[F_Z0][i];
  F.f[F_VX][i] = F.f[F_VX0][i]; F.f[F_VY][i] = F.f[F_VY0][i]; F.f[F_VZ][i] = F.f[F_VZ0][i];
  F.f[F_RHO][i] = F.f[F_RHO0][i]; F.f[F_EPS][i] = F.f[F_EPS0][i]; F.f[F_HINV][i] = F.f[F_HINV0][i];
  if (tensor)
#pragma unroll
    for (int k = 0; k < 6; ++k) F.f[F_HT_XX + k][i] = F.f[F_HT0_XX + k][i];
  if (crk) F.f[F_VOL][i] = F.f[F_VOL0][i];
}

// Extent of tensor H (ASPH): smallest eigenvalue -> F_HINV (cell size,
// neighbour pre-filter), largest -> F_HLMAX (dt node scale).
__device__ __forceinline__ void storeExtent(Fields& F, long i, const Sym& h) {
  double lmin, lmax;
  symExtent(h, lmin, lmax);
  F.f[F_HINV][i] = lmin;
  F.f[F_HLMAX][i] = lmax;
}
// Mixed mode: the same extents from an FP32 Jacobi decomposition (GB300's
// FP64 transcendental sequences would dominate the update).  The smallest
// eigenvalue only has to bound |H r| / |r| from below (neighbour pre-filter),
// so it is lowered by a margin far above the FP32 eigenvalue error; the
// largest feeds the FP32 dt vote.
__device__ __forceinline__ void storeExtent32(Fields& F, long i, const Sym& h) {
  const SymT<float> hf{(float)h.xx, (float)h.xy, (float)h.xz, (float)h.yy, (float)h.yz, (float)h.zz};
  float val[3], V[3][3];
  symEigen(hf, val, V);
  F.f[F_HINV][i] = (double)fminf(val[0], fminf(val[1], val[2])) * (1.0 - 1.0e-5);
  F.f[F_HLMAX][i] = (double)fmaxf(val[0], fmaxf(val[1], val[2]));
}
// ASPH radialOnly: the radius of every node at the start of the step
// (SmoothingScaleBase::preStepInitialize).
__global__ void radius0Kernel(Fields F, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = F.f[F_X][i], y = F.f[F_Y][i], z = F.f[F_Z][i];
  F.f[F_RAD0][i] = sqrt(x * x + y * y + z * z);
}
// ASPHSmoothingScale::finalize (src/SmoothingScale/ASPHSmoothingScale.cc:157-380)
// in its fixShape and radialOnly forms, gathered: the zeroth moment of the
// end-of-step state over the step's neighbour lists (fweight_ij WSPH(|H_i r_ij|)),
// the IdealH size ratio, H scaled (fixShape) or reshaped radially about the
// origin (radialOnly), then the eigenvalue limits; with IntegrateH or FixedH
// only the limits.  FP64 in both precision modes; in the mixed mode the FP32
// extents and mirrors of the new H are written as the update writes them.
__global__ void __launch_bounds__(128) asphEndKernel(Fields F, Fields32 P, const int* __restrict__ list, long n,
                                                    Grid g, NeighborLists nl, TableDev t, HydroParams hp) {
  extern __shared__ double smem[];   // dW/deta coefficients
  const int ntab = 3 * (hp.tableN1 + 1);
  for (int k = threadIdx.x; k < ntab; k += blockDim.x) smem[k] = t.g[k];
  __syncthreads();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int li = list[i];
  const NodeListParams L = hp.lists[li];
  const Sym Hi = loadSym(F, F_HT_XX, i);
  Sym Hn;
  if (hp.hUpdate != 0) {
    Hn = limitASPH(Hi, L.hminInv, L.hmaxInv, L.hminratio);
  } else {
    int hc[3];
    unpackCell(nl.cell[i], hc);
    const double* __restrict__ X = F.f[F_X];
    const double* __restrict__ Y = F.f[F_Y];
    const double* __restrict__ Z = F.f[F_Z];
    const double xi = X[i], yi = Y[i], zi = Z[i];
    const double mi = F.f[F_MASS][i], rhoi = F.f[F_RHO][i];
    const bool multi = hp.numLists > 1;
    double m0 = 0.0;
    const int cnt = nl.count[i];
    for (int q = 0; q < cnt; ++q) {
      const uint32_t ent = nl.nbr[nbSlot(i, q, nl.cap)];
      const int j = (int)(ent & kIndexMask), code = imageCode(g, hc, (int)(ent >> kIndexBits));
      double xj = X[j], yj = Y[j], zj = Z[j];
      imagePos(g, code, xj, yj, zj);
      double ex, ey, ez;
      symDot(Hi, xi - xj, yi - yj, zi - zj, ex, ey, ez);
      const double eta = sqrt(ex * ex + ey * ey + ez * ez);
      if (eta < hp.extent) {
        const double wsph = fabs(tableEval(smem, tableIndex(eta, hp.tableN1, hp.tableXstep), eta));
        const double fw = (multi && list[j] != li) ? F.f[F_MASS][j] * rhoi / (mi * F.f[F_RHO][j]) : 1.0;
        m0 += fw * wsph;
      }
    }
    const double mz = rootnu3T(fmax(0.0, m0));
    F.f[F_M0][i] = mz;
    const bool isolated = fabs(mz) <= 1.0e-15 * fmax(1.0, fabs(mz));
    const double cur = isolated ? 0.5 * L.nPerh : fmax(0.0, hermiteLookup(t.herm, hp, mz));
    const double s = fmin(4.0, fmax(0.25, L.nPerh / (cur + 1.0e-30)));
    const double aa = s < 1.0 ? 0.4 * (1.0 + s * s) : 0.4 * (1.0 + 1.0 / (s * s * s));
    const double f = 1.0 - aa + aa * s;
    const Sym Hid = hp.fixShape ? symDiv(Hi, f) : radialEvolution(Hi, xi, yi, zi, f, F.f[F_RAD0][i]);
    Hn = limitASPH(Hid, L.hminInv, L.hmaxInv, L.hminratio);
    storeSym(F, F_HIDEALT_XX, i, Hn);
  }
  storeSym(F, F_HT_XX, i, Hn);
  if (P.posh) {
    storeExtent32(F, i, Hn);
    P.posh[i].w = (float)F.f[F_HINV][i];
    writeTensorMirror(F, P, i);
  } else {
    storeExtent(F, i, Hn);
  }
}

__global__ void tensorExtentKernel(Fields F, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  storeExtent(F, i, loadSym(F, F_HT_XX, i));
}

// P != nullptr (mixed mode): the FP32 mirrors of the new state are written
// here as well (the prepare pass folded into the update).
// tensor (ASPH): H is the symmetric tensor, bounded on its eigenvalues
// (IncrementBoundedState / ReplaceBoundedState with SymTensor min/max).
// hUpdate: HEvolutionType -- 0 IdealH (the full update replaces H by Hideal),
// 1 IntegrateH (both updates increment H by DHDt), 2 FixedH (H never changes).
// asphEnd (ASPHSmoothingScale): both updates integrate H with
// IncrementASPHHtensor (fixShape / radialOnly forms) unless FixedH.
template <bool TENSOR>
__global__ void updateKernel(Fields F, const int* __restrict__ list, long n, const NodeListParams* __restrict__ lists,
                             double mult, int mid, int gravity, int epsIncrement, int hUpdate, int totalEnergy,
                             int crk, Fields32 P, Grid g, int asphEnd, int fixShape, int radialOnly) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const NodeListParams L = lists[list[i]];
  // the position before this update (the radial direction of radialOnly:
  // State::update applies the "H" policy before the "position" one)
  const double xOld = F.f[F_X][i], yOld = F.f[F_Y][i], zOld = F.f[F_Z][i];
  // the half-step update first takes the beginning-of-step copy (state0)
  if (mid) {
    F.f[F_X0][i] = F.f[F_X][i]; F.f[F_Y0][i] = F.f[F_Y][i]; F.f[F_Z0][i] = F.f[F_Z][i];
    F.f[F_VX0][i] = F.f[F_VX][i]; F.f[F_VY0][i] = F.f[F_VY][i]; F.f[F_VZ0][i] = F.f[F_VZ][i];
    F.f[F_RHO0][i] = F.f[F_RHO][i]; F.f[F_EPS0][i] = F.f[F_EPS][i]; F.f[F_HINV0][i] = F.f[F_HINV][i];
    if (TENSOR)
#pragma unroll
      for (int k = 0; k < 6; ++k) F.f[F_HT0_XX + k][i] = F.f[F_HT_XX + k][i];
    if (crk) F.f[F_VOL0][i] = F.f[F_VOL][i];
  }
  if (epsIncrement) {
    if (totalEnergy) {
      // SpecificFromTotalThermalEnergyPolicy::update: eps from the total
      // energy m (v^2/2 + eps) advanced by DEDt, with the hydro acceleration
      // for the new kinetic part (it fires before the velocity update)
      const double mi = F.f[F_MASS][i];
      const double v0x = F.f[F_VX][i], v0y = F.f[F_VY][i], v0z = F.f[F_VZ][i];
      const double v1x = v0x + mult * F.f[F_DVDT_X][i], v1y = v0y + mult * F.f[F_DVDT_Y][i],
                   v1z = v0z + mult * F.f[F_DVDT_Z][i];
      const double E0 = mi * (0.5 * (v0x * v0x + v0y * v0y + v0z * v0z) + F.f[F_EPS][i]);
      const double E1 = E0 + mult * F.f[F_DEPSDT][i];
      F.f[F_EPS][i] = E1 / mi - 0.5 * (v1x * v1x + v1y * v1y + v1z * v1z);
    } else {
      F.f[F_EPS][i] += mult * F.f[F_DEPSDT][i];
    }
  }
  const double x = F.f[F_X][i] + mult * F.f[F_DXDT_X][i];
  const double y = F.f[F_Y][i] + mult * F.f[F_DXDT_Y][i];
  const double z = F.f[F_Z][i] + mult * F.f[F_DXDT_Z][i];
  F.f[F_X][i] = x;
  F.f[F_Y][i] = y;
  F.f[F_Z][i] = z;
  // velocity: "delta velocity hydro" sorts before "delta velocity" (gravity)
  double vx = F.f[F_VX][i] + mult * F.f[F_DVDT_X][i];
  double vy = F.f[F_VY][i] + mult * F.f[F_DVDT_Y][i];
  double vz = F.f[F_VZ][i] + mult * F.f[F_DVDT_Z][i];
  if (gravity) {
    vx += mult * F.f[F_GRAV_X][i];
    vy += mult * F.f[F_GRAV_Y][i];
    vz += mult * F.f[F_GRAV_Z][i];
  }
  F.f[F_VX][i] = vx;
  F.f[F_VY][i] = vy;
  F.f[F_VZ][i] = vz;
  const double rho = fmin(L.rhoMax, fmax(L.rhoMin, F.f[F_RHO][i] + mult * F.f[F_DRHODT][i]));
  F.f[F_RHO][i] = rho;
  const double hminInv = L.hminInv, hmaxInv = L.hmaxInv;
  double h;
  const bool increment = mid || hUpdate == 1;
  if (hUpdate == 2) {
    h = F.f[F_HINV][i];
  } else if (TENSOR && asphEnd) {
    const Sym t = incrementASPHHtensor(loadSym(F, F_HT_XX, i), loadSym(F, F_DHDTT_XX, i), mult, xOld, yOld, zOld,
                                       fixShape != 0, radialOnly != 0, hminInv, hmaxInv, L.hminratio);
    storeSym(F, F_HT_XX, i, t);
    if (P.posh) storeExtent32(F, i, t);
    else storeExtent(F, i, t);
    h = F.f[F_HINV][i];
  } else if (TENSOR) {
    Sym t;
    if (increment) {
      t = loadSym(F, F_HT_XX, i);
      const Sym d = loadSym(F, F_DHDTT_XX, i);
      t = Sym{t.xx + mult * d.xx, t.xy + mult * d.xy, t.xz + mult * d.xz, t.yy + mult * d.yy, t.yz + mult * d.yz,
              t.zz + mult * d.zz};
    } else {
      t = loadSym(F, F_HIDEALT_XX, i);
    }
    t = symBound(t, hmaxInv, hminInv);
    storeSym(F, F_HT_XX, i, t);
    if (P.posh) storeExtent32(F, i, t);
    else storeExtent(F, i, t);
    h = F.f[F_HINV][i];
  } else {
    h = increment ? F.f[F_HINV][i] + mult * F.f[F_DHDT][i] : F.f[F_HIDEAL][i];
    if (h < hmaxInv) h = hmaxInv;
    if (h > hminInv) h = hminInv;
    F.f[F_HINV][i] = h;
  }
  if (crk) {
    // ContinuityVolumePolicy::update (src/RK/ContinuityVolumePolicy.cc:40-75):
    // it depends on the mass density, so it sees the updated rho and H
    const double mi = F.f[F_MASS][i];
    const double volMin = 0.5 * mi * safeInvVarD(rho);
    const double volMax = 4.0 * 3.141592653589793 / (3.0 * ((h * h) * h));
    const double dVdt = -mi * safeInvVarD(rho * rho) * F.f[F_DRHODT][i];
    F.f[F_VOL][i] = fmax(volMin, fmin(volMax, F.f[F_VOL][i] + mult * dVdt));
  }
  if (P.posh) {
    // Mixed mode.  The sound speed feeds only FP32 sweeps (Q, dt vote), so it
    // is evaluated in FP32; the conversions between double and float take
    // the integer pipe (convert.cuh) and the cell origins an integer-built
    // index: GB300's FP64 pipe, which runs FP64 arithmetic and the
    // conversion instructions at ~1/64 of the FP32 rate, bounds this kernel.
    const double eps = F.f[F_EPS][i];
    double p = L.gm1 * rho * eps;
    p = p < L.minP ? L.minP : (p > L.maxP ? L.maxP : p);
    F.f[F_P][i] = p;
    const float cs = sqrtf(fmaxf(0.0f, toFloatRN(L.ggm1 * eps)));
    F.f[F_CS][i] = toDouble(cs);
    int c[3];
    unpackCell(P.cell[i], c);
    const double ox = g.lo[0] + smallIntToDouble(c[0]) * g.cell[0];
    const double oy = g.lo[1] + smallIntToDouble(c[1]) * g.cell[1];
    const double oz = g.lo[2] + smallIntToDouble(c[2]) * g.cell[2];
    P.posh[i] = make_float4(toFloatRN(x - ox), toFloatRN(y - oy), toFloatRN(z - oz), toFloatRN(h));
    P.velm[i] = make_float4(toFloatRN(vx), toFloatRN(vy), toFloatRN(vz), toFloatRN(F.f[F_MASS][i]));
    const float om = toFloatRN(F.f[F_OMEGA][i]);
    P.thermo[i] = make_float4(toFloatRN(rho), toFloatRN(p), cs, om / (om * om + 1.0e-30f));
    if (TENSOR) writeTensorMirror(F, P, i);
    if (crk && P.vol) P.vol[i] = toFloatRN(F.f[F_VOL][i]);
  } else {
    eosNode(F, i, L);
  }
}

__global__ void eosKernel(Fields F, const int* __restrict__ list, long n, const NodeListParams* __restrict__ lists) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  eosNode(F, i, lists[list[i]]);
}

// Boundary::setAllViolationNodes + enforceBoundary (PlanarBoundary.cc:153-190,
// ReflectingBoundary.cc:465-473): nodes strictly outside a plane are mapped
// back; reflecting walls also mirror the velocity.
__device__ __forceinline__ bool fuzzyZero(double x) { return fabs(x) <= 1.0e-15 * fmax(1.0, fabs(x)); }
// A signed integer with the order of the double x (for non-NaN x; -0 sorts
// just below +0, which only sends a node at a wall to the exact test).
__device__ __forceinline__ long long orderKey(double x) {
  const long long b = __double_as_longlong(x);
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
// tensor: the H of a node mapped back through a reflecting wall is reflected
// too (PlanarBoundary::updateViolationNodes -> enforceBoundary(Hfield),
// (R H R).Symmetric()).
__global__ void enforceKernel(Fields F, long n, Grid g, int tensor) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  auto reflectH = [&](int a) {
    if (!tensor) return;
    if (a == 0) { F.f[F_HT_XY][i] = -F.f[F_HT_XY][i]; F.f[F_HT_XZ][i] = -F.f[F_HT_XZ][i]; }
    else if (a == 1) { F.f[F_HT_XY][i] = -F.f[F_HT_XY][i]; F.f[F_HT_YZ][i] = -F.f[F_HT_YZ][i]; }
    else { F.f[F_HT_XZ][i] = -F.f[F_HT_XZ][i]; F.f[F_HT_YZ][i] = -F.f[F_HT_YZ][i]; }
  };
  double* P[3] = {F.f[F_X], F.f[F_Y], F.f[F_Z]};
  double* V[3] = {F.f[F_VX], F.f[F_VY], F.f[F_VZ]};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double lo = g.wallLo[a], hi = g.wallHi[a];
    double p = P[a][i];
    // Integer pre-test on order-preserving keys of the bit patterns: a node
    // strictly inside (lo, hi) needs nothing, and the FP64 tests below (the
    // FP64 pipe is narrow) run only for the few on or beyond a wall.
    if (orderKey(p) > orderKey(lo) && orderKey(p) < orderKey(hi)) continue;
    const double sdLo = p - lo, sdHi = hi - p;
    if (g.kindLo[a] == AXIS_PERIODIC) {
      if (sdLo < 0.0 && !fuzzyZero(sdLo)) p = imageCoord(p, 2, AXIS_PERIODIC, AXIS_PERIODIC, lo, hi);
      else if (sdHi < 0.0 && !fuzzyZero(sdHi)) p = imageCoord(p, 1, AXIS_PERIODIC, AXIS_PERIODIC, lo, hi);
      P[a][i] = p;
    } else {
      if (g.kindLo[a] == AXIS_REFLECT && sdLo < 0.0 && !fuzzyZero(sdLo)) {
        p = imageCoord(p, 1, AXIS_REFLECT, g.kindHi[a], lo, hi);
        P[a][i] = p;
        V[a][i] = -V[a][i];
        reflectH(a);
      }
      const double sdHi2 = hi - p;
      if (g.kindHi[a] == AXIS_REFLECT && sdHi2 < 0.0 && !fuzzyZero(sdHi2)) {
        p = imageCoord(p, 2, g.kindLo[a], AXIS_REFLECT, lo, hi);
        P[a][i] = p;
        V[a][i] = -V[a][i];
        reflectH(a);
      }
    }
  }
}

// SpheralConservation totals (SpheralConservation.py:54-150) in FP64:
// mass, momentum, kinetic, thermal, gravitational (1/2 m phi).
__global__ void conservationKernel(Fields F, long n, int gravity, double* __restrict__ part) {
  __shared__ double sm[32];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double m = F.f[F_MASS][i], vx = F.f[F_VX][i], vy = F.f[F_VY][i], vz = F.f[F_VZ][i];
    acc[0] += m;
    acc[1] += m * vx; acc[2] += m * vy; acc[3] += m * vz;
    acc[4] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
    acc[5] += m * F.f[F_EPS][i];
    if (gravity) acc[6] += 0.5 * m * F.f[F_POT][i];
  }
  for (int k = 0; k < 7; ++k) {
    const double r = blockSum(acc[k], sm);
    if (threadIdx.x == 0) part[blockIdx.x * 7 + k] = r;
  }
}
__global__ void conservationFinalKernel(const double* __restrict__ part, int nb, double* __restrict__ out) {
  __shared__ double sm[32];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int k = 0; k < 7; ++k) acc[k] += part[b * 7 + k];
  for (int k = 0; k < 7; ++k) {
    const double r = blockSum(acc[k], sm);
    if (threadIdx.x == 0) out[k] = r;
  }
  if (threadIdx.x == 0) out[7] = out[4] + out[5] + out[6];
}

__global__ void checkStateKernel(Fields F, long n, int* __restrict__ flag) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double m = F.f[F_MASS][i], rho = F.f[F_RHO][i], a = F.f[F_HINV][i], eps = F.f[F_EPS][i];
  const double x = F.f[F_X][i], y = F.f[F_Y][i], z = F.f[F_Z][i];
  const double vx = F.f[F_VX][i], vy = F.f[F_VY][i], vz = F.f[F_VZ][i];
  const bool bad = !(m > 0.0) || !(rho > 0.0) || !(a > 0.0) || !isfinite(eps) || !isfinite(x) || !isfinite(y) ||
                   !isfinite(z) || !isfinite(vx) || !isfinite(vy) || !isfinite(vz) || !isfinite(rho) || !isfinite(a);
  if (bad) atomicExch(flag, 1);
}

// Caller-order transfers: stage[orig[k] * stride + c] <-> F[first + c][k].
__global__ void gatherOutKernel(Fields F, const int* __restrict__ orig, double* __restrict__ stage, int first,
                                int ncomp, int stride, long n) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long o = (long)orig[k] * stride;
  for (int c = 0; c < ncomp; ++c) stage[o + c] = F.f[first + c][k];
}
// Domain-decomposition exchange: rows of `w` values of the fields ids[0..w)
// for caller indices idx (get), or for the halo nodes, caller indices
// nOwn..nOwn+count-1 in order (put).  inv: internal index of each caller index.
__global__ void exchangeGetKernel(Fields F, const int* __restrict__ inv, const int* __restrict__ idx, long count,
                                  ExchangeFields ef, double* __restrict__ out) {
  const long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r >= count) return;
  const long k = inv[idx[r]];
  for (int c = 0; c < ef.w; ++c) out[r * ef.w + c] = F.f[ef.ids[c]][k];
}
__global__ void exchangePutKernel(Fields F, Fields32 P, const int* __restrict__ inv, long nOwn, long count,
                                  ExchangeFields ef, const double* __restrict__ in) {
  const long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r >= count) return;
  const long k = inv[nOwn + r];
  for (int c = 0; c < ef.w; ++c) F.f[ef.ids[c]][k] = in[r * ef.w + c];
  // the FP32 mirror entries the sweeps read next, written as their own
  // kernels write them for owned nodes
  if (P.thermo) {
    if (ef.mirror == 1) P.thermo[k].x = (float)F.f[F_RHO][k];
    if (ef.mirror == 2) {
      const float om = (float)F.f[F_OMEGA][k];
      P.thermo[k].w = om / (om * om + 1.0e-30f);
    }
  }
}

__global__ void scatterInKernel(Fields F, const int* __restrict__ orig, const double* __restrict__ stage, int first,
                                int ncomp, int stride, long n) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long o = (long)orig[k] * stride;
  for (int c = 0; c < ncomp; ++c) F.f[first + c][k] = stage[o + c];
}
// Caller-order transfers that address a pinned host array in place: the
// threads walk the flat host array (n records of `stride` doubles), so the
// host link sees contiguous reads (writes), and the permutation to the
// internal order (inv: caller index -> internal index) lands on the device
// side.  Components past ncomp are skipped on the way in; on the way out an
// isotropic H (isoH) is written as the SymTensor (a, 0, 0, a, 0, a).
__global__ void inverseOrderKernel(const int* __restrict__ orig, int* __restrict__ inv, long n) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k < n) inv[orig[k]] = (int)k;
}
__global__ void scatterInHostKernel(Fields F, const int* __restrict__ inv, const double* __restrict__ src, int first,
                                    int ncomp, int stride, long n) {
  const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (e >= n * stride) return;
  const long m = e / stride;
  const int c = (int)(e - m * stride);
  if (c < ncomp) F.f[first + c][inv[m]] = src[e];
}
__global__ void gatherOutHostKernel(Fields F, const int* __restrict__ inv, double* __restrict__ dst, int first,
                                    int ncomp, int stride, int isoH, long n) {
  const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (e >= n * stride) return;
  const long m = e / stride;
  const int c = (int)(e - m * stride);
  double v;
  if (isoH) v = (c == 0 || c == 3 || c == 5) ? F.f[first][inv[m]] : 0.0;
  else v = c < ncomp ? F.f[first + c][inv[m]] : 0.0;
  dst[e] = v;
}
// H as SymTensor (xx, xy, xz, yy, yz, zz) <-> isotropic hinv.
__global__ void gatherOutHKernel(Fields F, const int* __restrict__ orig, double* __restrict__ stage, int field,
                                 long n) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  double* o = stage + (long)orig[k] * 6;
  const double a = F.f[field][k];
  o[0] = a; o[1] = 0.0; o[2] = 0.0; o[3] = a; o[4] = 0.0; o[5] = a;
}
__global__ void countsOutKernel(const int* __restrict__ counts, const int* __restrict__ orig,
                                double* __restrict__ stage, long n) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  stage[orig[k]] = (double)counts[k];
}

inline unsigned gridFor(long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

//==============================================================================
// Launchers
//==============================================================================
void launchBounds(const Fields& F, long n, bool tensor, double* dScratch, int nScratch, double* dOut, cudaStream_t s,
                  LaunchCounter* lc) {
  int nb = (int)std::min<long>((n + 255) / 256, nScratch / kBoundsVals);
  if (nb < 1) nb = 1;
  boundsKernel<<<nb, 256, 0, s>>>(F, n, tensor ? 1 : 0, dScratch);
  boundsFinalKernel<<<1, 256, 0, s>>>(dScratch, nb, dOut);
  lc->add(2);
}
void launchCellKeys(const Fields& F, long n, Grid g, uint32_t* keys, int* vals, uint32_t* cellc, cudaStream_t s,
                    LaunchCounter* lc) {
  cellKeyKernel<<<gridFor(n, 256), 256, 0, s>>>(F, n, g, keys, vals, cellc);
  lc->add(1);
}
// ArtificialViscosityHandle::postStateUpdate: the Q's DvDx = the hydro DvDx.
__global__ void copyQGradientKernel(Fields F, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int k = 0; k < 9; ++k) F.f[F_DVDXQ_XX + k][i] = F.f[F_DVDX_XX + k][i];
}
// FP32 mirror of the Q's DvDx for the mixed pair sweep.
__global__ void qGradient32Kernel(Fields F, float4* __restrict__ dvq, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float v[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) v[k] = (float)F.f[F_DVDXQ_XX + k][i];
  dvq[3 * i] = make_float4(v[0], v[1], v[2], v[3]);
  dvq[3 * i + 1] = make_float4(v[4], v[5], v[6], v[7]);
  dvq[3 * i + 2] = make_float4(v[8], 0.0f, 0.0f, 0.0f);
}
void launchCopyQGradient(Fields F, long n, cudaStream_t s, LaunchCounter* lc) {
  copyQGradientKernel<<<gridFor(n, 256), 256, 0, s>>>(F, n);
  lc->add(1);
}
void launchQGradient32(Fields F, float4* dvq, long n, cudaStream_t s, LaunchCounter* lc) {
  qGradient32Kernel<<<gridFor(n, 256), 256, 0, s>>>(F, dvq, n);
  lc->add(1);
}
void launchPermute(const Fields& Fin, Fields Fout, const int* perm, const int* origIn, int* origOut,
                   const int* listIn, int* listOut, const uint32_t* cellIn, uint32_t* cellOut, long n,
                   bool carriedOnly, bool tensor, bool crk, cudaStream_t s, LaunchCounter* lc) {
  // the tensor-H fields (the end of the carried block and of the permuted
  // block) move only in ASPH mode, the RK volume and corrections (the end of
  // the permuted block) only in CRKSPH mode
  FieldRanges sel{};
  auto add = [&](int a, int b) { sel.first[sel.n] = a; sel.last[sel.n] = b; ++sel.n; };
  add(0, tensor ? (int)F_NUM_CARRIED : (int)F_HT_XX);
  if (!carriedOnly) {
    add(F_NUM_CARRIED, tensor ? (int)F_VOL : (int)F_HIDEALT_XX);
    if (crk) add(F_VOL, F_NUM_PERMUTED);
  }
  permuteKernel<<<gridFor(n, 256), 256, 0, s>>>(Fin, Fout, perm, origIn, origOut, listIn, listOut, cellIn, cellOut, n,
                                                sel);
  lc->add(1);
}
void launchCellRanges(const uint32_t* sortedKeys, long n, int shift, int* cellStart, int* cellEnd, cudaStream_t s,
                      LaunchCounter* lc) {
  cellRangeKernel<<<gridFor(n, 256), 256, 0, s>>>(sortedKeys, n, shift, cellStart, cellEnd);
  lc->add(1);
}
void launchItemBoxes(const int* items, const long long* dItems, int nItemsBound, long n, int width, Fields32 P,
                     float4* box, int* chunkOf, cudaStream_t s, LaunchCounter* lc) {
  itemBoxKernel<<<gridFor(std::max(1, nItemsBound), 256), 256, 0, s>>>(items, dItems, n, width, P, box, chunkOf);
  lc->add(1);
}
// Band of the FP32 pre-filter on e2 = min(a_i, a_j)^2 r^2 around ext^2
// (a = 1/h).  Every cell-relative coordinate is within about one cell size C
// of its cell origin, so each FP32 separation component carries at most
// ~10 u C of rounding (u = 2^-24: the cell-relative positions, the mirror,
// the difference and the periodic offset), and near the threshold
// (a r ~ ext) |e2_fp32 - e2| <= ext^2 (20 sqrt(3) u C a / ext + 7 u).  The
// band used is four times that bound, evaluated with a = a_i >= min(a_i, a_j):
// delta_i = bandA a_i + bandB.  A node whose delta reaches 1/2 takes the exact
// test on every candidate.
static void neighborBand(const Grid& g, double ext2, float& bandA, float& bandB) {
  const double u = 1.0 / 16777216.0;
  const double cmax = std::max(g.cell[0], std::max(g.cell[1], g.cell[2]));
  const double ext = std::sqrt(ext2);
  bandA = (float)(4.0 * 20.0 * std::sqrt(3.0) * u * cmax / ext);
  bandB = (float)(4.0 * 7.0 * u);
}
void launchSumDensity(Fields F, const int* list, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                      cudaStream_t s, LaunchCounter* lc) {
  const size_t sm = sizeof(double) * 3 * (hp.tableN1 + 1);
  if (hp.asph) sumDensityKernel<true><<<gridFor(n, 128), 128, sm, s>>>(F, list, n, g, nl, t, hp);
  else sumDensityKernel<false><<<gridFor(n, 128), 128, sm, s>>>(F, list, n, g, nl, t, hp);
  lc->add(1);
}
void launchGradh(Fields F, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp, cudaStream_t s,
                 LaunchCounter* lc) {
  const size_t sm = sizeof(double) * 6 * (hp.tableN1 + 1);
  if (hp.asph) gradhKernel<true><<<gridFor(n, 128), 128, sm, s>>>(F, n, g, nl, t, hp);
  else gradhKernel<false><<<gridFor(n, 128), 128, sm, s>>>(F, n, g, nl, t, hp);
  lc->add(1);
}
void launchPairFP64(Fields F, const int* list, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                    double* pacc, int blockSize, cudaStream_t s, LaunchCounter* lc) {
  const size_t sm = sizeof(double) * 6 * (hp.tableN1 + 1);
  const int b = 128;
  (void)blockSize;
#define SPH_PAIR64(X, C, T) pairKernelFP64<X, C, T><<<gridFor(n, b), b, sm, s>>>(F, list, n, g, nl, t, hp, pacc)
  if (hp.asph) {
    if (hp.xsph) {
      if (hp.compatible) SPH_PAIR64(true, true, true); else SPH_PAIR64(true, false, true);
    } else {
      if (hp.compatible) SPH_PAIR64(false, true, true); else SPH_PAIR64(false, false, true);
    }
  } else if (hp.xsph) {
    if (hp.compatible) SPH_PAIR64(true, true, false); else SPH_PAIR64(true, false, false);
  } else {
    if (hp.compatible) SPH_PAIR64(false, true, false); else SPH_PAIR64(false, false, false);
  }
#undef SPH_PAIR64
  lc->add(1);
}
void launchDt(Fields F, const int* list, long n, Grid g, NeighborLists nl, HydroParams hp,
              double maxNperh, double* dScratch, int nScratch, double* dOut,
              cudaStream_t s, LaunchCounter* lc) {
  const int nb = (int)gridFor(n, 128);
  (void)nScratch;
  dtKernel<<<nb, 128, 0, s>>>(F, list, n, g, nl, hp, maxNperh, dScratch);
  dtFinalKernel<<<1, 256, 0, s>>>(dScratch, nb, dOut);
  lc->add(2);
}
void launchCompatibleEnergy(Fields F, long n, Grid g, NeighborLists nl, const double* pacc, const float* pacc32,
                            double dt, cudaStream_t s, LaunchCounter* lc) {
  if (pacc32) energyKernel<true><<<gridFor(n, 128), 128, 0, s>>>(F, n, g, nl, pacc, pacc32, dt);
  else energyKernel<false><<<gridFor(n, 128), 128, 0, s>>>(F, n, g, nl, pacc, pacc32, dt);
  lc->add(1);
}
void launchRestoreState0(Fields F, long n, bool tensor, bool crk, cudaStream_t s, LaunchCounter* lc) {
  restoreState0Kernel<<<gridFor(n, 256), 256, 0, s>>>(F, n, tensor ? 1 : 0, crk ? 1 : 0);
  lc->add(1);
}
void launchRadius0(Fields F, long n, cudaStream_t s, LaunchCounter* lc) {
  radius0Kernel<<<gridFor(n, 256), 256, 0, s>>>(F, n);
  lc->add(1);
}
void launchTensorExtent(Fields F, long n, cudaStream_t s, LaunchCounter* lc) {
  tensorExtentKernel<<<gridFor(n, 256), 256, 0, s>>>(F, n);
  lc->add(1);
}
void launchUpdate(Fields F, const int* list, long n, HydroParams hp, double mult,
                  bool mid, bool gravity, const Fields32* mirror, const Grid& g, cudaStream_t s, LaunchCounter* lc) {
  const int epsInc = (mid || !hp.compatible) ? 1 : 0;
  Fields32 P{};
  if (mirror) P = *mirror;
  if (hp.asph)
    updateKernel<true><<<gridFor(n, 256), 256, 0, s>>>(F, list, n, hp.lists, mult, mid ? 1 : 0, gravity ? 1 : 0, epsInc,
                                                       hp.hUpdate, hp.totalEnergy, 0, P, g, hp.asphEnd, hp.fixShape,
                                                       hp.radialOnly);
  else
    updateKernel<false><<<gridFor(n, 256), 256, 0, s>>>(F, list, n, hp.lists, mult, mid ? 1 : 0, gravity ? 1 : 0,
                                                        epsInc, hp.hUpdate, hp.totalEnergy, hp.crk, P, g, 0, 0, 0);
  lc->add(1);
}
void launchASPHEnd(Fields F, Fields32 P, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                   HydroParams hp, cudaStream_t s, LaunchCounter* lc) {
  const size_t smem = 3 * (size_t)(hp.tableN1 + 1) * sizeof(double);
  asphEndKernel<<<gridFor(n, 128), 128, smem, s>>>(F, P, list, n, g, nl, t, hp);
  lc->add(1);
}
void launchEOS(Fields F, const int* list, long n, const NodeListParams* lists, cudaStream_t s, LaunchCounter* lc) {
  eosKernel<<<gridFor(n, 256), 256, 0, s>>>(F, list, n, lists);
  lc->add(1);
}
void launchEnforce(Fields F, long n, Grid g, bool tensor, cudaStream_t s, LaunchCounter* lc) {
  enforceKernel<<<gridFor(n, 256), 256, 0, s>>>(F, n, g, tensor ? 1 : 0);
  lc->add(1);
}
void launchConservation(Fields F, long n, bool gravity, double* dScratch, int nScratch, double* dOut, cudaStream_t s,
                        LaunchCounter* lc) {
  int nb = (int)std::min<long>((n + 255) / 256, nScratch / 7);
  if (nb < 1) nb = 1;
  conservationKernel<<<nb, 256, 0, s>>>(F, n, gravity ? 1 : 0, dScratch);
  conservationFinalKernel<<<1, 256, 0, s>>>(dScratch, nb, dOut);
  lc->add(2);
}
void launchCheckState(Fields F, long n, int* dFlag, cudaStream_t s, LaunchCounter* lc) {
  checkStateKernel<<<gridFor(n, 256), 256, 0, s>>>(F, n, dFlag);
  lc->add(1);
}

void launchExchangeGet(Fields F, const int* inv, const int* idx, long count, ExchangeFields ef, double* out,
                       cudaStream_t s, LaunchCounter* lc) {
  if (count <= 0) return;
  exchangeGetKernel<<<gridFor(count, 256), 256, 0, s>>>(F, inv, idx, count, ef, out);
  lc->add(1);
}
void launchExchangePut(Fields F, Fields32 P, const int* inv, long nOwn, long count, ExchangeFields ef,
                       const double* in, cudaStream_t s, LaunchCounter* lc) {
  if (count <= 0) return;
  exchangePutKernel<<<gridFor(count, 256), 256, 0, s>>>(F, P, inv, nOwn, count, ef, in);
  lc->add(1);
}

void launchGatherOut(Fields F, const int* orig, double* stage, int first, int ncomp, int stride, long n,
                     cudaStream_t s, LaunchCounter* lc) {
  gatherOutKernel<<<gridFor(n, 256), 256, 0, s>>>(F, orig, stage, first, ncomp, stride, n);
  lc->add(1);
}
void launchScatterIn(Fields F, const int* orig, const double* stage, int first, int ncomp, int stride, long n,
                     cudaStream_t s, LaunchCounter* lc) {
  scatterInKernel<<<gridFor(n, 256), 256, 0, s>>>(F, orig, stage, first, ncomp, stride, n);
  lc->add(1);
}
void launchInverseOrder(const int* orig, int* inv, long n, cudaStream_t s, LaunchCounter* lc) {
  inverseOrderKernel<<<gridFor(n, 256), 256, 0, s>>>(orig, inv, n);
  lc->add(1);
}
void launchScatterInHost(Fields F, const int* inv, const double* src, int first, int ncomp, int stride, long n,
                         cudaStream_t s, LaunchCounter* lc) {
  scatterInHostKernel<<<gridFor(n * stride, 256), 256, 0, s>>>(F, inv, src, first, ncomp, stride, n);
  lc->add(1);
}
void launchGatherOutHost(Fields F, const int* inv, double* dst, int first, int ncomp, int stride, bool isoH, long n,
                         cudaStream_t s, LaunchCounter* lc) {
  gatherOutHostKernel<<<gridFor(n * stride, 256), 256, 0, s>>>(F, inv, dst, first, ncomp, stride, isoH ? 1 : 0, n);
  lc->add(1);
}
void launchGatherOutH(Fields F, const int* orig, double* stage, int field, long n, cudaStream_t s, LaunchCounter* lc) {
  gatherOutHKernel<<<gridFor(n, 256), 256, 0, s>>>(F, orig, stage, field, n);
  lc->add(1);
}
void launchCountsOut(const int* counts, const int* orig, double* stage, long n, cudaStream_t s, LaunchCounter* lc) {
  countsOutKernel<<<gridFor(n, 256), 256, 0, s>>>(counts, orig, stage, n);
  lc->add(1);
}

void launchItemFlags(const uint32_t* keys, long n, int shift, const int* cellStart, int width, int* flag,
                     cudaStream_t s, LaunchCounter* lc) {
  itemFlagKernel<<<gridFor(n, 256), 256, 0, s>>>(keys, n, shift, cellStart, width, flag);
  lc->add(1);
}
void launchItemFill(const int* flag, const long long* pos, long n, int* items, cudaStream_t s, LaunchCounter* lc) {
  itemFillKernel<<<gridFor(n, 256), 256, 0, s>>>(flag, pos, n, items);
  lc->add(1);
}
void launchNeighborsWarp(const Fields& F, Fields32 P, long n, const int* items, int nItems, const long long* dItems,
                         int width, Grid g, const int* cellStart, const int* cellEnd, int* counts, int* maxCount,
                         uint32_t* nbr, int cap, double ext2, bool tensor, const float4* box, const int* chunkOf,
                         cudaStream_t s, LaunchCounter* lc) {
  float lo, hi;
  neighborBand(g, ext2, lo, hi);
  const long threads = (long)nItems * width;
  const unsigned gb = (unsigned)((threads + 127) / 128);
#define SPH_NBR(WR, WD, TE)                                                                                        \
  neighborWarpKernel<WR, WD, TE><<<gb, 128, 0, s>>>(F, P, n, items, nItems, g, cellStart, cellEnd, counts,        \
                                                    WR ? nbr : nullptr, ext2, lo, hi, WR ? cap : 0, maxCount, dItems, \
                                                    box, chunkOf)
  if (tensor) {
    if (nbr) {
      if (width == 8) SPH_NBR(true, 8, true); else if (width == 16) SPH_NBR(true, 16, true); else SPH_NBR(true, 32, true);
    } else {
      if (width == 8) SPH_NBR(false, 8, true); else if (width == 16) SPH_NBR(false, 16, true); else SPH_NBR(false, 32, true);
    }
  } else if (nbr) {
    if (width == 8) SPH_NBR(true, 8, false); else if (width == 16) SPH_NBR(true, 16, false); else SPH_NBR(true, 32, false);
  } else {
    if (width == 8) SPH_NBR(false, 8, false); else if (width == 16) SPH_NBR(false, 16, false); else SPH_NBR(false, 32, false);
  }
#undef SPH_NBR
  lc->add(1);
}

}  // namespace sph
