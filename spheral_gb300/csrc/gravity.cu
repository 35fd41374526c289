// Octree gravity of libsphgpu: the TreeGravity build and walk
// (src/Gravity/TreeGravity.cc:362-480, 819-932; TreeGravityInline.hh:38-165)
// as a linear octree over Morton-sorted nodes.
//
// The reference inserts nodes one at a time into per-level hash maps: a cell
// is created holding a single node and split when a second node arrives,
// down to level 20 where nodes accumulate in one leaf.  The resulting tree
// does not depend on the insertion order: the cell (l, key) exists when it
// holds a node and its parent holds at least two (or l == 0); it is a leaf
// when it holds one node or l == 20.  Here every node gets the reference's
// level-20 integer coordinates (same floating-point expression), the nodes
// are sorted by the 60-bit Morton key of those coordinates, and the cells are
// read off the sorted keys:
//
//   cpl(k)  = deepest level at which sorted nodes k-1 and k share a cell
//             (-1 for k = 0 and k = n);
//   the cells that start at node k are the levels cpl(k)+1 .. leaf(k),
//   leaf(k) = min(20, max(cpl(k), cpl(k+1)) + 1).
//
// Listing those chains in node order gives the cells in depth-first
// pre-order; each cell stores the index of the first cell after its subtree
// (`skip`), so the walk needs no stack.  Monopoles (mass, centre of mass) are
// summed bottom-up, level by level.
//
// Walk.  The reference walks level by level per node and, per cell, applies
// the far-field monopole when r^2 > cellsize^2 / theta^2 + |xcm - centre|^2,
// sums the leaf's nodes directly when the cell is a leaf, and descends
// otherwise (TreeGravity.cc:845-905).  The per-node set of far cells and
// opened leaves does not depend on the visiting order, so here the 32 nodes
// of a warp (neighbours in Morton order) walk the pre-order cell array
// together: a lane that applies a cell (far or leaf) skips that cell's
// subtree; the warp descends into a cell while any lane still needs it open.
// Forces, potentials and the decision are evaluated in FP64 with the
// reference's expressions (no fused multiply-add in the opening test);
// summation order is pre-order instead of level order.
//
// Mixed precision (the mixed-mode package).  GB300's FP64 pipe is thin, so
// the mixed walk evaluates each interaction in FP32 on double-float
// (hi + lo) coordinates -- the separation (hi_c - hi_i) + (lo_c - lo_i)
// carries FP32 relative precision at any distance -- and sums the terms with
// compensated (Kahan) FP32 accumulators that leave the kernel as the FP64
// value s - c.  The far/near decision compares the FP32 r^2 with the FP32
// threshold; inside a guard band of +-4e-6 (far above the FP32 error of both)
// it is retaken in FP64 with the reference's expression, so the set of far
// cells and opened leaves is the FP64 walk's.
#include "kernels.cuh"
#include "sort.cuh"
#include "../../include/sphgpu.h"

#include <cfloat>
#include <cstdio>
#include <cstring>
#include <string>

namespace sph {

namespace {

constexpr int kMaxLevel = 20;   // num1dbits - 1 (TreeGravity.hh: num1dbits = 21)
constexpr int kThreads = 256;

inline int blocksFor(long n, int t) { return (int)((n + t - 1) / t); }

// 64 bytes: one cell read by a whole warp is two 32-byte sectors.
struct __align__(32) TreeCell {
  double x, y, z, M;   // centre of mass and mass (Mglobal on one process)
  double r2cc;         // |xcm - geometric centre|^2 (rcm2cc2)
  double spare;
  int skip;            // first pre-order index after this cell's subtree
  int start;           // first node (tree order)
  int count;           // nodes in the cell
  int lvl;             // level | leaf << 8
};
static_assert(sizeof(TreeCell) == 64, "TreeCell layout");

// Node in tree order: position and mass.
struct __align__(32) TreeNode {
  double x, y, z, m;
};

__device__ __forceinline__ TreeNode loadNode(const TreeNode* __restrict__ p) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
  return TreeNode{a.x, a.y, b.x, b.y};
}

// Mixed-walk copies: double-float centre of mass, FP32 mass, FP32 opening
// threshold thr[level] + rcm2cc2; same skip/start/count/lvl.
struct __align__(16) TreeCell32 {
  float xh, yh, zh, M;
  float xl, yl, zl, open2;
  int skip, start, count, lvl;
};
static_assert(sizeof(TreeCell32) == 48, "TreeCell32 layout");

struct __align__(32) TreeNode32 {
  float xh, yh, zh, m;
  float xl, yl, zl, pad;
};

__device__ __forceinline__ void splitDF(double x, float& h, float& l) {
  h = (float)x;
  l = (float)(x - (double)h);
}

struct GBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t b) {
    if (b <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    const cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

__device__ __forceinline__ uint64_t spread3(uint64_t v) {
  // 20-bit integer -> every third bit of a 60-bit word.
  v &= 0xFFFFFull;
  v = (v | (v << 32)) & 0x001F00000000FFFFull;
  v = (v | (v << 16)) & 0x001F0000FF0000FFull;
  v = (v | (v << 8)) & 0x100F00F00F00F00Full;
  v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

__device__ __forceinline__ uint64_t compact3(uint64_t v) {
  v &= 0x1249249249249249ull;
  v = (v | (v >> 2)) & 0x10C30C30C30C30C3ull;
  v = (v | (v >> 4)) & 0x100F00F00F00F00Full;
  v = (v | (v >> 8)) & 0x001F0000FF0000FFull;
  v = (v | (v >> 16)) & 0x001F00000000FFFFull;
  v = (v | (v >> 32)) & 0xFFFFFull;
  return v;
}

// TreeGravity::buildCellKey at the deepest level: min(ncell-1, (x - xmin) /
// boxLength * ncell) truncated, ncell = 2^20.
__device__ __forceinline__ uint64_t cellCoord(double x, double xmin, double L) {
  const double u = __dmul_rn(__ddiv_rn(__dsub_rn(x, xmin), L), 1048576.0);
  const uint64_t c = (uint64_t)u;
  return c < 1048575ull ? c : 1048575ull;
}

//------------------------------------------------------------------------------
// Bounding box (TreeGravity::initialize: xmin, xmax, boxLength).
//------------------------------------------------------------------------------
__global__ void boxPartialKernel(Fields F, long n, double* __restrict__ part) {
  __shared__ double sm[6][kThreads / 32];
  double v[6] = {DBL_MAX, DBL_MAX, DBL_MAX, DBL_MAX, DBL_MAX, DBL_MAX};   // min x,y,z, -max x,y,z
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double x = F.f[F_X][i], y = F.f[F_Y][i], z = F.f[F_Z][i];
    v[0] = fmin(v[0], x); v[1] = fmin(v[1], y); v[2] = fmin(v[2], z);
    v[3] = fmin(v[3], -x); v[4] = fmin(v[4], -y); v[5] = fmin(v[5], -z);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] = fmin(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
    if (lane == 0) sm[k][warp] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double r = DBL_MAX;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmin(r, sm[threadIdx.x][w]);
    part[blockIdx.x * 6 + threadIdx.x] = r;
  }
}

// box = {xmin, ymin, zmin, boxLength, boxLength^2, -, -, -};
// also resets the dt-vote slot and the per-level opening thresholds.
__global__ void boxFinalKernel(const double* __restrict__ part, int nb, double opening, double* __restrict__ box,
                               double* __restrict__ thr, unsigned long long* __restrict__ dtBits) {
  __shared__ double v[6];
  __shared__ double sL2;
  if (threadIdx.x < 6) {
    double r = DBL_MAX;
    for (int b = 0; b < nb; ++b) r = fmin(r, part[b * 6 + threadIdx.x]);
    v[threadIdx.x] = r;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double xmin = v[0], ymin = v[1], zmin = v[2];
    const double xmax = -v[3], ymax = -v[4], zmax = -v[5];
    // boxLength = max(xmax - xmin, max(ymax - ymin, zmax - zmin))
    const double L = fmax(__dsub_rn(xmax, xmin), fmax(__dsub_rn(ymax, ymin), __dsub_rn(zmax, zmin)));
    sL2 = __dmul_rn(L, L);
    box[0] = xmin; box[1] = ymin; box[2] = zmin; box[3] = L; box[4] = sL2;
    *dtBits = __double_as_longlong(DBL_MAX);
  }
  __syncthreads();
  if (threadIdx.x <= kMaxLevel) {
    // cellsize2 / opening2 with cellsize2 = boxLength2 / 2^(2 level)
    const double cs2 = __ddiv_rn(sL2, (double)(1ull << (2 * threadIdx.x)));
    thr[threadIdx.x] = __ddiv_rn(cs2, __dmul_rn(opening, opening));
  }
}

//------------------------------------------------------------------------------
// Morton keys of the level-20 cell coordinates; sort by (hi 30, lo 30) bits.
//------------------------------------------------------------------------------
__global__ void treeKeyKernel(Fields F, long n, const double* __restrict__ box, uint64_t* __restrict__ key64,
                              uint32_t* __restrict__ lo, int* __restrict__ vals) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double L = box[3];
  uint64_t key = 0;
  if (L > 0.0) {
    const uint64_t ix = cellCoord(F.f[F_X][i], box[0], L);
    const uint64_t iy = cellCoord(F.f[F_Y][i], box[1], L);
    const uint64_t iz = cellCoord(F.f[F_Z][i], box[2], L);
    key = spread3(ix) | (spread3(iy) << 1) | (spread3(iz) << 2);
  }
  key64[i] = key;
  lo[i] = (uint32_t)(key & 0x3FFFFFFFull);
  vals[i] = (int)i;
}

__global__ void gatherHiKernel(const uint64_t* __restrict__ key64, const int* __restrict__ vals, long n,
                               uint32_t* __restrict__ hi) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  hi[k] = (uint32_t)(key64[vals[k]] >> 30);
}

// Tree-ordered node data and the shared-level count cpl(k).
__global__ void treeNodesKernel(Fields F, const uint64_t* __restrict__ key64, const int* __restrict__ vals, long n,
                                uint64_t* __restrict__ skey, TreeNode* __restrict__ tpos,
                                TreeNode32* __restrict__ tpos32) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int i = vals[k];
  skey[k] = key64[i];
  const double x = F.f[F_X][i], y = F.f[F_Y][i], z = F.f[F_Z][i], m = F.f[F_MASS][i];
  tpos[k] = TreeNode{x, y, z, m};
  if (tpos32) {
    TreeNode32 t;
    splitDF(x, t.xh, t.xl);
    splitDF(y, t.yh, t.yl);
    splitDF(z, t.zh, t.zl);
    t.m = (float)m;
    t.pad = 0.0f;
    tpos32[k] = t;
  }
}

__device__ __forceinline__ int sharedLevels(const uint64_t* __restrict__ skey, long n, long k) {
  if (k <= 0 || k >= n) return -1;
  const uint64_t x = skey[k] ^ skey[k - 1];
  if (x == 0) return kMaxLevel;
  const int b = 63 - __clzll((long long)x);
  return kMaxLevel - 1 - b / 3;
}

__device__ __forceinline__ int leafLevel(int c0, int c1) {
  const int m = (c0 > c1 ? c0 : c1) + 1;
  return m < kMaxLevel ? m : kMaxLevel;
}

__global__ void chainCountKernel(const uint64_t* __restrict__ skey, long n, int* __restrict__ nc) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int c0 = sharedLevels(skey, n, k), c1 = sharedLevels(skey, n, k + 1);
  nc[k] = leafLevel(c0, c1) - c0;
}

// First node after k whose level-l cell differs from k's (sorted keys).
__device__ __forceinline__ long cellEnd(const uint64_t* __restrict__ skey, long n, long k, int l) {
  const int sh = 3 * (kMaxLevel - l);
  const uint64_t p = skey[k] >> sh;
  long lo = k + 1, hi = n;
  while (lo < hi) {
    const long mid = (lo + hi) >> 1;
    if ((skey[mid] >> sh) == p) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void cellBuildKernel(const uint64_t* __restrict__ skey, long n, const long long* __restrict__ off,
                                long long numCells, TreeCell* __restrict__ cells) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int c0 = sharedLevels(skey, n, k), c1 = sharedLevels(skey, n, k + 1);
  const int lf = leafLevel(c0, c1);
  const long long base = off[k];
  for (int l = c0 + 1; l <= lf; ++l) {
    const long e = (l == lf && l < kMaxLevel) ? k + 1 : cellEnd(skey, n, k, l);
    TreeCell c;
    c.x = c.y = c.z = c.M = c.r2cc = c.spare = 0.0;
    c.skip = (int)(e < n ? off[e] : numCells);
    c.start = (int)k;
    c.count = (int)(e - k);
    c.lvl = l | ((l == lf) ? 256 : 0);
    cells[base + (l - c0 - 1)] = c;
  }
}

// Monopoles of the cells of one level (children are one level deeper and
// already done).  Leaves sum their nodes; a one-node leaf keeps the node's
// position exactly, as the reference's single-node cell does.
__global__ void momentKernel(TreeCell* __restrict__ cells, long long numCells, int level,
                             const TreeNode* __restrict__ tpos, const uint64_t* __restrict__ skey,
                             const double* __restrict__ box, double* __restrict__ mx) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= numCells) return;
  TreeCell cl = cells[c];
  if ((cl.lvl & 255) != level) return;
  double M = 0.0, sx = 0.0, sy = 0.0, sz = 0.0, x, y, z;
  if (cl.lvl >> 8) {
    if (cl.count == 1) {
      const TreeNode p = tpos[cl.start];
      M = p.m; x = p.x; y = p.y; z = p.z;
      sx = p.m * p.x; sy = p.m * p.y; sz = p.m * p.z;
    } else {
      for (int j = cl.start; j < cl.start + cl.count; ++j) {
        const TreeNode p = tpos[j];
        M += p.m; sx += p.m * p.x; sy += p.m * p.y; sz += p.m * p.z;
      }
      x = sx / M; y = sy / M; z = sz / M;
    }
  } else {
    for (long long ch = c + 1; ch < cl.skip; ch = cells[ch].skip) {
      M += cells[ch].M;
      sx += mx[3 * ch]; sy += mx[3 * ch + 1]; sz += mx[3 * ch + 2];
    }
    x = sx / M; y = sy / M; z = sz / M;
  }
  mx[3 * c] = sx; mx[3 * c + 1] = sy; mx[3 * c + 2] = sz;
  // Geometric centre: xmin + (ix + 0.5) * cellsize, cellsize = boxLength / 2^level.
  const uint64_t key = skey[cl.start];
  const int sh = kMaxLevel - level;
  const double cs = __ddiv_rn(box[3], (double)(1u << level));
  const double cx = __dadd_rn(box[0], __dmul_rn((double)(compact3(key) >> sh) + 0.5, cs));
  const double cy = __dadd_rn(box[1], __dmul_rn((double)(compact3(key >> 1) >> sh) + 0.5, cs));
  const double cz = __dadd_rn(box[2], __dmul_rn((double)(compact3(key >> 2) >> sh) + 0.5, cs));
  const double dx = __dsub_rn(x, cx), dy = __dsub_rn(y, cy), dz = __dsub_rn(z, cz);
  cl.x = x; cl.y = y; cl.z = z; cl.M = M;
  cl.r2cc = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  cells[c] = cl;
}

//------------------------------------------------------------------------------
// Walk (TreeGravity::applyTreeForces, TreeGravity.cc:819-932).
//------------------------------------------------------------------------------
__device__ __forceinline__ void addMonopole(double M, double dx, double dy, double dz, double r2, double soft2,
                                            double& ax, double& ay, double& az, double& phi) {
  // nhat = unitVector(xji); rji2 += soft2; a += M/rji2 nhat; phi -= M/sqrt(rji2)
  double nx = 1.0, ny = 0.0, nz = 0.0;
  const double r = sqrt(r2);
  if (r > 1.0e-50) {
    const double ir = 1.0 / r;
    nx = dx * ir; ny = dy * ir; nz = dz * ir;
  }
  const double r2s = r2 + soft2;
  const double irs = rsqrt(r2s);
  const double f = M * (irs * irs);
  ax += f * nx; ay += f * ny; az += f * nz;
  phi -= M * irs;
}

__global__ void __launch_bounds__(128) treeWalkKernel(const TreeCell* __restrict__ cells, long long numCells,
                                                     const TreeNode* __restrict__ tpos, const int* __restrict__ vals,
                                                     long n, const double* __restrict__ thrLevel, double soft2,
                                                     double softening, double G, Fields F,
                                                     unsigned long long* __restrict__ dtBits,
                                                     double* __restrict__ energyPart) {
  __shared__ double thr[kMaxLevel + 1];
  __shared__ double esum[4];
  __shared__ double dmin[4];
  if (threadIdx.x <= kMaxLevel) thr[threadIdx.x] = thrLevel[threadIdx.x];
  __syncthreads();
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const bool valid = k < n;
  double xi = 0, yi = 0, zi = 0, mi = 0;
  if (valid) {
    const TreeNode p = tpos[k];
    xi = p.x; yi = p.y; zi = p.z; mi = p.m;
  }
  double ax = 0, ay = 0, az = 0, phi = 0;
  // until: this lane ignores cells below this pre-order index
  unsigned until = valid ? 0u : 0xFFFFFFFFu;
  unsigned c = 1;   // the walk starts at the root's daughters
  const unsigned nc = (unsigned)numCells;
  if (__all_sync(0xffffffffu, !valid)) c = nc;
  while (c < nc) {
    const double2* cp = reinterpret_cast<const double2*>(cells + c);
    const double2 qa = __ldg(cp), qb = __ldg(cp + 1), qc = __ldg(cp + 2);
    const int4 qi = __ldg(reinterpret_cast<const int4*>(cp + 3));
    const double cxm = qa.x, cym = qa.y, czm = qb.x, cM = qb.y, r2cc = qc.x;
    const unsigned skip = (unsigned)qi.x;
    const int start = qi.y, count = qi.z, level = qi.w & 255, leaf = qi.w >> 8;
    bool descend = false;
    if (c >= until) {
      const double dx = __dsub_rn(cxm, xi), dy = __dsub_rn(cym, yi), dz = __dsub_rn(czm, zi);
      const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
      if (r2 > __dadd_rn(thr[level], r2cc)) {
        addMonopole(cM, dx, dy, dz, r2, soft2, ax, ay, az, phi);
        until = skip;
      } else if (leaf) {
        for (int j = start; j < start + count; ++j) {
          const TreeNode p = loadNode(tpos + j);
          const double ex = __dsub_rn(p.x, xi), ey = __dsub_rn(p.y, yi), ez = __dsub_rn(p.z, zi);
          const double s2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
          if (__ddiv_rn(s2, soft2) > 1.0e-10) addMonopole(p.m, ex, ey, ez, s2, soft2, ax, ay, az, phi);
        }
        until = skip;
      } else {
        descend = true;
      }
    }
    if (__any_sync(0xffffffffu, descend)) ++c;
    else c = __reduce_min_sync(0xffffffffu, until);
  }
  // Outputs: a, phi times G; dt vote sqrt(softening / |a|) before G.
  double vote = DBL_MAX, e = 0.0;
  if (valid) {
    const int i = vals[k];
    F.f[F_GRAV_X][i] = G * ax;
    F.f[F_GRAV_Y][i] = G * ay;
    F.f[F_GRAV_Z][i] = G * az;
    const double pot = G * phi;
    F.f[F_POT][i] = pot;
    const double amag = sqrt(ax * ax + ay * ay + az * az);
    if (amag > 0.0) vote = sqrt(softening / amag);
    e = 0.5 * mi * pot;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    vote = fmin(vote, __shfl_xor_sync(0xffffffffu, vote, o));
    e += __shfl_xor_sync(0xffffffffu, e, o);
  }
  if (lane == 0) { dmin[warp] = vote; esum[warp] = e; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = dmin[0], s = esum[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { v = fmin(v, dmin[w]); s += esum[w]; }
    energyPart[blockIdx.x] = s;
    atomicMin(dtBits, (unsigned long long)__double_as_longlong(v));   // positive doubles order as integers
  }
}

__global__ void cells32Kernel(const TreeCell* __restrict__ cells, long long numCells,
                              const double* __restrict__ thrLevel, TreeCell32* __restrict__ c32) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= numCells) return;
  const TreeCell cl = cells[c];
  TreeCell32 o;
  splitDF(cl.x, o.xh, o.xl);
  splitDF(cl.y, o.yh, o.yl);
  splitDF(cl.z, o.zh, o.zl);
  o.M = (float)cl.M;
  o.open2 = (float)__dadd_rn(thrLevel[cl.lvl & 255], cl.r2cc);
  o.skip = cl.skip;
  o.start = cl.start;
  o.count = cl.count;
  o.lvl = cl.lvl;
  c32[c] = o;
}

__device__ __forceinline__ void kahan(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// FP32 monopole term on a double-float separation: a += M/(r^2+eps^2) rhat,
// phi -= M/sqrt(r^2+eps^2), compensated sums.
struct Acc32 {
  float sx, sy, sz, sp, cx, cy, cz, cp;
};

__device__ __forceinline__ void addMonopole32(float M, float dx, float dy, float dz, float r2, float soft2,
                                              Acc32& a) {
  const float ir = r2 > 1.0e-30f ? rsqrtf(r2) : 0.0f;
  const float nx = r2 > 1.0e-30f ? dx * ir : 1.0f, ny = dy * ir, nz = dz * ir;
  const float irs = rsqrtf(r2 + soft2);
  const float f = M * (irs * irs);
  kahan(a.sx, a.cx, f * nx);
  kahan(a.sy, a.cy, f * ny);
  kahan(a.sz, a.cz, f * nz);
  kahan(a.sp, a.cp, -M * irs);
}

__global__ void __launch_bounds__(128) treeWalkMixedKernel(
    const TreeCell32* __restrict__ c32, const TreeCell* __restrict__ cells, long long numCells,
    const TreeNode32* __restrict__ t32, const TreeNode* __restrict__ tpos, const int* __restrict__ vals, long n,
    const double* __restrict__ thrLevel, double soft2d, double softening, double G, Fields F,
    unsigned long long* __restrict__ dtBits, double* __restrict__ energyPart) {
  __shared__ double thr[kMaxLevel + 1];
  __shared__ double esum[4];
  __shared__ double dmin[4];
  if (threadIdx.x <= kMaxLevel) thr[threadIdx.x] = thrLevel[threadIdx.x];
  __syncthreads();
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const bool valid = k < n;
  TreeNode32 me{0, 0, 0, 0, 0, 0, 0, 0};
  double xd = 0, yd = 0, zd = 0, mi = 0;
  if (valid) {
    me = t32[k];
    const TreeNode p = tpos[k];
    xd = p.x; yd = p.y; zd = p.z; mi = p.m;
  }
  const float soft2 = (float)soft2d;
  constexpr float kBand = 4.0e-6f;
  Acc32 acc{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  unsigned until = valid ? 0u : 0xFFFFFFFFu;
  unsigned c = 1;
  const unsigned nc = (unsigned)numCells;
  if (__all_sync(0xffffffffu, !valid)) c = nc;
  while (c < nc) {
    const float4* cp = reinterpret_cast<const float4*>(c32 + c);
    const float4 qa = __ldg(cp), qb = __ldg(cp + 1);
    const int4 qi = __ldg(reinterpret_cast<const int4*>(cp + 2));
    const unsigned skip = (unsigned)qi.x;
    const int start = qi.y, count = qi.z, level = qi.w & 255, leaf = qi.w >> 8;
    bool descend = false;
    if (c >= until) {
      const float dx = __fadd_rn(__fsub_rn(qa.x, me.xh), __fsub_rn(qb.x, me.xl));
      const float dy = __fadd_rn(__fsub_rn(qa.y, me.yh), __fsub_rn(qb.y, me.yl));
      const float dz = __fadd_rn(__fsub_rn(qa.z, me.zh), __fsub_rn(qb.z, me.zl));
      const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
      const float o2 = qb.w;
      bool far;
      if (r2 > o2 * (1.0f + kBand)) far = true;
      else if (r2 < o2 * (1.0f - kBand)) far = false;
      else {   // guard band: the reference's FP64 test
        const TreeCell& cd = cells[c];
        const double ex = __dsub_rn(cd.x, xd), ey = __dsub_rn(cd.y, yd), ez = __dsub_rn(cd.z, zd);
        const double q2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
        far = q2 > __dadd_rn(thr[level], cd.r2cc);
      }
      if (far) {
        addMonopole32(qa.w, dx, dy, dz, r2, soft2, acc);
        until = skip;
      } else if (leaf) {
        for (int j = start; j < start + count; ++j) {
          const TreeNode32 p = t32[j];
          const float ex = __fadd_rn(__fsub_rn(p.xh, me.xh), __fsub_rn(p.xl, me.xl));
          const float ey = __fadd_rn(__fsub_rn(p.yh, me.yh), __fsub_rn(p.yl, me.yl));
          const float ez = __fadd_rn(__fsub_rn(p.zh, me.zh), __fsub_rn(p.zl, me.zl));
          const float q2 = __fmaf_rn(ez, ez, __fmaf_rn(ey, ey, __fmul_rn(ex, ex)));
          const float lim = 1.0e-10f * soft2;
          bool use;
          if (q2 > lim * 1.001f) use = true;
          else if (q2 < lim * 0.999f) use = false;
          else {   // the reference's r2 / soft2 > 1e-10 in FP64
            const TreeNode pd = tpos[j];
            const double fx = __dsub_rn(pd.x, xd), fy = __dsub_rn(pd.y, yd), fz = __dsub_rn(pd.z, zd);
            const double w2 = __dadd_rn(__dadd_rn(__dmul_rn(fx, fx), __dmul_rn(fy, fy)), __dmul_rn(fz, fz));
            use = __ddiv_rn(w2, soft2d) > 1.0e-10;
          }
          if (use) addMonopole32(p.m, ex, ey, ez, q2, soft2, acc);
        }
        until = skip;
      } else {
        descend = true;
      }
    }
    if (__any_sync(0xffffffffu, descend)) ++c;
    else c = __reduce_min_sync(0xffffffffu, until);
  }
  double vote = DBL_MAX, e = 0.0;
  if (valid) {
    const double ax = (double)acc.sx - (double)acc.cx, ay = (double)acc.sy - (double)acc.cy;
    const double az = (double)acc.sz - (double)acc.cz, phi = (double)acc.sp - (double)acc.cp;
    const int i = vals[k];
    F.f[F_GRAV_X][i] = G * ax;
    F.f[F_GRAV_Y][i] = G * ay;
    F.f[F_GRAV_Z][i] = G * az;
    const double pot = G * phi;
    F.f[F_POT][i] = pot;
    const double amag = sqrt(ax * ax + ay * ay + az * az);
    if (amag > 0.0) vote = sqrt(softening / amag);
    e = 0.5 * mi * pot;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    vote = fmin(vote, __shfl_xor_sync(0xffffffffu, vote, o));
    e += __shfl_xor_sync(0xffffffffu, e, o);
  }
  if (lane == 0) { dmin[warp] = vote; esum[warp] = e; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = dmin[0], sm = esum[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { v = fmin(v, dmin[w]); sm += esum[w]; }
    energyPart[blockIdx.x] = sm;
    atomicMin(dtBits, (unsigned long long)__double_as_longlong(v));
  }
}

__global__ void walkFinalKernel(const double* __restrict__ energyPart, int nb, const unsigned long long* dtBits,
                                double G, double* __restrict__ out) {
  __shared__ double sm[32];
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += energyPart[b];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) sm[warp] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
    out[0] = __longlong_as_double((long long)*dtBits) / sqrt(G);   // dtMinAcc
    out[1] = t;                                                      // extraEnergy
  }
}

__global__ void zeroGravityKernel(Fields F, long n, double G, double* __restrict__ out) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i == 0) { out[0] = DBL_MAX / sqrt(G); out[1] = 0.0; }
  if (i >= n) return;
  F.f[F_GRAV_X][i] = F.f[F_GRAV_Y][i] = F.f[F_GRAV_Z][i] = 0.0;
  F.f[F_POT][i] = 0.0;
}

}  // namespace

struct GravityWork {
  GBuf part, box, thr, dtBits, key64, lo, lo2, vals, vals2, sortWs, skey, tpos, nc, off, scanWs, total, cells, mx,
      energy, tpos32, cells32;
  long long* hTotal = nullptr;
  long long lastCells = 0;
};

GravityWork* gravityCreate() {
  GravityWork* w = new GravityWork();
  if (cudaMallocHost(&w->hTotal, sizeof(long long)) != cudaSuccess) w->hTotal = nullptr;
  return w;
}

void gravityDestroy(GravityWork* w) {
  if (!w) return;
  GBuf* all[] = {&w->part, &w->box, &w->thr, &w->dtBits, &w->key64, &w->lo, &w->lo2, &w->vals, &w->vals2,
                 &w->sortWs, &w->skey, &w->tpos, &w->nc, &w->off, &w->scanWs, &w->total, &w->cells, &w->mx,
                 &w->energy, &w->tpos32, &w->cells32};
  for (GBuf* b : all) b->release();
  if (w->hTotal) cudaFreeHost(w->hTotal);
  delete w;
}

long long gravityNumCells(const GravityWork* w) { return w ? w->lastCells : 0; }

int gravityEvaluate(GravityWork* w, Fields F, long n, double G, double softening, double opening, bool mixed,
                    double* dOut, cudaStream_t s, LaunchCounter* lc, char* err, int errlen) {
#define GCHK(expr)                                                                     \
  do {                                                                                 \
    const cudaError_t e_ = (expr);                                                     \
    if (e_ != cudaSuccess) {                                                           \
      std::snprintf(err, errlen, "%s: %s", #expr, cudaGetErrorString(e_));             \
      return SPHGPU_E_CUDA;                                                            \
    }                                                                                  \
  } while (0)
  if (!w || !w->hTotal) { std::snprintf(err, errlen, "gravity work space missing"); return SPHGPU_E_STATE; }
  if (!(softening > 0.0) || !(opening > 0.0) || !(G > 0.0)) {
    std::snprintf(err, errlen, "TreeGravity needs G, softening and opening > 0");
    return SPHGPU_E_ARG;
  }
  if (n <= 1) {
    zeroGravityKernel<<<blocksFor(n > 0 ? n : 1, kThreads), kThreads, 0, s>>>(F, n, G, dOut);
    lc->add(1);
    w->lastCells = n;
    GCHK(cudaGetLastError());
    return SPHGPU_OK;
  }
  const int nbBox = 304;
  GCHK(w->part.ensure(nbBox * 6 * sizeof(double)));
  GCHK(w->box.ensure(8 * sizeof(double)));
  GCHK(w->thr.ensure(32 * sizeof(double)));
  GCHK(w->dtBits.ensure(sizeof(unsigned long long)));
  GCHK(w->key64.ensure(n * sizeof(uint64_t)));
  GCHK(w->skey.ensure(n * sizeof(uint64_t)));
  GCHK(w->lo.ensure(n * sizeof(uint32_t)));
  GCHK(w->lo2.ensure(n * sizeof(uint32_t)));
  GCHK(w->vals.ensure(n * sizeof(int)));
  GCHK(w->vals2.ensure(n * sizeof(int)));
  GCHK(w->sortWs.ensure(radixSortWorkspaceBytes(n)));
  GCHK(w->tpos.ensure(n * sizeof(TreeNode)));
  if (mixed) GCHK(w->tpos32.ensure(n * sizeof(TreeNode32)));
  GCHK(w->nc.ensure(n * sizeof(int)));
  GCHK(w->off.ensure((n + 1) * sizeof(long long)));
  GCHK(w->scanWs.ensure(scanWorkspaceBytes(n)));
  GCHK(w->total.ensure(sizeof(long long)));
  const int nbWalk = blocksFor(n, 128);
  GCHK(w->energy.ensure(nbWalk * sizeof(double)));

  boxPartialKernel<<<nbBox, kThreads, 0, s>>>(F, n, w->part.as<double>());
  boxFinalKernel<<<1, 32, 0, s>>>(w->part.as<double>(), nbBox, opening, w->box.as<double>(), w->thr.as<double>(),
                                 w->dtBits.as<unsigned long long>());
  treeKeyKernel<<<blocksFor(n, kThreads), kThreads, 0, s>>>(F, n, w->box.as<double>(), w->key64.as<uint64_t>(),
                                                           w->lo.as<uint32_t>(), w->vals.as<int>());
  lc->add(3);
  uint32_t* keys = w->lo.as<uint32_t>();
  uint32_t* keysAlt = w->lo2.as<uint32_t>();
  int* vals = w->vals.as<int>();
  int* valsAlt = w->vals2.as<int>();
  radixSortPairs(keys, vals, keysAlt, valsAlt, n, 30, w->sortWs.p, s, lc);
  gatherHiKernel<<<blocksFor(n, kThreads), kThreads, 0, s>>>(w->key64.as<uint64_t>(), vals, n, keys);
  lc->add(1);
  radixSortPairs(keys, vals, keysAlt, valsAlt, n, 30, w->sortWs.p, s, lc);
  treeNodesKernel<<<blocksFor(n, kThreads), kThreads, 0, s>>>(F, w->key64.as<uint64_t>(), vals, n,
                                                             w->skey.as<uint64_t>(), w->tpos.as<TreeNode>(),
                                                             mixed ? w->tpos32.as<TreeNode32>() : nullptr);
  chainCountKernel<<<blocksFor(n, kThreads), kThreads, 0, s>>>(w->skey.as<uint64_t>(), n, w->nc.as<int>());
  lc->add(2);
  scanExclusive<int>(w->nc.as<int>(), w->off.as<long long>(), n, w->scanWs.p, w->total.as<long long>(), s, lc);
  GCHK(cudaMemcpyAsync(w->hTotal, w->total.p, sizeof(long long), cudaMemcpyDeviceToHost, s));
  GCHK(cudaStreamSynchronize(s));
  const long long numCells = *w->hTotal;
  if (numCells <= 0 || numCells > 0x7FFFFFFFll) {
    std::snprintf(err, errlen, "octree cell count %lld out of range", numCells);
    return SPHGPU_E_OVERFLOW;
  }
  w->lastCells = numCells;
  GCHK(w->cells.ensure(numCells * sizeof(TreeCell)));
  GCHK(w->mx.ensure(numCells * 3 * sizeof(double)));
  TreeCell* cells = w->cells.as<TreeCell>();
  cellBuildKernel<<<blocksFor(n, kThreads), kThreads, 0, s>>>(w->skey.as<uint64_t>(), n, w->off.as<long long>(),
                                                             numCells, cells);
  lc->add(1);
  const int nbCells = (int)((numCells + kThreads - 1) / kThreads);
  for (int l = kMaxLevel; l >= 0; --l) {
    momentKernel<<<nbCells, kThreads, 0, s>>>(cells, numCells, l, w->tpos.as<TreeNode>(), w->skey.as<uint64_t>(),
                                              w->box.as<double>(), w->mx.as<double>());
  }
  lc->add(kMaxLevel + 1);
  if (mixed) {
    GCHK(w->cells32.ensure(numCells * sizeof(TreeCell32)));
    cells32Kernel<<<nbCells, kThreads, 0, s>>>(cells, numCells, w->thr.as<double>(), w->cells32.as<TreeCell32>());
    treeWalkMixedKernel<<<nbWalk, 128, 0, s>>>(w->cells32.as<TreeCell32>(), cells, numCells,
                                               w->tpos32.as<TreeNode32>(), w->tpos.as<TreeNode>(), vals, n,
                                               w->thr.as<double>(), softening * softening, softening, G, F,
                                               w->dtBits.as<unsigned long long>(), w->energy.as<double>());
    lc->add(1);
  } else {
    treeWalkKernel<<<nbWalk, 128, 0, s>>>(cells, numCells, w->tpos.as<TreeNode>(), vals, n, w->thr.as<double>(),
                                          softening * softening, softening, G, F,
                                          w->dtBits.as<unsigned long long>(), w->energy.as<double>());
  }
  walkFinalKernel<<<1, 256, 0, s>>>(w->energy.as<double>(), nbWalk, w->dtBits.as<unsigned long long>(), G, dOut);
  lc->add(2);
  GCHK(cudaGetLastError());
  return SPHGPU_OK;
#undef GCHK
}

}  // namespace sph
