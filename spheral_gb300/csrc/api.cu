// libsphgpu host runtime: device-resident state, the neighbour-list build,
// the CheapSynchronousRK2 step orchestration and the C ABI of include/sphgpu.h.
#include "../../include/sphgpu.h"
#include "kernels.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace sph {
namespace table {
int buildBSplineTable(int numPoints, double* w, double* g, double* g2, double* nperh, double* wsum, double* meta);
int buildKernelTable(int kernel, int order, int numPoints, double* w, double* g, double* g2, double* nperh,
                     double* wsum, double* meta);
double kernelExtent(int kernel, int order);
}

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CUDA_OK(expr)                                                                        \
  do {                                                                                       \
    cudaError_t e_ = (expr);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      throw ::sph::Error(SPHGPU_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Grow-only device buffer.
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  void ensure(size_t b) {
    if (b <= bytes) return;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    CUDA_OK(cudaMalloc(&p, b));
    bytes = b;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

struct Profiler {
  bool on = false;
  struct Rec { std::string name; cudaEvent_t a, b; };
  std::vector<Rec> pending;
  std::map<std::string, std::pair<long, double>> acc;
  cudaStream_t s = nullptr;
  void begin(const char* name, cudaEvent_t* a) {
    if (!on) return;
    CUDA_OK(cudaEventCreate(a));
    CUDA_OK(cudaEventRecord(*a, s));
    (void)name;
  }
  void end(const char* name, cudaEvent_t a) {
    if (!on) return;
    cudaEvent_t b;
    CUDA_OK(cudaEventCreate(&b));
    CUDA_OK(cudaEventRecord(b, s));
    pending.push_back({name, a, b});
  }
  void collect() {
    if (pending.empty()) return;
    CUDA_OK(cudaStreamSynchronize(s));
    for (auto& r : pending) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r.a, r.b);
      auto& e = acc[r.name];
      e.first += 1;
      e.second += ms;
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    pending.clear();
  }
};

struct Scope {
  Profiler& p;
  const char* n;
  cudaEvent_t a{};
  Scope(Profiler& p_, const char* n_) : p(p_), n(n_) { p.begin(n, &a); }
  ~Scope() {
    try { p.end(n, a); } catch (...) {}
  }
};

struct Boundary {
  int type, axis;
  double lo, hi;
  int wallHigh;
};

}  // namespace sph

using namespace sph;

struct sphgpu_ctx {
  sphgpu_config cfg{};
  std::string err;
  cudaStream_t stream = nullptr;
  LaunchCounter lc;
  Profiler prof;

  // parameters
  NodeListParams lists[kMaxNodeLists]{};
  DBuf dLists;   // device copy of lists
  DBuf dvq;      // limited Q, mixed mode: FP32 copy of the Q's DvDx (3 float4 per node)
  int numLists = 0;
  std::vector<Boundary> bcs;
  HydroParams hp{};
  bool haveTable = false;
  std::vector<double> tw, tg, tg2, therm, twsum;
  double tmeta[9]{};
  DBuf dTable;   // w | g | herm (FP64) then w32 | g32

  // particles
  long n = 0;
  DBuf bankA, bankB;   // F_NUM_FIELDS * cap doubles each
  Fields F{}, Falt{};
  DBuf orig[2], list[2], cellc[2];
  DBuf inv;                  // internal index of each caller index (in-place host transfers)
  long permVersion = 0;      // bumped whenever the internal order changes
  long invVersion = -1;      // permVersion the inverse was built for
  DBuf posh, velm, thermo;   // FP32 mirrors of the pair-loop inputs
  DBuf hten;                 // ASPH: FP32 mirror of tensor H (2 float4 per node)
  DBuf vol32, rkc32;         // CRKSPH, mixed mode: FP32 mirrors of the RK volume and corrections
  double kernelExtent = 2.0; // extent of the configured base kernel (BSpline 2, NBSpline (order+1)/2)
  DBuf stage;                // host <-> device staging for caller-order transfers
  // domain decomposition: the last nGhost caller indices are halo copies of
  // other domains' nodes; xfn is called at the step's exchange points
  long nGhost = 0;
  sphgpu_exchange_fn xfn = nullptr;
  void* xuser = nullptr;
  DBuf xstage, xidx;         // exchange rows and caller indices
  DBuf v12;                  // half-step velocities + DepsDt0 of the mixed-mode energy sweep
  int cur = 0;
  long cap = 0;
  // neighbour build
  Grid grid{};
  DBuf keys, vals, keysAlt, valsAlt, sortWs, cellStart, cellEnd, counts, nbrStart, nbr, scanWs, pacc;
  size_t cellSpace = 0;
  long long nnbr = 0;
  int nbCap = 0;             // slots per node of the warp-interleaved neighbour lists (0: not sized yet)
  int nbCapNext = 0;         // smaller capacity to adopt at the next build (0: keep)
  DBuf itemFlag, items;      // work items of the warp-cooperative neighbour search
  bool haveNeighbors = false;
  // scratch
  DBuf scratch, small;
  double* hsmall = nullptr;   // pinned
  // integrator
  double time = 0.0, lastDt = 1e-5, dtMultiplier = 1.0;
  long cycle = 0;
  double dtMinAcc = 1e300, extraEnergy = 0.0;
  GravityWork* grav = nullptr;
  bool initialized = false;
  cudaEvent_t tA = nullptr, tB = nullptr;
  int itemWidth = 32;        // lanes per work item of the neighbour search
  int itemBound = 0;         // upper bound on the number of work items
  int energyVariant = -1;    // autotuned batch depth of the FP32 energy sweep
  long energyTunedN = 0;
  bool energyPinned = false; // batch depth set by the caller
  DBuf itemBox, chunkOf;     // bounding boxes of the search's work chunks, chunk of each chunk's first node
  int tunedWidth = 0;        // autotuned group width (0: not tuned yet)
  int pinnedWidth = 0;       // group width set by the caller (0: autotuned)
  // The autotuners time their options at the first use for a problem size
  // and once more kRetuneAfter uses later, when the state has moved away
  // from its initial conditions (ASPH H fields, for one, relax in the first
  // steps and change which search width is fastest).
  long listBuilds = 0, widthRetuneAt = -1;
  long pairEvals = 0, pairRetuneAt = -1;
  long energyEvals = 0, energyRetuneAt = -1;
  long widthTunedN = 0;      // node count it was tuned at
  DBuf itemCount;            // device: number of work items
  bool capCheckPending = false, totalPending = false;
  double cachedBounds[kBoundsVals] = {};   // min h^-1, min x y z, max x y z, tensor extents of the current state
  bool boundsValid = false;      // cachedBounds describe the current state
  int pairVariant = -1;      // autotuned FP32 pair-kernel variant (-1: not tuned yet)
  bool omegaStale = false;   // the end-of-step grad-h correction is owed (computed on first read)
  bool pinnedVariant = false;  // set by sphgpu_set_pair_variant
  long tunedN = 0;

  Fields fieldsOf(DBuf& bank) {
    Fields f{};
    for (int k = 0; k < F_NUM_FIELDS; ++k) f.f[k] = bank.as<double>() + (size_t)k * cap;
    return f;
  }
  int* origp() { return orig[cur].as<int>(); }
  int* listp() { return list[cur].as<int>(); }
  uint32_t* cellp() { return cellc[cur].as<uint32_t>(); }
  double maxNperh() const {
    double m = 0.0;
    for (int k = 0; k < std::max(1, numLists); ++k) m = std::max(m, lists[k].nPerh);
    return m;
  }
  TableDev tableDev() {
    TableDev t;
    const size_t nc = tw.size();
    double* base = dTable.as<double>();
    t.w = base;
    t.g = base + nc;
    t.herm = base + 2 * nc;
    float* b32 = reinterpret_cast<float*>(base + 2 * nc + therm.size());
    t.w32 = b32;
    t.g32 = b32 + nc;
    t.p32a = reinterpret_cast<const float4*>(b32 + 2 * nc);
    t.p32b = reinterpret_cast<const float2*>(b32 + 2 * nc + 4 * (nc / 3));
    return t;
  }
  NeighborLists nl() { return NeighborLists{nbr.as<uint32_t>(), counts.as<int>(), nbCap, cellp()}; }
  size_t nbSlots() const { return (size_t)((n + 31) / 32) * 32 * (size_t)nbCap; }
  Fields32 f32() {
    Fields32 p;
    p.posh = posh.as<float4>();
    p.velm = velm.as<float4>();
    p.thermo = thermo.as<float4>();
    p.cell = cellp();
    p.dvq = dvq.p ? dvq.as<float4>() : nullptr;
    p.hten = cfg.smoothing_scale != SPHGPU_SMOOTHING_SPH ? hten.as<float4>() : nullptr;
    p.vol = vol32.p ? vol32.as<float>() : nullptr;
    p.rkc = rkc32.p ? rkc32.as<float4>() : nullptr;
    return p;
  }
  bool fp32() const { return cfg.precision != SPHGPU_PRECISION_FP64; }   // FP32 sweeps (compensated or plain)
  void check() { CUDA_OK(cudaGetLastError()); }
};

namespace {

void ensureCapacity(sphgpu_ctx* c, long n) {
  if (n <= c->cap) return;
  c->cap = n;
  const size_t bytes = (size_t)F_NUM_FIELDS * n * sizeof(double);
  c->bankA.release();
  c->bankB.release();
  c->bankA.ensure(bytes);
  c->bankB.ensure(bytes);
  c->posh.release(); c->posh.ensure(n * sizeof(float4));
  c->velm.release(); c->velm.ensure(n * sizeof(float4));
  c->thermo.release(); c->thermo.ensure(n * sizeof(float4));
  c->hten.release();
  if (c->cfg.smoothing_scale != SPHGPU_SMOOTHING_SPH) c->hten.ensure(2 * n * sizeof(float4));
  c->vol32.release();
  c->rkc32.release();
  if (c->cfg.hydro == SPHGPU_HYDRO_CRKSPH && c->fp32()) {
    c->vol32.ensure(n * sizeof(float));
    c->rkc32.ensure(4 * n * sizeof(float4));
  }
  for (int k = 0; k < 2; ++k) {
    c->orig[k].release(); c->orig[k].ensure(n * sizeof(int));
    c->list[k].release(); c->list[k].ensure(n * sizeof(int));
    c->cellc[k].release(); c->cellc[k].ensure(n * sizeof(uint32_t));
  }
}

void setTable(sphgpu_ctx* c, const double* w, const double* g, const double* g2, const double* nperh,
              const double* wsum, const double* meta) {
  const int N1 = (int)meta[0];
  const int nh = (int)meta[2];
  if (N1 < 1 || 3 * (N1 + 1) > kMaxTable || nh < 3) throw Error(SPHGPU_E_ARG, "kernel table size out of range");
  const size_t nc = 3 * (size_t)(N1 + 1);
  c->tw.assign(w, w + nc);
  c->tg.assign(g, g + nc);
  c->tg2.assign(g2, g2 + nc);
  c->therm.assign(nperh, nperh + 2 * nh);
  c->twsum.assign(wsum, wsum + 2 * nh);
  std::memcpy(c->tmeta, meta, sizeof(c->tmeta));
  std::vector<double> host(2 * nc + c->therm.size());
  std::copy(c->tw.begin(), c->tw.end(), host.begin());
  std::copy(c->tg.begin(), c->tg.end(), host.begin() + nc);
  std::copy(c->therm.begin(), c->therm.end(), host.begin() + 2 * nc);
  // FP32: plain copies (2 nc floats), then packed intervals (N1+1) x (w0 w1 w2 g0) and (N1+1) x (g1 g2)
  const size_t nint = (size_t)(N1 + 1);
  std::vector<float> h32(2 * nc + 4 * nint + 2 * nint);
  for (size_t k = 0; k < nc; ++k) { h32[k] = (float)c->tw[k]; h32[nc + k] = (float)c->tg[k]; }
  for (size_t k = 0; k < nint; ++k) {
    float* A = &h32[2 * nc + 4 * k];
    A[0] = (float)c->tw[3 * k]; A[1] = (float)c->tw[3 * k + 1]; A[2] = (float)c->tw[3 * k + 2];
    A[3] = (float)c->tg[3 * k];
    float* B = &h32[2 * nc + 4 * nint + 2 * k];
    B[0] = (float)c->tg[3 * k + 1]; B[1] = (float)c->tg[3 * k + 2];
  }
  const size_t bytes = host.size() * sizeof(double) + h32.size() * sizeof(float);
  c->dTable.ensure(bytes);
  CUDA_OK(cudaMemcpy(c->dTable.p, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_OK(cudaMemcpy(static_cast<char*>(c->dTable.p) + host.size() * sizeof(double), h32.data(),
                     h32.size() * sizeof(float), cudaMemcpyHostToDevice));
  // Derived constants
  auto& hp = c->hp;
  hp.tableN1 = N1;
  hp.tableXstep = meta[1];
  hp.extent = c->kernelExtent;
  hp.W0 = 1.0 * (c->tw[0] + (c->tw[1] + c->tw[2] * 0.0) * 0.0);
  hp.hermN = nh;
  hp.hermXmin = meta[3];
  hp.hermXmax = meta[4];
  hp.hermXstep = (meta[4] - meta[3]) / (nh - 1);
  c->haveTable = true;
}

double tableW(const sphgpu_ctx* c, double eta) {   // TableKernel::kernelValue(eta, 1)
  if (!(eta < c->hp.extent)) return 0.0;
  const size_t i0 = 3u * std::min((size_t)c->hp.tableN1, size_t(std::max(0.0, eta) / c->hp.tableXstep));
  return 1.0 * (c->tw[i0] + (c->tw[i0 + 1] + c->tw[i0 + 2] * eta) * eta);
}

void refreshParams(sphgpu_ctx* c) {
  auto& hp = c->hp;
  const auto& g = c->cfg;
  hp.compatible = g.compatible_energy;
  hp.gradh = g.gradh_correction;
  hp.xsph = g.xsph;
  hp.correctVelGrad = g.correct_velocity_gradient;
  hp.sumAllLists = g.sum_mass_density_over_all_nodelists;
  hp.densityUpdate = g.density_update;
  hp.linearInExpansion = g.linear_in_expansion;
  hp.quadraticInExpansion = g.quadratic_in_expansion;
  hp.useVelMagDt = g.use_velocity_magnitude_for_dt;
  hp.epsTensile = g.eps_tensile;
  hp.nTensile = g.n_tensile;
  hp.Cl = g.Cl;
  hp.Cq = g.Cq;
  hp.eps2 = g.eps2;
  hp.cfl = g.cfl;
  hp.numLists = std::max(1, c->numLists);
  // LimitedMonaghanGingoldViscosity: etaCrit = etaCritFrac / nPerh of the first
  // NodeList (LimitedMonaghanGingoldViscosity.cc:148-154)
  hp.limitedQ = g.viscosity == SPHGPU_VISCOSITY_LIMITED_MONAGHAN_GINGOLD ? 1 : 0;
  hp.etaCrit = g.eta_crit_frac / c->lists[0].nPerh;
  hp.etaFold = g.eta_fold_frac / c->lists[0].nPerh;
  hp.asph = g.smoothing_scale != SPHGPU_SMOOTHING_SPH ? 1 : 0;   // tensor H
  hp.asphEnd = g.smoothing_scale == SPHGPU_SMOOTHING_ASPH ? 1 : 0;
  hp.fixShape = g.fix_shape ? 1 : 0;
  hp.hUpdate = g.h_update;
  hp.totalEnergy = g.evolve_total_energy ? 1 : 0;
  hp.radialOnly = g.radial_only ? 1 : 0;
  hp.crk = g.hydro == SPHGPU_HYDRO_CRKSPH ? 1 : 0;
  hp.rkVolume = g.rk_volume;
  hp.plainSums = g.precision == SPHGPU_PRECISION_FP32_PLAIN ? 1 : 0;
  if (c->haveTable) hp.WnPerh = tableW(c, 1.0 / c->lists[0].nPerh);
  // NodeList table in device memory, one per handle (handles on different
  // streams never share it).
  for (auto& L : c->lists) {
    L.gm1 = L.gamma - 1.0;
    L.ggm1 = L.gamma * L.gm1;
  }
  c->dLists.ensure(sizeof(c->lists));
  CUDA_OK(cudaMemcpyAsync(c->dLists.p, c->lists, sizeof(c->lists), cudaMemcpyHostToDevice, c->stream));
  hp.lists = c->dLists.as<NodeListParams>();
}

void requireState(sphgpu_ctx* c) {
  if (!c->haveTable) throw Error(SPHGPU_E_STATE, "no kernel table installed");
  if (c->n <= 0) throw Error(SPHGPU_E_STATE, "no particles");
}

//------------------------------------------------------------------------------
// Grid for the cell list: periodic axes span their planes, reflecting walls
// bound their side, open sides follow the bounding box.  Cells are at least
// kernelExtent * hmax (strictly larger, so every interacting pair lies in
// adjacent cells).
//------------------------------------------------------------------------------
void buildGrid(sphgpu_ctx* c) {
  Scope sc(c->prof, "bounds");
  if (!c->boundsValid) {   // the bounds of the last step's check describe a changed state
    double* d = c->small.as<double>() + 20;
    c->scratch.ensure(kBoundsVals * sizeof(double) * 4096);
    launchBounds(c->F, c->n, c->hp.asph != 0, c->scratch.as<double>(), kBoundsVals * 4096, d, c->stream, &c->lc);
    c->check();
    CUDA_OK(cudaMemcpyAsync(c->hsmall + 20, d, kBoundsVals * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_OK(cudaStreamSynchronize(c->stream));
    std::memcpy(c->cachedBounds, c->hsmall + 20, sizeof(c->cachedBounds));
  }
  c->boundsValid = false;   // consumed: the step moves the nodes
  const double* bnd = c->cachedBounds;
  const double minHinv = bnd[0];
  if (!(minHinv > 0.0) || !std::isfinite(minHinv)) throw Error(SPHGPU_E_NAN, "non-positive or non-finite H");
  const double hmax = 1.0 / minHinv;
  const double support = c->hp.extent * hmax * (1.0 + 1.0e-9);
  // tensor H: every neighbour r_ij lies in ext E_i or ext E_j (E the unit
  // ellipsoid of H), whose half-width along axis a is sqrt((H^-2)_aa): the
  // cells follow the largest half-width per axis (with a margin for the
  // rounding of the inverse)
  double supportAxis[3] = {support, support, support};
  if (c->hp.asph)
    for (int a = 0; a < 3; ++a) supportAxis[a] = c->hp.extent * bnd[7 + a] * (1.0 + 1.0e-9);
  Grid g{};
  for (int a = 0; a < 3; ++a) {
    g.kindLo[a] = g.kindHi[a] = AXIS_OPEN;
    g.wallLo[a] = bnd[1 + a];
    g.wallHi[a] = bnd[4 + a];
  }
  for (const auto& b : c->bcs) {
    if (b.type == SPHGPU_BOUNDARY_PERIODIC) {
      g.kindLo[b.axis] = g.kindHi[b.axis] = AXIS_PERIODIC;
      g.wallLo[b.axis] = b.lo;
      g.wallHi[b.axis] = b.hi;
    } else if (b.wallHigh) {
      g.kindHi[b.axis] = AXIS_REFLECT;
      g.wallHi[b.axis] = b.hi;
    } else {
      g.kindLo[b.axis] = AXIS_REFLECT;
      g.wallLo[b.axis] = b.lo;
    }
  }
  int ncA[3];
  for (int a = 0; a < 3; ++a) {
    const double lo = g.kindLo[a] == AXIS_OPEN ? bnd[1 + a] : g.wallLo[a];
    const double hi = g.kindHi[a] == AXIS_OPEN ? bnd[4 + a] : g.wallHi[a];
    int nc = (int)std::min(1024.0, std::floor((hi - lo) / supportAxis[a]));
    if (g.kindLo[a] == AXIS_PERIODIC) {
      if (nc < 3)
        throw Error(SPHGPU_E_UNSUPPORTED,
                    "periodic box narrower than three kernel supports on axis " + std::to_string(a));
    } else {
      nc = std::max(1, nc);
    }
    ncA[a] = nc;
  }
  // A sparse or spread-out node set would ask for far more cells than nodes
  // (and cell tables as large as the key space): coarsen the widest axis
  // until the cells number at most max(4096, 8 n).  Larger cells only add
  // candidates; periodic axes keep at least three.
  const double cellCap = std::max(4096.0, 8.0 * (double)c->n);
  while ((double)ncA[0] * ncA[1] * ncA[2] > cellCap) {
    int a = -1;
    for (int b = 0; b < 3; ++b) {
      const int minNc = g.kindLo[b] == AXIS_PERIODIC ? 3 : 1;
      if (ncA[b] > minNc && (a < 0 || ncA[b] > ncA[a])) a = b;
    }
    if (a < 0) break;
    const int minNc = g.kindLo[a] == AXIS_PERIODIC ? 3 : 1;
    ncA[a] = std::max(minNc, (int)(ncA[a] * 0.8));
  }
  for (int a = 0; a < 3; ++a) {
    const double lo = g.kindLo[a] == AXIS_OPEN ? bnd[1 + a] : g.wallLo[a];
    const double hi = g.kindHi[a] == AXIS_OPEN ? bnd[4 + a] : g.wallHi[a];
    const double L = hi - lo;
    const double support = supportAxis[a];
    const int nc = ncA[a];
    // cell >= support: every interacting pair sits in adjacent cells
    const double cell = std::max(L / nc, support);
    g.lo[a] = lo;
    g.hi[a] = hi;
    g.cell[a] = cell;
    g.inv2[a] = 2.0 / cell;
    g.cellf[a] = (float)cell;
    g.nc[a] = nc;
    if (g.kindLo[a] != AXIS_PERIODIC) {   // open sides: the grid origin follows the data
      if (g.kindLo[a] == AXIS_OPEN) g.wallLo[a] = lo;
      if (g.kindHi[a] == AXIS_OPEN) g.wallHi[a] = hi;
    }
  }
  g.ext2f = (float)(c->hp.extent * c->hp.extent);
  c->grid = g;
}

int capFor(int m) { return std::max(32, ((m + m / 8 + 16 + 31) / 32) * 32); }
int* maxCountPtr(sphgpu_ctx* c) { return reinterpret_cast<int*>(c->small.as<double>() + 40); }
int readMaxCount(sphgpu_ctx* c) {
  CUDA_OK(cudaMemcpyAsync(c->hsmall + 40, maxCountPtr(c), sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  int m;
  std::memcpy(&m, c->hsmall + 40, sizeof(int));
  return m;
}
// Write pass of the neighbour search into lists of capacity nbCap; the
// largest count lands in the maxCount slot.
void writeLists(sphgpu_ctx* c) {
  c->nbr.ensure(std::max<size_t>(1, c->nbSlots()) * sizeof(uint32_t));
  CUDA_OK(cudaMemsetAsync(maxCountPtr(c), 0, sizeof(int), c->stream));
  Scope sc(c->prof, "neighbors");
  launchNeighborsWarp(c->F, c->f32(), c->n, c->items.as<int>(), c->itemBound, c->itemCount.as<long long>(),
                      c->itemWidth, c->grid, c->cellStart.as<int>(), c->cellEnd.as<int>(), c->counts.as<int>(),
                      maxCountPtr(c), c->nbr.as<uint32_t>(), c->nbCap, c->hp.extent * c->hp.extent, c->hp.asph != 0,
                      c->itemBox.as<float4>(), c->chunkOf.as<int>(), c->stream, &c->lc);
  c->check();
}
// CSR offsets of the lists (caller-order transfers) and their total, read
// back without a synchronisation.
void scanTotals(sphgpu_ctx* c) {
  const long n = c->n;
  long long* dTot = c->nbrStart.as<long long>() + n;
  scanExclusive<int>(c->counts.as<int>(), c->nbrStart.as<long long>(), n, c->scanWs.p, dTot, c->stream, &c->lc);
  c->check();
  CUDA_OK(cudaMemcpyAsync(c->hsmall + 42, dTot, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
  c->totalPending = true;
}
bool resolveNeighbors(sphgpu_ctx* c);

//------------------------------------------------------------------------------
// Neighbour build: cell keys -> stable radix sort -> permute every field ->
// cell ranges -> count -> scan -> fill.
//------------------------------------------------------------------------------
// inStep: called at the start of sphgpu_step -- the capacity check is left
// to the step's dt synchronisation and only the carried fields are permuted
// (the step rewrites the others before it returns).
void buildNeighbors(sphgpu_ctx* c, bool inStep = false) {
  const bool deferCheck = inStep;
  const long n = c->n;
  buildGrid(c);
  int bitsAxis = 0;
  while ((1 << bitsAxis) < std::max(c->grid.nc[0], std::max(c->grid.nc[1], c->grid.nc[2]))) ++bitsAxis;
  // one sub-cell Morton level in the sort key while it fits 30 bits
  c->grid.subShift = bitsAxis <= 9 ? 3 : 0;
  const Grid& g = c->grid;
  const int keyBits = std::max(1, 3 * bitsAxis);            // bits of the cell key
  const int sortBits = keyBits + g.subShift;                // bits of the sort key
  c->keys.ensure(n * sizeof(uint32_t));
  c->keysAlt.ensure(n * sizeof(uint32_t));
  c->vals.ensure(n * sizeof(int));
  c->valsAlt.ensure(n * sizeof(int));
  c->sortWs.ensure(radixSortWorkspaceBytes(n));
  {
    Scope sc(c->prof, "cell_keys");
    launchCellKeys(c->F, n, g, c->keys.as<uint32_t>(), c->vals.as<int>(), c->cellp(), c->stream, &c->lc);
  }
  uint32_t* k = c->keys.as<uint32_t>();
  int* v = c->vals.as<int>();
  uint32_t* ka = c->keysAlt.as<uint32_t>();
  int* va = c->valsAlt.as<int>();
  {
    Scope sc(c->prof, "radix_sort");
    radixSortPairs(k, v, ka, va, n, ((sortBits + 7) / 8) * 8, c->sortWs.p, c->stream, &c->lc);
  }
  c->check();
  {
    Scope sc(c->prof, "permute");
    const int nx = 1 - c->cur;
    launchPermute(c->F, c->Falt, v, c->orig[c->cur].as<int>(), c->orig[nx].as<int>(), c->list[c->cur].as<int>(),
                  c->list[nx].as<int>(), c->cellc[c->cur].as<uint32_t>(), c->cellc[nx].as<uint32_t>(), n,
                  inStep, c->hp.asph != 0, c->hp.crk != 0, c->stream, &c->lc);
    std::swap(c->bankA, c->bankB);
    std::swap(c->F, c->Falt);
    c->cur = nx;
    ++c->permVersion;
  }
  c->check();
  const size_t space = (size_t)1 << keyBits;
  if (space > c->cellSpace) {
    c->cellStart.release(); c->cellEnd.release();
    c->cellStart.ensure(space * sizeof(int));
    c->cellEnd.ensure(space * sizeof(int));
    c->cellSpace = space;
  }
  CUDA_OK(cudaMemsetAsync(c->cellStart.p, 0, space * sizeof(int), c->stream));
  CUDA_OK(cudaMemsetAsync(c->cellEnd.p, 0, space * sizeof(int), c->stream));
  {
    Scope sc(c->prof, "cell_ranges");
    launchCellRanges(k, n, g.subShift, c->cellStart.as<int>(), c->cellEnd.as<int>(), c->stream, &c->lc);
  }
  {
    Scope sc(c->prof, "prepare_fp32");
    launchPrepareFP32(c->F, c->f32(), n, g, c->stream, &c->lc);
  }
  c->counts.ensure(n * sizeof(int));
  c->nbrStart.ensure((n + 1) * sizeof(long long));
  c->scanWs.ensure(scanWorkspaceBytes(n) + 64);
  c->itemCount.ensure(sizeof(long long));
  // work items: first node of every chunk of up to `width` nodes of a cell.
  // The first guess of the group width follows the mean occupancy of the
  // cells so that few lanes of a group idle; the autotuner below then times
  // the widths once per problem size.
  const double cellsTotal = (double)g.nc[0] * g.nc[1] * g.nc[2];
  const double occupancy = (double)n / cellsTotal;
  const int guess = occupancy >= 24.0 ? 32 : (occupancy >= 12.0 ? 16 : 8);
  ++c->listBuilds;
  const bool retuneWidth = c->widthRetuneAt >= 0 && c->listBuilds >= c->widthRetuneAt;
  const bool tuned = c->pinnedWidth > 0 ||
                     (!retuneWidth && c->tunedWidth > 0 && std::labs(n - c->widthTunedN) <= c->widthTunedN / 8);
  c->itemFlag.ensure(n * sizeof(int));
  c->items.ensure(n * sizeof(int));
  c->itemBox.ensure(2 * (size_t)n * sizeof(float4));
  c->chunkOf.ensure(n * sizeof(int));
  auto makeItems = [&](int width) {
    c->itemWidth = width;
    // every non-empty cell adds at most one partial chunk
    c->itemBound = (int)std::min<double>((double)n, (double)(n / width) + cellsTotal);
    Scope sc(c->prof, "neighbor_items");
    long long* pos = c->nbrStart.as<long long>();
    launchItemFlags(k, n, g.subShift, c->cellStart.as<int>(), width, c->itemFlag.as<int>(), c->stream, &c->lc);
    scanExclusive<int>(c->itemFlag.as<int>(), pos, n, c->scanWs.p, c->itemCount.as<long long>(), c->stream, &c->lc);
    launchItemFill(c->itemFlag.as<int>(), pos, n, c->items.as<int>(), c->stream, &c->lc);
    launchItemBoxes(c->items.as<int>(), c->itemCount.as<long long>(), c->itemBound, n, width, c->f32(),
                    c->itemBox.as<float4>(), c->chunkOf.as<int>(), c->stream, &c->lc);
    c->check();
  };
  makeItems(c->pinnedWidth > 0 ? c->pinnedWidth : (tuned ? c->tunedWidth : guess));
  if (c->nbCapNext > 0) {   // adopt a smaller capacity decided at the previous build
    c->nbCap = c->nbCapNext;
    c->nbCapNext = 0;
  }
  if (c->nbCap == 0) {   // first build: size the lists with a counting pass
    int* dMax = maxCountPtr(c);
    CUDA_OK(cudaMemsetAsync(dMax, 0, sizeof(int), c->stream));
    Scope sc(c->prof, "neighbor_count");
    launchNeighborsWarp(c->F, c->f32(), n, c->items.as<int>(), c->itemBound, c->itemCount.as<long long>(),
                        c->itemWidth, g, c->cellStart.as<int>(), c->cellEnd.as<int>(), c->counts.as<int>(), dMax,
                        nullptr, 0, c->hp.extent * c->hp.extent, c->hp.asph != 0, c->itemBox.as<float4>(),
                        c->chunkOf.as<int>(), c->stream, &c->lc);
    c->check();
    c->nbCap = capFor(readMaxCount(c));
  }
  if (!tuned) {
    // Autotuner: the lists do not depend on the group width (the candidate
    // order is the cell order in every width), so each width writes them
    // once, timed, and the fastest is kept for this problem size.
    cudaEvent_t e0, e1;
    CUDA_OK(cudaEventCreate(&e0));
    CUDA_OK(cudaEventCreate(&e1));
    // two rounds, best time per width: the first launches after a new
    // build run on cold caches
    float best = 1e30f;
    int bestW = guess;
    for (int round = 0; round < 2; ++round)
      for (const int w : {8, 16, 32}) {
        if (w != c->itemWidth) makeItems(w);
        CUDA_OK(cudaEventRecord(e0, c->stream));
        writeLists(c);
        CUDA_OK(cudaEventRecord(e1, c->stream));
        CUDA_OK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) { best = ms; bestW = w; }
      }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->tunedWidth = bestW;
    c->widthTunedN = n;
    c->widthRetuneAt = retuneWidth ? -1 : c->listBuilds + kRetuneAfter;
    if (bestW != c->itemWidth) makeItems(bestW);
  }
  writeLists(c);
  if (deferCheck) {
    // The capacity check and the entry total are read at the caller's next
    // stream synchronisation (resolveNeighbors).
    CUDA_OK(cudaMemcpyAsync(c->hsmall + 40, maxCountPtr(c), sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    c->capCheckPending = true;
  } else {
    while (true) {
      const int m = readMaxCount(c);
      if (m <= c->nbCap) {
        if (capFor(m) * 2 < c->nbCap) c->nbCapNext = capFor(m);   // shrink at the next build, not now
        break;
      }
      c->nbCap = capFor(m);   // overflow: enlarge and rewrite
      writeLists(c);
    }
  }
  scanTotals(c);
  c->haveNeighbors = true;
  if (!deferCheck) resolveNeighbors(c);
}

// Reads the deferred capacity check and entry total after a stream
// synchronisation.  Returns true when the lists overflowed and were rewritten
// with a larger capacity (the caller must redo sweeps that used them).
bool resolveNeighbors(sphgpu_ctx* c) {
  bool regrown = false;
  if (c->capCheckPending) {
    c->capCheckPending = false;
    int m;
    std::memcpy(&m, c->hsmall + 40, sizeof(int));
    if (m > c->nbCap) {
      do {
        c->nbCap = capFor(m);
        writeLists(c);
        m = readMaxCount(c);
      } while (m > c->nbCap);
      scanTotals(c);
      regrown = true;
    } else if (capFor(m) * 2 < c->nbCap) {
      c->nbCapNext = capFor(m);
    }
  }
  if (c->totalPending) {
    CUDA_OK(cudaStreamSynchronize(c->stream));
    std::memcpy(&c->nnbr, c->hsmall + 42, sizeof(long long));
    c->totalPending = false;
  }
  return regrown;
}

void ensurePacc(sphgpu_ctx* c) {
  const size_t per = c->fp32() ? sizeof(float) : sizeof(double);
  c->pacc.ensure(std::max<size_t>(1, c->nbSlots()) * 3 * per);
}

// LimitedMonaghanGingoldViscosity reads the Q's own copy of DvDx, refreshed
// from the hydro's at every postStateUpdate (ArtificialViscosityHandle.cc:167-183).
void copyQGradient(sphgpu_ctx* c) {
  if (!c->hp.limitedQ) return;
  Scope sc(c->prof, "update");
  launchCopyQGradient(c->F, c->n, c->stream, &c->lc);
  c->check();
}

void prepare32(sphgpu_ctx* c) {
  if (!c->fp32()) return;
  Scope sc(c->prof, "prepare_fp32");
  launchPrepareFP32(c->F, c->f32(), c->n, c->grid, c->stream, &c->lc);
  c->check();
}
void sumDensity(sphgpu_ctx* c) {
  Scope sc(c->prof, "sum_density");
  if (c->hp.crk && c->fp32())   // computeCRKSPHSumMassDensity with the current RK volumes
    launchCRKDensityFP32(c->F, c->f32(), c->listp(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
  else if (c->hp.crk)
    launchCRKDensity(c->F, c->listp(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
  else if (c->fp32())
    launchSumDensityFP32(c->F, c->f32(), c->listp(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
  else
    launchSumDensity(c->F, c->listp(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
  c->check();
}
void gradh(sphgpu_ctx* c) {
  Scope sc(c->prof, "gradh");
  if (c->fp32())
    launchGradhFP32(c->F, c->f32(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
  else
    launchGradh(c->F, c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
  c->check();
}
void settleOmega(sphgpu_ctx* c) {
  if (!c->omegaStale) return;
  gradh(c);
  c->omegaStale = false;
}

void evalDerivs(sphgpu_ctx* c) {
  ensurePacc(c);
  if (c->fp32() && c->hp.limitedQ) {   // FP32 mirror of the Q's DvDx in the current node order
    c->dvq.ensure((size_t)c->n * 3 * sizeof(float4));
    launchQGradient32(c->F, c->dvq.as<float4>(), c->n, c->stream, &c->lc);
    c->check();
  }
  // Autotuner of the mixed pair kernels: time each variant (register budget,
  // loop form) twice per problem size and again two uses later (the kernel
  // is a pure function of its inputs and every variant gives the same bits,
  // so the trial launches leave the results unchanged) and keep the fastest.
  auto tunePair = [&](int nv, auto launch) {
    ++c->pairEvals;
    const bool retune = c->pairRetuneAt >= 0 && c->pairEvals >= c->pairRetuneAt;
    if (c->pinnedVariant || !(c->pairVariant < 0 || c->tunedN != c->n || retune)) return;
    cudaEvent_t e0, e1;
    CUDA_OK(cudaEventCreate(&e0));
    CUDA_OK(cudaEventCreate(&e1));
    float best = 1e30f;
    int bestV = 0;
    for (int t = 0; t < 2 * nv; ++t) {   // two rounds, best time per variant
      const int v = t % nv;
      CUDA_OK(cudaEventRecord(e0, c->stream));
      launch(v);
      CUDA_OK(cudaEventRecord(e1, c->stream));
      CUDA_OK(cudaEventSynchronize(e1));
      c->check();
      float ms = 0.f;
      CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) { best = ms; bestV = v; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->pairVariant = bestV;
    c->tunedN = c->n;
    c->pairRetuneAt = retune ? -1 : c->pairEvals + kRetuneAfter;
  };
  if (c->hp.crk && c->fp32()) {
    // RKCorrections::initialize, then CRKSPH::evaluateDerivatives, FP32 sweeps
    {
      Scope sc(c->prof, "rk_corrections");
      launchRKCorrectionsFP32(c->F, c->f32(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
    }
    auto crkPair = [&](int v) {
      launchPairCRKFP32(c->F, c->f32(), c->listp(), c->n, c->grid, c->nl(), c->tableDev(), c->hp,
                        c->pacc.as<float>(), v, c->stream, &c->lc);
    };
    tunePair(kPairVariantsCRK, crkPair);
    Scope sc(c->prof, "pair_crk");
    crkPair(c->pairVariant);
  } else if (c->fp32()) {
    auto pair = [&](int v) {
      launchPairFP32(c->F, c->f32(), c->listp(), c->n, c->grid, c->nl(), c->tableDev(), c->hp,
                     c->pacc.as<float>(), v, c->stream, &c->lc);
    };
    tunePair(c->hp.asph ? kPairVariantsTensor : kPairVariants, pair);
    Scope sc(c->prof, "pair_fp32");
    pair(c->pairVariant);
  } else if (c->hp.crk) {
    // RKCorrections::initialize (the integrator's initializeDerivatives) on
    // the state being evaluated, then CRKSPH::evaluateDerivatives
    {
      Scope sc(c->prof, "rk_corrections");
      launchRKCorrections(c->F, c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
    }
    Scope sc(c->prof, "pair_crk");
    launchPairCRK(c->F, c->listp(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->pacc.as<double>(), c->stream,
                  &c->lc);
  } else {
    Scope sc(c->prof, "pair_fp64");
    launchPairFP64(c->F, c->listp(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->pacc.as<double>(),
                   128, c->stream, &c->lc);
  }
  c->check();
  if (c->cfg.gravity) {
    Scope sc(c->prof, "gravity");
    char msg[256] = {0};
    double* d = c->small.as<double>() + 16;
    const int rc = gravityEvaluate(c->grav, c->F, c->n, c->cfg.G, c->cfg.softening, c->cfg.opening, c->fp32(), d,
                                   c->stream,
                                   &c->lc, msg, sizeof(msg));
    if (rc != SPHGPU_OK) throw Error(rc, std::string("gravity: ") + msg);
    CUDA_OK(cudaMemcpyAsync(c->hsmall + 16, d, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_OK(cudaStreamSynchronize(c->stream));
    c->dtMinAcc = c->hsmall[16];
    c->extraEnergy = c->hsmall[17];
  }
}

// Integrator::selectDt (src/Integrator/Integrator.cc:116-169).
// fusedDone: the mixed-mode density sweep already left the dt vote in small[0..1].
// Halo copies take no part in the dt vote: the vote kernels read the caller
// index of each sorted node (the current bank) and the owned count.
void setGhostParams(sphgpu_ctx* c) {
  c->hp.ghostOrig = c->nGhost > 0 ? c->origp() : nullptr;
  c->hp.nOwn = c->n - c->nGhost;
}

double packageDt(sphgpu_ctx* c, int* reason, bool fusedDone = false) {
  Scope sc(c->prof, "dt");
  setGhostParams(c);
  const long nb = (c->n + 127) / 128;
  c->scratch.ensure(std::max<size_t>(2 * nb * sizeof(double), 7 * sizeof(double) * 4096));
  double* d = c->small.as<double>();
  if (fusedDone) {
  } else if (c->fp32())
    launchDtFP32(c->F, c->f32(), c->listp(), c->n, c->grid, c->nl(), c->hp, c->maxNperh(),
                 c->scratch.as<double>(), (int)(2 * nb), d, c->stream, &c->lc);
  else
    launchDt(c->F, c->listp(), c->n, c->grid, c->nl(), c->hp, c->maxNperh(), c->scratch.as<double>(),
             (int)(2 * nb), d, c->stream, &c->lc);
  c->check();
  CUDA_OK(cudaMemcpyAsync(c->hsmall, d, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  double dt = c->hsmall[0] * c->cfg.cfl;
  int r = (int)c->hsmall[1];
  if (c->cfg.gravity) {
    const double gdt = c->cfg.ftimestep * c->dtMinAcc;
    if (gdt < dt) { dt = gdt; r = 6; }
  }
  if (reason) *reason = r;
  return dt;
}

double selectDt(sphgpu_ctx* c, double dtMin, double dtMax, bool fusedDone = false) {
  double dt = dtMax;
  int r;
  const double v = packageDt(c, &r, fusedDone);
  if (v > 0.0 && v < dt) dt = v;
  dt *= c->dtMultiplier;
  dt = std::min(dt, c->cfg.dt_growth * c->lastDt);
  dt = std::min(dtMax, std::max(dtMin, dt));
  return dt;
}

// The end-of-step check also takes the bounds the next neighbour build needs
// (min h^-1, bounding box), read back in the same synchronisation.
void checkState(sphgpu_ctx* c, const char* where) {
  int* flag = reinterpret_cast<int*>(c->small.as<double>() + 30);
  CUDA_OK(cudaMemsetAsync(flag, 0, sizeof(int), c->stream));
  launchCheckState(c->F, c->n, flag, c->stream, &c->lc);
  double* b = c->small.as<double>() + 20;
  c->scratch.ensure(kBoundsVals * sizeof(double) * 4096);
  launchBounds(c->F, c->n, c->hp.asph != 0, c->scratch.as<double>(), kBoundsVals * 4096, b, c->stream, &c->lc);
  CUDA_OK(cudaMemcpyAsync(c->hsmall + 20, b, kBoundsVals * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaMemcpyAsync(c->hsmall + 30, flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  int h;
  std::memcpy(&h, c->hsmall + 30, sizeof(int));
  if (h) throw Error(SPHGPU_E_NAN, std::string("non-finite or non-positive state after ") + where);
  std::memcpy(c->cachedBounds, c->hsmall + 20, sizeof(c->cachedBounds));
  c->boundsValid = true;
}

// Domain decomposition (DistributedBoundary::applyGhostBoundaries,
// src/Distributed/DistributedBoundary.cc): the caller's exchange function
// refreshes the halo copies at the points of the step where a neighbour sum
// has changed a field they are read for.  Every domain reaches the same
// points in the same order once per step.
void exchangePoint(sphgpu_ctx* c, int point, double* dt = nullptr) {
  if (!c->xfn) return;
  const int rc = c->xfn(c->xuser, point, dt);
  if (rc != 0) throw Error(SPHGPU_E_STATE, "the domain exchange function failed at point " + std::to_string(point));
}

// CheapSynchronousRK2::step (src/Integrator/CheapSynchronousRK2.cc:40-132).
double step(sphgpu_ctx* c, double maxTime) {
  requireState(c);
  refreshParams(c);
  buildNeighbors(c, true);                           // Integrator::setGhostNodes + connectivity
  bool fused = false;
  auto preStep = [&]() {
    if (c->hp.radialOnly) launchRadius0(c->F, c->n, c->stream, &c->lc);   // SmoothingScaleBase::preStepInitialize
    if (c->hp.crk) {   // RKCorrections::preStepInitialize: the RK volumes
      Scope sc(c->prof, "rk_volume");
      if (c->fp32())
        launchRKVolumesFP32(c->F, c->f32(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
      else
        launchRKVolumes(c->F, c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
    }
    if (c->cfg.density_update == SPHGPU_DENSITY_RIGOROUS_SUM) {   // preStepInitialize (+ dt vote when mixed SPH)
      if (c->fp32() && !c->hp.crk) {
        Scope sc(c->prof, "density_dt");
        const long nb = (c->n + 127) / 128;
        c->scratch.ensure(std::max<size_t>(2 * nb * sizeof(double), 7 * sizeof(double) * 4096));
        setGhostParams(c);
        launchDensityDtFP32(c->F, c->f32(), c->listp(), c->n, c->grid, c->nl(), c->tableDev(), c->hp,
                            c->maxNperh(), c->scratch.as<double>(), c->small.as<double>(), c->stream, &c->lc);
        c->check();
        fused = true;
      } else {
        sumDensity(c);
      }
    }
  };
  preStep();
  const double t = c->time;
  double dt = selectDt(c, std::min(c->cfg.dt_min, maxTime - t), std::min(c->cfg.dt_max, maxTime - t), fused);
  // The dt read synchronised the stream: settle the deferred list check.  A
  // list that overflowed its capacity was rewritten larger; redo the sweeps
  // that read it.
  if (resolveNeighbors(c)) {
    preStep();
    dt = selectDt(c, std::min(c->cfg.dt_min, maxTime - t), std::min(c->cfg.dt_max, maxTime - t), fused);
  }
  if (c->xfn) {
    exchangePoint(c, SPHGPU_EXCHANGE_DENSITY);   // the halo's summed densities
    exchangePoint(c, SPHGPU_EXCHANGE_DT, &dt);   // the smallest vote of all domains
    if (!(dt > 0.0) || !std::isfinite(dt)) throw Error(SPHGPU_E_STATE, "the domain exchange returned a bad dt");
  }
  const double hdt = 0.5 * dt;
  {
    Scope sc(c->prof, "update");   // the half-step update also saves state0
    const Fields32 m32 = c->f32();
    launchUpdate(c->F, c->listp(), c->n, c->hp, hdt, true, c->cfg.gravity != 0, c->fp32() ? &m32 : nullptr, c->grid,
                 c->stream, &c->lc);
  }
  c->check();
  c->time = t + hdt;
  copyQGradient(c);                                  // postStateUpdate (mid): the Q's DvDx
  if (c->cfg.gradh_correction) gradh(c);             // postStateUpdate (mid)
  c->omegaStale = false;
  if (c->cfg.gradh_correction) exchangePoint(c, SPHGPU_EXCHANGE_OMEGA);
  evalDerivs(c);                                     // derivs.Zero(); evaluateDerivatives(t + dt/2)
  exchangePoint(c, SPHGPU_EXCHANGE_DERIVS);          // the halo's accelerations and energy rates
  {
    Scope sc(c->prof, "update");
    launchRestoreState0(c->F, c->n, c->hp.asph != 0, c->hp.crk != 0, c->stream, &c->lc);
  }
  if (c->cfg.compatible_energy) {
    Scope sc(c->prof, "energy");
    if (c->fp32()) {
      c->v12.ensure(c->n * 2 * sizeof(float4));
      ++c->energyEvals;
      const bool retune = c->energyRetuneAt >= 0 && c->energyEvals >= c->energyRetuneAt;
      if (!c->energyPinned &&
          (c->energyVariant < 0 || std::labs(c->n - c->energyTunedN) > c->energyTunedN / 8 || retune)) {
        // Autotuner: time each batch depth once per problem size.  The trial
        // launches take dt = 0, so they add nothing to the energies; the
        // real launch below recomputes everything they wrote.
        cudaEvent_t e0, e1;
        CUDA_OK(cudaEventCreate(&e0));
        CUDA_OK(cudaEventCreate(&e1));
        float best = 1e30f;
        int bestV = 0;
        for (int t = 0; t < 2 * kEnergyVariants; ++t) {   // two rounds, best time per variant
          const int v = t % kEnergyVariants;
          CUDA_OK(cudaEventRecord(e0, c->stream));
          launchCompatibleEnergyFP32(c->F, c->n, c->grid, c->nl(), c->pacc.as<float>(), c->v12.as<float4>(),
                                     c->v12.as<float4>() + c->n, 0.0, v, c->stream, &c->lc);
          CUDA_OK(cudaEventRecord(e1, c->stream));
          CUDA_OK(cudaEventSynchronize(e1));
          c->check();
          float ms = 0.f;
          CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
          if (ms < best) { best = ms; bestV = v; }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        c->energyVariant = bestV;
        c->energyTunedN = c->n;
        c->energyRetuneAt = retune ? -1 : c->energyEvals + kRetuneAfter;
      }
      launchCompatibleEnergyFP32(c->F, c->n, c->grid, c->nl(), c->pacc.as<float>(), c->v12.as<float4>(),
                                 c->v12.as<float4>() + c->n, dt, c->energyVariant, c->stream, &c->lc);
    }
    else
      launchCompatibleEnergy(c->F, c->n, c->grid, c->nl(), c->pacc.as<double>(), nullptr, dt, c->stream, &c->lc);
  }
  {
    Scope sc(c->prof, "update");
    const Fields32 m32 = c->f32();
    launchUpdate(c->F, c->listp(), c->n, c->hp, dt, false, c->cfg.gravity != 0, c->fp32() ? &m32 : nullptr, c->grid,
                 c->stream, &c->lc);
  }
  c->check();
  c->time = t + dt;
  copyQGradient(c);                                  // postStateUpdate (end): the Q's DvDx
  // postStateUpdate (end): the grad-h correction of the new state.  Nothing
  // of the next step reads it before the half-step postStateUpdate computes
  // it again (the density sum, the dt vote and the half-step update do not
  // use it), so it is owed rather than computed: every read of the state
  // outside a step (fields, derivatives, checkpoints, a refresh of the FP32
  // mirror) settles it first on these same lists.  The FP32 sweep reads only
  // the mirror this update wrote, which the boundary enforcement below leaves
  // alone, so the settled values are those of an eager evaluation; the FP64
  // sweep reads the FP64 positions, so it is owed only when no wall or period
  // can move a node after it.
  if (c->cfg.gradh_correction) {
    // ASPHSmoothingScale changes H after this point: its Omega is the one of
    // the H before that change, so it is computed now
    if ((c->fp32() || c->bcs.empty()) && !c->hp.asphEnd) c->omegaStale = true;
    else gradh(c);
  }
  if (c->hp.asphEnd) {   // postStepFinalize: ASPHSmoothingScale::finalize
    Scope sc(c->prof, "asph_end");
    launchASPHEnd(c->F, c->fp32() ? c->f32() : Fields32{}, c->listp(), c->n, c->grid, c->nl(), c->tableDev(), c->hp,
                  c->stream, &c->lc);
    c->check();
  }
  {
    Scope sc(c->prof, "enforce");
    launchEnforce(c->F, c->n, c->grid, c->hp.asph != 0, c->stream, &c->lc);
  }
  c->check();
  checkState(c, "the step");
  c->cycle += 1;
  c->lastDt = dt;
  return dt;
}

struct FieldSpec {
  int first;
  int ncomp;
};
// asph: H, Hideal and DHDt are the tensor fields (and massSecondMoment exists).
bool fieldSpec(const std::string& s, FieldSpec& fs, bool& isH, bool& isNumNb, bool asph, bool crk) {
  isH = false;
  isNumNb = false;
  if (crk && (s == "volume" || s == "rkCorrections")) {   // RKCorrections state (LinearOrder)
    fs = {s == "volume" ? F_VOL : F_RKC_0, s == "volume" ? 1 : 16};
    return true;
  }
  static const std::map<std::string, FieldSpec> m = {
      {"position", {F_X, 3}}, {"velocity", {F_VX, 3}}, {"mass", {F_MASS, 1}}, {"massDensity", {F_RHO, 1}},
      {"specificThermalEnergy", {F_EPS, 1}}, {"pressure", {F_P, 1}}, {"soundSpeed", {F_CS, 1}},
      {"omegaGradh", {F_OMEGA, 1}}, {"massDensitySum", {F_RHOSUM, 1}}, {"normalization", {F_NORM, 1}},
      {"DxDt", {F_DXDT_X, 3}}, {"DvDt", {F_DVDT_X, 3}}, {"DrhoDt", {F_DRHODT, 1}}, {"DepsDt", {F_DEPSDT, 1}},
      {"DvDx", {F_DVDX_XX, 9}}, {"internalDvDx", {F_DVDX_XX, 9}}, {"gradRho", {F_GRADRHO_X, 3}},
      {"M", {F_M_XX, 9}}, {"localM", {F_M_XX, 9}}, {"maxViscousPressure", {F_MAXQ, 1}},
      {"effViscousPressure", {F_EFFQ, 1}}, {"XSPHWeightSum", {F_XSPHW, 1}}, {"XSPHDeltaV", {F_XSPHDV_X, 3}},
      {"massZerothMoment", {F_M0, 1}}, {"massFirstMoment", {F_M1_X, 3}}, {"DvDtGravity", {F_GRAV_X, 3}},
      {"potential", {F_POT, 1}}, {"DepsDtCompatible", {F_DEPS_COMPAT, 1}},
      {"ArtificialViscosityVelocityGradient", {F_DVDXQ_XX, 9}}};
  if (asph && (s == "H" || s == "Hideal" || s == "DHDt" || s == "massSecondMoment")) {
    fs = {s == "H" ? F_HT_XX : (s == "Hideal" ? F_HIDEALT_XX : (s == "DHDt" ? F_DHDTT_XX : F_M2_XX)), 6};
    return true;
  }
  if (s == "H" || s == "Hideal" || s == "DHDt") {
    isH = true;
    fs = {s == "H" ? F_HINV : (s == "Hideal" ? F_HIDEAL : F_DHDT), 6};
    return true;
  }
  if (s == "numNeighbors") {
    isNumNb = true;
    fs = {0, 1};
    return true;
  }
  auto it = m.find(s);
  if (it == m.end()) return false;
  fs = it->second;
  return true;
}

int fail(sphgpu_ctx* c, const Error& e) {
  if (c) c->err = e.what();
  return e.code;
}
int failStd(sphgpu_ctx* c, const std::exception& e) {
  if (c) c->err = e.what();
  return SPHGPU_E_CUDA;
}

#define API_BEGIN(h) \
  if (!(h)) return SPHGPU_E_ARG; \
  try {
#define API_RETURN_OK(h) return SPHGPU_OK
#define API_END(h)                        \
  }                                       \
  catch (const Error& e) {                \
    return fail(h, e);                    \
  }                                       \
  catch (const std::exception& e) {       \
    return failStd(h, e);                 \
  }                                       \
  return SPHGPU_OK;

}  // namespace

namespace {
struct CheckpointHeader {
  char magic[8];
  int32_t version, nfields;
  int64_t n, cycle;
  double time, lastDt, dtMultiplier, dtMinAcc, extraEnergy;
  int32_t precision, numLists, pairVariant, viscosity, smoothingScale, fixShape;
  // version 3: the package and kernel the image belongs to
  int32_t hydro, rkVolume, radialOnly, pad;
  uint64_t tableHash;   // FNV-1a of the W and grad W table coefficients
};
constexpr int32_t kCheckpointVersion = 3;

// FNV-1a over the bytes of the kernel table the handle evaluates, so an image
// written with another TableKernel (base kernel, order or number of points,
// or a table set by the caller) is told apart from this handle's.
uint64_t tableHash(const sphgpu_ctx* c) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&h](const void* p, size_t bytes) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t k = 0; k < bytes; ++k) { h ^= b[k]; h *= 1099511628211ull; }
  };
  mix(c->tw.data(), c->tw.size() * sizeof(double));
  mix(c->tg.data(), c->tg.size() * sizeof(double));
  return h;
}
constexpr char kCheckpointMagic[8] = {'S', 'P', 'H', 'G', 'P', 'U', 'C', 'K'};
size_t checkpointBytes(long n) {
  return sizeof(CheckpointHeader) + (size_t)F_NUM_PERMUTED * n * sizeof(double) + 2 * (size_t)n * sizeof(int);
}
}  // namespace

extern "C" {

void sphgpu_default_config(sphgpu_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->num_table_points = 1000;
  c->cfl = 0.25;
  c->use_velocity_magnitude_for_dt = 0;
  c->compatible_energy = 1;
  c->gradh_correction = 1;
  c->xsph = 0;
  c->correct_velocity_gradient = 1;
  c->sum_mass_density_over_all_nodelists = 1;
  c->density_update = SPHGPU_DENSITY_RIGOROUS_SUM;
  c->eps_tensile = 0.0;
  c->n_tensile = 4.0;
  c->Cl = 1.0;
  c->Cq = 1.0;
  c->eps2 = 1.0e-2;
  c->dt_min = 0.0;
  c->dt_max = 1.0e300;
  c->dt_growth = 2.0;
  c->last_dt = 1.0e-5;
  c->time = 0.0;
  c->gravity = 0;
  c->G = 1.0;
  c->softening = 0.01;
  c->opening = 0.5;
  c->ftimestep = 0.1;
  c->precision = SPHGPU_PRECISION_FP64;
  c->device = 0;
  c->viscosity = SPHGPU_VISCOSITY_MONAGHAN_GINGOLD;
  c->eta_crit_frac = 1.0;
  c->eta_fold_frac = 0.2;
  c->smoothing_scale = SPHGPU_SMOOTHING_SPH;
  c->fix_shape = 0;
  c->h_update = SPHGPU_H_IDEAL;
  c->evolve_total_energy = 0;
  c->radial_only = 0;
  c->hydro = SPHGPU_HYDRO_SPH;
  c->rk_volume = SPHGPU_RK_VOLUME_SUM;
  c->kernel = SPHGPU_KERNEL_BSPLINE;
  c->kernel_order = 3;
}

int sphgpu_create(const sphgpu_config* cfg, sphgpu_handle* out) {
  if (!cfg || !out) return SPHGPU_E_ARG;
  *out = nullptr;
  auto* c = new sphgpu_ctx();
  try {
    c->cfg = *cfg;
    if (cfg->precision != SPHGPU_PRECISION_FP64 && cfg->precision != SPHGPU_PRECISION_FP32 &&
        cfg->precision != SPHGPU_PRECISION_FP32_PLAIN)
      throw Error(SPHGPU_E_ARG, "unknown precision mode");
    if (cfg->precision == SPHGPU_PRECISION_FP32_PLAIN && cfg->hydro == SPHGPU_HYDRO_CRKSPH)
      throw Error(SPHGPU_E_UNSUPPORTED, "the plain-sum FP32 mode covers the SPH sweeps");
    if (cfg->viscosity != SPHGPU_VISCOSITY_MONAGHAN_GINGOLD && cfg->viscosity != SPHGPU_VISCOSITY_LIMITED_MONAGHAN_GINGOLD)
      throw Error(SPHGPU_E_UNSUPPORTED, "unknown artificial viscosity");
    if (cfg->viscosity == SPHGPU_VISCOSITY_LIMITED_MONAGHAN_GINGOLD && !(cfg->eta_fold_frac > 0.0))
      throw Error(SPHGPU_E_ARG, "etaFoldFrac must be positive");
    if (cfg->density_update != SPHGPU_DENSITY_RIGOROUS_SUM && cfg->density_update != SPHGPU_DENSITY_INTEGRATE)
      throw Error(SPHGPU_E_UNSUPPORTED, "only RigorousSumDensity and IntegrateDensity are on this path");
    if (cfg->smoothing_scale != SPHGPU_SMOOTHING_SPH && cfg->smoothing_scale != SPHGPU_SMOOTHING_ASPH_CLASSIC &&
        cfg->smoothing_scale != SPHGPU_SMOOTHING_ASPH)
      throw Error(SPHGPU_E_UNSUPPORTED, "unknown smoothing-scale package");
    if (cfg->smoothing_scale == SPHGPU_SMOOTHING_ASPH && !cfg->fix_shape && !cfg->radial_only)
      throw Error(SPHGPU_E_UNSUPPORTED, "ASPHSmoothingScale without fixShape or radialOnly shapes H from Voronoi "
                                        "cells, which are not built");
    if (cfg->h_update != SPHGPU_H_IDEAL && cfg->h_update != SPHGPU_H_INTEGRATE && cfg->h_update != SPHGPU_H_FIXED)
      throw Error(SPHGPU_E_UNSUPPORTED, "unknown H evolution");
    if (cfg->fix_shape && cfg->radial_only)   // ASPHClassicSmoothingScale: not both
      throw Error(SPHGPU_E_ARG, "fixShape and radialOnly cannot both be set");
    if (cfg->radial_only && cfg->smoothing_scale == SPHGPU_SMOOTHING_SPH)
      throw Error(SPHGPU_E_ARG, "radialOnly needs the ASPH smoothing scale");
    if (cfg->compatible_energy && cfg->evolve_total_energy)   // SPH.cc:97-98
      throw Error(SPHGPU_E_ARG, "compatibleEnergyEvolution and evolveTotalEnergy cannot both be set");
    if (cfg->hydro != SPHGPU_HYDRO_SPH && cfg->hydro != SPHGPU_HYDRO_CRKSPH)
      throw Error(SPHGPU_E_UNSUPPORTED, "unknown hydro package");
    if (cfg->hydro == SPHGPU_HYDRO_CRKSPH) {
      if (cfg->rk_volume != SPHGPU_RK_VOLUME_MASS_OVER_DENSITY && cfg->rk_volume != SPHGPU_RK_VOLUME_SUM &&
          cfg->rk_volume != SPHGPU_RK_VOLUME_H)
        throw Error(SPHGPU_E_UNSUPPORTED, "RK volume types with a tessellation are not built");
      if (cfg->smoothing_scale != SPHGPU_SMOOTHING_SPH)
        throw Error(SPHGPU_E_UNSUPPORTED, "CRKSPH runs with the SPH smoothing scale (isotropic H)");
      if (cfg->gradh_correction)
        throw Error(SPHGPU_E_ARG, "CRKSPH has no grad-h correction");
    }
    CUDA_OK(cudaSetDevice(cfg->device));
    CUDA_OK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->prof.s = c->stream;
    c->small.ensure(64 * sizeof(double));
    CUDA_OK(cudaMallocHost(&c->hsmall, 64 * sizeof(double)));
    c->time = cfg->time;
    c->lastDt = cfg->last_dt;
    for (int k = 0; k < kMaxNodeLists; ++k)
      c->lists[k] = NodeListParams{1.51, 1e-20, 1e20, 1e-10, 1e10, 5.0 / 3.0, -1.79e308, 1.79e308, 1e20, 1e-20, 0.1};
    c->numLists = 0;
    if (cfg->gravity) c->grav = gravityCreate();
    // Build the table of the configured base kernel (TableKernel(BSplineKernel(), n)
    // by default, or TableKernel(NBSplineKernel(order), n)).
    if (cfg->kernel != SPHGPU_KERNEL_BSPLINE && cfg->kernel != SPHGPU_KERNEL_NBSPLINE &&
        cfg->kernel != SPHGPU_KERNEL_WENDLAND_C2 && cfg->kernel != SPHGPU_KERNEL_WENDLAND_C4)
      throw Error(SPHGPU_E_UNSUPPORTED, "unknown base kernel");
    if (cfg->kernel == SPHGPU_KERNEL_NBSPLINE && (cfg->kernel_order < 2 || cfg->kernel_order > 9))
      throw Error(SPHGPU_E_ARG, "NBSplineKernel order must be 2..9");
    const int np = cfg->num_table_points > 0 ? cfg->num_table_points : 1000;
    const int nq = np | 1;
    std::vector<double> w(3 * ((nq - 1) / 2)), g(w.size()), g2(w.size()), nh(2 * np), ws(2 * np), meta(10);
    if (table::buildKernelTable(cfg->kernel, cfg->kernel_order, np, w.data(), g.data(), g2.data(), nh.data(),
                                ws.data(), meta.data()) != 0)
      throw Error(SPHGPU_E_ARG, "bad num_table_points");
    c->kernelExtent = meta[9];
    setTable(c, w.data(), g.data(), g2.data(), nh.data(), ws.data(), meta.data());
    refreshParams(c);
  } catch (const Error& e) {
    const int code = e.code;
    sphgpu_destroy(c);
    return code;
  } catch (const std::exception& e) {
    sphgpu_destroy(c);
    return SPHGPU_E_CUDA;
  }
  *out = c;
  return SPHGPU_OK;
}

int sphgpu_destroy(sphgpu_handle c) {
  if (!c) return SPHGPU_E_ARG;
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->prof.on = false;
  for (auto& r : c->prof.pending) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  DBuf* bufs[] = {&c->dTable, &c->bankA, &c->bankB, &c->keys, &c->vals, &c->keysAlt, &c->valsAlt, &c->sortWs,
                  &c->cellStart, &c->cellEnd, &c->counts, &c->nbrStart, &c->nbr, &c->scanWs, &c->pacc,
                  &c->scratch, &c->small, &c->posh, &c->velm, &c->thermo, &c->hten, &c->stage, &c->v12, &c->itemFlag,
                  &c->items, &c->dLists, &c->dvq, &c->inv, &c->vol32, &c->rkc32, &c->xstage, &c->xidx,
                  &c->itemBox, &c->chunkOf, &c->itemCount};
  for (auto* b : bufs) b->release();
  for (int k = 0; k < 2; ++k) { c->orig[k].release(); c->list[k].release(); c->cellc[k].release(); }
  if (c->grav) gravityDestroy(c->grav);
  if (c->tA) cudaEventDestroy(c->tA);
  if (c->tB) cudaEventDestroy(c->tB);
  if (c->hsmall) cudaFreeHost(c->hsmall);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return SPHGPU_OK;
}

const char* sphgpu_last_error(sphgpu_handle c) { return c ? c->err.c_str() : "null handle"; }

int sphgpu_build_bspline_table(int num_points, double* w, double* grad, double* grad2, double* nperh, double* wsum,
                               double* meta) {
  if (!w || !grad || !grad2 || !nperh || !wsum || !meta) return SPHGPU_E_ARG;
  return sph::table::buildBSplineTable(num_points, w, grad, grad2, nperh, wsum, meta) == 0 ? SPHGPU_OK
                                                                                           : SPHGPU_E_ARG;
}

int sphgpu_build_kernel_table(int kernel, int order, int num_points, double* w, double* grad, double* grad2,
                              double* nperh, double* wsum, double* meta) {
  if (!w || !grad || !grad2 || !nperh || !wsum || !meta) return SPHGPU_E_ARG;
  return sph::table::buildKernelTable(kernel, order, num_points, w, grad, grad2, nperh, wsum, meta) == 0
             ? SPHGPU_OK
             : SPHGPU_E_ARG;
}

int sphgpu_set_kernel_table(sphgpu_handle c, const double* w, const double* grad, const double* grad2,
                            const double* nperh, const double* wsum, const double* meta) {
  API_BEGIN(c)
  if (!w || !grad || !grad2 || !nperh || !wsum || !meta) throw Error(SPHGPU_E_ARG, "null table pointer");
  setTable(c, w, grad, grad2, nperh, wsum, meta);
  refreshParams(c);
  API_END(c)
}

int sphgpu_set_nodelist(sphgpu_handle c, int k, double nPerh, double hmin, double hmax, double rhoMin, double rhoMax,
                        double gamma) {
  API_BEGIN(c)
  if (k < 0 || k >= kMaxNodeLists) throw Error(SPHGPU_E_ARG, "nodelist index out of range");
  if (!(nPerh > 0.0) || !(hmin > 0.0) || !(hmax >= hmin) || !(gamma > 1.0))
    throw Error(SPHGPU_E_ARG, "bad nodelist parameters");
  c->lists[k] = NodeListParams{nPerh, hmin, hmax, rhoMin, rhoMax, gamma, -1.7976931348623157e308,
                               1.7976931348623157e308, 1.0 / hmin, 1.0 / hmax, c->lists[k].hminratio};
  c->numLists = std::max(c->numLists, k + 1);
  refreshParams(c);
  API_END(c)
}

int sphgpu_set_nodelist_hminratio(sphgpu_handle c, int k, double hminratio) {
  API_BEGIN(c)
  if (k < 0 || k >= kMaxNodeLists) throw Error(SPHGPU_E_ARG, "nodelist index out of range");
  if (!(hminratio > 0.0) || hminratio > 1.0) throw Error(SPHGPU_E_ARG, "hminratio must be in (0, 1]");
  c->lists[k].hminratio = hminratio;
  refreshParams(c);
  API_END(c)
}

int sphgpu_add_boundary(sphgpu_handle c, int type, int axis, double lo, double hi, int wall_high) {
  API_BEGIN(c)
  if (axis < 0 || axis > 2) throw Error(SPHGPU_E_ARG, "axis must be 0, 1 or 2");
  if (type == SPHGPU_BOUNDARY_PERIODIC) {
    if (!(hi > lo)) throw Error(SPHGPU_E_ARG, "periodic boundary needs hi > lo");
  } else if (type != SPHGPU_BOUNDARY_REFLECTING) {
    throw Error(SPHGPU_E_ARG, "unknown boundary type");
  }
  c->bcs.push_back(Boundary{type, axis, lo, hi, wall_high});
  API_END(c)
}

int sphgpu_set_particles(sphgpu_handle c, long n, const double* pos, const double* vel, const double* mass,
                         const double* rho, const double* eps, const double* H, const int* nodelist) {
  API_BEGIN(c)
  c->boundsValid = false;   // the state changes: bounds are measured again
  if (n <= 0 || n >= kMaxNodes) throw Error(SPHGPU_E_ARG, "particle count out of range");
  if (!pos || !vel || !mass || !rho || !eps || !H) throw Error(SPHGPU_E_ARG, "null particle array");
  if (c->numLists == 0) c->numLists = 1;
  const bool asph = c->cfg.smoothing_scale != SPHGPU_SMOOTHING_SPH;
  for (long i = 0; i < n; ++i) {
    const double* h = H + 6 * i;
    if (asph) {   // symmetric positive definite: leading minors positive (Sylvester)
      const double m2 = h[0] * h[3] - h[1] * h[1];
      const double m3 = h[0] * (h[3] * h[5] - h[4] * h[4]) - h[1] * (h[1] * h[5] - h[4] * h[2]) +
                        h[2] * (h[1] * h[4] - h[3] * h[2]);
      if (!(h[0] > 0.0) || !(m2 > 0.0) || !(m3 > 0.0))
        throw Error(SPHGPU_E_NAN, "H not positive definite on node " + std::to_string(i));
    } else {
      if (h[1] != 0.0 || h[2] != 0.0 || h[4] != 0.0 || h[0] != h[3] || h[0] != h[5])
        throw Error(SPHGPU_E_UNSUPPORTED, "H must be isotropic (H = I/h) on node " + std::to_string(i));
      if (!(h[0] > 0.0)) throw Error(SPHGPU_E_NAN, "non-positive H on node " + std::to_string(i));
    }
    if (nodelist && (nodelist[i] < 0 || nodelist[i] >= c->numLists))
      throw Error(SPHGPU_E_ARG, "nodelist id out of range on node " + std::to_string(i));
  }
  ensureCapacity(c, n);
  c->n = n;
  c->cur = 0;
  c->F = c->fieldsOf(c->bankA);
  c->Falt = c->fieldsOf(c->bankB);
  CUDA_OK(cudaMemsetAsync(c->bankA.p, 0, c->bankA.bytes, c->stream));
  std::vector<double> tmp(n);
  auto up = [&](int f, const double* src, int stride, int comp) {
    for (long i = 0; i < n; ++i) tmp[i] = src[(size_t)stride * i + comp];
    CUDA_OK(cudaMemcpyAsync(c->F.f[f], tmp.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CUDA_OK(cudaStreamSynchronize(c->stream));
  };
  for (int a = 0; a < 3; ++a) { up(F_X + a, pos, 3, a); up(F_VX + a, vel, 3, a); }
  up(F_MASS, mass, 1, 0);
  up(F_RHO, rho, 1, 0);
  up(F_EPS, eps, 1, 0);
  if (asph) {
    for (int k = 0; k < 6; ++k) up(F_HT_XX + k, H, 6, k);
    launchTensorExtent(c->F, n, c->stream, &c->lc);
    c->check();
  } else {
    up(F_HINV, H, 6, 0);
  }
  for (long i = 0; i < n; ++i) tmp[i] = 1.0;
  CUDA_OK(cudaMemcpyAsync(c->F.f[F_OMEGA], tmp.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  std::vector<int> ids(n);
  for (long i = 0; i < n; ++i) ids[i] = (int)i;
  CUDA_OK(cudaMemcpy(c->orig[0].p, ids.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  ++c->permVersion;
  for (long i = 0; i < n; ++i) ids[i] = nodelist ? nodelist[i] : 0;
  CUDA_OK(cudaMemcpy(c->list[0].p, ids.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  c->haveNeighbors = false;
  c->initialized = false;
  c->omegaStale = false;
  refreshParams(c);
  API_END(c)
}

//------------------------------------------------------------------------------
// Checkpoint / restart (the package's dumpState / restoreState,
// src/SPH/SPHBase.cc:711-768, plus the integrator's time, last dt and cycle).
// The image keeps the internal node order, so a restored run continues
// bitwise as the uninterrupted one.
//------------------------------------------------------------------------------

int sphgpu_checkpoint_size(sphgpu_handle c, size_t* bytes) {
  API_BEGIN(c)
  if (!bytes) throw Error(SPHGPU_E_ARG, "null size");
  requireState(c);
  *bytes = checkpointBytes(c->n);
  API_END(c)
}

int sphgpu_checkpoint(sphgpu_handle c, void* buffer, size_t bytes) {
  API_BEGIN(c)
  requireState(c);
  settleOmega(c);
  if (!buffer || bytes < checkpointBytes(c->n)) throw Error(SPHGPU_E_ARG, "checkpoint buffer too small");
  const long n = c->n;
  CheckpointHeader h{};
  std::memcpy(h.magic, kCheckpointMagic, 8);
  h.version = kCheckpointVersion;
  h.nfields = F_NUM_PERMUTED;
  h.n = n;
  h.cycle = c->cycle;
  h.time = c->time;
  h.lastDt = c->lastDt;
  h.dtMultiplier = c->dtMultiplier;
  h.dtMinAcc = c->dtMinAcc;
  h.extraEnergy = c->extraEnergy;
  h.precision = c->cfg.precision;
  h.numLists = c->numLists;
  h.pairVariant = c->pairVariant;
  h.viscosity = c->cfg.viscosity;
  h.smoothingScale = c->cfg.smoothing_scale;
  h.fixShape = c->cfg.fix_shape;
  h.hydro = c->cfg.hydro;
  h.rkVolume = c->cfg.rk_volume;
  h.radialOnly = c->cfg.radial_only;
  h.tableHash = tableHash(c);
  char* out = static_cast<char*>(buffer);
  std::memcpy(out, &h, sizeof(h));
  out += sizeof(h);
  for (int f = 0; f < F_NUM_PERMUTED; ++f, out += n * sizeof(double))
    CUDA_OK(cudaMemcpyAsync(out, c->F.f[f], n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaMemcpyAsync(out, c->origp(), n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  out += n * sizeof(int);
  CUDA_OK(cudaMemcpyAsync(out, c->listp(), n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

int sphgpu_restore(sphgpu_handle c, const void* buffer, size_t bytes) {
  API_BEGIN(c)
  c->boundsValid = false;   // the state changes: bounds are measured again
  if (!buffer || bytes < sizeof(CheckpointHeader)) throw Error(SPHGPU_E_ARG, "checkpoint buffer too small");
  CheckpointHeader h;
  std::memcpy(&h, buffer, sizeof(h));
  if (std::memcmp(h.magic, kCheckpointMagic, 8) != 0 || h.version != kCheckpointVersion ||
      h.nfields != F_NUM_PERMUTED)
    throw Error(SPHGPU_E_ARG, "not a checkpoint of this library version");
  if (h.n <= 0 || h.n >= kMaxNodes || bytes < checkpointBytes((long)h.n))
    throw Error(SPHGPU_E_ARG, "checkpoint size does not match its node count");
  if (h.precision != c->cfg.precision || h.viscosity != c->cfg.viscosity ||
      h.smoothingScale != c->cfg.smoothing_scale || h.fixShape != c->cfg.fix_shape ||
      h.radialOnly != c->cfg.radial_only)
    throw Error(SPHGPU_E_STATE, "checkpoint written with another precision mode, viscosity or smoothing scale");
  if (h.hydro != c->cfg.hydro || (c->cfg.hydro == SPHGPU_HYDRO_CRKSPH && h.rkVolume != c->cfg.rk_volume))
    throw Error(SPHGPU_E_STATE, "checkpoint written by another hydro package or RK volume type");
  if (h.tableHash != tableHash(c))
    throw Error(SPHGPU_E_STATE, "checkpoint written with another kernel table");
  if (h.numLists < 1 || h.numLists > std::max(1, c->numLists))
    throw Error(SPHGPU_E_STATE, "checkpoint uses NodeLists that are not set on this handle");
  const long n = (long)h.n;
  {
    // The caller-order map must be a permutation of 0..n-1 and every NodeList
    // id must name a NodeList of the image: both index device tables and
    // caller arrays, so a truncated or corrupted image is refused here.
    const char* tail = static_cast<const char*>(buffer) + sizeof(h) + (size_t)F_NUM_PERMUTED * n * sizeof(double);
    std::vector<int> orig((size_t)n), ids((size_t)n);
    std::memcpy(orig.data(), tail, n * sizeof(int));
    std::memcpy(ids.data(), tail + n * sizeof(int), n * sizeof(int));
    std::vector<unsigned char> seen((size_t)n, 0);
    for (long k = 0; k < n; ++k) {
      const int o = orig[k];
      if (o < 0 || o >= n || seen[o]) throw Error(SPHGPU_E_ARG, "checkpoint node order is not a permutation");
      seen[o] = 1;
      if (ids[k] < 0 || ids[k] >= h.numLists) throw Error(SPHGPU_E_ARG, "checkpoint NodeList id out of range");
    }
  }
  ensureCapacity(c, n);
  c->n = n;
  c->cur = 0;
  c->F = c->fieldsOf(c->bankA);
  c->Falt = c->fieldsOf(c->bankB);
  CUDA_OK(cudaMemsetAsync(c->bankA.p, 0, c->bankA.bytes, c->stream));
  const char* in = static_cast<const char*>(buffer) + sizeof(h);
  for (int f = 0; f < F_NUM_PERMUTED; ++f, in += n * sizeof(double))
    CUDA_OK(cudaMemcpyAsync(c->F.f[f], in, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_OK(cudaMemcpyAsync(c->orig[0].p, in, n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  ++c->permVersion;
  in += n * sizeof(int);
  CUDA_OK(cudaMemcpyAsync(c->list[0].p, in, n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  c->numLists = std::max(c->numLists, (int)h.numLists);
  c->cycle = h.cycle;
  c->time = h.time;
  c->lastDt = h.lastDt;
  c->dtMultiplier = h.dtMultiplier;
  c->dtMinAcc = h.dtMinAcc;
  c->extraEnergy = h.extraEnergy;
  c->pairVariant = h.pairVariant;   // same kernel variant: same rounding as the uninterrupted run
  c->tunedN = n;
  c->nbCap = 0;
  c->nbCapNext = 0;
  c->haveNeighbors = false;
  c->initialized = true;
  c->omegaStale = false;
  refreshParams(c);
  API_END(c)
}

int sphgpu_initialize(sphgpu_handle c) {
  API_BEGIN(c)
  requireState(c);
  refreshParams(c);
  launchEOS(c->F, c->listp(), c->n, c->hp.lists, c->stream, &c->lc);
  c->check();
  buildNeighbors(c);
  if (c->cfg.gradh_correction) gradh(c);
  c->omegaStale = false;
  if (c->hp.crk) {
    // RKCorrections::initializeProblemStartupDependencies
    // (src/RK/RKCorrections.cc:85-150): volumes, then corrections
    if (c->fp32()) {
      launchRKVolumesFP32(c->F, c->f32(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
      launchRKCorrectionsFP32(c->F, c->f32(), c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
    } else {
      launchRKVolumes(c->F, c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
      launchRKCorrections(c->F, c->n, c->grid, c->nl(), c->tableDev(), c->hp, c->stream, &c->lc);
    }
    c->check();
  }
  CUDA_OK(cudaStreamSynchronize(c->stream));
  c->initialized = true;
  API_END(c)
}

int sphgpu_connectivity(sphgpu_handle c) {
  API_BEGIN(c)
  requireState(c);
  refreshParams(c);
  settleOmega(c);   // on the lists the owed correction belongs to
  buildNeighbors(c);
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

int sphgpu_sum_density(sphgpu_handle c) {
  API_BEGIN(c)
  requireState(c);
  settleOmega(c);
  if (!c->haveNeighbors) buildNeighbors(c);
  prepare32(c);
  sumDensity(c);
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

int sphgpu_gradh(sphgpu_handle c) {
  API_BEGIN(c)
  requireState(c);
  if (!c->haveNeighbors) buildNeighbors(c);
  prepare32(c);
  gradh(c);
  c->omegaStale = false;
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

int sphgpu_evaluate_derivatives(sphgpu_handle c) {
  API_BEGIN(c)
  requireState(c);
  refreshParams(c);
  settleOmega(c);
  if (!c->haveNeighbors) buildNeighbors(c);
  prepare32(c);
  evalDerivs(c);
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

int sphgpu_dt(sphgpu_handle c, double* dt, int* reason) {
  API_BEGIN(c)
  requireState(c);
  settleOmega(c);
  refreshParams(c);
  if (!c->haveNeighbors) buildNeighbors(c);
  prepare32(c);
  const double v = packageDt(c, reason);
  if (dt) *dt = v;
  API_END(c)
}

int sphgpu_step(sphgpu_handle c, double max_time, double* dt_out) {
  API_BEGIN(c)
  const double dt = step(c, max_time);
  if (dt_out) *dt_out = dt;
  API_END(c)
}

int sphgpu_advance(sphgpu_handle c, int nsteps, double max_time) {
  API_BEGIN(c)
  for (int k = 0; k < nsteps && c->time < max_time; ++k) step(c, max_time);
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

int sphgpu_set_pair_variant(sphgpu_handle c, int variant) {
  API_BEGIN(c)
  if (variant < -1 || variant >= kPairVariants) throw Error(SPHGPU_E_ARG, "pair variant out of range");
  c->pairVariant = variant;
  c->pinnedVariant = variant >= 0;
  API_END(c)
}

int sphgpu_set_neighbor_width(sphgpu_handle c, int width) {
  API_BEGIN(c)
  if (width != 0 && width != 8 && width != 16 && width != 32) throw Error(SPHGPU_E_ARG, "group width not 0, 8, 16 or 32");
  c->pinnedWidth = width;
  if (width == 0) c->tunedWidth = 0;   // time the widths again at the next build
  API_END(c)
}

int sphgpu_set_energy_variant(sphgpu_handle c, int variant) {
  API_BEGIN(c)
  if (variant < -1 || variant >= kEnergyVariants) throw Error(SPHGPU_E_ARG, "energy variant out of range");
  c->energyPinned = variant >= 0;
  c->energyVariant = variant;
  API_END(c)
}

int sphgpu_get_energy_variant(sphgpu_handle c, int* variant, int* nvariants) {
  API_BEGIN(c)
  if (variant) *variant = c->energyVariant;
  if (nvariants) *nvariants = kEnergyVariants;
  API_END(c)
}

int sphgpu_get_neighbor_width(sphgpu_handle c, int* width) {
  API_BEGIN(c)
  if (!width) throw Error(SPHGPU_E_ARG, "null width");
  *width = c->itemWidth;
  API_END(c)
}

int sphgpu_get_pair_variant(sphgpu_handle c, int* variant, int* nvariants) {
  API_BEGIN(c)
  if (variant) *variant = c->pairVariant;
  if (nvariants)
    *nvariants = c->cfg.hydro == SPHGPU_HYDRO_CRKSPH
                     ? kPairVariantsCRK
                     : (c->cfg.smoothing_scale != SPHGPU_SMOOTHING_SPH ? kPairVariantsTensor : kPairVariants);
  API_END(c)
}

int sphgpu_ensemble_advance(sphgpu_handle* handles, int nboxes, int nsteps, double max_time, int nthreads,
                            int* failed) {
  if (failed) *failed = -1;
  if (!handles || nboxes <= 0 || nsteps < 0) return SPHGPU_E_ARG;
  {
    std::vector<sphgpu_handle> seen(handles, handles + nboxes);
    std::sort(seen.begin(), seen.end());
    if (!seen.front() || std::adjacent_find(seen.begin(), seen.end()) != seen.end()) return SPHGPU_E_ARG;
  }
  int nt = nthreads > 0 ? nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
  nt = std::max(1, std::min(nt, nboxes));
  // Longest-processing-time first: boxes by particle count, each onto the
  // least-loaded thread.
  std::vector<int> order(nboxes);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return handles[a]->n > handles[b]->n; });
  std::vector<std::vector<int>> work(nt);
  std::vector<long> load(nt, 0);
  for (int b : order) {
    const int t = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    work[t].push_back(b);
    load[t] += std::max(1L, handles[b]->n);
  }
  std::vector<int> rc(nboxes, SPHGPU_OK);
  std::atomic<int> stop{0};
  auto body = [&](int t) {
    auto run = [&](int b, bool finish) {
      sphgpu_ctx* c = handles[b];
      try {
        CUDA_OK(cudaSetDevice(c->cfg.device));
        if (finish) CUDA_OK(cudaStreamSynchronize(c->stream));
        else if (c->time < max_time) step(c, max_time);
      } catch (const Error& e) {
        rc[b] = fail(c, e);
      } catch (const std::exception& e) {
        rc[b] = failStd(c, e);
      }
      if (rc[b] != SPHGPU_OK) stop.store(1);
    };
    for (int k = 0; k < nsteps && !stop.load(); ++k)
      for (int b : work[t])
        if (rc[b] == SPHGPU_OK && !stop.load()) run(b, false);
    for (int b : work[t])
      if (rc[b] == SPHGPU_OK) run(b, true);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(body, t);
  body(0);
  for (auto& th : pool) th.join();
  for (int b = 0; b < nboxes; ++b)
    if (rc[b] != SPHGPU_OK) {
      if (failed) *failed = b;
      return rc[b];
    }
  return SPHGPU_OK;
}

int sphgpu_get_field(sphgpu_handle c, const char* name, double* out, int* ncomp) {
  API_BEGIN(c)
  if (!name) throw Error(SPHGPU_E_ARG, "null field name");
  FieldSpec fs;
  bool isH, isNb;
  if (!fieldSpec(name, fs, isH, isNb, c->hp.asph != 0, c->hp.crk != 0)) throw Error(SPHGPU_E_ARG, std::string("unknown field ") + name);
  if (fs.first == F_DVDXQ_XX && !c->hp.limitedQ)
    throw Error(SPHGPU_E_STATE, "ArtificialViscosityVelocityGradient exists only with the limited Q");
  if (ncomp) *ncomp = fs.ncomp;
  if (!out) return SPHGPU_OK;
  requireState(c);
  settleOmega(c);
  const long n = c->n;
  c->stage.ensure((size_t)n * fs.ncomp * sizeof(double));
  double* st = c->stage.as<double>();
  if (isNb) {
    if (!c->haveNeighbors) throw Error(SPHGPU_E_STATE, "no neighbour lists yet");
    launchCountsOut(c->counts.as<int>(), c->origp(), st, n, c->stream, &c->lc);
  } else if (isH) {
    launchGatherOutH(c->F, c->origp(), st, fs.first, n, c->stream, &c->lc);
  } else {
    launchGatherOut(c->F, c->origp(), st, fs.first, fs.ncomp, fs.ncomp, n, c->stream, &c->lc);
  }
  c->check();
  CUDA_OK(cudaMemcpyAsync(out, st, (size_t)n * fs.ncomp * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

int sphgpu_set_field(sphgpu_handle c, const char* name, const double* in) {
  API_BEGIN(c)
  if (c->n > 0 && c->haveTable) settleOmega(c);   // the state it belongs to is about to change
  c->boundsValid = false;   // the state changes: bounds are measured again
  if (!name || !in) throw Error(SPHGPU_E_ARG, "null argument");
  FieldSpec fs;
  bool isH, isNb;
  if (!fieldSpec(name, fs, isH, isNb, c->hp.asph != 0, c->hp.crk != 0) || isNb)
    throw Error(SPHGPU_E_ARG, std::string("unknown field ") + name);
  requireState(c);
  const long n = c->n;
  c->stage.ensure((size_t)n * fs.ncomp * sizeof(double));
  double* st = c->stage.as<double>();
  CUDA_OK(cudaMemcpyAsync(st, in, (size_t)n * fs.ncomp * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (isH) launchScatterIn(c->F, c->origp(), st, fs.first, 1, 6, n, c->stream, &c->lc);
  else launchScatterIn(c->F, c->origp(), st, fs.first, fs.ncomp, fs.ncomp, n, c->stream, &c->lc);
  if (fs.first == F_HT_XX) launchTensorExtent(c->F, n, c->stream, &c->lc);
  c->check();
  if (c->haveNeighbors) prepare32(c);
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

// The internal index of each caller index, rebuilt after a reordering.
const int* invOrder(sphgpu_ctx* c) {
  if (c->invVersion != c->permVersion) {
    c->inv.ensure((size_t)c->n * sizeof(int));
    launchInverseOrder(c->origp(), c->inv.as<int>(), c->n, c->stream, &c->lc);
    c->invVersion = c->permVersion;
  }
  return c->inv.as<int>();
}
// The device address of a host array of `bytes` bytes when it lies in
// page-locked memory the device can address (both ends checked); nullptr for
// pageable memory, which takes the staged copy instead.  Kernels then read or
// write the pinned array in place over the host link.
void* mappedHost(const void* p, size_t bytes) {
  if (!p || bytes == 0) return nullptr;
  cudaPointerAttributes a{}, b{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  const char* last = static_cast<const char*>(p) + bytes - 1;
  if (cudaPointerGetAttributes(&b, last) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  if (b.type != cudaMemoryTypeHost || !b.devicePointer) return nullptr;
  if (static_cast<char*>(b.devicePointer) - static_cast<char*>(a.devicePointer) != (ptrdiff_t)(bytes - 1))
    return nullptr;
  return a.devicePointer;
}

int sphgpu_upload_state(sphgpu_handle c, const double* pos, const double* vel, const double* mass, const double* rho,
                        const double* eps, const double* H) {
  API_BEGIN(c)
  if (c->n > 0 && c->haveTable) settleOmega(c);   // the state it belongs to is about to change
  c->boundsValid = false;   // the state changes: bounds are measured again
  requireState(c);
  const long n = c->n;
  c->stage.ensure((size_t)n * 15 * sizeof(double));
  double* st = c->stage.as<double>();
  struct Item { const double* p; int first, ncomp, stride; };
  const bool asph = c->hp.asph != 0;
  const Item items[] = {{pos, F_X, 3, 3}, {vel, F_VX, 3, 3}, {mass, F_MASS, 1, 1}, {rho, F_RHO, 1, 1},
                        {eps, F_EPS, 1, 1}, {H, asph ? (int)F_HT_XX : (int)F_HINV, asph ? 6 : 1, 6}};
  size_t off = 0;
  for (const auto& it : items) {
    if (!it.p) continue;
    const size_t bytes = (size_t)n * it.stride * sizeof(double);
    if (const void* dp = mappedHost(it.p, bytes)) {   // pinned: read in place, caller order
      launchScatterInHost(c->F, invOrder(c), static_cast<const double*>(dp), it.first, it.ncomp, it.stride, n,
                          c->stream, &c->lc);
      continue;
    }
    CUDA_OK(cudaMemcpyAsync(st + off, it.p, bytes, cudaMemcpyHostToDevice, c->stream));
    launchScatterIn(c->F, c->origp(), st + off, it.first, it.ncomp, it.stride, n, c->stream, &c->lc);
    off += (size_t)n * it.stride;
  }
  if (asph && H) launchTensorExtent(c->F, n, c->stream, &c->lc);
  c->check();
  // The FP32 mirror is not refreshed here: the step rebuilds it with the
  // lists, and every other entry that sweeps it refreshes it first.
  API_END(c)
}

int sphgpu_download_state(sphgpu_handle c, double* pos, double* vel, double* rho, double* eps, double* H) {
  API_BEGIN(c)
  requireState(c);
  const long n = c->n;
  c->stage.ensure((size_t)n * 14 * sizeof(double));
  double* st = c->stage.as<double>();
  struct Item { double* p; int first, ncomp, stride; };
  const bool asph = c->hp.asph != 0;
  const Item items[] = {{pos, F_X, 3, 3}, {vel, F_VX, 3, 3}, {rho, F_RHO, 1, 1}, {eps, F_EPS, 1, 1},
                        {H, asph ? (int)F_HT_XX : (int)F_HINV, asph ? 6 : 1, 6}};
  size_t off = 0;
  for (const auto& it : items) {
    if (!it.p) continue;
    const size_t bytes = (size_t)n * it.stride * sizeof(double);
    if (void* dp = mappedHost(it.p, bytes)) {   // pinned: written in place, caller order
      launchGatherOutHost(c->F, invOrder(c), static_cast<double*>(dp), it.first, it.ncomp, it.stride,
                          it.first == F_HINV && !asph, n, c->stream, &c->lc);
      continue;
    }
    if (it.first == F_HINV && !asph) launchGatherOutH(c->F, c->origp(), st + off, F_HINV, n, c->stream, &c->lc);
    else launchGatherOut(c->F, c->origp(), st + off, it.first, it.ncomp, it.stride, n, c->stream, &c->lc);
    CUDA_OK(cudaMemcpyAsync(it.p, st + off, (size_t)n * it.stride * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    off += (size_t)n * it.stride;
  }
  c->check();
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

int sphgpu_get_pairs(sphgpu_handle c, int* i_out, int* j_out, int* image, long* npairs) {
  API_BEGIN(c)
  if (!npairs) throw Error(SPHGPU_E_ARG, "null npairs");
  if (!c->haveNeighbors) throw Error(SPHGPU_E_STATE, "no neighbour lists yet");
  resolveNeighbors(c);
  *npairs = (long)c->nnbr;
  if (!i_out) return SPHGPU_OK;
  const long n = c->n;
  const int cap = c->nbCap;
  std::vector<int> orig(n), cnt(n);
  std::vector<uint32_t> nb(std::max<size_t>(1, c->nbSlots())), cells(n);
  CUDA_OK(cudaMemcpyAsync(cells.data(), c->cellp(), n * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaMemcpyAsync(orig.data(), c->origp(), n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaMemcpyAsync(cnt.data(), c->counts.p, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaMemcpyAsync(nb.data(), c->nbr.p, c->nbSlots() * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  long long k = 0;
  for (long i = 0; i < n; ++i)
    for (int q = 0; q < cnt[i]; ++q, ++k) {
      const uint32_t e = nb[((size_t)(i >> 5) * cap + q) * 32 + (i & 31)];
      i_out[k] = orig[i];
      j_out[k] = orig[e & kIndexMask];
      if (image) {
        const int d = (int)(e >> kIndexBits);
        int code = 0;
        for (int a = 0; a < 3; ++a) {
          const int ca = (int)((cells[i] >> (10 * a)) & 1023u);
          const int da = (d >> (2 * a)) & 3;
          if (da == 1 && ca == 0) code |= 1 << (2 * a);
          else if (da == 2 && ca == c->grid.nc[a] - 1) code |= 2 << (2 * a);
        }
        image[k] = code;
      }
    }
  API_END(c)
}

namespace {
ExchangeFields exchangeFields(int point) {
  ExchangeFields ef{};
  if (point == SPHGPU_EXCHANGE_DENSITY) {
    ef.w = 1; ef.mirror = 1; ef.ids[0] = F_RHO;
  } else if (point == SPHGPU_EXCHANGE_OMEGA) {
    ef.w = 1; ef.mirror = 2; ef.ids[0] = F_OMEGA;
  } else if (point == SPHGPU_EXCHANGE_DERIVS) {
    ef.w = 4; ef.mirror = 0;
    ef.ids[0] = F_DVDT_X; ef.ids[1] = F_DVDT_Y; ef.ids[2] = F_DVDT_Z; ef.ids[3] = F_DEPSDT;
  } else {
    throw Error(SPHGPU_E_ARG, "not a row exchange point");
  }
  return ef;
}
}  // namespace

int sphgpu_set_domain(sphgpu_handle c, long n_ghost, sphgpu_exchange_fn fn, void* user) {
  API_BEGIN(c)
  requireState(c);
  if (n_ghost < 0 || n_ghost >= c->n) throw Error(SPHGPU_E_ARG, "halo count out of range");
  if (n_ghost > 0 && !fn) throw Error(SPHGPU_E_ARG, "a halo needs an exchange function");
  if (fn && (c->cfg.gravity || c->hp.crk))
    throw Error(SPHGPU_E_UNSUPPORTED, "domain decomposition covers the SPH hydro step without gravity");
  c->nGhost = n_ghost;
  c->xfn = fn;
  c->xuser = user;
  API_END(c)
}

int sphgpu_exchange_width(sphgpu_handle c, int point, int* width) {
  API_BEGIN(c)
  if (!width) throw Error(SPHGPU_E_ARG, "null width");
  *width = point == SPHGPU_EXCHANGE_DT ? 0 : exchangeFields(point).w;
  API_END(c)
}

int sphgpu_exchange_get(sphgpu_handle c, int point, const int* idx, long count, double* out) {
  API_BEGIN(c)
  requireState(c);
  const ExchangeFields ef = exchangeFields(point);
  if (count < 0 || (count > 0 && (!idx || !out))) throw Error(SPHGPU_E_ARG, "bad exchange rows");
  if (count == 0) API_RETURN_OK(c);
  for (long r = 0; r < count; ++r)
    if (idx[r] < 0 || idx[r] >= c->n - c->nGhost) throw Error(SPHGPU_E_ARG, "exchange row is not an owned node");
  c->xidx.ensure((size_t)count * sizeof(int));
  c->xstage.ensure((size_t)count * ef.w * sizeof(double));
  CUDA_OK(cudaMemcpyAsync(c->xidx.p, idx, (size_t)count * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  launchExchangeGet(c->F, invOrder(c), c->xidx.as<int>(), count, ef, c->xstage.as<double>(), c->stream, &c->lc);
  c->check();
  CUDA_OK(cudaMemcpyAsync(out, c->xstage.p, (size_t)count * ef.w * sizeof(double), cudaMemcpyDeviceToHost,
                          c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

int sphgpu_exchange_put(sphgpu_handle c, int point, const double* in) {
  API_BEGIN(c)
  requireState(c);
  const ExchangeFields ef = exchangeFields(point);
  const long count = c->nGhost;
  if (count == 0) API_RETURN_OK(c);
  if (!in) throw Error(SPHGPU_E_ARG, "null exchange rows");
  c->xstage.ensure((size_t)count * ef.w * sizeof(double));
  CUDA_OK(cudaMemcpyAsync(c->xstage.p, in, (size_t)count * ef.w * sizeof(double), cudaMemcpyHostToDevice,
                          c->stream));
  Fields32 m32{};
  if (c->fp32()) m32 = c->f32();
  launchExchangePut(c->F, m32, invOrder(c), c->n - count, count, ef, c->xstage.as<double>(), c->stream, &c->lc);
  c->check();
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

int sphgpu_image_layout(sphgpu_handle c, const char* field, size_t* header_bytes, int* row, int* nrows) {
  API_BEGIN(c)
  if (header_bytes) *header_bytes = sizeof(CheckpointHeader);
  if (nrows) *nrows = F_NUM_PERMUTED;
  if (row) {
    if (!field) throw Error(SPHGPU_E_ARG, "null field name");
    FieldSpec fs;
    bool isH, isNumNb;
    if (!fieldSpec(field, fs, isH, isNumNb, c->hp.asph != 0, c->hp.crk != 0) || isNumNb || fs.first >= F_NUM_PERMUTED)
      throw Error(SPHGPU_E_ARG, std::string("no image row for ") + field);
    *row = fs.first;
  }
  API_END(c)
}

int sphgpu_conservation(sphgpu_handle c, double out[8]) {
  API_BEGIN(c)
  requireState(c);
  if (!out) throw Error(SPHGPU_E_ARG, "null output");
  c->scratch.ensure(7 * sizeof(double) * 4096);
  double* d = c->small.as<double>() + 32;
  launchConservation(c->F, c->n, c->cfg.gravity != 0, c->scratch.as<double>(), 7 * 4096, d, c->stream, &c->lc);
  c->check();
  CUDA_OK(cudaMemcpyAsync(c->hsmall + 32, d, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 8; ++k) out[k] = c->hsmall[32 + k];
  API_END(c)
}

int sphgpu_get_time(sphgpu_handle c, double* time, double* last_dt, long* cycle) {
  API_BEGIN(c)
  if (time) *time = c->time;
  if (last_dt) *last_dt = c->lastDt;
  if (cycle) *cycle = c->cycle;
  API_END(c)
}

int sphgpu_num_particles(sphgpu_handle c, long* n) {
  API_BEGIN(c)
  if (n) *n = c->n;
  API_END(c)
}

int sphgpu_profile_enable(sphgpu_handle c, int enable) {
  API_BEGIN(c)
  c->prof.collect();
  c->prof.on = enable != 0;
  API_END(c)
}
int sphgpu_profile_get(sphgpu_handle c, const char* name, long* launches, double* ms) {
  API_BEGIN(c)
  c->prof.collect();
  auto it = c->prof.acc.find(name ? name : "");
  if (launches) *launches = it == c->prof.acc.end() ? 0 : it->second.first;
  if (ms) *ms = it == c->prof.acc.end() ? 0.0 : it->second.second;
  API_END(c)
}
int sphgpu_profile_reset(sphgpu_handle c) {
  API_BEGIN(c)
  c->prof.collect();
  c->prof.acc.clear();
  API_END(c)
}
int sphgpu_launch_count(sphgpu_handle c, long* launches) {
  API_BEGIN(c)
  if (launches) *launches = c->lc.n;
  API_END(c)
}
int sphgpu_timer_start(sphgpu_handle c) {
  API_BEGIN(c)
  if (!c->tA) CUDA_OK(cudaEventCreate(&c->tA));
  if (!c->tB) CUDA_OK(cudaEventCreate(&c->tB));
  CUDA_OK(cudaEventRecord(c->tA, c->stream));
  API_END(c)
}
int sphgpu_timer_stop(sphgpu_handle c, double* ms) {
  API_BEGIN(c)
  if (!c->tA || !c->tB) throw Error(SPHGPU_E_STATE, "timer not started");
  CUDA_OK(cudaEventRecord(c->tB, c->stream));
  CUDA_OK(cudaEventSynchronize(c->tB));
  float f = 0.f;
  CUDA_OK(cudaEventElapsedTime(&f, c->tA, c->tB));
  if (ms) *ms = f;
  API_END(c)
}
int sphgpu_neighbor_count(sphgpu_handle c, long* entries) {
  API_BEGIN(c)
  if (c->haveNeighbors) resolveNeighbors(c);
  if (entries) *entries = (long)c->nnbr;
  API_END(c)
}
int sphgpu_synchronize(sphgpu_handle c) {
  API_BEGIN(c)
  CUDA_OK(cudaStreamSynchronize(c->stream));
  API_END(c)
}

}  // extern "C"
