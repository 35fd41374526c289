// Host-callable launchers of the hydro kernels (defined in hydro.cu) and the
// gravity kernels (gravity.cu).
#pragma once
#include "fields.cuh"
#include "sort.cuh"

namespace sph {

struct TableDev {
  const double* w;      // 3*(N1+1) quadratic coefficients of W
  const double* g;      // 3*(N1+1) quadratic coefficients of dW/deta
  const double* herm;   // 2*hermN Hermite knots of the nperh lookup (values, slopes)
  const float* w32;     // FP32 copies for the FP32 pair loop
  const float* g32;
  const float4* p32a;   // per interval (w0, w1, w2, g0) in FP32
  const float2* p32b;   // per interval (g1, g2) in FP32
};

struct NeighborLists {
  const uint32_t* nbr;      // entries (index | cell-offset code << 26), warp-interleaved with capacity cap
  const int* count;         // neighbours per node
  int cap;                  // slots per node
  const uint32_t* cell;     // home cell of every node (packed, 10 bits per axis)
};

// Reductions ------------------------------------------------------------------
// out[0] = min hinv, out[1..3] = min x,y,z, out[4..6] = max x,y,z,
// out[7..9] = (tensor H) max over nodes of sqrt((H^-2)_aa) per axis, else 0
constexpr int kBoundsVals = 10;
void launchBounds(const Fields& F, long n, bool tensor, double* dScratch, int nScratch, double* dOut, cudaStream_t s,
                  LaunchCounter* lc);

// Neighbour build -------------------------------------------------------------
void launchCellKeys(const Fields& F, long n, Grid g, uint32_t* keys, int* vals, uint32_t* cellc, cudaStream_t s,
                    LaunchCounter* lc);
// carriedOnly: move only the state and the derivatives the next step reads
// before recomputing them (the step rewrites every other field before it
// returns); otherwise every permuted field.
void launchPermute(const Fields& Fin, Fields Fout, const int* perm, const int* origIn, int* origOut,
                   const int* listIn, int* listOut, const uint32_t* cellIn, uint32_t* cellOut, long n,
                   bool carriedOnly, bool tensor, bool crk, cudaStream_t s, LaunchCounter* lc);
// The limited Q's DvDx <- the hydro DvDx; and its FP32 mirror (3 float4 per node).
void launchCopyQGradient(Fields F, long n, cudaStream_t s, LaunchCounter* lc);
void launchQGradient32(Fields F, float4* dvq, long n, cudaStream_t s, LaunchCounter* lc);
// shift: sub-cell key bits below the cell key (Grid::subShift).
void launchCellRanges(const uint32_t* sortedKeys, long n, int shift, int* cellStart, int* cellEnd, cudaStream_t s,
                      LaunchCounter* lc);
// Bounding boxes of the work chunks (for the batch culling of the search).
void launchItemBoxes(const int* items, const long long* dItems, int nItemsBound, long n, int width, Fields32 P,
                     float4* box, int* chunkOf, cudaStream_t s, LaunchCounter* lc);
// Group-cooperative neighbour search over items (first node of each chunk of
// up to `width` nodes of a cell).
// width: nodes per work item of the group-cooperative search (8, 16 or 32).
void launchItemFlags(const uint32_t* keys, long n, int shift, const int* cellStart, int width, int* flag,
                     cudaStream_t s, LaunchCounter* lc);
void launchItemFill(const int* flag, const long long* pos, long n, int* items, cudaStream_t s, LaunchCounter* lc);
// nItems: an upper bound on the item count (sizes the grid); *dItems (device)
// holds the count itself.
void launchNeighborsWarp(const Fields& F, Fields32 P, long n, const int* items, int nItems, const long long* dItems,
                         int width, Grid g, const int* cellStart, const int* cellEnd, int* counts, int* maxCount,
                         uint32_t* nbr, int cap, double ext2, bool tensor, const float4* box, const int* chunkOf,
                         cudaStream_t s, LaunchCounter* lc);

// Sweeps ---------------------------------------------------------------------
void launchSumDensity(Fields F, const int* list, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                      cudaStream_t s, LaunchCounter* lc);
void launchGradh(Fields F, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp, cudaStream_t s,
                 LaunchCounter* lc);
void launchPairFP64(Fields F, const int* list, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                    double* pacc, int blockSize, cudaStream_t s, LaunchCounter* lc);
constexpr int kPairVariants = 4;   // autotuned variants of launchPairFP32 (common path)
constexpr int kRetuneAfter = 2;    // uses between an autotuner's first timing and its one retiming
constexpr int kPairVariantsTensor = 4;   // of its tensor-H (ASPH) path
constexpr int kPairVariantsCRK = 2;      // of the mixed CRKSPH pair kernel
void launchPairFP32(Fields F, Fields32 F32, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                    HydroParams hp, float* pacc, int variant, cudaStream_t s,
                    LaunchCounter* lc);
void launchPrepareFP32(Fields F, Fields32 F32, long n, Grid g, cudaStream_t s, LaunchCounter* lc);
void launchSumDensityFP32(Fields F, Fields32 F32, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                          HydroParams hp, cudaStream_t s, LaunchCounter* lc);
void launchGradhFP32(Fields F, Fields32 F32, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                     cudaStream_t s, LaunchCounter* lc);
void launchDtFP32(Fields F, Fields32 F32, const int* list, long n, Grid g, NeighborLists nl, HydroParams hp,
                  double maxNperh, double* dScratch, int nScratch, double* dOut,
                  cudaStream_t s, LaunchCounter* lc);
// Mixed mode: density sum and dt vote fused in one sweep (dOut as launchDt).
void launchDensityDtFP32(Fields F, Fields32 F32, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                         HydroParams hp, double maxNperh, double* dScratch,
                         double* dOut, cudaStream_t s, LaunchCounter* lc);
// dt: writes per-block (value, reason) pairs then a final min into dOut[0], dOut[1] (reason as double)
void launchDt(Fields F, const int* list, long n, Grid g, NeighborLists nl, HydroParams hp,
              double maxNperh, double* dScratch, int nScratch, double* dOut,
              cudaStream_t s, LaunchCounter* lc);
void launchCompatibleEnergy(Fields F, long n, Grid g, NeighborLists nl, const double* pacc, const float* pacc32,
                            double dt, cudaStream_t s, LaunchCounter* lc);
// variant: slots per batch of the sweep, 0 -> 4, 1 -> 8, 2 -> 2 (the same
// result for every variant; picked by the autotuner).
constexpr int kEnergyVariants = 3;
void launchCompatibleEnergyFP32(Fields F, long n, Grid g, NeighborLists nl, const float* pacc, float4* vhi,
                                float4* vlo, double dt, int variant, cudaStream_t s, LaunchCounter* lc);
// state0 -> state (the copy is taken by the half-step update); tensor: also
// the tensor H (ASPH)
void launchRestoreState0(Fields F, long n, bool tensor, bool crk, cudaStream_t s, LaunchCounter* lc);
// CRKSPH (crk.cu): the RK volumes (RKCorrections::preStepInitialize), the CRK
// mass density sum (CRKSPHBase::preStepInitialize), the LinearOrder
// corrections (RKCorrections::initialize) and the CRKSPH pair loop with the
// SPHSmoothingScale moments and node finalize (FP64).
void launchRKVolumes(Fields F, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp, cudaStream_t s,
                     LaunchCounter* lc);
void launchCRKDensity(Fields F, const int* list, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                      cudaStream_t s, LaunchCounter* lc);
void launchRKCorrections(Fields F, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp, cudaStream_t s,
                         LaunchCounter* lc);
void launchPairCRK(Fields F, const int* list, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                   double* pacc, cudaStream_t s, LaunchCounter* lc);
// Mixed-precision CRKSPH (crk32.cu): FP32 sweeps on the FP32 mirror, FP64
// per-node completions; the volume and correction mirrors are written too.
void launchRKVolumesFP32(Fields F, Fields32 P, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                         cudaStream_t s, LaunchCounter* lc);
void launchCRKDensityFP32(Fields F, Fields32 P, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                          HydroParams hp, cudaStream_t s, LaunchCounter* lc);
void launchRKCorrectionsFP32(Fields F, Fields32 P, long n, Grid g, NeighborLists nl, TableDev t, HydroParams hp,
                             cudaStream_t s, LaunchCounter* lc);
// variant: 0 one neighbour slot per loop iteration, 1 two (autotuned,
// kPairVariantsCRK; the same bits either way)
void launchPairCRKFP32(Fields F, Fields32 P, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                       HydroParams hp, float* pacc, int variant, cudaStream_t s, LaunchCounter* lc);
// ASPH: F_HINV / F_HLMAX <- smallest / largest eigenvalue of the tensor H
void launchTensorExtent(Fields F, long n, cudaStream_t s, LaunchCounter* lc);
// ASPH radialOnly: F_RAD0 <- |x|
void launchRadius0(Fields F, long n, cudaStream_t s, LaunchCounter* lc);
// mid == true: save the beginning-of-step copies (state0), then the
// timeAdvanceOnly increment with multiplier; else full update (eps
// already advanced by the compatible-energy sweep when compatible).  mirror:
// also refresh the FP32 mirrors of the new state (mixed mode), cells of grid g.
void launchUpdate(Fields F, const int* list, long n, HydroParams hp, double mult,
                  bool mid, bool gravity, const Fields32* mirror, const Grid& g, cudaStream_t s, LaunchCounter* lc);
// ASPHSmoothingScale end of step: zeroth moment, IdealH and limits of H
// (P.posh non-null: the mixed mode's FP32 extents and mirrors are refreshed).
void launchASPHEnd(Fields F, Fields32 P, const int* list, long n, Grid g, NeighborLists nl, TableDev t,
                   HydroParams hp, cudaStream_t s, LaunchCounter* lc);
// lists: device table of NodeListParams (HydroParams::lists).
void launchEOS(Fields F, const int* list, long n, const NodeListParams* lists, cudaStream_t s, LaunchCounter* lc);
void launchEnforce(Fields F, long n, Grid g, bool tensor, cudaStream_t s, LaunchCounter* lc);
// out[0..7] conservation totals
void launchConservation(Fields F, long n, bool gravity, double* dScratch, int nScratch, double* dOut, cudaStream_t s,
                        LaunchCounter* lc);
// Domain-decomposition exchange rows: w field ids; mirror 1 refreshes the FP32
// density mirror, 2 the FP32 grad-h mirror of the halo nodes after a put.
struct ExchangeFields {
  int w, mirror;
  int ids[8];
};
void launchExchangeGet(Fields F, const int* inv, const int* idx, long count, ExchangeFields ef, double* out,
                       cudaStream_t s, LaunchCounter* lc);
void launchExchangePut(Fields F, Fields32 P, const int* inv, long nOwn, long count, ExchangeFields ef,
                       const double* in, cudaStream_t s, LaunchCounter* lc);
// caller-order transfers through a device staging buffer (stride doubles per node)
void launchGatherOut(Fields F, const int* orig, double* stage, int first, int ncomp, int stride, long n,
                     cudaStream_t s, LaunchCounter* lc);
void launchScatterIn(Fields F, const int* orig, const double* stage, int first, int ncomp, int stride, long n,
                     cudaStream_t s, LaunchCounter* lc);
void launchGatherOutH(Fields F, const int* orig, double* stage, int field, long n, cudaStream_t s, LaunchCounter* lc);
// caller-order transfers on pinned host arrays addressed in place (inv: the
// internal index of each caller index)
void launchInverseOrder(const int* orig, int* inv, long n, cudaStream_t s, LaunchCounter* lc);
void launchScatterInHost(Fields F, const int* inv, const double* src, int first, int ncomp, int stride, long n,
                         cudaStream_t s, LaunchCounter* lc);
void launchGatherOutHost(Fields F, const int* inv, double* dst, int first, int ncomp, int stride, bool isoH, long n,
                         cudaStream_t s, LaunchCounter* lc);
void launchCountsOut(const int* counts, const int* orig, double* stage, long n, cudaStream_t s, LaunchCounter* lc);
// check finite / positive state: writes a flag
void launchCheckState(Fields F, long n, int* dFlag, cudaStream_t s, LaunchCounter* lc);

// Gravity (gravity.cu) ---------------------------------------------------------
struct GravityWork;
GravityWork* gravityCreate();
void gravityDestroy(GravityWork* w);
// Build the octree of the current positions and walk it; writes F_GRAV_*,
// F_POT (already multiplied by G) and returns dtMinAcc via dOut[0], extra
// energy via dOut[1].
// mixed: FP32 interaction terms on double-float coordinates with compensated
// accumulation (decisions as in FP64); otherwise FP64 throughout.
int gravityEvaluate(GravityWork* w, Fields F, long n, double G, double softening, double opening, bool mixed,
                    double* dOut,
                    cudaStream_t s, LaunchCounter* lc, char* err, int errlen);

}  // namespace sph
