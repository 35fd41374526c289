// Device-wide exclusive scan and stable LSD radix sort (uint32 keys, int32
// values), written for the cell-list build of the neighbour search.
// Both are deterministic: equal keys keep their input order, so the particle
// order -- and with it every summation order downstream -- is reproducible.
#include "sort.cuh"

namespace sph {

namespace {
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T>
__device__ __forceinline__ T blockExclusiveScan(T v, T* smem, T* total) {
  // Warp-level inclusive scan then a scan over warp totals.
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    T w = lane < nw ? smem[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) smem[lane] = w;   // inclusive warp totals
  }
  __syncthreads();
  const T warpPrefix = warp > 0 ? smem[warp - 1] : T(0);
  const T result = warpPrefix + x - v;
  if (total) *total = smem[(blockDim.x >> 5) - 1];
  __syncthreads();
  return result;
}

template <typename Tin>
__global__ void scanReduceKernel(const Tin* __restrict__ in, long n, long long* __restrict__ blockSums) {
  __shared__ long long smem[32];
  const long base = (long)blockIdx.x * kScanTile;
  long long s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const long idx = base + (long)threadIdx.x * kScanItems + k;
    if (idx < n) s += (long long)in[idx];
  }
  long long tot;
  blockExclusiveScan<long long>(s, smem, &tot);
  if (threadIdx.x == 0) blockSums[blockIdx.x] = tot;
}

__global__ void scanBlockSumsKernel(long long* __restrict__ sums, int nb, long long* __restrict__ grandTotal) {
  __shared__ long long smem[32];
  const int per = (nb + blockDim.x - 1) / blockDim.x;
  const int beg = threadIdx.x * per;
  long long local = 0;
  for (int k = 0; k < per; ++k) if (beg + k < nb) local += sums[beg + k];
  long long tot;
  long long run = blockExclusiveScan<long long>(local, smem, &tot);
  for (int k = 0; k < per; ++k) {
    if (beg + k < nb) { const long long v = sums[beg + k]; sums[beg + k] = run; run += v; }
  }
  if (threadIdx.x == 0 && grandTotal) *grandTotal = tot;
}

template <typename Tin>
__global__ void scanDownsweepKernel(const Tin* __restrict__ in, long n, const long long* __restrict__ blockSums,
                                    long long* __restrict__ out) {
  __shared__ long long smem[32];
  const long base = (long)blockIdx.x * kScanTile;
  long long vals[kScanItems];
  long long s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const long idx = base + (long)threadIdx.x * kScanItems + k;
    vals[k] = idx < n ? (long long)in[idx] : 0;
    s += vals[k];
  }
  long long run = blockExclusiveScan<long long>(s, smem, nullptr) + blockSums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const long idx = base + (long)threadIdx.x * kScanItems + k;
    if (idx < n) out[idx] = run;
    run += vals[k];
  }
}
}  // namespace

size_t scanWorkspaceBytes(long n) {
  const long nb = (n + kScanTile - 1) / kScanTile;
  return (size_t)(nb + 2) * sizeof(long long);
}

template <typename Tin>
void scanExclusive(const Tin* in, long long* out, long n, void* workspace, long long* dTotal, cudaStream_t s,
                   LaunchCounter* lc) {
  const long nb = (n + kScanTile - 1) / kScanTile;
  long long* sums = static_cast<long long*>(workspace);
  if (n == 0) {
    cudaMemsetAsync(dTotal, 0, sizeof(long long), s);
    return;
  }
  scanReduceKernel<Tin><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, sums);
  scanBlockSumsKernel<<<1, 1024, 0, s>>>(sums, (int)nb, dTotal);
  scanDownsweepKernel<Tin><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, sums, out);
  if (lc) lc->add(3);
}
template void scanExclusive<int>(const int*, long long*, long, void*, long long*, cudaStream_t, LaunchCounter*);
template void scanExclusive<long long>(const long long*, long long*, long, void*, long long*, cudaStream_t,
                                       LaunchCounter*);

//------------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.
//------------------------------------------------------------------------------
namespace {
constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortThreads * kSortRounds;
constexpr int kWarps = kSortThreads / 32;

__global__ void radixHistKernel(const uint32_t* __restrict__ keys, long n, int shift, int numBlocks,
                                unsigned* __restrict__ blockHist) {
  __shared__ unsigned hist[256];
  hist[threadIdx.x] = 0;
  __syncthreads();
  const long base = (long)blockIdx.x * kSortTile;
#pragma unroll
  for (int r = 0; r < kSortRounds; ++r) {
    const long idx = base + (long)r * kSortThreads + threadIdx.x;
    if (idx < n) atomicAdd(&hist[(keys[idx] >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  blockHist[(long)threadIdx.x * numBlocks + blockIdx.x] = hist[threadIdx.x];
}

__global__ void radixScatterKernel(const uint32_t* __restrict__ keysIn, const int* __restrict__ valsIn, long n,
                                   int shift, int numBlocks, const long long* __restrict__ offsets,
                                   uint32_t* __restrict__ keysOut, int* __restrict__ valsOut) {
  __shared__ unsigned warpCnt[kWarps][256];
  __shared__ unsigned running[256];
  __shared__ unsigned roundTot[256];
  __shared__ long long blockOff[256];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  running[t] = 0;
  blockOff[t] = offsets[(long)t * numBlocks + blockIdx.x];
  const long base = (long)blockIdx.x * kSortTile;
  const unsigned lanemaskLt = (1u << lane) - 1u;
  for (int r = 0; r < kSortRounds; ++r) {
#pragma unroll
    for (int w = 0; w < kWarps; ++w) warpCnt[w][t] = 0;
    __syncthreads();
    const long idx = base + (long)r * kSortThreads + t;
    const bool valid = idx < n;
    uint32_t key = 0;
    int val = 0;
    unsigned digit = 256u + (unsigned)lane;   // unique dummy digit for idle lanes
    if (valid) { key = keysIn[idx]; val = valsIn[idx]; digit = (key >> shift) & 0xffu; }
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const unsigned rankInWarp = __popc(peers & lanemaskLt);
    const int leader = __ffs(peers) - 1;
    if (valid && lane == leader) warpCnt[warp][digit] = __popc(peers);
    __syncthreads();
    unsigned tot = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) tot += warpCnt[w][t];
    roundTot[t] = tot;
    if (valid) {
      unsigned before = 0;
      for (int w = 0; w < warp; ++w) before += warpCnt[w][digit];
      const long long pos = blockOff[digit] + running[digit] + before + rankInWarp;
      keysOut[pos] = key;
      valsOut[pos] = val;
    }
    __syncthreads();
    running[t] += roundTot[t];
    __syncthreads();
  }
}
}  // namespace

size_t radixSortWorkspaceBytes(long n) {
  const long nb = (n + kSortTile - 1) / kSortTile;
  const long nh = nb * 256;
  return (size_t)nh * sizeof(unsigned) + (size_t)nh * sizeof(long long) + scanWorkspaceBytes(nh) + 64;
}

void radixSortPairs(uint32_t*& keys, int*& vals, uint32_t*& keysAlt, int*& valsAlt, long n, int bits,
                    void* workspace, cudaStream_t s, LaunchCounter* lc) {
  if (n <= 1) return;
  const long nb = (n + kSortTile - 1) / kSortTile;
  const long nh = nb * 256;
  char* ws = static_cast<char*>(workspace);
  unsigned* hist = reinterpret_cast<unsigned*>(ws);
  long long* offs = reinterpret_cast<long long*>(ws + ((nh * sizeof(unsigned) + 15) / 16) * 16);
  void* scanWs = reinterpret_cast<char*>(offs) + nh * sizeof(long long);
  long long* dTot = reinterpret_cast<long long*>(static_cast<char*>(scanWs) + scanWorkspaceBytes(nh) - 16);
  for (int shift = 0; shift < bits; shift += 8) {
    radixHistKernel<<<(unsigned)nb, kSortThreads, 0, s>>>(keys, n, shift, (int)nb, hist);
    scanExclusive<unsigned>(hist, offs, nh, scanWs, dTot, s, lc);
    radixScatterKernel<<<(unsigned)nb, kSortThreads, 0, s>>>(keys, vals, n, shift, (int)nb, offs, keysAlt, valsAlt);
    if (lc) lc->add(2);
    std::swap(keys, keysAlt);
    std::swap(vals, valsAlt);
  }
}
template void scanExclusive<unsigned>(const unsigned*, long long*, long, void*, long long*, cudaStream_t,
                                      LaunchCounter*);

}  // namespace sph
