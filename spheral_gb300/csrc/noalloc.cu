// Conserved totals of caller-owned device arrays without any allocation.
//
// Some callers of this library cannot allocate GPU memory while they run: a
// host code that hands the library slices of its own pre-allocated device
// pools (with a memory pool that forbids outside cudaMalloc/cudaFree), code
// running inside a region where allocation would synchronise the device, or
// a driver that must keep its footprint fixed once it has started.  For them
// sphgpu_conservation_noalloc computes the same totals as sphgpu_conservation
// from device arrays they pass in, using a fixed scratch array that lives in
// the library itself.
//
// The scratch is a file-scope __device__ array of kNoAllocBlocks x 7 doubles
// (57,344 bytes).  Every GPU that loads the library holds it until the
// process exits, and all calls on a device share it: calls that overlap on
// the GPU (on different streams, or from different host threads) race on it
// and must be serialised by the caller.
#include "../../include/sphgpu.h"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocBlocks = 1024;                   // one partial set per block
constexpr long kNoAllocMaxNodes = 1L << 26;            // 67,108,864 nodes
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noallocPartials[kNoAllocBlocks * 7];

// Device address of the scratch array per device ordinal.  In host code the
// symbol g_noallocPartials is only a host-side stand-in, so the address must
// come from cudaGetSymbolAddress with that device current.
std::mutex g_mutex;
double* g_partialsPtr[kMaxDevices] = {};

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

// Per-block partial sums: mass, momentum (3), kinetic, thermal, 1/2 m phi.
__global__ void noallocPartialKernel(const double* __restrict__ mass, const double* __restrict__ vel,
                                     const double* __restrict__ eps, const double* __restrict__ pot, long n,
                                     double* __restrict__ partials) {
  __shared__ double sm[32];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double m = mass[i], vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
    acc[0] += m;
    acc[1] += m * vx;
    acc[2] += m * vy;
    acc[3] += m * vz;
    acc[4] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
    acc[5] += m * eps[i];
    if (pot) acc[6] += 0.5 * m * pot[i];
  }
  for (int k = 0; k < 7; ++k) {
    const double r = blockSum(acc[k], sm);
    if (threadIdx.x == 0) partials[blockIdx.x * 7 + k] = r;
  }
}

__global__ void noallocFinalKernel(const double* __restrict__ partials, int nb, double* __restrict__ out) {
  __shared__ double sm[32];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int k = 0; k < 7; ++k) acc[k] += partials[b * 7 + k];
  for (int k = 0; k < 7; ++k) {
    const double r = blockSum(acc[k], sm);
    if (threadIdx.x == 0) out[k] = r;
  }
  if (threadIdx.x == 0) out[7] = out[4] + out[5] + out[6];
}

}  // namespace

extern "C" int sphgpu_conservation_noalloc(const double* mass, const double* vel, const double* eps,
                                           const double* pot, long n, double* out, void* stream) {
  if (!mass || !vel || !eps || !out || n <= 0) return SPHGPU_E_ARG;
  if (n > kNoAllocMaxNodes) return SPHGPU_E_OVERFLOW;   // beyond the fixed-scratch limit
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SPHGPU_E_CUDA;
  double* partials;
  {
    // First call on this device: look up the scratch address with the device
    // current.  Make that first call before any stream capture begins.
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_partialsPtr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noallocPartials) != cudaSuccess || !p) return SPHGPU_E_CUDA;
      g_partialsPtr[dev] = static_cast<double*>(p);
    }
    partials = g_partialsPtr[dev];
  }
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  long nb = (n + kNoAllocThreads - 1) / kNoAllocThreads;
  if (nb > kNoAllocBlocks) nb = kNoAllocBlocks;
  // Every block overwrites its own partials and the final pass reads only
  // those nb sets, so nothing from an earlier call needs clearing.  The
  // launches go through cudaLaunchKernel, whose return code is this launch's
  // own: an error left pending by some earlier, unrelated launch on the
  // thread is neither reported as this call's failure nor cleared by it.
  int nbi = (int)nb;
  void* partialArgs[] = {(void*)&mass, (void*)&vel, (void*)&eps, (void*)&pot, (void*)&n, (void*)&partials};
  if (cudaLaunchKernel((const void*)noallocPartialKernel, dim3((unsigned)nb), dim3(kNoAllocThreads), partialArgs,
                       0, s) != cudaSuccess)
    return SPHGPU_E_CUDA;
  void* finalArgs[] = {(void*)&partials, (void*)&nbi, (void*)&out};
  if (cudaLaunchKernel((const void*)noallocFinalKernel, dim3(1), dim3(kNoAllocThreads), finalArgs, 0, s) !=
      cudaSuccess)
    return SPHGPU_E_CUDA;
  return SPHGPU_OK;
}
