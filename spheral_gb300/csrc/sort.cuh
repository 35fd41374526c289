// Scan / sort utilities of libsphgpu.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <utility>

namespace sph {

// Counts kernel launches issued by the library (reported by sphgpu_launch_count).
struct LaunchCounter {
  long n = 0;
  void add(long k) { n += k; }
};

size_t scanWorkspaceBytes(long n);
// out[i] = sum_{k<i} in[k] (int64); *dTotal (device) = sum of all.
template <typename Tin>
void scanExclusive(const Tin* in, long long* out, long n, void* workspace, long long* dTotal, cudaStream_t s,
                   LaunchCounter* lc);

size_t radixSortWorkspaceBytes(long n);
// Stable sort of (keys, vals) by the low `bits` bits of keys.  The pointers are
// ping-ponged: on return keys/vals point at the sorted data.
void radixSortPairs(uint32_t*& keys, int*& vals, uint32_t*& keysAlt, int*& valsAlt, long n, int bits,
                    void* workspace, cudaStream_t s, LaunchCounter* lc);

}  // namespace sph
