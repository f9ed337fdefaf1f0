// kcheck.cu -- count the non-finite values (NaN or +-Inf) of a job's state.
//
// A value is non-finite when all bits of its exponent field are set.  One
// launch per buffer: each thread counts over a grid-stride range, each warp
// sums its threads' counts (__reduce_add_sync) and one lane adds the sum to
// the device counter.
#include <cuda_runtime.h>

#include <cstdint>

#include "fdtd_internal.h"

namespace fdtd {
namespace {

template <typename U, U kExp>
__global__ void __launch_bounds__(256) count_nonfinite(const U *__restrict__ a, size_t n,
                                                       unsigned long long *__restrict__ out) {
  unsigned cnt = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    cnt += (__ldg(a + i) & kExp) == kExp;
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(out, (unsigned long long)cnt);
}

}  // namespace

// bytes of float (esz 4) or double (esz 8) elements at p, counted into *out
int launch_count_nonfinite(const void *p, size_t bytes, int esz, unsigned long long *out, int num_sms,
                           void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const size_t n = bytes / (size_t)esz;
  if (n == 0) return 0;
  const size_t want = (n + 255) / 256;
  const int blocks = (int)(want < (size_t)num_sms * 8 ? want : (size_t)num_sms * 8);
  if (esz == 4)
    count_nonfinite<uint32_t, 0x7f800000u><<<blocks, 256, 0, s>>>((const uint32_t *)p, n, out);
  else
    count_nonfinite<uint64_t, 0x7ff0000000000000ull><<<blocks, 256, 0, s>>>((const uint64_t *)p, n, out);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace fdtd
