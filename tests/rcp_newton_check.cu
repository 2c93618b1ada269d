// Exhaustive check of nbd::rcp_newton (nb_device.cuh) against the correctly rounded division:
// every float b in [kRcpNewtonMin, kRcpNewtonMax).  Prints the count of differing results and
// the first differing input; exits 1 on any difference.  Built and run by
// tests/test_gpu_reciprocal.py with the library's own compiler flags.
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "nb_device.cuh"

__global__ void k_check(uint32_t lo, uint32_t hi, unsigned long long* bad, uint32_t* first) {
  for (uint64_t i = (uint64_t)lo + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < hi;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float b = __uint_as_float((uint32_t)i);
    const float r = nbd::rcp_newton(b), ref = 1.0f / b;
    if (__float_as_uint(r) != __float_as_uint(ref)) {
      atomicAdd(bad, 1ull);
      atomicMin(first, (uint32_t)i);
    }
  }
}

int main() {
  const float lo_f = nbd::kRcpNewtonMin, hi_f = nbd::kRcpNewtonMax;
  uint32_t lo, hi;
  std::memcpy(&lo, &lo_f, 4);
  std::memcpy(&hi, &hi_f, 4);
  unsigned long long* bad = nullptr;
  uint32_t* first = nullptr;
  if (cudaMalloc(&bad, 8) != cudaSuccess || cudaMalloc(&first, 4) != cudaSuccess) return 2;
  cudaMemset(bad, 0, 8);
  cudaMemset(first, 0xFF, 4);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  k_check<<<sms * 16, 256>>>(lo, hi, bad, first);
  const cudaError_t e = cudaDeviceSynchronize();
  unsigned long long n_bad = 0;
  uint32_t first_bad = 0;
  cudaMemcpy(&n_bad, bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(&first_bad, first, 4, cudaMemcpyDeviceToHost);
  std::printf("cuda=%d values=%u mismatches=%llu first=%08x\n", (int)e, hi - lo, n_bad, first_bad);
  cudaFree(bad);
  cudaFree(first);
  return (e != cudaSuccess || n_bad) ? 1 : 0;
}
