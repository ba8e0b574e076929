// Self-test of the integer-pipe binary64 multiply (spd_emul.cuh) against the
// FP64 multiply on the device, over generated operand pairs covering the
// whole exponent range, ties and sticky bits, and special values.
#include <cuda_runtime.h>

#include "../../include/spd_gb300.h"
#include "spd_emul.cuh"

namespace {

__device__ __forceinline__ unsigned long long splitmix(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ double make_operand(unsigned long long r, int mode) {
  const unsigned long long sign = r & 0x8000000000000000ull;
  unsigned long long frac = r & 0x000FFFFFFFFFFFFFull;
  unsigned long long e;
  if (mode <= 4) {
    e = 1 + (r >> 52) % 2046;                      // any normal exponent
  } else if (mode == 5) {
    e = 1023 - 40 + (r >> 52) % 80;                // everyday magnitudes
  } else if (mode == 6) {
    e = 1023 - 40 + (r >> 52) % 80;
    const unsigned k = (unsigned)((r >> 40) % 53);  // many trailing zeros: ties and sticky edges
    frac &= ~((1ull << k) - 1ull);
  } else {
    const unsigned pick = (unsigned)((r >> 52) % 8);
    if (pick == 0) return __longlong_as_double((long long)sign);                 // +-0
    if (pick == 1) return __longlong_as_double((long long)(sign | (frac | 1)));  // subnormal
    if (pick == 2) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));  // inf
    if (pick == 3) return __longlong_as_double((long long)(0x7FF8000000000000ull | frac));  // NaN
    if (pick == 4) e = 2046;
    else if (pick == 5) e = 1;
    else e = 1 + (r >> 52) % 2046;
  }
  return __longlong_as_double((long long)(sign | (e << 52) | frac));
}

__global__ void k_selftest_mul(long long n, unsigned long long seed, unsigned long long* mismatches) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  unsigned bad = 0;
  if (i < n) {
    const int mode = (int)(i % 8);
    const double a = make_operand(splitmix(seed + 2 * (unsigned long long)i), mode);
    const double b = make_operand(splitmix(seed + 2 * (unsigned long long)i + 1), (mode == 7) ? 7 : mode);
    const double x = __dmul_rn(a, b);
    const double y = spd::emul_mul(a, b);
    const bool both_nan = (x != x) && (y != y);
    bad = (!both_nan && __double_as_longlong(x) != __double_as_longlong(y)) ? 1u : 0u;
  }
  const unsigned b = __ballot_sync(0xffffffffu, bad);
  if (b && (threadIdx.x & 31) == 0) atomicAdd(mismatches, (unsigned long long)__popc(b));
}

}  // namespace

extern "C" int spd_selftest_fp64(long long n, unsigned long long seed, unsigned long long* mismatches_out) {
  if (n <= 0 || mismatches_out == nullptr) return SPD_ERR_ARG;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return SPD_ERR_CUDA;
  cudaMemset(d, 0, sizeof(unsigned long long));
  const int bs = 256;
  const long long chunk = 1LL << 28;
  for (long long off = 0; off < n; off += chunk) {
    const long long m = (n - off < chunk) ? n - off : chunk;
    k_selftest_mul<<<(unsigned)((m + bs - 1) / bs), bs>>>(m, seed + 2 * (unsigned long long)off, d);
  }
  const cudaError_t e = cudaDeviceSynchronize();
  unsigned long long h = 0;
  cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return SPD_ERR_CUDA;
  *mismatches_out = h;
  return SPD_OK;
}
