// CFL time step from device-resident primitive subcell averages, without
// any device allocation.
//
// Who needs this: callers that may not call cudaMalloc -- solvers embedded
// in a host framework whose caching allocator owns all device memory, and
// real-time loops that forbid allocation after start-up.  The dt is the
// inviscid CFL limit (compute_dt's viscous limit is not applied).  They hand in their own
// input and output buffers; the only scratch this entry point uses is the
// fixed array below, which lives in the library image.
//
// Scratch: kNoAllocMaxBlocks partial maxima (one per 256-thread block, 128 KB)
// in a file-scope __device__ array, so at most
// kNoAllocMaxBlocks * 256 = 4,194,304 subcells per call (a 512x512 grid at
// p = 3).  Every GPU that loads the library keeps this array until the
// process exits.  Each call writes every slot it reads, so nothing has to be
// cleared between calls; calls that overlap on the GPU (two streams, or two
// host threads) share the array and race.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "../../include/spd_gb300.h"
#include "spd_device.cuh"

namespace {

constexpr int kNoAllocBlock = 256;
constexpr long long kNoAllocMaxBlocks = 16384;

__device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks];

// device address of g_noalloc_partials, looked up once per device
constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

// pass 1: per-block maximum of ndim*c_s + sum |v| over the block's subcells
// (src/sd_simulator.py:214-222); a NaN anywhere in the block becomes the
// block's partial so that it propagates like np.max.
template <int D>
__global__ void k_noalloc_cmax(const double* __restrict__ W, long long nq, double gamma, double min_c2,
                               double* __restrict__ partials) {
  constexpr int P_ = D + 1;
  __shared__ double red[kNoAllocBlock];
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double c = 0.0;
  if (q < nq) {
    c = spd::sound_speed(W[(long long)P_ * nq + q], W[q], gamma, min_c2) * (double)D;
#pragma unroll
    for (int v = 1; v <= D; ++v) c = c + fabs(W[(long long)v * nq + q]);
  }
  red[threadIdx.x] = c;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = spd::np_max(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

// pass 2: one block reduces the partials; dt = cfl * (h / c_max)
__global__ void k_noalloc_dt(const double* __restrict__ partials, int nblocks, double h, double cfl,
                             double* __restrict__ dt_out) {
  __shared__ double red[kNoAllocBlock];
  double m = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) m = spd::np_max(m, partials[i]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = spd::np_max(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double dt = h / red[0];
    *dt_out = cfl * dt;
  }
}

// Looks up the device address of the scratch array for the current device
// (first call on each device; cudaGetSymbolAddress allocates nothing).
int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SPD_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_ptr[dev] == nullptr) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_partials) != cudaSuccess || ptr == nullptr) return SPD_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(ptr);
  }
  *out = g_scratch_ptr[dev];
  return SPD_OK;
}

}  // namespace

extern "C" int spd_cfl_dt_noalloc(const double* W_cv_dev, long long n_subcells, int ndim, double gamma,
                                  double min_c2, double cfl_coeff, double h, double* dt_dev, void* stream) {
  if (W_cv_dev == nullptr || dt_dev == nullptr || n_subcells <= 0 || ndim < 1 || ndim > 3) return SPD_ERR_ARG;
  const long long nblocks = (n_subcells + kNoAllocBlock - 1) / kNoAllocBlock;
  if (nblocks > kNoAllocMaxBlocks) return SPD_ERR_ARG;  // more than 4,194,304 subcells
  double* partials = nullptr;
  if (int rc = scratch_for_current_device(&partials)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (ndim) {
    case 1: k_noalloc_cmax<1><<<(unsigned)nblocks, kNoAllocBlock, 0, s>>>(W_cv_dev, n_subcells, gamma, min_c2, partials); break;
    case 2: k_noalloc_cmax<2><<<(unsigned)nblocks, kNoAllocBlock, 0, s>>>(W_cv_dev, n_subcells, gamma, min_c2, partials); break;
    default: k_noalloc_cmax<3><<<(unsigned)nblocks, kNoAllocBlock, 0, s>>>(W_cv_dev, n_subcells, gamma, min_c2, partials); break;
  }
  if (cudaGetLastError() != cudaSuccess) return SPD_ERR_CUDA;
  k_noalloc_dt<<<1, kNoAllocBlock, 0, s>>>(partials, (int)nblocks, h, cfl_coeff, dt_dev);
  if (cudaGetLastError() != cudaSuccess) return SPD_ERR_CUDA;
  return SPD_OK;
}
