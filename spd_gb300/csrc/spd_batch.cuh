// Batched launches: one kernel launch runs one stage of the step for many
// independent problem instances at once.
//
// Every step kernel is a body ``Body::run(Blk, args...)`` (spd_kernels.cuh,
// spd_fv.cuh, spd_stepper.cuh).  A batched launch k_batched<Body, A...>
// covers the blocks of all instances back to back; a per-instance table of
// block offsets (boff[i] = first block of instance i, boff[n] = total) maps
// each block to its instance, whose argument pack (geometry, operators,
// buffer pointers, its own dt pointer) is read from device memory, and to
// its block index within that instance.  Each block thus does exactly what
// it does in the instance's own launch, so results are bit-identical.
//
// The host side records the launch sequence of one step per instance
// (BatchRec: the stepper runs with launches and zero-fills intercepted),
// checks that all instances produced the same sequence of bodies, block
// shapes and shared-memory sizes, and merges the i-th launch of every
// instance into one batched launch (Site).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "spd_device.cuh"

namespace spd_batch {
using spd::Blk;

// ---------------------------------------------------------------------------
// argument packs (same layout on host and device)
// ---------------------------------------------------------------------------
template <class... A>
struct Pack {};
template <class H, class... R>
struct Pack<H, R...> {
  H h;
  Pack<R...> r;
};

template <class... A>
struct PackBuild;
template <>
struct PackBuild<> {
  static Pack<> make() { return {}; }
};
template <class H, class... R>
struct PackBuild<H, R...> {
  template <class X, class... Y>
  static Pack<H, R...> make(X&& x, Y&&... y) {
    Pack<H, R...> p;
    p.h = static_cast<H>(std::forward<X>(x));
    p.r = PackBuild<R...>::make(std::forward<Y>(y)...);
    return p;
  }
};

#ifdef __CUDACC__
template <class Body, class... Got>
__device__ __forceinline__ void pack_call(const Blk& B, const Pack<>&, const Got&... got) {
  Body::run(B, got...);
}
template <class Body, class H, class... R, class... Got>
__device__ __forceinline__ void pack_call(const Blk& B, const Pack<H, R...>& p, const Got&... got) {
  pack_call<Body>(B, p.r, got..., p.h);
}

// instance of block b: the last i < n with boff[i] <= b (instances with no
// blocks have boff[i] == boff[i+1] and are skipped)
__host__ __device__ __forceinline__ int instance_of(const unsigned* __restrict__ boff, int n, unsigned b) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (boff[mid] <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <class Body, class... A>
__global__ void k_batched(const Pack<A...>* __restrict__ packs, const unsigned* __restrict__ boff, int n) {
  const int i = instance_of(boff, n, blockIdx.x);
  pack_call<Body>(Blk{blockIdx.x - boff[i], boff[i + 1] - boff[i]}, packs[i]);
}

struct ZeroRange {
  unsigned char* p;
  unsigned long long bytes;
};

// zero-fills of many instances' buffers in one launch: head bytes up to an
// 8-byte boundary, 8-byte words, tail bytes
static __global__ void k_zero_ranges(const ZeroRange* __restrict__ r, const unsigned* __restrict__ boff, int n) {
  const int i = instance_of(boff, n, blockIdx.x);
  const ZeroRange z = r[i];
  const unsigned long long t = (unsigned long long)(blockIdx.x - boff[i]) * blockDim.x + threadIdx.x;
  const unsigned long long stride = (unsigned long long)(boff[i + 1] - boff[i]) * blockDim.x;
  unsigned long long head = (8 - ((uintptr_t)z.p & 7)) & 7;
  if (head > z.bytes) head = z.bytes;
  const unsigned long long nw = (z.bytes - head) / 8;
  const unsigned long long tail = z.bytes - head - nw * 8;
  if (t < head) z.p[t] = 0;
  unsigned long long* w = reinterpret_cast<unsigned long long*>(z.p + head);
  for (unsigned long long k = t; k < nw; k += stride) w[k] = 0ULL;
  if (t < tail) z.p[head + nw * 8 + t] = 0;
}
#endif

// ---------------------------------------------------------------------------
// host: launch sites and the recorder
// ---------------------------------------------------------------------------
constexpr unsigned MAX_GRID = 0x7fffffffu;

struct SiteBase {
  const char* name = "";
  dim3 block{1, 1, 1};
  size_t smem = 0;
  std::vector<unsigned> boff{0};
  unsigned* d_boff = nullptr;
  virtual ~SiteBase() {
    if (d_boff) cudaFree(d_boff);
  }
  int count() const { return (int)boff.size() - 1; }
  virtual cudaError_t upload() = 0;
  virtual cudaError_t launch(cudaStream_t s) = 0;

 protected:
  cudaError_t upload_offsets() {
    cudaError_t e = cudaMalloc(&d_boff, sizeof(unsigned) * boff.size());
    if (e != cudaSuccess) return e;
    return cudaMemcpy(d_boff, boff.data(), sizeof(unsigned) * boff.size(), cudaMemcpyHostToDevice);
  }
};

#ifdef __CUDACC__
template <class Body, class... A>
struct Site : SiteBase {
  std::vector<Pack<A...>> packs;
  Pack<A...>* d_packs = nullptr;
  ~Site() override {
    if (d_packs) cudaFree(d_packs);
  }
  cudaError_t upload() override {
    cudaError_t e = upload_offsets();
    if (e != cudaSuccess) return e;
    e = cudaMalloc(&d_packs, sizeof(Pack<A...>) * packs.size());
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(d_packs, packs.data(), sizeof(Pack<A...>) * packs.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    if (smem > 48 * 1024)
      e = cudaFuncSetAttribute(k_batched<Body, A...>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return e;
  }
  cudaError_t launch(cudaStream_t s) override {
    if (boff.back() == 0) return cudaSuccess;
    k_batched<Body, A...><<<boff.back(), block, smem, s>>>(d_packs, d_boff, count());
    return cudaGetLastError();
  }
};

struct ZeroSite : SiteBase {
  std::vector<ZeroRange> ranges;
  ZeroRange* d_ranges = nullptr;
  ~ZeroSite() override {
    if (d_ranges) cudaFree(d_ranges);
  }
  cudaError_t upload() override {
    cudaError_t e = upload_offsets();
    if (e != cudaSuccess) return e;
    e = cudaMalloc(&d_ranges, sizeof(ZeroRange) * ranges.size());
    if (e != cudaSuccess) return e;
    return cudaMemcpy(d_ranges, ranges.data(), sizeof(ZeroRange) * ranges.size(), cudaMemcpyHostToDevice);
  }
  cudaError_t launch(cudaStream_t s) override {
    if (boff.back() == 0) return cudaSuccess;
    k_zero_ranges<<<boff.back(), block, 0, s>>>(d_ranges, d_boff, count());
    return cudaGetLastError();
  }
};
#endif

// Records the launch sequence of one step per instance.  The first instance
// creates the sites; every further instance must produce the same sequence.
struct BatchRec {
  std::vector<std::unique_ptr<SiteBase>> sites;
  size_t cursor = 0;
  bool first = true;
  std::string err;

  void begin_instance(bool is_first) {
    first = is_first;
    cursor = 0;
  }
  bool end_instance() {
    if (err.empty() && cursor != sites.size()) err = "instances record different step sequences (options differ)";
    return err.empty();
  }

#ifdef __CUDACC__
  template <class Body, class... A>
  void add(const char* name, dim3 grid, dim3 block, size_t smem, const Pack<A...>& p) {
    if (!err.empty()) return;
    if (grid.y != 1 || grid.z != 1) {
      err = std::string("batched launch needs a 1D grid: ") + name;
      return;
    }
    Site<Body, A...>* s = nullptr;
    if (first) {
      sites.emplace_back(new Site<Body, A...>());
      s = static_cast<Site<Body, A...>*>(sites.back().get());
      s->name = name;
      s->block = block;
      s->smem = smem;
    } else {
      if (cursor >= sites.size()) {
        err = "instances record different step sequences (options differ)";
        return;
      }
      s = dynamic_cast<Site<Body, A...>*>(sites[cursor].get());
      if (!s || s->block.x != block.x || s->block.y != block.y || s->block.z != block.z || s->smem != smem) {
        err = std::string("instances differ at launch ") + std::to_string(cursor) + " (" + name +
              "): options, degree or cells per block";
        return;
      }
    }
    ++cursor;
    if ((unsigned long long)s->boff.back() + grid.x > MAX_GRID) {
      err = std::string("batched grid too large at ") + name;
      return;
    }
    s->packs.push_back(p);
    s->boff.push_back(s->boff.back() + grid.x);
  }

  void add_zero(void* ptr, size_t bytes) {
    if (!err.empty()) return;
    ZeroSite* s = nullptr;
    if (first) {
      sites.emplace_back(new ZeroSite());
      s = static_cast<ZeroSite*>(sites.back().get());
      s->name = "k_zero_ranges";
      s->block = dim3(256, 1, 1);
    } else {
      if (cursor >= sites.size() || !(s = dynamic_cast<ZeroSite*>(sites[cursor].get()))) {
        err = "instances record different step sequences (options differ)";
        return;
      }
    }
    ++cursor;
    unsigned long long words = bytes / 8 + 1;
    unsigned long long nb = (words + 255) / 256;
    if (nb > 1024) nb = 1024;
    s->ranges.push_back(ZeroRange{static_cast<unsigned char*>(ptr), (unsigned long long)bytes});
    s->boff.push_back(s->boff.back() + (unsigned)nb);
  }
#endif

  cudaError_t upload() {
    for (auto& s : sites) {
      cudaError_t e = s->upload();
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  // enqueue every batched launch of the recorded steps on stream s
  cudaError_t launch(cudaStream_t s) {
    for (auto& site : sites) {
      cudaError_t e = site->launch(s);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
};

}  // namespace spd_batch
