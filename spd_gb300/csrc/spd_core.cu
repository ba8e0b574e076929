// Host side of the C ABI declared in include/spd_gb300.h: context
// allocation, layout conversion at the boundary and the launch sequence of
// one SD-ADER step (src/sdader_simulator.py:361-378).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/spd_gb300.h"
#include "spd_fv.cuh"

using namespace spd;

namespace {

const char* kVersion = "spd_gb300 0.1 (sm_103a, FP64)";

struct StepperBase;

}  // namespace

struct spd_ctx {
  spd_config cfg{};
  Ops ops{};
  Geo geo{};
  FvGeo fvg{};
  int D = 0, P = 0, n = 0, nf = 0, T = 0, V = 0, NS = 0, NJ = 0;
  double h_dt = 0.0;  // h_min / (p+1)
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<void*> allocs;
  // state
  double *U_sp = nullptr, *U_cv = nullptr, *W_cv = nullptr, *U_new = nullptr;
  double* dt = nullptr;
  // predictor scratch
  double* U_ader = nullptr;
  double* trace[3] = {nullptr, nullptr, nullptr};
  double* Fi[3] = {nullptr, nullptr, nullptr};
  double* Ffp[3] = {nullptr, nullptr, nullptr};
  double* bcfix[3] = {nullptr, nullptr, nullptr};
  // FV scratch
  double* F_HO[3] = {nullptr, nullptr, nullptr};
  double *ext_old = nullptr, *ext_new = nullptr, *theta_src = nullptr, *theta_a = nullptr, *theta_b = nullptr;
  double* theta_final = nullptr;
  double* bcbuf[3] = {nullptr, nullptr, nullptr};
  unsigned char *mask = nullptr, *mark_cell = nullptr, *mark_q = nullptr;
  int* flags = nullptr;  // [0] any possible trouble, [1] nan in cmax, [2] marked faces
  unsigned long long* counts = nullptr;  // [0] cells, [1] subcells, [2] cmax bits
  long long *list_cell = nullptr, *list_q = nullptr;
  double* troubles = nullptr;
  double* aff[3] = {nullptr, nullptr, nullptr};
  double* F_FB[3] = {nullptr, nullptr, nullptr};
  double *Mpred = nullptr, *S = nullptr;
  double *K_sp_to_cv = nullptr, *K_cv_to_sp = nullptr;
  double* geo_arrays = nullptr;
  double* staging = nullptr;
  size_t staging_len = 0;
  StepperBase* stepper = nullptr;
  bool fb_ran = false;
  // stream and launch accounting
  cudaStream_t own_stream = nullptr;
  long long launches = 0;
  bool prof = false;
  struct Rec {
    const char* name;
    cudaEvent_t a, b;
  };
  std::vector<Rec> rec;
  std::vector<cudaEvent_t> pool;
};

namespace {

int fail(spd_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                                    \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return fail(C, SPD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));             \
  } while (0)

#define CKL()                                                                                       \
  do {                                                                                              \
    cudaError_t e_ = cudaGetLastError();                                                            \
    if (e_ != cudaSuccess) return fail(C, SPD_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e_)); \
  } while (0)

inline unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

cudaEvent_t get_event(spd_ctx* C) {
  if (!C->pool.empty()) {
    cudaEvent_t e = C->pool.back();
    C->pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Counts every kernel launch of the context and, while profiling is on,
// brackets it with CUDA events on the context's stream.
struct ProfScope {
  spd_ctx* C;
  const char* name;
  cudaEvent_t a = nullptr;
  ProfScope(spd_ctx* c, const char* n) : C(c), name(n) {
    ++C->launches;
    if (C->prof) {
      a = get_event(C);
      cudaEventRecord(a, C->stream);
    }
  }
  ~ProfScope() {
    if (C->prof) {
      cudaEvent_t b = get_event(C);
      cudaEventRecord(b, C->stream);
      C->rec.push_back({name, a, b});
    }
  }
};

template <class T>
int dalloc(spd_ctx* C, T** p, size_t count) {
  void* ptr = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(&ptr, count * sizeof(T));
  if (e != cudaSuccess) return fail(C, SPD_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  C->allocs.push_back(ptr);
  *p = static_cast<T*>(ptr);
  return 0;
}

// --------------------------------------------------------------------------
// layout conversion at the boundary
// --------------------------------------------------------------------------
// reference SD layout (V, [Nz,] [Ny,] Nx, [nz,] [ny,] nx) <-> device
// [v][s][c] (to_dev = 1) or FV [v][q] (fv = 1)
__global__ void k_sd_layout(Geo g, int D, int n, int V, const double* __restrict__ src, double* __restrict__ dst,
                            int to_dev, int fv) {
  const long long NS = (D == 1) ? n : (D == 2 ? n * n : n * n * n);
  const long long total = (long long)V * g.Nc * NS;
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= total) return;
  // decompose the reference index (C order, fastest = kx)
  long long t = r;
  int k[3] = {0, 0, 0}, c[3] = {0, 0, 0};
  for (int d = 0; d < D; ++d) { k[d] = (int)(t % n); t /= n; }
  for (int d = 0; d < D; ++d) { c[d] = (int)(t % g.N[d]); t /= g.N[d]; }
  const int v = (int)t;
  long long di;
  if (fv) {
    const long long q = (c[0] * n + k[0]) + (long long)g.X[0] * ((D >= 2 ? c[1] * n + k[1] : 0) +
                                                                (long long)g.X[1] * (D >= 3 ? c[2] * n + k[2] : 0));
    di = (long long)v * g.Nq + q;
  } else {
    const long long s = k[0] + n * (k[1] + (long long)n * k[2]);
    const long long cc = c[0] + (long long)g.N[0] * (c[1] + (long long)g.N[1] * c[2]);
    di = ((long long)v * NS + s) * g.Nc + cc;
  }
  if (to_dev) dst[di] = src[r];
  else dst[r] = src[di];
}

__global__ void k_zero_d(double* p, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.0;
}

// --------------------------------------------------------------------------
// per-(D,P) launch sequence
// --------------------------------------------------------------------------
struct StepperBase {
  virtual ~StepperBase() {}
  virtual int update(spd_ctx* C) = 0;    // perform_update with the current dt
  virtual int wcv(spd_ctx* C) = 0;       // W_cv = prim(U_cv)
  virtual int cmax(spd_ctx* C) = 0;      // dt from W_cv
  virtual int sp_to_cv(spd_ctx* C) = 0;  // U_cv = sp_to_cv(U_sp)
  virtual int configure(spd_ctx* C) = 0;
  int cpb = 32;
  size_t smem = 0;
};

template <int D, int P>
__global__ void k_cmax_only(Geo g, const double* __restrict__ W_cv, unsigned long long* __restrict__ cmax_bits,
                            int* __restrict__ nan_flag) {
  constexpr int P_ = D + 1;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double cval = 0.0;
  bool isnan_c = false;
  if (q < g.Nq) {
    double c = sound_speed(W_cv[(long long)P_ * g.Nq + q], W_cv[q], g.gamma, g.min_c2) * (double)D;
#pragma unroll
    for (int v = 1; v <= D; ++v) c = c + fabs(W_cv[(long long)v * g.Nq + q]);
    if (c != c) isnan_c = true;
    else cval = c;
  }
  for (int off = 16; off > 0; off >>= 1) {
    const double o = __shfl_down_sync(0xffffffffu, cval, off);
    cval = (o > cval) ? o : cval;
  }
  const unsigned nb = __ballot_sync(0xffffffffu, isnan_c);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(cmax_bits, (unsigned long long)__double_as_longlong(cval));
    if (nb) atomicOr(nan_flag, 1);
  }
}

template <int D>
__global__ void k_prim_only(Geo g, const double* __restrict__ U_cv, double* __restrict__ W_cv) {
  constexpr int V = D + 2;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= g.Nq) return;
  double u[V], W[V];
#pragma unroll
  for (int v = 0; v < V; ++v) u[v] = U_cv[(long long)v * g.Nq + q];
  prim<D>(u, W, g.gamma, 0);
#pragma unroll
  for (int v = 0; v < V; ++v) W_cv[(long long)v * g.Nq + q] = W[v];
}

constexpr int BS = 256;
constexpr int PERSIST_BLOCKS = 152 * 8;

template <int D, int P>
struct Stepper : StepperBase {
  using k = K<D, P>;

  int configure(spd_ctx* C) override {
    // cells per block of the interior kernel: bounded by 200 KB of shared memory
    const size_t per_cell = (size_t)k::V * k::NS * C->T * sizeof(double);
    cpb = 32;
    while (cpb > 1 && per_cell * cpb > 200 * 1024) cpb /= 2;
    smem = per_cell * cpb;
    CK(cudaFuncSetAttribute(k_interior<D, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return 0;
  }

  int predictor(spd_ctx* C, int final_mode) {
    const Geo& g = C->geo;
    {
      ProfScope ps_(C, "k_traces_sp");
      k_traces_sp<D, P><<<blocks_for(g.Nc, 128), 128, 0, C->stream>>>(C->ops, g, C->U_sp, C->trace[0], C->trace[1],
                                                                     C->trace[2]);
    }
    CKL();
    const int m = C->T - 1;
    for (int it = 0; it <= m; ++it) {
      const int Teff = (it == 0) ? 1 : C->T;
      const int solver = C->cfg.riemann_solver_sd;
      for (int d = 0; d < D; ++d) {
        const long long tot = (long long)Teff * k::NJ * n_iface(g, d);
        {
          ProfScope ps_(C, "k_riemann_sd");
          k_riemann_sd<D, P><<<blocks_for(tot, 128), 128, 0, C->stream>>>(g, d, Teff, solver, C->trace[d],
                                                                          C->bcfix[d], C->Fi[d]);
        }
        CKL();
      }
      const int mode = (it < m) ? 0 : final_mode;
      const double* Uin = (it == 0) ? C->U_sp : C->U_ader;
      const int Tu = (it == 0) ? 1 : C->T;
      dim3 block(cpb, Teff);
      const size_t sm = (mode == 2) ? 0 : (size_t)k::V * k::NS * Teff * cpb * sizeof(double);
      {
        ProfScope ps_(C, "k_interior");
        k_interior<D, P><<<blocks_for(g.Nc, cpb), block, sm, C->stream>>>(
            C->ops, g, mode, Teff, Uin, Tu, C->dt, C->U_sp, C->U_ader, C->Fi[0], C->Fi[1], C->Fi[2], C->trace[0],
            C->trace[1], C->trace[2], C->Ffp[0], C->Ffp[1], C->Ffp[2]);
      }
      CKL();
    }
    return 0;
  }

  int sp_to_cv(spd_ctx* C) override {
    const Geo& g = C->geo;
    {
      ProfScope ps_(C, "k_sp_to_cv");
      k_sp_to_cv<D, P><<<blocks_for(g.Nc * k::V, 128), 128, 0, C->stream>>>(g, C->K_sp_to_cv, C->U_sp, C->U_cv);
    }
    CKL();
    return 0;
  }

  int wcv(spd_ctx* C) override {
    const Geo& g = C->geo;
    {
      ProfScope ps_(C, "k_prim_only");
      k_prim_only<D><<<blocks_for(g.Nq, BS), BS, 0, C->stream>>>(g, C->U_cv, C->W_cv);
    }
    CKL();
    return 0;
  }

  int cmax(spd_ctx* C) override {
    const Geo& g = C->geo;
    CK(cudaMemsetAsync(C->flags + 1, 0, sizeof(int), C->stream));
    CK(cudaMemsetAsync(C->counts + 2, 0, sizeof(unsigned long long), C->stream));
    {
      ProfScope ps_(C, "k_cmax_only");
      k_cmax_only<D, P><<<blocks_for(g.Nq, BS), BS, 0, C->stream>>>(g, C->W_cv, C->counts + 2, C->flags + 1);
    }
    CKL();
    {
      ProfScope ps_(C, "k_dt_final");
      k_dt_final<<<1, 1, 0, C->stream>>>(C->h_dt, C->cfg.cfl_coeff, C->counts + 2, C->flags + 1, C->dt);
    }
    CKL();
    return 0;
  }

  int fv_update(spd_ctx* C) {
    const Geo& g = C->geo;
    const spd_config& cf = C->cfg;
    // switch_to_finite_volume (src/sdader_simulator.py:288-298)
    if (int r = sp_to_cv(C)) return r;
    for (int d = 0; d < D; ++d) {
      {
        ProfScope ps_(C, "k_integrate_faces");
        k_integrate_faces<D, P><<<blocks_for(g.Nc * g.T * k::nf, 128), 128, 0, C->stream>>>(C->ops, g, d, C->Ffp[d],
                                                                                            C->F_HO[d]);
      }
      CKL();
    }
    long long nface[3] = {1, 1, 1};
    for (int d = 0; d < D; ++d) nface[d] = n_faces(g, d);
    for (int i = 0; i < C->T; ++i) {
      const double w_i = C->ops.w_tp[i];
      const double* FH[3] = {nullptr, nullptr, nullptr};
      for (int d = 0; d < D; ++d) FH[d] = C->F_HO[d] + (long long)i * k::V * nface[d];
      {
        ProfScope ps_(C, "k_fv_candidate");
        k_fv_candidate<D><<<blocks_for(g.Nq, BS), BS, 0, C->stream>>>(g, C->fvg, C->dt, w_i, FH[0], FH[1], FH[2],
                                                                       C->U_cv, C->U_new, C->ext_old, C->ext_new,
                                                                       cf.FB ? 1 : 0);
      }
      CKL();
      if (cf.FB) {
        // detect_troubles (src/trouble_detection.py:5-87)
        for (int d = 0; d < D; ++d) {
          if (int r = ghost(C, d, 1, k::V, C->ext_old, nullptr)) return r;
        }
        CK(cudaMemsetAsync(C->flags, 0, sizeof(int), C->stream));
        {
          ProfScope ps_(C, "k_nad");
          k_nad<D><<<blocks_for(g.Nq, BS), BS, 0, C->stream>>>(g, cf.tolerance, cf.NAD_delta, P > 0 ? 1 : 0, C->ext_old,
                                                               C->ext_new, C->mask, C->flags);
        }
        CKL();
        const int sed = (P > 1 && cf.SED) ? 1 : 0;
        if (sed) {
          for (int d = 0; d < D; ++d) {
            if (int r = ghost(C, d, 1, k::V, C->ext_new, C->flags)) return r;
          }
        }
        {
          ProfScope ps_(C, "k_troubles");
          k_troubles<D><<<blocks_for(g.Nq, BS), BS, 0, C->stream>>>(g, C->fvg, sed, cf.PAD, cf.min_rho, cf.max_rho,
                                                                    cf.min_P, C->mask, C->flags, C->ext_new,
                                                                    C->theta_src, C->troubles);
        }
        CKL();
        for (int d = 0; d < D; ++d) {
          if (int r = ghost(C, d, 0, 1, C->theta_src, nullptr)) return r;
        }
        double* th = C->theta_src;
        if (cf.blending) {
          {
            ProfScope ps_(C, "k_blend_neighbours");
            k_blend_neighbours<D><<<blocks_for(g.Nqe, BS), BS, 0, C->stream>>>(g, C->theta_src, C->theta_a);
          }
          CKL();
          double* in = C->theta_a;
          double* out = C->theta_b;
          for (int d = 0; d < D; ++d) {
            {
              ProfScope ps_(C, "k_blend_last");
              k_blend_last<D><<<blocks_for(g.Nqe, BS), BS, 0, C->stream>>>(g, d, in, out);
            }
            CKL();
            std::swap(in, out);
          }
          th = in;
        }
        C->theta_final = th;
        // affected faces, marks and the fallback fluxes (src/sdader_simulator.py:343-346)
        CK(cudaMemsetAsync(C->mark_cell, 0, (size_t)g.Nqe, C->stream));
        CK(cudaMemsetAsync(C->mark_q, 0, (size_t)g.Nq, C->stream));
        CK(cudaMemsetAsync(C->counts, 0, 2 * sizeof(unsigned long long), C->stream));
        for (int d = 0; d < D; ++d) {
          {
            ProfScope ps_(C, "k_affected");
            k_affected<D><<<blocks_for(nface[d], BS), BS, 0, C->stream>>>(g, d, cf.godunov, th, C->aff[d],
                                                                          C->mark_cell, C->mark_q, C->flags + 2);
          }
          CKL();
        }
        {
          ProfScope ps_(C, "k_compact");
          k_compact<<<blocks_for(g.Nqe, BS), BS, 0, C->stream>>>(g.Nqe, C->mark_cell, C->list_cell, C->counts);
        }
        CKL();
        {
          ProfScope ps_(C, "k_compact");
          k_compact<<<blocks_for(g.Nq, BS), BS, 0, C->stream>>>(g.Nq, C->mark_q, C->list_q, C->counts + 1);
        }
        CKL();
        k_muscl_cells_grid(C, w_i);
        CKL();
        for (int d = 0; d < D; ++d) {
          {
            ProfScope ps_(C, "k_muscl_faces");
            k_muscl_faces<D><<<blocks_for(nface[d], BS), BS, 0, C->stream>>>(g, d, cf.riemann_solver_fv, cf.godunov,
                                                                             C->aff[d], C->Mpred, C->S, C->F_FB[d]);
          }
          CKL();
        }
        k_fv_correct_grid(C, w_i, FH);
        CKL();
        C->fb_ran = true;
      }
      std::swap(C->U_cv, C->U_new);
    }
    // switch_to_high_order (src/sdader_simulator.py:300-307)
    {
      ProfScope ps_(C, "k_cv_to_sp");
      k_cv_to_sp<D, P><<<blocks_for(g.Nc * k::V, 128), 128, 0, C->stream>>>(g, C->K_cv_to_sp, C->U_cv, C->U_sp);
    }
    CKL();
    return 0;
  }

  void k_muscl_cells_grid(spd_ctx* C, double w_i) {
    const Geo& g = C->geo;
    const long long nb = std::min<long long>(PERSIST_BLOCKS, blocks_for(g.Nqe, 128));
    {
      ProfScope ps_(C, "k_muscl_cells");
      k_muscl_cells<D><<<(unsigned)nb, 128, 0, C->stream>>>(g, C->fvg, C->cfg.slope_limiter, C->dt, w_i, C->list_cell,
                                                            C->counts, C->ext_old, C->Mpred, C->S);
    }
  }

  void k_fv_correct_grid(spd_ctx* C, double w_i, const double* const* FH) {
    const Geo& g = C->geo;
    const long long nb = std::min<long long>(PERSIST_BLOCKS, blocks_for(g.Nq, 128));
    {
      ProfScope ps_(C, "k_fv_correct");
      k_fv_correct<D><<<(unsigned)nb, 128, 0, C->stream>>>(g, C->fvg, C->dt, w_i, C->cfg.godunov, C->list_q,
                                                           C->counts + 1, FH[0], FH[1], FH[2], C->F_FB[0], C->F_FB[1],
                                                           C->F_FB[2], C->aff[0], C->aff[1], C->aff[2], C->U_cv,
                                                           C->U_new);
    }
  }

  int ghost(spd_ctx* C, int d, int all, int nv, double* ext, const int* gate) {
    const Geo& g = C->geo;
    const int o0 = (d == 0) ? 1 : 0;
    const int o1 = (d == 2) ? 1 : 2;
    const long long tot = 2LL * nv * NGH * g.Xe[o0] * g.Xe[o1];
    {
      ProfScope ps_(C, "k_ghost");
      k_ghost<D><<<blocks_for(tot, BS), BS, 0, C->stream>>>(g, d, all, nv, k::V, ext, C->bcbuf[d], gate);
    }
    CKL();
    return 0;
  }

  int update(spd_ctx* C) override {
    const int final_mode = (C->cfg.update == SPD_UPDATE_SD) ? 1 : 2;
    if (int r = predictor(C, final_mode)) return r;
    if (C->cfg.update == SPD_UPDATE_FV) {
      if (int r = fv_update(C)) return r;
    }
    // W_cv = prim(U_cv) (src/sdader_simulator.py:376)
    return wcv(C);
  }
};

}  // namespace


namespace {

template <int D>
StepperBase* make_stepper_d(int P) {
  switch (P) {
    case 1: return new Stepper<D, 1>();
    case 2: return new Stepper<D, 2>();
    case 3: return new Stepper<D, 3>();
    case 4: return new Stepper<D, 4>();
    default: return nullptr;
  }
}

StepperBase* make_stepper(int D, int P) {
  switch (D) {
    case 1: return make_stepper_d<1>(P);
    case 2: return make_stepper_d<2>(P);
    case 3: return make_stepper_d<3>(P);
    default: return nullptr;
  }
}

long long ipow(long long b, int e) {
  long long r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}

int ensure_staging(spd_ctx* C, size_t count) {
  if (C->staging_len >= count) return 0;
  if (C->staging) {
    cudaFree(C->staging);
    C->allocs.erase(std::remove(C->allocs.begin(), C->allocs.end(), (void*)C->staging), C->allocs.end());
    C->staging = nullptr;
    C->staging_len = 0;
  }
  if (int r = dalloc(C, &C->staging, count)) return r;
  C->staging_len = count;
  return 0;
}

long long n_faces_host(const Geo& g, int d) {
  return (long long)(g.X[0] + (d == 0)) * (g.X[1] + (d == 1)) * (g.X[2] + (d == 2));
}

long long n_other_ext(const Geo& g, int d) {
  const int o0 = (d == 0) ? 1 : 0;
  const int o1 = (d == 2) ? 1 : 2;
  return (long long)g.Xe[o0] * g.Xe[o1];
}

}  // namespace

extern "C" {

const char* spd_version(void) { return kVersion; }

const char* spd_last_error(const spd_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int spd_create(const spd_config* cfg, const spd_operators* ops, spd_ctx** out) {
  if (!cfg || !ops || !out) return SPD_ERR_ARG;
  *out = nullptr;
  std::unique_ptr<spd_ctx> holder(new spd_ctx());
  spd_ctx* C = holder.get();
  C->cfg = *cfg;
  const int D = cfg->ndim, P = cfg->p, m = cfg->m;
  if (D < 1 || D > 3) return fail(C, SPD_ERR_ARG, "ndim must be 1, 2 or 3");
  if (P < 1 || P > 4) return fail(C, SPD_ERR_ARG, "p must be in 1..4");
  if (m < 0 || m + 1 > MAXT) return fail(C, SPD_ERR_ARG, "m must be in 0..5");
  for (int d = 0; d < D; ++d) {
    if (cfg->N[d] < 1) return fail(C, SPD_ERR_ARG, "N must be positive");
    for (int s = 0; s < 2; ++s)
      if (cfg->BC[d][s] < 0 || cfg->BC[d][s] > SPD_BC_PRESSURE) return fail(C, SPD_ERR_ARG, "bad boundary kind");
  }
  if (cfg->riemann_solver_sd < 0 || cfg->riemann_solver_sd > 2 || cfg->riemann_solver_fv < 0 ||
      cfg->riemann_solver_fv > 2)
    return fail(C, SPD_ERR_ARG, "bad Riemann solver");
  if (cfg->slope_limiter < 0 || cfg->slope_limiter > 1) return fail(C, SPD_ERR_ARG, "bad slope limiter");
  if (cfg->update != SPD_UPDATE_SD && cfg->update != SPD_UPDATE_FV) return fail(C, SPD_ERR_ARG, "bad update");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(C, SPD_ERR_CUDA, "no CUDA device available (spd_gb300 has no CPU path)");

  C->D = D;
  C->P = P;
  C->n = P + 1;
  C->nf = P + 2;
  C->T = m + 1;
  C->V = D + 2;
  C->NS = (int)ipow(C->n, D);
  C->NJ = C->NS / C->n;
  Geo& g = C->geo;
  g.T = C->T;
  g.Nc = 1;
  g.Nq = 1;
  g.Nqe = 1;
  double h_min = 1e10;
  for (int d = 0; d < 3; ++d) {
    if (d < D) {
      g.N[d] = cfg->N[d];
      g.X[d] = cfg->N[d] * C->n;
      g.Xe[d] = g.X[d] + 2 * NGH;
      g.h[d] = (cfg->lim[d][1] - cfg->lim[d][0]) / cfg->N[d];
      h_min = std::min(h_min, g.h[d]);
      g.bc[d][0] = cfg->BC[d][0];
      g.bc[d][1] = cfg->BC[d][1];
    } else {
      g.N[d] = 1;
      g.X[d] = 1;
      g.Xe[d] = 1;
      g.h[d] = 1.0;
      g.bc[d][0] = g.bc[d][1] = SPD_BC_PERIODIC;
    }
    g.Nc *= g.N[d];
    g.Nq *= g.X[d];
    g.Nqe *= g.Xe[d];
  }
  g.gamma = cfg->gamma;
  g.min_c2 = cfg->min_c2;
  C->h_dt = h_min / (double)(P + 1);

  const int n = C->n, nf = C->nf, T = C->T, V = C->V, NS = C->NS, NJ = C->NJ;
  std::memcpy(C->ops.sp_to_fp, ops->sp_to_fp, sizeof(double) * nf * n);
  std::memcpy(C->ops.dfp_to_sp, ops->dfp_to_sp, sizeof(double) * n * nf);
  std::memcpy(C->ops.sp_to_cv, ops->sp_to_cv, sizeof(double) * n * n);
  std::memcpy(C->ops.invader, ops->invader, sizeof(double) * T * T);
  std::memcpy(C->ops.w_tp, ops->w_tp, sizeof(double) * T);

  CK(cudaStreamCreateWithFlags(&C->own_stream, cudaStreamNonBlocking));
  C->stream = C->own_stream;

  // whole-cell operator products ((A*A)*A) for sp_to_cv and cv_to_sp
  {
    std::vector<double> K1((size_t)NS * NS), K2((size_t)NS * NS);
    const double* mats[2] = {ops->sp_to_cv, ops->cv_to_sp};
    std::vector<double>* outs[2] = {&K1, &K2};
    for (int w = 0; w < 2; ++w) {
      const double* A = mats[w];
      for (int o = 0; o < NS; ++o) {
        const int oi = o % n, oj = (o / n) % n, ok = o / (n * n);
        for (int in = 0; in < NS; ++in) {
          const int l = in % n, mm = (in / n) % n, a = in / (n * n);
          double val;
          if (D == 1) val = A[oi * n + l];
          else if (D == 2) val = A[oj * n + mm] * A[oi * n + l];
          else val = (A[ok * n + a] * A[oj * n + mm]) * A[oi * n + l];
          (*outs[w])[(size_t)o * NS + in] = val;
        }
      }
    }
    if (int r = dalloc(C, &C->K_sp_to_cv, K1.size())) return r;
    if (int r = dalloc(C, &C->K_cv_to_sp, K2.size())) return r;
    CK(cudaMemcpy(C->K_sp_to_cv, K1.data(), K1.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(C->K_cv_to_sp, K2.data(), K2.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  // subcell geometry (src/sdader_simulator.py:61-92, src/fv_simulator.py:195)
  {
    std::vector<double> buf;
    size_t off[3][4];
    for (int d = 0; d < D; ++d) {
      const int Xd = g.X[d], Xe = g.Xe[d];
      const double* fp = ops->faces[d];
      off[d][0] = buf.size();
      for (int k2 = 0; k2 < Xd; ++k2) buf.push_back(fp[NGH + 1 + k2] - fp[NGH + k2]);
      off[d][1] = buf.size();
      std::vector<double> cen(Xe);
      for (int e = 0; e < Xe; ++e) cen[e] = 0.5 * (fp[e + 1] + fp[e]);
      buf.insert(buf.end(), cen.begin(), cen.end());
      off[d][2] = buf.size();
      for (int e = 0; e < Xe; ++e) buf.push_back(fp[e + 1] - fp[e]);
      off[d][3] = buf.size();
      for (int e = 0; e + 1 < Xe; ++e) buf.push_back(cen[e + 1] - cen[e]);
    }
    if (int r = dalloc(C, &C->geo_arrays, buf.size())) return r;
    CK(cudaMemcpy(C->geo_arrays, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice));
    for (int d = 0; d < D; ++d) {
      C->fvg.dx[d] = C->geo_arrays + off[d][0];
      C->fvg.centers[d] = C->geo_arrays + off[d][1];
      C->fvg.hfp[d] = C->geo_arrays + off[d][2];
      C->fvg.hcv[d] = C->geo_arrays + off[d][3];
    }
  }
  // state and scratch
  const long long Nc = g.Nc, Nq = g.Nq, Nqe = g.Nqe;
  if (int r = dalloc(C, &C->U_sp, (size_t)V * NS * Nc)) return r;
  if (int r = dalloc(C, &C->U_ader, (size_t)V * T * NS * Nc)) return r;
  if (int r = dalloc(C, &C->U_cv, (size_t)V * Nq)) return r;
  if (int r = dalloc(C, &C->W_cv, (size_t)V * Nq)) return r;
  if (int r = dalloc(C, &C->dt, 1)) return r;
  if (int r = dalloc(C, &C->flags, 4)) return r;
  if (int r = dalloc(C, &C->counts, 4)) return r;
  for (int d = 0; d < D; ++d) {
    const long long nI = Nc / g.N[d] * (g.N[d] + 1);
    if (int r = dalloc(C, &C->trace[d], (size_t)2 * V * T * NJ * Nc)) return r;
    if (int r = dalloc(C, &C->Fi[d], (size_t)V * T * NJ * nI)) return r;
    if (int r = dalloc(C, &C->bcfix[d], (size_t)2 * V * NJ * (Nc / g.N[d]))) return r;
    CK(cudaMemset(C->bcfix[d], 0, sizeof(double) * 2 * V * NJ * (Nc / g.N[d])));
  }
  if (cfg->update == SPD_UPDATE_FV) {
    if (int r = dalloc(C, &C->U_new, (size_t)V * Nq)) return r;
    for (int d = 0; d < D; ++d) {
      const long long nfc = n_faces_host(g, d);
      if (int r = dalloc(C, &C->Ffp[d], (size_t)V * T * NJ * nf * Nc)) return r;
      if (int r = dalloc(C, &C->F_HO[d], (size_t)T * V * nfc)) return r;
      if (int r = dalloc(C, &C->bcbuf[d], (size_t)2 * V * NGH * n_other_ext(g, d))) return r;
      CK(cudaMemset(C->bcbuf[d], 0, sizeof(double) * 2 * V * NGH * n_other_ext(g, d)));
    }
    if (cfg->FB) {
      if (int r = dalloc(C, &C->ext_old, (size_t)V * Nqe)) return r;
      if (int r = dalloc(C, &C->ext_new, (size_t)V * Nqe)) return r;
      if (int r = dalloc(C, &C->theta_src, (size_t)Nqe)) return r;
      if (int r = dalloc(C, &C->theta_a, (size_t)Nqe)) return r;
      if (int r = dalloc(C, &C->theta_b, (size_t)Nqe)) return r;
      if (int r = dalloc(C, &C->mask, (size_t)Nq)) return r;
      if (int r = dalloc(C, &C->mark_cell, (size_t)Nqe)) return r;
      if (int r = dalloc(C, &C->mark_q, (size_t)Nq)) return r;
      if (int r = dalloc(C, &C->list_cell, (size_t)Nqe)) return r;
      if (int r = dalloc(C, &C->list_q, (size_t)Nq)) return r;
      if (int r = dalloc(C, &C->troubles, (size_t)Nq)) return r;
      if (int r = dalloc(C, &C->Mpred, (size_t)V * Nqe)) return r;
      if (int r = dalloc(C, &C->S, (size_t)D * V * Nqe)) return r;
      CK(cudaMemset(C->ext_old, 0, sizeof(double) * V * Nqe));
      CK(cudaMemset(C->ext_new, 0, sizeof(double) * V * Nqe));
      CK(cudaMemset(C->theta_src, 0, sizeof(double) * Nqe));
      CK(cudaMemset(C->troubles, 0, sizeof(double) * Nq));
      C->theta_final = C->theta_src;
      for (int d = 0; d < D; ++d) {
        const long long nfc = n_faces_host(g, d);
        if (int r = dalloc(C, &C->aff[d], (size_t)nfc)) return r;
        if (int r = dalloc(C, &C->F_FB[d], (size_t)V * nfc)) return r;
        CK(cudaMemset(C->aff[d], 0, sizeof(double) * nfc));
      }
    }
  }
  C->stepper = make_stepper(D, P);
  if (!C->stepper) return fail(C, SPD_ERR_ARG, "unsupported (ndim, p)");
  if (int r = C->stepper->configure(C)) return r;
  *out = holder.release();
  return SPD_OK;
}

int spd_destroy(spd_ctx* C) {
  if (!C) return SPD_ERR_ARG;
  if (C->stream) cudaStreamSynchronize(C->stream);
  for (void* p : C->allocs) cudaFree(p);
  for (auto& r : C->rec) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (cudaEvent_t e : C->pool) cudaEventDestroy(e);
  if (C->own_stream) cudaStreamDestroy(C->own_stream);
  delete C->stepper;
  delete C;
  return SPD_OK;
}

int spd_set_stream(spd_ctx* C, void* stream) {
  if (!C) return SPD_ERR_ARG;
  CK(cudaStreamSynchronize(C->stream));
  C->stream = stream ? static_cast<cudaStream_t>(stream) : C->own_stream;
  return SPD_OK;
}

int spd_profile(spd_ctx* C, int enable) {
  if (!C) return SPD_ERR_ARG;
  C->prof = enable != 0;
  return SPD_OK;
}

int spd_profile_report(spd_ctx* C, char* buf, size_t len) {
  if (!C || !buf || len == 0) return SPD_ERR_ARG;
  CK(cudaStreamSynchronize(C->stream));
  std::vector<std::string> names;
  std::vector<double> ms;
  std::vector<long long> cnt;
  for (auto& r : C->rec) {
    float t = 0.f;
    cudaEventElapsedTime(&t, r.a, r.b);
    size_t k = 0;
    while (k < names.size() && names[k] != r.name) ++k;
    if (k == names.size()) {
      names.push_back(r.name);
      ms.push_back(0.0);
      cnt.push_back(0);
    }
    ms[k] += t;
    cnt[k] += 1;
    C->pool.push_back(r.a);
    C->pool.push_back(r.b);
  }
  C->rec.clear();
  std::string out;
  char line[256];
  for (size_t k = 0; k < names.size(); ++k) {
    std::snprintf(line, sizeof(line), "%s %lld %.6f\n", names[k].c_str(), cnt[k], ms[k]);
    out += line;
  }
  std::snprintf(buf, len, "%s", out.c_str());
  return out.size() + 1 > len ? fail(C, SPD_ERR_ARG, "profile report truncated") : SPD_OK;
}

int spd_launch_count(const spd_ctx* C, long long* count) {
  if (!C || !count) return SPD_ERR_ARG;
  *count = C->launches;
  return SPD_OK;
}

int spd_synchronize(spd_ctx* C) {
  if (!C) return SPD_ERR_ARG;
  CK(cudaStreamSynchronize(C->stream));
  return SPD_OK;
}

static size_t field_count(spd_ctx* C, int field) {
  const Geo& g = C->geo;
  const int V = C->V, D = C->D;
  switch (field) {
    case SPD_U_SP:
    case SPD_U_CV:
    case SPD_W_CV: return (size_t)V * C->NS * g.Nc;
    case SPD_TROUBLES: return (size_t)g.Nq;
    case SPD_THETA: return (size_t)g.Nqe;
    case SPD_AFFECTED_X:
    case SPD_AFFECTED_Y:
    case SPD_AFFECTED_Z: {
      const int d = field - SPD_AFFECTED_X;
      return d < D ? (size_t)n_faces_host(g, d) : 0;
    }
    case SPD_BC_FP_X:
    case SPD_BC_FP_Y:
    case SPD_BC_FP_Z: {
      const int d = field - SPD_BC_FP_X;
      return d < D ? (size_t)2 * V * C->T * C->NJ * (g.Nc / g.N[d]) : 0;
    }
    case SPD_BC_FV_X:
    case SPD_BC_FV_Y:
    case SPD_BC_FV_Z: {
      const int d = field - SPD_BC_FV_X;
      return d < D ? (size_t)2 * V * NGH * n_other_ext(g, d) : 0;
    }
    default: return 0;
  }
}

// reference BC_fv layout (2, V, Ze', Ye', Xe') with NGH along d <-> device
// [side][v][g][other]
static void bcfv_map(const spd_ctx* C, int d, std::vector<size_t>& ref_to_dev) {
  const Geo& g = C->geo;
  const int V = C->V;
  int ext[3] = {g.Xe[0], g.Xe[1], g.Xe[2]};
  ext[d] = NGH;
  const int o0 = (d == 0) ? 1 : 0;
  const int o1 = (d == 2) ? 1 : 2;
  const long long nother = n_other_ext(g, d);
  ref_to_dev.resize((size_t)2 * V * ext[0] * ext[1] * ext[2]);
  size_t r = 0;
  for (int side = 0; side < 2; ++side)
    for (int v = 0; v < V; ++v)
      for (int z = 0; z < ext[2]; ++z)
        for (int y = 0; y < ext[1]; ++y)
          for (int x = 0; x < ext[0]; ++x) {
            const int c[3] = {x, y, z};
            const long long other = c[o0] + (long long)g.Xe[o0] * c[o1];
            ref_to_dev[r++] = ((((size_t)side * V + v) * NGH + c[d]) * nother) + other;
          }
}

int spd_upload(spd_ctx* C, int field, const double* host, size_t count) {
  if (!C || !host) return SPD_ERR_ARG;
  const size_t need = field_count(C, field);
  if (need == 0 || count != need) return fail(C, SPD_ERR_ARG, "upload: wrong field or element count");
  const Geo& g = C->geo;
  if (field == SPD_U_SP || field == SPD_U_CV || field == SPD_W_CV) {
    if (int r = ensure_staging(C, need)) return r;
    CK(cudaMemcpyAsync(C->staging, host, need * sizeof(double), cudaMemcpyHostToDevice, C->stream));
    double* dst = (field == SPD_U_SP) ? C->U_sp : (field == SPD_U_CV ? C->U_cv : C->W_cv);
    k_sd_layout<<<blocks_for((long long)need, BS), BS, 0, C->stream>>>(g, C->D, C->n, C->V, C->staging, dst, 1,
                                                                       field == SPD_U_SP ? 0 : 1);
    CKL();
    CK(cudaStreamSynchronize(C->stream));
    return SPD_OK;
  }
  if (field >= SPD_BC_FP_X && field <= SPD_BC_FP_Z) {
    const int d = field - SPD_BC_FP_X;
    const long long ntrans = g.Nc / g.N[d];
    std::vector<double> tmp((size_t)2 * C->V * C->NJ * ntrans);
    for (int side = 0; side < 2; ++side)
      for (int v = 0; v < C->V; ++v)
        for (long long ct = 0; ct < ntrans; ++ct)
          for (int j = 0; j < C->NJ; ++j) {
            const size_t ri = ((((size_t)side * C->V + v) * C->T + 0) * ntrans + ct) * C->NJ + j;
            tmp[(((size_t)side * C->V + v) * C->NJ + j) * ntrans + ct] = host[ri];
          }
    CK(cudaMemcpy(C->bcfix[d], tmp.data(), tmp.size() * sizeof(double), cudaMemcpyHostToDevice));
    return SPD_OK;
  }
  if (field >= SPD_BC_FV_X && field <= SPD_BC_FV_Z) {
    const int d = field - SPD_BC_FV_X;
    if (!C->bcbuf[d]) return SPD_OK;  // only used by the FV update
    std::vector<size_t> map;
    bcfv_map(C, d, map);
    std::vector<double> tmp(map.size());
    for (size_t r = 0; r < map.size(); ++r) tmp[map[r]] = host[r];
    CK(cudaMemcpy(C->bcbuf[d], tmp.data(), tmp.size() * sizeof(double), cudaMemcpyHostToDevice));
    return SPD_OK;
  }
  return fail(C, SPD_ERR_ARG, "upload: field is read-only");
}

int spd_download(spd_ctx* C, int field, double* host, size_t count) {
  if (!C || !host) return SPD_ERR_ARG;
  const size_t need = field_count(C, field);
  if (need == 0 || count != need) return fail(C, SPD_ERR_ARG, "download: wrong field or element count");
  const Geo& g = C->geo;
  if (field == SPD_U_SP || field == SPD_U_CV || field == SPD_W_CV) {
    if (int r = ensure_staging(C, need)) return r;
    const double* src = (field == SPD_U_SP) ? C->U_sp : (field == SPD_U_CV ? C->U_cv : C->W_cv);
    k_sd_layout<<<blocks_for((long long)need, BS), BS, 0, C->stream>>>(g, C->D, C->n, C->V, src, C->staging, 0,
                                                                       field == SPD_U_SP ? 0 : 1);
    CKL();
    CK(cudaMemcpyAsync(host, C->staging, need * sizeof(double), cudaMemcpyDeviceToHost, C->stream));
    CK(cudaStreamSynchronize(C->stream));
    return SPD_OK;
  }
  const double* src = nullptr;
  if (field == SPD_TROUBLES) src = C->troubles;
  else if (field == SPD_THETA) src = C->theta_final;
  else if (field >= SPD_AFFECTED_X && field <= SPD_AFFECTED_Z) src = C->aff[field - SPD_AFFECTED_X];
  if (field >= SPD_BC_FV_X && field <= SPD_BC_FV_Z) {
    const int d = field - SPD_BC_FV_X;
    if (!C->bcbuf[d]) return fail(C, SPD_ERR_ARG, "download: no FV boundary buffers (update is SD)");
    std::vector<double> tmp(need);
    CK(cudaStreamSynchronize(C->stream));
    CK(cudaMemcpy(tmp.data(), C->bcbuf[d], need * sizeof(double), cudaMemcpyDeviceToHost));
    std::vector<size_t> map;
    bcfv_map(C, d, map);
    for (size_t r = 0; r < map.size(); ++r) host[r] = tmp[map[r]];
    return SPD_OK;
  }
  if (!src) return fail(C, SPD_ERR_ARG, "download: field not available for this configuration");
  CK(cudaMemcpyAsync(host, src, need * sizeof(double), cudaMemcpyDeviceToHost, C->stream));
  CK(cudaStreamSynchronize(C->stream));
  return SPD_OK;
}

int spd_compute_dt(spd_ctx* C, double* dt_out) {
  if (!C) return SPD_ERR_ARG;
  if (int r = C->stepper->cmax(C)) return r;
  double dt = 0.0;
  CK(cudaMemcpyAsync(&dt, C->dt, sizeof(double), cudaMemcpyDeviceToHost, C->stream));
  CK(cudaStreamSynchronize(C->stream));
  if (dt_out) *dt_out = dt;
  return SPD_OK;
}

int spd_set_dt(spd_ctx* C, double dt) {
  if (!C) return SPD_ERR_ARG;
  CK(cudaMemcpyAsync(C->dt, &dt, sizeof(double), cudaMemcpyHostToDevice, C->stream));
  CK(cudaStreamSynchronize(C->stream));
  return SPD_OK;
}

int spd_get_dt(spd_ctx* C, double* dt_out) {
  if (!C || !dt_out) return SPD_ERR_ARG;
  CK(cudaMemcpyAsync(dt_out, C->dt, sizeof(double), cudaMemcpyDeviceToHost, C->stream));
  CK(cudaStreamSynchronize(C->stream));
  return SPD_OK;
}

int spd_perform_update(spd_ctx* C, double* time_inout) {
  if (!C) return SPD_ERR_ARG;
  if (int r = C->stepper->update(C)) return r;
  double dt = 0.0;
  CK(cudaMemcpyAsync(&dt, C->dt, sizeof(double), cudaMemcpyDeviceToHost, C->stream));
  CK(cudaStreamSynchronize(C->stream));
  if (time_inout) *time_inout += dt;
  return SPD_OK;
}

int spd_step(spd_ctx* C, int nsteps, double t_end, int mode, double* time_inout, int* nsteps_done) {
  if (!C || !time_inout) return SPD_ERR_ARG;
  int done = 0;
  if (mode == 0) {
    for (int i = 0; i < nsteps; ++i) {
      if (int r = C->stepper->cmax(C)) return r;
      if (int r = spd_perform_update(C, time_inout)) return r;
      ++done;
    }
  } else {
    while (*time_inout < t_end) {
      double dt = 0.0;
      if (int r = spd_compute_dt(C, &dt)) return r;
      if (*time_inout + dt >= t_end) {
        dt = t_end - *time_inout;
        if (int r = spd_set_dt(C, dt)) return r;
      }
      if (dt < 1e-14) break;
      if (int r = spd_perform_update(C, time_inout)) return r;
      ++done;
      if (nsteps > 0 && done >= nsteps) break;
    }
  }
  if (nsteps_done) *nsteps_done = done;
  return SPD_OK;
}

int spd_end_sim(spd_ctx* C) {
  if (!C) return SPD_ERR_ARG;
  if (int r = C->stepper->sp_to_cv(C)) return r;
  if (int r = C->stepper->wcv(C)) return r;
  CK(cudaStreamSynchronize(C->stream));
  return SPD_OK;
}

}  // extern "C"
