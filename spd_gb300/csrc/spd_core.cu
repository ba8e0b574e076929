// Host side of the C ABI declared in include/spd_gb300.h: context
// allocation, layout conversion at the boundary and the step drivers
// (src/sdader_simulator.py:361-413).
#include <memory>

#include "spd_ctx.cuh"

using namespace spd;
using namespace spd_host;

namespace {

const char* kVersion = "spd_gb300 0.1 (sm_103a, FP64)";

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

__global__ void k_time_add_dev(double* t, const double* dt) { *t = *t + *dt; }
// perform_time_evolution's clip (src/sdader_simulator.py:406-409) on the
// device: t[0] = time, t[1] = t_end
__global__ void k_clip_dt(const double* t, double* dt) {
  const double d = *dt;
  if (t[0] + d >= t[1]) *dt = t[1] - t[0];
}

StepperBase* make_stepper(int D, int P) {
  switch (D) {
    case 1: return make_stepper_d1(P);
    case 2: return make_stepper_d2(P);
    case 3: return make_stepper_d3(P);
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

// Device address of a host buffer the GPU can read and write directly
// (pinned or registered host memory, reached over NVLink-C2C on GB300), or
// null for any other pointer (pageable host memory, device memory).
const double* device_alias(const double* host) {
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (attr.type != cudaMemoryTypeHost || attr.devicePointer == nullptr) return nullptr;
  return static_cast<const double*>(attr.devicePointer);
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
  if (cfg->viscosity && cfg->update == SPD_UPDATE_FV && cfg->FB)
    return fail(C, SPD_ERR_ARG,
                "viscosity with the FV update and FB: the reference's viscous fallback fluxes raise "
                "AttributeError (src/muscl.py:253 calls compute_slopes, which calls a missing method)");
  if (cfg->viscosity && !(cfg->nu >= 0.0)) return fail(C, SPD_ERR_ARG, "nu must be >= 0");
  if (cfg->update == SPD_UPDATE_FV && cfg->FB && !cfg->WB) {
    // src/fv_simulator.py:251-253 fills "eq" ghost subcells with zeros (the
    // perturbation of the well-balanced mode, which is not implemented), so
    // the reference's fallback flux at those faces is 0*NaN and its first
    // step turns the boundary cells into NaN, its second step every cell
    for (int d = 0; d < D; ++d)
      for (int s = 0; s < 2; ++s)
        if (cfg->BC[d][s] == SPD_BC_EQ)
          return fail(C, SPD_ERR_ARG,
                      "boundary 'eq' with the FV update and FB: the reference's fallback fluxes there are NaN "
                      "(zero-density ghost subcells), which this build does not reproduce");
  }
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
      {
        int ex = 0;
        const double mant = std::frexp(g.h[d], &ex);
        g.h_pow2[d] = (mant == 0.5) ? 1 : 0;
        g.inv_h[d] = 1.0 / g.h[d];
      }
      h_min = std::min(h_min, g.h[d]);
      g.bc[d][0] = cfg->BC[d][0];
      g.bc[d][1] = cfg->BC[d][1];
    } else {
      g.N[d] = 1;
      g.X[d] = 1;
      g.Xe[d] = 1;
      g.h[d] = 1.0;
      g.inv_h[d] = 1.0;
      g.h_pow2[d] = 1;
      g.bc[d][0] = g.bc[d][1] = SPD_BC_PERIODIC;
    }
    g.Nc *= g.N[d];
    g.Nq *= g.X[d];
    g.Nqe *= g.Xe[d];
  }
  g.gamma = cfg->gamma;
  g.min_c2 = cfg->min_c2;
  g.iso = cfg->isothermal ? 1 : 0;
  C->h_dt = h_min / (double)(P + 1);
  // viscous dt limit h**2/nu*.25 (src/sd_simulator.py:223-224); h*h is the
  // correctly rounded square, as Python's h**2
  if (cfg->viscosity && cfg->nu > 0.0) C->dt_visc = C->h_dt * C->h_dt / cfg->nu * 0.25;

  const int n = C->n, nf = C->nf, T = C->T, V = C->V, NS = C->NS, NJ = C->NJ;
  std::memcpy(C->ops.sp_to_fp, ops->sp_to_fp, sizeof(double) * nf * n);
  std::memcpy(C->ops.dfp_to_sp, ops->dfp_to_sp, sizeof(double) * n * nf);
  std::memcpy(C->ops.sp_to_cv, ops->sp_to_cv, sizeof(double) * n * n);
  std::memcpy(C->ops.invader, ops->invader, sizeof(double) * T * T);
  std::memcpy(C->ops.w_tp, ops->w_tp, sizeof(double) * T);
  for (int d = 0; d < 3; ++d)
    for (int i = 0; i < n * nf; ++i) C->ops.dfp_h[d][i] = C->ops.dfp_to_sp[i] * g.inv_h[d];

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
    size_t off[3][8];
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
      off[d][4] = buf.size();
      for (int k2 = 0; k2 < Xd; ++k2) buf.push_back(1.0 / buf[off[d][0] + k2]);
      off[d][5] = buf.size();
      for (int e = 0; e + 1 < Xe; ++e) buf.push_back(1.0 / buf[off[d][3] + e]);
      off[d][6] = buf.size();
      for (int e = 0; e < Xe; ++e) buf.push_back((e >= 1 && e + 1 < Xe) ? cen[e + 1] - cen[e - 1] : 1.0);
      off[d][7] = buf.size();
      for (int e = 0; e < Xe; ++e) buf.push_back(1.0 / buf[off[d][6] + e]);
    }
    if (int r = dalloc(C, &C->geo_arrays, buf.size())) return r;
    CK(cudaMemcpy(C->geo_arrays, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice));
    for (int d = 0; d < D; ++d) {
      C->fvg.dx[d] = C->geo_arrays + off[d][0];
      C->fvg.centers[d] = C->geo_arrays + off[d][1];
      C->fvg.hfp[d] = C->geo_arrays + off[d][2];
      C->fvg.hcv[d] = C->geo_arrays + off[d][3];
      C->fvg.rdx[d] = C->geo_arrays + off[d][4];
      C->fvg.rhcv[d] = C->geo_arrays + off[d][5];
      C->fvg.c2[d] = C->geo_arrays + off[d][6];
      C->fvg.rc2[d] = C->geo_arrays + off[d][7];
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
  if (int r = dalloc(C, &C->counts, 8)) return r;
  for (int d = 0; d < D; ++d) {
    const long long nI = Nc / g.N[d] * (g.N[d] + 1);
    if (int r = dalloc(C, &C->trace[d], (size_t)2 * V * T * NJ * Nc)) return r;
    if (int r = dalloc(C, &C->Fi[d], (size_t)V * T * NJ * nI)) return r;
    if (int r = dalloc(C, &C->bcfix[d], (size_t)2 * V * NJ * (Nc / g.N[d]))) return r;
    CK(cudaMemset(C->bcfix[d], 0, sizeof(double) * 2 * V * NJ * (Nc / g.N[d])));
  }
  if (cfg->WB) {
    if (int r = dalloc(C, &C->Ueq_sp, (size_t)V * NS * Nc)) return r;
    if (int r = dalloc(C, &C->Ueq_cv, (size_t)V * Nq)) return r;
    if (int r = dalloc(C, &C->Weq_cv, (size_t)V * Nq)) return r;
    CK(cudaMemset(C->Ueq_sp, 0, sizeof(double) * V * NS * Nc));
    CK(cudaMemset(C->Ueq_cv, 0, sizeof(double) * V * Nq));
    CK(cudaMemset(C->Weq_cv, 0, sizeof(double) * V * Nq));
    for (int d = 0; d < D; ++d) {
      if (int r = dalloc(C, &C->Meq_fp[d], (size_t)V * NJ * nf * Nc)) return r;
      if (int r = dalloc(C, &C->Feq_fp[d], (size_t)V * NJ * nf * Nc)) return r;
      CK(cudaMemset(C->Meq_fp[d], 0, sizeof(double) * V * NJ * nf * Nc));
      CK(cudaMemset(C->Feq_fp[d], 0, sizeof(double) * V * NJ * nf * Nc));
      if (cfg->update == SPD_UPDATE_FV) {
        const long long nfc = n_faces_host(g, d);
        if (int r = dalloc(C, &C->Meq_faces[d], (size_t)V * nfc)) return r;
        if (int r = dalloc(C, &C->Feq_faces[d], (size_t)V * nfc)) return r;
        CK(cudaMemset(C->Meq_faces[d], 0, sizeof(double) * V * nfc));
        CK(cudaMemset(C->Feq_faces[d], 0, sizeof(double) * V * nfc));
      }
    }
    if (cfg->update == SPD_UPDATE_FV) {
      if (int r = dalloc(C, &C->Meq_fv, (size_t)V * Nqe)) return r;
      CK(cudaMemset(C->Meq_fv, 0, sizeof(double) * V * Nqe));
    }
  }
  if (cfg->potential) {
    if (int r = dalloc(C, &C->gphi_sp, (size_t)D * NS * Nc)) return r;
    if (int r = dalloc(C, &C->gphi_fv, (size_t)D * Nq)) return r;
    CK(cudaMemset(C->gphi_sp, 0, sizeof(double) * D * NS * Nc));
    CK(cudaMemset(C->gphi_fv, 0, sizeof(double) * D * Nq));
  }
  if (cfg->viscosity) {
    if (int r = dalloc(C, &C->dWsp, (size_t)D * V * T * NS * Nc)) return r;
    for (int d = 0; d < D; ++d) {
      if (int r = dalloc(C, &C->Wfp[d], (size_t)V * T * NJ * nf * Nc)) return r;
      if (int r = dalloc(C, &C->Gv[d], (size_t)V * T * NJ * nf * Nc)) return r;
    }
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
      // whole 32-bit words: k_sed clears mask bits with a word-wide atomic AND
      if (int r = dalloc(C, &C->mask, (size_t)(Nq + 3) / 4 * 4)) return r;
      if (int r = dalloc(C, &C->mark_cell, (size_t)Nqe)) return r;
      if (int r = dalloc(C, &C->mark_q, (size_t)Nq)) return r;
      if (int r = dalloc(C, &C->list_cell, (size_t)Nqe)) return r;
      if (int r = dalloc(C, &C->list_q, (size_t)Nq)) return r;
      if (int r = dalloc(C, &C->list_sed, (size_t)2 * Nq)) return r;
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
        if (int r = dalloc(C, &C->list_face[d], (size_t)nfc)) return r;
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
  if (C->step_exec) cudaGraphExecDestroy(C->step_exec);
  if (C->step_graph) cudaGraphDestroy(C->step_graph);
  if (C->dt_exec) cudaGraphExecDestroy(C->dt_exec);
  if (C->dt_graph) cudaGraphDestroy(C->dt_graph);
  for (void* p : C->allocs) cudaFree(p);
  for (void* p : C->adj_allocs) cudaFree(p);
  for (void* p : C->tape_allocs) cudaFree(p);
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
    case SPD_U_SP_ADJ: return C->Usp_a ? (size_t)V * C->NS * g.Nc : 0;
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
    case SPD_GRAD_PHI_SP:
    case SPD_GRAD_PHI_CV: return C->gphi_sp ? (size_t)D * C->NS * g.Nc : 0;
    case SPD_U_EQ_SP:
    case SPD_U_EQ_CV: return C->Ueq_sp ? (size_t)V * C->NS * g.Nc : 0;
    case SPD_M_EQ_FP_X:
    case SPD_M_EQ_FP_Y:
    case SPD_M_EQ_FP_Z:
    case SPD_F_EQ_FP_X:
    case SPD_F_EQ_FP_Y:
    case SPD_F_EQ_FP_Z: {
      const int d = (field - SPD_M_EQ_FP_X) % 3;
      return (d < D && C->Meq_fp[d]) ? (size_t)V * C->NJ * C->nf * g.Nc : 0;
    }
    case SPD_M_EQ_FACES_X:
    case SPD_M_EQ_FACES_Y:
    case SPD_M_EQ_FACES_Z:
    case SPD_F_EQ_FACES_X:
    case SPD_F_EQ_FACES_Y:
    case SPD_F_EQ_FACES_Z: {
      const int d = (field - SPD_M_EQ_FACES_X) % 3;
      return (d < D && C->Meq_faces[d]) ? (size_t)V * n_faces_host(g, d) : 0;
    }
    case SPD_M_EQ_FV: return C->Meq_fv ? (size_t)V * g.Nqe : 0;
    case SPD_F_FACES_X:
    case SPD_F_FACES_Y:
    case SPD_F_FACES_Z: {
      const int d = field - SPD_F_FACES_X;
      return (d < D && C->F_HO[d]) ? (size_t)C->T * V * n_faces_host(g, d) : 0;
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
  if (field == SPD_U_SP || field == SPD_U_CV || field == SPD_W_CV || field == SPD_U_SP_ADJ) {
    double* dst = (field == SPD_U_SP) ? C->U_sp
                  : (field == SPD_U_CV ? C->U_cv : (field == SPD_W_CV ? C->W_cv : C->Usp_a));
    // pinned host buffers are read by the layout kernel itself (one pass
    // over the host link); any other pointer goes through a device copy
    const double* src = device_alias(host);
    if (!src) {
      if (int r = ensure_staging(C, need)) return r;
      CK(cudaMemcpyAsync(C->staging, host, need * sizeof(double), cudaMemcpyDefault, C->stream));
      src = C->staging;
    }
    k_sd_layout<<<blocks_for((long long)need, BS), BS, 0, C->stream>>>(g, C->D, C->n, C->V, src, dst, 1,
                                                                       (field == SPD_U_SP || field == SPD_U_SP_ADJ) ? 0 : 1);
    CKL();
    CK(cudaStreamSynchronize(C->stream));
    return SPD_OK;
  }
  if (field == SPD_U_EQ_SP || field == SPD_U_EQ_CV) {
    if (int r = ensure_staging(C, need)) return r;
    CK(cudaMemcpyAsync(C->staging, host, need * sizeof(double), cudaMemcpyDefault, C->stream));
    double* dst = (field == SPD_U_EQ_SP) ? C->Ueq_sp : C->Ueq_cv;
    k_sd_layout<<<blocks_for((long long)need, BS), BS, 0, C->stream>>>(g, C->D, C->n, C->V, C->staging, dst, 1,
                                                                       field == SPD_U_EQ_SP ? 0 : 1);
    CKL();
    // the equilibrium's primitives (src/trouble_detection.py:59-60,
    // src/sdader_simulator.py:351-356 compute them from U_eq_cv)
    if (field == SPD_U_EQ_CV)
      if (int r = C->stepper->eq_prims(C)) return r;
    CK(cudaStreamSynchronize(C->stream));
    return SPD_OK;
  }
  if (field >= SPD_M_EQ_FP_X && field <= SPD_F_EQ_FP_Z) {
    // reference (V, cells z..x, points z..x), p+2 points along d -> [v][j][f][cell]
    const int d = (field - SPD_M_EQ_FP_X) % 3;
    double* dst = (field <= SPD_M_EQ_FP_Z) ? C->Meq_fp[d] : C->Feq_fp[d];
    const int n = C->n, nf = C->nf, NJ = C->NJ, V = C->V, D = C->D;
    std::vector<double> tmp(need);
    int np[3] = {1, 1, 1};
    for (int e = 0; e < D; ++e) np[e] = (e == d) ? nf : n;
    size_t r = 0;
    for (int v = 0; v < V; ++v)
      for (int cz = 0; cz < g.N[2]; ++cz)
        for (int cy = 0; cy < g.N[1]; ++cy)
          for (int cx = 0; cx < g.N[0]; ++cx)
            for (int kz = 0; kz < np[2]; ++kz)
              for (int ky = 0; ky < np[1]; ++ky)
                for (int kx = 0; kx < np[0]; ++kx) {
                  const int k[3] = {kx, ky, kz};
                  int j = 0;
                  if (d == 0) j = ky + n * kz;
                  else if (d == 1) j = kx + n * kz;
                  else j = kx + n * ky;
                  const long long c = cx + (long long)g.N[0] * (cy + (long long)g.N[1] * cz);
                  tmp[(((size_t)v * NJ + j) * nf + k[d]) * g.Nc + c] = host[r++];
                }
    CK(cudaMemcpy(dst, tmp.data(), need * sizeof(double), cudaMemcpyHostToDevice));
    return SPD_OK;
  }
  if (field >= SPD_M_EQ_FACES_X && field <= SPD_M_EQ_FV) {
    // the FV face and extended layouts are the reference's C order
    double* dst = (field == SPD_M_EQ_FV) ? C->Meq_fv
                  : (field <= SPD_M_EQ_FACES_Z ? C->Meq_faces[field - SPD_M_EQ_FACES_X]
                                               : C->Feq_faces[field - SPD_F_EQ_FACES_X]);
    CK(cudaMemcpy(dst, host, need * sizeof(double), cudaMemcpyHostToDevice));
    return SPD_OK;
  }
  if (field == SPD_GRAD_PHI_SP || field == SPD_GRAD_PHI_CV) {
    // ndim components in the SD layout: to [d][s][cell] (solution points)
    // or the FV layout [d][subcell] (subcell averages)
    if (int r = ensure_staging(C, need)) return r;
    CK(cudaMemcpyAsync(C->staging, host, need * sizeof(double), cudaMemcpyDefault, C->stream));
    double* dst = (field == SPD_GRAD_PHI_SP) ? C->gphi_sp : C->gphi_fv;
    k_sd_layout<<<blocks_for((long long)need, BS), BS, 0, C->stream>>>(g, C->D, C->n, C->D, C->staging, dst, 1,
                                                                       field == SPD_GRAD_PHI_SP ? 0 : 1);
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
  if (field == SPD_U_SP || field == SPD_U_CV || field == SPD_W_CV || field == SPD_U_SP_ADJ) {
    const double* src = (field == SPD_U_SP) ? C->U_sp
                        : (field == SPD_U_CV ? C->U_cv : (field == SPD_W_CV ? C->W_cv : C->Usp_a));
    const int fv = (field == SPD_U_SP || field == SPD_U_SP_ADJ) ? 0 : 1;
    // pinned host buffers are written by the layout kernel itself
    if (double* dst = const_cast<double*>(device_alias(host))) {
      k_sd_layout<<<blocks_for((long long)need, BS), BS, 0, C->stream>>>(g, C->D, C->n, C->V, src, dst, 0, fv);
      CKL();
      CK(cudaStreamSynchronize(C->stream));
      return SPD_OK;
    }
    if (int r = ensure_staging(C, need)) return r;
    k_sd_layout<<<blocks_for((long long)need, BS), BS, 0, C->stream>>>(g, C->D, C->n, C->V, src, C->staging, 0, fv);
    CKL();
    CK(cudaMemcpyAsync(host, C->staging, need * sizeof(double), cudaMemcpyDefault, C->stream));
    CK(cudaStreamSynchronize(C->stream));
    return SPD_OK;
  }
  const double* src = nullptr;
  if (field == SPD_TROUBLES) src = C->troubles;
  else if (field == SPD_THETA) src = C->theta_final;
  else if (field >= SPD_AFFECTED_X && field <= SPD_AFFECTED_Z) src = C->aff[field - SPD_AFFECTED_X];
  else if (field >= SPD_F_FACES_X && field <= SPD_F_FACES_Z) src = C->F_HO[field - SPD_F_FACES_X];
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

// Capture one step into two graphs: the dt graph (CFL reduction, then the
// clip of perform_time_evolution: dt = t_end - t where t + dt >= t_end, with
// t and t_end in t_dev[0..1]) and the update graph (update, t_dev[0] += dt).
// Returns false (and leaves the context as it was) when capture is not
// possible; the caller then steps launch by launch.
static bool capture(spd_ctx* C, int part, cudaGraph_t* gout, cudaGraphExec_t* xout) {
  cudaStream_t s = C->stream;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
  int rc;
  if (part == 0) {
    rc = C->stepper->cmax(C);
    if (!rc) {
      k_clip_dt<<<1, 1, 0, s>>>(C->t_dev, C->dt);
      if (cudaGetLastError() != cudaSuccess) rc = SPD_ERR_CUDA;
    }
  } else {
    rc = C->stepper->update(C);
    if (!rc) {
      k_time_add_dev<<<1, 1, 0, s>>>(C->t_dev, C->dt);
      if (cudaGetLastError() != cudaSuccess) rc = SPD_ERR_CUDA;
    }
  }
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(s, &g);
  if (rc || ec != cudaSuccess || cudaGraphInstantiate(xout, g, 0) != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    *xout = nullptr;
    cudaGetLastError();
    return false;
  }
  *gout = g;
  return true;
}

static bool build_step_graph(spd_ctx* C) {
  if (C->step_exec) return true;
  if (C->step_graph_failed) return false;
  if (!C->t_dev_pair) {
    void* p = nullptr;
    if (cudaMalloc(&p, 2 * sizeof(double)) != cudaSuccess) {
      C->step_graph_failed = true;
      return false;
    }
    C->allocs.push_back(p);
    C->t_dev_pair = static_cast<double*>(p);
  }
  double* keep_t = C->t_dev;
  C->t_dev = C->t_dev_pair;
  double* keep_cv = C->U_cv;
  double* keep_new = C->U_new;
  double* keep_theta = C->theta_final;
  const long long launches = C->launches;
  const bool ok = capture(C, 0, &C->dt_graph, &C->dt_exec) && capture(C, 1, &C->step_graph, &C->step_exec);
  C->graph_kernels = C->launches - launches + 2;  // the step's kernels, the clip and the time add
  C->launches = launches;                          // capture launched nothing
  C->graph_U_cv = C->U_cv;
  C->graph_U_new = C->U_new;
  C->graph_theta = C->theta_final;
  C->t_dev = keep_t;
  if (!ok) {
    if (C->dt_exec) cudaGraphExecDestroy(C->dt_exec);
    if (C->dt_graph) cudaGraphDestroy(C->dt_graph);
    C->dt_exec = nullptr;
    C->dt_graph = nullptr;
    C->step_exec = nullptr;
    C->U_cv = keep_cv;
    C->U_new = keep_new;
    C->theta_final = keep_theta;
    C->step_graph_failed = true;
    return false;
  }
  return true;
}

int spd_step(spd_ctx* C, int nsteps, double t_end, int mode, double* time_inout, int* nsteps_done) {
  if (!C || !time_inout) return SPD_ERR_ARG;
  int done = 0;
  bool nonfinite = false;
  const bool graphs = !C->prof && C->tape_mode == 0 && !C->recording && build_step_graph(C);
  if (graphs) {
    // the step as two graph launches; time and the clip in the same double
    // operations as the host loop below
    const double te = (mode == 0) ? HUGE_VAL : t_end;
    const double tt[2] = {*time_inout, te};
    CK(cudaMemcpyAsync(C->t_dev_pair, tt, sizeof(tt), cudaMemcpyHostToDevice, C->stream));
    if (mode == 0) {
      for (int i = 0; i < nsteps; ++i) {
        CK(cudaGraphLaunch(C->dt_exec, C->stream));
        CK(cudaGraphLaunch(C->step_exec, C->stream));
      }
      done = nsteps > 0 ? nsteps : 0;
    } else {
      double t = *time_inout;
      while (t < t_end) {
        CK(cudaGraphLaunch(C->dt_exec, C->stream));
        double dt = 0.0;
        CK(cudaMemcpyAsync(&dt, C->dt, sizeof(double), cudaMemcpyDeviceToHost, C->stream));
        CK(cudaStreamSynchronize(C->stream));
        if (dt < 1e-14) break;
        CK(cudaGraphLaunch(C->step_exec, C->stream));
        t = t + dt;
        nonfinite = nonfinite || !std::isfinite(dt);
        ++done;
        if (nsteps > 0 && done >= nsteps) break;
      }
    }
    C->launches += (long long)done * C->graph_kernels;
    CK(cudaMemcpyAsync(time_inout, C->t_dev_pair, sizeof(double), cudaMemcpyDeviceToHost, C->stream));
    CK(cudaStreamSynchronize(C->stream));
    if (done) {
      C->U_cv = C->graph_U_cv;
      C->U_new = C->graph_U_new;
      C->theta_final = C->graph_theta;
      if (C->cfg.update == SPD_UPDATE_FV && C->cfg.FB) C->fb_ran = true;
    }
    nonfinite = nonfinite || !std::isfinite(*time_inout);
  } else if (mode == 0) {
    for (int i = 0; i < nsteps; ++i) {
      if (int r = C->stepper->cmax(C)) return r;
      if (int r = spd_perform_update(C, time_inout)) return r;
      nonfinite = nonfinite || !std::isfinite(*time_inout);
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
      nonfinite = nonfinite || !std::isfinite(dt);
      ++done;
      if (nsteps > 0 && done >= nsteps) break;
    }
  }
  if (nsteps_done) *nsteps_done = done;
  // the steps ran as the reference runs them; the status reports the blow-up
  return nonfinite ? fail(C, SPD_ERR_NONFINITE, "step: dt is not finite (the state holds NaN or inf)") : SPD_OK;
}

int spd_end_sim(spd_ctx* C) {
  if (!C) return SPD_ERR_ARG;
  if (int r = C->stepper->sp_to_cv(C)) return r;
  if (int r = C->stepper->wcv(C)) return r;
  CK(cudaStreamSynchronize(C->stream));
  return SPD_OK;
}

}  // extern "C"
