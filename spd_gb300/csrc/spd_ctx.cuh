// Host-side context of the C ABI (include/spd_gb300.h) shared by the
// translation units of the library: the spd_ctx struct, launch accounting
// and the per-(D,P) stepper interface.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/spd_gb300.h"
#include "spd_batch.cuh"
#include "spd_fv.cuh"
#include "spd_visc.cuh"

namespace spd_host {
struct StepperBase;
}

struct spd_ctx {
  spd_config cfg{};
  spd::Ops ops{};
  spd::Geo geo{};
  spd::FvGeo fvg{};
  int D = 0, P = 0, n = 0, nf = 0, T = 0, V = 0, NS = 0, NJ = 0;
  double h_dt = 0.0;  // h_min / (p+1)
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<void*> allocs;
  // state
  double *U_sp = nullptr, *U_cv = nullptr, *W_cv = nullptr, *U_new = nullptr;
  double* dt = nullptr;
  double* t_dev = nullptr;  // simulated time kept on the device (ensemble driver, step graph)
  // one captured step (dt graph: CFL dt and the t_end clip; update graph:
  // update and time += dt) replayed by spd_step; the host-side buffer roles
  // it leaves behind are restored after each replay
  cudaGraph_t step_graph = nullptr, dt_graph = nullptr;
  cudaGraphExec_t step_exec = nullptr, dt_exec = nullptr;
  double* t_dev_pair = nullptr;  // [time, t_end] of the step graphs
  bool step_graph_failed = false;
  double *graph_U_cv = nullptr, *graph_U_new = nullptr, *graph_theta = nullptr;
  long long graph_kernels = 0;
  // adjoint: record slots of forward intermediates and the adjoint work
  // arrays (allocated by spd_adjoint_enable, freed on re-enable and destroy)
  bool recording = false;
  // decision tapes: per step, the affected faces and the branch outcomes of
  // every Riemann problem and limited slope (spd_tape_enable / spd_tape_step)
  int tape_mode = 0;  // 0 off, 1 record, 2 replay
  int tape_step = 0, tape_steps = 0;
  std::vector<void*> tape_allocs;
  unsigned* tape_rs[3] = {nullptr, nullptr, nullptr};
  unsigned* tape_fb[3] = {nullptr, nullptr, nullptr};
  unsigned char* tape_lim = nullptr;
  double* tape_aff = nullptr;
  int adj_depth = 0;
  std::vector<void*> adj_allocs;
  size_t rec_usp_n = 0, rec_ader_n = 0, rec_ucv_n = 0, rec_aff_n = 0, rec_mpred_n = 0;
  double *rec_usp = nullptr, *rec_ader = nullptr, *rec_ucv = nullptr, *rec_aff = nullptr, *rec_dt = nullptr;
  double* rec_mpred = nullptr;
  double* hist_usp = nullptr;   // U_sp at the start of the recorded step
  double* hist_ader = nullptr;  // U_ader after each Picard iteration but the last (m slots)
  double* hist_ucv = nullptr;   // U_cv at the start of each FV substep (T slots)
  double* hist_aff = nullptr;   // affected faces of each substep (T slots, all directions)
  double* hist_dt = nullptr;    // dt of the recorded step
  double* hist_mpred = nullptr; // MUSCL-Hancock predictions and slope terms of each substep (T slots)
  double* Usp_a = nullptr;
  double* Ua = nullptr;
  double* dudt_a = nullptr;
  double* Ea[3] = {nullptr, nullptr, nullptr};
  double* Tra[3] = {nullptr, nullptr, nullptr};
  double* Upart[3] = {nullptr, nullptr, nullptr};  // per-direction interior shares of Ua
  double* Ffa[3] = {nullptr, nullptr, nullptr};
  double* FHa[3] = {nullptr, nullptr, nullptr};
  double* Fba[3] = {nullptr, nullptr, nullptr};
  double* FA[3] = {nullptr, nullptr, nullptr};  // reconstructed-state adjoints per fallback face
  double* LA = nullptr;                          // limiter adjoints per extended cell
  double *Ucv_a = nullptr, *Unew_a = nullptr, *W_a = nullptr, *W_ext = nullptr;
  double* bcbuf_a[3] = {nullptr, nullptr, nullptr};
  // predictor scratch
  double* U_ader = nullptr;
  double* trace[3] = {nullptr, nullptr, nullptr};
  double* Fi[3] = {nullptr, nullptr, nullptr};
  double* Ffp[3] = {nullptr, nullptr, nullptr};
  double* bcfix[3] = {nullptr, nullptr, nullptr};
  // viscosity scratch: primitives at the flux points (left interface
  // states), their gradients at the solution points, viscous fluxes
  double* Wfp[3] = {nullptr, nullptr, nullptr};
  double* dWsp = nullptr;
  double* Gv[3] = {nullptr, nullptr, nullptr};
  double dt_visc = -1.0;  // h^2 / nu / 4 of the viscous dt limit, or < 0
  // gravity potential gradients: [d][s][cell] at the solution points and
  // [d][subcell] as subcell averages (FV layout)
  double* gphi_sp = nullptr;
  double* gphi_fv = nullptr;
  // well-balanced mode: equilibrium U_eq_sp [v][s][cell]; U_eq_cv and its
  // primitives [v][subcell]; per direction the conservative state and flux
  // at the flux points [v][j][f][cell]; with the FV update the primitive
  // state and flux at the subcell faces [v][face] and the primitives on the
  // extended subcell grid [v][ext]
  double *Ueq_sp = nullptr, *Ueq_cv = nullptr, *Weq_cv = nullptr, *Meq_fv = nullptr;
  double* Meq_fp[3] = {nullptr, nullptr, nullptr};
  double* Feq_fp[3] = {nullptr, nullptr, nullptr};
  double* Meq_faces[3] = {nullptr, nullptr, nullptr};
  double* Feq_faces[3] = {nullptr, nullptr, nullptr};
  // FV scratch
  double* F_HO[3] = {nullptr, nullptr, nullptr};
  double *ext_old = nullptr, *ext_new = nullptr, *theta_src = nullptr, *theta_a = nullptr, *theta_b = nullptr;
  double* theta_final = nullptr;
  double* bcbuf[3] = {nullptr, nullptr, nullptr};
  unsigned char *mask = nullptr, *mark_cell = nullptr, *mark_q = nullptr;
  int* flags = nullptr;  // [0] any possible trouble, [1] nan in cmax, [2] marked faces
  // [0] marked extended cells, [1] marked subcells, [2] cmax bits, [3] subcells
  // with a NAD flag on density or pressure, [4 + d] affected faces of direction d
  unsigned long long* counts = nullptr;
  // compacted index lists: marked extended cells, marked subcells, subcells
  // needing the smoothness check, affected faces per direction
  long long *list_cell = nullptr, *list_q = nullptr, *list_sed = nullptr;
  long long* list_face[3] = {nullptr, nullptr, nullptr};
  double* troubles = nullptr;
  double* aff[3] = {nullptr, nullptr, nullptr};
  double* F_FB[3] = {nullptr, nullptr, nullptr};
  double *Mpred = nullptr, *S = nullptr;
  double *K_sp_to_cv = nullptr, *K_cv_to_sp = nullptr;
  double* geo_arrays = nullptr;
  double* staging = nullptr;
  size_t staging_len = 0;
  spd_host::StepperBase* stepper = nullptr;
  bool fb_ran = false;
  // while non-null, the step's launches and zero-fills are recorded into
  // this batch recorder instead of being issued (packed ensembles)
  spd_batch::BatchRec* brec = nullptr;
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

namespace spd_host {
using namespace spd;

inline int fail(spd_ctx* c, int code, const std::string& msg) {
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

// Launch of the step kernel ``kern`` whose body is ``Body`` on the context's
// stream, or, while a batch recorder is attached, the record of that launch
// (its grid, block shape and argument pack) for a batched launch.
template <class Body, class... P, class... A>
void launch(spd_ctx* C, const char* name, void (*kern)(P...), dim3 grid, dim3 block, size_t smem, A&&... a) {
  if (C->brec) {
    C->brec->add<Body>(name, grid, block, smem, spd_batch::PackBuild<P...>::make(std::forward<A>(a)...));
    return;
  }
  kern<<<grid, block, smem, C->stream>>>(std::forward<A>(a)...);
}

// zero-fill of device bytes on the context's stream (recorded while a batch
// recorder is attached)
inline cudaError_t zero_fill(spd_ctx* C, void* p, size_t bytes) {
  if (C->brec) {
    C->brec->add_zero(p, bytes);
    return cudaSuccess;
  }
  return cudaMemsetAsync(p, 0, bytes, C->stream);
}

inline cudaEvent_t get_event(spd_ctx* C) {
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
// per-(D,P) launch sequence
// --------------------------------------------------------------------------
struct StepperBase {
  virtual ~StepperBase() {}
  virtual int update(spd_ctx* C) = 0;    // perform_update with the current dt
  virtual int wcv(spd_ctx* C) = 0;       // W_cv = prim(U_cv)
  virtual int cmax(spd_ctx* C) = 0;      // dt from W_cv
  virtual int sp_to_cv(spd_ctx* C) = 0;  // U_cv = sp_to_cv(U_sp)
  virtual int configure(spd_ctx* C) = 0;
  virtual int vjp(spd_ctx* C) = 0;       // Usp_a <- (d U_sp_new / d U_sp)^T Usp_a of the recorded step
  virtual int eq_prims(spd_ctx* C) = 0;  // Weq_cv = prim(Ueq_cv) (well-balanced mode)
  int cpb = 32;       // cells per block of k_interior (a power of two <= max_cpb)
  int max_cpb = 32;   // largest cpb whose shared-memory tile fits
  size_t smem = 0;
};

constexpr int BS = 256;
constexpr int PERSIST_BLOCKS = 152 * 8;

StepperBase* make_stepper_d1(int P);
StepperBase* make_stepper_d2(int P);
StepperBase* make_stepper_d3(int P);

}  // namespace spd_host
