// Batched ensembles: many independent SD-ADER problems of different sizes
// advanced together.  The per-instance step sequences (CFL dt reduction,
// predictor, FV update, device-side time accumulation) are recorded once
// into a CUDA graph whose branches run on several streams, so small
// instances fill the GPU concurrently and a whole ensemble step costs one
// graph launch instead of ~100 kernel launches and a host round trip per
// instance.  Each instance keeps its own dt (its own device reduction).
//
// The packed form (spd_ensemble_create_packed) instead merges the i-th
// launch of every instance into one batched launch indexed by a per-instance
// block-offset table (spd_batch.cuh): a whole ensemble step is then ~100
// launches however many instances there are.
#include <memory>

#include "spd_ctx.cuh"

using namespace spd;
using namespace spd_host;

struct spd_ensemble {
  std::vector<spd_ctx*> ctx;
  // buffer roles of each context at the end of the captured steps (the graph
  // replays leave the data there)
  std::vector<double*> roles;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> join;
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int steps_per_launch = 1;
  // packed form: the batched launch sites (argument packs and block-offset
  // tables in device memory) replayed by the graph
  std::unique_ptr<spd_batch::BatchRec> packed;
  std::string err;
};

namespace {

struct TimeAdd {
  static __device__ __forceinline__ void run(Blk, double* t, const double* dt) {
    if (threadIdx.x == 0) *t = *t + *dt;
  }
};
__global__ void k_time_add(double* t, const double* dt) { TimeAdd::run(hw_blk(), t, dt); }

// the calling thread's most recent ensemble error (also of a failed create,
// whose ensemble no longer exists)
thread_local std::string t_last_err;

int efail(spd_ensemble* E, int code, const std::string& msg) {
  if (E) E->err = msg;
  t_last_err = msg;
  return code;
}

#define ECK(call)                                                                                   \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return efail(E, SPD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Host-side buffer roles of the contexts.  Recording or capturing a step
// leaves them as after one step although no step has run yet; the guard
// puts back the roles of before on every exit of the create function, and
// spd_ensemble_step applies the roles of after once a step has run.
struct RolesGuard {
  std::vector<spd_ctx*> cs;
  std::vector<double*> pre;
  explicit RolesGuard(const std::vector<spd_ctx*>& c) : cs(c) {
    for (spd_ctx* C : cs) {
      pre.push_back(C->U_cv);
      pre.push_back(C->U_new);
      pre.push_back(C->theta_final);
    }
  }
  ~RolesGuard() {
    for (size_t i = 0; i < cs.size(); ++i) {
      cs[i]->U_cv = pre[3 * i];
      cs[i]->U_new = pre[3 * i + 1];
      cs[i]->theta_final = pre[3 * i + 2];
    }
  }
};

// one step of one instance on stream s, no host synchronisation
int enqueue_step(spd_ctx* C, cudaStream_t s) {
  cudaStream_t keep = C->stream;
  C->stream = s;
  int rc = C->stepper->cmax(C);
  if (!rc) rc = C->stepper->update(C);
  if (!rc) {
    ProfScope ps_(C, "k_time_add");
    k_time_add<<<1, 1, 0, s>>>(C->t_dev, C->dt);
    if (cudaGetLastError() != cudaSuccess) rc = SPD_ERR_CUDA;
  }
  C->stream = keep;
  return rc;
}

}  // namespace

extern "C" {

int spd_ensemble_create(spd_ctx** ctxs, int n, int nstreams, int steps_per_launch, spd_ensemble** out) {
  if (!ctxs || n <= 0 || nstreams <= 0 || steps_per_launch <= 0 || !out) return SPD_ERR_ARG;
  std::unique_ptr<spd_ensemble> holder(new spd_ensemble());
  spd_ensemble* E = holder.get();
  E->steps_per_launch = steps_per_launch;
  for (int i = 0; i < n; ++i) {
    if (!ctxs[i]) return efail(E, SPD_ERR_ARG, "null context");
    E->ctx.push_back(ctxs[i]);
    spd_ctx* C = ctxs[i];
    if (!C->t_dev) {
      void* p = nullptr;
      ECK(cudaMalloc(&p, sizeof(double)));
      C->allocs.push_back(p);
      C->t_dev = static_cast<double*>(p);
    }
    ECK(cudaStreamSynchronize(C->stream));
    ECK(cudaMemset(C->t_dev, 0, sizeof(double)));
  }
  ECK(cudaStreamCreateWithFlags(&E->main, cudaStreamNonBlocking));
  ECK(cudaEventCreateWithFlags(&E->fork, cudaEventDisableTiming));
  E->streams.resize(nstreams);
  E->join.resize(nstreams);
  for (int s = 0; s < nstreams; ++s) {
    ECK(cudaStreamCreateWithFlags(&E->streams[s], cudaStreamNonBlocking));
    ECK(cudaEventCreateWithFlags(&E->join[s], cudaEventDisableTiming));
  }
  // longest-processing-time assignment of instances to streams (work ~ subcells)
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return E->ctx[a]->geo.Nq > E->ctx[b]->geo.Nq; });
  std::vector<long long> load(nstreams, 0);
  std::vector<int> lane(n, 0);
  for (int i : order) {
    int best = 0;
    for (int s = 1; s < nstreams; ++s)
      if (load[s] < load[best]) best = s;
    lane[i] = best;
    load[best] += E->ctx[i]->geo.Nq;
  }
  const RolesGuard roles_before(E->ctx);
  ECK(cudaStreamBeginCapture(E->main, cudaStreamCaptureModeThreadLocal));
  cudaEventRecord(E->fork, E->main);
  for (int s = 0; s < nstreams; ++s) cudaStreamWaitEvent(E->streams[s], E->fork, 0);
  int rc = 0;
  for (int step = 0; step < steps_per_launch && !rc; ++step)
    for (int i : order)
      if (!rc) rc = enqueue_step(E->ctx[i], E->streams[lane[i]]);
  for (int s = 0; s < nstreams; ++s) {
    cudaEventRecord(E->join[s], E->streams[s]);
    cudaStreamWaitEvent(E->main, E->join[s], 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(E->main, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return efail(E, rc, "capture of an instance step failed");
  }
  if (ec != cudaSuccess) return efail(E, SPD_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ec));
  E->graph = g;
  ECK(cudaGraphInstantiate(&E->exec, E->graph, 0));
  for (spd_ctx* C : E->ctx) {
    E->roles.push_back(C->U_cv);
    E->roles.push_back(C->U_new);
    E->roles.push_back(C->theta_final);
  }
  *out = holder.release();
  return SPD_OK;
}

int spd_ensemble_create_packed(spd_ctx** ctxs, int n, int steps_per_launch, spd_ensemble** out) {
  if (!ctxs || n <= 0 || steps_per_launch <= 0 || !out) return SPD_ERR_ARG;
  std::unique_ptr<spd_ensemble> holder(new spd_ensemble());
  spd_ensemble* E = holder.get();
  E->steps_per_launch = steps_per_launch;
  for (int i = 0; i < n; ++i) {
    spd_ctx* C = ctxs[i];
    if (!C) return efail(E, SPD_ERR_ARG, "null context");
    if (C->recording || C->tape_mode != 0)
      return efail(E, SPD_ERR_ARG, "packed ensembles do not record adjoint intermediates or decision tapes");
    if (C->D != ctxs[0]->D || C->P != ctxs[0]->P || C->T != ctxs[0]->T)
      return efail(E, SPD_ERR_ARG, "packed ensembles need one dimension, degree and time order");
    E->ctx.push_back(C);
    if (!C->t_dev) {
      void* p = nullptr;
      ECK(cudaMalloc(&p, sizeof(double)));
      C->allocs.push_back(p);
      C->t_dev = static_cast<double*>(p);
    }
    ECK(cudaStreamSynchronize(C->stream));
    ECK(cudaMemset(C->t_dev, 0, sizeof(double)));
  }
  // record each instance's launch sequence (nothing is issued) and merge the
  // i-th launch of every instance into one batched launch
  E->packed.reset(new spd_batch::BatchRec());
  spd_batch::BatchRec* R = E->packed.get();
  const RolesGuard roles_before(E->ctx);
  for (int i = 0; i < n && R->err.empty(); ++i) {
    spd_ctx* C = E->ctx[i];
    const bool prof = C->prof;
    C->prof = false;
    C->brec = R;
    R->begin_instance(i == 0);
    int rc = 0;
    for (int step = 0; step < steps_per_launch && !rc && R->err.empty(); ++step) {
      rc = C->stepper->cmax(C);
      if (!rc) rc = C->stepper->update(C);
      if (!rc) launch<TimeAdd>(C, "k_time_add", k_time_add, 1, 1, 0, C->t_dev, C->dt);
    }
    C->brec = nullptr;
    C->prof = prof;
    if (rc) return efail(E, rc, std::string("recording instance ") + std::to_string(i) + ": " + C->err);
    R->end_instance();
  }
  if (!R->err.empty()) return efail(E, SPD_ERR_ARG, R->err);
  ECK(R->upload());
  ECK(cudaStreamCreateWithFlags(&E->main, cudaStreamNonBlocking));
  ECK(cudaStreamBeginCapture(E->main, cudaStreamCaptureModeThreadLocal));
  const cudaError_t el = R->launch(E->main);
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(E->main, &g);
  if (el != cudaSuccess || ec != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return efail(E, SPD_ERR_CUDA,
                 std::string("capture: ") + cudaGetErrorString(el != cudaSuccess ? el : ec));
  }
  E->graph = g;
  ECK(cudaGraphInstantiate(&E->exec, E->graph, 0));
  for (spd_ctx* C : E->ctx) {
    E->roles.push_back(C->U_cv);
    E->roles.push_back(C->U_new);
    E->roles.push_back(C->theta_final);
  }
  *out = holder.release();
  return SPD_OK;
}

int spd_ensemble_graph_nodes(const spd_ensemble* E, long long* nodes) {
  if (!E || !nodes) return SPD_ERR_ARG;
  size_t n = 0;
  if (E->graph && cudaGraphGetNodes(E->graph, nullptr, &n) != cudaSuccess) return SPD_ERR_CUDA;
  *nodes = (long long)n;
  return SPD_OK;
}

int spd_ensemble_step(spd_ensemble* E, int nlaunch) {
  if (!E || nlaunch < 0) return SPD_ERR_ARG;
  for (int i = 0; i < nlaunch; ++i) ECK(cudaGraphLaunch(E->exec, E->main));
  for (size_t i = 0; i < E->ctx.size(); ++i) {
    E->ctx[i]->U_cv = E->roles[3 * i];
    E->ctx[i]->U_new = E->roles[3 * i + 1];
    E->ctx[i]->theta_final = E->roles[3 * i + 2];
  }
  return SPD_OK;
}

int spd_ensemble_synchronize(spd_ensemble* E) {
  if (!E) return SPD_ERR_ARG;
  ECK(cudaStreamSynchronize(E->main));
  return SPD_OK;
}

int spd_ensemble_time(spd_ensemble* E, int i, double* t_out) {
  if (!E || !t_out || i < 0 || i >= (int)E->ctx.size()) return SPD_ERR_ARG;
  ECK(cudaStreamSynchronize(E->main));
  ECK(cudaMemcpy(t_out, E->ctx[i]->t_dev, sizeof(double), cudaMemcpyDeviceToHost));
  return SPD_OK;
}

int spd_ensemble_set_time(spd_ensemble* E, int i, double t) {
  if (!E || i < 0 || i >= (int)E->ctx.size()) return SPD_ERR_ARG;
  ECK(cudaStreamSynchronize(E->main));
  ECK(cudaMemcpy(E->ctx[i]->t_dev, &t, sizeof(double), cudaMemcpyHostToDevice));
  return SPD_OK;
}

int spd_ensemble_destroy(spd_ensemble* E) {
  if (!E) return SPD_ERR_ARG;
  if (E->main) cudaStreamSynchronize(E->main);
  if (E->exec) cudaGraphExecDestroy(E->exec);
  if (E->graph) cudaGraphDestroy(E->graph);
  for (auto s : E->streams) cudaStreamDestroy(s);
  for (auto e : E->join) cudaEventDestroy(e);
  if (E->fork) cudaEventDestroy(E->fork);
  if (E->main) cudaStreamDestroy(E->main);
  delete E;
  return SPD_OK;
}

const char* spd_ensemble_last_error(const spd_ensemble* E) { return E ? E->err.c_str() : t_last_err.c_str(); }

int spd_set_cells_per_block(spd_ctx* C, int cpb) {
  if (!C || cpb < 1 || cpb > C->stepper->max_cpb || (cpb & (cpb - 1))) return SPD_ERR_ARG;
  if (C->stepper->cpb != cpb && C->step_exec) {
    // the captured step carries the old launch shape
    cudaStreamSynchronize(C->stream);
    cudaGraphExecDestroy(C->step_exec);
    cudaGraphDestroy(C->step_graph);
    cudaGraphExecDestroy(C->dt_exec);
    cudaGraphDestroy(C->dt_graph);
    C->step_exec = nullptr;
    C->step_graph = nullptr;
    C->dt_exec = nullptr;
    C->dt_graph = nullptr;
  }
  C->stepper->cpb = cpb;
  return SPD_OK;
}

int spd_get_cells_per_block(const spd_ctx* C, int* cpb, int* max_cpb) {
  if (!C || !cpb || !max_cpb) return SPD_ERR_ARG;
  *cpb = C->stepper->cpb;
  *max_cpb = C->stepper->max_cpb;
  return SPD_OK;
}

}  // extern "C"
