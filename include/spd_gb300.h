/*
 * spd_gb300 -- C ABI of the GB300 (sm_103a) SD-ADER step for the
 * compressible Euler equations.
 *
 * The reference (jpalafou/spd) has no foreign-function layer: its operator
 * interface is the Python class SDADER_Simulator
 * (src/sdader_simulator.py:14).  Each entry point below replaces one method
 * of that class; the Python package spd_gb300 binds them with ctypes and
 * keeps the class surface.  All arrays crossing this boundary are FP64
 * arrays in the reference's C-order layouts (host arrays; U_sp, U_cv, W_cv
 * and the adjoint field may also be device arrays):
 *
 *   U_sp, U_cv, W_cv   (V, Nz, Ny, Nx, nz, ny, nx)          SD layout
 *   troubles           (1, Z, Y, X)                         Z = Nz*(p+1) ...
 *   theta              (1, Z+4, Y+4, X+4)
 *   affected_faces_x   (1, Z, Y, X+1)   (_y: (1, Z, Y+1, X), _z: (1, Z+1, Y, X))
 *   BC_fp_<dim>        (2, V, m+1, other cells..., other points...)
 *   BC_fv_<dim>        (2, V, extended extents with 2 along <dim>)
 *
 * with absent dimensions dropped (1D: (V, Nx, nx); 2D: (V, Ny, Nx, ny, nx)).
 * V = ndim + 2 variables ordered (rho, v_x[, v_y[, v_z]], P or E).
 *
 * Every function returns 0 on success and a nonzero spd_status otherwise;
 * spd_last_error() gives the message.  A context owns one CUDA stream and
 * its device buffers; it is not thread-safe, separate contexts may be used
 * from separate threads.  There is no CPU fallback: spd_create fails when
 * no CUDA device is available.
 */
#ifndef SPD_GB300_H
#define SPD_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct spd_ctx spd_ctx;
typedef struct spd_ensemble spd_ensemble;

enum spd_status {
  SPD_OK = 0,
  SPD_ERR_ARG = 1,      /* invalid argument or unsupported option */
  SPD_ERR_CUDA = 2,     /* CUDA runtime error */
  SPD_ERR_NONFINITE = 3 /* dt is not finite */
};

enum spd_riemann { SPD_LLF = 0, SPD_HLLC = 1, SPD_LHLLC = 2 };
enum spd_limiter { SPD_MINMOD = 0, SPD_MONCEN = 1 };
enum spd_update { SPD_UPDATE_SD = 0, SPD_UPDATE_FV = 1 };
enum spd_bc {
  SPD_BC_PERIODIC = 0,
  SPD_BC_REFLECTIVE = 1,
  SPD_BC_GRADFREE = 2,
  SPD_BC_IC = 3,
  SPD_BC_EQ = 4,
  SPD_BC_PRESSURE = 5
};

enum spd_field {
  SPD_U_SP = 0,
  SPD_U_CV = 1,
  SPD_W_CV = 2,
  SPD_TROUBLES = 3,
  SPD_THETA = 4,
  SPD_AFFECTED_X = 5,
  SPD_AFFECTED_Y = 6,
  SPD_AFFECTED_Z = 7,
  SPD_BC_FP_X = 8,
  SPD_BC_FP_Y = 9,
  SPD_BC_FP_Z = 10,
  SPD_BC_FV_X = 11,
  SPD_BC_FV_Y = 12,
  SPD_BC_FV_Z = 13,
  SPD_U_SP_ADJ = 14, /* adjoint of U_sp (U_sp layout), input and output of spd_vjp_step */
  /* read-only, update FV only: the flux-point fluxes of the last step's
   * final Picard iteration after the transverse subcell averaging, i.e. the
   * reference's F_ader_fp_<dim> after switch_to_finite_volume
   * (src/sdader_simulator.py:297-298); raw device layout [t][v][face], faces
   * x-fastest with N_d*(p+1)+1 faces along d and N*(p+1) along the others */
  SPD_F_FACES_X = 15,
  SPD_F_FACES_Y = 16,
  SPD_F_FACES_Z = 17,
  /* write-only, with potential: the gravity potential's gradient
   * (src/sdader_simulator.py:425-434) at the solution points, (ndim, Nz, Ny,
   * Nx, nz, ny, nx), and its subcell averages in the same SD layout
   * (compute_cv_from_sp of the former; the reference keeps them transposed
   * to the FV layout) */
  SPD_GRAD_PHI_SP = 18,
  SPD_GRAD_PHI_CV = 19,
  /* write-only, with WB: the equilibrium of the well-balanced mode
   * (src/sdader_simulator.py:436-481), in the reference's layouts --
   * U_eq_sp (SD layout), U_eq_cv (cell averages, SD layout), per direction
   * M_eq_fp / F_eq_fp (conservative state and flux at the flux points,
   * (V, cells..., points...) with p+2 points along the direction), with the
   * FV update per direction M_eq_faces / F_eq_faces (primitive state and
   * flux at the subcell faces, FV face layout) and M_eq_fv (primitives on
   * the subcell grid with 2 ghost layers) */
  SPD_U_EQ_SP = 20,
  SPD_U_EQ_CV = 21,
  SPD_M_EQ_FP_X = 22,
  SPD_M_EQ_FP_Y = 23,
  SPD_M_EQ_FP_Z = 24,
  SPD_F_EQ_FP_X = 25,
  SPD_F_EQ_FP_Y = 26,
  SPD_F_EQ_FP_Z = 27,
  SPD_M_EQ_FACES_X = 28,
  SPD_M_EQ_FACES_Y = 29,
  SPD_M_EQ_FACES_Z = 30,
  SPD_F_EQ_FACES_X = 31,
  SPD_F_EQ_FACES_Y = 32,
  SPD_F_EQ_FACES_Z = 33,
  SPD_M_EQ_FV = 34
};

/* Constructor options of SDADER_Simulator (src/simulator.py:10-36,
 * src/sd_simulator.py:20-26, src/fv_simulator.py:11-17,
 * src/sdader_simulator.py:15-27).  Strings become the enums above. */
typedef struct spd_config {
  int ndim;              /* 1, 2 or 3 */
  int N[3];              /* cells per direction, x first */
  int p;                 /* polynomial degree, 1..4 */
  int m;                 /* time order (m+1 ADER nodes), 0..5 */
  double lim[3][2];      /* xlim, ylim, zlim */
  double gamma;
  double cfl_coeff;
  double min_c2;
  int riemann_solver_sd; /* spd_riemann */
  int riemann_solver_fv; /* spd_riemann */
  int slope_limiter;     /* spd_limiter */
  int update;            /* spd_update */
  int FB;
  double tolerance;
  int SED;
  int NAD_delta;         /* NAD == "delta" */
  int PAD;
  int blending;
  double min_rho, max_rho, min_P;
  int godunov;
  int BC[3][2];          /* spd_bc per direction and side */
  /* viscosity (src/simulator.py:23-28, src/sdader_simulator.py:245-268):
   * the SD update, or the FV update without FB (the reference's viscous
   * fallback fluxes raise AttributeError, src/muscl.py:253) */
  int viscosity;
  double nu;
  double beta;
  /* gravity potential source terms (src/simulator.py:197-203) in the
   * predictor's dUdt and the subcell update; gradients by spd_upload */
  int potential;
  /* isothermal system (src/hydro.py:84,123,169, src/riemann_solver.py:142,210) */
  int isothermal;
  /* well-balanced mode (src/sdader_simulator.py:361-378 and callees): the
   * step advances U - U_eq; the equilibrium arrays by spd_upload */
  int WB;
} spd_config;

/* Constant operators built at setup on the host
 * (src/sd_simulator.py:30-52, src/sdader_simulator.py:40-46,61-92),
 * row-major. */
typedef struct spd_operators {
  const double* sp_to_fp;      /* (p+2) x (p+1) */
  const double* dfp_to_sp;     /* (p+1) x (p+2) */
  const double* sp_to_cv;      /* (p+1) x (p+1) */
  const double* cv_to_sp;      /* (p+1) x (p+1) */
  const double* invader;       /* (m+1) x (m+1), already weighted by w_tp */
  const double* w_tp;          /* m+1 */
  const double* faces[3];      /* subcell face positions with 2 ghost layers:
                                  N*(p+1) + 5 values per direction */
} spd_operators;

/* SDADER_Simulator.__init__ (device part): allocate the context. */
int spd_create(const spd_config* cfg, const spd_operators* ops, spd_ctx** out);
/* Copy a host array in the reference layout into the context. */
int spd_upload(spd_ctx* ctx, int field, const double* host, size_t count);
/* Copy a context array into a host buffer in the reference layout. */
int spd_download(spd_ctx* ctx, int field, double* host, size_t count);
/* SD_Simulator.compute_dt (src/sd_simulator.py:214-227). */
int spd_compute_dt(spd_ctx* ctx, double* dt_out);
/* Assign dm.dt (src/sdader_simulator.py:408). */
int spd_set_dt(spd_ctx* ctx, double dt);
int spd_get_dt(spd_ctx* ctx, double* dt_out);
/* SDADER_Simulator.perform_update (src/sdader_simulator.py:361-378) with
 * the current dt; *time_inout += dt on return. */
int spd_perform_update(spd_ctx* ctx, double* time_inout);
/* The loop bodies of perform_iterations (:394-399) and
 * perform_time_evolution (:401-413), without init_sim / end_sim.
 * mode 0: n_step iterations of (compute_dt, perform_update);
 * mode 1: advance while *time_inout < t_end with the t_end clip and the
 *         dt < 1e-14 stop.  *nsteps_done receives the steps taken.
 * A non-finite dt does not stop the loop (the reference runs on with it);
 * the call then returns SPD_ERR_NONFINITE with the steps done. */
int spd_step(spd_ctx* ctx, int nsteps, double t_end, int mode, double* time_inout, int* nsteps_done);
/* SDADER_Simulator.end_sim (:385-392): U_cv = sp_to_cv(U_sp), W_cv = prim(U_cv). */
int spd_end_sim(spd_ctx* ctx);
/* Wait for all work of the context. */
int spd_synchronize(spd_ctx* ctx);
/* Launch subsequent work on an external CUDA stream (a cudaStream_t, for
 * example the current stream of a framework); NULL restores the context's
 * own stream.  No reference counterpart (the reference runs on the host or
 * on CuPy's default stream). */
int spd_set_stream(spd_ctx* ctx, void* stream);
/* Per-kernel CUDA-event timing of subsequent launches on the context's
 * stream (enable = 1) -- the measurement hook of the benchmark; no
 * reference counterpart (the reference's only timer is the wall clock in
 * src/sdader_simulator.py:383,387). */
int spd_profile(spd_ctx* ctx, int enable);
/* One line "kernel launches total_ms" per kernel recorded since the last
 * report; clears the record. */
int spd_profile_report(spd_ctx* ctx, char* buf, size_t len);
/* Kernels launched by the context since it was created. */
int spd_launch_count(const spd_ctx* ctx, long long* count);
int spd_destroy(spd_ctx* ctx);
/* CFL time step dt = cfl_coeff * (h / max(ndim*c_s + sum |v|)) from
 * primitive subcell averages already on the device, without allocating
 * device memory (the inviscid limit; the viscous one of compute_dt is not
 * applied).  No counterpart in the reference: it serves callers that must
 * not call cudaMalloc -- a host framework whose allocator owns all device
 * memory, real-time loops that forbid allocation after start-up.  W_cv_dev holds
 * ndim + 2 variables one after the other, n_subcells values each (any
 * subcell order); h = h_min / (p + 1); dt_dev receives one double; the
 * work is queued on ``stream`` (a cudaStream_t, NULL = default stream).
 * At most 4,194,304 subcells per call (larger returns SPD_ERR_ARG).  Its
 * scratch is a fixed 128 KB array in the library image: the first call on
 * each device looks up that array's device address (make the first call
 * before any stream capture); calls that overlap on the GPU share the
 * array and race. */
int spd_cfl_dt_noalloc(const double* W_cv_dev, long long n_subcells, int ndim, double gamma, double min_c2,
                       double cfl_coeff, double h, double* dt_dev, void* stream);
const char* spd_last_error(const spd_ctx* ctx);
const char* spd_version(void);

/* ---- batched ensembles (no reference counterpart) ----------------------
 * Many independent contexts of different sizes advanced together: the step
 * of every instance (its own CFL dt, predictor, FV update and a device-side
 * time accumulator) is recorded once into one CUDA graph whose branches run
 * on ``nstreams`` streams (instances assigned largest-first to the least
 * loaded stream); one launch advances every instance ``steps_per_launch``
 * steps.  The contexts stay owned by the caller and must outlive the
 * ensemble; their simulated time restarts at 0 in the device accumulator. */
int spd_ensemble_create(spd_ctx** ctxs, int n, int nstreams, int steps_per_launch, spd_ensemble** out);
/* Packed form of the same ensemble: every kernel launch of the step covers
 * all instances at once.  A per-instance table of block offsets maps each
 * thread block to its instance (geometry, buffers, its own dt) and to its
 * block within that instance, so each instance computes exactly what its own
 * step computes (bit-identical) while a whole ensemble step costs ~100
 * launches instead of ~100 per instance; the sequence is captured in one
 * CUDA graph.  The instances must share the dimension, degree, options and
 * cells per block (they may differ in grid size, domain and boundary
 * conditions); otherwise SPD_ERR_ARG with the reason in
 * spd_ensemble_last_error(NULL). */
int spd_ensemble_create_packed(spd_ctx** ctxs, int n, int steps_per_launch, spd_ensemble** out);
/* Number of nodes (kernel launches, zero-fills, stream joins) of the
 * ensemble's CUDA graph. */
int spd_ensemble_graph_nodes(const spd_ensemble* ens, long long* nodes);
/* Enqueue nlaunch graph launches (asynchronous). */
int spd_ensemble_step(spd_ensemble* ens, int nlaunch);
int spd_ensemble_synchronize(spd_ensemble* ens);
/* Simulated time of instance i kept on the device (each step adds its dt). */
int spd_ensemble_time(spd_ensemble* ens, int i, double* t_out);
int spd_ensemble_set_time(spd_ensemble* ens, int i, double t);
int spd_ensemble_destroy(spd_ensemble* ens);
/* Last error of ``ens``; with NULL, the calling thread's most recent
 * ensemble error (e.g. why a create failed). */
const char* spd_ensemble_last_error(const spd_ensemble* ens);
/* Cells per thread block of the predictor's fused interior kernel (a power
 * of two up to the shared-memory bound reported by the getter); a tuning
 * knob of the ensemble autotuner, results are independent of it. */
int spd_set_cells_per_block(spd_ctx* ctx, int cpb);
int spd_get_cells_per_block(const spd_ctx* ctx, int* cpb, int* max_cpb);

/* ---- adjoint (no reference counterpart) --------------------------------
 * Vector-Jacobian product of one SD-ADER step U_sp -> U_sp'.  The step is
 * differentiated with dt, the trouble masks, theta, the affected faces, the
 * slope-limiter branches and the Riemann-solver branches frozen at their
 * values in a recorded forward step.
 * spd_adjoint_enable allocates ``depth`` record slots (the forward
 * intermediates of one step each: U_sp, the Picard iterates, the FV substep
 * states and affected faces) and the adjoint work arrays.
 * spd_record_step advances U_sp by one step with the given dt (no CFL
 * reduction) and records it into ``slot``; the step is bit-identical to
 * spd_set_dt + spd_perform_update.
 * spd_vjp_step replaces the SPD_U_SP_ADJ field a by J^T a, J the Jacobian of
 * the step recorded in ``slot``.
 * Decision tapes (for finite-difference checks of the adjoint):
 * spd_tape_enable allocates tapes for ``nsteps`` steps; spd_tape_step
 * advances U_sp by one step with the given dt and, with mode 1, records the
 * step's decisions into tape ``step`` (the affected faces and the branch
 * outcomes of every Riemann problem and limited slope) or, with mode 2,
 * replays them instead of taking them: the frozen-decision step whose
 * Jacobian spd_vjp_step applies.  Mode 1 is bit-identical to
 * spd_set_dt + spd_perform_update.
 * Uploads and downloads of U_sp, U_cv, W_cv and SPD_U_SP_ADJ accept host or
 * device pointers. */
int spd_adjoint_enable(spd_ctx* ctx, int depth);
int spd_adjoint_depth(const spd_ctx* ctx, int* depth);
int spd_record_step(spd_ctx* ctx, int slot, double dt);
int spd_vjp_step(spd_ctx* ctx, int slot);
int spd_tape_enable(spd_ctx* ctx, int nsteps);
int spd_tape_step(spd_ctx* ctx, int step, double dt, int mode);

#ifdef __cplusplus
}
#endif

#endif /* SPD_GB300_H */
