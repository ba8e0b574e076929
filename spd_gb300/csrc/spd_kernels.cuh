// SD-ADER step kernels for sm_103a, templated on the space dimension D and
// the polynomial degree P.  FP64 on the CUDA cores; bit-identical to the
// reference's NumPy path (src/sdader_simulator.py and callees).
//
// Device layouts (cells and subcells x-fastest):
//   U_sp   [v][s][c]        s = kx + n*(ky + n*kz),  c = cx + Nx*(cy + Ny*cz)
//   U_ader [v][t][s][c]
//   trace  [d][side][v][t][j][c]   edge-point states of direction d,
//                                  j = transverse point of the cell face
//   Fi     [d][v][t][j][iface]     element-interface Riemann fluxes
//   Ffp    [d][v][t][j][f][c]      flux-point fluxes (FV update only)
//   FV     [v][iz][iy][ix]         subcell arrays (U_cv, W_cv, U_new)
//   ext    [v][ze][ye][xe]         subcell arrays with 2 ghost layers
#pragma once
#include "spd_device.cuh"

namespace spd {

struct Ops {
  double sp_to_fp[MAXNF * MAXN];
  double dfp_to_sp[MAXN * MAXNF];
  double sp_to_cv[MAXN * MAXN];
  double invader[MAXT * MAXT];
  double w_tp[MAXT];
  // dfp_to_sp * (1/h_d) for directions whose h_d is a power of two: scaling
  // every product and partial sum of the derivative by 2^k is exact (away
  // from underflow and overflow), so sum(dfp*F)*(1/h) == sum((dfp/h)*F)
  double dfp_h[3][MAXN * MAXNF];
};

struct Geo {
  int N[3];        // cells per direction (1 for absent directions)
  int X[3];        // subcells per direction (N*n, 1 for absent)
  int Xe[3];       // extended subcells per direction (X+4, 1 for absent)
  int T;           // ADER time nodes
  long long Nc;    // cells
  long long Nq;    // subcells
  long long Nqe;   // extended subcells
  double h[3];
  double inv_h[3];  // 1/h, used only when h is a power of two (then x/h == x*(1/h) exactly)
  int h_pow2[3];
  double gamma, min_c2;
  int bc[3][2];
  int iso;  // isothermal (src/hydro.py:84,123,169)
};

template <int D, int P>
struct K {
  static constexpr int n = P + 1;
  static constexpr int nf = P + 2;
  static constexpr int V = D + 2;
  static constexpr int NS = (D == 1) ? n : (D == 2 ? n * n : n * n * n);
  static constexpr int NJ = NS / n;
};

// in-cell point index of point k along direction d on transverse line j
template <int D, int P>
__device__ __forceinline__ int sp_index(int d, int j, int k) {
  constexpr int n = P + 1;
  if (d == 0) return k + n * j;
  if (d == 1) return (j % n) + n * k + n * n * (j / n);
  return j + n * n * k;
}

__device__ __forceinline__ void cell_coords(const Geo& g, long long c, int& cx, int& cy, int& cz) {
  cx = (int)(c % g.N[0]);
  long long r = c / g.N[0];
  cy = (int)(r % g.N[1]);
  cz = (int)(r / g.N[1]);
}

// interface id along d for the cell with coordinates (cx,cy,cz), index i along d
__device__ __forceinline__ long long iface_id(const Geo& g, int d, int cx, int cy, int cz, int i) {
  if (d == 0) return (long long)i + (long long)(g.N[0] + 1) * (cy + (long long)g.N[1] * cz);
  if (d == 1) return (long long)cx + (long long)g.N[0] * (i + (long long)(g.N[1] + 1) * cz);
  return (long long)cx + (long long)g.N[0] * (cy + (long long)g.N[1] * i);
}

__host__ __device__ __forceinline__ long long n_iface(const Geo& g, int d) {
  return g.Nc / g.N[d] * (g.N[d] + 1);
}

// ---------------------------------------------------------------------------
// edge traces of one (cell, time node): sp -> fp 0 and fp nf-1 along every
// direction (src/sdader_simulator.py:220, src/transforms.py:3-25)
// ---------------------------------------------------------------------------
template <int D, int P>
__device__ __forceinline__ void write_traces(const Ops& op, const Geo& g, const double* __restrict__ U, int Tu,
                                             int tu, long long c, double* const* trace, int t_out) {
  using k = K<D, P>;
  for (int d = 0; d < D; ++d) {
    for (int j = 0; j < k::NJ; ++j) {
#pragma unroll
      for (int v = 0; v < k::V; ++v) {
        double x[k::n];
#pragma unroll
        for (int s = 0; s < k::n; ++s)
          x[s] = U[(((long long)v * Tu + tu) * k::NS + sp_index<D, P>(d, j, s)) * g.Nc + c];
        const double l = dot_dir<k::n>(op.sp_to_fp, x, d);
        const double r = dot_dir<k::n>(op.sp_to_fp + (k::nf - 1) * k::n, x, d);
        trace[d][(((long long)(0 * k::V + v) * g.T + t_out) * k::NJ + j) * g.Nc + c] = l;
        trace[d][(((long long)(1 * k::V + v) * g.T + t_out) * k::NJ + j) * g.Nc + c] = r;
      }
    }
  }
}

// Every kernel of the step is a body ``run(Blk, args...)`` plus a plain
// ``__global__`` wrapper that passes the hardware block index; the batched
// ensemble launches the same bodies over many instances at once.
template <int D, int P>
struct TracesSp {
  static __device__ __forceinline__ void run(Blk B, const Ops& op, const Geo& g, const double* __restrict__ U_sp,
                                             double* t0, double* t1, double* t2) {
    const long long c = B.id * (long long)blockDim.x + threadIdx.x;
    if (c >= g.Nc) return;
    double* tr[3] = {t0, t1, t2};
    write_traces<D, P>(op, g, U_sp, 1, 0, c, tr, 0);
  }
};
template <int D, int P>
__global__ void k_traces_sp(Ops op, Geo g, const double* __restrict__ U_sp, double* t0, double* t1, double* t2) {
  TracesSp<D, P>::run(hw_blk(), op, g, U_sp, t0, t1, t2);
}

// traces of every (cell, time node) of an iterate U (Tu time nodes stored)
template <int D, int P>
__global__ void k_traces_ader(Ops op, Geo g, const double* __restrict__ U, int Tu, int Teff, double* t0, double* t1,
                              double* t2) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= g.Nc * Teff) return;
  const long long c = tid % g.Nc;
  const int t = (int)(tid / g.Nc);
  double* tr[3] = {t0, t1, t2};
  write_traces<D, P>(op, g, U, Tu, (Tu == 1) ? 0 : t, c, tr, t);
}

// ---------------------------------------------------------------------------
// element-interface Riemann fluxes for direction d
// (src/sdader_simulator.py:225-234, src/sd_boundary.py:7-76)
// ---------------------------------------------------------------------------
// DIR >= 0 fixes the direction at compile time (the rotated velocity
// indices become constants); DIR = -1 takes it from d_rt.
template <int D, int P, int BM = 0, int DIR = -1, bool EQ = false>
struct RiemannSd {
static __device__ __forceinline__ void run(Blk B, const Geo& g, int d_rt, int Teff, int solver,
                                           const double* __restrict__ trace, const double* __restrict__ bcfix,
                                           double* __restrict__ Fi, unsigned* tape,
                                           const double* __restrict__ meq) {
  using k = K<D, P>;
  const int d = (DIR >= 0) ? DIR : d_rt;
  const long long nI = n_iface(g, d);
  const long long total = (long long)Teff * k::NJ * nI;
  const long long tid = B.id * (long long)blockDim.x + threadIdx.x;
  if (tid >= total) return;
  const long long iface = tid % nI;
  const long long r = tid / nI;
  const int j = (int)(r % k::NJ);
  const int t = (int)(r / k::NJ);
  // decode interface -> (i along d, transverse cell coords)
  int cx = 0, cy = 0, cz = 0, i = 0;
  if (d == 0) {
    i = (int)(iface % (g.N[0] + 1));
    long long q = iface / (g.N[0] + 1);
    cy = (int)(q % g.N[1]);
    cz = (int)(q / g.N[1]);
  } else if (d == 1) {
    cx = (int)(iface % g.N[0]);
    long long q = iface / g.N[0];
    i = (int)(q % (g.N[1] + 1));
    cz = (int)(q / (g.N[1] + 1));
  } else {
    cx = (int)(iface % g.N[0]);
    long long q = iface / g.N[0];
    cy = (int)(q % g.N[1]);
    i = (int)(q / g.N[1]);
  }
  const int Nd = g.N[d];
  auto cell_at = [&](int idx) -> long long {
    int x = cx, y = cy, z = cz;
    if (d == 0) x = idx; else if (d == 1) y = idx; else z = idx;
    return x + (long long)g.N[0] * (y + (long long)g.N[1] * z);
  };
  // transverse cell index of the face plane
  const long long ct = (d == 0) ? (cy + (long long)g.N[1] * cz) : (d == 1 ? (cx + (long long)g.N[0] * cz)
                                                                            : (cx + (long long)g.N[0] * cy));
  const long long ntrans = g.Nc / Nd;
  // the edge state: the trace of the iterate, plus (well-balanced mode,
  // src/sdader_simulator.py:221-223) the equilibrium at that flux point
  auto tr = [&](int side, int v, long long cell) -> double {
    double val = trace[(((long long)(side * k::V + v) * g.T + t) * k::NJ + j) * g.Nc + cell];
    if constexpr (EQ) {
      if (meq) val = val + meq[(((long long)v * k::NJ + j) * k::nf + (side ? k::nf - 1 : 0)) * g.Nc + cell];
    }
    return val;
  };
  auto fix = [&](int side, int v) -> double {
    return bcfix[(((long long)side * k::V + v) * k::NJ + j) * ntrans + ct];
  };
  double ML[k::V], MR[k::V];
  const int b0 = g.bc[d][0], b1 = g.bc[d][1];
  if (i == 0) {
    const long long c0 = cell_at(0);
#pragma unroll
    for (int v = 0; v < k::V; ++v) {
      double val;
      if (b0 == BC_PERIODIC) val = tr(1, v, cell_at(Nd - 1));
      else if (b0 == BC_REFLECTIVE) val = (v == d + 1) ? tr(0, v, c0) * -1.0 : tr(0, v, c0);
      else if (b0 == BC_GRADFREE) val = tr(0, v, c0);
      else val = fix(0, v);
      ML[v] = val;
      MR[v] = (b0 == BC_PRESSURE) ? fix(0, v) : tr(0, v, c0);
    }
    if (Nd == 1 && b1 == BC_PRESSURE) { /* right trace of the same cell is not used here */ }
  } else if (i == Nd) {
    const long long cl = cell_at(Nd - 1);
#pragma unroll
    for (int v = 0; v < k::V; ++v) {
      double val;
      if (b1 == BC_PERIODIC) val = (b0 == BC_PRESSURE) ? fix(0, v) : tr(0, v, cell_at(0));
      else if (b1 == BC_REFLECTIVE) val = (v == d + 1) ? tr(1, v, cl) * -1.0 : tr(1, v, cl);
      else if (b1 == BC_GRADFREE) val = tr(1, v, cl);
      else val = fix(1, v);
      MR[v] = val;
      ML[v] = (b1 == BC_PRESSURE) ? fix(1, v) : tr(1, v, cl);
    }
  } else {
    const long long cl = cell_at(i - 1), cr = cell_at(i);
#pragma unroll
    for (int v = 0; v < k::V; ++v) {
      ML[v] = tr(1, v, cl);
      MR[v] = tr(0, v, cr);
    }
  }
  double F[k::V];
  Br<BM> br;
  if (BM == 2) br.w = tape[tid];
  // the isothermal system only in the EQ form: a runtime flag costs the
  // plain form an FP64 multiply per flux (the compiler predicates it)
  riemann<D, double, BM>(solver, ML, MR, F, g.gamma, g.min_c2, d, false, &br, EQ && g.iso != 0);
  if (BM == 1) tape[tid] = br.w;
#pragma unroll
  for (int v = 0; v < k::V; ++v) Fi[(((long long)v * g.T + t) * k::NJ + j) * nI + iface] = F[v];
}
};
// EQ: the form for the well-balanced mode (meq non-null: the equilibrium
// at the flux points added to every edge state) and the isothermal system;
// the plain form reads neither
template <int D, int P, int BM = 0, int DIR = -1, bool EQ = false>
__global__ void k_riemann_sd(Geo g, int d_rt, int Teff, int solver, const double* __restrict__ trace,
                             const double* __restrict__ bcfix, double* __restrict__ Fi, unsigned* tape,
                             const double* __restrict__ meq) {
  RiemannSd<D, P, BM, DIR, EQ>::run(hw_blk(), g, d_rt, Teff, solver, trace, bcfix, Fi, tape, meq);
}

// ---------------------------------------------------------------------------
// interior flux points, derivative, Picard update (src/sdader_simulator.py:
// 148-200) or the final SD update (:202-208) or the flux-point output for
// the FV update (:288-298).  Block = (CPB cells) x (rows >= Teff): rows
// tl < Teff compute the flux derivative of time node tl (Teff = 1 in the
// first Picard iteration, else T); after the barrier every row writes its
// share of the outputs (time node t_out = tl, tl + rows, ...), so the first
// iteration may run with T rows and its single computed node spread over
// them (CPB a multiple of 32 keeps every warp in one row).
// mode: 0 = Picard (writes U_ader and next traces), 1 = SD update of U_sp,
//       2 = write Ffp.
// ---------------------------------------------------------------------------
// EXT: optional terms, each present when its pointer is not null -- the
// viscous fluxes G[d] (src/sdader_simulator.py:268, layout of Ffp),
// subtracted from the flux at every flux point, Riemann edges included,
// before the derivative (spd_visc.cuh); the gravity source of the
// potential gradient gphi [d][s][cell] added to the derivative
// (src/sdader_simulator.py:154-157, src/simulator.py:197-203).
template <int D, int P, bool EXT = false>
struct Interior {
static __device__ __forceinline__ void run(Blk B, const Ops& op, const Geo& g, int mode, int Teff,
                                           const double* __restrict__ Uin, int Tu, const double* __restrict__ dt_ptr,
                                           double* __restrict__ U_sp, double* __restrict__ U_ader, const double* Fi0,
                                           const double* Fi1, const double* Fi2, double* tr0, double* tr1,
                                           double* tr2, double* Ffp0, double* Ffp1, double* Ffp2,
                                           const double* G0 = nullptr, const double* G1 = nullptr,
                                           const double* G2 = nullptr, const double* gphi = nullptr,
                                           const double* const* meqs = nullptr,
                                           const double* const* feqs = nullptr) {
  using k = K<D, P>;
  const double* Gv[3] = {G0, G1, G2};
  const bool visc = EXT && G0 != nullptr;
  const bool pot = EXT && gphi != nullptr;
  const bool wb = EXT && meqs != nullptr;
  // the isothermal system runs in the EXT form only (a runtime flag would
  // cost the plain form a predicated FP64 multiply per flux point)
  const bool iso = EXT && g.iso != 0;
  extern __shared__ double dudt_s[];  // [(v*NS + s)*Teff + tl][CPB]
  const int CPB = blockDim.x;
  const int cl = threadIdx.x, tl = threadIdx.y;
  const long long c = B.id * (long long)CPB + cl;
  const bool active = c < g.Nc;
  const double* Fi[3] = {Fi0, Fi1, Fi2};
  double* Ffp[3] = {Ffp0, Ffp1, Ffp2};
  const int tu = (Tu == 1) ? 0 : tl;
  if (active && tl < Teff) {
    int cx, cy, cz;
    cell_coords(g, c, cx, cy, cz);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const long long nI = n_iface(g, d);
      const int cd = (d == 0) ? cx : (d == 1 ? cy : cz);
      const long long il = iface_id(g, d, cx, cy, cz, cd);
      const long long ir = iface_id(g, d, cx, cy, cz, cd + 1);
      for (int j = 0; j < k::NJ; ++j) {
        double u[k::V][k::n];
#pragma unroll
        for (int v = 0; v < k::V; ++v)
#pragma unroll
          for (int s = 0; s < k::n; ++s)
            u[v][s] = Uin[(((long long)v * Tu + tu) * k::NS + sp_index<D, P>(d, j, s)) * g.Nc + c];
        double Fl[k::V][k::nf];
#pragma unroll
        for (int f = 1; f < k::nf - 1; ++f) {
          double M[k::V], W[k::V], F[k::V];
#pragma unroll
          for (int v = 0; v < k::V; ++v) M[v] = dot_dir<k::n>(op.sp_to_fp + f * k::n, u[v], d);
          if (wb) {
#pragma unroll
            for (int v = 0; v < k::V; ++v)
              M[v] = M[v] + meqs[d][((((long long)v * k::NJ + j) * k::nf + f)) * g.Nc + c];
          }
          prim<D>(M, W, g.gamma, 0, (double*)nullptr, iso);
          flux<D>(W, F, g.gamma, d, iso);
#pragma unroll
          for (int v = 0; v < k::V; ++v) Fl[v][f] = F[v];
        }
#pragma unroll
        for (int v = 0; v < k::V; ++v) {
          Fl[v][0] = Fi[d][(((long long)v * g.T + tl) * k::NJ + j) * nI + il];
          Fl[v][k::nf - 1] = Fi[d][(((long long)v * g.T + tl) * k::NJ + j) * nI + ir];
        }
        if (wb) {
          // F -> F' (src/sdader_simulator.py:235-237), before the viscous flux
#pragma unroll
          for (int v = 0; v < k::V; ++v)
#pragma unroll
            for (int f = 0; f < k::nf; ++f)
              Fl[v][f] = Fl[v][f] - feqs[d][(((long long)v * k::NJ + j) * k::nf + f) * g.Nc + c];
        }
        if (visc) {
#pragma unroll
          for (int v = 0; v < k::V; ++v)
#pragma unroll
            for (int f = 0; f < k::nf; ++f)
              Fl[v][f] = Fl[v][f] - Gv[d][((((long long)v * g.T + tl) * k::NJ + j) * k::nf + f) * g.Nc + c];
        }
        if (mode == 2) {
#pragma unroll
          for (int v = 0; v < k::V; ++v)
#pragma unroll
            for (int f = 0; f < k::nf; ++f)
              Ffp[d][((((long long)v * g.T + tl) * k::NJ + j) * k::nf + f) * g.Nc + c] = Fl[v][f];
        } else {
          const double hd = g.h[d], ihd = g.inv_h[d];
          const bool pow2 = g.h_pow2[d] != 0;
#pragma unroll
          for (int v = 0; v < k::V; ++v) {
#pragma unroll
            for (int so = 0; so < k::n; ++so) {
              const double val = pow2 ? dot_dir<k::nf>(op.dfp_h[d] + so * k::nf, Fl[v], d)
                                      : div_rcp(dot_dir<k::nf>(op.dfp_to_sp + so * k::nf, Fl[v], d), hd, ihd);
              const int s = sp_index<D, P>(d, j, so);
              double* slot = &dudt_s[(((long long)v * k::NS + s) * Teff + tl) * CPB + cl];
              *slot = (d == 0) ? val : *slot + val;
            }
          }
        }
      }
    }
    if (pot && mode != 2) {
      // dUdt[vel] += rho * dphi_vel, dUdt[P] += m_vel * dphi_vel, direction by
      // direction, with the iterate the fluxes came from
      for (int s = 0; s < k::NS; ++s) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const double gp = gphi[((long long)d * k::NS + s) * g.Nc + c];
          const double u0 = Uin[(((long long)0 * Tu + tu) * k::NS + s) * g.Nc + c];
          const double uv = Uin[(((long long)(d + 1) * Tu + tu) * k::NS + s) * g.Nc + c];
          double* sv = &dudt_s[((((long long)(d + 1)) * k::NS + s) * Teff + tl) * CPB + cl];
          *sv = *sv + u0 * gp;
          if (!iso) {
            double* sp = &dudt_s[((((long long)(D + 1)) * k::NS + s) * Teff + tl) * CPB + cl];
            *sp = *sp + uv * gp;
          }
        }
      }
    }
  }
  if (mode == 2) return;
  __syncthreads();
  if (!active) return;
  const double dt = *dt_ptr;
  auto dudt = [&](int v, int s, int p) -> double {
    return dudt_s[(((long long)v * k::NS + s) * Teff + (Teff == 1 ? 0 : p)) * CPB + cl];
  };
  if (mode == 0) {
    double* tr[3] = {tr0, tr1, tr2};
    for (int t_out = tl; t_out < g.T; t_out += (int)blockDim.y) {
      for (int v = 0; v < k::V; ++v) {
        for (int s = 0; s < k::NS; ++s) {
          double acc = op.invader[t_out * g.T + 0] * dudt(v, s, 0);
          for (int p = 1; p < g.T; ++p) acc = acc + op.invader[t_out * g.T + p] * dudt(v, s, p);
          const double usp = U_sp[((long long)v * k::NS + s) * g.Nc + c];
          U_ader[(((long long)v * g.T + t_out) * k::NS + s) * g.Nc + c] = usp - acc * dt;
        }
      }
      write_traces<D, P>(op, g, U_ader, g.T, t_out, c, tr, t_out);
    }
  } else {
    for (int kk = tl; kk < k::V * k::NS; kk += (int)blockDim.y) {
      const int v = kk / k::NS, s = kk % k::NS;
      double acc = op.w_tp[0] * dudt(v, s, 0);
      for (int t = 1; t < g.T; ++t) acc = acc + op.w_tp[t] * dudt(v, s, t);
      double* u = &U_sp[((long long)v * k::NS + s) * g.Nc + c];
      *u = *u - acc * dt;
    }
  }
}
};
template <int D, int P>
__global__ void k_interior(Ops op, Geo g, int mode, int Teff, const double* __restrict__ Uin, int Tu,
                           const double* __restrict__ dt_ptr, double* __restrict__ U_sp, double* __restrict__ U_ader,
                           const double* Fi0, const double* Fi1, const double* Fi2, double* tr0, double* tr1,
                           double* tr2, double* Ffp0, double* Ffp1, double* Ffp2) {
  Interior<D, P>::run(hw_blk(), op, g, mode, Teff, Uin, Tu, dt_ptr, U_sp, U_ader, Fi0, Fi1, Fi2, tr0, tr1, tr2, Ffp0,
                      Ffp1, Ffp2);
}
template <int D, int P>
struct InteriorExt {
  static __device__ __forceinline__ void run(Blk B, const Ops& op, const Geo& g, int mode, int Teff,
                                             const double* __restrict__ Uin, int Tu, const double* __restrict__ dt_ptr,
                                             double* __restrict__ U_sp, double* __restrict__ U_ader,
                                             const double* Fi0, const double* Fi1, const double* Fi2, double* tr0,
                                             double* tr1, double* tr2, double* Ffp0, double* Ffp1, double* Ffp2,
                                             const double* G0, const double* G1, const double* G2,
                                             const double* gphi, const double* M0, const double* M1,
                                             const double* M2, const double* E0, const double* E1,
                                             const double* E2) {
    const double* meqs[3] = {M0, M1, M2};
    const double* feqs[3] = {E0, E1, E2};
    Interior<D, P, true>::run(B, op, g, mode, Teff, Uin, Tu, dt_ptr, U_sp, U_ader, Fi0, Fi1, Fi2, tr0, tr1, tr2, Ffp0,
                              Ffp1, Ffp2, G0, G1, G2, gphi, M0 ? meqs : nullptr, feqs);
  }
};
template <int D, int P>
__global__ void k_interior_ext(Ops op, Geo g, int mode, int Teff, const double* __restrict__ Uin, int Tu,
                               const double* __restrict__ dt_ptr, double* __restrict__ U_sp,
                               double* __restrict__ U_ader, const double* Fi0, const double* Fi1, const double* Fi2,
                               double* tr0, double* tr1, double* tr2, double* Ffp0, double* Ffp1, double* Ffp2,
                               const double* G0, const double* G1, const double* G2, const double* gphi,
                               const double* M0, const double* M1, const double* M2, const double* E0,
                               const double* E1, const double* E2) {
  InteriorExt<D, P>::run(hw_blk(), op, g, mode, Teff, Uin, Tu, dt_ptr, U_sp, U_ader, Fi0, Fi1, Fi2, tr0, tr1, tr2,
                         Ffp0, Ffp1, Ffp2, G0, G1, G2, gphi, M0, M1, M2, E0, E1, E2);
}

// ---------------------------------------------------------------------------
// transverse subcell averaging of the flux points and scatter to the FV face
// arrays of time node t (src/sd_simulator.py:208-212,
// src/sdader_simulator.py:310-323).  One thread per (cell, t, fp along d).
// F_HO layout [t][v][face], faces x-fastest with X_d + 1 along d.
// ---------------------------------------------------------------------------
template <int D, int P>
struct IntegrateFaces {
static __device__ __forceinline__ void run(Blk B, const Ops& op, const Geo& g, int d, const double* __restrict__ Ffp,
                                           double* __restrict__ F_HO) {
  using k = K<D, P>;
  const long long total = g.Nc * g.T * k::nf;
  const long long tid = B.id * (long long)blockDim.x + threadIdx.x;
  if (tid >= total) return;
  const long long c = tid % g.Nc;
  const long long r = tid / g.Nc;
  const int f = (int)(r % k::nf);
  const int t = (int)(r / k::nf);
  int cx, cy, cz;
  cell_coords(g, c, cx, cy, cz);
  const int cd = (d == 0) ? cx : (d == 1 ? cy : cz);
  if (f == k::nf - 1 && cd != g.N[d] - 1) return;
  const int fd = (f == k::nf - 1) ? g.N[d] * k::n : cd * k::n + f;
  const int FX = g.X[0] + (d == 0), FY = g.X[1] + (d == 1);
  const long long nface = (long long)FX * FY * (g.X[2] + (d == 2));
  // the other directions in increasing order
  int o0 = -1, o1 = -1;
  for (int e = 0; e < D; ++e) {
    if (e == d) continue;
    if (o0 < 0) o0 = e; else o1 = e;
  }
  for (int v = 0; v < k::V; ++v) {
    double G[k::NJ];
#pragma unroll
    for (int j = 0; j < k::NJ; ++j)
      G[j] = Ffp[((((long long)v * g.T + t) * k::NJ + j) * k::nf + f) * g.Nc + c];
    // transverse index j = a + n*b where a is the lower other direction
    if (D >= 2) {
      double G1[k::NJ];
      // along o0 (index a)
#pragma unroll
      for (int b = 0; b < k::NJ / k::n; ++b) {
        double x[k::n];
#pragma unroll
        for (int a = 0; a < k::n; ++a) x[a] = G[a + k::n * b];
#pragma unroll
        for (int ao = 0; ao < k::n; ++ao) G1[ao + k::n * b] = dot_dir<k::n>(op.sp_to_cv + ao * k::n, x, o0);
      }
      if (D == 3) {
#pragma unroll
        for (int a = 0; a < k::n; ++a) {
          double x[k::n];
#pragma unroll
          for (int b = 0; b < k::n; ++b) x[b] = G1[a + k::n * b];
#pragma unroll
          for (int bo = 0; bo < k::n; ++bo) G[a + k::n * bo] = dot_dir<k::n>(op.sp_to_cv + bo * k::n, x, o1);
        }
      } else {
#pragma unroll
        for (int jj = 0; jj < k::NJ; ++jj) G[jj] = G1[jj];
      }
    }
    for (int j = 0; j < k::NJ; ++j) {
      const int a = j % k::n, b = j / k::n;
      int fc[3] = {0, 0, 0};
      fc[d] = fd;
      const int cc[3] = {cx, cy, cz};
      if (o0 >= 0) fc[o0] = cc[o0] * k::n + a;
      if (o1 >= 0) fc[o1] = cc[o1] * k::n + b;
      const long long fid = fc[0] + (long long)FX * (fc[1] + (long long)FY * fc[2]);
      F_HO[((long long)t * k::V + v) * nface + fid] = G[j];
    }
  }
}
};
template <int D, int P>
__global__ void k_integrate_faces(Ops op, Geo g, int d, const double* __restrict__ Ffp, double* __restrict__ F_HO) {
  IntegrateFaces<D, P>::run(hw_blk(), op, g, d, Ffp, F_HO);
}

// ---------------------------------------------------------------------------
// whole-cell transforms sp <-> subcell averages (src/transforms.py:27-45)
// Kfull[o][i] holds the operator product ((A*A)*A) of output point o and
// input point i, formed exactly as the reference's einsum does.
// rows = false: one left-to-right sum over all input points (contiguous
//               input), 1D: two-lane sum, 2D with n = 2: row pairs;
// rows = true : per-row sums along x, then the row sums in order (strided
//               input, src/sdader_simulator.py:302-307).
// ---------------------------------------------------------------------------
template <int D, int P>
__device__ __forceinline__ double full_dot(const double* __restrict__ Krow, const double* x, bool rows) {
  using k = K<D, P>;
  if (D == 1) return dot_lanes2<k::n>(Krow, x);
  if (rows || (D == 2 && k::n == 2)) {
    double acc = 0.0;
#pragma unroll
    for (int r = 0; r < k::NS / k::n; ++r) {
      double rs = Krow[r * k::n] * x[r * k::n];
#pragma unroll
      for (int l = 1; l < k::n; ++l) rs = rs + Krow[r * k::n + l] * x[r * k::n + l];
      acc = (r == 0) ? rs : acc + rs;
    }
    return acc;
  }
  return dot_seq<k::NS>(Krow, x);
}

// U_cv (FV layout) = sp_to_cv(U_sp) for every cell and variable
template <int D, int P>
struct SpToCv {
static __device__ __forceinline__ void run(Blk B, const Geo& g, const double* __restrict__ Kfull,
                                           const double* __restrict__ U_sp, double* __restrict__ U_cv) {
  using k = K<D, P>;
  const long long tid = B.id * (long long)blockDim.x + threadIdx.x;
  if (tid >= g.Nc * k::V) return;
  const long long c = tid % g.Nc;
  const int v = (int)(tid / g.Nc);
  int cx, cy, cz;
  cell_coords(g, c, cx, cy, cz);
  double x[k::NS];
#pragma unroll
  for (int s = 0; s < k::NS; ++s) x[s] = U_sp[((long long)v * k::NS + s) * g.Nc + c];
  for (int o = 0; o < k::NS; ++o) {
    const int kx = o % k::n, ky = (o / k::n) % k::n, kz = o / (k::n * k::n);
    const long long q = (cx * k::n + kx) + (long long)g.X[0] * ((D >= 2 ? cy * k::n + ky : 0) +
                                                               (long long)g.X[1] * (D >= 3 ? cz * k::n + kz : 0));
    U_cv[(long long)v * g.Nq + q] = full_dot<D, P>(Kfull + (long long)o * k::NS, x, false);
  }
}
};
template <int D, int P>
__global__ void k_sp_to_cv(Geo g, const double* __restrict__ Kfull, const double* __restrict__ U_sp,
                           double* __restrict__ U_cv) {
  SpToCv<D, P>::run(hw_blk(), g, Kfull, U_sp, U_cv);
}

// U_sp = cv_to_sp(U_cv) (strided view order)
template <int D, int P>
struct CvToSp {
static __device__ __forceinline__ void run(Blk B, const Geo& g, const double* __restrict__ Kfull,
                                           const double* __restrict__ U_cv, double* __restrict__ U_sp) {
  using k = K<D, P>;
  const long long tid = B.id * (long long)blockDim.x + threadIdx.x;
  if (tid >= g.Nc * k::V) return;
  const long long c = tid % g.Nc;
  const int v = (int)(tid / g.Nc);
  int cx, cy, cz;
  cell_coords(g, c, cx, cy, cz);
  double x[k::NS];
#pragma unroll
  for (int s = 0; s < k::NS; ++s) {
    const int kx = s % k::n, ky = (s / k::n) % k::n, kz = s / (k::n * k::n);
    const long long q = (cx * k::n + kx) + (long long)g.X[0] * ((D >= 2 ? cy * k::n + ky : 0) +
                                                               (long long)g.X[1] * (D >= 3 ? cz * k::n + kz : 0));
    x[s] = U_cv[(long long)v * g.Nq + q];
  }
  for (int o = 0; o < k::NS; ++o) U_sp[((long long)v * k::NS + o) * g.Nc + c] = full_dot<D, P>(Kfull + (long long)o * k::NS, x, true);
}
};
template <int D, int P>
__global__ void k_cv_to_sp(Geo g, const double* __restrict__ Kfull, const double* __restrict__ U_cv,
                           double* __restrict__ U_sp) {
  CvToSp<D, P>::run(hw_blk(), g, Kfull, U_cv, U_sp);
}

}  // namespace spd
