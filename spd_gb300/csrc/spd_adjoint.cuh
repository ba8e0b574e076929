// Adjoint (vector-Jacobian product) of one SD-ADER step, hand-written for
// sm_103a.  The step is differentiated with dt, the trouble masks, the
// blending weights theta, the minmod branches and the Riemann-solver
// branches frozen at their forward values.  Linear pieces (interpolation,
// derivative, Picard sums, subcell transforms, flux divergence, boundary
// copies) are transposed directly; the pointwise nonlinear maps
// (primitives, Euler flux, LLF/HLLC, the MUSCL-Hancock half-step
// predictor) use hand-derived reverse-mode products (spd_vjp.cuh,
// predictor_vjp).  Adjoint arrays use the forward layouts
// (spd_kernels.cuh, spd_fv.cuh); suffix _a.
#pragma once
#include "spd_fv.cuh"
#include "spd_vjp.cuh"

namespace spd {

// ---------------------------------------------------------------------------
// predictor
// ---------------------------------------------------------------------------
// Adjoint of one fused interior kernel launch (k_interior), one thread per
// (cell c, time node t, direction d, transverse line j).  Input: the
// adjoint of dudt (mode 0/1) or of the flux points (mode 2).  Output: the
// line's share of the adjoint of this iteration's input U[t] (Upart[d],
// written; each point of a cell lies on exactly one line per direction)
// and the edge adjoints Ea of the line.
template <int D, int P>
__global__ void k_adj_interior(Ops op, Geo g, int mode, int Teff, const double* __restrict__ Uin, int Tu,
                               const double* __restrict__ dudt_a, const double* Ffa0, const double* Ffa1,
                               const double* Ffa2, double* Up0, double* Up1, double* Up2, double* Ea0, double* Ea1,
                               double* Ea2) {
  using k = K<D, P>;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const unsigned nc = (unsigned)g.Nc;
  if (tid >= (long long)nc * Teff * D * k::NJ) return;
  const unsigned ut = (unsigned)tid;
  const unsigned c = ut % nc;
  unsigned rest = ut / nc;
  const int j = (int)(rest % k::NJ);
  rest /= k::NJ;
  const int d = (int)(rest % D);
  const int t = (int)(rest / D);
  const int tu = (Tu == 1) ? 0 : t;
  const double* Ffa = (d == 0) ? Ffa0 : (d == 1 ? Ffa1 : Ffa2);
  double* Up = (d == 0) ? Up0 : (d == 1 ? Up1 : Up2);
  double* Ea = (d == 0) ? Ea0 : (d == 1 ? Ea1 : Ea2);
  double Fla[k::V][k::nf];
  if (mode == 2) {
#pragma unroll
    for (int v = 0; v < k::V; ++v)
#pragma unroll
      for (int f = 0; f < k::nf; ++f) Fla[v][f] = Ffa[((((long long)v * g.T + t) * k::NJ + j) * k::nf + f) * nc + c];
  } else {
    // derivative transpose: val = (sum_f dfp_to_sp[so][f] F[f]) / h; rh is
    // the correctly rounded 1/h the host stores for every active direction
    const double rh = g.inv_h[d];
#pragma unroll
    for (int v = 0; v < k::V; ++v) {
#pragma unroll
      for (int f = 0; f < k::nf; ++f) Fla[v][f] = 0.0;
#pragma unroll
      for (int so = 0; so < k::n; ++so) {
        const int s = sp_index<D, P>(d, j, so);
        const double da = dudt_a[(((long long)v * g.T + t) * k::NS + s) * nc + c] * rh;
#pragma unroll
        for (int f = 0; f < k::nf; ++f) Fla[v][f] += op.dfp_to_sp[so * k::nf + f] * da;
      }
    }
  }
  // edge flux points: adjoint of the interface fluxes
#pragma unroll
  for (int v = 0; v < k::V; ++v) {
    Ea[(((long long)(0 * k::V + v) * g.T + t) * k::NJ + j) * nc + c] = Fla[v][0];
    Ea[(((long long)(1 * k::V + v) * g.T + t) * k::NJ + j) * nc + c] = Fla[v][k::nf - 1];
  }
  // interior flux points
  double u[k::V][k::n], acc[k::V][k::n];
#pragma unroll
  for (int v = 0; v < k::V; ++v)
#pragma unroll
    for (int s = 0; s < k::n; ++s) {
      u[v][s] = Uin[(((long long)v * Tu + tu) * k::NS + sp_index<D, P>(d, j, s)) * nc + c];
      acc[v][s] = 0.0;
    }
#pragma unroll
  for (int f = 1; f < k::nf - 1; ++f) {
    double M[k::V], W[k::V], Wa[k::V], Ma[k::V];
#pragma unroll
    for (int v = 0; v < k::V; ++v) {
      M[v] = dot_dir<k::n>(op.sp_to_fp + f * k::n, u[v], d);
      Wa[v] = 0.0;
      Ma[v] = 0.0;
    }
    prim<D>(M, W, g.gamma, 0);
    double Fa[k::V];
#pragma unroll
    for (int v = 0; v < k::V; ++v) Fa[v] = Fla[v][f];
    flux_vjp_add<D>(W, Fa, Wa, g.gamma, d);
    prim_vjp_add<D>(M, Wa, Ma, g.gamma);
#pragma unroll
    for (int v = 0; v < k::V; ++v)
#pragma unroll
      for (int s = 0; s < k::n; ++s) acc[v][s] += op.sp_to_fp[f * k::n + s] * Ma[v];
  }
#pragma unroll
  for (int v = 0; v < k::V; ++v)
#pragma unroll
    for (int s = 0; s < k::n; ++s)
      Up[(((long long)v * Teff + t) * k::NS + sp_index<D, P>(d, j, s)) * nc + c] = acc[v][s];
}

// Adjoint of the element-interface Riemann fluxes of direction d: the
// interface adjoint is the sum of the edge adjoints of the cells that use
// the flux; (ML, MR) adjoints go (atomically) to the traces they came from.
template <int D, int P>
__global__ void k_adj_riemann(Geo g, int d, int Teff, int solver, const double* __restrict__ trace,
                              const double* __restrict__ bcfix, const double* __restrict__ Ea,
                              double* __restrict__ Tra) {
  using k = K<D, P>;
  const long long nI = n_iface(g, d);
  const long long total = (long long)Teff * k::NJ * nI;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= total) return;
  const long long iface = tid % nI;
  const long long r = tid / nI;
  const int j = (int)(r % k::NJ);
  const int t = (int)(r / k::NJ);
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
  const long long ntrans = g.Nc / Nd;
  const long long ct = (d == 0) ? (cy + (long long)g.N[1] * cz) : (d == 1 ? (cx + (long long)g.N[0] * cz)
                                                                            : (cx + (long long)g.N[0] * cy));
  auto tidx = [&](int side, int v, long long cell) -> long long {
    return (((long long)(side * k::V + v) * g.T + t) * k::NJ + j) * g.Nc + cell;
  };
  auto fix = [&](int side, int v) -> double {
    return bcfix[(((long long)side * k::V + v) * k::NJ + j) * ntrans + ct];
  };
  // forward inputs and where their adjoints go: trace (cell, side, negate)
  // or nowhere (a fixed boundary state)
  double ML[k::V], MR[k::V];
  long long srcL = -1, srcR = -1;
  int sideL = 1, sideR = 0;
  int fixL = 0, fixR = 0;  // boundary-state side used where a state is fixed
  bool negL = false, negR = false;
  const int b0 = g.bc[d][0], b1 = g.bc[d][1];
  double Fa[k::V];
  if (i == 0) {
    const long long c0 = cell_at(0);
    if (b0 == BC_PERIODIC) { srcL = cell_at(Nd - 1); sideL = 1; }
    else if (b0 == BC_REFLECTIVE) { srcL = c0; sideL = 0; negL = true; }
    else if (b0 == BC_GRADFREE) { srcL = c0; sideL = 0; }
    srcR = (b0 == BC_PRESSURE) ? -1 : c0;
    sideR = 0;
    fixL = 0;
    fixR = 0;
#pragma unroll
    for (int v = 0; v < k::V; ++v) Fa[v] = Ea[tidx(0, v, c0)];
  } else if (i == Nd) {
    const long long cl = cell_at(Nd - 1);
    if (b1 == BC_PERIODIC) { srcR = (b0 == BC_PRESSURE) ? -1 : cell_at(0); sideR = 0; }
    else if (b1 == BC_REFLECTIVE) { srcR = cl; sideR = 1; negR = true; }
    else if (b1 == BC_GRADFREE) { srcR = cl; sideR = 1; }
    srcL = (b1 == BC_PRESSURE) ? -1 : cl;
    sideL = 1;
    fixL = 1;
    fixR = (b1 == BC_PERIODIC) ? 0 : 1;
#pragma unroll
    for (int v = 0; v < k::V; ++v) Fa[v] = Ea[tidx(1, v, cl)];
  } else {
    srcL = cell_at(i - 1);
    srcR = cell_at(i);
#pragma unroll
    for (int v = 0; v < k::V; ++v) Fa[v] = Ea[tidx(1, v, srcL)] + Ea[tidx(0, v, srcR)];
  }
#pragma unroll
  for (int v = 0; v < k::V; ++v) {
    // values, exactly as the forward selected them
    if (srcL >= 0) {
      const double x = trace[tidx(sideL, v, srcL)];
      ML[v] = (negL && v == d + 1) ? x * -1.0 : x;
    } else {
      ML[v] = fix(fixL, v);
    }
    if (srcR >= 0) {
      const double x = trace[tidx(sideR, v, srcR)];
      MR[v] = (negR && v == d + 1) ? x * -1.0 : x;
    } else {
      MR[v] = fix(fixR, v);
    }
  }
  double MLa[k::V], MRa[k::V];
  riemann_vjp_rev<D>(solver, ML, MR, Fa, MLa, MRa, g.gamma, g.min_c2, d, false);
#pragma unroll
  for (int v = 0; v < k::V; ++v) {
    if (srcL >= 0) atomicAdd(&Tra[tidx(sideL, v, srcL)], (negL && v == d + 1) ? -MLa[v] : MLa[v]);
    if (srcR >= 0) atomicAdd(&Tra[tidx(sideR, v, srcR)], (negR && v == d + 1) ? -MRa[v] : MRa[v]);
  }
}

// Ua[t] = sum over directions of the interior partials (Upart, from
// k_adj_interior) + (edge traces)^T Tra, for cell c and node t; one thread
// per (cell, node, direction-d line j), adding in a fixed order.
template <int D, int P>
__global__ void k_adj_traces(Ops op, Geo g, int Teff, const double* __restrict__ Tra0, const double* Tra1,
                             const double* Tra2, const double* Up0, const double* Up1, const double* Up2,
                             double* __restrict__ Ua) {
  using k = K<D, P>;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const unsigned nc = (unsigned)g.Nc;
  if (tid >= (long long)nc * Teff * k::NS) return;
  const unsigned ut = (unsigned)tid;
  const unsigned c = ut % nc;
  const unsigned rest = ut / nc;
  const int s = (int)(rest % k::NS);
  const int t = (int)(rest / k::NS);
  const double* Tra[3] = {Tra0, Tra1, Tra2};
  const double* Up[3] = {Up0, Up1, Up2};
  // coordinates of point s: index along each direction and transverse line
  const int kx = s % k::n, ky = (s / k::n) % k::n, kz = s / (k::n * k::n);
#pragma unroll
  for (int v = 0; v < k::V; ++v) {
    const long long ui = (((long long)v * Teff + t) * k::NS + s) * nc + c;
    double a = Up[0][ui];
#pragma unroll
    for (int d = 1; d < D; ++d) a += Up[d][ui];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const int kd = (d == 0) ? kx : (d == 1 ? ky : kz);
      const int j = (d == 0) ? (ky + k::n * kz) : (d == 1 ? (kx + k::n * kz) : (kx + k::n * ky));
      const double l = Tra[d][(((long long)(0 * k::V + v) * g.T + t) * k::NJ + j) * nc + c];
      const double r = Tra[d][(((long long)(1 * k::V + v) * g.T + t) * k::NJ + j) * nc + c];
      a += op.sp_to_fp[kd] * l + op.sp_to_fp[(k::nf - 1) * k::n + kd] * r;
    }
    Ua[ui] = a;
  }
}

// Picard transpose: U_ader[t] = U_sp - dt * sum_p invader[t][p] dudt[p].
// Usp_a += sum_t Ua[t]; dudt_a[p] = -dt sum_t invader[t][p] Ua[t].  When
// the lower iteration is the first one (all nodes share one dudt),
// ``collapse`` sums dudt_a over p into node 0.
template <int D, int P>
__global__ void k_adj_picard(Ops op, Geo g, const double* __restrict__ dt_ptr, const double* __restrict__ Ua,
                             double* __restrict__ Usp_a, double* __restrict__ dudt_a, int collapse) {
  using k = K<D, P>;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= g.Nc * k::V * k::NS) return;
  const long long c = tid % g.Nc;
  const long long vs = tid / g.Nc;
  const int v = (int)(vs / k::NS), s = (int)(vs % k::NS);
  const double dt = *dt_ptr;
  double sum = 0.0;
  for (int t = 0; t < g.T; ++t) sum += Ua[(((long long)v * g.T + t) * k::NS + s) * g.Nc + c];
  Usp_a[((long long)v * k::NS + s) * g.Nc + c] += sum;
  double tot = 0.0;
  for (int p = 0; p < g.T; ++p) {
    double a = 0.0;
    for (int t = 0; t < g.T; ++t) a += op.invader[t * g.T + p] * Ua[(((long long)v * g.T + t) * k::NS + s) * g.Nc + c];
    a = -dt * a;
    if (collapse) tot += a;
    else dudt_a[(((long long)v * g.T + p) * k::NS + s) * g.Nc + c] = a;
  }
  if (collapse) dudt_a[(((long long)v * g.T + 0) * k::NS + s) * g.Nc + c] = tot;
}

// SD update transpose: U_new = U_sp - dt * sum_t w[t] dudt[t]:
// dudt_a[t] = -dt w[t] Usp_new_a (Usp_a keeps the identity part).
template <int D, int P>
__global__ void k_adj_sd_update(Ops op, Geo g, const double* __restrict__ dt_ptr, const double* __restrict__ Usp_a,
                                double* __restrict__ dudt_a, int Teff) {
  using k = K<D, P>;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= g.Nc * k::V * k::NS) return;
  const long long c = tid % g.Nc;
  const long long vs = tid / g.Nc;
  const int v = (int)(vs / k::NS), s = (int)(vs % k::NS);
  const double a = Usp_a[((long long)v * k::NS + s) * g.Nc + c];
  const double dt = *dt_ptr;
  double tot = 0.0;
  for (int t = 0; t < g.T; ++t) {
    const double x = -dt * op.w_tp[t] * a;
    if (Teff == 1) tot += x;
    else dudt_a[(((long long)v * g.T + t) * k::NS + s) * g.Nc + c] = x;
  }
  if (Teff == 1) dudt_a[(((long long)v * g.T + 0) * k::NS + s) * g.Nc + c] = tot;
}

// Usp_a += Ua (node 0) -- the first iteration reads U_sp directly
template <int D, int P>
__global__ void k_adj_add_first(Geo g, const double* __restrict__ Ua, double* __restrict__ Usp_a) {
  using k = K<D, P>;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= g.Nc * k::V * k::NS) return;
  Usp_a[i] += Ua[i];
}

// ---------------------------------------------------------------------------
// FV update
// ---------------------------------------------------------------------------
// Ucv_a (FV layout) = cv_to_sp^T Usp_a for every cell (cv_to_sp over the
// whole cell, Kfull[o][i])
template <int D, int P>
__global__ void k_adj_cv_to_sp(Geo g, const double* __restrict__ Kfull, const double* __restrict__ Usp_a,
                               double* __restrict__ Ucv_a) {
  using k = K<D, P>;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= g.Nc * k::V) return;
  const long long c = tid % g.Nc;
  const int v = (int)(tid / g.Nc);
  int cx, cy, cz;
  cell_coords(g, c, cx, cy, cz);
  double a[k::NS];
#pragma unroll
  for (int o = 0; o < k::NS; ++o) a[o] = Usp_a[((long long)v * k::NS + o) * g.Nc + c];
  for (int in = 0; in < k::NS; ++in) {
    double s = 0.0;
#pragma unroll
    for (int o = 0; o < k::NS; ++o) s += Kfull[(long long)o * k::NS + in] * a[o];
    const int kx = in % k::n, ky = (in / k::n) % k::n, kz = in / (k::n * k::n);
    const long long q = (cx * k::n + kx) + (long long)g.X[0] * ((D >= 2 ? cy * k::n + ky : 0) +
                                                               (long long)g.X[1] * (D >= 3 ? cz * k::n + kz : 0));
    Ucv_a[(long long)v * g.Nq + q] = s;
  }
}

// Usp_a += sp_to_cv^T Ucv_a
template <int D, int P>
__global__ void k_adj_sp_to_cv(Geo g, const double* __restrict__ Kfull, const double* __restrict__ Ucv_a,
                               double* __restrict__ Usp_a) {
  using k = K<D, P>;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= g.Nc * k::V) return;
  const long long c = tid % g.Nc;
  const int v = (int)(tid / g.Nc);
  int cx, cy, cz;
  cell_coords(g, c, cx, cy, cz);
  double a[k::NS];
#pragma unroll
  for (int o = 0; o < k::NS; ++o) {
    const int kx = o % k::n, ky = (o / k::n) % k::n, kz = o / (k::n * k::n);
    const long long q = (cx * k::n + kx) + (long long)g.X[0] * ((D >= 2 ? cy * k::n + ky : 0) +
                                                               (long long)g.X[1] * (D >= 3 ? cz * k::n + kz : 0));
    a[o] = Ucv_a[(long long)v * g.Nq + q];
  }
  for (int in = 0; in < k::NS; ++in) {
    double s = 0.0;
#pragma unroll
    for (int o = 0; o < k::NS; ++o) s += Kfull[(long long)o * k::NS + in] * a[o];
    Usp_a[((long long)v * k::NS + in) * g.Nc + c] += s;
  }
}

// Transpose of k_integrate_faces: F_HO_a (faces of node t) -> Ffp_a
template <int D, int P>
__global__ void k_adj_integrate_faces(Ops op, Geo g, int d, const double* __restrict__ FHa,
                                      double* __restrict__ Ffa) {
  using k = K<D, P>;
  const long long total = g.Nc * g.T * k::nf;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= total) return;
  const long long c = tid % g.Nc;
  const long long r = tid / g.Nc;
  const int f = (int)(r % k::nf);
  const int t = (int)(r / k::nf);
  int cx, cy, cz;
  cell_coords(g, c, cx, cy, cz);
  const int cd = (d == 0) ? cx : (d == 1 ? cy : cz);
  const bool used = !(f == k::nf - 1 && cd != g.N[d] - 1);
  const int fd = (f == k::nf - 1) ? g.N[d] * k::n : cd * k::n + f;
  const int FX = g.X[0] + (d == 0), FY = g.X[1] + (d == 1);
  const long long nface = (long long)FX * FY * (g.X[2] + (d == 2));
  int o0 = -1, o1 = -1;
  for (int e = 0; e < D; ++e) {
    if (e == d) continue;
    if (o0 < 0) o0 = e; else o1 = e;
  }
  for (int v = 0; v < k::V; ++v) {
    double G[k::NJ];
    if (!used) {
#pragma unroll
      for (int jj = 0; jj < k::NJ; ++jj) G[jj] = 0.0;
    } else {
      for (int jj = 0; jj < k::NJ; ++jj) {
        const int a = jj % k::n, b = jj / k::n;
        int fc[3] = {0, 0, 0};
        fc[d] = fd;
        const int cc[3] = {cx, cy, cz};
        if (o0 >= 0) fc[o0] = cc[o0] * k::n + a;
        if (o1 >= 0) fc[o1] = cc[o1] * k::n + b;
        const long long fid = fc[0] + (long long)FX * (fc[1] + (long long)FY * fc[2]);
        G[jj] = FHa[((long long)t * k::V + v) * nface + fid];
      }
      if (D == 3) {  // transpose of the second (o1) averaging
        double G1[k::NJ];
#pragma unroll
        for (int a = 0; a < k::n; ++a)
#pragma unroll
          for (int b = 0; b < k::n; ++b) {
            double s = 0.0;
#pragma unroll
            for (int bo = 0; bo < k::n; ++bo) s += op.sp_to_cv[bo * k::n + b] * G[a + k::n * bo];
            G1[a + k::n * b] = s;
          }
#pragma unroll
        for (int jj = 0; jj < k::NJ; ++jj) G[jj] = G1[jj];
      }
      if (D >= 2) {  // transpose of the first (o0) averaging
        double G0[k::NJ];
#pragma unroll
        for (int b = 0; b < k::NJ / k::n; ++b)
#pragma unroll
          for (int a = 0; a < k::n; ++a) {
            double s = 0.0;
#pragma unroll
            for (int ao = 0; ao < k::n; ++ao) s += op.sp_to_cv[ao * k::n + a] * G[ao + k::n * b];
            G0[a + k::n * b] = s;
          }
#pragma unroll
        for (int jj = 0; jj < k::NJ; ++jj) G[jj] = G0[jj];
      }
    }
#pragma unroll
    for (int jj = 0; jj < k::NJ; ++jj)
      Ffa[((((long long)v * g.T + t) * k::NJ + jj) * k::nf + f) * g.Nc + c] = G[jj];
  }
}

// Flux-divergence transpose of substep i and the split of the corrected
// flux adjoint: F_a[face] = dt_i (U_new_a[right]/dx[right] - U_new_a[left]/dx[left]),
// F_HO_a += (1 - theta) F_a (or F_a without limiting), and Fb_a = theta F_a
// (godunov: F_a) on the faces whose fallback flux was used.
template <int D>
__global__ void k_adj_faces(Geo g, FvGeo fg, int d, const double* __restrict__ dt_ptr, double w_i, int fb,
                            int godunov, const double* __restrict__ aff, const double* __restrict__ Unew_a,
                            double* __restrict__ FHa_i, double* __restrict__ Fba) {
  constexpr int V = D + 2;
  const long long nf = n_faces(g, d);
  const long long fidx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (fidx >= nf) return;
  const int FX = g.X[0] + (d == 0), FY = g.X[1] + (d == 1);
  int f[3];
  f[0] = (int)(fidx % FX);
  long long r = fidx / FX;
  f[1] = (int)(r % FY);
  f[2] = (int)(r / FY);
  const double dti = *dt_ptr * w_i;
  const int Xd = g.X[d];
  const double a = fb ? aff[fidx] : 0.0;
  const bool use_fb = fb && (godunov || a != 0.0);
  for (int v = 0; v < V; ++v) {
    double Fa = 0.0;
    int q[3] = {f[0], f[1], f[2]};
    // quotients by the subcell widths from their correctly rounded
    // reciprocals (div_rcp: the IEEE quotient's bits in 3 FP64 operations)
    if (f[d] >= 1) {  // right face of subcell f-1
      q[d] = f[d] - 1;
      const long long qi = q[0] + (long long)g.X[0] * (q[1] + (long long)g.X[1] * q[2]);
      Fa += div_rcp(-dti * Unew_a[(long long)v * g.Nq + qi], fg.dx[d][q[d]], fg.rdx[d][q[d]]);
    }
    if (f[d] < Xd) {  // left face of subcell f
      q[d] = f[d];
      const long long qi = q[0] + (long long)g.X[0] * (q[1] + (long long)g.X[1] * q[2]);
      Fa += div_rcp(dti * Unew_a[(long long)v * g.Nq + qi], fg.dx[d][q[d]], fg.rdx[d][q[d]]);
    }
    double ho = Fa, fbv = 0.0;
    if (use_fb) {
      if (godunov) { ho = 0.0; fbv = Fa; }
      else { ho = (1.0 - a) * Fa; fbv = a * Fa; }
    }
    FHa_i[(long long)v * nf + fidx] += ho;
    if (fb) Fba[(long long)v * nf + fidx] = fbv;
  }
}

// limiter transpose with the forward branch: returns (SL_a, SR_a).  At a
// kink of |x| the derivative taken is 0 (torch.abs's subgradient).
__device__ __forceinline__ double sign0(double x) { return (x > 0.0) ? 1.0 : ((x < 0.0) ? -1.0 : 0.0); }
__device__ __forceinline__ void limiter_vjp(int limiter, double SL, double SR, double hl, double hr, double hm,
                                            double a, double& SLa, double& SRa) {
  SLa = 0.0;
  SRa = 0.0;
  if (limiter == LIM_MINMOD) {
    const double ratio = SR / SL;
    if (ratio < 1.0) {
      if (ratio > 0.0) SRa = a;  // ratio * SL = SR
    } else {
      SLa = a;                   // ratio >= 1 or NaN: SL
    }
    return;
  }
  if (!(SL * SR >= 0.0)) return;
  const double dUC = (hl * SL + hr * SR) / (hl + hr);
  const double q1 = 2.0 * SL * hl / hm, q2 = 2.0 * SR * hr / hm;
  const double c1 = fabs(q1), c2 = fabs(q2), c3 = fabs(dUC);
  const double sg = sign0(dUC);
  // slope = sg * min(min(c1, c2), c3): the derivative weight of each
  // argument of a minimum is 1 / 0 by the comparison, 1/2 each at a tie
  const double m12 = np_min(c1, c2);
  double wm, w3;
  if (m12 == c3) { wm = 0.5; w3 = 0.5; }
  else if (m12 < c3 || m12 != m12) { wm = 1.0; w3 = 0.0; }
  else { wm = 0.0; w3 = 1.0; }
  double w1, w2;
  if (c1 == c2) { w1 = 0.5 * wm; w2 = 0.5 * wm; }
  else if (c1 < c2 || c1 != c1) { w1 = wm; w2 = 0.0; }
  else { w1 = 0.0; w2 = wm; }
  const double dq1 = sign0(q1) * 2.0 * hl / hm, dq2 = sign0(q2) * 2.0 * hr / hm;
  const double s3 = sign0(dUC);
  SLa = sg * (w1 * dq1 + w3 * s3 * hl / (hl + hr)) * a;
  SRa = sg * (w2 * dq2 + w3 * s3 * hr / (hl + hr)) * a;
}

// Limited gradients of extended cell e in every direction (the forward's
// k_muscl_cells arithmetic: values and branches as in the recorded step).
template <int D>
__device__ __forceinline__ void muscl_cell_forward(const Geo& g, const FvGeo& fg, int limiter, long long e,
                                                   const double* __restrict__ W_ext, double* W, double (*SLs)[D + 2],
                                                   double (*SRs)[D + 2], double (*dMh)[D + 2]) {
  constexpr int V = D + 2;
  int ec[3];
  e_coords(g, e, ec[0], ec[1], ec[2]);
  for (int v = 0; v < V; ++v) W[v] = W_ext[(long long)v * g.Nqe + e];
  for (int dd = 0; dd < D; ++dd) {
    const long long st = ext_stride(g, dd);
    const int cdd = ec[dd];
    const double hl = fg.hcv[dd][cdd - 1], hr = fg.hcv[dd][cdd], hm = fg.hfp[dd][cdd];
    const double rhl = fg.rhcv[dd][cdd - 1], rhr = fg.rhcv[dd][cdd];
    for (int v = 0; v < V; ++v) {
      const double* M = W_ext + (long long)v * g.Nqe;
      const double SL = div_rcp(M[e] - M[e - st], hl, rhl);
      const double SR = div_rcp(M[e + st] - M[e], hr, rhr);
      SLs[dd][v] = SL;
      SRs[dd][v] = SR;
      dMh[dd][v] = (limiter == LIM_MINMOD) ? minmod(SL, SR) : moncen(SL, SR, hl, hr, hm);
    }
  }
}

// Transpose of the half-step prediction pr = W + 0.5 dti dtW(W, dMh)
// (k_muscl_cells; the pressure component of dtW is multiplied by 0):
// in_a[0..V) += dpr/dW^T pra, in_a[V + dd V + v] += dpr/d(dMh[dd][v])^T pra.
template <int D>
SPD_FN void predictor_vjp(const double* W, const double (*dMh)[D + 2], double dti, const double* pra,
                          double* in_a) {
  constexpr int V = D + 2, P_ = D + 1;
  double dta[V];
  for (int v = 0; v < V; ++v) {
    in_a[v] += pra[v];
    dta[v] = 0.5 * dti * pra[v];
  }
  dta[P_] = 0.0;
  const double rw0 = 1.0 / W[0];
  for (int dd = 0; dd < D; ++dd) {
    const int vel = dd + 1;
    double* dma = in_a + V + dd * V;
    // dtW[0] -= W[vel] dm[0] + W[0] dm[vel]
    in_a[vel] -= dta[0] * dMh[dd][0];
    dma[0] -= dta[0] * W[vel];
    in_a[0] -= dta[0] * dMh[dd][vel];
    dma[vel] -= dta[0] * W[0];
    // dtW[vel] -= W[vel] dm[vel] + dm[P] / W[0]
    in_a[vel] -= dta[vel] * dMh[dd][vel];
    dma[vel] -= dta[vel] * W[vel];
    dma[P_] -= dta[vel] * rw0;
    in_a[0] += dta[vel] * dMh[dd][P_] * rw0 * rw0;
    // dtW[v2] -= W[vel] dm[v2], v2 = 2..D
    for (int v2 = 2; v2 <= D; ++v2) {
      in_a[vel] -= dta[v2] * dMh[dd][v2];
      dma[v2] -= dta[v2] * W[vel];
    }
  }
}

// MUSCL-Hancock adjoint, phase 1: on every face of direction d whose
// fallback flux was used, the Riemann VJP of Fb_a onto the two
// reconstructed states, FA[side][v][face] (side 0 = left state).  The
// states are the recorded forward's predictions and slope terms
// (Mpred [v][e], S [dir][v][e]; valid on the cells of used faces).
//
// The used faces and the cells next to them are compacted into index lists
// first (warp ballot): an FP64 warp instruction costs the same with 1 or 32
// active lanes, so the VJPs run on full warps over the lists.
template <int D>
__global__ void k_adj_used_faces(Geo g, int d, int godunov, const double* __restrict__ aff,
                                 long long* __restrict__ list, unsigned long long* __restrict__ count) {
  const long long nf = n_faces(g, d);
  const long long fidx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const bool used = fidx < nf && (godunov || aff[fidx] != 0.0);
  warp_append(used, fidx, list, count);
}

template <int D>
__device__ __forceinline__ void adj_muscl_riemann_face(const Geo& g, int d, int solver, long long fidx,
                                                       const double* __restrict__ Mpred,
                                                       const double* __restrict__ S, const double* __restrict__ Fba,
                                                       double* __restrict__ FA) {
  constexpr int V = D + 2;
  const long long nf = n_faces(g, d);
  const int FX = g.X[0] + (d == 0), FY = g.X[1] + (d == 1);
  int f[3];
  f[0] = (int)(fidx % FX);
  long long r = fidx / FX;
  f[1] = (int)(r % FY);
  f[2] = (int)(r / FY);
  int e1c[3];
  for (int kk = 0; kk < 3; ++kk) e1c[kk] = (kk < D) ? f[kk] + NGH : 0;
  e1c[d] = f[d] + 1;
  const long long e1 = e1c[0] + (long long)g.Xe[0] * (e1c[1] + (long long)g.Xe[1] * e1c[2]);
  const long long e2 = e1 + ext_stride(g, d);
  double M[2][V];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    M[0][v] = Mpred[(long long)v * g.Nqe + e1] + S[((long long)d * V + v) * g.Nqe + e1];
    M[1][v] = Mpred[(long long)v * g.Nqe + e2] - S[((long long)d * V + v) * g.Nqe + e2];
  }
  double Fa[V], MLa[V], MRa[V];
  for (int v = 0; v < V; ++v) Fa[v] = Fba[(long long)v * nf + fidx];
  riemann_vjp_rev<D>(solver, M[0], M[1], Fa, MLa, MRa, g.gamma, g.min_c2, d, true);
  for (int v = 0; v < V; ++v) {
    FA[(long long)v * nf + fidx] = MLa[v];
    FA[(long long)(V + v) * nf + fidx] = MRa[v];
  }
}

template <int D>
__global__ void k_adj_muscl_riemann(Geo g, int d, int solver, const long long* __restrict__ list,
                                    const unsigned long long* __restrict__ count, const double* __restrict__ Mpred,
                                    const double* __restrict__ S, const double* __restrict__ Fba,
                                    double* __restrict__ FA) {
  const unsigned long long cnt = *count;
  for (unsigned long long idx = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; idx < cnt;
       idx += (unsigned long long)gridDim.x * blockDim.x)
    adj_muscl_riemann_face<D>(g, d, solver, list[idx], Mpred, S, Fba, FA);
}

// whether extended cell e borders a used face (its state and slopes fed a
// fallback flux)
template <int D>
__device__ __forceinline__ bool borders_used_face(const Geo& g, int godunov, const double* const* AF, long long e) {
  int ec[3];
  e_coords(g, e, ec[0], ec[1], ec[2]);
  for (int dd = 0; dd < D; ++dd) {
    bool inside = true;
    int fc[3] = {0, 0, 0};
    for (int o = 0; o < D; ++o) {
      if (o == dd) continue;
      fc[o] = ec[o] - NGH;
      inside = inside && fc[o] >= 0 && fc[o] < g.X[o];
    }
    if (!inside) continue;
    for (int k = 0; k < 2; ++k) {
      fc[dd] = ec[dd] - 1 - k;
      if (fc[dd] < 0 || fc[dd] > g.X[dd]) continue;
      if (godunov || AF[dd][face_id(g, dd, fc[0], fc[1], fc[2])] != 0.0) return true;
    }
  }
  return false;
}

template <int D>
__global__ void k_adj_used_cells(Geo g, int godunov, const double* aff0, const double* aff1, const double* aff2,
                                 long long* __restrict__ list, unsigned long long* __restrict__ count) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const double* AF[3] = {aff0, aff1, aff2};
  const bool used = e < g.Nqe && borders_used_face<D>(g, godunov, AF, e);
  warp_append(used, e, list, count);
}

// Phase 2, one thread per listed extended cell e (the cells bordering a
// used face; W_a and LA are zero elsewhere): gathers (in a fixed order) the
// adjoints of its predicted state and slopes from the used faces it
// borders, takes them back through the prediction and the limiter, writes
// W_a(e) = the part that lands on W(e) itself and LA[dd][0|1][v](e) =
// SL_a / hl, SR_a / hr (the parts that land on W(e - st) and W(e + st)).
template <int D>
__device__ __forceinline__ void adj_muscl_cell(const Geo& g, const FvGeo& fg, int limiter, int godunov,
                                               const double* __restrict__ dt_ptr, double w_i, const double* aff0,
                                               const double* aff1, const double* aff2, const double* FA0,
                                               const double* FA1, const double* FA2,
                                               const double* __restrict__ W_ext, long long e,
                                               double* __restrict__ W_a, double* __restrict__ LA) {
  constexpr int V = D + 2, NT = V * (1 + D);
  const double* AF[3] = {aff0, aff1, aff2};
  const double* FA[3] = {FA0, FA1, FA2};
  int ec[3];
  e_coords(g, e, ec[0], ec[1], ec[2]);
  double Mpa[V], Sa[D][V];
  for (int v = 0; v < V; ++v) Mpa[v] = 0.0;
  bool any = false;
  for (int dd = 0; dd < D; ++dd) {
    for (int v = 0; v < V; ++v) Sa[dd][v] = 0.0;
    bool inside = true;
    int fc[3] = {0, 0, 0};
    for (int o = 0; o < D; ++o) {
      if (o == dd) continue;
      fc[o] = ec[o] - NGH;
      inside = inside && fc[o] >= 0 && fc[o] < g.X[o];
    }
    if (!inside) continue;
    const long long nf = n_faces(g, dd);
    for (int k = 0; k < 2; ++k) {
      // k = 0: the face on the right of e (e is its left state);
      // k = 1: the face on the left of e (e is its right state)
      fc[dd] = ec[dd] - 1 - k;
      if (fc[dd] < 0 || fc[dd] > g.X[dd]) continue;
      const long long fidx = face_id(g, dd, fc[0], fc[1], fc[2]);
      if (!(godunov || AF[dd][fidx] != 0.0)) continue;
      any = true;
      for (int v = 0; v < V; ++v) {
        const double a = FA[dd][(long long)(k * V + v) * nf + fidx];
        Mpa[v] += a;
        Sa[dd][v] += (k == 0) ? a : -a;
      }
    }
  }
  if (!any) {
    for (int v = 0; v < V; ++v) W_a[(long long)v * g.Nqe + e] = 0.0;
    for (int dd = 0; dd < D; ++dd)
      for (int k = 0; k < 2; ++k)
        for (int v = 0; v < V; ++v) LA[((long long)(dd * 2 + k) * V + v) * g.Nqe + e] = 0.0;
    return;
  }
  const double dti = *dt_ptr * w_i;
  double W[V], SLs[D][V], SRs[D][V], dMh[D][V];
  muscl_cell_forward<D>(g, fg, limiter, e, W_ext, W, SLs, SRs, dMh);
  double in_a[NT];
  for (int i2 = 0; i2 < NT; ++i2) in_a[i2] = 0.0;
  predictor_vjp<D>(W, dMh, dti, Mpa, in_a);
  for (int dd = 0; dd < D; ++dd) {
    const double hm = fg.hfp[dd][ec[dd]];
    for (int v = 0; v < V; ++v) in_a[V + dd * V + v] += Sa[dd][v] * 0.5 * hm;
  }
  double own[V];
  for (int v = 0; v < V; ++v) own[v] = in_a[v];
  for (int dd = 0; dd < D; ++dd) {
    const int cdd = ec[dd];
    const double hl = fg.hcv[dd][cdd - 1], hr = fg.hcv[dd][cdd], hm = fg.hfp[dd][cdd];
    for (int v = 0; v < V; ++v) {
      double SLa, SRa;
      limiter_vjp(limiter, SLs[dd][v], SRs[dd][v], hl, hr, hm, in_a[V + dd * V + v], SLa, SRa);
      const double l = SLa * fg.rhcv[dd][cdd - 1], rr = SRa * fg.rhcv[dd][cdd];
      // SL = (W(e) - W(e-st)) / hl ; SR = (W(e+st) - W(e)) / hr
      own[v] = own[v] + l - rr;
      LA[((long long)(dd * 2 + 0) * V + v) * g.Nqe + e] = l;
      LA[((long long)(dd * 2 + 1) * V + v) * g.Nqe + e] = rr;
    }
  }
  for (int v = 0; v < V; ++v) W_a[(long long)v * g.Nqe + e] = own[v];
}

template <int D>
__global__ void k_adj_muscl_cells(Geo g, FvGeo fg, int limiter, int godunov, const double* __restrict__ dt_ptr,
                                  double w_i, const double* aff0, const double* aff1, const double* aff2,
                                  const double* FA0, const double* FA1, const double* FA2,
                                  const double* __restrict__ W_ext, const long long* __restrict__ list,
                                  const unsigned long long* __restrict__ count, double* __restrict__ W_a,
                                  double* __restrict__ LA) {
  const unsigned long long cnt = *count;
  for (unsigned long long idx = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; idx < cnt;
       idx += (unsigned long long)gridDim.x * blockDim.x)
    adj_muscl_cell<D>(g, fg, limiter, godunov, dt_ptr, w_i, aff0, aff1, aff2, FA0, FA1, FA2, W_ext, list[idx], W_a,
                      LA);
}

// Phase 3: W_a(e) += sum over directions of -SL_a/hl of e+st and +SR_a/hr
// of e-st (fixed order, no atomics).
template <int D>
__global__ void k_adj_muscl_gather(Geo g, const double* __restrict__ LA, double* __restrict__ W_a) {
  constexpr int V = D + 2;
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= g.Nqe) return;
  int ec[3];
  e_coords(g, e, ec[0], ec[1], ec[2]);
  for (int v = 0; v < V; ++v) {
    double acc = W_a[(long long)v * g.Nqe + e];
    for (int dd = 0; dd < D; ++dd) {
      const long long st = ext_stride(g, dd);
      if (ec[dd] + 1 < g.Xe[dd]) acc = acc - LA[((long long)(dd * 2 + 0) * V + v) * g.Nqe + e + st];
      if (ec[dd] >= 1) acc = acc + LA[((long long)(dd * 2 + 1) * V + v) * g.Nqe + e - st];
    }
    W_a[(long long)v * g.Nqe + e] = acc;
  }
}

// Transpose of one side of one direction's ghost fill (all = true form):
// the adjoint of each ghost value goes to the cell it was copied from
// (sign-flipped for the normal velocity at reflective sides) and the ghost
// adjoint is cleared.  Launched for the directions in reverse order, one
// side at a time (both sides may share a source cell on tiny grids).
template <int D>
__global__ void k_adj_ghost(Geo g, int d, int side, double* __restrict__ W_a) {
  constexpr int V = D + 2;
  const int o0 = (d == 0) ? 1 : 0;
  const int o1 = (d == 2) ? 1 : 2;
  const long long nother = (long long)g.Xe[o0] * g.Xe[o1];
  const long long total = (long long)V * NGH * nother;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= total) return;
  const long long other = tid % nother;
  long long r = tid / nother;
  const int gi = (int)(r % NGH);
  const int v = (int)(r / NGH);
  const int a = (int)(other % g.Xe[o0]);
  const int b = (int)(other / g.Xe[o0]);
  const int Xd = g.X[d];
  const int kind = g.bc[d][side];
  auto ext_index = [&](int e) -> long long {
    int c[3];
    c[d] = e;
    c[o0] = a;
    c[o1] = b;
    return c[0] + (long long)g.Xe[0] * (c[1] + (long long)g.Xe[1] * c[2]);
  };
  const int dst = (side == 0) ? gi : Xd + NGH + gi;
  const long long di = (long long)v * g.Nqe + ext_index(dst);
  const double ga = W_a[di];
  if (ga == 0.0) return;
  int src = -1;
  if (kind == BC_PERIODIC) src = (side == 0) ? Xd + gi : NGH + gi;
  else if (kind == BC_REFLECTIVE || kind == BC_GRADFREE) src = (side == 0) ? NGH + gi : Xd + gi;
  W_a[di] = 0.0;
  if (src < 0) return;  // fixed boundary state: no dependence on the solution
  const double val = (kind == BC_REFLECTIVE && v == d + 1) ? -ga : ga;
  // within one side every ghost has its own source cell
  W_a[(long long)v * g.Nqe + ext_index(src)] += val;
}

// Ucv_a(i) = U_new_a + prim^T(W_a) for the active subcells; clears W_a.
template <int D>
__global__ void k_adj_prim_cv(Geo g, const double* __restrict__ U_cv, const double* __restrict__ Unew_a,
                              double* __restrict__ W_a, double* __restrict__ Ucv_a) {
  constexpr int V = D + 2;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= g.Nq) return;
  int ix, iy, iz;
  q_coords(g, q, ix, iy, iz);
  const long long e = ext_of<D>(g, ix, iy, iz);
  double U[V], Wa[V], Ua[V];
  bool any = false;
#pragma unroll
  for (int v = 0; v < V; ++v) {
    U[v] = U_cv[(long long)v * g.Nq + q];
    Wa[v] = W_a[(long long)v * g.Nqe + e];
    W_a[(long long)v * g.Nqe + e] = 0.0;
    any = any || (Wa[v] != 0.0);
  }
  if (any) {
#pragma unroll
    for (int v = 0; v < V; ++v) Ua[v] = 0.0;
    prim_vjp_add<D>(U, Wa, Ua, g.gamma);
  }
#pragma unroll
  for (int v = 0; v < V; ++v)
    Ucv_a[(long long)v * g.Nq + q] = Unew_a[(long long)v * g.Nq + q] + (any ? Ua[v] : 0.0);
}

// W_old with ghosts for the adjoint's recompute of the fallback fluxes
template <int D>
__global__ void k_prim_ext(Geo g, const double* __restrict__ U_cv, double* __restrict__ W_ext) {
  constexpr int V = D + 2;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= g.Nq) return;
  int ix, iy, iz;
  q_coords(g, q, ix, iy, iz);
  const long long e = ext_of<D>(g, ix, iy, iz);
  double u[V], W[V];
#pragma unroll
  for (int v = 0; v < V; ++v) u[v] = U_cv[(long long)v * g.Nq + q];
  prim<D>(u, W, g.gamma, 0);
#pragma unroll
  for (int v = 0; v < V; ++v) W_ext[(long long)v * g.Nqe + e] = W[v];
}

}  // namespace spd
