// Viscous fluxes of the SD-ADER predictor (src/sdader_simulator.py:245-268,
// src/hydro.py:172-241), added after the element-interface Riemann solves of
// every Picard iteration and subtracted from the flux at every flux point by
// the interior kernel.  Bit-identical to the reference's NumPy path:
//
//  * ViscGrad: the primitives W at the nf flux points of every direction d
//    (interpolation of the iterate, then U -> W in the plain velocity
//    order), with both edge points replaced by the LEFT state of their
//    element interface (ML: the right-edge state of the cell on the left,
//    or the domain-boundary state of src/sd_boundary.py:32-68), stored as
//    Wfp[d]; their derivative along d at the solution points, divided by h_d,
//    stored as dWsp[d];
//  * ViscFlux: for every flux direction d and gradient direction e, dWsp[e]
//    interpolated to the flux points of d, with both edge points replaced by
//    the RIGHT state of their interface (MR: the left-edge value of the cell
//    on the right, or the boundary state); the viscous flux from Wfp[d] and
//    these gradients, times rho and nu, stored as G[d] (layout of the
//    flux-point fluxes, [v][t][j][f][cell]).
//
// Boundary states (store_BC / apply_BC of src/sd_boundary.py, applied to the
// primitive and gradient arrays as the reference does): periodic -> the
// opposite edge; reflective -> the cell's own edge with the normal-velocity
// component negated; gradfree -> the cell's own edge; ic, eq -> the stored
// initial conservative edge traces, unchanged; pressure -> the same stored
// values, which also overwrite the domain-edge point of the array itself.
#pragma once
#include "spd_kernels.cuh"

namespace spd {

template <int D, int P>
struct ViscGrad {
  static __device__ __forceinline__ void run(Blk B, const Ops& op, const Geo& g, int Teff,
                                             const double* __restrict__ Uin, int Tu, const double* tr0,
                                             const double* tr1, const double* tr2, const double* bf0,
                                             const double* bf1, const double* bf2, double* W0, double* W1,
                                             double* W2, double* __restrict__ dWsp, const double* mq0,
                                             const double* mq1, const double* mq2) {
    using k = K<D, P>;
    // well-balanced mode: the conservative equilibrium at the flux points is
    // part of the state whose primitives are taken (src/sdader_simulator.py:221-223)
    const double* meq[3] = {mq0, mq1, mq2};
    const long long tid = B.id * (long long)blockDim.x + threadIdx.x;
    if (tid >= g.Nc * Teff) return;
    const long long c = tid % g.Nc;
    const int t = (int)(tid / g.Nc);
    const int tu = (Tu == 1) ? 0 : t;
    const double* trace[3] = {tr0, tr1, tr2};
    const double* bcfix[3] = {bf0, bf1, bf2};
    double* Wfp[3] = {W0, W1, W2};
    int cx, cy, cz;
    cell_coords(g, c, cx, cy, cz);
#pragma unroll 1
    for (int d = 0; d < D; ++d) {
      const int cd = (d == 0) ? cx : (d == 1 ? cy : cz);
      const int Nd = g.N[d];
      const int b0 = g.bc[d][0], b1 = g.bc[d][1];
      const long long step = (d == 0) ? 1 : (d == 1 ? g.N[0] : (long long)g.N[0] * g.N[1]);
      const long long ntrans = g.Nc / Nd;
      const long long ct = (d == 0) ? (cy + (long long)g.N[1] * cz) : (d == 1 ? (cx + (long long)g.N[0] * cz)
                                                                              : (cx + (long long)g.N[0] * cy));
      for (int j = 0; j < k::NJ; ++j) {
        auto tr = [&](int side, int v, long long cell) -> double {
          double val = trace[d][(((long long)(side * k::V + v) * g.T + t) * k::NJ + j) * g.Nc + cell];
          if (meq[0]) val = val + meq[d][(((long long)v * k::NJ + j) * k::nf + (side ? k::nf - 1 : 0)) * g.Nc + cell];
          return val;
        };
        auto fix = [&](int side, int v) -> double {
          return bcfix[d][(((long long)side * k::V + v) * k::NJ + j) * ntrans + ct];
        };
        double Wf[k::V][k::nf];
        double u[k::V][k::n];
#pragma unroll
        for (int v = 0; v < k::V; ++v)
#pragma unroll
          for (int s = 0; s < k::n; ++s)
            u[v][s] = Uin[(((long long)v * Tu + tu) * k::NS + sp_index<D, P>(d, j, s)) * g.Nc + c];
#pragma unroll
        for (int f = 1; f < k::nf - 1; ++f) {
          double M[k::V], W[k::V];
#pragma unroll
          for (int v = 0; v < k::V; ++v) {
            M[v] = dot_dir<k::n>(op.sp_to_fp + f * k::n, u[v], d);
            if (meq[0]) M[v] = M[v] + meq[d][(((long long)v * k::NJ + j) * k::nf + f) * g.Nc + c];
          }
          prim<D>(M, W, g.gamma, 0, (double*)nullptr, g.iso != 0);
#pragma unroll
          for (int v = 0; v < k::V; ++v) Wf[v][f] = W[v];
        }
        // right edge: the cell's own right-edge state (its trace), or the
        // stored state on a "pressure" side
        {
          double M[k::V], W[k::V];
          if (cd == Nd - 1 && b1 == BC_PRESSURE) {
#pragma unroll
            for (int v = 0; v < k::V; ++v) W[v] = fix(1, v);
          } else {
#pragma unroll
            for (int v = 0; v < k::V; ++v) M[v] = tr(1, v, c);
            prim<D>(M, W, g.gamma, 0, (double*)nullptr, g.iso != 0);
          }
#pragma unroll
          for (int v = 0; v < k::V; ++v) Wf[v][k::nf - 1] = W[v];
        }
        // left edge: the right-edge state of the cell on the left, or the
        // boundary state
        {
          double M[k::V], W[k::V];
          if (cd > 0 || b0 == BC_PERIODIC || b0 == BC_REFLECTIVE || b0 == BC_GRADFREE) {
            const long long src = (cd > 0) ? c - step : (b0 == BC_PERIODIC ? c + (Nd - 1) * step : c);
            const int side = (cd > 0 || b0 == BC_PERIODIC) ? 1 : 0;
#pragma unroll
            for (int v = 0; v < k::V; ++v) M[v] = tr(side, v, src);
            prim<D>(M, W, g.gamma, 0, (double*)nullptr, g.iso != 0);
            if (cd == 0 && b0 == BC_REFLECTIVE) W[d + 1] = W[d + 1] * -1.0;
          } else {
#pragma unroll
            for (int v = 0; v < k::V; ++v) W[v] = fix(0, v);
          }
#pragma unroll
          for (int v = 0; v < k::V; ++v) Wf[v][0] = W[v];
        }
#pragma unroll
        for (int v = 0; v < k::V; ++v) {
#pragma unroll
          for (int f = 0; f < k::nf; ++f)
            Wfp[d][((((long long)v * g.T + t) * k::NJ + j) * k::nf + f) * g.Nc + c] = Wf[v][f];
        }
        const double hd = g.h[d], ihd = g.inv_h[d];
        const bool pow2 = g.h_pow2[d] != 0;
#pragma unroll
        for (int v = 0; v < k::V; ++v) {
#pragma unroll
          for (int so = 0; so < k::n; ++so) {
            const double val = pow2 ? dot_dir<k::nf>(op.dfp_h[d] + so * k::nf, Wf[v], d)
                                    : div_rcp(dot_dir<k::nf>(op.dfp_to_sp + so * k::nf, Wf[v], d), hd, ihd);
            dWsp[((((long long)d * k::V + v) * g.T + t) * k::NS + sp_index<D, P>(d, j, so)) * g.Nc + c] = val;
          }
        }
      }
    }
  }
};
template <int D, int P>
__global__ void k_visc_grad(Ops op, Geo g, int Teff, const double* __restrict__ Uin, int Tu, const double* tr0,
                            const double* tr1, const double* tr2, const double* bf0, const double* bf1,
                            const double* bf2, double* W0, double* W1, double* W2, double* __restrict__ dWsp,
                            const double* mq0, const double* mq1, const double* mq2) {
  ViscGrad<D, P>::run(hw_blk(), op, g, Teff, Uin, Tu, tr0, tr1, tr2, bf0, bf1, bf2, W0, W1, W2, dWsp, mq0, mq1, mq2);
}

template <int D, int P>
struct ViscFlux {
  static __device__ __forceinline__ void run(Blk B, const Ops& op, const Geo& g, int Teff,
                                             const double* __restrict__ dWsp, const double* W0, const double* W1,
                                             const double* W2, const double* bf0, const double* bf1,
                                             const double* bf2, double nu, double beta, double* G0, double* G1,
                                             double* G2) {
    using k = K<D, P>;
    constexpr int P_ = D + 1;
    const long long tid = B.id * (long long)blockDim.x + threadIdx.x;
    if (tid >= g.Nc * Teff) return;
    const long long c = tid % g.Nc;
    const int t = (int)(tid / g.Nc);
    const double* bcfix[3] = {bf0, bf1, bf2};
    const double* Wfp[3] = {W0, W1, W2};
    double* G[3] = {G0, G1, G2};
    int cx, cy, cz;
    cell_coords(g, c, cx, cy, cz);
#pragma unroll 1
    for (int d = 0; d < D; ++d) {
      const int cd = (d == 0) ? cx : (d == 1 ? cy : cz);
      const int Nd = g.N[d];
      const int b0 = g.bc[d][0], b1 = g.bc[d][1];
      const long long step = (d == 0) ? 1 : (d == 1 ? g.N[0] : (long long)g.N[0] * g.N[1]);
      const long long ntrans = g.Nc / Nd;
      const long long ct = (d == 0) ? (cy + (long long)g.N[1] * cz) : (d == 1 ? (cx + (long long)g.N[0] * cz)
                                                                              : (cx + (long long)g.N[0] * cy));
      const int v1 = rvel<D>(d, 0);
      for (int j = 0; j < k::NJ; ++j) {
        auto fix = [&](int side, int v) -> double {
          return bcfix[d][(((long long)side * k::V + v) * k::NJ + j) * ntrans + ct];
        };
        auto sp_val = [&](int e, int v, int s, long long cell) -> double {
          return dWsp[((((long long)e * k::V + v) * g.T + t) * k::NS + sp_index<D, P>(d, j, s)) * g.Nc + cell];
        };
        // gradients along every direction e at the flux points of d
        double gf[D][k::V][k::nf];
#pragma unroll
        for (int e = 0; e < D; ++e) {
#pragma unroll
          for (int v = 0; v < k::V; ++v) {
            double x[k::n];
#pragma unroll
            for (int s = 0; s < k::n; ++s) x[s] = sp_val(e, v, s, c);
#pragma unroll
            for (int f = 0; f < k::nf; ++f) gf[e][v][f] = dot_dir<k::n>(op.sp_to_fp + f * k::n, x, d);
            // left edge: the cell's own left-edge value (MR of its left
            // interface) unless a "pressure" side overwrote it
            if (cd == 0 && b0 == BC_PRESSURE) gf[e][v][0] = fix(0, v);
            // right edge: the left-edge value of the cell on the right, or
            // the boundary state
            double r;
            if (cd < Nd - 1 || b1 == BC_PERIODIC) {
              const long long nb = (cd < Nd - 1) ? c + step : c - (Nd - 1) * step;
              double xn[k::n];
#pragma unroll
              for (int s = 0; s < k::n; ++s) xn[s] = sp_val(e, v, s, nb);
              r = dot_dir<k::n>(op.sp_to_fp, xn, d);
            } else if (b1 == BC_REFLECTIVE || b1 == BC_GRADFREE) {
              r = gf[e][v][k::nf - 1];
              if (b1 == BC_REFLECTIVE && v == d + 1) r = r * -1.0;
            } else {
              r = fix(1, v);
            }
            gf[e][v][k::nf - 1] = r;
          }
        }
#pragma unroll
        for (int f = 0; f < k::nf; ++f) {
          double W[k::V];
#pragma unroll
          for (int v = 0; v < k::V; ++v)
            W[v] = Wfp[d][((((long long)v * g.T + t) * k::NJ + j) * k::nf + f) * g.Nc + c];
          double F[k::V];
          F[v1] = 2.0 * gf[d][v1][f] - beta * gf[d][v1][f];
          F[P_] = W[v1] * F[v1];
#pragma unroll
          for (int kk = 1; kk < D; ++kk) {
            const int vel = rvel<D>(d, kk);
            F[v1] = F[v1] - beta * gf[vel - 1][vel][f];
            F[vel] = gf[d][vel][f] + gf[vel - 1][v1][f];
            F[P_] = F[P_] + W[vel] * F[vel];
          }
          F[0] = 0.0;
#pragma unroll
          for (int v = 0; v < k::V; ++v)
            G[d][((((long long)v * g.T + t) * k::NJ + j) * k::nf + f) * g.Nc + c] = F[v] * W[0] * nu;
        }
      }
    }
  }
};
template <int D, int P>
__global__ void k_visc_flux(Ops op, Geo g, int Teff, const double* __restrict__ dWsp, const double* W0,
                            const double* W1, const double* W2, const double* bf0, const double* bf1,
                            const double* bf2, double nu, double beta, double* G0, double* G1, double* G2) {
  ViscFlux<D, P>::run(hw_blk(), op, g, Teff, dWsp, W0, W1, W2, bf0, bf1, bf2, nu, beta, G0, G1, G2);
}

}  // namespace spd
