// Device-side building blocks of the SD-ADER step: Euler thermodynamics,
// the LLF / HLLC / low-Mach HLLC Riemann solvers and the fixed-order
// contractions.  Every routine reproduces the operation order of the
// reference's NumPy expressions (file:line cited per function) so that the
// FP64 results are bit-identical to it; this file must be compiled with
// --fmad=false so that no a*b+c is fused.
#pragma once
#include <cstdint>
#include <cmath>

namespace spd {


constexpr int MAXN = 5;   // p <= 4
constexpr int MAXNF = 6;
constexpr int MAXT = 6;   // m <= 5
constexpr int NGH = 2;    // subcell ghost layers (Nghc)

enum Riemann : int { RS_LLF = 0, RS_HLLC = 1, RS_LHLLC = 2 };
enum Limiter : int { LIM_MINMOD = 0, LIM_MONCEN = 1 };
enum BcKind : int { BC_PERIODIC = 0, BC_REFLECTIVE = 1, BC_GRADFREE = 2, BC_IC = 3, BC_EQ = 4, BC_PRESSURE = 5 };

// NumPy's maximum / minimum: NaN in either argument propagates.
__device__ __forceinline__ double np_max(double a, double b) { return (a >= b || a != a) ? a : b; }
__device__ __forceinline__ double np_min(double a, double b) { return (a <= b || a != a) ? a : b; }

// Velocity index k (0-based) of the rotated frame used for direction idim:
// np.roll(vels, -idim) (src/sdader_simulator.py:219).
template <int D>
__device__ __forceinline__ int rvel(int idim, int k) { return 1 + (idim + k) % D; }

// U -> W (src/hydro.py:48-86); the kinetic term sums in the order of the
// velocity list, which is the rotated list inside the Riemann wrapper
// (src/riemann_solver.py:10-29) and the plain list elsewhere.
template <int D>
__device__ __forceinline__ void prim(const double* U, double* W, double gamma, int idim_order) {
  constexpr int P_ = D + 1;
  W[0] = U[0];
  double K = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const int v = rvel<D>(idim_order, k);
    W[v] = U[v] / U[0];
    const double w2 = W[v] * W[v];
    K = (k == 0) ? w2 : K + w2;
  }
  K = K * (0.5 * U[0]);
  W[P_] = (gamma - 1.0) * (U[P_] - K);
}

// W -> U (src/hydro.py:88-125).
template <int D>
__device__ __forceinline__ void cons(const double* W, double* U, double gamma, int idim_order) {
  constexpr int P_ = D + 1;
  U[0] = W[0];
  double K = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const int v = rvel<D>(idim_order, k);
    U[v] = W[v] * W[0];
    const double w2 = W[v] * W[v];
    K = (k == 0) ? w2 : K + w2;
  }
  K = K * (0.5 * W[0]);
  U[P_] = W[P_] / (gamma - 1.0) + K;
}

// Euler flux in the rotated frame of direction idim (src/hydro.py:127-170).
template <int D>
__device__ __forceinline__ void flux(const double* W, double* F, double gamma, int idim) {
  constexpr int P_ = D + 1;
  const int v1 = rvel<D>(idim, 0);
  double K = 0.0, m = 0.0;
#pragma unroll
  for (int k = D - 1; k >= 0; --k) {
    const int v = rvel<D>(idim, k);
    m = W[0] * W[v];
    const double mv = m * W[v];
    K = (k == D - 1) ? mv : K + mv;
    F[v] = m * W[v1];
  }
  const double E = W[P_] / (gamma - 1.0) + 0.5 * K;
  F[0] = m;
  F[v1] = m * W[v1] + W[P_];
  F[P_] = W[v1] * (E + W[P_]);
}

// Sound speed with floor (src/hydro.py:3-46).
__device__ __forceinline__ double sound_speed(double P, double rho, double gamma, double min_c2) {
  double c2 = gamma * P / rho;
  c2 = (c2 > min_c2) ? c2 : min_c2;
  return sqrt(c2);
}

// LLF (src/riemann_solver.py:31-65).
template <int D>
__device__ __forceinline__ void llf(const double* WL, const double* WR, const double* UL, const double* UR,
                                    double* F, double gamma, double min_c2, int idim) {
  constexpr int V = D + 2, P_ = D + 1;
  const int v1 = rvel<D>(idim, 0);
  double FL[V], FR[V];
  flux<D>(WL, FL, gamma, idim);
  flux<D>(WR, FR, gamma, idim);
  const double cL = sound_speed(WL[P_], WL[0], gamma, min_c2) + fabs(WL[v1]);
  const double cR = sound_speed(WR[P_], WR[0], gamma, min_c2) + fabs(WR[v1]);
  const double cmax = (cL > cR) ? cL : cR;
  const double hc = 0.5 * cmax;
#pragma unroll
  for (int v = 0; v < V; ++v) F[v] = 0.5 * (FR[v] + FL[v]) - hc * (UR[v] - UL[v]);
}

// HLLC (src/riemann_solver.py:67-145) and its low-Mach variant (:147-212).
// Only the branch the reference's np.where chain selects is evaluated.
template <int D>
__device__ __forceinline__ void hllc(const double* WL, const double* WR, const double* UL, const double* UR,
                                     double* F, double gamma, double min_c2, int idim, bool low_mach) {
  constexpr int P_ = D + 1;
  const int v1 = rvel<D>(idim, 0);
  const double cL = sound_speed(WL[P_], WL[0], gamma, min_c2) + fabs(WL[v1]);
  const double cR = sound_speed(WR[P_], WR[0], gamma, min_c2) + fabs(WR[v1]);
  const double cmax = (cL > cR) ? cL : cR;
  const double vL = WL[v1], vR = WR[v1];
  const double sL = ((vL < vR) ? vL : vR) - cmax;
  const double sR = ((vL > vR) ? vL : vR) + cmax;
  const double rcL = WL[0] * (vL - sL);
  const double rcR = WR[0] * (sR - vR);
  const double den = rcR + rcL;
  const double vstar = (rcR * vR + rcL * vL + (WL[P_] - WR[P_])) / den;
  double Pstar;
  if (low_mach) {
    const double mx = np_max(fabs(vL), fabs(vR)) / cmax;
    const double Mach = np_min(1.0, mx);
    const double phi = Mach * (2.0 - Mach);
    Pstar = (rcR * WL[P_] + rcL * WR[P_] + phi * rcL * rcR * (vL - vR)) / den;
  } else {
    Pstar = (rcR * WL[P_] + rcL * WR[P_] + rcL * rcR * (vL - vR)) / den;
  }
  double r, vg, Pg, e;
  if (sL > 0) {
    r = WL[0]; vg = vL; Pg = WL[P_]; e = UL[P_];
  } else if (vstar > 0) {
    const double d = sL - vstar;
    r = WL[0] * (sL - vL) / d;
    e = ((sL - vL) * UL[P_] - WL[P_] * vL + Pstar * vstar) / d;
    vg = vstar; Pg = Pstar;
  } else if (sR > 0) {
    const double d = sR - vstar;
    r = WR[0] * (sR - vR) / d;
    e = ((sR - vR) * UR[P_] - WR[P_] * vR + Pstar * vstar) / d;
    vg = vstar; Pg = Pstar;
  } else {
    r = WR[0]; vg = vR; Pg = WR[P_]; e = UR[P_];
  }
  F[0] = r * vg;
  F[v1] = F[0] * vg + Pg;
  F[P_] = vg * (e + Pg);
#pragma unroll
  for (int k = 1; k < D; ++k) {
    const int v = rvel<D>(idim, k);
    F[v] = F[0] * ((vstar > 0) ? WL[v] : WR[v]);
  }
}

// Riemann wrapper (src/riemann_solver.py:10-29): inputs conservative
// (prims=false) or primitive (prims=true); rotated velocity order.
template <int D>
__device__ __forceinline__ void riemann(int solver, const double* ML, const double* MR, double* F, double gamma,
                                        double min_c2, int idim, bool prims) {
  constexpr int V = D + 2;
  double WL[V], WR[V], UL[V], UR[V];
  if (prims) {
#pragma unroll
    for (int v = 0; v < V; ++v) { WL[v] = ML[v]; WR[v] = MR[v]; }
    cons<D>(WL, UL, gamma, idim);
    cons<D>(WR, UR, gamma, idim);
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v) { UL[v] = ML[v]; UR[v] = MR[v]; }
    prim<D>(UL, WL, gamma, idim);
    prim<D>(UR, WR, gamma, idim);
  }
  if (solver == RS_LLF) llf<D>(WL, WR, UL, UR, F, gamma, min_c2, idim);
  else hllc<D>(WL, WR, UL, UR, F, gamma, min_c2, idim, solver == RS_LHLLC);
}

// One output of a 1D operator contraction: sum_s A[s] * x[s].  ``lanes2``
// is the order of an einsum over the contiguous x axis (even and odd terms
// accumulated separately, then added); otherwise a left-to-right sum
// (src/transforms.py:3-25).
template <int L>
__device__ __forceinline__ double dot_seq(const double* A, const double* x) {
  double acc = A[0] * x[0];
#pragma unroll
  for (int s = 1; s < L; ++s) acc = acc + A[s] * x[s];
  return acc;
}
template <int L>
__device__ __forceinline__ double dot_lanes2(const double* A, const double* x) {
  double e = A[0] * x[0];
  if (L == 1) return e;
  double o = A[1] * x[1];
#pragma unroll
  for (int s = 2; s < L; ++s) {
    if (s % 2 == 0) e = e + A[s] * x[s];
    else o = o + A[s] * x[s];
  }
  return e + o;
}
template <int L>
__device__ __forceinline__ double dot_dir(const double* A, const double* x, int idim) {
  return idim == 0 ? dot_lanes2<L>(A, x) : dot_seq<L>(A, x);
}

// Limiters (src/muscl.py:12-59); NaN semantics follow the np.where forms.
__device__ __forceinline__ double minmod(double SL, double SR) {
  double r = SR / SL;
  r = (r < 1.0) ? r : 1.0;
  return ((r > 0.0) ? r : 0.0) * SL;
}
__device__ __forceinline__ double np_sign(double x) {
  return (x > 0.0) ? 1.0 : ((x < 0.0) ? -1.0 : ((x == 0.0) ? 0.0 : x));
}
__device__ __forceinline__ double moncen(double dUL, double dUR, double dxL, double dxR, double dxM) {
  const double dUC = (dxL * dUL + dxR * dUR) / (dxL + dxR);
  double slope = np_min(fabs(2.0 * dUL * dxL / dxM), fabs(2.0 * dUR * dxR / dxM));
  slope = np_sign(dUC) * np_min(slope, fabs(dUC));
  return (dUL * dUR >= 0.0) ? slope : 0.0;
}

}  // namespace spd
