// Reverse-mode vector-Jacobian products of the pointwise Euler maps of the
// step (primitive/conservative conversion, Euler flux, LLF and HLLC /
// low-Mach HLLC Riemann solvers, src/hydro.py and src/riemann_solver.py).
// Each routine recomputes the forward values with the forward's own
// arithmetic (so every branch is taken as in the forward step) and then
// accumulates the adjoints of its inputs.  Derivative conventions at kinks
// follow the dual-number forms in spd_device.cuh: |x| has derivative 0 at
// 0, a tie of numpy-style maximum/minimum gives each argument half, and a
// select (a > b ? a : b) differentiates the selected argument.
#pragma once
#include "spd_device.cuh"

namespace spd {

SPD_FN double sgn0(double x) { return (x > 0.0) ? 1.0 : ((x < 0.0) ? -1.0 : 0.0); }

// W = prim(U): Ua += (dW/dU)^T Wa
// (Adjoint-only arithmetic below uses reciprocals freely: its values need
// no bitwise match; values that decide a branch are recomputed exactly.)
template <int D>
SPD_FN void prim_vjp_add(const double* U, const double* Wa, double* Ua, double gamma) {
  constexpr int P_ = D + 1;
  const double r = U[0];
  const double rr = 1.0 / r;
  double w[D + 2], ks = 0.0;
#pragma unroll
  for (int v = 1; v <= D; ++v) {
    w[v] = U[v] * rr;
    ks += w[v] * w[v];
  }
  const double Pa = Wa[P_];
  Ua[P_] += (gamma - 1.0) * Pa;
  const double Ka = -(gamma - 1.0) * Pa;
  const double ksa = Ka * 0.5 * r;
  double ra = Wa[0] + Ka * 0.5 * ks;
#pragma unroll
  for (int v = 1; v <= D; ++v) {
    const double wa = (Wa[v] + 2.0 * w[v] * ksa) * rr;
    Ua[v] += wa;
    ra -= wa * w[v];
  }
  Ua[0] += ra;
}

// U = cons(W): Wa += (dU/dW)^T Ua
template <int D>
SPD_FN void cons_vjp_add(const double* W, const double* Ua, double* Wa, double gamma) {
  constexpr int P_ = D + 1;
  const double r = W[0];
  double ks = 0.0;
#pragma unroll
  for (int v = 1; v <= D; ++v) ks += W[v] * W[v];
  Wa[P_] += Ua[P_] * (1.0 / (gamma - 1.0));
  const double ksa = Ua[P_] * 0.5 * r;
  double ra = Ua[0] + Ua[P_] * 0.5 * ks;
#pragma unroll
  for (int v = 1; v <= D; ++v) {
    Wa[v] += 2.0 * W[v] * ksa + Ua[v] * r;
    ra += Ua[v] * W[v];
  }
  Wa[0] += ra;
}

// F = flux(W) in direction idim: Wa += (dF/dW)^T Fa
template <int D>
SPD_FN void flux_vjp_add(const double* W, const double* Fa, double* Wa, double gamma, int idim) {
  constexpr int P_ = D + 1;
  const int v1 = rvel<D>(idim, 0);
  const double r = W[0], u = W[v1], P = W[P_];
  double ks = 0.0;
#pragma unroll
  for (int v = 1; v <= D; ++v) ks += W[v] * W[v];
  const double rg = 1.0 / (gamma - 1.0);
  const double E = P * rg + 0.5 * r * ks;
  double ra = Fa[0] * u + Fa[v1] * u * u;
  double ua = Fa[0] * r + Fa[v1] * 2.0 * r * u + Fa[P_] * (E + P);
  double Pa = Fa[v1] + Fa[P_] * u;
  const double Ea = Fa[P_] * u;
#pragma unroll
  for (int k = 1; k < D; ++k) {
    const int vt = rvel<D>(idim, k);
    ra += Fa[vt] * W[vt] * u;
    ua += Fa[vt] * r * W[vt];
    Wa[vt] += Fa[vt] * r * u;
  }
  Pa += Ea * rg;
  ra += Ea * 0.5 * ks;
#pragma unroll
  for (int v = 1; v <= D; ++v) Wa[v] += Ea * r * W[v];
  Wa[0] += ra;
  Wa[v1] += ua;
  Wa[P_] += Pa;
}

// c = sound_speed(P, rho) (floored): adds dc/dP * ca, dc/drho * ca
SPD_FN void sound_speed_vjp_add(double P, double rho, double gamma, double min_c2, double ca, double& Pa,
                                double& ra) {
  const double rr = 1.0 / rho;
  const double c2 = div_rcp(gamma * P, rho, rr);  // the forward's quotient (decides the floor)
  if (!(c2 > min_c2)) return;
  const double c2a = ca * (0.5 / sqrt(c2));
  Pa += c2a * gamma * rr;
  ra -= c2a * c2 * rr;
}

// LLF / HLLC flux F(ML, MR): (MLa, MRa) = J^T Fa (written).  prims: the
// inputs are primitive states (else conservative), as in riemann().
template <int D>
SPD_FN void riemann_vjp_rev(int solver, const double* ML, const double* MR, const double* Fa, double* MLa,
                            double* MRa, double gamma, double min_c2, int idim, bool prims) {
  constexpr int V = D + 2, P_ = D + 1;
  const int v1 = rvel<D>(idim, 0);
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
  double WLa[V], WRa[V], ULa[V], URa[V];
#pragma unroll
  for (int v = 0; v < V; ++v) { WLa[v] = 0.0; WRa[v] = 0.0; ULa[v] = 0.0; URa[v] = 0.0; }
  const double cL = sound_speed(WL[P_], WL[0], gamma, min_c2) + fabs(WL[v1]);
  const double cR = sound_speed(WR[P_], WR[0], gamma, min_c2) + fabs(WR[v1]);
  const bool Lmax = cL > cR;
  const double cmax = Lmax ? cL : cR;
  double cmax_a = 0.0;
  if (solver == RS_LLF) {
    const double hc = 0.5 * cmax;
    double FLa[V], FRa[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      FLa[v] = 0.5 * Fa[v];
      FRa[v] = 0.5 * Fa[v];
      URa[v] -= hc * Fa[v];
      ULa[v] += hc * Fa[v];
      cmax_a -= 0.5 * Fa[v] * (UR[v] - UL[v]);
    }
    flux_vjp_add<D>(WL, FLa, WLa, gamma, idim);
    flux_vjp_add<D>(WR, FRa, WRa, gamma, idim);
  } else {
    const bool low_mach = solver == RS_LHLLC;
    const double vL = WL[v1], vR = WR[v1];
    const bool minL = vL < vR, maxL = vL > vR;
    const double sL = (minL ? vL : vR) - cmax;
    const double sR = (maxL ? vL : vR) + cmax;
    const double rcL = WL[0] * (vL - sL);
    const double rcR = WR[0] * (sR - vR);
    const double den = rcR + rcL;
    const double rden = 1.0 / den;
    const double vstar = div_rcp(rcR * vR + rcL * vL + (WL[P_] - WR[P_]), den, rden);
    double phi = 1.0, Mach = 0.0, mx = 0.0;
    if (low_mach) {
      mx = np_max(fabs(vL), fabs(vR)) / cmax;
      Mach = np_min(1.0, mx);
      phi = Mach * (2.0 - Mach);
    }
    const double Pstar = low_mach ? div_rcp(rcR * WL[P_] + rcL * WR[P_] + phi * rcL * rcR * (vL - vR), den, rden)
                                  : div_rcp(rcR * WL[P_] + rcL * WR[P_] + rcL * rcR * (vL - vR), den, rden);
    int region;
    double r, vg, Pg, e, dd = 1.0, rdd = 1.0;
    if (sL > 0.0) {
      region = 0; r = WL[0]; vg = vL; Pg = WL[P_]; e = UL[P_];
    } else if (vstar > 0.0 || sR > 0.0) {
      // left (region 1) and right (region 2) star states: one path with
      // per-lane operands (both sides of a warp evaluate it once)
      const bool lft = vstar > 0.0;
      region = lft ? 1 : 2;
      const double s = lft ? sL : sR, v = lft ? vL : vR;
      const double w0 = lft ? WL[0] : WR[0], wP = lft ? WL[P_] : WR[P_], uP = lft ? UL[P_] : UR[P_];
      dd = s - vstar;
      rdd = 1.0 / dd;
      r = div_rcp(w0 * (s - v), dd, rdd);
      e = div_rcp((s - v) * uP - wP * v + Pstar * vstar, dd, rdd);
      vg = vstar; Pg = Pstar;
    } else {
      region = 3; r = WR[0]; vg = vR; Pg = WR[P_]; e = UR[P_];
    }
    const double F0 = r * vg;
    const bool left = vstar > 0.0;
    // reverse of the flux assembly
    double F0a = Fa[0] + Fa[v1] * vg;
#pragma unroll
    for (int k = 1; k < D; ++k) {
      const int vt = rvel<D>(idim, k);
      const double wv = left ? WL[vt] : WR[vt];
      F0a += Fa[vt] * wv;
      if (left) WLa[vt] += Fa[vt] * F0;
      else WRa[vt] += Fa[vt] * F0;
    }
    const double ra = F0a * vg;
    const double vga = F0a * r + Fa[v1] * F0 + Fa[P_] * (e + Pg);
    const double Pga = Fa[v1] + Fa[P_] * vg;
    const double ea = Fa[P_] * vg;
    double vstar_a = 0.0, Pstar_a = 0.0, sL_a = 0.0, sR_a = 0.0, vL_a = 0.0, vR_a = 0.0;
    if (region == 0) {
      WLa[0] += ra; vL_a += vga; WLa[P_] += Pga; ULa[P_] += ea;
    } else if (region == 3) {
      WRa[0] += ra; vR_a += vga; WRa[P_] += Pga; URa[P_] += ea;
    } else {
      vstar_a += vga;
      Pstar_a += Pga;
      const bool isL = region == 1;
      const double rho = isL ? WL[0] : WR[0];
      const double vK = isL ? vL : vR;
      const double sK = isL ? sL : sR;
      const double EK = isL ? UL[P_] : UR[P_];
      const double PK = isL ? WL[P_] : WR[P_];
      // r = rho (sK - vK) / dd, dd = sK - vstar (rdd = 1 / dd from above)
      double rho_a = ra * (sK - vK) * rdd;
      double sK_a = (ra * rho - ra * r) * rdd;
      double vK_a = -ra * rho * rdd;
      vstar_a += ra * r * rdd;
      // e = ((sK - vK) EK - PK vK + Pstar vstar) / dd
      const double na = ea * rdd;
      sK_a += -na * e + na * EK;
      vstar_a += na * e + na * Pstar;
      vK_a += -na * EK - na * PK;
      const double EK_a = na * (sK - vK);
      const double PK_a = -na * vK;
      Pstar_a += na * vstar;
      if (isL) {
        WLa[0] += rho_a; vL_a += vK_a; sL_a += sK_a; ULa[P_] += EK_a; WLa[P_] += PK_a;
      } else {
        WRa[0] += rho_a; vR_a += vK_a; sR_a += sK_a; URa[P_] += EK_a; WRa[P_] += PK_a;
      }
    }
    // Pstar = (rcR PL + rcL PR + phi rcL rcR (vL - vR)) / den
    double rcL_a = 0.0, rcR_a = 0.0, den_a = 0.0;
    {
      const double na = Pstar_a * rden;
      den_a -= na * Pstar;
      rcR_a += na * WL[P_] + na * phi * rcL * (vL - vR);
      rcL_a += na * WR[P_] + na * phi * rcR * (vL - vR);
      WLa[P_] += na * rcR;
      WRa[P_] += na * rcL;
      vL_a += na * phi * rcL * rcR;
      vR_a -= na * phi * rcL * rcR;
      if (low_mach) {
        const double phi_a = na * rcL * rcR * (vL - vR);
        const double Mach_a = phi_a * (2.0 - 2.0 * Mach);
        // Mach = np_min(1, mx)
        const double wmx = (mx == 1.0) ? 0.5 : ((1.0 <= mx || mx != mx) ? 0.0 : 1.0);
        const double mx_a = Mach_a * wmx;
        // mx = np_max(|vL|, |vR|) / cmax
        cmax_a -= mx_a * mx / cmax;
        const double aL = fabs(vL), aR = fabs(vR);
        const double m_a = mx_a / cmax;
        double wL, wR;
        if (aL == aR) { wL = 0.5; wR = 0.5; }
        else if (aL >= aR || aL != aL) { wL = 1.0; wR = 0.0; }
        else { wL = 0.0; wR = 1.0; }
        vL_a += m_a * wL * sgn0(vL);
        vR_a += m_a * wR * sgn0(vR);
      }
    }
    // vstar = (rcR vR + rcL vL + (PL - PR)) / den
    {
      const double na = vstar_a * rden;
      den_a -= na * vstar;
      rcR_a += na * vR;
      rcL_a += na * vL;
      vR_a += na * rcR;
      vL_a += na * rcL;
      WLa[P_] += na;
      WRa[P_] -= na;
    }
    rcR_a += den_a;
    rcL_a += den_a;
    // rcL = rhoL (vL - sL); rcR = rhoR (sR - vR)
    WLa[0] += rcL_a * (vL - sL);
    vL_a += rcL_a * WL[0];
    sL_a -= rcL_a * WL[0];
    WRa[0] += rcR_a * (sR - vR);
    sR_a += rcR_a * WR[0];
    vR_a -= rcR_a * WR[0];
    // sL = min-select(vL, vR) - cmax; sR = max-select(vL, vR) + cmax
    if (minL) vL_a += sL_a; else vR_a += sL_a;
    cmax_a -= sL_a;
    if (maxL) vL_a += sR_a; else vR_a += sR_a;
    cmax_a += sR_a;
    WLa[v1] += vL_a;
    WRa[v1] += vR_a;
  }
  // cmax = select(cL, cR); c = sound_speed(P, rho) + |v|
  {
    const double cLa = Lmax ? cmax_a : 0.0, cRa = Lmax ? 0.0 : cmax_a;
    sound_speed_vjp_add(WL[P_], WL[0], gamma, min_c2, cLa, WLa[P_], WLa[0]);
    sound_speed_vjp_add(WR[P_], WR[0], gamma, min_c2, cRa, WRa[P_], WRa[0]);
    WLa[v1] += cLa * sgn0(WL[v1]);
    WRa[v1] += cRa * sgn0(WR[v1]);
  }
  // back to the inputs
#pragma unroll
  for (int v = 0; v < V; ++v) { MLa[v] = 0.0; MRa[v] = 0.0; }
  if (prims) {
#pragma unroll
    for (int v = 0; v < V; ++v) { MLa[v] = WLa[v]; MRa[v] = WRa[v]; }
    cons_vjp_add<D>(WL, ULa, MLa, gamma);
    cons_vjp_add<D>(WR, URa, MRa, gamma);
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v) { MLa[v] = ULa[v]; MRa[v] = URa[v]; }
    prim_vjp_add<D>(UL, WLa, MLa, gamma);
    prim_vjp_add<D>(UR, WRa, MRa, gamma);
  }
}

}  // namespace spd
