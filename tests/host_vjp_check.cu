// Host-side check of the reverse-mode vector-Jacobian products of the
// pointwise Euler maps (spd_vjp.cuh) against products formed with the
// dual-number forms of the same maps (spd_device.cuh) and of the
// MUSCL-Hancock half-step prediction: random states in 1D,
// 2D and 3D, every Riemann solver, conservative and primitive inputs, and
// mirrored states (the velocity ties of reflective walls); and the
// Markstein quotient div_rcp against IEEE division, bit for bit.  Exit
// status 0 when every relative difference is below 1e-12 and no quotient
// differs.
#include <cstdio>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>
#include "spd_adjoint.cuh"
using namespace spd;

template <int D>
void dual_riemann_vjp(int solver, const double* ML, const double* MR, const double* Fa, double* MLa, double* MRa,
                      double gamma, double min_c2, int d, bool prims) {
  constexpr int V = D + 2;
  Dual<2 * V> l[V], r[V], f[V];
  for (int i = 0; i < V; ++i) {
    l[i] = Dual<2 * V>(ML[i]); l[i].d[i] = 1.0;
    r[i] = Dual<2 * V>(MR[i]); r[i].d[V + i] = 1.0;
  }
  riemann<D>(solver, l, r, f, gamma, min_c2, d, prims);
  for (int i = 0; i < 2 * V; ++i) {
    double s = 0.0;
    for (int v = 0; v < V; ++v) s += Fa[v] * f[v].d[i];
    if (i < V) MLa[i] = s; else MRa[i - V] = s;
  }
}

template <int D>
double check(std::mt19937_64& rng, int solver, bool prims, int d, bool ties) {
  constexpr int V = D + 2;
  std::normal_distribution<double> N(0.0, 1.0);
  std::uniform_real_distribution<double> Uu(0.5, 2.0);
  double WL[V], WR[V];
  WL[0] = Uu(rng); WR[0] = Uu(rng);
  WL[D + 1] = Uu(rng); WR[D + 1] = Uu(rng);
  for (int v = 1; v <= D; ++v) { WL[v] = 0.7 * N(rng); WR[v] = 0.7 * N(rng); }
  if (ties) { for (int v = 1; v <= D; ++v) WR[v] = -WL[v]; }
  double ML[V], MR[V];
  if (prims) { for (int v = 0; v < V; ++v) { ML[v] = WL[v]; MR[v] = WR[v]; } }
  else { cons<D>(WL, ML, 1.4, 0); cons<D>(WR, MR, 1.4, 0); }
  double Fa[V];
  for (int v = 0; v < V; ++v) Fa[v] = N(rng);
  double a1[V], b1[V], a2[V], b2[V];
  dual_riemann_vjp<D>(solver, ML, MR, Fa, a1, b1, 1.4, 1e-10, d, prims);
  riemann_vjp_rev<D>(solver, ML, MR, Fa, a2, b2, 1.4, 1e-10, d, prims);
  double err = 0.0, nrm = 0.0;
  for (int v = 0; v < V; ++v) {
    err += (a1[v] - a2[v]) * (a1[v] - a2[v]) + (b1[v] - b2[v]) * (b1[v] - b2[v]);
    nrm += a1[v] * a1[v] + b1[v] * b1[v];
  }
  return sqrt(err / nrm);
}

template <int D>
double check_flux_prim(std::mt19937_64& rng, int d) {
  constexpr int V = D + 2;
  std::normal_distribution<double> N(0.0, 1.0);
  std::uniform_real_distribution<double> Uu(0.5, 2.0);
  double W[V], U[V];
  W[0] = Uu(rng); W[D + 1] = Uu(rng);
  for (int v = 1; v <= D; ++v) W[v] = N(rng);
  cons<D>(W, U, 1.4, 0);
  double Fa[V];
  for (int v = 0; v < V; ++v) Fa[v] = N(rng);
  // dual: F = flux(prim(U))
  Dual<V> u[V], w[V], f[V];
  for (int i = 0; i < V; ++i) { u[i] = Dual<V>(U[i]); u[i].d[i] = 1.0; }
  prim<D>(u, w, 1.4, 0);
  flux<D>(w, f, 1.4, d);
  double g1[V], g2[V], Wa[V], Wv[V];
  for (int i = 0; i < V; ++i) { double s = 0; for (int v = 0; v < V; ++v) s += Fa[v] * f[v].d[i]; g1[i] = s; }
  prim<D>(U, Wv, 1.4, 0);
  for (int v = 0; v < V; ++v) { Wa[v] = 0.0; g2[v] = 0.0; }
  flux_vjp_add<D>(Wv, Fa, Wa, 1.4, d);
  prim_vjp_add<D>(U, Wa, g2, 1.4);
  double err = 0, nrm = 0;
  for (int v = 0; v < V; ++v) { err += (g1[v] - g2[v]) * (g1[v] - g2[v]); nrm += g1[v] * g1[v]; }
  return sqrt(err / nrm);
}

// div_rcp (Markstein's correction from a correctly rounded reciprocal)
// against the correctly rounded IEEE quotient: returns the mismatch count.
// The operands cover the step's range, zeros, infinities and NaN, and the
// edges of the exponent range: subnormal and huge divisors, numerators and
// quotients near underflow and overflow, and subnormal quotients.
long long check_div_rcp(std::mt19937_64& rng, long long n) {
  std::uniform_int_distribution<int> ea(-80, 80), eb(-40, 40), wide(-1074, 1023), edge(0, 120);
  std::uniform_real_distribution<double> m(1.0, 2.0);
  long long bad = 0;
  const double specials[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 1.0, -1.0, 0.4, 3.0};
  const double tiny[] = {4.9406564584124654e-324, 2.2250738585072009e-308, 2.2250738585072014e-308,
                         1.0e-310, 1.7976931348623157e308, 8.98846567431158e307};
  for (long long i = 0; i < n; ++i) {
    double a = std::ldexp(m(rng), ea(rng)) * ((rng() & 1) ? -1.0 : 1.0);
    double b = std::ldexp(m(rng), eb(rng)) * ((rng() & 1) ? -1.0 : 1.0);
    if (i % 97 == 0) a = specials[(i / 97) % 9];
    if (i % 89 == 0) b = specials[5 + (i / 89) % 4];
    if (i % 7 == 0) b = 0.4;  // gamma - 1
    if (i % 5 == 1) {
      // anywhere in the exponent range, incl. subnormal operands
      a = std::ldexp(m(rng), wide(rng)) * ((rng() & 1) ? -1.0 : 1.0);
      b = std::ldexp(m(rng), wide(rng)) * ((rng() & 1) ? -1.0 : 1.0);
    } else if (i % 5 == 3) {
      // quotients and operands at the window's edges: near 2^-1022 and 2^1023
      const int k = edge(rng);
      a = std::ldexp(m(rng), (i & 8) ? -1080 + k : 1023 - k) * ((rng() & 1) ? -1.0 : 1.0);
      b = std::ldexp(m(rng), (i & 16) ? 60 - k : k - 60);
      if (i % 55 == 3) b = tiny[(i / 55) % 6];
      if (i % 65 == 3) a = tiny[(i / 65) % 6];
    }
    volatile double rb = 1.0 / b;
    const double got = div_rcp(a, b, rb);
    const double want = a / b;
    if (!(std::memcmp(&got, &want, sizeof(double)) == 0 || (got != got && want != want))) ++bad;
  }
  return bad;
}

// dual-number form of the MUSCL-Hancock half-step prediction (the forward's
// k_muscl_cells arithmetic) and its Jacobian-transpose product
template <int D>
double check_predictor(std::mt19937_64& rng) {
  constexpr int V = D + 2, P_ = D + 1, NT = V * (1 + D);
  std::normal_distribution<double> N(0.0, 1.0);
  std::uniform_real_distribution<double> Uu(0.5, 2.0);
  double W[V], dMh[D][V], pra[V];
  W[0] = Uu(rng);
  W[P_] = Uu(rng);
  for (int v = 1; v <= D; ++v) W[v] = N(rng);
  for (int dd = 0; dd < D; ++dd)
    for (int v = 0; v < V; ++v) dMh[dd][v] = N(rng);
  for (int v = 0; v < V; ++v) pra[v] = N(rng);
  const double dti = 0.01 + 0.1 * Uu(rng);
  Dual<NT> w[V], dm[D][V], dtW[V];
  for (int v = 0; v < V; ++v) { w[v] = Dual<NT>(W[v]); w[v].d[v] = 1.0; }
  for (int dd = 0; dd < D; ++dd)
    for (int v = 0; v < V; ++v) { dm[dd][v] = Dual<NT>(dMh[dd][v]); dm[dd][v].d[V + dd * V + v] = 1.0; }
  for (int v = 0; v < V; ++v) dtW[v] = Dual<NT>(0.0);
  for (int dd = 0; dd < D; ++dd) {
    const int vel = dd + 1;
    dtW[0] = dtW[0] - (w[vel] * dm[dd][0] + w[0] * dm[dd][vel]);
    dtW[P_] = dtW[P_] - (w[vel] * dm[dd][P_] + 1.4 * w[P_] * dm[dd][vel]);
    dtW[vel] = dtW[vel] - (w[vel] * dm[dd][vel] + dm[dd][P_] / w[0]);
    for (int v2 = 2; v2 <= D; ++v2) dtW[v2] = dtW[v2] - w[vel] * dm[dd][v2];
  }
  dtW[P_] = dtW[P_] * 0.0;
  double ref[NT], got[NT];
  for (int i = 0; i < NT; ++i) { ref[i] = 0.0; got[i] = 0.0; }
  for (int v = 0; v < V; ++v) {
    const Dual<NT> pr = w[v] + 0.5 * dtW[v] * dti;
    for (int i = 0; i < NT; ++i) ref[i] += pra[v] * pr.d[i];
  }
  predictor_vjp<D>(W, dMh, dti, pra, got);
  double err = 0.0, nrm = 0.0;
  for (int i = 0; i < NT; ++i) { err += (got[i] - ref[i]) * (got[i] - ref[i]); nrm += ref[i] * ref[i]; }
  return sqrt(err / nrm);
}

// ieee_key / ieee_key_inverse (the integer keys of the device max / min
// and of the trouble detection) against IEEE comparison: every ordered
// pair of non-NaN values, specials included, compares the same way on the
// keys, and the inverse returns the value (+0 for either zero); and the
// word-based predicates nan_w, nonzero_w, gt0_w against x != x, x != 0,
// x > 0.
long long check_order_keys(std::mt19937_64& rng, long long n) {
  auto bits = [](double x) { long long b; memcpy(&b, &x, 8); return b; };
  auto val = [](long long b) { double x; memcpy(&x, &b, 8); return x; };
  const double specials[] = {0.0, -0.0, 1.0, -1.0, 4.9e-324, -4.9e-324, 2.2250738585072014e-308,
                             -2.2250738585072014e-308, 1.7976931348623157e308, -1.7976931348623157e308,
                             INFINITY, -INFINITY, 0.75, -0.25, 1e-300, -1e300};
  std::uniform_int_distribution<unsigned long long> U;
  long long bad = 0;
  auto one = [&](double a, double b) {
    if (a != a || b != b) return;
    const long long ka = ieee_key(bits(a)), kb = ieee_key(bits(b));
    bad += ((ka < kb) != (a < b)) + ((ka == kb) != (a == b)) + ((ka > kb) != (a > b));
  };
  auto preds = [&](double a) {
    bad += (nan_w(a) != (a != a)) + (nonzero_w(a) != (a != 0.0)) + (gt0_w(a) != (a > 0.0));
  };
  for (double a : specials) {
    preds(a);
    for (double b : specials) one(a, b);
  }
  preds(NAN);
  preds(-NAN);
  preds(val(0x7ff0000000000001LL));
  preds(val((long long)0xfff0000000000001ULL));
  for (long long i = 0; i < n; ++i) {
    const double a = val((long long)U(rng)), b = val((long long)U(rng));
    one(a, b);
    one(a, -a);
    preds(a);
    if (a == a) {
      const double back = val(ieee_key_inverse(ieee_key(bits(a))));
      bad += (a == 0.0) ? (bits(back) != 0) : (bits(back) != bits(a));
    }
  }
  return bad;
}

int main() {
  std::mt19937_64 rng(42);
  double worst = 0.0;
  const long long key_bad = check_order_keys(rng, 5000000);
  printf("order-key mismatches: %lld\n", key_bad);
  if (key_bad) return 1;
  const long long div_bad = check_div_rcp(rng, 20000000);
  printf("div_rcp mismatches: %lld of 20000000\n", div_bad);
  if (div_bad) return 1;
  for (int trial = 0; trial < 4000; ++trial) {
    for (int solver = 0; solver < 3; ++solver)
      for (int prims = 0; prims < 2; ++prims) {
        const bool ties = (trial % 7) == 0;
        double e;
        e = check<1>(rng, solver, prims, 0, ties); worst = e > worst ? e : worst;
        for (int d = 0; d < 2; ++d) { e = check<2>(rng, solver, prims, d, ties); worst = e > worst ? e : worst; }
        for (int d = 0; d < 3; ++d) { e = check<3>(rng, solver, prims, d, ties); worst = e > worst ? e : worst; }
      }
    double e = check_flux_prim<2>(rng, trial % 2); worst = e > worst ? e : worst;
    e = check_predictor<1>(rng); worst = e > worst ? e : worst;
    e = check_predictor<2>(rng); worst = e > worst ? e : worst;
    e = check_predictor<3>(rng); worst = e > worst ? e : worst;
    e = check_flux_prim<3>(rng, trial % 3); worst = e > worst ? e : worst;
    e = check_flux_prim<1>(rng, 0); worst = e > worst ? e : worst;
  }
  printf("worst relative difference reverse vs dual: %.3e\n", worst);
  return worst < 1e-12 ? 0 : 1;
}
