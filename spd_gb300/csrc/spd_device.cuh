// Device-side building blocks of the SD-ADER step: Euler thermodynamics,
// the LLF / HLLC / low-Mach HLLC Riemann solvers and the fixed-order
// contractions.  Every routine reproduces the operation order of the
// reference's NumPy expressions (file:line cited per function) so that the
// FP64 results are bit-identical to it; this file must be compiled with
// --fmad=false so that no a*b+c is fused.
#pragma once
#include <cstdint>
#include <cmath>
#include <cstring>

// device code; also host-callable so the scalar maps can be checked on a CPU
#ifndef SPD_FN
#define SPD_FN __host__ __device__ __forceinline__
#endif

namespace spd {


constexpr int MAXN = 5;   // p <= 4
constexpr int MAXNF = 6;
constexpr int MAXT = 6;   // m <= 5
constexpr int NGH = 2;    // subcell ghost layers (Nghc)

// Block index a kernel body works on and the number of blocks of its grid.
// A plain launch passes the hardware indices; a batched launch over many
// instances passes the block's index within its own instance's share of the
// grid and the size of that share.
struct Blk {
  unsigned id, n;
};
#ifdef __CUDACC__
__device__ __forceinline__ Blk hw_blk() { return Blk{blockIdx.x, gridDim.x}; }
#endif

enum Riemann : int { RS_LLF = 0, RS_HLLC = 1, RS_LHLLC = 2 };
enum Limiter : int { LIM_MINMOD = 0, LIM_MONCEN = 1 };
enum BcKind : int { BC_PERIODIC = 0, BC_REFLECTIVE = 1, BC_GRADFREE = 2, BC_IC = 3, BC_EQ = 4, BC_PRESSURE = 5 };

// ---------------------------------------------------------------------------
// Scalars: the physics below is written for a generic scalar S, instantiated
// with double (the step itself, same arithmetic as written) and with the
// forward-mode dual number Dual<N> (value plus N tangents), which the
// adjoint kernels use for the Jacobian-transpose products of local maps.
// ---------------------------------------------------------------------------
template <int N>
struct Dual {
  double v;
  double d[N];
  SPD_FN Dual() {}
  SPD_FN Dual(double x) : v(x) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
};
template <int N>
SPD_FN Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
SPD_FN Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
SPD_FN Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r; r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
SPD_FN Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N>
SPD_FN Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N> SPD_FN Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> SPD_FN Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> SPD_FN Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> SPD_FN Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N>
SPD_FN Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N> SPD_FN Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N> SPD_FN Dual<N> operator/(const Dual<N>& a, double b) { return a / Dual<N>(b); }
template <int N> SPD_FN Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> SPD_FN bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> SPD_FN bool operator>(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N> SPD_FN bool operator<=(const Dual<N>& a, const Dual<N>& b) { return a.v <= b.v; }
template <int N> SPD_FN bool operator>=(const Dual<N>& a, const Dual<N>& b) { return a.v >= b.v; }
template <int N> SPD_FN bool operator!=(const Dual<N>& a, const Dual<N>& b) { return a.v != b.v; }
template <int N> SPD_FN bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> SPD_FN bool operator>(const Dual<N>& a, double b) { return a.v > b; }

// Correctly rounded a / b from a correctly rounded reciprocal rb = RN(1/b)
// by Markstein's correction (P. Markstein, IBM J. Res. Dev. 34(1), 1990;
// Muller et al., Handbook of Floating-Point Arithmetic, 2nd ed., Thm. 5.3):
// q = RN(a*rb) is within one ulp of a/b, the residual a - b*q is exact in
// one fused multiply-add, and RN(q + r*rb) is RN(a/b).  The theorem needs
// every quantity away from underflow and overflow, so the corrected quotient
// is used only when the biased exponents of b lie in [23, 2023] and those of
// a and q in [63, 2023] (then rb and q are normal, and the exact residual, a
// multiple of ulp(b)*ulp(q) >= 2^-1074, is representable).  Outside that
// window: a zero, infinite or NaN numerator or divisor makes q itself the
// IEEE quotient (value and sign) and q is returned; any other operand pair
// (subnormal or huge b, a or q near underflow or overflow) is divided by
// IEEE division.  Three FP64 operations instead of a full division where
// one divisor serves several quotients.
#ifdef __CUDA_ARCH__
__device__ __noinline__ double div_ieee_slow(double a, double b) { return a / b; }
#else
inline double div_ieee_slow(double a, double b) { return a / b; }
#endif
// Predicates on a double's bit pattern evaluated on its two 32-bit words
// (integer pipes).  The same tests written on the 64-bit pattern (for
// instance (bits & ~sign) > bits(inf) for NaN) were compiled to FP64-pipe
// instructions, measured with ncu (one per test), on the pipe that bounds
// the step's kernels.
SPD_FN unsigned hi_word(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned)__double2hiint(x);
#else
  unsigned long long b;
  memcpy(&b, &x, sizeof(b));
  return (unsigned)(b >> 32);
#endif
}
SPD_FN unsigned lo_word(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned)__double2loint(x);
#else
  unsigned long long b;
  memcpy(&b, &x, sizeof(b));
  return (unsigned)b;
#endif
}
// x is a NaN
SPD_FN bool nan_w(double x) {
  const unsigned h = hi_word(x) & 0x7fffffffu;
  return h > 0x7ff00000u || (h == 0x7ff00000u && lo_word(x) != 0u);
}
// x != 0 (true for NaN, false for both zeros)
SPD_FN bool nonzero_w(double x) { return ((hi_word(x) & 0x7fffffffu) | lo_word(x)) != 0u; }
// x > 0 (false for zeros, negatives and NaN)
SPD_FN bool gt0_w(double x) {
  const unsigned h = hi_word(x), l = lo_word(x);
  return (h >> 31) == 0u && (h | l) != 0u && (h < 0x7ff00000u || (h == 0x7ff00000u && l == 0u));
}

SPD_FN double div_rcp(double a, double b, double rb) {
  const double q = a * rb;
  const double r = fma(-q, b, a);
  const double q2 = fma(r, rb, q);
  // the window tests on the high words (|x|'s exponent is bits 30..20 of
  // the high word; |x| is zero when both words of |x| are, infinite or NaN
  // when the high word of |x| is >= that of infinity): integer pipes, where
  // the same tests on the 64-bit patterns cost about one FP64 instruction
  // per quotient (measured with ncu)
  const unsigned ha = hi_word(a) & 0x7fffffffu, hb = hi_word(b) & 0x7fffffffu, hq = hi_word(q) & 0x7fffffffu;
  const unsigned ea = ha >> 20, eb = hb >> 20, eq = hq >> 20;
  if (eb >= 23u && eb <= 2023u) {
    if ((ha | lo_word(a)) == 0u || ha >= 0x7ff00000u) return q;
    if (ea >= 63u && ea <= 2023u && eq >= 63u && eq <= 2023u) return q2;
  } else if ((hb | lo_word(b)) == 0u || hb >= 0x7ff00000u) {
    return q;
  }
  return div_ieee_slow(a, b);
}

SPD_FN double sval(double x) { return x; }
template <int N> SPD_FN double sval(const Dual<N>& x) { return x.v; }
SPD_FN double ad_sqrt(double x) { return sqrt(x); }
template <int N>
SPD_FN Dual<N> ad_sqrt(const Dual<N>& x) {
  Dual<N> r; r.v = sqrt(x.v);
  const double k = 0.5 / r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = x.d[i] * k;
  return r;
}
// |x| by clearing the sign bit (integer pipe; the same bits as fabs)
SPD_FN double abs_bits(double x) {
#ifdef __CUDA_ARCH__
  return __hiloint2double(__double2hiint(x) & 0x7fffffff, __double2loint(x));
#else
  return fabs(x);
#endif
}
SPD_FN double ad_abs(double x) { return abs_bits(x); }
template <int N>
SPD_FN Dual<N> ad_abs(const Dual<N>& x) {
  if (x.v > 0) return x;
  if (x.v < 0) return -x;
  return Dual<N>(fabs(x.v));
}

// a / b with b's reciprocal rb precomputed (double: Markstein; dual numbers:
// plain division, rb unused)
SPD_FN double div_by(double a, double b, double rb) { return div_rcp(a, b, rb); }
template <int N>
SPD_FN Dual<N> div_by(const Dual<N>& a, const Dual<N>& b, const Dual<N>&) { return a / b; }
template <int N>
SPD_FN Dual<N> div_by(const Dual<N>& a, double b, double) { return a / b; }
SPD_FN double recip_of(double b) { return 1.0 / b; }
template <int N>
SPD_FN Dual<N> recip_of(const Dual<N>&) { return Dual<N>(0.0); }

// NumPy's maximum / minimum: NaN in either argument propagates.
template <class S>
SPD_FN S np_max(const S& a, const S& b) { return (a >= b || a != a) ? a : b; }
template <class S>
SPD_FN S np_min(const S& a, const S& b) { return (a <= b || a != a) ? a : b; }
// Order-preserving int64 key of a double's bit pattern b: negatives
// reflected and moved up by one, so that -0 and +0 share the key 0 and every
// other pair of non-NaN values compares as in IEEE (shifts, xor and a
// subtraction on the integer pipes).
SPD_FN long long ieee_key(long long b) {
  const long long s = b >> 63;  // 0 or -1
  return (b ^ (s & 0x7fffffffffffffffLL)) - s;
}
// its inverse (the key 0 gives +0)
SPD_FN long long ieee_key_inverse(long long k) {
  const long long s = k >> 63;
  return (k + s) ^ (s & 0x7fffffffffffffffLL);
}
// The same two functions for doubles on the device, evaluated on the
// integer keys (NaN first): identical results, no FP64-pipe comparison.
#ifdef __CUDA_ARCH__
template <>
__device__ __forceinline__ double np_max<double>(const double& a, const double& b) {
  const long long ba = __double_as_longlong(a), bb = __double_as_longlong(b);
  return (nan_w(a) || (!nan_w(b) && ieee_key(ba) >= ieee_key(bb))) ? a : b;
}
template <>
__device__ __forceinline__ double np_min<double>(const double& a, const double& b) {
  const long long ba = __double_as_longlong(a), bb = __double_as_longlong(b);
  return (nan_w(a) || (!nan_w(b) && ieee_key(ba) <= ieee_key(bb))) ? a : b;
}
#endif
// a > b with IEEE semantics (false when either is NaN; -0 equals +0).  For
// doubles on the device it is evaluated on the integer keys: an FP64
// comparison issues on the FP64 pipe, which bounds the Riemann solvers.
SPD_FN bool fgt(double a, double b) {
#ifdef __CUDA_ARCH__
  return !nan_w(a) && !nan_w(b) && ieee_key(__double_as_longlong(a)) > ieee_key(__double_as_longlong(b));
#else
  return a > b;
#endif
}
// a >= b with IEEE semantics, the same way
SPD_FN bool fge(double a, double b) {
#ifdef __CUDA_ARCH__
  return !nan_w(a) && !nan_w(b) && ieee_key(__double_as_longlong(a)) >= ieee_key(__double_as_longlong(b));
#else
  return a >= b;
#endif
}
template <int N> SPD_FN bool fgt(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N> SPD_FN bool fgt(const Dual<N>& a, double b) { return a.v > b; }
template <int N> SPD_FN bool fgt(double a, const Dual<N>& b) { return a > b.v; }

// Dual forms: same value; at a tie the derivative is the mean of the two
// arguments' derivatives (the subgradient torch.maximum / torch.minimum
// propagate).
template <int N>
SPD_FN Dual<N> tie_mean(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.5 * (a.d[i] + b.d[i]);
  return r;
}
template <int N>
SPD_FN Dual<N> np_max(const Dual<N>& a, const Dual<N>& b) {
  if (a.v == b.v) return tie_mean(a, b);
  return (a.v >= b.v || a.v != a.v) ? a : b;
}
template <int N>
SPD_FN Dual<N> np_min(const Dual<N>& a, const Dual<N>& b) {
  if (a.v == b.v) return tie_mean(a, b);
  return (a.v <= b.v || a.v != a.v) ? a : b;
}

// Branch control of the piecewise-smooth maps (Riemann solvers, slope
// limiters).  BM = 0: live comparisons (the step); BM = 1: live, and each
// comparison's outcome is appended to ``w`` (a decision tape word);
// BM = 2: the outcomes are read back from ``w`` instead of compared, which
// evaluates the same smooth branch at a perturbed state (the frozen-branch
// map that the adjoint differentiates).
template <int BM>
struct Br {
  unsigned w = 0;
  int k = 0;
};
template <int BM>
SPD_FN bool pick(Br<BM>* br, bool live) {
  if (BM == 0) return live;
  if (BM == 1) {
    if (live) br->w |= (1u << br->k);
    ++br->k;
    return live;
  }
  const bool b = (br->w >> br->k) & 1u;
  ++br->k;
  return b;
}
// |x| whose sign is a recorded decision under BM != 0
template <int BM, class S>
SPD_FN S abs_br(const S& x, Br<BM>* br) {
  if (BM == 0) return ad_abs(x);
  return pick(br, sval(x) >= 0.0) ? x : -x;
}

// Velocity index k (0-based) of the rotated frame used for direction idim:
// np.roll(vels, -idim) (src/sdader_simulator.py:219).
template <int D>
SPD_FN int rvel(int idim, int k) { return 1 + (idim + k) % D; }

// U -> W (src/hydro.py:48-86); the kinetic term sums in the order of the
// velocity list, which is the rotated list inside the Riemann wrapper
// (src/riemann_solver.py:10-29) and the plain list elsewhere.
// ``r0_out`` (optional) receives 1/rho for later quotients by rho.
// ``iso``: the isothermal system (src/hydro.py:84,123,169): the kinetic term
// of the energy is multiplied by 0 and the energy flux by 0.
template <int D, class S>
SPD_FN void prim(const S* U, S* W, double gamma, int idim_order, S* r0_out = nullptr, bool iso = false) {
  constexpr int P_ = D + 1;
  W[0] = U[0];
  S K = 0.0;
  const S r0 = recip_of(U[0]);
  if (r0_out) *r0_out = r0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const int v = rvel<D>(idim_order, k);
    W[v] = (D == 1 && !r0_out) ? U[v] / U[0] : div_by(U[v], U[0], r0);
    const S w2 = W[v] * W[v];
    K = (k == 0) ? w2 : K + w2;
  }
  K = K * (0.5 * U[0]);
  if (iso) K = K * 0.0;
  W[P_] = (gamma - 1.0) * (U[P_] - K);
}

// W -> U (src/hydro.py:88-125).
template <int D, class S>
SPD_FN void cons(const S* W, S* U, double gamma, int idim_order, bool iso = false) {
  constexpr int P_ = D + 1;
  U[0] = W[0];
  S K = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const int v = rvel<D>(idim_order, k);
    U[v] = W[v] * W[0];
    const S w2 = W[v] * W[v];
    K = (k == 0) ? w2 : K + w2;
  }
  K = K * (0.5 * W[0]);
  if (iso) K = K * 0.0;
  U[P_] = div_by(W[P_], gamma - 1.0, 1.0 / (gamma - 1.0)) + K;
}

// Euler flux in the rotated frame of direction idim (src/hydro.py:127-170).
template <int D, class S>
SPD_FN void flux(const S* W, S* F, double gamma, int idim, bool iso = false) {
  constexpr int P_ = D + 1;
  const int v1 = rvel<D>(idim, 0);
  S K = 0.0, m = 0.0;
#pragma unroll
  for (int k = D - 1; k >= 0; --k) {
    const int v = rvel<D>(idim, k);
    m = W[0] * W[v];
    const S mv = m * W[v];
    K = (k == D - 1) ? mv : K + mv;
    F[v] = m * W[v1];
  }
  const S E = div_by(W[P_], gamma - 1.0, 1.0 / (gamma - 1.0)) + 0.5 * K;
  F[0] = m;
  F[v1] = m * W[v1] + W[P_];
  F[P_] = W[v1] * (E + W[P_]);
  if (iso) F[P_] = F[P_] * 0.0;
}

// Sound speed with floor (src/hydro.py:3-46).
template <class S, int BM = 0>
SPD_FN S sound_speed(const S& P, const S& rho, double gamma, double min_c2,
                                         Br<BM>* br = nullptr, const S* rrho = nullptr) {
  S c2 = rrho ? div_by(gamma * P, rho, *rrho) : gamma * P / rho;
  c2 = pick(br, fgt(c2, min_c2)) ? c2 : S(min_c2);
  return ad_sqrt(c2);
}

// LLF (src/riemann_solver.py:31-65).
template <int D, class S, int BM = 0>
SPD_FN void llf(const S* WL, const S* WR, const S* UL, const S* UR, S* F, double gamma,
                                    double min_c2, int idim, Br<BM>* br = nullptr, const S* rL = nullptr,
                                    const S* rR = nullptr, bool iso = false) {
  constexpr int V = D + 2, P_ = D + 1;
  const int v1 = rvel<D>(idim, 0);
  S FL[V], FR[V];
  flux<D>(WL, FL, gamma, idim, iso);
  flux<D>(WR, FR, gamma, idim, iso);
  const S cL = sound_speed(WL[P_], WL[0], gamma, min_c2, br, rL) + abs_br(WL[v1], br);
  const S cR = sound_speed(WR[P_], WR[0], gamma, min_c2, br, rR) + abs_br(WR[v1], br);
  const S cmax = pick(br, fgt(cL, cR)) ? cL : cR;
  const S hc = 0.5 * cmax;
#pragma unroll
  for (int v = 0; v < V; ++v) F[v] = 0.5 * (FR[v] + FL[v]) - hc * (UR[v] - UL[v]);
}

// HLLC (src/riemann_solver.py:67-145) and its low-Mach variant (:147-212).
// Only the branch the reference's np.where chain selects is evaluated.
template <int D, class S, int BM = 0>
SPD_FN void hllc(const S* WL, const S* WR, const S* UL, const S* UR, S* F, double gamma,
                                     double min_c2, int idim, bool low_mach, Br<BM>* br = nullptr,
                                     const S* rL = nullptr, const S* rR = nullptr, bool iso = false) {
  constexpr int P_ = D + 1;
  const int v1 = rvel<D>(idim, 0);
  const S cL = sound_speed(WL[P_], WL[0], gamma, min_c2, br, rL) + abs_br(WL[v1], br);
  const S cR = sound_speed(WR[P_], WR[0], gamma, min_c2, br, rR) + abs_br(WR[v1], br);
  const S cmax = pick(br, fgt(cL, cR)) ? cL : cR;
  const S vL = WL[v1], vR = WR[v1];
  const S sL = (pick(br, fgt(vR, vL)) ? vL : vR) - cmax;
  const S sR = (pick(br, fgt(vL, vR)) ? vL : vR) + cmax;
  const S rcL = WL[0] * (vL - sL);
  const S rcR = WR[0] * (sR - vR);
  const S den = rcR + rcL;
  const S rden = recip_of(den);
  const S vstar = div_by(rcR * vR + rcL * vL + (WL[P_] - WR[P_]), den, rden);
  S Pstar;
  if (low_mach) {
    S mx, Mach;
    if (BM == 0) {
      mx = np_max(ad_abs(vL), ad_abs(vR)) / cmax;
      Mach = np_min(S(1.0), mx);
    } else {
      const S aL = abs_br(vL, br), aR = abs_br(vR, br);
      mx = (pick(br, aL >= aR || aL != aL) ? aL : aR) / cmax;
      Mach = pick(br, S(1.0) <= mx) ? S(1.0) : mx;
    }
    const S phi = Mach * (2.0 - Mach);
    Pstar = div_by(rcR * WL[P_] + rcL * WR[P_] + phi * rcL * rcR * (vL - vR), den, rden);
  } else {
    Pstar = div_by(rcR * WL[P_] + rcL * WR[P_] + rcL * rcR * (vL - vR), den, rden);
  }
  S r, vg, Pg, e;
  if constexpr (BM == 0) {
    // the left and right star states are the same formulas with the sides
    // swapped: one path with per-lane operands, so a warp whose lanes take
    // both sides (an FP64 warp instruction costs the same with any number of
    // active lanes) evaluates the reciprocal and quotients once
    if (fgt(sL, 0.0)) {
      r = WL[0]; vg = vL; Pg = WL[P_]; e = UL[P_];
    } else if (fgt(vstar, 0.0) || fgt(sR, 0.0)) {
      const bool lft = fgt(vstar, 0.0);
      const S s = lft ? sL : sR, v = lft ? vL : vR;
      const S w0 = lft ? WL[0] : WR[0], wP = lft ? WL[P_] : WR[P_], uP = lft ? UL[P_] : UR[P_];
      const S d = s - vstar;
      const S rd = recip_of(d);
      r = div_by(w0 * (s - v), d, rd);
      e = div_by((s - v) * uP - wP * v + Pstar * vstar, d, rd);
      vg = vstar; Pg = Pstar;
    } else {
      r = WR[0]; vg = vR; Pg = WR[P_]; e = UR[P_];
    }
  } else if (pick(br, fgt(sL, 0.0))) {
    r = WL[0]; vg = vL; Pg = WL[P_]; e = UL[P_];
  } else if (pick(br, fgt(vstar, 0.0))) {
    const S d = sL - vstar;
    const S rd = recip_of(d);
    r = div_by(WL[0] * (sL - vL), d, rd);
    e = div_by((sL - vL) * UL[P_] - WL[P_] * vL + Pstar * vstar, d, rd);
    vg = vstar; Pg = Pstar;
  } else if (pick(br, fgt(sR, 0.0))) {
    const S d = sR - vstar;
    const S rd = recip_of(d);
    r = div_by(WR[0] * (sR - vR), d, rd);
    e = div_by((sR - vR) * UR[P_] - WR[P_] * vR + Pstar * vstar, d, rd);
    vg = vstar; Pg = Pstar;
  } else {
    r = WR[0]; vg = vR; Pg = WR[P_]; e = UR[P_];
  }
  F[0] = r * vg;
  F[v1] = F[0] * vg + Pg;
  F[P_] = vg * (e + Pg);
  if (D > 1) {
    const bool left = pick(br, fgt(vstar, 0.0));
#pragma unroll
    for (int k = 1; k < D; ++k) {
      const int v = rvel<D>(idim, k);
      F[v] = F[0] * (left ? WL[v] : WR[v]);
    }
  }
  if (iso) F[P_] = F[P_] * 0.0;
}

// Riemann wrapper (src/riemann_solver.py:10-29): inputs conservative
// (prims=false) or primitive (prims=true); rotated velocity order.
template <int D, class S, int BM = 0>
SPD_FN void riemann(int solver, const S* ML, const S* MR, S* F, double gamma, double min_c2,
                                        int idim, bool prims, Br<BM>* br = nullptr, bool iso = false) {
  constexpr int V = D + 2;
  S WL[V], WR[V], UL[V], UR[V];
  S rL, rR;  // 1/rho of the two states when the conversion computed it
  const S* prL = nullptr;
  const S* prR = nullptr;
  if (prims) {
#pragma unroll
    for (int v = 0; v < V; ++v) { WL[v] = ML[v]; WR[v] = MR[v]; }
    cons<D>(WL, UL, gamma, idim, iso);
    cons<D>(WR, UR, gamma, idim, iso);
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v) { UL[v] = ML[v]; UR[v] = MR[v]; }
    prim<D>(UL, WL, gamma, idim, &rL, iso);
    prim<D>(UR, WR, gamma, idim, &rR, iso);
    prL = &rL;
    prR = &rR;
  }
  if (solver == RS_LLF) llf<D, S, BM>(WL, WR, UL, UR, F, gamma, min_c2, idim, br, prL, prR, iso);
  else hllc<D, S, BM>(WL, WR, UL, UR, F, gamma, min_c2, idim, solver == RS_LHLLC, br, prL, prR, iso);
}

// One output of a 1D operator contraction: sum_s A[s] * x[s].  ``lanes2``
// is the order of an einsum over the contiguous x axis (even and odd terms
// accumulated separately, then added); otherwise a left-to-right sum
// (src/transforms.py:3-25).
template <int L>
SPD_FN double dot_seq(const double* A, const double* x) {
  double acc = A[0] * x[0];
#pragma unroll
  for (int s = 1; s < L; ++s) acc = acc + A[s] * x[s];
  return acc;
}
template <int L>
SPD_FN double dot_lanes2(const double* A, const double* x) {
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
SPD_FN double dot_dir(const double* A, const double* x, int idim) {
  return idim == 0 ? dot_lanes2<L>(A, x) : dot_seq<L>(A, x);
}

// Limiters (src/muscl.py:12-59); NaN semantics follow the np.where forms.
// (comparisons through fgt / fge: integer keys on the device)
SPD_FN double minmod(double SL, double SR) {
  double r = SR / SL;
  r = fgt(1.0, r) ? r : 1.0;
  return (fgt(r, 0.0) ? r : 0.0) * SL;
}
SPD_FN double np_sign(double x) {
  return fgt(x, 0.0) ? 1.0 : (fgt(0.0, x) ? -1.0 : ((fge(x, 0.0) && fge(0.0, x)) ? 0.0 : x));
}
SPD_FN double moncen(double dUL, double dUR, double dxL, double dxR, double dxM) {
  const double dUC = (dxL * dUL + dxR * dUR) / (dxL + dxR);
  double slope = np_min(abs_bits(2.0 * dUL * dxL / dxM), abs_bits(2.0 * dUR * dxR / dxM));
  slope = np_sign(dUC) * np_min(slope, abs_bits(dUC));
  return fge(dUL * dUR, 0.0) ? slope : 0.0;
}

// Limited slope with its branch as a decision code (BM as in Br): minmod
// code = 0 (0*SL), 1 (ratio*SL), 2 (SL); moncen code = bit 0 zero slope,
// bits 1-2 sign of the centred slope (0, +, -), bits 3-4 the minimum taken
// (1: left, 2: right, 3: centred), bits 5-6 the sign inside its |.|.
SPD_FN int sign_code(double x) { return (x > 0.0) ? 1 : ((x < 0.0) ? 2 : 0); }
SPD_FN double code_sign(int c) { return c == 1 ? 1.0 : (c == 2 ? -1.0 : 0.0); }
template <int BM>
SPD_FN double limiter_br(int limiter, double SL, double SR, double hl, double hr, double hm,
                                             unsigned char* code) {
  if (limiter == LIM_MINMOD) {
    if (BM == 2) {
      const int c = *code;
      if (c == 1) return (SR / SL) * SL;
      return (c == 2 ? 1.0 : 0.0) * SL;
    }
    const double v = minmod(SL, SR);
    if (BM == 1) {
      const double r = SR / SL;
      *code = (unsigned char)((r < 1.0) ? ((r > 0.0) ? 1 : 0) : 2);
    }
    return v;
  }
  const double dUC = (hl * SL + hr * SR) / (hl + hr);
  const double q1 = 2.0 * SL * hl / hm, q2 = 2.0 * SR * hr / hm;
  if (BM == 2) {
    const int c = *code;
    if (c & 1) return 0.0;
    const int sel = (c >> 3) & 3;
    const double q = sel == 1 ? q1 : (sel == 2 ? q2 : dUC);
    return code_sign((c >> 1) & 3) * (code_sign((c >> 5) & 3) * q);
  }
  const double v = moncen(SL, SR, hl, hr, hm);
  if (BM == 1) {
    const double c1 = fabs(q1), c2 = fabs(q2), c3 = fabs(dUC);
    const double m12 = np_min(c1, c2);
    const int sel12 = (c1 <= c2 || c1 != c1) ? 1 : 2;
    const int sel = (m12 <= c3 || m12 != m12) ? sel12 : 3;
    const double q = sel == 1 ? q1 : (sel == 2 ? q2 : dUC);
    const int zero = (SL * SR >= 0.0) ? 0 : 1;
    *code = (unsigned char)(zero | (sign_code(dUC) << 1) | (sel << 3) | (sign_code(q) << 5));
  }
  return v;
}

}  // namespace spd
