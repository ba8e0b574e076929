// Subcell finite-volume update with a-posteriori limiting for sm_103a:
// high-order flux application, ghost fills, NAD/SED/PAD trouble detection,
// blending, MUSCL-Hancock fallback fluxes on the affected faces only, and
// the CFL reduction.  Bit-identical to src/sdader_simulator.py:333-349,
// src/fv_simulator.py, src/trouble_detection.py and src/muscl.py.
#pragma once
#include "spd_kernels.cuh"

namespace spd {

struct FvGeo {
  const double* dx[3];       // active subcell widths, X_d values
  const double* centers[3];  // extended subcell centres, Xe_d values
  const double* hfp[3];      // extended subcell widths, Xe_d values
  const double* hcv[3];      // extended centre distances, Xe_d - 1 values
  const double* rdx[3];      // 1 / dx (correctly rounded)
  const double* rhcv[3];     // 1 / hcv (correctly rounded)
  const double* c2[3];       // centres[j+1] - centres[j-1], Xe_d values (ends unused)
  const double* rc2[3];      // 1 / c2 (correctly rounded)
};

__device__ __forceinline__ void q_coords(const Geo& g, long long q, int& ix, int& iy, int& iz) {
  ix = (int)(q % g.X[0]);
  long long r = q / g.X[0];
  iy = (int)(r % g.X[1]);
  iz = (int)(r / g.X[1]);
}

template <int D>
__device__ __forceinline__ long long ext_of(const Geo& g, int ix, int iy, int iz) {
  const int xe = ix + NGH, ye = (D >= 2) ? iy + NGH : 0, ze = (D >= 3) ? iz + NGH : 0;
  return xe + (long long)g.Xe[0] * (ye + (long long)g.Xe[1] * ze);
}

__device__ __forceinline__ long long ext_stride(const Geo& g, int d) {
  return d == 0 ? 1LL : (d == 1 ? (long long)g.Xe[0] : (long long)g.Xe[0] * g.Xe[1]);
}

__device__ __forceinline__ long long face_id(const Geo& g, int d, int fx, int fy, int fz) {
  const int FX = g.X[0] + (d == 0), FY = g.X[1] + (d == 1);
  return fx + (long long)FX * (fy + (long long)FY * fz);
}

__host__ __device__ __forceinline__ long long n_faces(const Geo& g, int d) {
  return (long long)(g.X[0] + (d == 0)) * (g.X[1] + (d == 1)) * (g.X[2] + (d == 2));
}

// Order-preserving int64 key of a double (ieee_key of its bits: the two
// zeros share a key, as they compare equal in IEEE) and its inverse (the
// key of either zero gives +0); NaN test on the bits.
__device__ __forceinline__ long long order_key(double x) { return ieee_key(__double_as_longlong(x)); }
__device__ __forceinline__ double from_order_key(long long k) { return __longlong_as_double(ieee_key_inverse(k)); }
__device__ __forceinline__ bool is_nan_bits(double x) { return nan_w(x); }
// NumPy maximum (a if a >= b or a is NaN, else b) on the integer pipes
__device__ __forceinline__ double np_max_key(double a, double b) {
  if (is_nan_bits(a)) return a;
  if (is_nan_bits(b)) return b;
  return order_key(a) >= order_key(b) ? a : b;
}
// x != 0.0 on the bits (true for NaN, false for both zeros)
__device__ __forceinline__ bool nonzero_bits(double x) { return nonzero_w(x); }
// x > 0 on the bits (false for zeros, negatives and NaN)
__device__ __forceinline__ bool gt0_key(double x) { return gt0_w(x); }

// gravity source of one subcell (src/fv_simulator.py:200-203 with
// src/simulator.py:197-203): dUdt[vel] += rho * dphi_vel, dUdt[P] +=
// m_vel * dphi_vel, direction by direction; gphi [d][subcell]
template <int D>
__device__ __forceinline__ void potential_source(const Geo& g, const double* __restrict__ gphi, long long q,
                                                 const double* u, double* dudt) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const double gp = gphi[(long long)d * g.Nq + q];
    dudt[d + 1] = dudt[d + 1] + u[0] * gp;
    if (!g.iso) dudt[D + 1] = dudt[D + 1] + u[d + 1] * gp;
  }
}

// Primitives of one subcell's state (src/sdader_simulator.py:351-356): in
// the well-balanced mode (Ueq non-null) the perturbation
// prim(U + U_eq) - prim(U_eq), with prim(U_eq) given as Weq; [v][subcell]
template <int D>
__device__ __forceinline__ void prims_cv(const Geo& g, const double* u, double* W, const double* __restrict__ Ueq,
                                         const double* __restrict__ Weq, long long q) {
  constexpr int V = D + 2;
  if (Ueq == nullptr) {
    prim<D>(u, W, g.gamma, 0, (double*)nullptr, g.iso != 0);
    return;
  }
  double uf[V];
#pragma unroll
  for (int v = 0; v < V; ++v) uf[v] = u[v] + Ueq[(long long)v * g.Nq + q];
  prim<D>(uf, W, g.gamma, 0, (double*)nullptr, g.iso != 0);
#pragma unroll
  for (int v = 0; v < V; ++v) W[v] = W[v] - Weq[(long long)v * g.Nq + q];
}

// dUdt of one subcell from the face fluxes (src/fv_simulator.py:189-205)
template <int D>
__device__ __forceinline__ void flux_divergence(const Geo& g, const FvGeo& fg, int ix, int iy, int iz,
                                                const double* const* F, int v, double& out) {
  const int ii[3] = {ix, iy, iz};
  double acc = 0.0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const long long nf = n_faces(g, d);
    const long long fl = face_id(g, d, ix, iy, iz);
    const long long fr = face_id(g, d, ix + (d == 0), iy + (d == 1), iz + (d == 2));
    const double part = div_rcp(F[d][(long long)v * nf + fr] - F[d][(long long)v * nf + fl], fg.dx[d][ii[d]],
                                fg.rdx[d][ii[d]]);
    acc = (d == 0) ? part : acc + part;
  }
  out = acc;
}

// candidate update with the high-order fluxes of time node i, W_old and
// W_new into the extended arrays (src/sdader_simulator.py:336-340,
// src/trouble_detection.py:10-13)
template <int D>
struct FvCandidate {
// write_ext: 0 = no primitives (no limiting); 1 = W_old = prim(U_cv) and
// W_new = prim(U_new) into ext_old / ext_new; 2 = as 1 with W_old read from
// ext_new, which holds prim(U_cv) at this point (the previous substep's
// W_new, refreshed by k_fv_correct where the fallback changed U_cv): the
// same values without a second primitive conversion.
static __device__ __forceinline__ void run(Blk B, const Geo& g, const FvGeo& fg, const double* __restrict__ dt_ptr,
                                           double w_i, const double* F0, const double* F1, const double* F2,
                                           const double* __restrict__ U_cv, double* __restrict__ U_new,
                                           double* ext_old, double* ext_new, int write_ext,
                                           const double* __restrict__ gphi, const double* __restrict__ Ueq,
                                           const double* __restrict__ Weq) {
  constexpr int V = D + 2;
  const long long q = B.id * (long long)blockDim.x + threadIdx.x;
  if (q >= g.Nq) return;
  int ix, iy, iz;
  q_coords(g, q, ix, iy, iz);
  const double* F[3] = {F0, F1, F2};
  const double dti = *dt_ptr * w_i;
  double u[V], un[V], dudt[V];
#pragma unroll
  for (int v = 0; v < V; ++v) u[v] = U_cv[(long long)v * g.Nq + q];
#pragma unroll
  for (int v = 0; v < V; ++v) flux_divergence<D>(g, fg, ix, iy, iz, F, v, dudt[v]);
  if (gphi != nullptr) potential_source<D>(g, gphi, q, u, dudt);
#pragma unroll
  for (int v = 0; v < V; ++v) {
    un[v] = u[v] - dudt[v] * dti;
    U_new[(long long)v * g.Nq + q] = un[v];
  }
  if (write_ext) {
    const long long e = ext_of<D>(g, ix, iy, iz);
    double W[V];
    if (write_ext == 2) {
#pragma unroll
      for (int v = 0; v < V; ++v) W[v] = ext_new[(long long)v * g.Nqe + e];
    } else {
      prims_cv<D>(g, u, W, Ueq, Weq, q);
    }
#pragma unroll
    for (int v = 0; v < V; ++v) ext_old[(long long)v * g.Nqe + e] = W[v];
    prims_cv<D>(g, un, W, Ueq, Weq, q);
#pragma unroll
    for (int v = 0; v < V; ++v) ext_new[(long long)v * g.Nqe + e] = W[v];
  }
}
};
template <int D>
__global__ void k_fv_candidate(Geo g, FvGeo fg, const double* __restrict__ dt_ptr, double w_i,
                               const double* F0, const double* F1, const double* F2,
                               const double* __restrict__ U_cv, double* __restrict__ U_new, double* ext_old,
                               double* ext_new, int write_ext, const double* __restrict__ gphi,
                               const double* __restrict__ Ueq, const double* __restrict__ Weq) {
  FvCandidate<D>::run(hw_blk(), g, fg, dt_ptr, w_i, F0, F1, F2, U_cv, U_new, ext_old, ext_new, write_ext, gphi, Ueq,
                      Weq);
}

// W_cv (subcell layout) from the active region of an extended primitive
// array: the end-of-step primitives when ext_new holds prim of the final
// subcell state (src/sdader_simulator.py:351-359 computed once, in the last
// substep's candidate update and corrected update)
template <int D>
struct ExtToPlain {
  static __device__ __forceinline__ void run(Blk B, const Geo& g, const double* __restrict__ ext,
                                             double* __restrict__ W_cv) {
    constexpr int V = D + 2;
    const long long q = B.id * (long long)blockDim.x + threadIdx.x;
    if (q >= g.Nq) return;
    int ix, iy, iz;
    q_coords(g, q, ix, iy, iz);
    const long long e = ext_of<D>(g, ix, iy, iz);
#pragma unroll
    for (int v = 0; v < V; ++v) W_cv[(long long)v * g.Nq + q] = ext[(long long)v * g.Nqe + e];
  }
};
template <int D>
__global__ void k_ext_to_plain(Geo g, const double* __restrict__ ext, double* __restrict__ W_cv) {
  ExtToPlain<D>::run(hw_blk(), g, ext, W_cv);
}

// ghost fill of one direction (src/fv_simulator.py:224-273): store the
// boundary buffer when the reference does, then copy it into the ghost
// layers.  bcbuf layout [side][v][g][other], other = the extended index of
// the remaining directions (lower direction fastest).  When ``gate`` is
// non-null the fill runs only if *gate != 0.
template <int D>
struct Ghost {
static __device__ __forceinline__ void run(Blk B, const Geo& g, int d, int all, int nv, int nv_buf, double* ext,
                                           double* bcbuf, const int* gate) {
  if (gate != nullptr && *gate == 0) return;
  const int o0 = (d == 0) ? 1 : 0;
  const int o1 = (d == 2) ? 1 : 2;
  const long long nother = (long long)g.Xe[o0] * g.Xe[o1];
  const long long total = 2LL * nv * NGH * nother;
  const long long tid = B.id * (long long)blockDim.x + threadIdx.x;
  if (tid >= total) return;
  const long long other = tid % nother;
  long long r = tid / nother;
  const int gi = (int)(r % NGH);
  r /= NGH;
  const int v = (int)(r % nv);
  const int side = (int)(r / nv);
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
  const long long bidx = (((long long)side * nv_buf + v) * NGH + gi) * nother + other;
  double val;
  bool store = false;
  int src = 0;
  if (kind == BC_PERIODIC) { store = true; src = (side == 0) ? Xd + gi : NGH + gi; }
  else if ((kind == BC_REFLECTIVE || kind == BC_GRADFREE) && all) { store = true; src = (side == 0) ? NGH + gi : Xd + gi; }
  if (store) {
    val = ext[(long long)v * g.Nqe + ext_index(src)];
    if (kind == BC_REFLECTIVE && v == d + 1) val = val * -1.0;
    bcbuf[bidx] = val;
  } else if (kind == BC_EQ && all) {
    val = 0.0;
    bcbuf[bidx] = val;
  } else {
    val = bcbuf[bidx];
  }
  const int dst = (side == 0) ? gi : Xd + NGH + gi;
  ext[(long long)v * g.Nqe + ext_index(dst)] = val;
}
};
template <int D>
__global__ void k_ghost(Geo g, int d, int all, int nv, int nv_buf, double* ext, double* bcbuf, const int* gate) {
  Ghost<D>::run(hw_blk(), g, d, all, nv, nv_buf, ext, bcbuf, gate);
}

// NAD: relaxed discrete maximum principle over the cross stencil
// (src/trouble_detection.py:14-38).  mask bit v = possible trouble of var v.
template <int D>
struct Nad {
// With sed_list non-null, the flagged (subcell, density / pressure) pairs
// are also appended to sed_list (item 2*q + is_pressure) for k_sed.
static __device__ __forceinline__ void run(Blk B, const Geo& g, double tol, int delta, int relax,
                                           const double* __restrict__ ext_old, const double* __restrict__ ext_new,
                                           unsigned char* __restrict__ mask, int* any_flag,
                                           long long* __restrict__ sed_list, unsigned long long* __restrict__ sed_count) {
  constexpr int V = D + 2;
  const long long q = B.id * (long long)blockDim.x + threadIdx.x;
  unsigned int m = 0;
  if (q < g.Nq) {
    int ix, iy, iz;
    q_coords(g, q, ix, iy, iz);
    const long long e = ext_of<D>(g, ix, iy, iz);
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const double* W = ext_old + (long long)v * g.Nqe;
      // maximum / minimum of the cross stencil on order-preserving integer
      // keys (integer pipes; the FP64 pipe is the step's bottleneck).  A NaN
      // anywhere makes NumPy's maximum/minimum NaN and the point troubled.
      const double c0 = W[e];
      bool nan = is_nan_bits(c0);
      long long kmx = order_key(c0), kmn = kmx;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const long long st = ext_stride(g, d);
        const double a = W[e - st], b = W[e + st];
        nan = nan || is_nan_bits(a) || is_nan_bits(b);
        const long long ka = order_key(a), kb = order_key(b);
        kmx = max(kmx, max(ka, kb));
        kmn = min(kmn, min(ka, kb));
      }
      double mx = from_order_key(kmx), mn = from_order_key(kmn);
      if (relax) {
        if (delta) {
          const double eps = tol * (mx - mn);
          mn = mn - eps;
          mx = mx + eps;
        } else {
          mn = mn - abs_bits(mn) * tol;
          mx = mx + abs_bits(mx) * tol;
        }
      }
      const double wn = ext_new[(long long)v * g.Nqe + e];
      // !(wn >= mn) || !(wn <= mx) on the integer keys: true when any of the
      // three is NaN, else the ordered comparison (the keys equate -0, +0)
      const long long kw = order_key(wn);
      const bool pt = nan || is_nan_bits(wn) || is_nan_bits(mn) || is_nan_bits(mx) || kw < order_key(mn) ||
                      kw > order_key(mx);
      m |= (pt ? 1u : 0u) << v;
    }
    mask[q] = (unsigned char)m;
  }
  const unsigned ballot = __ballot_sync(0xffffffffu, m != 0);
  if (ballot != 0 && (threadIdx.x & 31) == 0) atomicOr(any_flag, 1);
  if (sed_list != nullptr && ballot != 0) {
    constexpr int P_ = D + 1;
    const bool f0 = m & 1u, fP = (m >> P_) & 1u;
    const unsigned b0 = __ballot_sync(0xffffffffu, f0), bP = __ballot_sync(0xffffffffu, fP);
    if (b0 | bP) {
      const int lane = threadIdx.x & 31;
      const unsigned lt = (1u << lane) - 1u;
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(sed_count, (unsigned long long)(__popc(b0) + __popc(bP)));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (f0) sed_list[base + __popc(b0 & lt)] = 2 * q;
      if (fP) sed_list[base + __popc(b0) + __popc(bP & lt)] = 2 * q + 1;
    }
  }
}
};
template <int D>
__global__ void k_nad(Geo g, double tol, int delta, int relax, const double* __restrict__ ext_old,
                      const double* __restrict__ ext_new, unsigned char* __restrict__ mask, int* any_flag,
                      long long* __restrict__ sed_list, unsigned long long* __restrict__ sed_count) {
  Nad<D>::run(hw_blk(), g, tol, delta, relax, ext_old, ext_new, mask, any_flag, sed_list, sed_count);
}

// smooth-extrema relaxation factor of one variable along direction d at
// active subcell i (src/trouble_detection.py:104-137, including its
// one-sided minimum at the first and last active subcell).
__device__ __forceinline__ double sed_alpha_dir(const double* W, long long e0, long long st, int i, int Xd,
                                                const double* c2, const double* rc2, const double* hfp) {
  // line accessors in extended coordinates j along d; c2[j] = cen[j+1] -
  // cen[j-1] and rc2[j] its correctly rounded reciprocal (the quotients
  // below are the IEEE ones, div_rcp)
  auto U = [&](int j) { return W[e0 + (long long)j * st]; };
  const int k = i + NGH;
  const int lo = (i == 0) ? k - 1 : k - 2;
  const int hi = (i == Xd - 1) ? k + 1 : k + 2;
  double dUs[5];
#pragma unroll
  for (int o = 0; o < 5; ++o) {
    const int j = k - 2 + o;
    if (j >= lo && j <= hi) dUs[o] = div_rcp(U(j + 1) - U(j - 1), c2[j], rc2[j]);
  }
  auto dU = [&](int j) { return dUs[j - (k - 2)]; };
  auto aLR = [&](int kk, double& aL, double& aR) {
    const double dUm = dU(kk - 1), dU0 = dU(kk), dUp = dU(kk + 1);
    const double d2U = div_rcp(dUp - dUm, c2[kk], rc2[kk]);
    const double dv = 0.5 * hfp[kk] * d2U;
    const double rdv = 1.0 / dv;
    const double vL = dUm - dU0;
    const double vR = dUp - dU0;
    // comparisons on the integer keys / words (IEEE semantics)
    const double selL = fgt(0.0, dv) ? (fgt(vL, 0.0) ? vL : 0.0) : (fgt(0.0, vL) ? vL : 0.0);
    aL = div_rcp(-selL, dv, rdv);
    if (!nonzero_w(dv)) aL = 1.0;  // |dv| <= 0
    aL = fgt(1.0, aL) ? aL : 1.0;
    const double selR = fgt(dv, 0.0) ? (fgt(vR, 0.0) ? vR : 0.0) : (fgt(0.0, vR) ? vR : 0.0);
    aR = div_rcp(selR, dv, rdv);
    if (!nonzero_w(dv)) aR = 1.0;
    aR = fgt(1.0, aR) ? aR : 1.0;
  };
  auto A = [&](int kk) {
    double aL, aR;
    aLR(kk, aL, aR);
    return fgt(aL, aR) ? aR : aL;
  };
  if (i == 0) return np_min(A(k), A(k + 1));
  if (i == Xd - 1) {
    double aL, aR;
    aLR(k, aL, aR);
    return np_min(A(k - 1), aL);
  }
  return np_min(A(k - 1), np_min(A(k), A(k + 1)));
}

// SED (k_sed) and the trouble flags with PAD (k_troubles),
// src/trouble_detection.py:40-70.
template <int D>
struct Sed {
// smooth-extrema relaxation of the NAD flags of density and pressure: one
// list item per flagged (subcell, variable) pair, item = 2*q + (variable is
// pressure), compacted by k_nad so that this FP64 work runs on full warps.
// A pair whose smoothness indicator alpha is not < 1 clears its bit of the
// NAD mask (bytes of one 32-bit word may belong to other items, hence the
// atomic AND).
static __device__ __forceinline__ void run(Blk B, const Geo& g, const FvGeo& fg, const long long* __restrict__ list,
                                           const unsigned long long* __restrict__ count,
                                           const double* __restrict__ ext_new, unsigned char* mask) {
  constexpr int P_ = D + 1;
  const unsigned long long cnt = *count;
  for (unsigned long long idx = B.id * (unsigned long long)blockDim.x + threadIdx.x; idx < cnt;
       idx += (unsigned long long)B.n * blockDim.x) {
    const long long item = list[idx];
    const long long q = item >> 1;
    const int var = (item & 1) ? P_ : 0;
    int ix, iy, iz;
    q_coords(g, q, ix, iy, iz);
    const long long e = ext_of<D>(g, ix, iy, iz);
    const int ii[3] = {ix, iy, iz};
    const double* W = ext_new + (long long)var * g.Nqe;
    double alpha = W[e] * 0.0 + 1.0;
    for (int d = 0; d < D; ++d) {
      const long long st = ext_stride(g, d);
      const long long e0 = e - (long long)(ii[d] + NGH) * st;
      const double an = sed_alpha_dir(W, e0, st, ii[d], g.X[d], fg.c2[d], fg.rc2[d], fg.hfp[d]);
      alpha = (an < alpha) ? an : alpha;
    }
    if (!(alpha < 1.0))
      atomicAnd(reinterpret_cast<unsigned*>(mask) + (q >> 2), ~(1u << (8 * (unsigned)(q & 3) + var)));
  }
}
};
template <int D>
__global__ void k_sed(Geo g, FvGeo fg, const long long* __restrict__ list, const unsigned long long* __restrict__ count,
                      const double* __restrict__ ext_new, unsigned char* mask) {
  Sed<D>::run(hw_blk(), g, fg, list, count, ext_new, mask);
}

// trouble flags (NAD flags of density or pressure after the smooth-extrema
// relaxation) and PAD; writes the troubles into var 0 of the theta-source
// extended array and the troubles array.
template <int D>
struct Troubles {
static __device__ __forceinline__ void run(Blk B, const Geo& g, int pad, double min_rho, double max_rho, double min_P,
                                           const unsigned char* __restrict__ mask,
                                           const double* __restrict__ ext_new, double* __restrict__ theta_src,
                                           double* __restrict__ troubles, const double* __restrict__ Weq) {
  constexpr int P_ = D + 1;
  const long long q = B.id * (long long)blockDim.x + threadIdx.x;
  if (q >= g.Nq) return;
  int ix, iy, iz;
  q_coords(g, q, ix, iy, iz);
  const long long e = ext_of<D>(g, ix, iy, iz);
  const unsigned m = mask[q];
  const int pt0 = m & 1u, ptP = (m >> P_) & 1u;
  // max(pt0, ptP) as a double: constants, no conversion on the FP64 pipe
  double t = (pt0 | ptP) ? 1.0 : 0.0;
  if (pad) {
    double r = ext_new[e];
    double P = ext_new[(long long)P_ * g.Nqe + e];
    if (Weq) {
      // the full state's primitives (src/trouble_detection.py:59-60)
      r = r + Weq[q];
      P = P + Weq[(long long)P_ * g.Nq + q];
    }
    // comparisons on the integer keys (IEEE semantics: NaN fails them)
    t = fge(r, min_rho) ? t : 1.0;
    t = fge(max_rho, r) ? t : 1.0;
    t = fge(P, min_P) ? t : 1.0;
  }
  theta_src[e] = t;
  troubles[q] = t;
}
};
template <int D>
__global__ void k_troubles(Geo g, int pad, double min_rho, double max_rho, double min_P,
                           const unsigned char* __restrict__ mask, const double* __restrict__ ext_new,
                           double* __restrict__ theta_src, double* __restrict__ troubles,
                           const double* __restrict__ Weq) {
  Troubles<D>::run(hw_blk(), g, pad, min_rho, max_rho, min_P, mask, ext_new, theta_src, troubles, Weq);
}

// extended-grid coordinates
__device__ __forceinline__ void e_coords(const Geo& g, long long e, int& xe, int& ye, int& ze) {
  xe = (int)(e % g.Xe[0]);
  long long r = e / g.Xe[0];
  ye = (int)(r % g.Xe[1]);
  ze = (int)(r / g.Xe[1]);
}

// first / second (/ third) neighbour blending (src/trouble_detection.py:
// 139-164); the 3D neighbour pairs are those the reference's index tuples
// select.
template <int D>
struct BlendNeighbours {
static __device__ __forceinline__ void run(Blk B, const Geo& g, const double* __restrict__ src,
                                           double* __restrict__ out) {
  const long long e = B.id * (long long)blockDim.x + threadIdx.x;
  if (e >= g.Nqe) return;
  int c[3];
  e_coords(g, e, c[0], c[1], c[2]);
  auto at = [&](int x, int y, int z) { return src[x + (long long)g.Xe[0] * (y + (long long)g.Xe[1] * z)]; };
  auto inb = [&](int d, int v) { return v >= 0 && v < g.Xe[d]; };
  double th = src[e];
  for (int d = 0; d < D; ++d) {
    for (int s = -1; s <= 1; s += 2) {
      int cc[3] = {c[0], c[1], c[2]};
      cc[d] += s;
      if (inb(d, cc[d])) th = np_max_key(0.75 * at(cc[0], cc[1], cc[2]), th);
    }
  }
  if (D == 2) {
    for (int sy = -1; sy <= 1; sy += 2)
      for (int sx = -1; sx <= 1; sx += 2)
        if (inb(0, c[0] + sx) && inb(1, c[1] + sy)) th = np_max_key(0.5 * at(c[0] + sx, c[1] + sy, 0), th);
  } else if (D == 3) {
    // (axis pair, offsets) per (i, idim); axes listed as (first, second)
    // cut axis; offset 0 with range e < last (cut a) or e >= 1 (cut b)
    const int axes[3][2] = {{1, 0}, {2, 1}, {0, 2}};  // idim 0: (y,x); 1: (z,y); 2: (x,z)
    // per i: (offset, cutkind) for the first and the second cut axis;
    // cutkind 0 = a (target e < last), 1 = b (target e >= 1)
    const int offs[4][2] = {{+1, +1}, {0, -1}, {-1, +1}, {0, -1}};
    const int kinds[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};
    for (int i = 0; i < 4; ++i) {
      for (int idim = 0; idim < 3; ++idim) {
        bool ok = true;
        int cc[3] = {c[0], c[1], c[2]};
        for (int k2 = 0; k2 < 2; ++k2) {
          const int ax = axes[idim][k2];
          const int last = g.Xe[ax] - 1;
          if (kinds[i][k2] == 0 && c[ax] >= last) ok = false;
          if (kinds[i][k2] == 1 && c[ax] < 1) ok = false;
          cc[ax] += offs[i][k2];
        }
        if (ok) th = np_max_key(0.5 * at(cc[0], cc[1], cc[2]), th);
      }
    }
    // third neighbours: offsets on (z, y, x)
    const int t3[4][3] = {{+1, +1, +1}, {+1, +1, -1}, {+1, -1, +1}, {+1, -1, -1}};
    for (int i = 0; i < 4; ++i) {
      const int oz = t3[i][0], oy = t3[i][1], ox = t3[i][2];
      const bool ok = (oz > 0 ? c[2] < g.Xe[2] - 1 : c[2] >= 1) && (oy > 0 ? c[1] < g.Xe[1] - 1 : c[1] >= 1) &&
                      (ox > 0 ? c[0] < g.Xe[0] - 1 : c[0] >= 1);
      if (ok) th = np_max_key(0.375 * at(c[0] + ox, c[1] + oy, c[2] + oz), th);
    }
  }
  out[e] = th;
}
};
template <int D>
__global__ void k_blend_neighbours(Geo g, const double* __restrict__ src, double* __restrict__ out) {
  BlendNeighbours<D>::run(hw_blk(), g, src, out);
}

// last blending layer along direction d (src/trouble_detection.py:167-169):
// two sequential in-place sweeps, fused with a one-cell halo.
template <int D>
struct BlendLast {
static __device__ __forceinline__ void run(Blk B, const Geo& g, int d, const double* __restrict__ in,
                                           double* __restrict__ out) {
  const long long e = B.id * (long long)blockDim.x + threadIdx.x;
  if (e >= g.Nqe) return;
  int c[3];
  e_coords(g, e, c[0], c[1], c[2]);
  const long long st = ext_stride(g, d);
  const int last = g.Xe[d] - 1;
  auto th_a = [&](int k, long long ek) {  // after the first sweep
    const double t = in[ek];
    if (k < last) return np_max_key(gt0_key(in[ek + st]) ? 0.25 : 0.0, t);
    return t;
  };
  const int k = c[d];
  const double a0 = th_a(k, e);
  if (k >= 1) {
    const double am = th_a(k - 1, e - st);
    out[e] = np_max_key(gt0_key(am) ? 0.25 : 0.0, a0);
  } else {
    out[e] = a0;
  }
}
};
template <int D>
__global__ void k_blend_last(Geo g, int d, const double* __restrict__ in, double* __restrict__ out) {
  BlendLast<D>::run(hw_blk(), g, d, in, out);
}

// affected faces of direction d (src/trouble_detection.py:81-87) and the
// marks for the fallback fluxes and the corrected update.  With theta ==
// nullptr the affected faces already in ``aff`` are used (replayed
// decisions).
template <int D>
struct Affected {
static __device__ __forceinline__ void run(Blk B, const Geo& g, int d, int godunov, const double* __restrict__ theta,
                                           double* __restrict__ aff, unsigned char* __restrict__ mark_cell,
                                           unsigned char* __restrict__ mark_q, int* __restrict__ nmarked,
                                           long long* __restrict__ flist, unsigned long long* __restrict__ fcount) {
  const long long nf = n_faces(g, d);
  const long long fidx = B.id * (long long)blockDim.x + threadIdx.x;
  bool need = false;
  if (fidx < nf) {
    const int FX = g.X[0] + (d == 0), FY = g.X[1] + (d == 1);
    int f[3];
    f[0] = (int)(fidx % FX);
    long long r = fidx / FX;
    f[1] = (int)(r % FY);
    f[2] = (int)(r / FY);
    int e1[3], e2[3];
    for (int k = 0; k < 3; ++k) {
      const int base = (k < D) ? f[k] + NGH : 0;
      e1[k] = base;
      e2[k] = base;
    }
    e1[d] = f[d] + 1;
    e2[d] = f[d] + 2;
    const long long i1 = e1[0] + (long long)g.Xe[0] * (e1[1] + (long long)g.Xe[1] * e1[2]);
    const long long i2 = e2[0] + (long long)g.Xe[0] * (e2[1] + (long long)g.Xe[1] * e2[2]);
    double a;
    if (theta) {
      a = np_max_key(theta[i1], theta[i2]);
      aff[fidx] = a;
    } else {
      a = aff[fidx];
    }
    need = godunov || nonzero_bits(a);
    if (need) {
      mark_cell[i1] = 1;
      mark_cell[i2] = 1;
      int q[3] = {f[0], f[1], f[2]};
      if (f[d] >= 1) {
        q[d] = f[d] - 1;
        mark_q[q[0] + (long long)g.X[0] * (q[1] + (long long)g.X[1] * q[2])] = 1;
      }
      if (f[d] < g.X[d]) {
        q[d] = f[d];
        mark_q[q[0] + (long long)g.X[0] * (q[1] + (long long)g.X[1] * q[2])] = 1;
      }
    }
  }
  const unsigned b = __ballot_sync(0xffffffffu, need);
  if (b != 0) {
    // the faces that need a fallback flux, compacted by warp ballot: an FP64
    // warp instruction costs the same with 1 or 32 active lanes, so the
    // fallback Riemann problems run on full warps over this list
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == 0) {
      atomicAdd(nmarked, __popc(b));
      base = atomicAdd(fcount, (unsigned long long)__popc(b));
    }
    base = __shfl_sync(0xffffffffu, base, 0);
    if (need) flist[base + __popc(b & ((1u << lane) - 1u))] = fidx;
  }
}
};
template <int D>
__global__ void k_affected(Geo g, int d, int godunov, const double* __restrict__ theta, double* __restrict__ aff,
                           unsigned char* __restrict__ mark_cell, unsigned char* __restrict__ mark_q,
                           int* __restrict__ nmarked, long long* __restrict__ flist,
                           unsigned long long* __restrict__ fcount) {
  Affected<D>::run(hw_blk(), g, d, godunov, theta, aff, mark_cell, mark_q, nmarked, flist, fcount);
}

// compaction of marked indices by warp ballot: writes the marked indices
// into list and their count into *count.
// Appends ``value`` of every lane with ``keep`` to list (order within the
// list unspecified), one atomic per warp.  All 32 lanes of the warp must
// call it.
__device__ __forceinline__ void warp_append(bool keep, long long value, long long* __restrict__ list,
                                            unsigned long long* __restrict__ count) {
  const unsigned b = __ballot_sync(0xffffffffu, keep);
  if (b == 0) return;
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(b));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (keep) list[base + __popc(b & ((1u << lane) - 1u))] = value;
}

struct Compact {
  static __device__ __forceinline__ void run(Blk B, long long total, const unsigned char* __restrict__ mark,
                                             long long* __restrict__ list, unsigned long long* __restrict__ count) {
    const long long i = B.id * (long long)blockDim.x + threadIdx.x;
    const bool m = (i < total) && mark[i];
    const unsigned b = __ballot_sync(0xffffffffu, m);
    if (b == 0) return;
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(b));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (m) list[base + __popc(b & ((1u << lane) - 1u))] = i;
  }
};
static __global__ void k_compact(long long total, const unsigned char* __restrict__ mark, long long* __restrict__ list,
                          unsigned long long* __restrict__ count) {
  Compact::run(hw_blk(), total, mark, list, count);
}

// MUSCL-Hancock: limited gradients, slopes and the half-step primitive
// predictor of one extended subcell (src/muscl.py:61-75,129-173,175-216).
template <int D, int BM = 0>
struct MusclCells {
static __device__ __forceinline__ void run(Blk B, const Geo& g, const FvGeo& fg, int limiter,
                                           const double* __restrict__ dt_ptr, double w_i,
                                           const long long* __restrict__ list,
                                           const unsigned long long* __restrict__ count,
                                           const double* __restrict__ W_ext, double* __restrict__ Mpred,
                                           double* __restrict__ S, unsigned char* ltape,
                                           const double* __restrict__ Meq, const double* __restrict__ gphi) {
  constexpr int V = D + 2, P_ = D + 1;
  const unsigned long long cnt = *count;
  const double dti = *dt_ptr * w_i;
  const bool wb = Meq != nullptr;
  for (unsigned long long idx = B.id * (unsigned long long)blockDim.x + threadIdx.x; idx < cnt;
       idx += (unsigned long long)B.n * blockDim.x) {
  const long long e = list[idx];
  int c[3];
  e_coords(g, e, c[0], c[1], c[2]);
  double W[V], dMh[3][V], dMq[3][V];
#pragma unroll
  for (int v = 0; v < V; ++v) W[v] = W_ext[(long long)v * g.Nqe + e];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const long long st = ext_stride(g, d);
    const int k = c[d];
    const double hl = fg.hcv[d][k - 1], hr = fg.hcv[d][k], hm = fg.hfp[d][k];
    const double rhl = fg.rhcv[d][k - 1], rhr = fg.rhcv[d][k];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const double* M = W_ext + (long long)v * g.Nqe;
      const double SL = div_rcp(M[e] - M[e - st], hl, rhl);
      const double SR = div_rcp(M[e + st] - M[e], hr, rhr);
      double dm;
      if (BM == 0) dm = (limiter == LIM_MINMOD) ? minmod(SL, SR) : moncen(SL, SR, hl, hr, hm);
      else dm = limiter_br<BM>(limiter, SL, SR, hl, hr, hm, &ltape[((long long)d * V + v) * g.Nqe + e]);
      dMh[d][v] = dm;
      S[((long long)d * V + v) * g.Nqe + e] = 0.5 * dm * hm;
      if (wb) {
        // the equilibrium's limited gradient (src/muscl.py:203-204)
        const double* Q = Meq + (long long)v * g.Nqe;
        const double QL = div_rcp(Q[e] - Q[e - st], hl, rhl);
        const double QR = div_rcp(Q[e + st] - Q[e], hr, rhr);
        dMq[d][v] = (limiter == LIM_MINMOD) ? minmod(QL, QR) : moncen(QL, QR, hl, hr, hm);
      }
    }
  }
  // the prediction takes the full state in the well-balanced mode
  // (src/muscl.py:205-207); the state it is added to is (M + M_eq) - M_eq
  double Wf[V];
#pragma unroll
  for (int v = 0; v < V; ++v) Wf[v] = wb ? W[v] + Meq[(long long)v * g.Nqe + e] : W[v];
  double dtW[V];
#pragma unroll
  for (int v = 0; v < V; ++v) dtW[v] = 0.0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const int vel = d + 1;
    const double* dW = dMh[d];
    dtW[0] = dtW[0] - (Wf[vel] * dW[0] + Wf[0] * dW[vel]);
    dtW[P_] = dtW[P_] - (Wf[vel] * dW[P_] + g.gamma * Wf[P_] * dW[vel]);
    dtW[vel] = dtW[vel] - (Wf[vel] * dW[vel] + dW[P_] / Wf[0]);
    if (wb) {
      // src/muscl.py:167-170; the transverse terms then use the
      // equilibrium gradient, as the reference's reassigned dW does
      dW = dMq[d];
      dtW[0] = dtW[0] - (Wf[vel] * dW[0]);
      dtW[P_] = dtW[P_] - (Wf[vel] * dW[P_]);
    }
#pragma unroll
    for (int v2 = 2; v2 <= D; ++v2) dtW[v2] = dtW[v2] - Wf[vel] * dW[v2];
  }
  dtW[P_] = dtW[P_] * 0.0;
  if (wb && gphi != nullptr) {
    // gravity in the prediction (src/muscl.py:208-212), active subcells only
    bool active = true;
#pragma unroll
    for (int d = 0; d < D; ++d) active = active && c[d] >= NGH && c[d] < NGH + g.X[d];
    if (active) {
      const double drho = (Wf[0] - Meq[e]) / Wf[0];
      const long long q = (c[0] - NGH) + (long long)g.X[0] * ((D > 1 ? c[1] - NGH : 0) +
                                                            (long long)g.X[1] * (D > 2 ? c[2] - NGH : 0));
#pragma unroll
      for (int d = 0; d < D; ++d) dtW[d + 1] = dtW[d + 1] + drho * gphi[(long long)d * g.Nq + q];
    }
  }
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const double base = wb ? Wf[v] - Meq[(long long)v * g.Nqe + e] : W[v];
    Mpred[(long long)v * g.Nqe + e] = base + 0.5 * dtW[v] * dti;
  }
  }
}
};
template <int D, int BM = 0>
__global__ void k_muscl_cells(Geo g, FvGeo fg, int limiter, const double* __restrict__ dt_ptr, double w_i,
                              const long long* __restrict__ list, const unsigned long long* __restrict__ count,
                              const double* __restrict__ W_ext, double* __restrict__ Mpred, double* __restrict__ S,
                              unsigned char* ltape, const double* __restrict__ Meq, const double* __restrict__ gphi) {
  MusclCells<D, BM>::run(hw_blk(), g, fg, limiter, dt_ptr, w_i, list, count, W_ext, Mpred, S, ltape, Meq, gphi);
}

// fallback Riemann flux on the affected faces of direction d
// (src/muscl.py:217-221, src/fv_simulator.py:88-165)
template <int D, int BM = 0>
struct MusclFaces {
// the affected faces of direction d from their compacted list (k_affected),
// a grid-stride loop over full warps
static __device__ __forceinline__ void run(Blk B, const Geo& g, int d, int solver,
                                           const long long* __restrict__ flist,
                                           const unsigned long long* __restrict__ fcount,
                                           const double* __restrict__ Mpred, const double* __restrict__ S,
                                           double* __restrict__ F_FB, unsigned* ftape,
                                           const double* __restrict__ Mq, const double* __restrict__ Fq) {
  const unsigned long long cnt = *fcount;
  for (unsigned long long idx = B.id * (unsigned long long)blockDim.x + threadIdx.x; idx < cnt;
       idx += (unsigned long long)B.n * blockDim.x)
    face(g, d, solver, flist[idx], Mpred, S, F_FB, ftape, Mq, Fq);
}
// Mq, Fq (well-balanced mode): the equilibrium's primitive state and flux
// at the faces, added to both states and subtracted from the flux
// (src/fv_simulator.py:150-165)
static __device__ __forceinline__ void face(const Geo& g, int d, int solver, long long fidx,
                                            const double* __restrict__ Mpred, const double* __restrict__ S,
                                            double* __restrict__ F_FB, unsigned* ftape,
                                            const double* __restrict__ Mq = nullptr,
                                            const double* __restrict__ Fq = nullptr) {
  constexpr int V = D + 2;
  const long long nf = n_faces(g, d);
  const int FX = g.X[0] + (d == 0), FY = g.X[1] + (d == 1);
  int f[3];
  f[0] = (int)(fidx % FX);
  long long r = fidx / FX;
  f[1] = (int)(r % FY);
  f[2] = (int)(r / FY);
  int e1[3];
  for (int k = 0; k < 3; ++k) e1[k] = (k < D) ? f[k] + NGH : 0;
  e1[d] = f[d] + 1;
  const long long i1 = e1[0] + (long long)g.Xe[0] * (e1[1] + (long long)g.Xe[1] * e1[2]);
  const long long i2 = i1 + ext_stride(g, d);
  double ML[V], MR[V], F[V];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    ML[v] = Mpred[(long long)v * g.Nqe + i1] + S[((long long)d * V + v) * g.Nqe + i1];
    MR[v] = Mpred[(long long)v * g.Nqe + i2] - S[((long long)d * V + v) * g.Nqe + i2];
    if (Mq) {
      MR[v] = MR[v] + Mq[(long long)v * nf + fidx];
      ML[v] = ML[v] + Mq[(long long)v * nf + fidx];
    }
  }
  Br<BM> br;
  if (BM == 2) br.w = ftape[fidx];
  riemann<D, double, BM>(solver, ML, MR, F, g.gamma, g.min_c2, d, true, &br, g.iso != 0);
  if (BM == 1) ftape[fidx] = br.w;
#pragma unroll
  for (int v = 0; v < V; ++v) F_FB[(long long)v * nf + fidx] = Fq ? F[v] - Fq[(long long)v * nf + fidx] : F[v];
}
};
template <int D, int BM = 0>
__global__ void k_muscl_faces(Geo g, int d, int solver, const long long* __restrict__ flist,
                              const unsigned long long* __restrict__ fcount, const double* __restrict__ Mpred,
                              const double* __restrict__ S, double* __restrict__ F_FB, unsigned* ftape,
                              const double* __restrict__ Mq, const double* __restrict__ Fq) {
  MusclFaces<D, BM>::run(hw_blk(), g, d, solver, flist, fcount, Mpred, S, F_FB, ftape, Mq, Fq);
}

// corrected update of the subcells next to an affected face
// (src/sdader_simulator.py:325-331,346)
template <int D>
struct FvCorrect {
static __device__ __forceinline__ void run(Blk B, const Geo& g, const FvGeo& fg, const double* __restrict__ dt_ptr,
                                           double w_i, int godunov, const long long* __restrict__ list,
                                           const unsigned long long* __restrict__ count, const double* F0,
                                           const double* F1, const double* F2, const double* B0, const double* B1,
                                           const double* B2, const double* A0, const double* A1, const double* A2,
                                           const double* __restrict__ U_cv, double* __restrict__ U_new,
                                           double* __restrict__ ext_new, const double* __restrict__ gphi,
                                           const double* __restrict__ Ueq, const double* __restrict__ Weq) {
  constexpr int V = D + 2;
  const unsigned long long cnt = *count;
  const double* FH[3] = {F0, F1, F2};
  const double* FB[3] = {B0, B1, B2};
  const double* AF[3] = {A0, A1, A2};
  const double dti = *dt_ptr * w_i;
  for (unsigned long long idx = B.id * (unsigned long long)blockDim.x + threadIdx.x; idx < cnt;
       idx += (unsigned long long)B.n * blockDim.x) {
  const long long q = list[idx];
  int ix, iy, iz;
  q_coords(g, q, ix, iy, iz);
  const int ii[3] = {ix, iy, iz};
  double un[V], dudt[V], u[V];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    u[v] = U_cv[(long long)v * g.Nq + q];
    double acc = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const long long nf = n_faces(g, d);
      const long long fl = face_id(g, d, ix, iy, iz);
      const long long fr = face_id(g, d, ix + (d == 0), iy + (d == 1), iz + (d == 2));
      double Fv[2];
      const long long fs[2] = {fl, fr};
      for (int s = 0; s < 2; ++s) {
        const double ho = FH[d][(long long)v * nf + fs[s]];
        const double a = AF[d][fs[s]];
        if (godunov) Fv[s] = 1.0 * FB[d][(long long)v * nf + fs[s]] + (1.0 - 1.0) * ho;
        else if (a != 0.0) Fv[s] = a * FB[d][(long long)v * nf + fs[s]] + (1.0 - a) * ho;
        else Fv[s] = ho;
      }
      const double part = div_rcp(Fv[1] - Fv[0], fg.dx[d][ii[d]], fg.rdx[d][ii[d]]);
      acc = (d == 0) ? part : acc + part;
    }
    dudt[v] = acc;
  }
  if (gphi != nullptr) potential_source<D>(g, gphi, q, u, dudt);
#pragma unroll
  for (int v = 0; v < V; ++v) {
    un[v] = u[v] - dudt[v] * dti;
    U_new[(long long)v * g.Nq + q] = un[v];
  }
  if (ext_new != nullptr) {
    // the primitives of the corrected state: the next substep's W_old
    // (k_fv_candidate with write_ext == 2) or, after the last substep, W_cv
    // (k_ext_to_plain)
    double W[V];
    prims_cv<D>(g, un, W, Ueq, Weq, q);
    const long long e = ext_of<D>(g, ix, iy, iz);
#pragma unroll
    for (int v = 0; v < V; ++v) ext_new[(long long)v * g.Nqe + e] = W[v];
  }
  }
}
};
template <int D>
__global__ void k_fv_correct(Geo g, FvGeo fg, const double* __restrict__ dt_ptr, double w_i, int godunov,
                             const long long* __restrict__ list, const unsigned long long* __restrict__ count,
                             const double* F0, const double* F1, const double* F2, const double* B0,
                             const double* B1, const double* B2, const double* A0, const double* A1,
                             const double* A2, const double* __restrict__ U_cv, double* __restrict__ U_new,
                             double* __restrict__ ext_new, const double* __restrict__ gphi,
                             const double* __restrict__ Ueq, const double* __restrict__ Weq) {
  FvCorrect<D>::run(hw_blk(), g, fg, dt_ptr, w_i, godunov, list, count, F0, F1, F2, B0, B1, B2, A0, A1, A2, U_cv,
                    U_new, ext_new, gphi, Ueq, Weq);
}

// Well-balanced mode around the step (src/sdader_simulator.py:363-376):
// sign -1: U_sp -= U_eq_sp before the predictor; sign +1: U_sp += U_eq_sp
// after the update.  One thread per solution-point value.
struct WbShift {
  static __device__ __forceinline__ void run(Blk B, long long n, double sign, double* __restrict__ U_sp,
                                             const double* __restrict__ Ueq) {
    const long long i = B.id * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    U_sp[i] = (sign < 0.0) ? U_sp[i] - Ueq[i] : U_sp[i] + Ueq[i];
  }
};
static __global__ void k_wb_shift(long long n, double sign, double* __restrict__ U_sp, const double* __restrict__ Ueq) {
  WbShift::run(hw_blk(), n, sign, U_sp, Ueq);
}
// U_cv += U_eq_cv, then W_cv = prim(U_cv) (src/sdader_simulator.py:375-376)
template <int D>
struct WbEnd {
  static __device__ __forceinline__ void run(Blk B, const Geo& g, double* __restrict__ U_cv,
                                             const double* __restrict__ Ueq, double* __restrict__ W_cv) {
    constexpr int V = D + 2;
    const long long q = B.id * (long long)blockDim.x + threadIdx.x;
    if (q >= g.Nq) return;
    double u[V], W[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      u[v] = U_cv[(long long)v * g.Nq + q] + Ueq[(long long)v * g.Nq + q];
      U_cv[(long long)v * g.Nq + q] = u[v];
    }
    prim<D>(u, W, g.gamma, 0, (double*)nullptr, g.iso != 0);
#pragma unroll
    for (int v = 0; v < V; ++v) W_cv[(long long)v * g.Nq + q] = W[v];
  }
};
template <int D>
__global__ void k_wb_end(Geo g, double* __restrict__ U_cv, const double* __restrict__ Ueq, double* __restrict__ W_cv) {
  WbEnd<D>::run(hw_blk(), g, U_cv, Ueq, W_cv);
}

// dt = cfl * h / cmax from the reduced maximum of d*c_s + sum |v| (NaN when
// a NaN entered the reduction) (src/sd_simulator.py:214-227)
// dt = cfl * min(h / c_max, h^2 / nu / 4) (src/sd_simulator.py:214-227; the
// viscous limit only when dt_visc >= 0; Python's min keeps its first
// argument unless the second is smaller, so a NaN dt stays NaN)
struct DtFinal {
  static __device__ __forceinline__ void run(Blk, double h, double cfl, const unsigned long long* cmax_bits,
                                             const int* nan_flag, double* dt, double dt_visc) {
    if (threadIdx.x != 0) return;
    const double cmax = *nan_flag ? __longlong_as_double(0x7ff8000000000000LL)
                                  : __longlong_as_double((long long)*cmax_bits);
    double dtt = h / cmax;
    if (dt_visc >= 0.0 && dt_visc < dtt) dtt = dt_visc;
    *dt = cfl * dtt;
  }
};
static __global__ void k_dt_final(double h, double cfl, const unsigned long long* cmax_bits, const int* nan_flag,
                           double* dt, double dt_visc) {
  DtFinal::run(hw_blk(), h, cfl, cmax_bits, nan_flag, dt, dt_visc);
}

}  // namespace spd
