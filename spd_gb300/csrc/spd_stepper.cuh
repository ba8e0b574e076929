// Launch sequence of one SD-ADER step for dimension D and degree P
// (src/sdader_simulator.py:361-378); instantiated per dimension in
// spd_step_d1.cu, spd_step_d2.cu and spd_step_d3.cu.
#pragma once
#include "spd_ctx.cuh"

namespace spd_host {

template <int D, int P>
int adjoint_vjp(spd_ctx* C);

template <int D, int P>
struct CmaxOnly {
static __device__ __forceinline__ void run(Blk B, const Geo& g, const double* __restrict__ W_cv,
                                           unsigned long long* __restrict__ cmax_bits, int* __restrict__ nan_flag) {
  constexpr int P_ = D + 1;
  const long long q = B.id * (long long)blockDim.x + threadIdx.x;
  double cval = 0.0;
  bool isnan_c = false;
  if (q < g.Nq) {
    double c = sound_speed(W_cv[(long long)P_ * g.Nq + q], W_cv[q], g.gamma, g.min_c2) * (double)D;
#pragma unroll
    for (int v = 1; v <= D; ++v) c = c + abs_bits(W_cv[(long long)v * g.Nq + q]);
    if (nan_w(c)) isnan_c = true;
    else cval = c;
  }
  // the warp's maximum (comparisons on the integer keys)
  for (int off = 16; off > 0; off >>= 1) {
    const double o = __shfl_down_sync(0xffffffffu, cval, off);
    cval = fgt(o, cval) ? o : cval;
  }
  const unsigned nb = __ballot_sync(0xffffffffu, isnan_c);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(cmax_bits, (unsigned long long)__double_as_longlong(cval));
    if (nb) atomicOr(nan_flag, 1);
  }
}
};
template <int D, int P>
__global__ void k_cmax_only(Geo g, const double* __restrict__ W_cv, unsigned long long* __restrict__ cmax_bits,
                            int* __restrict__ nan_flag) {
  CmaxOnly<D, P>::run(hw_blk(), g, W_cv, cmax_bits, nan_flag);
}

template <int D>
struct PrimOnly {
  static __device__ __forceinline__ void run(Blk B, const Geo& g, const double* __restrict__ U_cv,
                                             double* __restrict__ W_cv) {
    constexpr int V = D + 2;
    const long long q = B.id * (long long)blockDim.x + threadIdx.x;
    if (q >= g.Nq) return;
    double u[V], W[V];
#pragma unroll
    for (int v = 0; v < V; ++v) u[v] = U_cv[(long long)v * g.Nq + q];
    prim<D>(u, W, g.gamma, 0, (double*)nullptr, g.iso != 0);
#pragma unroll
    for (int v = 0; v < V; ++v) W_cv[(long long)v * g.Nq + q] = W[v];
  }
};
template <int D>
__global__ void k_prim_only(Geo g, const double* __restrict__ U_cv, double* __restrict__ W_cv) {
  PrimOnly<D>::run(hw_blk(), g, U_cv, W_cv);
}


template <int D, int P>
struct Stepper : StepperBase {
  using k = K<D, P>;

  int configure(spd_ctx* C) override {
    // cells per block of the interior kernel: bounded by the 227 KB of shared
    // memory a block may use
    const size_t per_cell = (size_t)k::V * k::NS * C->T * sizeof(double);
    max_cpb = 64;
    while (max_cpb > 1 && per_cell * max_cpb > 227 * 1024) max_cpb /= 2;
    cpb = std::min(32, max_cpb);
    smem = per_cell * max_cpb;
    CK(cudaFuncSetAttribute(k_interior<D, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaFuncSetAttribute(k_interior_ext<D, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return 0;
  }

  // the Riemann problems of one Picard iteration, one instantiation per
  // direction; EQ: the form with the well-balanced mode's equilibrium edge
  // values and the isothermal system
  template <bool EQ>
  void riemann_plain(spd_ctx* C, int d, unsigned nb, int Teff, int solver) {
    const Geo& g = C->geo;
    constexpr int D1 = (D > 1 ? 1 : 0), D2 = (D > 2 ? 2 : 0);
    unsigned* no_tape = nullptr;
    const double* meq = C->Meq_fp[d];
    if (d == 0)
      launch<RiemannSd<D, P, 0, 0, EQ>>(C, "k_riemann_sd", k_riemann_sd<D, P, 0, 0, EQ>, nb, 128, 0, g, d, Teff,
                                        solver, C->trace[d], C->bcfix[d], C->Fi[d], no_tape, meq);
    else if (d == 1)
      launch<RiemannSd<D, P, 0, D1, EQ>>(C, "k_riemann_sd", k_riemann_sd<D, P, 0, D1, EQ>, nb, 128, 0, g, d, Teff,
                                         solver, C->trace[d], C->bcfix[d], C->Fi[d], no_tape, meq);
    else
      launch<RiemannSd<D, P, 0, D2, EQ>>(C, "k_riemann_sd", k_riemann_sd<D, P, 0, D2, EQ>, nb, 128, 0, g, d, Teff,
                                         solver, C->trace[d], C->bcfix[d], C->Fi[d], no_tape, meq);
  }

  // the Riemann problems of one Picard iteration with every branch taped
  // (BM 1) or replayed (BM 2), one instantiation per direction as in the
  // plain form.  The runtime-direction instantiation is not used: on
  // sm_103a its LLF branch returned NaN for every flux in 2D (HLLC, 1D and
  // the same device function called from a plain kernel were exact).
  template <int BM>
  void riemann_taped(spd_ctx* C, int d, unsigned nb, int Teff, int solver, unsigned* tp) {
    const Geo& g = C->geo;
    constexpr int D1 = (D > 1 ? 1 : 0), D2 = (D > 2 ? 2 : 0);
    if (d == 0)
      k_riemann_sd<D, P, BM, 0><<<nb, 128, 0, C->stream>>>(g, d, Teff, solver, C->trace[d], C->bcfix[d], C->Fi[d],
                                                          tp, nullptr);
    else if (d == 1)
      k_riemann_sd<D, P, BM, D1><<<nb, 128, 0, C->stream>>>(g, d, Teff, solver, C->trace[d], C->bcfix[d], C->Fi[d],
                                                           tp, nullptr);
    else
      k_riemann_sd<D, P, BM, D2><<<nb, 128, 0, C->stream>>>(g, d, Teff, solver, C->trace[d], C->bcfix[d], C->Fi[d],
                                                           tp, nullptr);
  }

  int predictor(spd_ctx* C, int final_mode) {
    const Geo& g = C->geo;
    if (C->recording)
      CK(cudaMemcpyAsync(C->hist_usp, C->U_sp, sizeof(double) * k::V * k::NS * g.Nc, cudaMemcpyDeviceToDevice,
                         C->stream));
    {
      ProfScope ps_(C, "k_traces_sp");
      launch<TracesSp<D, P>>(C, "k_traces_sp", k_traces_sp<D, P>, blocks_for(g.Nc, 128), 128, 0, C->ops, g, C->U_sp,
                             C->trace[0], C->trace[1], C->trace[2]);
    }
    CKL();
    const int m = C->T - 1;
    for (int it = 0; it <= m; ++it) {
      const int Teff = (it == 0) ? 1 : C->T;
      const int solver = C->cfg.riemann_solver_sd;
      for (int d = 0; d < D; ++d) {
        const long long tot = (long long)Teff * k::NJ * n_iface(g, d);
        {
          ProfScope ps_(C, "k_riemann_sd");
          if (C->tape_mode == 0) {
            const unsigned nb = blocks_for(tot, 128);
            if (C->Meq_fp[d] || C->cfg.isothermal)
              riemann_plain<true>(C, d, nb, Teff, solver);
            else
              riemann_plain<false>(C, d, nb, Teff, solver);
          } else {
            unsigned* tp = C->tape_rs[d] + ((size_t)C->tape_step * C->T + it) * C->T * k::NJ * n_iface(g, d);
            if (C->tape_mode == 1)
              riemann_taped<1>(C, d, blocks_for(tot, 128), Teff, solver, tp);
            else
              riemann_taped<2>(C, d, blocks_for(tot, 128), Teff, solver, tp);
          }
        }
        CKL();
      }
      const int mode = (it < m) ? 0 : final_mode;
      const double* Uin = (it == 0) ? C->U_sp : C->U_ader;
      const int Tu = (it == 0) ? 1 : C->T;
      const bool visc = C->cfg.viscosity != 0;
      if (visc) {
        // viscous fluxes of this iteration (src/sdader_simulator.py:239-268)
        {
          ProfScope ps_(C, "k_visc_grad");
          launch<ViscGrad<D, P>>(C, "k_visc_grad", k_visc_grad<D, P>, blocks_for(g.Nc * Teff, 128), 128, 0, C->ops,
                                 g, Teff, Uin, Tu, C->trace[0], C->trace[1], C->trace[2], C->bcfix[0], C->bcfix[1],
                                 C->bcfix[2], C->Wfp[0], C->Wfp[1], C->Wfp[2], C->dWsp, (const double*)C->Meq_fp[0],
                                 (const double*)C->Meq_fp[1], (const double*)C->Meq_fp[2]);
        }
        CKL();
        {
          ProfScope ps_(C, "k_visc_flux");
          launch<ViscFlux<D, P>>(C, "k_visc_flux", k_visc_flux<D, P>, blocks_for(g.Nc * Teff, 128), 128, 0, C->ops,
                                 g, Teff, C->dWsp, C->Wfp[0], C->Wfp[1], C->Wfp[2], C->bcfix[0], C->bcfix[1],
                                 C->bcfix[2], C->cfg.nu, C->cfg.beta, C->Gv[0], C->Gv[1], C->Gv[2]);
        }
        CKL();
      }
      // the first Picard iteration computes one time node but writes all T:
      // T thread rows share its output (whole warps per row when cpb is a
      // multiple of 32)
      const int rows = (mode == 0 && Teff == 1 && cpb % 32 == 0) ? C->T : Teff;
      dim3 block(cpb, rows);
      const size_t sm = (mode == 2) ? 0 : (size_t)k::V * k::NS * Teff * cpb * sizeof(double);
      if (visc || C->gphi_sp || C->Ueq_sp || C->cfg.isothermal) {
        ProfScope ps_(C, "k_interior");
        launch<InteriorExt<D, P>>(C, "k_interior", k_interior_ext<D, P>, blocks_for(g.Nc, cpb), block, sm, C->ops,
                                  g, mode, Teff, Uin, Tu, C->dt, C->U_sp, C->U_ader, C->Fi[0], C->Fi[1], C->Fi[2],
                                  C->trace[0], C->trace[1], C->trace[2], C->Ffp[0], C->Ffp[1], C->Ffp[2],
                                  visc ? C->Gv[0] : nullptr, C->Gv[1], C->Gv[2], (const double*)C->gphi_sp,
                                  (const double*)C->Meq_fp[0], (const double*)C->Meq_fp[1],
                                  (const double*)C->Meq_fp[2], (const double*)C->Feq_fp[0],
                                  (const double*)C->Feq_fp[1], (const double*)C->Feq_fp[2]);
      } else {
        ProfScope ps_(C, "k_interior");
        launch<Interior<D, P>>(C, "k_interior", k_interior<D, P>, blocks_for(g.Nc, cpb), block, sm, C->ops, g, mode,
                               Teff, Uin, Tu, C->dt, C->U_sp, C->U_ader, C->Fi[0], C->Fi[1], C->Fi[2], C->trace[0],
                               C->trace[1], C->trace[2], C->Ffp[0], C->Ffp[1], C->Ffp[2]);
      }
      CKL();
      if (C->recording && mode == 0) {
        const size_t n = (size_t)k::V * C->T * k::NS * g.Nc;
        CK(cudaMemcpyAsync(C->hist_ader + (size_t)it * n, C->U_ader, n * sizeof(double), cudaMemcpyDeviceToDevice,
                           C->stream));
      }
    }
    return 0;
  }

  int sp_to_cv(spd_ctx* C) override {
    const Geo& g = C->geo;
    {
      ProfScope ps_(C, "k_sp_to_cv");
      launch<SpToCv<D, P>>(C, "k_sp_to_cv", k_sp_to_cv<D, P>, blocks_for(g.Nc * k::V, 128), 128, 0, g, C->K_sp_to_cv,
                           C->U_sp, C->U_cv);
    }
    CKL();
    return 0;
  }

  int wcv(spd_ctx* C) override {
    const Geo& g = C->geo;
    {
      ProfScope ps_(C, "k_prim_only");
      launch<PrimOnly<D>>(C, "k_prim_only", k_prim_only<D>, blocks_for(g.Nq, BS), BS, 0, g, C->U_cv, C->W_cv);
    }
    CKL();
    return 0;
  }

  int cmax(spd_ctx* C) override {
    const Geo& g = C->geo;
    CK(zero_fill(C, C->flags + 1, sizeof(int)));
    CK(zero_fill(C, C->counts + 2, sizeof(unsigned long long)));
    {
      ProfScope ps_(C, "k_cmax_only");
      launch<CmaxOnly<D, P>>(C, "k_cmax_only", k_cmax_only<D, P>, blocks_for(g.Nq, BS), BS, 0, g, C->W_cv,
                             C->counts + 2, C->flags + 1);
    }
    CKL();
    {
      ProfScope ps_(C, "k_dt_final");
      launch<DtFinal>(C, "k_dt_final", k_dt_final, 1, 1, 0, C->h_dt, C->cfg.cfl_coeff, C->counts + 2, C->flags + 1,
                      C->dt, C->dt_visc);
    }
    CKL();
    return 0;
  }

  // affected faces of all directions per substep in a record slot or tape
  static size_t hist_aff_stride(const spd_ctx* C) {
    size_t per = 0;
    for (int d = 0; d < D; ++d) per += (size_t)n_faces(C->geo, d);
    return per;
  }
  static double* tape_aff(spd_ctx* C, int i) {
    return C->tape_aff + ((size_t)C->tape_step * C->T + i) * hist_aff_stride(C);
  }

  int fv_update(spd_ctx* C) {
    const Geo& g = C->geo;
    const spd_config& cf = C->cfg;
    // switch_to_finite_volume (src/sdader_simulator.py:288-298)
    if (int r = sp_to_cv(C)) return r;
    for (int d = 0; d < D; ++d) {
      {
        ProfScope ps_(C, "k_integrate_faces");
        launch<IntegrateFaces<D, P>>(C, "k_integrate_faces", k_integrate_faces<D, P>,
                                     blocks_for(g.Nc * g.T * k::nf, 128), 128, 0, C->ops, g, d, C->Ffp[d], C->F_HO[d]);
      }
      CKL();
    }
    long long nface[3] = {1, 1, 1};
    for (int d = 0; d < D; ++d) nface[d] = n_faces(g, d);
    for (int i = 0; i < C->T; ++i) {
      const double w_i = C->ops.w_tp[i];
      if (C->recording)
        CK(cudaMemcpyAsync(C->hist_ucv + (size_t)i * k::V * g.Nq, C->U_cv, sizeof(double) * k::V * g.Nq,
                           cudaMemcpyDeviceToDevice, C->stream));
      const double* FH[3] = {nullptr, nullptr, nullptr};
      for (int d = 0; d < D; ++d) FH[d] = C->F_HO[d] + (long long)i * k::V * nface[d];
      {
        ProfScope ps_(C, "k_fv_candidate");
        launch<FvCandidate<D>>(C, "k_fv_candidate", k_fv_candidate<D>, blocks_for(g.Nq, BS), BS, 0, g, C->fvg, C->dt,
                               w_i, FH[0], FH[1], FH[2], C->U_cv, C->U_new, C->ext_old, C->ext_new,
                               cf.FB ? (i == 0 ? 1 : 2) : 0, (const double*)C->gphi_fv, (const double*)C->Ueq_cv,
                               (const double*)C->Weq_cv);
      }
      CKL();
      if (cf.FB && C->tape_mode == 2) {
        // the affected faces of the taped step instead of trouble detection
        size_t off = 0;
        for (int d = 0; d < D; ++d) {
          CK(cudaMemcpyAsync(C->aff[d], tape_aff(C, i) + off, sizeof(double) * nface[d], cudaMemcpyDeviceToDevice,
                             C->stream));
          off += (size_t)nface[d];
        }
        for (int d = 0; d < D; ++d) {
          if (int r = ghost(C, d, 1, k::V, C->ext_old, nullptr)) return r;
        }
      } else if (cf.FB) {
        // detect_troubles (src/trouble_detection.py:5-87)
        for (int d = 0; d < D; ++d) {
          if (int r = ghost(C, d, 1, k::V, C->ext_old, nullptr)) return r;
        }
        const int sed = (P > 1 && cf.SED) ? 1 : 0;
        CK(zero_fill(C, C->flags, sizeof(int)));
        if (sed) CK(zero_fill(C, C->counts + 3, sizeof(unsigned long long)));
        {
          ProfScope ps_(C, "k_nad");
          long long* sed_list = sed ? C->list_sed : nullptr;
          launch<Nad<D>>(C, "k_nad", k_nad<D>, blocks_for(g.Nq, BS), BS, 0, g, cf.tolerance, cf.NAD_delta,
                         P > 0 ? 1 : 0, C->ext_old, C->ext_new, C->mask, C->flags, sed_list, C->counts + 3);
        }
        CKL();
        if (sed) {
          for (int d = 0; d < D; ++d) {
            if (int r = ghost(C, d, 1, k::V, C->ext_new, C->flags)) return r;
          }
          ProfScope ps_(C, "k_sed");
          const unsigned nb = (unsigned)std::min<long long>(PERSIST_BLOCKS, blocks_for(2 * g.Nq, BS));
          launch<Sed<D>>(C, "k_sed", k_sed<D>, nb, BS, 0, g, C->fvg, C->list_sed, C->counts + 3, C->ext_new,
                         C->mask);
          CKL();
        }
        {
          ProfScope ps_(C, "k_troubles");
          launch<Troubles<D>>(C, "k_troubles", k_troubles<D>, blocks_for(g.Nq, BS), BS, 0, g, cf.PAD, cf.min_rho,
                              cf.max_rho, cf.min_P, C->mask, C->ext_new, C->theta_src, C->troubles,
                              (const double*)C->Weq_cv);
        }
        CKL();
        for (int d = 0; d < D; ++d) {
          if (int r = ghost(C, d, 0, 1, C->theta_src, nullptr)) return r;
        }
        double* th = C->theta_src;
        if (cf.blending) {
          {
            ProfScope ps_(C, "k_blend_neighbours");
            launch<BlendNeighbours<D>>(C, "k_blend_neighbours", k_blend_neighbours<D>, blocks_for(g.Nqe, BS), BS, 0, g,
                                       C->theta_src, C->theta_a);
          }
          CKL();
          double* in = C->theta_a;
          double* out = C->theta_b;
          for (int d = 0; d < D; ++d) {
            {
              ProfScope ps_(C, "k_blend_last");
              launch<BlendLast<D>>(C, "k_blend_last", k_blend_last<D>, blocks_for(g.Nqe, BS), BS, 0, g, d, in, out);
            }
            CKL();
            std::swap(in, out);
          }
          th = in;
        }
        C->theta_final = th;
      }
      if (cf.FB) {
        // affected faces, marks and the fallback fluxes (src/sdader_simulator.py:343-346)
        CK(zero_fill(C, C->mark_cell, (size_t)g.Nqe));
        CK(zero_fill(C, C->mark_q, (size_t)g.Nq));
        CK(zero_fill(C, C->counts, 2 * sizeof(unsigned long long)));
        CK(zero_fill(C, C->counts + 4, D * sizeof(unsigned long long)));
        for (int d = 0; d < D; ++d) {
          {
            ProfScope ps_(C, "k_affected");
            const double* th = C->tape_mode == 2 ? nullptr : C->theta_final;
            launch<Affected<D>>(C, "k_affected", k_affected<D>, blocks_for(nface[d], BS), BS, 0, g, d, cf.godunov, th,
                                C->aff[d], C->mark_cell, C->mark_q, C->flags + 2, C->list_face[d],
                                C->counts + 4 + d);
          }
          CKL();
        }
        {
          ProfScope ps_(C, "k_compact");
          launch<Compact>(C, "k_compact", k_compact, blocks_for(g.Nqe, BS), BS, 0, g.Nqe, C->mark_cell, C->list_cell,
                          C->counts);
        }
        CKL();
        {
          ProfScope ps_(C, "k_compact");
          launch<Compact>(C, "k_compact", k_compact, blocks_for(g.Nq, BS), BS, 0, g.Nq, C->mark_q, C->list_q,
                          C->counts + 1);
        }
        CKL();
        if (C->tape_mode == 1) {
          size_t off = 0;
          for (int d = 0; d < D; ++d) {
            CK(cudaMemcpyAsync(tape_aff(C, i) + off, C->aff[d], sizeof(double) * nface[d], cudaMemcpyDeviceToDevice,
                               C->stream));
            off += (size_t)nface[d];
          }
        }
        k_muscl_cells_grid(C, w_i, i);
        CKL();
        if (C->recording) {
          const size_t nq = (size_t)k::V * g.Nqe;
          double* dst = C->hist_mpred + (size_t)i * (1 + D) * nq;
          CK(cudaMemcpyAsync(dst, C->Mpred, sizeof(double) * nq, cudaMemcpyDeviceToDevice, C->stream));
          CK(cudaMemcpyAsync(dst + nq, C->S, sizeof(double) * D * nq, cudaMemcpyDeviceToDevice, C->stream));
        }
        for (int d = 0; d < D; ++d) {
          {
            ProfScope ps_(C, "k_muscl_faces");
            // grid-stride over the compacted list of affected faces
            const unsigned nb = (unsigned)std::min<long long>(PERSIST_BLOCKS, blocks_for(nface[d], BS));
            const unsigned long long* fcount = C->counts + 4 + d;
            if (C->tape_mode == 0) {
              unsigned* no_tape = nullptr;
              launch<MusclFaces<D>>(C, "k_muscl_faces", k_muscl_faces<D>, nb, BS, 0, g, d, cf.riemann_solver_fv,
                                    C->list_face[d], fcount, C->Mpred, C->S, C->F_FB[d], no_tape,
                                    (const double*)C->Meq_faces[d], (const double*)C->Feq_faces[d]);
            } else {
              unsigned* tp = C->tape_fb[d] + ((size_t)C->tape_step * C->T + i) * nface[d];
              if (C->tape_mode == 1)
                k_muscl_faces<D, 1><<<nb, BS, 0, C->stream>>>(g, d, cf.riemann_solver_fv, C->list_face[d], fcount,
                                                             C->Mpred, C->S, C->F_FB[d], tp, nullptr, nullptr);
              else
                k_muscl_faces<D, 2><<<nb, BS, 0, C->stream>>>(g, d, cf.riemann_solver_fv, C->list_face[d], fcount,
                                                             C->Mpred, C->S, C->F_FB[d], tp, nullptr, nullptr);
            }
          }
          CKL();
        }
        k_fv_correct_grid(C, w_i, FH, C->ext_new);
        CKL();
        C->fb_ran = true;
        if (C->recording) {
          size_t off = 0;
          const size_t per = hist_aff_stride(C);
          for (int d = 0; d < D; ++d) {
            CK(cudaMemcpyAsync(C->hist_aff + (size_t)i * per + off, C->aff[d], sizeof(double) * nface[d],
                               cudaMemcpyDeviceToDevice, C->stream));
            off += (size_t)nface[d];
          }
        }
      }
      std::swap(C->U_cv, C->U_new);
    }
    // switch_to_high_order (src/sdader_simulator.py:300-307)
    {
      ProfScope ps_(C, "k_cv_to_sp");
      launch<CvToSp<D, P>>(C, "k_cv_to_sp", k_cv_to_sp<D, P>, blocks_for(g.Nc * k::V, 128), 128, 0, g, C->K_cv_to_sp,
                           C->U_cv, C->U_sp);
    }
    CKL();
    return 0;
  }

  void k_muscl_cells_grid(spd_ctx* C, double w_i, int i) {
    const Geo& g = C->geo;
    const long long nb = std::min<long long>(PERSIST_BLOCKS, blocks_for(g.Nqe, 128));
    ProfScope ps_(C, "k_muscl_cells");
    if (C->tape_mode == 0) {
      unsigned char* no_tape = nullptr;
      launch<MusclCells<D>>(C, "k_muscl_cells", k_muscl_cells<D>, (unsigned)nb, 128, 0, g, C->fvg,
                            C->cfg.slope_limiter, C->dt, w_i, C->list_cell, C->counts, C->ext_old, C->Mpred, C->S,
                            no_tape, (const double*)C->Meq_fv, (const double*)C->gphi_fv);
      return;
    }
    unsigned char* lt = C->tape_lim + ((size_t)C->tape_step * C->T + i) * D * k::V * g.Nqe;
    if (C->tape_mode == 1)
      k_muscl_cells<D, 1><<<(unsigned)nb, 128, 0, C->stream>>>(g, C->fvg, C->cfg.slope_limiter, C->dt, w_i,
                                                               C->list_cell, C->counts, C->ext_old, C->Mpred, C->S, lt,
                                                               nullptr, nullptr);
    else
      k_muscl_cells<D, 2><<<(unsigned)nb, 128, 0, C->stream>>>(g, C->fvg, C->cfg.slope_limiter, C->dt, w_i,
                                                               C->list_cell, C->counts, C->ext_old, C->Mpred, C->S, lt,
                                                               nullptr, nullptr);
  }

  // ext_new non-null: also the primitives of the corrected subcells (the
  // next substep's W_old, or the step's W_cv after the last substep)
  void k_fv_correct_grid(spd_ctx* C, double w_i, const double* const* FH, double* ext_new) {
    const Geo& g = C->geo;
    const long long nb = std::min<long long>(PERSIST_BLOCKS, blocks_for(g.Nq, 128));
    {
      ProfScope ps_(C, "k_fv_correct");
      launch<FvCorrect<D>>(C, "k_fv_correct", k_fv_correct<D>, (unsigned)nb, 128, 0, g, C->fvg, C->dt, w_i,
                           C->cfg.godunov, C->list_q, C->counts + 1, FH[0], FH[1], FH[2], C->F_FB[0], C->F_FB[1],
                           C->F_FB[2], C->aff[0], C->aff[1], C->aff[2], C->U_cv, C->U_new, ext_new,
                           (const double*)C->gphi_fv, (const double*)C->Ueq_cv, (const double*)C->Weq_cv);
    }
  }

  int ghost(spd_ctx* C, int d, int all, int nv, double* ext, const int* gate) {
    const Geo& g = C->geo;
    const int o0 = (d == 0) ? 1 : 0;
    const int o1 = (d == 2) ? 1 : 2;
    const long long tot = 2LL * nv * NGH * g.Xe[o0] * g.Xe[o1];
    {
      ProfScope ps_(C, "k_ghost");
      launch<Ghost<D>>(C, "k_ghost", k_ghost<D>, blocks_for(tot, BS), BS, 0, g, d, all, nv, k::V, ext, C->bcbuf[d],
                       gate);
    }
    CKL();
    return 0;
  }

  // adjoint of the recorded step (spd_adjoint_exec.cuh, compiled in its own
  // translation units)
  int vjp(spd_ctx* C) override { return adjoint_vjp<D, P>(C); }

  // well-balanced mode: U_sp -/+ U_eq_sp around the step
  int wb_shift(spd_ctx* C, double sign) {
    const Geo& g = C->geo;
    const long long n = (long long)k::V * k::NS * g.Nc;
    {
      ProfScope ps_(C, "k_wb_shift");
      launch<WbShift>(C, "k_wb_shift", k_wb_shift, blocks_for(n, BS), BS, 0, n, sign, C->U_sp,
                      (const double*)C->Ueq_sp);
    }
    CKL();
    return 0;
  }

  int eq_prims(spd_ctx* C) override {
    const Geo& g = C->geo;
    {
      ProfScope ps_(C, "k_prim_only");
      launch<PrimOnly<D>>(C, "k_prim_only", k_prim_only<D>, blocks_for(g.Nq, BS), BS, 0, g, C->Ueq_cv, C->Weq_cv);
    }
    CKL();
    return 0;
  }

  int update(spd_ctx* C) override {
    const int final_mode = (C->cfg.update == SPD_UPDATE_SD) ? 1 : 2;
    if (C->Ueq_sp) {
      // src/sdader_simulator.py:363-365, 372-376: the step advances the
      // perturbation; afterwards U_sp += U_eq_sp, U_cv += U_eq_cv (with the
      // SD update U_cv is the previous step's) and W_cv = prim(U_cv)
      if (int r = wb_shift(C, -1.0)) return r;
      if (int r = predictor(C, final_mode)) return r;
      if (C->cfg.update == SPD_UPDATE_FV)
        if (int r = fv_update(C)) return r;
      if (int r = wb_shift(C, 1.0)) return r;
      const Geo& g = C->geo;
      {
        ProfScope ps_(C, "k_wb_end");
        launch<WbEnd<D>>(C, "k_wb_end", k_wb_end<D>, blocks_for(g.Nq, BS), BS, 0, g, C->U_cv,
                         (const double*)C->Ueq_cv, C->W_cv);
      }
      CKL();
      return 0;
    }
    if (int r = predictor(C, final_mode)) return r;
    if (C->cfg.update == SPD_UPDATE_FV) {
      if (int r = fv_update(C)) return r;
      if (C->cfg.FB) {
        // W_cv = prim(U_cv) (src/sdader_simulator.py:376): ext_new already
        // holds it (the last substep's W_new, refreshed where corrected)
        const Geo& g = C->geo;
        {
          ProfScope ps_(C, "k_ext_to_plain");
          launch<ExtToPlain<D>>(C, "k_ext_to_plain", k_ext_to_plain<D>, blocks_for(g.Nq, BS), BS, 0, g, C->ext_new,
                                C->W_cv);
        }
        CKL();
        return 0;
      }
    }
    // W_cv = prim(U_cv) (src/sdader_simulator.py:376)
    return wcv(C);
  }
};

template <int D>
StepperBase* make_stepper_for(int P) {
  switch (P) {
    case 1: return new Stepper<D, 1>();
    case 2: return new Stepper<D, 2>();
    case 3: return new Stepper<D, 3>();
    case 4: return new Stepper<D, 4>();
    default: return nullptr;
  }
}

}  // namespace spd_host
