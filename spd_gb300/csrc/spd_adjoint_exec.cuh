// Launch sequence of the adjoint of one recorded SD-ADER step (the kernels
// are in spd_adjoint.cuh), instantiated in spd_adj_d1.cu, spd_adj_d2.cu and
// spd_adj_d3.cu.  Like the step they are compiled without FMA contraction:
// the adjoint recomputes forward values (traces, reconstructed states,
// limiter arguments) whose branch decisions, ties included, must be the
// recorded step's.  (Measured: contracting the adjoint units saved 8% of
// the backward and moved moncen ties in the Kelvin-Helmholtz golden case.)
#pragma once
#include "spd_adjoint.cuh"
#include "spd_ctx.cuh"

namespace spd_host {

template <int D, int P>
int adj_traces_of(spd_ctx* C, const double* U, int Tu, int Teff) {
  const Geo& g = C->geo;
  ProfScope ps_(C, "k_adj_traces_fwd");
  k_traces_ader<D, P><<<blocks_for(g.Nc * Teff, 128), 128, 0, C->stream>>>(C->ops, g, U, Tu, Teff, C->trace[0],
                                                                          C->trace[1], C->trace[2]);
  CKL();
  return 0;
}

// adjoint of one predictor iteration: dudt_a (or Ffa) -> Ua (written)
template <int D, int P>
int adj_iteration(spd_ctx* C, int mode, const double* Uin, int Tu, int Teff) {
  using k = K<D, P>;
  const Geo& g = C->geo;
  if (int r = adj_traces_of<D, P>(C, Uin, Tu, Teff)) return r;
  {
    ProfScope ps_(C, "k_adj_interior");
    k_adj_interior<D, P><<<blocks_for(g.Nc * Teff * D * k::NJ, 128), 128, 0, C->stream>>>(
        C->ops, g, mode, Teff, Uin, Tu, C->dudt_a, C->Ffa[0], C->Ffa[1], C->Ffa[2], C->Upart[0], C->Upart[1],
        C->Upart[2], C->Ea[0], C->Ea[1], C->Ea[2]);
  }
  CKL();
  for (int d = 0; d < D; ++d) {
    CK(cudaMemsetAsync(C->Tra[d], 0, sizeof(double) * 2 * k::V * g.T * k::NJ * g.Nc, C->stream));
    const long long tot = (long long)Teff * k::NJ * n_iface(g, d);
    ProfScope ps_(C, "k_adj_riemann");
    k_adj_riemann<D, P><<<blocks_for(tot, 64), 64, 0, C->stream>>>(g, d, Teff, C->cfg.riemann_solver_sd,
                                                                  C->trace[d], C->bcfix[d], C->Ea[d], C->Tra[d]);
    CKL();
  }
  {
    ProfScope ps_(C, "k_adj_traces");
    k_adj_traces<D, P><<<blocks_for(g.Nc * Teff * k::NS, 128), 128, 0, C->stream>>>(
        C->ops, g, Teff, C->Tra[0], C->Tra[1], C->Tra[2], C->Upart[0], C->Upart[1], C->Upart[2], C->Ua);
  }
  CKL();
  return 0;
}

template <int D, int P>
int adjoint_vjp(spd_ctx* C) {
  using k = K<D, P>;
  const Geo& g = C->geo;
  const spd_config& cf = C->cfg;
  const int m = C->T - 1;
  const long long nsp = (long long)k::V * k::NS * g.Nc;
  const size_t nader = (size_t)k::V * C->T * k::NS * g.Nc;
  int final_mode = 1;
  if (cf.update == SPD_UPDATE_FV) {
    final_mode = 2;
    long long nface[3] = {1, 1, 1};
    size_t per = 0;
    for (int d = 0; d < D; ++d) {
      nface[d] = n_faces(g, d);
      per += (size_t)nface[d];
      CK(cudaMemsetAsync(C->FHa[d], 0, sizeof(double) * C->T * k::V * nface[d], C->stream));
    }
    {
      ProfScope ps_(C, "k_adj_cv_to_sp");
      k_adj_cv_to_sp<D, P><<<blocks_for(g.Nc * k::V, 128), 128, 0, C->stream>>>(g, C->K_cv_to_sp, C->Usp_a,
                                                                               C->Unew_a);
    }
    CKL();
    CK(cudaMemsetAsync(C->Usp_a, 0, sizeof(double) * nsp, C->stream));
    if (cf.FB) {
      CK(cudaMemsetAsync(C->W_a, 0, sizeof(double) * k::V * g.Nqe, C->stream));
      // fixed-state ghost sides read the boundary buffers, which no step overwrites
      for (int d = 0; d < D; ++d) {
        const int o0 = (d == 0) ? 1 : 0;
        const int o1 = (d == 2) ? 1 : 2;
        CK(cudaMemcpyAsync(C->bcbuf_a[d], C->bcbuf[d], sizeof(double) * 2 * k::V * NGH * g.Xe[o0] * g.Xe[o1],
                           cudaMemcpyDeviceToDevice, C->stream));
      }
    }
    for (int i = C->T - 1; i >= 0; --i) {
      const double w_i = C->ops.w_tp[i];
      const double* Ucv_i = C->hist_ucv + (size_t)i * k::V * g.Nq;
      size_t off = 0;
      for (int d = 0; d < D; ++d) {
        const double* aff = cf.FB ? C->hist_aff + (size_t)i * per + off : nullptr;
        ProfScope ps_(C, "k_adj_faces");
        k_adj_faces<D><<<blocks_for(nface[d], BS), BS, 0, C->stream>>>(
            g, C->fvg, d, C->hist_dt, w_i, cf.FB ? 1 : 0, cf.godunov, aff, C->Unew_a,
            C->FHa[d] + (size_t)i * k::V * nface[d], C->Fba[d]);
        CKL();
        off += (size_t)nface[d];
      }
      if (cf.FB) {
        {
          ProfScope ps_(C, "k_prim_ext");
          k_prim_ext<D><<<blocks_for(g.Nq, BS), BS, 0, C->stream>>>(g, Ucv_i, C->W_ext);
        }
        CKL();
        for (int d = 0; d < D; ++d) {
          const int o0 = (d == 0) ? 1 : 0;
          const int o1 = (d == 2) ? 1 : 2;
          const long long tot = 2LL * k::V * NGH * g.Xe[o0] * g.Xe[o1];
          ProfScope ps_(C, "k_ghost");
          k_ghost<D><<<blocks_for(tot, BS), BS, 0, C->stream>>>(g, d, 1, k::V, k::V, C->W_ext, C->bcbuf_a[d],
                                                                nullptr);
          CKL();
        }
        // the used faces and the cells bordering them, compacted into the
        // forward step's scratch lists (same stream, never live at once)
        const double* affd[3] = {nullptr, nullptr, nullptr};
        off = 0;
        for (int d = 0; d < D; ++d) {
          affd[d] = C->hist_aff + (size_t)i * per + off;
          off += (size_t)nface[d];
        }
        CK(cudaMemsetAsync(C->counts, 0, sizeof(unsigned long long), C->stream));
        CK(cudaMemsetAsync(C->counts + 4, 0, D * sizeof(unsigned long long), C->stream));
        for (int d = 0; d < D; ++d) {
          ProfScope ps_(C, "k_adj_used_faces");
          k_adj_used_faces<D><<<blocks_for(nface[d], BS), BS, 0, C->stream>>>(g, d, cf.godunov, affd[d],
                                                                               C->list_face[d], C->counts + 4 + d);
          CKL();
        }
        {
          ProfScope ps_(C, "k_adj_used_cells");
          k_adj_used_cells<D><<<blocks_for(g.Nqe, BS), BS, 0, C->stream>>>(g, cf.godunov, affd[0], affd[1], affd[2],
                                                                            C->list_cell, C->counts);
        }
        CKL();
        for (int d = 0; d < D; ++d) {
          ProfScope ps_(C, "k_adj_muscl_riemann");
          const double* mp = C->hist_mpred + (size_t)i * (1 + D) * k::V * g.Nqe;
          const unsigned nb = (unsigned)std::min<long long>(PERSIST_BLOCKS, blocks_for(nface[d], 64));
          k_adj_muscl_riemann<D><<<nb, 64, 0, C->stream>>>(g, d, cf.riemann_solver_fv, C->list_face[d],
                                                           C->counts + 4 + d, mp, mp + (size_t)k::V * g.Nqe,
                                                           C->Fba[d], C->FA[d]);
          CKL();
        }
        // W_a and LA are zero on the cells that border no used face
        CK(cudaMemsetAsync(C->W_a, 0, sizeof(double) * k::V * g.Nqe, C->stream));
        CK(cudaMemsetAsync(C->LA, 0, sizeof(double) * 2 * D * k::V * g.Nqe, C->stream));
        {
          ProfScope ps_(C, "k_adj_muscl_cells");
          const unsigned nb = (unsigned)std::min<long long>(PERSIST_BLOCKS, blocks_for(g.Nqe, 64));
          k_adj_muscl_cells<D><<<nb, 64, 0, C->stream>>>(g, C->fvg, cf.slope_limiter, cf.godunov, C->hist_dt, w_i,
                                                         affd[0], affd[1], affd[2], C->FA[0], C->FA[1], C->FA[2],
                                                         C->W_ext, C->list_cell, C->counts, C->W_a, C->LA);
        }
        CKL();
        {
          ProfScope ps_(C, "k_adj_muscl_gather");
          k_adj_muscl_gather<D><<<blocks_for(g.Nqe, BS), BS, 0, C->stream>>>(g, C->LA, C->W_a);
        }
        CKL();
        for (int d = D - 1; d >= 0; --d) {
          const int o0 = (d == 0) ? 1 : 0;
          const int o1 = (d == 2) ? 1 : 2;
          const long long tot = (long long)k::V * NGH * g.Xe[o0] * g.Xe[o1];
          for (int side = 0; side < 2; ++side) {
            ProfScope ps_(C, "k_adj_ghost");
            k_adj_ghost<D><<<blocks_for(tot, BS), BS, 0, C->stream>>>(g, d, side, C->W_a);
            CKL();
          }
        }
      }
      if (cf.FB) {
        {
          ProfScope ps_(C, "k_adj_prim_cv");
          k_adj_prim_cv<D><<<blocks_for(g.Nq, BS), BS, 0, C->stream>>>(g, Ucv_i, C->Unew_a, C->W_a, C->Ucv_a);
        }
        CKL();
        std::swap(C->Ucv_a, C->Unew_a);  // the adjoint of this substep's input feeds the previous one
      }
      // without limiting the substep's input enters only through the
      // identity (its primitives feed no fallback flux): Unew_a already is
      // the adjoint of the input, and W_a (allocated with FB only) is unused
    }
    {
      ProfScope ps_(C, "k_adj_sp_to_cv");
      k_adj_sp_to_cv<D, P><<<blocks_for(g.Nc * k::V, 128), 128, 0, C->stream>>>(g, C->K_sp_to_cv, C->Unew_a,
                                                                                C->Usp_a);
    }
    CKL();
    for (int d = 0; d < D; ++d) {
      ProfScope ps_(C, "k_adj_integrate_faces");
      k_adj_integrate_faces<D, P><<<blocks_for(g.Nc * g.T * k::nf, 128), 128, 0, C->stream>>>(C->ops, g, d,
                                                                                              C->FHa[d], C->Ffa[d]);
      CKL();
    }
  } else {
    ProfScope ps_(C, "k_adj_sd_update");
    k_adj_sd_update<D, P><<<blocks_for(nsp, BS), BS, 0, C->stream>>>(C->ops, g, C->hist_dt, C->Usp_a, C->dudt_a,
                                                                     m == 0 ? 1 : C->T);
    CKL();
  }
  // predictor iterations, last to first
  for (int it = m; it >= 0; --it) {
    const int mode = (it == m) ? final_mode : 0;
    if (it < m) {
      ProfScope ps_(C, "k_adj_picard");
      k_adj_picard<D, P><<<blocks_for(nsp, BS), BS, 0, C->stream>>>(C->ops, g, C->hist_dt, C->Ua, C->Usp_a, C->dudt_a,
                                                                    it == 0 ? 1 : 0);
      CKL();
    }
    const double* Uin = (it == 0) ? C->hist_usp : C->hist_ader + (size_t)(it - 1) * nader;
    const int Tu = (it == 0) ? 1 : C->T;
    const int Teff = (it == 0) ? 1 : C->T;
    if (int r = adj_iteration<D, P>(C, mode, Uin, Tu, Teff)) return r;
    if (it == 0) {
      ProfScope ps_(C, "k_adj_add_first");
      k_adj_add_first<D, P><<<blocks_for(nsp, BS), BS, 0, C->stream>>>(g, C->Ua, C->Usp_a);
      CKL();
    }
  }
  return 0;
}

}  // namespace spd_host

#define SPD_INSTANTIATE_ADJOINT(D)                        \
  namespace spd_host {                                    \
  template int adjoint_vjp<D, 1>(spd_ctx*);               \
  template int adjoint_vjp<D, 2>(spd_ctx*);               \
  template int adjoint_vjp<D, 3>(spd_ctx*);               \
  template int adjoint_vjp<D, 4>(spd_ctx*);               \
  }
