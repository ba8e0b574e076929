// C ABI of the adjoint: record slots of forward intermediates, recorded
// steps and the vector-Jacobian product of one recorded step.  The step is
// differentiated with dt, the trouble masks, theta, the affected faces, the
// minmod/moncen branches and the Riemann-solver branches frozen at their
// values in the recorded forward step.
#include "spd_ctx.cuh"

using namespace spd;
using namespace spd_host;

namespace {

int adj_alloc(spd_ctx* C, double** p, size_t count) {
  void* q = nullptr;
  CK(cudaMalloc(&q, count * sizeof(double)));
  C->adj_allocs.push_back(q);
  *p = static_cast<double*>(q);
  return 0;
}

void adj_free(spd_ctx* C) {
  if (C->stream) cudaStreamSynchronize(C->stream);
  for (void* p : C->adj_allocs) cudaFree(p);
  C->adj_allocs.clear();
  C->adj_depth = 0;
}

// point the hist_* pointers at record slot `slot`
void select_slot(spd_ctx* C, int slot) {
  C->hist_usp = C->rec_usp + (size_t)slot * C->rec_usp_n;
  C->hist_ader = C->rec_ader_n ? C->rec_ader + (size_t)slot * C->rec_ader_n : nullptr;
  C->hist_ucv = C->rec_ucv_n ? C->rec_ucv + (size_t)slot * C->rec_ucv_n : nullptr;
  C->hist_aff = C->rec_aff_n ? C->rec_aff + (size_t)slot * C->rec_aff_n : nullptr;
  C->hist_dt = C->rec_dt + slot;
  C->hist_mpred = C->rec_mpred_n ? C->rec_mpred + (size_t)slot * C->rec_mpred_n : nullptr;
}

}  // namespace

extern "C" {

int spd_adjoint_enable(spd_ctx* C, int depth) {
  if (!C || depth < 1) return SPD_ERR_ARG;
  if (C->cfg.viscosity || C->cfg.potential || C->cfg.isothermal || C->cfg.WB)
    return fail(C, SPD_ERR_ARG,
                "the adjoint does not differentiate the viscous fluxes, the gravity source, the isothermal "
                "system or the well-balanced mode");
  if (C->adj_depth >= depth) return SPD_OK;
  adj_free(C);
  const Geo& g = C->geo;
  const int D = C->D, V = C->V, T = C->T, NS = C->NS, NJ = C->NJ, m = T - 1;
  const bool fv = C->cfg.update == SPD_UPDATE_FV;
  const bool fb = fv && C->cfg.FB;
  long long nface[3] = {0, 0, 0};
  size_t faces_total = 0;
  for (int d = 0; d < D; ++d) {
    nface[d] = n_faces(g, d);
    faces_total += (size_t)nface[d];
  }
  C->rec_usp_n = (size_t)V * NS * g.Nc;
  C->rec_ader_n = (size_t)m * V * T * NS * g.Nc;
  C->rec_ucv_n = fv ? (size_t)T * V * g.Nq : 0;
  C->rec_aff_n = fb ? (size_t)T * faces_total : 0;
  C->rec_mpred_n = fb ? (size_t)T * (1 + D) * V * g.Nqe : 0;
  if (int r = adj_alloc(C, &C->rec_usp, C->rec_usp_n * depth)) return r;
  if (C->rec_ader_n)
    if (int r = adj_alloc(C, &C->rec_ader, C->rec_ader_n * depth)) return r;
  if (C->rec_ucv_n)
    if (int r = adj_alloc(C, &C->rec_ucv, C->rec_ucv_n * depth)) return r;
  if (C->rec_aff_n)
    if (int r = adj_alloc(C, &C->rec_aff, C->rec_aff_n * depth)) return r;
  if (C->rec_mpred_n)
    if (int r = adj_alloc(C, &C->rec_mpred, C->rec_mpred_n * depth)) return r;
  if (int r = adj_alloc(C, &C->rec_dt, (size_t)depth)) return r;
  if (int r = adj_alloc(C, &C->Usp_a, (size_t)V * NS * g.Nc)) return r;
  CK(cudaMemset(C->Usp_a, 0, sizeof(double) * V * NS * g.Nc));
  if (int r = adj_alloc(C, &C->Ua, (size_t)V * T * NS * g.Nc)) return r;
  if (int r = adj_alloc(C, &C->dudt_a, (size_t)V * T * NS * g.Nc)) return r;
  for (int d = 0; d < D; ++d) {
    if (int r = adj_alloc(C, &C->Ea[d], (size_t)2 * V * T * NJ * g.Nc)) return r;
    if (int r = adj_alloc(C, &C->Tra[d], (size_t)2 * V * T * NJ * g.Nc)) return r;
    if (int r = adj_alloc(C, &C->Upart[d], (size_t)V * T * NS * g.Nc)) return r;
    if (fv) {
      if (int r = adj_alloc(C, &C->Ffa[d], (size_t)V * T * NJ * C->nf * g.Nc)) return r;
      if (int r = adj_alloc(C, &C->FHa[d], (size_t)T * V * nface[d])) return r;
    }
    if (fb) {
      const int o0 = (d == 0) ? 1 : 0;
      const int o1 = (d == 2) ? 1 : 2;
      if (int r = adj_alloc(C, &C->Fba[d], (size_t)V * nface[d])) return r;
      if (int r = adj_alloc(C, &C->FA[d], (size_t)2 * V * nface[d])) return r;
      if (int r = adj_alloc(C, &C->bcbuf_a[d], (size_t)2 * V * NGH * g.Xe[o0] * g.Xe[o1])) return r;
    }
  }
  if (fv) {
    if (int r = adj_alloc(C, &C->Ucv_a, (size_t)V * g.Nq)) return r;
    if (int r = adj_alloc(C, &C->Unew_a, (size_t)V * g.Nq)) return r;
  }
  if (fb) {
    if (int r = adj_alloc(C, &C->W_a, (size_t)V * g.Nqe)) return r;
    if (int r = adj_alloc(C, &C->W_ext, (size_t)V * g.Nqe)) return r;
    if (int r = adj_alloc(C, &C->LA, (size_t)2 * D * V * g.Nqe)) return r;
    CK(cudaMemset(C->W_ext, 0, sizeof(double) * V * g.Nqe));
  }
  C->adj_depth = depth;
  select_slot(C, 0);
  return SPD_OK;
}

int spd_adjoint_depth(const spd_ctx* C, int* depth) {
  if (!C || !depth) return SPD_ERR_ARG;
  *depth = C->adj_depth;
  return SPD_OK;
}

int spd_record_step(spd_ctx* C, int slot, double dt) {
  if (!C) return SPD_ERR_ARG;
  if (slot < 0 || slot >= C->adj_depth) return fail(C, SPD_ERR_ARG, "record_step: slot out of range (spd_adjoint_enable)");
  select_slot(C, slot);
  CK(cudaMemcpyAsync(C->dt, &dt, sizeof(double), cudaMemcpyHostToDevice, C->stream));
  CK(cudaMemcpyAsync(C->hist_dt, C->dt, sizeof(double), cudaMemcpyDeviceToDevice, C->stream));
  C->recording = true;
  const int rc = C->stepper->update(C);
  C->recording = false;
  if (rc) return rc;
  CK(cudaStreamSynchronize(C->stream));
  return SPD_OK;
}

int spd_tape_enable(spd_ctx* C, int nsteps) {
  if (!C || nsteps < 1) return SPD_ERR_ARG;
  if (C->cfg.viscosity || C->cfg.potential || C->cfg.isothermal || C->cfg.WB)
    return fail(C, SPD_ERR_ARG,
                "decision tapes do not cover the viscous fluxes, the gravity source, the isothermal system or "
                "the well-balanced mode");
  if (C->tape_steps >= nsteps) return SPD_OK;
  if (C->stream) cudaStreamSynchronize(C->stream);
  for (void* p : C->tape_allocs) cudaFree(p);
  C->tape_allocs.clear();
  C->tape_steps = 0;
  const Geo& g = C->geo;
  const int D = C->D, V = C->V, T = C->T, NJ = C->NJ;
  const bool fb = C->cfg.update == SPD_UPDATE_FV && C->cfg.FB;
  auto alloc = [&](void** p, size_t bytes) -> int {
    CK(cudaMalloc(p, bytes));
    C->tape_allocs.push_back(*p);
    return 0;
  };
  size_t faces_total = 0;
  for (int d = 0; d < D; ++d) {
    const size_t nI = (size_t)n_iface(g, d);
    if (int r = alloc((void**)&C->tape_rs[d], sizeof(unsigned) * nsteps * T * T * NJ * nI)) return r;
    if (fb) {
      const size_t nfc = (size_t)n_faces(g, d);
      faces_total += nfc;
      if (int r = alloc((void**)&C->tape_fb[d], sizeof(unsigned) * nsteps * T * nfc)) return r;
    }
  }
  if (fb) {
    if (int r = alloc((void**)&C->tape_lim, (size_t)nsteps * T * D * V * g.Nqe)) return r;
    if (int r = alloc((void**)&C->tape_aff, sizeof(double) * nsteps * T * faces_total)) return r;
  }
  C->tape_steps = nsteps;
  return SPD_OK;
}

int spd_tape_step(spd_ctx* C, int step, double dt, int mode) {
  if (!C) return SPD_ERR_ARG;
  if (step < 0 || step >= C->tape_steps) return fail(C, SPD_ERR_ARG, "tape_step: step out of range (spd_tape_enable)");
  if (mode != 1 && mode != 2) return fail(C, SPD_ERR_ARG, "tape_step: mode is 1 (record) or 2 (replay)");
  CK(cudaMemcpyAsync(C->dt, &dt, sizeof(double), cudaMemcpyHostToDevice, C->stream));
  C->tape_mode = mode;
  C->tape_step = step;
  const int rc = C->stepper->update(C);
  C->tape_mode = 0;
  if (rc) return rc;
  CK(cudaStreamSynchronize(C->stream));
  return SPD_OK;
}

int spd_vjp_step(spd_ctx* C, int slot) {
  if (!C) return SPD_ERR_ARG;
  if (slot < 0 || slot >= C->adj_depth) return fail(C, SPD_ERR_ARG, "vjp_step: slot out of range (spd_adjoint_enable)");
  select_slot(C, slot);
  if (int r = C->stepper->vjp(C)) return r;
  CK(cudaStreamSynchronize(C->stream));
  return SPD_OK;
}

}  // extern "C"
