// Reverse mode of the RK4 step (the derivative the reference takes with jax.grad of
// l3es/spectral_solver.py:50-80): per-step checkpoints are the caller's; the three
// inner stage states are recomputed by the forward stage kernels, then four RHS
// vector-Jacobian products run in reverse stage order (adjoint_kernels.cuh):
//   lam = lam1;  g4 = dt/6 lam1
//   r4 = vjp(Uc, g4); lam += r4; g3 = dt/3 lam1 + dt r4
//   r3 = vjp(Ub, g3); lam += r3; g2 = dt/3 lam1 + dt/2 r3
//   r2 = vjp(Ua, g2); lam += r2; g1 = dt/6 lam1 + dt/2 r2
//   r1 = vjp(U0, g1); lam += r1
// The accumulation and the next stage's cotangent are written by the epilogue of the
// last pass of each product.
#include <cuda_runtime.h>

#include <string>

#include "l3es_internal.h"

using namespace l3es;

static int adj_prepare(l3es_plan* p) {
  AdjWork& w = p->adj;
  if (w.Ua) return L3ES_OK;
  const Ctx& c = p->ctx;
  const size_t spec = sizeof(float2) * 3 * (size_t)c.cs * c.batch;
  float2** bufs[] = {&w.Ua, &w.Ub, &w.Uc, &w.Wm, &w.LAM, &w.G};
  for (float2** b : bufs) {
    cudaError_t e = cudaMalloc((void**)b, spec);
    if (e != cudaSuccess) {
      cudaGetLastError();
      for (void* a : w.allocs) cudaFree(a);
      w = AdjWork();
      return fail(L3ES_ENOMEM, std::string("adjoint workspace: ") + cudaGetErrorString(e));
    }
    w.allocs.push_back(*b);
  }
  cudaError_t e = cudaMalloc((void**)&w.Y6, 2 * spec);
  if (e == cudaSuccess) {
    w.allocs.push_back(w.Y6);
    e = cudaMalloc((void**)&w.band, sizeof(double) * 2 * c.batch);
    if (e == cudaSuccess) w.allocs.push_back(w.band);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    for (void* a : w.allocs) cudaFree(a);
    w = AdjWork();
    return fail(L3ES_ENOMEM, std::string("adjoint workspace: ") + cudaGetErrorString(e));
  }
  return L3ES_OK;
}

static int adj_check(l3es_plan* p, const char* who) {
  if (p->desc.forcing == L3ES_FORCING_EKIN_TOT)
    return fail(L3ES_EINVAL, std::string(who) +
                                 ": the ekin_tot rescaling after each step has no adjoint here "
                                 "(use forcing none or const_power)");
  if (p->desc.scheme != L3ES_SCHEME_EXPLICIT)
    return fail(L3ES_EINVAL, std::string(who) + ": the adjoint follows the explicit RK4 step only "
                                                "(L3ES_SCHEME_EXPLICIT)");
  return adj_prepare(p);
}

static AdjEpi adj_epi(const l3es_plan* p) {
  AdjEpi a{};
  a.drag = (float)p->desc.drag;
  a.band_kf2 = p->desc.forcing == L3ES_FORCING_CONST_POWER ? p->desc.kf * p->desc.kf : 0;
  a.band_adj = p->adj.band;
  return a;
}

extern "C" {

int l3es_plan_adjoint_prepare(l3es_plan* plan) {
  if (!plan) return fail(L3ES_EINVAL, "l3es_plan_adjoint_prepare: null plan");
  return adj_check(plan, "l3es_plan_adjoint_prepare");
}

int l3es_rhs_vjp(l3es_plan* plan, const void* u_hat, const void* g, void* out, void* stream) {
  if (!plan || !u_hat || !g || !out) return fail(L3ES_EINVAL, "l3es_rhs_vjp: null argument");
  if (out == u_hat) return fail(L3ES_EINVAL, "l3es_rhs_vjp: out must not alias u_hat");
  if (misaligned16(u_hat) || misaligned16(g) || misaligned16(out))
    return fail(L3ES_EINVAL, "l3es_rhs_vjp: arrays must be 16-byte aligned");
  int rc = adj_check(plan, "l3es_rhs_vjp");
  if (rc != L3ES_OK) return rc;
  AdjEpi a = adj_epi(plan);
  a.us = (const float2*)u_hat;
  a.g = (const float2*)g;
  a.gscale = 1.f;
  a.lam_out = (float2*)out;
  plan->tab.vjp(plan->ctx, a, plan->adj.Wm, plan->adj.Y6, (cudaStream_t)stream);
  return cuda_check(cudaGetLastError(), "l3es_rhs_vjp launch");
}

int l3es_adjoint_step(l3es_plan* plan, const void* u_hat_n, void* lam, void* stream) {
  if (!plan || !u_hat_n || !lam) return fail(L3ES_EINVAL, "l3es_adjoint_step: null argument");
  if (lam == u_hat_n) return fail(L3ES_EINVAL, "l3es_adjoint_step: lam must not alias u_hat_n");
  if (misaligned16(u_hat_n) || misaligned16(lam))
    return fail(L3ES_EINVAL, "l3es_adjoint_step: arrays must be 16-byte aligned");
  int rc = adj_check(plan, "l3es_adjoint_step");
  if (rc != L3ES_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const Ctx& c = plan->ctx;
  const l3es_plan_desc& d = plan->desc;
  AdjWork& w = plan->adj;
  float2* U0 = const_cast<float2*>((const float2*)u_hat_n);  // read only (rk < 3 never writes S)
  float2* L1 = (float2*)lam;
  // recompute the stage states Ua, Ub, Uc (forward stages rk = 0, 1, 2)
  static const double a_rk4[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
  static const double b_rk4[3] = {0.5, 0.5, 1.0};
  float2* stage_out[3] = {w.Ua, w.Ub, w.Uc};
  for (int rk = 0; rk < 3; ++rk) {
    EpiParams prm;
    prm.a_dt = (float)(a_rk4[rk] * d.dt);
    prm.b_dt = (float)(b_rk4[rk] * d.dt);
    prm.nu = (float)d.nu;
    prm.drag = (float)d.drag;
    prm.kolm_amp = (float)d.kolm_amp;
    prm.kolm_k = d.kolm_k;
    prm.band_kf2 = d.forcing == L3ES_FORCING_CONST_POWER ? d.kf * d.kf : 0;
    prm.rk = rk;
    prm.if_h = 0.f;
    plan->tab.stage(c, rk == 0 ? U0 : stage_out[rk - 1], U0, stage_out[rk], rk, prm, s);
  }
  const float dt = (float)d.dt;
  const float2* us[4] = {w.Uc, w.Ub, w.Ua, U0};
  const float a_next[4] = {(float)(d.dt / 3.0), (float)(d.dt / 3.0), (float)(d.dt / 6.0), 0.f};
  const float b_next[4] = {dt, 0.5f * dt, 0.5f * dt, 0.f};
  for (int j = 0; j < 4; ++j) {
    AdjEpi a = adj_epi(plan);
    a.us = us[j];
    a.lam1 = L1;
    if (j == 0) {  // g4 = dt/6 lam1, lam_in = lam1
      a.g = L1;
      a.gscale = (float)(d.dt / 6.0);
      a.lam_in = nullptr;
    } else {
      a.g = w.G;
      a.gscale = 1.f;
      a.lam_in = w.LAM;
    }
    if (j < 3) {
      a.lam_out = w.LAM;
      a.g_out = w.G;
      a.a_next = a_next[j];
      a.b_next = b_next[j];
    } else {
      a.lam_out = L1;  // lam1 is not read after the first three products
      a.g_out = nullptr;
    }
    plan->tab.vjp(c, a, w.Wm, w.Y6, s);
  }
  return cuda_check(cudaGetLastError(), "l3es_adjoint_step launch");
}

}  // extern "C"
