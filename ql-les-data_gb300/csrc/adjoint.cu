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

namespace l3es {

// Adjoint of the ekin_tot rescaling u_new = u_rk (alpha mask + 1 - mask) after the RK4
// update (spectral_solver.py:82-112), alpha = sqrt(max(0, (E0 - E_high) / (E_low + eps))),
// E = sum w |u|^2 / (2 N^(2d)) (E_low over the band 0 < |k|^2 <= kf^2, E_high the rest).
// For the cotangent lam of u_new, with beta = Re sum_band conj(lam) u_rk:
//   lam_rk = lam - c_h w u_rk (outside the band),  alpha lam - c_l w u_rk (inside),
//   c_h = beta / (2 alpha (E_low + eps) N^(2d)),  c_l = beta alpha / (2 (E_low + eps) N^(2d))
// (no alpha term where the rescaling saturates at alpha = 0). One CTA per trajectory
// forms (alpha, c_h, c_l) from the energy partials of u_rk and the band sums.
template <int DIM>
__global__ void __launch_bounds__(256)
k_ekin_adj_coef(const float2* __restrict__ urk, const float2* __restrict__ lam, long long cs,
                const double* __restrict__ partial, int npartial, const double* __restrict__ e0, int N, int kf,
                double inv_n2d, double eps, double* __restrict__ coef) {
  const int batch = blockIdx.x;
  const float2* ub = urk + (long long)batch * 3 * cs;
  const float2* lb = lam + (long long)batch * 3 * cs;
  __shared__ double red[3][32];
  double s = 0.0, lo = 0.0, be = 0.0;
  for (int i = threadIdx.x; i < npartial; i += blockDim.x) s += partial[(long long)batch * npartial + i];
  const int nb = band_count<DIM>(kf);
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    long long idx;
    int wg;
    if (!band_mode<DIM>(i, N, kf, idx, wg)) continue;
    for (int c = 0; c < 3; ++c) {
      const float2 v = ub[c * cs + idx], l = lb[c * cs + idx];
      lo += wg * ((double)v.x * v.x + (double)v.y * v.y);
      be += (double)l.x * v.x + (double)l.y * v.y;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    lo += __shfl_xor_sync(0xffffffffu, lo, o);
    be += __shfl_xor_sync(0xffffffffu, be, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    red[0][wid] = s;
    red[1][wid] = lo;
    red[2][wid] = be;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0.0, L = 0.0, B = 0.0;
    for (int i = 0; i < nw; ++i) {
      S += red[0][i];
      L += red[1][i];
      B += red[2][i];
    }
    const double e_low = 0.5 * L * inv_n2d, e_high = 0.5 * S * inv_n2d - e_low;
    const double arg = (e0[batch] - e_high) / (e_low + eps);
    const double alpha = sqrt(arg > 0.0 ? arg : 0.0);
    double ch = 0.0, cl = 0.0;
    if (alpha > 0.0) {
      ch = B * inv_n2d / (2.0 * alpha * (e_low + eps));
      cl = B * alpha * inv_n2d / (2.0 * (e_low + eps));
    }
    coef[3 * batch] = alpha;
    coef[3 * batch + 1] = ch;
    coef[3 * batch + 2] = cl;
  }
}

// lam <- lam_rk over all modes (two per thread, float4), from (alpha, c_h, c_l)
template <int DIM>
__global__ void __launch_bounds__(256)
k_ekin_adj_apply(float2* __restrict__ lam, const float2* __restrict__ urk, long long cs, int N, int kf,
                 const double* __restrict__ coef) {
  const int batch = blockIdx.y;
  const long long pairs = 3 * cs / 2;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= pairs) return;
  const float alpha = (float)coef[3 * batch], ch = (float)coef[3 * batch + 1], cl = (float)coef[3 * batch + 2];
  const long long bo = (long long)batch * 3 * cs;
  float4* lp = reinterpret_cast<float4*>(lam + bo) + q;
  const float4 l4 = *lp;
  const float4 u4 = reinterpret_cast<const float4*>(urk + bo)[q];
  const unsigned H = (unsigned)(N / 2 + 1), NMID = DIM == 3 ? (unsigned)N : 1u, ucs = (unsigned)cs;
  float r[4] = {l4.x, l4.y, l4.z, l4.w};
  const float u[4] = {u4.x, u4.y, u4.z, u4.w};
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const unsigned g = (unsigned)(2 * q + h) % ucs;  // mode index inside its component
    const int kh = (int)(g % H);
    const unsigned rest = g / H;
    const int km = DIM == 3 ? kfull((int)(rest % NMID), N) : 0;
    const int kx = kfull((int)(rest / NMID), N);
    const int k2 = kx * kx + km * km + kh * kh;
    const float w = (kh == 0 || kh == N / 2) ? 1.f : 2.f;
    const bool band = k2 > 0 && k2 <= kf * kf;
    const float a = band ? alpha : 1.f, c = (band ? cl : ch) * w;
    r[2 * h] = a * r[2 * h] - c * u[2 * h];
    r[2 * h + 1] = a * r[2 * h + 1] - c * u[2 * h + 1];
  }
  *lp = make_float4(r[0], r[1], r[2], r[3]);
}

}  // namespace l3es

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
  if (e == cudaSuccess) w.allocs.push_back(w.Y6);
  const size_t wbytes = sizeof(float2) * 6 * (size_t)c.fs * c.batch;  // the size of the plan's W
  for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
    e = cudaMalloc((void**)&w.Wst[i], wbytes);
    if (e == cudaSuccess) w.allocs.push_back(w.Wst[i]);
  }
  if (e == cudaSuccess) {
    e = cudaMalloc((void**)&w.band, sizeof(double) * 2 * c.batch);
    if (e == cudaSuccess) w.allocs.push_back(w.band);
  }
  if (e == cudaSuccess) {
    e = cudaMalloc((void**)&w.ekin, sizeof(double) * 3 * c.batch);
    if (e == cudaSuccess) w.allocs.push_back(w.ekin);
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
    // the stage's u, curl u lines stay in Wst[rk] for the VJP at the same state
    Ctx cw = c;
    cw.W = w.Wst[rk];
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
    plan->tab.stage(cw, rk == 0 ? U0 : stage_out[rk - 1], U0, stage_out[rk], rk, prm, s);
  }
  if (d.forcing == L3ES_FORCING_EKIN_TOT) {
    // the step ends with the ekin_tot rescaling of the RK4 result u_rk: recompute u_rk
    // (the last stage, written to Wm, which is free until the products below) and turn
    // lam = dL/du_new into dL/du_rk
    EpiParams prm;
    prm.a_dt = (float)(a_rk4[3] * d.dt);
    prm.b_dt = 0.f;
    prm.nu = (float)d.nu;
    prm.drag = (float)d.drag;
    prm.kolm_amp = (float)d.kolm_amp;
    prm.kolm_k = d.kolm_k;
    prm.band_kf2 = 0;
    prm.rk = 3;
    prm.if_h = 0.f;
    plan->tab.stage(c, w.Uc, w.Wm, c.Tb, 3, prm, s);
    const int nke = energy_partials(c, w.Wm, s);
    const double inv_n2d = 1.0 / std::pow((double)c.n, 2 * c.dim);
    const double eps64 = 2.220446049250313e-16;  // jnp.finfo(float).eps, spectral_solver.py:23
    const long long pairs = 3 * c.cs / 2;
    const dim3 eb((unsigned)((pairs + 255) / 256), c.batch);
    if (c.dim == 3) {
      k_ekin_adj_coef<3><<<c.batch, 256, 0, s>>>(w.Wm, L1, c.cs, c.partial, nke, c.e0, c.n, d.kf, inv_n2d, eps64,
                                                 w.ekin);
      k_ekin_adj_apply<3><<<eb, 256, 0, s>>>(L1, w.Wm, c.cs, c.n, d.kf, w.ekin);
    } else {
      k_ekin_adj_coef<2><<<c.batch, 256, 0, s>>>(w.Wm, L1, c.cs, c.partial, nke, c.e0, c.n, d.kf, inv_n2d, eps64,
                                                 w.ekin);
      k_ekin_adj_apply<2><<<eb, 256, 0, s>>>(L1, w.Wm, c.cs, c.n, d.kf, w.ekin);
    }
  }
  const float dt = (float)d.dt;
  const float2* us[4] = {w.Uc, w.Ub, w.Ua, U0};
  const float a_next[4] = {(float)(d.dt / 3.0), (float)(d.dt / 3.0), (float)(d.dt / 6.0), 0.f};
  const float b_next[4] = {dt, 0.5f * dt, 0.5f * dt, 0.f};
  for (int j = 0; j < 4; ++j) {
    AdjEpi a = adj_epi(plan);
    a.us = us[j];
    a.wlines = j > 0 ? w.Wst[3 - j] : nullptr;  // Ub, Ua, U0: recomputed above; Uc: not
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
