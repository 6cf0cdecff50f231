// Adjoint (vector-Jacobian product) kernels of the pseudo-spectral RHS for sm_103a.
//
// For du = P D F(u x w) - (nu k^2 + drag) u_hat + f(u_hat) with u = irfftn(u_hat),
// w = irfftn(i k x u_hat) (l3es/spectral_solver.py:50-60) and a cotangent g of du,
// the cotangent of u_hat is
//   vjp = wt [F(w x m) + i k x F(m x u)] - (nu k^2 + drag) g + f'(u_hat)^T g,
//   m = irfftn(D P g / wt),
// wt = 1 on the half-axis planes 0 and N/2 and 2 elsewhere (a stored mode's
// multiplicity in the full spectrum), gradients in the dL/dRe + i dL/dIm convention.
// One evaluation:
//   kx_inv (curl)      u, w lines (the forward kernel)
//   kx_inv_adjproj     m lines: dealias mask, Leray projection and 1/wt in the prologue
//                      (block 0 also reduces the constant-power band terms)
//   ky_pass inverse    (3D) on the 9 fields
//   line_cross_adj     c2r of m (parked), u and w; r2c of m x u and m x w, all modes
//   ky_pass forward    (3D) on the 6 products
//   kx_fwd_plain       x-axis forward FFT of the 6 products
//   k_adj_epi          elementwise vjp assembly and the RK4 reverse recursion
#pragma once

#include "dns_kernels.cuh"

namespace l3es {

// Constant-power band force derivative terms of one stage field, by all threads of
// one block (blockDim a multiple of 32, at most 1024):
//   s = eps / (2 E_f + tiny), c = -2 eps beta / (2 E_f + tiny)^2 / N^(2d),
//   E_f = sum_band wt |us|^2 / (2 N^(2d)), beta = Re sum_band conj(gscale g) us.
template <int DIM>
__device__ __forceinline__ void band_adj_terms(const float2* __restrict__ us, const float2* __restrict__ g,
                                               long long cs, float gscale, int N, int kf, double inv_n2d,
                                               double eps_inj, double* out) {
  __shared__ double red_e[32], red_b[32];
  double e = 0.0, beta = 0.0;
  const int nb = band_count<DIM>(kf);
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    long long idx;
    int wg;
    if (!band_mode<DIM>(i, N, kf, idx, wg)) continue;
    for (int c = 0; c < 3; ++c) {
      const float2 v = us[c * cs + idx];
      const float2 gv = g[c * cs + idx];
      e += wg * ((double)v.x * v.x + (double)v.y * v.y);
      beta += (double)gscale * ((double)gv.x * v.x + (double)gv.y * v.y);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_xor_sync(0xffffffffu, e, o);
    beta += __shfl_xor_sync(0xffffffffu, beta, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
    red_e[wid] = e;
    red_b[wid] = beta;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double E = 0.0, B = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      E += red_e[i];
      B += red_b[i];
    }
    const double den = 2.0 * (0.5 * E * inv_n2d) + 1e-30;  // as band_coefficient
    out[0] = eps_inj / den;
    out[1] = -2.0 * eps_inj * B / (den * den) * inv_n2d;
  }
}

// ------------------------------------------------------------------------------
// x-axis inverse pass of m = D P (gscale g) / wt (3 fields), columns like kx_inv.
// D: the cube band |kx|, |kmid|, khalf <= kd; P: Leray projection (k = 0 untouched).
// With band_kf > 0, block (0, b) also writes the band terms of trajectory b.
// ------------------------------------------------------------------------------
template <int N, int DIM>
__global__ void __launch_bounds__(TW * Fft<N>::T)
kx_inv_adjproj(const float2* __restrict__ g, long long cs, float gscale, int kd, float2* __restrict__ w,
               long long fs, const float2* __restrict__ tw, const float2* __restrict__ us, int band_kf,
               double inv_n2d, double eps_inj, double* __restrict__ band_out) {
  constexpr int E = Fft<N>::E, T = Fft<N>::T, H = N / 2 + 1;
  constexpr int NMID = DIM == 3 ? N : 1;
  constexpr int MC = NMID * H;
  __shared__ float2 sm[xpad_len<TW>(N) * TW];
  const int p = threadIdx.x % TW, t = threadIdx.x / TW;
  const int m = blockIdx.x * TW + p;
  const bool ok = m < MC;
  const long long bg = (long long)blockIdx.y * 3 * cs, bw = (long long)blockIdx.y * 3 * fs;
  if (band_kf > 0 && blockIdx.x == 0)
    band_adj_terms<DIM>(us + bg, g + bg, cs, gscale, N, band_kf, inv_n2d, eps_inj, band_out + 2 * blockIdx.y);
  const int kh = m % H;
  const int km = DIM == 3 ? kfull(m / H, N) : 0;
  const float inv_wt = (kh == 0 || kh == N / 2) ? gscale : 0.5f * gscale;
  // band membership as unsigned offsets: -kd <= k <= kd  <=>  (unsigned)(k + kd) <= 2 kd
  // (the signed two-sided form was observed to keep out-of-band rows on the GPU)
  const unsigned span = 2u * (unsigned)kd;
  const bool col_keep = ok && (unsigned)(km + kd) <= span && (unsigned)kh <= (unsigned)kd;
  float2 a[3][E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int kx = kfull(t + T * e, N);
    const bool keep = col_keep && (unsigned)(kx + kd) <= span;
    float2 v0 = make_float2(0.f, 0.f), v1 = v0, v2 = v0;
    if (keep) {
      const long long o = bg + (long long)(t + T * e) * MC + m;
      v0 = g[o];
      v1 = g[o + cs];
      v2 = g[o + 2 * cs];
    }
    float k0, k1, k2;
    kvec<DIM>(kx, km, kh, k0, k1, k2);
    const int ik2 = kx * kx + km * km + kh * kh;
    const float inv = 1.0f / (ik2 == 0 ? 1.0f : (float)ik2);
    const float pr = (v0.x * k0 + v1.x * k1 + v2.x * k2) * inv;
    const float pi_ = (v0.y * k0 + v1.y * k1 + v2.y * k2) * inv;
    a[0][e] = make_float2(inv_wt * (v0.x - pr * k0), inv_wt * (v0.y - pi_ * k0));
    a[1][e] = make_float2(inv_wt * (v1.x - pr * k1), inv_wt * (v1.y - pi_ * k1));
    a[2][e] = make_float2(inv_wt * (v2.x - pr * k2), inv_wt * (v2.y - pi_ * k2));
  }
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    block_fft<N, E, kInv, TW>(a[f], sm + p, t, tw, 1);
    if (ok) {
#pragma unroll
      for (int e = 0; e < E; ++e) w[bw + f * fs + (long long)(t + T * e) * MC + m] = a[f][e];
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------
// Half-axis line pass of the adjoint: c2r of the 3 m lines (parked in shared memory,
// same thread writes and reads), then of the 3 u lines and the 3 w lines; C = m x u
// and A = m x w accumulate in registers and are r2c'd (every half-axis mode) when
// their triple is complete: out fields 0..2 = C, 3..5 = A.
// wm: [batch][3][fs] (m), wuw: [batch][6][fs] (u, w), out: [batch][6][cs].
// ------------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(LineCfg<N>::THREADS, 3)
line_cross_adj(const float2* __restrict__ wm, const float2* __restrict__ wuw, long long fs,
               float2* __restrict__ out, long long cs, float scale, const float2* __restrict__ twN, int nlines) {
  using C = LineCfg<N>;
  constexpr int M = C::M, H = N / 2 + 1, E = C::E, T = C::T, LPC = C::LPC;
  __shared__ float2 s_x[LPC * C::XS];
  __shared__ float2 s_m[LPC * C::PS];
  const int batch = blockIdx.y;
  const int q = threadIdx.x / T, t = threadIdx.x % T;
  const long long line_raw = (long long)blockIdx.x * LPC + q;
  const bool valid = line_raw < nlines;
  const long long line = valid ? line_raw : nlines - 1;  // idle lines mirror a valid one
  const float2* srcm = wm + (long long)batch * 3 * fs + line * H;
  const float2* srcy = wuw + (long long)batch * 6 * fs + line * H;
  float2* xs = s_x + q * C::XS;
  float2* sm_ = s_m + q * C::PS;
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    float2 v[E];
    c2r_load_pack<M, E>(srcm + f * fs, t, v, twN, scale);
    warp_fft<M, E, kInv>(v, xs, t, twN + N);
#pragma unroll
    for (int e = 0; e < E; ++e) sm_[f * M + t + T * e] = v[e];  // physical values at 2n, 2n+1
    __syncwarp();
  }
  float2* ob = out + (long long)batch * 6 * cs + line * H;
#pragma unroll 1
  for (int grp = 0; grp < 2; ++grp) {
    float2 cr[3][E];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int e = 0; e < E; ++e) cr[c][e] = make_float2(0.f, 0.f);
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      float2 v[E];
      c2r_load_pack<M, E>(srcy + (3 * grp + f) * fs, t, v, twN, scale);
      warp_fft<M, E, kInv>(v, xs, t, twN + N);
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int n = t + T * e;
        const float2 y = v[e];
        if (f == 0) {  // Y_x: (m x Y)_y += m_z Y_x, (m x Y)_z -= m_y Y_x
          const float2 mz = sm_[2 * M + n], my = sm_[M + n];
          cr[1][e].x = fmaf(mz.x, y.x, cr[1][e].x);
          cr[1][e].y = fmaf(mz.y, y.y, cr[1][e].y);
          cr[2][e].x = fmaf(-my.x, y.x, cr[2][e].x);
          cr[2][e].y = fmaf(-my.y, y.y, cr[2][e].y);
        } else if (f == 1) {  // Y_y: (m x Y)_x -= m_z Y_y, (m x Y)_z += m_x Y_y
          const float2 mz = sm_[2 * M + n], mx = sm_[n];
          cr[0][e].x = fmaf(-mz.x, y.x, cr[0][e].x);
          cr[0][e].y = fmaf(-mz.y, y.y, cr[0][e].y);
          cr[2][e].x = fmaf(mx.x, y.x, cr[2][e].x);
          cr[2][e].y = fmaf(mx.y, y.y, cr[2][e].y);
        } else {  // Y_z: (m x Y)_x += m_y Y_z, (m x Y)_y -= m_x Y_z
          const float2 my = sm_[M + n], mx = sm_[n];
          cr[0][e].x = fmaf(my.x, y.x, cr[0][e].x);
          cr[0][e].y = fmaf(my.y, y.y, cr[0][e].y);
          cr[1][e].x = fmaf(-mx.x, y.x, cr[1][e].x);
          cr[1][e].y = fmaf(-mx.y, y.y, cr[1][e].y);
        }
      }
      __syncwarp();
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      warp_fft<M, E, kFwd>(cr[c], xs, t, twN + N);
      float2 X[E];
      r2c_unpack_regs<M, E>(cr[c], t, twN, X);
      if (valid) {
        float2* dst = ob + (3 * grp + c) * cs;
#pragma unroll
        for (int e = 0; e < E; ++e) dst[t + T * e] = X[e];
        if (t == 0) dst[M] = make_float2(cr[c][0].x - cr[c][0].y, 0.f);  // X[M] = Re Z0 - Im Z0
      }
      __syncwarp();
    }
  }
}

// Epilogue operands of k_adj_epi. The stage's cotangent is gscale * g; the step's
// accumulated cotangent becomes lam_out = lam_in + vjp (lam_in = lam1 when null, and
// lam1 = 0 when null) and the next stage's cotangent g_out = a_next lam1 + b_next vjp
// (skipped when null). g_out may alias g and lam_out may alias lam_in or lam1 (each
// element is read and written by the same thread, reads first).
struct AdjEpi {
  const float2* us;
  const float2* g;
  float gscale;
  const float2* lam1;
  const float2* lam_in;
  float2* lam_out;
  float2* g_out;
  float a_next, b_next;
  float drag;
  int band_kf2;             // constant-power band 0 < |k|^2 <= band_kf2 (0 = off)
  const double* band_adj;   // [batch][2]: s, c
  const float2* wlines;     // u, curl u lines of us when already computed (else nullptr)
};

// ------------------------------------------------------------------------------
// Elementwise vjp assembly, two modes per thread (float4), all 3 components:
//   vjp = wt (i k x Cp - Ap) - (nu k^2 + drag) g [+ s g + c wt us on the band]
// with Cp = F(m x u) (fields 0..2 of y), Ap = F(m x w) (fields 3..5), then the RK4
// reverse recursion (AdjEpi). cs is even (N even), so a float4 never straddles a
// component.
// ------------------------------------------------------------------------------
template <int N, int DIM>
__global__ void __launch_bounds__(256)
k_adj_epi(const float2* __restrict__ y, long long cs, AdjEpi a, const float* __restrict__ nu_b) {
  constexpr unsigned H = N / 2 + 1;
  constexpr unsigned NMID = DIM == 3 ? N : 1;
  const int batch = blockIdx.y;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // pair index in one component
  if (q >= cs / 2) return;
  const long long by = (long long)batch * 6 * cs, bo = (long long)batch * 3 * cs;
  const float nu = nu_b[batch];
  float fs_ = 0.f, fc = 0.f;
  if (a.band_kf2 > 0) {
    fs_ = (float)a.band_adj[2 * batch];
    fc = (float)a.band_adj[2 * batch + 1];
  }
  float4 cp[3], ap[3], gg[3], l1[3], li[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    cp[c] = reinterpret_cast<const float4*>(y + by + c * cs)[q];
    ap[c] = reinterpret_cast<const float4*>(y + by + (3 + c) * cs)[q];
    gg[c] = reinterpret_cast<const float4*>(a.g + bo + c * cs)[q];
    l1[c] = a.lam1 ? reinterpret_cast<const float4*>(a.lam1 + bo + c * cs)[q] : make_float4(0.f, 0.f, 0.f, 0.f);
    li[c] = a.lam_in ? reinterpret_cast<const float4*>(a.lam_in + bo + c * cs)[q] : l1[c];
  }
  float4 lo[3], go[3];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const unsigned i = (unsigned)(2 * q + h);  // < cs < 2^31
    const int kh = (int)(i % H);
    const unsigned rest = i / H;
    const int km = DIM == 3 ? kfull((int)(rest % NMID), N) : 0;
    const int kx = kfull((int)(rest / NMID), N);
    float k0, k1, k2;
    kvec<DIM>(kx, km, kh, k0, k1, k2);
    const int ik2 = kx * kx + km * km + kh * kh;
    const float wt = (kh == 0 || kh == N / 2) ? 1.f : 2.f;
    const float lin = nu * (float)ik2 + a.drag;
    const bool band = a.band_kf2 > 0 && ik2 > 0 && ik2 <= a.band_kf2;
    float2 C[3], A[3], G[3], L1[3], LI[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      C[c] = h ? make_float2(cp[c].z, cp[c].w) : make_float2(cp[c].x, cp[c].y);
      A[c] = h ? make_float2(ap[c].z, ap[c].w) : make_float2(ap[c].x, ap[c].y);
      G[c] = h ? make_float2(gg[c].z, gg[c].w) : make_float2(gg[c].x, gg[c].y);
      G[c].x *= a.gscale;
      G[c].y *= a.gscale;
      L1[c] = h ? make_float2(l1[c].z, l1[c].w) : make_float2(l1[c].x, l1[c].y);
      LI[c] = h ? make_float2(li[c].z, li[c].w) : make_float2(li[c].x, li[c].y);
    }
    // k x C
    const float2 xc[3] = {make_float2(k1 * C[2].x - k2 * C[1].x, k1 * C[2].y - k2 * C[1].y),
                          make_float2(k2 * C[0].x - k0 * C[2].x, k2 * C[0].y - k0 * C[2].y),
                          make_float2(k0 * C[1].x - k1 * C[0].x, k0 * C[1].y - k1 * C[0].y)};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      // wt (i (k x C) - A),  i (x + i y) = -y + i x
      float2 r = make_float2(wt * (-xc[c].y - A[c].x), wt * (xc[c].x - A[c].y));
      r.x -= lin * G[c].x;
      r.y -= lin * G[c].y;
      if (band) {
        const float2 uv = a.us[bo + c * cs + i];
        r.x += fs_ * G[c].x + fc * wt * uv.x;
        r.y += fs_ * G[c].y + fc * wt * uv.y;
      }
      const float2 lv = make_float2(LI[c].x + r.x, LI[c].y + r.y);
      const float2 gv = make_float2(a.a_next * L1[c].x + a.b_next * r.x, a.a_next * L1[c].y + a.b_next * r.y);
      if (h == 0) {
        lo[c].x = lv.x;
        lo[c].y = lv.y;
        go[c].x = gv.x;
        go[c].y = gv.y;
      } else {
        lo[c].z = lv.x;
        lo[c].w = lv.y;
        go[c].z = gv.x;
        go[c].w = gv.y;
      }
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    reinterpret_cast<float4*>(a.lam_out + bo + c * cs)[q] = lo[c];
    if (a.g_out) reinterpret_cast<float4*>(a.g_out + bo + c * cs)[q] = go[c];
  }
}

}  // namespace l3es
