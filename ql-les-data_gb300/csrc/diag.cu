// Diagnostics of the drivers (l3es/spectral_solver.py:123-127, :318-320;
// l3es/utils.py:35-97, :300-315) with FP64 partial sums. Each point's or mode's
// contribution is formed in FP32 and accumulated in float-float (Ff, ~48 bits) or FP64
// (field statistics); FP64 arithmetic is scarce on this GPU. The spectral loops run one
// warp per contiguous half-axis row, so no per-element index division is needed.
//   l3es_field_stats      max |u_c| per component and 0.5 mean sum u^2 of a physical field
//   l3es_dissipation      nu <|curl u|^2> by Parseval on the half spectrum
//   l3es_energy_spectrum  shell sums E(k), shells int(|k| + 0.5)
#include <cuda_runtime.h>

#include <cmath>

#include "l3es_internal.h"

namespace l3es {

// per block: max |u_c| for c = 0..2 and sum_c u_c^2, over ps values per component
__global__ void __launch_bounds__(256)
k_field_stats(const float* __restrict__ u, long long ps, int nblk, double* __restrict__ partial) {
  const int batch = blockIdx.y;
  const float* ub = u + (long long)batch * 3 * ps;
  float mx[3] = {0.f, 0.f, 0.f};
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < ps; i += (long long)nblk * blockDim.x) {
    float e = 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = ub[c * ps + i];
      mx[c] = fmaxf(mx[c], fabsf(v));
      e = fmaf(v, v, e);
    }
    s += (double)e;
  }
  __shared__ float smx[3][32];
  __shared__ double ss[32];
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
#pragma unroll
    for (int c = 0; c < 3; ++c) mx[c] = fmaxf(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    ss[wid] = s;
    for (int c = 0; c < 3; ++c) smx[c][wid] = mx[c];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    float m[3] = {0.f, 0.f, 0.f};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      t += ss[w];
      for (int c = 0; c < 3; ++c) m[c] = fmaxf(m[c], smx[c][w]);
    }
    double* o = partial + ((long long)batch * nblk + blockIdx.x) * 4;
    o[0] = m[0];
    o[1] = m[1];
    o[2] = m[2];
    o[3] = t;
  }
}

// out[batch*4 + {0,1,2}] = max |u_c|, out[batch*4 + 3] = 0.5 mean sum u^2
__global__ void k_field_stats_final(const double* __restrict__ partial, int nblk, double inv_ps,
                                    double* __restrict__ out) {
  const int batch = blockIdx.x;
  if (threadIdx.x != 0) return;
  double m[3] = {0.0, 0.0, 0.0}, s = 0.0;
  for (int b = 0; b < nblk; ++b) {
    const double* p = partial + ((long long)batch * nblk + b) * 4;
    for (int c = 0; c < 3; ++c) m[c] = fmax(m[c], p[c]);
    s += p[3];
  }
  for (int c = 0; c < 3; ++c) out[batch * 4 + c] = m[c];
  out[batch * 4 + 3] = 0.5 * s * inv_ps;
}

// dissipation partials: Parseval sum of w |C|^2 over the half spectrum, C = k x u_hat
// with the reference kkk. irfftn keeps only the Hermitian part of the kh = 0 and
// kh = N/2 planes, and i C is not Hermitian there (kz = +N/2 for both partners), so
// those planes use |(C(k) - conj C(-k)) / 2|^2 with weight 1 (utils.py:312-315).
template <int DIM>
__device__ __forceinline__ void curl_at(const float2* __restrict__ ub, long long cs, int n, int kxi, int mid, int kh,
                                        float* re, float* im) {
  const int h = n / 2 + 1;
  const int nmid = DIM == 3 ? n : 1;
  const long long i = ((long long)kxi * nmid + mid) * h + kh;
  float k0, k1, k2;
  kvec<DIM>(kfull(kxi, n), DIM == 3 ? kfull(mid, n) : 0, kh, k0, k1, k2);
  const float2 a = ub[i], b = ub[cs + i], c = ub[2 * cs + i];
  // (k x u)_x = k1 c - k2 b, (k x u)_y = k2 a - k0 c, (k x u)_z = k0 b - k1 a
  re[0] = k1 * c.x - k2 * b.x;
  im[0] = k1 * c.y - k2 * b.y;
  re[1] = k2 * a.x - k0 * c.x;
  im[1] = k2 * a.y - k0 * c.y;
  re[2] = k0 * b.x - k1 * a.x;
  im[2] = k0 * b.y - k1 * a.y;
}

template <int DIM>
__global__ void __launch_bounds__(256)
k_diss_partial(const float2* __restrict__ uh, long long cs, int n, int nblk, double* __restrict__ partial) {
  const int batch = blockIdx.y;
  const float2* ub = uh + (long long)batch * 3 * cs;
  const int h = n / 2 + 1;
  const int nmid = DIM == 3 ? n : 1;
  const long long rows = cs / h;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  Ff s{0.f, 0.f};
  for (long long r = (long long)blockIdx.x * wpb + (threadIdx.x >> 5); r < rows; r += (long long)nblk * wpb) {
    const int mid = (int)(r % nmid), kxi = (int)(r / nmid);
    for (int kh = lane; kh < h; kh += 32) {
      float re[3], im[3];
      curl_at<DIM>(ub, cs, n, kxi, mid, kh, re, im);
      float e = 0.f;
      if (kh == 0 || kh == n / 2) {
        float re2[3], im2[3];
        curl_at<DIM>(ub, cs, n, (n - kxi) % n, DIM == 3 ? (n - mid) % n : 0, kh, re2, im2);
        // Hermitian part of i C is i (C(k) - conj C(-k)) / 2
        for (int c = 0; c < 3; ++c) {
          const float hr = 0.5f * (re[c] - re2[c]), hi = 0.5f * (im[c] + im2[c]);
          e = fmaf(hr, hr, fmaf(hi, hi, e));
        }
      } else {
        for (int c = 0; c < 3; ++c) e = fmaf(re[c], re[c], fmaf(im[c], im[c], e));
        e *= 2.f;
      }
      s = ff_add(s, e);
    }
  }
  block_sum_store_ff(s, partial, batch * nblk + blockIdx.x);
}

// energy spectrum: per-block shared-memory histograms of (weight, weight*|u_hat|^2)
// over shells int(|k| + 0.5) < n, merged with FP64 atomics into acc[batch][2][n]
template <int DIM>
__global__ void __launch_bounds__(256)
k_spectrum(const float2* __restrict__ uh, long long cs, int n, int nblk, double scale, double* __restrict__ acc) {
  extern __shared__ double hist[];  // [2][n]
  const int batch = blockIdx.y;
  for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) hist[i] = 0.0;
  __syncthreads();
  const float2* ub = uh + (long long)batch * 3 * cs;
  const int h = n / 2 + 1;
  const int nmid = DIM == 3 ? n : 1;
  const long long rows = cs / h;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (long long r = (long long)blockIdx.x * wpb + (threadIdx.x >> 5); r < rows; r += (long long)nblk * wpb) {
    const int kx = kfull((int)(r / nmid), n);
    const int km = DIM == 3 ? kfull((int)(r % nmid), n) : 0;
    const float2* row = ub + r * h;
    for (int kh = lane; kh < h; kh += 32) {
      // shell int(|k| + 0.5): |k|^2 is an integer below 3 (n/2)^2, whose square root is
      // never within 1/(8|k|) of a half integer, far more than the FP32 rounding
      const int k2 = kx * kx + km * km + kh * kh;
      const int shell = (int)(sqrtf((float)k2) + 0.5f);
      float e = 0.f;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float2 v = row[c * cs + kh];
        e = fmaf(v.x, v.x, fmaf(v.y, v.y, e));
      }
      if (shell < n) {
        const double w = (kh == 0 || kh == n / 2) ? 1.0 : 2.0;
        atomicAdd(&hist[shell], w);
        atomicAdd(&hist[n + shell], w * scale * (double)e);
      }
    }
  }
  __syncthreads();
  double* a = acc + (long long)batch * 2 * n;
  for (int i = threadIdx.x; i < 2 * n; i += blockDim.x)
    if (hist[i] != 0.0) atomicAdd(&a[i], hist[i]);
}

// sum of n partials per trajectory times scale
__global__ void __launch_bounds__(256)
k_diag_sum(const double* __restrict__ partial, int n, double scale, double* __restrict__ out) {
  __shared__ double red[32];
  const int batch = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[(long long)batch * n + i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
    out[batch] = t * scale;
  }
}

__global__ void k_spectrum_final(const double* __restrict__ acc, int n, double eps, double* __restrict__ ek) {
  const int batch = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double* a = acc + (long long)batch * 2 * n;
  const double pi = 3.14159265358979323846;
  ek[(long long)batch * n + k] = a[n + k] * 4.0 * pi * (double)k * k / (a[k] + eps);
}

}  // namespace l3es

using namespace l3es;

extern "C" {

int l3es_field_stats(l3es_plan* plan, const float* u, double* out_dev, void* stream) {
  if (!plan || !u || !out_dev) return fail(L3ES_EINVAL, "l3es_field_stats: null argument");
  const Ctx& c = plan_ctx(plan);
  cudaStream_t s = (cudaStream_t)stream;
  const int nblk = (int)std::min<long long>(608, (c.ps + 255) / 256);
  L3ES_LAUNCH(c, KK_REDUCE, 4.0 * 3.0 * c.ps * c.batch, s,
              k_field_stats<<<dim3(nblk, c.batch), 256, 0, s>>>(u, c.ps, nblk, c.partial));
  L3ES_LAUNCH(c, KK_REDUCE, 0.0, s,
              k_field_stats_final<<<c.batch, 32, 0, s>>>(c.partial, nblk, 1.0 / (double)c.ps, out_dev));
  return cuda_check(cudaGetLastError(), "l3es_field_stats launch");
}

int l3es_dissipation(l3es_plan* plan, const void* u_hat, double nu, double* out_dev, void* stream) {
  if (!plan || !u_hat || !out_dev) return fail(L3ES_EINVAL, "l3es_dissipation: null argument");
  const Ctx& c = plan_ctx(plan);
  cudaStream_t s = (cudaStream_t)stream;
  const int nblk = (int)std::min<long long>(608, (c.cs / c.h + 7) / 8);  // one warp per row
  const double scale = nu / std::pow((double)c.n, 2 * c.dim);
  if (c.dim == 3)
    L3ES_LAUNCH(c, KK_REDUCE, 8.0 * 3.0 * c.cs * c.batch, s,
                k_diss_partial<3><<<dim3(nblk, c.batch), 256, 0, s>>>((const float2*)u_hat, c.cs, c.n, nblk,
                                                                     c.partial));
  else
    L3ES_LAUNCH(c, KK_REDUCE, 8.0 * 3.0 * c.cs * c.batch, s,
                k_diss_partial<2><<<dim3(nblk, c.batch), 256, 0, s>>>((const float2*)u_hat, c.cs, c.n, nblk,
                                                                     c.partial));
  L3ES_LAUNCH(c, KK_REDUCE, 0.0, s, k_diag_sum<<<c.batch, 256, 0, s>>>(c.partial, nblk, scale, out_dev));
  return cuda_check(cudaGetLastError(), "l3es_dissipation launch");
}

int l3es_energy_spectrum(l3es_plan* plan, const void* u_hat, double mul_fac, double* ek_dev, void* stream) {
  if (!plan || !u_hat || !ek_dev) return fail(L3ES_EINVAL, "l3es_energy_spectrum: null argument");
  const Ctx& c = plan_ctx(plan);
  cudaStream_t s = (cudaStream_t)stream;
  const int n = c.n;
  int rc = cuda_check(cudaMemsetAsync(c.partial, 0, sizeof(double) * 2 * n * c.batch, s), "l3es_energy_spectrum");
  if (rc != L3ES_OK) return rc;
  const int nblk = (int)std::min<long long>(608, (c.cs / c.h + 7) / 8);  // one warp per row
  // |u_hat / n^dim|^2 * mul_fac (utils.py:82-86)
  const double scale = mul_fac / std::pow((double)n, 2 * c.dim);
  const size_t smem = sizeof(double) * 2 * n;
  if (c.dim == 3)
    L3ES_LAUNCH(c, KK_REDUCE, 8.0 * 3.0 * c.cs * c.batch, s,
                k_spectrum<3><<<dim3(nblk, c.batch), 256, smem, s>>>((const float2*)u_hat, c.cs, n, nblk, scale,
                                                                    c.partial));
  else
    L3ES_LAUNCH(c, KK_REDUCE, 8.0 * 3.0 * c.cs * c.batch, s,
                k_spectrum<2><<<dim3(nblk, c.batch), 256, smem, s>>>((const float2*)u_hat, c.cs, n, nblk, scale,
                                                                    c.partial));
  L3ES_LAUNCH(c, KK_REDUCE, 0.0, s,
              k_spectrum_final<<<dim3((n + 127) / 128, c.batch), 128, 0, s>>>(c.partial, n, 2.220446049250313e-16,
                                                                              ek_dev));
  return cuda_check(cudaGetLastError(), "l3es_energy_spectrum launch");
}

}  // extern "C"
