// Coarsening and exact spectral interpolation kernels shared by the particle
// entry points (templates, so every translation unit may instantiate them).
#pragma once

#include <cuda_runtime.h>

#include "fft_core.cuh"

namespace l3es {

// ------------------------------------------------------------------------------
// Coarse spectrum of spectral_filtering: Hh(f) = 0.5 (C(f) + conj C(p)), with
// C(f) = U_fine(f) / (N/c)^dim on the crop set f in [-c/2, c/2-1]^dim and p the
// crop-set representative of -f mod c. The half-average is fftn(real(ifftn(crop)))
// (utils.py:126-127): it only changes modes with a component at -c/2.
// Output: rfftn layout of the coarse grid, half axis index iz in [0, c/2].
// ------------------------------------------------------------------------------
__device__ __forceinline__ int crop_freq(int i, int c) { return i < c / 2 ? i : i - c; }  // [-c/2, c/2)
__device__ __forceinline__ int crop_wrap(int f, int c) {  // -> [-c/2, c/2)
  f %= c;
  if (f < -c / 2) f += c;
  if (f >= c / 2) f -= c;
  return f;
}

template <int DIM>
__device__ __forceinline__ float2 fine_full(const float2* __restrict__ uh, int N, int fx, int fy, int fz) {
  // full-spectrum value of the rfftn half spectrum at signed frequencies (3D: fx, fy,
  // fz with fz on the half axis; 2D: fx, fy with fy on the half axis)
  const int H = N / 2 + 1;
  if (DIM == 3) {
    if (fz >= 0) return __ldg(uh + ((long long)((fx + N) % N) * N + (fy + N) % N) * H + fz);
    const float2 v = __ldg(uh + ((long long)((-fx + N) % N) * N + (-fy + N) % N) * H + (-fz));
    return make_float2(v.x, -v.y);
  } else {
    if (fy >= 0) return __ldg(uh + (long long)((fx + N) % N) * H + fy);
    const float2 v = __ldg(uh + (long long)((-fx + N) % N) * H + (-fy));
    return make_float2(v.x, -v.y);
  }
}

template <int DIM>
__global__ void __launch_bounds__(256)
k_crop(const float2* __restrict__ uh, long long cs, int N, float2* __restrict__ hh, long long hcs, int c,
       float scale) {
  const int hc = c / 2 + 1;
  const long long per = DIM == 3 ? (long long)c * c * hc : (long long)c * hc;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int comp = blockIdx.y;
  if (i >= per) return;
  int ix, iy, iz;
  if (DIM == 3) {
    iz = (int)(i % hc);
    iy = (int)((i / hc) % c);
    ix = (int)(i / ((long long)hc * c));
  } else {
    iz = 0;
    iy = (int)(i % hc);
    ix = (int)(i / hc);
  }
  const float2* u = uh + comp * cs;
  float2 a, b;
  if (DIM == 3) {
    const int fx = crop_freq(ix, c), fy = crop_freq(iy, c), fz = iz < c / 2 ? iz : -c / 2;
    a = fine_full<3>(u, N, fx, fy, fz);
    b = fine_full<3>(u, N, crop_wrap(-fx, c), crop_wrap(-fy, c), crop_wrap(-fz, c));
  } else {
    const int fx = crop_freq(ix, c), fy = iy < c / 2 ? iy : -c / 2;
    a = fine_full<2>(u, N, fx, fy, 0);
    b = fine_full<2>(u, N, crop_wrap(-fx, c), crop_wrap(-fy, c), 0);
  }
  hh[comp * hcs + i] = make_float2(0.5f * scale * (a.x + b.x), 0.5f * scale * (a.y - b.y));
}

// ------------------------------------------------------------------------------
// Exact spectral interpolation (interp_backend="dft", integrator.py:62-91):
// u_r[j] = Re sum_{k in [-c/2, c/2-1]^dim} Hhat(k) exp(i k.x_j) / c^dim.
// Separable: per (kx[, ky]) an inner sum over the last axis with per-thread phase
// tables in shared memory (exp(i k x) per particle and axis by an FP64 recurrence).
// ------------------------------------------------------------------------------
template <int DIM>
__global__ void __launch_bounds__(128)
k_dft_interp(const float2* __restrict__ hh, long long hcs, int c, int ncomp, const double* __restrict__ r,
             long long np, double* __restrict__ u_r, double dt, double* __restrict__ r_out) {
  extern __shared__ float2 ph[];  // [DIM][c][128]
  const long long j_raw = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = j_raw < np;
  const long long j = valid ? j_raw : 0;
  const int tid = threadIdx.x;
  for (int d = 0; d < DIM; ++d) {
    // exp(i k x) for k = -c/2 .. c/2-1: two FP64 sincos, then p_{k+1} = p_k exp(i x)
    // in FP64 (the recurrence adds ~c ulp; FP64 transcendentals are slow on this GPU)
    const double x = r[j * DIM + d];
    double sn, co, pi, pr;
    sincos(x, &sn, &co);
    sincos(-(double)(c / 2) * x, &pi, &pr);
    for (int k = 0; k < c; ++k) {
      ph[(d * c + k) * 128 + tid] = make_float2((float)pr, (float)pi);
      const double tr = pr * co - pi * sn;
      pi = fma(pr, sn, pi * co);
      pr = tr;
    }
  }
  const int hc = c / 2 + 1;
  double ur[3] = {0.0, 0.0, 0.0};
  for (int comp = 0; comp < ncomp; ++comp) {
    const float2* h = hh + comp * hcs;
    double tot = 0.0;
    if (DIM == 3) {
      for (int kx = -c / 2; kx < c / 2; ++kx) {
        const float2 ex = ph[(0 * c + kx + c / 2) * 128 + tid];
        float2 sx = make_float2(0.f, 0.f);
        for (int ky = -c / 2; ky < c / 2; ++ky) {
          float2 sy = make_float2(0.f, 0.f);
          for (int kz = -c / 2; kz < c / 2; ++kz) {
            float2 v;
            if (kz >= 0) {
              v = __ldg(h + ((long long)((kx + c) % c) * c + (ky + c) % c) * hc + kz);
            } else {
              const float2 t = __ldg(h + ((long long)((-kx + c) % c) * c + (-ky + c) % c) * hc - kz);
              v = make_float2(t.x, -t.y);
            }
            const float2 ez = ph[(2 * c + kz + c / 2) * 128 + tid];
            sy = make_float2(sy.x + v.x * ez.x - v.y * ez.y, sy.y + v.x * ez.y + v.y * ez.x);
          }
          const float2 ey = ph[(1 * c + ky + c / 2) * 128 + tid];
          sx = make_float2(sx.x + sy.x * ey.x - sy.y * ey.y, sx.y + sy.x * ey.y + sy.y * ey.x);
        }
        tot += (double)sx.x * ex.x - (double)sx.y * ex.y;
      }
    } else {
      for (int kx = -c / 2; kx < c / 2; ++kx) {
        const float2 ex = ph[(0 * c + kx + c / 2) * 128 + tid];
        float2 sy = make_float2(0.f, 0.f);
        for (int ky = -c / 2; ky < c / 2; ++ky) {
          float2 v;
          if (ky >= 0) {
            v = __ldg(h + (long long)((kx + c) % c) * hc + ky);
          } else {
            const float2 t = __ldg(h + (long long)((-kx + c) % c) * hc - ky);
            v = make_float2(t.x, -t.y);
          }
          const float2 ey = ph[(1 * c + ky + c / 2) * 128 + tid];
          sy = make_float2(sy.x + v.x * ey.x - v.y * ey.y, sy.y + v.x * ey.y + v.y * ey.x);
        }
        tot += (double)sy.x * ex.x - (double)sy.y * ex.y;
      }
    }
    ur[comp] = tot / pow((double)c, DIM);
  }
  if (!valid) return;
  for (int comp = 0; comp < ncomp; ++comp) u_r[j * ncomp + comp] = ur[comp];
  if (r_out) {
    const double two_pi = 2.0 * 3.14159265358979323846;
    for (int d = 0; d < DIM; ++d) {
      double x = r[j * DIM + d] + dt * ur[d];
      x = x - two_pi * floor(x / two_pi);
      if (x >= two_pi) x -= two_pi;
      r_out[j * DIM + d] = x;
    }
  }
}

}  // namespace l3es
