// Spectral coarsening, type-2 NUFFT interpolation to particles and periodic
// advection (l3es/utils.py:100-138, l3es/integrator.py:21-91, l3es/combined.py:
// 122-130, :199) for sm_103a.
//
// Data flow of one particle update (fused path of the combined loop):
//   fine u_hat (N)  --k_crop-->  coarse half spectrum Hh (c)       [spectral_filtering]
//   Hh --k_nufft_prep--> fine NUFFT grid G (n = 2c), deconvolved by the ES kernel's
//   Fourier transform --3 c2c passes--> Re g (float) --k_nufft_gather--> u_r,
//   advected r (particles binned by cell so warps gather neighbouring grid points)
// and, when the coarse field itself is wanted, irfftn(Hh) at c (write_u / plots).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "dns_ops.cuh"
#include "l3es_internal.h"
#include "particle_kernels.cuh"

namespace l3es {

// ------------------------------------------------------------------------------
// NUFFT grid: G(g) = Hhat(k) / (psi(kx) psi(ky) psi(kz)) at g = k mod n for k in
// [-c/2, c/2-1]^dim (modes in fftshift order, as finufft receives them from
// integrator.py:38-44), zero elsewhere. Hhat from the coarse half spectrum via
// Hermitian symmetry. inv_psi: 1/psi_hat(k), k = -c/2..c/2-1.
// ------------------------------------------------------------------------------
template <int DIM>
__global__ void __launch_bounds__(256)
k_nufft_prep(const float2* __restrict__ hh, long long hcs, int c, const float* __restrict__ inv_psi,
             float2* __restrict__ g, long long gcs, int n) {
  const long long per = DIM == 3 ? (long long)n * n * n : (long long)n * n;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int comp = blockIdx.y;
  if (i >= per) return;
  int gx, gy, gz;
  if (DIM == 3) {
    gz = (int)(i % n);
    gy = (int)((i / n) % n);
    gx = (int)(i / ((long long)n * n));
  } else {
    gz = 0;
    gy = (int)(i % n);
    gx = (int)(i / n);
  }
  const int kx = gx < n / 2 ? gx : gx - n, ky = gy < n / 2 ? gy : gy - n, kz = gz < n / 2 ? gz : gz - n;
  const int lo = -c / 2, hi = c / 2 - 1;
  float2 out = make_float2(0.f, 0.f);
  const bool in = kx >= lo && kx <= hi && ky >= lo && ky <= hi && (DIM == 2 || (kz >= lo && kz <= hi));
  if (in) {
    const int hc = c / 2 + 1;
    const float2* h = hh + comp * hcs;
    float2 v;
    if (DIM == 3) {
      if (kz >= 0) {
        v = __ldg(h + ((long long)((kx + c) % c) * c + (ky + c) % c) * hc + kz);
      } else {
        const float2 t = __ldg(h + ((long long)((-kx + c) % c) * c + (-ky + c) % c) * hc + (-kz));
        v = make_float2(t.x, -t.y);
      }
      const float s = inv_psi[kx + c / 2] * inv_psi[ky + c / 2] * inv_psi[kz + c / 2];
      out = make_float2(v.x * s, v.y * s);
    } else {
      if (ky >= 0) {
        v = __ldg(h + (long long)((kx + c) % c) * hc + ky);
      } else {
        const float2 t = __ldg(h + (long long)((-kx + c) % c) * hc + (-ky));
        v = make_float2(t.x, -t.y);
      }
      const float s = inv_psi[kx + c / 2] * inv_psi[ky + c / 2];
      out = make_float2(v.x * s, v.y * s);
    }
  }
  g[comp * gcs + i] = out;
}

// ------------------------------------------------------------------------------
// Last NUFFT grid pass: c2c inverse FFT of contiguous lines of n complex values,
// writing only the real part (the interpolant of a real kernel needs no more).
// ------------------------------------------------------------------------------
template <int NL>
__global__ void __launch_bounds__(128)
line_c2c_re(const float2* __restrict__ g, float* __restrict__ gre, long long nlines, const float2* __restrict__ tw,
            float scale) {
  constexpr int E = Fft<NL>::E, T = Fft<NL>::T;
  static_assert(T <= 32, "line inside one warp");
  constexpr int LPC = (32 / T) * 4;
  constexpr int XS = xpad_len<1>(NL);
  __shared__ float2 s_x[LPC * XS];
  const int q = threadIdx.x / T, t = threadIdx.x % T;
  const long long line_raw = (long long)blockIdx.x * LPC + q;
  const bool valid = line_raw < nlines;
  const long long line = valid ? line_raw : nlines - 1;
  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = __ldg(g + line * NL + t + T * e);
  block_fft<NL, E, kInv, 1, true>(v, s_x + q * XS, t, tw, 1);
  if (valid) {
#pragma unroll
    for (int e = 0; e < E; ++e) gre[line * NL + t + T * e] = scale * v[e].x;
  }
}

// ------------------------------------------------------------------------------
// Particle binning by cell (counting sort) so that consecutive threads of the
// gather work on neighbouring grid points. Bins: cubes of (n/nb)^dim fine cells.
// ------------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ int particle_bin(const double* __restrict__ r, long long j, int nb) {
  const double inv = nb / (2.0 * 3.14159265358979323846);
  int b = 0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    int cidx = (int)floor(r[j * DIM + d] * inv);
    cidx = cidx < 0 ? 0 : (cidx >= nb ? nb - 1 : cidx);
    b = b * nb + cidx;
  }
  return b;
}

// Batched plans: trajectory blockIdx.y (blockIdx.x for the scan) has its positions at
// r + b np dim, its bins at count / start + b nbins and its permutation at perm + b np.
template <int DIM>
__global__ void k_bin_count(const double* __restrict__ r, long long np, int nb, int nbins, int* __restrict__ count) {
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  r += (long long)blockIdx.y * np * DIM;
  count += (long long)blockIdx.y * nbins;
  if (j < np) atomicAdd(count + particle_bin<DIM>(r, j, nb), 1);
}

// exclusive scan of nbins counts by one CTA of 1024 threads (chunked)
__global__ void __launch_bounds__(1024) k_bin_scan(const int* __restrict__ count, int nbins, int* __restrict__ start) {
  __shared__ int part[1024];
  count += (long long)blockIdx.x * nbins;
  start += (long long)blockIdx.x * nbins;
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nbins; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < nbins ? count[i] : 0;
    part[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int add = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
      __syncthreads();
      part[threadIdx.x] += add;
      __syncthreads();
    }
    if (i < nbins) start[i] = carry + part[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += part[1023];
    __syncthreads();
  }
}

template <int DIM>
__global__ void k_bin_scatter(const double* __restrict__ r, long long np, int nb, int nbins, int* __restrict__ cursor,
                              int* __restrict__ perm) {
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  r += (long long)blockIdx.y * np * DIM;
  cursor += (long long)blockIdx.y * nbins;
  perm += (long long)blockIdx.y * np;
  if (j < np) perm[atomicAdd(cursor + particle_bin<DIM>(r, j, nb), 1)] = (int)j;
}

// ------------------------------------------------------------------------------
// ES-kernel gather + Euler advection. For particle j (in binned order):
//   u_r[j] = (1 / (n^dim c^dim)) sum_l Re g(l) prod_d phi((x_d/h - l_d) / (w/2))
//   r_out[j] = (r[j] + dt u_r[j]) mod 2 pi                 (integrator.py:21-23)
// phi(z) = exp(beta (sqrt(1 - z^2) - 1)); w-point support per axis.
// Eight lanes per particle (four particles per warp): lane q < W takes support index q
// of the innermost (contiguous) axis and sums over the W^(dim-1) outer support rows, so
// the group's loads of one row are W adjacent floats (one L1 wavefront instead of one
// per particle); the group adds its partial sums by shuffles and lane 0 writes.
// ------------------------------------------------------------------------------
constexpr int kGatherLanes = 8;

template <int DIM, int W>
__global__ void __launch_bounds__(128)
k_nufft_gather(const float* __restrict__ gre, long long gcs, int n, int ncomp, float beta, double norm,
               const double* __restrict__ r, const int* __restrict__ perm, long long np, double* __restrict__ u_r,
               double dt, double* __restrict__ r_out) {
  static_assert(W <= kGatherLanes, "one support row per lane");
  {  // batched plans: trajectory blockIdx.y (its 3-field grid, positions, order, outputs)
    const long long b = blockIdx.y;
    gre += b * 3 * gcs;
    r += b * np * DIM;
    if (perm) perm += b * np;
    u_r += b * np * ncomp;
    if (r_out) r_out += b * np * DIM;
  }
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long i = gt / kGatherLanes;
  const int a = (int)(gt % kGatherLanes);
  const bool live = i < np;  // every lane stays for the group shuffles
  const long long j = live ? (perm ? perm[i] : i) : 0;
  const double two_pi = 2.0 * 3.14159265358979323846;
  const double inv_h = n / two_pi;
  float wk[DIM][W];
  int id[DIM][W];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    // grid coordinate and its offset from the first support point in FP64 (3 FP64
    // operations per axis; FP64 division is avoided: it is slow on this GPU), the W
    // kernel arguments z = (t - a) / (W/2) in FP32
    const double xs = (live ? r[j * DIM + d] : 0.0) * inv_h;
    const double l0 = ceil(xs - 0.5 * W);
    const int il0 = (int)l0;
    const float t = (float)(xs - l0);
#pragma unroll
    for (int q = 0; q < W; ++q) {
      const float z = (t - (float)q) * (2.0f / W);
      const float qq = 1.f - z * z;
      wk[d][q] = qq > 0.f ? expf(beta * (sqrtf(qq) - 1.f)) : 0.f;
      id[d][q] = (il0 + q) & (n - 1);  // n is a power of two; two's complement wraps negatives
    }
  }
  const bool col = live && a < W;
  float wl = 0.f;  // this lane's innermost-axis weight and grid index
  int il = 0;
#pragma unroll
  for (int q = 0; q < W; ++q)
    if (q == a) {
      wl = wk[DIM - 1][q];
      il = id[DIM - 1][q];
    }
  double ur[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    if (comp >= ncomp) break;
    const float* gc = gre + comp * gcs + il;
    float acc = 0.f;
    if (col) {
      if (DIM == 3) {
#pragma unroll
        for (int q0 = 0; q0 < W; ++q0) {
          float sb = 0.f;
#pragma unroll
          for (int q1 = 0; q1 < W; ++q1)
            sb = fmaf(__ldg(gc + ((long long)id[0][q0] * n + id[1][q1]) * n), wk[1][q1], sb);
          acc = fmaf(sb, wk[0][q0], acc);
        }
      } else {
#pragma unroll
        for (int q0 = 0; q0 < W; ++q0) acc = fmaf(__ldg(gc + (long long)id[0][q0] * n), wk[0][q0], acc);
      }
      acc *= wl;
    }
#pragma unroll
    for (int o = kGatherLanes / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    ur[comp] = (double)acc * norm;
  }
  if (!live || a != 0) return;
  for (int comp = 0; comp < ncomp; ++comp) u_r[j * ncomp + comp] = ur[comp];
  if (r_out) {
    for (int d = 0; d < DIM; ++d) {
      double x = r[j * DIM + d] + dt * ur[d];
      x = x - two_pi * floor(x / two_pi);
      if (x >= two_pi) x -= two_pi;  // Python % never returns the modulus itself
      r_out[j * DIM + d] = x;
    }
  }
}

// ------------------------------------------------------------------------------
// Adjoint of the particle interpolation (u_r of l3es_interp as a function of the fine
// half spectrum, at fixed positions), for a cotangent lam = dL/du_r (np, dim):
//   NUFFT: spread (the transpose of k_nufft_gather) -> forward FFT of the n-grid ->
//          k_box_to_half_adj with the deconvolution factors -> k_crop_adj
//   DFT:   k_p2g_dft (sum_j lam_j exp(-i k.r_j) on the c-grid) -> k_box_to_half_adj
//          -> k_crop_adj
// Gradients of complex arrays follow dL = Re sum conj(grad) d(array).
// ------------------------------------------------------------------------------
// gbar[comp](l) += norm lam[j][comp] prod_d phi((x_d / h - l_d) / (w / 2)); lanes as
// in the gather (lane q < W: support column q of the contiguous axis, all outer rows).
// FP32 atomic additions: the order of a grid point's contributions is not fixed.
template <int DIM, int W>
__global__ void __launch_bounds__(128)
k_nufft_spread(float* __restrict__ gbar, long long gcs, int n, int ncomp, float beta, double norm,
               const double* __restrict__ r, const int* __restrict__ perm, long long np,
               const double* __restrict__ lam) {
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long i = gt / kGatherLanes;
  const int a = (int)(gt % kGatherLanes);
  if (i >= np || a >= W) return;
  const long long j = perm ? perm[i] : i;
  const double two_pi = 2.0 * 3.14159265358979323846;
  const double inv_h = n / two_pi;
  float wk[DIM][W];
  int id[DIM][W];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const double xs = r[j * DIM + d] * inv_h;
    const double l0 = ceil(xs - 0.5 * W);
    const int il0 = (int)l0;
    const float t = (float)(xs - l0);
#pragma unroll
    for (int q = 0; q < W; ++q) {
      const float z = (t - (float)q) * (2.0f / W);
      const float qq = 1.f - z * z;
      wk[d][q] = qq > 0.f ? expf(beta * (sqrtf(qq) - 1.f)) : 0.f;
      id[d][q] = (il0 + q) & (n - 1);
    }
  }
  float wl = 0.f;
  int il = 0;
#pragma unroll
  for (int q = 0; q < W; ++q)
    if (q == a) {
      wl = wk[DIM - 1][q];
      il = id[DIM - 1][q];
    }
  for (int comp = 0; comp < ncomp; ++comp) {
    const float v = (float)(norm * lam[j * ncomp + comp]) * wl;
    float* gc = gbar + comp * gcs + il;
    if (DIM == 3) {
#pragma unroll
      for (int q0 = 0; q0 < W; ++q0) {
        const float v0 = v * wk[0][q0];
#pragma unroll
        for (int q1 = 0; q1 < W; ++q1) atomicAdd(gc + ((long long)id[0][q0] * n + id[1][q1]) * n, v0 * wk[1][q1]);
      }
    } else {
#pragma unroll
      for (int q0 = 0; q0 < W; ++q0) atomicAdd(gc + (long long)id[0][q0] * n, v * wk[0][q0]);
    }
  }
}

// forward c2c FFT of contiguous lines of NL real values (imaginary part zero)
template <int NL>
__global__ void __launch_bounds__(128)
line_fft_real_fwd(const float* __restrict__ x, float2* __restrict__ g, long long nlines,
                  const float2* __restrict__ tw) {
  constexpr int E = Fft<NL>::E, T = Fft<NL>::T;
  static_assert(T <= 32, "line inside one warp");
  constexpr int LPC = (32 / T) * 4;
  constexpr int XS = xpad_len<1>(NL);
  __shared__ float2 s_x[LPC * XS];
  const int q = threadIdx.x / T, t = threadIdx.x % T;
  const long long line_raw = (long long)blockIdx.x * LPC + q;
  const bool valid = line_raw < nlines;
  const long long line = valid ? line_raw : nlines - 1;
  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = make_float2(__ldg(x + line * NL + t + T * e), 0.f);
  block_fft<NL, E, kFwd, 1, true>(v, s_x + q * XS, t, tw, 1);
  if (valid) {
#pragma unroll
    for (int e = 0; e < E; ++e) g[line * NL + t + T * e] = v[e];
  }
}

// Adjoint of the reads of the coarse half spectrum by k_nufft_prep (inv_psi: its
// deconvolution factors) or by k_dft_interp (inv_psi == nullptr: factors 1): the box
// mode k in [-c/2, c/2 - 1]^dim reads Hh(k) for a half-axis frequency >= 0 and
// conj Hh(-k) below, so
//   Hb(q) = scale ([q_h <= c/2 - 1] s(k1) G(k1) + [q_h >= 1] s(k2) conj G(k2)),
//   k1 = (cf(q_x), [cf(q_y),] q_h), k2 = (cf(-q_x), [cf(-q_y),] -q_h),
// G on a gn^dim grid in fftfreq order (index k mod gn), cf: the frequency in [-c/2, c/2).
template <int DIM>
__global__ void __launch_bounds__(256)
k_box_to_half_adj(const float2* __restrict__ G, long long gcs, int gn, int c, const float* __restrict__ inv_psi,
                  float scale, float2* __restrict__ hb, long long hcs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int comp = blockIdx.y;
  if (i >= hcs) return;
  const int hc = c / 2 + 1;
  const int qh = (int)(i % hc);
  const int qy = DIM == 3 ? (int)((i / hc) % c) : 0;
  const int qx = DIM == 3 ? (int)(i / ((long long)hc * c)) : (int)(i / hc);
  const float2* g = G + comp * gcs;
  auto cf = [c](int v) { return v < c / 2 ? v : v - c; };
  auto gidx = [gn](int k) { return (k % gn + gn) % gn; };
  auto sfac = [&](int kx, int ky, int kh) {
    if (!inv_psi) return 1.f;
    const float sx = inv_psi[kx + c / 2], sh = inv_psi[kh + c / 2];
    return DIM == 3 ? sx * inv_psi[ky + c / 2] * sh : sx * sh;
  };
  float2 acc = make_float2(0.f, 0.f);
  if (qh <= c / 2 - 1) {
    const int kx = cf(qx), ky = DIM == 3 ? cf(qy) : 0, kh = qh;
    const long long o = DIM == 3 ? ((long long)gidx(kx) * gn + gidx(ky)) * gn + gidx(kh) : (long long)gidx(kx) * gn + gidx(kh);
    const float s = sfac(kx, ky, kh);
    acc.x += s * g[o].x;
    acc.y += s * g[o].y;
  }
  if (qh >= 1) {
    const int kx = cf((c - qx) % c), ky = DIM == 3 ? cf((c - qy) % c) : 0, kh = -qh;
    const long long o = DIM == 3 ? ((long long)gidx(kx) * gn + gidx(ky)) * gn + gidx(kh) : (long long)gidx(kx) * gn + gidx(kh);
    const float s = sfac(kx, ky, kh);
    acc.x += s * g[o].x;
    acc.y -= s * g[o].y;
  }
  hb[comp * hcs + i] = make_float2(scale * acc.x, scale * acc.y);
}

// The coarse real-field cotangent v = c^d irfftn_c(Hb / w) (w: half-axis multiplicity,
// the adjoint of rfftn_c) seen through rfftn_c again: V = rfftn_c(v) = c^d P(Hb / w),
// P the projection onto spectra of real fields, i.e. V = c^d Hb / 2 inside the half
// axis and c^d (Hb(q) + conj Hb(q*)) / 2 on its planes 0 and c/2 (q* = (-q_x, [-q_y,]
// q_h) mod c). k_uncrop_grad then maps V to the fine half spectrum (the adjoint of
// spectral_filtering(irfftn(.)), the convention of the loss gradients).
template <int DIM>
__global__ void __launch_bounds__(256)
k_herm_project(const float2* __restrict__ hb, long long hcs, int c, float cd, float2* __restrict__ V) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int comp = blockIdx.y;
  if (i >= hcs) return;
  const int hc = c / 2 + 1;
  const int qh = (int)(i % hc);
  const float2* h = hb + comp * hcs;
  float2 v = h[i];
  if (qh == 0 || qh == c / 2) {
    const int qy = DIM == 3 ? (int)((i / hc) % c) : 0;
    const int qx = DIM == 3 ? (int)(i / ((long long)hc * c)) : (int)(i / hc);
    const int mx = (c - qx) % c, my = (c - qy) % c;
    const long long m = DIM == 3 ? ((long long)mx * c + my) * hc + qh : (long long)mx * hc + qh;
    const float2 w = h[m];
    v = make_float2(v.x + w.x, v.y - w.y);
  }
  V[comp * hcs + i] = make_float2(0.5f * cd * v.x, 0.5f * cd * v.y);
}

// ------------------------------------------------------------------------------
// Particle -> grid spectrum (turbulence.py:299-339, ur_to_u_dft_wrapper):
// S_c(k) = sum_j u_r[j][c] exp(-i k . r_j) for every k of the N^dim grid in fftfreq
// order. One thread per mode; particles streamed through shared memory in tiles of
// 128 with per-particle 1D phase tables exp(-i k_d x_d) (FP64 recurrence, stored FP32);
// tile sums in FP32, running total in FP64.
// ------------------------------------------------------------------------------
template <int DIM>
__global__ void __launch_bounds__(128)
k_p2g_dft(const double* __restrict__ r, const double* __restrict__ u_r, long long np, int ncomp, int n,
          float2* __restrict__ S, long long scs) {
  extern __shared__ float2 sh[];            // [128][DIM][n] phases
  __shared__ float su[128][3];              // velocities of the tile
  const long long modes = DIM == 3 ? (long long)n * n * n : (long long)n * n;
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = m < modes;
  int ki[3] = {0, 0, 0};
  {
    long long mm = valid ? m : 0;
    for (int d = DIM - 1; d >= 0; --d) {
      const int idx = (int)(mm % n);
      mm /= n;
      ki[d] = idx;  // index in [0, n); frequency kfull(idx, n)
    }
  }
  double acc[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  for (long long base = 0; base < np; base += 128) {
    const int cnt = (int)min((long long)128, np - base);
    __syncthreads();
    // phase tables: thread i fills particle i
    if ((int)threadIdx.x < cnt) {
      const long long j = base + threadIdx.x;
      for (int d = 0; d < DIM; ++d) {
        // exp(-i m x) for m = 0..n/2 by the recurrence p_{m+1} = p_m exp(-i x) in FP64
        // (one sincos per axis; the recurrence adds ~m ulp), negative k by conjugation
        const double x = r[j * DIM + d];
        double sn, cs;
        sincos(-x, &sn, &cs);
        double pr = 1.0, pi = 0.0;
        float2* row = sh + ((long long)threadIdx.x * DIM + d) * n;
        for (int mm = 0; mm <= n / 2; ++mm) {
          const float2 v = make_float2((float)pr, (float)pi);
          if (mm < n / 2) row[mm] = v;
          if (mm > 0) row[n - mm] = make_float2(v.x, -v.y);
          const double tr = pr * cs - pi * sn;
          pi = fma(pr, sn, pi * cs);
          pr = tr;
        }
      }
      for (int c = 0; c < 3; ++c) su[threadIdx.x][c] = c < ncomp ? (float)u_r[j * ncomp + c] : 0.f;
    }
    __syncthreads();
    if (valid) {
      float tacc[3][2] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      for (int q = 0; q < cnt; ++q) {
        float2 ph = sh[((long long)q * DIM + 0) * n + ki[0]];
        for (int d = 1; d < DIM; ++d) {
          const float2 b = sh[((long long)q * DIM + d) * n + ki[d]];
          ph = make_float2(ph.x * b.x - ph.y * b.y, ph.x * b.y + ph.y * b.x);
        }
        for (int c = 0; c < 3; ++c) {
          tacc[c][0] = fmaf(su[q][c], ph.x, tacc[c][0]);
          tacc[c][1] = fmaf(su[q][c], ph.y, tacc[c][1]);
        }
      }
      for (int c = 0; c < 3; ++c) {
        acc[c][0] += tacc[c][0];
        acc[c][1] += tacc[c][1];
      }
    }
  }
  if (valid)
    for (int c = 0; c < 3; ++c) S[c * scs + m] = make_float2((float)acc[c][0], (float)acc[c][1]);
}

// Stages of classical RK4 particle advection through a field held fixed (extension),
// elementwise over the n = np * dim coordinates; v: the velocity at the stage positions.
//   stage 0: acc = v,    rs = wrap(r0 + dt/2 v)
//   stage 1: acc += 2 v, rs = wrap(r0 + dt/2 v)
//   stage 2: acc += 2 v, rs = wrap(r0 + dt v)
//   stage 3: rs = wrap(r0 + dt/6 (acc + v))          (rs = the caller's r_out)
__global__ void k_rk4_particles(int stage, const double* __restrict__ r0, const double* __restrict__ v,
                                double* __restrict__ acc, double* __restrict__ rs, double dt, long long n,
                                double box) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double vi = v[i];
  double x;
  if (stage == 0) {
    acc[i] = vi;
    x = r0[i] + 0.5 * dt * vi;
  } else if (stage == 1) {
    acc[i] += 2.0 * vi;
    x = r0[i] + 0.5 * dt * vi;
  } else if (stage == 2) {
    acc[i] += 2.0 * vi;
    x = r0[i] + dt * vi;
  } else {
    x = r0[i] + dt / 6.0 * (acc[i] + vi);
  }
  x = x - box * floor(x / box);
  if (x >= box) x -= box;
  rs[i] = x;
}

// shift_fn(r, dr) = (r + scale * dr) mod box (integrator.py:21-23), elementwise
__global__ void k_shift(const double* __restrict__ r, const double* __restrict__ dr, long long n, double scale,
                        double box, double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x = r[i] + scale * dr[i];
  x = x - box * floor(x / box);
  if (x >= box) x -= box;
  out[i] = x;
}

// ------------------------------------------------------------------------------
// Coarse-grid MSE loss and its gradient with respect to the fine half spectrum.
// k_mse_resid: in place uc <- 2 (uc - target) / size (components >= ncomp <- 0), FP64
// per-block partial sums of (uc - target)^2.
// k_uncrop_grad: G(k) = wt n(k) / (2 N^d) V(k mod c), V = rfftn_c of the residual,
// n(k) = [k in box] + [-k in box], box = [-c/2, c/2 - 1]^d with fine frequencies in
// [-N/2, N/2 - 1]: the adjoint of irfftn_c(crop(.)) (the crop averages each coarse
// mode with the conjugate of its mirror, and irfftn drops the imaginary part of the
// half-axis planes 0 and N/2, so every stored fine mode inside the box or whose
// mirror is inside contributes with that mode's multiplicity).
// ------------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_mse_resid(float* __restrict__ uc, const float* __restrict__ tgt, long long per, int ncomp, double inv_size,
            double* __restrict__ partial) {
  double acc = 0.0;
  const long long total = 3 * per;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    float v = 0.f;
    if (i < ncomp * per) {
      const double d = (double)uc[i] - (double)tgt[i];
      acc += d * d;
      v = (float)(2.0 * d * inv_size);
    }
    uc[i] = v;
  }
  block_sum_store(acc, partial, blockIdx.x);
}

__global__ void __launch_bounds__(256)
k_mse_sum(const double* __restrict__ partial, int n, double inv_size, double* __restrict__ out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
  __shared__ double tot[1];
  block_sum_store(acc, tot, 0);
  __syncthreads();
  if (threadIdx.x == 0) out[0] = tot[0] * inv_size;
}

__device__ __forceinline__ int signed_freq(int i, int n) { return i < n / 2 ? i : i - n; }

template <int DIM>
__global__ void __launch_bounds__(256)
k_uncrop_grad(const float2* __restrict__ V, long long hcs, int c, int N, long long cs, int ncomp, float scale,
              float2* __restrict__ G) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int comp = blockIdx.y;
  if (i >= cs) return;
  const int H = N / 2 + 1, hc = c / 2 + 1;
  const int kh = (int)(i % H);
  const long long rest = i / H;
  const int mid = DIM == 3 ? (int)(rest % N) : 0;
  const int xi = DIM == 3 ? (int)(rest / N) : (int)rest;
  const int lo = -c / 2, hi = c / 2 - 1;
  const int sx = signed_freq(xi, N), sm = signed_freq(mid, N), sh = signed_freq(kh, N);
  const int nx = signed_freq((N - xi) % N, N), nm = signed_freq((N - mid) % N, N), nh = signed_freq((N - kh) % N, N);
  const bool in_k = sx >= lo && sx <= hi && (DIM == 2 || (sm >= lo && sm <= hi)) && sh >= lo && sh <= hi;
  const bool in_m = nx >= lo && nx <= hi && (DIM == 2 || (nm >= lo && nm <= hi)) && nh >= lo && nh <= hi;
  const int n = (int)in_k + (int)in_m;
  float2 out = make_float2(0.f, 0.f);
  if (n > 0 && comp < ncomp) {
    const int wt = (kh == 0 || kh == N / 2) ? 1 : 2;
    const long long ci = DIM == 3 ? ((long long)(xi % c) * c + (mid % c)) * hc + kh : (long long)(xi % c) * hc + kh;
    const float2 v = V[comp * hcs + ci];
    const float f = scale * (float)(wt * n);
    out = make_float2(f * v.x, f * v.y);
  }
  G[comp * cs + i] = out;
}

}  // namespace l3es

using namespace l3es;

// ES kernel Fourier transform psi_hat(k) = (w / (2n)) int_{-1}^{1} phi(z) cos(pi k z w / n) dz
// by Gauss-Legendre quadrature in FP64 (nodes from Newton iteration on P_m).
static void gauss_legendre(int m, std::vector<double>& x, std::vector<double>& wt) {
  x.resize(m);
  wt.resize(m);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < m; ++i) {
    double z = std::cos(pi * (i + 0.75) / (m + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= m; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      const double dp = m * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= m; ++k) {
      const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    const double dp = m * (z * p1 - p0) / (z * z - 1.0);
    x[i] = z;
    wt[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

struct l3es_interp_plan {
  int dim = 3, c = 32, n = 64, w = 6, n_fine = 0;
  int batch = 1;  // trajectories (batched plans: set_spectrum and the NUFFT interpolation only)
  long long np_max = 0;
  int nb = 16;  // bins per axis
  double beta = 0.0;
  float2* tw = nullptr;      // n-point twiddles
  float2* hh = nullptr;      // [3][coarse half spectrum]
  float2* g = nullptr;       // [3][n^dim]
  float* gre = nullptr;      // [3][n^dim]
  float* inv_psi = nullptr;  // [c]
  float2* twc = nullptr;     // c-point twiddles (particle -> grid inverse transform)
  int* count = nullptr;      // [nb^dim]
  int* start = nullptr;      // [nb^dim]
  int* perm = nullptr;       // [np_max]
  double* red = nullptr;     // [1024] loss partial sums
  double* rk_acc = nullptr;  // [np_max][dim] RK4 advection: velocity accumulator
  double* rk_pos = nullptr;  // [np_max][dim]   stage positions
  double* rk_vel = nullptr;  // [np_max][dim]   stage velocities
  float2* hb = nullptr;      // [3][coarse half spectrum] interpolation adjoint
  l3es_plan* coarse = nullptr;  // size-c transforms (irfftn of Hh, rfftn of a coarse field)
  long long hcs = 0, gcs = 0;
  Ctx gctx;                  // geometry for the grid passes (twiddles only)
  KTimer* timer = nullptr;
  std::vector<void*> allocs;
};

static int ip_alloc(l3es_interp_plan* p, void** ptr, size_t bytes, const char* what) {
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(L3ES_ENOMEM, std::string("cudaMalloc(") + what + "): " + cudaGetErrorString(e));
  }
  p->allocs.push_back(*ptr);
  return L3ES_OK;
}

static void ip_free(l3es_interp_plan* p) {
  for (void* a : p->allocs) cudaFree(a);
  p->allocs.clear();
  if (p->coarse) l3es_plan_destroy(p->coarse);
  p->coarse = nullptr;
}

// inverse c2c of a full 3-component grid of NG^dim complex values (g, in place for
// the strided axes), real part times scale into gre
template <int NG>
static void c2c_inverse_re(int dim, float2* g, float* gre, const float2* tw, float scale, cudaStream_t s) {
  using KY = KyCfg<NG>;
  constexpr int TX = KY::THREADS, TWY = KY::TWY;
  const long long per = dim == 3 ? (long long)NG * NG * NG : (long long)NG * NG;
  if (dim == 3) {
    ky_pass<NG, kInv><<<dim3((NG * NG + TWY - 1) / TWY, 1, 3), TX, 0, s>>>(g, per, NG * NG, NG * NG, NG / 2, tw);
    ky_pass<NG, kInv><<<dim3((NG + TWY - 1) / TWY, NG, 3), TX, 0, s>>>(g, per, NG, NG, NG / 2, tw);
  } else {
    ky_pass<NG, kInv><<<dim3((NG + TWY - 1) / TWY, 1, 3), TX, 0, s>>>(g, per, NG, NG, NG / 2, tw);
  }
  const long long lines = 3 * per / NG;
  constexpr int LPC = (32 / Fft<NG>::T) * 4;
  line_c2c_re<NG><<<(unsigned)((lines + LPC - 1) / LPC), 128, 0, s>>>(g, gre, lines, tw, scale);
}

// strided c2c passes of the NUFFT grid (inverse), via the ky_pass kernel
template <int NG>
static void grid_passes(const l3es_interp_plan* p, cudaStream_t s) {
  using KY = KyCfg<NG>;
  constexpr int TX = KY::THREADS, TWY = KY::TWY;
  const long long per = p->gcs;
  const unsigned nf = 3u * (unsigned)p->batch;  // fields of every trajectory, one after another
  if (p->dim == 3) {
    // x: pencils of stride n^2, columns = (y, z) flattened
    ky_pass<NG, kInv><<<dim3((NG * NG + TWY - 1) / TWY, 1, nf), TX, 0, s>>>(p->g, per, NG * NG, NG * NG, NG / 2, p->tw);
    // y: pencils of stride n inside each x-plane, columns = z
    ky_pass<NG, kInv><<<dim3((NG + TWY - 1) / TWY, NG, nf), TX, 0, s>>>(p->g, per, NG, NG, NG / 2, p->tw);
  } else {
    ky_pass<NG, kInv><<<dim3((NG + TWY - 1) / TWY, 1, nf), TX, 0, s>>>(p->g, per, NG, NG, NG / 2, p->tw);
  }
  const long long lines = (long long)nf * per / NG;
  constexpr int LPC = (32 / Fft<NG>::T) * 4;
  line_c2c_re<NG><<<(unsigned)((lines + LPC - 1) / LPC), 128, 0, s>>>(p->g, p->gre, lines, p->tw, 1.0f);
}

// forward c2c passes of the real NUFFT grid gre (the adjoint of the inverse passes):
// the contiguous axis (real -> complex, into g), then the strided axes in place
template <int NG>
static void grid_fwd_passes(const l3es_interp_plan* p, cudaStream_t s) {
  using KY = KyCfg<NG>;
  constexpr int TX = KY::THREADS, TWY = KY::TWY;
  const long long per = p->gcs;
  const long long lines = 3 * per / NG;
  constexpr int LPC = (32 / Fft<NG>::T) * 4;
  line_fft_real_fwd<NG><<<(unsigned)((lines + LPC - 1) / LPC), 128, 0, s>>>(p->gre, p->g, lines, p->tw);
  if (p->dim == 3) {
    ky_pass<NG, kFwd><<<dim3((NG + TWY - 1) / TWY, NG, 3), TX, 0, s>>>(p->g, per, NG, NG, NG / 2, p->tw);
    ky_pass<NG, kFwd><<<dim3((NG * NG + TWY - 1) / TWY, 1, 3), TX, 0, s>>>(p->g, per, NG * NG, NG * NG, NG / 2, p->tw);
  } else {
    ky_pass<NG, kFwd><<<dim3((NG + TWY - 1) / TWY, 1, 3), TX, 0, s>>>(p->g, per, NG, NG, NG / 2, p->tw);
  }
}

static int run_grid_fwd_passes(const l3es_interp_plan* p, cudaStream_t s) {
  switch (p->n) {
    case 16: grid_fwd_passes<16>(p, s); return L3ES_OK;
    case 32: grid_fwd_passes<32>(p, s); return L3ES_OK;
    case 64: grid_fwd_passes<64>(p, s); return L3ES_OK;
    case 128: grid_fwd_passes<128>(p, s); return L3ES_OK;
    case 256: grid_fwd_passes<256>(p, s); return L3ES_OK;
    default: return fail(L3ES_EINVAL, "NUFFT grid size not supported");
  }
}

static int run_grid_passes(const l3es_interp_plan* p, cudaStream_t s) {
  switch (p->n) {
    case 16: grid_passes<16>(p, s); return L3ES_OK;
    case 32: grid_passes<32>(p, s); return L3ES_OK;
    case 64: grid_passes<64>(p, s); return L3ES_OK;
    case 128: grid_passes<128>(p, s); return L3ES_OK;
    case 256: grid_passes<256>(p, s); return L3ES_OK;
    default: return fail(L3ES_EINVAL, "NUFFT grid size not supported");
  }
}

extern "C" {

int l3es_interp_plan_create(int32_t dim, int32_t n_fine, int32_t ckp_n, int32_t width, int64_t np_max,
                            l3es_interp_plan** out) {
  return l3es_interp_plan_create_batch(dim, n_fine, ckp_n, width, np_max, 1, out);
}

int l3es_interp_plan_create_batch(int32_t dim, int32_t n_fine, int32_t ckp_n, int32_t width, int64_t np_max,
                                  int32_t batch, l3es_interp_plan** out) {
  if (!out) return fail(L3ES_EINVAL, "l3es_interp_plan_create: null out");
  *out = nullptr;
  if (batch < 1) return fail(L3ES_EINVAL, "l3es_interp_plan_create_batch: batch < 1");
  if (batch > 1 && n_fine <= 0)
    return fail(L3ES_EINVAL, "l3es_interp_plan_create_batch: a batched plan needs a fine grid (n_fine > 0)");
  if (dim != 2 && dim != 3) return fail(L3ES_EINVAL, "dim must be 2 or 3");
  if (ckp_n != 8 && ckp_n != 16 && ckp_n != 32 && ckp_n != 64 && ckp_n != 128)
    return fail(L3ES_EINVAL, "ckp_N must be 8, 16, 32, 64 or 128");
  if (n_fine != 0 && (n_fine < ckp_n || (n_fine & (n_fine - 1)) != 0))
    return fail(L3ES_EINVAL, "ckp_N must be <= N (powers of two)");
  if (width != 6 && width != 8 && width != 4) return fail(L3ES_EINVAL, "kernel width must be 4, 6 or 8");
  if (np_max < 0) return fail(L3ES_EINVAL, "np_max < 0");
  auto* p = new l3es_interp_plan();
  p->dim = dim;
  p->c = ckp_n;
  p->n = 2 * ckp_n;
  p->w = width;
  p->n_fine = n_fine;
  p->np_max = np_max;
  p->batch = batch;
  p->beta = 2.30 * width;
  p->nb = p->n / 4;
  const int hc = ckp_n / 2 + 1;
  p->hcs = dim == 3 ? (long long)ckp_n * ckp_n * hc : (long long)ckp_n * hc;
  p->gcs = dim == 3 ? (long long)p->n * p->n * p->n : (long long)p->n * p->n;
  const long long nbins = dim == 3 ? (long long)p->nb * p->nb * p->nb : (long long)p->nb * p->nb;
  int rc = L3ES_OK;
  rc = rc ? rc : ip_alloc(p, (void**)&p->tw, sizeof(float2) * p->n, "twiddles");
  rc = rc ? rc : ip_alloc(p, (void**)&p->hh, sizeof(float2) * 3 * batch * p->hcs, "coarse spectrum");
  rc = rc ? rc : ip_alloc(p, (void**)&p->g, sizeof(float2) * 3 * batch * p->gcs, "nufft grid");
  rc = rc ? rc : ip_alloc(p, (void**)&p->gre, sizeof(float) * 3 * batch * p->gcs, "nufft grid re");
  rc = rc ? rc : ip_alloc(p, (void**)&p->inv_psi, sizeof(float) * ckp_n, "deconvolution");
  rc = rc ? rc : ip_alloc(p, (void**)&p->twc, sizeof(float2) * ckp_n, "coarse twiddles");
  rc = rc ? rc : ip_alloc(p, (void**)&p->count, sizeof(int) * batch * nbins, "bins");
  rc = rc ? rc : ip_alloc(p, (void**)&p->start, sizeof(int) * batch * nbins, "bin starts");
  rc = rc ? rc : ip_alloc(p, (void**)&p->perm, sizeof(int) * batch * (np_max > 0 ? np_max : 1), "permutation");
  rc = rc ? rc : ip_alloc(p, (void**)&p->red, sizeof(double) * 1024, "loss partials");
  const size_t rk_bytes = sizeof(double) * dim * (np_max > 0 ? np_max : 1);
  rc = rc ? rc : ip_alloc(p, (void**)&p->rk_acc, rk_bytes, "rk4 accumulator");
  rc = rc ? rc : ip_alloc(p, (void**)&p->rk_pos, rk_bytes, "rk4 stage positions");
  rc = rc ? rc : ip_alloc(p, (void**)&p->rk_vel, rk_bytes, "rk4 stage velocities");
  rc = rc ? rc : ip_alloc(p, (void**)&p->hb, sizeof(float2) * 3 * p->hcs, "coarse spectrum adjoint");
  if (rc == L3ES_OK) {
    l3es_plan_desc d{};
    d.dim = dim;
    d.n = ckp_n;
    d.batch = 1;
    d.nu = 0.0;
    d.dt = 1.0;
    rc = l3es_plan_create(&d, &p->coarse);
  }
  if (rc != L3ES_OK) {
    ip_free(p);
    delete p;
    return rc;
  }
  // host tables: n-point twiddles (FP64 -> FP32), 1/psi_hat(k) by quadrature
  std::vector<float2> tw(p->n);
  const double pi = 3.14159265358979323846;
  for (int m = 0; m < p->n; ++m) {
    const double a = -2.0 * pi * m / p->n;
    tw[m] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  std::vector<double> zq, wq;
  gauss_legendre(100, zq, wq);
  std::vector<float> ipsi(ckp_n);
  for (int i = 0; i < ckp_n; ++i) {
    const double k = i - ckp_n / 2;
    double sum = 0.0;
    for (size_t q = 0; q < zq.size(); ++q) {
      const double phi = std::exp(p->beta * (std::sqrt(1.0 - zq[q] * zq[q]) - 1.0));
      sum += wq[q] * phi * std::cos(pi * k * zq[q] * width / p->n);
    }
    ipsi[i] = (float)(1.0 / ((double)width / (2.0 * p->n) * sum));
  }
  std::vector<float2> twc(ckp_n);
  for (int m = 0; m < ckp_n; ++m) {
    const double a = -2.0 * pi * m / ckp_n;
    twc[m] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  cudaError_t e = cudaMemcpy(p->tw, tw.data(), sizeof(float2) * p->n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->inv_psi, ipsi.data(), sizeof(float) * ckp_n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->twc, twc.data(), sizeof(float2) * ckp_n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    rc = cuda_check(e, "l3es_interp_plan_create");
    ip_free(p);
    delete p;
    return rc;
  }
  *out = p;
  return L3ES_OK;
}

int l3es_interp_plan_destroy(l3es_interp_plan* p) {
  if (!p) return L3ES_OK;
  ip_free(p);
  delete p;
  return L3ES_OK;
}

int l3es_interp_set_spectrum(l3es_interp_plan* p, const void* u_hat_fine, void* stream) {
  if (!p || !u_hat_fine) return fail(L3ES_EINVAL, "l3es_interp_set_spectrum: null argument");
  if (p->n_fine <= 0) return fail(L3ES_ESTATE, "plan was created without a fine grid (n_fine = 0)");
  cudaStream_t s = (cudaStream_t)stream;
  const int N = p->n_fine, c = p->c;
  const long long cs = p->dim == 3 ? (long long)N * N * (N / 2 + 1) : (long long)N * (N / 2 + 1);
  const float scale = (float)std::pow((double)c / N, p->dim);
  const unsigned blocks = (unsigned)((p->hcs + 255) / 256);
  const unsigned nf = 3u * (unsigned)p->batch;  // batched: [batch][3] fine spectra in, [batch][3] coarse out
  if (p->dim == 3)
    k_crop<3><<<dim3(blocks, nf), 256, 0, s>>>((const float2*)u_hat_fine, cs, N, p->hh, p->hcs, c, scale);
  else
    k_crop<2><<<dim3(blocks, nf), 256, 0, s>>>((const float2*)u_hat_fine, cs, N, p->hh, p->hcs, c, scale);
  return cuda_check(cudaGetLastError(), "l3es_interp_set_spectrum launch");
}

int l3es_interp_set_field(l3es_interp_plan* p, const float* u_coarse, void* stream) {
  if (!p || !u_coarse) return fail(L3ES_EINVAL, "l3es_interp_set_field: null argument");
  if (p->batch > 1) return fail(L3ES_EINVAL, "l3es_interp_set_field: not for batched plans");
  return l3es_rfftn(p->coarse, u_coarse, p->hh, stream);
}

int l3es_interp_coarse_field(l3es_interp_plan* p, float* u_coarse, void* stream) {
  if (!p || !u_coarse) return fail(L3ES_EINVAL, "l3es_interp_coarse_field: null argument");
  if (p->batch > 1) return fail(L3ES_EINVAL, "l3es_interp_coarse_field: not for batched plans");
  return l3es_irfftn(p->coarse, p->hh, u_coarse, stream);
}

int l3es_interp_coarse_spectrum(l3es_interp_plan* p, void* out, void* stream) {
  if (!p || !out) return fail(L3ES_EINVAL, "l3es_interp_coarse_spectrum: null argument");
  if (p->batch > 1) return fail(L3ES_EINVAL, "l3es_interp_coarse_spectrum: not for batched plans");
  return cuda_check(cudaMemcpyAsync(out, p->hh, sizeof(float2) * 3 * p->hcs, cudaMemcpyDeviceToDevice,
                                    (cudaStream_t)stream),
                    "l3es_interp_coarse_spectrum");
}

}  // extern "C"

// Exact interpolation (dft backend) at r into u_r, with the fused Euler shift when r_out.
static int dft_eval(l3es_interp_plan* p, const double* r, int64_t np, double* u_r, double dt, double* r_out,
                    cudaStream_t s) {
  const int ncomp = p->dim;
  const unsigned pb = (unsigned)((np + 127) / 128);
  const size_t smem = sizeof(float2) * p->dim * p->c * 128;
  if (p->dim == 3) {
    cudaFuncSetAttribute(k_dft_interp<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_dft_interp<3><<<pb, 128, smem, s>>>(p->hh, p->hcs, p->c, ncomp, r, np, u_r, dt, r_out);
  } else {
    cudaFuncSetAttribute(k_dft_interp<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_dft_interp<2><<<pb, 128, smem, s>>>(p->hh, p->hcs, p->c, ncomp, r, np, u_r, dt, r_out);
  }
  return cuda_check(cudaGetLastError(), "l3es_interp (dft) launch");
}

// NUFFT gather at r from the prepared fine grid (nufft_grid), visiting particles in the
// bin order of the positions nufft_grid was given; fused Euler shift when r_out.
static int nufft_eval(l3es_interp_plan* p, const double* r, int64_t np, double* u_r, double dt, double* r_out,
                      cudaStream_t s) {
  const int ncomp = p->dim;
  const double norm = 1.0 / (std::pow((double)p->n, p->dim) * std::pow((double)p->c, p->dim));
  const float beta = (float)p->beta;
  const dim3 gblk((unsigned)((np * kGatherLanes + 127) / 128), (unsigned)p->batch);
#define L3ES_GATHER(D, W)                                                                                   \
  k_nufft_gather<D, W><<<gblk, 128, 0, s>>>(p->gre, p->gcs, p->n, ncomp, beta, norm, r, p->perm, np, u_r, dt, \
                                          r_out)
  if (p->dim == 3) {
    if (p->w == 6) L3ES_GATHER(3, 6);
    else if (p->w == 8) L3ES_GATHER(3, 8);
    else L3ES_GATHER(3, 4);
  } else {
    if (p->w == 6) L3ES_GATHER(2, 6);
    else if (p->w == 8) L3ES_GATHER(2, 8);
    else L3ES_GATHER(2, 4);
  }
#undef L3ES_GATHER
  return cuda_check(cudaGetLastError(), "l3es_interp launch");
}

static int nufft_grid(l3es_interp_plan* p, const double* r, int64_t np, cudaStream_t s);

extern "C" {

int l3es_interp(l3es_interp_plan* p, const double* r, int64_t np, double* u_r, int32_t backend, double dt,
                double* r_out, void* stream) {
  if (!p || !r || !u_r) return fail(L3ES_EINVAL, "l3es_interp: null argument");
  if (np < 0 || np > p->np_max) return fail(L3ES_EINVAL, "l3es_interp: np outside [0, np_max]");
  if (backend != 0 && backend != 1) return fail(L3ES_EINVAL, "l3es_interp: backend must be 0 (nufft) or 1 (dft)");
  if (p->batch > 1 && backend != 0) return fail(L3ES_EINVAL, "l3es_interp: batched plans interpolate by NUFFT only");
  if (np == 0) return L3ES_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (backend == 1) return dft_eval(p, r, np, u_r, dt, r_out, s);
  const int rc = nufft_grid(p, r, np, s);
  return rc != L3ES_OK ? rc : nufft_eval(p, r, np, u_r, dt, r_out, s);
}

int l3es_interp_advect_rk4(l3es_interp_plan* p, const double* r, int64_t np, double* u_r, int32_t backend,
                           double dt, double* r_out, void* stream) {
  if (!p || !r || !u_r || !r_out) return fail(L3ES_EINVAL, "l3es_interp_advect_rk4: null argument");
  if (np < 0 || np > p->np_max) return fail(L3ES_EINVAL, "l3es_interp_advect_rk4: np outside [0, np_max]");
  if (backend != 0 && backend != 1)
    return fail(L3ES_EINVAL, "l3es_interp_advect_rk4: backend must be 0 (nufft) or 1 (dft)");
  if (r_out == r || u_r == r || u_r == r_out)
    return fail(L3ES_EINVAL, "l3es_interp_advect_rk4: r, u_r and r_out must be separate arrays");
  if (p->batch > 1) return fail(L3ES_EINVAL, "l3es_interp_advect_rk4: not for batched plans");
  if (np == 0) return L3ES_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = backend == 0 ? nufft_grid(p, r, np, s) : L3ES_OK;  // one grid, bins of r reused by every stage
  const long long n = np * p->dim;
  const unsigned eb = (unsigned)((n + 255) / 256);
  const double box = 2.0 * 3.14159265358979323846;
  for (int stage = 0; stage < 4 && rc == L3ES_OK; ++stage) {
    const double* pos = stage == 0 ? r : p->rk_pos;
    double* vel = stage == 0 ? u_r : p->rk_vel;  // u_r: the velocity at the old positions
    rc = backend == 0 ? nufft_eval(p, pos, np, vel, 0.0, nullptr, s) : dft_eval(p, pos, np, vel, 0.0, nullptr, s);
    if (rc != L3ES_OK) break;
    k_rk4_particles<<<eb, 256, 0, s>>>(stage, r, vel, p->rk_acc, stage == 3 ? r_out : p->rk_pos, dt, n, box);
    rc = cuda_check(cudaGetLastError(), "l3es_interp_advect_rk4 launch");
  }
  return rc;
}

}  // extern "C"

// Fine NUFFT grid of the plan's coarse spectrum (deconvolve, zero-pad, 3 c2c passes, Re)
// and the bin order of the positions r.
static int bin_particles(l3es_interp_plan* p, const double* r, int64_t np, cudaStream_t s);

static int nufft_grid(l3es_interp_plan* p, const double* r, int64_t np, cudaStream_t s) {
  const unsigned gb = (unsigned)((p->gcs + 255) / 256);
  const unsigned nf = 3u * (unsigned)p->batch;
  if (p->dim == 3)
    k_nufft_prep<3><<<dim3(gb, nf), 256, 0, s>>>(p->hh, p->hcs, p->c, p->inv_psi, p->g, p->gcs, p->n);
  else
    k_nufft_prep<2><<<dim3(gb, nf), 256, 0, s>>>(p->hh, p->hcs, p->c, p->inv_psi, p->g, p->gcs, p->n);
  const int rc = run_grid_passes(p, s);
  return rc != L3ES_OK ? rc : bin_particles(p, r, np, s);
}

// counting sort of the particles by cell into p->perm
static int bin_particles(l3es_interp_plan* p, const double* r, int64_t np, cudaStream_t s) {
  const dim3 pb((unsigned)((np + 127) / 128), (unsigned)p->batch);
  const int nbins = p->dim == 3 ? p->nb * p->nb * p->nb : p->nb * p->nb;
  int rc = cuda_check(cudaMemsetAsync(p->count, 0, sizeof(int) * nbins * p->batch, s), "l3es_interp memset");
  if (rc != L3ES_OK) return rc;
  if (p->dim == 3) {
    k_bin_count<3><<<pb, 128, 0, s>>>(r, np, p->nb, nbins, p->count);
    k_bin_scan<<<p->batch, 1024, 0, s>>>(p->count, nbins, p->start);
    k_bin_scatter<3><<<pb, 128, 0, s>>>(r, np, p->nb, nbins, p->start, p->perm);
  } else {
    k_bin_count<2><<<pb, 128, 0, s>>>(r, np, p->nb, nbins, p->count);
    k_bin_scan<<<p->batch, 1024, 0, s>>>(p->count, nbins, p->start);
    k_bin_scatter<2><<<pb, 128, 0, s>>>(r, np, p->nb, nbins, p->start, p->perm);
  }
  return cuda_check(cudaGetLastError(), "l3es_interp grid launch");
}

extern "C" {

int l3es_interp_vjp(l3es_interp_plan* p, const double* r, int64_t np, const double* lam, int32_t backend,
                    void* grad_fine, void* stream) {
  if (!p || !r || !lam || !grad_fine) return fail(L3ES_EINVAL, "l3es_interp_vjp: null argument");
  if (p->batch > 1) return fail(L3ES_EINVAL, "l3es_interp_vjp: not for batched plans");
  if (p->n_fine <= 0) return fail(L3ES_ESTATE, "l3es_interp_vjp: plan was created without a fine grid (n_fine = 0)");
  if (np < 0 || np > p->np_max) return fail(L3ES_EINVAL, "l3es_interp_vjp: np outside [0, np_max]");
  if (backend != 0 && backend != 1) return fail(L3ES_EINVAL, "l3es_interp_vjp: backend must be 0 (nufft) or 1 (dft)");
  cudaStream_t s = (cudaStream_t)stream;
  const int N = p->n_fine, c = p->c, dim = p->dim;
  const long long cs = dim == 3 ? (long long)N * N * (N / 2 + 1) : (long long)N * (N / 2 + 1);
  int rc = L3ES_OK;
  if (np == 0) return cuda_check(cudaMemsetAsync(grad_fine, 0, sizeof(float2) * 3 * cs, s), "l3es_interp_vjp memset");
  const unsigned hbk = (unsigned)((p->hcs + 255) / 256);
  if (backend == 1) {
    // S(k) = sum_j lam_j exp(-i k.r_j) on the c-grid (into p->g), then / c^dim
    const long long modes = dim == 3 ? (long long)c * c * c : (long long)c * c;
    const size_t smem = sizeof(float2) * 128 * dim * c;
    if (smem > 200 * 1024) return fail(L3ES_EINVAL, "l3es_interp_vjp: ckp_N too large for the dft backend");
    const float scale = (float)(1.0 / (double)modes);
    if (dim == 3) {
      cudaFuncSetAttribute(k_p2g_dft<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_p2g_dft<3><<<(unsigned)((modes + 127) / 128), 128, smem, s>>>(r, lam, np, 3, c, p->g, modes);
      k_box_to_half_adj<3><<<dim3(hbk, 3), 256, 0, s>>>(p->g, modes, c, c, nullptr, scale, p->hb, p->hcs);
    } else {
      cudaFuncSetAttribute(k_p2g_dft<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_p2g_dft<2><<<(unsigned)((modes + 127) / 128), 128, smem, s>>>(r, lam, np, 2, c, p->g, modes);
      k_box_to_half_adj<2><<<dim3(hbk, 3), 256, 0, s>>>(p->g, modes, c, c, nullptr, scale, p->hb, p->hcs);
    }
  } else {
    rc = bin_particles(p, r, np, s);
    if (rc == L3ES_OK) rc = cuda_check(cudaMemsetAsync(p->gre, 0, sizeof(float) * 3 * p->gcs, s), "l3es_interp_vjp memset");
    if (rc != L3ES_OK) return rc;
    const double norm = 1.0 / (std::pow((double)p->n, dim) * std::pow((double)c, dim));
    const float beta = (float)p->beta;
    const unsigned gblk = (unsigned)((np * kGatherLanes + 127) / 128);
#define L3ES_SPREAD(D, W) \
  k_nufft_spread<D, W><<<gblk, 128, 0, s>>>(p->gre, p->gcs, p->n, dim, beta, norm, r, p->perm, np, lam)
    if (dim == 3) {
      if (p->w == 6) L3ES_SPREAD(3, 6);
      else if (p->w == 8) L3ES_SPREAD(3, 8);
      else L3ES_SPREAD(3, 4);
    } else {
      if (p->w == 6) L3ES_SPREAD(2, 6);
      else if (p->w == 8) L3ES_SPREAD(2, 8);
      else L3ES_SPREAD(2, 4);
    }
#undef L3ES_SPREAD
    rc = run_grid_fwd_passes(p, s);
    if (rc != L3ES_OK) return rc;
    if (dim == 3)
      k_box_to_half_adj<3><<<dim3(hbk, 3), 256, 0, s>>>(p->g, p->gcs, p->n, c, p->inv_psi, 1.f, p->hb, p->hcs);
    else
      k_box_to_half_adj<2><<<dim3(hbk, 3), 256, 0, s>>>(p->g, p->gcs, p->n, c, p->inv_psi, 1.f, p->hb, p->hcs);
  }
  // coarse cotangent -> fine half spectrum (p->g is free again: V goes there)
  const float cd = (float)std::pow((double)c, dim);
  const float uscale = (float)(0.5 / std::pow((double)N, dim));
  const dim3 gb((unsigned)((cs + 255) / 256), 3);
  if (dim == 3) {
    k_herm_project<3><<<dim3(hbk, 3), 256, 0, s>>>(p->hb, p->hcs, c, cd, p->g);
    k_uncrop_grad<3><<<gb, 256, 0, s>>>(p->g, p->hcs, c, N, cs, 3, uscale, (float2*)grad_fine);
  } else {
    k_herm_project<2><<<dim3(hbk, 3), 256, 0, s>>>(p->hb, p->hcs, c, cd, p->g);
    k_uncrop_grad<2><<<gb, 256, 0, s>>>(p->g, p->hcs, c, N, cs, 2, uscale, (float2*)grad_fine);
  }
  return cuda_check(cudaGetLastError(), "l3es_interp_vjp launch");
}

int l3es_interp_particles_to_grid(l3es_interp_plan* p, const double* r, const double* u_r, int64_t np,
                                  float* u_grid, void* stream) {
  if (!p || !r || !u_r || !u_grid) return fail(L3ES_EINVAL, "l3es_interp_particles_to_grid: null argument");
  if (p->batch > 1) return fail(L3ES_EINVAL, "l3es_interp_particles_to_grid: not for batched plans");
  if (np < 0) return fail(L3ES_EINVAL, "l3es_interp_particles_to_grid: np < 0");
  cudaStream_t s = (cudaStream_t)stream;
  const int c = p->c;
  const long long modes = p->dim == 3 ? (long long)c * c * c : (long long)c * c;
  // the NUFFT grid buffers (n = 2c) hold the c^dim spectrum and its real transform
  const size_t smem = sizeof(float2) * 128 * p->dim * c;
  if (smem > 200 * 1024) return fail(L3ES_EINVAL, "l3es_interp_particles_to_grid: grid too large");
  if (p->dim == 3) {
    cudaFuncSetAttribute(k_p2g_dft<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_p2g_dft<3><<<(unsigned)((modes + 127) / 128), 128, smem, s>>>(r, u_r, np, 3, c, p->g, modes);
  } else {
    cudaFuncSetAttribute(k_p2g_dft<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_p2g_dft<2><<<(unsigned)((modes + 127) / 128), 128, smem, s>>>(r, u_r, np, 2, c, p->g, modes);
  }
  // u_grid = real(ifftn(S)) (ifftn carries 1/c^dim)
  const float scale = (float)(1.0 / (double)modes);
  switch (c) {
    case 8: c2c_inverse_re<8>(p->dim, p->g, u_grid, p->twc, scale, s); break;
    case 16: c2c_inverse_re<16>(p->dim, p->g, u_grid, p->twc, scale, s); break;
    case 32: c2c_inverse_re<32>(p->dim, p->g, u_grid, p->twc, scale, s); break;
    case 64: c2c_inverse_re<64>(p->dim, p->g, u_grid, p->twc, scale, s); break;
    case 128: c2c_inverse_re<128>(p->dim, p->g, u_grid, p->twc, scale, s); break;
    default: return fail(L3ES_EINVAL, "l3es_interp_particles_to_grid: unsupported grid");
  }
  return cuda_check(cudaGetLastError(), "l3es_interp_particles_to_grid launch");
}

int l3es_interp_coarse_mse(l3es_interp_plan* p, const void* u_hat_fine, const float* target, double* loss_dev,
                           void* grad, void* stream) {
  if (!p || !u_hat_fine || !target || !loss_dev) return fail(L3ES_EINVAL, "l3es_interp_coarse_mse: null argument");
  if (p->batch > 1) return fail(L3ES_EINVAL, "l3es_interp_coarse_mse: not for batched plans");
  if (p->n_fine <= 0) return fail(L3ES_ESTATE, "plan was created without a fine grid (n_fine = 0)");
  if (grad == u_hat_fine) return fail(L3ES_EINVAL, "l3es_interp_coarse_mse: grad must not alias u_hat_fine");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = l3es_interp_set_spectrum(p, u_hat_fine, stream);
  if (rc == L3ES_OK) rc = l3es_irfftn(p->coarse, p->hh, p->gre, stream);  // coarse field (3, c^d)
  if (rc != L3ES_OK) return rc;
  const int c = p->c, N = p->n_fine;
  const long long per = p->dim == 3 ? (long long)c * c * c : (long long)c * c;
  const double inv_size = 1.0 / ((double)p->dim * per);
  const int nblk = (int)std::min<long long>(1024, (3 * per + 255) / 256);
  k_mse_resid<<<nblk, 256, 0, s>>>(p->gre, target, per, p->dim, inv_size, p->red);
  k_mse_sum<<<1, 256, 0, s>>>(p->red, nblk, inv_size, loss_dev);
  rc = cuda_check(cudaGetLastError(), "l3es_interp_coarse_mse launch");
  if (rc != L3ES_OK || !grad) return rc;
  rc = l3es_rfftn(p->coarse, p->gre, p->g, stream);  // V = rfftn_c(residual)
  if (rc != L3ES_OK) return rc;
  const long long cs = p->dim == 3 ? (long long)N * N * (N / 2 + 1) : (long long)N * (N / 2 + 1);
  const float scale = (float)(0.5 / std::pow((double)N, p->dim));
  const dim3 gb((unsigned)((cs + 255) / 256), 3);
  if (p->dim == 3)
    k_uncrop_grad<3><<<gb, 256, 0, s>>>(p->g, p->hcs, c, N, cs, 3, scale, (float2*)grad);
  else
    k_uncrop_grad<2><<<gb, 256, 0, s>>>(p->g, p->hcs, c, N, cs, 2, scale, (float2*)grad);
  return cuda_check(cudaGetLastError(), "l3es_interp_coarse_mse launch");
}

int l3es_shift(const double* r, const double* dr, int64_t n, double scale, double box, double* out, void* stream) {
  if (!r || !dr || !out) return fail(L3ES_EINVAL, "l3es_shift: null argument");
  if (n <= 0) return n == 0 ? L3ES_OK : fail(L3ES_EINVAL, "l3es_shift: n < 0");
  k_shift<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(r, dr, n, scale, box, out);
  return cuda_check(cudaGetLastError(), "l3es_shift launch");
}

}  // extern "C"
