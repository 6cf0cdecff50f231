// SPH particle relaxation and density on a periodic box (l3es/relax.py:16-178,
// l3es/utils.py:169-218, relaxation block of l3es/combined.py:132-142) for sm_103a.
//
// Particles: n per axis at rest (spacing dx = L / n, mass dx^dim, reference density 1),
// quintic spline kernel with smoothing length dx and cutoff 3 dx, Tait EoS with gamma 1
// and sound speed 10 u_ref.
//
// Neighbour search is a cell list rebuilt on every call:
//   k_sph_bin      wrap (optionally after an Euler predictor), cell id, cell counts
//   k_sph_scan     exclusive scan of the counts (one CTA)
//   k_sph_scatter  slot per particle (atomic, unordered)
//   k_sph_order    stable order inside each cell (rank by input index), so that neighbour
//                  sums run in a fixed order and results are bitwise reproducible; stores
//                  cell-local FP32 coordinates
//   k_sph_density  rho = m sum_j W(|r_ij|)            (kSphLanes lanes per particle, cell order)
//   k_sph_accel    pressure + transport-velocity (and viscous) accelerations
// Cells are cubes of side L / floor(n / 3) >= cutoff, so a 3^dim stencil holds every
// neighbour. Pair geometry is FP32 from cell-local coordinates (offsets below one cell
// side, so the FP32 rounding of a pair distance is ~1e-7 of dx); each lane sums its
// neighbours' FP32 terms in float-float (Ff, error-free FP32 additions: FP64 arithmetic
// is scarce on this GPU and FP64 accumulators kept its FP64 pipe 73-85% busy), the lanes
// combine in FP64, and the density-to-pressure step (rho - 1) is FP64.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "l3es_internal.h"

namespace l3es {

constexpr int kSphThreads = 128;
// Lanes per particle in the neighbour sums: lane q visits candidates q, q + 8, ... of every
// stencil cell and the lanes' FP64 partial sums are added by a fixed shuffle tree, so the
// summation order stays fixed (bitwise reproducible). With one thread per particle a 32^3
// relaxation call kept ~7 warps per SM, each walking ~900 candidates one load after the
// other.
constexpr int kSphLanes = 8;

struct SphGeom {
  double L;      // box side
  double inv_cs; // cells per unit length (nc / L)
  double cs_d;   // cell side L / nc (cell origins; nc * cs_d == L up to FP64 rounding)
  float cs;      // cell side (stencil offsets)
  float Lf;      // box side (FP32, for the nc == 1 minimum image)
  int nc;        // cells per axis (1: every particle is a candidate, minimum image)
  float inv_h;   // 1 / dx
  float cut2;    // (3 dx)^2
};

// position wrapped into [0, L), as the periodic shift of integrator.py:21-23 leaves it
__device__ __forceinline__ double wrap_box(double x, double L) {
  x = x - L * floor(x / L);
  return x >= L ? x - L : x;
}

__device__ __forceinline__ int cell_coord(double x, const SphGeom& g) {
  int c = (int)(x * g.inv_cs);
  return c < 0 ? 0 : (c >= g.nc ? g.nc - 1 : c);
}

// Morris (1997) quintic spline without its normalisation sigma:
//   w(q) = (3-q)_+^5 - 6 (2-q)_+^5 + 15 (1-q)_+^5,  dw/dq = -5 (3-q)_+^4 + 30 (2-q)_+^4 - 75 (1-q)_+^4
__device__ __forceinline__ float quintic_w(float q) {
  const float q3 = fmaxf(0.f, 3.f - q), q2 = fmaxf(0.f, 2.f - q), q1 = fmaxf(0.f, 1.f - q);
  const float a = q3 * q3, b = q2 * q2, c = q1 * q1;
  return a * a * q3 - 6.f * (b * b * q2) + 15.f * (c * c * q1);
}
__device__ __forceinline__ float quintic_dw(float q) {
  const float q3 = fmaxf(0.f, 3.f - q), q2 = fmaxf(0.f, 2.f - q), q1 = fmaxf(0.f, 1.f - q);
  const float a = q3 * q3, b = q2 * q2, c = q1 * q1;
  return -5.f * (a * a) + 30.f * (b * b) - 75.f * (c * c);
}

template <int DIM>
__device__ __forceinline__ int cell_index(const int* ci, int nc) {
  int c = 0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) c = c * nc + ci[d];
  return c;
}

// wrapped position (after x += dt * u when u != null), its cell, cell counts
template <int DIM>
__global__ void __launch_bounds__(kSphThreads)
k_sph_bin(const double* __restrict__ r, const double* __restrict__ u, double dt, long long np, SphGeom g,
          double* __restrict__ xw, int* __restrict__ cell, int* __restrict__ count) {
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= np) return;
  int ci[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    double x = r[j * DIM + d];
    if (u) x += dt * u[j * DIM + d];
    x = wrap_box(x, g.L);
    xw[j * DIM + d] = x;
    ci[d] = cell_coord(x, g);
  }
  const int c = cell_index<DIM>(ci, g.nc);
  cell[j] = c;
  atomicAdd(count + c, 1);
}

// exclusive scan of ncell counts by one CTA of 1024 threads: each thread sums a
// contiguous segment, the segment sums are scanned with warp shuffles
__global__ void __launch_bounds__(1024)
k_sph_scan(const int* __restrict__ count, int ncell, int* __restrict__ start, int* __restrict__ cursor) {
  __shared__ int warp_sum[32];
  const int seg = (ncell + 1023) / 1024;
  const int b = threadIdx.x * seg, e = min(ncell, b + seg);
  int s = 0;
  for (int i = b; i < e; ++i) s += count[i];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_sum[w] = incl;
  __syncthreads();
  if (w == 0) {
    int v = warp_sum[lane], iv = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, iv, o);
      if (lane >= o) iv += t;
    }
    warp_sum[lane] = iv - v;
  }
  __syncthreads();
  int run = warp_sum[w] + incl - s;
  for (int i = b; i < e; ++i) {
    start[i] = run;
    cursor[i] = run;
    run += count[i];
  }
  if (threadIdx.x == 1023) start[ncell] = run;
}

__global__ void __launch_bounds__(kSphThreads)
k_sph_scatter(const int* __restrict__ cell, long long np, int* __restrict__ cursor, int* __restrict__ perm0) {
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < np) perm0[atomicAdd(cursor + cell[j], 1)] = (int)j;
}

// slot of particle perm0[s] = cell start + number of cell members with a smaller input
// index; cell-local FP32 coordinates (and the velocity, when given) in that order
template <int DIM>
__global__ void __launch_bounds__(kSphThreads)
k_sph_order(const int* __restrict__ perm0, const int* __restrict__ cell, const int* __restrict__ start,
            const double* __restrict__ xw, const double* __restrict__ u, long long np, SphGeom g,
            int* __restrict__ perm, float4* __restrict__ xs, float4* __restrict__ us) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= np) return;
  const int j = perm0[s];
  const int c = cell[j];
  const int b = start[c], e = start[c + 1];
  int rank = 0;
  for (int m = b; m < e; ++m) rank += perm0[m] < j;
  const int t = b + rank;
  perm[t] = j;
  float loc[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const double x = xw[(long long)j * DIM + d];
    loc[d] = (float)(x - (double)cell_coord(x, g) * g.cs_d);
  }
  xs[t] = make_float4(loc[0], loc[1], loc[2], 0.f);
  if (us) {
    float v[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < DIM; ++d) v[d] = (float)u[(long long)j * DIM + d];
    us[t] = make_float4(v[0], v[1], v[2], 0.f);
  }
}

// Visits every candidate neighbour of the particle at slot i (cell-local position xi in
// cell ci): f(slot j, dx, dy, dz, r^2) for pairs with r^2 < cut2, the particle itself
// included (r = 0). Cells of the 3^dim stencil are wrapped; the displacement r_i - r_j
// is formed from cell-local coordinates and the stencil offset.
template <int DIM, class F>
__device__ __forceinline__ void for_neighbours(const float4 xi, const int3 ci, const SphGeom& g,
                                               const int* __restrict__ start, const float4* __restrict__ xs, int lane,
                                               F&& f) {
  const int R = g.nc >= 3 ? 1 : 0;
  const int nc = g.nc;
  for (int oz = (DIM == 3 ? -R : 0); oz <= (DIM == 3 ? R : 0); ++oz) {
    int cz = ci.z + oz;
    cz = cz < 0 ? cz + nc : (cz >= nc ? cz - nc : cz);
    for (int oy = -R; oy <= R; ++oy) {
      int cy = ci.y + oy;
      cy = cy < 0 ? cy + nc : (cy >= nc ? cy - nc : cy);
      for (int ox = -R; ox <= R; ++ox) {
        int cx = ci.x + ox;
        cx = cx < 0 ? cx + nc : (cx >= nc ? cx - nc : cx);
        const int c = DIM == 3 ? (cx * nc + cy) * nc + cz : cx * nc + cy;
        const float px = xi.x - (float)ox * g.cs, py = xi.y - (float)oy * g.cs, pz = xi.z - (float)oz * g.cs;
        const int b = start[c], e = start[c + 1];
        for (int jj = b + lane; jj < e; jj += kSphLanes) {
          const float4 xj = xs[jj];
          float dx = px - xj.x, dy = py - xj.y, dz = DIM == 3 ? pz - xj.z : 0.f;
          if (R == 0) {  // one cell: minimum image
            dx -= g.Lf * rintf(dx / g.Lf);
            dy -= g.Lf * rintf(dy / g.Lf);
            if (DIM == 3) dz -= g.Lf * rintf(dz / g.Lf);
          }
          const float r2 = dx * dx + dy * dy + dz * dz;
          if (r2 < g.cut2) f(jj, dx, dy, dz, r2);
        }
      }
    }
  }
}

// sum of v over the kSphLanes lanes of a particle (fixed order), in every lane
__device__ __forceinline__ double lanes_sum(double v) {
#pragma unroll
  for (int o = 1; o < kSphLanes; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// cell coordinates of the particle at slot i, from its FP64 wrapped position
template <int DIM>
__device__ __forceinline__ int3 slot_cell(long long i, const int* __restrict__ perm, const double* __restrict__ xw,
                                          const SphGeom& g) {
  const long long j = perm[i];
  int3 c;
  c.x = cell_coord(xw[j * DIM], g);
  c.y = cell_coord(xw[j * DIM + 1], g);
  c.z = DIM == 3 ? cell_coord(xw[j * DIM + 2], g) : 0;
  return c;
}

// rho[slot] = m sigma sum_j w(r_ij / h); rp[slot] = (rho, p = p_ref (rho - 1)) in FP32
// for the acceleration pass; rho_out[input index] when requested
template <int DIM>
__global__ void __launch_bounds__(kSphThreads)
k_sph_density(const float4* __restrict__ xs, const int* __restrict__ start, const int* __restrict__ perm,
              const double* __restrict__ xw, long long np, SphGeom g, double m_sigma, double p_ref,
              float2* __restrict__ rp, double* __restrict__ rho_out) {
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long i = gt / kSphLanes;
  const int lane = (int)(gt % kSphLanes);
  const bool live = i < np;  // every lane stays for the shuffles
  Ff part{0.f, 0.f};
  if (live) {
    const float4 xi = xs[i];
    const int3 ci = slot_cell<DIM>(i, perm, xw, g);
    const float inv_h = g.inv_h;
    for_neighbours<DIM>(xi, ci, g, start, xs, lane, [&](int, float, float, float, float r2) {
      part = ff_add(part, quintic_w(sqrtf(r2) * inv_h));
    });
  }
  const double acc = lanes_sum((double)part.hi + (double)part.lo);
  if (!live || lane != 0) return;
  const double rho = m_sigma * acc;
  rp[i] = make_float2((float)rho, (float)(p_ref * (rho - 1.0)));
  if (rho_out) rho_out[perm[i]] = rho;
}

enum SphMode { kSphRelaxAcc = 0, kSphRelaxVel = 1, kSphForces = 2 };

struct SphAccelArgs {
  const float4* xs;
  const int* start;
  const int* perm;
  const double* xw;     // wrapped (predicted) positions, input order
  const float2* rp;     // (rho, p) per slot
  const float4* us;     // velocities per slot (forces only)
  long long np;
  float mass, grad_scale, p_ref, eps;  // grad_scale = sigma / h
  // relaxation velocity (combined.py:132-142)
  const double* r0;
  double kick;  // (relax_dt_factor * dt)^2
  double dt;
  double* out0;  // acc | u_out | acc_p
  double* out1;  // r_out (may be null) | acc_visc
  double* out2;  // acc_tvf
};

// Per pair (Adami 2012 eqs. 8, 10, 13 with constant mass, as relax.py:88-105/139-159):
//   pref = m (1/rho_i^2 + 1/rho_j^2), p_ij = (rho_j p_i + rho_i p_j) / (rho_i + rho_j)
//   grad = dW/dr * r_ij / (r + eps)
//   acc_p = -pref p_ij grad, acc_tvf = -pref p_ref grad, acc_visc = pref u_ij dW/dr / (r + eps)
// Relaxation acceleration = acc_p + acc_tvf / 2.
template <int DIM, int MODE>
__global__ void __launch_bounds__(kSphThreads) k_sph_accel(SphAccelArgs a, SphGeom g) {
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long i = gt / kSphLanes;
  const int lane = (int)(gt % kSphLanes);
  const bool live = i < a.np;  // every lane stays for the shuffles
  const long long is = live ? i : 0;
  const float4 xi = a.xs[is];
  const int3 ci = slot_cell<DIM>(is, a.perm, a.xw, g);
  const float2 rpi = a.rp[is];
  const float inv_ri2 = 1.f / (rpi.x * rpi.x);
  const float4 ui = MODE == kSphForces ? a.us[is] : make_float4(0.f, 0.f, 0.f, 0.f);
  Ff fp[3] = {}, ft[3] = {}, fv[3] = {};
  if (live) for_neighbours<DIM>(xi, ci, g, a.start, a.xs, lane, [&](int jj, float dx, float dy, float dz, float r2) {
    const float2 rpj = a.rp[jj];
    const float r = sqrtf(r2);
    const float dw = a.grad_scale * quintic_dw(r * g.inv_h);
    const float pref = a.mass * (inv_ri2 + 1.f / (rpj.x * rpj.x));
    const float pij = (rpj.x * rpi.y + rpi.x * rpj.y) / (rpi.x + rpj.x);
    const float s = dw / (r + a.eps);
    if (MODE == kSphForces) {
      const float cp = -pref * pij * s, ct = -pref * a.p_ref * s;
      fp[0] = ff_add(fp[0], cp * dx); fp[1] = ff_add(fp[1], cp * dy); fp[2] = ff_add(fp[2], cp * dz);
      ft[0] = ff_add(ft[0], ct * dx); ft[1] = ff_add(ft[1], ct * dy); ft[2] = ff_add(ft[2], ct * dz);
      const float4 uj = a.us[jj];
      const float cv = pref * s;
      fv[0] = ff_add(fv[0], cv * (ui.x - uj.x));
      fv[1] = ff_add(fv[1], cv * (ui.y - uj.y));
      fv[2] = ff_add(fv[2], cv * (ui.z - uj.z));
    } else {
      const float cp = -pref * (pij + 0.5f * a.p_ref) * s;
      fp[0] = ff_add(fp[0], cp * dx); fp[1] = ff_add(fp[1], cp * dy); fp[2] = ff_add(fp[2], cp * dz);
    }
  });
  double ap[3], at[3] = {0.0, 0.0, 0.0}, av[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    ap[d] = lanes_sum((double)fp[d].hi + (double)fp[d].lo);
    if (MODE == kSphForces) {
      at[d] = lanes_sum((double)ft[d].hi + (double)ft[d].lo);
      av[d] = lanes_sum((double)fv[d].hi + (double)fv[d].lo);
    }
  }
  if (!live || lane != 0) return;
  const long long j = a.perm[i];
  if (MODE == kSphRelaxAcc) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) a.out0[j * DIM + d] = ap[d];
  } else if (MODE == kSphRelaxVel) {
    // r_temp <- shift(r_temp, kick * acc); u = displacement(r_temp, r0) / dt, with the
    // periodic displacement mod(d + L/2, L) - L/2; optionally r_out = shift(r0, dt u)
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const double x = wrap_box(a.xw[j * DIM + d] + a.kick * ap[d], g.L);
      double dd = x - a.r0[j * DIM + d] + 0.5 * g.L;
      dd = dd - g.L * floor(dd / g.L);
      if (dd >= g.L) dd -= g.L;
      const double uv = (dd - 0.5 * g.L) / a.dt;
      a.out0[j * DIM + d] = uv;
      if (a.out1) a.out1[j * DIM + d] = wrap_box(a.r0[j * DIM + d] + a.dt * uv, g.L);
    }
  } else {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      a.out0[j * DIM + d] = ap[d];
      a.out1[j * DIM + d] = av[d];
      a.out2[j * DIM + d] = at[d];
    }
  }
}

}  // namespace l3es

using namespace l3es;

struct l3es_sph_plan {
  int dim = 3, n = 0;
  long long np_max = 0;
  int ncell = 0;
  SphGeom g{};
  double dx = 0.0, mass = 0.0, sigma = 0.0;
  double* xw = nullptr;    // [np_max * dim] wrapped / predicted positions
  int* cell = nullptr;     // [np_max]
  int* count = nullptr;    // [ncell]
  int* start = nullptr;    // [ncell + 1]
  int* cursor = nullptr;   // [ncell]
  int* perm0 = nullptr;    // [np_max] unordered slots
  int* perm = nullptr;     // [np_max] slot -> input index
  float4* xs = nullptr;    // [np_max] cell-local coordinates per slot
  float4* us = nullptr;    // [np_max] velocity per slot (forces)
  float2* rp = nullptr;    // [np_max] (rho, p) per slot
  std::vector<void*> allocs;
};

static int sph_alloc(l3es_sph_plan* p, void** ptr, size_t bytes, const char* what) {
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(L3ES_ENOMEM, std::string("cudaMalloc(") + what + "): " + cudaGetErrorString(e));
  }
  p->allocs.push_back(*ptr);
  return L3ES_OK;
}

static void sph_free(l3es_sph_plan* p) {
  for (void* a : p->allocs) cudaFree(a);
  p->allocs.clear();
}

// cell list of r (+ dt u_pred when given); leaves xw, perm, xs (and us when u != null)
static int sph_build(l3es_sph_plan* p, const double* r, const double* u_pred, double dt, const double* u,
                     long long np, cudaStream_t s) {
  int rc = cuda_check(cudaMemsetAsync(p->count, 0, sizeof(int) * p->ncell, s), "l3es_sph memset");
  if (rc != L3ES_OK) return rc;
  const unsigned pb = (unsigned)((np + kSphThreads - 1) / kSphThreads);
  if (p->dim == 3) {
    k_sph_bin<3><<<pb, kSphThreads, 0, s>>>(r, u_pred, dt, np, p->g, p->xw, p->cell, p->count);
  } else {
    k_sph_bin<2><<<pb, kSphThreads, 0, s>>>(r, u_pred, dt, np, p->g, p->xw, p->cell, p->count);
  }
  k_sph_scan<<<1, 1024, 0, s>>>(p->count, p->ncell, p->start, p->cursor);
  k_sph_scatter<<<pb, kSphThreads, 0, s>>>(p->cell, np, p->cursor, p->perm0);
  if (p->dim == 3)
    k_sph_order<3><<<pb, kSphThreads, 0, s>>>(p->perm0, p->cell, p->start, p->xw, u, np, p->g, p->perm, p->xs,
                                               u ? p->us : nullptr);
  else
    k_sph_order<2><<<pb, kSphThreads, 0, s>>>(p->perm0, p->cell, p->start, p->xw, u, np, p->g, p->perm, p->xs,
                                               u ? p->us : nullptr);
  return cuda_check(cudaGetLastError(), "l3es_sph cell list");
}

static void sph_density(l3es_sph_plan* p, long long np, double p_ref, double* rho_out, cudaStream_t s) {
  const unsigned pb = (unsigned)((np * kSphLanes + kSphThreads - 1) / kSphThreads);
  const double m_sigma = p->mass * p->sigma;
  if (p->dim == 3)
    k_sph_density<3><<<pb, kSphThreads, 0, s>>>(p->xs, p->start, p->perm, p->xw, np, p->g, m_sigma, p_ref, p->rp,
                                                 rho_out);
  else
    k_sph_density<2><<<pb, kSphThreads, 0, s>>>(p->xs, p->start, p->perm, p->xw, np, p->g, m_sigma, p_ref, p->rp,
                                                 rho_out);
}

template <int MODE>
static void sph_accel(l3es_sph_plan* p, SphAccelArgs& a, cudaStream_t s) {
  const unsigned pb = (unsigned)((a.np * kSphLanes + kSphThreads - 1) / kSphThreads);
  if (p->dim == 3)
    k_sph_accel<3, MODE><<<pb, kSphThreads, 0, s>>>(a, p->g);
  else
    k_sph_accel<2, MODE><<<pb, kSphThreads, 0, s>>>(a, p->g);
}

static SphAccelArgs sph_args(l3es_sph_plan* p, long long np, double u_ref) {
  SphAccelArgs a{};
  a.xs = p->xs;
  a.start = p->start;
  a.perm = p->perm;
  a.xw = p->xw;
  a.rp = p->rp;
  a.us = p->us;
  a.np = np;
  a.mass = (float)p->mass;
  a.grad_scale = (float)(p->sigma / p->dx);
  a.p_ref = (float)(100.0 * u_ref * u_ref);
  a.eps = 2.220446049250313e-16f;
  return a;
}

// plan and particle count; with np == 0 the arrays may be null (the call does nothing)
static int sph_check(l3es_sph_plan* p, const void* r, long long np, const char* who) {
  if (!p) return fail(L3ES_EINVAL, std::string(who) + ": null plan");
  if (np < 0 || np > p->np_max) return fail(L3ES_EINVAL, std::string(who) + ": np outside [0, np_max]");
  if (np > 0 && !r) return fail(L3ES_EINVAL, std::string(who) + ": null positions");
  return L3ES_OK;
}

extern "C" {

int l3es_sph_plan_create(int32_t dim, int32_t n, double box, int64_t np_max, l3es_sph_plan** out) {
  if (!out) return fail(L3ES_EINVAL, "l3es_sph_plan_create: null out");
  *out = nullptr;
  if (dim != 2 && dim != 3) return fail(L3ES_EINVAL, "l3es_sph_plan_create: dim must be 2 or 3");
  if (n < 1 || n > 1024) return fail(L3ES_EINVAL, "l3es_sph_plan_create: n must be in [1, 1024]");
  if (!(box > 0.0) || !std::isfinite(box)) return fail(L3ES_EINVAL, "l3es_sph_plan_create: box must be > 0");
  if (np_max < 1 || np_max > (1LL << 30)) return fail(L3ES_EINVAL, "l3es_sph_plan_create: np_max out of range");
  auto* p = new l3es_sph_plan();
  p->dim = dim;
  p->n = n;
  p->np_max = np_max;
  p->dx = box / n;
  p->mass = std::pow(p->dx, dim);
  // quintic normalisation (Morris 1997): 7 / (478 pi h^2) in 2D, 3 / (359 pi h^3) in 3D
  p->sigma = dim == 3 ? 3.0 / (359.0 * M_PI * p->dx * p->dx * p->dx) : 7.0 / (478.0 * M_PI * p->dx * p->dx);
  int nc = n / 3;  // cell side L / nc >= cutoff 3 dx
  if (nc < 3) nc = 1;
  p->g.L = box;
  p->g.nc = nc;
  p->g.inv_cs = nc / box;
  p->g.cs_d = box / nc;
  p->g.cs = (float)(box / nc);
  p->g.Lf = (float)box;
  p->g.inv_h = (float)(1.0 / p->dx);
  p->g.cut2 = (float)(9.0 * p->dx * p->dx);
  p->ncell = dim == 3 ? nc * nc * nc : nc * nc;
  int rc = L3ES_OK;
  const size_t npm = (size_t)np_max;
  if (rc == L3ES_OK) rc = sph_alloc(p, (void**)&p->xw, sizeof(double) * npm * dim, "xw");
  if (rc == L3ES_OK) rc = sph_alloc(p, (void**)&p->cell, sizeof(int) * npm, "cell");
  if (rc == L3ES_OK) rc = sph_alloc(p, (void**)&p->perm0, sizeof(int) * npm, "perm0");
  if (rc == L3ES_OK) rc = sph_alloc(p, (void**)&p->perm, sizeof(int) * npm, "perm");
  if (rc == L3ES_OK) rc = sph_alloc(p, (void**)&p->xs, sizeof(float4) * npm, "xs");
  if (rc == L3ES_OK) rc = sph_alloc(p, (void**)&p->us, sizeof(float4) * npm, "us");
  if (rc == L3ES_OK) rc = sph_alloc(p, (void**)&p->rp, sizeof(float2) * npm, "rp");
  if (rc == L3ES_OK) rc = sph_alloc(p, (void**)&p->count, sizeof(int) * p->ncell, "count");
  if (rc == L3ES_OK) rc = sph_alloc(p, (void**)&p->cursor, sizeof(int) * p->ncell, "cursor");
  if (rc == L3ES_OK) rc = sph_alloc(p, (void**)&p->start, sizeof(int) * (p->ncell + 1), "start");
  if (rc != L3ES_OK) {
    sph_free(p);
    delete p;
    return rc;
  }
  *out = p;
  return L3ES_OK;
}

int l3es_sph_plan_destroy(l3es_sph_plan* p) {
  if (!p) return L3ES_OK;
  sph_free(p);
  delete p;
  return L3ES_OK;
}

int l3es_sph_density(l3es_sph_plan* p, const double* r, int64_t np, double* rho, void* stream) {
  int rc = sph_check(p, r, np, "l3es_sph_density");
  if (rc != L3ES_OK) return rc;
  if (np == 0) return L3ES_OK;
  if (!rho) return fail(L3ES_EINVAL, "l3es_sph_density: null rho");
  cudaStream_t s = (cudaStream_t)stream;
  rc = sph_build(p, r, nullptr, 0.0, nullptr, np, s);
  if (rc != L3ES_OK) return rc;
  sph_density(p, np, 0.0, rho, s);
  return cuda_check(cudaGetLastError(), "l3es_sph_density launch");
}

int l3es_sph_relax_acceleration(l3es_sph_plan* p, const double* r, int64_t np, double u_ref, double* acc,
                                void* stream) {
  int rc = sph_check(p, r, np, "l3es_sph_relax_acceleration");
  if (rc != L3ES_OK) return rc;
  if (np == 0) return L3ES_OK;
  if (!acc) return fail(L3ES_EINVAL, "l3es_sph_relax_acceleration: null acc");
  cudaStream_t s = (cudaStream_t)stream;
  rc = sph_build(p, r, nullptr, 0.0, nullptr, np, s);
  if (rc != L3ES_OK) return rc;
  const double p_ref = 100.0 * u_ref * u_ref;
  sph_density(p, np, p_ref, nullptr, s);
  SphAccelArgs a = sph_args(p, np, u_ref);
  a.out0 = acc;
  sph_accel<kSphRelaxAcc>(p, a, s);
  return cuda_check(cudaGetLastError(), "l3es_sph_relax_acceleration launch");
}

int l3es_sph_forces(l3es_sph_plan* p, const double* r, const double* u, int64_t np, double u_ref, double* acc_p,
                    double* acc_visc, double* acc_tvf, void* stream) {
  int rc = sph_check(p, r, np, "l3es_sph_forces");
  if (rc != L3ES_OK) return rc;
  if (np == 0) return L3ES_OK;
  if (!u || !acc_p || !acc_visc || !acc_tvf) return fail(L3ES_EINVAL, "l3es_sph_forces: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  rc = sph_build(p, r, nullptr, 0.0, u, np, s);
  if (rc != L3ES_OK) return rc;
  const double p_ref = 100.0 * u_ref * u_ref;
  sph_density(p, np, p_ref, nullptr, s);
  SphAccelArgs a = sph_args(p, np, u_ref);
  a.out0 = acc_p;
  a.out1 = acc_visc;
  a.out2 = acc_tvf;
  sph_accel<kSphForces>(p, a, s);
  return cuda_check(cudaGetLastError(), "l3es_sph_forces launch");
}

int l3es_sph_relax_velocity(l3es_sph_plan* p, const double* r0, const double* u_r, int64_t np, double dt,
                            double relax_dt_factor, double u_ref, double* u_out, double* r_out, void* stream) {
  int rc = sph_check(p, r0, np, "l3es_sph_relax_velocity");
  if (rc != L3ES_OK) return rc;
  if (!(dt != 0.0) || !std::isfinite(dt)) return fail(L3ES_EINVAL, "l3es_sph_relax_velocity: dt must be nonzero");
  if (np == 0) return L3ES_OK;
  if (!u_r || !u_out) return fail(L3ES_EINVAL, "l3es_sph_relax_velocity: null argument");
  if (u_out == u_r || u_out == r0 || (r_out && (r_out == r0 || r_out == u_r || r_out == u_out)))
    return fail(L3ES_EINVAL, "l3es_sph_relax_velocity: outputs must not alias the inputs");
  cudaStream_t s = (cudaStream_t)stream;
  rc = sph_build(p, r0, u_r, dt, nullptr, np, s);
  if (rc != L3ES_OK) return rc;
  const double p_ref = 100.0 * u_ref * u_ref;
  sph_density(p, np, p_ref, nullptr, s);
  SphAccelArgs a = sph_args(p, np, u_ref);
  a.r0 = r0;
  a.kick = (relax_dt_factor * dt) * (relax_dt_factor * dt);
  a.dt = dt;
  a.out0 = u_out;
  a.out1 = r_out;
  sph_accel<kSphRelaxVel>(p, a, s);
  return cuda_check(cudaGetLastError(), "l3es_sph_relax_velocity launch");
}

}  // extern "C"
