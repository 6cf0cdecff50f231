// Internal host-side declarations shared by the l3es_gb300 translation units.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/l3es_gb300.h"
#include "adjoint_kernels.cuh"
#include "dns_kernels.cuh"

namespace l3es {

// Kernel kinds for the per-launch CUDA-event timer (l3es_plan_kernel_stats).
enum KernelKind {
  KK_X_INV = 0,     // kx_inv with curl prologue (3D RHS: 5 fields, 2D: 6)
  KK_Y_INV,         // ky_pass inverse
  KK_LINE_CROSS,    // line_cross
  KK_Y_FWD,         // ky_pass forward (truncated)
  KK_X_EPI,         // kx_fwd_band (band x-FFT + projection)
  KK_FORCE,         // k_force_ekin
  KK_X_INV_PLAIN,   // kx_inv without curl (irfftn)
  KK_LINE_C2R,      // line_c2r
  KK_LINE_R2C,      // line_r2c
  KK_X_FWD_PLAIN,   // kx_fwd_plain (rfftn)
  KK_REDUCE,        // energy / diagnostic reductions
  KK_FILTER,        // spectral coarsening
  KK_NUFFT_PREP,    // NUFFT deconvolve + pad
  KK_NUFFT_FFT,     // NUFFT fine-grid FFT passes
  KK_NUFFT_GATHER,  // NUFFT gather + advection
  KK_PARTICLE_SORT, // particle binning
  KK_RK_UPDATE,     // k_rk_update (elementwise RK4 combination)
  KK_ADJ_X_INV,     // kx_inv_adjproj (projected cotangent, x inverse, band terms)
  KK_ADJ_LINE,      // line_cross_adj (both adjoint products)
  KK_ADJ_EPI,       // k_adj_epi (vjp assembly + RK4 reverse recursion)
  KK_COUNT
};
const char* kernel_kind_name(int k);

// Records an event pair around every launch while enabled; collect() sums the
// elapsed times per kind after the work has finished.
struct KTimer {
  struct Rec {
    int kind;
    double bytes;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  double ms[KK_COUNT] = {};
  double bytes[KK_COUNT] = {};
  long long launches[KK_COUNT] = {};
  cudaEvent_t get() {
    cudaEvent_t e;
    if (!pool.empty()) {
      e = pool.back();
      pool.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    return e;
  }
  void start(int kind, double nbytes, cudaStream_t s) {
    Rec r{kind, nbytes, get(), get()};
    cudaEventRecord(r.a, s);
    recs.push_back(r);
  }
  void stop(cudaStream_t s) { cudaEventRecord(recs.back().b, s); }
  void collect() {
    for (auto& r : recs) {
      cudaEventSynchronize(r.b);
      float t = 0.f;
      cudaEventElapsedTime(&t, r.a, r.b);
      ms[r.kind] += t;
      bytes[r.kind] += r.bytes;
      launches[r.kind] += 1;
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    recs.clear();
  }
  void reset() {
    collect();
    for (int k = 0; k < KK_COUNT; ++k) {
      ms[k] = 0.0;
      bytes[k] = 0.0;
      launches[k] = 0;
    }
  }
  ~KTimer() {
    for (auto& r : recs) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// Launch with optional per-kernel timing: kind, algorithmic bytes of the launch.
#define L3ES_LAUNCH(ctx, kind, nbytes, stream, ...)                   \
  do {                                                                \
    ::l3es::KTimer* _tm = (ctx).timer;                                \
    if (_tm) _tm->start((kind), (double)(nbytes), (stream));          \
    __VA_ARGS__;                                                      \
    if (_tm) _tm->stop(stream);                                       \
  } while (0)

// Encodes a tiled tensor map of 8-byte elements (no swizzle, no interleave) for bulk
// tensor loads: rank dims (dims[0] contiguous), byte strides of dims 1..rank-1 in
// strides[0..rank-2], box extents `box`. False if the driver entry point is unavailable,
// an address or stride is not 16-byte aligned, or the encoding is rejected.
bool tma_encode(CUtensorMap* map, const void* base, int rank, const unsigned long long* dims,
                const unsigned long long* strides, const unsigned* box);

// Spectra handed to the elementwise and energy kernels are read as float4 (two modes):
// caller arrays must start on a 16-byte boundary (checked at the C entry points).
inline bool misaligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) != 0; }

// Kernel variants of one plan's step (chosen by l3es_plan_autotune; the defaults are the
// measured best at 256^3 on GB300).
struct Schedule {
  int x_bulk = 1;     // 3D x passes by the persistent bulk-tensor-copy kernels (else one tile per CTA);
                      // 2D: the step's x passes in 2-column tiles (else 8)
  int y_var = 0;      // y-pass schedule: KyCfg variant (0: radix 16 from N = 128, 1: radix 8)
  int line_pair = 1;  // line pass: 1 two-for-one (64 <= N <= 256), 2 two-for-one radix 16 and 3 the same
                      // fed by bulk copies (N = 256; 3 is its default), 0 packed
  int band_bulk = -1; // persistent bulk-copy band pass (-1: from N = 256, the measured default)
};

// Geometry + scratch of one plan, handed to the per-N launch wrappers.
struct Ctx {
  int dim = 3, n = 0, h = 0, batch = 1;
  int kd = 0;           // largest kept |k| of the 2/3 cube mask (|k| < 2/3 (N/2+1))
  int kt = 0;           // stored half-axis columns of the nonlinear term (kd+1 -> multiple of TW)
  long long nmid = 1;   // middle-axis length (3D: N, 2D: 1)
  long long cs = 0;     // complex elements per spectral component (nmid*N*H)
  long long fs = 0;     // per field of the 6-field scratch W (== cs)
  long long ds = 0;     // per component of the nonlinear scratch DU (nmid*N*kt)
  long long ps = 0;     // real elements per physical component (N^dim)
  int npartial = 0;     // upper bound on the energy pass's CTAs per trajectory
  long long partial_len = 0;  // doubles per trajectory in `partial`
  float2* tw = nullptr;        // N-point twiddle table + compact table of the N/2-point line FFT
  float2* W = nullptr;         // [batch][6][cs]
  float2* Wx = nullptr;        // 3D: [batch][2][cs] x-transformed u_y, u_z of the RHS
  float2* DU = nullptr;        // [batch][3][ds]
  float2* Tb = nullptr;        // [batch][3][cs] RK stage field
  float2* C = nullptr;         // [batch][3][cs] RK accumulator
  float2* P = nullptr;         // [batch][3][pcs] projected nonlinear term on the kept band
  long long pcs = 0;           // per component of P ((2kd+1)^(dim-1) * kt)
  double* partial = nullptr;   // [batch][partial_len]: reduction partials, any layout of
                               // at most partial_len doubles per trajectory
  double* band = nullptr;      // [batch] constant-power coefficient
  double* e0 = nullptr;        // [batch] ekin_tot targets
  double* einj = nullptr;      // [batch] scratch e_inj
  float* nu_b = nullptr;       // [batch] viscosity per trajectory
  int* err = nullptr;          // device error word: nonzero after a kernel wait timed out
  int step_form = 2;           // explicit RK4 step (run_steps): 0 per-mode update of the whole
                               // spectrum, 1 closed-form stages outside the stage region, 2 the
                               // stage combination fused into the band pass (l3es_plan_set_step_form;
                               // plans start at 2 in 3D, 1 in 2D)
  Schedule sched;              // kernel variants of the step
  int kf = 0;                  // forcing band 0 < |k|^2 <= kf^2
  double eps_inj = 0.0;        // constant-power injection rate
  KTimer* timer = nullptr;     // per-launch timing (nullptr = off)
};

// Launch wrappers for one grid size N (both dims), explicitly instantiated per N.
struct DnsTable {
  // one RK stage: RHS of `us` + epilogue (rk 0..3) into the state S / stage field
  // `out`; rk = -1 writes the RHS itself to `out`
  void (*stage)(const Ctx&, const float2* us, float2* S, float2* out, int rk, const EpiParams& prm,
                cudaStream_t s);
  void (*irfftn)(const Ctx&, const float2* uh, float* u, cudaStream_t s);
  void (*rfftn)(const Ctx&, const float* u, float2* uh, cudaStream_t s);
  // vector-Jacobian product of the RHS at a.us with cotangent a.gscale * a.g, folded
  // into the RK4 reverse recursion (AdjEpi); Wm: [batch][3][cs], Y6: [batch][6][cs]
  void (*vjp)(const Ctx&, const AdjEpi& a, float2* Wm, float2* Y6, cudaStream_t s);
};

// Adjoint scratch of a plan, allocated by the first adjoint call.
struct AdjWork {
  float2* Ua = nullptr;   // [batch][3][cs] RK stage states recomputed from the checkpoint
  float2* Ub = nullptr;
  float2* Uc = nullptr;
  float2* Wm = nullptr;   // [batch][3][cs] projected cotangent lines
  float2* Y6 = nullptr;   // [batch][6][cs] product spectra
  float2* LAM = nullptr;  // [batch][3][cs] accumulated cotangent
  float2* G = nullptr;    // [batch][3][cs] stage cotangent
  float2* Wst[3] = {nullptr, nullptr, nullptr};  // [batch][6][fs] u, curl u lines of U0, Ua, Ub, kept
                                                 // from the stage recomputation for the VJPs
  double* band = nullptr; // [batch][2]
  double* ekin = nullptr; // [batch][3] ekin_tot adjoint: alpha, c_high, c_low
  std::vector<void*> allocs;
};

}  // namespace l3es

struct l3es_plan {
  l3es_plan_desc desc;
  l3es::Ctx ctx;
  l3es::KTimer timer;
  l3es::DnsTable tab;
  int device = 0;
  long long ws_bytes = 0;
  std::vector<void*> allocs;
  l3es::AdjWork adj;
};

namespace l3es {

// Launch table of grid size N (defined in dns_ops.cuh, instantiated per N in dns_n*.cu).
template <int N>
DnsTable make_dns_table();
bool dns_table(int n, DnsTable* out);  // false if N is not compiled in
const Ctx& plan_ctx(const l3es_plan* p);

// Per-block float-float partial sums of w |u_hat|^2 of the plan's trajectories into
// c.partial ([batch][nblk]); returns nblk (plan.cu).
int energy_partials(const Ctx& c, const float2* uh, cudaStream_t s);

// thread-local error reporting
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

}  // namespace l3es
