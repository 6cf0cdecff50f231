// Plan management and the C ABI of the DNS step (include/l3es_gb300.h).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "l3es_internal.h"

namespace l3es {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return L3ES_OK;
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return L3ES_ECUDA;
}

const char* kernel_kind_name(int k) {
  static const char* names[KK_COUNT] = {
      "kx_inv_curl", "ky_pass_inv", "line_cross", "ky_pass_fwd", "kx_fwd_band",
      "force_ekin", "kx_inv", "line_c2r", "line_r2c", "kx_fwd", "reduce",
      "filter", "nufft_prep", "nufft_fft", "nufft_gather", "particle_sort", "rk_update",
      "kx_inv_adjproj", "line_cross_adj", "adj_epilogue"};
  return (k >= 0 && k < KK_COUNT) ? names[k] : "";
}

const Ctx& plan_ctx(const l3es_plan* p) { return p->ctx; }

bool tma_encode(CUtensorMap* map, const void* base, int rank, const unsigned long long* dims,
                const unsigned long long* strides, const unsigned* box) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      fn = nullptr;
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode || rank < 1 || rank > 5 || ((uintptr_t)base & 15u)) return false;
  cuuint64_t d[5];
  cuuint64_t st[4];
  cuuint32_t b[5], es[5];
  for (int i = 0; i < rank; ++i) {
    d[i] = dims[i];
    b[i] = box[i];
    es[i] = 1;
    if (i + 1 < rank) {
      if (strides[i] & 15u) return false;
      st[i] = strides[i];
    }
  }
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_INT64, (cuuint32_t)rank, const_cast<void*>(base), d, st, b, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool dns_table(int n, DnsTable* out) {
  switch (n) {
    case 8: *out = make_dns_table<8>(); return true;
    case 16: *out = make_dns_table<16>(); return true;
    case 32: *out = make_dns_table<32>(); return true;
    case 64: *out = make_dns_table<64>(); return true;
    case 128: *out = make_dns_table<128>(); return true;
    case 256: *out = make_dns_table<256>(); return true;
    case 512: *out = make_dns_table<512>(); return true;
    default: return false;
  }
}

// Largest |k| kept by the cube mask |k_i| < 2/3 (N/2+1) (spectral_solver.py:42-48),
// with the reference's float64 comparison.
static int dealias_kd(int n) {
  const double kmax = 2.0 / 3.0 * (double)(n / 2 + 1);
  int kd = 0;
  while ((double)(kd + 1) < kmax) ++kd;
  return kd;
}

static float2 twiddle(long long m, long long n) {
  const double pi = 3.14159265358979323846;
  const double a = -2.0 * pi * (double)m / (double)n;
  return make_float2((float)std::cos(a), (float)std::sin(a));
}

// Appends the compact per-stage table of an m-point FFT (stages of radix radix_max until
// the remainder is smaller; Sched::ctoff layout): for stage s >= 1 of radix R with Ns points per sub-transform, entries
// r = 1..R-1, jm = 0..Ns-1 hold exp(-2 pi i r jm / (Ns R)). Same FP64 angles (scaled by
// powers of two) as the strided table, so both give the same FP32 values.
static void push_compact_table(std::vector<float2>& t, int m, int radix_max = 8) {
  const int E = m >= radix_max ? radix_max : m;
  std::vector<int> radix;
  int rem = m;
  while (E > 1 && rem >= E) {
    radix.push_back(E);
    rem /= E;
  }
  if (rem > 1) radix.push_back(rem);
  long long ns = 1;
  for (size_t st = 0; st < radix.size(); ++st) {
    const int R = radix[st];
    if (st >= 1)
      for (int r = 1; r < R; ++r)
        for (long long jm = 0; jm < ns; ++jm) t.push_back(twiddle(r * jm, ns * R));
    ns *= R;
  }
}

// FP64 -> FP32 twiddle table exp(-2 pi i m / n), m in [0, n), followed by the compact
// table of the n/2-point line FFT, that of the n-point FFT (the two-for-one line pass,
// at line2_ct_offset<n>()) and that of the n-point FFT in radix-16 stages (at
// line3_ct16_offset<n>()).
static std::vector<float2> twiddles(int n) {
  std::vector<float2> t(n);
  for (int m = 0; m < n; ++m) t[m] = twiddle(m, n);
  push_compact_table(t, n / 2);
  push_compact_table(t, n);
  push_compact_table(t, n, 16);  // radix-16 line pass (line3_ct16_offset<n>())
  return t;
}

// Parseval kinetic energy: per-block partial sums of w |u_hat|^2 over 3 components.
// The 3 components of a trajectory are one flat array of 3 cs modes read as float4
// (two modes) in a grid-stride loop, every lane busy; a component holds whole half-axis
// rows of h modes (cs is a multiple of h and even), so mode i has half-axis index
// i mod h and weight 1 on the planes 0 and h-1, else 2. Each pair's energy is formed in
// FP32 and accumulated in float-float (Ff), combined across warps and blocks in FP64.
__global__ void __launch_bounds__(256)
k_energy_partial(const float2* __restrict__ uh, long long cs, int h, int nblk, double* __restrict__ partial) {
  const int batch = blockIdx.y;
  const float4* ub = reinterpret_cast<const float4*>(uh + (long long)batch * 3 * cs);
  const unsigned pairs = (unsigned)(3 * cs / 2), uh_ = (unsigned)h;  // 3 cs < 2^32 for N <= 512
  Ff s{0.f, 0.f};
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < pairs; q += (unsigned)nblk * blockDim.x) {
    const float4 v = __ldg(ub + q);
    const unsigned k0 = (2u * q) % uh_, k1 = k0 + 1u == uh_ ? 0u : k0 + 1u;
    const float w0 = (k0 == 0u || k0 == uh_ - 1u) ? 1.f : 2.f;
    const float w1 = (k1 == 0u || k1 == uh_ - 1u) ? 1.f : 2.f;
    s = ff_add(s, fmaf(w0, fmaf(v.x, v.x, v.y * v.y), w1 * fmaf(v.z, v.z, v.w * v.w)));
  }
  block_sum_store_ff(s, partial, batch * nblk + blockIdx.x);
}

__global__ void __launch_bounds__(256)
k_sum_partials(const double* __restrict__ partial, int n, double scale, double* __restrict__ out) {
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

}  // namespace l3es

using namespace l3es;

#define L3ES_TRY_CUDA(expr, what)                          \
  do {                                                     \
    int _rc = cuda_check((expr), (what));                  \
    if (_rc != L3ES_OK) return _rc;                        \
  } while (0)

static int plan_alloc(l3es_plan* p, void** ptr, size_t bytes, const char* what) {
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(L3ES_ENOMEM, std::string("cudaMalloc(") + what + ", " + std::to_string(bytes) +
                                 " B): " + cudaGetErrorString(e));
  }
  p->allocs.push_back(*ptr);
  p->ws_bytes += (long long)bytes;
  return L3ES_OK;
}

static void plan_free(l3es_plan* p) {
  for (void* a : p->allocs) cudaFree(a);
  p->allocs.clear();
  for (void* a : p->adj.allocs) cudaFree(a);
  p->adj = AdjWork();
}

extern "C" {

const char* l3es_last_error(void) { return g_err.c_str(); }

const char* l3es_version(void) { return "l3es_gb300 0.1 (sm_103a)"; }

int l3es_plan_create(const l3es_plan_desc* desc, l3es_plan** out) {
  if (!desc || !out) return fail(L3ES_EINVAL, "l3es_plan_create: null argument");
  *out = nullptr;
  const int n = desc->n, dim = desc->dim;
  if (dim != 2 && dim != 3) return fail(L3ES_EINVAL, "dim must be 2 or 3, got " + std::to_string(dim));
  DnsTable tab;
  if (!dns_table(n, &tab))
    return fail(L3ES_EINVAL, "N=" + std::to_string(n) + " not supported (8, 16, 32, 64, 128, 256, 512)");
  if (desc->batch < 1) return fail(L3ES_EINVAL, "batch must be >= 1");
  if (!(desc->dt > 0.0) || !(desc->nu >= 0.0)) return fail(L3ES_EINVAL, "need dt > 0 and nu >= 0");
  if (desc->forcing < L3ES_FORCING_NONE || desc->forcing > L3ES_FORCING_CONST_POWER)
    return fail(L3ES_EINVAL, "unknown forcing mode " + std::to_string(desc->forcing));
  if (desc->forcing != L3ES_FORCING_NONE && (desc->kf < 1 || desc->kf > n / 4))
    return fail(L3ES_EINVAL, "forcing needs 1 <= kf <= N/4");
  if (desc->kolm_k != 0 && (dim != 2 || desc->kolm_k < 0 || desc->kolm_k >= n / 2))
    return fail(L3ES_EINVAL, "Kolmogorov forcing is 2D with 0 < kolm_k < N/2");
  if (desc->scheme != L3ES_SCHEME_EXPLICIT && desc->scheme != L3ES_SCHEME_INTEGRATING_FACTOR)
    return fail(L3ES_EINVAL, "unknown time-stepping scheme " + std::to_string(desc->scheme));

  auto* p = new l3es_plan();
  p->desc = *desc;
  cudaGetDevice(&p->device);
  Ctx& c = p->ctx;
  c.dim = dim;
  c.n = n;
  c.h = n / 2 + 1;
  c.batch = desc->batch;
  c.kd = dealias_kd(n);
  c.kt = ((c.kd + 1 + TW - 1) / TW) * TW;
  if (n == 256) c.sched.line_pair = 3;  // the staged radix-16 line pass (measured best at 256)
  // the band-fused step in 3D; a 2D band pass has one CTA per 8 half-axis columns (11 at
  // 256^2), too few to hide its epilogue's loads (2D Kolmogorov 256^2 with particles:
  // 104.5 us per step fused, 101.4 us with the elementwise update)
  c.step_form = dim == 3 ? 2 : 1;
  c.nmid = dim == 3 ? n : 1;
  c.cs = c.nmid * n * c.h;
  c.fs = c.cs;
  c.ds = c.nmid * n * c.kt;
  c.ps = dim == 3 ? (long long)n * n * n : (long long)n * n;
  c.npartial = (int)((3 * c.cs / 2 + 255) / 256);
  c.pcs = (long long)(2 * c.kd + 1) * (dim == 3 ? (2 * c.kd + 1) : 1) * c.kt;
  // room for the RK energy partials, the diagnostics' 608 blocks x 4 values and a
  // 2 x N spectrum accumulator
  c.partial_len = std::max<long long>(std::max<long long>(c.npartial, 4LL * 608), 2LL * n);
  c.kf = desc->kf;
  c.eps_inj = desc->eps_inj;
  p->tab = tab;

  const size_t B = (size_t)c.batch;
  int rc = L3ES_OK;
  const std::vector<float2> tw = twiddles(n);
  rc = rc ? rc : plan_alloc(p, (void**)&c.tw, sizeof(float2) * tw.size(), "twiddles");
  rc = rc ? rc : plan_alloc(p, (void**)&c.W, sizeof(float2) * B * 6 * c.fs, "W");
  if (dim == 3) rc = rc ? rc : plan_alloc(p, (void**)&c.Wx, sizeof(float2) * B * 2 * c.fs, "Wx");
  rc = rc ? rc : plan_alloc(p, (void**)&c.DU, sizeof(float2) * B * 3 * c.ds, "DU");
  rc = rc ? rc : plan_alloc(p, (void**)&c.Tb, sizeof(float2) * B * 3 * c.cs, "stage");
  rc = rc ? rc : plan_alloc(p, (void**)&c.C, sizeof(float2) * B * 3 * c.cs, "accumulator");
  rc = rc ? rc : plan_alloc(p, (void**)&c.P, sizeof(float2) * B * 3 * c.pcs, "band");
  rc = rc ? rc : plan_alloc(p, (void**)&c.partial, sizeof(double) * B * c.partial_len, "partials");
  rc = rc ? rc : plan_alloc(p, (void**)&c.band, sizeof(double) * B, "band");
  rc = rc ? rc : plan_alloc(p, (void**)&c.e0, sizeof(double) * B, "e0");
  rc = rc ? rc : plan_alloc(p, (void**)&c.einj, sizeof(double) * B, "einj");
  rc = rc ? rc : plan_alloc(p, (void**)&c.nu_b, sizeof(float) * B, "viscosities");
  rc = rc ? rc : plan_alloc(p, (void**)&c.err, sizeof(int), "error word");
  if (rc != L3ES_OK) {
    plan_free(p);
    delete p;
    return rc;
  }
  std::vector<double> e0(B, desc->e_kin_init);
  std::vector<float> nus(B, (float)desc->nu);
  cudaError_t e = cudaMemcpy(c.tw, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(c.nu_b, nus.data(), sizeof(float) * B, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(c.e0, e0.data(), sizeof(double) * B, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(c.band, 0, sizeof(double) * B);
  if (e == cudaSuccess) e = cudaMemset(c.err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    rc = cuda_check(e, "l3es_plan_create");
    plan_free(p);
    delete p;
    return rc;
  }
  *out = p;
  return L3ES_OK;
}

int l3es_plan_check(l3es_plan* plan) {
  if (!plan) return fail(L3ES_EINVAL, "l3es_plan_check: null plan");
  int h = 0;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&h, plan->ctx.err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_check(e, "l3es_plan_check");
  if (h) {
    cudaMemset(plan->ctx.err, 0, sizeof(int));
    if (h & kErrTimeout)
      return fail(L3ES_ETIMEOUT, std::string("l3es_plan_check: a kernel's wait on its bulk copies timed out") +
                                     ((h & kErrNonFinite) ? " (and the state held non-finite values)" : ""));
    return fail(L3ES_ENONFINITE, "l3es_plan_check: a step produced non-finite values (the flow blew up; "
                                 "a smaller dt or a larger viscosity is needed)");
  }
  return L3ES_OK;
}

namespace l3es {
// One CTA waits on an mbarrier that expects 16 bytes no copy will deliver (nothing is
// issued, so nothing is in flight when it gives up); the bounded wait must run out and
// set *err.
__global__ void k_wait_selftest(int* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar, 16);
  __syncthreads();
  const bool got = mbar_wait(&bar, 0);
  if (__syncthreads_or(!got) && threadIdx.x == 0) *err = kErrTimeout;
}
}  // namespace l3es

int l3es_selftest_bounded_wait(void* stream) {
  int* d = nullptr;
  int h = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMalloc(&d, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(int), s);
  if (e == cudaSuccess) {
    k_wait_selftest<<<1, 32, 0, s>>>(d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (d) cudaFree(d);
  if (e != cudaSuccess) return cuda_check(e, "l3es_selftest_bounded_wait");
  return h ? fail(L3ES_ETIMEOUT, "l3es_selftest_bounded_wait: the wait ran out as expected") : L3ES_OK;
}

int l3es_plan_destroy(l3es_plan* plan) {
  if (!plan) return L3ES_OK;
  plan_free(plan);
  delete plan;
  return L3ES_OK;
}

int l3es_plan_set_e0(l3es_plan* plan, const double* e0_host, int32_t count) {
  if (!plan || !e0_host) return fail(L3ES_EINVAL, "l3es_plan_set_e0: null argument");
  if (count != plan->ctx.batch) return fail(L3ES_EINVAL, "l3es_plan_set_e0: count != batch");
  return cuda_check(cudaMemcpy(plan->ctx.e0, e0_host, sizeof(double) * count, cudaMemcpyHostToDevice),
                    "l3es_plan_set_e0");
}

int l3es_plan_set_nu(l3es_plan* plan, const double* nu_host, int32_t count) {
  if (!plan || !nu_host) return fail(L3ES_EINVAL, "l3es_plan_set_nu: null argument");
  if (count != plan->ctx.batch) return fail(L3ES_EINVAL, "l3es_plan_set_nu: count != batch");
  std::vector<float> v(count);
  for (int i = 0; i < count; ++i) {
    if (!(nu_host[i] >= 0.0)) return fail(L3ES_EINVAL, "l3es_plan_set_nu: viscosity must be >= 0");
    v[i] = (float)nu_host[i];
  }
  return cuda_check(cudaMemcpy(plan->ctx.nu_b, v.data(), sizeof(float) * count, cudaMemcpyHostToDevice),
                    "l3es_plan_set_nu");
}

int64_t l3es_plan_workspace_bytes(const l3es_plan* plan) { return plan ? plan->ws_bytes : 0; }

int l3es_plan_timing(l3es_plan* plan, int32_t enable) {
  if (!plan) return fail(L3ES_EINVAL, "l3es_plan_timing: null plan");
  plan->timer.reset();
  plan->ctx.timer = enable ? &plan->timer : nullptr;
  return cuda_check(cudaGetLastError(), "l3es_plan_timing");
}

int l3es_plan_kernel_stats(l3es_plan* plan, int32_t kind, double* total_ms, int64_t* launches,
                           double* algo_bytes) {
  if (!plan || !total_ms || !launches || !algo_bytes) return fail(L3ES_EINVAL, "l3es_plan_kernel_stats: null");
  if (kind < 0 || kind >= KK_COUNT) return fail(L3ES_EINVAL, "l3es_plan_kernel_stats: bad kind");
  plan->timer.collect();
  *total_ms = plan->timer.ms[kind];
  *launches = plan->timer.launches[kind];
  *algo_bytes = plan->timer.bytes[kind];
  return cuda_check(cudaGetLastError(), "l3es_plan_kernel_stats");
}

int32_t l3es_kernel_kind_count(void) { return KK_COUNT; }

const char* l3es_kernel_kind_name(int32_t kind) { return kernel_kind_name(kind); }

int l3es_plan_get_schedule(const l3es_plan* plan, int32_t* sched4) {
  if (!plan || !sched4) return fail(L3ES_EINVAL, "l3es_plan_get_schedule: null argument");
  const Schedule& s = plan->ctx.sched;
  sched4[0] = s.x_bulk;
  sched4[1] = s.y_var;
  sched4[2] = s.line_pair;
  sched4[3] = s.band_bulk < 0 ? (plan->ctx.n >= 256 ? 1 : 0) : s.band_bulk;
  return L3ES_OK;
}

int l3es_plan_set_schedule(l3es_plan* plan, const int32_t* sched4) {
  if (!plan || !sched4) return fail(L3ES_EINVAL, "l3es_plan_set_schedule: null argument");
  for (int i = 0; i < 4; ++i)
    if (sched4[i] != 0 && sched4[i] != 1 && !(i == 2 && (sched4[i] == 2 || sched4[i] == 3)))
      return fail(L3ES_EINVAL, "l3es_plan_set_schedule: values are 0 or 1 (line pass: 0 to 3)");
  if (sched4[2] >= 2 && plan->ctx.n != 256)
    return fail(L3ES_EINVAL, "l3es_plan_set_schedule: the radix-16 line passes (2, 3) exist for N = 256 only");
  Schedule& s = plan->ctx.sched;
  s.x_bulk = sched4[0];
  s.y_var = sched4[1];
  s.line_pair = sched4[2];
  s.band_bulk = sched4[3];
  return L3ES_OK;
}

int l3es_plan_get_step_form(const l3es_plan* plan, int32_t* form) {
  if (!plan || !form) return fail(L3ES_EINVAL, "l3es_plan_get_step_form: null argument");
  *form = plan->ctx.step_form;
  return L3ES_OK;
}

int l3es_plan_set_step_form(l3es_plan* plan, int32_t form) {
  if (!plan) return fail(L3ES_EINVAL, "l3es_plan_set_step_form: null plan");
  if (form < 0 || form > 2) return fail(L3ES_EINVAL, "l3es_plan_set_step_form: form is 0, 1 or 2");
  plan->ctx.step_form = form;
  return L3ES_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// Autotuner: picks the plan's kernel variants (bulk-copy or one-tile x passes, radix-16 or
// radix-8 y passes, two-for-one or packed line pass, bulk-copy or one-tile band pass) by
// timing the right-hand side on the plan's own scratch (coordinate descent, each knob
// with the others at their current choice), and caches the result in a text file, one
// line per (GPU, dim, N, batch): "<key> x_bulk y_var line_pair band_bulk".
// ---------------------------------------------------------------------------------
static std::string tune_key(const l3es_plan* p) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, p->device);
  std::string name = prop.name;
  for (char& ch : name)
    if (ch == ' ') ch = '_';
  return name + "|sm" + std::to_string(prop.major) + std::to_string(prop.minor) + "|d" + std::to_string(p->ctx.dim) +
         "|n" + std::to_string(p->ctx.n) + "|b" + std::to_string(p->ctx.batch) + "|f" +
         std::to_string(p->ctx.step_form);
}

static bool tune_cache_read(const char* path, const std::string& key, int32_t* v) {
  if (!path) return false;
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (std::fgets(line, sizeof line, f)) {
    char k[400];
    int a, b, c, d;
    if (std::sscanf(line, "%399s %d %d %d %d", k, &a, &b, &c, &d) == 5 && key == k) {
      v[0] = a;
      v[1] = b;
      v[2] = c;
      v[3] = d;
      found = true;  // the last entry of a key wins
    }
  }
  std::fclose(f);
  return found;
}

static void tune_cache_write(const char* path, const std::string& key, const int32_t* v) {
  if (!path) return;
  std::vector<std::string> keep;
  if (FILE* f = std::fopen(path, "r")) {
    char line[512];
    while (std::fgets(line, sizeof line, f)) {
      char k[400];
      if (std::sscanf(line, "%399s", k) == 1 && key == k) continue;
      keep.emplace_back(line);
    }
    std::fclose(f);
  }
  FILE* f = std::fopen(path, "w");
  if (!f) return;  // an unwritable cache only costs a re-tune
  for (const auto& l : keep) std::fputs(l.c_str(), f);
  std::fprintf(f, "%s %d %d %d %d\n", key.c_str(), v[0], v[1], v[2], v[3]);
  std::fclose(f);
}

// The four stages of one RK4 step of the state S in the plan's step form
// (spectral_solver.py:65-80; the forcing rescale of ekin_tot follows in run_steps).
static void rk4_stages(l3es_plan* plan, float2* S, cudaStream_t s) {
  const Ctx& c = plan->ctx;
  const l3es_plan_desc& d = plan->desc;
  static const double a_rk4[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
  static const double b_rk4[3] = {0.5, 0.5, 1.0};
  // closed-form stages outside the stage region (k_rk_update): explicit scheme, forcing
  // terms inside the region (band forcing |k| <= kf, Kolmogorov mode kh = kolm_k)
  const int kf_band = d.forcing == L3ES_FORCING_CONST_POWER ? d.kf : 0;
  const int lin_ok = c.step_form >= 1 && d.scheme != L3ES_SCHEME_INTEGRATING_FACTOR && kf_band <= c.kd &&
                     kf_band < c.kt && (d.kolm_k <= 0 || d.kolm_k < c.kt);
  // the band-fused form: the band pass combines the stages on the band in place in S,
  // the x inverse applies the closed form to every other mode; its accumulator lives in
  // C in the band's compact layout (kt <= N/2 + 1, i.e. N >= 16, keeps that inside C)
  const int band_rk = lin_ok && c.step_form >= 2 && c.kt <= c.h;
  for (int rk = 0; rk < 4; ++rk) {
    EpiParams prm;
    prm.a_dt = (float)(a_rk4[rk] * d.dt);
    prm.b_dt = rk < 3 ? (float)(b_rk4[rk] * d.dt) : 0.f;
    prm.nu = (float)d.nu;
    prm.drag = (float)d.drag;
    prm.kolm_amp = (float)d.kolm_amp;
    prm.kolm_k = d.kolm_k;
    prm.band_kf2 = d.forcing == L3ES_FORCING_CONST_POWER ? d.kf * d.kf : 0;
    prm.rk = rk;
    prm.if_h = d.scheme == L3ES_SCHEME_INTEGRATING_FACTOR ? (float)d.dt : 0.f;
    prm.dt = (float)d.dt;
    prm.lin = lin_ok;
    prm.band_rk = band_rk;
    if (band_rk)
      plan->tab.stage(c, S, S, S, rk, prm, s);
    else
      plan->tab.stage(c, rk == 0 ? S : c.Tb, S, c.Tb, rk, prm, s);
  }
}

// mean milliseconds of one RK4 step in the plan's step form with its current schedule,
// on the zeroed stage scratch T as the state (timing only: the explicit forms then alias
// their stage field with the state; zeros stay finite through every term)
static float time_step(l3es_plan* p, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1) {
  const Ctx& c = p->ctx;
  rk4_stages(p, c.Tb, s);
  const int reps = c.cs * c.batch > (1 << 20) ? 2 : 5;
  cudaEventRecord(e0, s);
  for (int i = 0; i < reps; ++i) rk4_stages(p, c.Tb, s);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  return ms / reps;
}

extern "C" int l3es_plan_autotune(l3es_plan* plan, const char* cache_path, void* stream) {
  if (!plan) return fail(L3ES_EINVAL, "l3es_plan_autotune: null plan");
  cudaStream_t s = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  int rc = cuda_check(cudaStreamIsCapturing(s, &cap), "l3es_plan_autotune");
  if (rc != L3ES_OK) return rc;
  if (cap != cudaStreamCaptureStatusNone) return fail(L3ES_ESTATE, "l3es_plan_autotune: not while recording a graph");
  const std::string key = tune_key(plan);
  int32_t v[4];
  if (tune_cache_read(cache_path, key, v)) return l3es_plan_set_schedule(plan, v);
  Ctx& c = plan->ctx;
  KTimer* timer = c.timer;
  c.timer = nullptr;  // untimed by the per-kernel timer
  // the timed steps run on scratch; whatever they flag in the error word (a constant-power
  // coefficient of a zero field can overflow) is not the caller's: keep the word as it was
  int err_word = 0;
  rc = cuda_check(cudaMemcpyAsync(&err_word, c.err, sizeof(int), cudaMemcpyDeviceToHost, s),
                  "l3es_plan_autotune error word");
  if (rc == L3ES_OK) rc = cuda_check(cudaStreamSynchronize(s), "l3es_plan_autotune sync");
  if (rc == L3ES_OK)
    rc = cuda_check(cudaMemsetAsync(c.Tb, 0, sizeof(float2) * 3 * c.cs * c.batch, s), "l3es_plan_autotune memset");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (rc == L3ES_OK) rc = cuda_check(cudaEventCreate(&e0), "l3es_plan_autotune event");
  if (rc == L3ES_OK) rc = cuda_check(cudaEventCreate(&e1), "l3es_plan_autotune event");
  if (rc == L3ES_OK) {
    l3es_plan_get_schedule(plan, v);
    l3es_plan_set_schedule(plan, v);
    // knobs that change anything for this plan
    const int n = c.n;
    const bool knob[4] = {(c.dim == 3 && n >= 64) || c.dim == 2, c.dim == 3 && n >= 128, n >= 64 && n <= 256,
                          c.dim == 3 && n >= 64};
    const int nval[4] = {2, 2, n == 256 ? 4 : 2, 2};  // the line pass has two radix-16 forms at 256
    float best = time_step(plan, s, e0, e1);
    for (int k = 0; k < 4; ++k) {
      if (!knob[k]) continue;
      const int keep = v[k];
      int pick = keep;
      for (int val = 0; val < nval[k]; ++val) {
        if (val == keep) continue;
        v[k] = val;
        l3es_plan_set_schedule(plan, v);
        const float t = time_step(plan, s, e0, e1);
        if (t < best) {
          best = t;
          pick = val;
        }
      }
      v[k] = pick;
      l3es_plan_set_schedule(plan, v);
    }
    rc = cuda_check(cudaGetLastError(), "l3es_plan_autotune launch");
    if (rc == L3ES_OK) tune_cache_write(cache_path, key, v);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  c.timer = timer;
  const int rc2 = cuda_check(cudaMemcpyAsync(c.err, &err_word, sizeof(int), cudaMemcpyHostToDevice, s),
                             "l3es_plan_autotune error word");
  const int rc3 = cuda_check(cudaStreamSynchronize(s), "l3es_plan_autotune sync");
  return rc != L3ES_OK ? rc : rc2 != L3ES_OK ? rc2 : rc3;
}

// per-block partial sums of w |u_hat|^2 into c.partial ([batch][nblk]); returns nblk
int l3es::energy_partials(const Ctx& c, const float2* uh, cudaStream_t s) {
  // 8 blocks of 256 threads per SM of a 152-SM GB300, fewer when the field is small
  const int nblk = (int)std::min<long long>(std::min<long long>(c.npartial, 8 * 152), (3 * c.cs / 2 + 255) / 256);
  L3ES_LAUNCH(c, KK_REDUCE, 8.0 * 3.0 * c.cs * c.batch, s,
              k_energy_partial<<<dim3(nblk, c.batch), 256, 0, s>>>(uh, c.cs, c.h, nblk, c.partial));
  return nblk;
}

// nsteps RK4 steps in place; ke_dev (optional): kinetic energy of the final state per
// trajectory (for ekin_tot forcing: of the rescaled state)
static int run_steps(l3es_plan* plan, void* u_hat, float* u_out, int32_t nsteps, double* e_inj_dev, double* ke_dev,
                     void* stream) {
  if (!plan || !u_hat) return fail(L3ES_EINVAL, "l3es_step: null plan or u_hat");
  if (misaligned16(u_hat)) return fail(L3ES_EINVAL, "l3es_step: u_hat must be 16-byte aligned");
  if (nsteps < 0) return fail(L3ES_EINVAL, "l3es_step: nsteps < 0");
  cudaStream_t s = (cudaStream_t)stream;
  const Ctx& c = plan->ctx;
  const l3es_plan_desc& d = plan->desc;
  float2* S = (float2*)u_hat;
  const double inv_n2d = 1.0 / std::pow((double)c.n, 2 * c.dim);
  const double eps64 = 2.220446049250313e-16;  // jnp.finfo(float).eps, spectral_solver.py:23
  for (int st = 0; st < nsteps; ++st) {
    rk4_stages(plan, S, s);
    double* einj = e_inj_dev ? e_inj_dev + (long long)st * c.batch : c.einj;
    double* ke_final = (ke_dev && st == nsteps - 1) ? ke_dev : nullptr;
    // energy partials of the new state by the row-wise float-float pass (a separate
    // pass is cheaper than reducing inside the elementwise RK update)
    int nke = 0;
    if (d.forcing == L3ES_FORCING_EKIN_TOT || ke_final) nke = energy_partials(c, S, s);
    if (d.forcing == L3ES_FORCING_EKIN_TOT) {
      if (c.dim == 3)
        L3ES_LAUNCH(c, KK_FORCE, 0.0, s,
                    k_force_ekin<3><<<c.batch, 256, 0, s>>>(S, c.cs, c.partial, nke, c.e0, d.dt, c.n, d.kf,
                                                            inv_n2d, eps64, einj, ke_final));
      else
        L3ES_LAUNCH(c, KK_FORCE, 0.0, s,
                    k_force_ekin<2><<<c.batch, 256, 0, s>>>(S, c.cs, c.partial, nke, c.e0, d.dt, c.n, d.kf,
                                                            inv_n2d, eps64, einj, ke_final));
    } else {
      if (e_inj_dev) L3ES_TRY_CUDA(cudaMemsetAsync(einj, 0, sizeof(double) * c.batch, s), "l3es_step memset");
      if (ke_final)
        L3ES_LAUNCH(c, KK_REDUCE, 0.0, s, k_sum_partials<<<c.batch, 256, 0, s>>>(c.partial, nke, 0.5 * inv_n2d, ke_final));
    }
  }
  if (nsteps == 0 && ke_dev) {
    const int rc = l3es_kinetic_energy(plan, u_hat, ke_dev, stream);
    if (rc != L3ES_OK) return rc;
  }
  if (u_out) plan->tab.irfftn(c, S, u_out, s);
  return cuda_check(cudaGetLastError(), "l3es_step launch");
}

extern "C" {

int l3es_step(l3es_plan* plan, void* u_hat, float* u_out, int32_t nsteps, double* e_inj_dev, void* stream) {
  return run_steps(plan, u_hat, u_out, nsteps, e_inj_dev, nullptr, stream);
}

int l3es_step_energy(l3es_plan* plan, void* u_hat, float* u_out, int32_t nsteps, double* e_inj_dev, double* ke_dev,
                     void* stream) {
  if (!ke_dev) return fail(L3ES_EINVAL, "l3es_step_energy: null ke_dev");
  return run_steps(plan, u_hat, u_out, nsteps, e_inj_dev, ke_dev, stream);
}

int l3es_rhs(l3es_plan* plan, const void* u_hat, void* du, void* stream) {
  if (!plan || !u_hat || !du) return fail(L3ES_EINVAL, "l3es_rhs: null argument");
  if (u_hat == du) return fail(L3ES_EINVAL, "l3es_rhs: du must not alias u_hat");
  if (misaligned16(u_hat) || misaligned16(du)) return fail(L3ES_EINVAL, "l3es_rhs: u_hat and du must be 16-byte aligned");
  const l3es_plan_desc& d = plan->desc;
  EpiParams prm;
  prm.a_dt = 0.f;
  prm.b_dt = 0.f;
  prm.nu = (float)d.nu;
  prm.drag = (float)d.drag;
  prm.kolm_amp = (float)d.kolm_amp;
  prm.kolm_k = d.kolm_k;
  prm.band_kf2 = d.forcing == L3ES_FORCING_CONST_POWER ? d.kf * d.kf : 0;
  prm.rk = -1;
  prm.if_h = 0.f;  // rhs_fn itself: the full right-hand side, viscous term included
  plan->tab.stage(plan->ctx, (const float2*)u_hat, nullptr, (float2*)du, -1, prm, (cudaStream_t)stream);
  return cuda_check(cudaGetLastError(), "l3es_rhs launch");
}

int l3es_rfftn(l3es_plan* plan, const float* u, void* u_hat, void* stream) {
  if (!plan || !u || !u_hat) return fail(L3ES_EINVAL, "l3es_rfftn: null argument");
  plan->tab.rfftn(plan->ctx, u, (float2*)u_hat, (cudaStream_t)stream);
  return cuda_check(cudaGetLastError(), "l3es_rfftn launch");
}

int l3es_irfftn(l3es_plan* plan, const void* u_hat, float* u, void* stream) {
  if (!plan || !u || !u_hat) return fail(L3ES_EINVAL, "l3es_irfftn: null argument");
  plan->tab.irfftn(plan->ctx, (const float2*)u_hat, u, (cudaStream_t)stream);
  return cuda_check(cudaGetLastError(), "l3es_irfftn launch");
}

int l3es_kinetic_energy(l3es_plan* plan, const void* u_hat, double* out_dev, void* stream) {
  if (!plan || !u_hat || !out_dev) return fail(L3ES_EINVAL, "l3es_kinetic_energy: null argument");
  if (misaligned16(u_hat)) return fail(L3ES_EINVAL, "l3es_kinetic_energy: u_hat must be 16-byte aligned");
  const Ctx& c = plan->ctx;
  cudaStream_t s = (cudaStream_t)stream;
  const int nblk = energy_partials(c, (const float2*)u_hat, s);
  const double scale = 0.5 / std::pow((double)c.n, 2 * c.dim);
  L3ES_LAUNCH(c, KK_REDUCE, 0.0, s, k_sum_partials<<<c.batch, 256, 0, s>>>(c.partial, nblk, scale, out_dev));
  return cuda_check(cudaGetLastError(), "l3es_kinetic_energy launch");
}

}  // extern "C"
