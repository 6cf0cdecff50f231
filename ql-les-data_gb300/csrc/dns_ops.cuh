// Host launch wrappers for the DNS kernels of one grid size N. Each dns_n*.cu
// translation unit instantiates make_dns_table<N>() for its sizes, so the sizes
// compile in parallel.
#pragma once

#include "l3es_internal.h"

namespace l3es {

template <int N>
struct DnsOps {
  static constexpr int H = N / 2 + 1;
  static constexpr int TX = TW * Fft<N>::T;  // threads of the strided passes
  using L = LineCfg<N>;

  static size_t cross_smem() { return (size_t)(6 * L::LPC * H + L::LPC * xpad_len(L::M)) * sizeof(float2); }
  static size_t c2r_smem() { return (size_t)(L::LPC * H + L::LPC * xpad_len(L::M)) * sizeof(float2); }
  static size_t r2c_smem() { return (size_t)(L::LPC * xpad_len(L::M)) * sizeof(float2); }

  static void init_attrs() {
    cudaFuncSetAttribute(line_cross<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cross_smem());
    cudaFuncSetAttribute(line_c2r<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c2r_smem());
    cudaFuncSetAttribute(line_r2c<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)r2c_smem());
  }

  // us: field the RHS is evaluated on; S: state; out: RK stage field (or du for rk=-1)
  template <int DIM>
  static void stage_dim(const Ctx& c, const float2* us, float2* S, float2* out, int rk, const EpiParams& prm,
                        cudaStream_t s) {
    const long long mc = c.nmid * H;
    const long long lines = c.nmid * N;
    const float scale = (float)(1.0 / (DIM == 3 ? (double)N * N * N : (double)N * N));
    kx_inv<N, DIM, true><<<dim3((unsigned)((mc + TW - 1) / TW), c.batch), TX, 0, s>>>(us, c.cs, c.W, c.fs, c.tw);
    if (DIM == 3)
      ky_pass<N, kInv><<<dim3((H + TW - 1) / TW, N, 6 * c.batch), TX, 0, s>>>(c.W, c.fs, H, H, N / 2, c.tw);
    line_cross<N><<<dim3((unsigned)(lines / L::LPC), c.batch), L::THREADS, cross_smem(), s>>>(
        c.W, c.fs, c.DU, c.ds, c.kt, c.kd, scale, c.tw, (int)lines);
    if (DIM == 3)
      ky_pass<N, kFwd><<<dim3(c.kt / TW, N, 3 * c.batch), TX, 0, s>>>(c.DU, c.ds, c.kt, c.kt, c.kd, c.tw);
    if (prm.band_kf2 > 0) {
      const double inv_n2d = 1.0 / (DIM == 3 ? std::pow((double)N, 6) : std::pow((double)N, 4));
      k_band_scale<DIM><<<c.batch, 256, 0, s>>>(us, c.cs, N, c.kf, inv_n2d, c.eps_inj, 1e-30, c.band);
    }
    kx_fwd_epi<N, DIM><<<dim3((H + TW - 1) / TW, (unsigned)c.nmid, c.batch), TX, 0, s>>>(
        c.DU, c.ds, c.kt, c.kd, us, S, c.C, out, S, c.cs, prm, c.band, c.partial, c.tw);
  }

  static void stage(const Ctx& c, const float2* us, float2* S, float2* out, int rk, const EpiParams& prm,
                    cudaStream_t s) {
    if (c.dim == 3)
      stage_dim<3>(c, us, S, out, rk, prm, s);
    else
      stage_dim<2>(c, us, S, out, rk, prm, s);
  }

  template <int DIM>
  static void irfftn_dim(const Ctx& c, const float2* uh, float* u, cudaStream_t s) {
    const long long mc = c.nmid * H;
    const long long lines = c.nmid * N;
    const float scale = (float)(1.0 / (DIM == 3 ? (double)N * N * N : (double)N * N));
    kx_inv<N, DIM, false><<<dim3((unsigned)((mc + TW - 1) / TW), c.batch), TX, 0, s>>>(uh, c.cs, c.W, c.fs, c.tw);
    if (DIM == 3)
      ky_pass<N, kInv><<<dim3((H + TW - 1) / TW, N, 3 * c.batch), TX, 0, s>>>(c.W, c.fs, H, H, N / 2, c.tw);
    line_c2r<N><<<dim3((unsigned)(lines / L::LPC), c.batch), L::THREADS, c2r_smem(), s>>>(c.W, c.fs, u, c.ps,
                                                                                          scale, c.tw);
  }

  static void irfftn(const Ctx& c, const float2* uh, float* u, cudaStream_t s) {
    if (c.dim == 3)
      irfftn_dim<3>(c, uh, u, s);
    else
      irfftn_dim<2>(c, uh, u, s);
  }

  template <int DIM>
  static void rfftn_dim(const Ctx& c, const float* u, float2* uh, cudaStream_t s) {
    const long long mc = c.nmid * H;
    const long long lines = c.nmid * N;
    line_r2c<N><<<dim3((unsigned)(lines / L::LPC), c.batch), L::THREADS, r2c_smem(), s>>>(u, c.ps, c.W, c.fs, c.tw);
    if (DIM == 3)
      ky_pass<N, kFwd><<<dim3((H + TW - 1) / TW, N, 3 * c.batch), TX, 0, s>>>(c.W, c.fs, H, H, N / 2, c.tw);
    kx_fwd_plain<N, DIM><<<dim3((unsigned)((mc + TW - 1) / TW), c.batch), TX, 0, s>>>(c.W, c.fs, uh, c.cs, c.tw);
  }

  static void rfftn(const Ctx& c, const float* u, float2* uh, cudaStream_t s) {
    if (c.dim == 3)
      rfftn_dim<3>(c, u, uh, s);
    else
      rfftn_dim<2>(c, u, uh, s);
  }
};

template <int N>
DnsTable make_dns_table() {
  DnsOps<N>::init_attrs();
  DnsTable t;
  t.stage = &DnsOps<N>::stage;
  t.irfftn = &DnsOps<N>::irfftn;
  t.rfftn = &DnsOps<N>::rfftn;
  return t;
}

}  // namespace l3es
