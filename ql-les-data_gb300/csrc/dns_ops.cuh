// Host launch wrappers for the DNS kernels of one grid size N. Each dns_n*.cu
// translation unit instantiates make_dns_table<N>() for its sizes, so the sizes
// compile in parallel.
#pragma once

#include "l3es_internal.h"

namespace l3es {

template <int N>
struct DnsOps {
  static constexpr int H = N / 2 + 1;
  static constexpr int TX = TW * Fft<N>::T;  // threads of the strided x passes
  // 2D x passes in narrow tiles (schedule entry [0] in 2D): XN columns per CTA, so a
  // 256^2 field's 129 columns spread over 65 CTAs instead of 17
  static constexpr int XN = 2;
  static constexpr int TXN = XN * Fft<N>::T;
  using L = LineCfg<N>;
  using KY = KyCfg<N>;
  static constexpr unsigned ky_tiles(int ncols) { return (unsigned)((ncols + KY::TWY - 1) / KY::TWY); }

  static unsigned line_blocks(long long lines) { return (unsigned)((lines + L::LPC - 1) / L::LPC); }

  // persistent CTAs of the bulk-copy x inverse pass (0: use kx_inv)
  static inline int tma_ctas = 0;

  static inline int tma_band_ctas = 0;
  static inline int tma_plain_ctas = 0;  // x inverse without curl (irfftn)
  static inline int tma_lin_ctas = 0;    // band-fused RK step: x inverse and band pass
  static inline int tma_band_fused_ctas = 0;

  // resident CTAs (all SMs) of a persistent kernel with K::SMEM dynamic shared memory
  template <typename F>
  static int persistent_ctas(F kernel) {
    int nb = 0, dev = 0, sms = 0;
    const int smem = KxTma<N>::SMEM;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, TX, smem) == cudaSuccess &&
        cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
      return nb * sms;
    cudaGetLastError();
    return 0;
  }

  static inline bool lc3_staged_ok = false;  // dynamic shared memory of the staged line pass granted

  static void init_attrs() {
    if constexpr (N == 256) {
      lc3_staged_ok = cudaFuncSetAttribute(line_cross3<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           Line3Cfg<N>::SMEM_STAGED) == cudaSuccess;
      cudaGetLastError();
    }
    if constexpr (N >= 64) {
      tma_ctas = persistent_ctas(kx_inv_tma<N, true, true>);
      tma_band_ctas = persistent_ctas(kx_fwd_band_tma<N>);
      tma_plain_ctas = persistent_ctas(kx_inv_tma<N, false>);
      tma_lin_ctas = persistent_ctas(kx_inv_tma<N, true, true, true>);
      tma_band_fused_ctas = persistent_ctas(kx_fwd_band_tma<N, true>);
    }
  }

  // y pass of `nz` fields (columns [0, ncols) of rows of ncols values) in the plan's
  // y schedule (KyCfg variant)
  template <int DIR>
  static void y_pass(const Ctx& c, int kind, double bytes, float2* w, long long fs, int ncols, int kd_store, int nz,
                     cudaStream_t s) {
    const dim3 g(ky_tiles(ncols), N, nz);
    if (c.sched.y_var == 1)
      L3ES_LAUNCH(c, kind, bytes, s,
                  ky_pass<N, DIR, 1><<<g, KyCfg<N, 1>::THREADS, 0, s>>>(w, fs, ncols, ncols, kd_store, c.tw));
    else
      L3ES_LAUNCH(c, kind, bytes, s, ky_pass<N, DIR, 0><<<g, KY::THREADS, 0, s>>>(w, fs, ncols, ncols, kd_store, c.tw));
  }

  // the RHS's y inverse (six one-FFT jobs per tile) in the plan's y schedule
  static void y_inv_rhs(const Ctx& c, double bytes, cudaStream_t s) {
    const dim3 g(6 * ky_tiles(H), N, c.batch);
    if (c.sched.y_var == 1)
      L3ES_LAUNCH(c, KK_Y_INV, bytes, s, ky_inv_rhs<N, 1><<<g, KyCfg<N, 1>::THREADS, 0, s>>>(c.W, c.Wx, c.fs, c.tw));
    else
      L3ES_LAUNCH(c, KK_Y_INV, bytes, s, ky_inv_rhs<N, 0><<<g, KY::THREADS, 0, s>>>(c.W, c.Wx, c.fs, c.tw));
  }

  // x inverse pass with curl prologue: us -> W (6 fields); xl: the x inverse of a
  // band-fused RK stage (us is then the state xl->S)
  template <int DIM>
  static void x_inverse(const Ctx& c, const float2* us, double bytes, cudaStream_t s, const XLin* xl = nullptr) {
    const long long mc = c.nmid * H;
    if constexpr (DIM == 3 && N >= 64) {
      CUtensorMap map;
      const unsigned long long dims[3] = {(unsigned long long)mc, N, 3ull * c.batch};
      const unsigned long long strides[2] = {8ull * mc, 8ull * c.cs};
      const unsigned box[3] = {TW, KxTma<N>::NY, 3};
      const int ctas = xl ? tma_lin_ctas : tma_ctas;
      if (c.sched.x_bulk && ctas > 0 && tma_encode(&map, us, 3, dims, strides, box)) {
        const int ntiles = (int)(mc / TW);
        const int gx = std::max(1, std::min(ntiles, ctas / c.batch));
        if (xl)
          L3ES_LAUNCH(c, KK_X_INV, bytes, s,
                      kx_inv_tma<N, true, true, true><<<dim3(gx, c.batch), TX, KxTma<N>::SMEM, s>>>(
                          map, c.W, c.fs, c.tw, ntiles, c.err, c.Wx, *xl));
        else
          L3ES_LAUNCH(c, KK_X_INV, bytes, s,
                      kx_inv_tma<N, true, true><<<dim3(gx, c.batch), TX, KxTma<N>::SMEM, s>>>(
                          map, c.W, c.fs, c.tw, ntiles, c.err, c.Wx, XLin{}));
        return;
      }
    }
    if constexpr (DIM == 2) {
      if (c.sched.x_bulk) {
        const dim3 gn((unsigned)((mc + XN - 1) / XN), c.batch);
        if (xl)
          L3ES_LAUNCH(c, KK_X_INV, bytes, s,
                      kx_inv<N, 2, true, false, true, XN><<<gn, TXN, 0, s>>>(us, c.cs, c.W, c.fs, c.tw, c.Wx, *xl,
                                                                            c.err));
        else
          L3ES_LAUNCH(c, KK_X_INV, bytes, s,
                      kx_inv<N, 2, true, false, false, XN><<<gn, TXN, 0, s>>>(us, c.cs, c.W, c.fs, c.tw, c.Wx,
                                                                             XLin{}, c.err));
        return;
      }
    }
    const dim3 g((unsigned)((mc + TW - 1) / TW), c.batch);
    if (xl)
      L3ES_LAUNCH(c, KK_X_INV, bytes, s,
                  kx_inv<N, DIM, true, DIM == 3, true><<<g, TX, 0, s>>>(us, c.cs, c.W, c.fs, c.tw, c.Wx, *xl, c.err));
    else
      L3ES_LAUNCH(c, KK_X_INV, bytes, s,
                  kx_inv<N, DIM, true, DIM == 3><<<g, TX, 0, s>>>(us, c.cs, c.W, c.fs, c.tw, c.Wx));
  }

  // us: field the RHS is evaluated on; S: state; out: RK stage field (or du for rk=-1)
  template <int DIM>
  static void stage_dim(const Ctx& c, const float2* us, float2* S, float2* out, int rk, const EpiParams& prm,
                        cudaStream_t s) {
    const long long mc = c.nmid * H;
    const long long lines = c.nmid * N;
    const float scale = (float)(1.0 / (DIM == 3 ? (double)N * N * N : (double)N * N));
    const double B = c.batch, A = 8.0 * 3.0 * c.cs * B;  // bytes of one 3-component spectrum
    const double Adu = 8.0 * 3.0 * c.ds * B;               // bytes of the truncated DU field
    const double rows = DIM == 3 ? (2.0 * c.kd + 1.0) / N : 1.0;  // kept y rows
    const double inv_n2d = 1.0 / (DIM == 3 ? std::pow((double)N, 6) : std::pow((double)N, 4));
    // band-fused RK step (XLin): us == S; fb = the band's share of the modes
    const bool fused = prm.band_rk && rk >= 0;
    const double fb = (double)c.pcs / (double)c.cs;
    XLin xl{};
    if (fused) {
      xl.S = S;
      xl.cs = c.cs;
      xl.nu_b = c.nu_b;
      xl.drag = prm.drag;
      xl.dt = prm.dt;
      xl.kd = c.kd;
      xl.kt = c.kt;
      xl.rk = rk;
      xl.band_kf = prm.band_kf2 > 0 ? c.kf : 0;
      xl.inv_n2d = inv_n2d;
      xl.eps_inj = c.eps_inj;
      xl.band_scale = c.band;
    }
    // 3D: the x pass stores u_x, curl_y, curl_z in W and u_y, u_z in the side buffer
    // Wx (curl_x is not stored); the y pass writes all six fields of W. The last
    // band-fused stage also writes the new state outside the band.
    x_inverse<DIM>(c, us, (DIM == 3 ? 8.0 : 9.0) / 3.0 * A + (fused && rk == 3 ? (1.0 - fb) * A : 0.0), s,
                   fused ? &xl : nullptr);
    if (DIM == 3) y_inv_rhs(c, 11.0 / 3.0 * A, s);
    bool line_done = false;
    if constexpr (N >= 64 && N <= 256) {  // two real lines per complex FFT, persistent
      if constexpr (N == 256) {
        if (c.sched.line_pair >= 2) {  // radix-16 lines, 16 lanes per line
          using L3 = Line3Cfg<N>;
          const float s2 = 0.5f * scale * scale;
          const long long tiles = (lines + L3::LPC - 1) / L3::LPC;
          if (c.sched.line_pair == 3 && lc3_staged_ok && lines % L3::LPC == 0)
            L3ES_LAUNCH(c, KK_LINE_CROSS, 2.0 * A + Adu, s,
                        line_cross3<N, true><<<dim3((unsigned)tiles, c.batch), L3::THREADS, L3::SMEM_STAGED, s>>>(
                            c.W, c.fs, c.DU, c.ds, c.kt, c.kd, s2, c.tw + line2_ct_offset<N>(),
                            c.tw + line3_ct16_offset<N>(), (int)lines, c.err));
          else
            L3ES_LAUNCH(c, KK_LINE_CROSS, 2.0 * A + Adu, s,
                        line_cross3<N, false><<<dim3((unsigned)tiles, c.batch), L3::THREADS, 0, s>>>(
                            c.W, c.fs, c.DU, c.ds, c.kt, c.kd, s2, c.tw + line2_ct_offset<N>(),
                            c.tw + line3_ct16_offset<N>(), (int)lines, c.err));
          line_done = true;
        }
      }
      if (!line_done && c.sched.line_pair) {
        using L2 = Line2Cfg<N>;
        const float s2 = 0.5f * scale * scale;
        const long long tiles = (lines + L2::LPC - 1) / L2::LPC;
        L3ES_LAUNCH(c, KK_LINE_CROSS, 2.0 * A + Adu, s,
                    line_cross2<N><<<dim3((unsigned)tiles, c.batch), L2::THREADS, 0, s>>>(
                        c.W, c.fs, c.DU, c.ds, c.kt, c.kd, s2, c.tw + line2_ct_offset<N>(), (int)lines));
        line_done = true;
      }
    }
    if (!line_done)
      L3ES_LAUNCH(c, KK_LINE_CROSS, 2.0 * A + Adu, s,
                  line_cross<N><<<dim3(line_blocks(lines), c.batch), L::THREADS, 0, s>>>(
                      c.W, c.fs, c.DU, c.ds, c.kt, c.kd, scale, c.tw, (int)lines));
    if (DIM == 3) y_pass<kFwd>(c, KK_Y_FWD, Adu * (1.0 + rows), c.DU, c.ds, c.kt, c.kd, 3 * c.batch, s);
    // band x-FFT + projection into P, then the elementwise RK update
    const int nb = 2 * c.kd + 1;
    const double Ap = 8.0 * 3.0 * c.pcs * B;
    if (fused) {
      // the stage combination on the band: rk 0 reads S and writes P (= u0) and S; rk 1
      // reads S, P and writes acc, S; rk 2 reads S, P, acc and writes acc, S; rk 3 reads
      // S, acc and writes S
      const BandRk br{S, c.C, c.cs, prm, c.band, c.nu_b, c.err};
      const double bb = Adu * rows + Ap * (rk == 0 ? 3.0 : rk == 1 ? 4.0 : rk == 2 ? 5.0 : 3.0);
      if constexpr (DIM == 3 && N >= 64) {
        const bool bulk = c.sched.band_bulk < 0 ? N >= 256 : c.sched.band_bulk != 0;
        CUtensorMap map;
        const unsigned long long dims[4] = {(unsigned long long)c.kt, N, N, 3ull * c.batch};
        const unsigned long long strides[3] = {8ull * c.kt, 8ull * N * c.kt, 8ull * c.ds};
        const unsigned box[4] = {TW, 1, KxTma<N>::NY, 3};
        if (bulk && tma_band_fused_ctas > 0 && tma_encode(&map, c.DU, 4, dims, strides, box)) {
          const int ntiles = (c.kt / TW) * nb;
          const int gx = std::max(1, std::min(ntiles, tma_band_fused_ctas / c.batch));
          L3ES_LAUNCH(c, KK_X_EPI, bb, s,
                      kx_fwd_band_tma<N, true><<<dim3(gx, c.batch), TX, KxTma<N>::SMEM, s>>>(
                          map, c.kt, c.kd, c.P, c.pcs, c.tw, us, c.cs, 0, inv_n2d, c.eps_inj, c.band, c.err, br));
          return;
        }
      }
      if (DIM == 2 && c.sched.x_bulk)
        L3ES_LAUNCH(c, KK_X_EPI, bb, s,
                    kx_fwd_band<N, DIM, true, XN><<<dim3(c.kt / XN, 1, c.batch), TXN, 0, s>>>(
                        c.DU, c.ds, c.kt, c.kd, c.P, c.pcs, c.tw, us, c.cs, 0, inv_n2d, c.eps_inj, c.band, br));
      else
        L3ES_LAUNCH(c, KK_X_EPI, bb, s,
                    kx_fwd_band<N, DIM, true><<<dim3(c.kt / TW, DIM == 3 ? nb : 1, c.batch), TX, 0, s>>>(
                        c.DU, c.ds, c.kt, c.kd, c.P, c.pcs, c.tw, us, c.cs, 0, inv_n2d, c.eps_inj, c.band, br));
      return;
    }
    // (block 0 of each trajectory also computes the constant-power coefficient of us)
    bool band_done = false;
    // by default from 256^3: smaller grids have too few band tiles per persistent CTA to
    // pipeline (measured at 128^3: 9.5 us persistent vs 8.4 us one-shot)
    if constexpr (DIM == 3 && N >= 64) {
      const bool bulk = c.sched.band_bulk < 0 ? N >= 256 : c.sched.band_bulk != 0;
      CUtensorMap map;
      const unsigned long long dims[4] = {(unsigned long long)c.kt, N, N, 3ull * c.batch};
      const unsigned long long strides[3] = {8ull * c.kt, 8ull * N * c.kt, 8ull * c.ds};
      const unsigned box[4] = {TW, 1, KxTma<N>::NY, 3};
      if (bulk && tma_band_ctas > 0 && tma_encode(&map, c.DU, 4, dims, strides, box)) {
        const int ntiles = (c.kt / TW) * nb;
        const int gx = std::max(1, std::min(ntiles, tma_band_ctas / c.batch));
        L3ES_LAUNCH(c, KK_X_EPI, Adu * rows + Ap, s,
                    kx_fwd_band_tma<N><<<dim3(gx, c.batch), TX, KxTma<N>::SMEM, s>>>(
                        map, c.kt, c.kd, c.P, c.pcs, c.tw, us, c.cs, prm.band_kf2 > 0 ? c.kf : 0, inv_n2d,
                        c.eps_inj, c.band, c.err, BandRk{}));
        band_done = true;
      }
    }
    if (!band_done && DIM == 2 && c.sched.x_bulk)
      L3ES_LAUNCH(c, KK_X_EPI, Adu * rows + Ap, s,
                  kx_fwd_band<N, DIM, false, XN><<<dim3(c.kt / XN, 1, c.batch), TXN, 0, s>>>(
                      c.DU, c.ds, c.kt, c.kd, c.P, c.pcs, c.tw, us, c.cs, prm.band_kf2 > 0 ? c.kf : 0, inv_n2d,
                      c.eps_inj, c.band));
    else if (!band_done)
      L3ES_LAUNCH(c, KK_X_EPI, Adu * rows + Ap, s,
                  kx_fwd_band<N, DIM><<<dim3(c.kt / TW, DIM == 3 ? nb : 1, c.batch), TX, 0, s>>>(
                      c.DU, c.ds, c.kt, c.kd, c.P, c.pcs, c.tw, us, c.cs, prm.band_kf2 > 0 ? c.kf : 0, inv_n2d,
                      c.eps_inj, c.band));
    // rk -1: us -> du; 0: us -> out; 1: us, u0 -> acc, out; 2: us, u0, acc -> acc, out;
    // 3: us, acc -> fin
    double upd = Ap + A * (rk < 0 ? 2.0 : rk == 0 ? 2.0 : rk == 1 ? 4.0 : rk == 2 ? 5.0 : 3.0);
    if (prm.lin && rk >= 0 && !(prm.if_h > 0.f)) {  // outside the stage region: u0 in, one field out
      const double fr = DIM == 3 ? (2.0 * c.kd + 1.0) / N : (double)c.kt / H;
      upd = Ap + A * (fr * (rk == 0 ? 2.0 : rk == 1 ? 4.0 : rk == 2 ? 5.0 : 3.0) + (1.0 - fr) * 2.0);
    }
    const long long pairs = 3 * c.cs / 2;
    const dim3 ug((unsigned)((pairs + 255) / 256), c.batch);
    if (prm.lin && rk >= 0 && !(prm.if_h > 0.f))
      L3ES_LAUNCH(c, KK_RK_UPDATE, upd, s,
                  k_rk_update_lin<N, DIM><<<ug, 256, 0, s>>>(c.P, c.pcs, c.kt, c.kd, us, S, c.C, out, S, c.cs, prm,
                                                            c.band, c.nu_b, c.err));
    else if (prm.if_h > 0.f && rk >= 0)
      L3ES_LAUNCH(c, KK_RK_UPDATE, upd, s,
                  k_rk_update<N, DIM, true><<<ug, 256, 0, s>>>(c.P, c.pcs, c.kt, c.kd, us, S, c.C, out, S, c.cs, prm,
                                                                c.band, c.nu_b, c.err));
    else
      L3ES_LAUNCH(c, KK_RK_UPDATE, upd, s,
                  k_rk_update<N, DIM><<<ug, 256, 0, s>>>(c.P, c.pcs, c.kt, c.kd, us, S, c.C, out, S, c.cs, prm,
                                                          c.band, c.nu_b, c.err));
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
    const double A = 8.0 * 3.0 * c.cs * c.batch, P = 4.0 * 3.0 * c.ps * c.batch;
    bool x_done = false;
    if constexpr (DIM == 3 && N >= 64) {  // persistent, next tile by one bulk tensor load
      CUtensorMap map;
      const unsigned long long dims[3] = {(unsigned long long)mc, N, 3ull * c.batch};
      const unsigned long long strides[2] = {8ull * mc, 8ull * c.cs};
      const unsigned box[3] = {TW, KxTma<N>::NY, 3};
      if (c.sched.x_bulk && tma_plain_ctas > 0 && tma_encode(&map, uh, 3, dims, strides, box)) {
        const int ntiles = (int)(mc / TW);
        const int gx = std::max(1, std::min(ntiles, tma_plain_ctas / c.batch));
        L3ES_LAUNCH(c, KK_X_INV_PLAIN, 2.0 * A, s,
                    kx_inv_tma<N, false><<<dim3(gx, c.batch), TX, KxTma<N>::SMEM, s>>>(map, c.W, c.fs, c.tw, ntiles,
                                                                                        c.err, nullptr, XLin{}));
        x_done = true;
      }
    }
    if (!x_done)
      L3ES_LAUNCH(c, KK_X_INV_PLAIN, 2.0 * A, s,
                  kx_inv<N, DIM, false><<<dim3((unsigned)((mc + TW - 1) / TW), c.batch), TX, 0, s>>>(
                      uh, c.cs, c.W, c.fs, c.tw));
    if (DIM == 3) y_pass<kInv>(c, KK_Y_INV, 2.0 * A, c.W, c.fs, H, N / 2, 3 * c.batch, s);
    L3ES_LAUNCH(c, KK_LINE_C2R, A + P, s,
                line_c2r<N><<<dim3(line_blocks(lines), c.batch), L::THREADS, 0, s>>>(
                    c.W, c.fs, u, c.ps, scale, c.tw, (int)lines));
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
    const double A = 8.0 * 3.0 * c.cs * c.batch, P = 4.0 * 3.0 * c.ps * c.batch;
    L3ES_LAUNCH(c, KK_LINE_R2C, A + P, s,
                line_r2c<N><<<dim3(line_blocks(lines), c.batch), L::THREADS, 0, s>>>(
                    u, c.ps, c.W, c.fs, c.tw, (int)lines));
    if (DIM == 3) y_pass<kFwd>(c, KK_Y_FWD, 2.0 * A, c.W, c.fs, H, N / 2, 3 * c.batch, s);
    L3ES_LAUNCH(c, KK_X_FWD_PLAIN, 2.0 * A, s,
                kx_fwd_plain<N, DIM><<<dim3((unsigned)((mc + TW - 1) / TW), c.batch), TX, 0, s>>>(
                    c.W, c.fs, uh, c.cs, c.tw));
  }

  static void rfftn(const Ctx& c, const float* u, float2* uh, cudaStream_t s) {
    if (c.dim == 3)
      rfftn_dim<3>(c, u, uh, s);
    else
      rfftn_dim<2>(c, u, uh, s);
  }

  // Vector-Jacobian product of the RHS (adjoint_kernels.cuh): u/curl x-inverse,
  // projected-cotangent x-inverse (+ band terms), y inverse (3D), one line pass for
  // both products, y forward (3D), x forward, elementwise epilogue.
  template <int DIM>
  static void vjp_dim(const Ctx& c, const AdjEpi& a, float2* Wm, float2* Y6, cudaStream_t s) {
    const long long mc = c.nmid * H;
    const long long lines = c.nmid * N;
    const float scale = (float)(1.0 / (DIM == 3 ? (double)N * N * N : (double)N * N));
    const double A = 8.0 * 3.0 * c.cs * c.batch;  // bytes of one 3-component spectrum
    const unsigned xb = (unsigned)((mc + TW - 1) / TW);
    const double inv_n2d = 1.0 / (DIM == 3 ? std::pow((double)N, 6) : std::pow((double)N, 4));
    // u and curl u lines of the stage field: the forward RHS's x and y inverse passes, or
    // the lines the stage recomputation left (a.wlines)
    const float2* wuw = a.wlines ? a.wlines : c.W;
    if (!a.wlines) x_inverse<DIM>(c, a.us, (DIM == 3 ? 8.0 : 9.0) / 3.0 * A, s);
    L3ES_LAUNCH(c, KK_ADJ_X_INV, 2.0 * A, s,
                kx_inv_adjproj<N, DIM><<<dim3(xb, c.batch), TX, 0, s>>>(
                    a.g, c.cs, a.gscale, c.kd, Wm, c.fs, c.tw, a.us, a.band_kf2 > 0 ? c.kf : 0, inv_n2d,
                    c.eps_inj, const_cast<double*>(a.band_adj)));
    if (DIM == 3) {
      if (!a.wlines) y_inv_rhs(c, 11.0 / 3.0 * A, s);
      y_pass<kInv>(c, KK_Y_INV, 2.0 * A, Wm, c.fs, H, N / 2, 3 * c.batch, s);
    }
    L3ES_LAUNCH(c, KK_ADJ_LINE, 5.0 * A, s,
                line_cross_adj<N><<<dim3(line_blocks(lines), c.batch), L::THREADS, 0, s>>>(
                    Wm, wuw, c.fs, Y6, c.cs, scale, c.tw, (int)lines));
    if (DIM == 3) y_pass<kFwd>(c, KK_Y_FWD, 4.0 * A, Y6, c.cs, H, N / 2, 6 * c.batch, s);
    // Y6 (6 fields per trajectory) -> W, as 2 * batch groups of 3 fields
    L3ES_LAUNCH(c, KK_X_FWD_PLAIN, 4.0 * A, s,
                kx_fwd_plain<N, DIM><<<dim3(xb, 2 * c.batch), TX, 0, s>>>(Y6, c.cs, c.W, c.fs, c.tw));
    const long long pairs = c.cs / 2;
    // reads: 2 product spectra, g, lam1, lam_in; writes: lam_out, g_out
    const double epi = (3.0 + (a.lam1 ? 1.0 : 0.0) + (a.lam_in ? 1.0 : 0.0) + 1.0 + (a.g_out ? 1.0 : 0.0)) * A;
    L3ES_LAUNCH(c, KK_ADJ_EPI, epi, s,
                k_adj_epi<N, DIM><<<dim3((unsigned)((pairs + 255) / 256), c.batch), 256, 0, s>>>(c.W, c.cs, a,
                                                                                                 c.nu_b));
  }

  static void vjp(const Ctx& c, const AdjEpi& a, float2* Wm, float2* Y6, cudaStream_t s) {
    if (c.dim == 3)
      vjp_dim<3>(c, a, Wm, Y6, s);
    else
      vjp_dim<2>(c, a, Wm, Y6, s);
  }
};

template <int N>
DnsTable make_dns_table() {
  DnsOps<N>::init_attrs();
  DnsTable t;
  t.stage = &DnsOps<N>::stage;
  t.irfftn = &DnsOps<N>::irfftn;
  t.rfftn = &DnsOps<N>::rfftn;
  t.vjp = &DnsOps<N>::vjp;
  return t;
}

}  // namespace l3es
