// Register/shared-memory FFT building blocks for sm_103a.
//
// An N-point complex FFT is computed cooperatively by T = N/E threads of a CTA,
// each holding E = 8 complex values in registers. The algorithm is Stockham
// autosort (Govindaraju et al., SC'08): radix-R stages (R <= E), E/R butterflies
// per thread and stage, data exchanged through shared memory between stages.
// Input element n and output element k both live in thread n % T, slot n / T,
// so a forward FFT can consume the register output of an inverse FFT directly.
//
// Twiddles come from a table tw[m] = exp(-2 pi i m / Ntab) computed in FP64 on the
// host and stored FP32; an N-point FFT indexes it with stride Ntab / N. FFTs whose
// threads sit in one warp can instead read a compact per-stage table (CT = true, see
// Sched::ctoff) in which the twiddles of one stage are contiguous in the thread index,
// so a warp's twiddle load touches one or two 128-byte lines instead of up to eight.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace l3es {

constexpr int kFwd = -1;  // exp(-i ...): numpy fft / rfft
constexpr int kInv = +1;  // exp(+i ...): numpy ifft / irfft (unnormalised)

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
// multiply by exp(DIR * i * pi / 2): DIR=-1 -> -i, DIR=+1 -> +i
template <int DIR>
__device__ __forceinline__ float2 mul_i(float2 a) {
  return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}
// twiddle from the FP32 table, conjugated for the inverse direction
template <int DIR>
__device__ __forceinline__ float2 twid(const float2* __restrict__ tw, int idx) {
  float2 w = __ldg(tw + idx);
  return DIR < 0 ? w : conjf2(w);
}

// cos/sin(2 pi k / 16), k = 0..3 (first quadrant), exact decimal constants
__device__ __forceinline__ float c16(int k) {
  return k == 0 ? 1.0f : k == 1 ? 0.92387953251128674f : k == 2 ? 0.70710678118654752f : 0.38268343236508978f;
}

// In-register DFT of size R (2, 4, 8, 16), natural order in and out.
template <int R, int DIR>
struct Dft;

template <int DIR>
struct Dft<1, DIR> {
  static __device__ __forceinline__ void run(float2*) {}
};

template <int DIR>
struct Dft<2, DIR> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <int DIR>
struct Dft<4, DIR> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    float2 s13 = cadd(v[1], v[3]), d13 = mul_i<DIR>(csub(v[1], v[3]));
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
  }
};

// radix-2 decimation in time on top of two half-size DFTs
template <int R, int DIR>
struct DftSplit {
  static __device__ __forceinline__ void run(float2* v) {
    float2 e[R / 2], o[R / 2];
#pragma unroll
    for (int i = 0; i < R / 2; ++i) {
      e[i] = v[2 * i];
      o[i] = v[2 * i + 1];
    }
    Dft<R / 2, DIR>::run(e);
    Dft<R / 2, DIR>::run(o);
#pragma unroll
    for (int k = 0; k < R / 2; ++k) {
      float2 t;
      // W_R^k = exp(DIR * 2 pi i k / R) expressed in sixteenths of a turn
      const int q = k * (16 / R);  // 0..7
      if (q == 0) {
        t = o[k];
      } else if (q == 4) {
        t = mul_i<DIR>(o[k]);
      } else {
        // angle 2 pi q / 16 in (0, pi): cos = c16(q) (q<4) or -c16(8-q) ...
        float cr, si;
        if (q < 4) {
          cr = c16(q);
          si = c16(4 - q);
        } else {
          cr = -c16(8 - q);
          si = c16(q - 4);
        }
        const float2 w = make_float2(cr, DIR * si);
        t = cmul(o[k], w);
      }
      v[k] = cadd(e[k], t);
      v[k + R / 2] = csub(e[k], t);
    }
  }
};

template <int DIR>
struct Dft<8, DIR> {
  static __device__ __forceinline__ void run(float2* v) { DftSplit<8, DIR>::run(v); }
};
template <int DIR>
struct Dft<16, DIR> {
  static __device__ __forceinline__ void run(float2* v) { DftSplit<16, DIR>::run(v); }
};

// Compile-time stage schedule: radix E until the remainder is smaller than E.
template <int N, int E>
struct Sched {
  static constexpr int ilog(int n, int e) { return n < e ? 0 : 1 + ilog(n / e, e); }
  static constexpr int ipow(int e, int k) { return k == 0 ? 1 : e * ipow(e, k - 1); }
  static constexpr int kFull = ilog(N, E);           // number of radix-E stages
  static constexpr int kRem = N / ipow(E, kFull);    // last radix (1 if none)
  static constexpr int kStages = kFull + (kRem > 1 ? 1 : 0);
  static constexpr int radix(int s) { return s < kFull ? E : kRem; }
  static constexpr int ns(int s) { return ipow(E, s); }  // Ns before stage s
  // compact twiddle table: stage s >= 1 holds (radix(s) - 1) x ns(s) entries
  // ct[ctoff(s) + (r - 1) ns(s) + jm] = exp(-2 pi i r jm / (ns(s) radix(s))), r >= 1,
  // jm < ns(s); stage 0 (Ns = 1) needs none
  static constexpr int ctoff(int s) { return s <= 1 ? 0 : ctoff(s - 1) + (radix(s - 1) - 1) * ns(s - 1); }
  static constexpr int ctlen() { return ctoff(kStages); }
};

// Exchange index per layout, chosen with a shared-memory bank model (8-byte
// accesses served per half warp) of every Stockham read/write pattern:
//  - column-interleaved buffers (SS > 1): one spare slot every 8 elements;
//  - contiguous per-line buffers (SS == 1): XOR swizzle of the low 4 bits (a
//    permutation inside aligned blocks of 16) by bits 3..6 when a thread holds 8
//    elements, by bits 4..7 when it holds 16; lines M + 8 slots apart.
template <int SS, int E = 8>
__device__ __forceinline__ int xpad(int n) {
  return SS == 1 ? (E == 16 ? n ^ ((n >> 4) & 15) : n ^ ((n >> 3) & 15)) : n + (n >> 3);
}
template <int SS>
__host__ __device__ constexpr int xpad_len(int n) { return SS == 1 ? n + 8 : n + n / 8; }

template <bool WARP>
__device__ __forceinline__ void fft_sync() {
  if (WARP)
    __syncwarp();
  else
    __syncthreads();
}

// One Stockham stage. FIRST: inputs from registers; LAST: outputs to registers.
// sm: exchange buffer, element n at sm[xpad<SS>(n) * SS]. WARP: all T threads of the
// FFT are in one warp, so __syncwarp orders the exchanges.
// CT: tw is the compact table at this stage's offset (tws unused).
template <int N, int E, int R, int NS, int DIR, int SS, bool WARP, bool FIRST, bool LAST, bool CT = false>
__device__ __forceinline__ void stockham_stage(float2 (&v)[E], float2* sm, int t,
                                               const float2* __restrict__ tw, int tws) {
  constexpr int T = N / E;
  constexpr int BPT = E / R;  // butterflies per thread
  float2 x[BPT][R];
#pragma unroll
  for (int b = 0; b < BPT; ++b) {
    const int j = t + T * b;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      x[b][r] = FIRST ? v[b + r * BPT] : sm[xpad<SS, E>(j + r * (N / R)) * SS];
    }
  }
  if (!FIRST && !LAST) fft_sync<WARP>();  // all reads done before the in-place writes
#pragma unroll
  for (int b = 0; b < BPT; ++b) {
    const int j = t + T * b;
    if (NS > 1) {
      const int jm = j % NS;
#pragma unroll
      for (int r = 1; r < R; ++r)
        x[b][r] = cmul(x[b][r], twid<DIR>(tw, CT ? (r - 1) * NS + jm : r * jm * (N / (NS * R)) * tws));
    }
    Dft<R, DIR>::run(x[b]);
    if (LAST) {
#pragma unroll
      for (int r = 0; r < R; ++r) v[b + r * BPT] = x[b][r];
    } else {
      const int base = (j / NS) * NS * R + (j % NS);
#pragma unroll
      for (int r = 0; r < R; ++r) sm[xpad<SS, E>(base + r * NS) * SS] = x[b][r];
    }
  }
  if (!LAST) fft_sync<WARP>();
}

template <int N, int E, int DIR, int SS, bool WARP, bool CT, int S, bool DONE = (S >= Sched<N, E>::kStages)>
struct Stages;
template <int N, int E, int DIR, int SS, bool WARP, bool CT, int S>
struct Stages<N, E, DIR, SS, WARP, CT, S, false> {
  using Sc = Sched<N, E>;
  static __device__ __forceinline__ void run(float2 (&v)[E], float2* sm, int t,
                                             const float2* __restrict__ tw, int tws) {
    stockham_stage<N, E, Sc::radix(S), Sc::ns(S), DIR, SS, WARP, S == 0, S == Sc::kStages - 1, CT>(
        v, sm, t, CT ? tw + Sc::ctoff(S) : tw, tws);
    Stages<N, E, DIR, SS, WARP, CT, S + 1>::run(v, sm, t, tw, tws);
  }
};
template <int N, int E, int DIR, int SS, bool WARP, bool CT, int S>
struct Stages<N, E, DIR, SS, WARP, CT, S, true> {
  static __device__ __forceinline__ void run(float2 (&)[E], float2*, int, const float2* __restrict__, int) {}
};

// N-point FFT by T = N/E threads; every thread of the CTA (WARP = false) or of the
// warp (WARP = true) must call it, since it synchronises between stages. v[e] holds
// element t + T*e on entry and on exit. tws: stride into the twiddle table (table
// length / N); with CT, tw is the compact table of the N-point FFT instead. The exchange buffer is free on return only after the caller's next
// barrier of the same scope.
template <int N, int E, int DIR, int SS, bool WARP = false, bool CT = false>
__device__ __forceinline__ void block_fft(float2 (&v)[E], float2* sm, int t,
                                          const float2* __restrict__ tw, int tws) {
  Stages<N, E, DIR, SS, WARP, CT, 0>::run(v, sm, t, tw, tws);
}

// N-point FFT whose T = N/E threads sit in one warp (per-line buffers, SS = 1). For
// N = 2 E^2 (e.g. 128 = 8 x 8 x 2) the final radix-2 stage pairs element j with
// j + N/2; after the second stage they sit in the same register slot of lanes t and
// t ^ E, so that stage exchanges by warp shuffle instead of a shared-memory round
// trip. Other sizes use the shared-memory Stockham schedule. ct: the compact twiddle
// table of the N-point FFT (Sched<N, E>::ctoff layout, length Sched<N, E>::ctlen()).
template <int N, int E, int DIR>
__device__ __forceinline__ void warp_fft(float2 (&v)[E], float2* sm, int t, const float2* __restrict__ ct) {
  using Sc = Sched<N, E>;
  constexpr bool kTail2 = Sc::kStages == 3 && Sc::radix(0) == E && Sc::radix(1) == E && Sc::radix(2) == 2 &&
                          N / E == 2 * E && N / E <= 32;
  if constexpr (!kTail2) {
    block_fft<N, E, DIR, 1, true, true>(v, sm, t, ct, 0);
  } else {
    constexpr int T = N / E;
    // stage 0: radix E on the registers, out to shared memory
    stockham_stage<N, E, E, 1, DIR, 1, true, true, false>(v, sm, t, ct, 0);
    // stage 1: radix E (Ns = E), one butterfly per thread, outputs stay in registers:
    // slot r holds element (t / E) N/2 + t % E + r E
    {
      float2 x[E];
#pragma unroll
      for (int r = 0; r < E; ++r) x[r] = sm[xpad<1, E>(t + r * (N / E))];
      const int jm = t % E;
#pragma unroll
      for (int r = 1; r < E; ++r) x[r] = cmul(x[r], twid<DIR>(ct, Sc::ctoff(1) + (r - 1) * E + jm));
      Dft<E, DIR>::run(x);
#pragma unroll
      for (int r = 0; r < E; ++r) v[r] = x[r];
    }
    // stage 2: radix 2 (Ns = N/2) between lanes t and t ^ E
    {
      const bool hi = t >= E;
      const int partner = (threadIdx.x & 31) ^ E;
      float2 y[E];
#pragma unroll
      for (int b = 0; b < E / 2; ++b) {
        const float2 give = hi ? v[2 * b] : v[2 * b + 1];
        float2 got;
        got.x = __shfl_sync(0xffffffffu, give.x, partner);
        got.y = __shfl_sync(0xffffffffu, give.y, partner);
        const float2 a = hi ? got : v[2 * b];
        float2 c = hi ? v[2 * b + 1] : got;
        const int j = t + T * b;
        c = cmul(c, twid<DIR>(ct, Sc::ctoff(2) + j));
        y[b] = cadd(a, c);
        y[b + E / 2] = csub(a, c);
      }
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = y[e];
    }
  }
}

// Elements per thread used for an N-point FFT (radix-8 stages).
template <int N>
struct Fft {
  static constexpr int E = N >= 8 ? 8 : N;
  static constexpr int T = N / E;
};

// Radix-16 variant: one exchange for N = 256 (16 x 16), half the shared-memory
// traffic of the radix-8 schedule; used where registers allow 16 values per thread.
template <int N>
struct Fft16 {
  static constexpr int E = N >= 16 ? 16 : N;
  static constexpr int T = N / E;
};

// signed integer wavenumber of FFT index i on a full axis of length n (fftfreq)
__device__ __forceinline__ int kfull(int i, int n) { return i < n / 2 ? i : i - n; }

}  // namespace l3es
