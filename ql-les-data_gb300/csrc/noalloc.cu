// Allocation-free particle interpolation: l3es_interp_dft_noalloc.
//
// Some hosts cannot let a library allocate device memory. A JAX/XLA program that
// calls this library through an FFI custom call is the common case: XLA reserves
// most of the GPU for its own pool at start-up (the reference exposes that
// fraction as its xla_mem_fraction option), so a cudaMalloc from inside the call
// can fail or fragment memory that XLA believes it owns. Hosts that run under a
// fixed device-memory budget are in the same position. For them this entry point
// computes the same result as l3es_interp_set_spectrum followed by l3es_interp
// with the exact (dft) backend, but keeps its only scratch buffer, the coarse
// spectrum, in a fixed-size array that is part of the loaded library image.
//
// Limits and sharing rules:
//  - the scratch holds kNoallocScratchElems complex64 values (417,792 bytes), the
//    coarse spectrum of ckp_N = 32 in 3D; requests above ckp_N = 32 in 3D or
//    ckp_N = 64 in 2D (where the kernel's per-block phase tables reach the shared
//    memory limit) are rejected with L3ES_EINVAL;
//  - every GPU that loads the library keeps this array for the life of the
//    process;
//  - all calls share the one array and it keeps the previous call's contents.
//    Each call writes every scratch element it reads before reading it, so
//    nothing has to start at zero; but two calls whose work overlaps on the GPU
//    (different streams, or different host threads, without ordering between
//    them) race on the array and give wrong results;
//  - the host symbol of the array is only a stand-in and must never be handed to a
//    kernel; every call outside stream capture looks up the array's device address
//    on the current device (cheap), so the address stays right after a
//    cudaDeviceReset reloads the library's device code; a call made while the
//    stream is being captured uses the address found by the last call outside
//    capture on that device, so make one call on each device before any capture;
//  - CUDA loads a library's device code lazily by default: the first call on a
//    device (the look-up above) loads the module and so places the array in device
//    memory. A host whose device memory is spoken for should make that first call
//    (a warm-up call with a small np) before it hands the device to its own pool,
//    or run with CUDA_MODULE_LOADING=EAGER;
//  - np is at most 128 (2^31 - 1) particles (one thread per particle, the grid-x
//    limit).
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <mutex>
#include <string>

#include "l3es_internal.h"
#include "particle_kernels.cuh"

namespace l3es {

constexpr long long kNoallocScratchElems = 3LL * 32 * 32 * (32 / 2 + 1);  // 52,224 complex64

static __device__ __align__(256) float2 g_noalloc_scratch[kNoallocScratchElems];

constexpr int kMaxDevices = 64;
constexpr long long kNoallocMaxParticles = 128LL * 2147483647LL;
static std::atomic<float2*> g_scratch_ptr[kMaxDevices];
static std::mutex g_scratch_mu;

// Device address of g_noalloc_scratch on the current device: looked up on every call
// outside stream capture (after a cudaDeviceReset the module is reloaded and the
// array may move), the cached value of this device while `stream` is capturing.
static int noalloc_scratch(cudaStream_t stream, float2** out) {
  int dev = -1;
  int rc = cuda_check(cudaGetDevice(&dev), "l3es_interp_dft_noalloc: cudaGetDevice");
  if (rc != L3ES_OK) return rc;
  if (dev < 0 || dev >= kMaxDevices) return fail(L3ES_ESTATE, "l3es_interp_dft_noalloc: device index out of range");
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  rc = cuda_check(cudaStreamIsCapturing(stream, &cap), "l3es_interp_dft_noalloc: cudaStreamIsCapturing");
  if (rc != L3ES_OK) return rc;
  if (cap != cudaStreamCaptureStatusNone) {
    float2* p = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!p)
      return fail(L3ES_ESTATE,
                  "l3es_interp_dft_noalloc: the first call on a device must come before any stream capture");
    *out = p;
    return L3ES_OK;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  void* addr = nullptr;
  rc = cuda_check(cudaGetSymbolAddress(&addr, g_noalloc_scratch),
                  "l3es_interp_dft_noalloc: cudaGetSymbolAddress(scratch)");
  if (rc != L3ES_OK) return rc;
  g_scratch_ptr[dev].store(static_cast<float2*>(addr), std::memory_order_release);
  *out = static_cast<float2*>(addr);
  return L3ES_OK;
}

}  // namespace l3es

using namespace l3es;

extern "C" int l3es_interp_dft_noalloc(int32_t dim, int32_t n_fine, int32_t ckp_n, const void* u_hat_fine,
                                       const double* r, int64_t np, double* u_r, void* stream) {
  if (!u_hat_fine || !r || !u_r) return fail(L3ES_EINVAL, "l3es_interp_dft_noalloc: null argument");
  if (dim != 2 && dim != 3) return fail(L3ES_EINVAL, "l3es_interp_dft_noalloc: dim must be 2 or 3");
  if (ckp_n < 2 || (ckp_n & (ckp_n - 1)) != 0 || n_fine < ckp_n || (n_fine & (n_fine - 1)) != 0)
    return fail(L3ES_EINVAL, "l3es_interp_dft_noalloc: need powers of two with 2 <= ckp_N <= N");
  if (np < 0) return fail(L3ES_EINVAL, "l3es_interp_dft_noalloc: np < 0");
  if (np > kNoallocMaxParticles)
    return fail(L3ES_EINVAL, "l3es_interp_dft_noalloc: np above 128 (2^31 - 1), the one-thread-per-particle grid limit");
  const int c = ckp_n, hc = c / 2 + 1;
  const long long hcs = dim == 3 ? (long long)c * c * hc : (long long)c * hc;
  if (3 * hcs > kNoallocScratchElems || (dim == 2 && c > 64))
    return fail(L3ES_EINVAL, "l3es_interp_dft_noalloc: ckp_N=" + std::to_string(c) + " in " + std::to_string(dim) +
                                 "D is above the limit of the fixed " + std::to_string(kNoallocScratchElems * 8) +
                                 "-byte scratch (3D ckp_N <= 32, 2D ckp_N <= 64)");
  cudaStream_t s = (cudaStream_t)stream;
  float2* hh = nullptr;
  int rc = noalloc_scratch(s, &hh);
  if (rc != L3ES_OK) return rc;
  if (np == 0) return L3ES_OK;
  const int N = n_fine;
  const long long cs = dim == 3 ? (long long)N * N * (N / 2 + 1) : (long long)N * (N / 2 + 1);
  const float scale = (float)std::pow((double)c / N, dim);
  const unsigned blocks = (unsigned)((hcs + 255) / 256);
  const unsigned pb = (unsigned)((np + 127) / 128);
  const size_t smem = sizeof(float2) * dim * c * 128;
  if (dim == 3) {
    k_crop<3><<<dim3(blocks, 3), 256, 0, s>>>((const float2*)u_hat_fine, cs, N, hh, hcs, c, scale);
    rc = cuda_check(cudaFuncSetAttribute(k_dft_interp<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "l3es_interp_dft_noalloc: shared memory attribute");
    if (rc != L3ES_OK) return rc;
    k_dft_interp<3><<<pb, 128, smem, s>>>(hh, hcs, c, 3, r, np, u_r, 0.0, nullptr);
  } else {
    k_crop<2><<<dim3(blocks, 3), 256, 0, s>>>((const float2*)u_hat_fine, cs, N, hh, hcs, c, scale);
    rc = cuda_check(cudaFuncSetAttribute(k_dft_interp<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "l3es_interp_dft_noalloc: shared memory attribute");
    if (rc != L3ES_OK) return rc;
    k_dft_interp<2><<<pb, 128, smem, s>>>(hh, hcs, c, 2, r, np, u_r, 0.0, nullptr);
  }
  return cuda_check(cudaGetLastError(), "l3es_interp_dft_noalloc launch");
}
