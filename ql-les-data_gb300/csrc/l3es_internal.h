// Internal host-side declarations shared by the l3es_gb300 translation units.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "../../include/l3es_gb300.h"
#include "dns_kernels.cuh"

namespace l3es {

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
  int npartial = 0;     // CTAs of kx_fwd_epi per trajectory
  float2* tw = nullptr;        // N-point twiddle table
  float2* W = nullptr;         // [batch][6][cs]
  float2* DU = nullptr;        // [batch][3][ds]
  float2* Tb = nullptr;        // [batch][3][cs] RK stage field
  float2* C = nullptr;         // [batch][3][cs] RK accumulator
  double* partial = nullptr;   // [batch][npartial]
  double* band = nullptr;      // [batch] constant-power coefficient
  double* e0 = nullptr;        // [batch] ekin_tot targets
  double* einj = nullptr;      // [batch] scratch e_inj
  int kf = 0;                  // forcing band 0 < |k|^2 <= kf^2
  double eps_inj = 0.0;        // constant-power injection rate
};

// Launch wrappers for one grid size N (both dims), explicitly instantiated per N.
struct DnsTable {
  // one RK stage: RHS of `us` + epilogue (rk 0..3) into the state S / stage field
  // `out`; rk = -1 writes the RHS itself to `out`
  void (*stage)(const Ctx&, const float2* us, float2* S, float2* out, int rk, const EpiParams& prm,
                cudaStream_t s);
  void (*irfftn)(const Ctx&, const float2* uh, float* u, cudaStream_t s);
  void (*rfftn)(const Ctx&, const float* u, float2* uh, cudaStream_t s);
};

// Launch table of grid size N (defined in dns_ops.cuh, instantiated per N in dns_n*.cu).
template <int N>
DnsTable make_dns_table();
bool dns_table(int n, DnsTable* out);  // false if N is not compiled in

// thread-local error reporting
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

}  // namespace l3es
