// fom.cu -- matrix-free FOM velocity-stress leapfrog for sm_103a.
//
// The reference assembles two CRS Jacobians (src/kokkos/shwavepp.hpp:319-466) and
// advances with two Kokkos-Kernels SpMV/SpMM calls per step
// (src/kokkos/fom_update_kernels.hpp:60-181).  Here the sparsity is implicit: the
// library checks once that the mesh is the mesher's structured full grid and then
// computes neighbour gids from (j, i).  Only the stencil values are stored, one
// coefficient array per neighbour slot (SoA), with dt folded in:
//   vp point p:  v[p] = v[p] + cN*s[N] + cS*s[S] + cW*s[W] + cE*s[E]  (+ forcing)
//   sp point q:  s[q] = s[q] + cA*v[A] + cB*v[B]
// which is the reference's y + dt*(J x) re-associated to four (two) FMAs per
// entry: on GB300 the FP64 pipe, not HBM, is the tighter roof for this update.
//
// State layout in HBM: row-major [gid][M] (M = number of forcings, m fastest),
// i.e. gid order of the reference, so snapshots need no permutation.  Each thread
// owns VEC consecutive columns of one point (16-byte vector loads when M is even).
// Source injection (RankOneForcing / AddForcingRank2) is fused into the velocity
// kernel: the one thread that owns (src_gid[m], m) evaluates the signal on device.
// The seismogram receiver gather is fused into the stress launch as extra blocks
// (they read the velocity of the same step, which that launch does not modify).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "fom_sweep.h"
#include "fom_band.h"
#include "shaw_internal.h"

namespace shaw {

namespace {
thread_local std::string t_err;
}

void set_error(const std::string& msg) { t_err = msg; }
int fail(int code, const std::string& msg) {
  t_err = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  t_err = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? SHAW_ERR_OUT_OF_MEMORY : SHAW_ERR_CUDA;
}

}  // namespace shaw

extern "C" const char* shaw_last_error(void) { return shaw::t_err.c_str(); }
extern "C" const char* shaw_version(void) { return "shaw_gb300 0.1 (sm_103a)"; }

using shaw::FastDiv;

namespace {

constexpr int kThreads = 256;
constexpr uint32_t kGraphChunk = 64;  // leapfrog steps per captured CUDA graph
constexpr uint64_t kBandSteps = 1 << 16;  // leapfrog steps per persistent band launch

using shaw::FomCtl;
namespace sweep = shaw::sweep;

// Arguments shared by both half-step kernels (passed by value, < 4 KB).  The state
// and the folded stencil values are FP64 (SHAW_FP64) or FP32 (SHAW_MIXED_FP32).
struct FomArgs {
  void* xv;            // [nvp][M]
  void* xs;            // [nsp][M]
  const void* cvp;     // 4 planes of nvp: N, S, W, E (dt folded)
  const void* csp;     // 2 planes of nsp: A, B (dt folded)
  const double* rho_inv;
  const unsigned long long* src;  // [M] source vp gid per column
  const int* kind;
  const double* period;
  const double* delay;
  const unsigned long long* rcv;  // [R]
  double* seis;                   // [R x T x M] LayoutLeft
  FomCtl* ctl;
  double dt;
  uint32_t nth, nr, M, chunks;    // chunks = M / VEC
  uint32_t vp_items, sp_items;    // nvp*chunks, nsp*chunks
  uint32_t sp_row;                // 2*nth - 1
  uint32_t R, seis_freq, seis_T;
  uint32_t sp_blocks;             // blocks of the stress part of the stress launch
  int rank2;
  FastDiv chunks_div, nth_div, sprow_div;
};

// VEC consecutive columns of one point as one vector load/store (16 bytes at most).
template <typename T, int VEC>
struct VecT;
template <typename T>
struct VecT<T, 1> {
  using type = T;
  __device__ static T ld(const T* p) { return *p; }
  __device__ static void st(T* p, T v) { *p = v; }
};
template <>
struct VecT<double, 2> {
  using type = double2;
  __device__ static double2 ld(const double* p) { return *reinterpret_cast<const double2*>(p); }
  __device__ static void st(double* p, double2 v) { *reinterpret_cast<double2*>(p) = v; }
};
template <>
struct VecT<float, 2> {
  using type = float2;
  __device__ static float2 ld(const float* p) { return *reinterpret_cast<const float2*>(p); }
  __device__ static void st(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
};
template <>
struct VecT<float, 4> {
  using type = float4;
  __device__ static float4 ld(const float* p) { return *reinterpret_cast<const float4*>(p); }
  __device__ static void st(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
};

__device__ __forceinline__ void fma_into(double& acc, double c, double x) { acc = fma(c, x, acc); }
__device__ __forceinline__ void fma_into(double2& acc, double c, double2 x) {
  acc.x = fma(c, x.x, acc.x);
  acc.y = fma(c, x.y, acc.y);
}
__device__ __forceinline__ void fma_into(float& acc, float c, float x) { acc = fmaf(c, x, acc); }
__device__ __forceinline__ void fma_into(float2& acc, float c, float2 x) {
  acc.x = fmaf(c, x.x, acc.x);
  acc.y = fmaf(c, x.y, acc.y);
}
__device__ __forceinline__ void fma_into(float4& acc, float c, float4 x) {
  acc.x = fmaf(c, x.x, acc.x);
  acc.y = fmaf(c, x.y, acc.y);
  acc.z = fmaf(c, x.z, acc.z);
  acc.w = fmaf(c, x.w, acc.w);
}
__device__ __forceinline__ double& lane(double& v, int) { return v; }
__device__ __forceinline__ double& lane(double2& v, int e) { return e == 0 ? v.x : v.y; }
__device__ __forceinline__ float& lane(float& v, int) { return v; }
__device__ __forceinline__ float& lane(float2& v, int e) { return e == 0 ? v.x : v.y; }
__device__ __forceinline__ float& lane(float4& v, int e) { return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w; }

// sp gid of the stp point of cell (j, i): interleaved numbering of the mesher.
__device__ __forceinline__ uint32_t stp_gid(uint32_t j, uint32_t i, const FomArgs& a) {
  return (j + 1 < a.nr) ? j * a.sp_row + 2 * i + 1 : j * a.sp_row + i;
}

// Source term of column m at vp point p for step n (1-based), signal at t = (n-1)*dt.
// Out of line: only the one thread that owns (src[m], m) ever calls it.
__device__ __noinline__ double add_forcing(double x, const FomArgs& a, uint32_t m, uint32_t p, uint32_t k_local,
                                           unsigned long long host_step) {
  const unsigned long long n = (host_step ? host_step : a.ctl->step_base + k_local + 1);
  const double t = (double)(n - 1) * a.dt;
  const double f = shaw::signal_value(a.kind[m], a.delay[m], a.period[m], t);
  const double ri = a.rho_inv[p];
  // explicit roundings (no FMA contraction), as in the reference's host kernels
  if (a.rank2) return __dadd_rn(x, __dmul_rn(__dmul_rn(ri, f), a.dt));  // AddForcingRank2: x += rhoInv*f*dt
  return __dadd_rn(x, __dmul_rn(__dmul_rn(a.dt, ri), f));              // KokkosBlas::mult(1, x, dt, rhoInv, f)
}
// FP32 state: the source increment in FP64, in the same order, rounded once.
__device__ __noinline__ float add_forcing(float x, const FomArgs& a, uint32_t m, uint32_t p, uint32_t k_local,
                                          unsigned long long host_step) {
  const unsigned long long n = (host_step ? host_step : a.ctl->step_base + k_local + 1);
  const double t = (double)(n - 1) * a.dt;
  const double f = shaw::signal_value(a.kind[m], a.delay[m], a.period[m], t);
  const double ri = a.rho_inv[p];
  const double inc = a.rank2 ? __dmul_rn(__dmul_rn(ri, f), a.dt) : __dmul_rn(__dmul_rn(a.dt, ri), f);
  return x + __double2float_rn(inc);
}

// Forcing of the VEC columns c*VEC.. that this thread owns at vp point p.
template <typename V, int VEC>
__device__ __forceinline__ void apply_forcing(V& v, const FomArgs& a, uint32_t c, uint32_t p, uint32_t k_local,
                                              unsigned long long host_step) {
  if (VEC == 1) {
    if (a.src[c] == p) lane(v, 0) = add_forcing(lane(v, 0), a, c, p, k_local, host_step);
  } else {
#pragma unroll
    for (int h = 0; h < VEC / 2; ++h) {
      const ulonglong2 s2 = __ldg(reinterpret_cast<const ulonglong2*>(a.src) + (VEC / 2) * c + h);
      const uint32_t m0 = VEC * c + 2 * h;
      if (s2.x == p) lane(v, 2 * h) = add_forcing(lane(v, 2 * h), a, m0, p, k_local, host_step);
      if (s2.y == p) lane(v, 2 * h + 1) = add_forcing(lane(v, 2 * h + 1), a, m0 + 1, p, k_local, host_step);
    }
  }
}

// updateVelocity (fom_update_kernels.hpp:60-90 rank-1, :132-167 rank-2) for one step.
// Programmatic dependent launch: the two half-step kernels are launched so that the next
// one may be scheduled while this one drains.  Each waits for the complete previous
// grid (and its memory) before touching any state, and releases its dependents once
// its own stores are issued.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_next_grid() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename T, int VEC>
__global__ void __launch_bounds__(kThreads) fom_velocity_kernel(FomArgs a, uint32_t k_local,
                                                                unsigned long long host_step) {
  using V = VecT<T, VEC>;
  wait_prior_grid();
  T* const xv = static_cast<T*>(a.xv);
  const T* const xs = static_cast<const T*>(a.xs);
  const T* const cvp = static_cast<const T*>(a.cvp);
  const uint32_t item = blockIdx.x * kThreads + threadIdx.x;
  if (item >= a.vp_items) return;
  const uint32_t p = shaw::fast_div(item, a.chunks_div);
  const uint32_t c = item - p * a.chunks;
  const uint32_t j = shaw::fast_div(p, a.nth_div);
  const uint32_t i = p - j * a.nth;
  T* xp = xv + (size_t)p * a.M + c * VEC;
  typename V::type v = V::ld(xp);
  if (i != 0 && i + 1 != a.nth) {
    // interior theta: N/S are srp points, W/E stp points.  At the CMB (j == 0)
    // and the surface (j == nr-1) N and S are the same srp (merged coefficient in cN).
    const uint32_t rowN = (j + 1 < a.nr) ? j : j - 1;
    const uint32_t rowS = (j > 0) ? j - 1 : 0;
    const uint32_t gN = rowN * a.sp_row + 2 * i;
    const uint32_t gS = rowS * a.sp_row + 2 * i;
    const uint32_t gW = stp_gid(j, i - 1, a);
    const uint32_t gE = stp_gid(j, i, a);
    const size_t nvp = (size_t)a.nth * a.nr;
    const T cN = __ldg(cvp + p);
    const T cS = __ldg(cvp + nvp + p);
    const T cW = __ldg(cvp + 2 * nvp + p);
    const T cE = __ldg(cvp + 3 * nvp + p);
    const size_t off = (size_t)c * VEC;
    fma_into(v, cN, V::ld(xs + (size_t)gN * a.M + off));
    fma_into(v, cS, V::ld(xs + (size_t)gS * a.M + off));
    fma_into(v, cW, V::ld(xs + (size_t)gW * a.M + off));
    fma_into(v, cE, V::ld(xs + (size_t)gE * a.M + off));
  }
  // forcing: the thread owning (src[m], m) adds it, evaluating the signal at t_{n-1}
  apply_forcing<typename V::type, VEC>(v, a, c, p, k_local, host_step);
  V::st(xp, v);
  allow_next_grid();
}

// updateStress (fom_update_kernels.hpp:93-104, :170-181) + fused receiver gather.
template <typename T, int VEC>
__global__ void __launch_bounds__(kThreads) fom_stress_kernel(FomArgs a, uint32_t k_local,
                                                              unsigned long long host_step) {
  using V = VecT<T, VEC>;
  wait_prior_grid();
  const T* const xv = static_cast<const T*>(a.xv);
  T* const xs = static_cast<T*>(a.xs);
  const T* const csp = static_cast<const T*>(a.csp);
  if (blockIdx.x >= a.sp_blocks) {
    // Seismogram::storeVelocitySignalAtReceivers (seismogram.hpp:193-214)
    const unsigned long long n = (host_step ? host_step : a.ctl->step_base + k_local + 1);
    if (a.seis_freq == 0 || n % a.seis_freq != 0) return;
    const uint32_t idx = (blockIdx.x - a.sp_blocks) * kThreads + threadIdx.x;
    if (idx >= a.R * a.M) return;
    const uint32_t r = idx % a.R, m = idx / a.R;
    const unsigned long long cnt = n / a.seis_freq - 1;
    const double val = (double)xv[(size_t)a.rcv[r] * a.M + m];
    a.seis[r + (size_t)a.R * (cnt + (size_t)a.seis_T * m)] = val;
    if (!isfinite(val)) atomicOr(&a.ctl->nonfinite, 1u);
    return;
  }
  const uint32_t item = blockIdx.x * kThreads + threadIdx.x;
  if (item >= a.sp_items) return;
  const uint32_t q = shaw::fast_div(item, a.chunks_div);
  const uint32_t c = item - q * a.chunks;
  const uint32_t j = shaw::fast_div(q, a.sprow_div);
  const uint32_t rem = q - j * a.sp_row;
  uint32_t gA, gB;
  if (j + 1 < a.nr && (rem & 1u) == 0) {
    // srp of cell (j, i): north vp (j+1, i), south vp (j, i)
    const uint32_t i = rem >> 1;
    gA = (j + 1) * a.nth + i;
    gB = j * a.nth + i;
  } else {
    // stp of cell (j, i): west vp (j, i), east vp (j, i+1)
    const uint32_t i = (j + 1 < a.nr) ? (rem >> 1) : rem;
    gA = j * a.nth + i;
    gB = gA + 1;
  }
  const size_t nsp = (size_t)(a.nr - 1) * a.nth + (size_t)a.nr * (a.nth - 1);
  const T cA = __ldg(csp + q);
  const T cB = __ldg(csp + nsp + q);
  T* sp = xs + (size_t)q * a.M + c * VEC;
  typename V::type s = V::ld(sp);
  const size_t off = (size_t)c * VEC;
  fma_into(s, cA, V::ld(xv + (size_t)gA * a.M + off));
  fma_into(s, cB, V::ld(xv + (size_t)gB * a.M + off));
  V::st(sp, s);
  allow_next_grid();
}

// y = Jvp x (Jvp: nvp x nsp) or y = Jsp x (nsp x nvp) on column-major multivectors
// (one column per blockIdx.y), with the unfolded stencil values: the multivector
// SpMV of computeRomOperatorsUsingFomJacsWithMatProp (rom_compute_jacobians.hpp:88-101).
// Rows row0 .. row0+nrows-1 of the product are computed (x holds full columns, y
// holds nrows rows per column).  Per row the products are summed in the CRS entry
// order (N, S, W, E / A, B).
__global__ void fom_apply_vp_kernel(const double* __restrict__ craw, const double* __restrict__ x,
                                    double* __restrict__ y, uint32_t nth, uint32_t nr, size_t nsp, uint32_t row0,
                                    uint32_t nrows) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const uint32_t p = row0 + r;
  const size_t nvp = (size_t)nth * nr;
  const double* xc = x + (size_t)blockIdx.y * nsp;
  const uint32_t j = p / nth, i = p - j * nth;
  double sum = 0.0;
  if (i != 0 && i + 1 != nth) {
    const uint32_t row = 2 * nth - 1;
    const uint32_t gN = ((j + 1 < nr) ? j : j - 1) * row + 2 * i;
    const uint32_t gS = ((j > 0) ? j - 1 : 0) * row + 2 * i;
    const uint32_t gW = (j + 1 < nr) ? j * row + 2 * (i - 1) + 1 : j * row + i - 1;
    const uint32_t gE = (j + 1 < nr) ? j * row + 2 * i + 1 : j * row + i;
    sum = __dadd_rn(sum, __dmul_rn(craw[p], xc[gN]));
    if (gS != gN) sum = __dadd_rn(sum, __dmul_rn(craw[nvp + p], xc[gS]));
    sum = __dadd_rn(sum, __dmul_rn(craw[2 * nvp + p], xc[gW]));
    sum = __dadd_rn(sum, __dmul_rn(craw[3 * nvp + p], xc[gE]));
  }
  y[(size_t)blockIdx.y * nrows + r] = sum;
}

__global__ void fom_apply_sp_kernel(const double* __restrict__ craw, const double* __restrict__ x,
                                    double* __restrict__ y, uint32_t nth, uint32_t nr, size_t nsp, uint32_t row0,
                                    uint32_t nrows) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const uint32_t q = row0 + r;
  const size_t nvp = (size_t)nth * nr;
  const double* xc = x + (size_t)blockIdx.y * nvp;
  const uint32_t row = 2 * nth - 1;
  const uint32_t j = q / row, rem = q - j * row;
  uint32_t gA, gB;
  if (j + 1 < nr && (rem & 1u) == 0) {
    gA = (j + 1) * nth + (rem >> 1);
    gB = j * nth + (rem >> 1);
  } else {
    gA = j * nth + ((j + 1 < nr) ? (rem >> 1) : rem);
    gB = gA + 1;
  }
  double sum = __dmul_rn(craw[q], xc[gA]);
  sum = __dadd_rn(sum, __dmul_rn(craw[nsp + q], xc[gB]));
  y[(size_t)blockIdx.y * nrows + r] = sum;
}

// dt folded into the stencil values in FP64, then stored in the state's precision.
template <typename T>
__global__ void fom_fold_kernel(const double* raw, T* folded, double dt, size_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    folded[k] = (T)(dt * raw[k]);
}

// Point-major copies of the folded stencil values for the single sweep:
// out[(shift + p) * planes + c] = dt * raw[c * n + p] in the state's precision.
template <typename T>
__global__ void fom_fold_aos_kernel(const double* raw, T* out, double dt, size_t n, uint32_t planes, size_t shift) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n * planes; k += (size_t)gridDim.x * blockDim.x) {
    const size_t p = k / planes, c = k - p * planes;
    out[(shift + p) * planes + c] = (T)(dt * raw[c * n + p]);
  }
}

__global__ void fom_advance_base_kernel(FomCtl* ctl, unsigned int by) { ctl->step_base += by; }
__global__ void fom_set_base_kernel(FomCtl* ctl, unsigned long long v) { ctl->step_base = v; }

// [N][M] -> [M][N] FP64 for the LayoutLeft snapshot copy.
template <typename T>
__global__ void fom_transpose_kernel(const T* in, double* out, uint32_t N, uint32_t M) {
  __shared__ double tile[32][33];
  const uint32_t n0 = blockIdx.x * 32, m0 = blockIdx.y * 32;
  for (uint32_t r = threadIdx.y; r < 32; r += 8) {
    const uint32_t n = n0 + r, m = m0 + threadIdx.x;
    if (n < N && m < M) tile[r][threadIdx.x] = (double)in[(size_t)n * M + m];
  }
  __syncthreads();
  for (uint32_t r = threadIdx.y; r < 32; r += 8) {
    const uint32_t m = m0 + r, n = n0 + threadIdx.x;
    if (n < N && m < M) out[(size_t)m * N + n] = tile[threadIdx.x][r];
  }
}

}  // namespace

struct shaw_fom_s {
  uint64_t nth = 0, nr = 0, nvp = 0, nsp = 0;
  uint32_t M = 1;
  int rank = 1;
  int precision = SHAW_FP64;
  cudaStream_t stream = nullptr;
  size_t esz = sizeof(double);  // bytes per state value and folded stencil value
  // device buffers
  void* xv = nullptr;
  void* xs = nullptr;
  double* cvp_raw = nullptr;
  double* csp_raw = nullptr;
  void* cvp = nullptr;
  void* csp = nullptr;
  double* rho_inv = nullptr;
  unsigned long long* src = nullptr;
  int* kind = nullptr;
  double* period = nullptr;
  double* delay = nullptr;
  unsigned long long* rcv = nullptr;
  double* seis = nullptr;
  // snapshot copies: two staging buffers ([M][N] FP64 columns) filled on the compute stream,
  // read back on the copy stream while the time loop goes on
  double* stage[2] = {nullptr, nullptr};
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_ready[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr};
  bool stage_used[2] = {false, false};
  int stage_next = 0;
  FomCtl* ctl = nullptr;
  bool sources_set = false;
  // receivers / snapshots
  uint32_t R = 0;
  uint64_t seis_freq = 0, seis_T = 0, seis_nsteps = 0;
  uint64_t snap_fvp = 0, snap_fsp = 0, snap_nsteps = 0, snap_cvp = 0, snap_csp = 0;
  double* host_vp = nullptr;
  double* host_sp = nullptr;
  // run state
  double folded_dt = std::nan("");
  uint64_t step = 0;  // completed steps since reset
  uint64_t launches = 0;
  // graph cache (a chunk of graph_len steps)
  cudaGraphExec_t graph = nullptr;
  double graph_dt = std::nan("");
  uint64_t graph_len = 0;
  // single-sweep path (M a multiple of 32): the state alternates between two buffers each
  // step; xv / xs above always point at the current one, xvb[cur] / xsb[cur]
  bool sweep = false;                // the sweep is in use
  bool sweep_ok = false;             // its buffers exist (M a multiple of 32)
  sweep::Form form = sweep::kF64;
  void* xvb[2] = {nullptr, nullptr};
  void* xsb[2] = {nullptr, nullptr};
  int cur = 0;
  CUtensorMap tv[2], ts[2];          // tensor maps over the buffers (v box: strip + 1, sp box)
  void* cv4 = nullptr;               // point-major folded stencil values of the sweep (state precision)
  void* cs2 = nullptr;
  int sms = 0;
  // rank-1 persistent band path (small FP64 grids): bands, rows per band, shared memory
  bool band_ok = false, use_band = false;
  uint32_t band_n = 0, band_rows = 0, band_cols = 0;  // band width (rows or columns), column bands
  size_t band_smem = 0;
  double* ftab = nullptr;                 // [kBandSteps] forcing increments of one band launch
  unsigned long long* xwords = nullptr;   // halo exchange words, down then up
  unsigned long long* rcv_sorted = nullptr;  // [R][2] (key, receiver) pairs in key order (band ranges)
  uint32_t band_tag = 0;                  // last tag used in xwords (0: cleared)
  uint64_t src0 = 0;  // the rank-1 source: gid, kind, period, delay
  int kind0 = 0;
  double period0 = 0, delay0 = 0;
  cudaGraphExec_t sweep_graph[2] = {nullptr, nullptr};  // a chunk of steps starting from buffer 0 / 1
  double sweep_graph_dt[2] = {std::nan(""), std::nan("")};
  uint64_t sweep_graph_len[2] = {0, 0};
};

namespace {

using H = shaw_fom_s;

// Columns per thread: one 16-byte vector where M allows it.
uint32_t state_vec(const H* h) {
  if (h->esz == sizeof(float)) return (h->M % 4 == 0) ? 4u : (h->M % 2 == 0) ? 2u : 1u;
  return (h->M % 2 == 0) ? 2u : 1u;
}

FomArgs make_args(const H* h, double dt) {
  FomArgs a;
  std::memset(&a, 0, sizeof(a));
  a.xv = h->xv;
  a.xs = h->xs;
  a.cvp = h->cvp;
  a.csp = h->csp;
  a.rho_inv = h->rho_inv;
  a.src = h->src;
  a.kind = h->kind;
  a.period = h->period;
  a.delay = h->delay;
  a.rcv = h->rcv;
  a.seis = h->seis;
  a.ctl = h->ctl;
  a.dt = dt;
  a.nth = (uint32_t)h->nth;
  a.nr = (uint32_t)h->nr;
  a.M = h->M;
  a.chunks = h->M / state_vec(h);
  a.vp_items = (uint32_t)(h->nvp * a.chunks);
  a.sp_items = (uint32_t)(h->nsp * a.chunks);
  a.sp_row = (uint32_t)(2 * h->nth - 1);
  a.R = h->R;
  a.seis_freq = (uint32_t)h->seis_freq;
  a.seis_T = (uint32_t)h->seis_T;
  a.sp_blocks = (a.sp_items + kThreads - 1) / kThreads;
  a.rank2 = h->rank == 2 ? 1 : 0;
  a.chunks_div = shaw::make_fastdiv(a.chunks);
  a.nth_div = shaw::make_fastdiv(a.nth);
  a.sprow_div = shaw::make_fastdiv(a.sp_row);
  return a;
}

// A half-step kernel on h's stream with programmatic stream serialization.
template <typename K, typename... X>
int launch_half_step(H* h, K kern, uint32_t blocks, const FomArgs& a, X... args) {
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(kThreads);
  cfg.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SHAW_CUDA(cudaLaunchKernelEx(&cfg, kern, a, args...));
  h->launches++;
  return SHAW_OK;
}

int launch_velocity(H* h, const FomArgs& a, uint32_t k_local, unsigned long long host_step) {
  const uint32_t blocks = (a.vp_items + kThreads - 1) / kThreads;
  const uint32_t vec = h->M / a.chunks;
  if (h->esz == sizeof(float)) {
    if (vec == 4) return launch_half_step(h, fom_velocity_kernel<float, 4>, blocks, a, k_local, host_step);
    if (vec == 2) return launch_half_step(h, fom_velocity_kernel<float, 2>, blocks, a, k_local, host_step);
    return launch_half_step(h, fom_velocity_kernel<float, 1>, blocks, a, k_local, host_step);
  }
  if (vec == 2) return launch_half_step(h, fom_velocity_kernel<double, 2>, blocks, a, k_local, host_step);
  return launch_half_step(h, fom_velocity_kernel<double, 1>, blocks, a, k_local, host_step);
}

int launch_stress(H* h, const FomArgs& a, uint32_t k_local, unsigned long long host_step) {
  uint32_t blocks = a.sp_blocks;
  if (a.R && a.seis_freq) blocks += (a.R * a.M + kThreads - 1) / kThreads;
  const uint32_t vec = h->M / a.chunks;
  if (h->esz == sizeof(float)) {
    if (vec == 4) return launch_half_step(h, fom_stress_kernel<float, 4>, blocks, a, k_local, host_step);
    if (vec == 2) return launch_half_step(h, fom_stress_kernel<float, 2>, blocks, a, k_local, host_step);
    return launch_half_step(h, fom_stress_kernel<float, 1>, blocks, a, k_local, host_step);
  }
  if (vec == 2) return launch_half_step(h, fom_stress_kernel<double, 2>, blocks, a, k_local, host_step);
  return launch_half_step(h, fom_stress_kernel<double, 1>, blocks, a, k_local, host_step);
}

int ensure_folded(H* h, double dt) {
  if (h->folded_dt == dt) return SHAW_OK;
  if (h->esz == sizeof(float)) {
    fom_fold_kernel<float><<<1024, 256, 0, h->stream>>>(h->cvp_raw, (float*)h->cvp, dt, 4 * h->nvp);
    fom_fold_kernel<float><<<1024, 256, 0, h->stream>>>(h->csp_raw, (float*)h->csp, dt, 2 * h->nsp);
  } else {
    fom_fold_kernel<double><<<1024, 256, 0, h->stream>>>(h->cvp_raw, (double*)h->cvp, dt, 4 * h->nvp);
    fom_fold_kernel<double><<<1024, 256, 0, h->stream>>>(h->csp_raw, (double*)h->csp, dt, 2 * h->nsp);
  }
  h->launches += 2;
  if (h->sweep) {
    if (h->form == sweep::kF64) {
      fom_fold_aos_kernel<double><<<1024, 256, 0, h->stream>>>(h->cvp_raw, (double*)h->cv4, dt, h->nvp, 4, 0);
      fom_fold_aos_kernel<double><<<1024, 256, 0, h->stream>>>(h->csp_raw, (double*)h->cs2, dt, h->nsp, 2, 1);
    } else {
      fom_fold_aos_kernel<float><<<1024, 256, 0, h->stream>>>(h->cvp_raw, (float*)h->cv4, dt, h->nvp, 4, 0);
      fom_fold_aos_kernel<float><<<1024, 256, 0, h->stream>>>(h->csp_raw, (float*)h->cs2, dt, h->nsp, 2, 1);
    }
    h->launches += 2;
  }
  SHAW_CUDA(cudaGetLastError());
  h->folded_dt = dt;
  return SHAW_OK;
}

// ---- the single-sweep path --------------------------------------------------------------

sweep::Params sweep_params(const H* h, double dt, int from) {
  sweep::Params p;
  std::memset(&p, 0, sizeof(p));
  p.xv_new = h->xvb[from ^ 1];
  p.xs_new = h->xsb[from ^ 1];
  p.xv_old = h->xvb[from];
  p.cvp = h->cv4;
  p.csp = h->cs2;
  p.rho_inv = h->rho_inv;
  p.src = h->src;
  p.kind = h->kind;
  p.period = h->period;
  p.delay = h->delay;
  p.rcv = h->rcv;
  p.seis = h->seis;
  p.ctl = h->ctl;
  p.dt = dt;
  p.nth = (uint32_t)h->nth;
  p.nr = (uint32_t)h->nr;
  p.M = h->M;
  p.sp_row = (uint32_t)(2 * h->nth - 1);
  p.R = h->R;
  p.seis_freq = (uint32_t)h->seis_freq;
  p.seis_T = (uint32_t)h->seis_T;
  p.rank2 = h->rank == 2 ? 1 : 0;
  sweep::plan(p, h->sms, (uint32_t)h->esz);
  return p;
}

// One leapfrog step from buffer `from` into the other one.
int launch_sweep(H* h, double dt, int from, uint32_t k_local, unsigned long long host_step) {
  const sweep::Params p = sweep_params(h, dt, from);
  int rc = sweep::launch(h->form, h->tv[from], h->ts[from], p, k_local, host_step, h->stream, true);
  if (rc) return rc;
  h->launches++;
  return SHAW_OK;
}

void set_current(H* h, int cur) {
  h->cur = cur;
  h->xv = h->xvb[cur];
  h->xs = h->xsb[cur];
}

// The seismogram of the current step (the sweep records step n - 1 during step n).
int flush_gather(H* h, double dt) {
  if (!h->R || !h->seis_freq || h->step == 0) return SHAW_OK;
  const sweep::Params p = sweep_params(h, dt, h->cur);
  int rc = sweep::launch_gather(h->form, p, h->xv, h->step, h->stream);
  if (rc) return rc;
  h->launches++;
  return SHAW_OK;
}

// Graph of `len` sweep steps starting from buffer `from` (it ends on buffer from ^ (len & 1)),
// step numbers read from ctl->step_base.
int ensure_sweep_graph(H* h, double dt, int from, uint64_t len) {
  if (h->sweep_graph[from] && h->sweep_graph_dt[from] == dt && h->sweep_graph_len[from] == len) return SHAW_OK;
  if (h->sweep_graph[from]) {
    cudaGraphExecDestroy(h->sweep_graph[from]);
    h->sweep_graph[from] = nullptr;
  }
  cudaGraph_t g = nullptr;
  SHAW_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  const uint64_t before = h->launches;
  int rc = SHAW_OK;
  for (uint32_t k = 0; k < len && rc == SHAW_OK; ++k) rc = launch_sweep(h, dt, from ^ (int)(k & 1), k, 0);
  if (rc == SHAW_OK) fom_advance_base_kernel<<<1, 1, 0, h->stream>>>(h->ctl, (unsigned int)len);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  h->launches = before;
  if (rc != SHAW_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return shaw::cuda_fail(e, "cudaStreamEndCapture (sweep)");
  e = cudaGraphInstantiate(&h->sweep_graph[from], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return shaw::cuda_fail(e, "cudaGraphInstantiate (sweep)");
  h->sweep_graph_dt[from] = dt;
  h->sweep_graph_len[from] = len;
  return SHAW_OK;
}

// SHAW_FOM_SCHEDULE_AUTO: the faster schedule of the handle's precision (measured on GB300 at
// 1000 x 2000, M = 256: FP32 sweep 1.84 ms vs two-pass 2.66 ms per step; FP64 two-pass 6.73 ms
// vs the sweep 7.49 ms, both bound by the FP64 pipe).
bool auto_sweep(const H* h) { return h->sweep_ok && h->precision == SHAW_MIXED_FP32; }

void drop_graphs(H* h) {
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  for (int b = 0; b < 2; ++b)
    if (h->sweep_graph[b]) { cudaGraphExecDestroy(h->sweep_graph[b]); h->sweep_graph[b] = nullptr; }
}

// Copy the current vp (dof 0) or sp (dof 1) state into column `col` of the host snapshot
// matrix (StateObserver::observe, state_observer.hpp:175-203).  The state is transposed
// (or copied, for one FP64 column) into a staging buffer on the compute stream; the copy to
// the page-locked host matrix runs on the copy stream, overlapping the next steps.  The two
// staging buffers alternate; a buffer is refilled only after its previous copy is done.
int snapshot_copy(H* h, int dof, uint64_t col) {
  const uint64_t N = dof == 0 ? h->nvp : h->nsp;
  const uint64_t T = h->snap_nsteps / (dof == 0 ? h->snap_fvp : h->snap_fsp);
  double* host = dof == 0 ? h->host_vp : h->host_sp;
  const void* dev = dof == 0 ? h->xv : h->xs;
  const int b = h->stage_next;
  h->stage_next ^= 1;
  if (h->stage_used[b]) SHAW_CUDA(cudaStreamWaitEvent(h->stream, h->ev_free[b], 0));
  if (h->M == 1 && h->esz == sizeof(double)) {
    SHAW_CUDA(cudaMemcpyAsync(h->stage[b], dev, N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  } else {
    dim3 grid((unsigned)((N + 31) / 32), (h->M + 31) / 32);
    if (h->esz == sizeof(float))
      fom_transpose_kernel<float><<<grid, dim3(32, 8), 0, h->stream>>>((const float*)dev, h->stage[b], (uint32_t)N,
                                                                       h->M);
    else
      fom_transpose_kernel<double><<<grid, dim3(32, 8), 0, h->stream>>>((const double*)dev, h->stage[b], (uint32_t)N,
                                                                        h->M);
    h->launches++;
    SHAW_CUDA(cudaGetLastError());
  }
  SHAW_CUDA(cudaEventRecord(h->ev_ready[b], h->stream));
  SHAW_CUDA(cudaStreamWaitEvent(h->copy_stream, h->ev_ready[b], 0));
  SHAW_CUDA(cudaMemcpy2DAsync(host + N * col, N * T * sizeof(double), h->stage[b], N * sizeof(double),
                              N * sizeof(double), h->M, cudaMemcpyDeviceToHost, h->copy_stream));
  SHAW_CUDA(cudaEventRecord(h->ev_free[b], h->copy_stream));
  h->stage_used[b] = true;
  return SHAW_OK;
}

// The snapshots of step h->step that fall due.
int snapshots_due(H* h) {
  const uint64_t n = h->step;
  int rc = SHAW_OK;
  if (n % h->snap_fvp == 0) {
    if ((rc = snapshot_copy(h, 0, h->snap_cvp))) return rc;
    h->snap_cvp++;
  }
  if (n % h->snap_fsp == 0) {
    if ((rc = snapshot_copy(h, 1, h->snap_csp))) return rc;
    h->snap_csp++;
  }
  return SHAW_OK;
}

int check_ready(H* h, double dt) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (!(dt > 0.0) || !std::isfinite(dt)) return shaw::fail(SHAW_ERR_INVALID_ARG, "dt must be > 0");
  if (!h->sources_set) return shaw::fail(SHAW_ERR_STATE, "shaw_fom_set_sources must be called before stepping");
  return SHAW_OK;
}

// Build (once per dt and length) a graph of `len` steps that reads its step numbers
// from the device-side step_base and advances it at the end.
int ensure_graph(H* h, double dt, uint64_t len) {
  if (h->graph && h->graph_dt == dt && h->graph_len == len) return SHAW_OK;
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  const FomArgs a = make_args(h, dt);
  cudaGraph_t g = nullptr;
  SHAW_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  const uint64_t before = h->launches;
  int rc = SHAW_OK;
  for (uint32_t k = 0; k < len && rc == SHAW_OK; ++k) {
    rc = launch_velocity(h, a, k, 0);
    if (rc == SHAW_OK) rc = launch_stress(h, a, k, 0);
  }
  if (rc == SHAW_OK) {
    fom_advance_base_kernel<<<1, 1, 0, h->stream>>>(h->ctl, (unsigned int)len);
  }
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  h->launches = before;  // captured launches are counted when the graph is replayed
  if (rc != SHAW_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return shaw::cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&h->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return shaw::cuda_fail(e, "cudaGraphInstantiate");
  h->graph_dt = dt;
  h->graph_len = len;
  return SHAW_OK;
}

int set_step_base(H* h) {
  fom_set_base_kernel<<<1, 1, 0, h->stream>>>(h->ctl, (unsigned long long)h->step);
  h->launches++;
  SHAW_CUDA(cudaGetLastError());
  return SHAW_OK;
}

// The first vp / sp row whose graph entries differ from the structured full mesh's, or
// the row count when all match (rows checked in parallel on the host threads).
uint64_t first_bad_vp(const shaw_fom_operator_desc* d) {
  const uint64_t nth = d->nth, nr = d->nr, row = 2 * nth - 1;
  auto srp = [&](uint64_t j, uint64_t i) { return j * row + 2 * i; };
  auto stp = [&](uint64_t j, uint64_t i) { return (j + 1 < nr) ? j * row + 2 * i + 1 : j * row + i; };
  uint64_t bad = d->nvp;
#pragma omp parallel for reduction(min : bad) schedule(static)
  for (int64_t pp = 0; pp < (int64_t)d->nvp; ++pp) {
    const uint64_t p = (uint64_t)pp, j = p / nth, i = p % nth;
    const int64_t* g = d->graph_vp + p * 5;
    const int64_t eW = (i >= 1) ? (int64_t)stp(j, i - 1) : (int64_t)stp(j, i);
    const int64_t eE = (i + 1 < nth) ? (int64_t)stp(j, i) : (int64_t)stp(j, i - 1);
    const int64_t eN = (j + 1 < nr) ? (int64_t)srp(j, i) : (int64_t)srp(j - 1, i);
    const int64_t eS = (j >= 1) ? (int64_t)srp(j - 1, i) : (int64_t)srp(j, i);
    if (g[0] != (int64_t)p || g[1] != eW || g[2] != eN || g[3] != eE || g[4] != eS) bad = std::min(bad, p);
  }
  return bad;
}

uint64_t first_bad_sp(const shaw_fom_operator_desc* d) {
  const uint64_t nth = d->nth, nr = d->nr, row = 2 * nth - 1;
  uint64_t bad = d->nsp;
#pragma omp parallel for reduction(min : bad) schedule(static)
  for (int64_t qq = 0; qq < (int64_t)d->nsp; ++qq) {
    const uint64_t q = (uint64_t)qq, j = q / row, rem = q % row;
    const int64_t* g = d->graph_sp + q * 3;
    int64_t eA, eB;
    int lab;
    if (j + 1 < nr && rem % 2 == 0) {
      const uint64_t i = rem / 2;
      lab = 1; eA = (int64_t)((j + 1) * nth + i); eB = (int64_t)(j * nth + i);
    } else {
      const uint64_t i = (j + 1 < nr) ? rem / 2 : rem;
      lab = 2; eA = (int64_t)(j * nth + i); eB = eA + 1;
    }
    if (g[0] != (int64_t)q || g[1] != eA || g[2] != eB || d->labels_sp[q] != lab) bad = std::min(bad, q);
  }
  return bad;
}

bool valid_structured_mesh(const shaw_fom_operator_desc* d, std::string& why) {
  const uint64_t nth = d->nth, nr = d->nr;
  if (nth < 2 || nr < 2) { why = "nth and nr must be >= 2"; return false; }
  if (d->nvp != nth * nr) { why = "numPtsVp != nth*nr"; return false; }
  if (d->nsp != (nr - 1) * nth + nr * (nth - 1)) { why = "numPtsSp != (nr-1)*nth + nr*(nth-1)"; return false; }
  if (d->nvp * 4 >= (1ull << 32) || d->nsp * 2 >= (1ull << 32)) { why = "mesh too large for 32-bit indexing"; return false; }
  const uint64_t bv = first_bad_vp(d);
  if (bv != d->nvp) {
    why = "graph_vp row " + std::to_string(bv) + " does not match the structured full mesh";
    return false;
  }
  const uint64_t bs = first_bad_sp(d);
  if (bs != d->nsp) {
    why = "graph_sp row " + std::to_string(bs) + " does not match the structured full mesh";
    return false;
  }
  return true;
}

}  // namespace

extern "C" {

int shaw_fom_create(const shaw_fom_operator_desc* d, int rank, uint32_t M, int precision, shaw_fom_t* out) {
  if (!d || !out) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (M == 0) return shaw::fail(SHAW_ERR_INVALID_ARG, "num_forcings must be >= 1");
  if (rank != 1 && rank != 2) return shaw::fail(SHAW_ERR_INVALID_ARG, "rank must be 1 or 2");
  if (rank == 1 && M != 1) return shaw::fail(SHAW_ERR_INVALID_ARG, "the rank-1 form has exactly one forcing");
  if (precision != SHAW_FP64 && precision != SHAW_MIXED_FP32)
    return shaw::fail(SHAW_ERR_UNSUPPORTED, "FOM precision must be SHAW_FP64 or SHAW_MIXED_FP32");
  if (!d->graph_vp || !d->graph_sp || !d->labels_sp || !d->coords_vp || !d->coords_sp || !d->cot_vp ||
      !d->cot_sp || !d->coeff_vp || !d->rho_inv_vp || !d->shear_mod_sp)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "operator descriptor has a null array");
  std::string why;
  if (!valid_structured_mesh(d, why)) return shaw::fail(SHAW_ERR_MESH, why);
  if ((uint64_t)d->nsp * M >= (1ull << 32) || (uint64_t)d->nvp * M >= (1ull << 32))
    return shaw::fail(SHAW_ERR_UNSUPPORTED, "mesh points x forcings must stay below 2^32");

  // Stencil values in the reference's expression order (shwavepp.hpp:361-364, 441-454).
  const uint64_t nvp = d->nvp, nsp = d->nsp;
  // every entry is written below (in parallel, which also spreads the first touch)
  std::unique_ptr<double[]> cv(new double[4 * nvp]), cs(new double[2 * nsp]);
  const double three = 3.0, oneHalf = 1.0 / 2.0;
#pragma omp parallel for schedule(static)
  for (int64_t pp = 0; pp < (int64_t)nvp; ++pp) {
    const uint64_t p = (uint64_t)pp;
    const int64_t* g = d->graph_vp + p * 5;
    const double rInv = d->coords_vp[p * 2 + 1];
    const double cot = d->cot_vp[p];
    const double rhoInv = d->rho_inv_vp[p];
    const double* c = d->coeff_vp + p * 4;
    const double cW = (-rInv * d->dth_inv + rInv * cot) * c[0] * rhoInv;
    const double cN = (d->drr_inv + three * oneHalf * rInv) * c[1] * rhoInv;
    const double cE = (rInv * d->dth_inv + rInv * cot) * c[2] * rhoInv;
    const double cS = (-d->drr_inv + three * oneHalf * rInv) * c[3] * rhoInv;
    if (g[2] == g[4]) { cv[p] = cN + cS; cv[nvp + p] = 0.0; }
    else { cv[p] = cN; cv[nvp + p] = cS; }
    if (g[1] == g[3]) { cv[2 * nvp + p] = cW + cE; cv[3 * nvp + p] = 0.0; }
    else { cv[2 * nvp + p] = cW; cv[3 * nvp + p] = cE; }
  }
#pragma omp parallel for schedule(static)
  for (int64_t qq = 0; qq < (int64_t)nsp; ++qq) {
    const uint64_t q = (uint64_t)qq;
    const double rInv = d->coords_sp[q * 2 + 1];
    const double G = d->shear_mod_sp[q];
    if (d->labels_sp[q] == 1) {
      cs[q] = (d->drr_inv - rInv * oneHalf) * G;
      cs[nsp + q] = (-d->drr_inv - rInv * oneHalf) * G;
    } else {
      cs[q] = (-d->dth_inv - oneHalf * d->cot_sp[q]) * rInv * G;
      cs[nsp + q] = (d->dth_inv - oneHalf * d->cot_sp[q]) * rInv * G;
    }
  }

  H* h = new H();
  h->nth = d->nth; h->nr = d->nr; h->nvp = nvp; h->nsp = nsp; h->M = M; h->rank = rank;
  h->precision = precision;
  h->esz = precision == SHAW_MIXED_FP32 ? sizeof(float) : sizeof(double);
  auto bail = [&](int rc) { shaw_fom_destroy(h); return rc; };
  cudaError_t e;
#define SHAW_TRY(call) do { e = (call); if (e != cudaSuccess) return bail(shaw::cuda_fail(e, #call)); } while (0)
  SHAW_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  SHAW_TRY(cudaMalloc(&h->xv, nvp * M * h->esz));
  SHAW_TRY(cudaMalloc(&h->xs, nsp * M * h->esz));
  SHAW_TRY(cudaMalloc(&h->cvp_raw, 4 * nvp * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->csp_raw, 2 * nsp * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->cvp, 4 * nvp * h->esz));
  SHAW_TRY(cudaMalloc(&h->csp, 2 * nsp * h->esz));
  SHAW_TRY(cudaMalloc(&h->rho_inv, nvp * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->src, M * sizeof(unsigned long long)));
  SHAW_TRY(cudaMalloc(&h->kind, M * sizeof(int)));
  SHAW_TRY(cudaMalloc(&h->period, M * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->delay, M * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->ctl, sizeof(FomCtl)));
  SHAW_TRY(cudaMemcpyAsync(h->cvp_raw, cv.get(), 4 * nvp * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SHAW_TRY(cudaMemcpyAsync(h->csp_raw, cs.get(), 2 * nsp * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SHAW_TRY(cudaMemcpyAsync(h->rho_inv, d->rho_inv_vp, nvp * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SHAW_TRY(cudaMemsetAsync(h->ctl, 0, sizeof(FomCtl), h->stream));
  SHAW_TRY(cudaMemsetAsync(h->xv, 0, nvp * M * h->esz, h->stream));
  SHAW_TRY(cudaMemsetAsync(h->xs, 0, nsp * M * h->esz, h->stream));
  // the single sweep: every column block of 32 forcings is a tile column
  h->xvb[0] = h->xv;
  h->xsb[0] = h->xs;
  if (M % sweep::kTM == 0) {
    int dev = 0;
    SHAW_TRY(cudaGetDevice(&dev));
    SHAW_TRY(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, dev));
    SHAW_TRY(cudaMalloc(&h->xvb[1], nvp * M * h->esz));
    SHAW_TRY(cudaMalloc(&h->xsb[1], nsp * M * h->esz));
    SHAW_TRY(cudaMemsetAsync(h->xvb[1], 0, nvp * M * h->esz, h->stream));
    SHAW_TRY(cudaMemsetAsync(h->xsb[1], 0, nsp * M * h->esz, h->stream));
    h->form = precision == SHAW_MIXED_FP32 ? sweep::kF32 : sweep::kF64;
    const size_t cv_bytes = (nvp + sweep::kCoefPadV) * 4 * h->esz, cs_bytes = (1 + nsp + sweep::kCoefPadS) * 2 * h->esz;
    SHAW_TRY(cudaMalloc(&h->cv4, cv_bytes));
    SHAW_TRY(cudaMalloc(&h->cs2, cs_bytes));
    SHAW_TRY(cudaMemsetAsync(h->cv4, 0, cv_bytes, h->stream));
    SHAW_TRY(cudaMemsetAsync(h->cs2, 0, cs_bytes, h->stream));
    for (int b = 0; b < 2; ++b) {
      int rc = sweep::encode_map(&h->tv[b], h->xvb[b], nvp, M, (uint32_t)h->esz, sweep::kRowsV);
      if (rc == SHAW_OK) rc = sweep::encode_map(&h->ts[b], h->xsb[b], nsp, M, (uint32_t)h->esz, sweep::kRowsS);
      if (rc) return bail(rc);
    }
    h->sweep_ok = true;
    h->sweep = auto_sweep(h);
  }
  if (rank == 1 && precision == SHAW_FP64)
    h->band_ok = h->use_band = shaw::band::plan((uint32_t)h->nth, (uint32_t)h->nr, &h->band_n, &h->band_rows,
                                                &h->band_cols, &h->band_smem);
  SHAW_TRY(cudaStreamSynchronize(h->stream));
#undef SHAW_TRY
  *out = h;
  return SHAW_OK;
}

void shaw_fom_destroy(shaw_fom_t h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
  drop_graphs(h);
  if (h->host_vp) cudaHostUnregister(h->host_vp);
  if (h->host_sp) cudaHostUnregister(h->host_sp);
  if (!h->xvb[0]) { h->xvb[0] = h->xv; h->xsb[0] = h->xs; }
  void* bufs[] = {h->xvb[0], h->xsb[0], h->xvb[1], h->xsb[1], h->cvp_raw, h->csp_raw, h->cvp, h->csp,
                  h->cv4, h->cs2, h->ftab, h->xwords, h->rcv_sorted, h->rho_inv, h->src, h->kind, h->period, h->delay, h->rcv, h->seis,
                  h->stage[0], h->stage[1], h->ctl};
  for (void* b : bufs)
    if (b) cudaFree(b);
  for (int b = 0; b < 2; ++b) {
    if (h->ev_ready[b]) cudaEventDestroy(h->ev_ready[b]);
    if (h->ev_free[b]) cudaEventDestroy(h->ev_free[b]);
  }
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int shaw_fom_set_sources(shaw_fom_t h, const uint64_t* gid, const int32_t* kind, const double* period,
                         const double* delay) {
  if (!h || !gid || !kind || !period || !delay) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  for (uint32_t m = 0; m < h->M; ++m) {
    if (gid[m] >= h->nvp) return shaw::fail(SHAW_ERR_INVALID_ARG, "source gid out of range");
    if (kind[m] < SHAW_SIGNAL_RICKER || kind[m] > SHAW_SIGNAL_GAUSS_DER)
      return shaw::fail(SHAW_ERR_INVALID_ARG, "unknown signal kind");
    if (!(period[m] > 0.0)) return shaw::fail(SHAW_ERR_INVALID_ARG, "Period for signal must be positive.");
    if (!(delay[m] >= 0.0)) return shaw::fail(SHAW_ERR_INVALID_ARG, "Delay time of the signal must be >=0");
  }
  static_assert(sizeof(unsigned long long) == sizeof(uint64_t), "gid width");
  SHAW_CUDA(cudaMemcpyAsync(h->src, gid, h->M * sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream));
  SHAW_CUDA(cudaMemcpyAsync(h->kind, kind, h->M * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  SHAW_CUDA(cudaMemcpyAsync(h->period, period, h->M * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SHAW_CUDA(cudaMemcpyAsync(h->delay, delay, h->M * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  h->src0 = gid[0];
  h->kind0 = kind[0];
  h->period0 = period[0];
  h->delay0 = delay[0];
  h->sources_set = true;
  return SHAW_OK;
}

int shaw_fom_set_receivers(shaw_fom_t h, const uint64_t* gid, uint32_t R, uint64_t freq, uint64_t nsteps) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  if (h->rcv) { cudaFree(h->rcv); h->rcv = nullptr; }
  if (h->rcv_sorted) { cudaFree(h->rcv_sorted); h->rcv_sorted = nullptr; }
  if (h->seis) { cudaFree(h->seis); h->seis = nullptr; }
  h->R = 0; h->seis_freq = 0; h->seis_T = 0; h->seis_nsteps = 0;
  drop_graphs(h);
  if (R == 0) return SHAW_OK;
  if (!gid) return shaw::fail(SHAW_ERR_INVALID_ARG, "null receiver gids");
  if (freq == 0) return shaw::fail(SHAW_ERR_INVALID_ARG, "cannot have seismoFreq <=0 ");
  if (nsteps % freq != 0)
    return shaw::fail(SHAW_ERR_FREQ_DIVISOR, "Seismogram sampling frequency not a divisor of steps");
  for (uint32_t r = 0; r < R; ++r)
    if (gid[r] >= h->nvp) return shaw::fail(SHAW_ERR_INVALID_ARG, "receiver gid out of range");
  const uint64_t T = nsteps / freq;
  if ((uint64_t)R * h->M >= (1ull << 31) || T >= (1ull << 32))
    return shaw::fail(SHAW_ERR_UNSUPPORTED, "seismogram too large");
  SHAW_CUDA(cudaMalloc(&h->rcv, R * sizeof(unsigned long long)));
  SHAW_CUDA(cudaMalloc(&h->seis, (size_t)R * T * h->M * sizeof(double)));
  SHAW_CUDA(cudaMemcpyAsync(h->rcv, gid, R * sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream));
  if (h->band_ok) {  // (key, receiver) pairs in key order: each band reads a contiguous range
    // key: the gid (row-major) for row bands, i nr + j (column-major) for column bands
    auto key = [&](uint64_t g) -> unsigned long long {
      return h->band_cols ? (unsigned long long)(g % h->nth) * h->nr + g / h->nth : (unsigned long long)g;
    };
    std::vector<unsigned long long> pairs(2 * (size_t)R);
    std::vector<uint32_t> order(R);
    for (uint32_t r = 0; r < R; ++r) order[r] = r;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return key(gid[x]) < key(gid[y]); });
    for (uint32_t q = 0; q < R; ++q) {
      pairs[2 * (size_t)q] = key(gid[order[q]]);
      pairs[2 * (size_t)q + 1] = order[q];
    }
    SHAW_CUDA(cudaMalloc(&h->rcv_sorted, 2 * (size_t)R * sizeof(unsigned long long)));
    SHAW_CUDA(cudaMemcpyAsync(h->rcv_sorted, pairs.data(), 2 * (size_t)R * sizeof(unsigned long long),
                              cudaMemcpyHostToDevice, h->stream));
    SHAW_CUDA(cudaStreamSynchronize(h->stream));
  }
  SHAW_CUDA(cudaMemsetAsync(h->seis, 0, (size_t)R * T * h->M * sizeof(double), h->stream));
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  h->R = R; h->seis_freq = freq; h->seis_T = T; h->seis_nsteps = nsteps;
  return SHAW_OK;
}

int shaw_fom_set_snapshots(shaw_fom_t h, uint64_t fvp, uint64_t fsp, uint64_t nsteps, double* host_vp,
                           double* host_sp) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  if (h->copy_stream) SHAW_CUDA(cudaStreamSynchronize(h->copy_stream));
  if (h->host_vp) cudaHostUnregister(h->host_vp);
  if (h->host_sp) cudaHostUnregister(h->host_sp);
  h->host_vp = h->host_sp = nullptr;
  h->snap_fvp = h->snap_fsp = h->snap_nsteps = 0;
  if (fvp == 0 && fsp == 0) return SHAW_OK;
  if (fvp == 0 || fsp == 0 || !host_vp || !host_sp)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "snapshot frequencies and arrays are required for both dofs");
  if (nsteps % fvp != 0) return shaw::fail(SHAW_ERR_FREQ_DIVISOR, "Snapshot Vp frequency not a divisor of steps");
  if (nsteps % fsp != 0) return shaw::fail(SHAW_ERR_FREQ_DIVISOR, "Snapshot Sp frequency not a divisor of steps");
  const size_t bvp = h->nvp * (nsteps / fvp) * h->M * sizeof(double);
  const size_t bsp = h->nsp * (nsteps / fsp) * h->M * sizeof(double);
  SHAW_CUDA(cudaHostRegister(host_vp, bvp, cudaHostRegisterDefault));
  cudaError_t e = cudaHostRegister(host_sp, bsp, cudaHostRegisterDefault);
  if (e != cudaSuccess) {
    cudaHostUnregister(host_vp);
    return shaw::cuda_fail(e, "cudaHostRegister(host_sp)");
  }
  if (!h->copy_stream) {
    e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking);
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
      e = cudaEventCreateWithFlags(&h->ev_ready[b], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_free[b], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
      cudaHostUnregister(host_vp);
      cudaHostUnregister(host_sp);
      return shaw::cuda_fail(e, "snapshot copy stream / events");
    }
  }
  for (int b = 0; b < 2; ++b) {
    if (h->stage[b]) continue;
    e = cudaMalloc(&h->stage[b], std::max(h->nvp, h->nsp) * h->M * sizeof(double));
    if (e != cudaSuccess) {
      cudaHostUnregister(host_vp);
      cudaHostUnregister(host_sp);
      return shaw::cuda_fail(e, "cudaMalloc(snapshot staging)");
    }
  }
  h->stage_used[0] = h->stage_used[1] = false;
  h->stage_next = 0;
  h->host_vp = host_vp; h->host_sp = host_sp;
  h->snap_fvp = fvp; h->snap_fsp = fsp; h->snap_nsteps = nsteps;
  return SHAW_OK;
}

int shaw_fom_reset(shaw_fom_t h) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaMemsetAsync(h->xv, 0, h->nvp * h->M * h->esz, h->stream));
  SHAW_CUDA(cudaMemsetAsync(h->xs, 0, h->nsp * h->M * h->esz, h->stream));
  SHAW_CUDA(cudaMemsetAsync(h->ctl, 0, sizeof(FomCtl), h->stream));
  if (h->seis)
    SHAW_CUDA(cudaMemsetAsync(h->seis, 0, (size_t)h->R * h->seis_T * h->M * sizeof(double), h->stream));
  h->step = 0;
  h->snap_cvp = h->snap_csp = 0;
  return SHAW_OK;
}

int shaw_fom_advance(shaw_fom_t h, double dt, uint64_t nsteps) {
  int rc = check_ready(h, dt);
  if (rc) return rc;
  if (h->seis_freq && h->step + nsteps > h->seis_nsteps)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "advancing past the step count the seismogram was sized for");
  if (h->snap_fvp && h->step + nsteps > h->snap_nsteps)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "advancing past the step count the snapshots were sized for");
  if ((rc = ensure_folded(h, dt))) return rc;
  if (h->use_band && h->snap_fvp == 0 && nsteps > 0) {
    // all the steps of this call in one persistent launch of row bands
    shaw::band::Args c;
    std::memset(&c, 0, sizeof(c));
    c.cvp = static_cast<const double*>(h->cvp);
    c.csp = static_cast<const double*>(h->csp);
    c.xv = static_cast<double*>(h->xv);
    c.xs = static_cast<double*>(h->xs);
    c.rho_inv = h->rho_inv;
    c.src = h->src0;
    c.kind = h->kind0;
    c.period = h->period0;
    c.delay = h->delay0;
    c.dt = dt;
    c.rcv_sorted = h->rcv_sorted;
    c.seis = h->seis;
    c.ctl = h->ctl;
    c.nth = (uint32_t)h->nth;
    c.nr = (uint32_t)h->nr;
    c.rows = h->band_rows;
    c.cols = h->band_cols;
    c.R = h->R;
    c.seis_freq = (uint32_t)h->seis_freq;
    c.seis_T = (uint32_t)h->seis_T;
    const uint32_t L = h->band_cols ? (uint32_t)h->nr : (uint32_t)h->nth;  // points of a band's edge line
    const size_t dw = shaw::band::down_words(h->band_n, L);
    const size_t words = dw + shaw::band::up_words(h->band_n, L);
    if (!h->ftab) {
      SHAW_CUDA(cudaMalloc(&h->ftab, kBandSteps * sizeof(double)));
      SHAW_CUDA(cudaMalloc(&h->xwords, words * sizeof(unsigned long long)));
      SHAW_CUDA(cudaMemsetAsync(h->xwords, 0, words * sizeof(unsigned long long), h->stream));
      h->band_tag = 0;
    }
    c.ftab = h->ftab;
    c.xdown = h->xwords;
    c.xup = h->xwords + dw;
    // launches of at most kBandSteps steps, each filling the forcing table it reads
    for (uint64_t done = 0; done < nsteps;) {
      c.step0 = h->step;
      c.nsteps = std::min<uint64_t>(kBandSteps, nsteps - done);
      if ((uint64_t)h->band_tag + c.nsteps >= 0xffffffffull) {  // tags would wrap: clear the words
        SHAW_CUDA(cudaMemsetAsync(h->xwords, 0, words * sizeof(unsigned long long), h->stream));
        h->band_tag = 0;
      }
      c.tag0 = h->band_tag + 1;
      if ((rc = shaw::band::launch(c, h->band_n, h->band_smem, h->stream))) return rc;
      h->band_tag += (uint32_t)c.nsteps;
      h->launches += 2;
      h->step += c.nsteps;
      done += c.nsteps;
    }
    return SHAW_OK;
  }
  // Steps run as replays of a captured chunk (64 steps; with snapshots, the steps between
  // two sample steps, so that every chunk ends on one) and single launches before and after.
  // The snapshots of a sample step are taken right after it (both half-steps done: the
  // velocity of step n is not changed by its stress half-step).
  const bool snaps = h->snap_fvp != 0;
  const uint64_t len = snaps ? std::gcd(h->snap_fvp, h->snap_fsp) : kGraphChunk;
  const bool graphs = len >= 4 && len <= 4096;
  bool base_valid = false;  // ctl->step_base == h->step
  const FomArgs a = make_args(h, dt);
  uint64_t done = 0;
  while (done < nsteps) {
    if (graphs && nsteps - done >= len && (!snaps || h->step % len == 0)) {
      if (h->sweep) {
        if ((rc = ensure_sweep_graph(h, dt, h->cur, len))) return rc;
      } else if ((rc = ensure_graph(h, dt, len))) {
        return rc;
      }
      if (!base_valid) {
        if ((rc = set_step_base(h))) return rc;
        base_valid = true;
      }
      if (h->sweep) {
        SHAW_CUDA(cudaGraphLaunch(h->sweep_graph[h->cur], h->stream));
        h->launches += len + 1;
        set_current(h, h->cur ^ (int)(len & 1));
      } else {
        SHAW_CUDA(cudaGraphLaunch(h->graph, h->stream));
        h->launches += 2 * len + 1;
      }
      done += len;
      h->step += len;
    } else {
      const unsigned long long n = h->step + 1;
      if (h->sweep) {
        if ((rc = launch_sweep(h, dt, h->cur, 0, n))) return rc;
        set_current(h, h->cur ^ 1);
      } else {
        if ((rc = launch_velocity(h, a, 0, n))) return rc;
        if ((rc = launch_stress(h, a, 0, n))) return rc;
      }
      ++done;
      ++h->step;
      base_valid = false;
    }
    if (snaps && (rc = snapshots_due(h))) return rc;
  }
  return h->sweep ? flush_gather(h, dt) : SHAW_OK;
}

int shaw_fom_synchronize(shaw_fom_t h) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  if (h->copy_stream) SHAW_CUDA(cudaStreamSynchronize(h->copy_stream));
  FomCtl c;
  SHAW_CUDA(cudaMemcpy(&c, h->ctl, sizeof(c), cudaMemcpyDeviceToHost));
  if (c.error & 1u)
    return shaw::fail(SHAW_ERR_CUDA,
                      "a bounded wait of a persistent FOM kernel ran out (a tile copy or a neighbour's row never "
                      "arrived)");
  if (c.nonfinite) return shaw::fail(SHAW_ERR_NONFINITE, "NaN/Inf in a sampled velocity (seismogram)");
  return SHAW_OK;
}

int shaw_fom_run(shaw_fom_t h, double dt, uint64_t nsteps) {
  int rc = check_ready(h, dt);
  if (rc) return rc;
  if (h->seis_freq && nsteps != h->seis_nsteps)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "nsteps differs from the seismogram's step count");
  if (h->snap_fvp && nsteps != h->snap_nsteps)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "nsteps differs from the snapshots' step count");
  if ((rc = shaw_fom_reset(h))) return rc;
  if ((rc = shaw_fom_advance(h, dt, nsteps))) return rc;
  return shaw_fom_synchronize(h);
}

int shaw_fom_update_velocity(shaw_fom_t h, double dt, uint64_t step) {
  int rc = check_ready(h, dt);
  if (rc) return rc;
  if (step == 0) return shaw::fail(SHAW_ERR_INVALID_ARG, "steps are 1-based");
  if ((rc = ensure_folded(h, dt))) return rc;
  const FomArgs a = make_args(h, dt);
  return launch_velocity(h, a, 0, step);
}

int shaw_fom_update_stress(shaw_fom_t h, double dt) {
  int rc = check_ready(h, dt);
  if (rc) return rc;
  if ((rc = ensure_folded(h, dt))) return rc;
  FomArgs a = make_args(h, dt);
  a.seis_freq = 0;  // a bare half-step records no seismogram
  return launch_stress(h, a, 0, 1);
}

int shaw_fom_get_seismogram(shaw_fom_t h, double* out) {
  if (!h || !out) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  if (!h->seis) return shaw::fail(SHAW_ERR_STATE, "no receivers set");
  SHAW_CUDA(cudaMemcpyAsync(out, h->seis, (size_t)h->R * h->seis_T * h->M * sizeof(double),
                            cudaMemcpyDeviceToHost, h->stream));
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  return SHAW_OK;
}

}  // extern "C"

namespace {

// host LayoutLeft FP64 [N x M] <-> device row-major [N][M] in the state's precision
// (FP32 states are written rounded to nearest and read back exactly).
template <typename T>
int copy_state_t(shaw_fom_t h, double* host, const double* chost, uint64_t N, void* dev, bool to_host) {
  std::vector<T> tmp(N * h->M);
  const uint32_t M = h->M;
  if (to_host) {
    SHAW_CUDA(cudaMemcpyAsync(tmp.data(), dev, tmp.size() * sizeof(T), cudaMemcpyDeviceToHost, h->stream));
    SHAW_CUDA(cudaStreamSynchronize(h->stream));
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < (int64_t)N; ++n)
      for (uint32_t m = 0; m < M; ++m) host[n + N * m] = (double)tmp[n * M + m];
  } else {
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < (int64_t)N; ++n)
      for (uint32_t m = 0; m < M; ++m) tmp[n * M + m] = (T)chost[n + N * m];
    SHAW_CUDA(cudaMemcpyAsync(dev, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
    SHAW_CUDA(cudaStreamSynchronize(h->stream));
  }
  return SHAW_OK;
}

int copy_state(shaw_fom_t h, double* host, const double* chost, uint64_t N, void* dev, bool to_host) {
  if (h->esz == sizeof(float)) return copy_state_t<float>(h, host, chost, N, dev, to_host);
  if (h->M == 1) {
    if (to_host) SHAW_CUDA(cudaMemcpyAsync(host, dev, N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    else SHAW_CUDA(cudaMemcpyAsync(dev, chost, N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    SHAW_CUDA(cudaStreamSynchronize(h->stream));
    return SHAW_OK;
  }
  return copy_state_t<double>(h, host, chost, N, dev, to_host);
}

}  // namespace

extern "C" {

int shaw_fom_get_state(shaw_fom_t h, double* vp, double* sp) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  int rc = SHAW_OK;
  if (vp && (rc = copy_state(h, vp, nullptr, h->nvp, h->xv, true))) return rc;
  if (sp && (rc = copy_state(h, sp, nullptr, h->nsp, h->xs, true))) return rc;
  return SHAW_OK;
}

int shaw_fom_set_state(shaw_fom_t h, const double* vp, const double* sp) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  int rc = SHAW_OK;
  if (vp && (rc = copy_state(h, nullptr, vp, h->nvp, h->xv, false))) return rc;
  if (sp && (rc = copy_state(h, nullptr, sp, h->nsp, h->xs, false))) return rc;
  return SHAW_OK;
}

int shaw_fom_set_schedule(shaw_fom_t h, int schedule) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (schedule < SHAW_FOM_SCHEDULE_AUTO || schedule > SHAW_FOM_SCHEDULE_PERSISTENT)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "unknown FOM schedule");
  if (schedule == SHAW_FOM_SCHEDULE_SWEEP && !h->sweep_ok)
    return shaw::fail(SHAW_ERR_UNSUPPORTED, "the single sweep needs a multiple of 32 forcing columns");
  if (schedule == SHAW_FOM_SCHEDULE_PERSISTENT && !h->band_ok)
    return shaw::fail(SHAW_ERR_UNSUPPORTED,
                      "the persistent schedule needs a rank-1 FP64 handle on a grid of at least two r rows "
                      "whose row bands (one per SM) fit a CTA");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  drop_graphs(h);
  h->folded_dt = std::nan("");  // fold the stencil values of the new form on the next step
  h->sweep = schedule == SHAW_FOM_SCHEDULE_AUTO ? auto_sweep(h) : schedule == SHAW_FOM_SCHEDULE_SWEEP;
  h->use_band = schedule == SHAW_FOM_SCHEDULE_AUTO ? h->band_ok : schedule == SHAW_FOM_SCHEDULE_PERSISTENT;
  return SHAW_OK;
}

void* shaw_fom_stream(shaw_fom_t h) { return h ? (void*)h->stream : nullptr; }
uint64_t shaw_fom_kernel_launches(shaw_fom_t h) { return h ? h->launches : 0; }

}  // extern "C"

namespace shaw {

// Column-major multivector products with the FOM operators (no dt, no forcing):
// dof 0: y = (Jvp x)[row0 : row0+nrows, :] with x nsp x ncols;
// dof 1: y = (Jsp x)[row0 : row0+nrows, :] with x nvp x ncols; y is nrows x ncols.
// The handle is only read (its stencil values are immutable after shaw_fom_create),
// so a caller may run this on its own stream while another thread steps the FOM.
int fom_apply(shaw_fom_t h, int dof, const double* x, double* y, uint64_t row0, uint64_t nrows, uint32_t ncols,
              cudaStream_t s) {
  if (!h || !x || !y) return fail(SHAW_ERR_INVALID_ARG, "null argument");
  if (ncols == 0 || nrows == 0) return SHAW_OK;
  if (ncols > 65535) return fail(SHAW_ERR_UNSUPPORTED, "at most 65535 columns per operator product");
  const uint64_t rows = dof == 0 ? h->nvp : h->nsp;
  if (row0 > rows || nrows > rows - row0) return fail(SHAW_ERR_INVALID_ARG, "row range outside the operator");
  dim3 grid((unsigned)((nrows + 255) / 256), ncols);
  if (dof == 0)
    fom_apply_vp_kernel<<<grid, 256, 0, s>>>(h->cvp_raw, x, y, (uint32_t)h->nth, (uint32_t)h->nr, h->nsp,
                                             (uint32_t)row0, (uint32_t)nrows);
  else
    fom_apply_sp_kernel<<<grid, 256, 0, s>>>(h->csp_raw, x, y, (uint32_t)h->nth, (uint32_t)h->nr, h->nsp,
                                             (uint32_t)row0, (uint32_t)nrows);
  SHAW_CUDA(cudaGetLastError());
  return SHAW_OK;
}

void fom_sizes(shaw_fom_t h, uint64_t* nvp, uint64_t* nsp) {
  *nvp = h->nvp;
  *nsp = h->nsp;
}

}  // namespace shaw
