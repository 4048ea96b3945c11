// rom.cu -- Galerkin ROM leapfrog on the reduced operators, for sm_103a.
//
// Reference: runRomRankOneForcing (src/kokkos/rom_run_rank_one.hpp:112-151) and the
// rank-2 form runRomRankTwoForcing (src/kokkos/torevise/run_rom_rank_two_forcing.hpp:149-188):
//   xv += dt * Av xs ;  xv[:,j] += (f_j(t_{n-1}) * dt) * b[:,j] ;  xs += dt * As xv
// with Av = PhiVp^T Jvp PhiSp (kv x ks), As = PhiSp^T Jsp PhiVp (ks x kv).
//
// Rank 1 (one forcing) is 2 x 20000 dependent GEMVs on a few hundred modes: latency
// bound.  It runs as ONE persistent launch on a thread-block cluster: each CTA
// keeps its slice of operator rows in shared memory and a full copy of both
// reduced states; after each half-step every CTA pushes its new rows into all
// CTAs' copies of the next state with asynchronous distributed-shared-memory stores
// that complete on the receiving CTA's mbarrier (st.async ... complete_tx), and each
// CTA waits (bounded) on its own mbarrier for the full vector.  Two arithmetics:
//   SHAW_FP64        FP64 products and state (the oracle-parity path);
//   SHAW_MIXED_FP32  "double-float": operators and states split into FP32 hi+lo,
//                    error-free products (FMA) with compensated FP32 sums
//                    (Ogita-Rump-Oishi Dot2) and a compensated (Kahan-style)
//                    state update, so every flop runs on the FP32 pipe.
// Rank 2 (M forcings) in FP64 is two cuBLAS DGEMMs per step plus a fused forcing
// kernel that evaluates the M signals on the device.
#include <cooperative_groups.h>
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "l2_exchange.cuh"
#include "rom_oz.h"
#include "rom_tc.h"
#include "shaw_internal.h"

namespace cg = cooperative_groups;

namespace {

constexpr int kRomThreads = 256;
// rank-1 cluster kernel: 16 warps, so that at k = 256 over 16 CTAs every warp owns one
// velocity row and one stress row (no serial rows per warp on the latency-bound path)
constexpr int kR1Threads = 512;
constexpr int kR1Warps = kR1Threads / 32;
constexpr uint64_t kR1MaxSteps = 1 << 16;  // leapfrog steps per rank-1 launch

// ---- double-float (hi + lo FP32) arithmetic ------------------------------------
struct df {
  float h, l;
};

__device__ __forceinline__ df df_split(double x) {
  df r;
  r.h = (float)x;
  r.l = (float)(x - (double)r.h);
  return r;
}
__device__ __forceinline__ double df_val(df a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float z = s - a;
  return {s, (a - (s - z)) + (b - z)};
}
__device__ __forceinline__ df df_norm(float s, float c) { return two_sum(s, c); }
// a + b in double-float
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.h, b.h);
  s.l += a.l + b.l;
  return df_norm(s.h, s.l);
}
// a * b in double-float (error-free product of the hi parts + cross terms)
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return df_norm(p, e);
}
// accumulate a*x into (s, c): Dot2 with cross terms
__device__ __forceinline__ void df_dot_acc(float& s, float& c, df a, df x) {
  const float p = a.h * x.h;
  const float e = fmaf(a.h, x.h, -p);
  const df t = two_sum(s, p);
  s = t.h;
  c += t.l + e;
  c = fmaf(a.h, x.l, c);
  c = fmaf(a.l, x.h, c);
}

struct RomArgs {
  const double* Av;   // kv x ks row-major
  const double* As;   // ks x kv row-major
  const double* b;    // kv (rank-1 forcing vector)
  double* xv;         // kv  (initial state in, final state out)
  double* xs;         // ks
  const void* fdt_t;  // [nsteps]: f(t_{n-1}) * dt of the launch's steps, as the kernel's element type
  double dt;
  uint32_t kv, ks, rows_v, rows_s;  // rows per CTA
  unsigned long long step0, nsteps;
  uint32_t fvp, fsp;
  double* snap_vp;  // kv x Tvp (device)
  double* snap_sp;  // ks x Tsp
  unsigned long long Tvp, Tsp;
  uint32_t fseis;
  double* hist;                 // kv x (samples of this launch): XV on the seismogram's sample steps
  unsigned long long hist_t0;   // sample index of hist's first column
  unsigned int* error;          // set when an exchange wait runs out
  // band kernel (FP64): each CTA's mailbox of tagged words, [CTA][2 slots][kv][2] and
  // [CTA][2 slots][ks][2]
  unsigned long long* xw_v;
  unsigned long long* xw_s;
  uint32_t tag0;  // tag of the launch's first step (>= 1); step it carries tag0 + it
};

// Dynamic shared memory of the rank-1 kernel, in elements of T (double or df):
//   xv_full[2][kv] | xs_full[2][ks] (both alternating by step) | Av rows [rows_v x ks] |
//   As rows [rows_s x kv] | b rows [rows_v]
template <typename T>
size_t rank1_smem_bytes(uint32_t kv, uint32_t ks, uint32_t rv, uint32_t rs) {
  return sizeof(T) * (2 * (size_t)kv + 2 * (size_t)ks + (size_t)rv * ks + (size_t)rs * kv + rv);
}

// ---- cluster exchange: st.async into the peers' shared memory, completing on their mbarrier
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t peer_addr(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_async8(uint32_t raddr, uint64_t v, uint32_t rbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(raddr), "l"(v),
               "r"(rbar)
               : "memory");
}
__device__ __forceinline__ void xbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)));
}
// this CTA's single arrival of the phase, announcing the bytes the peers will deliver
__device__ __forceinline__ void xbar_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// Bounded wait for the phase with the given parity (acquire at cluster scope: the
// peers' stores are visible afterwards).  False when the limit ran out.
__device__ __forceinline__ bool xbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_addr(bar);
  for (unsigned long long i = 0; i < (1ull << 24); ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
template <typename T>
__device__ __forceinline__ uint64_t bits8(T x) {
  static_assert(sizeof(T) == 8, "8-byte state elements");
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ void warp_sum_df(float& s, float& c) {
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
    const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
    const df t = two_sum(s, s2);
    s = t.h;
    c = c + c2 + t.l;
  }
}

template <bool MIXED>
struct Arith;

template <>
struct Arith<false> {
  using T = double;
  __device__ static T load(double x) { return x; }
  __device__ static double value(T x) { return x; }
  // warp dot product of row[0:n] with vec[0:n]
  __device__ static T dot(const T* row, const T* vec, uint32_t n, int lane) {
    double acc = 0.0;
    for (uint32_t k = lane; k < n; k += 32) acc = fma(row[k], vec[k], acc);
    return warp_sum(acc);
  }
  // x + dt*y, then + fdt*b when b != null: KokkosBlas::gemv then axpy roundings
  __device__ static T update(T x, T y, T dt) { return __dadd_rn(x, __dmul_rn(dt, y)); }
  __device__ static T axpy(T x, T a, T b) { return __dadd_rn(x, __dmul_rn(a, b)); }
  // an output sample (seismogram): the value itself
  __device__ static void store_sample(double* p, T x) { *p = x; }
};

template <>
struct Arith<true> {
  using T = df;
  __device__ static T load(double x) { return df_split(x); }
  __device__ static double value(T x) { return df_val(x); }
  __device__ static T dot(const T* row, const T* vec, uint32_t n, int lane) {
    float s = 0.f, c = 0.f;
    for (uint32_t k = lane; k < n; k += 32) df_dot_acc(s, c, row[k], vec[k]);
    warp_sum_df(s, c);
    return df_norm(s, c);
  }
  // dt and a arrive already split (once per launch / per step, not per row)
  __device__ static T update(T x, T y, T dt) { return df_add(x, df_mul(dt, y)); }
  __device__ static T axpy(T x, T a, T b) { return df_add(x, df_mul(a, b)); }
  // an output sample: the FP32 pair in the double's 8 bytes, widened to FP64 after the
  // launch (rom_samples_to_fp64_kernel), so the time loop issues no FP64 instruction
  __device__ static void store_sample(double* p, T x) { *reinterpret_cast<df*>(p) = x; }
};

// The observers' sample steps, counted instead of divided (a 64-bit division per step and
// thread sat on the latency-bound loop): at step n, `due` when n is a multiple of freq,
// with `index` = n / freq - 1 - base.  Start with the launch's first step step0 + 1.
struct SampleClock {
  uint32_t freq, phase;
  unsigned long long next;  // index of the next sample
  __device__ SampleClock(uint32_t f, unsigned long long step0, unsigned long long base)
      : freq(f), phase(f ? (uint32_t)(step0 % f) : 0), next(f ? step0 / f - base : 0) {}
  // advance to the next step; true (and the sample index in *idx) on a sample step
  __device__ __forceinline__ bool tick(unsigned long long* idx) {
    if (!freq || ++phase != freq) return false;
    phase = 0;
    *idx = next++;
    return true;
  }
};

// One persistent launch for nsteps ROM rank-1 leapfrog steps (one cluster).
template <bool MIXED>
__global__ void __launch_bounds__(kR1Threads) rom_rank1_cluster_kernel(RomArgs a) {
  using A = Arith<MIXED>;
  using T = typename A::T;
  cg::cluster_group cluster = cg::this_cluster();
  const uint32_t crank = cluster.block_rank();
  const uint32_t csize = cluster.num_blocks();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // Both states alternate between two full copies: step it reads copy it % 2 and writes
  // its new rows into copy (it + 1) % 2 of every CTA.  A CTA reaches the step that
  // overwrites a copy only after every peer has sent the rows of the step in between,
  // i.e. after every peer has finished reading that copy.
  T* const xvb = reinterpret_cast<T*>(smem_raw);
  T* const xsb = xvb + 2 * (size_t)a.kv;
  T* Av = xsb + 2 * (size_t)a.ks;
  // xbar[c]: the XV copy c is complete; xbar[2 + c]: the XS copy c is complete
  __shared__ __align__(8) uint64_t xbar[4];
  T* As = Av + (size_t)a.rows_v * a.ks;
  T* bv = As + (size_t)a.rows_s * a.kv;
  // row slices of this CTA (empty for trailing ranks when the rows do not divide evenly)
  const uint32_t v0 = min(a.kv, crank * a.rows_v), v1 = min(a.kv, v0 + a.rows_v);
  const uint32_t s0 = min(a.ks, crank * a.rows_s), s1 = min(a.ks, s0 + a.rows_s);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  if (threadIdx.x == 0) {
    for (int i = 0; i < 4; ++i) xbar_init(&xbar[i]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (uint32_t k = threadIdx.x; k < a.kv; k += kR1Threads) xvb[k] = A::load(a.xv[k]);
  for (uint32_t k = threadIdx.x; k < a.ks; k += kR1Threads) xsb[k] = A::load(a.xs[k]);
  for (size_t e = threadIdx.x; e < (size_t)(v1 - v0) * a.ks; e += kR1Threads)
    Av[e] = A::load(a.Av[(size_t)v0 * a.ks + e]);
  for (size_t e = threadIdx.x; e < (size_t)(s1 - s0) * a.kv; e += kR1Threads)
    As[e] = A::load(a.As[(size_t)s0 * a.kv + e]);
  for (uint32_t r = v0 + threadIdx.x; r < v1; r += kR1Threads) bv[r - v0] = A::load(a.b[r]);
  cluster.sync();

  const T dtT = A::load(a.dt);
  SampleClock clk_v(a.fvp, a.step0, 0), clk_s(a.fsp, a.step0, 0), clk_h(a.hist ? a.fseis : 0, a.step0, a.hist_t0);
  for (unsigned long long it = 0; it < a.nsteps; ++it) {
    // rom_run_rank_one.hpp:118 fValDt = f(t_{n-1}) * dt, from the table filled before the launch
    // (RankOneForcing keeps the whole signal time series too: forcing_rank_one.hpp:169-178)
    const T fdt = static_cast<const T*>(a.fdt_t)[it];
    // sample steps of the observers, decided once per step
    unsigned long long iv = 0, is = 0, ih = 0;
    const bool snap_v = clk_v.tick(&iv), snap_s = clk_s.tick(&is);
    // the ROM seismogram S = PhiVp[gid_r, :] XV (main_reconstruct_seismo.cc:157-185) is one
    // GEMM kernel after the launch over the XV of the sample steps, kept here in hist
    double* const hcol = clk_h.tick(&ih) ? a.hist + (size_t)a.kv * ih : nullptr;
    const uint32_t cur = (uint32_t)(it & 1), nxt = cur ^ 1u, par = (uint32_t)((it >> 1) & 1);
    const T* const xvc = xvb + (size_t)cur * a.kv;
    const T* const xsc = xsb + (size_t)cur * a.ks;
    T* const xv = xvb + (size_t)nxt * a.kv;  // the new states
    T* const xs = xsb + (size_t)nxt * a.ks;
    // 1. velocity rows of this CTA, sent to copy nxt of every CTA (lane l -> CTA l)
    if (threadIdx.x == 0) xbar_expect(&xbar[nxt], a.kv * (uint32_t)sizeof(T));
    for (uint32_t r = v0 + warp; r < v1; r += kR1Warps) {
      const T y = A::dot(Av + (size_t)(r - v0) * a.ks, xsc, a.ks, lane);
      if (lane < (int)csize) {
        T x = A::update(xvc[r], y, dtT);
        x = A::axpy(x, fdt, bv[r - v0]);
        st_async8(peer_addr(smem_addr(xv + r), lane), bits8(x), peer_addr(smem_addr(&xbar[nxt]), lane));
        if (lane == 0 && snap_v)
          a.snap_vp[r + (size_t)a.kv * iv] = A::value(x);
        if (lane == 0 && hcol) A::store_sample(hcol + r, x);
      }
    }
    bool ok = xbar_wait(&xbar[nxt], par);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(a.error, 1u);
      break;
    }
    // 2. stress rows of this CTA
    if (threadIdx.x == 0) xbar_expect(&xbar[2 + nxt], a.ks * (uint32_t)sizeof(T));
    for (uint32_t r = s0 + warp; r < s1; r += kR1Warps) {
      const T y = A::dot(As + (size_t)(r - s0) * a.kv, xv, a.kv, lane);
      if (lane < (int)csize) {
        const T x = A::update(xsc[r], y, dtT);
        st_async8(peer_addr(smem_addr(xs + r), lane), bits8(x), peer_addr(smem_addr(&xbar[2 + nxt]), lane));
        if (lane == 0 && snap_s)
          a.snap_sp[r + (size_t)a.ks * is] = A::value(x);
      }
    }
    ok = xbar_wait(&xbar[2 + nxt], par);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(a.error, 2u);
      break;
    }
  }
  const T* const xvf = xvb + (size_t)(a.nsteps & 1) * a.kv;
  const T* const xsf = xsb + (size_t)(a.nsteps & 1) * a.ks;
  for (uint32_t r = v0 + threadIdx.x; r < v1; r += kR1Threads) a.xv[r] = A::value(xvf[r]);
  for (uint32_t r = s0 + threadIdx.x; r < s1; r += kR1Threads) a.xs[r] = A::value(xsf[r]);
  // no CTA leaves while a peer may still deliver rows into its shared memory
  cluster.sync();
}

// ---- FP64 rank 1 over many SMs: one cooperative launch of row bands ----------------
//
// The cluster kernel above keeps its 16 CTAs' FP64 pipes busy (a row dot is 8 dependent
// FMAs and 5 shuffle adds per lane, ~64 cycles per warp FP64 instruction on a sub-
// partition of GB300's narrow FP64 pipe).  Here a cooperative grid of up to one CTA per
// SM runs the same steps with a few rows per CTA: CTA c owns velocity rows [c rv, ...)
// and stress rows [c rs, ...), one warp per row (so four rows run on the four sub-
// partitions side by side), and keeps full copies of both states.  After each half-step
// every CTA writes its new rows as tagged words into every CTA's own mailbox and
// gathers its mailbox through L2 (l2_exchange.cuh).  Private mailboxes keep the polls of
// different CTAs on different lines: with one shared copy, every CTA polled the same
// few lines and the writers' stores queued behind the polls (7.0 us per step at k = 256
// against 5.7 for the cluster).  Two slots per state by step parity: a CTA overwrites
// a slot of step n only after it has gathered step n - 1, which every CTA published after
// it had gathered step n - 2 from that slot.  The row arithmetic (Arith<false>: the same warp
// dot, update and forcing) is the cluster kernel's, so the results are bit-identical.
// A row's own old value is read before the row is published, so the gather that
// overwrites it cannot run ahead of that read; other rows of the state being gathered are
// not read in that half-step.  Every wait is bounded (error bit 1 velocity, 2 stress).
constexpr int kR1BandThreads = 256;
constexpr int kR1BandWarps = kR1BandThreads / 32;
constexpr int kR1BandRecv = 4;  // gathered points per thread: k <= 1024

__device__ __forceinline__ bool gather_state(double* x, const unsigned long long* w, uint32_t k, uint32_t tag) {
  const unsigned long long* src[kR1BandRecv];
  double* dst[kR1BandRecv];
  uint32_t pending = 0;
#pragma unroll
  for (int j = 0; j < kR1BandRecv; ++j) {
    const uint32_t q = threadIdx.x + j * kR1BandThreads;
    src[j] = nullptr;
    dst[j] = nullptr;
    if (q < k) {
      src[j] = w + 2 * (size_t)q;
      dst[j] = x + q;
      pending |= 1u << j;
    }
  }
  return shaw::l2x::poll<kR1BandRecv>(src, dst, pending, tag);
}

__global__ void __launch_bounds__(kR1BandThreads, 1) rom_rank1_band_kernel(RomArgs a) {
  using A = Arith<false>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* const xv = reinterpret_cast<double*>(smem_raw);  // [kv]
  double* const xs = xv + a.kv;                            // [ks]
  double* const Av = xs + a.ks;                            // rows_v x ks
  double* const As = Av + (size_t)a.rows_v * a.ks;         // rows_s x kv
  double* const bv = As + (size_t)a.rows_s * a.kv;         // rows_v
  const uint32_t c = blockIdx.x;
  const uint32_t v0 = min(a.kv, c * a.rows_v), v1 = min(a.kv, v0 + a.rows_v);
  const uint32_t s0 = min(a.ks, c * a.rows_s), s1 = min(a.ks, s0 + a.rows_s);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  for (uint32_t k = threadIdx.x; k < a.kv; k += kR1BandThreads) xv[k] = a.xv[k];
  for (uint32_t k = threadIdx.x; k < a.ks; k += kR1BandThreads) xs[k] = a.xs[k];
  for (size_t e = threadIdx.x; e < (size_t)(v1 - v0) * a.ks; e += kR1BandThreads) Av[e] = a.Av[(size_t)v0 * a.ks + e];
  for (size_t e = threadIdx.x; e < (size_t)(s1 - s0) * a.kv; e += kR1BandThreads) As[e] = a.As[(size_t)s0 * a.kv + e];
  for (uint32_t r = v0 + threadIdx.x; r < v1; r += kR1BandThreads) bv[r - v0] = a.b[r];
  __syncthreads();

  const double dt = a.dt;
  SampleClock clk_v(a.fvp, a.step0, 0), clk_s(a.fsp, a.step0, 0), clk_h(a.hist ? a.fseis : 0, a.step0, a.hist_t0);
  for (unsigned long long it = 0; it < a.nsteps; ++it) {
    const uint32_t tag = a.tag0 + (uint32_t)it;
    const size_t slot = (size_t)(it & 1);
    const double fdt = static_cast<const double*>(a.fdt_t)[it];  // rom_run_rank_one.hpp:118 fValDt
    unsigned long long iv = 0, is = 0, ih = 0;
    const bool snap_v = clk_v.tick(&iv), snap_s = clk_s.tick(&is);
    double* const hcol = clk_h.tick(&ih) ? a.hist + (size_t)a.kv * ih : nullptr;
    // 1. velocity rows of this CTA, written into every CTA's mailbox as they are formed
    //    (every lane holds the row's sum and forms the same new value)
    const uint32_t G = gridDim.x;
    for (uint32_t r = v0 + warp; r < v1; r += kR1BandWarps) {
      const double y = A::dot(Av + (size_t)(r - v0) * a.ks, xs, a.ks, lane);
      double x = A::update(xv[r], y, dt);
      x = A::axpy(x, fdt, bv[r - v0]);
      for (uint32_t c = lane; c < G; c += 32) shaw::l2x::put(a.xw_v + ((2 * (size_t)c + slot) * a.kv + r) * 2, tag, x);
      if (lane == 0) {
        if (snap_v) a.snap_vp[r + (size_t)a.kv * iv] = x;
        if (hcol) hcol[r] = x;
      }
    }
    bool ok = gather_state(xv, a.xw_v + (2 * (size_t)blockIdx.x + slot) * a.kv * 2, a.kv, tag);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(a.error, 1u);
      break;
    }
    // 2. stress rows of this CTA
    for (uint32_t r = s0 + warp; r < s1; r += kR1BandWarps) {
      const double y = A::dot(As + (size_t)(r - s0) * a.kv, xv, a.kv, lane);
      const double x = A::update(xs[r], y, dt);
      for (uint32_t c = lane; c < G; c += 32) shaw::l2x::put(a.xw_s + ((2 * (size_t)c + slot) * a.ks + r) * 2, tag, x);
      if (lane == 0 && snap_s) a.snap_sp[r + (size_t)a.ks * is] = x;
    }
    ok = gather_state(xs, a.xw_s + (2 * (size_t)blockIdx.x + slot) * a.ks * 2, a.ks, tag);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(a.error, 2u);
      break;
    }
  }
  for (uint32_t r = v0 + threadIdx.x; r < v1; r += kR1BandThreads) a.xv[r] = xv[r];
  for (uint32_t r = s0 + threadIdx.x; r < s1; r += kR1BandThreads) a.xs[r] = xs[r];
}

// FP64 -> FP32 hi + lo; in and out may be the same array (each element is read before
// it is overwritten, by the same thread).
__global__ void rom_split_df_kernel(const double* in, df* out, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const double v = in[e];
    out[e] = df_split(v);
  }
}

// out (R x T, leading dimension R) = phi (R x k row-major) * hist (k x T): one 16 x 16
// output tile per block, the k sum in ascending order with FMAs, so every element's
// arithmetic is independent of how the columns are split across launches.
__global__ void rom_seis_gemm_kernel(const double* __restrict__ phi, const double* __restrict__ hist, uint32_t R,
                                     uint32_t k, uint32_t T, double* __restrict__ out) {
  __shared__ double ps[16][17], hs[16][17];
  const uint32_t tx = threadIdx.x, ty = threadIdx.y;
  const uint32_t r = blockIdx.x * 16 + ty, t = blockIdx.y * 16 + tx;
  double acc = 0.0;
  for (uint32_t k0 = 0; k0 < k; k0 += 16) {
    const uint32_t rr = blockIdx.x * 16 + ty, kk = k0 + tx;
    ps[ty][tx] = (rr < R && kk < k) ? phi[(size_t)rr * k + kk] : 0.0;
    const uint32_t kh = k0 + ty, th = blockIdx.y * 16 + tx;
    hs[ty][tx] = (kh < k && th < T) ? hist[(size_t)th * k + kh] : 0.0;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 16; ++j) acc = fma(ps[ty][j], hs[j][tx], acc);
    __syncthreads();
  }
  if (r < R && t < T) out[(size_t)t * R + r] = acc;
}

// Samples stored as FP32 hi + lo pairs in place of doubles -> FP64, in place.
__global__ void rom_samples_to_fp64_kernel(double* p, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const df v = *reinterpret_cast<const df*>(p + e);
    p[e] = df_val(v);
  }
}

// table[s] = f(t) * dt at t = (step0 + s) * dt: the forcing of step step0 + s + 1.
__global__ void rom_signal_table_kernel(int kind, double delay, double period, double dt, unsigned long long step0,
                                        unsigned long long n, double* table) {
  const unsigned long long s = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  if (s < n) table[s] = shaw::signal_value(kind, delay, period, (double)(step0 + s) * dt) * dt;
}

// Rank-2 forcing: XV[:, j] += (f_j(t_{n-1}) * dt) * b[:, j]   (one block per column)
__global__ void rom_forcing_rank2_kernel(double* xv, const double* b, const int* kind, const double* period,
                                         const double* delay, double dt, unsigned long long n, uint32_t kv) {
  __shared__ double fdt;
  const uint32_t j = blockIdx.x;
  if (threadIdx.x == 0) fdt = shaw::signal_value(kind[j], delay[j], period[j], (double)(n - 1) * dt) * dt;
  __syncthreads();
  double* col = xv + (size_t)j * kv;
  const double* bc = b + (size_t)j * kv;
  for (uint32_t i = threadIdx.x; i < kv; i += blockDim.x) col[i] = __dadd_rn(col[i], __dmul_rn(fdt, bc[i]));
}

}  // namespace

struct shaw_rom_s {
  uint64_t kv = 0, ks = 0;
  uint32_t M = 1;
  int rank = 1, precision = SHAW_FP64;
  shaw::tc::Plan* tc = nullptr;  // rank-2 tensor-core TF32x3 path
  shaw::oz::Batch* oz = nullptr;  // rank-2 tensor-core Ozaki BF16 path (a batch of one)
  bool persistent2() const { return tc != nullptr || oz != nullptr; }
  cudaStream_t stream = nullptr;
  cublasHandle_t blas = nullptr;
  double *Av = nullptr, *As = nullptr, *b = nullptr, *xv = nullptr, *xs = nullptr;
  int* kind = nullptr;
  double *period = nullptr, *delay = nullptr;
  std::vector<int> h_kind;
  std::vector<double> h_period, h_delay;
  bool signals_set = false;
  // observers
  uint64_t fvp = 0, fsp = 0, snap_nsteps = 0;
  double *snap_vp = nullptr, *snap_sp = nullptr;  // device
  double *host_vp = nullptr, *host_sp = nullptr;  // caller arrays
  uint32_t R = 0;
  uint64_t fseis = 0, seis_T = 0, seis_nsteps = 0;
  double *phi_rcv = nullptr, *seis = nullptr;
  double* fdt = nullptr;  // rank-1 forcing table of the current launch
  uint64_t fdt_cap = 0;
  double* hist = nullptr;  // rank-1: XV on the sample steps of a launch (seismogram GEMM input)
  size_t hist_cap = 0;
  unsigned int* r1_err = nullptr;  // rank-1 kernel: an exchange wait ran out
  // rank-1 launch shape: cluster (rom_rank1_cluster_kernel) or bands (rom_rank1_band_kernel)
  uint32_t cluster = 1, rows_v = 0, rows_s = 0;
  size_t smem = 0;
  bool band = false, band_ok = false, cluster_ok = false;  // band: the launch in use
  uint32_t band_n = 0, band_rv = 0, band_rs = 0;
  size_t band_smem = 0;
  unsigned long long* xw = nullptr;  // band mailboxes: [CTA][2][kv][2] then [CTA][2][ks][2]
  uint32_t band_tag = 0;             // last tag used in xw (0: cleared)
  uint64_t step = 0;
  uint64_t launches = 0;
};

namespace {

using RH = shaw_rom_s;

// FP64 rank 1 on row bands: a few rows per CTA (one warp each), one CTA per SM at most;
// every state gathered by 256 threads of at most four points.
bool rank1_band_plan(RH* h, int sms, size_t budget) {
  const uint64_t k = std::max(h->kv, h->ks);
  if (k > (uint64_t)kR1BandRecv * kR1BandThreads || k < 2) return false;
  // rows per CTA: measured at k = 128 .. 1024 (steps of 2000 with a 181-receiver seismogram),
  // 4 rows per CTA up to k = 256 and 8 beyond were fastest: fewer CTAs write fewer mailboxes
  // and stay on one die, more rows per CTA queue more warps on the FP64 pipe
  uint64_t rpc = std::max<uint64_t>(4, (k + 63) / 64);
  uint32_t g = 0, rv = 0, rs = 0;
  size_t bytes = 0;
  for (;; rpc = (rpc + 1) / 2) {
    g = (uint32_t)std::max<uint64_t>(2, (k + rpc - 1) / rpc);
    rv = (uint32_t)((h->kv + g - 1) / g);
    rs = (uint32_t)((h->ks + g - 1) / g);
    bytes = sizeof(double) * ((size_t)h->kv + h->ks + (size_t)rv * h->ks + (size_t)rs * h->kv + rv);
    if (bytes <= budget || rpc == 1) break;
  }
  if (bytes > budget || g > (uint32_t)sms) return false;
  if (cudaFuncSetAttribute(rom_rank1_band_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
      cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rom_rank1_band_kernel, kR1BandThreads, bytes) !=
          cudaSuccess ||
      (uint64_t)per_sm * sms < g) {
    cudaGetLastError();
    return false;
  }
  h->band_ok = true;
  h->band_n = g;
  h->band_rv = rv;
  h->band_rs = rs;
  h->band_smem = bytes;
  return true;
}

template <bool MIXED>
int rank1_configure(RH* h) {
  using T = typename Arith<MIXED>::T;
  int dev = 0, maxOptin = 0, sms = 0;
  SHAW_CUDA(cudaGetDevice(&dev));
  SHAW_CUDA(cudaDeviceGetAttribute(&maxOptin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  SHAW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const size_t budget = (size_t)maxOptin;
  // FP64: row bands over the GPU when they fit (the default), else the cluster
  if (!MIXED) h->band = rank1_band_plan(h, sms, budget);
  for (uint32_t c : {1u, 2u, 4u, 8u, 16u}) {
    const uint32_t rv = (uint32_t)((h->kv + c - 1) / c), rs = (uint32_t)((h->ks + c - 1) / c);
    const size_t bytes = rank1_smem_bytes<T>((uint32_t)h->kv, (uint32_t)h->ks, rv, rs);
    if (bytes <= budget) {
      // prefer the smallest cluster whose per-CTA row slice keeps the warps busy
      // FP64 GEMV rows are the cost on GB300's narrow FP64 pipe: spread them over up
      // to 16 CTAs (the cluster exchange costs less than the extra rows per CTA)
      if (rv > 16 && c < 16) continue;
      h->cluster = c; h->rows_v = rv; h->rows_s = rs; h->smem = bytes;
      h->cluster_ok = true;
      return SHAW_OK;
    }
  }
  if (h->band_ok) return SHAW_OK;
  return shaw::fail(SHAW_ERR_UNSUPPORTED, "reduced operators too large for the on-chip rank-1 ROM kernel");
}

template <bool MIXED>
int rank1_launch(RH* h, double dt, uint64_t nsteps) {
  RomArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Av = h->Av; a.As = h->As; a.b = h->b; a.xv = h->xv; a.xs = h->xs;
  if (h->fdt_cap < nsteps) {
    if (h->fdt) cudaFree(h->fdt);
    h->fdt = nullptr;
    h->fdt_cap = 0;
    SHAW_CUDA(cudaMalloc(&h->fdt, nsteps * sizeof(double)));
    h->fdt_cap = nsteps;
  }
  rom_signal_table_kernel<<<(unsigned)((nsteps + 255) / 256), 256, 0, h->stream>>>(
      h->h_kind[0], h->h_delay[0], h->h_period[0], dt, h->step, nsteps, h->fdt);
  h->launches++;
  SHAW_CUDA(cudaGetLastError());
  if (MIXED) {  // the forcing table as FP32 hi + lo, in place
    rom_split_df_kernel<<<(unsigned)((nsteps + 255) / 256), 256, 0, h->stream>>>(h->fdt, reinterpret_cast<df*>(h->fdt),
                                                                                  nsteps);
    h->launches++;
    SHAW_CUDA(cudaGetLastError());
  }
  if (!h->r1_err) {
    SHAW_CUDA(cudaMalloc(&h->r1_err, sizeof(unsigned int)));
    SHAW_CUDA(cudaMemsetAsync(h->r1_err, 0, sizeof(unsigned int), h->stream));
  }
  a.error = h->r1_err;
  a.fdt_t = h->fdt; a.dt = dt;
  a.kv = (uint32_t)h->kv; a.ks = (uint32_t)h->ks; a.rows_v = h->rows_v; a.rows_s = h->rows_s;
  a.step0 = h->step; a.nsteps = nsteps;
  a.fvp = (uint32_t)h->fvp; a.fsp = (uint32_t)h->fsp; a.snap_vp = h->snap_vp; a.snap_sp = h->snap_sp;
  // seismogram samples of this launch: XV history in the kernel, one GEMM kernel afterwards
  const uint64_t t0 = h->fseis ? h->step / h->fseis : 0, t1 = h->fseis ? (h->step + nsteps) / h->fseis : 0;
  if (h->seis && t1 > t0) {
    const size_t need = (size_t)h->kv * (t1 - t0);
    if (h->hist_cap < need) {
      if (h->hist) cudaFree(h->hist);
      h->hist = nullptr;
      h->hist_cap = 0;
      SHAW_CUDA(cudaMalloc(&h->hist, need * sizeof(double)));
      h->hist_cap = need;
    }
    a.hist = h->hist;
    a.hist_t0 = t0;
    a.fseis = (uint32_t)h->fseis;
  }
  if (!MIXED && h->band) {
    const size_t words = 4 * (size_t)h->band_n * ((size_t)h->kv + h->ks);  // a mailbox per CTA
    if (!h->xw) {
      SHAW_CUDA(cudaMalloc(&h->xw, words * sizeof(unsigned long long)));
      SHAW_CUDA(cudaMemsetAsync(h->xw, 0, words * sizeof(unsigned long long), h->stream));
      h->band_tag = 0;
    }
    if ((uint64_t)h->band_tag + nsteps >= 0xffffffffull) {  // tags would wrap: clear the words
      SHAW_CUDA(cudaMemsetAsync(h->xw, 0, words * sizeof(unsigned long long), h->stream));
      h->band_tag = 0;
    }
    a.xw_v = h->xw;
    a.xw_s = h->xw + 4 * (size_t)h->band_n * h->kv;
    a.tag0 = h->band_tag + 1;
    a.rows_v = h->band_rv;
    a.rows_s = h->band_rs;
    // per launch: another handle's plan may have set the kernel's limit for fewer modes
    SHAW_CUDA(cudaFuncSetAttribute(rom_rank1_band_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)h->band_smem));
    cudaLaunchConfig_t cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(h->band_n);
    cfg.blockDim = dim3(kR1BandThreads);
    cfg.dynamicSmemBytes = h->band_smem;
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // every band co-resident, or the launch fails
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SHAW_CUDA(cudaLaunchKernelEx(&cfg, rom_rank1_band_kernel, a));
    h->band_tag += (uint32_t)nsteps;
  } else {
  auto kern = rom_rank1_cluster_kernel<MIXED>;
  SHAW_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h->smem));
  if (h->cluster > 8) SHAW_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(h->cluster);
  cfg.blockDim = dim3(kR1Threads);
  cfg.dynamicSmemBytes = h->smem;
  cfg.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = h->cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SHAW_CUDA(cudaLaunchKernelEx(&cfg, kern, a));
  }
  h->launches++;
  if (a.hist) {
    const size_t cnt = (size_t)h->kv * (t1 - t0);
    if (MIXED) {  // the history as FP32 pairs -> FP64
      rom_samples_to_fp64_kernel<<<(unsigned)std::min<size_t>((cnt + 255) / 256, 1024), 256, 0, h->stream>>>(h->hist,
                                                                                                             cnt);
      h->launches++;
      SHAW_CUDA(cudaGetLastError());
    }
    // S(:, t0:t1) = PhiRcv (R x kv, row-major) * hist (kv x (t1 - t0))
    const dim3 grid((unsigned)((h->R + 15) / 16), (unsigned)((t1 - t0 + 15) / 16));
    rom_seis_gemm_kernel<<<grid, dim3(16, 16), 0, h->stream>>>(h->phi_rcv, h->hist, (uint32_t)h->R, (uint32_t)h->kv,
                                                              (uint32_t)(t1 - t0), h->seis + (size_t)h->R * t0);
    h->launches++;
    SHAW_CUDA(cudaGetLastError());
  }
  return SHAW_OK;
}

int rank2_step(RH* h, double dt, uint64_t n) {
  const double one = 1.0;
  // xv = xv + dt * Av xs  (Av row-major kv x ks == column-major ks x kv -> op T)
  if (cublasDgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)h->kv, (int)h->M, (int)h->ks, &dt, h->Av, (int)h->ks,
                  h->xs, (int)h->ks, &one, h->xv, (int)h->kv) != CUBLAS_STATUS_SUCCESS)
    return shaw::fail(SHAW_ERR_CUDA, "cublasDgemm (velocity) failed");
  rom_forcing_rank2_kernel<<<h->M, 128, 0, h->stream>>>(h->xv, h->b, h->kind, h->period, h->delay, dt, n,
                                                        (uint32_t)h->kv);
  h->launches += 2;
  SHAW_CUDA(cudaGetLastError());
  if (h->fvp && n % h->fvp == 0) {
    const uint64_t T = h->snap_nsteps / h->fvp;
    SHAW_CUDA(cudaMemcpy2DAsync(h->host_vp + h->kv * (n / h->fvp - 1), h->kv * T * sizeof(double), h->xv,
                                h->kv * sizeof(double), h->kv * sizeof(double), h->M, cudaMemcpyDeviceToHost,
                                h->stream));
  }
  if (h->fseis && n % h->fseis == 0) {
    const double zero = 0.0;
    // S(:, t, :) = PhiRcv (R x kv) * XV (kv x M) into the R x T x M seismogram
    if (cublasDgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)h->R, (int)h->M, (int)h->kv, &one, h->phi_rcv,
                    (int)h->kv, h->xv, (int)h->kv, &zero, h->seis + (size_t)h->R * (n / h->fseis - 1),
                    (int)(h->R * h->seis_T)) != CUBLAS_STATUS_SUCCESS)
      return shaw::fail(SHAW_ERR_CUDA, "cublasDgemm (seismogram) failed");
    h->launches++;
  }
  // xs = xs + dt * As xv
  if (cublasDgemm(h->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)h->ks, (int)h->M, (int)h->kv, &dt, h->As, (int)h->kv,
                  h->xv, (int)h->kv, &one, h->xs, (int)h->ks) != CUBLAS_STATUS_SUCCESS)
    return shaw::fail(SHAW_ERR_CUDA, "cublasDgemm (stress) failed");
  h->launches++;
  if (h->fsp && n % h->fsp == 0) {
    const uint64_t T = h->snap_nsteps / h->fsp;
    SHAW_CUDA(cudaMemcpy2DAsync(h->host_sp + h->ks * (n / h->fsp - 1), h->ks * T * sizeof(double), h->xs,
                                h->ks * sizeof(double), h->ks * sizeof(double), h->M, cudaMemcpyDeviceToHost,
                                h->stream));
  }
  return SHAW_OK;
}

}  // namespace

extern "C" {

int shaw_rom_create(uint64_t kv, uint64_t ks, const double* Av, const double* As, int rank, uint32_t M,
                    const double* b, int precision, shaw_rom_t* out) {
  if (!out || !Av || !As || !b) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (kv == 0 || ks == 0 || M == 0) return shaw::fail(SHAW_ERR_INVALID_ARG, "sizes must be positive");
  if (kv > 65535 || ks > 65535) return shaw::fail(SHAW_ERR_UNSUPPORTED, "at most 65535 modes");
  if (rank != 1 && rank != 2) return shaw::fail(SHAW_ERR_INVALID_ARG, "rank must be 1 or 2");
  if (rank == 1 && M != 1) return shaw::fail(SHAW_ERR_INVALID_ARG, "the rank-1 form has exactly one forcing");
  if (rank == 1 && precision != SHAW_FP64 && precision != SHAW_MIXED_FP32)
    return shaw::fail(SHAW_ERR_UNSUPPORTED, "rank-1 ROM precision must be SHAW_FP64 or SHAW_MIXED_FP32");
  if (rank == 2 && precision != SHAW_FP64 && precision != SHAW_MIXED_TF32X3 && precision != SHAW_MIXED_OZAKI_BF16 &&
      precision != SHAW_OZAKI_FP64)
    return shaw::fail(SHAW_ERR_UNSUPPORTED,
                      "rank-2 ROM precision must be SHAW_FP64, SHAW_MIXED_TF32X3, SHAW_MIXED_OZAKI_BF16 or "
                      "SHAW_OZAKI_FP64");
  RH* h = new RH();
  h->kv = kv; h->ks = ks; h->M = M; h->rank = rank; h->precision = precision;
  auto bail = [&](int rc) { shaw_rom_destroy(h); return rc; };
  cudaError_t e;
#define SHAW_TRY(call) do { e = (call); if (e != cudaSuccess) return bail(shaw::cuda_fail(e, #call)); } while (0)
  SHAW_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  SHAW_TRY(cudaMalloc(&h->Av, kv * ks * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->As, kv * ks * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->b, kv * M * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->xv, kv * M * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->xs, ks * M * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->kind, M * sizeof(int)));
  SHAW_TRY(cudaMalloc(&h->period, M * sizeof(double)));
  SHAW_TRY(cudaMalloc(&h->delay, M * sizeof(double)));
  SHAW_TRY(cudaMemcpyAsync(h->Av, Av, kv * ks * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SHAW_TRY(cudaMemcpyAsync(h->As, As, kv * ks * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SHAW_TRY(cudaMemcpyAsync(h->b, b, kv * M * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SHAW_TRY(cudaMemsetAsync(h->xv, 0, kv * M * sizeof(double), h->stream));
  SHAW_TRY(cudaMemsetAsync(h->xs, 0, ks * M * sizeof(double), h->stream));
  SHAW_TRY(cudaStreamSynchronize(h->stream));
#undef SHAW_TRY
  int rc = SHAW_OK;
  if (rank == 1) {
    rc = precision == SHAW_FP64 ? rank1_configure<false>(h) : rank1_configure<true>(h);
  } else if (precision == SHAW_MIXED_TF32X3) {
    rc = shaw::tc::create(h->tc, (uint32_t)kv, (uint32_t)ks, h->Av, h->As, M, h->b, h->stream);
    if (rc == SHAW_OK && cudaStreamSynchronize(h->stream) != cudaSuccess)
      rc = shaw::fail(SHAW_ERR_CUDA, "tensor-core ROM setup failed");
  } else if (precision == SHAW_MIXED_OZAKI_BF16 || precision == SHAW_OZAKI_FP64) {
    shaw::oz::InstanceDesc d;
    d.kv = (uint32_t)kv; d.ks = (uint32_t)ks; d.M = M; d.Av = Av; d.As = As; d.b = b;
    rc = shaw::oz::create(h->oz, 1, &d, h->stream, precision == SHAW_OZAKI_FP64 ? 9 : 6);
    if (rc == SHAW_OK) rc = shaw::oz::set_signals(h->oz, 0, h->kind, h->period, h->delay);
    if (rc == SHAW_OK && cudaStreamSynchronize(h->stream) != cudaSuccess)
      rc = shaw::fail(SHAW_ERR_CUDA, "Ozaki tensor-core ROM setup failed");
  } else {
    if (cublasCreate(&h->blas) != CUBLAS_STATUS_SUCCESS) rc = shaw::fail(SHAW_ERR_CUDA, "cublasCreate failed");
    else if (cublasSetStream(h->blas, h->stream) != CUBLAS_STATUS_SUCCESS)
      rc = shaw::fail(SHAW_ERR_CUDA, "cublasSetStream failed");
  }
  if (rc) return bail(rc);
  *out = h;
  return SHAW_OK;
}

void shaw_rom_destroy(shaw_rom_t h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->blas) cublasDestroy(h->blas);
  if (h->tc) shaw::tc::destroy(h->tc);
  if (h->oz) shaw::oz::destroy(h->oz);
  if (h->rank == 2 && !h->persistent2()) {
    if (h->host_vp) cudaHostUnregister(h->host_vp);
    if (h->host_sp) cudaHostUnregister(h->host_sp);
  }
  void* bufs[] = {h->Av, h->As, h->b, h->xv, h->xs, h->kind, h->period, h->delay,
                  h->snap_vp, h->snap_sp, h->phi_rcv, h->seis, h->fdt, h->hist, h->r1_err, h->xw};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int shaw_rom_set_signals(shaw_rom_t h, const int32_t* kind, const double* period, const double* delay) {
  if (!h || !kind || !period || !delay) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  for (uint32_t j = 0; j < h->M; ++j) {
    if (kind[j] < SHAW_SIGNAL_RICKER || kind[j] > SHAW_SIGNAL_GAUSS_DER)
      return shaw::fail(SHAW_ERR_INVALID_ARG, "unknown signal kind");
    if (!(period[j] > 0.0)) return shaw::fail(SHAW_ERR_INVALID_ARG, "Period for signal must be positive. ");
    if (!(delay[j] >= 0.0)) return shaw::fail(SHAW_ERR_INVALID_ARG, "Delay time of the signal must be >=0");
  }
  h->h_kind.assign(kind, kind + h->M);
  h->h_period.assign(period, period + h->M);
  h->h_delay.assign(delay, delay + h->M);
  SHAW_CUDA(cudaMemcpyAsync(h->kind, h->h_kind.data(), h->M * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  SHAW_CUDA(cudaMemcpyAsync(h->period, period, h->M * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SHAW_CUDA(cudaMemcpyAsync(h->delay, delay, h->M * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  h->signals_set = true;
  return SHAW_OK;
}

int shaw_rom_set_snapshots(shaw_rom_t h, uint64_t fvp, uint64_t fsp, uint64_t nsteps, double* host_vp,
                           double* host_sp) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  const bool device_snaps = h->rank == 1 || h->persistent2();  // collected on the device by persistent kernels
  if (!device_snaps) {
    if (h->host_vp) cudaHostUnregister(h->host_vp);
    if (h->host_sp) cudaHostUnregister(h->host_sp);
  }
  if (h->snap_vp) { cudaFree(h->snap_vp); h->snap_vp = nullptr; }
  if (h->snap_sp) { cudaFree(h->snap_sp); h->snap_sp = nullptr; }
  h->host_vp = h->host_sp = nullptr;
  h->fvp = h->fsp = h->snap_nsteps = 0;
  if (fvp == 0 && fsp == 0) return SHAW_OK;
  if (fvp == 0 || fsp == 0 || !host_vp || !host_sp)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "snapshot frequencies and arrays are required for both dofs");
  if (nsteps % fvp) return shaw::fail(SHAW_ERR_FREQ_DIVISOR, "Snapshot Vp frequency not a divisor of steps");
  if (nsteps % fsp) return shaw::fail(SHAW_ERR_FREQ_DIVISOR, "Snapshot Sp frequency not a divisor of steps");
  const size_t bvp = h->kv * (nsteps / fvp) * h->M * sizeof(double);
  const size_t bsp = h->ks * (nsteps / fsp) * h->M * sizeof(double);
  if (device_snaps) {
    SHAW_CUDA(cudaMalloc(&h->snap_vp, bvp));
    SHAW_CUDA(cudaMalloc(&h->snap_sp, bsp));
  } else {
    SHAW_CUDA(cudaHostRegister(host_vp, bvp, cudaHostRegisterDefault));
    const cudaError_t e = cudaHostRegister(host_sp, bsp, cudaHostRegisterDefault);
    if (e != cudaSuccess) {
      cudaHostUnregister(host_vp);
      return shaw::cuda_fail(e, "cudaHostRegister");
    }
  }
  h->host_vp = host_vp; h->host_sp = host_sp;
  h->fvp = fvp; h->fsp = fsp; h->snap_nsteps = nsteps;
  return SHAW_OK;
}

int shaw_rom_set_receivers(shaw_rom_t h, const double* phi_rows, uint32_t R, uint64_t freq, uint64_t nsteps) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  if (h->phi_rcv) { cudaFree(h->phi_rcv); h->phi_rcv = nullptr; }
  if (h->seis) { cudaFree(h->seis); h->seis = nullptr; }
  h->R = 0; h->fseis = 0; h->seis_T = 0; h->seis_nsteps = 0;
  if (h->oz)
    if (int rc = shaw::oz::set_receivers(h->oz, 0, nullptr, 0, nullptr, 0, 0, h->stream)) return rc;
  if (R == 0) return SHAW_OK;
  if (h->tc)
    return shaw::fail(SHAW_ERR_UNSUPPORTED,
                      "the TF32x3 rank-2 ROM records snapshots; form the seismogram from them");
  if (!phi_rows) return shaw::fail(SHAW_ERR_INVALID_ARG, "null receiver rows");
  if (freq == 0) return shaw::fail(SHAW_ERR_INVALID_ARG, "cannot have seismoFreq <=0 ");
  if (nsteps % freq) return shaw::fail(SHAW_ERR_FREQ_DIVISOR, "Seismogram sampling frequency not a divisor of steps");
  const uint64_t T = nsteps / freq;
  if (h->oz) {
    // the tensor-core kernel forms the seismogram in the loop, as an exact (Ozaki) product
    // of the sliced receiver rows with the sliced velocity state
    if (h->kv > 65535 || freq > 0xFFFFFFFFull) return shaw::fail(SHAW_ERR_UNSUPPORTED, "receiver setup too large");
    SHAW_CUDA(cudaMalloc(&h->seis, (size_t)R * T * h->M * sizeof(double)));
    SHAW_CUDA(cudaMemsetAsync(h->seis, 0, (size_t)R * T * h->M * sizeof(double), h->stream));
    if (int rc = shaw::oz::set_receivers(h->oz, 0, phi_rows, R, h->seis, T, (uint32_t)freq, h->stream)) return rc;
    h->R = R; h->fseis = freq; h->seis_T = T; h->seis_nsteps = nsteps;
    return SHAW_OK;
  }
  SHAW_CUDA(cudaMalloc(&h->phi_rcv, (size_t)R * h->kv * sizeof(double)));
  SHAW_CUDA(cudaMalloc(&h->seis, (size_t)R * T * h->M * sizeof(double)));
  SHAW_CUDA(cudaMemcpyAsync(h->phi_rcv, phi_rows, (size_t)R * h->kv * sizeof(double), cudaMemcpyHostToDevice,
                            h->stream));
  SHAW_CUDA(cudaMemsetAsync(h->seis, 0, (size_t)R * T * h->M * sizeof(double), h->stream));
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  h->R = R; h->fseis = freq; h->seis_T = T; h->seis_nsteps = nsteps;
  return SHAW_OK;
}

int shaw_rom_reset(shaw_rom_t h) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaMemsetAsync(h->xv, 0, h->kv * h->M * sizeof(double), h->stream));
  SHAW_CUDA(cudaMemsetAsync(h->xs, 0, h->ks * h->M * sizeof(double), h->stream));
  if (h->seis) SHAW_CUDA(cudaMemsetAsync(h->seis, 0, (size_t)h->R * h->seis_T * h->M * sizeof(double), h->stream));
  if (h->r1_err) SHAW_CUDA(cudaMemsetAsync(h->r1_err, 0, sizeof(unsigned int), h->stream));
  if (h->tc || h->oz) {
    const int rc = h->tc ? shaw::tc::reset(h->tc, h->stream) : shaw::oz::reset(h->oz, h->stream);
    if (rc) return rc;
  }
  h->step = 0;
  return SHAW_OK;
}

int shaw_rom_set_schedule(shaw_rom_t h, int schedule) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (schedule < SHAW_ROM_SCHEDULE_AUTO || schedule > SHAW_ROM_SCHEDULE_BANDS)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "unknown ROM schedule");
  if (schedule == SHAW_ROM_SCHEDULE_AUTO) {
    if (h->rank == 1 && h->precision == SHAW_FP64) h->band = h->band_ok;
    return SHAW_OK;
  }
  if (h->rank != 1 || h->precision != SHAW_FP64)
    return shaw::fail(SHAW_ERR_UNSUPPORTED, "ROM schedules other than AUTO apply to rank-1 FP64 handles");
  if (schedule == SHAW_ROM_SCHEDULE_BANDS && !h->band_ok)
    return shaw::fail(SHAW_ERR_UNSUPPORTED, "the row-band schedule needs at most 1024 modes per dof");
  if (schedule == SHAW_ROM_SCHEDULE_CLUSTER && !h->cluster_ok)
    return shaw::fail(SHAW_ERR_UNSUPPORTED, "the reduced operators do not fit the cluster kernel");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  h->band = schedule == SHAW_ROM_SCHEDULE_BANDS;
  return SHAW_OK;
}

int shaw_rom_advance(shaw_rom_t h, double dt, uint64_t nsteps) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (!(dt > 0.0) || !std::isfinite(dt)) return shaw::fail(SHAW_ERR_INVALID_ARG, "dt must be > 0");
  if (!h->signals_set) return shaw::fail(SHAW_ERR_STATE, "shaw_rom_set_signals must be called before stepping");
  if (h->fseis && h->step + nsteps > h->seis_nsteps)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "advancing past the step count the seismogram was sized for");
  if (h->fvp && h->step + nsteps > h->snap_nsteps)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "advancing past the step count the snapshots were sized for");
  if (nsteps == 0) return SHAW_OK;
  int rc = SHAW_OK;
  if (h->rank == 1) {  // launches of at most kR1MaxSteps steps (bounded forcing table and history)
    for (uint64_t done = 0; done < nsteps;) {
      const uint64_t k = std::min<uint64_t>(kR1MaxSteps, nsteps - done);
      rc = h->precision == SHAW_FP64 ? rank1_launch<false>(h, dt, k) : rank1_launch<true>(h, dt, k);
      if (rc) return rc;
      h->step += k;
      done += k;
    }
    return SHAW_OK;
  }
  if (h->tc || h->oz) {
    const unsigned long long Tv = h->fvp ? h->snap_nsteps / h->fvp : 0, Ts = h->fsp ? h->snap_nsteps / h->fsp : 0;
    if (h->tc) {
      rc = shaw::tc::advance(h->tc, h->stream, dt, h->step, nsteps, h->kind, h->period, h->delay, h->snap_vp,
                             h->snap_sp, Tv, Ts, (uint32_t)h->fvp, (uint32_t)h->fsp);
    } else {
      rc = shaw::oz::set_snapshots(h->oz, 0, h->snap_vp, h->snap_sp, Tv, Ts, (uint32_t)h->fvp, (uint32_t)h->fsp);
      if (rc == SHAW_OK) rc = shaw::oz::advance(h->oz, h->stream, dt, h->step, nsteps);
    }
    if (rc) return rc;
    h->launches++;
    h->step += nsteps;
    return SHAW_OK;
  }
  for (uint64_t s = 0; s < nsteps; ++s) {
    if ((rc = rank2_step(h, dt, h->step + 1))) return rc;
    h->step++;
  }
  return SHAW_OK;
}

int shaw_rom_synchronize(shaw_rom_t h) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  if (h->rank == 1 && h->r1_err) {
    unsigned int err = 0;
    SHAW_CUDA(cudaMemcpy(&err, h->r1_err, sizeof(err), cudaMemcpyDeviceToHost));
    if (err)
      return shaw::fail(SHAW_ERR_CUDA, "rank-1 ROM kernel: a row exchange wait ran out (code " +
                                           std::to_string(err) + ")");
  }
  if (h->rank == 1 && h->fvp) {
    // rank-1 snapshots are collected on the device; copy what the run produced
    const uint64_t Tv = std::min<uint64_t>(h->step / h->fvp, h->snap_nsteps / h->fvp);
    const uint64_t Ts = std::min<uint64_t>(h->step / h->fsp, h->snap_nsteps / h->fsp);
    SHAW_CUDA(cudaMemcpy(h->host_vp, h->snap_vp, h->kv * Tv * sizeof(double), cudaMemcpyDeviceToHost));
    SHAW_CUDA(cudaMemcpy(h->host_sp, h->snap_sp, h->ks * Ts * sizeof(double), cudaMemcpyDeviceToHost));
  }
  if (h->tc || h->oz) {
    const int rc = h->tc ? shaw::tc::check(h->tc, h->stream) : shaw::oz::check(h->oz, h->stream);
    if (rc) return rc;
    if (h->fvp) {
      const uint64_t Tv = h->snap_nsteps / h->fvp, Ts = h->snap_nsteps / h->fsp;
      SHAW_CUDA(cudaMemcpy(h->host_vp, h->snap_vp, h->kv * Tv * h->M * sizeof(double), cudaMemcpyDeviceToHost));
      SHAW_CUDA(cudaMemcpy(h->host_sp, h->snap_sp, h->ks * Ts * h->M * sizeof(double), cudaMemcpyDeviceToHost));
    }
  }
  return SHAW_OK;
}

int shaw_rom_run(shaw_rom_t h, double dt, uint64_t nsteps) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (h->fseis && nsteps != h->seis_nsteps)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "nsteps differs from the seismogram's step count");
  if (h->fvp && nsteps != h->snap_nsteps)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "nsteps differs from the snapshots' step count");
  int rc = shaw_rom_reset(h);
  if (rc) return rc;
  if ((rc = shaw_rom_advance(h, dt, nsteps))) return rc;
  return shaw_rom_synchronize(h);
}

int shaw_rom_get_state(shaw_rom_t h, double* xv, double* xs) {
  if (!h) return shaw::fail(SHAW_ERR_INVALID_ARG, "null handle");
  if (h->tc || h->oz) {
    const int rc = h->tc ? shaw::tc::get_state(h->tc, h->stream, h->xv, h->xs)
                         : shaw::oz::get_state(h->oz, 0, h->stream, h->xv, h->xs);
    if (rc) return rc;
  }
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  if (xv) SHAW_CUDA(cudaMemcpy(xv, h->xv, h->kv * h->M * sizeof(double), cudaMemcpyDeviceToHost));
  if (xs) SHAW_CUDA(cudaMemcpy(xs, h->xs, h->ks * h->M * sizeof(double), cudaMemcpyDeviceToHost));
  return SHAW_OK;
}

int shaw_rom_get_seismogram(shaw_rom_t h, double* out) {
  if (!h || !out) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  if (!h->seis) return shaw::fail(SHAW_ERR_STATE, "no receivers set");
  SHAW_CUDA(cudaStreamSynchronize(h->stream));
  SHAW_CUDA(cudaMemcpy(out, h->seis, (size_t)h->R * h->seis_T * h->M * sizeof(double), cudaMemcpyDeviceToHost));
  return SHAW_OK;
}

void* shaw_rom_stream(shaw_rom_t h) { return h ? (void*)h->stream : nullptr; }
uint64_t shaw_rom_kernel_launches(shaw_rom_t h) { return h ? h->launches : 0; }

// computeRomOperatorsUsingFomJacsWithMatProp (rom_compute_jacobians.hpp:83-102), FP64 on the GPU:
// tmp = J Phi with the matrix-free operator, then a cuBLAS DGEMM for Phi^T tmp.
int shaw_rom_project(shaw_fom_t fom, const double* phi_vp, uint64_t kv, const double* phi_sp, uint64_t ks,
                     double* rom_jvp, double* rom_jsp) {
  if (!fom || !phi_vp || !phi_sp || !rom_jvp || !rom_jsp) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  if (kv == 0 || ks == 0 || kv > 65535 || ks > 65535) return shaw::fail(SHAW_ERR_INVALID_ARG, "bad mode counts");
  uint64_t nvp = 0, nsp = 0;
  shaw::fom_sizes(fom, &nvp, &nsp);
  cudaStream_t s = (cudaStream_t)shaw_fom_stream(fom);
  cublasHandle_t blas = nullptr;
  double *pv = nullptr, *ps = nullptr, *tmp = nullptr, *out = nullptr;
  int rc = SHAW_OK;
  auto cleanup = [&]() {
    if (blas) cublasDestroy(blas);
    cudaFree(pv); cudaFree(ps); cudaFree(tmp); cudaFree(out);
  };
  cudaError_t e;
  if ((e = cudaMalloc(&pv, nvp * kv * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&ps, nsp * ks * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&tmp, std::max(nvp * ks, nsp * kv) * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&out, kv * ks * sizeof(double))) != cudaSuccess) {
    cleanup();
    return shaw::cuda_fail(e, "cudaMalloc (projection)");
  }
  if (cublasCreate(&blas) != CUBLAS_STATUS_SUCCESS || cublasSetStream(blas, s) != CUBLAS_STATUS_SUCCESS) {
    cleanup();
    return shaw::fail(SHAW_ERR_CUDA, "cublas init failed");
  }
  const double one = 1.0, zero = 0.0;
  do {
    if ((e = cudaMemcpyAsync(pv, phi_vp, nvp * kv * sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(ps, phi_sp, nsp * ks * sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess) {
      rc = shaw::cuda_fail(e, "cudaMemcpyAsync (basis)");
      break;
    }
    // tmp (nvp x ks) = Jvp PhiSp ; romJvp row-major kv x ks == column-major ks x kv = tmp^T PhiVp
    if ((rc = shaw::fom_apply(fom, 0, ps, tmp, 0, nvp, (uint32_t)ks, s))) break;
    if (cublasDgemm(blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)ks, (int)kv, (int)nvp, &one, tmp, (int)nvp, pv, (int)nvp,
                    &zero, out, (int)ks) != CUBLAS_STATUS_SUCCESS) {
      rc = shaw::fail(SHAW_ERR_CUDA, "cublasDgemm (projection vp)");
      break;
    }
    if ((e = cudaMemcpyAsync(rom_jvp, out, kv * ks * sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess) {
      rc = shaw::cuda_fail(e, "cudaMemcpyAsync (romJvp)");
      break;
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) { rc = shaw::cuda_fail(e, "sync"); break; }
    // tmp (nsp x kv) = Jsp PhiVp ; romJsp row-major ks x kv == column-major kv x ks = tmp^T PhiSp
    if ((rc = shaw::fom_apply(fom, 1, pv, tmp, 0, nsp, (uint32_t)kv, s))) break;
    if (cublasDgemm(blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)kv, (int)ks, (int)nsp, &one, tmp, (int)nsp, ps, (int)nsp,
                    &zero, out, (int)kv) != CUBLAS_STATUS_SUCCESS) {
      rc = shaw::fail(SHAW_ERR_CUDA, "cublasDgemm (projection sp)");
      break;
    }
    if ((e = cudaMemcpyAsync(rom_jsp, out, kv * ks * sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess) {
      rc = shaw::cuda_fail(e, "cudaMemcpyAsync (romJsp)");
      break;
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) { rc = shaw::cuda_fail(e, "sync"); break; }
  } while (false);
  cudaStreamSynchronize(s);
  cleanup();
  return rc;
}

}  // extern "C"

// ---- projection without allocation --------------------------------------------------
// Some callers cannot allocate device memory during a call: a host application that
// hands the library a fixed memory budget up front, a code path that runs where
// allocation is forbidden or would synchronise the device, or a runtime that
// manages every device allocation itself.  For them the projection below keeps
// its intermediate J * Phi block in one fixed, statically sized device array.
//
// The projection runs over blocks of mesh rows: for rows n0 .. n1 of the output
// dof, T = (J PhiIn)[n0:n1, :] (all k_in columns) goes to the array, and
// out += PhiOut[n0:n1, :]^T T accumulates in a tiled FP64 kernel, blocks in a fixed
// order.  Every basis value is read about once, so the cost grows with
// n * k_in * k_out flops, like the allocating path's DGEMM, for any mesh size.
//
// The array lives for as long as the library is loaded, on every GPU that loads
// it.  Host code must not pass the array's name to a kernel (in host code that
// name is a host-side stand-in, not a device address): its device address is
// looked up with cudaGetSymbolAddress on each call, for the current device.  All
// calls share the array, so calls whose work overlaps on the GPU (different
// streams, or threads without ordering) race on it; the array keeps whatever the
// last call left in it, and every element this code reads is written first within
// the same call.
namespace {

constexpr uint64_t kProjectScratchDoubles = 1ull << 21;  // 16 MiB of FP64
static __device__ __align__(256) double g_project_scratch[kProjectScratchDoubles];

// Device address of the scratch array on the current device.  The lookup does not
// allocate; the first one on a device may load the module, so a caller makes its
// first call before any stream capture.
int project_scratch(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_project_scratch);
  if (e != cudaSuccess) return shaw::cuda_fail(e, "cudaGetSymbolAddress(project scratch)");
  *out = static_cast<double*>(p);
  return SHAW_OK;
}

constexpr int kProjTile = 32;  // output tile (k_out x k_in) of one CTA, and rows per K step

// out[i * k_in + j] (=, or += when accumulate) sum_{r < nrows} phi_out[(row0 + r) + n_out * i] * t[r + nrows * j]
// for i < k_out, j < k_in: a 32 x 32 output tile per CTA, 256 threads with 2 x 2 outputs
// each, both operands staged through shared memory 32 rows at a time (FP64 FMAs).
__global__ void __launch_bounds__(256) rom_project_accum_kernel(const double* __restrict__ phi_out, uint64_t n_out,
                                                                uint64_t row0, uint32_t nrows,
                                                                const double* __restrict__ t, uint32_t k_out,
                                                                uint32_t k_in, double* __restrict__ out,
                                                                int accumulate) {
  __shared__ double sa[kProjTile][kProjTile + 1];
  __shared__ double sb[kProjTile][kProjTile + 1];
  const uint32_t i0 = blockIdx.y * kProjTile, j0 = blockIdx.x * kProjTile;
  const uint32_t tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (uint32_t r0 = 0; r0 < nrows; r0 += kProjTile) {
    // 32 rows x 32 columns of each operand: thread (tid & 31) walks the rows (coalesced)
    for (uint32_t e = tid; e < kProjTile * kProjTile; e += 256) {
      const uint32_t rr = e & 31, cc = e >> 5;
      const bool in_r = r0 + rr < nrows;
      sa[rr][cc] = (in_r && i0 + cc < k_out) ? phi_out[(row0 + r0 + rr) + n_out * (i0 + cc)] : 0.0;
      sb[rr][cc] = (in_r && j0 + cc < k_in) ? t[(r0 + rr) + (size_t)nrows * (j0 + cc)] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (uint32_t rr = 0; rr < kProjTile; ++rr) {
      const double a0 = sa[rr][2 * ty], a1 = sa[rr][2 * ty + 1];
      const double b0 = sb[rr][2 * tx], b1 = sb[rr][2 * tx + 1];
      acc[0][0] = fma(a0, b0, acc[0][0]);
      acc[0][1] = fma(a0, b1, acc[0][1]);
      acc[1][0] = fma(a1, b0, acc[1][0]);
      acc[1][1] = fma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const uint32_t i = i0 + 2 * ty + a, j = j0 + 2 * tx + b;
      if (i < k_out && j < k_in) {
        double* o = out + (size_t)i * k_in + j;
        *o = accumulate ? *o + acc[a][b] : acc[a][b];
      }
    }
}

// out (k_out x k_in, row-major) = PhiOut^T (J PhiIn), over row blocks of the scratch array.
int project_block(shaw_fom_t fom, int dof, const double* phi_in, uint64_t k_in, const double* phi_out,
                  uint64_t n_out, uint64_t k_out, double* out, double* scratch, cudaStream_t s) {
  uint64_t rows = kProjectScratchDoubles / k_in;  // >= 32 for k_in <= 65535
  rows -= rows % kProjTile;
  const dim3 grid((unsigned)((k_in + kProjTile - 1) / kProjTile), (unsigned)((k_out + kProjTile - 1) / kProjTile));
  for (uint64_t n0 = 0; n0 < n_out; n0 += rows) {
    const uint64_t nb = (n_out - n0 < rows) ? n_out - n0 : rows;
    int rc = shaw::fom_apply(fom, dof, phi_in, scratch, n0, nb, (uint32_t)k_in, s);
    if (rc) return rc;
    rom_project_accum_kernel<<<grid, 256, 0, s>>>(phi_out, n_out, n0, (uint32_t)nb, scratch, (uint32_t)k_out,
                                                  (uint32_t)k_in, out, n0 == 0 ? 0 : 1);
    SHAW_CUDA(cudaGetLastError());
  }
  return SHAW_OK;
}

}  // namespace

extern "C" int shaw_rom_project_noalloc(shaw_fom_t fom, const double* d_phi_vp, uint64_t kv, const double* d_phi_sp,
                                        uint64_t ks, double* d_rom_jvp, double* d_rom_jsp, void* stream) {
  if (!fom || !d_phi_vp || !d_phi_sp || !d_rom_jvp || !d_rom_jsp)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  if (kv == 0 || ks == 0 || kv > 65535 || ks > 65535)
    return shaw::fail(SHAW_ERR_INVALID_ARG,
                      "bad mode counts for the allocation-free projection: kv and ks must be in 1..65535 "
                      "(a row block of J*Phi with every mode column must fit the 16 MiB scratch array)");
  uint64_t nvp = 0, nsp = 0;
  shaw::fom_sizes(fom, &nvp, &nsp);
  double* scratch = nullptr;
  int rc = project_scratch(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // romJvp (kv x ks) = PhiVp^T (Jvp PhiSp);  romJsp (ks x kv) = PhiSp^T (Jsp PhiVp)
  if ((rc = project_block(fom, 0, d_phi_sp, ks, d_phi_vp, nvp, kv, d_rom_jvp, scratch, s))) return rc;
  return project_block(fom, 1, d_phi_vp, kv, d_phi_sp, nsp, ks, d_rom_jsp, scratch, s);
}
