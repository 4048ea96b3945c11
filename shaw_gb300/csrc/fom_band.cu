// fom_band.cu -- the rank-1 FOM leapfrog of a small grid as ONE persistent cooperative launch.
//
// runFom (src/kokkos/fom_run.hpp:97-149) on a grid such as 101 theta x 201 r (60,601
// DOFs) does a fraction of a microsecond of FP64 work per step spread over the GPU, so
// the two half-step launches, not arithmetic, bound the step.  Here one cooperative grid
// (all CTAs co-resident, one per SM) runs all the steps of a call.  CTA b owns a band of
// `rows` r rows and keeps in shared memory its velocity rows plus the row above (a halo),
// its srp rows plus the row below (a halo), its stp rows, and the folded stencil values
// of all of them.  Per step:
//   1. v of the band (the two-pass velocity kernel's FMAs, same order) and the forcing;
//      the band's lowest v row goes straight from the registers to band b - 1;
//   2. wait for the halo v row from band b + 1; the receivers of the band;
//   3. sigma of the band (the stress kernel's FMAs, same order); the band's highest srp
//      row goes straight to band b + 1;
//   4. wait for the halo srp row from band b - 1.
// Rows travel through L2 as self-validating 8-byte words: each carries 32 bits of the
// double and a 32-bit tag naming the step, so a reader polls the data itself; no flag,
// fence or second round trip follows the data.  Each 8-byte word is written and read by
// single-copy-atomic accesses, so a word is never seen half old and half new.  Tags grow
// monotonically over the life of the buffers (the host clears them before the 32-bit tag
// would wrap), so a word left by an earlier step or launch never matches.  One word pair
// per point and direction suffices: band b overwrites its row of step n only after it
// has received the neighbour's row of step n - 1, which that neighbour sends after it has
// consumed b's row of step n - 1.
// Results are bit-identical to the two half-step kernels.  Every wait is bounded: a wait
// that runs out sets ctl->error bit 1 and the CTA leaves the loop; its neighbours' waits
// then run out in turn, so the launch always ends.
#include <cuda_runtime.h>

#include <cstring>

#include "fom_band.h"
#include "shaw_internal.h"

namespace shaw {
namespace band {

constexpr uint32_t kThreads = 256;
constexpr int kBatch = 4;                      // elements of a phase per thread, processed side by side
constexpr uint32_t kPollLimit = 1u << 22;      // polls of one word pair before a wait gives up (about a second)

// Doubles of shared memory a CTA with `rows` rows needs.
inline size_t smem_doubles(uint32_t nth, uint32_t rows) {
  return (size_t)(rows + 1) * nth * 2 + (size_t)rows * (nth - 1) + (size_t)4 * rows * nth + (size_t)2 * rows * nth +
         (size_t)2 * rows * (nth - 1);
}

namespace {

// One point of a halo row: two words (tag | high half, tag | low half), one 16-byte store.
// The vector access is two 8-byte accesses, each single-copy atomic; each is validated alone.
__device__ __forceinline__ void put(unsigned long long* w, uint32_t tag, double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const unsigned long long t = (unsigned long long)tag << 32;
  asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(w), "l"(t | (u >> 32)),
               "l"(t | (u & 0xffffffffull))
               : "memory");
}
// Bounded wait for the point tagged `tag`; false when the poll limit runs out.
__device__ __forceinline__ bool get(const unsigned long long* w, uint32_t tag, double* v) {
  for (uint32_t k = 0; k < kPollLimit; ++k) {
    unsigned long long hi, lo;
    asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(hi), "=l"(lo) : "l"(w) : "memory");
    if ((uint32_t)(hi >> 32) == tag && (uint32_t)(lo >> 32) == tag) {
      *v = __longlong_as_double((long long)((hi << 32) | (lo & 0xffffffffull)));
      return true;
    }
  }
  return false;
}

// The forcing increments of the steps of a launch: ftab[s] = (dt rhoInv[src]) f(t) at
// t = (step0 + s) dt, rounded as KokkosBlas::mult(1, x, dt, rhoInv, f) forms them, so the
// kernel adds each with one FP64 add (the same roundings as the half-step kernels).
__global__ void fom_band_forcing_kernel(Args a) {
  const unsigned long long s = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  if (s >= a.nsteps) return;
  const double f = shaw::signal_value(a.kind, a.delay, a.period, (double)(a.step0 + s) * a.dt);
  a.ftab[s] = __dmul_rn(__dmul_rn(a.dt, a.rho_inv[a.src]), f);
}

__global__ void __launch_bounds__(kThreads, 1) fom_band_kernel(const Args a) {
  const uint32_t b = blockIdx.x;
  const uint32_t nth = a.nth, nr = a.nr, rows = a.rows;
  const uint32_t j0 = b * rows, j1 = min(nr, j0 + rows), nrow = j1 - j0;  // plan: every band owns rows
  const bool up = j1 < nr;   // a band above exists (halo row v(j1) from it, srp row j1 - 1 to it)
  const bool down = j0 > 0;  // a band below exists (halo row srp(j0 - 1) from it, v row j0 to it)
  const uint32_t sp_row = 2 * nth - 1;
  const size_t nvp = (size_t)nth * nr, nsp = (size_t)(nr - 1) * nth + (size_t)nr * (nth - 1);
  extern __shared__ __align__(16) double sm[];
  double* const V = sm;                                // (rows + 1) x nth: v rows j0 .. j1
  double* const SRP = V + (size_t)(rows + 1) * nth;    // (rows + 1) x nth: srp rows j0 - 1 .. j1 - 1
  double* const STP = SRP + (size_t)(rows + 1) * nth;  // rows x (nth - 1)
  double* const CV = STP + (size_t)rows * (nth - 1);   // 4 x rows x nth
  double* const CSR = CV + (size_t)4 * rows * nth;     // 2 x rows x nth (srp rows j0 .. j1 - 1)
  double* const CST = CSR + (size_t)2 * rows * nth;    // 2 x rows x (nth - 1)
  const uint32_t nv = rows * nth, ns = rows * (nth - 1);
  unsigned long long* const send_down = a.xdown + (size_t)b * nth * 2;
  unsigned long long* const send_up = a.xup + (size_t)b * nth * 2;
  const unsigned long long* const recv_above = up ? a.xdown + (size_t)(b + 1) * nth * 2 : nullptr;
  const unsigned long long* const recv_below = down ? a.xup + (size_t)(b - 1) * nth * 2 : nullptr;

  // the band, its halos and its stencil values
  for (uint32_t e = threadIdx.x; e < (nrow + (up ? 1 : 0)) * nth; e += kThreads) V[e] = a.xv[(size_t)j0 * nth + e];
  for (uint32_t e = threadIdx.x; e < (rows + 1) * nth; e += kThreads) {
    const uint32_t rl = e / nth, i = e - rl * nth;
    const int j = (int)j0 - 1 + (int)rl;  // srp row
    SRP[e] = (j >= 0 && j + 1 < (int)nr && j < (int)j1) ? a.xs[(size_t)j * sp_row + 2 * i] : 0.0;
  }
  for (uint32_t e = threadIdx.x; e < nrow * (nth - 1); e += kThreads) {
    const uint32_t rl = e / (nth - 1), i = e - rl * (nth - 1), j = j0 + rl;
    const size_t q = (j + 1 < nr) ? (size_t)j * sp_row + 2 * i + 1 : (size_t)j * sp_row + i;
    STP[e] = a.xs[q];
    CST[e] = a.csp[q];
    CST[ns + e] = a.csp[nsp + q];
  }
  for (uint32_t e = threadIdx.x; e < nrow * nth; e += kThreads) {
    const size_t p = (size_t)j0 * nth + e;
    for (int c = 0; c < 4; ++c) CV[c * nv + e] = a.cvp[c * nvp + p];
    const uint32_t rl = e / nth, i = e - rl * nth, j = j0 + rl;
    if (j + 1 < nr) {
      const size_t q = (size_t)j * sp_row + 2 * i;
      CSR[e] = a.csp[q];
      CSR[nv + e] = a.csp[nsp + q];
    }
  }
  // This thread's elements, fixed for every step.  Velocity element k is band point
  // e = t + k kThreads in row order, so the lowest row (sent down) comes first.  Stress
  // element k counts the rows from the top, so the highest srp row (sent up) comes first.
  int ev[kBatch], eN[kBatch], eS[kBatch], eW[kBatch], es[kBatch], est[kBatch], estW[kBatch];
  bool interior[kBatch], send_v[kBatch], send_s[kBatch];
  int src_k = -1;
#pragma unroll
  for (int k = 0; k < kBatch; ++k) {
    const uint32_t e = threadIdx.x + k * kThreads;
    ev[k] = es[k] = est[k] = -1;
    interior[k] = send_v[k] = send_s[k] = false;
    if (e < nrow * nth) {
      const uint32_t rl = e / nth, i = e - rl * nth, j = j0 + rl;
      ev[k] = (int)e;
      interior[k] = i != 0 && i + 1 != nth;
      eN[k] = (j + 1 < nr) ? (int)((rl + 1) * nth + i) : (int)(rl * nth + i);  // srp(j) or, at the surface, srp(j - 1)
      eS[k] = (j > 0) ? (int)(rl * nth + i) : (int)((rl + 1) * nth + i);      // srp(j - 1) or, at the CMB, srp(j)
      eW[k] = (int)(rl * (nth - 1) + i) - 1;                                   // stp(j, i - 1); stp(j, i) follows
      send_v[k] = down && rl == 0;
      if ((unsigned long long)j * nth + i == a.src) src_k = k;
      const uint32_t rs = nrow - 1 - rl;  // stress: the same point set, rows counted from the top
      if (j0 + rs + 1 < nr) {
        es[k] = (int)(rs * nth + i);  // srp(j0 + rs, i) is SRP[es + nth]; v(j0 + rs, i) is V[es]
        send_s[k] = up && rs == nrow - 1;
      }
    }
    if (e < nrow * (nth - 1)) {
      const uint32_t rs = nrow - 1 - e / (nth - 1), i = e % (nth - 1);
      est[k] = (int)(rs * (nth - 1) + i);
      estW[k] = (int)(rs * nth + i);  // v(j, i) in V; v(j, i + 1) follows
    }
  }
  __syncthreads();

  for (unsigned long long it = 0; it < a.nsteps; ++it) {
    const unsigned long long n = a.step0 + it + 1;
    const uint32_t tag = a.tag0 + (uint32_t)it;
    // 1. velocity (each thread reads and writes only its own v elements in this phase)
    {
      double v[kBatch], c[kBatch][4], x[kBatch][4];
#pragma unroll
      for (int k = 0; k < kBatch; ++k) {
        if (ev[k] < 0) continue;
        v[k] = V[ev[k]];
        if (interior[k]) {
#pragma unroll
          for (int q = 0; q < 4; ++q) c[k][q] = CV[q * nv + ev[k]];
          x[k][0] = SRP[eN[k]];
          x[k][1] = SRP[eS[k]];
          x[k][2] = STP[eW[k]];
          x[k][3] = STP[eW[k] + 1];
        }
      }
      const double fdt = src_k >= 0 ? a.ftab[it] : 0.0;
#pragma unroll
      for (int k = 0; k < kBatch; ++k) {
        if (ev[k] < 0) continue;
        if (interior[k]) {
#pragma unroll
          for (int q = 0; q < 4; ++q) v[k] = fma(c[k][q], x[k][q], v[k]);
        }
        if (k == src_k) v[k] = __dadd_rn(v[k], fdt);
        if (send_v[k]) put(send_down + 2 * ev[k], tag, v[k]);
        V[ev[k]] = v[k];
      }
    }
    // 2. the halo v row j1 from the band above
    bool ok = true;
    if (up)
      for (uint32_t i = threadIdx.x; i < nth; i += kThreads) {
        double x;
        if (get(recv_above + 2 * i, tag, &x))
          V[(size_t)nrow * nth + i] = x;
        else
          ok = false;
      }
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(&a.ctl->error, 1u);
      break;
    }
    // the receivers of the band (Seismogram::storeVelocitySignalAtReceivers)
    if (a.seis_freq && n % a.seis_freq == 0) {
      const unsigned long long cnt = n / a.seis_freq - 1;
      for (uint32_t r = threadIdx.x; r < a.R; r += kThreads) {
        const unsigned long long g = a.rcv[r];
        if (g >= (unsigned long long)j0 * nth && g < (unsigned long long)j1 * nth && cnt < a.seis_T) {
          const double val = V[g - (unsigned long long)j0 * nth];
          a.seis[r + (size_t)a.R * cnt] = val;
          if (!isfinite(val)) atomicOr(&a.ctl->nonfinite, 1u);
        }
      }
    }
    // 3. stress (each thread reads and writes only its own stress elements; v is fixed)
    {
      double sr[kBatch], st[kBatch];
#pragma unroll
      for (int k = 0; k < kBatch; ++k) {
        if (es[k] >= 0) {
          const int e = es[k];
          sr[k] = SRP[e + nth];
          sr[k] = fma(CSR[e], V[e + nth], sr[k]);  // north v(j + 1, i)
          sr[k] = fma(CSR[nv + e], V[e], sr[k]);   // south v(j, i)
          if (send_s[k]) put(send_up + 2 * (e - (nrow - 1) * nth), tag, sr[k]);
        }
        if (est[k] >= 0) {
          const int e = est[k];
          st[k] = STP[e];
          st[k] = fma(CST[e], V[estW[k]], st[k]);           // west v(j, i)
          st[k] = fma(CST[ns + e], V[estW[k] + 1], st[k]);  // east v(j, i + 1)
        }
      }
#pragma unroll
      for (int k = 0; k < kBatch; ++k) {
        if (es[k] >= 0) SRP[es[k] + nth] = sr[k];
        if (est[k] >= 0) STP[est[k]] = st[k];
      }
    }
    // 4. the halo srp row j0 - 1 from the band below
    if (down)
      for (uint32_t i = threadIdx.x; i < nth; i += kThreads) {
        double x;
        if (get(recv_below + 2 * i, tag, &x))
          SRP[i] = x;
        else
          ok = false;
      }
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(&a.ctl->error, 1u);
      break;
    }
  }
  // the band back to the state
  for (uint32_t e = threadIdx.x; e < nrow * nth; e += kThreads) a.xv[(size_t)j0 * nth + e] = V[e];
  for (uint32_t e = threadIdx.x; e < nrow * nth; e += kThreads) {
    const uint32_t rl = e / nth, i = e - rl * nth, j = j0 + rl;
    if (j + 1 < nr) a.xs[(size_t)j * sp_row + 2 * i] = SRP[(rl + 1) * nth + i];
  }
  for (uint32_t e = threadIdx.x; e < nrow * (nth - 1); e += kThreads) {
    const uint32_t rl = e / (nth - 1), i = e - rl * (nth - 1), j = j0 + rl;
    const size_t q = (j + 1 < nr) ? (size_t)j * sp_row + 2 * i + 1 : (size_t)j * sp_row + i;
    a.xs[q] = STP[e];
  }
}

}  // namespace

bool plan(uint32_t nth, uint32_t nr, uint32_t* bands, uint32_t* rows, size_t* smem) {
  if (nth < 3 || nr < 2) return false;
  int dev = 0, sms = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return false;
  // the fewest rows per band with one band per SM; the grid needs at least two bands
  const uint32_t r = (nr + (uint32_t)sms - 1) / (uint32_t)sms;
  const uint32_t g = (nr + r - 1) / r;
  if (g < 2) return false;
  if ((size_t)r * nth > (size_t)kBatch * kThreads) return false;  // a band is at most kBatch points a thread
  const size_t bytes = smem_doubles(nth, r) * sizeof(double);
  if (bytes + 1024 > (size_t)optin) return false;
  if (cudaFuncSetAttribute(fom_band_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fom_band_kernel, kThreads, bytes) != cudaSuccess ||
      (size_t)per_sm * sms < g) {
    cudaGetLastError();
    return false;
  }
  *bands = g;
  *rows = r;
  *smem = bytes;
  return true;
}

int launch(const Args& a, uint32_t bands, size_t smem, cudaStream_t s) {
  fom_band_forcing_kernel<<<(unsigned)((a.nsteps + 255) / 256), 256, 0, s>>>(a);
  SHAW_CUDA(cudaGetLastError());
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(bands);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;  // every band co-resident, or the launch fails
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SHAW_CUDA(cudaLaunchKernelEx(&cfg, fom_band_kernel, a));
  return SHAW_OK;
}

}  // namespace band
}  // namespace shaw
