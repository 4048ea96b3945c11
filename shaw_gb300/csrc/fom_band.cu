// fom_band.cu -- the rank-1 FOM leapfrog of a small grid as ONE persistent cooperative launch.
//
// runFom (src/kokkos/fom_run.hpp:97-149) on a grid such as 101 theta x 201 r (60,601
// DOFs) does a fraction of a microsecond of FP64 work per step spread over the GPU, so
// the two half-step launches, not arithmetic, bound the step.  Here one cooperative grid
// (all CTAs co-resident, one per SM) runs all the steps of a call.  CTA b owns a band of
// `rows` r rows j0 .. j1 - 1 and keeps in shared memory its velocity rows plus v(j1), its
// srp rows plus srp(j0 - 1) and srp(j1), its stp rows plus stp(j1, .), and the folded
// stencil values of all of them.  Row j1 belongs to band b + 1, which computes the same
// v(j1) from the same inputs; computing it here too spares one exchange per step.
//
// The step is ordered so that only what a neighbour waits for lies between receiving and
// sending.  The "edge" velocity rows are those that read a received row: j0 (when a band
// exists below) and j1 (when one exists above); all other velocity rows are "interior".
//   1. v of the edge rows (the two-pass velocity kernel's FMAs, same order, and the
//      forcing);
//   2. sigma of the srp rows and of the stp row j0 (the stress kernel's FMAs, same order);
//      the band's lowest srp and stp rows go straight from the registers to band b - 1,
//      its highest srp row to band b + 1;
//   3. while those rows travel: sigma of the other stp rows, the receivers of the band,
//      and v of the interior rows for the NEXT step (they read only this band's rows);
//   4. wait for srp(j1) and stp(j1, .) from band b + 1 and srp(j0 - 1) from band b - 1.
// When the step-3 work fits the warps left over, 3 and 4 run side by side: the first
// warps (one lane per received point) poll from the moment their rows are sent, the others
// do the step-3 work, and the two groups meet at a named barrier before v is overwritten.
// Rows travel through L2 as tagged words (l2_exchange.cuh), the tag naming the step; the
// host clears the words before the 32-bit tag would wrap.  Each direction has two slots,
// by step parity: band b writes its rows of step n + 2 into the slot of step n only after
// it has received the neighbour's rows of step n + 1, which that neighbour sends after it
// has read b's rows of step n.
// Results are bit-identical to the two half-step kernels.  Every wait is bounded: a wait
// that runs out sets ctl->error bit 1 and the CTA leaves the loop; its neighbours' waits
// then run out in turn, so the launch always ends.
#include <cuda_runtime.h>

#include <cstring>

#include "fom_band.h"
#include "l2_exchange.cuh"
#include "shaw_internal.h"

namespace shaw {
namespace band {

constexpr uint32_t kThreads = 512;
constexpr int kBatch = 2;                      // elements of a set per thread, processed side by side

// Doubles of shared memory a CTA with `rows` rows needs.
inline size_t smem_doubles(uint32_t nth, uint32_t rows) {
  return (size_t)(rows + 1) * nth + (size_t)(rows + 2) * nth + (size_t)(rows + 1) * (nth - 1) +
         (size_t)4 * (rows + 1) * nth + (size_t)2 * rows * nth + (size_t)2 * rows * (nth - 1);
}

namespace {

// The forcing increments of the steps of a launch: ftab[s] = (dt rhoInv[src]) f(t) at
// t = (step0 + s) dt, rounded as KokkosBlas::mult(1, x, dt, rhoInv, f) forms them, so the
// kernel adds each with one FP64 add (the same roundings as the half-step kernels).
__global__ void fom_band_forcing_kernel(Args a) {
  const unsigned long long s = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  if (s >= a.nsteps) return;
  const double f = shaw::signal_value(a.kind, a.delay, a.period, (double)(a.step0 + s) * a.dt);
  a.ftab[s] = __dmul_rn(__dmul_rn(a.dt, a.rho_inv[a.src]), f);
}

// A set of velocity points of this thread: p = place in V (-1 when absent) and a packed
// word m: bit 0 = interior theta point (the stencil applies), bit 1 = N is srp(j) (else
// srp(j - 1), at the surface), bit 2 = S is srp(j - 1) (else srp(j), at the CMB), bits 3..
// = the local row rl.  In SRP, srp(j) is at p + nth and srp(j - 1) at p; in STP,
// stp(j, i - 1) is at p - rl - 1 and stp(j, i) follows.
struct VelSet {
  int p[kBatch], m[kBatch];
};

// updateVelocity of a set (fom_velocity_kernel's FMAs, same order), plus the forcing of the
// source point when FORCE: only the warp holding the source runs that form, so the other
// warps issue no FP64 add on the narrow FP64 pipe.
template <bool FORCE>
__device__ __forceinline__ void velocity(const VelSet& e, double* V, const double* SRP, const double* STP,
                                         const double* CV, uint32_t nv, uint32_t nth, int src_p, double fdt) {
#pragma unroll
  for (int k = 0; k < kBatch; ++k) {
    if (e.p[k] < 0) continue;
    const int p = e.p[k], m = e.m[k];
    double v = V[p];
    if (m & 1) {
      const int w = p - (m >> 3) - 1;
      v = fma(CV[p], SRP[(m & 2) ? p + (int)nth : p], v);           // N
      v = fma(CV[nv + p], SRP[(m & 4) ? p : p + (int)nth], v);      // S
      v = fma(CV[2 * nv + p], STP[w], v);                           // W
      v = fma(CV[3 * nv + p], STP[w + 1], v);                       // E
    }
    if (FORCE && p == src_p) v = __dadd_rn(v, fdt);  // after the FMAs, as the half-step kernel
    V[p] = v;
  }
}

// The halo rows of a step, points q = t, t + nt, ... (at most kRecvMax) of the received set:
// first the message from above (srp(j1) when it exists, then stp(j1, .)), then srp(j0 - 1)
// from below.  Each round issues the loads of all the thread's pending points before it
// checks any, so their round trips overlap.
constexpr int kRecvMax = 3;  // received points per thread: 3 nth - 1 <= 3 kThreads for nth <= 512
__device__ __forceinline__ bool receive(const unsigned long long* recv_above, const unsigned long long* recv_below,
                                        uint32_t slot, uint32_t tag, size_t down_pts, size_t up_pts,
                                        uint32_t n_above, uint32_t n_recv, bool srp_above, uint32_t nth,
                                        uint32_t nrow, double* SRP, double* STP, uint32_t t, uint32_t nt) {
  const unsigned long long* src[kRecvMax];
  double* dst[kRecvMax];  // (both filled for the pending points only)
  uint32_t pending = 0;
#pragma unroll
  for (int k = 0; k < kRecvMax; ++k) {
    const uint32_t q = t + k * nt;
    src[k] = nullptr;
    dst[k] = nullptr;
    if (q >= n_recv) continue;
    pending |= 1u << k;
    if (q < n_above) {
      const uint32_t pa = srp_above ? q : q + nth;  // point of the message from above
      src[k] = recv_above + (size_t)slot * down_pts * 2 + 2 * pa;
      dst[k] = pa < nth ? SRP + (size_t)(nrow + 1) * nth + pa : STP + (size_t)nrow * (nth - 1) + (pa - nth);
    } else {
      const uint32_t pb = q - n_above;
      src[k] = recv_below + (size_t)slot * up_pts * 2 + 2 * pb;
      dst[k] = SRP + pb;
    }
  }
  return l2x::poll<kRecvMax>(src, dst, pending, tag);
}

// The time loop shared by the row and the column band kernels (steps 1-4 above, the roles,
// the barriers and the bounded waits).  The orientation's work comes in as callables:
// vel_edge(it) / vel_int(it) the velocity of the edge / interior lines of step it,
// send(tag, slot) the stress of the lines a neighbour waits for (each put as it is formed),
// unsent() the stress of the other lines, recv(slot, tag, t, nt) the halo lines (points t,
// t + nt, ...).  V is the band's velocity; the band's receivers have keys in [key0, key1)
// of the key-ordered list, each at V[key - key0].
template <class VelE, class VelI, class Send, class Unsent, class Recv>
__device__ __forceinline__ void band_steps(const Args& a, const double* V, unsigned long long key0,
                                           unsigned long long key1, bool split, bool poller, bool worker, uint32_t wt,
                                           uint32_t nwt, uint32_t npt, VelE vel_edge, VelI vel_int, Send send,
                                           Unsent unsent, Recv recv) {
  // the receivers: a range of the list; the sampling phase and the sample count before the
  // launch's first step (step step0 + 1)
  __shared__ uint32_t s_rcv[2];
  if (threadIdx.x < 2) {
    const unsigned long long key = threadIdx.x ? key1 : key0;
    uint32_t lo = 0, hi = a.R;  // first entry with key >= key
    while (lo < hi) {
      const uint32_t mid = lo + (hi - lo) / 2;
      if (a.rcv_sorted[2 * (size_t)mid] < key) lo = mid + 1; else hi = mid;
    }
    s_rcv[threadIdx.x] = lo;
  }
  uint32_t phase = a.seis_freq ? (uint32_t)(a.step0 % a.seis_freq) : 0;
  uint32_t sample = 0;  // clamped at seis_T: samples past the seismogram's length are dropped
  if (a.seis_freq) {
    const unsigned long long s0 = a.step0 / a.seis_freq;
    sample = s0 < a.seis_T ? (uint32_t)s0 : a.seis_T;
  }
  __syncthreads();
  const uint32_t rcv_lo = s_rcv[0], rcv_hi = s_rcv[1];

  if (a.nsteps > 0) vel_int(0ull);  // the interior lines of the first step
  for (unsigned long long it = 0; it < a.nsteps; ++it) {
    const uint32_t tag = a.tag0 + (uint32_t)it;
    const uint32_t slot = (uint32_t)(it & 1);
    // 1. velocity of the edge lines (each thread reads and writes only its own v elements)
    vel_edge(it);
    __syncthreads();
    // 2. stress of the lines a neighbour waits for; each goes out as soon as it is formed
    //    (each thread reads and writes only its own stress elements; v is fixed)
    send(tag, slot);
    // 3. while the lines travel: the other stress lines, the receivers, the next interior
    //    velocity (workers); 4. the halo lines (pollers).  Work and polls touch different
    //    lines: the polls write only the halo lines.
    const bool sampling = a.seis_freq && ++phase == a.seis_freq;
    if (sampling) phase = 0;
    bool ok = true;
    if (split && poller) {
      asm volatile("bar.arrive 1, %0;" ::"r"(kThreads) : "memory");  // this thread's reads of v are done
      ok = recv(slot, tag, threadIdx.x, npt);
    }
    if (worker) {
      unsent();
      // the receivers of the band (Seismogram::storeVelocitySignalAtReceivers)
      if (sampling && sample < a.seis_T) {
        for (uint32_t q = rcv_lo + wt; q < rcv_hi; q += nwt) {
          const unsigned long long g = a.rcv_sorted[2 * (size_t)q], r = a.rcv_sorted[2 * (size_t)q + 1];
          const double val = V[g - key0];
          a.seis[r + (size_t)a.R * sample] = val;
          if (!isfinite(val)) atomicOr(&a.ctl->nonfinite, 1u);
        }
      }
      // every read of this step's v and every stress line is done
      if (split)
        asm volatile("bar.sync 1, %0;" ::"r"(kThreads) : "memory");
      else
        __syncthreads();
      if (it + 1 < a.nsteps) vel_int(it + 1);
    }
    if (sampling && sample < a.seis_T) ++sample;
    if (!split) ok = recv(slot, tag, threadIdx.x, npt);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(&a.ctl->error, 1u);
      break;
    }
  }
}

__global__ void __launch_bounds__(kThreads, 1) fom_band_kernel(const Args a) {
  const uint32_t b = blockIdx.x;
  const uint32_t nth = a.nth, nr = a.nr, rows = a.rows;
  const uint32_t j0 = b * rows, j1 = min(nr, j0 + rows), nrow = j1 - j0;  // plan: every band owns rows
  const bool up = j1 < nr;   // a band above exists: v(j1) computed here, srp(j1), stp(j1, .) from it
  const bool down = j0 > 0;  // a band below exists: srp(j0 - 1) from it
  const bool srp_above = j1 + 1 < nr;  // srp(j1) exists
  const uint32_t vrows = nrow + (up ? 1 : 0);
  const uint32_t sp_row = 2 * nth - 1;
  const size_t nvp = (size_t)nth * nr, nsp = (size_t)(nr - 1) * nth + (size_t)nr * (nth - 1);
  extern __shared__ __align__(16) double sm[];
  double* const V = sm;                                     // (rows + 1) x nth: v rows j0 .. j1
  double* const SRP = V + (size_t)(rows + 1) * nth;         // (rows + 2) x nth: srp rows j0 - 1 .. j1
  double* const STP = SRP + (size_t)(rows + 2) * nth;       // (rows + 1) x (nth - 1): stp rows j0 .. j1
  double* const CV = STP + (size_t)(rows + 1) * (nth - 1);  // 4 x (rows + 1) x nth: rows j0 .. j1
  double* const CSR = CV + (size_t)4 * (rows + 1) * nth;    // 2 x rows x nth: srp rows j0 .. j1 - 1
  double* const CST = CSR + (size_t)2 * rows * nth;         // 2 x rows x (nth - 1)
  const uint32_t nv = (rows + 1) * nth, nsr = rows * nth, ns = rows * (nth - 1);
  // messages: down = srp(j0, .) then stp(j0, .) (2 nth - 1 points), up = srp(j1 - 1, .) (nth)
  const size_t down_pts = 2 * (size_t)nth - 1, up_pts = nth;
  unsigned long long* const send_down = a.xdown + (size_t)b * 2 * down_pts * 2;  // + slot * down_pts * 2
  unsigned long long* const send_up = a.xup + (size_t)b * 2 * up_pts * 2;
  const unsigned long long* const recv_above = up ? a.xdown + (size_t)(b + 1) * 2 * down_pts * 2 : nullptr;
  const unsigned long long* const recv_below = down ? a.xup + (size_t)(b - 1) * 2 * up_pts * 2 : nullptr;

  // the band, its halos and its stencil values
  for (uint32_t e = threadIdx.x; e < vrows * nth; e += kThreads) V[e] = a.xv[(size_t)j0 * nth + e];
  for (uint32_t e = threadIdx.x; e < (nrow + 2) * nth; e += kThreads) {
    const uint32_t rl = e / nth, i = e - rl * nth;
    const int j = (int)j0 - 1 + (int)rl;  // srp row
    SRP[e] = (j >= 0 && j + 1 < (int)nr && j <= (int)j1) ? a.xs[(size_t)j * sp_row + 2 * i] : 0.0;
  }
  for (uint32_t e = threadIdx.x; e < vrows * (nth - 1); e += kThreads) {
    const uint32_t rl = e / (nth - 1), i = e - rl * (nth - 1), j = j0 + rl;
    const size_t q = (j + 1 < nr) ? (size_t)j * sp_row + 2 * i + 1 : (size_t)j * sp_row + i;
    STP[e] = a.xs[q];
    if (rl < nrow) {
      CST[e] = a.csp[q];
      CST[ns + e] = a.csp[nsp + q];
    }
  }
  for (uint32_t e = threadIdx.x; e < vrows * nth; e += kThreads) {
    const size_t p = (size_t)j0 * nth + e;
    for (int c = 0; c < 4; ++c) CV[c * nv + e] = a.cvp[c * nvp + p];
    const uint32_t rl = e / nth, i = e - rl * nth, j = j0 + rl;
    if (rl < nrow && j + 1 < nr) {
      const size_t q = (size_t)j * sp_row + 2 * i;
      CSR[e] = a.csp[q];
      CSR[nsr + e] = a.csp[nsp + q];
    }
  }

  // This thread's elements, fixed for every step.  The velocity rows in band order, edge
  // rows first: local rows 0 (if down) and nrow (if up) are edge rows; e counts the edge
  // points, then the interior points.
  const uint32_t n_edge_rows = (down ? 1 : 0) + (up ? 1 : 0);
  const uint32_t n_int_rows = vrows - n_edge_rows;
  const uint32_t stp2_row0 = down ? 1 : 0, n_s2 = (nrow - stp2_row0) * (nth - 1);
  // Roles while the rows travel.  The received points: srp(j1) (when it exists) and
  // stp(j1, .) from above, srp(j0 - 1) from below.  When the other work fits the warps
  // left over, the first warps (one lane per received point) poll from the moment the
  // band's own rows are sent, and the other warps compute the other stp rows, the
  // receivers and the next step's interior velocity meanwhile; otherwise every thread
  // does that work first and polls afterwards.
  const uint32_t n_above = up ? (srp_above ? nth : 0) + nth - 1 : 0;
  const uint32_t n_recv = n_above + (down ? nth : 0);
  const uint32_t poll_threads = min(kThreads, 32 * ((n_recv + 31) / 32));
  const uint32_t work_threads = kThreads - poll_threads;
  const bool split = work_threads > 0 && n_s2 <= kBatch * work_threads && n_int_rows * nth <= kBatch * work_threads;
  const bool poller = !split || threadIdx.x < poll_threads;
  const bool worker = !split || threadIdx.x >= poll_threads;
  const uint32_t wt = split ? threadIdx.x - poll_threads : threadIdx.x;  // index among the workers
  const uint32_t nwt = split ? work_threads : kThreads;
  const uint32_t npt = split ? poll_threads : kThreads;
  auto vel_row = [&](bool edge, uint32_t r) -> uint32_t {  // local v row of the r-th edge / interior row
    if (edge) return (down && r == 0) ? 0 : nrow;
    return r + (down ? 1 : 0);
  };
  VelSet ve, vi;
  const int src_p = (a.src >= (unsigned long long)j0 * nth && a.src < (unsigned long long)(j0 + vrows) * nth)
                        ? (int)(a.src - (unsigned long long)j0 * nth)
                        : -1;
  bool ve_src = false, vi_src = false;
#pragma unroll
  for (int k = 0; k < kBatch; ++k) {
#pragma unroll
    for (int set = 0; set < 2; ++set) {
      VelSet& vs = set ? vi : ve;
      const uint32_t nrows_set = set ? n_int_rows : n_edge_rows;
      // the edge rows over all threads, the interior rows over the workers
      const uint32_t e = set ? (worker ? wt + k * nwt : ~0u) : threadIdx.x + k * kThreads;
      vs.p[k] = -1;
      vs.m[k] = 0;
      if (e < nrows_set * nth) {
        const uint32_t rl = vel_row(set == 0, e / nth), i = e % nth, j = j0 + rl;
        const uint32_t pt = rl * nth + i;
        vs.p[k] = (int)pt;
        vs.m[k] = (i != 0 && i + 1 != nth ? 1 : 0) | (j + 1 < nr ? 2 : 0) | (j > 0 ? 4 : 0) | (int)(rl << 3);
        if ((int)pt == src_p) (set ? vi_src : ve_src) = true;
      }
    }
  }
  // stress, first set: the srp rows, then stp row j0 when it is sent down; second set: the
  // other stp rows.  Message points: -1 when the element is not sent.
  const uint32_t n_srp = (up ? nrow : nrow - 1) * nth;  // srp(j) exists for j <= nr - 2
  const uint32_t n_s1 = n_srp + (down ? nth - 1 : 0);
  // First set: s1a = place (-1 when absent) and s1m: bit 0 = srp element (else stp),
  // bit 1 = sent up, bit 2 = sent down, bits 3.. = the message point.  An srp(j0 + rl, i)
  // element is SRP[s1a + nth] and reads V[s1a], V[s1a + nth]; the stp(j0, i) element is
  // STP[s1a] and reads V[s1a], V[s1a + 1].  Second set: stp(j, i) at STP[s2a], v(j, i) at V[s2w].
  int s1a[kBatch], s1m[kBatch], s2a[kBatch], s2w[kBatch];
#pragma unroll
  for (int k = 0; k < kBatch; ++k) {
    const uint32_t e = threadIdx.x + k * kThreads;
    s1a[k] = s2a[k] = -1;
    s1m[k] = 0;
    if (e < n_srp) {  // srp(j0 + rl, i), rows from the top so that srp(j1 - 1) leads
      const uint32_t rl = n_srp / nth - 1 - e / nth, i = e % nth;
      s1a[k] = (int)(rl * nth + i);
      s1m[k] = 1 | (up && j0 + rl == j1 - 1 ? 2 : 0) | (down && rl == 0 ? 4 : 0) | (int)(i << 3);
    } else if (e < n_s1) {  // stp(j0, i), sent down
      const uint32_t i = e - n_srp;
      s1a[k] = (int)i;
      s1m[k] = 4 | (int)((nth + i) << 3);
    }
    const uint32_t e2 = worker ? wt + k * nwt : ~0u;  // the other stp rows over the workers
    if (e2 < n_s2) {
      const uint32_t rl = stp2_row0 + e2 / (nth - 1), i = e2 % (nth - 1);
      s2a[k] = (int)(rl * (nth - 1) + i);
      s2w[k] = (int)(rl * nth + i);  // v(j, i) in V; v(j, i + 1) follows
    }
  }
  // the warps that hold the source run the forcing form of their velocity set
  const bool ve_force = __any_sync(0xffffffffu, ve_src), vi_force = __any_sync(0xffffffffu, vi_src);

  auto vel_edge = [&](unsigned long long it) {
    if (ve_force) velocity<true>(ve, V, SRP, STP, CV, nv, nth, src_p, a.ftab[it]);
    else velocity<false>(ve, V, SRP, STP, CV, nv, nth, -1, 0.0);
  };
  auto vel_int = [&](unsigned long long it) {
    if (vi_force) velocity<true>(vi, V, SRP, STP, CV, nv, nth, src_p, a.ftab[it]);
    else velocity<false>(vi, V, SRP, STP, CV, nv, nth, -1, 0.0);
  };
  auto send = [&](uint32_t tag, uint32_t slot) {
    unsigned long long* const sd = send_down + (size_t)slot * down_pts * 2;
    unsigned long long* const su = send_up + (size_t)slot * up_pts * 2;
#pragma unroll
    for (int k = 0; k < kBatch; ++k) {
      if (s1a[k] < 0) continue;
      const int e = s1a[k], m = s1m[k];
      double y;
      if (m & 1) {
        y = SRP[e + nth];
        y = fma(CSR[e], V[e + nth], y);  // north v(j + 1, i)
        y = fma(CSR[nsr + e], V[e], y);  // south v(j, i)
        SRP[e + nth] = y;
      } else {
        y = STP[e];
        y = fma(CST[e], V[e], y);           // west v(j0, i)
        y = fma(CST[ns + e], V[e + 1], y);  // east v(j0, i + 1)
        STP[e] = y;
      }
      if (m & 2) l2x::put(su + 2 * (m >> 3), tag, y);
      if (m & 4) l2x::put(sd + 2 * (m >> 3), tag, y);
    }
  };
  auto unsent = [&]() {
#pragma unroll
    for (int k = 0; k < kBatch; ++k) {
      if (s2a[k] < 0) continue;
      const int e = s2a[k];
      double y = STP[e];
      y = fma(CST[e], V[s2w[k]], y);
      y = fma(CST[ns + e], V[s2w[k] + 1], y);
      STP[e] = y;
    }
  };
  auto recv = [&](uint32_t slot, uint32_t tag, uint32_t t, uint32_t nt) {
    return receive(recv_above, recv_below, slot, tag, down_pts, up_pts, n_above, n_recv, srp_above, nth, nrow, SRP,
                   STP, t, nt);
  };
  band_steps(a, V, (unsigned long long)j0 * nth, (unsigned long long)j1 * nth, split, poller, worker, wt, nwt, npt,
             vel_edge, vel_int, send, unsent, recv);
  // the band back to the state (its own rows only)
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


// ---- the same leapfrog on column bands (grids wider than tall) ------------------------
//
// CTA b owns theta columns i0 .. i1 - 1 for every r row: its v columns plus v(., i1), its
// srp columns plus srp(., i1), its stp columns plus stp(., i0 - 1) and stp(., i1), and the
// folded stencil values of all of them; the shared arrays are column-major (stride nr for
// v and stp, nr - 1 for srp).  The roles of the row bands swap: the edge velocity columns
// are i0 (reading the received stp(., i0 - 1)) and i1 (computed here from the received
// srp(., i1) and stp(., i1) -- band b + 1 computes the same values); band b sends srp(., i0)
// and stp(., i0) to band b - 1 and stp(., i1 - 1) to band b + 1.  Same step order, roles,
// slots and bounded waits as the row kernel; bit-identical to the half-step kernels.

// Column-band velocity set: p = c nr + j (column c = i - i0) and m: bit 0 interior theta
// point, bit 1 N is srp(j) (else srp(j - 1)), bit 2 S is srp(j - 1) (else srp(j)), bits 3..
// = c.  srp(j, i) is SRP[p - c], srp(j - 1, i) is SRP[p - c - 1]; stp(j, i - 1) is STP[p]
// and stp(j, i) is STP[p + nr].
template <bool FORCE>
__device__ __forceinline__ void velocity_cols(const VelSet& e, double* V, const double* SRP, const double* STP,
                                              const double* CV, uint32_t nv, uint32_t nr, int src_p, double fdt) {
#pragma unroll
  for (int k = 0; k < kBatch; ++k) {
    if (e.p[k] < 0) continue;
    const int p = e.p[k], m = e.m[k], c = m >> 3;
    double v = V[p];
    if (m & 1) {
      v = fma(CV[p], SRP[(m & 2) ? p - c : p - c - 1], v);           // N
      v = fma(CV[nv + p], SRP[(m & 4) ? p - c - 1 : p - c], v);      // S
      v = fma(CV[2 * nv + p], STP[p], v);                           // W
      v = fma(CV[3 * nv + p], STP[p + (int)nr], v);                 // E
    }
    if (FORCE && p == src_p) v = __dadd_rn(v, fdt);  // after the FMAs, as the half-step kernel
    V[p] = v;
  }
}

// Received points of a column band: first the message from the right (srp(., i1), nr - 1
// points, then stp(., i1), nr points, when it exists), then stp(., i0 - 1) from the left.
__device__ __forceinline__ bool receive_cols(const unsigned long long* recv_right, const unsigned long long* recv_left,
                                             uint32_t slot, uint32_t tag, size_t left_pts, size_t right_pts,
                                             uint32_t n_right, uint32_t n_recv, uint32_t nr, uint32_t ncol,
                                             double* SRP, double* STP, uint32_t t, uint32_t nt) {
  const unsigned long long* src[kRecvMax];
  double* dst[kRecvMax];
  uint32_t pending = 0;
#pragma unroll
  for (int k = 0; k < kRecvMax; ++k) {
    const uint32_t q = t + k * nt;
    src[k] = nullptr;
    dst[k] = nullptr;
    if (q >= n_recv) continue;
    pending |= 1u << k;
    if (q < n_right) {  // the right band's left message: srp(., i1) then stp(., i1)
      src[k] = recv_right + (size_t)slot * left_pts * 2 + 2 * q;
      dst[k] = q < nr - 1 ? SRP + (size_t)ncol * (nr - 1) + q : STP + (size_t)(ncol + 1) * nr + (q - (nr - 1));
    } else {  // the left band's right message: stp(., i0 - 1)
      const uint32_t pb = q - n_right;
      src[k] = recv_left + (size_t)slot * right_pts * 2 + 2 * pb;
      dst[k] = STP + pb;
    }
  }
  return l2x::poll<kRecvMax>(src, dst, pending, tag);
}

__global__ void __launch_bounds__(kThreads, 1) fom_bandc_kernel(const Args a) {
  const uint32_t b = blockIdx.x;
  const uint32_t nth = a.nth, nr = a.nr, cw = a.rows;  // cw: columns per band
  const uint32_t i0 = b * cw, i1 = min(nth, i0 + cw), ncol = i1 - i0;  // plan: every band owns columns
  const bool right = i1 < nth;  // a band on the right: v(., i1) computed here, srp(., i1), stp(., i1) from it
  const bool left = i0 > 0;     // a band on the left: stp(., i0 - 1) from it
  const bool stp_right = i1 + 1 < nth;  // stp(., i1) exists
  const uint32_t vcols = ncol + (right ? 1 : 0);
  const uint32_t sp_row = 2 * nth - 1, ns1 = nr - 1;
  const size_t nvp = (size_t)nth * nr, nsp = (size_t)(nr - 1) * nth + (size_t)nr * (nth - 1);
  extern __shared__ __align__(16) double sm[];
  double* const V = sm;                                   // (cw + 1) x nr: columns i0 .. i1
  double* const SRP = V + (size_t)(cw + 1) * nr;          // (cw + 1) x (nr - 1): columns i0 .. i1
  double* const STP = SRP + (size_t)(cw + 1) * ns1;       // (cw + 2) x nr: columns i0 - 1 .. i1
  double* const CV = STP + (size_t)(cw + 2) * nr;         // 4 x (cw + 1) x nr: columns i0 .. i1
  double* const CSR = CV + (size_t)4 * (cw + 1) * nr;     // 2 x cw x (nr - 1): own srp columns
  double* const CST = CSR + (size_t)2 * cw * ns1;         // 2 x cw x nr: own stp columns
  const uint32_t nv = (cw + 1) * nr, nsr = cw * ns1, nst = cw * nr;
  // messages: left = srp(., i0) then stp(., i0) (2 nr - 1 points), right = stp(., i1 - 1) (nr)
  const size_t left_pts = 2 * (size_t)nr - 1, right_pts = nr;
  unsigned long long* const send_left = a.xdown + (size_t)b * 2 * left_pts * 2;  // + slot * left_pts * 2
  unsigned long long* const send_right = a.xup + (size_t)b * 2 * right_pts * 2;
  const unsigned long long* const recv_right = right ? a.xdown + (size_t)(b + 1) * 2 * left_pts * 2 : nullptr;
  const unsigned long long* const recv_left = left ? a.xup + (size_t)(b - 1) * 2 * right_pts * 2 : nullptr;
  auto stp_q = [&](uint32_t j, uint32_t i) -> size_t {  // stp(j, i) in the sp state
    return (j + 1 < nr) ? (size_t)j * sp_row + 2 * i + 1 : (size_t)j * sp_row + i;
  };

  // the band, its halos and its stencil values
  for (uint32_t e = threadIdx.x; e < vcols * nr; e += kThreads) {
    const uint32_t c = e / nr, j = e - c * nr;
    const size_t p = (size_t)j * nth + i0 + c;
    V[e] = a.xv[p];
    for (int q = 0; q < 4; ++q) CV[q * nv + e] = a.cvp[q * nvp + p];
  }
  for (uint32_t e = threadIdx.x; e < vcols * ns1; e += kThreads) {
    const uint32_t c = e / ns1, j = e - c * ns1;
    const size_t q = (size_t)j * sp_row + 2 * (i0 + c);
    SRP[e] = a.xs[q];
    if (c < ncol) {
      CSR[e] = a.csp[q];
      CSR[nsr + e] = a.csp[nsp + q];
    }
  }
  for (uint32_t e = threadIdx.x; e < (ncol + 2) * nr; e += kThreads) {
    const uint32_t c = e / nr, j = e - c * nr;
    const int i = (int)i0 - 1 + (int)c;  // stp column
    if (i >= 0 && i + 1 < (int)nth && i <= (int)i1) STP[e] = a.xs[stp_q(j, (uint32_t)i)];
    if (c >= 1 && c <= ncol && i + 1 < (int)nth) {  // own stp column c - 1
      const size_t q = stp_q(j, (uint32_t)i);
      CST[e - nr] = a.csp[q];
      CST[nst + e - nr] = a.csp[nsp + q];
    }
  }

  // Roles, as in the row kernel.  Received: srp(., i1) (nr - 1) and stp(., i1) (nr, when it
  // exists) from the right, stp(., i0 - 1) (nr) from the left.
  const uint32_t n_edge_cols = (left ? 1 : 0) + (right ? 1 : 0);
  const uint32_t n_int_cols = vcols - n_edge_cols;
  const uint32_t c_first_int = left ? 1 : 0;
  const bool stp_left_msg = left && i0 + 1 < nth;           // stp(., i0) exists and goes left
  const uint32_t n_s2_srp = (ncol - (left ? 1 : 0)) * ns1;  // srp columns not sent
  // stp columns sent: 0 (to the left, when it exists) and ncol - 1 (to the right)
  const bool c0_sent = stp_left_msg, clast_sent = right;  // (ncol - 1 == 0 is one column, sent both ways)
  const uint32_t last_stp_col = right ? ncol : ncol - 1;  // own stp columns [0, last_stp_col): stp(., i) for i <= nth - 2
  const uint32_t n_right = right ? ns1 + (stp_right ? nr : 0) : 0;
  const uint32_t n_recv = n_right + (left ? nr : 0);
  const uint32_t poll_threads = min(kThreads, 32 * ((n_recv + 31) / 32));
  const uint32_t work_threads = kThreads - poll_threads;
  // unsent stress elements: srp of columns c_first_int .. ncol - 1, stp of the columns that
  // are not sent
  uint32_t n_s2_stp = 0;
  for (uint32_t c = 0; c < last_stp_col; ++c)
    if (!((c == 0 && c0_sent) || (c + 1 == ncol && clast_sent))) n_s2_stp += nr;
  const uint32_t n_s2 = n_s2_srp + n_s2_stp;
  const bool split = work_threads > 0 && n_s2 <= kBatch * work_threads && n_int_cols * nr <= kBatch * work_threads;
  const bool poller = !split || threadIdx.x < poll_threads;
  const bool worker = !split || threadIdx.x >= poll_threads;
  const uint32_t wt = split ? threadIdx.x - poll_threads : threadIdx.x;
  const uint32_t nwt = split ? work_threads : kThreads;
  const uint32_t npt = split ? poll_threads : kThreads;

  VelSet ve, vi;
  int src_p = -1;
  {
    const unsigned long long js = a.src / nth, is = a.src - js * nth;
    if (is >= i0 && is < i0 + vcols) src_p = (int)((is - i0) * nr + js);
  }
  bool ve_src = false, vi_src = false;
#pragma unroll
  for (int k = 0; k < kBatch; ++k) {
#pragma unroll
    for (int set = 0; set < 2; ++set) {
      VelSet& vs = set ? vi : ve;
      const uint32_t ncols_set = set ? n_int_cols : n_edge_cols;
      const uint32_t e = set ? (worker ? wt + k * nwt : ~0u) : threadIdx.x + k * kThreads;
      vs.p[k] = -1;
      vs.m[k] = 0;
      if (e < ncols_set * nr) {
        const uint32_t r = e / nr, j = e - r * nr;
        const uint32_t c = set ? c_first_int + r : ((left && r == 0) ? 0 : ncol);  // the column
        const uint32_t i = i0 + c, pt = c * nr + j;
        vs.p[k] = (int)pt;
        vs.m[k] = (i != 0 && i + 1 != nth ? 1 : 0) | (j + 1 < nr ? 2 : 0) | (j > 0 ? 4 : 0) | (int)(c << 3);
        if ((int)pt == src_p) (set ? vi_src : ve_src) = true;
      }
    }
  }
  // Sent stress elements (all threads): s1t = target (SRP or STP place), s1v = the first v
  // input (the second is s1v + 1 for srp, s1v + nr for stp), s1m: bit 0 srp, bit 1 to the
  // right, bit 2 to the left, bits 3.. = the message point.  Unsent ones (workers): s2t,
  // s2v, s2m likewise (bit 0 srp).  Coefficients: CSR[t] / CST[t - nr] for srp / stp.
  const uint32_t n_s1_srp = left ? ns1 : 0;
  const uint32_t n_s1_stp = ((c0_sent ? 1u : 0u) + ((clast_sent && !(ncol == 1 && c0_sent)) ? 1u : 0u)) * nr;
  const uint32_t n_s1 = n_s1_srp + n_s1_stp;
  int s1t[kBatch], s1v[kBatch], s1m[kBatch], s2t[kBatch], s2v[kBatch], s2m[kBatch];
#pragma unroll
  for (int k = 0; k < kBatch; ++k) {
    const uint32_t e = threadIdx.x + k * kThreads;
    s1t[k] = s2t[k] = -1;
    s1v[k] = s1m[k] = s2v[k] = s2m[k] = 0;
    if (e < n_s1_srp) {  // srp(j, i0), to the left
      const uint32_t j = e;
      s1t[k] = (int)j;
      s1v[k] = (int)j;  // v(j, i0) at V[j]; v(j + 1, i0) follows
      s1m[k] = 1 | 4 | (int)(j << 3);
    } else if (e < n_s1) {  // stp(j, i0) (left and/or right) or stp(j, i1 - 1) (right)
      const uint32_t f = e - n_s1_srp, which = f / nr, j = f - which * nr;
      const uint32_t c = (which == 0 && c0_sent) ? 0 : ncol - 1;
      s1t[k] = (int)((c + 1) * nr + j);
      s1v[k] = (int)(c * nr + j);
      const bool to_left = c == 0 && c0_sent, to_right = c + 1 == ncol && clast_sent;
      const uint32_t lp = (uint32_t)ns1 + j;  // the left message's stp points follow its srp points
      s1m[k] = (to_right ? 2 : 0) | (to_left ? 4 : 0) | (int)((to_left ? lp : j) << 3);
      if (to_left && to_right) s1m[k] |= (int)(1u << 30);  // right point = j (low bits carry lp)
    }
    const uint32_t e2 = worker ? wt + k * nwt : ~0u;
    if (e2 < n_s2_srp) {
      const uint32_t c = c_first_int + e2 / ns1, j = e2 % ns1;
      s2t[k] = (int)(c * ns1 + j);
      s2v[k] = (int)(c * nr + j);
      s2m[k] = 1;
    } else if (e2 < n_s2) {
      uint32_t f = e2 - n_s2_srp, c = 0;
      for (; c < last_stp_col; ++c) {  // the f-th unsent stp element
        if ((c == 0 && c0_sent) || (c + 1 == ncol && clast_sent)) continue;
        if (f < nr) break;
        f -= nr;
      }
      s2t[k] = (int)((c + 1) * nr + f);
      s2v[k] = (int)(c * nr + f);
      s2m[k] = 0;
    }
  }
  const bool ve_force = __any_sync(0xffffffffu, ve_src), vi_force = __any_sync(0xffffffffu, vi_src);

  auto stress = [&](int t, int v0, int m) -> double {  // one element, the stress kernel's FMAs
    if (m & 1) {  // srp(j, i): north v(j + 1, i), south v(j, i)
      double y = SRP[t];
      y = fma(CSR[t], V[v0 + 1], y);
      y = fma(CSR[nsr + t], V[v0], y);
      SRP[t] = y;
      return y;
    }
    double y = STP[t];  // stp(j, i): west v(j, i), east v(j, i + 1)
    y = fma(CST[t - (int)nr], V[v0], y);
    y = fma(CST[nst + t - (int)nr], V[v0 + (int)nr], y);
    STP[t] = y;
    return y;
  };
  auto vel_edge = [&](unsigned long long it) {
    if (ve_force) velocity_cols<true>(ve, V, SRP, STP, CV, nv, nr, src_p, a.ftab[it]);
    else velocity_cols<false>(ve, V, SRP, STP, CV, nv, nr, -1, 0.0);
  };
  auto vel_int = [&](unsigned long long it) {
    if (vi_force) velocity_cols<true>(vi, V, SRP, STP, CV, nv, nr, src_p, a.ftab[it]);
    else velocity_cols<false>(vi, V, SRP, STP, CV, nv, nr, -1, 0.0);
  };
  auto send = [&](uint32_t tag, uint32_t slot) {
    unsigned long long* const sl = send_left + (size_t)slot * left_pts * 2;
    unsigned long long* const sr = send_right + (size_t)slot * right_pts * 2;
#pragma unroll
    for (int k = 0; k < kBatch; ++k) {
      if (s1t[k] < 0) continue;
      const int m = s1m[k];
      const double y = stress(s1t[k], s1v[k], m);
      const int pt = (m >> 3) & ((1 << 27) - 1);
      if (m & 4) l2x::put(sl + 2 * pt, tag, y);
      if (m & 2) l2x::put(sr + 2 * ((m & (1 << 30)) ? pt - (int)ns1 : pt), tag, y);
    }
  };
  auto unsent = [&]() {
#pragma unroll
    for (int k = 0; k < kBatch; ++k)
      if (s2t[k] >= 0) stress(s2t[k], s2v[k], s2m[k]);
  };
  auto recv = [&](uint32_t slot, uint32_t tag, uint32_t t, uint32_t nt) {
    return receive_cols(recv_right, recv_left, slot, tag, left_pts, right_pts, n_right, n_recv, nr, ncol, SRP, STP,
                        t, nt);
  };
  // receivers in column-major key order (key = i nr + j = V place + i0 nr)
  band_steps(a, V, (unsigned long long)i0 * nr, (unsigned long long)i1 * nr, split, poller, worker, wt, nwt, npt,
             vel_edge, vel_int, send, unsent, recv);
  // the band back to the state (its own columns only)
  for (uint32_t e = threadIdx.x; e < ncol * nr; e += kThreads) {
    const uint32_t c = e / nr, j = e - c * nr;
    a.xv[(size_t)j * nth + i0 + c] = V[e];
  }
  for (uint32_t e = threadIdx.x; e < ncol * ns1; e += kThreads) {
    const uint32_t c = e / ns1, j = e - c * ns1;
    a.xs[(size_t)j * sp_row + 2 * (i0 + c)] = SRP[e];
  }
  for (uint32_t e = threadIdx.x; e < last_stp_col * nr; e += kThreads) {
    const uint32_t c = e / nr, j = e - c * nr;
    a.xs[stp_q(j, i0 + c)] = STP[e + nr];
  }
}
}  // namespace

// Doubles of shared memory a column band of cw theta columns needs.
inline size_t smem_doubles_cols(uint32_t nr, uint32_t cw) {
  return (size_t)(cw + 1) * nr + (size_t)(cw + 1) * (nr - 1) + (size_t)(cw + 2) * nr + (size_t)4 * (cw + 1) * nr +
         (size_t)2 * cw * (nr - 1) + (size_t)2 * cw * nr;
}

namespace {

// Whether kern fits `need` co-resident CTAs with `bytes` of shared memory each.
bool fits(void (*kern)(Args), size_t bytes, int sms, int optin, uint32_t need) {
  if (bytes + 1024 > (size_t)optin) return false;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, bytes) != cudaSuccess ||
      (size_t)per_sm * sms < need) {
    cudaGetLastError();
    return false;
  }
  return true;
}

}  // namespace

bool plan(uint32_t nth, uint32_t nr, uint32_t* bands, uint32_t* width, uint32_t* cols, size_t* smem) {
  if (nth < 3 || nr < 2) return false;
  int dev = 0, sms = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return false;
  // the narrowest bands with one band per SM; at least two bands.  Cost: the points between
  // receiving and sending (edge velocity rows plus the stress rows sent), per band.
  const uint32_t r = (nr + (uint32_t)sms - 1) / (uint32_t)sms, gr = (nr + r - 1) / r;
  const uint32_t w = (nth + (uint32_t)sms - 1) / (uint32_t)sms, gc = (nth + w - 1) / w;
  const size_t br = smem_doubles(nth, r) * sizeof(double), bc = smem_doubles_cols(nr, w) * sizeof(double);
  const bool row_ok = gr >= 2 && (size_t)(r + 1) * nth <= (size_t)kBatch * kThreads &&
                      3 * (size_t)nth <= (size_t)kRecvMax * kThreads && fits(fom_band_kernel, br, sms, optin, gr);
  const bool col_ok = gc >= 2 && (size_t)(w + 1) * nr <= (size_t)kBatch * kThreads &&
                      3 * (size_t)nr <= (size_t)kRecvMax * kThreads && fits(fom_bandc_kernel, bc, sms, optin, gc);
  const size_t cost_r = (size_t)(r + 3) * nth, cost_c = (size_t)(w >= 2 ? 5 : 4) * nr;
  if (col_ok && (!row_ok || cost_c < cost_r)) {
    *bands = gc;
    *width = w;
    *cols = 1;
    *smem = bc;
    return true;
  }
  if (!row_ok) return false;
  *bands = gr;
  *width = r;
  *cols = 0;
  *smem = br;
  return true;
}

int launch(const Args& a, uint32_t bands, size_t smem, cudaStream_t s) {
  fom_band_forcing_kernel<<<(unsigned)((a.nsteps + 255) / 256), 256, 0, s>>>(a);
  SHAW_CUDA(cudaGetLastError());
  // per launch: another handle's plan may have set the kernel's limit for a smaller grid
  void (*kern)(Args) = a.cols ? fom_bandc_kernel : fom_band_kernel;
  SHAW_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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
  SHAW_CUDA(cudaLaunchKernelEx(&cfg, kern, a));
  return SHAW_OK;
}

}  // namespace band
}  // namespace shaw
