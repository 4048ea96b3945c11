// fom_sweep.cu -- the FOM velocity-stress leapfrog as one sweep per step (sm_103a).
//
// The reference advances with two CRS products per step (updateVelocity, then
// updateStress: src/kokkos/fom_update_kernels.hpp:60-181), i.e. two passes over the
// state: the stress pass re-reads every velocity value and the velocity pass every
// stress value, 24 bytes of HBM traffic per FP64 DOF-update.  Here one kernel advances
// both half-steps: a CTA owns a tile of the grid (a strip of kTI theta points x a chunk
// of forcing columns x a segment of r rows) and sweeps it row by row along r.  For row r
//   1. a copy warp stages v(r, strip + 1), the sp row r (stp and srp of the strip, one
//      point of halo either side) and the row's stencil values in shared memory (two
//      TMA tensor copies and two bulk copies into a ring of 3-4 rows, issued as soon as a
//      slot is released, completing on mbarriers);
//   2. eight compute warps form v_new(r, i) = v + cN s_N + cS s_S + cW s_W + cE s_E
//      (+ forcing) for the strip and its east neighbour (s_S is row r-1's srp, still in
//      the ring);
//   3. then sigma_new of row r-1 from v_new of rows r-1 and r (kept in a 3-slot shared
//      buffer): srp(r-1, i) = s + cA v(r, i) + cB v(r-1, i) and
//      stp(r-1, i) = s + cA v(r-1, i) + cB v(r-1, i+1).
// Each value is read once and written once per step (16 B per FP64 DOF-update), plus
// the strip's halo points (mostly L2 hits: neighbouring strips run side by side) and
// one recomputed v row per segment.  The old and new states are separate buffers (the
// handle alternates them), so halo values read by one CTA are never overwritten by
// another during the step.  A lane owns 1, 2 or 4 consecutive forcing columns (16-byte
// vector accesses), which spreads the per-point index work over the columns.
//
// The seismogram (Seismogram::storeVelocitySignalAtReceivers, seismogram.hpp:193-214)
// of step n-1 is gathered by extra blocks of step n from the old velocity buffer, which
// step n does not modify; the last step of a call is gathered by launch_gather.
//
// Forms: FP64 state with FP64 FMAs (the two-pass kernels' arithmetic in the same order,
// so the results are bit-identical to theirs), or FP32 state with FP32 FMAs.
//
// Every wait is bounded: a wait that runs out sets ctl->error bit 1 and the CTA stops
// issuing copies; before it exits it waits (bounded again) for the copies it issued.
#include "fom_sweep.h"

#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>
#include <string>

#include "shaw_internal.h"
#include "tc_ptx.cuh"

namespace shaw {
namespace sweep {

namespace {

using ptx::kWaitLimit;
using ptx::mbar_expect_tx;
using ptx::mbar_init;
using ptx::mbar_init_fence;
using ptx::smem_u32;

template <int F>
struct FT;
template <>
struct FT<kF64> {
  using S = double;   // state
  using CV = double;  // folded stencil value of a vp point (velocity half-step)
  using CS = double;  // folded stencil value of an sp point (stress half-step)
  using V = double;   // v_new as kept for the stress half-step
};
template <>
struct FT<kF32> {
  using S = float;
  using CV = float;
  using CS = float;
  using V = float;
};

// ---- the per-point updates -----------------------------------------------------------

template <int F>
struct Arith;

template <>
struct Arith<kF64> {
  __device__ static double vel(double v, double cN, double sN, double cS, double sS, double cW, double sW, double cE,
                               double sE) {
    v = fma(cN, sN, v);
    v = fma(cS, sS, v);
    v = fma(cW, sW, v);
    return fma(cE, sE, v);
  }
  __device__ static double str(double s, double cA, double vA, double cB, double vB) {
    s = fma(cA, vA, s);
    return fma(cB, vB, s);
  }
};

template <>
struct Arith<kF32> {
  __device__ static float vel(float v, float cN, float sN, float cS, float sS, float cW, float sW, float cE,
                              float sE) {
    v = fmaf(cN, sN, v);
    v = fmaf(cS, sS, v);
    v = fmaf(cW, sW, v);
    return fmaf(cE, sE, v);
  }
  __device__ static float str(float s, float cA, float vA, float cB, float vB) {
    s = fmaf(cA, vA, s);
    return fmaf(cB, vB, s);
  }
};

// ---- forcing (the same arithmetic as the two-pass kernels) -----------------------------

__device__ __noinline__ double forced(double x, const Params& a, uint32_t m, uint32_t p, unsigned long long n) {
  const double t = (double)(n - 1) * a.dt;
  const double f = shaw::signal_value(a.kind[m], a.delay[m], a.period[m], t);
  const double ri = a.rho_inv[p];
  if (a.rank2) return __dadd_rn(x, __dmul_rn(__dmul_rn(ri, f), a.dt));  // AddForcingRank2
  return __dadd_rn(x, __dmul_rn(__dmul_rn(a.dt, ri), f));              // KokkosBlas::mult(1, x, dt, rhoInv, f)
}
__device__ __noinline__ float forced(float x, const Params& a, uint32_t m, uint32_t p, unsigned long long n) {
  const double t = (double)(n - 1) * a.dt;
  const double f = shaw::signal_value(a.kind[m], a.delay[m], a.period[m], t);
  const double ri = a.rho_inv[p];
  const double inc = a.rank2 ? __dmul_rn(__dmul_rn(ri, f), a.dt) : __dmul_rn(__dmul_rn(a.dt, ri), f);
  return x + __double2float_rn(inc);
}

__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_next_grid() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Bounded wait on an mbarrier phase; false when the poll limit ran out.
__device__ __forceinline__ bool wait_full(uint64_t* bar, uint32_t parity) {
  return ptx::mbar_wait_n(bar, parity, kWaitLimit);
}

// Stencil values staged with each row: 4 per vp point (N, S, W, E) and 2 per sp point
// (A, B), copied from the point-major copies of the coefficients (Params::cvp / csp).
// An sp copy may start up to kPtsPer16 - 1 points early so that it is 16-byte aligned.
template <int F>
struct Coef {
  using C = typename FT<F>::CS;
  static constexpr uint32_t kPtsPer16 = 16 / (2 * sizeof(C));  // sp points per 16 bytes (1 or 2)
  // sp points a row copy spans: the box and the alignment shift, rounded to whole 16 bytes
  static constexpr uint32_t kCsPts = (kRowsS + kPtsPer16 - 1 + kPtsPer16 - 1) / kPtsPer16 * kPtsPer16;
};

// VEC consecutive values of one lane as one vector access (16 bytes at most).
template <typename T, int VEC>
struct alignas(sizeof(T) * VEC) Vec {
  T x[VEC];
};
template <typename T, int VEC>
__device__ __forceinline__ Vec<T, VEC> ldv(const T* p) {
  return *reinterpret_cast<const Vec<T, VEC>*>(p);
}
template <typename T, int VEC>
__device__ __forceinline__ void stv(T* p, const Vec<T, VEC>& v) {
  *reinterpret_cast<Vec<T, VEC>*>(p) = v;
}

// Tile geometry of a (form, columns-per-lane) pair: kTM * VEC columns per tile; a ring of 4
// rows where a row of the tile is at most 16 KB, else 3 (two rows in use, the rest loading).
template <int F, int VEC>
struct Geo {
  using S = typename FT<F>::S;
  static constexpr uint32_t TM = kTM * VEC;
  static constexpr uint32_t STAGES = (sizeof(S) * VEC >= 16) ? 3 : 4;
};

template <int F, int VEC>
struct Smem {
  using S = typename FT<F>::S;
  using V = typename FT<F>::V;
  using CV = typename FT<F>::CV;
  using CS = typename FT<F>::CS;
  static constexpr uint32_t TM = Geo<F, VEC>::TM, ST = Geo<F, VEC>::STAGES;
  S v[ST][kRowsV][TM];
  S s[ST][kRowsS][TM];
  V vb[3][kRowsV][TM];
  CV cv[ST][kRowsV][4];
  CS cs[ST][Coef<F>::kCsPts][2];
  uint64_t full[ST];   // the copies of a row have landed
  uint64_t empty[ST];  // the 8 compute warps are done with a row's slot
  unsigned int abort;
  unsigned int t_waited;  // the last row index the compute warps waited for
};

// sp-box offset of stp(row, i0 + li) (li may be -1): interleaved rows / the last row.
__device__ __forceinline__ uint32_t stp_off(int li, bool last) {
  return last ? (uint32_t)(li + 1) : (uint32_t)(2 * li + 2);
}
__device__ __forceinline__ uint32_t srp_off(int li) { return (uint32_t)(2 * li + 1); }

template <int F>
__device__ void gather_prev(const Params& p, uint32_t k_local, unsigned long long host_step) {
  using S = typename FT<F>::S;
  const unsigned long long n = host_step ? host_step : p.ctl->step_base + k_local + 1;
  if (n < 2 || p.seis_freq == 0) return;
  const unsigned long long prev = n - 1;
  if (prev % p.seis_freq != 0) return;
  const uint32_t idx = (blockIdx.x - p.n_tiles) * blockDim.x + threadIdx.x;
  if (idx >= p.R * p.M) return;
  const uint32_t r = idx % p.R, m = idx / p.R;
  const unsigned long long cnt = prev / p.seis_freq - 1;
  if (cnt >= p.seis_T) return;
  const double val = (double)static_cast<const S*>(p.xv_old)[(size_t)p.rcv[r] * p.M + m];
  p.seis[r + (size_t)p.R * (cnt + (size_t)p.seis_T * m)] = val;
  if (!isfinite(val)) atomicOr(&p.ctl->nonfinite, 1u);
}

__device__ __forceinline__ void compute_barrier() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

constexpr uint32_t kBlock = kThreads + 32;  // 8 compute warps + 1 copy warp

template <int F, int VEC>
__global__ void __launch_bounds__(kBlock, 2) fom_sweep_kernel(const __grid_constant__ CUtensorMap tv,
                                                              const __grid_constant__ CUtensorMap ts,
                                                              const Params p, uint32_t k_local,
                                                              unsigned long long host_step) {
  using S = typename FT<F>::S;
  using CV = typename FT<F>::CV;
  using CS = typename FT<F>::CS;
  using V = typename FT<F>::V;
  using A = Arith<F>;
  using SV = Vec<S, VEC>;
  using VV = Vec<V, VEC>;
  constexpr uint32_t TM = Geo<F, VEC>::TM, ST = Geo<F, VEC>::STAGES;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem<F, VEC>& sm = *reinterpret_cast<Smem<F, VEC>*>(smem_raw);

  if (blockIdx.x >= p.n_tiles) {
    wait_prior_grid();
    gather_prev<F>(p, k_local, host_step);
    return;
  }
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // tile: strip fastest (neighbouring strips run side by side and share their halo in L2)
  uint32_t b = blockIdx.x;
  const uint32_t strip = b % p.strips;
  b /= p.strips;
  const uint32_t chunk = b % p.chunks;
  const uint32_t seg = b / p.chunks;
  const uint32_t i0 = strip * kTI, m0 = chunk * TM, j0 = seg * p.tj;
  const uint32_t nth = p.nth, nr = p.nr;
  const uint32_t jend = min(j0 + p.tj, nr - 1);  // last v row computed (j0 + tj: a halo row)
  const uint32_t jown = min(j0 + p.tj, nr);       // rows j0 .. jown - 1 are written by this tile
  const bool pre = j0 > 0;                         // row j0 - 1 staged (sp only)
  const uint32_t base = pre ? 0u : 1u;             // row index t = r - j0 + 1 of the first copy
  constexpr uint32_t kPpa = Coef<F>::kPtsPer16;
  auto sp_y0 = [&](uint32_t r) {  // first sp point of row r's box
    return (r + 1 < nr) ? (int)(r * p.sp_row + 2 * i0) - 1 : (int)(r * p.sp_row + i0) - 1;
  };
  auto cs_shift = [&](uint32_t r) { return (uint32_t)(sp_y0(r) + 1) % kPpa; };

  if (tid == 0) {
    for (uint32_t k = 0; k < ST; ++k) {
      mbar_init(&sm.full[k], 1);
      mbar_init(&sm.empty[k], kThreads / 32);
    }
    sm.abort = 0;
    sm.t_waited = 0;
    mbar_init_fence();
  }
  __syncthreads();
  wait_prior_grid();  // the previous step's state is complete from here on
  volatile unsigned int* abort_flag = &sm.abort;

  if (warp == kThreads / 32) {
    // ---- copy warp: row r = j0 - 1 + t into slot (t - base) % ST as soon as it is free ----
    uint32_t t_last = 0;
    if (lane == 0) {
      prefetch_map(&tv);
      prefetch_map(&ts);
      const CV* cv4 = static_cast<const CV*>(p.cvp);  // [nvp + pad][4]
      const CS* cs2 = static_cast<const CS*>(p.csp);  // [1 + nsp + pad][2]: sp point q at q + 1
      constexpr uint32_t kBytesV = kRowsV * TM * sizeof(S), kBytesS = kRowsS * TM * sizeof(S);
      constexpr uint32_t kBytesCv = kRowsV * 4 * sizeof(CV), kBytesCs = Coef<F>::kCsPts * 2 * sizeof(CS);
      for (uint32_t t = base; j0 - 1 + t <= jend; ++t) {
        const uint32_t u = t - base, k = u % ST;
        if (u >= ST && !ptx::mbar_wait_n(&sm.empty[k], ((u / ST) - 1) & 1u, kWaitLimit)) {
          atomicOr(&p.ctl->error, 1u);
          *abort_flag = 1;
        }
        if (*abort_flag) break;
        const uint32_t r = j0 - 1 + t;
        const int ys = sp_y0(r);
        if (t == 0) {
          mbar_expect_tx(&sm.full[k], kBytesS);
        } else {
          mbar_expect_tx(&sm.full[k], kBytesV + kBytesS + kBytesCv + kBytesCs);
          tma_load_2d(&sm.v[k][0][0], &tv, (int)m0, (int)(r * nth + i0), &sm.full[k]);
          ptx::bulk_g2s(&sm.cv[k][0][0], cv4 + (size_t)(r * nth + i0) * 4, kBytesCv, &sm.full[k]);
          const uint32_t c0 = (uint32_t)(ys + 1) - cs_shift(r);  // padded index, a multiple of kPpa
          ptx::bulk_g2s(&sm.cs[k][0][0], cs2 + (size_t)c0 * 2, kBytesCs, &sm.full[k]);
        }
        tma_load_2d(&sm.s[k][0][0], &ts, (int)m0, ys, &sm.full[k]);
        t_last = t + 1;
      }
    }
    __syncthreads();  // the compute warps are done
    // an aborted CTA waits (bounded) for the copies it issued and did not consume before it exits
    if (lane == 0 && *abort_flag) {
      for (uint32_t t = max(sm.t_waited + 1, base); t < t_last; ++t) {
        const uint32_t u = t - base;
        wait_full(&sm.full[u % ST], (u / ST) & 1u);
      }
    }
    return;
  }

  // ---- compute warps: warp w owns the points li = 2w, 2w + 1 of the strip (warp 7 also the
  //      east neighbour li = kTI) and the lane's VEC columns ----
  const uint32_t col = m0 + lane * VEC;
  const uint32_t nq = (warp == 7) ? 3u : 2u;
  uint32_t hit_row[3][VEC];  // the row of the lane's source in column col + c at point q, else ~0
  bool any_hit[3];
#pragma unroll
  for (uint32_t q = 0; q < 3; ++q) {
    any_hit[q] = false;
    const uint32_t i = i0 + 2 * warp + q;
#pragma unroll
    for (int c = 0; c < VEC; ++c) {
      const unsigned long long g = p.src[col + c];
      const uint32_t sj = (uint32_t)(g / nth), si = (uint32_t)(g - (unsigned long long)sj * nth);
      hit_row[q][c] = (q < nq && si == i) ? sj : 0xFFFFFFFFu;
      any_hit[q] = any_hit[q] || hit_row[q][c] != 0xFFFFFFFFu;
    }
  }
  const unsigned long long n_step = host_step ? host_step : p.ctl->step_base + k_local + 1;
  S* const xv_new = static_cast<S*>(p.xv_new);
  S* const xs_new = static_cast<S*>(p.xs_new);
  const size_t M = p.M;
  S carry[3][VEC];  // srp of the previous row at each point (the next row's S neighbour)

  for (uint32_t t = 1;; ++t) {
    const uint32_t r = j0 - 1 + t;
    if (r > jend) break;
    // ---- stage(t) (and the pre-stage at t == 1) have arrived ----
    if (!*abort_flag) {
      const uint32_t u = t - base;
      bool ok = wait_full(&sm.full[u % ST], (u / ST) & 1u);
      if (t == 1 && pre) ok = wait_full(&sm.full[0], 0) && ok;
      if (!ok) {
        atomicOr(&p.ctl->error, 1u);
        *abort_flag = 1;
      } else if (tid == 0) {
        sm.t_waited = t;
      }
    }
    const uint32_t k = (t - base) % ST, kp = (t - 1 - base) % ST;
    const bool last = (r + 1 == nr);
    const S* sv = &sm.v[k][0][0] + lane * VEC;
    const S* ss = &sm.s[k][0][0] + lane * VEC;
    const S* ssp = &sm.s[kp][0][0] + lane * VEC;  // row r - 1 (interleaved)
    const bool fresh_S = (r == j0) || (r == 0);   // S neighbour not carried from the previous row
    // ---- v_new(r, i0 + li), li = 2w + q ----
    {
      VV* vb = reinterpret_cast<VV*>(&sm.vb[t % 3][0][0]);
      S eW[VEC];  // E neighbour of the previous point = W neighbour of this one
      bool have_e = false;
#pragma unroll
      for (uint32_t q = 0; q < 3; ++q) {
        const uint32_t li = 2 * warp + q;
        const uint32_t i = i0 + li;
        if (q >= nq || i >= nth) break;
        SV v = ldv<S, VEC>(sv + li * TM);
        if (i != 0 && i + 1 != nth) {
          const CV cN = sm.cv[k][li][0], cS = sm.cv[k][li][1], cW = sm.cv[k][li][2], cE = sm.cv[k][li][3];
          const SV rawE = ldv<S, VEC>(ss + stp_off((int)li, last) * TM);
          SV rawW, rawN, rawS;
          if (!have_e) rawW = ldv<S, VEC>(ss + stp_off((int)li - 1, last) * TM);
          if (fresh_S) rawS = ldv<S, VEC>((r > 0 ? ssp : ss) + srp_off(li) * TM);
          if (!last) rawN = ldv<S, VEC>(ss + srp_off(li) * TM);
#pragma unroll
          for (int c = 0; c < VEC; ++c) {
            const S oS = fresh_S ? rawS.x[c] : carry[q][c];
            const S oN = last ? oS : rawN.x[c];
            const S oW = have_e ? eW[c] : rawW.x[c];
            const S oE = rawE.x[c];
            v.x[c] = A::vel(v.x[c], cN, oN, cS, oS, cW, oW, cE, oE);
            carry[q][c] = oN;
            eW[c] = oE;
          }
          have_e = true;
        } else {
          have_e = false;
        }
        if (any_hit[q]) {
#pragma unroll
          for (int c = 0; c < VEC; ++c)
            if (r == hit_row[q][c]) v.x[c] = forced(v.x[c], p, col + c, r * nth + i, n_step);
        }
        if (li < kTI && r < jown) stv<S, VEC>(xv_new + ((size_t)r * nth + i) * M + col, v);
        vb[li * (TM / VEC) + lane] = v;
      }
    }
    compute_barrier();
    // ---- sigma_new of row r - 1 (interleaved row): srp and stp of li = 2w, 2w + 1 ----
    if (r > j0) {
      const uint32_t rq = r - 1;
      const VV* vn = reinterpret_cast<const VV*>(&sm.vb[t % 3][0][0]) + lane;        // v_new(r)
      const VV* vo = reinterpret_cast<const VV*>(&sm.vb[(t - 1) % 3][0][0]) + lane;  // v_new(r - 1)
      const CS(*csq)[2] = sm.cs[kp] + cs_shift(rq);  // indexed like the sp box of row r - 1
      constexpr uint32_t VS = TM / VEC;              // vb stride of one point (in vectors)
#pragma unroll
      for (uint32_t h = 0; h < 2; ++h) {
        const uint32_t li = 2 * warp + h;
        const uint32_t i = i0 + li;
        if (i >= nth) break;
        const size_t g = (size_t)rq * p.sp_row + 2 * i;  // srp(rq, i)
        {
          SV sg = ldv<S, VEC>(ssp + srp_off(li) * TM);
          const CS cA = csq[srp_off(li)][0], cB = csq[srp_off(li)][1];
          const VV a = vn[li * VS], bb = vo[li * VS];
#pragma unroll
          for (int c = 0; c < VEC; ++c) sg.x[c] = A::str(sg.x[c], cA, a.x[c], cB, bb.x[c]);
          stv<S, VEC>(xs_new + g * M + col, sg);
        }
        if (i + 1 < nth) {  // stp(rq, i)
          SV su = ldv<S, VEC>(ssp + stp_off((int)li, false) * TM);
          const CS cA = csq[stp_off((int)li, false)][0], cB = csq[stp_off((int)li, false)][1];
          const VV a = vo[li * VS], bb = vo[(li + 1) * VS];
#pragma unroll
          for (int c = 0; c < VEC; ++c) su.x[c] = A::str(su.x[c], cA, a.x[c], cB, bb.x[c]);
          stv<S, VEC>(xs_new + (g + 1) * M + col, su);
        }
      }
    }
    // ---- the surface row's stp (no srp there): sigma_new(r) from v_new(r) ----
    if (last && r < jown) {
      const VV* vn = reinterpret_cast<const VV*>(&sm.vb[t % 3][0][0]) + lane;
      const CS(*csc)[2] = sm.cs[k] + cs_shift(r);
      constexpr uint32_t VS = TM / VEC;
#pragma unroll
      for (uint32_t h = 0; h < 2; ++h) {
        const uint32_t li = 2 * warp + h;
        const uint32_t i = i0 + li;
        if (i + 1 >= nth) break;
        const size_t g = (size_t)r * p.sp_row + i;
        SV su = ldv<S, VEC>(ss + stp_off((int)li, true) * TM);
        const CS cA = csc[stp_off((int)li, true)][0], cB = csc[stp_off((int)li, true)][1];
        const VV a = vn[li * VS], bb = vn[(li + 1) * VS];
#pragma unroll
        for (int c = 0; c < VEC; ++c) su.x[c] = A::str(su.x[c], cA, a.x[c], cB, bb.x[c]);
        stv<S, VEC>(xs_new + g * M + col, su);
      }
    }
    // the slot of row r - 1 is free once every compute warp is past this point
    if (lane == 0 && (t >= 2 || pre)) ptx::mbar_arrive(&sm.empty[(t - 1 - base) % ST]);
  }
  allow_next_grid();
  __syncthreads();  // with the copy warp, which drains an aborted CTA's copies
}

template <int F>
__global__ void fom_gather_kernel(Params p, const void* xv, unsigned long long step) {
  using S = typename FT<F>::S;
  if (p.seis_freq == 0 || step == 0 || step % p.seis_freq != 0) return;
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= p.R * p.M) return;
  const uint32_t r = idx % p.R, m = idx / p.R;
  const unsigned long long cnt = step / p.seis_freq - 1;
  if (cnt >= p.seis_T) return;
  const double val = (double)static_cast<const S*>(xv)[(size_t)p.rcv[r] * p.M + m];
  p.seis[r + (size_t)p.R * (cnt + (size_t)p.seis_T * m)] = val;
  if (!isfinite(val)) atomicOr(&p.ctl->nonfinite, 1u);
}

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

template <int F, int VEC>
int launch_t(const CUtensorMap& tv, const CUtensorMap& ts, const Params& p, uint32_t k_local,
             unsigned long long host_step, cudaStream_t s, bool pdl) {
  static bool attr_set = false;  // per process: the kernel's dynamic shared-memory opt-in
  const size_t smem = sizeof(Smem<F, VEC>);
  if (!attr_set) {
    SHAW_CUDA(cudaFuncSetAttribute(fom_sweep_kernel<F, VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(p.n_tiles + p.gather_blocks);
  cfg.blockDim = dim3(kBlock);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  SHAW_CUDA(cudaLaunchKernelEx(&cfg, fom_sweep_kernel<F, VEC>, tv, ts, p, k_local, host_step));
  return SHAW_OK;
}

}  // namespace

uint32_t columns_per_lane(uint32_t M, uint32_t esz) {
  if (esz == 4 && M % (4 * kTM) == 0) return 4;
  if (M % (2 * kTM) == 0) return 2;
  return 1;
}

int encode_map(CUtensorMap* map, const void* base, uint64_t n, uint32_t M, uint32_t esz, uint32_t box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
  if (!enc) return fail(SHAW_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const cuuint64_t dims[2] = {M, n};
  const cuuint64_t strides[1] = {(cuuint64_t)M * esz};
  const cuuint32_t box[2] = {kTM * columns_per_lane(M, esz), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(map, esz == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                         const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(SHAW_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return SHAW_OK;
}

void plan(Params& p, int sm_count, uint32_t esz) {
  p.vec = columns_per_lane(p.M, esz);
  p.strips = (p.nth + kTI - 1) / kTI;
  p.chunks = p.M / (kTM * p.vec);
  // segments of tj rows: at least ~8 waves of 2 CTAs per SM, rows >= 32 (one halo row per segment)
  const uint64_t per_layer = (uint64_t)p.strips * p.chunks;
  const uint64_t want = (uint64_t)sm_count * 2 * 8;
  uint64_t segs = (want + per_layer - 1) / per_layer;
  uint64_t tj = (p.nr + segs - 1) / segs;
  if (tj < 32) tj = 32;
  if (tj > p.nr) tj = p.nr;
  p.tj = (uint32_t)tj;
  p.segs = (uint32_t)((p.nr + tj - 1) / tj);
  p.n_tiles = p.strips * p.chunks * p.segs;
  p.gather_blocks = (p.R && p.seis_freq) ? (p.R * p.M + kBlock - 1) / kBlock : 0;
}

int launch(Form f, const CUtensorMap& tv, const CUtensorMap& ts, const Params& p, uint32_t k_local,
           unsigned long long host_step, cudaStream_t s, bool pdl) {
  switch (f) {
    case kF64:
      return p.vec == 2 ? launch_t<kF64, 2>(tv, ts, p, k_local, host_step, s, pdl)
                        : launch_t<kF64, 1>(tv, ts, p, k_local, host_step, s, pdl);
    default:
      return p.vec == 4   ? launch_t<kF32, 4>(tv, ts, p, k_local, host_step, s, pdl)
             : p.vec == 2 ? launch_t<kF32, 2>(tv, ts, p, k_local, host_step, s, pdl)
                          : launch_t<kF32, 1>(tv, ts, p, k_local, host_step, s, pdl);
  }
}

int launch_gather(Form f, const Params& p, const void* xv, unsigned long long step, cudaStream_t s) {
  if (!p.R || !p.seis_freq) return SHAW_OK;
  const uint32_t blocks = (p.R * p.M + 255) / 256;
  if (f == kF32) fom_gather_kernel<kF32><<<blocks, 256, 0, s>>>(p, xv, step);
  else fom_gather_kernel<kF64><<<blocks, 256, 0, s>>>(p, xv, step);
  SHAW_CUDA(cudaGetLastError());
  return SHAW_OK;
}

}  // namespace sweep
}  // namespace shaw
