// rom_oz.cu -- rank-2 ROM leapfrog with FP64-grade reduced GEMMs on the BF16 tensor
// cores (tcgen05, kind::f16), using the Ozaki splitting scheme with exact accumulation,
// for one reduced system or a batch of uneven ones in a single persistent launch.
//
// Reference: runRomRankTwoForcing (src/kokkos/torevise/run_rom_rank_two_forcing.hpp:149-188)
//   XV += dt Av XS ;  XV[:,j] += (f_j dt) b[:,j] ;  XS += dt As XV
//
// Why not plain TF32x3 / BF16x3: the tensor pipe accumulates in FP32 with truncation,
// which biases every GEMM toward zero by ~1e-6 relative for K = 512; over 20000
// oscillating leapfrog steps that becomes a phase drift far above 1e-6.  Here the
// products are made EXACT instead (Ozaki, Ogita, Oishi & Rump 2012; "Ozaki scheme"):
//   * every operator row i is scaled by 2^alpha_i and every state column j by 2^beta_j
//     so its entries lie in (-1, 1), then cut into 6 slices of 6 bits:
//         a = sum_s a_s 2^(-6(s+1)),  a_s integers, |a_0| <= 64, |a_s>0| <= 32
//     (exact in BF16);
//   * a slice product is an integer below 2^12, a K-sum below 2^22 (K <= 1024) and a
//     diagonal d = s + t (up to 6 pairs) below 2^24: the FP32 accumulators in TMEM
//     hold every partial sum exactly, whatever their rounding mode;
//   * pairs with s + t <= 5 give ~2^-36 relative accuracy; they are issued as 6 MMAs
//     per K-step (operator slice s times the stacked state slices 0 .. 5-s), and the 6
//     diagonal sums are combined with error-free FP32 additions in the epilogue.
// State: FP32 hi + lo pairs (compensated) in global memory.  The epilogue slices each
// new state value into the next GEMM's BF16 B tiles as soon as it is computed, with a
// per-column exponent predicted from the previous half-step (one bit of headroom);
// columns whose new maximum leaves the predicted range are re-sliced exactly after
// the phase.
//
// Work decomposition: forcing columns are independent for the whole run, so the unit
// of work is a TILE = (instance, block of nb columns), advanced through all time steps
// by one CTA.  A persistent grid of at most one CTA per SM runs a host-built schedule:
// CTA c advances the tiles order[cta_begin[c] .. cta_begin[c+1]) one after another.
// Tile widths nb in {16, 32, 64} and the schedule (longest-processing-time-first over
// modelled or measured tile costs) are picked by the autotuner `tune`.
// Within a tile the producer, the MMA issuer and the epilogue warps run decoupled (stage
// metadata, accumulator barriers, and gates through which the epilogue releases each new
// state to the producer); block-wide barriers are taken only between tiles.
// All waits are bounded: a wait that runs out sets an error flag, every role leaves its
// loop (the epilogue at its next vote), the kernel releases TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <queue>
#include <string>
#include <vector>

#include "rom_oz.h"
#include "l2_exchange.cuh"
#include "shaw_internal.h"
#include "tc_ptx.cuh"

namespace shaw {
namespace oz {

using namespace shaw::ptx;

namespace {

// warps: 0 bulk-copy producer, 1 MMA issuer, 2 TMEM owner, 3 idle, 4..11 epilogue
// (two groups of four: warp w reads TMEM lanes 32*(w%4).., each group half the columns)
constexpr int kThreads = 384;
constexpr int kEpiThreads = 256;
constexpr int kKc = 32;                       // BF16 K-elements per pipeline stage (64 bytes per row)
constexpr uint32_t kRowBytes = kKc * 2;
constexpr uint32_t kATile = 128 * kRowBytes;  // one slice of a 128 x 32 operator tile: 8 KB
constexpr uint32_t kMaxNb = 64;               // widest tile of either form
constexpr int kMaxStages = 3;
constexpr uint32_t kLevels = 8;  // M-tiles per phase and CTA: at most 1024 / 128
// TMEM: two accumulator sets at columns 0 and 256 when S nb <= 256; otherwise one set at
// column 0 and the staging of its combined values at column S nb
constexpr uint32_t kTmemCols = 512;

// The two forms of the scheme, by slice count S (the diagonals d = s + t <= S - 1 kept):
//   S = 6: 36-bit slicing, FP32 hi + lo state (SHAW_MIXED_OZAKI_BF16);
//   S = 9: 54-bit slicing, FP64 state: FP64-grade results (SHAW_OZAKI_FP64).
// Exactness of the FP32 accumulators (K <= 1024): a diagonal d holds at most d + 1 slice
// pairs; the first slice of either operand is in [-64, 64], the others in [-32, 32], so
// d = 8 sums below 2 * 64 * 32 * 1024 + 7 * 32 * 32 * 1024 = 11 * 2^20 < 2^24.
template <int S>
struct Geo {
  static constexpr uint32_t kABytes = S * kATile;                              // 48 / 72 KB
  static constexpr uint32_t kMaxNb = S == 6 ? 64u : 32u;
  static constexpr uint32_t kStageBytes = kABytes + S * kMaxNb * kRowBytes;  // 72 / 90 KB
  static constexpr int kStages = S == 6 ? 3 : 2;
  __host__ __device__ static constexpr uint32_t bstage_bytes(uint32_t nb) { return S * nb * kRowBytes; }
  __host__ __device__ static constexpr uint32_t acc_buffers(uint32_t nb) { return (S * nb <= 256) ? 2u : 1u; }
};

// Byte offset of (row r, k) in a K-major, no-swizzle BF16 tile of 32 K-elements:
// core matrices of 8 rows x 16 bytes, K-direction stride 128 B, 8-row-group stride 512 B.
__host__ __device__ __forceinline__ uint32_t tile_off(uint32_t r, uint32_t k) {
  return (((r >> 3) * 4u + (k >> 3)) << 7) + ((r & 7u) << 4) + ((k & 7u) << 1);
}

// Byte offset of (slice s, column j, K-row k) in one pipeline stage of state slices (the
// B operand, MN-major, no swizzle): the S slices are stacked along N (n = s*nb + j); a
// core matrix is 8 K-rows x 16 bytes (8 consecutive n); N-direction stride 128 B,
// K-direction stride 16*S*nb B (all S*nb columns of one 8-row K group).  Eight
// consecutive columns of one row are 16 contiguous bytes; slice s starts 16*nb*s bytes
// after slice 0.
template <int S>
__host__ __device__ __forceinline__ uint32_t bslice_off(uint32_t nb, uint32_t s, uint32_t j, uint32_t k) {
  const uint32_t n = s * nb + j;
  return (k >> 3) * (16u * S * nb) + ((n >> 3) << 7) + ((k & 7u) << 4) + ((n & 7u) << 1);
}

// Global stores as inline PTX without a memory clobber: the epilogue's stores go to
// global memory only, so shared-memory values read around them need no reload.
__device__ __forceinline__ void st_f32(float* p, float v) { asm volatile("st.global.f32 [%0], %1;" ::"l"(p), "f"(v)); }
__device__ __forceinline__ void st_f64(double* p, double v) {
  asm volatile("st.global.f64 [%0], %1;" ::"l"(p), "d"(v));
}
__device__ __forceinline__ void st_v4(void* p, const uint32_t (&w)[4]) {
  asm volatile("st.global.v4.b32 [%0], {%1, %2, %3, %4};" ::"l"(p), "r"(w[0]), "r"(w[1]), "r"(w[2]), "r"(w[3]));
}

// One reduced system on the device.
struct OzInst {
  const uint8_t* Av;  // [kvp/128][ksp/32][slice][8 KB]
  const uint8_t* As;  // [ksp/128][kvp/32][slice][8 KB]
  const int* alpha_v;
  const int* alpha_s;
  const float* bh;
  const float* bl;  // [Mp][kvp]
  float *xvh, *xvl, *xsh, *xsl;  // 6-slice form: states as FP32 hi + lo, [Mp][kp]
  const double* b64;              // 9-slice form: forcing vectors and states in FP64
  double *xv64, *xs64;
  const int* kind;
  const double* period;
  const double* delay;
  double *snap_vp, *snap_sp;
  unsigned long long Tvp, Tsp;
  uint32_t fvp, fsp;
  int* expo;  // [3][Mp]: per column, the exponent of the current XS slices and the predicted
              // exponents of the next XV and XS slicing (kept across launches)
  // receivers: rows PhiVp[gid_r, :] sliced like an operator, seismogram R x T x M (device)
  const uint8_t* Ar;  // [Rp/128][kvp/32][slice][8 KB]
  const int* alpha_r;
  double* seis;
  unsigned long long Tseis;
  uint32_t fseis, R, Rp;
  uint32_t kv, ks, kvp, ksp, M, Mp;
};

// pinfo: bit 0 = part (0 or 1), bit 1 = paired, bits 2.. = pair slot.  A paired tile is
// advanced by two co-resident CTAs that split its 128-row M-tiles between them and share
// the B slices (global memory), the column maxima and a step barrier (pair_sync).
struct OzTile {
  uint32_t inst, col0, nb, pinfo;
};

struct OzArgs {
  const OzInst* inst;
  const OzTile* tiles;
  const uint32_t* order;      // tile indices, grouped by CTA
  const uint32_t* cta_begin;  // [ctas + 1]
  uint8_t* bvt;               // per CTA: slices of XV (B of the stress GEMM)
  uint8_t* bst;               // per CTA: slices of XS (B of the velocity GEMM)
  size_t bscratch;            // bytes of bvt / bst per CTA
  double dt;
  unsigned long long step0, nsteps;
  unsigned int* error;
  unsigned long long* tile_ns;  // per tile: device time of its last run
  unsigned int* pair_sync;      // per pair slot: arrival counter (zeroed before each launch)
  unsigned int* pair_levels;    // per pair slot and part: level gates opened (zeroed likewise)
  unsigned int* pair_colmax;    // per pair slot: [5][kMaxNb] column maxima; not zeroed: each part writes
                                // its maxima before the step barrier that its peer waits on before reading
};

struct Shared {
  uint64_t full[kMaxStages], empty[kMaxStages], acc_full[2], acc_empty[2], drain;
  uint64_t gate_lvl[kLevels], gate_full;  // opened by the epilogue once per new state (see the producer)
  uint32_t meta[kMaxStages];       // per pipeline stage: kMeta* flags
  int redo[2];                     // per new state (alternating): the settle re-sliced columns
  uint32_t tmem;
  int abort;
  // per-column arrays 16-byte aligned: the epilogue reads them 8 columns at a time
  __align__(16) int beta_v[kMaxNb];
  __align__(16) int beta_s[kMaxNb];   // exponents the current B tiles were sliced with
  __align__(16) int pred_v[kMaxNb];
  __align__(16) int pred_s[kMaxNb];   // predicted exponents for slicing the next new state
  unsigned int colmax[kMaxNb];
  unsigned long long reslice_v, reslice_s;  // columns to re-slice exactly after a phase
  __align__(16) float fdt_h[kMaxNb];   // f_j(t_{n-1}) * dt of the current step, as FP32 hi + lo
  __align__(16) float fdt_l[kMaxNb];
  __align__(16) double fdt64[kMaxNb];  // the same in FP64 (9-slice form)
  OzInst in;
  OzTile tile;
};

__device__ __forceinline__ void raise(Shared* sh, unsigned int* err, unsigned int code) {
  atomicOr(err, code);
  sh->abort = 1;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Accumulator set and its parity for the next M-tile; `uses` counts completed uses of
// each set.  Every role walks the same sequence, so they agree without communicating.
__device__ __forceinline__ void acc_next(uint32_t nbuf, uint32_t (&uses)[2], uint32_t& buf, uint32_t& par) {
  buf = (nbuf == 2) ? ((uses[0] + uses[1]) & 1u) : 0u;
  par = uses[buf] & 1u;
  uses[buf]++;
}

// Instruction-descriptor bit: B operand MN-major ("transpose B").
constexpr uint32_t kIdescBMnMajor = 1u << 16;

// The MMAs of one 32-wide K stage for tiles of NB columns.  The B slices of a stage are
// stacked along N (slice t = rows t*NB ..), and the diagonal accumulators along TMEM
// columns (diagonal d = columns d*NB ..), so operator slice sa times the state slices
// tb = 0 .. S-1-sa is ONE MMA of N = (S-sa)*NB whose output columns start at diagonal
// sa: S MMAs per K-step instead of S(S+1)/2 pair MMAs, each A slice read from shared
// memory once.  N is capped at 256: a longer stack is split into the fewest MMAs, with
// the slices spread evenly over them (an MMA costs ~N/2 cycles above N = 128, so 192 +
// 192 issues faster than 256 + 128).  The first MMA of a tile (sa = 0 covers every
// diagonal) starts the accumulation.  Descriptors of the stage's first A / B slice; the
// others differ only in the start-address field (16-byte units, no carry: shared
// addresses < 256 KB).
template <int S, uint32_t NB>
__device__ __forceinline__ void issue_stage(uint32_t dcol, uint32_t abase, uint32_t bbase, bool first_chunk) {
  const uint64_t adesc0 = smem_desc(abase, 128, 512);
  const uint64_t bdesc0 = smem_desc(bbase, 16u * S * NB, 128);  // MN-major state slices
  constexpr uint32_t kCap = 256u / NB;
#pragma unroll
  for (uint32_t k = 0; k < kKc / 16; ++k) {
#pragma unroll
    for (int sa = 0; sa < S; ++sa) {
      const uint64_t adesc = adesc0 + ((sa * kATile + k * 256) >> 4);
      const uint32_t acc = (!first_chunk || k > 0 || sa > 0) ? 1u : 0u;
      const uint32_t total = (uint32_t)(S - sa), parts = (total + kCap - 1) / kCap;
#pragma unroll
      for (uint32_t p = 0, tb = 0; p < parts; ++p) {
        const uint32_t take = (total - tb + (parts - p) - 1) / (parts - p);
        const uint64_t bdesc = bdesc0 + ((tb * 16u * NB + k * 32u * S * NB) >> 4);
        mma_f16(dcol + (sa + tb) * NB, adesc, bdesc, idesc_bf16(take * NB) | kIdescBMnMajor, acc);
        tb += take;
      }
    }
  }
}

// Stage metadata, written by the producer before it hands a stage over: the stage opens an
// M-tile (the issuer takes the next accumulator set), starts its accumulation, closes it
// (commit to acc_full after its MMAs), only closes it (no copies, no MMAs), or ends the
// tile (no copies, no MMAs).
constexpr uint32_t kMetaBegin = 1u, kMetaFirst = 2u, kMetaLast = 4u, kMetaEnd = 8u, kMetaCommit = 16u;

// Producer: hand the next pipeline stage over (bounded wait for it to be free), with its
// metadata and, unless it ends the tile, the bulk copies of one operator and one B stage.
template <int S>
__device__ __forceinline__ bool push_stage(uint8_t* stages, Shared* sh, uint32_t& it, uint32_t meta,
                                           const uint8_t* asrc, const uint8_t* bsrc, uint32_t bbytes,
                                           unsigned int* err) {
  using G = Geo<S>;
  const uint32_t s = it % G::kStages, ph = (it / G::kStages) & 1u;
  if (!mbar_wait(&sh->empty[s], ph ^ 1u)) {
    raise(sh, err, 1u);
    return false;
  }
  ++it;
  sh->meta[s] = meta;  // released to the issuer by the arrival below
  if (meta & (kMetaEnd | kMetaCommit)) {
    mbar_arrive(&sh->full[s]);
  } else {
    uint8_t* st = stages + (size_t)s * G::kStageBytes;
    mbar_expect_tx(&sh->full[s], G::kABytes + bbytes);
    bulk_g2s(st, asrc, G::kABytes, &sh->full[s]);
    bulk_g2s(st + G::kABytes, bsrc, bbytes, &sh->full[s]);
  }
  return true;
}

// Producer: wait (bounded) until `gate` has opened for the gi-th new state of the launch,
// then order its bulk copies after the generic-proxy writes the gate covers.
__device__ __forceinline__ bool wait_gate(Shared* sh, uint64_t* gate, uint32_t gi, unsigned int* err) {
  if (!mbar_wait(gate, gi & 1u)) {
    raise(sh, err, 64u);
    return false;
  }
  asm volatile("fence.proxy.async.global;" ::: "memory");
  return true;
}

// Acquire-poll of a global counter until it reaches target; false when `limit` polls ran out.
__device__ __forceinline__ bool poll_counter(const unsigned int* ctr, unsigned int target, unsigned long long limit) {
  for (unsigned long long i = 0; i < limit; ++i) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
    if (v >= target) return true;
  }
  return false;
}

// Producer of a paired tile: wait (bounded) until the peer part's counter of opened level
// gates (kLevels per new state) has reached `target`.
__device__ __forceinline__ bool wait_peer(Shared* sh, const unsigned int* ctr, uint32_t target, unsigned int* err) {
  if (!poll_counter(ctr, target, kWaitLimit)) {
    raise(sh, err, 128u);
    return false;
  }
  asm volatile("fence.proxy.async.global;" ::: "memory");
  return true;
}

// 2^e as an FP32 factor pair (e may leave the normal range of one factor).
__device__ __forceinline__ void pow2_pair(int e, float& f1, float& f2) {
  const int e1 = e / 2, e2 = e - e1;
  f1 = __int_as_float((e1 + 127) << 23);
  f2 = __int_as_float((e2 + 127) << 23);
}

// Read the 6 diagonal accumulators of 8 columns for this thread's row (TMEM lanes of
// quarter q) and combine them: every D_d is an integer below 2^24, so the terms
// D_d * 2^(6(5-d)) are exact in FP32 and their sum Y (< 2^55) is formed with error-free
// additions (TwoSum, smallest term first) into a double-float pair accurate to 2^-48;
// y = Y * 2^-42 (before the row / column scaling).  No integer or 64-bit conversions.
__device__ __forceinline__ void load_combine8(uint32_t tcols, uint32_t nb, int q, uint32_t j0, float* yh,
                                              float* yl) {
  constexpr int kDiags = 6;
  float D[kDiags][8];
#pragma unroll
  for (int d = 0; d < kDiags; ++d) tmem_ld8(tcols + ((uint32_t)(q * 32) << 16) + d * nb + j0, D[d]);
  tmem_wait_ld();
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) {
    float s = D[kDiags - 1][jj], e = 0.f;
#pragma unroll
    for (int d = kDiags - 2; d >= 0; --d) {
      float err;
      two_sum(s, D[d][jj] * __int_as_float((127 + 6 * (kDiags - 1 - d)) << 23), s, err);
      e += err;
    }
    const float h = s + e;
    const float l = e - (h - s);
    yh[jj] = h * 0x1p-42f;  // exact power-of-two scalings
    yl[jj] = l * 0x1p-42f;
  }
}

// With a single accumulator set (6 nb > 256, i.e. nb = 64) the TMEM columns after it,
// [6 nb, 8 nb), stage the combined values of one M-tile: the epilogue drains the
// accumulator into them (hi at +j, lo at +nb+j), hands it back to the MMA issuer, and
// finishes the state update while the next M-tile's MMAs run.
__device__ __forceinline__ bool stage_accumulator(uint32_t tcols, uint32_t spare, uint32_t nb, int q, uint32_t jbeg,
                                                  uint32_t jend, uint64_t* acc_empty) {
  for (uint32_t j0 = jbeg; j0 < jend; j0 += 8) {
    float yh[8], yl[8];
    load_combine8(tcols, nb, q, j0, yh, yl);
    tmem_st8(spare + j0, yh);
    tmem_st8(spare + nb + j0, yl);
  }
  tmem_wait_st();
  tc_fence_before();
  mbar_arrive(acc_empty);
  return true;
}

// Combined values of 8 columns: from the accumulator, or from the staging columns.
__device__ __forceinline__ void fetch_combined8(bool staged, uint32_t tcols, uint32_t spare, uint32_t nb, int q,
                                                uint32_t j0, float* yh, float* yl) {
  if (staged) {
    tmem_ld8(spare + j0, yh);
    tmem_ld8(spare + nb + j0, yl);
    tmem_wait_ld();
  } else {
    load_combine8(tcols, nb, q, j0, yh, yl);
  }
}

// x * 2^-e: one exact (or once-rounded) product when 2^-e is a normal FP32, else ldexpf.
__device__ __forceinline__ float scale_exp2f(float x, int e) {
  return (e >= -126 && e <= 126) ? x * __int_as_float((127 - e) << 23) : ldexpf(x, -e);
}

// Nearest integer of |x| < 2^22 (ties to even): adding 1.5 * 2^23 rounds x to the integer
// grid of that binade; two full-rate adds instead of a conversion-pipe rint.
__device__ __forceinline__ float round_int(float x) { return (x + 0x1.8p23f) - 0x1.8p23f; }

// The 6 balanced base-64 digits of v = h + l (|v| < 1, double-float): digits 0-2 from h
// alone (each step exact: th = 64 h, a = nearest integer of th, h = th - a), then l is
// folded in at its weight (2^18 after three steps) with one rounded add (error below
// 2^-42 of the unit), digits 3-5 from that sum.  Digit 0 is in [-64, 64], the others in
// [-32, 32]: integers, exact in BF16; the expansion matches v to within 2^-37 (the
// remainder after six digits) + 2^-43 (the rounding of the fold).
__device__ __forceinline__ void six_digits(float h, float l, float (&a)[6]) {
#pragma unroll
  for (int s = 0; s < 6; ++s) {
    if (s == 3) h += l * 0x1p18f;
    const float th = h * 64.f;
    a[s] = round_int(th);
    h = th - a[s];
  }
}

// Two FP32 values whose low 16 bits are zero (small integers) as one word of two BF16s.
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// Slice a state block (rows x nb, column-major with leading dimension kp, double-float)
// into the BF16 B tiles with per-column exponents beta[j] (|x| < 2^beta).
__device__ __forceinline__ void slice_state(const float* xh, const float* xl, uint32_t kp, uint32_t nb,
                                            const int* beta, uint8_t* tiles, unsigned long long mask, uint32_t r0,
                                            uint32_t r1) {
  const uint32_t t = threadIdx.x - 128;
  const uint32_t bbytes = Geo<6>::bstage_bytes(nb);
  const uint32_t nr = r1 - r0, n = nr * nb;
  for (uint32_t e0 = t; e0 < n; e0 += 4 * kEpiThreads) {
    float vh[4], vl[4];
    uint32_t jj[4], rr[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t e = e0 + u * kEpiThreads;
      jj[u] = e / (nr ? nr : 1);
      rr[u] = r0 + (e - jj[u] * nr);
      if (e < n && ((mask >> jj[u]) & 1ull)) {
        vh[u] = xh[(size_t)jj[u] * kp + rr[u]];
        vl[u] = xl[(size_t)jj[u] * kp + rr[u]];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (e0 + u * kEpiThreads >= n) break;
      if (!((mask >> jj[u]) & 1ull)) continue;
      float a[6];
      six_digits(scale_exp2f(vh[u], beta[jj[u]]), scale_exp2f(vl[u], beta[jj[u]]), a);
      uint8_t* base = tiles + (size_t)(rr[u] / kKc) * bbytes + bslice_off<6>(nb, 0, jj[u], rr[u] % kKc);
#pragma unroll
      for (int s = 0; s < 6; ++s)  // small integers: the upper half of the FP32 bits is the BF16
        *reinterpret_cast<uint16_t*>(base + s * 16u * nb) = (uint16_t)(__float_as_uint(a[s]) >> 16);
    }
  }
}

// Slice 8 state values of one row (columns j0 .. j0+7) into the B tiles with exponents
// e[jj] (the layout of slice_state): per slice one 16-byte store at dst + s*16*nb, dst =
// the (row, j0) byte of slice 0.  A value at or above 2^e gives meaningless slices (no
// clamp): the caller detects it from the column maximum and re-slices that column
// exactly.  Below 2^e the first slice is in [-64, 64] and every slice is exact in BF16.
__device__ __forceinline__ void slice_value8(const float* xh, const float* xl, const int* e, uint8_t* dst,
                                             uint32_t nb) {
  float a[8][6];
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) six_digits(scale_exp2f(xh[jj], e[jj]), scale_exp2f(xl[jj], e[jj]), a[jj]);
#pragma unroll
  for (int s = 0; s < 6; ++s) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = pack_bf16x2(a[2 * i][s], a[2 * i + 1][s]);
    st_v4(dst + s * 16u * nb, w);
  }
}

// ---- 9-slice form: FP64 state, integer combination and slicing -------------------

// v * 2^e for a power-of-two scaling, exact: an add to the exponent field when the
// result stays normal, ldexp otherwise.
__device__ __forceinline__ double scale_pow2(double v, int e) {
  const long long b = __double_as_longlong(v);
  const int ex = (int)((b >> 52) & 0x7FF) + e;
  if (v != 0.0 && ex > 0 && ex < 2047 && ((b >> 52) & 0x7FF) != 0) return __longlong_as_double(b + ((long long)e << 52));
  return ldexp(v, e);
}

// Read the 9 diagonal accumulators of 8 columns for this thread's row and combine them
// exactly in integers: D_d < 2^24 (integers held by FP32), Y = sum_d D_d 2^(6(8-d)) =
// H 2^36 + L with H = D_0 2^12 + D_1 2^6 + D_2 (|H| < 2^36) and L = sum_{d>=3} D_d
// 2^(6(8-d)) (|L| < 2^54); y = Y * 2^-60 before the row / column scaling.  Returned as
// the FP64 pair (H exact, L rounded once).
__device__ __forceinline__ void load_combine8_fp64(uint32_t tcols, uint32_t nb, int q, uint32_t j0, double* yH,
                                                   double* yL) {
  float D[9][8];
#pragma unroll
  for (int d = 0; d < 9; ++d) tmem_ld8(tcols + ((uint32_t)(q * 32) << 16) + d * nb + j0, D[d]);
  tmem_wait_ld();
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) {
    long long H = __float2int_rn(D[0][jj]);
    H = H * 64 + __float2int_rn(D[1][jj]);
    H = H * 64 + __float2int_rn(D[2][jj]);
    long long L = __float2int_rn(D[3][jj]);
#pragma unroll
    for (int d = 4; d < 9; ++d) L = L * 64 + __float2int_rn(D[d][jj]);
    yH[jj] = (double)H;
    yL[jj] = (double)L;
  }
}

// With one accumulator set (9 nb > 256, i.e. nb = 32) the columns after it, [9 nb, 13 nb),
// stage the combined pairs of one M-tile as raw FP64 words (yH at +2j, yL at +2nb+2j):
// the epilogue drains the accumulator, hands it back to the MMA issuer and finishes the
// state update while the next M-tile's MMAs run.
__device__ __forceinline__ void words_of(const double* y, float* w) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const long long b = __double_as_longlong(y[i]);
    w[2 * i] = __int_as_float((int)b);
    w[2 * i + 1] = __int_as_float((int)(b >> 32));
  }
}
__device__ __forceinline__ void doubles_of(const float* w, double* y) {
#pragma unroll
  for (int i = 0; i < 4; ++i)
    y[i] = __longlong_as_double(((long long)__float_as_int(w[2 * i + 1]) << 32) |
                                (unsigned int)__float_as_int(w[2 * i]));
}
__device__ __forceinline__ bool stage_accumulator_fp64(uint32_t tcols, uint32_t spare, uint32_t nb, int q,
                                                       uint32_t jbeg, uint32_t jend, uint64_t* acc_empty) {
  for (uint32_t j0 = jbeg; j0 < jend; j0 += 8) {
    double yH[8], yL[8];
    load_combine8_fp64(tcols, nb, q, j0, yH, yL);
    float w[8];
    words_of(yH, w);
    tmem_st8(spare + 2 * j0, w);
    words_of(yH + 4, w);
    tmem_st8(spare + 2 * j0 + 8, w);
    words_of(yL, w);
    tmem_st8(spare + 2 * nb + 2 * j0, w);
    words_of(yL + 4, w);
    tmem_st8(spare + 2 * nb + 2 * j0 + 8, w);
  }
  tmem_wait_st();
  tc_fence_before();
  mbar_arrive(acc_empty);
  return true;
}
__device__ __forceinline__ void fetch_combined8_fp64(bool staged, uint32_t tcols, uint32_t spare, uint32_t nb, int q,
                                                     uint32_t j0, double* yH, double* yL) {
  if (staged) {
    float w[4][8];
    tmem_ld8(spare + 2 * j0, w[0]);
    tmem_ld8(spare + 2 * j0 + 8, w[1]);
    tmem_ld8(spare + 2 * nb + 2 * j0, w[2]);
    tmem_ld8(spare + 2 * nb + 2 * j0 + 8, w[3]);
    tmem_wait_ld();
    doubles_of(w[0], yH);
    doubles_of(w[1], yH + 4);
    doubles_of(w[2], yL);
    doubles_of(w[3], yL + 4);
  } else {
    load_combine8_fp64(tcols, nb, q, j0, yH, yL);
  }
}

// x * 2^(54 - beta) rounded to an integer, from the bits of x (no FP64 arithmetic): the
// 54-bit fixed-point value of x / 2^beta for |x| < 2^beta.  Values at or above 2^beta
// give meaningless results; the caller re-slices such columns exactly.
__device__ __forceinline__ long long fixed54(double x, int beta) {
  const long long bits = __double_as_longlong(x);
  int e = (int)((bits >> 52) & 0x7FF);
  long long m = bits & 0xFFFFFFFFFFFFFLL;
  if (e == 0)
    e = 1;  // subnormal: no implicit bit
  else
    m |= 1LL << 52;
  const int sh = e - 1075 + 54 - beta;  // x / 2^beta * 2^54 = m * 2^sh
  long long v;
  if (sh >= 0)
    v = sh <= 9 ? (m << sh) : 0;
  else if (sh > -63)
    v = (m + (1LL << (-sh - 1))) >> (-sh);
  else
    v = 0;
  return bits < 0 ? -v : v;
}

// A small integer (|a| <= 256) as FP32 without a conversion: a + 1.5 * 2^23 as FP32 bits,
// back to the float a (whose low 16 bits are zero: its upper half is the BF16 of a).
__device__ __forceinline__ float float_of_int(int a) { return __int_as_float(0x4B400000 + a) - 12582912.0f; }
__device__ __forceinline__ uint32_t bf16_of_int(int a) { return __float_as_uint(float_of_int(a)) >> 16; }

// Balanced base-64 digit s (most significant first) of a 54-bit fixed-point value v;
// v keeps the remainder.  Digit 0 is in [-64, 64], digits 1-7 in [-32, 32], the last
// (the remainder itself) in [-32, 32).
template <int s>
__device__ __forceinline__ int take_digit(long long& v) {
  if constexpr (s == 8) {
    return (int)v;
  } else {
    constexpr int b = 6 * (8 - s);
    const long long a = (v + (1LL << (b - 1))) >> b;
    v -= a << b;
    return (int)a;
  }
}

template <int s>
__device__ __forceinline__ void slice9_step(long long (&v)[8], uint8_t* dst, uint32_t nb) {
  uint32_t w[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float lo = float_of_int(take_digit<s>(v[2 * i]));
    w[i] = pack_bf16x2(lo, float_of_int(take_digit<s>(v[2 * i + 1])));
  }
  st_v4(dst + s * 16u * nb, w);
  if constexpr (s < 8) slice9_step<s + 1>(v, dst, nb);
}

// 9-slice form of slice_value8: 8 FP64 values of one row into the B tiles.
__device__ __forceinline__ void slice_value8_fp64(const double* x, const int* e, uint8_t* dst, uint32_t nb) {
  long long v[8];
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) v[jj] = fixed54(x[jj], e[jj]);
  slice9_step<0>(v, dst, nb);
}

// 9-slice form of slice_state: rows [r0, r1) x nb of an FP64 state block.
__device__ __forceinline__ void slice_state_fp64(const double* x, uint32_t kp, uint32_t nb, const int* beta,
                                                 uint8_t* tiles, unsigned long long mask, uint32_t r0, uint32_t r1) {
  const uint32_t t = threadIdx.x - 128;
  const uint32_t bbytes = Geo<9>::bstage_bytes(nb);
  const uint32_t nr = r1 - r0, n = nr * nb;
  for (uint32_t e = t; e < n; e += kEpiThreads) {
    const uint32_t j = e / (nr ? nr : 1), r = r0 + (e - j * nr);
    if (!((mask >> j) & 1ull)) continue;
    long long v = fixed54(x[(size_t)j * kp + r], beta[j]);
    uint8_t* base = tiles + (size_t)(r / kKc) * bbytes + bslice_off<9>(nb, 0, j, r % kKc);
    int a[9];
    a[0] = take_digit<0>(v); a[1] = take_digit<1>(v); a[2] = take_digit<2>(v);
    a[3] = take_digit<3>(v); a[4] = take_digit<4>(v); a[5] = take_digit<5>(v);
    a[6] = take_digit<6>(v); a[7] = take_digit<7>(v); a[8] = take_digit<8>(v);
#pragma unroll
    for (int s = 0; s < 9; ++s) *reinterpret_cast<uint16_t*>(base + s * 16u * nb) = (uint16_t)bf16_of_int(a[s]);
  }
}

// Column-maximum key of an FP64 value: the upper 32 bits of |x| (monotonic in |x|).
__device__ __forceinline__ unsigned int max_key64(double x) {
  return (unsigned int)((__double_as_longlong(x) >> 32) & 0x7FFFFFFF);
}

// floor(log2 m) of a column maximum key (FP32 bits of |x| for S = 6, max_key64 for S = 9).
template <int S>
__device__ __forceinline__ int key_ilogb(unsigned int m) {
  if constexpr (S == 6)
    return ilogbf(__uint_as_float(m));
  else
    return (int)(m >> 20) - 1023;
}

// "no exponent yet": the int whose four bytes are 0x80 (what a byte-wise memset writes)
constexpr int kNoPrediction = (int)0x80808080;

// After a phase that sliced its new state with the predicted exponents pred[]: keep
// them (beta = pred) for every column whose new maximum m lies in [2^(pred-3), 2^pred)
// -- no value clamped, at most 2 bits of headroom -- and mark the other columns in
// *mask for an exact re-slice with beta = ilogb(m) + 1.  The next prediction is
// ilogb(m) + 2 (one bit of headroom).  Epilogue threads t < nb; colmax is consumed;
// *other (the other phase's mask, no longer read) is cleared.
template <int S>
__device__ __forceinline__ void settle_exponents(Shared* sh, uint32_t nb, int* beta, int* pred,
                                                 unsigned long long* mask, unsigned long long* other) {
  const uint32_t t = threadIdx.x - 128;
  if (t == 0) *other = 0ull;
  if (t < nb) {
    const unsigned int m = sh->colmax[t];
    sh->colmax[t] = 0u;
    const int p = pred[t];
    bool ok;
    if (m == 0u) {  // an all-zero column: its slices are zeros with any exponent
      ok = p != kNoPrediction;
      beta[t] = ok ? p : 0;
    } else {
      const int e = key_ilogb<S>(m);  // 2^e <= m < 2^(e+1)
      ok = p != kNoPrediction && e + 1 <= p && p <= e + 3;
      beta[t] = ok ? p : e + 1;
      pred[t] = e + 2;
    }
    if (!ok) atomicOr(mask, 1ull << t);
  }
}

// Column exponents from the maxima gathered in colmax: |x| < 2^beta.
template <int S>
__device__ __forceinline__ void column_exponents(Shared* sh, uint32_t nb, int* beta, int* pred) {
  const uint32_t t = threadIdx.x - 128;
  if (t < nb) {
    const unsigned int m = sh->colmax[t];
    beta[t] = (m != 0u) ? key_ilogb<S>(m) + 1 : 0;
    if (m != 0u) pred[t] = beta[t] + 1;
    sh->colmax[t] = 0u;
  }
}

// Column maxima over the warp's 32 rows for 8 columns j0 .. j0+7 of monotonic keys of
// |x|: eight warp reductions, then lane jj publishes column j0+jj with one shared atomic.
__device__ __forceinline__ void note_max8_keys(Shared* sh, uint32_t j0, const unsigned int* key) {
  const int lane = threadIdx.x & 31;
  unsigned int mine = 0u;
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) {
    const unsigned int m = __reduce_max_sync(0xffffffffu, key[jj]);
    if (lane == jj) mine = m;
  }
  if (lane < 8) atomicMax(&sh->colmax[j0 + lane], mine);
}
// keys of FP32 values: the bits of |x|
__device__ __forceinline__ void note_max8(Shared* sh, uint32_t j0, const float* xh) {
  unsigned int key[8];
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) key[jj] = __float_as_uint(fabsf(xh[jj]));
  note_max8_keys(sh, j0, key);
}

// 8 consecutive per-column values (j0 a multiple of 8) from shared memory as vector loads.
template <typename T>
__device__ __forceinline__ void ld8(const T* p, T* v) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
  if constexpr (sizeof(T) == 4) {
    const int4 a = reinterpret_cast<const int4*>(p)[0], b = reinterpret_cast<const int4*>(p)[1];
    const int w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
    for (int i = 0; i < 8; ++i) memcpy(v + i, w + i, 4);
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const double2 d = reinterpret_cast<const double2*>(p)[i];
      memcpy(v + 2 * i, &d.x, 8);
      memcpy(v + 2 * i + 1, &d.y, 8);
    }
  }
}

__device__ __forceinline__ void epi_barrier() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
// OR of a predicate over the 256 epilogue threads (named barrier 1).
__device__ __forceinline__ bool epi_any(bool p) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred a, b;\n setp.ne.u32 a, %1, 0;\n bar.red.or.pred b, 1, 256, a;\n selp.u32 %0, 1, 0, b;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)p)
      : "memory");
  return r != 0u;
}

// Step barrier of the two CTAs of a paired tile (called by all epilogue threads).  Thread
// 128 publishes the epilogue's global writes (release), counts its arrival and waits,
// bounded, until the peer has arrived as often; then it acquires the peer's writes for the
// generic and the bulk-copy (async) proxies.  A wait that runs out raises the error flag.
__device__ __forceinline__ void pair_sync(Shared* sh, unsigned int* ctr, uint32_t& nsync, unsigned int* err) {
  epi_barrier();
  ++nsync;
  if (threadIdx.x == 128 && !sh->abort) {
    // release this CTA's writes (ordered before by the block barrier) with the arrival,
    // acquire the peer's with the observing load; polled without sleeping (two CTAs)
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(ctr) : "memory");
    bool ok = false;
    for (unsigned long long i = 0; i < kWaitLimit; ++i) {
      unsigned int v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
      if (v >= 2u * nsync) {
        ok = true;
        break;
      }
    }
    if (!ok) raise(sh, err, 32u);
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  epi_barrier();
}

// S = 6: FP32 hi + lo state (SHAW_MIXED_OZAKI_BF16); S = 9: FP64 state (SHAW_OZAKI_FP64).
//
// Roles run decoupled within a tile: the producer (warp 0) walks the tile's phases and
// pushes pipeline stages, the MMA issuer (warp 1) consumes them in order, the epilogue
// warps (4..11) drain the accumulators, update and re-slice the state and open the gates
// through which the producer may read the new slices.  Block-wide barriers are taken only
// at tile boundaries; the epilogue warps synchronise among themselves on named barrier 1.
template <int S>
__global__ void __launch_bounds__(kThreads, 1) rom_rank2_ozaki_kernel(OzArgs a) {
  using G = Geo<S>;
  constexpr int kStages = G::kStages;
  constexpr uint32_t kABytes = G::kABytes, kStageBytes = G::kStageBytes;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* stages = smem;
  Shared* sh = reinterpret_cast<Shared*>(smem + kStages * kStageBytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ew = warp - 4;  // >= 0 on the epilogue warps
  const int q = warp & 3;   // TMEM lane quarter of this warp

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&sh->full[s], 1);
      mbar_init(&sh->empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sh->acc_full[b], 1);
      mbar_init(&sh->acc_empty[b], kEpiThreads);
    }
    mbar_init(&sh->drain, 1);
    for (uint32_t l = 0; l < kLevels; ++l) mbar_init(&sh->gate_lvl[l], 1);
    mbar_init(&sh->gate_full, 1);
    sh->abort = 0;
    mbar_init_fence();
  }
  if (warp == 2) tmem_alloc(&sh->tmem, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  const float dth = (float)a.dt, dtl = (float)(a.dt - (double)dth);
  // it: pipeline stages pushed (producer) / consumed (issuer); uses: accumulator sets taken
  // (issuer, epilogue); gbase: states produced before this tile (initial slicing + two per step)
  uint32_t it = 0, uses[2] = {0u, 0u}, gbase = 0;
  unsigned long long t_start = 0;
  for (uint32_t ti = a.cta_begin[blockIdx.x]; ti < a.cta_begin[blockIdx.x + 1]; ++ti) {
    if (threadIdx.x == 0) {
      t_start = global_ns();
      sh->tile = a.tiles[a.order[ti]];
      sh->in = a.inst[sh->tile.inst];
    }
    if (threadIdx.x < kMaxNb) {
      sh->colmax[threadIdx.x] = 0u;
      sh->beta_v[threadIdx.x] = 0;
      sh->beta_s[threadIdx.x] = 0;
      sh->pred_v[threadIdx.x] = kNoPrediction;
      sh->pred_s[threadIdx.x] = kNoPrediction;
    }
    if (threadIdx.x == 0) sh->reslice_v = sh->reslice_s = 0ull;
    if (__syncthreads_or(sh->abort != 0)) break;
    const OzInst& in = sh->in;
    const uint32_t nb = sh->tile.nb, col0 = sh->tile.col0;
    const bool paired = (sh->tile.pinfo & 2u) != 0u;
    const uint32_t part = sh->tile.pinfo & 1u, slot = sh->tile.pinfo >> 2;
    const uint32_t bbytes = G::bstage_bytes(nb);  // B stage bytes
    const uint32_t nbuf = G::acc_buffers(nb);
    const uint32_t n_mt_v = in.kvp / 128, n_mt_s = in.ksp / 128, n_kc_v = in.ksp / kKc, n_kc_s = in.kvp / kKc;
    // M-tiles of this CTA: all of them, or its half of a paired tile (part 0 the first
    // ceil(n/2), part 1 the rest); the B slices are then one buffer per pair
    auto half = [&](uint32_t n, uint32_t& m0, uint32_t& m1) {
      m0 = (paired && part) ? (n + 1) / 2 : 0u;
      m1 = (paired && !part) ? (n + 1) / 2 : n;
    };
    uint32_t mv0, mv1, ms0, ms1, mr0, mr1;
    half(n_mt_v, mv0, mv1);
    half(n_mt_s, ms0, ms1);
    half(in.Rp / 128, mr0, mr1);
    uint8_t* const bvt = a.bvt + (size_t)(paired ? slot : blockIdx.x) * a.bscratch;
    uint8_t* const bst = a.bst + (size_t)(paired ? slot : blockIdx.x) * a.bscratch;
    unsigned int* const pctr = paired ? a.pair_sync + slot : nullptr;
    unsigned int* const ectr = paired ? a.pair_levels + 2 * slot + part : nullptr;  // this part's level count
    unsigned int* const pcol = paired ? a.pair_colmax + (size_t)slot * 4 * kMaxNb : nullptr;  // [parity][part][nb]

    if (warp == 0) {
      // ---------------- producer ----------------
      // Phase by phase, the stages of its M-tiles.  The B operand of a phase is the state
      // produced before it (index g within the tile: 0 = the initial slicing, 2n + 1 = XV
      // of step n, 2n + 2 = XS of step n).  The first M-tile against a new state takes its
      // K-chunks level by level as the producing phase finishes its M-tiles -- level l =
      // the rows of the l-th M-tile of each part (level gates) -- and is closed once that
      // phase has settled its exponents (full gate): by a commit-only stage, or, if columns
      // were re-sliced, by issuing the M-tile again from chunk 0.  Every partial sum is
      // exact, so the K order does not change the result.
      if (lane == 0) {
        uint32_t passed = ~0u;  // the last full gate passed (index over the whole launch)
        const unsigned int* const peer_ctr = paired ? ectr - part + (part ^ 1u) : nullptr;
        auto phase = [&](const uint8_t* Aop, const uint8_t* Bop, uint32_t m0, uint32_t m1, uint32_t n_kc,
                         uint32_t n_src, uint32_t g) -> bool {
          const uint32_t gi = gbase + g;
          constexpr uint32_t kCpm = 128 / kKc;  // K-chunks per M-tile of the producing phase
          // M-tiles of the producing phase: this part's from own0, the peer's from peer0
          const uint32_t h = paired ? (n_src + 1) / 2 : n_src;
          const uint32_t own0 = part ? h : 0u, own_n = part ? n_src - h : h;
          const uint32_t peer0 = part ? 0u : h, peer_n = paired ? n_src - own_n : 0u;
          const uint32_t levels = max(own_n, peer_n);
          for (uint32_t mt = m0; mt < m1; ++mt) {
            const uint8_t* const arow = Aop + (size_t)mt * n_kc * kABytes;
            auto put = [&](uint32_t c, uint32_t meta) {
              return push_stage<S>(stages, sh, it, meta, arow + (size_t)c * kABytes, Bop + (size_t)c * bbytes,
                                   bbytes, a.error);
            };
            if (passed != gi) {
              uint32_t meta = kMetaBegin | kMetaFirst;
              for (uint32_t l = 0; l < levels; ++l) {
                if (!wait_gate(sh, &sh->gate_lvl[l], gi, a.error)) return false;
                if (paired && !wait_peer(sh, peer_ctr, kLevels * g + l + 1u, a.error)) return false;
                const uint32_t m_a = l < own_n ? own0 + l : ~0u, m_b = l < peer_n ? peer0 + l : ~0u;
                const uint32_t lo = min(m_a, m_b), hi = max(m_a, m_b);  // ascending K order
                for (uint32_t src : {lo, hi}) {
                  if (src == ~0u) continue;
                  for (uint32_t c = src * kCpm; c < (src + 1) * kCpm; ++c) {
                    if (!put(c, meta)) return false;
                    meta = 0u;
                  }
                }
              }
              if (!wait_gate(sh, &sh->gate_full, gi, a.error)) return false;
              passed = gi;
              if (sh->redo[gi & 1u] == 0) {
                if (!put(0u, kMetaCommit)) return false;
              } else {
                for (uint32_t c = 0; c < n_kc; ++c)
                  if (!put(c, (c == 0 ? kMetaFirst : 0u) | (c == n_kc - 1 ? kMetaLast : 0u))) return false;
              }
            } else {
              for (uint32_t c = 0; c < n_kc; ++c)
                if (!put(c, (c == 0 ? kMetaBegin | kMetaFirst : 0u) | (c == n_kc - 1 ? kMetaLast : 0u)))
                  return false;
            }
            if (sh->abort) return false;
          }
          return true;
        };
        bool ok = true;
        for (unsigned long long st = 0; st < a.nsteps && ok; ++st) {
          const unsigned long long n = a.step0 + st + 1;
          const uint32_t g = 2u * (uint32_t)st;
          ok = phase(in.Av, bst, mv0, mv1, n_kc_v, n_mt_s, g);
          if (ok && in.seis && in.fseis && n % in.fseis == 0) ok = phase(in.Ar, bvt, mr0, mr1, n_kc_s, n_mt_v, g + 1);
          if (ok) ok = phase(in.As, bvt, ms0, ms1, n_kc_s, n_mt_v, g + 1);
        }
        push_stage<S>(stages, sh, it, kMetaEnd, nullptr, nullptr, 0u, a.error);  // the issuer leaves the tile
      }
    } else if (warp == 1) {
      // ---------------- MMA issuer ----------------
      if (lane == 0) {
        uint32_t buf = 0u, dcol = sh->tmem;
        for (;;) {
          const uint32_t s = it % kStages, ph = (it / kStages) & 1u;
          if (!mbar_wait(&sh->full[s], ph)) {
            raise(sh, a.error, 4u);
            break;
          }
          ++it;
          tc_fence_after();
          const uint32_t meta = sh->meta[s];
          if (meta & kMetaEnd) {
            mbar_arrive(&sh->empty[s]);
            break;
          }
          if (meta & kMetaCommit) {  // the M-tile's MMAs are all issued: close it
            mma_commit(&sh->acc_full[buf]);
            mbar_arrive(&sh->empty[s]);
            continue;
          }
          if (meta & kMetaBegin) {
            uint32_t par;
            acc_next(nbuf, uses, buf, par);
            if (!mbar_wait(&sh->acc_empty[buf], par ^ 1u)) {
              raise(sh, a.error, 2u);
              break;
            }
            tc_fence_after();
            dcol = sh->tmem + buf * 256u;
          }
          const uint32_t abase = smem_u32(stages + (size_t)s * kStageBytes);
          const bool first = (meta & kMetaFirst) != 0u;
          // tile width as a compile-time constant: the issue sequence of a stage is then
          // straight-line code with constant descriptor offsets (a single thread issues
          // every MMA, and per-instruction index arithmetic would pace the tensor pipe)
          if (nb == 16)
            issue_stage<S, 16>(dcol, abase, abase + kABytes, first);
          else if (nb == 32)
            issue_stage<S, 32>(dcol, abase, abase + kABytes, first);
          else if constexpr (S * 64 <= 2 * 256)
            issue_stage<S, 64>(dcol, abase, abase + kABytes, first);
          mma_commit(&sh->empty[s]);
          if (meta & kMetaLast) mma_commit(&sh->acc_full[buf]);
        }
      }
    } else if (ew >= 0) {
      // ---------------- epilogue ----------------
      const uint32_t t = threadIdx.x - 128;
      const uint32_t jbeg = (uint32_t)((ew >> 2) * (nb / 2)), jend = jbeg + nb / 2;  // this group's columns
      // single accumulator set (6-slice form with nb = 64, 9-slice form with nb = 32):
      // stage its combined values in the TMEM columns after it
      const bool stage = nbuf == 1;
      const uint32_t spare = sh->tmem + ((uint32_t)(q * 32) << 16) + S * nb;
      float* const xvh = S == 6 ? in.xvh + (size_t)col0 * in.kvp : nullptr;
      float* const xvl = S == 6 ? in.xvl + (size_t)col0 * in.kvp : nullptr;
      float* const xsh = S == 6 ? in.xsh + (size_t)col0 * in.ksp : nullptr;
      float* const xsl = S == 6 ? in.xsl + (size_t)col0 * in.ksp : nullptr;
      const float* const bh = S == 6 ? in.bh + (size_t)col0 * in.kvp : nullptr;
      const float* const bl = S == 6 ? in.bl + (size_t)col0 * in.kvp : nullptr;
      double* const xv64 = S == 9 ? in.xv64 + (size_t)col0 * in.kvp : nullptr;
      double* const xs64 = S == 9 ? in.xs64 + (size_t)col0 * in.ksp : nullptr;
      const double* const b64 = S == 9 ? in.b64 + (size_t)col0 * in.kvp : nullptr;
      uint32_t nsync = 0, nx = 0, gp = gbase;
      // Paired: combine the column maxima of both parts.  Each part stores its own maxima,
      // both pass the step barrier, each folds in the peer's; the buffers alternate between
      // exchanges, so a part never overwrites maxima the peer has yet to read (it would
      // first have to pass the next barrier).
      auto exchange = [&]() {
        unsigned int* const xb = pcol + (size_t)(nx & 1u) * 2 * kMaxNb;
        ++nx;
        epi_barrier();
        if (t < nb) __stcg(xb + part * kMaxNb + t, sh->colmax[t]);
        pair_sync(sh, pctr, nsync, a.error);
        if (t < nb) sh->colmax[t] = max(sh->colmax[t], __ldcg(xb + (part ^ 1u) * kMaxNb + t));
      };
      // Level gate l of the state being produced: the slices of this part's l-th M-tile are
      // written (and, paired, the peer is told); after the last M-tile every remaining level
      // opens, so each level gate opens once per state.
      auto open_level = [&](uint32_t l, bool last) {
        asm volatile("fence.proxy.async.global;" ::: "memory");
        epi_barrier();
        if (t == 0) {
          const uint32_t top = last ? kLevels : l + 1u;
          for (uint32_t u = l; u < top; ++u) mbar_arrive(&sh->gate_lvl[u]);
          if (paired) asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(ectr), "r"(top - l) : "memory");
        }
      };
      // The full gate: every slice of the new state is final (both parts), with the re-slice
      // decision for the producer.
      auto open_full = [&](bool redo) {
        asm volatile("fence.proxy.async.global;" ::: "memory");
        epi_barrier();
        if (t == 0) {
          sh->redo[gp & 1u] = redo ? 1 : 0;
          mbar_arrive(&sh->gate_full);
        }
        ++gp;
      };
      // One phase: its M-tiles in order; a phase that produces a state opens a level gate
      // after each.
      auto epi_phase = [&](uint32_t m0, uint32_t m1, bool producing, auto&& epi) {
        for (uint32_t mt = m0; mt < m1; ++mt) {
          uint32_t buf, par;
          acc_next(nbuf, uses, buf, par);
          bool ok = !sh->abort;
          if (ok && !mbar_wait(&sh->acc_full[buf], par)) {
            raise(sh, a.error, 8u);
            ok = false;
          }
          if (ok) {
            tc_fence_after();
            // the epilogue may hand the accumulator back early (returns true once it has)
            const bool released = epi(mt, sh->tmem + buf * 256u, &sh->acc_empty[buf]);
            if (!released) {
              tc_fence_before();
              mbar_arrive(&sh->acc_empty[buf]);
            }
          }
          if (producing) open_level(mt - m0, mt + 1 == m1);
        }
      };
      // After a producing phase: settle its exponents (both parts), re-slice the columns that
      // left their predicted range, open the full gate.
      auto settle = [&](int* beta, int* pred, unsigned long long* mask, unsigned long long* other, auto&& reslice) {
        asm volatile("fence.proxy.async.global;" ::: "memory");  // slices written in the phase, for the peer's copies
        if (paired) exchange();
        epi_barrier();
        settle_exponents<S>(sh, nb, beta, pred, mask, other);
        epi_barrier();
        const unsigned long long redo = *mask;
        if (redo && !sh->abort) reslice(redo);
        asm volatile("fence.proxy.async.global;" ::: "memory");
        // paired: the re-sliced rows of both parts must land before either reads them (the
        // mask is the same in both parts, so both take this barrier or neither)
        if (paired && redo) pair_sync(sh, pctr, nsync, a.error);
        open_full(redo != 0ull);
      };

      // B tiles of the current XS (the state may be non-zero when advancing in pieces):
      // with the exponents the previous launch left (so a run in pieces slices exactly
      // as an uninterrupted run), or exact exponents for a fresh state
      {
        const uint32_t nr = (ms1 - ms0) * 128;
        for (uint32_t e = t; e < nr * nb; e += kEpiThreads) {
          const uint32_t j = e / nr, row = ms0 * 128 + (e - j * nr);
          const size_t si = (size_t)j * in.ksp + row;
          atomicMax(&sh->colmax[j], S == 6 ? __float_as_uint(fabsf(xsh[si])) : max_key64(xs64[si]));
        }
        if (paired) exchange();
        epi_barrier();
        column_exponents<S>(sh, nb, sh->beta_s, sh->pred_s);
        if (t < nb) {
          const int bs = in.expo[col0 + t];
          if (bs != kNoPrediction) {
            sh->beta_s[t] = bs;
            sh->pred_v[t] = in.expo[in.Mp + col0 + t];
            sh->pred_s[t] = in.expo[2 * in.Mp + col0 + t];
          }
        }
        epi_barrier();
        if constexpr (S == 6)
          slice_state(xsh, xsl, in.ksp, nb, sh->beta_s, bst, ~0ull, ms0 * 128, ms1 * 128);
        else
          slice_state_fp64(xs64, in.ksp, nb, sh->beta_s, bst, ~0ull, ms0 * 128, ms1 * 128);
        asm volatile("fence.proxy.async.global;" ::: "memory");
        if (paired) pair_sync(sh, pctr, nsync, a.error);  // both halves of the XS slices written
        open_level(0u, true);
        open_full(false);
      }

      for (unsigned long long st = 0; st < a.nsteps; ++st) {
        if (epi_any(sh->abort != 0)) break;
        const unsigned long long n = a.step0 + st + 1;
        if (t < nb) {
          const uint32_t col = col0 + t;
          const double f =
              col < in.M ? signal_value(in.kind[col], in.delay[col], in.period[col], (double)(n - 1) * a.dt) * a.dt
                         : 0.0;
          sh->fdt_h[t] = (float)f;
          sh->fdt_l[t] = (float)(f - (double)sh->fdt_h[t]);
          sh->fdt64[t] = f;
        }
        epi_barrier();
        // snapshot steps (StateObserver), decided once per step
        const bool snap_v = in.snap_vp && in.fvp && n % in.fvp == 0;
        const bool snap_s = in.snap_sp && in.fsp && n % in.fsp == 0;
        const unsigned long long tv = snap_v ? n / in.fvp - 1 : 0, ts = snap_s ? n / in.fsp - 1 : 0;
        // ---------------- velocity: XV += dt Av XS + fdt b ----------------
        if constexpr (S == 6)
          epi_phase(mv0, mv1, true, [&](uint32_t mt, uint32_t tcols, uint64_t* acc_empty) {
            const bool staged = stage && stage_accumulator(tcols, spare, nb, q, jbeg, jend, acc_empty);
            const uint32_t row = mt * 128 + q * 32 + lane;
            const int alpha = in.alpha_v[row];
            uint8_t* const brow = bvt + (size_t)(row / kKc) * bbytes + bslice_off<S>(nb, 0, 0, row % kKc);
            for (uint32_t j0 = jbeg; j0 < jend; j0 += 8) {
              float ph[8], pl[8], qh[8], ql[8];
              int pe[8];
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) {  // state and forcing loads ahead of the TMEM reads
                const size_t si = (size_t)(j0 + jj) * in.kvp + row;
                ph[jj] = xvh[si];
                pl[jj] = xvl[si];
                qh[jj] = bh[si];
                ql[jj] = bl[si];
              }
              float yh[8], yl[8];
              fetch_combined8(staged, tcols, spare, nb, q, j0, yh, yl);
              int b8[8], p8[8];
              float fh8[8], fl8[8];
              ld8(sh->beta_s + j0, b8);
              ld8(sh->pred_v + j0, p8);
              ld8(sh->fdt_h + j0, fh8);
              ld8(sh->fdt_l + j0, fl8);
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) {
                const uint32_t j = j0 + jj, col = col0 + j;
                const int e = alpha + b8[jj];
                const size_t si = (size_t)j * in.kvp + row;
                float xh = ph[jj], xl = pl[jj];
                float s1, s2;
                pow2_pair(e, s1, s2);
                df_fma(xh, xl, dth, dtl, yh[jj] * s1 * s2, yl[jj] * s1 * s2);
                df_fma(xh, xl, fh8[jj], fl8[jj], qh[jj], ql[jj]);
                st_f32(xvh + si, xh);
                st_f32(xvl + si, xl);
                ph[jj] = xh;
                pl[jj] = xl;
                // a column without a prediction is sliced with any exponent: it is re-sliced
                // exactly after the phase
                const int pv = p8[jj];
                pe[jj] = pv != kNoPrediction ? pv : 0;
                if (snap_v && row < in.kv && col < in.M)
                  st_f64(in.snap_vp + row + (size_t)in.kv * (tv + in.Tvp * col), (double)xh + (double)xl);
              }
              slice_value8(ph, pl, pe, brow + ((j0 >> 3) << 7), nb);
              note_max8(sh, j0, ph);
            }
            return staged;
          });
        else
          epi_phase(mv0, mv1, true, [&](uint32_t mt, uint32_t tcols, uint64_t* acc_empty) {
            const bool staged = stage && stage_accumulator_fp64(tcols, spare, nb, q, jbeg, jend, acc_empty);
            const uint32_t row = mt * 128 + q * 32 + lane;
            const int alpha = in.alpha_v[row] - 60;
            uint8_t* const brow = bvt + (size_t)(row / kKc) * bbytes + bslice_off<S>(nb, 0, 0, row % kKc);
            for (uint32_t j0 = jbeg; j0 < jend; j0 += 8) {
              double x[8], f[8];
              int pe[8];
              unsigned int key[8];
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) {  // state and forcing loads ahead of the TMEM reads
                const size_t si = (size_t)(j0 + jj) * in.kvp + row;
                x[jj] = xv64[si];
                f[jj] = b64[si];
              }
              double yH[8], yL[8];
              fetch_combined8_fp64(staged, tcols, spare, nb, q, j0, yH, yL);
              int b8[8], p8[8];
              double f8[8];
              ld8(sh->beta_s + j0, b8);
              ld8(sh->pred_v + j0, p8);
              ld8(sh->fdt64 + j0, f8);
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) {
                const uint32_t j = j0 + jj, col = col0 + j;
                const int e = alpha + b8[jj];
                // x += dt * y with y = (yH 2^36 + yL) 2^e, then x += fdt * b
                double xn = fma(scale_pow2(a.dt, e), yL[jj], x[jj]);
                xn = fma(scale_pow2(a.dt, e + 36), yH[jj], xn);
                xn = fma(f8[jj], f[jj], xn);
                st_f64(xv64 + (size_t)j * in.kvp + row, xn);
                x[jj] = xn;
                key[jj] = max_key64(xn);
                const int pv = p8[jj];
                pe[jj] = pv != kNoPrediction ? pv : 0;
                if (snap_v && row < in.kv && col < in.M)
                  st_f64(in.snap_vp + row + (size_t)in.kv * (tv + in.Tvp * col), xn);
              }
              slice_value8_fp64(x, pe, brow + ((j0 >> 3) << 7), nb);
              note_max8_keys(sh, j0, key);
            }
            return staged;
          });
        settle(sh->beta_v, sh->pred_v, &sh->reslice_v, &sh->reslice_s, [&](unsigned long long redo) {
          if constexpr (S == 6)
            slice_state(xvh, xvl, in.kvp, nb, sh->beta_v, bvt, redo, mv0 * 128, mv1 * 128);
          else
            slice_state_fp64(xv64, in.kvp, nb, sh->beta_v, bvt, redo, mv0 * 128, mv1 * 128);
        });
        if (epi_any(sh->abort != 0)) break;
        // ---------------- seismogram on sample steps: S(:, t, cols) = PhiRcv XV ----------------
        // (main_reconstruct_seismo.cc:157-185 in the loop; the XV slices of the stress GEMM
        // are its B operand, so the product is exact like the leapfrog's)
        if (in.seis && in.fseis && n % in.fseis == 0) {
          const unsigned long long tcnt = n / in.fseis - 1;
          epi_phase(mr0, mr1, false, [&](uint32_t mt, uint32_t tcols, uint64_t*) {
            const uint32_t r = mt * 128 + q * 32 + lane;
            const int alpha = in.alpha_r[r];
            for (uint32_t j0 = jbeg; j0 < jend; j0 += 8) {
              double v[8];
              if constexpr (S == 6) {
                float yh[8], yl[8];
                load_combine8(tcols, nb, q, j0, yh, yl);
#pragma unroll
                for (int jj = 0; jj < 8; ++jj)
                  v[jj] = ldexp((double)yh[jj] + (double)yl[jj], alpha + sh->beta_v[j0 + jj]);
              } else {
                double yH[8], yL[8];
                load_combine8_fp64(tcols, nb, q, j0, yH, yL);
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) {
                  const int e = alpha + sh->beta_v[j0 + jj] - 60;
                  v[jj] = fma(scale_pow2(1.0, e + 36), yH[jj], scale_pow2(yL[jj], e));
                }
              }
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) {
                const uint32_t col = col0 + j0 + jj;
                if (r < in.R && col < in.M) st_f64(in.seis + r + (size_t)in.R * (tcnt + in.Tseis * col), v[jj]);
              }
            }
            return false;
          });
          if (epi_any(sh->abort != 0)) break;
        }
        // ---------------- stress: XS += dt As XV ----------------
        if constexpr (S == 6)
          epi_phase(ms0, ms1, true, [&](uint32_t mt, uint32_t tcols, uint64_t* acc_empty) {
            const bool staged = stage && stage_accumulator(tcols, spare, nb, q, jbeg, jend, acc_empty);
            const uint32_t row = mt * 128 + q * 32 + lane;
            const int alpha = in.alpha_s[row];
            uint8_t* const brow = bst + (size_t)(row / kKc) * bbytes + bslice_off<S>(nb, 0, 0, row % kKc);
            for (uint32_t j0 = jbeg; j0 < jend; j0 += 8) {
              float ph[8], pl[8];
              int pe[8];
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) {
                const size_t si = (size_t)(j0 + jj) * in.ksp + row;
                ph[jj] = xsh[si];
                pl[jj] = xsl[si];
              }
              float yh[8], yl[8];
              fetch_combined8(staged, tcols, spare, nb, q, j0, yh, yl);
              int b8[8], p8[8];
              ld8(sh->beta_v + j0, b8);
              ld8(sh->pred_s + j0, p8);
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) {
                const uint32_t j = j0 + jj, col = col0 + j;
                const int e = alpha + b8[jj];
                const size_t si = (size_t)j * in.ksp + row;
                float xh = ph[jj], xl = pl[jj];
                float s1, s2;
                pow2_pair(e, s1, s2);
                df_fma(xh, xl, dth, dtl, yh[jj] * s1 * s2, yl[jj] * s1 * s2);
                st_f32(xsh + si, xh);
                st_f32(xsl + si, xl);
                ph[jj] = xh;
                pl[jj] = xl;
                const int ps = p8[jj];
                pe[jj] = ps != kNoPrediction ? ps : 0;
                if (snap_s && row < in.ks && col < in.M)
                  st_f64(in.snap_sp + row + (size_t)in.ks * (ts + in.Tsp * col), (double)xh + (double)xl);
              }
              slice_value8(ph, pl, pe, brow + ((j0 >> 3) << 7), nb);
              note_max8(sh, j0, ph);
            }
            return staged;
          });
        else
          epi_phase(ms0, ms1, true, [&](uint32_t mt, uint32_t tcols, uint64_t* acc_empty) {
            const bool staged = stage && stage_accumulator_fp64(tcols, spare, nb, q, jbeg, jend, acc_empty);
            const uint32_t row = mt * 128 + q * 32 + lane;
            const int alpha = in.alpha_s[row] - 60;
            uint8_t* const brow = bst + (size_t)(row / kKc) * bbytes + bslice_off<S>(nb, 0, 0, row % kKc);
            for (uint32_t j0 = jbeg; j0 < jend; j0 += 8) {
              double x[8];
              int pe[8];
              unsigned int key[8];
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) x[jj] = xs64[(size_t)(j0 + jj) * in.ksp + row];
              double yH[8], yL[8];
              fetch_combined8_fp64(staged, tcols, spare, nb, q, j0, yH, yL);
              int b8[8], p8[8];
              ld8(sh->beta_v + j0, b8);
              ld8(sh->pred_s + j0, p8);
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) {
                const uint32_t j = j0 + jj, col = col0 + j;
                const int e = alpha + b8[jj];
                double xn = fma(scale_pow2(a.dt, e), yL[jj], x[jj]);
                xn = fma(scale_pow2(a.dt, e + 36), yH[jj], xn);
                st_f64(xs64 + (size_t)j * in.ksp + row, xn);
                x[jj] = xn;
                key[jj] = max_key64(xn);
                const int ps = p8[jj];
                pe[jj] = ps != kNoPrediction ? ps : 0;
                if (snap_s && row < in.ks && col < in.M)
                  st_f64(in.snap_sp + row + (size_t)in.ks * (ts + in.Tsp * col), xn);
              }
              slice_value8_fp64(x, pe, brow + ((j0 >> 3) << 7), nb);
              note_max8_keys(sh, j0, key);
            }
            return staged;
          });
        settle(sh->beta_s, sh->pred_s, &sh->reslice_s, &sh->reslice_v, [&](unsigned long long redo) {
          if constexpr (S == 6)
            slice_state(xsh, xsl, in.ksp, nb, sh->beta_s, bst, redo, ms0 * 128, ms1 * 128);
          else
            slice_state_fp64(xs64, in.ksp, nb, sh->beta_s, bst, redo, ms0 * 128, ms1 * 128);
        });
      }
      if (t < nb && part == 0u) {  // exponents for the next launch
        in.expo[col0 + t] = sh->beta_s[t];
        in.expo[in.Mp + col0 + t] = sh->pred_v[t];
        in.expo[2 * in.Mp + col0 + t] = sh->pred_s[t];
      }
    }
    gbase += 2u * (uint32_t)a.nsteps + 1u;
    const bool stop = __syncthreads_or(sh->abort != 0);
    if (threadIdx.x == 0 && a.tile_ns) a.tile_ns[a.order[ti]] = global_ns() - t_start;
    if (stop) break;
  }
  // no bulk copy may still be landing in shared memory when the CTA leaves (after an
  // aborted run the issuer may not have consumed the last stages): wait, bounded, for the
  // full barriers of the producer's last pushes
  if (warp == 0 && lane == 0) {
    for (uint32_t i = it > (uint32_t)kStages ? it - kStages : 0u; i < it; ++i)
      if (!mbar_wait(&sh->full[i % kStages], (i / kStages) & 1u)) atomicOr(a.error, 16u);
  }
  // drain: no MMA may still be in flight when TMEM is released
  if (warp == 1 && lane == 0) {
    mma_commit(&sh->drain);
    if (!mbar_wait(&sh->drain, 0)) atomicOr(a.error, 16u);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) tmem_dealloc(sh->tmem, kTmemCols);
}

// Diagnostic of the bounded waits, each on an event that never happens: an mbarrier phase
// that nothing completes (the wait of gates, stages and accumulators) and a global counter
// that nothing increments (the wait on the peer of a paired tile).  Each must give up after
// `polls` polls; status gets the error bits the kernel uses for them (64, 128).
__global__ void oz_wait_selftest_kernel(unsigned long long polls, const unsigned int* ctr,
                                        const unsigned long long* word, unsigned int* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int s = 0u;
    if (!mbar_wait_n(&bar, 0u, polls)) s |= 64u;      // phase 0: nobody arrives
    if (!poll_counter(ctr, 1u, polls)) s |= 128u;     // the counter stays 0
    // the band kernels' row exchange: a tagged word that nobody writes (it stays 0, tag 1)
    double x = 0.0;
    const unsigned long long* const src[1] = {word};
    double* const dst[1] = {&x};
    const uint32_t lim = (uint32_t)(polls < shaw::l2x::kPollLimit ? polls : shaw::l2x::kPollLimit);
    if (!shaw::l2x::poll<1>(src, dst, 1u, 1u, lim)) s |= 256u;
    *status = s;
  }
}

// state (hi + lo, [Mp][kp]) -> FP64 LayoutLeft k x M
__global__ void oz_gather_state_kernel(const float* h, const float* l, uint32_t k, uint32_t M, uint32_t kp,
                                       double* out) {
  const size_t n = (size_t)k * M;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const uint32_t col = (uint32_t)(e / k), row = (uint32_t)(e % k);
    out[e] = (double)h[(size_t)col * kp + row] + (double)l[(size_t)col * kp + row];
  }
}

// FP64 state ([Mp][kp]) -> LayoutLeft k x M
__global__ void oz_gather_state64_kernel(const double* x, uint32_t k, uint32_t M, uint32_t kp, double* out) {
  const size_t n = (size_t)k * M;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const uint32_t col = (uint32_t)(e / k), row = (uint32_t)(e % k);
    out[e] = x[(size_t)col * kp + row];
  }
}

uint32_t round_up(uint32_t x, uint32_t m) { return (x + m - 1) / m * m; }

uint16_t bf16_bits_of_int(double a) {
  const float f = (float)a;  // |a| <= 64: exact in BF16
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (uint16_t)(u >> 16);
}

// Row-scaled 6-bit slices (S of them) of a row-major FP64 operator (rows x cols),
// padded, tiled as [rows_p/128][cols_p/32][slice][128 x 32 BF16 tile]; alpha[r] = row
// exponent.
void slice_operator(const double* A, uint32_t rows, uint32_t cols, uint32_t rows_p, uint32_t cols_p, int kSlices,
                    std::vector<uint16_t>& out, std::vector<int>& alpha) {
  const uint32_t n_kc = cols_p / kKc;
  out.assign((size_t)rows_p * cols_p * kSlices, 0);
  alpha.assign(rows_p, 0);
  for (uint32_t r = 0; r < rows; ++r) {
    double mx = 0.0;
    for (uint32_t c = 0; c < cols; ++c) mx = std::max(mx, std::fabs(A[(size_t)r * cols + c]));
    const int e = mx > 0.0 ? std::ilogb(mx) + 1 : 0;
    alpha[r] = e;
    for (uint32_t c = 0; c < cols; ++c) {
      double v = std::ldexp(A[(size_t)r * cols + c], -e);
      const uint32_t mt = r / 128, kc = c / kKc;
      const size_t tile = ((size_t)mt * n_kc + kc) * kSlices;
      const uint32_t off = tile_off(r % 128, c % kKc) / 2;
      for (int s = 0; s < kSlices; ++s) {
        const double t = v * 64.0;
        double q = std::nearbyint(t);
        q = std::min(64.0, std::max(-64.0, q));
        v = t - q;
        out[(tile + s) * (kATile / 2) + off] = bf16_bits_of_int(q);
      }
    }
  }
}

// Longest processing time first: tiles by decreasing cost, each to the least-loaded CTA.
void lpt_schedule(const std::vector<double>& cost, uint32_t ctas, std::vector<uint32_t>& order,
                  std::vector<uint32_t>& begin, double& makespan) {
  std::vector<uint32_t> idx(cost.size());
  std::iota(idx.begin(), idx.end(), 0u);
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t x, uint32_t y) { return cost[x] > cost[y]; });
  using Slot = std::pair<double, uint32_t>;
  std::priority_queue<Slot, std::vector<Slot>, std::greater<Slot>> pq;
  for (uint32_t c = 0; c < ctas; ++c) pq.push({0.0, c});
  std::vector<std::vector<uint32_t>> per(ctas);
  makespan = 0.0;
  for (uint32_t t : idx) {
    Slot s = pq.top();
    pq.pop();
    per[s.second].push_back(t);
    s.first += cost[t];
    makespan = std::max(makespan, s.first);
    pq.push(s);
  }
  order.clear();
  begin.assign(ctas + 1, 0u);
  for (uint32_t c = 0; c < ctas; ++c) {
    begin[c] = (uint32_t)order.size();
    order.insert(order.end(), per[c].begin(), per[c].end());
  }
  begin[ctas] = (uint32_t)order.size();
}

}  // namespace

struct Batch {
  std::vector<OzInst> inst;  // host copy of the device table
  OzInst* d_inst = nullptr;
  std::vector<void*> owned;  // device buffers of the instances
  // tiling
  int slices = 6;        // 6: FP32 hi + lo state; 9: FP64 state
  uint32_t max_nb = 64;  // widest tile of the form
  uint32_t width = 32;
  bool paired = false;  // every tile split over two co-resident CTAs (one tile part per CTA)
  std::string sched_source = "model";
  std::vector<OzTile> tiles;
  std::vector<uint32_t> order, begin;
  uint32_t ctas = 0, max_tiles = 0;
  double model_makespan = 0.0;
  OzTile* d_tiles = nullptr;
  uint32_t *d_order = nullptr, *d_begin = nullptr;
  uint8_t *bvt = nullptr, *bst = nullptr;
  size_t bscratch = 0;
  unsigned int* error = nullptr;
  unsigned long long* tile_ns = nullptr;
  unsigned int *pair_sync = nullptr, *pair_colmax = nullptr;
  size_t smem = 0;
  int sms = 0;
  bool table_dirty = true, tiles_dirty = true;
};

namespace {

uint32_t tile_width_for(uint32_t M, uint32_t W) {
  uint32_t nb = 16;
  while (nb < W && nb < M) nb *= 2;
  return nb;
}

// Modelled cost of one tile per step (arbitrary units): the 2 x S(S+1)/2 slice-pair MMAs
// of 128 x nb x 16 and the per-element epilogue and re-slicing work.
double tile_model_cost(const OzInst& in, uint32_t nb, int S) {
  return (double)nb * ((double)in.kvp * in.ksp * (S * (S + 1) / 2) / 2048.0 + 15.0 * (in.kvp + in.ksp)) + 2000.0;
}

// Paired tiling is possible when every instance has at least two M-tiles per phase and the
// tile parts fit one per SM (the two parts of a pair wait on each other, so all CTAs must
// be resident at once: the launch is cooperative).
bool pairing_fits(const Batch* p, uint32_t W) {
  uint32_t n = 0;
  for (const OzInst& in : p->inst) {
    if (in.kvp < 256 || in.ksp < 256) return false;
    const uint32_t nb = tile_width_for(in.M, W);
    n += (in.M + nb - 1) / nb;
  }
  return 2 * n <= (uint32_t)p->sms;
}

void build_tiles(Batch* p, uint32_t W, bool paired = false) {
  p->width = W;
  p->paired = paired;
  p->tiles.clear();
  uint32_t slot = 0;
  for (uint32_t i = 0; i < (uint32_t)p->inst.size(); ++i) {
    const uint32_t nb = tile_width_for(p->inst[i].M, W);
    for (uint32_t c = 0; c < p->inst[i].M; c += nb, ++slot) {
      if (!paired) {
        p->tiles.push_back({i, c, nb, 0u});
      } else {
        p->tiles.push_back({i, c, nb, (slot << 2) | 2u});
        p->tiles.push_back({i, c, nb, (slot << 2) | 3u});
      }
    }
  }
  p->ctas = std::min<uint32_t>((uint32_t)p->tiles.size(), (uint32_t)p->sms);
  if (paired) {  // one tile part per CTA
    p->order.resize(p->tiles.size());
    std::iota(p->order.begin(), p->order.end(), 0u);
    p->begin.resize(p->ctas + 1);
    std::iota(p->begin.begin(), p->begin.end(), 0u);
    p->model_makespan = tile_model_cost(p->inst[0], p->tiles[0].nb, p->slices) / 2;
    p->sched_source = "paired";
    p->tiles_dirty = true;
    return;
  }
  std::vector<double> cost(p->tiles.size());
  for (size_t t = 0; t < p->tiles.size(); ++t)
    cost[t] = tile_model_cost(p->inst[p->tiles[t].inst], p->tiles[t].nb, p->slices);
  lpt_schedule(cost, p->ctas, p->order, p->begin, p->model_makespan);
  p->sched_source = "model";
  p->tiles_dirty = true;
}

int upload(Batch* p, cudaStream_t s) {
  if (p->table_dirty) {
    SHAW_CUDA(cudaMemcpyAsync(p->d_inst, p->inst.data(), p->inst.size() * sizeof(OzInst), cudaMemcpyHostToDevice, s));
    p->table_dirty = false;
  }
  if (p->tiles_dirty) {
    SHAW_CUDA(cudaMemcpyAsync(p->d_tiles, p->tiles.data(), p->tiles.size() * sizeof(OzTile), cudaMemcpyHostToDevice, s));
    SHAW_CUDA(cudaMemcpyAsync(p->d_order, p->order.data(), p->order.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                              s));
    SHAW_CUDA(cudaMemcpyAsync(p->d_begin, p->begin.data(), p->begin.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                              s));
    p->tiles_dirty = false;
  }
  return SHAW_OK;
}

}  // namespace

int create(Batch*& p, uint32_t n, const InstanceDesc* d, cudaStream_t s, int slices) {
  p = nullptr;
  if (slices != 6 && slices != 9) return fail(SHAW_ERR_INVALID_ARG, "slice count must be 6 or 9");
  if (n == 0 || !d) return fail(SHAW_ERR_INVALID_ARG, "empty batch");
  for (uint32_t i = 0; i < n; ++i) {
    if (d[i].kv == 0 || d[i].ks == 0 || d[i].M == 0 || !d[i].Av || !d[i].As || !d[i].b)
      return fail(SHAW_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": empty sizes or null operator");
    if (d[i].kv > 1024 || d[i].ks > 1024)
      return fail(SHAW_ERR_UNSUPPORTED, "the Ozaki tensor-core ROM supports at most 1024 modes per dof");
  }
  Batch* b = new Batch();
  b->slices = slices;
  b->max_nb = slices == 6 ? Geo<6>::kMaxNb : Geo<9>::kMaxNb;
  int dev = 0;
  cudaError_t e;
  auto bail = [&](int rc) {
    destroy(b);
    return rc;
  };
#define OZ_TRY(call) do { e = (call); if (e != cudaSuccess) return bail(cuda_fail(e, #call)); } while (0)
  OZ_TRY(cudaGetDevice(&dev));
  OZ_TRY(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev));
  uint32_t kmax_p = 128;
  b->inst.resize(n);
  for (uint32_t i = 0; i < n; ++i) {
    OzInst& in = b->inst[i];
    std::memset(&in, 0, sizeof(in));
    in.kv = d[i].kv; in.ks = d[i].ks; in.M = d[i].M;
    in.kvp = round_up(in.kv, 128); in.ksp = round_up(in.ks, 128); in.Mp = round_up(in.M, kMaxNb);
    kmax_p = std::max(kmax_p, std::max(in.kvp, in.ksp));
    b->max_tiles += 2 * ((in.M + 15) / 16);
    std::vector<uint16_t> sv, ss;
    std::vector<int> av, as;
    slice_operator(d[i].Av, in.kv, in.ks, in.kvp, in.ksp, slices, sv, av);
    slice_operator(d[i].As, in.ks, in.kv, in.ksp, in.kvp, slices, ss, as);
    std::vector<float> bh, bl;
    std::vector<double> b64;
    if (slices == 6) {
      bh.assign((size_t)in.Mp * in.kvp, 0.f);
      bl.assign((size_t)in.Mp * in.kvp, 0.f);
    } else {
      b64.assign((size_t)in.Mp * in.kvp, 0.0);
    }
    for (uint32_t c = 0; c < in.M; ++c)
      for (uint32_t r = 0; r < in.kv; ++r) {
        const double v = d[i].b[(size_t)c * in.kv + r];
        if (slices == 6) {
          const float h = (float)v;
          bh[(size_t)c * in.kvp + r] = h;
          bl[(size_t)c * in.kvp + r] = (float)(v - (double)h);
        } else {
          b64[(size_t)c * in.kvp + r] = v;
        }
      }
    auto alloc = [&](void** ptr, size_t bytes) {
      const cudaError_t r = cudaMalloc(ptr, bytes);
      if (r == cudaSuccess) b->owned.push_back(*ptr);
      return r;
    };
    const size_t nv = (size_t)in.Mp * in.kvp, ns = (size_t)in.Mp * in.ksp;
    OZ_TRY(alloc((void**)&in.Av, sv.size() * 2));
    OZ_TRY(alloc((void**)&in.As, ss.size() * 2));
    OZ_TRY(alloc((void**)&in.alpha_v, in.kvp * sizeof(int)));
    OZ_TRY(alloc((void**)&in.alpha_s, in.ksp * sizeof(int)));
    if (slices == 6) {
      OZ_TRY(alloc((void**)&in.bh, nv * sizeof(float)));
      OZ_TRY(alloc((void**)&in.bl, nv * sizeof(float)));
      OZ_TRY(alloc((void**)&in.xvh, nv * sizeof(float)));
      OZ_TRY(alloc((void**)&in.xvl, nv * sizeof(float)));
      OZ_TRY(alloc((void**)&in.xsh, ns * sizeof(float)));
      OZ_TRY(alloc((void**)&in.xsl, ns * sizeof(float)));
    } else {
      OZ_TRY(alloc((void**)&in.b64, nv * sizeof(double)));
      OZ_TRY(alloc((void**)&in.xv64, nv * sizeof(double)));
      OZ_TRY(alloc((void**)&in.xs64, ns * sizeof(double)));
    }
    OZ_TRY(alloc((void**)&in.expo, 3 * (size_t)in.Mp * sizeof(int)));
    OZ_TRY(cudaMemcpyAsync((void*)in.Av, sv.data(), sv.size() * 2, cudaMemcpyHostToDevice, s));
    OZ_TRY(cudaMemcpyAsync((void*)in.As, ss.data(), ss.size() * 2, cudaMemcpyHostToDevice, s));
    OZ_TRY(cudaMemcpyAsync((void*)in.alpha_v, av.data(), av.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    OZ_TRY(cudaMemcpyAsync((void*)in.alpha_s, as.data(), as.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    if (slices == 6) {
      OZ_TRY(cudaMemcpyAsync((void*)in.bh, bh.data(), nv * sizeof(float), cudaMemcpyHostToDevice, s));
      OZ_TRY(cudaMemcpyAsync((void*)in.bl, bl.data(), nv * sizeof(float), cudaMemcpyHostToDevice, s));
    } else {
      OZ_TRY(cudaMemcpyAsync((void*)in.b64, b64.data(), nv * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    OZ_TRY(cudaStreamSynchronize(s));  // the host vectors go out of scope
  }
  b->bscratch = (size_t)(kmax_p / kKc) * kRowBytes * (size_t)slices * b->max_nb;  // one B operand, widest tile
  OZ_TRY(cudaMalloc(&b->d_inst, n * sizeof(OzInst)));
  OZ_TRY(cudaMalloc(&b->d_tiles, b->max_tiles * sizeof(OzTile)));
  OZ_TRY(cudaMalloc(&b->d_order, b->max_tiles * sizeof(uint32_t)));
  OZ_TRY(cudaMalloc(&b->d_begin, ((size_t)b->sms + 1) * sizeof(uint32_t)));
  OZ_TRY(cudaMalloc(&b->bvt, (size_t)b->sms * b->bscratch));
  OZ_TRY(cudaMalloc(&b->bst, (size_t)b->sms * b->bscratch));
  OZ_TRY(cudaMalloc(&b->error, sizeof(unsigned int)));
  OZ_TRY(cudaMalloc(&b->tile_ns, b->max_tiles * sizeof(unsigned long long)));
  OZ_TRY(cudaMalloc(&b->pair_sync, (size_t)2 * b->sms * sizeof(unsigned int)));  // step barrier, level gates
  OZ_TRY(cudaMalloc(&b->pair_colmax, (size_t)b->sms * 4 * kMaxNb * sizeof(unsigned int)));
#undef OZ_TRY
  b->smem = slices == 6 ? (size_t)Geo<6>::kStages * Geo<6>::kStageBytes + sizeof(Shared)
                         : (size_t)Geo<9>::kStages * Geo<9>::kStageBytes + sizeof(Shared);
  // default tiling: tiles split across CTA pairs where they fit (the widest tiles that
  // still occupy half the SMs, else the narrowest); otherwise 32-column tiles (64 when a
  // single wide system fills every SM twice), at most the form's widest tile
  uint32_t pw = 0;
  for (uint32_t W : {16u, 32u, 64u}) {
    if (W > b->max_nb || !pairing_fits(b, W)) continue;
    uint32_t parts = 0;
    for (const OzInst& in : b->inst) parts += 2 * ((in.M + tile_width_for(in.M, W) - 1) / tile_width_for(in.M, W));
    if (pw == 0 || 2 * parts >= (uint32_t)b->sms) pw = W;
  }
  if (pw)
    build_tiles(b, pw, true);
  else
    build_tiles(b, std::min(b->max_nb, (n == 1 && d[0].M >= 64u * (uint32_t)b->sms) ? 64u : 32u));
  p = b;
  return reset(p, s);
}

int set_signals(Batch* p, uint32_t i, const int* kind, const double* period, const double* delay) {
  if (!p || i >= p->inst.size()) return fail(SHAW_ERR_INVALID_ARG, "instance index out of range");
  p->inst[i].kind = kind;
  p->inst[i].period = period;
  p->inst[i].delay = delay;
  p->table_dirty = true;
  return SHAW_OK;
}

int set_snapshots(Batch* p, uint32_t i, double* snap_vp, double* snap_sp, unsigned long long Tvp,
                  unsigned long long Tsp, uint32_t fvp, uint32_t fsp) {
  if (!p || i >= p->inst.size()) return fail(SHAW_ERR_INVALID_ARG, "instance index out of range");
  OzInst& in = p->inst[i];
  if (in.snap_vp != snap_vp || in.snap_sp != snap_sp || in.Tvp != Tvp || in.Tsp != Tsp || in.fvp != fvp ||
      in.fsp != fsp) {
    in.snap_vp = snap_vp; in.snap_sp = snap_sp; in.Tvp = Tvp; in.Tsp = Tsp; in.fvp = fvp; in.fsp = fsp;
    p->table_dirty = true;
  }
  return SHAW_OK;
}

int set_receivers(Batch* p, uint32_t i, const double* rows, uint32_t R, double* d_seis, unsigned long long T,
                  uint32_t freq, cudaStream_t s) {
  if (!p || i >= p->inst.size()) return fail(SHAW_ERR_INVALID_ARG, "instance index out of range");
  OzInst& in = p->inst[i];
  SHAW_CUDA(cudaStreamSynchronize(s));
  if (in.Ar) cudaFree((void*)in.Ar);
  if (in.alpha_r) cudaFree((void*)in.alpha_r);
  in.Ar = nullptr; in.alpha_r = nullptr; in.seis = nullptr; in.R = in.Rp = in.fseis = 0; in.Tseis = 0;
  p->table_dirty = true;
  if (R == 0) return SHAW_OK;
  const uint32_t Rp = round_up(R, 128);
  std::vector<uint16_t> sl;
  std::vector<int> al;
  slice_operator(rows, R, in.kv, Rp, in.kvp, p->slices, sl, al);
  uint8_t* dA = nullptr;
  int* dal = nullptr;
  SHAW_CUDA(cudaMalloc(&dA, sl.size() * 2));
  cudaError_t e = cudaMalloc(&dal, Rp * sizeof(int));
  if (e != cudaSuccess) {
    cudaFree(dA);
    return cuda_fail(e, "cudaMalloc (receiver exponents)");
  }
  in.Ar = dA;
  in.alpha_r = dal;
  SHAW_CUDA(cudaMemcpyAsync(dA, sl.data(), sl.size() * 2, cudaMemcpyHostToDevice, s));
  SHAW_CUDA(cudaMemcpyAsync(dal, al.data(), Rp * sizeof(int), cudaMemcpyHostToDevice, s));
  SHAW_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
  in.seis = d_seis; in.R = R; in.Rp = Rp; in.Tseis = T; in.fseis = freq;
  return SHAW_OK;
}

int reset(Batch* p, cudaStream_t s) {
  for (const OzInst& in : p->inst) {
    const size_t nv = (size_t)in.Mp * in.kvp, ns = (size_t)in.Mp * in.ksp;
    if (p->slices == 6) {
      SHAW_CUDA(cudaMemsetAsync(in.xvh, 0, nv * sizeof(float), s));
      SHAW_CUDA(cudaMemsetAsync(in.xvl, 0, nv * sizeof(float), s));
      SHAW_CUDA(cudaMemsetAsync(in.xsh, 0, ns * sizeof(float), s));
      SHAW_CUDA(cudaMemsetAsync(in.xsl, 0, ns * sizeof(float), s));
    } else {
      SHAW_CUDA(cudaMemsetAsync(in.xv64, 0, nv * sizeof(double), s));
      SHAW_CUDA(cudaMemsetAsync(in.xs64, 0, ns * sizeof(double), s));
    }
    SHAW_CUDA(cudaMemsetAsync(in.expo, 0x80, 3 * (size_t)in.Mp * sizeof(int), s));  // kNoPrediction
  }
  SHAW_CUDA(cudaMemsetAsync(p->error, 0, sizeof(unsigned int), s));
  return SHAW_OK;
}

int advance(Batch* p, cudaStream_t s, double dt, unsigned long long step0, unsigned long long nsteps) {
  for (size_t i = 0; i < p->inst.size(); ++i)
    if (!p->inst[i].kind) return fail(SHAW_ERR_STATE, "instance " + std::to_string(i) + " has no signals");
  if (int rc = upload(p, s)) return rc;
  OzArgs a;
  std::memset(&a, 0, sizeof(a));
  a.inst = p->d_inst; a.tiles = p->d_tiles; a.order = p->d_order; a.cta_begin = p->d_begin;
  a.bvt = p->bvt; a.bst = p->bst; a.bscratch = p->bscratch;
  a.dt = dt; a.step0 = step0; a.nsteps = nsteps; a.error = p->error; a.tile_ns = p->tile_ns;
  a.pair_sync = p->pair_sync; a.pair_levels = p->pair_sync + p->sms; a.pair_colmax = p->pair_colmax;
  void (*kern)(OzArgs) = p->slices == 6 ? rom_rank2_ozaki_kernel<6> : rom_rank2_ozaki_kernel<9>;
  SHAW_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem));
  if (p->paired) {  // the parts of a pair wait on each other: all CTAs resident (cooperative launch)
    SHAW_CUDA(cudaMemsetAsync(p->pair_sync, 0, (size_t)2 * p->sms * sizeof(unsigned int), s));
    void* args[] = {&a};
    SHAW_CUDA(cudaLaunchCooperativeKernel((const void*)kern, dim3(p->ctas), dim3(kThreads), args, p->smem, s));
  } else {
    kern<<<p->ctas, kThreads, p->smem, s>>>(a);
  }
  SHAW_CUDA(cudaGetLastError());
  return SHAW_OK;
}

int check(Batch* p, cudaStream_t s) {
  unsigned int err = 0;
  SHAW_CUDA(cudaMemcpyAsync(&err, p->error, sizeof(err), cudaMemcpyDeviceToHost, s));
  SHAW_CUDA(cudaStreamSynchronize(s));
  if (err)
    return fail(SHAW_ERR_CUDA, "Ozaki tensor-core ROM kernel: a pipeline wait ran out (code " +
                                   std::to_string(err) + ")");
  return SHAW_OK;
}

int get_state(Batch* p, uint32_t i, cudaStream_t s, double* dxv, double* dxs) {
  if (i >= p->inst.size()) return fail(SHAW_ERR_INVALID_ARG, "instance index out of range");
  const OzInst& in = p->inst[i];
  if (p->slices == 6) {
    oz_gather_state_kernel<<<256, 256, 0, s>>>(in.xvh, in.xvl, in.kv, in.M, in.kvp, dxv);
    oz_gather_state_kernel<<<256, 256, 0, s>>>(in.xsh, in.xsl, in.ks, in.M, in.ksp, dxs);
  } else {
    oz_gather_state64_kernel<<<256, 256, 0, s>>>(in.xv64, in.kv, in.M, in.kvp, dxv);
    oz_gather_state64_kernel<<<256, 256, 0, s>>>(in.xs64, in.ks, in.M, in.ksp, dxs);
  }
  SHAW_CUDA(cudaGetLastError());
  return SHAW_OK;
}

int set_tiling(Batch* p, uint32_t width, bool paired) {
  if (width != 16 && width != 32 && width != 64) return fail(SHAW_ERR_INVALID_ARG, "tile width must be 16, 32 or 64");
  if (width > p->max_nb)
    return fail(SHAW_ERR_UNSUPPORTED, "tiles of the 9-slice (FP64-grade) form are at most 32 columns wide");
  if (paired && !pairing_fits(p, width))
    return fail(SHAW_ERR_UNSUPPORTED, "paired tiles need >= 256 modes per dof and two CTAs per tile on the SMs");
  build_tiles(p, width, paired);
  return SHAW_OK;
}

int tune(Batch* p, cudaStream_t s, double dt, unsigned long long trial_steps, std::string& report,
         unsigned long long& launches) {
  if (trial_steps == 0) trial_steps = 1;
  launches = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  SHAW_CUDA(cudaEventCreate(&e0));
  SHAW_CUDA(cudaEventCreate(&e1));
  int rc = SHAW_OK;
  auto timed = [&](float& ms) -> int {
    if (int r = reset(p, s)) return r;
    if (int r = upload(p, s)) return r;
    SHAW_CUDA(cudaEventRecord(e0, s));
    if (int r = advance(p, s, dt, 0, trial_steps)) return r;
    ++launches;
    SHAW_CUDA(cudaEventRecord(e1, s));
    if (int r = check(p, s)) return r;
    SHAW_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    return SHAW_OK;
  };
  struct Best {
    float ms = 1e30f;
    uint32_t width = 32;
    bool paired = false;
    std::vector<OzTile> tiles;
    std::vector<uint32_t> order, begin;
    uint32_t ctas = 0;
    std::string source;
  } best;
  char line[256];
  report.clear();
  do {
    float warm = 0.f;
    build_tiles(p, std::min(32u, p->max_nb));
    if ((rc = timed(warm))) break;  // first launch: module load, caches
    for (uint32_t W : {16u, 32u, 64u}) {
      if (W > p->max_nb) continue;
      build_tiles(p, W);
      float ms_model = 0.f;
      if ((rc = timed(ms_model))) break;
      std::vector<unsigned long long> ns(p->tiles.size());
      SHAW_CUDA(cudaMemcpyAsync(ns.data(), p->tile_ns, ns.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                s));
      SHAW_CUDA(cudaStreamSynchronize(s));
      std::snprintf(line, sizeof(line), "width %u: %zu tiles on %u CTAs, model schedule %.3f ms", W,
                    p->tiles.size(), p->ctas, ms_model);
      report += line;
      if (ms_model < best.ms) best = {ms_model, W, false, p->tiles, p->order, p->begin, p->ctas, "model"};
      // schedule from the measured tile times
      std::vector<double> cost(ns.begin(), ns.end());
      double mk = 0.0;
      lpt_schedule(cost, p->ctas, p->order, p->begin, mk);
      p->sched_source = "measured";
      p->tiles_dirty = true;
      float ms_meas = 0.f;
      if ((rc = timed(ms_meas))) break;
      std::snprintf(line, sizeof(line), ", measured schedule %.3f ms\n", ms_meas);
      report += line;
      if (ms_meas < best.ms) best = {ms_meas, W, false, p->tiles, p->order, p->begin, p->ctas, "measured"};
    }
    if (rc) break;
    for (uint32_t W : {16u, 32u, 64u}) {  // tiles split over CTA pairs, where they fit
      if (W > p->max_nb || !pairing_fits(p, W)) continue;
      build_tiles(p, W, true);
      float ms_pair = 0.f;
      if ((rc = timed(ms_pair))) break;
      std::snprintf(line, sizeof(line), "width %u paired: %zu tile parts on %u CTAs, %.3f ms\n", W, p->tiles.size(),
                    p->ctas, ms_pair);
      report += line;
      if (ms_pair < best.ms) best = {ms_pair, W, true, p->tiles, p->order, p->begin, p->ctas, "paired"};
    }
  } while (false);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  p->width = best.width;
  p->paired = best.paired;
  p->tiles = best.tiles;
  p->order = best.order;
  p->begin = best.begin;
  p->ctas = best.ctas;
  p->sched_source = best.source;
  p->tiles_dirty = true;
  std::snprintf(line, sizeof(line), "chosen: width %u, %s schedule, %.3f ms per %llu steps\n", best.width,
                best.source.c_str(), best.ms, trial_steps);
  report += line;
  return reset(p, s);
}

std::string describe(const Batch* p) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "tile width %u%s, %zu tiles, %u CTAs, %s schedule", p->width,
                p->paired ? " (each tile on a CTA pair)" : "", p->tiles.size(), p->ctas, p->sched_source.c_str());
  return buf;
}

uint32_t num_ctas(const Batch* p) { return p->ctas; }

int wait_selftest(unsigned long long polls, unsigned int* status) {
  unsigned int* d = nullptr;  // [0] the counter, [1] the status, [4..7] the tagged word pair
  SHAW_CUDA(cudaMalloc(&d, 8 * sizeof(unsigned int)));
  cudaError_t rc = cudaMemset(d, 0, 8 * sizeof(unsigned int));
  if (rc == cudaSuccess) {
    oz_wait_selftest_kernel<<<1, 32>>>(polls, d, reinterpret_cast<const unsigned long long*>(d + 4), d + 1);
    rc = cudaGetLastError();
  }
  if (rc == cudaSuccess) rc = cudaDeviceSynchronize();
  if (rc == cudaSuccess) rc = cudaMemcpy(status, d + 1, sizeof(unsigned int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (rc != cudaSuccess) return fail(SHAW_ERR_CUDA, std::string("bounded-wait self-test: ") + cudaGetErrorString(rc));
  return SHAW_OK;
}

void destroy(Batch* p) {
  if (!p) return;
  for (void* b : p->owned) cudaFree(b);
  for (OzInst& in : p->inst) {
    if (in.Ar) cudaFree((void*)in.Ar);
    if (in.alpha_r) cudaFree((void*)in.alpha_r);
  }
  void* bufs[] = {p->d_inst,  p->d_tiles, p->d_order,   p->d_begin,    p->bvt,
                  p->bst,     p->error,   p->tile_ns,   p->pair_sync,  p->pair_colmax};
  for (void* b : bufs)
    if (b) cudaFree(b);
  delete p;
}

}  // namespace oz
}  // namespace shaw
