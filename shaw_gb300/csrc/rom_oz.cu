// rom_oz.cu -- rank-2 ROM leapfrog with FP64-grade reduced GEMMs on the BF16 tensor
// cores (tcgen05, kind::f16), using the Ozaki splitting scheme with exact accumulation.
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
//   * pairs with s + t <= 5 (21 MMAs per K-step) give ~2^-36 relative accuracy; the 6
//     diagonal sums are combined in the epilogue in FP32 double-float and scaled back.
// State: FP32 hi + lo pairs (compensated) in global memory; the epilogue re-slices
// the new state into the next GEMM's BF16 B tiles after each half-step.
// Each CTA owns NB forcing columns and runs the whole time loop (persistent).
// All waits are bounded: a wait that runs out sets an error flag, the kernel leaves
// its loop, releases TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "rom_oz.h"
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
constexpr int kSlices = 6;
constexpr int kDiags = 6;                     // d = s + t in [0, 5]
constexpr int kKc = 32;                       // BF16 K-elements per pipeline stage (64 bytes per row)
constexpr uint32_t kRowBytes = kKc * 2;
constexpr uint32_t kATile = 128 * kRowBytes;  // one slice of a 128 x 32 operator tile: 8 KB
constexpr int kStages = 3;

template <int NB>
struct Cfg {
  static constexpr uint32_t kBTile = NB * kRowBytes;
  static constexpr uint32_t kABytes = kSlices * kATile;
  static constexpr uint32_t kBBytes = kSlices * kBTile;
  static constexpr uint32_t kStage = kABytes + kBBytes;
  static constexpr uint32_t kTmemCols = (kDiags * NB <= 256) ? 256 : 512;
};

// Byte offset of (row r, k) in a K-major, no-swizzle BF16 tile of 32 K-elements:
// core matrices of 8 rows x 16 bytes, K-direction stride 128 B, 8-row-group stride 512 B.
__host__ __device__ __forceinline__ uint32_t tile_off(uint32_t r, uint32_t k) {
  return (((r >> 3) * 4u + (k >> 3)) << 7) + ((r & 7u) << 4) + ((k & 7u) << 1);
}

struct OzArgs {
  const uint8_t* Av;  // [kvp/128][ksp/32][slice][8 KB]
  const uint8_t* As;  // [ksp/128][kvp/32][slice][8 KB]
  const int* alpha_v;
  const int* alpha_s;
  const float* bh;
  const float* bl;  // [Mp][kvp]
  float *xvh, *xvl, *xsh, *xsl;
  uint8_t* bvt;  // per CTA [kvp/32][slice][NB x 64 B]: slices of XV (B of the stress GEMM)
  uint8_t* bst;  // per CTA [ksp/32][slice][NB x 64 B]: slices of XS (B of the velocity GEMM)
  const int* kind;
  const double* period;
  const double* delay;
  double *snap_vp, *snap_sp;
  unsigned long long Tvp, Tsp;
  uint32_t fvp, fsp;
  uint32_t kv, ks, kvp, ksp, M;
  double dt;
  unsigned long long step0, nsteps;
  unsigned int* error;
};

struct Shared {
  uint64_t full[kStages], empty[kStages], acc_full, acc_empty;
  uint32_t tmem;
  int abort;
  int beta_v[64], beta_s[64];
  unsigned int colmax[64];
  double fdt[64];
};

__device__ __forceinline__ void raise(Shared* sh, unsigned int* err, unsigned int code) {
  atomicOr(err, code);
  sh->abort = 1;
}

// One GEMM phase: for every 128-row M-tile, D_d = sum over K of the slice pairs on
// diagonal d, then the epilogue `epi(mt)` runs on warps 4..7.
template <int NB, typename Epi>
__device__ __forceinline__ void gemm_phase(uint8_t* stages, Shared* sh, const uint8_t* Aop, const uint8_t* Bop,
                                           uint32_t n_mt, uint32_t n_kc, uint32_t& it, uint32_t& mtc,
                                           unsigned int* err, Epi epi) {
  using C = Cfg<NB>;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0 && lane == 0) {
    for (uint32_t q = 0; q < n_mt * n_kc && !sh->abort; ++q) {
      const uint32_t s = (it + q) % kStages, ph = ((it + q) / kStages) & 1u;
      if (!mbar_wait(&sh->empty[s], ph ^ 1u)) { raise(sh, err, 1u); break; }
      const uint32_t mt = q / n_kc, c = q - mt * n_kc;
      uint8_t* st = stages + (size_t)s * C::kStage;
      mbar_expect_tx(&sh->full[s], C::kStage);
      bulk_g2s(st, Aop + ((size_t)mt * n_kc + c) * C::kABytes, C::kABytes, &sh->full[s]);
      bulk_g2s(st + C::kABytes, Bop + (size_t)c * C::kBBytes, C::kBBytes, &sh->full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = idesc_bf16(NB);
    for (uint32_t mt = 0; mt < n_mt && !sh->abort; ++mt) {
      if (!mbar_wait(&sh->acc_empty, ((mtc + mt) & 1u) ^ 1u)) { raise(sh, err, 2u); break; }
      tc_fence_after();
      for (uint32_t c = 0; c < n_kc && !sh->abort; ++c) {
        const uint32_t q = mt * n_kc + c;
        const uint32_t s = (it + q) % kStages, ph = ((it + q) / kStages) & 1u;
        if (!mbar_wait(&sh->full[s], ph)) { raise(sh, err, 4u); break; }
        tc_fence_after();
        const uint32_t abase = smem_u32(stages + (size_t)s * C::kStage);
        // descriptors of the stage's first A / B slice; the others differ only in the
        // start-address field (16-byte units, no carry: shared addresses < 256 KB)
        const uint64_t adesc0 = smem_desc(abase, 128, 512);
        const uint64_t bdesc0 = smem_desc(abase + C::kABytes, 128, 512);
#pragma unroll
        for (uint32_t k = 0; k < kKc / 16; ++k) {
#pragma unroll
          for (int d = 0; d < kDiags; ++d) {
#pragma unroll
            for (int sa = 0; sa <= d; ++sa) {
              const int tb = d - sa;
              const uint64_t adesc = adesc0 + ((sa * kATile + k * 256) >> 4);
              const uint64_t bdesc = bdesc0 + ((tb * C::kBTile + k * 256) >> 4);
              mma_f16(sh->tmem + d * NB, adesc, bdesc, idesc, (c > 0 || k > 0 || sa > 0) ? 1u : 0u);
            }
          }
        }
        mma_commit(&sh->empty[s]);
      }
      mma_commit(&sh->acc_full);
    }
  } else if (warp >= 4) {
    for (uint32_t mt = 0; mt < n_mt; ++mt) {
      if (!mbar_wait(&sh->acc_full, (mtc + mt) & 1u)) { raise(sh, err, 8u); break; }
      tc_fence_after();
      if (!sh->abort) epi(mt);
      tc_fence_before();
      mbar_arrive(&sh->acc_empty);
    }
  }
  it += n_mt * n_kc;
  mtc += n_mt;
}

// 2^e as an FP32 factor pair (e may leave the normal range of one factor).
__device__ __forceinline__ void pow2_pair(int e, float& f1, float& f2) {
  const int e1 = e / 2, e2 = e - e1;
  f1 = __int_as_float((e1 + 127) << 23);
  f2 = __int_as_float((e2 + 127) << 23);
}

// Read the 6 diagonal accumulators of 8 columns for this thread's row (TMEM lanes of
// quarter q) and combine them exactly: every D_d is an integer below 2^24, so
// Y = sum_d D_d * 2^(6(5-d)) is an exact int64 and y = Y * 2^-42 (before scaling).
// Returns y as a double-float pair.
template <int NB>
__device__ __forceinline__ void load_combine8(uint32_t tmem, int q, uint32_t j0, float* yh, float* yl) {
  float D[kDiags][8];
#pragma unroll
  for (int d = 0; d < kDiags; ++d) tmem_ld8(tmem + ((uint32_t)(q * 32) << 16) + d * NB + j0, D[d]);
  tmem_wait_ld();
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) {
    long long Y = 0;
#pragma unroll
    for (int d = 0; d < kDiags; ++d) Y += (long long)__float2int_rn(D[d][jj]) << (6 * (kDiags - 1 - d));
    const float h = __ll2float_rn(Y);
    const float l = __ll2float_rn(Y - __float2ll_rn(h));
    yh[jj] = h * 0x1p-42f;  // exact power-of-two scalings
    yl[jj] = l * 0x1p-42f;
  }
}

// Slice a state block (rows x NB, column-major, double-float) into the BF16 B tiles
// with per-column exponents beta[j] (|x| < 2^beta).
template <int NB>
__device__ __forceinline__ void slice_state(const float* xh, const float* xl, uint32_t kp, uint32_t col0,
                                            const int* beta, uint8_t* tiles) {
  using C = Cfg<NB>;
  const uint32_t t = threadIdx.x - 128;
  for (uint32_t e = t; e < kp * NB; e += kEpiThreads) {
    const uint32_t j = e / kp, row = e - j * kp;
    const size_t si = (size_t)(col0 + j) * kp + row;
    float vh = ldexpf(xh[si], -beta[j]), vl = ldexpf(xl[si], -beta[j]);
    uint8_t* base = tiles + (size_t)(row / kKc) * C::kBBytes + tile_off(j, row % kKc);
#pragma unroll
    for (int s = 0; s < kSlices; ++s) {
      const float th = vh * 64.f, tl = vl * 64.f;
      float a = rintf(th);
      a = fminf(64.f, fmaxf(-64.f, a));
      two_sum(th - a, tl, vh, vl);
      *reinterpret_cast<__nv_bfloat16*>(base + s * C::kBTile) = __float2bfloat16_rn(a);
    }
  }
}

// Column exponents from the maxima gathered in colmax: |x| < 2^beta.
template <int NB>
__device__ __forceinline__ void column_exponents(Shared* sh, int* beta) {
  const uint32_t t = threadIdx.x - 128;
  if (t < NB) {
    const float m = __uint_as_float(sh->colmax[t]);
    beta[t] = (m > 0.f) ? ilogbf(m) + 1 : 0;
    sh->colmax[t] = 0u;
  }
}

__device__ __forceinline__ void note_max(Shared* sh, uint32_t j, float v) {
  const unsigned int m = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(v)));
  if ((threadIdx.x & 31) == 0) atomicMax(&sh->colmax[j], m);
}

template <int NB>
__global__ void __launch_bounds__(kThreads, 1) rom_rank2_ozaki_kernel(OzArgs a) {
  using C = Cfg<NB>;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* stages = smem;
  Shared* sh = reinterpret_cast<Shared*>(smem + kStages * C::kStage);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ew = warp - 4;                     // >= 0 on the epilogue warps
  const int q = warp & 3;                      // TMEM lane quarter of this warp
  const uint32_t jbeg = (uint32_t)((ew >> 2) * (NB / 2)), jend = jbeg + NB / 2;  // this group's columns
  const uint32_t n_mt_v = a.kvp / 128, n_mt_s = a.ksp / 128, n_kc_v = a.ksp / kKc, n_kc_s = a.kvp / kKc;
  const uint32_t col0 = blockIdx.x * NB;
  uint8_t* bvt = a.bvt + (size_t)blockIdx.x * n_kc_s * C::kBBytes;
  uint8_t* bst = a.bst + (size_t)blockIdx.x * n_kc_v * C::kBBytes;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&sh->full[s], 1);
      mbar_init(&sh->empty[s], 1);
    }
    mbar_init(&sh->acc_full, 1);
    mbar_init(&sh->acc_empty, kEpiThreads);
    sh->abort = 0;
    mbar_init_fence();
  }
  if (threadIdx.x < 64) {
    sh->colmax[threadIdx.x] = 0u;
    sh->beta_v[threadIdx.x] = 0;
    sh->beta_s[threadIdx.x] = 0;
  }
  if (warp == 2) tmem_alloc(&sh->tmem, C::kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  // B tiles of the current XS (the state may be non-zero when advancing in pieces)
  if (ew >= 0) {
    for (uint32_t e = threadIdx.x - 128; e < a.ksp * NB; e += kEpiThreads) {
      const uint32_t j = e / a.ksp, row = e - j * a.ksp;
      const float v = a.xsh[(size_t)(col0 + j) * a.ksp + row];
      atomicMax(&sh->colmax[j], __float_as_uint(fabsf(v)));
    }
    asm volatile("bar.sync 1, 256;" ::: "memory");
    column_exponents<NB>(sh, sh->beta_s);
    asm volatile("bar.sync 1, 256;" ::: "memory");
    slice_state<NB>(a.xsh, a.xsl, a.ksp, col0, sh->beta_s, bst);
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  __syncthreads();

  const float dth = (float)a.dt, dtl = (float)(a.dt - (double)dth);
  uint32_t it = 0, mtc = 0;
  for (unsigned long long st = 0; st < a.nsteps && !sh->abort; ++st) {
    const unsigned long long n = a.step0 + st + 1;
    if (ew >= 0) {
      const uint32_t t = threadIdx.x - 128;
      if (t < NB) {
        const uint32_t col = col0 + t;
        sh->fdt[t] = col < a.M
                         ? signal_value(a.kind[col], a.delay[col], a.period[col], (double)(n - 1) * a.dt) * a.dt
                         : 0.0;
      }
      asm volatile("bar.sync 1, 256;" ::: "memory");
    }
    // ---------------- velocity: XV += dt Av XS + fdt b ----------------
    gemm_phase<NB>(stages, sh, a.Av, bst, n_mt_v, n_kc_v, it, mtc, a.error, [&](uint32_t mt) {
      const uint32_t row = mt * 128 + q * 32 + lane;
      const int alpha = a.alpha_v[row];
      for (uint32_t j0 = jbeg; j0 < jend; j0 += 8) {
        float yh[8], yl[8];
        load_combine8<NB>(sh->tmem, q, j0, yh, yl);
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
          const uint32_t j = j0 + jj, col = col0 + j;
          const int e = alpha + sh->beta_s[j];
          const size_t si = (size_t)col * a.kvp + row;
          float xh = a.xvh[si], xl = a.xvl[si];
          float s1, s2;
          pow2_pair(e, s1, s2);
          df_fma(xh, xl, dth, dtl, yh[jj] * s1 * s2, yl[jj] * s1 * s2);
          const double f = sh->fdt[j];
          const float fh = (float)f, fl = (float)(f - (double)fh);
          df_fma(xh, xl, fh, fl, a.bh[si], a.bl[si]);
          a.xvh[si] = xh;
          a.xvl[si] = xl;
          note_max(sh, j, xh);
          if (a.snap_vp && a.fvp && n % a.fvp == 0 && row < a.kv && col < a.M)
            a.snap_vp[row + (size_t)a.kv * ((n / a.fvp - 1) + a.Tvp * col)] = (double)xh + (double)xl;
        }
      }
    });
    if (ew >= 0) {
      asm volatile("bar.sync 1, 256;" ::: "memory");
      column_exponents<NB>(sh, sh->beta_v);
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (!sh->abort) slice_state<NB>(a.xvh, a.xvl, a.kvp, col0, sh->beta_v, bvt);
      asm volatile("fence.proxy.async.global;" ::: "memory");
    }
    __syncthreads();
    if (sh->abort) break;
    // ---------------- stress: XS += dt As XV ----------------
    gemm_phase<NB>(stages, sh, a.As, bvt, n_mt_s, n_kc_s, it, mtc, a.error, [&](uint32_t mt) {
      const uint32_t row = mt * 128 + q * 32 + lane;
      const int alpha = a.alpha_s[row];
      for (uint32_t j0 = jbeg; j0 < jend; j0 += 8) {
        float yh[8], yl[8];
        load_combine8<NB>(sh->tmem, q, j0, yh, yl);
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
          const uint32_t j = j0 + jj, col = col0 + j;
          const int e = alpha + sh->beta_v[j];
          const size_t si = (size_t)col * a.ksp + row;
          float xh = a.xsh[si], xl = a.xsl[si];
          float s1, s2;
          pow2_pair(e, s1, s2);
          df_fma(xh, xl, dth, dtl, yh[jj] * s1 * s2, yl[jj] * s1 * s2);
          a.xsh[si] = xh;
          a.xsl[si] = xl;
          note_max(sh, j, xh);
          if (a.snap_sp && a.fsp && n % a.fsp == 0 && row < a.ks && col < a.M)
            a.snap_sp[row + (size_t)a.ks * ((n / a.fsp - 1) + a.Tsp * col)] = (double)xh + (double)xl;
        }
      }
    });
    if (ew >= 0) {
      asm volatile("bar.sync 1, 256;" ::: "memory");
      column_exponents<NB>(sh, sh->beta_s);
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (!sh->abort) slice_state<NB>(a.xsh, a.xsl, a.ksp, col0, sh->beta_s, bst);
      asm volatile("fence.proxy.async.global;" ::: "memory");
    }
    __syncthreads();
  }
  // drain: no MMA may still be in flight when TMEM is released
  if (warp == 1 && lane == 0) {
    mma_commit(&sh->acc_full);
    mbar_wait(&sh->acc_full, mtc & 1u);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) tmem_dealloc(sh->tmem, C::kTmemCols);
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

uint32_t round_up(uint32_t x, uint32_t m) { return (x + m - 1) / m * m; }

uint16_t bf16_bits_of_int(double a) {
  const float f = (float)a;  // |a| <= 64: exact in BF16
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (uint16_t)(u >> 16);
}

// Row-scaled 6-bit slices of a row-major FP64 operator (rows x cols), padded, tiled
// as [rows_p/128][cols_p/32][slice][128 x 32 BF16 tile]; alpha[r] = row exponent.
void slice_operator(const double* A, uint32_t rows, uint32_t cols, uint32_t rows_p, uint32_t cols_p,
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

}  // namespace

struct Plan {
  uint32_t kv = 0, ks = 0, kvp = 0, ksp = 0, M = 0, Mp = 0, nb = 32, ctas = 0;
  uint8_t *Av = nullptr, *As = nullptr, *bvt = nullptr, *bst = nullptr;
  int *alpha_v = nullptr, *alpha_s = nullptr;
  float *bh = nullptr, *bl = nullptr, *xvh = nullptr, *xvl = nullptr, *xsh = nullptr, *xsl = nullptr;
  unsigned int* error = nullptr;
  size_t smem = 0;
};

int create(Plan*& p, uint32_t kv, uint32_t ks, const double* hAv, const double* hAs, uint32_t M, const double* hb,
           cudaStream_t s) {
  if (kv > 1024 || ks > 1024)
    return fail(SHAW_ERR_UNSUPPORTED, "the Ozaki tensor-core ROM supports at most 1024 modes per dof");
  p = new Plan();
  p->kv = kv; p->ks = ks; p->M = M;
  p->kvp = round_up(kv, 128); p->ksp = round_up(ks, 128);
  p->nb = (M >= 64 * 152) ? 64 : 32;
  p->Mp = round_up(M, p->nb);
  p->ctas = p->Mp / p->nb;
  std::vector<uint16_t> sv, ss;
  std::vector<int> av, as;
  slice_operator(hAv, kv, ks, p->kvp, p->ksp, sv, av);
  slice_operator(hAs, ks, kv, p->ksp, p->kvp, ss, as);
  std::vector<float> bh((size_t)p->Mp * p->kvp, 0.f), bl((size_t)p->Mp * p->kvp, 0.f);
  for (uint32_t c = 0; c < M; ++c)
    for (uint32_t r = 0; r < kv; ++r) {
      const double v = hb[(size_t)c * kv + r];
      const float h = (float)v;
      bh[(size_t)c * p->kvp + r] = h;
      bl[(size_t)c * p->kvp + r] = (float)(v - (double)h);
    }
  const size_t btile_bytes = (size_t)kSlices * p->nb * kRowBytes;  // per K-chunk
  cudaError_t e;
  auto bail = [&](cudaError_t err, const char* w) {
    const int rc = cuda_fail(err, w);
    destroy(p);
    p = nullptr;
    return rc;
  };
#define OZ_TRY(call) do { e = (call); if (e != cudaSuccess) return bail(e, #call); } while (0)
  OZ_TRY(cudaMalloc(&p->Av, sv.size() * 2));
  OZ_TRY(cudaMalloc(&p->As, ss.size() * 2));
  OZ_TRY(cudaMalloc(&p->alpha_v, p->kvp * sizeof(int)));
  OZ_TRY(cudaMalloc(&p->alpha_s, p->ksp * sizeof(int)));
  OZ_TRY(cudaMalloc(&p->bh, bh.size() * sizeof(float)));
  OZ_TRY(cudaMalloc(&p->bl, bl.size() * sizeof(float)));
  OZ_TRY(cudaMalloc(&p->xvh, (size_t)p->Mp * p->kvp * sizeof(float)));
  OZ_TRY(cudaMalloc(&p->xvl, (size_t)p->Mp * p->kvp * sizeof(float)));
  OZ_TRY(cudaMalloc(&p->xsh, (size_t)p->Mp * p->ksp * sizeof(float)));
  OZ_TRY(cudaMalloc(&p->xsl, (size_t)p->Mp * p->ksp * sizeof(float)));
  OZ_TRY(cudaMalloc(&p->bvt, (size_t)p->ctas * (p->kvp / kKc) * btile_bytes));
  OZ_TRY(cudaMalloc(&p->bst, (size_t)p->ctas * (p->ksp / kKc) * btile_bytes));
  OZ_TRY(cudaMalloc(&p->error, sizeof(unsigned int)));
  OZ_TRY(cudaMemcpyAsync(p->Av, sv.data(), sv.size() * 2, cudaMemcpyHostToDevice, s));
  OZ_TRY(cudaMemcpyAsync(p->As, ss.data(), ss.size() * 2, cudaMemcpyHostToDevice, s));
  OZ_TRY(cudaMemcpyAsync(p->alpha_v, av.data(), av.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  OZ_TRY(cudaMemcpyAsync(p->alpha_s, as.data(), as.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  OZ_TRY(cudaMemcpyAsync(p->bh, bh.data(), bh.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  OZ_TRY(cudaMemcpyAsync(p->bl, bl.data(), bl.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  OZ_TRY(cudaStreamSynchronize(s));  // the host vectors go out of scope
#undef OZ_TRY
  const uint32_t stage = p->nb == 64 ? Cfg<64>::kStage : Cfg<32>::kStage;
  p->smem = (size_t)kStages * stage + sizeof(Shared);
  return reset(p, s);
}

int reset(Plan* p, cudaStream_t s) {
  const size_t btile_bytes = (size_t)kSlices * p->nb * kRowBytes;
  SHAW_CUDA(cudaMemsetAsync(p->xvh, 0, (size_t)p->Mp * p->kvp * sizeof(float), s));
  SHAW_CUDA(cudaMemsetAsync(p->xvl, 0, (size_t)p->Mp * p->kvp * sizeof(float), s));
  SHAW_CUDA(cudaMemsetAsync(p->xsh, 0, (size_t)p->Mp * p->ksp * sizeof(float), s));
  SHAW_CUDA(cudaMemsetAsync(p->xsl, 0, (size_t)p->Mp * p->ksp * sizeof(float), s));
  SHAW_CUDA(cudaMemsetAsync(p->bvt, 0, (size_t)p->ctas * (p->kvp / kKc) * btile_bytes, s));
  SHAW_CUDA(cudaMemsetAsync(p->bst, 0, (size_t)p->ctas * (p->ksp / kKc) * btile_bytes, s));
  SHAW_CUDA(cudaMemsetAsync(p->error, 0, sizeof(unsigned int), s));
  return SHAW_OK;
}

int advance(Plan* p, cudaStream_t s, double dt, unsigned long long step0, unsigned long long nsteps,
            const int* kind, const double* period, const double* delay, double* snap_vp, double* snap_sp,
            unsigned long long Tvp, unsigned long long Tsp, uint32_t fvp, uint32_t fsp) {
  OzArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Av = p->Av; a.As = p->As; a.alpha_v = p->alpha_v; a.alpha_s = p->alpha_s; a.bh = p->bh; a.bl = p->bl;
  a.xvh = p->xvh; a.xvl = p->xvl; a.xsh = p->xsh; a.xsl = p->xsl; a.bvt = p->bvt; a.bst = p->bst;
  a.kind = kind; a.period = period; a.delay = delay;
  a.snap_vp = snap_vp; a.snap_sp = snap_sp; a.Tvp = Tvp; a.Tsp = Tsp; a.fvp = fvp; a.fsp = fsp;
  a.kv = p->kv; a.ks = p->ks; a.kvp = p->kvp; a.ksp = p->ksp; a.M = p->M;
  a.dt = dt; a.step0 = step0; a.nsteps = nsteps; a.error = p->error;
  if (p->nb == 64) {
    SHAW_CUDA(cudaFuncSetAttribute(rom_rank2_ozaki_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)p->smem));
    rom_rank2_ozaki_kernel<64><<<p->ctas, kThreads, p->smem, s>>>(a);
  } else {
    SHAW_CUDA(cudaFuncSetAttribute(rom_rank2_ozaki_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)p->smem));
    rom_rank2_ozaki_kernel<32><<<p->ctas, kThreads, p->smem, s>>>(a);
  }
  SHAW_CUDA(cudaGetLastError());
  return SHAW_OK;
}

int check(Plan* p, cudaStream_t s) {
  unsigned int err = 0;
  SHAW_CUDA(cudaMemcpyAsync(&err, p->error, sizeof(err), cudaMemcpyDeviceToHost, s));
  SHAW_CUDA(cudaStreamSynchronize(s));
  if (err)
    return fail(SHAW_ERR_CUDA, "Ozaki tensor-core ROM kernel: a pipeline wait ran out (code " +
                                   std::to_string(err) + ")");
  return SHAW_OK;
}

int get_state(Plan* p, cudaStream_t s, double* dxv, double* dxs) {
  oz_gather_state_kernel<<<256, 256, 0, s>>>(p->xvh, p->xvl, p->kv, p->M, p->kvp, dxv);
  oz_gather_state_kernel<<<256, 256, 0, s>>>(p->xsh, p->xsl, p->ks, p->M, p->ksp, dxs);
  SHAW_CUDA(cudaGetLastError());
  return SHAW_OK;
}

void destroy(Plan* p) {
  if (!p) return;
  void* bufs[] = {p->Av, p->As, p->bvt, p->bst, p->alpha_v, p->alpha_s, p->bh, p->bl,
                  p->xvh, p->xvl, p->xsh, p->xsl, p->error};
  for (void* b : bufs)
    if (b) cudaFree(b);
  delete p;
}

}  // namespace oz
}  // namespace shaw
