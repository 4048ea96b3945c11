// rom_tc.cu -- mixed-precision rank-2 ROM leapfrog on the 5th-generation tensor cores
// (tcgen05 + TMEM + bulk-async copies), for sm_103a.
//
// Reference: runRomRankTwoForcing (src/kokkos/torevise/run_rom_rank_two_forcing.hpp:149-188)
//   XV += dt Av XS ;  XV[:,j] += (f_j dt) b[:,j] ;  XS += dt As XV
// Each CTA owns NB forcing columns and runs the whole time loop (persistent; the
// columns never interact, so no grid-wide synchronisation is needed).  Per half-step:
//   * the reduced operator (kv x ks, padded to multiples of 128) streams from L2 in
//     pre-tiled 128 x 32 TF32 tiles (hi and lo parts), the state block (K x NB)
//     in NB x 32 tiles, through a 4-stage cp.async.bulk / mbarrier pipeline;
//   * one thread issues tcgen05.mma kind::tf32 (M = 128, N = NB, K = 8) into FP32
//     accumulators in TMEM: D = Ahi Bhi + Ahi Blo + Alo Bhi  ("TF32x3" split);
//   * four epilogue warps read D with tcgen05.ld and update the state held as an
//     FP32 hi + lo pair (compensated, "Kahan") in global memory, add the forcing
//     and write the next GEMM's B tiles (TF32 hi / lo, rounded with cvt.rna).
// All waits are bounded: a wait that runs out sets an error flag and the kernel
// leaves its loop, releases TMEM and returns (the host reports SHAW_ERR_CUDA).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "rom_tc.h"
#include "shaw_internal.h"
#include "tc_ptx.cuh"

namespace shaw {
namespace tc {

using namespace shaw::ptx;

namespace {

constexpr int kThreads = 256;
constexpr int kStages = 4;
constexpr int kKc = 32;                        // K elements per pipeline stage
constexpr uint32_t kATileBytes = 128 * kKc * 4;  // 16 KB
// Byte offset of element (row r, k) inside a canonical K-major, no-swizzle tile of
// 32 K-elements (core matrices of 8 rows x 16 bytes; K-direction stride 128 B,
// 8-row-group stride 1024 B).
__host__ __device__ __forceinline__ uint32_t tile_off(uint32_t r, uint32_t k) {
  return (((r >> 3) * 8u + (k >> 2)) << 7) + ((r & 7u) << 4) + ((k & 3u) << 2);
}

struct TcArgs {
  const float* Av_t;  // [kvp/128][ksp/32] tiles of 128 x 32, hi then lo planes (each plane n_tiles * 16 KB)
  const float* As_t;  // [ksp/128][kvp/32]
  const float* bh;    // [Mp][kvp]
  const float* bl;
  float* xvh; float* xvl;  // [Mp][kvp]
  float* xsh; float* xsl;  // [Mp][ksp]
  float* bvt;  // per CTA: [kvp/32] tiles of NB x 32, hi plane then lo plane (B operand of the stress GEMM)
  float* bst;  // per CTA: [ksp/32] tiles (B operand of the velocity GEMM)
  const int* kind; const double* period; const double* delay;
  double* snap_vp; double* snap_sp;  // kv x T x M (device) or null
  unsigned long long Tvp, Tsp;
  uint32_t fvp, fsp;
  uint32_t kv, ks, kvp, ksp, M, Mp;
  double dt;
  unsigned long long step0, nsteps;
  unsigned int* error;
};

template <int NB>
struct Smem {
  static constexpr uint32_t kBTileBytes = NB * kKc * 4;
  static constexpr uint32_t kStageBytes = 2 * kATileBytes + 2 * kBTileBytes;
};

// One phase: D[mt] = sum_c A(mt, c) B(c) over all M-tiles of the output (rows) and
// K-chunks; A tiles from Aop (n_mt x n_kc tiles), B tiles from Bop (n_kc tiles).
template <int NB>
__device__ __forceinline__ void run_gemm_roles(int warp, int lane, uint8_t* stages, uint64_t* full,
                                               uint64_t* empty, uint64_t* accum, uint32_t tmem,
                                               const float* Aop, size_t a_plane, const float* Bop,
                                               size_t b_plane, uint32_t n_mt, uint32_t n_kc, uint32_t& it,
                                               volatile int* abort_flag, unsigned int* err) {
  constexpr uint32_t SB = Smem<NB>::kStageBytes;
  constexpr uint32_t BT = Smem<NB>::kBTileBytes;
  const uint32_t items = n_mt * n_kc;
  if (warp == 0 && lane == 0) {
    // producer: bulk copies of (A hi, A lo, B hi, B lo) for every (mt, c)
    for (uint32_t q = 0; q < items && !*abort_flag; ++q) {
      const uint32_t s = (it + q) % kStages, ph = ((it + q) / kStages) & 1u;
      if (!mbar_wait(&empty[s], ph ^ 1u)) { atomicOr(err, 1u); *abort_flag = 1; break; }
      const uint32_t mt = q / n_kc, c = q - mt * n_kc;
      uint8_t* st = stages + (size_t)s * SB;
      const float* a = Aop + ((size_t)mt * n_kc + c) * (kATileBytes / 4);
      const float* b = Bop + (size_t)c * (BT / 4);
      mbar_expect_tx(&full[s], SB);
      bulk_g2s(st, a, kATileBytes, &full[s]);
      bulk_g2s(st + kATileBytes, a + a_plane, kATileBytes, &full[s]);
      bulk_g2s(st + 2 * kATileBytes, b, BT, &full[s]);
      bulk_g2s(st + 2 * kATileBytes + BT, b + b_plane, BT, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = idesc_tf32(NB);
    for (uint32_t q = 0; q < items && !*abort_flag; ++q) {
      const uint32_t s = (it + q) % kStages, ph = ((it + q) / kStages) & 1u;
      if (!mbar_wait(&full[s], ph)) { atomicOr(err, 2u); *abort_flag = 1; break; }
      tc_fence_after();
      const uint32_t mt = q / n_kc, c = q - mt * n_kc;
      const uint32_t base = smem_u32(stages + (size_t)s * SB);
      const uint32_t d = tmem + mt * NB;
#pragma unroll
      for (uint32_t k = 0; k < kKc / 8; ++k) {
        const uint64_t ah = smem_desc(base + k * 256, 128, 1024);
        const uint64_t al = smem_desc(base + kATileBytes + k * 256, 128, 1024);
        const uint64_t bh = smem_desc(base + 2 * kATileBytes + k * 256, 128, 1024);
        const uint64_t bl = smem_desc(base + 2 * kATileBytes + BT + k * 256, 128, 1024);
        mma_tf32(d, ah, bh, idesc, (c > 0 || k > 0) ? 1u : 0u);
        mma_tf32(d, ah, bl, idesc, 1u);
        mma_tf32(d, al, bh, idesc, 1u);
      }
      mma_commit(&empty[s]);  // frees the stage once these MMAs have read it
    }
    mma_commit(accum);  // all MMAs of this phase complete -> epilogue may read D
  }
  it += items;
}

template <int NB>
__global__ void __launch_bounds__(kThreads, 1) rom_rank2_tc_kernel(TcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t SB = Smem<NB>::kStageBytes;
  constexpr uint32_t BT = Smem<NB>::kBTileBytes;
  uint8_t* stages = smem;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * SB);
  uint64_t* full = bars;
  uint64_t* empty = bars + kStages;
  uint64_t* accum = bars + 2 * kStages;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  double* fdt = reinterpret_cast<double*>(bars + 2 * kStages + 2);  // [NB]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t blk = blockIdx.x;
  const uint32_t n_mt_v = a.kvp / 128, n_mt_s = a.ksp / 128;
  const uint32_t n_kc_v = a.ksp / kKc, n_kc_s = a.kvp / kKc;  // K-chunks of the velocity / stress GEMM
  uint32_t tcols = 32;
  while (tcols < (n_mt_v > n_mt_s ? n_mt_v : n_mt_s) * NB) tcols <<= 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum, 1);
    *abort_flag = 0;
    mbar_init_fence();
  }
  if (warp == 2) tmem_alloc(tmem_slot, tcols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  // per-CTA operand planes
  const size_t av_plane = (size_t)n_mt_v * n_kc_v * (kATileBytes / 4);
  const size_t as_plane = (size_t)n_mt_s * n_kc_s * (kATileBytes / 4);
  const size_t bv_plane = (size_t)n_kc_s * (BT / 4);
  const size_t bs_plane = (size_t)n_kc_v * (BT / 4);
  float* bvt = a.bvt + (size_t)blk * 2 * bv_plane;
  float* bst = a.bst + (size_t)blk * 2 * bs_plane;
  const uint32_t col0 = blk * NB;
  uint32_t it = 0, acc_phase = 0;
  const int ew = warp - 4;  // epilogue warp index 0..3 (TMEM lane quarter)
  const float dth = (float)a.dt, dtl = (float)(a.dt - (double)dth);

  for (unsigned long long st = 0; st < a.nsteps; ++st) {
    const unsigned long long n = a.step0 + st + 1;
    // ---------------- velocity: XV += dt Av XS + fdt b ----------------
    if (ew >= 0 && ew < 4) {
      const uint32_t t = threadIdx.x - 128;
      for (uint32_t j = t; j < NB; j += 128) {
        const uint32_t col = col0 + j;
        fdt[j] = col < a.M ? signal_value(a.kind[col], a.delay[col], a.period[col], (double)(n - 1) * a.dt) * a.dt
                           : 0.0;
      }
      asm volatile("bar.sync 1, 128;" ::: "memory");
    }
    run_gemm_roles<NB>(warp, lane, stages, full, empty, accum, tmem, a.Av_t, av_plane, bst, bs_plane, n_mt_v,
                       n_kc_v, it, abort_flag, a.error);
    if (ew >= 0 && ew < 4) {
      if (!mbar_wait(accum, acc_phase)) { atomicOr(a.error, 4u); *abort_flag = 1; }
      tc_fence_after();
      if (!*abort_flag) {
        const uint32_t i_local = ew * 32 + lane;
        for (uint32_t mt = 0; mt < n_mt_v; ++mt) {
          const uint32_t row = mt * 128 + i_local;
          for (uint32_t j0 = 0; j0 < NB; j0 += 16) {
            float y[16];
            tmem_ld16(tmem + ((uint32_t)(ew * 32) << 16) + mt * NB + j0, y);
#pragma unroll
            for (int jj = 0; jj < 16; ++jj) {
              const uint32_t j = j0 + jj, col = col0 + j;
              const size_t si = (size_t)col * a.kvp + row;
              float xh = a.xvh[si], xl = a.xvl[si];
              df_fma(xh, xl, dth, dtl, y[jj], 0.f);
              const double f = fdt[j];
              const float fh = (float)f, fl = (float)(f - (double)fh);
              df_fma(xh, xl, fh, fl, a.bh[si], a.bl[si]);
              a.xvh[si] = xh;
              a.xvl[si] = xl;
              const float hi = tf32_rna(xh);
              const float lo = tf32_rna((xh - hi) + xl);
              const uint32_t c = row / kKc, kk = row % kKc;
              uint8_t* tb = reinterpret_cast<uint8_t*>(bvt) + (size_t)c * BT + tile_off(j, kk);
              *reinterpret_cast<float*>(tb) = hi;
              *reinterpret_cast<float*>(tb + bv_plane * 4) = lo;
              if (a.snap_vp && a.fvp && n % a.fvp == 0 && row < a.kv && col < a.M)
                a.snap_vp[row + (size_t)a.kv * ((n / a.fvp - 1) + a.Tvp * col)] = (double)xh + (double)xl;
            }
          }
        }
      }
      asm volatile("fence.proxy.async.global;" ::: "memory");
      tc_fence_before();
    }
    acc_phase ^= 1u;
    __syncthreads();
    tc_fence_after();
    if (*abort_flag) break;
    // ---------------- stress: XS += dt As XV ----------------
    run_gemm_roles<NB>(warp, lane, stages, full, empty, accum, tmem, a.As_t, as_plane, bvt, bv_plane, n_mt_s,
                       n_kc_s, it, abort_flag, a.error);
    if (ew >= 0 && ew < 4) {
      if (!mbar_wait(accum, acc_phase)) { atomicOr(a.error, 8u); *abort_flag = 1; }
      tc_fence_after();
      if (!*abort_flag) {
        const uint32_t i_local = ew * 32 + lane;
        for (uint32_t mt = 0; mt < n_mt_s; ++mt) {
          const uint32_t row = mt * 128 + i_local;
          for (uint32_t j0 = 0; j0 < NB; j0 += 16) {
            float y[16];
            tmem_ld16(tmem + ((uint32_t)(ew * 32) << 16) + mt * NB + j0, y);
#pragma unroll
            for (int jj = 0; jj < 16; ++jj) {
              const uint32_t j = j0 + jj, col = col0 + j;
              const size_t si = (size_t)col * a.ksp + row;
              float xh = a.xsh[si], xl = a.xsl[si];
              df_fma(xh, xl, dth, dtl, y[jj], 0.f);
              a.xsh[si] = xh;
              a.xsl[si] = xl;
              const float hi = tf32_rna(xh);
              const float lo = tf32_rna((xh - hi) + xl);
              const uint32_t c = row / kKc, kk = row % kKc;
              uint8_t* tb = reinterpret_cast<uint8_t*>(bst) + (size_t)c * BT + tile_off(j, kk);
              *reinterpret_cast<float*>(tb) = hi;
              *reinterpret_cast<float*>(tb + bs_plane * 4) = lo;
              if (a.snap_sp && a.fsp && n % a.fsp == 0 && row < a.ks && col < a.M)
                a.snap_sp[row + (size_t)a.ks * ((n / a.fsp - 1) + a.Tsp * col)] = (double)xh + (double)xl;
            }
          }
        }
      }
      asm volatile("fence.proxy.async.global;" ::: "memory");
      tc_fence_before();
    }
    acc_phase ^= 1u;
    __syncthreads();
    tc_fence_after();
    if (*abort_flag) break;
  }
  // drain: make sure no MMA is still reading smem / writing TMEM before releasing TMEM
  if (warp == 1 && lane == 0) {
    mma_commit(accum);
    mbar_wait(accum, acc_phase);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) {
    tmem_dealloc(tmem, tcols);
  }
}

// Tile an FP64 row-major operator (rows x cols) into TF32 hi/lo planes of 128 x 32 tiles.
__global__ void tile_operator_kernel(const double* A, uint32_t rows, uint32_t cols, uint32_t rows_p,
                                     uint32_t cols_p, float* out) {
  const size_t n = (size_t)rows_p * cols_p;
  const size_t plane = n;
  const uint32_t n_kc = cols_p / kKc;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(e / cols_p), c = (uint32_t)(e % cols_p);
    const double v = (r < rows && c < cols) ? A[(size_t)r * cols + c] : 0.0;
    const float hi = tf32_rna((float)v);
    const float lo = tf32_rna((float)(v - (double)hi));
    const uint32_t mt = r / 128, kc = c / kKc;
    const size_t tile = (size_t)mt * n_kc + kc;
    const size_t off = tile * (kATileBytes / 4) + tile_off(r % 128, c % kKc) / 4;
    out[off] = hi;
    out[plane + off] = lo;
  }
}

// b (kv x M, LayoutLeft FP64) -> FP32 hi/lo [Mp][kvp]
__global__ void split_b_kernel(const double* b, uint32_t kv, uint32_t M, uint32_t kvp, uint32_t Mp, float* bh,
                               float* bl) {
  const size_t n = (size_t)kvp * Mp;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const uint32_t col = (uint32_t)(e / kvp), row = (uint32_t)(e % kvp);
    const double v = (row < kv && col < M) ? b[(size_t)col * kv + row] : 0.0;
    const float h = (float)v;
    bh[e] = h;
    bl[e] = (float)(v - (double)h);
  }
}

// state (hi + lo, [Mp][kp]) -> FP64 LayoutLeft k x M
__global__ void gather_state_kernel(const float* h, const float* l, uint32_t k, uint32_t M, uint32_t kp,
                                    double* out) {
  const size_t n = (size_t)k * M;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const uint32_t col = (uint32_t)(e / k), row = (uint32_t)(e % k);
    out[e] = (double)h[(size_t)col * kp + row] + (double)l[(size_t)col * kp + row];
  }
}

uint32_t round_up(uint32_t x, uint32_t m) { return (x + m - 1) / m * m; }

}  // namespace

struct Plan {
  uint32_t kv = 0, ks = 0, kvp = 0, ksp = 0, M = 0, Mp = 0, nb = 32, ctas = 0;
  float *Av_t = nullptr, *As_t = nullptr, *bh = nullptr, *bl = nullptr;
  float *xvh = nullptr, *xvl = nullptr, *xsh = nullptr, *xsl = nullptr, *bvt = nullptr, *bst = nullptr;
  unsigned int* error = nullptr;
  size_t smem = 0;
};

int create(Plan*& p, uint32_t kv, uint32_t ks, const double* dAv, const double* dAs, uint32_t M, const double* db,
           cudaStream_t s) {
  p = new Plan();
  p->kv = kv; p->ks = ks; p->M = M;
  p->kvp = round_up(kv, 128); p->ksp = round_up(ks, 128);
  // columns per CTA: fill the 152 SMs where the column count allows it
  p->nb = (M >= 64 * 152) ? 64 : 32;
  p->Mp = round_up(M, p->nb);
  p->ctas = p->Mp / p->nb;
  const uint32_t tcols_needed = (p->kvp > p->ksp ? p->kvp : p->ksp) / 128 * p->nb;
  if (tcols_needed > 512) {
    destroy(p);
    p = nullptr;
    return fail(SHAW_ERR_UNSUPPORTED, "tensor-core ROM supports at most 1024 modes per dof");
  }
  const size_t nav = (size_t)p->kvp * p->ksp, nas = (size_t)p->ksp * p->kvp;
  const size_t bt = (size_t)p->nb * kKc;  // floats per B tile
  cudaError_t e;
  auto bail = [&](cudaError_t err, const char* w) {
    const int rc = cuda_fail(err, w);
    destroy(p);
    p = nullptr;
    return rc;
  };
#define TC_TRY(call) do { e = (call); if (e != cudaSuccess) return bail(e, #call); } while (0)
  TC_TRY(cudaMalloc(&p->Av_t, 2 * nav * sizeof(float)));
  TC_TRY(cudaMalloc(&p->As_t, 2 * nas * sizeof(float)));
  TC_TRY(cudaMalloc(&p->bh, (size_t)p->Mp * p->kvp * sizeof(float)));
  TC_TRY(cudaMalloc(&p->bl, (size_t)p->Mp * p->kvp * sizeof(float)));
  TC_TRY(cudaMalloc(&p->xvh, (size_t)p->Mp * p->kvp * sizeof(float)));
  TC_TRY(cudaMalloc(&p->xvl, (size_t)p->Mp * p->kvp * sizeof(float)));
  TC_TRY(cudaMalloc(&p->xsh, (size_t)p->Mp * p->ksp * sizeof(float)));
  TC_TRY(cudaMalloc(&p->xsl, (size_t)p->Mp * p->ksp * sizeof(float)));
  TC_TRY(cudaMalloc(&p->bvt, (size_t)p->ctas * 2 * (p->kvp / kKc) * bt * sizeof(float)));
  TC_TRY(cudaMalloc(&p->bst, (size_t)p->ctas * 2 * (p->ksp / kKc) * bt * sizeof(float)));
  TC_TRY(cudaMalloc(&p->error, sizeof(unsigned int)));
  tile_operator_kernel<<<1024, 256, 0, s>>>(dAv, kv, ks, p->kvp, p->ksp, p->Av_t);
  tile_operator_kernel<<<1024, 256, 0, s>>>(dAs, ks, kv, p->ksp, p->kvp, p->As_t);
  split_b_kernel<<<1024, 256, 0, s>>>(db, kv, M, p->kvp, p->Mp, p->bh, p->bl);
  TC_TRY(cudaGetLastError());
  const uint32_t SB = 2 * kATileBytes + 2 * p->nb * kKc * 4;
  p->smem = (size_t)kStages * SB + (2 * kStages + 2) * 8 + (size_t)p->nb * 8;
#undef TC_TRY
  return reset(p, s);
}

int reset(Plan* p, cudaStream_t s) {
  const size_t bt = (size_t)p->nb * kKc;
  SHAW_CUDA(cudaMemsetAsync(p->xvh, 0, (size_t)p->Mp * p->kvp * sizeof(float), s));
  SHAW_CUDA(cudaMemsetAsync(p->xvl, 0, (size_t)p->Mp * p->kvp * sizeof(float), s));
  SHAW_CUDA(cudaMemsetAsync(p->xsh, 0, (size_t)p->Mp * p->ksp * sizeof(float), s));
  SHAW_CUDA(cudaMemsetAsync(p->xsl, 0, (size_t)p->Mp * p->ksp * sizeof(float), s));
  SHAW_CUDA(cudaMemsetAsync(p->bvt, 0, (size_t)p->ctas * 2 * (p->kvp / kKc) * bt * sizeof(float), s));
  SHAW_CUDA(cudaMemsetAsync(p->bst, 0, (size_t)p->ctas * 2 * (p->ksp / kKc) * bt * sizeof(float), s));
  SHAW_CUDA(cudaMemsetAsync(p->error, 0, sizeof(unsigned int), s));
  return SHAW_OK;
}

int advance(Plan* p, cudaStream_t s, double dt, unsigned long long step0, unsigned long long nsteps,
            const int* kind, const double* period, const double* delay, double* snap_vp, double* snap_sp,
            unsigned long long Tvp, unsigned long long Tsp, uint32_t fvp, uint32_t fsp) {
  TcArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Av_t = p->Av_t; a.As_t = p->As_t; a.bh = p->bh; a.bl = p->bl;
  a.xvh = p->xvh; a.xvl = p->xvl; a.xsh = p->xsh; a.xsl = p->xsl; a.bvt = p->bvt; a.bst = p->bst;
  a.kind = kind; a.period = period; a.delay = delay;
  a.snap_vp = snap_vp; a.snap_sp = snap_sp; a.Tvp = Tvp; a.Tsp = Tsp; a.fvp = fvp; a.fsp = fsp;
  a.kv = p->kv; a.ks = p->ks; a.kvp = p->kvp; a.ksp = p->ksp; a.M = p->M; a.Mp = p->Mp;
  a.dt = dt; a.step0 = step0; a.nsteps = nsteps; a.error = p->error;
  if (p->nb == 64) {
    SHAW_CUDA(cudaFuncSetAttribute(rom_rank2_tc_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)p->smem));
    rom_rank2_tc_kernel<64><<<p->ctas, kThreads, p->smem, s>>>(a);
  } else {
    SHAW_CUDA(cudaFuncSetAttribute(rom_rank2_tc_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)p->smem));
    rom_rank2_tc_kernel<32><<<p->ctas, kThreads, p->smem, s>>>(a);
  }
  SHAW_CUDA(cudaGetLastError());
  return SHAW_OK;
}

int check(Plan* p, cudaStream_t s) {
  unsigned int err = 0;
  SHAW_CUDA(cudaMemcpyAsync(&err, p->error, sizeof(err), cudaMemcpyDeviceToHost, s));
  SHAW_CUDA(cudaStreamSynchronize(s));
  if (err) return fail(SHAW_ERR_CUDA, "tensor-core ROM kernel: a pipeline wait ran out (code " + std::to_string(err) + ")");
  return SHAW_OK;
}

int get_state(Plan* p, cudaStream_t s, double* dxv, double* dxs) {
  gather_state_kernel<<<256, 256, 0, s>>>(p->xvh, p->xvl, p->kv, p->M, p->kvp, dxv);
  gather_state_kernel<<<256, 256, 0, s>>>(p->xsh, p->xsl, p->ks, p->M, p->ksp, dxs);
  SHAW_CUDA(cudaGetLastError());
  return SHAW_OK;
}

void destroy(Plan* p) {
  if (!p) return;
  void* bufs[] = {p->Av_t, p->As_t, p->bh, p->bl, p->xvh, p->xvl, p->xsh, p->xsl, p->bvt, p->bst, p->error};
  for (void* b : bufs)
    if (b) cudaFree(b);
  delete p;
}

}  // namespace tc
}  // namespace shaw
