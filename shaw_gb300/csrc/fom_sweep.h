// fom_sweep.h -- the single-sweep FOM leapfrog (fom_sweep.cu), shared with fom.cu.
#pragma once

#include <cuda.h>  // CUtensorMap (header only: tensor maps are encoded through the runtime's driver entry point)
#include <cuda_runtime.h>

#include <cstdint>

namespace shaw {

// Device-side control block of a FOM handle.
struct FomCtl {
  unsigned long long step_base;  // steps completed before the current graph chunk
  unsigned int nonfinite;        // set when a gathered receiver value is NaN/Inf
  unsigned int error;            // 1: a bounded wait of the sweep kernel ran out
};

namespace sweep {

// Arithmetic of one sweep: FP64 state and FP64 FMAs (kF64, the two-pass kernels'
// arithmetic in one sweep) or FP32 state and FP32 FMAs (kF32).
enum Form { kF64 = 0, kF32 = 1 };

constexpr uint32_t kTI = 16;               // vp points per strip (theta)
constexpr uint32_t kTM = 32;               // forcing columns per tile at one column per lane
constexpr uint32_t kRowsV = kTI + 1;       // v box: the strip and its east neighbour
constexpr uint32_t kRowsS = 2 * kTI + 3;   // sp box: stp(i0-1), then srp(i), stp(i) for i0..i0+kTI
constexpr uint32_t kThreads = 256;         // 8 compute warps (plus one copy warp)
constexpr uint32_t kCoefPadV = 32;         // tail padding (points) of the point-major coefficient copies
constexpr uint32_t kCoefPadS = 40;

struct Params {
  void* xv_new;             // [nvp][M] state after the step
  void* xs_new;             // [nsp][M]
  const void* xv_old;       // [nvp][M] state before the step (seismogram of the previous step)
  const void* cvp;          // [nvp + kCoefPadV][4] (N, S, W, E per vp point), dt folded, in the state's type
  const void* csp;          // [1 + nsp + kCoefPadS][2] (A, B per sp point; sp point q at index q + 1)
  const double* rho_inv;
  const unsigned long long* src;  // [M] source vp gid per column
  const int* kind;
  const double* period;
  const double* delay;
  const unsigned long long* rcv;  // [R]
  double* seis;                   // [R x T x M] LayoutLeft
  FomCtl* ctl;
  double dt;
  uint32_t nth, nr, M, sp_row;   // sp_row = 2 nth - 1
  uint32_t vec;                  // forcing columns per lane (a tile is kTM * vec columns)
  uint32_t strips, chunks, segs, tj;  // tiles: strips of kTI points x column chunks x segments of tj rows
  uint32_t n_tiles, gather_blocks;
  uint32_t R, seis_freq, seis_T;
  int rank2;
};

// Forcing columns per lane for M columns of esz-byte values (1, 2 or 4: 16 bytes at most).
uint32_t columns_per_lane(uint32_t M, uint32_t esz);

// Tensor map over one state buffer ([n][M] row-major, 2-D {M, n}, box {kTM * vec, rows}).
int encode_map(CUtensorMap* map, const void* base, uint64_t n, uint32_t M, uint32_t esz, uint32_t box_rows);

// Tiling of a grid for the sweep (columns per lane, segment length and tile counts).
void plan(Params& p, int sm_count, uint32_t esz);

// One leapfrog step: v and sigma of every point, read from the old buffers (through the
// tensor maps), written to the new ones.  k_local / host_step as in the two-pass kernels.
int launch(Form f, const CUtensorMap& tv_old, const CUtensorMap& ts_old, const Params& p, uint32_t k_local,
           unsigned long long host_step, cudaStream_t s, bool pdl);

// The seismogram of step `step` from the state buffer xv (the sweep records step n-1 during
// step n; this records the last step of a call).
int launch_gather(Form f, const Params& p, const void* xv, unsigned long long step, cudaStream_t s);

}  // namespace sweep
}  // namespace shaw
