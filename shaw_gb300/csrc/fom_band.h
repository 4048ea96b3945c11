// fom_band.h -- the rank-1 FOM leapfrog of a small grid as one persistent cooperative
// launch (fom_band.cu), used by fom.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "fom_sweep.h"

namespace shaw {
namespace band {

struct Args {
  const double* cvp;  // 4 planes of nvp (N, S, W, E), dt folded
  const double* csp;  // 2 planes of nsp (A, B), dt folded
  double* xv;         // [nvp] state (read at the start, written at the end)
  double* xs;         // [nsp]
  const double* rho_inv;
  unsigned long long src;
  int kind;
  double period, delay, dt;
  const unsigned long long* rcv_sorted;  // [R][2]: (gid, receiver index) pairs in gid order
  double* seis;                          // [R x T]
  double* ftab;  // [nsteps]: the forcing increment of each step (filled by launch)
  FomCtl* ctl;
  // halo exchange words, a (tag, half of a double) pair per point, two slots per band:
  unsigned long long* xdown;  // [bands][2][2 nth - 1][2]: band b's lowest srp and stp rows, read by band b - 1
  unsigned long long* xup;    // [bands][2][nth][2]: band b's highest srp row, read by band b + 1
  unsigned long long step0, nsteps;
  uint32_t tag0;  // tag of the launch's first step (>= 1); step it carries tag0 + it
  uint32_t nth, nr, rows, R, seis_freq, seis_T;  // rows: r rows per band, or theta columns when cols
  uint32_t cols;  // 1: column bands (theta columns i0 .. i1 - 1, every r row), 0: row bands
};

// Bands for an nth x nr grid: row bands (r rows each) or column bands (theta columns
// each), whichever puts fewer points between receiving and sending; the band count, its
// width (rows or columns), the orientation and the shared memory.  False when the grid
// does not fit one co-resident band per CTA on this device.
bool plan(uint32_t nth, uint32_t nr, uint32_t* bands, uint32_t* width, uint32_t* cols, size_t* smem);

// Exchange words (unsigned long long) of each direction for `bands` bands whose rows (or
// columns) have L points: L = nth for row bands, nr for column bands.
inline size_t down_words(uint32_t bands, uint32_t L) { return (size_t)bands * 2 * (2 * (size_t)L - 1) * 2; }
inline size_t up_words(uint32_t bands, uint32_t L) { return (size_t)bands * 2 * L * 2; }

// nsteps leapfrog steps of the rank-1 FOM in one cooperative launch on stream s.
int launch(const Args& a, uint32_t bands, size_t smem, cudaStream_t s);

}  // namespace band
}  // namespace shaw
