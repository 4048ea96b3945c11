// rom_oz.h -- host interface of the Ozaki-scheme BF16 tensor-core rank-2 ROM leapfrog
// (rom_oz.cu).  One Batch advances one or many independent reduced systems (instances of
// their own kv, ks and forcing count M) in a single persistent launch.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

namespace shaw {
namespace oz {

// One reduced system: Av kv x ks and As ks x kv row-major, b kv x M LayoutLeft (host arrays).
struct InstanceDesc {
  uint32_t kv = 0, ks = 0, M = 0;
  const double *Av = nullptr, *As = nullptr, *b = nullptr;
};

struct Batch;

// Slice every instance's operators into row-scaled BF16 slices, allocate the states, and
// pick the default tiling.  slices = 6: 36-bit products, FP32 hi + lo states
// (SHAW_MIXED_OZAKI_BF16); slices = 9: 54-bit products and FP64 states, FP64-grade
// results (SHAW_OZAKI_FP64), tiles of at most 32 columns.
int create(Batch*& p, uint32_t n, const InstanceDesc* d, cudaStream_t s, int slices = 6);
// Per-column signals of instance i (device arrays of M entries, owned by the caller).
int set_signals(Batch* p, uint32_t i, const int* kind, const double* period, const double* delay);
// Device snapshot buffers of instance i (k x T x M LayoutLeft), or nullptr / frequency 0.
int set_snapshots(Batch* p, uint32_t i, double* snap_vp, double* snap_sp, unsigned long long Tvp,
                  unsigned long long Tsp, uint32_t fvp, uint32_t fsp);
// Receivers of instance i: rows = PhiVp[gid_r, :] (host, R x kv row-major); on every step n
// with n % freq == 0 the kernel writes S(r, n/freq - 1, j) = rows[r, :] . XV[:, j] into the
// device seismogram d_seis (R x T x M LayoutLeft).  R = 0 removes them.
int set_receivers(Batch* p, uint32_t i, const double* rows, uint32_t R, double* d_seis, unsigned long long T,
                  uint32_t freq, cudaStream_t s);
int reset(Batch* p, cudaStream_t s);
// nsteps leapfrog steps of every instance, starting after step step0: one persistent launch.
int advance(Batch* p, cudaStream_t s, double dt, unsigned long long step0, unsigned long long nsteps);
// SHAW_ERR_CUDA if a bounded pipeline wait ran out in the last launches.
int check(Batch* p, cudaStream_t s);
// FP64 copy of instance i's states (device buffers kv x M and ks x M, LayoutLeft).
int get_state(Batch* p, uint32_t i, cudaStream_t s, double* dxv, double* dxs);
// Autotuner: times every tile width in {16, 32, 64} with a model-cost LPT schedule and a
// schedule rebuilt from the measured per-tile times, and every width whose tiles fit
// the SMs twice over split across CTA pairs; keeps the fastest and leaves all states
// reset to zero.  `report` receives one line per candidate, `launches` the number of
// kernel launches made.
int tune(Batch* p, cudaStream_t s, double dt, unsigned long long trial_steps, std::string& report,
         unsigned long long& launches);
// Fixed tiling: tiles of `width` forcing columns (16, 32 or 64), optionally each split
// across two co-resident CTAs (SHAW_ERR_UNSUPPORTED where the pairs do not fit).
int set_tiling(Batch* p, uint32_t width, bool paired);
// The current tiling in words (width, tiles, CTAs, schedule source).
std::string describe(const Batch* p);
uint32_t num_ctas(const Batch* p);
void destroy(Batch* p);
// One small launch whose bounded waits (an mbarrier phase and a global counter that nothing
// completes) run out after `polls` polls; *status gets their error bits (64, 128).
int wait_selftest(unsigned long long polls, unsigned int* status);

}  // namespace oz
}  // namespace shaw
