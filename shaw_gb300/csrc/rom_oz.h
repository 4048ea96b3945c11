// rom_oz.h -- host interface of the Ozaki-scheme BF16 tensor-core rank-2 ROM leapfrog (rom_oz.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace shaw {
namespace oz {

struct Plan;

// Slice the FP64 reduced operators (HOST, row-major) into row-scaled BF16 slices and
// allocate the split state; hAv kv x ks, hAs ks x kv, hb kv x M (LayoutLeft), host arrays.
int create(Plan*& p, uint32_t kv, uint32_t ks, const double* hAv, const double* hAs, uint32_t M,
           const double* hb, cudaStream_t s);
int reset(Plan* p, cudaStream_t s);
// nsteps leapfrog steps starting after step step0, one persistent launch.
int advance(Plan* p, cudaStream_t s, double dt, unsigned long long step0, unsigned long long nsteps,
            const int* kind, const double* period, const double* delay, double* snap_vp, double* snap_sp,
            unsigned long long Tvp, unsigned long long Tsp, uint32_t fvp, uint32_t fsp);
// SHAW_ERR_CUDA if a bounded pipeline wait ran out in the last launches.
int check(Plan* p, cudaStream_t s);
// FP64 copy of the states (device buffers kv x M and ks x M, LayoutLeft).
int get_state(Plan* p, cudaStream_t s, double* dxv, double* dxs);
void destroy(Plan* p);

}  // namespace oz
}  // namespace shaw
