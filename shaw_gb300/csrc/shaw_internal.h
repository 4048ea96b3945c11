// shaw_internal.h -- helpers shared by the CUDA translation units of libshaw_gpu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "shaw_gpu.h"

namespace shaw {

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// Column-major multivector products with a FOM handle's operators (fom.cu).
int fom_apply(shaw_fom_t h, int dof, const double* x, double* y, uint64_t row0, uint64_t nrows, uint32_t ncols,
              cudaStream_t s);
void fom_sizes(shaw_fom_t h, uint64_t* nvp, uint64_t* nsp);

#define SHAW_CUDA(call)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return ::shaw::cuda_fail(e_, #call); \
  } while (0)

// Unsigned 32-bit division by a run-time invariant divisor (multiply-high method,
// Granlund & Montgomery 1994): q = (umulhi(n, m) + n) >> s, valid for every n < 2^32.
struct FastDiv {
  uint32_t d, m, s;
};

inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  f.d = d;
  uint32_t s = 0;
  while ((uint64_t(1) << s) < d) ++s;
  f.s = s;
  f.m = uint32_t(((uint64_t(1) << 32) * ((uint64_t(1) << s) - d)) / d + 1);
  return f;
}

__host__ __device__ inline uint32_t fast_div(uint32_t n, const FastDiv& f) {
#ifdef __CUDA_ARCH__
  const uint32_t hi = __umulhi(n, f.m);
#else
  const uint32_t hi = uint32_t((uint64_t(n) * f.m) >> 32);
#endif
  return uint32_t((uint64_t(hi) + n) >> f.s);
}

// Source time functions, src/shared/various/signal.hpp:86-128 (same operation order).
__host__ __device__ inline double signal_value(int kind, double delay, double period, double t) {
  const double pi = 3.14159265358979323846;
  const double freq = 1.0 / period;
  const double freqSq = freq * freq;
  if (kind == SHAW_SIGNAL_RICKER) {
    const double piSq = pi * pi;
    const double tDiffSq = (t - delay) * (t - delay);
    const double expTerm = exp(-piSq * freqSq * tDiffSq);
    return (1.0 - 2.0 * piSq * tDiffSq * freqSq) * expTerm;
  } else if (kind == SHAW_SIGNAL_SINUSOID) {
    const double rn = 0.001;
    const double term2 = rn / (rn + 2.0);
    if (t < period) {
      const double term1 = sin(rn * pi * t / period);
      const double term3 = sin((rn + 2.0) * pi * t / period);
      return term1 - term2 * term3;
    }
    const double term1 = sin(rn * pi);
    const double term3 = sin((rn + 2.0) * pi);
    return term1 - term2 * term3;
  }
  const double tDiff = (t - delay);
  const double tDiffSq = tDiff * tDiff;
  const double expTerm = exp(-freqSq * tDiffSq);
  return -2.0 * tDiff * freqSq * expTerm;
}

}  // namespace shaw
