// l2_exchange.cuh -- values passed between the CTAs of one cooperative launch through L2
// as self-validating tagged words, used by the persistent band kernels (fom_band.cu, rom.cu).
//
// A double travels as one 16-byte pair of 8-byte words, (tag | high half) and (tag | low
// half): a reader polls the data itself, so no flag, fence or second round trip follows
// it.  Each 8-byte word is written and read by a single-copy-atomic access (the 16-byte
// vector access is two of them), so a word is never seen half old and half new, and each
// word is validated alone.  Tags are step numbers that grow monotonically over the life of
// a buffer (its owner clears the buffer before a 32-bit tag would wrap), so a word left by
// an earlier step or launch never matches.
#pragma once

#include <cstdint>

namespace shaw {
namespace l2x {

// Polling rounds before a wait gives up: about a second of L2 round trips.
constexpr uint32_t kPollLimit = 1u << 22;

__device__ __forceinline__ void put(unsigned long long* w, uint32_t tag, double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const unsigned long long t = (unsigned long long)tag << 32;
  asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(w), "l"(t | (u >> 32)),
               "l"(t | (u & 0xffffffffull))
               : "memory");
}

// Bounded wait for the points src[k] (k with bit k of `pending` set) tagged `tag`, each
// stored to *dst[k] as it arrives.  Every round issues the loads of all pending points
// before it checks any, so their round trips overlap.  False when `limit` rounds ran out.
template <int N>
__device__ __forceinline__ bool poll(const unsigned long long* const (&src)[N], double* const (&dst)[N],
                                     uint32_t pending, uint32_t tag, uint32_t limit = kPollLimit) {
  for (uint32_t round = 0; pending && round < limit; ++round) {
    unsigned long long hi[N], lo[N];
#pragma unroll
    for (int k = 0; k < N; ++k)
      if (pending & (1u << k))
        asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(hi[k]), "=l"(lo[k]) : "l"(src[k]) : "memory");
#pragma unroll
    for (int k = 0; k < N; ++k)
      if ((pending & (1u << k)) && (uint32_t)(hi[k] >> 32) == tag && (uint32_t)(lo[k] >> 32) == tag) {
        *dst[k] = __longlong_as_double((long long)((hi[k] << 32) | (lo[k] & 0xffffffffull)));
        pending &= ~(1u << k);
      }
  }
  return pending == 0;
}

}  // namespace l2x
}  // namespace shaw
