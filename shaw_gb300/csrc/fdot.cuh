// fdot.cuh -- an FP64 stencil update v + sum_k c_k x_k on the integer pipes, rounded once.
//
// GB300's FP64 pipe issues about 2 FMA lanes per clock per SM; its integer pipes are far
// wider.  A "fused dot" here forms each product's top 64 bits from the two 53-bit
// significands (one 64 x 64 high multiply), aligns every term to the largest one (the base
// value included) with 4 bits of headroom, adds them exactly in a signed 64-bit integer,
// and rounds the sum to FP64 once (ties to even).  Each term keeps 60 significant bits
// before the sum, so the result is within 0.5 ulp + 2^-56 of the exact v + sum c_k x_k --
// closer than a chain of FMAs, which rounds after each term -- and, unlike a fixed-point
// scale shared by the whole state, every point keeps FP64's relative precision however
// small its values are.  It does not reproduce the FMA chain bit for bit.
//
// Range: normal and zero inputs; subnormal inputs count as zero.  A non-finite input or a
// result outside the normal range sets *bad, and the caller recomputes the point with FMAs.
// Both host and device compile this header (the host form is what the CPU tests check
// against exact rational arithmetic).
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define SHAW_FD_HD __host__ __device__ __forceinline__
#else
#define SHAW_FD_HD inline
#endif

namespace shaw {
namespace fd {

SHAW_FD_HD uint64_t mulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

SHAW_FD_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

SHAW_FD_HD uint64_t bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}

SHAW_FD_HD double from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}

// One term of the sum: t * 2^x with t < 2^64 (t = 0 for a zero term), negative when neg;
// special when an operand is infinite or NaN.
struct Term {
  uint64_t t;
  int x;
  uint32_t neg, special;
};

// c * x: the significands left-aligned (bit 63 set) and multiplied, top 64 bits kept.
// Value = mulhi(A, B) * 2^(ec + ex - 2108) for A = m_c 2^11, B = m_x 2^11 (m = the 53-bit
// significand, value m 2^(e - 1075)).  Exponent field 0 (zero, subnormal) gives a zero term.
SHAW_FD_HD Term product(double c, double x) {
  const uint64_t bc = bits(c), bx = bits(x);
  const int ec = (int)((bc >> 52) & 0x7FF), ex = (int)((bx >> 52) & 0x7FF);
  const uint64_t a = (bc << 11) | (1ull << 63), b = (bx << 11) | (1ull << 63);
  Term r;
  r.t = (ec != 0 && ex != 0) ? mulhi(a, b) : 0ull;
  r.x = ec + ex - 2108;
  r.neg = (uint32_t)((bc ^ bx) >> 63);
  r.special = (uint32_t)(ec == 2047 || ex == 2047);
  return r;
}

// The base value v: m_v 2^11 * 2^(ev - 1086).
SHAW_FD_HD Term base(double v) {
  const uint64_t bv = bits(v);
  const int ev = (int)((bv >> 52) & 0x7FF);
  Term r;
  r.t = ev != 0 ? ((bv << 11) | (1ull << 63)) : 0ull;
  r.x = ev - 1086;
  r.neg = (uint32_t)(bv >> 63);
  r.special = (uint32_t)(ev == 2047);
  return r;
}

// round(sum of the terms) to FP64, ties to even.  A special term (an infinite or NaN
// input) or a sum outside the normal range sets *bad.
template <int N>
SHAW_FD_HD double sum(const Term (&t)[N], bool* bad) {
  int xm = -100000;
  uint32_t special = 0;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    special |= t[k].special;
    if (t[k].t != 0 && t[k].x > xm) xm = t[k].x;
  }
  if (special) {
    *bad = true;
    return 0.0;
  }
  if (xm == -100000) return 0.0;  // every term is zero
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    const int d = xm + 4 - t[k].x;  // >= 4 for every nonzero term
    const uint64_t u = (t[k].t != 0 && d < 64) ? (t[k].t >> d) : 0ull;
    s += t[k].neg ? -(int64_t)u : (int64_t)u;
  }
  if (s == 0) return 0.0;
  const uint64_t neg = s < 0 ? 1ull : 0ull;
  const uint64_t a = neg ? (uint64_t)(-s) : (uint64_t)s;
  const int lz = clz64(a);
  const uint64_t n = a << lz;  // bit 63 set; value n 2^(xm + 4 - lz)
  uint64_t mant = n >> 11;
  const uint64_t rb = (n >> 10) & 1ull, sticky = (n & 0x3FFull) != 0 ? 1ull : 0ull;
  int e = xm + 1090 - lz;  // value mant 2^(e - 1075)
  if (rb && (sticky || (mant & 1ull))) {
    ++mant;
    if (mant >> 53) {
      mant >>= 1;
      ++e;
    }
  }
  if (e <= 0 || e >= 2047) {  // outside the normal range
    *bad = true;
    return 0.0;
  }
  return from_bits((neg << 63) | ((uint64_t)e << 52) | (mant & 0xFFFFFFFFFFFFFull));
}

// v + cN sN + cS sS + cW sW + cE sE and s + cA vA + cB vB, rounded once.
SHAW_FD_HD double vel(double v, double cN, double sN, double cS, double sS, double cW, double sW, double cE, double sE,
                      bool* bad) {
  const Term t[5] = {base(v), product(cN, sN), product(cS, sS), product(cW, sW), product(cE, sE)};
  return sum<5>(t, bad);
}
SHAW_FD_HD double str(double s, double cA, double vA, double cB, double vB, bool* bad) {
  const Term t[3] = {base(s), product(cA, vA), product(cB, vB)};
  return sum<3>(t, bad);
}

}  // namespace fd
}  // namespace shaw
