// xf64.cuh -- extended-precision arithmetic on the integer pipes for the
// FP64 dependency sweep of Brandes' algorithm.
//
// The reference keeps the dependencies in Float64: coeff = (1 + delta[w]) /
// sigma[w] and delta[v] += sigma[v] * coeff (src/centrality/betweenness.jl:
// 96-99).  On this GPU an FP64 instruction costs about 68 FP32 instructions of
// pipe time, and the dependency sweep adds one term per (DAG arc, source), so
// an FP64-pipe implementation is bound by the FP64 unit.  The sweep instead
// works on non-negative values in this format:
//
//   xf64{m, e}  =  m * 2^(e - 1085),   m in [2^62, 2^63)  or  m = 0 with e = 0.
//
// A finite positive double with biased exponent E and 53-bit significand M
// converts exactly to {M << 10, E}: the format is an IEEE binary64 value with
// 10 more significand bits and an integer exponent.  Every operation below
// truncates at most one unit of its 63-bit result (relative error < 2^-62),
// against the 2^-53 of one FP64 rounding; results go back to binary64 with
// round-to-nearest-even.  Path counts are exact uint64 integers, and their
// reciprocal is computed here by Newton iteration in 64-bit fixed point.
//
// All functions are __host__ __device__ so that the host tests check the same
// code against exact rational arithmetic; only the three primitives
// (high product, clamped right shift, leading zeros) differ by target.
#pragma once

#include <stdint.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace lgbc {

struct xf64 {
  uint64_t m;
  int32_t e;
};

constexpr int kXfBias = 1085;  // 1075 (binary64: value = M * 2^(E - 1075)) + 10 guard bits

// ---- primitives ------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t xf_mulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return static_cast<uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
#endif
}

// x >> n for any n >= 0 (0 once n >= 64).
__host__ __device__ __forceinline__ uint64_t xf_shr(uint64_t x, uint32_t n) {
#ifdef __CUDA_ARCH__
  uint64_t r;
  asm("shr.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(n));  // PTX clamps n to 64
  return r;
#else
  return n >= 64 ? 0 : x >> n;
#endif
}

__host__ __device__ __forceinline__ int xf_clz(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll(static_cast<long long>(x));
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// ---- conversions -------------------------------------------------------------
__host__ __device__ __forceinline__ xf64 xf_zero() { return xf64{0ull, 0}; }

// A non-negative binary64 value given by its bits (zero or normal).
__host__ __device__ __forceinline__ xf64 xf_from_bits(uint64_t b) {
  const int E = static_cast<int>(b >> 52);
  if (E == 0) return xf_zero();
  return xf64{((b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull) << 10, E};
}

// Round to the nearest binary64 value (ties to even); the bits of the result.
// Values stay inside the normal range here (2^-1022 <= x < 2^1024).
__host__ __device__ __forceinline__ uint64_t xf_to_bits(xf64 a) {
  if (a.m == 0) return 0ull;
  const uint64_t M = a.m >> 10;
  const uint32_t r = static_cast<uint32_t>(a.m & 1023u);
  const uint64_t up = (r > 512u || (r == 512u && (M & 1u))) ? 1ull : 0ull;
  // M carries the implicit bit 2^52, which adds one to the exponent field;
  // a round-up to 2^53 carries once more, as it must.
  return (static_cast<uint64_t>(a.e - 1) << 52) + M + up;
}

// ---- arithmetic on non-negative values ---------------------------------------
// a + b.  Both sums of terms < 2^63 fit 64 bits; one shift renormalises.
__host__ __device__ __forceinline__ xf64 xf_add(xf64 a, xf64 b) {
  const int E = a.e > b.e ? a.e : b.e;
  uint64_t m = xf_shr(a.m, static_cast<uint32_t>(E - a.e)) +
               xf_shr(b.m, static_cast<uint32_t>(E - b.e));
  const uint32_t c = static_cast<uint32_t>(m >> 63);
  m >>= c;
  return xf64{m, m ? E + static_cast<int>(c) : 0};
}

// a + x for a non-negative binary64 x given by its bits (zero or normal).
__host__ __device__ __forceinline__ xf64 xf_add_bits(xf64 a, uint64_t xb) {
  return xf_add(a, xf_from_bits(xb));
}

// (hi : lo) of a 64 x 64-bit product of normalised operands (hi >= 2^61),
// normalised to m in [2^62, 2^63); e_hi is the exponent the result would
// have with m = hi.
__host__ __device__ __forceinline__ xf64 xf_norm_product(uint64_t hi, uint64_t lo, int e_hi) {
  if (hi == 0 && lo == 0) return xf_zero();
  // hi >= 2^61 for normalised operands; move the top bit to position 62
  const int lz = xf_clz(hi) - 1;  // 0, 1 or 2 for normalised operands
  uint64_t m;
  if (lz >= 0)
    m = lz == 0 ? hi : ((hi << lz) | (lo >> (64 - lz)));
  else
    m = hi >> 1;
  return xf64{m, e_hi - lz};
}

// a * s for an integer s >= 1 (a path count).
__host__ __device__ __forceinline__ xf64 xf_mul_u64(xf64 a, uint64_t s) {
  if (a.m == 0 || s == 0) return xf_zero();
  const int lz = xf_clz(s);
  const uint64_t sn = s << lz;  // in [2^63, 2^64)
  // a.m * sn = (hi 2^64 + lo); value = a.m sn 2^(a.e - kXfBias - lz)
  return xf_norm_product(xf_mulhi(a.m, sn), a.m * sn, a.e + 64 - lz);
}

// a * b.
__host__ __device__ __forceinline__ xf64 xf_mul(xf64 a, xf64 b) {
  if (a.m == 0 || b.m == 0) return xf_zero();
  const uint64_t bn = b.m << 1;  // in [2^63, 2^64); b = bn 2^(b.e - kXfBias - 1)
  return xf_norm_product(xf_mulhi(a.m, bn), a.m * bn, a.e + b.e - kXfBias + 63);
}

// 1 / s for an integer s >= 1: R ~ 2^127 / sn (sn = s normalised to
// [2^63, 2^64)) from a double-float seed -- the FP32 reciprocal of sn's top
// 24 bits refined by one FP32 Newton step against its top 48 bits (about 46
// correct bits) -- and one Newton step in 64-bit fixed point (relative error
// < 2^-61).
__host__ __device__ __forceinline__ float xf_rcp_seed(float t) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(t));
  return r;
#else
  return 1.0f / t;
#endif
}

__host__ __device__ __forceinline__ float xf_fmaf(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return __builtin_fmaf(a, b, c);
#endif
}

__host__ __device__ __forceinline__ uint32_t xf_float_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  __builtin_memcpy(&u, &f, 4);
  return u;
#endif
}

__host__ __device__ __forceinline__ xf64 xf_recip_u64(uint64_t s) {
  const int lz = xf_clz(s);
  const uint64_t sn = s << lz;  // 1/s = 2^lz / sn
  if (sn == 0x8000000000000000ull) return xf64{1ull << 62, lz + 960};  // a power of two: exact
  // t = sn / 2^40 as a float pair: th in [2^23, 2^24) and tl in [0, 1), both exact
  const float th = static_cast<float>(static_cast<uint32_t>(sn >> 40));
  const float tl = static_cast<float>(static_cast<uint32_t>(sn >> 16) & 0xFFFFFFu) * 0x1p-24f;
  const float r0 = xf_rcp_seed(th);                                  // in (2^-24, 2^-23]
  const float e = xf_fmaf(-tl, r0, xf_fmaf(-th, r0, 1.0f));          // 1 - t r0
  const float c = r0 * e;                                            // 1/t ~ r0 + c
  // x ~ 2^127 / sn = 2^87 / t = (r0 + c) 2^87, r0 2^87 = mr 2^(er + 64) with er = -24, or
  // er = -23 at r0 = 2^-23 where r0 2^87 = 2^64 wraps to 0 and the negative c
  // brings x back below 2^64 (the sum is taken modulo 2^64; x itself fits)
  const uint32_t rb = xf_float_bits(r0);
  const int er = static_cast<int>((rb >> 23) & 0xFFu) - 127;
  const uint64_t mr = static_cast<uint64_t>((rb & 0x7FFFFFu) | 0x800000u);
  const int64_t cx = static_cast<int64_t>(static_cast<int32_t>(c * 0x1p70f)) << 17;  // c 2^87
  uint64_t x = (mr << (er + 64)) + static_cast<uint64_t>(cx);
  if (x == 0) x = 0xFFFFFFFFFFFFFFFFull;  // t = 2^23 exactly (sn < 2^63 + 2^16): seed 2^64
  {
    // err = 2^127 - sn x (two's complement over 128 bits), x += x err / 2^127
    const uint64_t plo = sn * x;
    const uint64_t phi = xf_mulhi(sn, x);
    const uint64_t elo = 0ull - plo;
    const uint64_t ehi = 0x8000000000000000ull - phi - (plo != 0 ? 1ull : 0ull);
    // err >> 63 as a signed 64-bit value (|err| < 2^84 after the seed)
    const int64_t e63 = static_cast<int64_t>((ehi << 1) | (elo >> 63));
    const uint64_t mag = static_cast<uint64_t>(e63 < 0 ? -e63 : e63);
    const uint64_t corr = xf_mulhi(x, mag);  // x |err| / 2^127 = (x |e63|) >> 64
    x = e63 < 0 ? x - corr : x + corr;
  }
  // 1/s = x 2^(lz - 127); x in (2^63, 2^64) up to the last units
  const int lx = xf_clz(x);  // 0 (or 1 if x fell just below 2^63)
  const uint64_t xn = x << lx;
  return xf64{xn >> 1, lz - 127 + 64 - lx + kXfBias - 63};
}

// ---- gather accumulator ------------------------------------------------------
// The dependency gathers add up to 32 terms (one 32-edge chunk) per lane
// between two renormalisations, so their accumulator skips the per-add
// renormalisation of xf_add:
//
//   xg{m, e}  =  m * 2^(e - 1080),   m in [2^57, 2^58) after xg_norm (or 0, e = 0),
//
// terms enter as (53-bit significand << 5) in [2^57, 2^58) and after k adds
// m < (k + 1) 2^58 < 2^64 for k <= 32.  Each add truncates less than one unit
// of the 58-bit scale (relative error < 2^-57, against binary64's 2^-53).
struct xg64 {
  uint64_t m;
  int32_t e;
};

__host__ __device__ __forceinline__ xg64 xg_zero() { return xg64{0ull, 0}; }

// x >> n for n in [0, 2046] (0 once n >= 64).
__host__ __device__ __forceinline__ uint64_t xg_shr(uint64_t x, uint32_t n) { return xf_shr(x, n); }

// a += x for a positive normal binary64 x given by its bits (psi > 0 always).
__host__ __device__ __forceinline__ void xg_add_bits(xg64& a, uint64_t xb) {
  const uint32_t hi = static_cast<uint32_t>(xb >> 32);
  const int ex = static_cast<int>(hi >> 20);
  const uint64_t t = (static_cast<uint64_t>((hi & 0xFFFFFu) | 0x100000u) << 37) |
                     (static_cast<uint64_t>(static_cast<uint32_t>(xb)) << 5);
  const int E = a.e > ex ? a.e : ex;
  a.m = xg_shr(a.m, static_cast<uint32_t>(E - a.e)) + xg_shr(t, static_cast<uint32_t>(E - ex));
  a.e = E;
}

// Back to m in [2^57, 2^58) after at most 32 adds.
__host__ __device__ __forceinline__ void xg_norm(xg64& a) {
  const int top = 63 - xf_clz(a.m);  // 57..63 (or -1 for 0)
  const int sh = top > 57 ? top - 57 : 0;
  a.m >>= sh;
  a.e += sh;
}

// The extended value of a normalised gather accumulator.
__host__ __device__ __forceinline__ xf64 xg_to_xf(xg64 a) { return xf64{a.m << 5, a.e}; }

}  // namespace lgbc
