// gbdx_f64i.cuh -- IEEE-754 binary64 operations evaluated on the integer
// pipes.  GB300 issues FP64 instructions at a small fraction of the FP32 rate,
// and the per-step time update of an FP32-state trajectory (the step size
// dt * factor, the new time t + dt and the FP32 copy of dt) is otherwise the
// only FP64 work of a step.  These routines return exactly the value the FP64
// instruction would (round to nearest, ties to even) for finite normal
// operands with a normal result; every other input takes the hardware
// instruction.  The algorithms are the textbook ones: align the significands
// with the shifted-out bits folded into a sticky bit, add or subtract, renormalise
// and round on the guard bits.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define GBDX_HD __host__ __device__ __forceinline__
#else
#define GBDX_HD inline
#endif

namespace gbdx {

GBDX_HD uint64_t f64i_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

GBDX_HD double f64i_double(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

GBDX_HD uint32_t f64i_fbits(float x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

GBDX_HD float f64i_float(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

// The hardware operations for the inputs the integer paths do not take.  Kept
// out of line on the device so the compiler cannot evaluate them
// speculatively beside the integer path (a select of both results would put
// the FP64 instruction back on every call).
#ifdef __CUDA_ARCH__
static __device__ __noinline__ double f64i_hw_add(double a, double b) { return a + b; }
static __device__ __noinline__ double f64i_hw_mul(double a, float f) { return a * double(f); }
static __device__ __noinline__ float f64i_hw_cvt(double a) { return float(a); }
static __device__ __noinline__ double f64i_hw_widen(float f) { return double(f); }
#else
inline double f64i_hw_add(double a, double b) { return a + b; }
inline double f64i_hw_mul(double a, float f) { return a * double(f); }
inline float f64i_hw_cvt(double a) { return float(a); }
inline double f64i_hw_widen(float f) { return double(f); }
#endif

GBDX_HD int f64i_clz(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

// double(f): binary32 -> binary64 (exact).
GBDX_HD double f64i_from_f32(float f) {
  const uint32_t u = f64i_fbits(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return f64i_hw_widen(f);  // zero, subnormal, inf, NaN
  // exponent rebias 127 -> 1023 (896 << 20 in the high word); the 23 fraction
  // bits become the top of the 52
  const uint32_t hi = (u & 0x80000000u) | (((u & 0x7fffffffu) >> 3) + (896u << 20));
  return f64i_double((uint64_t(hi) << 32) | uint64_t(u << 29));
}

// float(a): binary64 -> binary32, round to nearest even.
GBDX_HD float f64i_to_f32(double a) {
  const uint64_t u = f64i_bits(a);
  const uint32_t hi = uint32_t(u >> 32), lo = uint32_t(u);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  // binary32 normal exponents 1..254 are binary64 exponents 897..1150
  if (e < 897u || e > 1150u) return f64i_hw_cvt(a);
  uint32_t r = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  const uint32_t rem = lo & 0x1fffffffu;
  // a carry out of the significand steps the exponent; past 254 it is inf
  if (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) r++;
  return f64i_float((hi & 0x80000000u) | r);
}

// a * double(f), round to nearest even (the binary32 operand widens exactly).
GBDX_HD double f64i_mul_f32(double a, float f) {
  const uint64_t ua = f64i_bits(a);
  const uint32_t uf = f64i_fbits(f);
  const uint32_t ea = uint32_t(ua >> 52) & 0x7ffu, ef = (uf >> 23) & 0xffu;
  if (ea == 0u || ea == 0x7ffu || ef == 0u || ef == 0xffu) return f64i_hw_mul(a, f);
  const uint64_t ma = (ua & 0xfffffffffffffull) | (1ull << 52);  // 53 bits
  const uint32_t mf = (uf & 0x7fffffu) | 0x800000u;               // 24 bits
  // P = ma * mf < 2^77 as p1 * 2^32 + lo
  const uint64_t p0 = uint64_t(uint32_t(ma)) * mf;
  const uint64_t p1 = uint64_t(uint32_t(ma >> 32)) * mf + (p0 >> 32);
  const uint32_t lo = uint32_t(p0);
  int e = int(ea) + int(ef) - 127;
  uint64_t q;
  uint32_t r, half;
  if (p1 >> 44) {  // P >= 2^76: keep bits 76..24
    q = (p1 << 8) | (lo >> 24);
    r = lo & 0xffffffu;
    half = 0x800000u;
    e += 1;
  } else {  // P in [2^75, 2^76): keep bits 75..23
    q = (p1 << 9) | (lo >> 23);
    r = lo & 0x7fffffu;
    half = 0x400000u;
  }
  if (r > half || (r == half && (q & 1u))) q++;
  // q in [2^52, 2^53]; (e - 1) << 52 plus q carries a rounding overflow into e
  if (e < 1 || e + int(q >> 53) > 0x7fe) return f64i_hw_mul(a, f);
  const uint64_t sign = (ua ^ (uint64_t(uf) << 32)) & 0x8000000000000000ull;
  return f64i_double(sign | ((uint64_t(e - 1) << 52) + q));
}

// a + b, round to nearest even.
GBDX_HD double f64i_add(double a, double b) {
  uint64_t ua = f64i_bits(a), ub = f64i_bits(b);
  const uint64_t kAbs = 0x7fffffffffffffffull;
  if ((ua & kAbs) < (ub & kAbs)) {
    const uint64_t t = ua;
    ua = ub;
    ub = t;
  }
  const uint32_t ea = uint32_t(ua >> 52) & 0x7ffu, eb = uint32_t(ub >> 52) & 0x7ffu;
  // |a| >= |b|: a zero or subnormal b, or an inf/NaN a, goes to the hardware
  if (eb == 0u || ea == 0x7ffu) return f64i_hw_add(a, b);
  const uint64_t kFrac = 0xfffffffffffffull;
  // significands with 9 guard bits: the leading bit sits at bit 61
  const uint64_t ma = ((ua & kFrac) | (1ull << 52)) << 9;
  uint64_t mb = ((ub & kFrac) | (1ull << 52)) << 9;
  const uint32_t d = ea - eb;
  if (d != 0u) mb = d < 63u ? (mb >> d) | uint64_t((mb << (64u - d)) != 0ull) : 1ull;
  int e = int(ea);
  uint64_t m;
  if (((ua ^ ub) >> 63) == 0ull) {
    m = ma + mb;  // < 2^63
    if (m >> 62) {
      m = (m >> 1) | (m & 1ull);
      e++;
    }
  } else {
    m = ma - mb;
    if (m == 0ull) return 0.0;  // x + (-x) is +0 under round to nearest
    const int z = f64i_clz(m) - 2;
    m <<= z;
    e -= z;
    if (e <= 0) return f64i_hw_add(a, b);  // subnormal result
  }
  uint64_t q = m >> 9;
  const uint32_t r = uint32_t(m) & 0x1ffu;
  if (r > 0x100u || (r == 0x100u && (q & 1u))) q++;
  if (e + int(q >> 53) > 0x7fe) return f64i_hw_add(a, b);  // overflow
  return f64i_double((ua & 0x8000000000000000ull) | ((uint64_t(e - 1) << 52) + q));
}

}  // namespace gbdx
