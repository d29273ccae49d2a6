// wdem_dw.cuh -- double-word arithmetic on FP32: a value is hi + lo, two floats with |lo| <= ulp(hi) / 2,
// 48 significant bits.  On the GB300 the FP32 pipes issue 64 times the FP64 pipe's instructions, so a
// chain of double-word operations (5 to 20 FP32 instructions each) costs a fraction of the same chain in
// FP64.  The building blocks are the error-free transformations (Fast2Sum, 2Sum, 2Prod with FMA) and the
// double-word algorithms of Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic building
// blocks of double-word arithmetic" (ACM TOMS 44, 2017): with u = 2^-24, DWPlusDW (their Algorithm 6) is
// within 3u^2 relative, DWTimesDW (Algorithm 12) within 5u^2, DWTimesFP (Algorithm 9) within 2u^2,
// DWDivDW (Algorithm 18) within 15u^2.  The square root is one Newton step from the FP32 root, evaluated
// with an exact product (error near 2^-47 relative).
//
// Conversions go through the bit patterns on the integer pipe (a double's top 24 significant bits are the
// high word exactly; the remaining 29 are rounded into the low word), so no FP64 instruction is spent on
// them; doubles below 2^-100 in magnitude lose their low word (they are zero for the physics here).
// Arithmetic must be IEEE FP32 in round-to-nearest without flush-to-zero, as nvcc compiles it by default.
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>

namespace wdem {

struct dwf {
  float h, l;
};

#ifdef __CUDACC__
#define WDEM_DW __host__ __device__ __forceinline__
#else
#define WDEM_DW inline
#endif

WDEM_DW uint32_t dwF2U(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u; std::memcpy(&u, &f, 4); return u;
#endif
}
WDEM_DW float dwU2F(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f; std::memcpy(&f, &u, 4); return f;
#endif
}
WDEM_DW uint64_t dwD2U(double d) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u; std::memcpy(&u, &d, 8); return u;
#endif
}
WDEM_DW double dwU2D(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double d; std::memcpy(&d, &u, 8); return d;
#endif
}
WDEM_DW float dwFma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

// ---- error-free transformations
WDEM_DW dwf fast2Sum(float a, float b) {  // |a| >= |b| (or a's exponent >= b's)
  const float s = a + b;
  const float z = s - a;
  return {s, b - z};
}
WDEM_DW dwf twoSum(float a, float b) {
  const float s = a + b;
  const float ap = s - b;
  const float bp = s - ap;
  return {s, (a - ap) + (b - bp)};
}
WDEM_DW dwf twoProd(float a, float b) {
  const float p = a * b;
  return {p, dwFma(a, b, -p)};
}

// ---- conversions
// double -> double word: hi = the top 24 significant bits (exact), lo = the rest rounded to 24 bits
WDEM_DW dwf dwFrom(double d) {
  const uint64_t b = dwD2U(d);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff);          // biased exponent
  if (e == 0x7ff) {                                 // Inf / NaN: carried in hi
    const float v = (float)d;
    return {v, 0.f};
  }
  const int E = e - 1023;                           // unbiased
  if (E < -126) return {0.f, 0.f};                  // below FP32's normal range: zero here
  if (E > 127) return {dwU2F(sign | 0x7f800000u), 0.f};
  const uint64_t m = b & 0xFFFFFFFFFFFFFull;        // 52 mantissa bits
  const float h = dwU2F(sign | ((uint32_t)(E + 127) << 23) | (uint32_t)(m >> 29));
  const uint32_t mlo = (uint32_t)(m & 0x1FFFFFFFu); // the 29 bits below hi
  if (mlo == 0 || E < -100) return {h, 0.f};
  // lo = mlo * 2^(E - 52) with hi's sign: (float)mlo rounds to 24 bits, the scale is a power of two
  float l = (float)mlo * 1.862645149230957e-09f;    // * 2^-29, exact
  l *= dwU2F((uint32_t)(E - 23 + 127) << 23);       // * 2^(E - 23), exact (E - 23 >= -123)
  // hi was truncated, so lo may reach a whole ulp of hi: renormalise to |lo| <= ulp(hi) / 2
  return fast2Sum(h, sign ? -l : l);
}
WDEM_DW double dwTo(dwf x) { return (double)x.h + (double)x.l; }
WDEM_DW dwf dwF(float f) { return {f, 0.f}; }

// ---- arithmetic
WDEM_DW dwf dwNeg(dwf x) { return {-x.h, -x.l}; }
// DWPlusDW, accurate version (Algorithm 6)
WDEM_DW dwf dwAdd(dwf x, dwf y) {
  const dwf s = twoSum(x.h, y.h);
  const dwf t = twoSum(x.l, y.l);
  const float c = s.l + t.h;
  const dwf v = fast2Sum(s.h, c);
  const float w = t.l + v.l;
  return fast2Sum(v.h, w);
}
WDEM_DW dwf dwSub(dwf x, dwf y) { return dwAdd(x, dwNeg(y)); }
// DWPlusFP (Algorithm 4)
WDEM_DW dwf dwAddF(dwf x, float y) {
  const dwf s = twoSum(x.h, y);
  const float v = x.l + s.l;
  return fast2Sum(s.h, v);
}
// DWTimesDW with FMA (Algorithm 12)
WDEM_DW dwf dwMul(dwf x, dwf y) {
  const dwf c = twoProd(x.h, y.h);
  const float tl0 = x.l * y.l;
  const float tl1 = dwFma(x.h, y.l, tl0);
  const float cl2 = dwFma(x.l, y.h, tl1);
  const float cl3 = c.l + cl2;
  return fast2Sum(c.h, cl3);
}
// DWTimesFP with FMA (Algorithm 9)
WDEM_DW dwf dwMulF(dwf x, float y) {
  const dwf c = twoProd(x.h, y);
  const float cl3 = dwFma(x.l, y, c.l);
  return fast2Sum(c.h, cl3);
}
// x * 2^k for a power of two given as a float: exact
WDEM_DW dwf dwScale(dwf x, float p2) { return {x.h * p2, x.l * p2}; }
// DWDivDW (Algorithm 18 without the second correction: error below 15u^2 for the first quotient and one
// correction step, here as in their Algorithm 17 followed by Fast2Sum)
WDEM_DW dwf dwDiv(dwf x, dwf y) {
  const float th = x.h / y.h;
  const dwf r = dwMulF(y, th);
  const float pih = x.h - r.h;
  const float dl = x.l - r.l;
  const float d = pih + dl;
  const float tl = d / y.h;
  return fast2Sum(th, tl);
}
// square root: s = sqrt(hi), then s + (x - s^2) / (2 s) with s^2 exact
WDEM_DW dwf dwSqrt(dwf x) {
  if (!(x.h > 0.f)) return {x.h == 0.f ? 0.f : sqrtf(x.h), 0.f};
  const float s = sqrtf(x.h);
  const dwf p = twoProd(s, s);
  const float r = ((x.h - p.h) - p.l + x.l) / (2.f * s);
  return fast2Sum(s, r);
}
WDEM_DW dwf dwRecip(dwf y) { return dwDiv(dwF(1.f), y); }
WDEM_DW bool dwPos(dwf x) { return x.h > 0.f || (x.h == 0.f && x.l > 0.f); }
WDEM_DW bool dwNegative(dwf x) { return x.h < 0.f || (x.h == 0.f && x.l < 0.f); }
WDEM_DW bool dwGt(dwf x, dwf y) { return x.h > y.h || (x.h == y.h && x.l > y.l); }
WDEM_DW dwf dwAbs(dwf x) { return dwNegative(x) ? dwNeg(x) : x; }
WDEM_DW dwf dwMin(dwf x, dwf y) { return dwGt(x, y) ? y : x; }
WDEM_DW dwf dwMax(dwf x, dwf y) { return dwGt(x, y) ? x : y; }
WDEM_DW bool dwIsZero(dwf x) { return x.h == 0.f && x.l == 0.f; }

// ---- 3-vectors
struct dw3 {
  dwf x, y, z;
};
WDEM_DW dw3 dw3From(double a, double b, double c) { return {dwFrom(a), dwFrom(b), dwFrom(c)}; }
WDEM_DW dw3 dw3Add(dw3 a, dw3 b) { return {dwAdd(a.x, b.x), dwAdd(a.y, b.y), dwAdd(a.z, b.z)}; }
WDEM_DW dw3 dw3Sub(dw3 a, dw3 b) { return {dwSub(a.x, b.x), dwSub(a.y, b.y), dwSub(a.z, b.z)}; }
WDEM_DW dw3 dw3Mul(dw3 a, dwf s) { return {dwMul(a.x, s), dwMul(a.y, s), dwMul(a.z, s)}; }
WDEM_DW dw3 dw3MulF(dw3 a, float s) { return {dwMulF(a.x, s), dwMulF(a.y, s), dwMulF(a.z, s)}; }
WDEM_DW dwf dw3Dot(dw3 a, dw3 b) { return dwAdd(dwAdd(dwMul(a.x, b.x), dwMul(a.y, b.y)), dwMul(a.z, b.z)); }
WDEM_DW dw3 dw3Cross(dw3 a, dw3 b) {
  return {dwSub(dwMul(a.y, b.z), dwMul(a.z, b.y)), dwSub(dwMul(a.z, b.x), dwMul(a.x, b.z)),
          dwSub(dwMul(a.x, b.y), dwMul(a.y, b.x))};
}
WDEM_DW dwf dw3Sq(dw3 a) { return dw3Dot(a, a); }

}  // namespace wdem
