// wdem_math.cuh -- FP64 vector/quaternion helpers for the DEM kernels.
//
// Every helper performs the IEEE operations in the same order as Woo's Eigen expressions
// (left-to-right; dot = (a0 b0 + a1 b1) + a2 b2), and the kernels are compiled with
// --fmad=false, so per-contact results reproduce the CPU restatement bit for bit.  In the contracted
// variant (WDEM_FMA, wdem_variant.h) multiply-adds become FMAs and the helpers marked below divide by a
// scalar through one reciprocal (normalisations through one reciprocal square root).
#pragma once
#include <cuda_runtime.h>
#include "wdem_variant.h"

// Keeps the compiler from if-converting a skipped branch (which would issue the FP64 division
// sequence anyway under a predicate): the empty volatile asm marks the block as having effects.
#define WDEM_REAL_BRANCH() asm volatile("")

namespace wdem {
WDEM_VARIANT_BEGIN

struct d3 { double x, y, z; };

__device__ __forceinline__ d3 mk(double x, double y, double z) { d3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ d3 xyz(const double4_32a& v) { return mk(v.x, v.y, v.z); }
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ d3 operator-(d3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ d3 operator*(d3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ d3 operator*(double s, d3 a) { return mk(s * a.x, s * a.y, s * a.z); }
#ifdef WDEM_FMA
__device__ __forceinline__ d3 operator/(d3 a, double s) { const double r = 1.0 / s; return mk(a.x * r, a.y * r, a.z * r); }
#else
__device__ __forceinline__ d3 operator/(d3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
#endif
__device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double sqnorm(d3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
// sqnorm with every operation rounded on its own in both variants (never contracted): the contracted
// variant keeps the sphere distance, the near-cancelling overlap |d| - r1 - r2 and the position update
// identical to the exact variant, so that contact forces agree to rounding after a step from one state
__device__ __forceinline__ double sqnormExact(d3 a) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)), __dmul_rn(a.z, a.z));
}
// v + a s, never contracted (the position update pos + vel dt)
__device__ __forceinline__ double addMulExact(double v, double a, double s) { return __dadd_rn(v, __dmul_rn(a, s)); }
__device__ __forceinline__ d3 cross(d3 a, d3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ bool isZero(d3 a) { return a.x == 0 && a.y == 0 && a.z == 0; }

// Predicates on the bit patterns, evaluated on the integer pipe instead of FP64 compares (the FP64
// pipe is the binding unit of these kernels on GB300).  Each equals its FP64 counterpart exactly.  The
// two 32-bit halves come out of an asm move, which the compiler cannot see through: a 64-bit bit test
// such as (bits << 1) == 0 is recognised as x == 0 and turned back into an FP64 compare.
struct Halves { unsigned lo, hi; };
__device__ __forceinline__ Halves halvesOf(double x) {
  Halves h;
  asm("mov.b64 {%0, %1}, %2;" : "=r"(h.lo), "=r"(h.hi) : "d"(x));
  return h;
}
__device__ __forceinline__ double fromHalves(unsigned lo, unsigned hi) {
  double x;
  asm("mov.b64 %0, {%1, %2};" : "=d"(x) : "r"(lo), "r"(hi));
  return x;
}
__device__ __forceinline__ unsigned long long bitsOf(double x) {
  const Halves h = halvesOf(x);
  return ((unsigned long long)h.hi << 32) | h.lo;
}
__device__ __forceinline__ bool zeroBits(double x) { const Halves h = halvesOf(x); return ((h.hi << 1) | h.lo) == 0; }  // x == 0
__device__ __forceinline__ bool isZeroBits(d3 a) {
  const Halves x = halvesOf(a.x), y = halvesOf(a.y), z = halvesOf(a.z);
  return (((x.hi | y.hi | z.hi) << 1) | x.lo | y.lo | z.lo) == 0;
}
__device__ __forceinline__ bool negZero(double x) { const Halves h = halvesOf(x); return h.hi == 0x80000000u && h.lo == 0; }
__device__ __forceinline__ bool hasNegZero(d3 a) { return negZero(a.x) || negZero(a.y) || negZero(a.z); }
// y > 0 (positive, nonzero, not NaN; +inf included)
__device__ __forceinline__ bool positiveBits(double y) {
  const Halves h = halvesOf(y);
  const bool pos = !(h.hi & 0x80000000u) && (h.hi | h.lo) != 0;
  const bool notNaN = h.hi < 0x7ff00000u || (h.hi == 0x7ff00000u && h.lo == 0);
  return pos && notNaN;
}
// y < 0 (negative, nonzero, not NaN; -inf included)
__device__ __forceinline__ bool negativeBits(double y) {
  const Halves h = halvesOf(y);
  const unsigned m = h.hi & 0x7fffffffu;
  return (h.hi & 0x80000000u) && (m | h.lo) != 0 && (m < 0x7ff00000u || (m == 0x7ff00000u && h.lo == 0));
}
__device__ __forceinline__ bool nanBits(double x) {
  const Halves h = halvesOf(x);
  const unsigned m = h.hi & 0x7fffffffu;
  return m > 0x7ff00000u || (m == 0x7ff00000u && h.lo != 0);
}
__device__ __forceinline__ bool isOneBits(double x) { const Halves h = halvesOf(x); return h.hi == 0x3ff00000u && h.lo == 0; }  // x == 1.0
__device__ __forceinline__ bool finiteBits(double x) { return (halvesOf(x).hi & 0x7ff00000u) != 0x7ff00000u; }
// a * b for finite a and b == +-0: the zero with the product's sign
__device__ __forceinline__ double signedZero(double a, double b) {
  return fromHalves(0u, (halvesOf(a).hi ^ halvesOf(b).hi) & 0x80000000u);
}
// the sign bits of a and b differ
__device__ __forceinline__ bool signsDiffer(double a, double b) { return ((halvesOf(a).hi ^ halvesOf(b).hi) >> 31) != 0; }
// Eigen normalize().  When the squared norm is exactly 1, sqrt gives exactly 1 and the divisions
// are identities: skipping them changes no bit and saves FP64 issue slots.
__device__ __forceinline__ d3 normalized(d3 a) {
  double z = sqnorm(a);
#ifdef WDEM_FMA
  if (z > 0 && z != 1.0) { WDEM_REAL_BRANCH(); const double r = rsqrt(z); a.x *= r; a.y *= r; a.z *= r; }
#else
  if (z > 0 && z != 1.0) { WDEM_REAL_BRANCH(); double n = sqrt(z); a.x /= n; a.y /= n; a.z /= n; }
#endif
  return a;
}
// x / y for y > 0 finite or +inf: a zero numerator is its own quotient (keeping the sign of zero),
// so the software FP64 division is skipped bit-exactly.
__device__ __forceinline__ double qdiv(double x, double y) {
  double r = x;
  if (!(zeroBits(x) && positiveBits(y))) { WDEM_REAL_BRANCH(); r = x / y; }
  return r;
}
// v / s per component (v / m, the acceleration of a node): three qdiv; contracted variant: one reciprocal
__device__ __forceinline__ d3 divBy(d3 v, double s) {
#ifdef WDEM_FMA
  const double r = 1.0 / s;
  return mk(v.x * r, v.y * r, v.z * r);
#else
  return mk(qdiv(v.x, s), qdiv(v.y, s), qdiv(v.z, s));
#endif
}
// v / d per component (torque / inertia): three qdiv; contracted variant: one reciprocal when the three
// divisors are equal (spheres), else three
__device__ __forceinline__ d3 divByEach(d3 v, d3 d) {
#ifdef WDEM_FMA
  if (d.x == d.y && d.y == d.z) { const double r = 1.0 / d.x; return mk(v.x * r, v.y * r, v.z * r); }
  return mk(v.x / d.x, v.y / d.y, v.z / d.z);
#else
  return mk(qdiv(v.x, d.x), qdiv(v.y, d.y), qdiv(v.z, d.z));
#endif
}
__device__ __forceinline__ double comp(d3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ void setComp(d3& a, int i, double v) { if (i == 0) a.x = v; else if (i == 1) a.y = v; else a.z = v; }

// row-major 3x3 times vector, each row summed left to right
__device__ __forceinline__ d3 mvec(const double* m, d3 v) {
  return mk(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z, m[6] * v.x + m[7] * v.y + m[8] * v.z);
}

struct qd { double w, x, y, z; };

// Rotation matrix given by columns c0, c1, c2 -> unit quaternion (Shoemake: trace branch, else the
// largest diagonal element).  m(r,k) = column k, row r.
__device__ __forceinline__ qd quatFromCols(d3 c0, d3 c1, d3 c2) {
  const double m00 = c0.x, m10 = c0.y, m20 = c0.z;
  const double m01 = c1.x, m11 = c1.y, m21 = c1.z;
  const double m02 = c2.x, m12 = c2.y, m22 = c2.z;
  qd q;
  double t = m00 + m11 + m22;
  if (t > 0) {
    t = sqrt(t + 1.0);
    q.w = 0.5 * t;
    t = 0.5 / t;
    q.x = (m21 - m12) * t;
    q.y = (m02 - m20) * t;
    q.z = (m10 - m01) * t;
  } else {
    // largest diagonal element i, j = i+1, k = j+1 (mod 3), written out per case
    int i = 0;
    if (m11 > m00) i = 1;
    if (m22 > (i == 0 ? m00 : m11)) i = 2;
    if (i == 0) {         // j=1, k=2
      t = sqrt(m00 - m11 - m22 + 1.0);
      q.x = 0.5 * t; t = 0.5 / t;
      q.w = (m21 - m12) * t; q.y = (m10 + m01) * t; q.z = (m20 + m02) * t;
    } else if (i == 1) {  // j=2, k=0
      t = sqrt(m11 - m22 - m00 + 1.0);
      q.y = 0.5 * t; t = 0.5 / t;
      q.w = (m02 - m20) * t; q.z = (m21 + m12) * t; q.x = (m01 + m10) * t;
    } else {              // j=0, k=1
      t = sqrt(m22 - m00 - m11 + 1.0);
      q.z = 0.5 * t; t = 0.5 / t;
      q.w = (m10 - m01) * t; q.x = (m02 + m20) * t; q.y = (m12 + m21) * t;
    }
  }
  return q;
}

// v rotated by unit quaternion q: uv = q.vec x v; uv += uv; v + w uv + q.vec x uv
__device__ __forceinline__ d3 qrot(qd q, d3 v) {
  d3 qv = mk(q.x, q.y, q.z);
  d3 uv = cross(qv, v);
  uv = uv + uv;
  return v + q.w * uv + cross(qv, uv);
}

__device__ __forceinline__ qd qmul(qd a, qd b) {
  qd r;
  r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
  r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
  r.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
  r.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
  return r;
}

__device__ __forceinline__ qd qnormalized(qd q) {
  double z2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
#ifdef WDEM_FMA
  if (!isOneBits(z2) && z2 > 0) { WDEM_REAL_BRANCH(); const double r = rsqrt(z2); q.x *= r; q.y *= r; q.z *= r; q.w *= r; }
#else
  if (!isOneBits(z2) && z2 > 0) { WDEM_REAL_BRANCH(); double n = sqrt(z2); q.x /= n; q.y /= n; q.z /= n; q.w /= n; }
#endif
  return q;
}

// Eigen maxCoeff of a 3-vector: maxi(maxi(a0,a1),a2), maxi(a,b) = a<b ? b : a
__device__ __forceinline__ double dmax3(d3 a) {
  double m = (a.x < a.y) ? a.y : a.x;
  return (m < a.z) ? a.z : m;
}

__device__ __forceinline__ double signum(double f) { return f < 0 ? -1.0 : (f > 0 ? 1.0 : 0.0); }

__device__ __forceinline__ int expBits(double x) { return (int)((halvesOf(x).hi >> 20) & 0x7ff); }

// Mathr::Sign(F * u) (-1, 0, +1; 0 for NaN): the sign bits decide unless a factor is zero, not finite,
// subnormal, or the product could underflow to zero, in which case the product is formed.
__device__ __forceinline__ int signProd(double F, double u) {
  if (zeroBits(F) || zeroBits(u)) return 0;
  const int eF = expBits(F), eu = expBits(u);
  if (eF != 0 && eF != 0x7ff && eu != 0 && eu != 0x7ff && eF + eu > 1100)
    return signsDiffer(F, u) ? -1 : 1;
  WDEM_REAL_BRANCH();
  const double pr = F * u;
  return pr < 0 ? -1 : (pr > 0 ? 1 : 0);
}

// v + s a for a == +-0 and finite s: s a is a zero of sign(s) ^ sign(a), and adding a zero changes v only
// from -0 to +0 (round to nearest: -0 + +0 = +0); otherwise the operations are done.
__device__ __forceinline__ double addScaled(double v, double s, double a) {
  if (zeroBits(a) && finiteBits(s)) {
    const bool addendNeg = signsDiffer(s, a);
    return (negZero(v) && !addendNeg) ? 0.0 : v;
  }
  WDEM_REAL_BRANCH();
  return v + s * a;
}
// a * b with a of known class (0: +0, 1: -0, 2: exactly 1, 3: other; MCLS_* of the step parameters):
// a zero or unit factor times a finite b is formed on the integer pipe (IEEE: +-0 * b is the zero with
// the sign of the product, 1 * b is b)
__device__ __forceinline__ double mulC(double a, int cls, double b) {
  if (cls != 3 && finiteBits(b)) return cls == 2 ? b : signedZero(a, b);
  WDEM_REAL_BRANCH();
  return a * b;
}
// a * b where a zero a times a finite b is the signed zero
__device__ __forceinline__ double mulZ(double a, double b) {
  if (zeroBits(a) && finiteBits(b)) return signedZero(a, b);
  WDEM_REAL_BRANCH();
  return a * b;
}
// a + b; when an operand is a zero the sum is the other operand, except -0 + +0 = +0 (round to nearest)
__device__ __forceinline__ double addZ(double a, double b) {
  if (zeroBits(b)) return (negZero(a) && !negZero(b)) ? 0.0 : a;
  if (zeroBits(a)) return b;
  WDEM_REAL_BRANCH();
  return a + b;
}
__device__ __forceinline__ double negD(double a) { const Halves h = halvesOf(a); return fromHalves(h.lo, h.hi ^ 0x80000000u); }
// row-major m (entry classes cls) times v, each row summed left to right: mvec with the zero and unit
// entries' contributions formed exactly without FP64 operations
__device__ __forceinline__ d3 mvecC(const double* m, int cls, d3 v) {
  double r[3];
  for (int i = 0; i < 3; i++) {
    const double t0 = mulC(m[3 * i], (cls >> (6 * i)) & 3, v.x);
    const double t1 = mulC(m[3 * i + 1], (cls >> (6 * i + 2)) & 3, v.y);
    const double t2 = mulC(m[3 * i + 2], (cls >> (6 * i + 4)) & 3, v.z);
    r[i] = addZ(addZ(t0, t1), t2);
  }
  return mk(r[0], r[1], r[2]);
}

// v + a s (operands of the product in this order) for the position update pos + vel dt
__device__ __forceinline__ double addScaledR(double v, double a, double s) {
  if (zeroBits(a) && finiteBits(s)) {
    const bool addendNeg = signsDiffer(s, a);
    return (negZero(v) && !addendNeg) ? 0.0 : v;
  }
  WDEM_REAL_BRANCH();
  return addMulExact(v, a, s);
}

// double -> float by truncating the mantissa (error below 2^-23 relative) for values in the float normal
// range, on the integer pipe; zeros keep their sign; other values use the hardware conversion.
__device__ __forceinline__ float truncF(double x) {
  const Halves h = halvesOf(x);
  const int e = (int)((h.hi >> 20) & 0x7ff);
  // sign, rebased exponent, the top 23 of the 52 mantissa bits (20 in hi, 3 in lo)
  if (e >= 897 && e <= 1150)
    return __uint_as_float((h.hi & 0x80000000u) | ((unsigned)(e - 896) << 23) | ((h.hi & 0xfffffu) << 3) | (h.lo >> 29));
  if (((h.hi << 1) | h.lo) == 0) return __uint_as_float(h.hi & 0x80000000u);
  WDEM_REAL_BRANCH();
  return (float)x;
}

// x^n by squaring, n small and fixed (pown of Woo's Math.hpp)
__device__ __forceinline__ double pown3(double x) {
  // n=3: d=1, r=1 -> pown(x*x,1) * x ; pown(y,1): d=0,r=1 -> 1*y
  double y = x * x;
  double x2d = 1.0 * y;
  return x2d * x;
}
__device__ __forceinline__ double pown5(double x) {
  // n=5: d=2, r=1 -> pown(x*x,2)*x ; pown(y,2): d=1,r=0 -> pown(y*y,1)*1 = (1*(y*y))*1
  double y = x * x;
  double z = y * y;
  double p2 = (1.0 * z) * 1.0;
  return p2 * x;
}

WDEM_VARIANT_END
}  // namespace wdem
