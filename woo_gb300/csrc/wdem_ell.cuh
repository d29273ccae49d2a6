// wdem_ell.cuh -- ellipsoid contact geometry on the GPU.
//
// Cg2_Ellipsoid_Ellipsoid_L6Geom / Cg2_Sphere_Ellipsoid_L6Geom (Ellipsoid.cpp:259-351) use the
// Perram-Wertheim contact function S(l) = l (1-l) R^T G(l)^-1 R, G(l) = (1-l) A^-1 + l B^-1, with
// A = sum_k u_k u_k^T / a_k^2 built from the orientation columns u_k and semi-axes a_k; its maximum
// F_ab decides contact (F_ab <= 1) and gives the contact point and overlap.  Two maximisers:
//   - Brent's method on -S (the reference's, restated operation for operation, so that the result
//     equals the CPU restatement bit for bit), and
//   - Newton-Raphson on S'(l) = 0 (the reference leaves this branch unimplemented), safeguarded by
//     a bracket from the sign of S' (S is concave on [0,1]), converged when |dl| <= tol, started
//     from a cold guess, the previous step's l, or the learned warm start.
// All 3x3 matrices here are symmetric; they are stored as (m00 m01 m02 m11 m12 m22).  The inverse
// follows Eigen's 3x3 formula (cofactors, det from column 0, adjugate times 1/det), which for an
// exactly symmetric input yields an exactly symmetric result, so the 6-entry form is bit-identical to
// the general one.
#pragma once
#include "wdem_math.cuh"
#include "wdem_variant.h"

namespace wdem {
WDEM_VARIANT_BEGIN

struct s33 { double a, b, c, d, e, f; };  // (0,0) (0,1) (0,2) (1,1) (1,2) (2,2)

__device__ __forceinline__ s33 symInv(const s33& m) {
  const double c00 = m.d * m.f - m.e * m.e;
  const double c01 = m.c * m.e - m.b * m.f;
  const double c02 = m.b * m.e - m.c * m.d;
  const double c11 = m.a * m.f - m.c * m.c;
  const double c12 = m.c * m.b - m.a * m.e;
  const double c22 = m.a * m.d - m.b * m.b;
  const double det = c00 * m.a + c01 * m.b + c02 * m.c;
  const double inv = 1.0 / det;
  s33 r;
  r.a = c00 * inv; r.b = c01 * inv; r.c = c02 * inv; r.d = c11 * inv; r.e = c12 * inv; r.f = c22 * inv;
  return r;
}
// (1-l) A + l B, elementwise
__device__ __forceinline__ s33 symMix(const s33& A, const s33& B, double l) {
  const double w = 1 - l;
  s33 G;
  G.a = w * A.a + l * B.a; G.b = w * A.b + l * B.b; G.c = w * A.c + l * B.c;
  G.d = w * A.d + l * B.d; G.e = w * A.e + l * B.e; G.f = w * A.f + l * B.f;
  return G;
}
// M v, rows summed left to right
__device__ __forceinline__ d3 symMul(const s33& m, d3 v) {
  return mk(m.a * v.x + m.b * v.y + m.c * v.z, m.b * v.x + m.d * v.y + m.e * v.z, m.c * v.x + m.e * v.y + m.f * v.z);
}
// sum_k u_k u_k^T / a_k^2 accumulated from zero, u_k = q * e_k (Ellipsoid.cpp:286-289)
__device__ __forceinline__ s33 shapeMatrix(qd q, d3 semi) {
  const d3 u0 = qrot(q, mk(1, 0, 0)), u1 = qrot(q, mk(0, 1, 0)), u2 = qrot(q, mk(0, 0, 1));
  const double s0 = semi.x * semi.x, s1 = semi.y * semi.y, s2 = semi.z * semi.z;
  s33 A;
  A.a = 0.0 + (u0.x * u0.x) / s0; A.b = 0.0 + (u0.x * u0.y) / s0; A.c = 0.0 + (u0.x * u0.z) / s0;
  A.d = 0.0 + (u0.y * u0.y) / s0; A.e = 0.0 + (u0.y * u0.z) / s0; A.f = 0.0 + (u0.z * u0.z) / s0;
  A.a = A.a + (u1.x * u1.x) / s1; A.b = A.b + (u1.x * u1.y) / s1; A.c = A.c + (u1.x * u1.z) / s1;
  A.d = A.d + (u1.y * u1.y) / s1; A.e = A.e + (u1.y * u1.z) / s1; A.f = A.f + (u1.z * u1.z) / s1;
  A.a = A.a + (u2.x * u2.x) / s2; A.b = A.b + (u2.x * u2.y) / s2; A.c = A.c + (u2.x * u2.z) / s2;
  A.d = A.d + (u2.y * u2.y) / s2; A.e = A.e + (u2.y * u2.z) / s2; A.f = A.f + (u2.z * u2.z) / s2;
  return A;
}

// -l (1-l) R^T G(l)^-1 R as the reference's functor evaluates it (Ellipsoid.cpp:293)
__device__ __forceinline__ double pwNegS(const s33& Ai, const s33& Bi, d3 R, double l) {
  const s33 Gi = symInv(symMix(Ai, Bi, l));
  const double sc = -l * (1 - l);
  const d3 sR = sc * R;
  const d3 t = mk(sR.x * Gi.a + sR.y * Gi.b + sR.z * Gi.c, sR.x * Gi.b + sR.y * Gi.d + sR.z * Gi.e,
                  sR.x * Gi.c + sR.y * Gi.e + sR.z * Gi.f);
  return t.x * R.x + t.y * R.y + t.z * R.z;
}

// Brent's minimisation of -S on [0, 1] (R. P. Brent 1973, ch. 5, in the form of
// boost::math::tools::brent_find_minima used at Ellipsoid.cpp:309); tol = 2^(1-min(bits, 26)).
// Returns false when maxIter evaluations did not converge.
__device__ __forceinline__ bool brentMax(const s33& Ai, const s33& Bi, d3 R, double tol, int maxIter, double& L,
                                         double& Fab, int& evals) {
  const double golden = (double)0.3819660f;
  double lo = 0., hi = 1.;
  double x = hi, w = hi, v = hi;
  double fx = pwNegS(Ai, Bi, R, x), fw = fx, fv = fx;
  double step = 0, step2 = 0;
  int n = 1;
  bool ok = false;
  for (; n < maxIter;) {
    const double mid = (lo + hi) / 2;
    const double t1 = tol * fabs(x) + tol / 4;
    const double t2 = 2 * t1;
    if (fabs(x - mid) <= (t2 - (hi - lo) / 2)) { ok = true; break; }
    bool goldenStep = true;
    if (fabs(step2) > t1) {
      double r = (x - w) * (fx - fv);
      double q = (x - v) * (fx - fw);
      double p = (x - v) * q - (x - w) * r;
      q = 2 * (q - r);
      if (q > 0) p = -p;
      q = fabs(q);
      const double prev = step2;
      step2 = step;
      if (!((fabs(p) >= fabs(q * prev / 2)) || (p <= q * (lo - x)) || (p >= q * (hi - x)))) {
        goldenStep = false;
        step = p / q;
        const double u = x + step;
        if (((u - lo) < t2) || ((hi - u) < t2)) step = (mid - x) < 0 ? -fabs(t1) : fabs(t1);
      }
    }
    if (goldenStep) {
      step2 = (x >= mid) ? lo - x : hi - x;
      step = golden * step2;
    }
    const double u = (fabs(step) >= t1) ? x + step : (step > 0 ? x + fabs(t1) : x - fabs(t1));
    const double fu = pwNegS(Ai, Bi, R, u);
    n++;
    if (fu <= fx) {
      if (u >= x) lo = x; else hi = x;
      v = w; w = x; x = u;
      fv = fw; fw = fx; fx = fu;
    } else {
      if (u < x) lo = u; else hi = u;
      if ((fu <= fw) || (w == x)) { v = w; w = u; fv = fw; fw = fu; }
      else if ((fu <= fv) || (v == x) || (v == w)) { v = u; fv = fu; }
    }
  }
  evals += n;
  L = x;
  Fab = -fx;
  return ok;
}

// One Newton-Raphson step on S'(l) = 0 from l, with the bracket [lo, hi] of the root kept from the sign
// of S' (S' decreasing).  S' = (1-2l) h + l(1-l) h', S'' = -2h + 2(1-2l) h' + l(1-l) h'' with
// h = R^T x, h' = -x^T D x, h'' = 2 (D x)^T G^-1 D x, x = G^-1 R, D = B^-1 - A^-1.
__device__ __forceinline__ double newtonStep(const s33& Ai, const s33& Bi, const s33& D, d3 R, double l, double& lo,
                                             double& hi, double tol, bool& conv) {
  const s33 Gi = symInv(symMix(Ai, Bi, l));
  const d3 x = symMul(Gi, R);
  const d3 Dx = symMul(D, x);
  const d3 y = symMul(Gi, Dx);
  const double h = dot(R, x), h1 = -dot(x, Dx), h2 = 2 * dot(Dx, y);
  const double w = l * (1 - l), s = 1 - 2 * l;
  const double S1 = s * h + w * h1;
  const double S2 = -2 * h + 2 * s * h1 + w * h2;
  if (S1 > 0) lo = l; else hi = l;
  const double dl = -S1 / S2;
  // converged: the Newton correction itself is below the tolerance (it may sit on a bracket end)
  if (fabs(dl) <= tol) { conv = true; return l + dl; }
  double ln = l + dl;
  if (!(ln >= lo && ln <= hi)) ln = 0.5 * (lo + hi);  // outside the bracket (or NaN): bisect
  return ln;
}

// Newton-Raphson maximiser of S from l0; returns the number of iterations, or -1 when it did not converge
// within maxIter.  Converged when the correction |dl| <= tol, or when the error left after applying the
// correction, estimated from quadratic convergence as K dl^2 with K = |dl_k| / dl_{k-1}^2, is <= tol
// (only once the corrections shrink and |dl| < 1e-3, i.e. inside the quadratic regime).
__device__ __forceinline__ int newtonMax(const s33& Ai, const s33& Bi, d3 R, double l0, double tol, int maxIter,
                                         double& L) {
  s33 D;
  D.a = Bi.a - Ai.a; D.b = Bi.b - Ai.b; D.c = Bi.c - Ai.c; D.d = Bi.d - Ai.d; D.e = Bi.e - Ai.e; D.f = Bi.f - Ai.f;
  double lo = 0., hi = 1., l = l0, prev = 0.;
  for (int it = 1; it <= maxIter; it++) {
    bool conv = false;
    const double ln = newtonStep(Ai, Bi, D, R, l, lo, hi, tol, conv);
    if (conv) { L = ln; return it; }
    const double dl = fabs(ln - l);
    if (prev > 0. && dl < 1e-3 && dl <= prev && (dl / (prev * prev)) * (dl * dl) <= tol) { L = ln; return it; }
    prev = dl;
    l = ln;
  }
  L = l;
  return -1;
}

__device__ __forceinline__ double maxc(d3 v) { double r = v.x; if (v.y > r) r = v.y; if (v.z > r) r = v.z; return r; }
__device__ __forceinline__ qd qconj(qd q) { q.x = -q.x; q.y = -q.y; q.z = -q.z; return q; }

// Inputs of the learned warm start (13 numbers): the centre offset R in A's frame, the orientation of B
// relative to A (w >= 0), both semi-axis triples; lengths divided by s = max(a) + max(b) so that the
// map is scale-free.  ELL_FEATURES inputs + ELL_TARGETS outputs (lambda, contact point in A's frame / s)
// make one training record.
enum { ELL_FEATURES = 13, ELL_TARGETS = 4, ELL_RECORD = ELL_FEATURES + ELL_TARGETS };
__device__ __forceinline__ void ellFeatures(qd oa, d3 semiA, qd ob, d3 semiB, d3 R, float* f) {
  const double s = maxc(semiA) + maxc(semiB);
  const double is = 1.0 / s;
  const qd ca = qconj(oa);
  const d3 r = qrot(ca, R);
  qd q = qmul(ca, ob);
  if (q.w < 0) { q.w = -q.w; q.x = -q.x; q.y = -q.y; q.z = -q.z; }
  f[0] = (float)(r.x * is); f[1] = (float)(r.y * is); f[2] = (float)(r.z * is);
  f[3] = (float)q.w; f[4] = (float)q.x; f[5] = (float)q.y; f[6] = (float)q.z;
  f[7] = (float)(semiA.x * is); f[8] = (float)(semiA.y * is); f[9] = (float)(semiA.z * is);
  f[10] = (float)(semiB.x * is); f[11] = (float)(semiB.y * is); f[12] = (float)(semiB.z * is);
}

WDEM_VARIANT_END
}  // namespace wdem
