// wdem_peri.cuh -- the periodic pair predicate of InsertionSortCollider (spatialOverlapPeri and
// spatialOverlapPeri_axis, "new algorithm", src/dem/InsertionSortCollider.cpp:897-1044) on the GPU.
// Boxes are in unsheared coordinates and are not wrapped; the result also gives Contact.cellDist, the
// number of cells by which pB is shifted to overlap pA.  Same IEEE operations as the reference.
#pragma once
#include <cuda_runtime.h>
#include "wdem_variant.h"

namespace wdem {
WDEM_VARIANT_BEGIN

// InsertionSortCollider::cellWrapRel (InsertionSortCollider.cpp:624-628)
__device__ __forceinline__ double cellWrapRel(double x, double x0, double x1, int& period) {
  const double xNorm = (x - x0) / (x1 - x0);
  const double f = floor(xNorm);
  period = (int)f;
  return (xNorm - f) * (x1 - x0);
}

// one axis; *ambiguous is set when the boxes overlap on both sides (the reference throws)
__device__ __forceinline__ bool overlapPeriAxis(double min1, double max1, double min2, double max2, double dim,
                                                int& period, bool& ambiguous) {
  if (isinf(min1) || isinf(min2)) { period = 0; return true; }
  int pmn1_2, pmx1_2, pmn2_1, pmx2_1;
  const double mn1_2 = cellWrapRel(min1, min2, min2 + dim, pmn1_2);
  (void)cellWrapRel(max1, min2, min2 + dim, pmx1_2);
  const double mn2_1 = cellWrapRel(min2, min1, min1 + dim, pmn2_1);
  (void)cellWrapRel(max2, min1, min1 + dim, pmx2_1);
  if (pmn1_2 != pmx1_2 && pmn2_1 != pmx2_1) { ambiguous = true; period = 0; return false; }
  if (pmn2_1 == pmx2_1) { period = -pmn2_1; return mn2_1 < (max1 - min1); }
  period = pmn1_2;
  return mn1_2 < (max2 - min2);
}

__device__ __forceinline__ bool overlapPeri(const double4_32a& mn1, const double4_32a& mx1, const double4_32a& mn2,
                                            const double4_32a& mx2, const double* size, int4& per, bool& ambiguous) {
  int p0 = 0, p1 = 0, p2 = 0;
  if (!overlapPeriAxis(mn1.x, mx1.x, mn2.x, mx2.x, size[0], p0, ambiguous)) return false;
  if (!overlapPeriAxis(mn1.y, mx1.y, mn2.y, mx2.y, size[1], p1, ambiguous)) return false;
  if (!overlapPeriAxis(mn1.z, mx1.z, mn2.z, mx2.z, size[2], p2, ambiguous)) return false;
  per = make_int4(p0, p1, p2, 0);
  return true;
}

// FP32 screens of spatialOverlapPeri on wrapped box centres and half-widths.
// minimum-image centre distance on one axis (the image choice can differ from the exact one only where
// both images are about L/2 away, beyond any half-width sum below L/2)
__device__ __forceinline__ float periDist(float c1, float c2, float L, float invL) {
  const float d = c2 - c1;
  return fabsf(d - L * rintf(d * invL));
}
// the boxes are disjoint on this axis for every period shift: the rounding of the FP32 copies (centres
// wrapped to [0, L), half-widths) and of this arithmetic is a few 2^-24 L, the margin 1e-5 L
__device__ __forceinline__ bool periFar(float c1, float h1, float c2, float h2, float L, float invL) {
  return periDist(c1, c2, L, invL) > h1 + h2 + 1e-5f * L;
}
// ... or overlapping on this axis for the nearest image, by more than the same margin
__device__ __forceinline__ bool periNear(float c1, float h1, float c2, float h2, float L, float invL) {
  return periDist(c1, c2, L, invL) < h1 + h2 - 1e-5f * L;
}

WDEM_VARIANT_END
}  // namespace wdem
