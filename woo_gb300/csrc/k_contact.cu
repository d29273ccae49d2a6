// k_contact.cu -- fused contact kernel: the GB300 replacement of one pass of Woo's ContactLoop
// (src/dem/ContactLoop.cpp:93-268) with the functors
//   Cg2_Sphere_Sphere_L6Geom (src/dem/Sphere.cpp:92-117), Cg2_Wall_Sphere_L6Geom (src/dem/Wall.cpp:50-84),
//   Cg2_Any_Any_L6Geom__Base::handleSpheresLikeContact (src/dem/L6Geom.cpp:49-216),
//   Cp2_FrictMat_FrictPhys (src/dem/FrictMat.cpp:20-44), Cp2_HertzMat_HertzPhys (src/dem/Hertz.cpp:34-77),
//   Law2_L6Geom_FrictPhys_IdealElPl (src/dem/IdealElPl.cpp:15-125),
//   Law2_L6Geom_HertzPhys_DMT, DMT branch (src/dem/Hertz.cpp:85-114,170-210),
// and the force/torque branch of Contact::getForceTorqueBranch (src/dem/Contact.cpp:24-34).
//
// One thread per contact, contacts in SoA so every history load/store is coalesced.  Particle
// state is gathered as 32-byte double4_32a records (position+radius, velocity+mass, angular velocity).
// Instead of adding into particles under a mutex (DemData::addForceTorque, Particle.hpp:249) each
// real contact writes its global force and the torques on both particles; the integrator sums them
// per particle through the CSR in a fixed order.
#include <algorithm>

#include "wdem_internal.h"
#include "wdem_variant.h"
#include "wdem_math.cuh"
#include "wdem_peri.cuh"
#include "wdem_ell.cuh"
#include "wdem_dw.cuh"
#include "../../include/wdem.h"

namespace wdem {
WDEM_VARIANT_BEGIN

__constant__ DevMaterial c_mats[MAX_MATERIALS];

void upload_materials(const DevMaterial* m, int n) {
  cudaMemcpyToSymbol(c_mats, m, sizeof(DevMaterial) * (n < MAX_MATERIALS ? n : MAX_MATERIALS));
}

__device__ __forceinline__ bool overlapBoxes(const double4_32a& mn1, const double4_32a& mx1, const double4_32a& mn2, const double4_32a& mx2) {
  return (mn1.x <= mx2.x) && (mx1.x >= mn2.x) && (mn1.y <= mx2.y) && (mx1.y >= mn2.y) && (mn1.z <= mx2.z) && (mx1.z >= mn2.z);
}

__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }   // std::min
__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }   // std::max

// Physical constants of a new (or updated) contact, Cp2_*.  Writes tanPhi and, for FrictPhys,
// kn/kt; for HertzPhys the constants kn0, kt0, alpha_sqrtMK, Fna used by the DMT law each step.
template <int CP2>
__device__ __forceinline__ void cp2(const StepParams& P, int matA, int matB, double r1, double r2, double massA,
                                    double massB, double& kn, double& kt, double& tanPhi, double* hz) {
  const DevMaterial m1 = c_mats[matA];
  const DevMaterial m2 = c_mats[matB];
  // L6Geom.lens and contA with iniLensTouch (L6Geom.cpp:61-68)
  double l0 = fabs(r1), l1 = fabs(r2);
  if (CP2 == WDEM_CP2_FRICT) {
    const double rr = (r1 > 0 && r2 > 0) ? dmin(r1, r2) : (r1 > 0 ? r1 : r2);
    const double A = M_PI * (rr * rr);
    kn = 1 / (1 / (m1.young * A / l0) + 1 / (m2.young * A / l1));
    kt = .5 * (m1.ktDivKn + m2.ktDivKn) * kn;
    tanPhi = dmin(m1.tanPhi, m2.tanPhi);
  } else {
    const double nu1 = P.poisson, nu2 = P.poisson;
    double K = (4 / 3.) * 1. / ((1 - nu1 * nu1) / m1.young + (1 - nu2 * nu2) / m2.young);
    double R = 1. / (1. / l0 + 1. / l1);
    double kn0 = K * sqrt(R);
    double gamma = dmin(m1.surfEnergy, m2.surfEnergy);
    double G1 = m1.young / (2 * (1 + nu1)), G2 = m2.young / (2 * (1 + nu2));
    double G = .5 * (G1 + G2);
    double nu = .5 * (nu1 + nu2);
    double kt0 = 2 * sqrt(4 * R) * G / (2 - nu);
    tanPhi = dmin(m1.tanPhi, m2.tanPhi);
    double aSMK = 0.0;
    if (P.en > 0 && P.en < 1.) {
      double mbar = (massA <= 0 && massB > 0) ? massB : ((massA > 0 && massB <= 0) ? massA : (massA * massB) / (massA + massB));
      aSMK = dmax(0., P.viscAlpha * sqrt(mbar * kn0));
    }
    hz[0] = kn0;
    hz[1] = kt0;
    hz[2] = aSMK;
    hz[3] = 4 * M_PI * R * gamma;  // DMT adhesion force, constant per contact
  }
}

// warp-aggregated add of per-thread counters (one atomic per warp)
__device__ __forceinline__ void warpAdd(unsigned long long* dst, unsigned v) {
  const unsigned mask = __activemask();
  unsigned long long sum = v;
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(mask, sum, o);
  if ((threadIdx.x & 31) == (__ffs(mask) - 1) && sum) atomicAdd(dst, sum);
}

// Perram-Wertheim geometry of an ellipsoid (or sphere + ellipsoid) pair, Cg2_Ellipsoid_Ellipsoid_L6Geom::
// go_Ellipsoid_or_Sphere (Ellipsoid.cpp:270-351).  Returns false when the pair does not touch
// (F_ab > 1) and the contact is not real.
__device__ __noinline__ bool ellPairGeometry(const StepParams& P, const Particles& p, const Contacts& c, long long i,
                                             int a, int b, bool real, d3 pos1, d3 pos2, d3& normal, d3& contPt,
                                             double& uN, double& r1, double& r2, DeviceStatus* st) {
  const double4_32a SA = p.semi[a], SB = p.semi[b], OA = p.ori[a], OB = p.ori[b];
  qd oa, ob;
  oa.w = OA.x; oa.x = OA.y; oa.y = OA.z; oa.z = OA.w;
  ob.w = OB.x; ob.x = OB.y; ob.y = OB.z; ob.z = OB.w;
  const d3 semiA = xyz(SA), semiB = xyz(SB);
  const d3 R = pos2 - pos1;
  const s33 Ai = symInv(shapeMatrix(oa, semiA));
  const s33 Bi = symInv(shapeMatrix(ob, semiB));
  double L, Fab;
  unsigned iters = 0, fallback = 0;
  if (P.ellSolver == WDEM_ELL_BRENT) {
    int ev = 0;
    if (!brentMax(Ai, Bi, R, P.brentTol, 1000, L, Fab, ev)) {
      if (atomicCAS(&st->code, 0, WDEM_ERR_TIMEOUT) == 0) st->detail = a;
      return false;
    }
    iters = (unsigned)ev;
  } else {
    const double cold = maxc(semiA) / (maxc(semiA) + maxc(semiB));
    double l0 = cold;
    int budget = 60;
    const double lh = c.lam ? c.lam[i] : -1.0;
    const bool hist = lh > 0 && lh < 1;
    if ((P.warmStart == WDEM_WARM_HISTORY || P.warmStart == WDEM_WARM_HISTORY_MLP) && hist) {
      l0 = lh;
    } else if ((P.warmStart == WDEM_WARM_MLP || P.warmStart == WDEM_WARM_HISTORY_MLP) && c.lam0) {
      // the learned guess (for WDEM_WARM_HISTORY_MLP only where the pair has no previous maximiser),
      // judged by the plain solve: cold start after fallbackIters iterations without convergence
      const double lm = (double)c.lam0[i];
      if (lm > 0 && lm < 1) { l0 = lm; budget = P.fallbackIters; }
    }
    int it = newtonMax(Ai, Bi, R, l0, P.newtonTol, budget, L);
    if (it < 0 && budget < 60) {
      // the warm start did not converge within k iterations: plain cold-start Newton
      fallback = 1;
      iters += (unsigned)budget;
      it = newtonMax(Ai, Bi, R, cold, P.newtonTol, 60, L);
    }
    if (it < 0) {
      if (atomicCAS(&st->code, 0, WDEM_ERR_TIMEOUT) == 0) st->detail = a;
      return false;
    }
    iters += (unsigned)it;
    Fab = -pwNegS(Ai, Bi, R, L);
  }
  warpAdd(&st->ellSolves, 1u);
  warpAdd(&st->ellIters, iters);
  if (fallback) warpAdd(&st->ellFallbacks, fallback);
  if (c.lam) c.lam[i] = L;
  const bool touch = !(Fab > 1);
  if (!touch && !real) {
    if (P.ellLog) {
      const unsigned long long k = atomicAdd(P.ellLogCount, 1ull);
      if (k < (unsigned long long)P.ellLogCap) {
        float* rec = P.ellLog + k * ELL_RECORD;
        ellFeatures(oa, semiA, ob, semiB, R, rec);
        // contact point of the scaled ellipsoids, as in the touching case
        const s33 Gi = symInv(symMix(Ai, Bi, L));
        const d3 n = symMul(Gi, R);
        const double w = 1 - L;
        const d3 v = mk((w * Ai.a) * n.x + (w * Ai.b) * n.y + (w * Ai.c) * n.z,
                        (w * Ai.b) * n.x + (w * Ai.d) * n.y + (w * Ai.e) * n.z,
                        (w * Ai.c) * n.x + (w * Ai.e) * n.y + (w * Ai.f) * n.z);
        const d3 vl = qrot(qconj(oa), v);
        const double is = 1.0 / (maxc(semiA) + maxc(semiB));
        rec[13] = (float)L; rec[14] = (float)(vl.x * is); rec[15] = (float)(vl.y * is); rec[16] = (float)(vl.z * is);
      }
    }
    return false;
  }
  const s33 Gi = symInv(symMix(Ai, Bi, L));
  const d3 nUnnorm = symMul(Gi, R);
  const double w = 1 - L;
  const d3 v = mk((w * Ai.a) * nUnnorm.x + (w * Ai.b) * nUnnorm.y + (w * Ai.c) * nUnnorm.z,
                  (w * Ai.b) * nUnnorm.x + (w * Ai.d) * nUnnorm.y + (w * Ai.e) * nUnnorm.z,
                  (w * Ai.c) * nUnnorm.x + (w * Ai.e) * nUnnorm.y + (w * Ai.f) * nUnnorm.z);
  contPt = pos1 + v;
  const double mu = sqrt(Fab);
  const double Rnorm = sqrt(sqnorm(R));
  const d3 nUnit = normalized(nUnnorm);
  const d3 rUnit = R / Rnorm;
  uN = Rnorm * (1 - 1 / mu) * dot(rUnit, nUnit);
  normal = nUnit;
  r1 = sqrt(sqnorm(contPt - pos1));
  r2 = sqrt(sqnorm(contPt - pos2));
  if (P.ellLog) {
    const unsigned long long k = atomicAdd(P.ellLogCount, 1ull);
    if (k < (unsigned long long)P.ellLogCap) {
      float* rec = P.ellLog + k * ELL_RECORD;
      ellFeatures(oa, semiA, ob, semiB, R, rec);
      const d3 vl = qrot(qconj(oa), v);
      const double is = 1.0 / (maxc(semiA) + maxc(semiB));
      rec[13] = (float)L; rec[14] = (float)(vl.x * is); rec[15] = (float)(vl.y * is); rec[16] = (float)(vl.z * is);
    }
  }
  return true;
}

// Cg2_Wall_Ellipsoid_L6Geom::go (Ellipsoid.cpp:227-257); pA is the wall
__device__ __forceinline__ bool wallEllGeometry(const Particles& p, int a, int b, bool real, d3 pos1, d3 pos2,
                                                d3& normal, d3& contPt, double& uN, double& r1, double& r2) {
  const int wa = p.meta[a].x;
  const int ax = (wa >> 4) & 3, sense = ((wa >> 8) & 3) - 1;
  const double4_32a SB = p.semi[b], OB = p.ori[b];
  qd ob;
  ob.w = OB.x; ob.x = OB.y; ob.y = OB.z; ob.z = OB.w;
  const d3 c0 = qrot(ob, mk(SB.x, 0, 0)), c1 = qrot(ob, mk(0, SB.y, 0)), c2 = qrot(ob, mk(0, 0, SB.z));
  const double m0 = comp(c0, ax), m1 = comp(c1, ax), m2 = comp(c2, ax);
  const double extent = sqrt(m0 * m0 + m1 * m1 + m2 * m2);
  const double wp = comp(pos1, ax), ep = comp(pos2, ax);
  if (((wp < (ep - extent)) || (wp > (ep + extent))) && !real) return false;
  const double dist = ep - wp;
  const int sgn = (sense == 0) ? (dist > 0 ? 1 : -1) : (sense == 1 ? 1 : -1);
  const double ds = (double)sgn;
  normal = mk(ds * (ax == 0 ? 1. : 0.), ds * (ax == 1 ? 1. : 0.), ds * (ax == 2 ? 1. : 0.));
  uN = sgn * dist - extent;
  const d3 mp = normalized(mk(m0, m1, m2));
  const d3 col = mk(c0.x * mp.x + c1.x * mp.y + c2.x * mp.z, c0.y * mp.x + c1.y * mp.y + c2.y * mp.z,
                    c0.z * mp.x + c1.z * mp.y + c2.z * mp.z);
  contPt = pos2 + (double)(-sgn) * col;
  setComp(contPt, ax, wp);
  const double contR = sqrt(sqnorm(contPt - pos2));
  r1 = -contR;
  r2 = contR;
  return true;
}

// CompUtils::closestSegmentPt (CompUtils.cpp:59-65)
__device__ __forceinline__ d3 closestSegmentPt(d3 P, d3 A, d3 B) {
  const d3 BA = B - A;
  const double bb = sqnorm(BA);
  if (bb == 0.) return A;
  const double u = (dot(P, BA) - dot(A, BA)) / bb;
  const double lo = (0. < u) ? u : 0.;        // std::max(0., u)
  const double t = (lo < 1.) ? lo : 1.;       // std::min(1., .)
  return A + t * BA;
}

// Cg2_Facet_Sphere_L6Geom::go (Facet.cpp:333-390) for facets without neighbour angles (Facet.n21lim NaN: no
// boundary adjustment) and without fakeVel.  pA is the facet: node 0 at n0, nodes 1 and 2 in fv1/fv2,
// half-thickness ht; pB the sphere at sC.  The projected centre is classified against the outer vectors of
// the three edges (Facet::getOuterVectors, Facet.cpp:113-117) and snapped to the triangle, an edge or a node.
__device__ __forceinline__ bool facetSphereGeometry(const Particles& p, const Contacts& c, long long i, int a, bool real,
                                                    d3 n0, double ht, d3 sC, double r, d3& normal, d3& contPt,
                                                    double& uN, double& r1, double& r2, DeviceStatus* st) {
  const d3 n1 = xyz(p.fv1[a]), n2 = xyz(p.fv2[a]);
  const d3 nn = cross(n1 - n0, n2 - n0);
  const d3 fNormal = normalized(nn);
  const double planeDist = dot(sC - n0, fNormal);
  const double rh = r + ht;
  if (fabs(planeDist) > rh && !real) return false;
  const d3 fC = sC - planeDist * fNormal;
  const double l0 = dot(cross(n1 - n0, nn), fC - n0);
  const double l1 = dot(cross(n2 - n1, nn), fC - n1);
  const double l2 = dot(cross(n0 - n2, nn), fC - n2);
  const int w = (l0 > 0 ? 1 : 0) + (l1 > 0 ? 2 : 0) + (l2 > 0 ? 4 : 0);
  switch (w) {
    case 0: contPt = fC; break;
    case 1: contPt = closestSegmentPt(fC, n0, n1); break;
    case 2: contPt = closestSegmentPt(fC, n1, n2); break;
    case 4: contPt = closestSegmentPt(fC, n2, n0); break;
    case 3: contPt = n1; break;
    case 5: contPt = n0; break;
    case 6: contPt = n2; break;
    default:
      // outside all three edges: the reference throws logic_error
      if (atomicCAS(&st->code, 0, WDEM_ERR_UNSUPPORTED) == 0) st->detail = a;
      return false;
  }
  normal = sC - contPt;
  if (sqnorm(normal) > rh * rh && !real) return false;
  const double dist = sqrt(sqnorm(normal));
  if (dist != 0) normal = normal / dist;
  else if (real) {
    // the sphere's centre on the facet: the previous normal, L6Geom.node.ori * UnitX
    const d3 c0 = mk(c.hist[HIST_T0X][i], c.hist[HIST_T0Y][i], c.hist[HIST_T0Z][i]);
    const d3 c1 = mk(c.hist[HIST_T1X][i], c.hist[HIST_T1Y][i], c.hist[HIST_T1Z][i]);
    normal = qrot(quatFromCols(c0, c1, cross(c0, c1)), mk(1, 0, 0));
  } else normal = mk(1, 0, 0);
  if (ht > 0) contPt = contPt + normal * ht;
  uN = dist - r - ht;
  r1 = (ht < r) ? r : ht;  // std::max(halfThick, radius)
  r2 = r;
  return true;
}

// Facet::interpolatePtLinAngVel (Facet.cpp:161-179) at x without fakeVel: barycentric weights of x
// (CompUtils::triangleBarycentrics, CompUtils.cpp:94-112: the 2x2 system solved by Eigen's closed-form
// inverse) applied to the node velocities; node 0 moves with the particle, nodes 1 and 2 are at rest
__device__ __forceinline__ void facetPointVel(const Particles& p, int a, d3 n0, d3 x, d3& vel, d3& angVel) {
  const d3 n1 = xyz(p.fv1[a]), n2 = xyz(p.fv2[a]);
  const d3 vB = n1 - n0, vC = n2 - n0, vX = x - n0;
  const double m00 = dot(vB, vB), m01 = dot(vC, vB), m10 = dot(vB, vC), m11 = dot(vC, vC);
  const double invdet = 1. / (m00 * m11 - m10 * m01);
  const double i00 = m11 * invdet, i10 = -m10 * invdet, i01 = -m01 * invdet, i11 = m00 * invdet;
  const double b0 = dot(vX, vB), b1 = dot(vX, vC);
  const double u = i00 * b0 + i01 * b1, v = i10 * b0 + i11 * b1;
  const double a0 = 1 - u - v;
  const d3 v0 = vel, z = mk(0, 0, 0);
  vel = a0 * v0 + u * z + v * z;
  angVel = cross(n0 - x, v0) + cross(n1 - x, z) + cross(n2 - x, z);
}

// ------------------------------------------------------------------------------------ capsules
// Capsules keep (radius, shaft, 0) in Particles.semi and their bounding radius radius + shaft/2 in posr.w.
__device__ __forceinline__ qd oriOf(const Particles& p, int i) {
  const double4_32a o = p.ori[i];
  qd q;
  q.w = o.x; q.x = o.y; q.y = o.z; q.z = o.w;
  return q;
}

// Cg2_Sphere_Capsule_L6Geom::go (Capsule.cpp:198-216); pA is the sphere, pB the capsule
__device__ __noinline__ bool sphereCapsuleGeometry(const Particles& p, int a, int b, bool real, d3 spherePos, d3 capPos,
                                                   d3& normal, d3& contPt, double& uN, double& r1, double& r2) {
  const double rs = p.posr[a].w;
  const double4_32a cs = p.semi[b];
  const double rc = cs.x;
  const double rSum = rs + rc;
  const d3 half = qrot(oriOf(p, b), mk(cs.y / 2., 0, 0));
  const d3 pt = closestSegmentPt(spherePos, capPos - half, capPos + half);
  const double distSq = sqnorm(pt - spherePos);
  if (!real && distSq > rSum * rSum) return false;
  const double dist = sqrt(distSq);
  normal = (pt - spherePos) / dist;
  uN = dist - rSum;
  contPt = spherePos + normal * (rs + .5 * uN);
  r1 = rs;
  r2 = rc;
  return true;
}

// Cg2_Wall_Capsule_L6Geom::go (Capsule.cpp:116-164); pA is the wall.  The overlaps of the two end caps with
// the wall weight the contact point and give uN.
__device__ __noinline__ bool wallCapsuleGeometry(const Particles& p, const Contacts& c, long long i, int a, int b,
                                                 bool real, d3 wallPos, d3 capPos, d3& normal, d3& contPt,
                                                 double& uN, double& r1, double& r2) {
  const int wa = p.meta[a].x;
  const int ax = (wa >> 4) & 3, sense = ((wa >> 8) & 3) - 1;
  const double4_32a cs = p.semi[b];
  const double rc = cs.x;
  const d3 half = qrot(oriOf(p, b), mk(cs.y / 2., 0, 0));
  const d3 A = capPos - half, B = capPos + half;
  const double wp = comp(wallPos, ax);
  const double d0 = comp(A, ax) - wp, d1 = comp(B, ax) - wp;
  if (!real && (fabs(d0) > rc && fabs(d1) > rc)) return false;
  const double cDist = comp(capPos, ax) - wp;
  double nax;
  if (sense == 0) nax = real ? comp(mk(c.hist[HIST_T0X][i], c.hist[HIST_T0Y][i], c.hist[HIST_T0Z][i]), ax) : (cDist > 0 ? 1. : -1.);
  else nax = (sense == 1 ? 1. : -1);
  normal = mk(0, 0, 0);
  setComp(normal, ax, nax);
  const double u0 = d0 * nax - rc, u1 = d1 * nax - rc;
  if (u0 * u1 < 0) {
    // the ends on opposite sides of the wall: the overlapping one takes all
    contPt = u0 < 0 ? A : B;
    uN = u0 < 0 ? u0 : u1;
  } else if (u0 + u1 != 0.) {
    const double sum = u0 + u1;
    double w0 = u0 / sum, w1 = u1 / sum;
    if (u0 > 0) { const double t = w0; w0 = w1; w1 = t; }  // no overlap: the end closer to the wall weighs more
    contPt = w0 * A + w1 * B;
    uN = w0 * u0 + w1 * u1;
  } else {
    contPt = .5 * (A + B);
    uN = 0.;
  }
  setComp(contPt, ax, wp);
  r1 = -rc;
  r2 = rc;
  return true;
}

// CompUtils::distSq_SegmentSegment (CompUtils.cpp:260-592): D. Eberly's segment distance ("Distance Between
// Two Line Segments in 3D", Geometric Tools) as the reference has it -- the minimum of the quadratic in the
// segment parameters (s0, s1) classified into the nine regions of the parameter rectangle; on a side one
// parameter sits at its bound and the other is minimised and clamped, a corner tries one side and, when the
// clamp ends on the far bound, the other; nearly parallel segments take the symmetric average.  The
// comparisons and the additions of the distance formulas keep the reference's order in every region.
struct SegSeg {
  double a01, b0, b1, c, e0, e1;
  // s1 = f, s0 the clamped minimiser t = -(a01 f + b0); lowFirst: tested t < -e0, t <= e0, else, otherwise
  // t > e0, t >= -e0, else; far: the last branch was taken
  __device__ __forceinline__ double withS1(double f, bool lowFirst, double& s0, double& s1, bool& far) const {
    s1 = f;
    const double t = -(a01 * s1 + b0);
    bool inner = false;
    far = false;
    if (lowFirst) {
      if (t < -e0) s0 = -e0;
      else if (t <= e0) { s0 = t; inner = true; }
      else { s0 = e0; far = true; }
    } else {
      if (t > e0) s0 = e0;
      else if (t >= -e0) { s0 = t; inner = true; }
      else { s0 = -e0; far = true; }
    }
    const double x = inner ? -s0 * s0 : s0 * (s0 - 2. * t);
    return x + s1 * (s1 + 2. * b1) + c;
  }
  // s0 = f, s1 the clamped minimiser t = -(a01 f + b1)
  __device__ __forceinline__ double withS0(double f, bool lowFirst, double& s0, double& s1) const {
    s0 = f;
    const double t = -(a01 * s0 + b1);
    bool inner = false;
    if (lowFirst) {
      if (t < -e1) s1 = -e1;
      else if (t <= e1) { s1 = t; inner = true; }
      else s1 = e1;
    } else {
      if (t > e1) s1 = e1;
      else if (t >= -e1) { s1 = t; inner = true; }
      else s1 = -e1;
    }
    const double x = inner ? -s1 * s1 : s1 * (s1 - 2. * t);
    return x + s0 * (s0 + 2. * b0) + c;
  }
};
__device__ __forceinline__ double distSqSegSeg(d3 c0, d3 d0, double e0, d3 c1, d3 d1, double e1, double& s0, double& s1) {
  const d3 diff = c0 - c1;
  SegSeg g;
  g.a01 = -dot(d0, d1);
  g.b0 = dot(diff, d0);
  g.b1 = -dot(diff, d1);
  g.c = sqnorm(diff);
  g.e0 = e0;
  g.e1 = e1;
  const double a01 = g.a01, b0 = g.b0, b1 = g.b1, c = g.c;
  const double det = fabs(1. - a01 * a01);
  double d;
  bool far;
  if (det >= 1e-8) {
    s0 = a01 * b1 - b0;
    s1 = a01 * b0 - b1;
    const double ed0 = e0 * det, ed1 = e1 * det;
    if (s0 >= -ed0) {
      if (s0 <= ed0) {
        if (s1 >= -ed1) {
          if (s1 <= ed1) {  // interior
            const double inv = 1. / det;
            s0 *= inv;
            s1 *= inv;
            d = s0 * (s0 + a01 * s1 + 2. * b0) + s1 * (a01 * s0 + s1 + 2. * b1) + c;
          } else d = g.withS1(e1, true, s0, s1, far);
        } else d = g.withS1(-e1, true, s0, s1, far);
      } else {
        if (s1 >= -ed1) {
          if (s1 <= ed1) d = g.withS0(e0, true, s0, s1);
          else {
            d = g.withS1(e1, true, s0, s1, far);
            if (far) d = g.withS0(e0, true, s0, s1);
          }
        } else {
          d = g.withS1(-e1, true, s0, s1, far);
          if (far) d = g.withS0(e0, false, s0, s1);
        }
      }
    } else {
      if (s1 >= -ed1) {
        if (s1 <= ed1) d = g.withS0(-e0, true, s0, s1);
        else {
          d = g.withS1(e1, false, s0, s1, far);
          if (far) d = g.withS0(-e0, true, s0, s1);
        }
      } else {
        d = g.withS1(-e1, false, s0, s1, far);
        if (far) d = g.withS0(-e0, true, s0, s1);
      }
    }
  } else {
    // parallel: the averaged b0 makes the distance symmetric in the two segments
    const double e0pe1 = e0 + e1;
    const double sign = (a01 > 0. ? -1. : 1.);
    const double b0Avr = .5 * (b0 - sign * b1);
    double lambda = -b0Avr;
    if (lambda < -e0pe1) lambda = -e0pe1;
    else if (lambda > e0pe1) lambda = e0pe1;
    s1 = -sign * lambda * e1 / e0pe1;
    s0 = lambda + sign * s1;
    d = lambda * (lambda + 2. * b0Avr) + c;
  }
  if (d < 0.) d = 0.;
  return d;
}

// Cg2_Capsule_Capsule_L6Geom::go (Capsule.cpp:223-323): uN and the normal from the closest points of the axis
// segments; the contact point from those unless two or more end caps overlap the other capsule's axis, in
// which case the overlapping ends' points (moved from their closest point on the other axis towards the end
// by the other radius' share of rSum) are averaged with weights rSum - distance
__device__ __noinline__ bool capsuleCapsuleGeometry(const Particles& p, int a, int b, bool real, d3 pos1, d3 pos2,
                                                    d3& normal, d3& contPt, double& uN, double& r1, double& r2) {
  const double4_32a c1 = p.semi[a], c2 = p.semi[b];
  const d3 dir1 = qrot(oriOf(p, a), mk(1, 0, 0)), dir2 = qrot(oriOf(p, b), mk(1, 0, 0));
  const double rSum = c1.x + c2.x;
  double u, v;
  const double distSq = distSqSegSeg(pos1, dir1, .5 * c1.y, pos2, dir2, .5 * c2.y, u, v);
  if (!real && distSq > rSum * rSum) return false;
  const d3 close0 = pos1 + dir1 * u, close1 = pos2 + dir2 * v;
  const d3 h1 = .5 * c1.y * dir1, h2 = .5 * c2.y * dir2;
  const d3 ends[2][2] = {{pos1 - h1, pos1 + h1}, {pos2 - h2, pos2 + h2}};
  const double dist = sqrt(distSq);
  uN = dist - (c1.x + c2.x);
  normal = (close1 - close0) / dist;
  int bits = 0, nOver = 0;
  d3 eClose[2][2];
  double eDistSq[2][2];
  for (int s = 0; s < 2; s++) {
    const int t = 1 - s;
    for (int e = 0; e < 2; e++) {
      eClose[s][e] = closestSegmentPt(ends[s][e], ends[t][0], ends[t][1]);
      eDistSq[s][e] = sqnorm(eClose[s][e] - ends[s][e]);
      if (eDistSq[s][e] < rSum * rSum) { bits |= 1 << (2 * s + e); nOver++; }
    }
  }
  const double r1r = c1.x / rSum, r2r = c2.x / rSum;
  if (nOver < 2) contPt = close0 + (c1.x + 0.5 * uN) * normal;
  else if (nOver == 4) {
    d3 pp = mk(0, 0, 0);
    double ww = 0.;
    for (int s = 0; s < 2; s++)
      for (int e = 0; e < 2; e++) {
        const double w = rSum - sqrt(eDistSq[s][e]);
        pp = pp + w * (eClose[s][e] + (ends[s][e] - eClose[s][e]) * (s == 0 ? r2r : r1r));
        ww += w;
      }
    contPt = pp / ww;
  } else {
    // two or three overlapping ends (bit 2s+e for end e of capsule s): the two that place the contact; with
    // three, the two ends of the capsule whose both ends overlap (the reference's lookup table)
    int q0s = 0, q0e = 0, q1s = 0, q1e = 0;
    switch (bits) {
      case 3: case 7: case 11: q1e = 1; break;           // ends of capsule 0
      case 5: q1s = 1; break;                             // (0,0), (1,0)
      case 6: q0e = 1; q1s = 1; break;                    // (0,1), (1,0)
      case 9: q1s = 1; q1e = 1; break;                    // (0,0), (1,1)
      case 10: q0e = 1; q1s = 1; q1e = 1; break;          // (0,1), (1,1)
      case 12: case 13: case 14: q0s = 1; q1s = 1; q1e = 1; break;  // ends of capsule 1
      default: break;
    }
    const d3 p0 = eClose[q0s][q0e] + (ends[q0s][q0e] - eClose[q0s][q0e]) * (q0s == 0 ? r2r : r1r);
    const d3 p1 = eClose[q1s][q1e] + (ends[q1s][q1e] - eClose[q1s][q1e]) * (q1s == 0 ? r2r : r1r);
    const double w0 = rSum - sqrt(eDistSq[q0s][q0e]), w1 = rSum - sqrt(eDistSq[q1s][q1e]);
    contPt = (w0 * p0 + w1 * p1) / (w0 + w1);
  }
  r1 = c1.x;
  r2 = c2.x;
  return true;
}

// One contact of the work list: geometry, physics and law (ContactLoop.cpp:134-197).  PENDING
// contacts have been resolved and potential pairs that cannot touch culled by k_contacts_cull.
template <int LAW, int CP2, bool PERI, bool ELL>
__device__ __forceinline__ void contactBody(const StepParams& P, const Particles& p, const Contacts& c, long long i,
                                            DeviceStatus* st) {
  const uint8_t s0 = c.state[i];
  const uint8_t sb = s0 & CS_SHAPES;
  const uint8_t s = s0 & CS_MASK;
  const int2 id = c.ids[i];
  const int a = id.x, b = id.y;
  // batched scenes: the scene's dt (the material of pA belongs to its scene; walls too)
  const double dtC = P.matDt ? P.matDt[p.meta[a].y] : P.dt;
  const bool real = (s == CS_REAL);
  // periodic: pB is taken at its image hSize*cellDist (ContactLoop.cpp:156, Cell::intrShiftPos)
  int4 cd = make_int4(0, 0, 0, 0);
  if (PERI) cd = c.cdist[i];
  const double4_32a A4 = p.posr[a], B4 = p.posr[b];
  d3 pos1 = xyz(A4);
  d3 shift2 = mk(0, 0, 0);
  if (PERI) shift2 = mvec(P.hS, mk((double)cd.x, (double)cd.y, (double)cd.z));
  const d3 pos2 = PERI ? xyz(B4) + shift2 : xyz(B4);
  double r1, r2, uN;
  d3 normal, contPt;
  if (ELL && (sb & CS_ELL)) {
    // aspherical shapes: ellipsoids and capsules (pB is the capsule of a sphere or wall pair)
    if ((p.meta[b].x & 15) == WDEM_SHAPE_CAPSULE) {
      if (sb & CS_WALL_A) {
        if (!wallCapsuleGeometry(p, c, i, a, b, real, pos1, pos2, normal, contPt, uN, r1, r2)) return;
      } else if ((p.meta[a].x & 15) == WDEM_SHAPE_SPHERE) {
        if (!sphereCapsuleGeometry(p, a, b, real, pos1, pos2, normal, contPt, uN, r1, r2)) return;
      } else if (!capsuleCapsuleGeometry(p, a, b, real, pos1, pos2, normal, contPt, uN, r1, r2)) return;
    } else if (sb & CS_WALL_A) {
      if (!wallEllGeometry(p, a, b, real, pos1, pos2, normal, contPt, uN, r1, r2)) return;
    } else if (!ellPairGeometry(P, p, c, i, a, b, real, pos1, pos2, normal, contPt, uN, r1, r2, st)) return;
  } else if (!PERI && (sb & CS_FACET)) {  // facets are aperiodic only
    if (!facetSphereGeometry(p, c, i, a, real, pos1, A4.w, pos2, B4.w, normal, contPt, uN, r1, r2, st)) return;
  } else if (!(sb & CS_WALL_A)) {
    // Cg2_Sphere_Sphere_L6Geom::go
    r1 = A4.w; r2 = B4.w;
    d3 relPos = pos2 - pos1;
    double t = fabs(P.distFactor) * (r1 + r2);
    const double relSq = sqnormExact(relPos);
    double unDistSq = __dsub_rn(relSq, __dmul_rn(t, t));
    if (positiveBits(unDistSq) && !real) return;
    double dist = sqrt(relSq);
    uN = dist - (r1 + r2);
    normal = relPos / dist;
    contPt = pos1 + (r1 + 0.5 * uN) * normal;
  } else {
    // Cg2_Wall_Sphere_L6Geom::go (pA is the wall)
    const int wa = p.meta[a].x;
    const int ax = (wa >> 4) & 3, sense = ((wa >> 8) & 3) - 1;
    const double radius = B4.w;
    double dist = comp(pos2, ax) - comp(pos1, ax);
    if (!real && fabs(dist) > radius) return;
    contPt = pos2;
    setComp(contPt, ax, comp(pos1, ax));
    normal = mk(0, 0, 0);
    double nax;
    if (sense == 0) {
      if (!real) nax = dist > 0 ? 1. : -1.;
      else {
        d3 prev0 = mk(c.hist[HIST_T0X][i], c.hist[HIST_T0Y][i], c.hist[HIST_T0Z][i]);
        nax = comp(prev0, ax);
      }
    } else nax = (sense == 1 ? 1. : -1);
    setComp(normal, ax, nax);
    uN = nax * dist - radius;
    r1 = -radius; r2 = radius;
  }
  // materials are needed only when Cp2 runs
  int matA = 0, matB = 0;
  if (!real || P.updatePhysNow) { matA = p.meta[a].y; matB = p.meta[b].y; }

  double fx, fy, fz, kn, kt, tanPhi;
  double hz[4] = {0, 0, 0, 0};
  d3 cur0, cur1, gvel, gangVel;
  const double4_32a V1 = p.velm[a], V2 = p.velm[b];
  const double4_32a W1 = p.angw[a], W2 = p.angw[b];
  d3 vel1 = xyz(V1), angVel1 = xyz(W1);
  const d3 vel2 = xyz(V2), angVel2 = xyz(W2);
  if (!PERI && (sb & CS_FACET)) {
    // handleSpheresLikeContact gets the facet as a point at contPt moving with the interpolated velocities
    facetPointVel(p, a, pos1, contPt, vel1, angVel1);
    pos1 = contPt;
  }
  if (!real) {
    // new L6Geom: setInitialLocalCoords (L6Geom.cpp:25-36), node.pos = contPt
    d3 locX = normal;
    d3 e = fabs(locX.y) < fabs(locX.z) ? mk(0, 1, 0) : mk(0, 0, 1);
    d3 locY = cross(locX, e);
    locY = locY - locX * dot(locY, locX);
    locY = normalized(locY);
    cur0 = locX; cur1 = locY;
    gvel = mk(0, 0, 0); gangVel = mk(0, 0, 0);
    // new CPhys (ContactLoop.cpp:179-180)
    cp2<CP2>(P, matA, matB, r1, r2, V1.w, V2.w, kn, kt, tanPhi, hz);
    fx = 0; fy = 0; fz = 0;
    c.step0[i] = (int)stepOf(P, st);
  } else {
    // update (L6Geom.cpp:79-216)
    const d3 prevNormal = mk(c.hist[HIST_T0X][i], c.hist[HIST_T0Y][i], c.hist[HIST_T0Z][i]);
    const d3 prevT1 = mk(c.hist[HIST_T1X][i], c.hist[HIST_T1Y][i], c.hist[HIST_T1Z][i]);
    const d3 prevContPt = mk(c.hist[HIST_CX][i], c.hist[HIST_CY][i], c.hist[HIST_CZ][i]);
    const double dt = dtC;
    const int am = P.approxMask;
    const d3 currNormal = normal;
    d3 normRotVec = cross(prevNormal, currNormal);
    d3 midNormal = (am & 1) ? prevNormal : 0.5 * (prevNormal + currNormal);
    if (zeroBits(sqnorm(midNormal))) midNormal = currNormal;
    else if (!(am & 2) && !(am & 1)) midNormal = normalized(midNormal);
    d3 normTwistVec = midNormal * dt * 0.5 * dot(midNormal, angVel1 + angVel2);
    d3 rt = normRotVec + normTwistVec;
    d3 mid0, mid1;
    if (am & 4) { mid0 = prevNormal; mid1 = prevT1; }
    else { mid0 = midNormal; mid1 = prevT1 - cross(prevT1, rt) * 0.5; }
    d3 mid2 = cross(mid0, mid1);
    cur0 = currNormal;
    cur1 = prevT1 - cross(mid1, rt);
    if (P.trsfRenorm > 0 && (stepOf(P, st) % P.trsfRenorm) == 0) {
      cur0 = normalized(cur0);
      cur1 = cur1 - cur0 * dot(cur1, cur0);
      cur1 = normalized(cur1);
    }
    d3 midContPt, midPos1, midPos2;
    // periodic: velocity of the pB image, Cell::intrShiftVel = gradV * pprevHsize * cellDist
    d3 shiftVel2 = mk(0, 0, 0);
    if (PERI) shiftVel2 = mvec(P.shv, mk((double)cd.x, (double)cd.y, (double)cd.z));
    if (am & 8) { midContPt = contPt; midPos1 = pos1; midPos2 = pos2; }
    else {
      midContPt = 0.5 * (prevContPt + contPt);
      midPos1 = pos1 - (dt * 0.5) * vel1;
      midPos2 = PERI ? pos2 - (dt * 0.5) * (vel2 + shiftVel2) : pos2 - (dt * 0.5) * vel2;
    }
    d3 c1x = (P.noRatch && positiveBits(r1)) ? r1 * midNormal : midContPt - midPos1;
    d3 c2x = (P.noRatch && positiveBits(r2)) ? (-r2) * midNormal : midContPt - midPos2;
    d3 relVel = PERI ? (vel2 + shiftVel2 + cross(angVel2, c2x)) - (vel1 + cross(angVel1, c1x))
                     : (vel2 + cross(angVel2, c2x)) - (vel1 + cross(angVel1, c1x));
    gvel = mk(dot(mid0, relVel), dot(mid1, relVel), dot(mid2, relVel));
    // L6Geom.angVel feeds only the rolling/twisting resistance of IdealElPl and the downloaded geometry
    if (c.geom[0] || (LAW == WDEM_LAW_IDEALELPL && P.relRollStiff > 0. && P.rollTanPhi > 0.)) {
      const d3 dw = angVel2 - angVel1;
      gangVel = mk(dot(mid0, dw), dot(mid1, dw), dot(mid2, dw));
    } else {
      gangVel = mk(0, 0, 0);
    }
    fx = c.hist[HIST_FX][i]; fy = c.hist[HIST_FY][i]; fz = c.hist[HIST_FZ][i];
    kn = c.hist[HIST_KN][i]; kt = c.hist[HIST_KT][i];
    tanPhi = c.tanPhi[i];
    if (CP2 == WDEM_CP2_HERTZ) { hz[0] = c.hist[HIST_E0][i]; hz[1] = c.hist[HIST_E1][i]; hz[2] = c.hist[HIST_E2][i]; hz[3] = c.hist[HIST_E3][i]; }
    if (P.updatePhysNow) cp2<CP2>(P, matA, matB, r1, r2, V1.w, V2.w, kn, kt, tanPhi, hz);
  }
  const d3 cur2 = cross(cur0, cur1);

  // ---- Law2
  bool keep = true;
  double tqx = 0, tqy = 0, tqz = 0;
  const double dt = dtC;
  double eEl = 0, ePl = 0, eVN = 0, eVT = 0, eBr = 0;
  if (LAW == WDEM_LAW_IDEALELPL) {
    if (positiveBits(uN) && !P.noBreak) {
      keep = false;
      if (P.noSlip && P.trackEnergy) {
        // elastic potential lost when a contact breaks without slipping (IdealElPl.cpp:28-40)
        const double Fn = kn * uN;
        const double sc = dt * kt;
        const double ft0 = fy + sc * gvel.y, ft1 = fz + sc * gvel.z;
        eBr = .5 * (Fn * Fn / kn + (ft0 * ft0 + ft1 * ft1) / kt);
      }
    } else {
      fx = kn * uN;
      if (P.noFrict || zeroBits(tanPhi)) { fy = 0; fz = 0; }
      else {
        double sc = dt * kt;
        fy = fy + sc * gvel.y;
        fz = fz + sc * gvel.z;
        double maxFt = fabs(fx) * tanPhi;
        double ftSq = fy * fy + fz * fz;
        if (ftSq > maxFt * maxFt && !P.noSlip) {
          double FtNorm = sqrt(ftSq);
          double ratio = maxFt / FtNorm;
          if (zeroBits(FtNorm)) ratio = 0.;
          if (P.trackEnergy) ePl = (kt != 0. ? (maxFt) * (FtNorm - maxFt) / kt : 0.);
          fy *= ratio; fz *= ratio;
        }
        // Eigen maxCoeff = maxi(maxi(f0,f1),f2) with maxi(a,b) = a<b ? b : a
        double m01 = (fx < fy) ? fy : fx;
        double mm = (m01 < fz) ? fz : m01;
        if (nanBits(mm)) { if (atomicCAS(&st->code, 0, WDEM_ERR_NAN) == 0) st->detail = a; }
      }
      if (P.trackEnergy) {
        const double el = 0.5 * (fx * fx / kn + (kt != 0. ? (fy * fy + fz * fz) / kt : 0.));
        eEl = isnan(el) ? 0. : el;
      }
      if (P.relRollStiff > 0. && P.rollTanPhi > 0.) {
        double charLen = fabs(r1) + fabs(r2);
        double kr = kn * charLen;
        double tq0 = 0, tq1 = 0, tq2 = 0;  // the law resets CPhys.torque first (IdealElPl.cpp:34)
        if (P.relTwistStiff > 0) {
          tq0 = tq0 + dt * P.relTwistStiff * kr * gangVel.x;
          double maxTt = fabs(fx * P.rollTanPhi * charLen);
          if (fabs(tq0) > maxTt) tq0 = copysign(maxTt, tq0);
        }
        double sr = dt * kr;
        tq1 = tq1 + sr * gangVel.y;
        tq2 = tq2 + sr * gangVel.z;
        double maxTr = dmax(0., fabs(fx) * P.rollTanPhi * charLen);
        double trSq = tq1 * tq1 + tq2 * tq2;
        if (trSq > maxTr * maxTr) {
          double TrNorm = sqrt(trSq);
          double ratio = maxTr / TrNorm;
          if (TrNorm == 0.) ratio = 0.;
          tq1 *= ratio; tq2 *= ratio;
        }
        tqx = tq0; tqy = tq1; tqz = tq2;
      }
    }
  } else {
    const double velN = gvel.x;
    const double kn0 = hz[0];
#ifdef WDEM_FMA
    // one square root of the overlap for kn, Fne and kt, and its square root for the viscous coefficient
    const double sq = sqrt(dmax(-uN, 0.));
    kn = (3 / 2.) * kn0 * sq;
#else
    kn = (3 / 2.) * kn0 * sqrt(-uN);
#endif
    if (positiveBits(uN)) keep = false;
    else {
#ifdef WDEM_FMA
      double Fne = -kn0 * pown3(sq);
      double Fna = hz[3];
      double eta = (positiveBits(hz[2]) ? hz[2] * sqrt(sq) : 0.);
#else
      double Fne = -kn0 * pown3(sqrt(-uN));
      double Fna = hz[3];
      double eta = (positiveBits(hz[2]) ? hz[2] * sqrt(sqrt(dmax(-uN, 0.))) : 0.);
#endif
      double Fnv = eta * velN;
      // HertzPhys.alpha = mean of the materials' alpha (Hertz.cpp:52); the clamp applies when it is 0
      const double alphaC = .5 * (c_mats[p.meta[a].y].alpha + c_mats[p.meta[b].y].alpha);
      if (zeroBits(alphaC) && P.noAttraction && positiveBits(Fne + Fnv)) Fnv = -Fne;
      fx = Fne + Fna + Fnv;
      if (P.trackEnergy) eVN = Fnv * velN * dt;
#ifdef WDEM_FMA
      kt = hz[1] * sq;
#else
      kt = hz[1] * sqrt(negativeBits(uN) ? -uN : 0);
#endif
      double sc = dt * kt;
      fy = fy + sc * gvel.y;
      fz = fz + sc * gvel.z;
      double maxFt = fabs(dmin(0., fx) * tanPhi);
      double ftSq = fy * fy + fz * fz;
      if (ftSq > maxFt * maxFt) {
        double FtNorm = sqrt(ftSq);
        double ratio = maxFt / FtNorm;
        if (P.trackEnergy) ePl = (.5 * (FtNorm - maxFt) + maxFt) * (FtNorm - maxFt) / kt;
        fy *= ratio; fz *= ratio;
      } else {
        fy = fy + eta * gvel.y;
        fz = fz + eta * gvel.z;
        if (P.trackEnergy) eVT = eta * (gvel.y * gvel.y + gvel.z * gvel.z) * dt;
      }
      if (P.trackEnergy && uN < 0) eEl = kn0 * (2 / 5.) * pown5(sqrt(-uN)) + 0.5 * (fy * fy + fz * fz) / kt;
    }
  }

  if (P.trackEnergy) {
    c.energy[EC_ELAST][i] = eEl; c.energy[EC_PLAST][i] = ePl; c.energy[EC_VISCN][i] = eVN;
    c.energy[EC_VISCT][i] = eVT; c.energy[EC_BROKEN][i] = eBr;
  }
  if (!keep) {
    // ContactContainer::requestRemoval: geom and phys dropped, collider decides in the next step
    c.state[i] = CS_PENDING | sb;
    return;
  }
  // persistent history
  c.state[i] = CS_REAL | sb;
  if (p.touched) { p.touched[a] = 1; p.touched[b] = 1; }
  c.hist[HIST_T0X][i] = cur0.x; c.hist[HIST_T0Y][i] = cur0.y; c.hist[HIST_T0Z][i] = cur0.z;
  c.hist[HIST_T1X][i] = cur1.x; c.hist[HIST_T1Y][i] = cur1.y; c.hist[HIST_T1Z][i] = cur1.z;
  c.hist[HIST_CX][i] = contPt.x; c.hist[HIST_CY][i] = contPt.y; c.hist[HIST_CZ][i] = contPt.z;
  c.hist[HIST_FX][i] = fx; c.hist[HIST_FY][i] = fy; c.hist[HIST_FZ][i] = fz;
  c.hist[HIST_KN][i] = kn; c.hist[HIST_KT][i] = kt;
  if (!real || P.updatePhysNow) {
    c.tanPhi[i] = tanPhi;
    if (CP2 == WDEM_CP2_HERTZ) { c.hist[HIST_E0][i] = hz[0]; c.hist[HIST_E1][i] = hz[1]; c.hist[HIST_E2][i] = hz[2]; c.hist[HIST_E3][i] = hz[3]; }
  }
  if (c.geom[0]) {
    c.geom[0][i] = uN;
    c.geom[1][i] = gvel.x; c.geom[2][i] = gvel.y; c.geom[3][i] = gvel.z;
    c.geom[4][i] = gangVel.x; c.geom[5][i] = gangVel.y; c.geom[6][i] = gangVel.z;
  }
  // Contact::getForceTorqueBranch: F = ori*force, T = ori*torque (zero if torque is zero),
  // branch xc = contPt - node pos; the particle receives F and xc x F + T (sign -1 for pB)
  // (the quaternion of the frame, not the frame's columns: the frame update is first order and drifts from
  // orthonormality between renormalisations, which Quaternion(Matrix3) absorbs)
  const qd ori = quatFromCols(cur0, cur1, cur2);
  const d3 F = qrot(ori, mk(fx, fy, fz));
  const d3 tq = mk(tqx, tqy, tqz);
  const d3 T = isZeroBits(tq) ? mk(0, 0, 0) : qrot(ori, tq);
  const d3 xcA = contPt - pos1;
  const d3 xcB = contPt - pos2;
  const d3 TA = cross(xcA, F) + T;
  const d3 FB = F * -1.0;
  const d3 TB = cross(xcB, FB) + T * -1.0;
  // each particle's share at its CSR entry, stamped with this pass; a facet (pA) takes none
  // (ContactLoop::applyForceUninodal skips shapes with more than one node, ContactLoop.cpp:270-276)
  const int2 sl = c.slot[i];
  const double stamp = __longlong_as_double(seqOf(P, st));
  if (PERI || !(sb & CS_FACET)) {
    double4_32a* oa = c.out + OUT_RECORDS * (long long)sl.x;
    oa[OUT_F] = make_double4_32a(F.x, F.y, F.z, stamp);
    oa[OUT_T] = make_double4_32a(TA.x, TA.y, TA.z, 0.0);
  }
  double4_32a* ob = c.out + OUT_RECORDS * (long long)sl.y;
  ob[OUT_F] = make_double4_32a(FB.x, FB.y, FB.z, stamp);
  ob[OUT_T] = make_double4_32a(TB.x, TB.y, TB.z, 0.0);
  // the row positions this pass stamped, for the integrator's gather
  if (p.rowMask) {
    const uchar2 rb = c.rowBit[i];
    if (PERI || !(sb & CS_FACET)) atomicOr(&p.rowMask[a], 1u << rb.x);
    atomicOr(&p.rowMask[b], 1u << rb.y);
  }
}

#ifdef WDEM_FMA
// ---------------------------------------------------------------------------- double-word contact law
// The update of a real sphere-sphere or wall-sphere contact (L6Geom.cpp:79-216 with IdealElPl.cpp:15-92 or
// Hertz.cpp:85-114,170-210) with the frame, the law and the force rotation in double-word FP32 arithmetic
// (wdem_dw.cuh, 48 significant bits), selected by wdem_params.arith = WDEM_ARITH_DW.  FP64 stays where a
// difference cancels: the positions, the centre distance and the overlap uN = |d| - r1 - r2 (square root of
// the exactly rounded squared distance), the contact point, and the differences of positions and of
// velocities that the branch vectors and the relative velocity start from.  Everything else (the frame
// update, the local velocities, the Hertz or ideal-plastic law, the Coulomb cap, the quaternion of the frame
// and the rotation of the force, the branch torques) runs on the FP32 pipes.  New contacts, facets, rolling
// resistance, energy tracking, updatePhys and approxMask keep the FP64 law for the whole pass (the host
// decides, dwEligible); the double-word kernel takes the real contacts at the front of the work list and
// the FP64 kernel the potential pairs behind them, so that neither kernel carries both bodies.
__device__ __forceinline__ double fToD(float f) {  // exact, on the integer pipe (subnormals as zero)
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  const unsigned long long sgn = (unsigned long long)(u & 0x80000000u) << 32;
  if (e == 0) return __longlong_as_double((long long)sgn);
  if (e == 0xffu) return (double)f;
  return __longlong_as_double((long long)(sgn | ((unsigned long long)(e + 896u) << 52) |
                                          ((unsigned long long)(u & 0x7fffffu) << 29)));
}
__device__ __forceinline__ double dwToD(dwf x) { return fToD(x.h) + fToD(x.l); }
__device__ __forceinline__ dw3 dw3Of(d3 v) { return dw3From(v.x, v.y, v.z); }
__device__ __forceinline__ d3 dw3ToD(dw3 v) { return mk(dwToD(v.x), dwToD(v.y), dwToD(v.z)); }
__device__ __forceinline__ dw3 dw3Scale(dw3 a, float p2) { return {dwScale(a.x, p2), dwScale(a.y, p2), dwScale(a.z, p2)}; }
__device__ __forceinline__ dw3 dw3Normalized(dw3 a) { return dw3Mul(a, dwRecip(dwSqrt(dw3Sq(a)))); }
struct dwq {
  dwf w, x, y, z;
};
// Quaternion(Matrix3) of the frame with columns c0, c1, c2 (the branches of quatFromCols)
__device__ __forceinline__ dwq dwQuatFromCols(dw3 c0, dw3 c1, dw3 c2) {
  const dwf m00 = c0.x, m10 = c0.y, m20 = c0.z, m01 = c1.x, m11 = c1.y, m21 = c1.z, m02 = c2.x, m12 = c2.y, m22 = c2.z;
  dwq q;
  const dwf tr = dwAdd(dwAdd(m00, m11), m22);
  if (dwPos(tr)) {
    dwf t = dwSqrt(dwAddF(tr, 1.f));
    q.w = dwScale(t, 0.5f);
    t = dwScale(dwRecip(t), 0.5f);
    q.x = dwMul(dwSub(m21, m12), t);
    q.y = dwMul(dwSub(m02, m20), t);
    q.z = dwMul(dwSub(m10, m01), t);
  } else {
    int i = 0;
    if (dwGt(m11, m00)) i = 1;
    if (dwGt(m22, i == 0 ? m00 : m11)) i = 2;
    if (i == 0) {
      dwf t = dwSqrt(dwAddF(dwSub(dwSub(m00, m11), m22), 1.f));
      q.x = dwScale(t, 0.5f); t = dwScale(dwRecip(t), 0.5f);
      q.w = dwMul(dwSub(m21, m12), t); q.y = dwMul(dwAdd(m10, m01), t); q.z = dwMul(dwAdd(m20, m02), t);
    } else if (i == 1) {
      dwf t = dwSqrt(dwAddF(dwSub(dwSub(m11, m22), m00), 1.f));
      q.y = dwScale(t, 0.5f); t = dwScale(dwRecip(t), 0.5f);
      q.w = dwMul(dwSub(m02, m20), t); q.z = dwMul(dwAdd(m21, m12), t); q.x = dwMul(dwAdd(m01, m10), t);
    } else {
      dwf t = dwSqrt(dwAddF(dwSub(dwSub(m22, m00), m11), 1.f));
      q.z = dwScale(t, 0.5f); t = dwScale(dwRecip(t), 0.5f);
      q.w = dwMul(dwSub(m10, m01), t); q.x = dwMul(dwAdd(m02, m20), t); q.y = dwMul(dwAdd(m12, m21), t);
    }
  }
  return q;
}
// v rotated by q: uv = q.vec x v, uv += uv, v + w uv + q.vec x uv (as qrot)
__device__ __forceinline__ dw3 dwQrot(dwq q, dw3 v) {
  const dw3 qv = {q.x, q.y, q.z};
  const dw3 uv = dw3Scale(dw3Cross(qv, v), 2.f);
  return dw3Add(dw3Add(v, dw3Mul(uv, q.w)), dw3Cross(qv, uv));
}

template <int LAW, int CP2, bool PERI>
__device__ __forceinline__ void contactBodyDW(const StepParams& P, const Particles& p, const Contacts& c, long long i,
                                              DeviceStatus* st) {
  const uint8_t s0 = c.state[i];
  const uint8_t sb = s0 & CS_SHAPES;
  if ((s0 & CS_MASK) != CS_REAL) return;  // the front of the work list holds real contacts only
  const int2 id = c.ids[i];
  const int a = id.x, b = id.y;
  const double dtC = P.matDt ? P.matDt[p.meta[a].y] : P.dt;
  int4 cd = make_int4(0, 0, 0, 0);
  if (PERI) cd = c.cdist[i];
  const double4_32a A4 = p.posr[a], B4 = p.posr[b];
  const d3 pos1 = xyz(A4);
  d3 shift2 = mk(0, 0, 0);
  if (PERI) shift2 = mvec(P.hS, mk((double)cd.x, (double)cd.y, (double)cd.z));
  const d3 pos2 = PERI ? xyz(B4) + shift2 : xyz(B4);
  double r1, r2, uN;
  dw3 normal, d1, d2;  // d1, d2: the contact point's offsets from pA's and pB's node (the branch vectors)
  d3 contPt;
  if (!(sb & CS_WALL_A)) {
    // Cg2_Sphere_Sphere_L6Geom::go of a real contact: uN in FP64, the normal and the contact point's offset
    // from pA in double words
    r1 = A4.w; r2 = B4.w;
    const d3 relPos = pos2 - pos1;
    const double dist = sqrt(sqnormExact(relPos));
    uN = dist - (r1 + r2);
    const dw3 relPosW = dw3Of(relPos);
    normal = dw3Mul(relPosW, dwRecip(dwFrom(dist)));
    d1 = dw3Mul(normal, dwFrom(r1 + 0.5 * uN));
    d2 = dw3Sub(d1, relPosW);
    contPt = pos1 + dw3ToD(d1);
  } else {
    // Cg2_Wall_Sphere_L6Geom::go (pA is the wall)
    const int wa = p.meta[a].x;
    const int ax = (wa >> 4) & 3, sense = ((wa >> 8) & 3) - 1;
    const double radius = B4.w;
    const double dist = comp(pos2, ax) - comp(pos1, ax);
    contPt = pos2;
    setComp(contPt, ax, comp(pos1, ax));
    const double nax = sense == 0 ? comp(mk(c.hist[HIST_T0X][i], c.hist[HIST_T0Y][i], c.hist[HIST_T0Z][i]), ax)
                                  : (sense == 1 ? 1. : -1.);
    normal = {dwF(0.f), dwF(0.f), dwF(0.f)};
    if (ax == 0) normal.x = dwF((float)nax); else if (ax == 1) normal.y = dwF((float)nax); else normal.z = dwF((float)nax);
    uN = nax * dist - radius;
    r1 = -radius; r2 = radius;
    d1 = dw3Of(contPt - pos1);
    d2 = dw3Of(contPt - pos2);
  }
  // L6Geom update (L6Geom.cpp:79-216), approxMask 0
  const dw3 prevNormal = dw3From(c.hist[HIST_T0X][i], c.hist[HIST_T0Y][i], c.hist[HIST_T0Z][i]);
  const dw3 prevT1 = dw3From(c.hist[HIST_T1X][i], c.hist[HIST_T1Y][i], c.hist[HIST_T1Z][i]);
  const d3 prevContPt = mk(c.hist[HIST_CX][i], c.hist[HIST_CY][i], c.hist[HIST_CZ][i]);
  const dwf dt = dwFrom(dtC);
  const dwf dtHalf = dwScale(dt, 0.5f);
  const double4_32a V1 = p.velm[a], V2 = p.velm[b];
  const double4_32a W1 = p.angw[a], W2 = p.angw[b];
  const dw3 angVel1 = dw3From(W1.x, W1.y, W1.z), angVel2 = dw3From(W2.x, W2.y, W2.z);
  const dw3 currNormal = normal;
  const dw3 normRotVec = dw3Cross(prevNormal, currNormal);
  dw3 midNormal = dw3Scale(dw3Add(prevNormal, currNormal), 0.5f);
  if (dwIsZero(dw3Sq(midNormal))) midNormal = currNormal;
  else midNormal = dw3Normalized(midNormal);
  const dw3 normTwistVec = dw3Mul(midNormal, dwMul(dtHalf, dw3Dot(midNormal, dw3Add(angVel1, angVel2))));
  const dw3 rt = dw3Add(normRotVec, normTwistVec);
  const dw3 mid0 = midNormal;
  const dw3 mid1 = dw3Sub(prevT1, dw3Scale(dw3Cross(prevT1, rt), 0.5f));
  const dw3 mid2 = dw3Cross(mid0, mid1);
  dw3 cur0 = currNormal;
  dw3 cur1 = dw3Sub(prevT1, dw3Cross(mid1, rt));
  if (P.trsfRenorm > 0 && (stepOf(P, st) % P.trsfRenorm) == 0) {
    cur0 = dw3Normalized(cur0);
    cur1 = dw3Sub(cur1, dw3Mul(cur0, dw3Dot(cur1, cur0)));
    cur1 = dw3Normalized(cur1);
  }
  // branch vectors midContPt - midPos = (contPt - pos) + (prevContPt - contPt) / 2 + dt/2 vel: the offsets
  // d1, d2 and the FP64 difference of the two contact points, which are close together
  d3 shiftVel2 = mk(0, 0, 0);
  if (PERI) shiftVel2 = mvec(P.shv, mk((double)cd.x, (double)cd.y, (double)cd.z));
  const d3 vel1d = xyz(V1), vel2d = PERI ? xyz(V2) + shiftVel2 : xyz(V2);
  const dw3 halfPrev = dw3Scale(dw3Of(prevContPt - contPt), 0.5f);
  const dw3 c1x = (P.noRatch && positiveBits(r1)) ? dw3Mul(midNormal, dwFrom(r1))
                                                   : dw3Add(dw3Add(d1, halfPrev), dw3Mul(dw3Of(vel1d), dtHalf));
  const dw3 c2x = (P.noRatch && positiveBits(r2)) ? dw3Mul(midNormal, dwFrom(-r2))
                                                   : dw3Add(dw3Add(d2, halfPrev), dw3Mul(dw3Of(vel2d), dtHalf));
  const dw3 relVel = dw3Add(dw3Of(vel2d - vel1d), dw3Sub(dw3Cross(angVel2, c2x), dw3Cross(angVel1, c1x)));
  const dw3 gvel = {dw3Dot(mid0, relVel), dw3Dot(mid1, relVel), dw3Dot(mid2, relVel)};
  dwf fx = dwFrom(c.hist[HIST_FX][i]), fy = dwFrom(c.hist[HIST_FY][i]), fz = dwFrom(c.hist[HIST_FZ][i]);
  double knD = c.hist[HIST_KN][i], ktD = c.hist[HIST_KT][i];
  const dwf tanPhi = dwFrom(c.tanPhi[i]);
  const dw3 cur2 = dw3Cross(cur0, cur1);
  // ---- Law2
  bool keep = true;
  if (LAW == WDEM_LAW_IDEALELPL) {
    if (positiveBits(uN) && !P.noBreak) keep = false;
    else {
      fx = dwFrom(knD * uN);  // FP64: the normal force carries the relative error of uN only
      if (P.noFrict || zeroBits(c.tanPhi[i])) { fy = dwF(0.f); fz = dwF(0.f); }
      else {
        const dwf sc = dwFrom(dtC * ktD);
        fy = dwAdd(fy, dwMul(sc, gvel.y));
        fz = dwAdd(fz, dwMul(sc, gvel.z));
        const dwf maxFt = dwMul(dwAbs(fx), tanPhi);
        const dwf ftSq = dwAdd(dwMul(fy, fy), dwMul(fz, fz));
        if (dwGt(ftSq, dwMul(maxFt, maxFt)) && !P.noSlip) {
          const dwf FtNorm = dwSqrt(ftSq);
          const dwf ratio = dwIsZero(FtNorm) ? dwF(0.f) : dwDiv(maxFt, FtNorm);
          fy = dwMul(fy, ratio); fz = dwMul(fz, ratio);
        }
        if (isnan(fx.h) || isnan(fy.h) || isnan(fz.h)) { if (atomicCAS(&st->code, 0, WDEM_ERR_NAN) == 0) st->detail = a; }
      }
    }
  } else {
    const double kn0 = c.hist[HIST_E0][i];
    if (positiveBits(uN)) keep = false;
    else {
      // the normal force in FP64 as in the contracted FP64 body: near equilibrium the elastic and adhesive
      // terms cancel, and the sum must carry no more than the overlap's relative error
      const double velN = dwToD(gvel.x);
      const double sq = sqrt(dmax(-uN, 0.));
      knD = (3 / 2.) * kn0 * sq;
      const double Fne = -kn0 * pown3(sq);
      const double Fna = c.hist[HIST_E3][i];
      const double hz2 = c.hist[HIST_E2][i];
      const double etaD = positiveBits(hz2) ? hz2 * sqrt(sq) : 0.;
      double Fnv = etaD * velN;
      const double alphaC = .5 * (c_mats[p.meta[a].y].alpha + c_mats[p.meta[b].y].alpha);
      if (zeroBits(alphaC) && P.noAttraction && positiveBits(Fne + Fnv)) Fnv = -Fne;
      fx = dwFrom(Fne + Fna + Fnv);
      const dwf eta = dwFrom(etaD);
      ktD = c.hist[HIST_E1][i] * sq;
      const dwf sc = dwFrom(dtC * ktD);
      fy = dwAdd(fy, dwMul(sc, gvel.y));
      fz = dwAdd(fz, dwMul(sc, gvel.z));
      const dwf maxFt = dwMul(dwAbs(dwMin(dwF(0.f), fx)), tanPhi);
      const dwf ftSq = dwAdd(dwMul(fy, fy), dwMul(fz, fz));
      if (dwGt(ftSq, dwMul(maxFt, maxFt))) {
        const dwf ratio = dwDiv(maxFt, dwSqrt(ftSq));
        fy = dwMul(fy, ratio); fz = dwMul(fz, ratio);
      } else {
        fy = dwAdd(fy, dwMul(eta, gvel.y));
        fz = dwAdd(fz, dwMul(eta, gvel.z));
      }
    }
  }
  if (!keep) {
    c.state[i] = CS_PENDING | sb;
    return;
  }
  c.state[i] = CS_REAL | sb;
  if (p.touched) { p.touched[a] = 1; p.touched[b] = 1; }
  const d3 c0d = dw3ToD(cur0), c1d = dw3ToD(cur1);
  c.hist[HIST_T0X][i] = c0d.x; c.hist[HIST_T0Y][i] = c0d.y; c.hist[HIST_T0Z][i] = c0d.z;
  c.hist[HIST_T1X][i] = c1d.x; c.hist[HIST_T1Y][i] = c1d.y; c.hist[HIST_T1Z][i] = c1d.z;
  c.hist[HIST_CX][i] = contPt.x; c.hist[HIST_CY][i] = contPt.y; c.hist[HIST_CZ][i] = contPt.z;
  c.hist[HIST_FX][i] = dwToD(fx); c.hist[HIST_FY][i] = dwToD(fy); c.hist[HIST_FZ][i] = dwToD(fz);
  c.hist[HIST_KN][i] = knD; c.hist[HIST_KT][i] = ktD;
  if (c.geom[0]) {
    const dw3 dw_ = dw3Sub(angVel2, angVel1);
    c.geom[0][i] = uN;
    c.geom[1][i] = dwToD(gvel.x); c.geom[2][i] = dwToD(gvel.y); c.geom[3][i] = dwToD(gvel.z);
    c.geom[4][i] = dwToD(dw3Dot(mid0, dw_)); c.geom[5][i] = dwToD(dw3Dot(mid1, dw_)); c.geom[6][i] = dwToD(dw3Dot(mid2, dw_));
  }
  // Contact::getForceTorqueBranch: F = ori * force, branch torques xc x F (no CPhys torque on this path)
  const dw3 F = dwQrot(dwQuatFromCols(cur0, cur1, cur2), dw3{fx, fy, fz});
  const d3 Fd = dw3ToD(F);
  const d3 TA = dw3ToD(dw3Cross(d1, F));
  const d3 TB = dw3ToD(dw3Cross(d2, dw3Scale(F, -1.f)));
  const int2 sl = c.slot[i];
  const double stamp = __longlong_as_double(seqOf(P, st));
  if (PERI || !(sb & CS_FACET)) {
    double4_32a* oa = c.out + OUT_RECORDS * (long long)sl.x;
    oa[OUT_F] = make_double4_32a(Fd.x, Fd.y, Fd.z, stamp);
    oa[OUT_T] = make_double4_32a(TA.x, TA.y, TA.z, 0.0);
  }
  double4_32a* ob = c.out + OUT_RECORDS * (long long)sl.y;
  ob[OUT_F] = make_double4_32a(-Fd.x, -Fd.y, -Fd.z, stamp);
  ob[OUT_T] = make_double4_32a(TB.x, TB.y, TB.z, 0.0);
  if (p.rowMask) {
    const uchar2 rb = c.rowBit[i];
    if (PERI || !(sb & CS_FACET)) atomicOr(&p.rowMask[a], 1u << rb.x);
    atomicOr(&p.rowMask[b], 1u << rb.y);
  }
}
#endif

// BS threads a block and 512 threads an SM (<= 128 registers a thread, no spills); the grid (blocks per
// SM) and BS are the launch shape of the step parameters, chosen by the autotuner or the defaults (128
// threads, 4 blocks per SM: one wave)
template <int LAW, int CP2, bool PERI, bool ELL, int BS, bool DW = false>
__global__ void __launch_bounds__(BS, 512 / BS) k_contacts(StepParams P, Particles p, Contacts c, const unsigned* work,
                                                        const unsigned* count, long long nc, DeviceStatus* st,
                                                        int part) {
  // part 0: the whole work list; 1: the real contacts at its front; 2: the potential pairs behind them
  const unsigned k0 = part == 2 ? count[0] : 0u;
  const unsigned m = part == 1 ? count[0] : workLen(count);
  for (unsigned k = k0 + blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
#ifdef WDEM_FMA
    if (DW) {
      contactBodyDW<LAW, CP2, PERI>(P, p, c, (long long)workItem(work, count, nc, k), st);
      continue;
    }
#endif
    contactBody<LAW, CP2, PERI, ELL>(P, p, c, (long long)workItem(work, count, nc, k), st);
  }
}

// First pass over all contacts: resolves PENDING contacts (removePending of the collider: the broken
// contact dies when the boxes of the last rebuild no longer overlap, else it is potential again), skips
// dead pairs and wall+wall pairs (no Cg2 functor, ContactLoop.cpp:149-150), and culls potential pairs that
// cannot touch with FP32 tests whose margins exceed their rounding (the exact FP64 test would reject
// them too).  Survivors (real contacts and potential pairs near touching) are appended to the work list;
// the list order is irrelevant because each contact is processed independently.
// One contact of the cull (see k_contacts_cull): need = the FP64 pass must see it this step, real = it
// is a real contact; returns false when the contact can be left out of the pass until the next
// rebuild (dead, wall + wall, or far).
template <bool PERI, bool ELL>
__device__ __forceinline__ bool cullOne(const StepParams& P, const Particles& p, const Contacts& c, long long nc,
                                        long long i, uint8_t s0, DeviceStatus* st, bool& need, bool& realNow) {
  const uint8_t sb = s0 & CS_SHAPES;
  uint8_t s = s0 & CS_MASK;
  if (s == CS_POTENTIAL && !PERI && (s0 & CS_FAR)) {
    // cannot touch before the next rebuild: nothing to load
  } else if (s != CS_DEAD && sb != (CS_WALL_A | CS_WALL_B)) {
    const int2 id = c.ids[i];
    const int a = id.x, b = id.y;
    bool alive = true;
    if (s == CS_PENDING) {
      bool ov;
      if (PERI) {
        int4 per;
        bool amb = false;
        ov = overlapPeri(p.bbmin[a], p.bbmax[a], p.bbmin[b], p.bbmax[b], P.csize, per, amb);
        if (amb) { if (atomicCAS(&st->code, 0, WDEM_ERR_TOO_BIG) == 0) st->detail = a; ov = true; alive = false; }
      } else
        ov = overlapBoxes(p.bbmin[a], p.bbmax[a], p.bbmin[b], p.bbmax[b]);
      if (!ov) { c.state[i] = CS_DEAD | sb; alive = false; }
      else if (alive) { s = CS_POTENTIAL; c.state[i] = s | sb; }
    }
    if (alive) {
      if (s == CS_REAL) need = realNow = true;
      else if (sb & CS_FACET) need = true;  // facet + sphere: the FP64 functor decides every step
      else if (!(sb & CS_WALL_A)) {
        // Sphere/ellipsoid pairs: the FP32 copies carry a relative error below 2^-23 per coordinate and
        // radius; the margin (1e-5 relative on the contact distance plus 1e-6 x the sum of |coordinates|)
        // exceeds the accumulated FP32 error, so a pair rejected here fails the exact FP64 test of
        // Cg2_Sphere_Sphere_L6Geom (ellipsoids: it lies outside the bounding spheres, F_ab > 1).
        // Pairs close to touching, NaN and overflow fall through to the FP64 test.
        const float4 fa = p.posf[a];
        float4 fb = p.posf[b];
        float Sh = 0.f;
        if (PERI) {
          // FP32 image shift; its rounding is bounded by 2^-23 x sum |h_ij cellDist_j|, added to the margin
          const int4 cd = c.cdist[i];
          const float c0 = (float)cd.x, c1 = (float)cd.y, c2 = (float)cd.z;
          const float h[9] = {(float)P.hS[0], (float)P.hS[1], (float)P.hS[2], (float)P.hS[3], (float)P.hS[4],
                              (float)P.hS[5], (float)P.hS[6], (float)P.hS[7], (float)P.hS[8]};
          fb.x += h[0] * c0 + h[1] * c1 + h[2] * c2;
          fb.y += h[3] * c0 + h[4] * c1 + h[5] * c2;
          fb.z += h[6] * c0 + h[7] * c1 + h[8] * c2;
          for (int q = 0; q < 9; q++) Sh += fabsf(h[q]) * fabsf(q % 3 == 0 ? c0 : (q % 3 == 1 ? c1 : c2));
        }
        const float dx = fb.x - fa.x, dy = fb.y - fa.y, dz = fb.z - fa.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float S = fabsf(fa.x) + fabsf(fa.y) + fabsf(fa.z) + fabsf(fb.x) + fabsf(fb.y) + fabsf(fb.z) + 2.f * Sh;
        const float df = (ELL && (sb & CS_ELL)) ? 1.f : P.distFactorF;
        const float R = df * (fa.w + fb.w) * 1.00001f + 1e-6f * S;
        need = !(d2 > R * R);
        if (!PERI && !need) {
          // far: the distance exceeds the (error-padded) contact distance by 4 verletDist (CS_FAR)
          const float Rf = (R + 4.f * P.verletHiF) * 1.00001f;
          if (d2 > Rf * Rf) c.state[i] = (uint8_t)(CS_POTENTIAL | CS_FAR | sb);
        }
      } else {
        // wall + sphere/ellipsoid: the distance along the wall axis against the radius (ellipsoids: the
        // largest semi-axis, an upper bound of the extent), with the same kind of margin
        const int ax = (p.meta[a].x >> 4) & 3;
        const float4 fa = p.posf[a], fb = p.posf[b];
        const float ca = ax == 0 ? fa.x : (ax == 1 ? fa.y : fa.z), cb = ax == 0 ? fb.x : (ax == 1 ? fb.y : fb.z);
        const float dist = fabsf(cb - ca);
        need = !(dist > fb.w * 1.00001f + 1e-6f * (fabsf(ca) + fabsf(cb)));
      }
    }
  }
  const uint8_t s1 = c.state[i];
  return (s1 & CS_MASK) != CS_DEAD && (s1 & CS_SHAPES) != (CS_WALL_A | CS_WALL_B) && !(s1 & CS_FAR);
}

// warp-aggregated appends: the work list (real contacts from the front, potential pairs from the back)
// and, in the full pass, the active list
__device__ __forceinline__ void cullAppend(unsigned* work, unsigned* count, long long nc, long long i, bool need,
                                           bool realNow, unsigned* act, unsigned* actCount, bool active) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1;
  const unsigned bReal = __ballot_sync(0xffffffffu, need && realNow);
  const unsigned bPot = __ballot_sync(0xffffffffu, need && !realNow);
  if (bReal) {
    const int leader = __ffs(bReal) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(&count[0], (unsigned)__popc(bReal));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (need && realNow) work[base + __popc(bReal & below)] = (unsigned)i;
  }
  if (bPot) {
    const int leader = __ffs(bPot) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(&count[1], (unsigned)__popc(bPot));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (need && !realNow) work[nc - 1 - (base + __popc(bPot & below))] = (unsigned)i;
  }
  if (act) {
    const unsigned bAct = __ballot_sync(0xffffffffu, active);
    if (bAct) {
      const int leader = __ffs(bAct) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(actCount, (unsigned)__popc(bAct));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (active) act[base + __popc(bAct & below)] = (unsigned)i;
    }
  }
}

// First pass over the contacts: resolves PENDING contacts (removePending of the collider: the broken
// contact dies when the boxes of the last rebuild no longer overlap, else it is potential again), skips
// dead pairs and wall+wall pairs (no Cg2 functor, ContactLoop.cpp:149-150), and culls potential pairs that
// cannot touch with FP32 tests whose margins exceed their rounding (the exact FP64 test would reject
// them too).  Survivors (real contacts and potential pairs near touching) are appended to the work list;
// the list order is irrelevant because each contact is processed independently.  FULL: one thread per
// contact of the container, and the contacts that may need the pass before the next rebuild are
// listed (act); otherwise the grid walks that list only.
template <bool PERI, bool ELL, bool FULL, int BS>
__global__ void __launch_bounds__(BS) k_contacts_cull(StepParams P, Particles p, Contacts c, long long nc,
                                                       unsigned* work, unsigned* count, DeviceStatus* st) {
  const long long first = (long long)blockIdx.x * blockDim.x;
  const long long m = FULL ? nc : (long long)st->actCount;
  // a step queued behind a collider trigger: the work list stays empty, so the heavy pass is a no-op too
  if (haltedContacts(st, stepOf(P, st))) return;
  // the integrator's lists of this step have been consumed: their counters start the next step at 0
  if (first + threadIdx.x == 0) { st->rotCount = 0; st->touchCount = 0; }
  const long long stride = FULL ? m + 1 : (long long)gridDim.x * blockDim.x;
  for (long long base = first; base < m; base += stride) {
    const long long k = base + threadIdx.x;
    const long long i = k < m ? (FULL ? k : (long long)c.act[k]) : -1;
    bool need = false, realNow = false, active = false;
    if (i >= 0) active = cullOne<PERI, ELL>(P, p, c, nc, i, c.state[i], st, need, realNow);
    cullAppend(work, count, nc, i, need, realNow, FULL ? c.act : nullptr, &st->actCount, active && FULL);
  }
}

// the cull with the block size of the launch shape
template <bool PERI, bool ELL>
static void launchCull(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc, unsigned* count,
                       DeviceStatus* st, bool full) {
  const int bs = P.shCullBlock == 128 || P.shCullBlock == 512 ? P.shCullBlock : 256;
  const long long sms = P.numSMs > 0 ? P.numSMs : 152;
  // full pass: a thread per contact; list pass: a grid-stride walk of the active list (2048 threads an SM)
  const unsigned cb = full ? (unsigned)((nc + bs - 1) / bs) : (unsigned)std::min<long long>((nc + bs - 1) / bs, sms * (2048 / bs));
#define WDEM_CULL(BS_)                                                                                              \
  (full ? k_contacts_cull<PERI, ELL, true, BS_> : k_contacts_cull<PERI, ELL, false, BS_>)<<<cb, BS_, 0, s>>>(      \
      P, p, c, nc, c.work, count, st)
  if (bs == 128) WDEM_CULL(128);
  else if (bs == 512) WDEM_CULL(512);
  else WDEM_CULL(256);
#undef WDEM_CULL
  ++::wdem::g_kernel_launches;
}
#ifdef WDEM_FMA
// the double-word law applies to the whole pass: no facets, no energy tracking, no updatePhys, no approxMask,
// no rolling resistance
template <int LAW>
static bool dwEligible(const StepParams& P) {
  return P.dw && !P.hasFacets && !P.trackEnergy && !P.updatePhysNow && P.approxMask == 0 &&
         !(LAW == WDEM_LAW_IDEALELPL && P.relRollStiff > 0. && P.rollTanPhi > 0.);
}
#endif
// the FP64 pass with the block size and blocks per SM of the launch shape
template <int LAW, int CP2, bool PERI, bool ELL>
static void launchHeavy(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc, unsigned* count,
                        DeviceStatus* st) {
  const int bs = P.shContactsBlock == 64 || P.shContactsBlock == 256 ? P.shContactsBlock : 128;
  const long long sms = P.numSMs > 0 ? P.numSMs : 152;
  const long long perSM = P.shContactsPerSM > 0 ? P.shContactsPerSM : 512 / bs;
  const long long need = (nc + bs - 1) / bs;
  const unsigned hb = (unsigned)std::max<long long>(1, std::min(need, sms * perSM));
  int part = 0;
#ifdef WDEM_FMA
  if (!ELL && dwEligible<LAW>(P)) {
    // the double-word law for the real contacts, then the FP64 kernel for the potential pairs
    if (bs == 64) k_contacts<LAW, CP2, PERI, false, 64, true><<<hb, 64, 0, s>>>(P, p, c, c.work, count, nc, st, 1);
    else if (bs == 256) k_contacts<LAW, CP2, PERI, false, 256, true><<<hb, 256, 0, s>>>(P, p, c, c.work, count, nc, st, 1);
    else k_contacts<LAW, CP2, PERI, false, 128, true><<<hb, 128, 0, s>>>(P, p, c, c.work, count, nc, st, 1);
    ++::wdem::g_kernel_launches;
    part = 2;
  }
#endif
  if (bs == 64) k_contacts<LAW, CP2, PERI, ELL, 64><<<hb, 64, 0, s>>>(P, p, c, c.work, count, nc, st, part);
  else if (bs == 256) k_contacts<LAW, CP2, PERI, ELL, 256><<<hb, 256, 0, s>>>(P, p, c, c.work, count, nc, st, part);
  else k_contacts<LAW, CP2, PERI, ELL, 128><<<hb, 128, 0, s>>>(P, p, c, c.work, count, nc, st, part);
  ++::wdem::g_kernel_launches;
}

void launch_contacts(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc, DeviceStatus* st,
                     bool full, const uint16_t* warmBf, const float* warmF) {
  if (nc <= 0) {
    cudaMemsetAsync(&st->rotCount, 0, 2 * sizeof(unsigned), s);  // rotCount, touchCount; otherwise cleared by the cull kernel
    return;
  }
  unsigned* count = &st->workCount;  // workCount, workPot
  cudaMemsetAsync(count, 0, 2 * sizeof(unsigned), s);
  if (full) cudaMemsetAsync(&st->actCount, 0, sizeof(unsigned), s);
  // the FP64 pass loops over the work list (length known on the device only): by default 4 blocks of 128
  // per SM fill the GPU at its register count, and no more blocks are launched to find the list short
  if (P.hasEll) {
    // ellipsoid scenes: aperiodic, FrictMat + IdealElPl (checked on the host)
    launchCull<false, true>(s, P, p, c, nc, count, st, full);
    if (warmBf) mlp_launch_warm(s, p, c, nc, c.work, count, warmBf, warmF, P.warmStart == WDEM_WARM_HISTORY_MLP, st, P.numSMs);
    launchHeavy<WDEM_LAW_IDEALELPL, WDEM_CP2_FRICT, false, true>(s, P, p, c, nc, count, st);
  } else if (P.periodic) {
    launchCull<true, false>(s, P, p, c, nc, count, st, full);
    if (P.law == WDEM_LAW_IDEALELPL) launchHeavy<WDEM_LAW_IDEALELPL, WDEM_CP2_FRICT, true, false>(s, P, p, c, nc, count, st);
    else launchHeavy<WDEM_LAW_HERTZ_DMT, WDEM_CP2_HERTZ, true, false>(s, P, p, c, nc, count, st);
  } else {
    launchCull<false, false>(s, P, p, c, nc, count, st, full);
    if (P.law == WDEM_LAW_IDEALELPL) launchHeavy<WDEM_LAW_IDEALELPL, WDEM_CP2_FRICT, false, false>(s, P, p, c, nc, count, st);
    else launchHeavy<WDEM_LAW_HERTZ_DMT, WDEM_CP2_HERTZ, false, false>(s, P, p, c, nc, count, st);
  }
}

WDEM_VARIANT_END
}  // namespace wdem

namespace wdem {
WDEM_VARIANT_BEGIN

// HertzPhys constants (kn0, kt0, alpha_sqrtMK, adhesion) of uploaded real contacts: Woo stores them
// in HertzPhys (Hertz.hpp:16-31); they are pure functions of the materials, radii and masses.
__global__ void k_init_uploaded(StepParams P, Particles p, Contacts c, long long nc) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc || (c.state[i] & CS_MASK) != CS_REAL) return;
  const int2 id = c.ids[i];
  const int4 ma = p.meta[id.x], mb = p.meta[id.y];
  const double rb = p.posr[id.y].w;
  const double ra = p.posr[id.x].w;
  const double r1 = ((ma.x & 15) == WDEM_SHAPE_WALL) ? -rb : ((ma.x & 15) == WDEM_SHAPE_FACET ? ((ra < rb) ? rb : ra) : ra);
  const double r2 = rb;
  double kn, kt, tanPhi, hz[4];
  cp2<WDEM_CP2_HERTZ>(P, ma.y, mb.y, r1, r2, p.velm[id.x].w, p.velm[id.y].w, kn, kt, tanPhi, hz);
  c.hist[HIST_E0][i] = hz[0]; c.hist[HIST_E1][i] = hz[1]; c.hist[HIST_E2][i] = hz[2]; c.hist[HIST_E3][i] = hz[3];
}

void launch_init_uploaded(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc) {
  if (nc <= 0 || P.cp2 != WDEM_CP2_HERTZ) return;
  (k_init_uploaded<<<(unsigned)((nc + 127) / 128), 128, 0, s>>>(P, p, c, nc), ++::wdem::g_kernel_launches);
}

WDEM_VARIANT_END
}  // namespace wdem
