// k_leapfrog.cu -- fused integrator: the GB300 replacement of Woo's Leapfrog(reset=True)
// (src/dem/Leapfrog.cpp:104-255) with ForceResetter folded in, the per-node force accumulation of
// DemData::addForceTorque (src/dem/Particle.hpp:249) done as a deterministic CSR gather, and the
// collider's verlet trigger AabbCollider::aabbIsDirty (src/dem/Collision.cpp:80-123).
//
// One thread per particle.  The force on a particle is m*g (reset at the end of the previous step)
// plus the contributions of its real contacts, added in the order of the contacts' (min id, max id)
// keys; that fixed order makes the sum deterministic and identical to the CPU oracle's.
#include <algorithm>

#include "wdem_internal.h"
#include "wdem_variant.h"
#include "wdem_math.cuh"
#include "../../include/wdem.h"

namespace wdem {
WDEM_VARIANT_BEGIN

// F = m g (unless gravitySkip) + sum of contact forces; T = sum of contact torques
// Contact forces and torques of particle i from the previous contact pass: its CSR row's records, in the
// row's order (the partner ids'), those stamped by that pass only (contacts real after it).
__device__ __forceinline__ void gatherRow(long long want, int i, const Contacts& c, const Csr& csr, d3& F, d3& T) {
  const int e0 = csr.rowptr[i], e1 = csr.rowptr[i + 1];
  for (int e = e0; e < e1; e++) {
    const double4_32a* o = c.out + OUT_RECORDS * (long long)e;
    const double4_32a f4 = o[OUT_F];
    if (__double_as_longlong(f4.w) != want) continue;
    F = F + xyz(f4);
    T = T + xyz(o[OUT_T]);
  }
}

// The same sum over the entries of the row that the contact pass marked in the particle's row mask, in the
// row's order: an entry outside the mask was not stamped by that pass; a stale bit (from a pass before a
// rebuild) fails the stamp test as in gatherRow.
__device__ __forceinline__ void gatherRowMasked(long long want, int i, unsigned mask, const Contacts& c, const Csr& csr,
                                                d3& F, d3& T) {
  const int e0 = csr.rowptr[i], e1 = csr.rowptr[i + 1];
  unsigned lo = mask & 0x7fffffffu;
  while (lo) {
    const int e = e0 + __ffs(lo) - 1;
    lo &= lo - 1;
    if (e >= e1) break;
    const double4_32a* o = c.out + OUT_RECORDS * (long long)e;
    const double4_32a f4 = o[OUT_F];
    if (__double_as_longlong(f4.w) != want) continue;
    F = F + xyz(f4);
    T = T + xyz(o[OUT_T]);
  }
  if (mask & 0x80000000u) {
    for (int e = e0 + 31; e < e1; e++) {
      const double4_32a* o = c.out + OUT_RECORDS * (long long)e;
      const double4_32a f4 = o[OUT_F];
      if (__double_as_longlong(f4.w) != want) continue;
      F = F + xyz(f4);
      T = T + xyz(o[OUT_T]);
    }
  }
}

__device__ __forceinline__ void gatherForce(const StepParams& P, long long want, int i, double mass, unsigned flags,
                                            const Contacts& c, const Csr& csr, d3& F, d3& T) {
  const bool grav = P.hasGravity && !(flags & WDEM_GRAVITY_SKIP);
  if (grav) {
    // mass * g; a component of g that is exactly zero gives a zero of the sign of the (finite) mass,
    // set without the multiply (g is uniform over the scene, so the branch does not diverge)
    const bool mf = finiteBits(mass);
    F.x = (zeroBits(P.gravity[0]) && mf) ? signedZero(mass, P.gravity[0]) : mass * P.gravity[0];
    F.y = (zeroBits(P.gravity[1]) && mf) ? signedZero(mass, P.gravity[1]) : mass * P.gravity[1];
    F.z = (zeroBits(P.gravity[2]) && mf) ? signedZero(mass, P.gravity[2]) : mass * P.gravity[2];
  } else F = mk(0, 0, 0);
  T = mk(0, 0, 0);
  gatherRow(want, i, c, csr, F, T);
}

// Raises the collider trigger.  All particles of a free-falling cloud cross the verlet distance in the
// same step, and a million stores to one word serialise in the memory system: one store per warp, and
// none once the flag is seen set.
__device__ __forceinline__ void raiseDirty(DeviceStatus* st, bool dirty, long long step) {
  const unsigned am = __activemask();
  const unsigned b = __ballot_sync(am, dirty);
  if (b && (threadIdx.x & 31) == (unsigned)(__ffs(b) - 1))
    if (*(volatile int*)&st->dirty == 0) {
      st->dirty = 1;
      st->haltAt = step + 1;
    }
}

// Quaternion::toRotationMatrix (Eigen's formula), row-major
__device__ __forceinline__ void quatToMat(qd q, double* m) {
  const double tx = 2 * q.x, ty = 2 * q.y, tz = 2 * q.z;
  const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
  const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
  const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
  m[0] = 1 - (tyy + tzz); m[1] = txy - twz;       m[2] = txz + twy;
  m[3] = txy + twz;       m[4] = 1 - (txx + tzz); m[5] = tyz - twx;
  m[6] = txz - twy;       m[7] = tyz + twx;       m[8] = 1 - (txx + tyy);
}
__device__ __forceinline__ double minc(d3 v) { double r = v.x; if (v.y < r) r = v.y; if (v.z < r) r = v.z; return r; }
// Leapfrog::DotQ (Leapfrog.cpp:325-331)
__device__ __forceinline__ qd dotQ(d3 w, qd Q) {
  qd d;
  d.w = (-Q.x * w.x - Q.y * w.y - Q.z * w.z) / 2;
  d.x = (Q.w * w.x - Q.z * w.y + Q.y * w.z) / 2;
  d.y = (Q.z * w.x + Q.w * w.y - Q.x * w.z) / 2;
  d.z = (-Q.y * w.x + Q.x * w.y + Q.w * w.z) / 2;
  return d;
}
// coefficient-wise q1 + q2 f (Woo's quaternion operator+ and scalar operator*)
__device__ __forceinline__ qd qaxpy(qd q1, double f, qd q2) {
  qd r;
  r.w = q1.w + q2.w * f; r.x = q1.x + q2.x * f; r.y = q1.y + q2.y * f; r.z = q1.z + q2.z * f;
  return r;
}
// Leapfrog::leapfrogAsphericalRotate (Leapfrog.cpp:299-322): angular momentum leapfrog in the body frame
__device__ __noinline__ void asphericalRotate(const StepParams& P, Particles p, int i, d3 M, d3 inertia, qd& ori,
                                              d3& angVel, double dt) {
  d3 am = xyz(p.angMom[i]);
  double A[9];
  qd oc;
  oc.w = ori.w; oc.x = -ori.x; oc.y = -ori.y; oc.z = -ori.z;
  quatToMat(oc, A);
  if (isnan(minc(am))) {
    // inertia.asDiagonal() * ori.conjugate() * angVel
    double DR[9];
    for (int r = 0; r < 3; r++) {
      const double Ir = r == 0 ? inertia.x : (r == 1 ? inertia.y : inertia.z);
      for (int k = 0; k < 3; k++) DR[3 * r + k] = Ir * A[3 * r + k];
    }
    am = mvec(DR, angVel);
  }
  const d3 l_n = am + (dt / 2) * M;
  const d3 l_b_n = mvec(A, l_n);
  const d3 w_b_n = mk(l_b_n.x / inertia.x, l_b_n.y / inertia.y, l_b_n.z / inertia.z);
  const qd dq_n = dotQ(w_b_n, ori);
  const qd q_half = qaxpy(ori, dt / 2, dq_n);
  am = am + dt * M;
  const d3 l_b_h = mvec(A, am);
  const d3 w_b_h = mk(l_b_h.x / inertia.x, l_b_h.y / inertia.y, l_b_h.z / inertia.z);
  const qd dq_h = dotQ(w_b_h, q_half);
  ori = qaxpy(ori, dt, dq_h);
  angVel = qrot(ori, w_b_h);
  ori = qnormalized(ori);
  p.angMom[i] = make_double4_32a(am.x, am.y, am.z, 0);
}
// .5 w^T (T^T diag(I) T) w, T = rotation matrix of ori, all nine products kept as in the reference
__device__ __noinline__ double asphericalErot(qd ori, d3 inertia, d3 w) {
  double T[9], TI[9], M[9];
  quatToMat(ori, T);
  const double I[9] = {inertia.x, 0, 0, 0, inertia.y, 0, 0, 0, inertia.z};
  for (int r = 0; r < 3; r++)
    for (int k = 0; k < 3; k++) TI[3 * r + k] = T[0 * 3 + r] * I[0 * 3 + k] + T[1 * 3 + r] * I[1 * 3 + k] + T[2 * 3 + r] * I[2 * 3 + k];
  for (int r = 0; r < 3; r++)
    for (int k = 0; k < 3; k++) M[3 * r + k] = TI[3 * r + 0] * T[0 * 3 + k] + TI[3 * r + 1] * T[1 * 3 + k] + TI[3 * r + 2] * T[2 * 3 + k];
  return .5 * dot(w, mvec(M, w));
}

template <bool FROM_ARRAYS, bool PERI, bool ELL>
__global__ void __launch_bounds__(256) k_leapfrog(StepParams P, Particles p, int n, Contacts c, Csr csr, DeviceStatus* st) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  const long long step = stepOf(P, st);
  if (i >= n || haltedIntegrator(st, step)) return;
  if (p.rowMask) p.rowMask[i] = 0;  // this path gathers whole rows; the marks of the last pass are consumed
  const int4 meta = p.meta[i];
  const unsigned flags = (unsigned)meta.w;
  const bool asph = ELL && (meta.x & META_ASPH);
  const double4_32a vm = p.velm[i];
  const double mass = vm.w;
  const bool blockedAll = (flags & 63u) == 63u;
  const bool blockedNone = (flags & 63u) == 0u;
  d3 F, T;
  if (FROM_ARRAYS) {
    F = xyz(p.force[i]);
    T = xyz(p.torque[i]);
  } else if (!blockedAll) {
    gatherForce(P, seqOf(P, st) - 1, i, mass, flags, c, csr, F, T);
  } else {
    // the force on a fully blocked node changes nothing in its motion; it is materialised only
    // when downloaded (k_reduce_forces)
    F = mk(0, 0, 0); T = mk(0, 0, 0);
  }
  const double dt = dtOf(P, meta.y);
  const double damping = P.damping;
  const bool damp = (damping != 0. && !(flags & WDEM_DAMPING_SKIP));
  d3 vel = xyz(vm);
  const double4_32a w4 = p.angw[i];
  d3 angVel = xyz(w4);
  const double4_32a pr = p.posr[i];
  d3 pos = xyz(pr);
  const d3 inertia = xyz(p.inert[i]);
  if (P.lfEnergy) {
    // Leapfrog::doDampingDissipation and doGravityWork (Leapfrog.cpp:53-74), mid-step values
    double eDamp = 0, eGrav = 0;
    if (damp && !(flags & WDEM_ENERGY_SKIP)) {
      const d3 av = mk(fabs(vel.x), fabs(vel.y), fabs(vel.z)), af = mk(fabs(F.x), fabs(F.y), fabs(F.z));
      const d3 aw = mk(fabs(angVel.x), fabs(angVel.y), fabs(angVel.z)), at = mk(fabs(T.x), fabs(T.y), fabs(T.z));
      eDamp = dot(av, af) * damping * dt + dot(aw, at) * damping * dt;
    }
    if (P.hasGravity && !(flags & WDEM_GRAVITY_SKIP)) {
      const d3 g = mk(P.gravity[0], P.gravity[1], P.gravity[2]);
      if (blockedNone) eGrav = -dot(g, vel) * mass * dt;
      else {
        if (!(flags & 1u)) eGrav = eGrav - g.x * vel.x * mass * dt;
        if (!(flags & 2u)) eGrav = eGrav - g.y * vel.y * mass * dt;
        if (!(flags & 4u)) eGrav = eGrav - g.z * vel.z * mass * dt;
      }
    }
    p.energy[EP_DAMP][i] = eDamp;
    p.energy[EP_GRAV][i] = eGrav;
  }
  // fluctuation velocities (Cell::pprevFluctVel / pprevFluctAngVel, HOMO_GRADV2; Cell.cpp:36-57)
  d3 vel0 = vel, angVel0 = angVel;
  if (PERI && !blockedAll) {
    vel0 = vel - mvec(P.gradV, pos - P.dt / 2 * vel);
    angVel0 = angVel - mk(P.spinVec[0], P.spinVec[1], P.spinVec[2]);
  }
  d3 linAccelE = mk(0, 0, 0), angAccelE = mk(0, 0, 0);
  if (!blockedAll) {
    d3 linAccel;
    if (blockedNone) linAccel = divBy(F, mass);
    else {
      linAccel = mk(0, 0, 0);
      if (!(flags & 1u)) linAccel.x = linAccel.x + qdiv(F.x, mass);
      if (!(flags & 2u)) linAccel.y = linAccel.y + qdiv(F.y, mass);
      if (!(flags & 4u)) linAccel.z = linAccel.z + qdiv(F.z, mass);
    }
    // nonviscDamp2nd (Leapfrog.cpp:33-35)
    if (damp) {
      const double hd = 0.5 * dt;
      linAccel.x = linAccel.x * (1 - damping * signum(F.x * (vel0.x + hd * linAccel.x)));
      linAccel.y = linAccel.y * (1 - damping * signum(F.y * (vel0.y + hd * linAccel.y)));
      linAccel.z = linAccel.z * (1 - damping * signum(F.z * (vel0.z + hd * linAccel.z)));
    }
    // v(t+dt/2): plain, or the homothetic GRADV2 form (Leapfrog.cpp:189-190)
    if (PERI) vel = mvec(P.ImLL4hInv, mvec(P.LmL, pos) + mvec(P.IpLL4h, vel) + linAccel * dt);
    else vel = vel + dt * linAccel;
    linAccelE = linAccel;
    // a zero torque adds zeros to angVel, which changes no bit unless angVel holds a -0 (then the
    // reference's addition may turn it into +0): skip only when that cannot happen
    const bool inertiaPositive = positiveBits(inertia.x) && positiveBits(inertia.y) && positiveBits(inertia.z);
    if (ELL && asph) {
      if (!isZeroBits(inertia)) {
        // aspherical: blocked rotational DOFs zero the torque, then nonviscDamp1st (Leapfrog.cpp:176-179, 29-31)
        if (flags & 8u) T.x = 0;
        if (flags & 16u) T.y = 0;
        if (flags & 32u) T.z = 0;
        if (damp) {
          T.x = T.x * (1 - damping * signum(T.x * angVel0.x));
          T.y = T.y * (1 - damping * signum(T.y * angVel0.y));
          T.z = T.z * (1 - damping * signum(T.z * angVel0.z));
        }
      }
    } else if (!isZeroBits(inertia) && (PERI || !(isZeroBits(T) && inertiaPositive && !hasNegZero(angVel)))) {
      d3 angAccel;
      if (blockedNone) angAccel = divByEach(T, inertia);
      else {
        angAccel = mk(0, 0, 0);
        if (!(flags & 8u)) angAccel.x = angAccel.x + qdiv(T.x, inertia.x);
        if (!(flags & 16u)) angAccel.y = angAccel.y + qdiv(T.y, inertia.y);
        if (!(flags & 32u)) angAccel.z = angAccel.z + qdiv(T.z, inertia.z);
      }
      if (damp) {
        const double hd = 0.5 * dt;
        angAccel.x = angAccel.x * (1 - damping * signum(T.x * (angVel0.x + hd * angAccel.x)));
        angAccel.y = angAccel.y * (1 - damping * signum(T.y * (angVel0.y + hd * angAccel.y)));
        angAccel.z = angAccel.z * (1 - damping * signum(T.z * (angVel0.z + hd * angAccel.z)));
      }
      angVel = angVel + dt * angAccel;
      if (PERI) angVel = angVel - mk(P.dSpin[0], P.dSpin[1], P.dSpin[2]);
      angAccelE = angAccel;
    }
  } else if (PERI) {
    // fixed node with GRADV2: velocity correction without acceleration (Leapfrog.cpp:207-211)
    vel = mvec(P.ImLL4hInv, mvec(P.LmL, pos) + mvec(P.IpLL4h, vel));
  }
  if (P.lfEnergy) {
    // Leapfrog::doKineticEnergy, spherical (Leapfrog.cpp:76-98): on-step velocities
    double ek = 0;
    if (!(flags & WDEM_ENERGY_SKIP)) {
      const d3 pv = blockedAll ? mk(0, 0, 0) : vel0, pw = blockedAll ? mk(0, 0, 0) : angVel0;
      const d3 cfv = pv + .5 * dt * linAccelE, cfa = pw + .5 * dt * angAccelE;
      const double Etrans = .5 * mass * sqnorm(cfv);
      double Erot;
      const bool aspherical = !(inertia.x == inertia.y && inertia.y == inertia.z);
      if (ELL && aspherical) {
        qd o;
        const double4_32a o4e = p.ori[i];
        o.w = o4e.x; o.x = o4e.y; o.y = o4e.z; o.z = o4e.w;
        Erot = asphericalErot(o, inertia, cfa);
      } else Erot = 0.5 * dot(cfa, mk(inertia.x * cfa.x, inertia.y * cfa.y, inertia.z * cfa.z));
      const double imax = dmax3(inertia);
      if (isnan(Erot) || isinf(imax)) Erot = 0;
      ek = Etrans + Erot;
    }
    p.energy[EP_KIN][i] = ek;
  }
  // leapfrogTranslate (:275-278)
  pos = mk(addMulExact(pos.x, vel.x, dt), addMulExact(pos.y, vel.y, dt), addMulExact(pos.z, vel.z, dt));
  // leapfrogSphericalRotate (:280-297): q = AngleAxis(|w| dt, w/|w|) * q, normalised
  double4_32a o4 = p.ori[i];
  qd ori; ori.w = o4.x; ori.x = o4.y; ori.y = o4.z; ori.z = o4.w;
  if (ELL && asph) {
    if (isZeroBits(inertia)) { if (atomicCAS(&st->code, 0, WDEM_ERR_STATE) == 0) st->detail = i; }
    else asphericalRotate(P, p, i, T, inertia, ori, angVel, dt);
  } else {
  if (!isZeroBits(angVel)) {
    double angle = sqrt(sqnorm(angVel));
    d3 axis = angVel / angle;
    double ha = 0.5 * (angle * dt);
    double sh, ch;
    sincos(ha, &sh, &ch);
    qd q; q.w = ch; q.x = sh * axis.x; q.y = sh * axis.y; q.z = sh * axis.z;
    ori = qmul(q, ori);
  }
  ori = qnormalized(ori);
  }
  p.posr[i] = make_double4_32a(pos.x, pos.y, pos.z, pr.w);
  p.posf[i] = make_float4((float)pos.x, (float)pos.y, (float)pos.z, (float)pr.w);
  p.velm[i] = make_double4_32a(vel.x, vel.y, vel.z, mass);
  p.angw[i] = make_double4_32a(angVel.x, angVel.y, angVel.z, w4.w);
  p.ori[i] = make_double4_32a(ori.w, ori.x, ori.y, ori.z);
  // a non-finite position can never be collided again (NaN boxes overlap nothing): stop with an error,
  // as Woo stops on a NaN force
  if (!finiteBits(pos.x) || !finiteBits(pos.y) || !finiteBits(pos.z)) {
    if (atomicCAS(&st->code, 0, WDEM_ERR_NAN) == 0) st->detail = i;
  }
  // aabbIsDirty, run by the collider right after Leapfrog: moved^2 > verletDist^2
  const double4_32a lp = p.lastPos[i];
  const d3 dd = mk(lp.x, lp.y, lp.z) - pos;
  if (!ELL) {
    raiseDirty(st, sqnorm(dd) > P.maxD2, step);
  } else {
    // rotation-aware trigger for bounds that track it (maxRot >= 0; Collision.cpp:94-121)
    double moveDueToRot2 = 0.;
    const double mr = p.maxRot[i];
    bool dirty = false;
    if (mr >= 0.) {
      const double4_32a l4 = p.lastOri[i];
      qd lc;
      lc.w = l4.x; lc.x = -l4.y; lc.y = -l4.z; lc.z = -l4.w;
      const qd dq = qmul(lc, ori);
      const double nv = sqrt(dq.x * dq.x + dq.y * dq.y + dq.z * dq.z);
      const double ang = (nv != 0) ? 2 * atan2(nv, fabs(dq.w)) : 0.;
      const double rot = fmax(0., fabs(ang));
      if (rot > mr) dirty = true;
      const double4_32a bmn = p.bbmin[i], bmx = p.bbmax[i];
      const double arm = dmax3(mk(bmx.x - bmn.x, bmx.y - bmn.y, bmx.z - bmn.z));
      const double mv = .5 * arm * rot;
      moveDueToRot2 = mv * mv;
    }
    const double d2 = sqnorm(dd);
    raiseDirty(st, dirty || (d2 > 0. ? d2 : 0.) + moveDueToRot2 > P.maxD2, step);
  }
}

// leapfrogSphericalRotate of a sphere with angVel != 0: q = AngleAxis(|w| dt, w/|w|) q, normalised.
// A sphere's orientation feeds nothing else in the step (sphere contacts do not read it): it is
// integrated to within a few ulp of the reference's operations at a fraction of their cost.  For the
// half angles of a DEM step (h = |w| dt/2 < 1e-3) the Taylor polynomials sin h = h (1 - h^2/6 (1 -
// h^2/20)) and cos h = 1 - h^2/2 (1 - h^2/12) (truncation errors h^7/5040 and h^6/720, far below an
// ulp) need neither |w| nor the axis: the vector part sin(h) w/|w| = w dt/2 (1 - h^2/6 (1 - h^2/20))
// with h^2 = |w|^2 dt^2/4.  The normalisation 1/sqrt(z) of a product of unit quaternions (|z - 1| a
// few ulp) is its Taylor polynomial 1 - e/2 + 3e^2/8, e = z - 1 (error 5e^3/16, far below an ulp).
__device__ __forceinline__ void rotateSphere(const StepParams& P, const Particles& p, unsigned i, d3 angVel, int mat) {
  const double4_32a o4 = p.ori[i];
  qd ori; ori.w = o4.x; ori.x = o4.y; ori.y = o4.z; ori.z = o4.w;
  const double dt = dtOf(P, mat);
  const double w2 = sqnorm(angVel);
  const double h2 = 0.25 * (w2 * (dt * dt));
  qd q;
  if (h2 < 1e-6) {
    const double f = (0.5 * dt) * (1.0 - h2 * (1.0 / 6.0) * (1.0 - h2 * 0.05));
    q.w = 1.0 - h2 * 0.5 * (1.0 - h2 * (1.0 / 12.0));
    q.x = angVel.x * f; q.y = angVel.y * f; q.z = angVel.z * f;
  } else {
    WDEM_REAL_BRANCH();
    const double angle = sqrt(w2);
    const double inv = 1.0 / angle;
    double sh, ch;
    sincos(0.5 * (angle * dt), &sh, &ch);
    q.w = ch; q.x = sh * (angVel.x * inv); q.y = sh * (angVel.y * inv); q.z = sh * (angVel.z * inv);
  }
  ori = qmul(q, ori);
  const double z2 = ori.x * ori.x + ori.y * ori.y + ori.z * ori.z + ori.w * ori.w;
  if (!isOneBits(z2)) {
    double rn;
    const double e = z2 - 1.0;
    if (fabs(e) < 1e-6) rn = 1.0 - e * (0.5 - 0.375 * e);
    else {
      WDEM_REAL_BRANCH();
      rn = z2 > 0 ? 1.0 / sqrt(z2) : 1.0;
    }
    ori.x *= rn; ori.y *= rn; ori.z *= rn; ori.w *= rn;
  }
  p.ori[i] = make_double4_32a(ori.w, ori.x, ori.y, ori.z);
}

// The same step as k_leapfrog<false, PERI, false> without energy tracking, for one particle, issuing
// fewer FP64 operations with bit-identical results:
//  - the CSR gather runs only for particles that a real contact touched in the last contact pass
//    (p.touched, set by the contact kernel; those run in k_leapfrog_lists); the others get m g;
//  - Sign(F (v + dt/2 a)) of the damping comes from the sign bits (signProd) and the factor
//    1 - damping Sign(...) from two constants; zero accelerations and velocities skip their updates
//    (addScaled: adding a zero changes only -0);
//  - the verlet trigger is decided in FP32 with an error margin from the FP32 shadows of the new and
//    the last-rebuild positions, and in FP64 only when the margin does not decide it;
//  - an orientation that does not rotate and that the last normalisation left unchanged (meta bit
//    META_ORI_FIXED) is neither normalised again nor rewritten;
//  - the FP32 shadow is written by mantissa truncation on the integer pipe.
// m g along one axis: the signed zero of a zero g, nothing when the value is not used, else the product
__device__ __forceinline__ double gravForce(double mass, bool massFinite, double g, bool unused) {
  if (zeroBits(g) && massFinite) return signedZero(mass, g);
  if (unused) return 0.0;
  WDEM_REAL_BRANCH();
  return mass * g;
}

// The particle's records (meta, velm, angw, posr, lastPosf) are loaded by the caller, all at once.
struct FastRec {
  int4 meta;
  double4_32a vm, w4, pr;
  float4 lf;
};
__device__ __forceinline__ FastRec loadFast(const Particles& p, int i) {
  FastRec r;
  r.meta = p.meta[i];
  r.vm = p.velm[i];
  r.w4 = p.angw[i];
  r.pr = p.posr[i];
  r.lf = p.lastPosf[i];
  return r;
}

template <bool PERI>
__device__ __forceinline__ void integrateFast(const StepParams& P, const Particles& p, const int i, const int n, const Contacts& c,
                                              const Csr& csr, DeviceStatus* st, const bool touchedNow, const FastRec& rec,
                                              const unsigned rowMask) {
  const int4 meta = rec.meta;
  const unsigned flags = (unsigned)meta.w;
  const double4_32a vm = rec.vm;
  const double mass = vm.w;
  const bool blockedAll = (flags & 63u) == 63u;
  const bool blockedNone = (flags & 63u) == 0u;
  d3 F, T;
  const bool grav = P.hasGravity && !(flags & WDEM_GRAVITY_SKIP);
  const bool damp = (P.dampOn && !(flags & WDEM_DAMPING_SKIP));
  // the gravity-only path takes its acceleration from the cache; without damping nothing reads m g
  // along the gravity axis then
  const int skipAxis = (blockedNone && grav && !touchedNow && P.gravAxis >= 0 && !damp) ? P.gravAxis : -1;
  if (!blockedAll) {
    if (grav) {
      const bool mf = finiteBits(mass);
      F = mk(gravForce(mass, mf, P.gravity[0], skipAxis == 0), gravForce(mass, mf, P.gravity[1], skipAxis == 1),
             gravForce(mass, mf, P.gravity[2], skipAxis == 2));
    } else F = mk(0, 0, 0);
    T = mk(0, 0, 0);
    if (touchedNow) gatherRowMasked(seqOf(P, st) - 1, i, rowMask, c, csr, F, T);
  } else {
    F = mk(0, 0, 0); T = mk(0, 0, 0);
  }
  const double dt = dtOf(P, meta.y);
  d3 vel = xyz(vm);
  const double4_32a w4 = rec.w4;
  const double4_32a& w4c = w4;
  d3 angVel = xyz(w4);
  bool angChanged = false;
  const double4_32a pr = rec.pr;
  d3 pos = xyz(pr);
  if (!blockedAll) {
    d3 lin;
    if (blockedNone && grav && !touchedNow && P.gravAxis >= 0) {
      // F = m g exactly: the acceleration along the gravity axis is the cached qdiv(m g, m); the other
      // components are qdiv of signed zeros, i.e. the zeros themselves
      lin = F;
      if (P.gravAxis == 0) lin.x = w4c.w; else if (P.gravAxis == 1) lin.y = w4c.w; else lin.z = w4c.w;
    } else if (blockedNone) lin = divBy(F, mass);
    else {
      lin = mk(0, 0, 0);
      if (!(flags & 1u)) lin.x = lin.x + qdiv(F.x, mass);
      if (!(flags & 2u)) lin.y = lin.y + qdiv(F.y, mass);
      if (!(flags & 4u)) lin.z = lin.z + qdiv(F.z, mass);
    }
    if (damp) {
      // nonviscDamp2nd: a *= 1 - damping Sign(F (v + dt/2 a)); a zero F gives Sign 0 and factor 1.
      // Periodic: v is the fluctuation velocity v - gradV (x - dt/2 v) (Cell::pprevFluctVel)
      d3 v0 = vel;
      if (PERI) {
        const double hdt = P.dt / 2;
        const d3 w = mk(addZ(pos.x, negD(mulZ(vel.x, hdt))), addZ(pos.y, negD(mulZ(vel.y, hdt))),
                        addZ(pos.z, negD(mulZ(vel.z, hdt))));
        const d3 g = mvecC(P.gradV, P.clsGradV, w);
        v0 = mk(addZ(vel.x, negD(g.x)), addZ(vel.y, negD(g.y)), addZ(vel.z, negD(g.z)));
      }
      const double hd = 0.5 * dt;
      if (!zeroBits(F.x)) { const int sg = signProd(F.x, v0.x + hd * lin.x); if (sg) lin.x = lin.x * (sg > 0 ? P.dampM : P.dampP); }
      if (!zeroBits(F.y)) { const int sg = signProd(F.y, v0.y + hd * lin.y); if (sg) lin.y = lin.y * (sg > 0 ? P.dampM : P.dampP); }
      if (!zeroBits(F.z)) { const int sg = signProd(F.z, v0.z + hd * lin.z); if (sg) lin.z = lin.z * (sg > 0 ? P.dampM : P.dampP); }
    }
    if (PERI) {
      // GRADV2 (Leapfrog.cpp:189-190): v = (I - dt(L+ + L-)/4)^-1 ((L+ - L-) x + (I + dt(L+ + L-)/4) v + a dt)
      const d3 a = mvecC(P.LmL, P.clsLmL, pos);
      const d3 b = mvecC(P.IpLL4h, P.clsIpLL4h, vel);
      const d3 sum = mk(addZ(addZ(a.x, b.x), mulZ(lin.x, dt)), addZ(addZ(a.y, b.y), mulZ(lin.y, dt)),
                        addZ(addZ(a.z, b.z), mulZ(lin.z, dt)));
      vel = mvecC(P.ImLL4hInv, P.clsImLL4hInv, sum);
    } else {
      vel.x = addScaled(vel.x, dt, lin.x);
      vel.y = addScaled(vel.y, dt, lin.y);
      vel.z = addScaled(vel.z, dt, lin.z);
    }
    if (!isZeroBits(T)) {
      WDEM_REAL_BRANCH();
      const d3 inertia = xyz(p.inert[i]);
      if (!isZeroBits(inertia)) {
        d3 ang;
        if (blockedNone) ang = divByEach(T, inertia);
        else {
          ang = mk(0, 0, 0);
          if (!(flags & 8u)) ang.x = ang.x + qdiv(T.x, inertia.x);
          if (!(flags & 16u)) ang.y = ang.y + qdiv(T.y, inertia.y);
          if (!(flags & 32u)) ang.z = ang.z + qdiv(T.z, inertia.z);
        }
        if (damp) {
          const double hd = 0.5 * dt;
          // periodic: the fluctuation spin angVel - spinVec (Cell::pprevFluctAngVel)
          const d3 w0 = PERI ? mk(addZ(angVel.x, negD(P.spinVec[0])), addZ(angVel.y, negD(P.spinVec[1])),
                                  addZ(angVel.z, negD(P.spinVec[2])))
                             : angVel;
          if (!zeroBits(T.x)) { const int sg = signProd(T.x, w0.x + hd * ang.x); if (sg) ang.x = ang.x * (sg > 0 ? P.dampM : P.dampP); }
          if (!zeroBits(T.y)) { const int sg = signProd(T.y, w0.y + hd * ang.y); if (sg) ang.y = ang.y * (sg > 0 ? P.dampM : P.dampP); }
          if (!zeroBits(T.z)) { const int sg = signProd(T.z, w0.z + hd * ang.z); if (sg) ang.z = ang.z * (sg > 0 ? P.dampM : P.dampP); }
        }
        angVel.x = addScaled(angVel.x, dt, ang.x);
        angVel.y = addScaled(angVel.y, dt, ang.y);
        angVel.z = addScaled(angVel.z, dt, ang.z);
        angChanged = true;
      }
    } else {
      // a zero torque still divides by the inertia and adds to angVel: that changes angVel only when an
      // inertia component is not positive (0/0, 0/negative) or angVel holds a -0
      if (!(meta.x & META_IPOS) || hasNegZero(angVel)) {
        WDEM_REAL_BRANCH();
        const d3 inertia = xyz(p.inert[i]);
        if (!isZeroBits(inertia)) {
          d3 ang;
          if (blockedNone) ang = divByEach(T, inertia);
          else {
            ang = mk(0, 0, 0);
            if (!(flags & 8u)) ang.x = ang.x + qdiv(T.x, inertia.x);
            if (!(flags & 16u)) ang.y = ang.y + qdiv(T.y, inertia.y);
            if (!(flags & 32u)) ang.z = ang.z + qdiv(T.z, inertia.z);
          }
          angVel = angVel + dt * ang;
          angChanged = true;
        }
      }
    }
    // periodic spin correction angVel -= deltaSpinVec (Leapfrog.cpp:192-197), for nodes with inertia;
    // subtracting +0 leaves every value unchanged
    if (PERI && !P.dSpinZero) {
      const double4_32a in4 = p.inert[i];
      if (!isZeroBits(xyz(in4))) {
        angVel = mk(addZ(angVel.x, negD(P.dSpin[0])), addZ(angVel.y, negD(P.dSpin[1])), addZ(angVel.z, negD(P.dSpin[2])));
        angChanged = true;
      }
    }
  } else if (PERI) {
    // fixed node with GRADV2: velocity correction without acceleration (Leapfrog.cpp:207-211)
    const d3 a = mvecC(P.LmL, P.clsLmL, pos);
    const d3 b = mvecC(P.IpLL4h, P.clsIpLL4h, vel);
    vel = mvecC(P.ImLL4hInv, P.clsImLL4hInv, mk(addZ(a.x, b.x), addZ(a.y, b.y), addZ(a.z, b.z)));
  }
  pos.x = addScaledR(pos.x, vel.x, dt);
  pos.y = addScaledR(pos.y, vel.y, dt);
  pos.z = addScaledR(pos.z, vel.z, dt);
  // leapfrogSphericalRotate; an unrotated, already-normalised orientation is left alone
  int mx = meta.x;
  bool rotate = false;
  if (!isZeroBits(angVel)) {
    // untouched spheres: rotated from the rotation list in the second pass (spinning spheres are
    // scattered over most warps, whose FP64 pipe would wait for their few spinning lanes); the second
    // pass's own (touched) particles rotate here
    rotate = true;
    mx &= ~META_ORI_FIXED;
  } else if (!(mx & META_ORI_FIXED)) {
    const double4_32a o4 = p.ori[i];
    qd ori; ori.w = o4.x; ori.x = o4.y; ori.y = o4.z; ori.z = o4.w;
    const double z2 = ori.x * ori.x + ori.y * ori.y + ori.z * ori.z + ori.w * ori.w;
    if (isOneBits(z2)) mx |= META_ORI_FIXED;  // normalisation is the identity from now on
    else {
      ori = qnormalized(ori);
      p.ori[i] = make_double4_32a(ori.w, ori.x, ori.y, ori.z);
    }
  }
  if (mx != meta.x) reinterpret_cast<int*>(&p.meta[i])[0] = mx;
  p.posr[i] = make_double4_32a(pos.x, pos.y, pos.z, pr.w);
  const float4 pf = make_float4(truncF(pos.x), truncF(pos.y), truncF(pos.z), truncF(pr.w));
  p.posf[i] = pf;
  p.velm[i] = make_double4_32a(vel.x, vel.y, vel.z, mass);
  if (angChanged) p.angw[i] = make_double4_32a(angVel.x, angVel.y, angVel.z, w4.w);
  if (!finiteBits(pos.x) || !finiteBits(pos.y) || !finiteBits(pos.z)) {
    if (atomicCAS(&st->code, 0, WDEM_ERR_NAN) == 0) st->detail = i;
  }
  if (touchedNow) {
    if (rotate) rotateSphere(P, p, (unsigned)i, angVel, meta.y);
  } else {
    const unsigned am = __activemask();
    const unsigned b = __ballot_sync(am, rotate);
    if (b) {
      const int lane = threadIdx.x & 31, leader = __ffs(b) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(&st->rotCount, (unsigned)__popc(b));
      base = __shfl_sync(am, base, leader);
      const unsigned slot = base + __popc(b & ((1u << lane) - 1));
      if (rotate && slot < (unsigned)n) p.rotList[slot] = (unsigned)i;
    }
  }
  // aabbIsDirty (moved^2 > verletDist^2): FP32 distance of the shadows with a bound on its error
  // (truncation < 2^-23 relative per coordinate, FP32 arithmetic a few 2^-24 of the distance)
  const float4 lf = rec.lf;
  const float dx = pf.x - lf.x, dy = pf.y - lf.y, dz = pf.z - lf.z;
  const float df = sqrtf(dx * dx + dy * dy + dz * dz);
  const float S = fabsf(pf.x) + fabsf(pf.y) + fabsf(pf.z) + fabsf(lf.x) + fabsf(lf.y) + fabsf(lf.z);
  const float err = 2.5e-7f * S + 1e-6f * df;
  bool dirty = false;
  if (!(df + err < P.verletLoF)) {
    WDEM_REAL_BRANCH();
    const double4_32a lp = p.lastPos[i];
    const d3 dd = mk(lp.x, lp.y, lp.z) - pos;
    dirty = sqnorm(dd) > P.maxD2;
  }
  raiseDirty(st, dirty, stepOf(P, st));
}

// First pass: particles without contact forces this step.  Those that a real contact touched are
// compacted into touchList instead: their force gather and divisions would hold up the FP64 pipe
// for whole warps of gravity-only neighbours.  DENSE (many real contacts): a block that has touched
// particles also compacts its other particles to its first threads, so that their FP64 work issues in
// full warps, and appends its touched ones with one atomic.
template <bool PERI, int BS, bool DENSE>
__global__ void __launch_bounds__(BS, 1024 / BS) k_leapfrog_fast(StepParams P, Particles p, int n, Contacts c, Csr csr,
                                                               DeviceStatus* st) {
  if constexpr (!DENSE) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // all of the particle's loads are issued together, before the guard's and the list decision
    const FastRec rec = loadFast(p, i);
    const uint8_t tch = p.touched[i];
    if (haltedIntegrator(st, stepOf(P, st))) return;
    const bool listed = ((unsigned)rec.meta.w & 63u) != 63u && tch != 0;
    const unsigned am = __activemask();
    const unsigned b = __ballot_sync(am, listed);
    if (b) {
      const int lane = threadIdx.x & 31, leader = __ffs(b) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(&st->touchCount, (unsigned)__popc(b));
      base = __shfl_sync(am, base, leader);
      const unsigned slot = base + __popc(b & ((1u << lane) - 1));
      if (listed && slot < (unsigned)n) p.touchList[slot] = (unsigned)i;
    }
    if (listed) return;
    integrateFast<PERI>(P, p, i, n, c, csr, st, false, rec, 0u);
  } else {
    constexpr int NW = BS / 32;
    __shared__ unsigned sCnt[2][NW];
    __shared__ int sIdx[BS];
    __shared__ unsigned sBase;
    const int i = blockIdx.x * BS + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const bool live = i < n;
    FastRec rec;
    uint8_t tch = 0;
    if (live) {
      rec = loadFast(p, i);
      tch = p.touched[i];
    }
    const bool run = live && !haltedIntegrator(st, stepOf(P, st));
    const bool listed = run && ((unsigned)rec.meta.w & 63u) != 63u && tch != 0;
    const bool own = run && !listed;
    // every thread of the block reaches the barriers: none returns before them
    const unsigned lt = (1u << lane) - 1u;
    const unsigned bl = __ballot_sync(0xffffffffu, listed), bo = __ballot_sync(0xffffffffu, own);
    if (lane == 0) {
      sCnt[0][w] = (unsigned)__popc(bl);
      sCnt[1][w] = (unsigned)__popc(bo);
    }
    __syncthreads();
    unsigned preL = 0, preO = 0, nL = 0, nO = 0;
#pragma unroll
    for (int k = 0; k < NW; ++k) {
      const unsigned a = sCnt[0][k], b = sCnt[1][k];
      if (k < w) {
        preL += a;
        preO += b;
      }
      nL += a;
      nO += b;
    }
    bool mine = own;
    int j = i;
    if (nL != 0) {  // the same for every thread of the block
      if (threadIdx.x == 0) sBase = atomicAdd(&st->touchCount, nL);
      if (own) sIdx[preO + (unsigned)__popc(bo & lt)] = i;
      __syncthreads();
      if (listed) {
        const unsigned slot = sBase + preL + (unsigned)__popc(bl & lt);
        if (slot < (unsigned)n) p.touchList[slot] = (unsigned)i;
      }
      mine = threadIdx.x < nO;
      j = mine ? sIdx[threadIdx.x] : i;
      if (mine && j != i) rec = loadFast(p, j);  // the block loaded it a moment ago
    }
    if (!mine) return;
    integrateFast<PERI>(P, p, j, n, c, csr, st, false, rec, 0u);
  }
}

// Second pass, over two lists: the touched particles (CSR force gather, full integration, rotation
// inline), then the rotation list of the first pass.
template <bool PERI>
__global__ void __launch_bounds__(256) k_leapfrog_lists(StepParams P, Particles p, int n, Contacts c, Csr csr,
                                                         DeviceStatus* st) {
  if (haltedIntegrator(st, stepOf(P, st))) return;
  const unsigned nt = st->touchCount < (unsigned)n ? st->touchCount : (unsigned)n;
  const unsigned nr = st->rotCount < (unsigned)n ? st->rotCount : (unsigned)n;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < nt + nr; k += gridDim.x * blockDim.x) {
    if (k < nt) {
      const int i = (int)p.touchList[k];
      p.touched[i] = 0;
      const unsigned m = p.rowMask[i];
      p.rowMask[i] = 0;
      integrateFast<PERI>(P, p, i, n, c, csr, st, true, loadFast(p, i), m);
    } else {
      const unsigned i = p.rotList[k - nt];
      rotateSphere(P, p, i, xyz(p.angw[i]), p.meta[i].y);
    }
  }
}

// resident blocks of the list pass on the whole GPU (one wave; queried once per instantiation), or the
// launch shape's blocks per SM
template <bool PERI>
static unsigned listGrid(const StepParams& P) {
  static int per = 0;
  if (per == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_leapfrog_lists<PERI>, 256, 0);
    per = std::max(1, per);
  }
  const int sms = P.numSMs > 0 ? P.numSMs : 152;
  const int want = P.shListsPerSM > 0 ? std::min(P.shListsPerSM, per) : per;
  return (unsigned)sms * (unsigned)want;
}
// the first pass with the block size of the launch shape; the block-compacting one when the last step the
// host saw had many real contacts (either is exact: they differ only in which thread integrates a particle)
template <bool PERI>
static void launchFast(cudaStream_t s, const StepParams& P, Particles p, int n, Contacts c, Csr csr, DeviceStatus* st) {
  const int bs = P.shLeapBlock == 128 || P.shLeapBlock == 512 ? P.shLeapBlock : 256;
  const unsigned blocks = (unsigned)((n + bs - 1) / bs);
  if (P.denseTouch) {
    if (bs == 128) k_leapfrog_fast<PERI, 128, true><<<blocks, 128, 0, s>>>(P, p, n, c, csr, st);
    else if (bs == 512) k_leapfrog_fast<PERI, 512, true><<<blocks, 512, 0, s>>>(P, p, n, c, csr, st);
    else k_leapfrog_fast<PERI, 256, true><<<blocks, 256, 0, s>>>(P, p, n, c, csr, st);
  } else {
    if (bs == 128) k_leapfrog_fast<PERI, 128, false><<<blocks, 128, 0, s>>>(P, p, n, c, csr, st);
    else if (bs == 512) k_leapfrog_fast<PERI, 512, false><<<blocks, 512, 0, s>>>(P, p, n, c, csr, st);
    else k_leapfrog_fast<PERI, 256, false><<<blocks, 256, 0, s>>>(P, p, n, c, csr, st);
  }
  ++::wdem::g_kernel_launches;
}

void launch_leapfrog(cudaStream_t s, const StepParams& P, Particles p, int n, int fromArrays, Contacts c, Csr csr,
                     DeviceStatus* st) {
  if (n <= 0) return;
  unsigned blocks = (n + 255) / 256;
  if (!fromArrays && !P.hasEll && !P.lfEnergy && p.touched && p.rotList) {
    // st->rotCount and st->touchCount are zero here: k_contacts_cull clears them for the next step (and
    // the handle starts at zero)
    if (P.periodic) {
      const unsigned rb = std::min(blocks, listGrid<true>(P));
      launchFast<true>(s, P, p, n, c, csr, st);
      (k_leapfrog_lists<true><<<rb, 256, 0, s>>>(P, p, n, c, csr, st), ++::wdem::g_kernel_launches);
    } else {
      const unsigned rb = std::min(blocks, listGrid<false>(P));
      launchFast<false>(s, P, p, n, c, csr, st);
      (k_leapfrog_lists<false><<<rb, 256, 0, s>>>(P, p, n, c, csr, st), ++::wdem::g_kernel_launches);
    }
    return;
  }
  if (P.hasEll) {
    if (fromArrays) (k_leapfrog<true, false, true><<<blocks, 256, 0, s>>>(P, p, n, c, csr, st), ++::wdem::g_kernel_launches);
    else (k_leapfrog<false, false, true><<<blocks, 256, 0, s>>>(P, p, n, c, csr, st), ++::wdem::g_kernel_launches);
  } else if (P.periodic) {
    if (fromArrays) (k_leapfrog<true, true, false><<<blocks, 256, 0, s>>>(P, p, n, c, csr, st), ++::wdem::g_kernel_launches);
    else (k_leapfrog<false, true, false><<<blocks, 256, 0, s>>>(P, p, n, c, csr, st), ++::wdem::g_kernel_launches);
  } else {
    if (fromArrays) (k_leapfrog<true, false, false><<<blocks, 256, 0, s>>>(P, p, n, c, csr, st), ++::wdem::g_kernel_launches);
    else (k_leapfrog<false, false, false><<<blocks, 256, 0, s>>>(P, p, n, c, csr, st), ++::wdem::g_kernel_launches);
  }
}

// DynDt::nodalCritDtSq (DynDt.cpp:46-63) with nodalStiffAdd (DynDt.cpp:16-38): the squared critical
// step of a node from the stiffnesses of its real contacts, visited in the order of the partner ids
// (Particle::contacts, a map by id); the contact normal is the contact node's orientation applied to
// the x axis, Eigen's n.array().pow(2) is the squares n*n, L6Geom.lens of sphere contacts are the radii
// (a wall's lens is the sphere's radius).  The minimum over nodes is exact in any order: positive
// doubles order as their bit patterns (kept complemented, so that zero means none).
__global__ void k_dyndt(StepParams P, Particles p, int n, Contacts c, Csr csr, DeviceStatus* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned flags = (unsigned)p.meta[i].w;
  if ((flags & 63u) == 63u) return;  // completely blocked: always stable (Inf)
  d3 kt3 = mk(0, 0, 0), kr3 = mk(0, 0, 0);
  const int e0 = csr.rowptr[i], e1 = csr.rowptr[i + 1];
  for (int e = e0; e < e1; e++) {
    const unsigned en = csr.ent[e];
    const unsigned ci = en & 0x7fffffffu;
    if ((c.state[ci] & CS_MASK) != CS_REAL) continue;
    const bool isB = (en >> 31) != 0;
    const double kn = c.hist[HIST_KN][ci], kt = c.hist[HIST_KT][ci];
    const d3 c0 = mk(c.hist[HIST_T0X][ci], c.hist[HIST_T0Y][ci], c.hist[HIST_T0Z][ci]);
    const d3 c1 = mk(c.hist[HIST_T1X][ci], c.hist[HIST_T1Y][ci], c.hist[HIST_T1Z][ci]);
    const qd ori = quatFromCols(c0, c1, cross(c0, c1));
    const d3 nrm = qrot(ori, mk(1, 0, 0));
    const d3 n2 = mk(nrm.x * nrm.x, nrm.y * nrm.y, nrm.z * nrm.z);
    const double knt = kn - kt;
    kt3 = mk(kt3.x + (n2.x * knt + kt), kt3.y + (n2.y * knt + kt), kt3.z + (n2.z * knt + kt));
    // lens[ix]: the radius of this node's sphere; a wall takes the sphere's (|-r|)
    const int2 id = c.ids[ci];
    const int other = isB ? id.x : id.y;
    const bool wallA = (c.state[ci] & CS_WALL_A) != 0;
    const double len = (!isB && wallA) ? p.posr[other].w : p.posr[i].w;
    const double sc = (len * len) * kt;
    kr3 = mk(kr3.x + sc * (n2.y + n2.z), kr3.y + sc * (n2.z + n2.x), kr3.z + sc * (n2.x + n2.y));
  }
  const double mass = p.velm[i].w;
  const d3 inertia = xyz(p.inert[i]);
  double ret = __longlong_as_double(0x7ff0000000000000ll);
  const double kt[3] = {kt3.x, kt3.y, kt3.z}, kr[3] = {kr3.x, kr3.y, kr3.z}, in[3] = {inertia.x, inertia.y, inertia.z};
  for (int k = 0; k < 3; k++)
    if (kt[k] != 0 && mass > 0. && !(flags & (1u << k))) { const double v = mass / fabs(kt[k]); ret = v < ret ? v : ret; }
  for (int k = 0; k < 3; k++)
    if (kr[k] != 0 && in[k] > 0. && !(flags & (8u << k))) { const double v = in[k] / fabs(kr[k]); ret = v < ret ? v : ret; }
  ret = 2 * ret;
  if (!(ret < __longlong_as_double(0x7ff0000000000000ll))) return;  // Inf (or NaN): no bound from this node
  atomicMax(&st->dynNotMin, ~(unsigned long long)__double_as_longlong(ret));
}

void launch_dyndt(cudaStream_t s, const StepParams& P, Particles p, int n, Contacts c, Csr csr, DeviceStatus* st) {
  if (n <= 0) return;
  (k_dyndt<<<(n + 127) / 128, 128, 0, s>>>(P, p, n, c, csr, st), ++::wdem::g_kernel_launches);
}

// DemData.force/torque as Woo holds them after ContactLoop (reset to m*g by Leapfrog, then contacts)
__global__ void k_reduce_forces(StepParams P, Particles p, int n, Contacts c, Csr csr) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 meta = p.meta[i];
  d3 F, T;
  gatherForce(P, P.seq - 1, i, p.velm[i].w, (unsigned)meta.w, c, csr, F, T);
  p.force[i] = make_double4_32a(F.x, F.y, F.z, 0);
  p.torque[i] = make_double4_32a(T.x, T.y, T.z, 0);
}

void launch_reduce_forces(cudaStream_t s, const StepParams& P, Particles p, int n, Contacts c, Csr csr) {
  if (n <= 0) return;
  (k_reduce_forces<<<(n + 127) / 128, 128, 0, s>>>(P, p, n, c, csr), ++::wdem::g_kernel_launches);
}

WDEM_VARIANT_END
}  // namespace wdem

namespace wdem {
WDEM_VARIANT_BEGIN

// Kinematic state exchange with caller buffers (xyz-interleaved / wxyz) through a device staging
// area: scatter into the double4 records, or gather out of them.
__global__ void k_state_in(Particles p, int n, const double* pos, const double* vel, const double* angVel,
                           const double* ori) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (pos) {
    double4_32a v = p.posr[i]; v.x = pos[3 * i]; v.y = pos[3 * i + 1]; v.z = pos[3 * i + 2]; p.posr[i] = v;
    p.posf[i] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
  }
  if (vel) { double4_32a v = p.velm[i]; v.x = vel[3 * i]; v.y = vel[3 * i + 1]; v.z = vel[3 * i + 2]; p.velm[i] = v; }
  if (angVel) { double4_32a v = p.angw[i]; v.x = angVel[3 * i]; v.y = angVel[3 * i + 1]; v.z = angVel[3 * i + 2]; p.angw[i] = v; }
  if (ori) {
    p.ori[i] = make_double4_32a(ori[4 * i], ori[4 * i + 1], ori[4 * i + 2], ori[4 * i + 3]);
    reinterpret_cast<int*>(&p.meta[i])[0] &= ~META_ORI_FIXED;
  }
}
__global__ void k_state_out(Particles p, int n, double* pos, double* vel, double* angVel, double* ori) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (pos) { double4_32a v = p.posr[i]; pos[3 * i] = v.x; pos[3 * i + 1] = v.y; pos[3 * i + 2] = v.z; }
  if (vel) { double4_32a v = p.velm[i]; vel[3 * i] = v.x; vel[3 * i + 1] = v.y; vel[3 * i + 2] = v.z; }
  if (angVel) { double4_32a v = p.angw[i]; angVel[3 * i] = v.x; angVel[3 * i + 1] = v.y; angVel[3 * i + 2] = v.z; }
  if (ori) { double4_32a v = p.ori[i]; ori[4 * i] = v.x; ori[4 * i + 1] = v.y; ori[4 * i + 2] = v.z; ori[4 * i + 3] = v.w; }
}
void launch_state_in(cudaStream_t s, Particles p, int n, const double* pos, const double* vel, const double* angVel,
                     const double* ori) {
  if (n > 0) (k_state_in<<<(n + 255) / 256, 256, 0, s>>>(p, n, pos, vel, angVel, ori), ++::wdem::g_kernel_launches);
}
void launch_state_out(cudaStream_t s, Particles p, int n, double* pos, double* vel, double* angVel, double* ori) {
  if (n > 0) (k_state_out<<<(n + 255) / 256, 256, 0, s>>>(p, n, pos, vel, angVel, ori), ++::wdem::g_kernel_launches);
}

WDEM_VARIANT_END
}  // namespace wdem

namespace wdem {
WDEM_VARIANT_BEGIN

// FP64 issue-rate probe: independent chains of fused multiply-adds (explicit __fma_rn, so the
// no-contraction build flag does not split them).  2 flops per FMA.
__global__ void k_fp64_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
  double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
  for (int k = 0; k < iters; k++) {
    x0 = __fma_rn(x0, a, b); x1 = __fma_rn(x1, a, b); x2 = __fma_rn(x2, a, b); x3 = __fma_rn(x3, a, b);
    x4 = __fma_rn(x4, a, b); x5 = __fma_rn(x5, a, b); x6 = __fma_rn(x6, a, b); x7 = __fma_rn(x7, a, b);
  }
  double r = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (r == 1234.5678) out[blockIdx.x] = r;  // keeps the chains alive
}

double fp64_probe(cudaStream_t s, double* scratch, int sms, float* msOut) {
  const int iters = 4096, threads = 256, blocks = sms * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  (k_fp64_probe<<<blocks, threads, 0, s>>>(scratch, iters, 0.999999, 1e-7), ++::wdem::g_kernel_launches);  // warm-up
  cudaEventRecord(e0, s);
  (k_fp64_probe<<<blocks, threads, 0, s>>>(scratch, iters, 0.999999, 1e-7), ++::wdem::g_kernel_launches);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  if (msOut) *msOut = ms;
  double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
  return ms > 0 ? flops / (ms * 1e-3) / 1e9 : 0.0;
}

WDEM_VARIANT_END
}  // namespace wdem

namespace wdem {
WDEM_VARIANT_BEGIN
__global__ void k_refresh_posf(Particles p, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4_32a v = p.posr[i];
  p.posf[i] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
}
void launch_refresh_posf(cudaStream_t s, Particles p, int n) {
  if (n > 0) (k_refresh_posf<<<(n + 255) / 256, 256, 0, s>>>(p, n), ++::wdem::g_kernel_launches);
}

// The acceleration of a particle that only gravity acts on, qdiv(m g, m) with the integrator's own
// operations, cached in angw.w so that the integrator does not repeat the division every step.
__global__ void k_grav_acc(StepParams P, Particles p, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4_32a w = p.angw[i];
  if (P.gravAxis >= 0) {
    const double m = p.velm[i].w;
    w.w = qdiv(m * P.gravity[P.gravAxis], m);
  } else w.w = 0.;
  p.angw[i] = w;
}
void launch_grav_acc(cudaStream_t s, const StepParams& P, Particles p, int n) {
  if (n > 0) (k_grav_acc<<<(n + 255) / 256, 256, 0, s>>>(P, p, n), ++::wdem::g_kernel_launches);
}
WDEM_VARIANT_END
}  // namespace wdem

namespace wdem {
WDEM_VARIANT_BEGIN

// Deterministic sum: each block reduces a fixed slice in a fixed shared-memory tree, then one block
// sums the block partials the same way.  The result is independent of scheduling.
static const int ER_T = 256;
__global__ void k_esum(const double* x, long long n, double* partials) {
  __shared__ double sh[ER_T];
  long long base = (long long)blockIdx.x * ER_T * 8;
  double acc = 0;
  for (int k = 0; k < 8; k++) {
    long long i = base + (long long)k * ER_T + threadIdx.x;
    if (i < n) acc = acc + x[i];
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int off = ER_T / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}
__global__ void k_efinal(const double* partials, long long nb, double* acc, int reset) {
  __shared__ double sh[ER_T];
  double a = 0;
  for (long long i = threadIdx.x; i < nb; i += ER_T) a = a + partials[i];
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int off = ER_T / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) *acc = reset ? sh[0] : *acc + sh[0];
}
void energy_accumulate(cudaStream_t s, const double* x, long long n, double* partials, double* acc, bool reset) {
  long long nb = (n + ER_T * 8 - 1) / (ER_T * 8);
  if (nb > 0) (k_esum<<<(unsigned)nb, ER_T, 0, s>>>(x, n, partials), ++::wdem::g_kernel_launches);
  (k_efinal<<<1, ER_T, 0, s>>>(partials, nb, acc, reset ? 1 : 0), ++::wdem::g_kernel_launches);
}

WDEM_VARIANT_END
}  // namespace wdem
