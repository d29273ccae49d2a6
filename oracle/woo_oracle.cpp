/*
 * woo_oracle.cpp -- CPU ORACLE for the GB300 DEM engine.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++17 restatement of woodem/woo's DEM timestep (Leapfrog -> InsertionSortCollider ->
 * ContactLoop), written from the reference sources cited at each function.  The CUDA engine's results
 * are compared with it: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * The product library (libwdem.so) never links or calls it.
 *
 * Build: oracle/build.sh (g++ -O2 -std=c++17 -ffp-contract=off -fPIC -shared [-fopenmp]).
 * -ffp-contract=off keeps every a*b+c as two IEEE operations, as the reference's x86-64 build does.
 *
 * Pinning: Woo cannot be compiled here (Eigen3 and Boost are absent), so this restatement is pinned
 * by the reference's own known-answer tests re-stated in tests/test_oracle_known_answers.py
 * (py/tests/test_hertz.py:30-47 collision time, py/tests/test_demfield.py:24-51 updatePhys,
 * py/tests/test_energy.py gravity/damping skips) and by analytic cases.
 *
 * Third-party arithmetic restated here: Eigen3 (unpinned version; Ubuntu 20.04 libeigen3-dev in the
 * reference CI): cross/dot/norm/normalize, 3x3 matrix-vector, Quaternion(Matrix3) (Shoemake's
 * trace/largest-diagonal method), quaternion*vector (v + 2w(q x v) + q x (2 q x v)), quaternion
 * product, AngleAxis -> Quaternion (cos(a/2), sin(a/2) axis).  Each is written from the published
 * formula; evaluation order follows Eigen's left-to-right expression evaluation.
 *
 * Two switches make the oracle reproduce the GPU engine's documented conventions exactly:
 *   canonicalOrient: a new contact between two particles of the same shape gets pA = lower id
 *     (the reference takes the order in which the insertion sort met the pair, an artefact of the
 *     sort; InsertionSortCollider.cpp:102, :579).
 *   applyOrder: 0 = forces added in container order (ContactLoop.cpp:195-197 / :257-264),
 *     1 = added per contact sorted by (min id, max id), the GPU's CSR order.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#include <chrono>
#include <array>
#ifdef _OPENMP
#include <omp.h>
#include <parallel/algorithm>
#endif

#include "../include/wdem.h"

namespace orc {

static const double Inf = std::numeric_limits<double>::infinity();
static const double NaN = std::numeric_limits<double>::quiet_NaN();

/* ------------------------------------------------------------------ small linear algebra */
struct V3 {
  double x = 0, y = 0, z = 0;
  V3() {}
  V3(double a, double b, double c) : x(a), y(b), z(c) {}
  double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline V3 operator+(const V3& a, const V3& b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(const V3& a, const V3& b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator-(const V3& a) { return V3(-a.x, -a.y, -a.z); }
static inline V3 operator*(const V3& a, double s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline V3 operator*(double s, const V3& a) { return V3(s * a.x, s * a.y, s * a.z); }
static inline V3 operator/(const V3& a, double s) { return V3(a.x / s, a.y / s, a.z / s); }
static inline bool isZero(const V3& a) { return a.x == 0 && a.y == 0 && a.z == 0; }
/* Eigen redux on a fixed size-3 vector: (a0*b0 + a1*b1) + a2*b2 */
static inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double sqnorm(const V3& a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline double norm(const V3& a) { return std::sqrt(sqnorm(a)); }
static inline V3 cross(const V3& a, const V3& b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* Eigen normalize(): divide by sqrt(squaredNorm) when it is positive */
static inline void normalize(V3& a) {
  double z = sqnorm(a);
  if (z > 0) { double n = std::sqrt(z); a.x /= n; a.y /= n; a.z /= n; }
}
static inline double absmax(const V3& a) { return std::max(a.x, std::max(a.y, a.z)); }

/* 3x3 matrix stored by columns: c[0], c[1], c[2] */
struct M3 {
  V3 c[3];
  double operator()(int r, int k) const { return c[k][r]; }
};
/* M^T v: component i is column i dotted with v */
static inline V3 mulT(const M3& m, const V3& v) { return V3(dot(m.c[0], v), dot(m.c[1], v), dot(m.c[2], v)); }

/* general 3x3 helpers for the periodic cell, row-major r[i][k] */
struct Mat {
  double r[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  static Mat I() { Mat m; m.r[0][0] = m.r[1][1] = m.r[2][2] = 1; return m; }
  V3 col(int k) const { return V3(r[0][k], r[1][k], r[2][k]); }
};
static Mat mmul(const Mat& a, const Mat& b) {
  Mat c;
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) c.r[i][k] = a.r[i][0] * b.r[0][k] + a.r[i][1] * b.r[1][k] + a.r[i][2] * b.r[2][k];
  return c;
}
static V3 mvec(const Mat& a, const V3& v) {
  return V3(a.r[0][0] * v.x + a.r[0][1] * v.y + a.r[0][2] * v.z, a.r[1][0] * v.x + a.r[1][1] * v.y + a.r[1][2] * v.z,
            a.r[2][0] * v.x + a.r[2][1] * v.y + a.r[2][2] * v.z);
}
static V3 mvecI(const Mat& a, int c0, int c1, int c2) {
  return mvec(a, V3((double)c0, (double)c1, (double)c2));
}
static Mat madd(const Mat& a, const Mat& b, double sb) {
  Mat c;
  for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) c.r[i][k] = a.r[i][k] + sb * b.r[i][k];
  return c;
}
static Mat mscale(const Mat& a, double s) { Mat c; for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) c.r[i][k] = a.r[i][k] * s; return c; }
static Mat mtrans(const Mat& a) { Mat c; for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) c.r[i][k] = a.r[k][i]; return c; }
/* Eigen's 3x3 determinant: expansion along row 0, m00 (m11 m22 - m12 m21) - m01 (m10 m22 - m12 m20)
 * + m02 (m10 m21 - m11 m20) */
static double mdet(const Mat& m) {
  const double (*a)[3] = m.r;
  return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
         a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
}
/* Eigen's 3x3 inverse: cofactors, det = cofactors of column 0 dotted with column 0, then adjugate x (1/det) */
static Mat minv(const Mat& m) {
  const double (*a)[3] = m.r;
  Mat c;
  c.r[0][0] = a[1][1] * a[2][2] - a[1][2] * a[2][1];
  c.r[0][1] = a[0][2] * a[2][1] - a[0][1] * a[2][2];
  c.r[0][2] = a[0][1] * a[1][2] - a[0][2] * a[1][1];
  c.r[1][0] = a[1][2] * a[2][0] - a[1][0] * a[2][2];
  c.r[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0];
  c.r[1][2] = a[0][2] * a[1][0] - a[0][0] * a[1][2];
  c.r[2][0] = a[1][0] * a[2][1] - a[1][1] * a[2][0];
  c.r[2][1] = a[0][1] * a[2][0] - a[0][0] * a[2][1];
  c.r[2][2] = a[0][0] * a[1][1] - a[0][1] * a[1][0];
  double det = c.r[0][0] * a[0][0] + c.r[0][1] * a[1][0] + c.r[0][2] * a[2][0];
  double invdet = 1.0 / det;
  for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) c.r[i][k] = c.r[i][k] * invdet;
  return c;
}
/* leviCivita (src/supp/base/Math.hpp:223-228): (m12-m21, m20-m02, m01-m10) */
static V3 leviCivita(const Mat& m) { return V3(m.r[1][2] - m.r[2][1], m.r[2][0] - m.r[0][2], m.r[0][1] - m.r[1][0]); }

/* Cell (src/core/Cell.hpp:22-187, Cell.cpp), homoDeform = HOMO_GRADV2 only */
struct Cell {
  Mat trsf = Mat::I(), hSize = Mat::I(), pprevHsize = Mat::I(), gradV, nextGradV, W;
  V3 spinVec, size, cos;
  Mat shearTrsf = Mat::I(), unshearTrsf = Mat::I();
  bool hasShear = false;
  /* Cell::integrateAndUpdate (Cell.cpp:81-120) */
  void integrateAndUpdate(double dt) {
    Mat trsfInc = mscale(gradV, dt);
    trsf = madd(trsf, mmul(trsfInc, trsf), 1.0);
    Mat prevHsize = hSize;
    Mat gdt2 = mscale(mscale(gradV, dt), 1. / 2.);  /* gradV*dt/2. */
    Mat A = madd(Mat::I(), gdt2, -1.0), B = madd(Mat::I(), gdt2, 1.0);
    hSize = mmul(mmul(minv(A), B), hSize);
    pprevHsize = mscale(madd(prevHsize, hSize, 1.0), .5);
    if (mdet(hSize) == 0) throw std::runtime_error("Cell is degenerate (zero volume).");
    Mat Hnorm;
    for (int i = 0; i < 3; i++) {
      V3 base = hSize.col(i);
      size[i] = norm(base);
      base = base / size[i];
      Hnorm.r[0][i] = base.x; Hnorm.r[1][i] = base.y; Hnorm.r[2][i] = base.z;
    }
    for (int i = 0; i < 3; i++) {
      int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      cos[i] = sqnorm(cross(Hnorm.col(i1), Hnorm.col(i2)));
    }
    shearTrsf = Hnorm;
    unshearTrsf = minv(shearTrsf);
    const double (*h)[3] = hSize.r;
    hasShear = (h[0][1] != 0 || h[0][2] != 0 || h[1][0] != 0 || h[1][2] != 0 || h[2][0] != 0 || h[2][1] != 0);
  }
  /* Cell::setNextGradV (Cell.cpp:60-66) */
  void setNextGradV() {
    gradV = nextGradV;
    W = mscale(madd(gradV, mtrans(gradV), -1.0), .5);
    spinVec = .5 * leviCivita(W);
  }
  V3 intrShiftPos(const int* cd) const { return mvecI(hSize, cd[0], cd[1], cd[2]); }
  /* Cell::intrShiftVel, HOMO_GRADV2 (Cell.cpp:28-34): gradV*pprevHsize*cellDist */
  V3 intrShiftVel(const int* cd) const { return mvecI(mmul(gradV, pprevHsize), cd[0], cd[1], cd[2]); }
  /* Cell::shearAlignedExtents (Cell.cpp:68-78) */
  V3 shearAlignedExtents(const V3& perp) const {
    if (!hasShear) return perp;
    V3 ret = perp;
    for (int ax = 0; ax < 3; ax++) {
      int ax1 = (ax + 1) % 3, ax2 = (ax + 2) % 3;
      ret[ax1] += .5 * perp[ax1] * (1 / cos[ax] - 1);
      ret[ax2] += .5 * perp[ax2] * (1 / cos[ax] - 1);
    }
    return ret;
  }
};

struct Quat {
  double w = 1, x = 0, y = 0, z = 0;
  Quat() {}
  Quat(double w_, double x_, double y_, double z_) : w(w_), x(x_), y(y_), z(z_) {}
};
/* Hamilton product, written term by term as in Eigen's generic quat_product */
static inline Quat qmul(const Quat& a, const Quat& b) {
  return Quat(a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z,
              a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
              a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z,
              a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x);
}
/* rotate v by unit quaternion q: uv = 2 (q.vec x v); v + w uv + q.vec x uv */
static inline V3 qrot(const Quat& q, const V3& v) {
  V3 qv(q.x, q.y, q.z);
  V3 uv = cross(qv, v);
  uv = uv + uv;
  return v + q.w * uv + cross(qv, uv);
}
static inline void qnormalize(Quat& q) {
  /* coefficients stored (x,y,z,w): ((x^2+y^2)+z^2)+w^2 */
  double z2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
  if (z2 > 0) { double n = std::sqrt(z2); q.x /= n; q.y /= n; q.z /= n; q.w /= n; }
}
static inline Quat qconj(const Quat& q) { return Quat(q.w, -q.x, -q.y, -q.z); }
/* rotation matrix -> quaternion, Shoemake's method (trace branch, else largest diagonal) */
static Quat quatFromMatrix(const M3& m) {
  Quat q;
  double t = m(0, 0) + m(1, 1) + m(2, 2);
  if (t > 0) {
    t = std::sqrt(t + 1.0);
    q.w = 0.5 * t;
    t = 0.5 / t;
    q.x = (m(2, 1) - m(1, 2)) * t;
    q.y = (m(0, 2) - m(2, 0)) * t;
    q.z = (m(1, 0) - m(0, 1)) * t;
  } else {
    int i = 0;
    if (m(1, 1) > m(0, 0)) i = 1;
    if (m(2, 2) > m(i, i)) i = 2;
    int j = (i + 1) % 3, k = (j + 1) % 3;
    t = std::sqrt(m(i, i) - m(j, j) - m(k, k) + 1.0);
    double v[3];
    v[i] = 0.5 * t;
    t = 0.5 / t;
    q.w = (m(k, j) - m(j, k)) * t;
    v[j] = (m(j, i) + m(i, j)) * t;
    v[k] = (m(k, i) + m(i, k)) * t;
    q.x = v[0]; q.y = v[1]; q.z = v[2];
  }
  return q;
}
static inline double pow2(double x) { return x * x; }

/* Quaternion::toRotationMatrix, Eigen's formula with tx = 2x, twx = tx w, ... (row-major result) */
static Mat quatToMat(const Quat& q) {
  const double tx = 2 * q.x, ty = 2 * q.y, tz = 2 * q.z;
  const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
  const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
  const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
  Mat m;
  m.r[0][0] = 1 - (tyy + tzz); m.r[0][1] = txy - twz;       m.r[0][2] = txz + twy;
  m.r[1][0] = txy + twz;       m.r[1][1] = 1 - (txx + tzz); m.r[1][2] = tyz - twx;
  m.r[2][0] = txz - twy;       m.r[2][1] = tyz + twx;       m.r[2][2] = 1 - (txx + tyy);
  return m;
}
/* AngleAxis(q).angle(): 2 atan2(|q.vec|, |q.w|), 0 for a zero vector part */
static double quatAngle(const Quat& q) {
  const double n = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z);
  if (n != 0) return 2 * std::atan2(n, std::abs(q.w));
  return 0;
}
static inline double minCoeff(const V3& a) { double r = a.x; if (a.y < r) r = a.y; if (a.z < r) r = a.z; return r; }
static inline double maxCoeff(const V3& a) { double r = a.x; if (a.y > r) r = a.y; if (a.z > r) r = a.z; return r; }
/* Math::Sign (src/supp/base/Math.hpp:145) */
static inline double Sign(double f) { if (f < 0) return -1; if (f > 0) return 1; return 0; }
/* pown (src/supp/base/Math.hpp:166-175): x^n by squaring */
static double pown(double x, unsigned n) {
  unsigned d = n >> 1, r = n & 1;
  double x2d = d == 0 ? 1 : pown(x * x, d);
  double xr = r == 0 ? 1 : x;
  return x2d * xr;
}

/* ------------------------------------------------------------------ model */
struct Aabb {
  bool has = false;
  V3 min, max;
  V3 nodeLastPos;
  Quat nodeLastOri;
  double maxD2 = 0;
  double maxRot = -1;   /* < 0: rotation ignored (Sphere, Wall); Bo1_Ellipsoid_Aabb starts it at 0 */
};

struct Particle {
  int id = 0;
  int shape = WDEM_SHAPE_SPHERE;
  double radius = NaN;
  int axis = 0, sense = 0;
  int mat = 0;
  unsigned mask = 1;
  unsigned flags = 0;
  double mass = 0;
  V3 inertia;
  V3 pos, vel, angVel, force, torque;
  Quat ori;
  V3 semiAxes;                        /* Ellipsoid.semiAxes */
  V3 fv1, fv2;                        /* Facet nodes 1 and 2 (node 0 is pos; radius holds halfThick) */
  double shaft = NaN;                 /* Capsule.shaft (radius holds Capsule.radius) */
  V3 angMom = V3(NaN, NaN, NaN);      /* DemData.angMom (aspherical Leapfrog) */
  Aabb bound;
  std::map<int, std::shared_ptr<struct Contact>> contacts; /* Particle::contacts (Particle.hpp:36) */
  bool isBlockedNone() const { return (flags & 63u) == 0; }
  bool isBlockedAll() const { return (flags & 63u) == 63u; }
  bool isBlockedAllRot() const { return (flags & 56u) == 56u; }
  bool isBlockedAxisDOF(int ax, bool rot) const { return flags & (1u << (ax + (rot ? 3 : 0))); }
  bool isAspherical() const { return !(inertia.x == inertia.y && inertia.y == inertia.z); }
};

struct Contact {
  int pA = -1, pB = -1;
  int cellDist[3] = {0, 0, 0};
  bool geom = false, phys = false;
  int stepCreated = -1;
  double minDist00Sq = -1;
  size_t linIx = 0;
  /* L6Geom (src/dem/L6Geom.hpp:14-22) */
  V3 gvel, gangVel;
  double uN = NaN;
  double lens[2] = {0, 0};
  double contA = NaN;
  M3 trsf;
  V3 contPt;
  Quat gori;
  /* FrictPhys / HertzPhys (FrictMat.hpp:30-41, Hertz.hpp:16-31) */
  V3 force, torque;
  double kn = NaN, kt = NaN, tanPhi = NaN;
  double kt0 = 0, alpha_sqrtMK = 0, R = 0, K = 0, gamma = 0, alpha = 0, contRad = 0;
  bool isReal() const { return geom && phys; }
  bool isColliding() const { return stepCreated >= 0; }
  Contact() {
    trsf.c[0] = V3(1, 0, 0); trsf.c[1] = V3(0, 1, 0); trsf.c[2] = V3(0, 0, 1);
  }
};
typedef std::shared_ptr<Contact> CPtr;

struct Energy {
  double v[WDEM_E_COUNT] = {0};
  bool resettable[WDEM_E_COUNT] = {true, false, false, true, false, false, false, false};
  void resetResettables() { for (int i = 0; i < WDEM_E_COUNT; i++) if (resettable[i]) v[i] = 0; }
};

struct Bounds {
  double coord = 0;
  int id = 0;
  bool hasBB = false, isMin = false;
  Bounds() {}
  Bounds(double c, int i, bool mn) : coord(c), id(i), hasBB(false), isMin(mn) {}
  /* InsertionSortCollider.hpp:132-140 */
  bool operator<(const Bounds& b) const {
    if (id == b.id && coord == b.coord) return isMin;
    return coord < b.coord;
  }
  bool operator>(const Bounds& b) const {
    if (id == b.id && coord == b.coord) return !isMin;
    return coord > b.coord;
  }
};

struct Scene {
  /* Scene + DemField + engine attributes */
  wdem_params P;
  std::vector<wdem_material> mats;
  long step = 0;
  double time = 0;
  std::vector<Particle> par;
  /* ContactContainer */
  std::vector<CPtr> linView;
  std::vector<std::pair<CPtr, bool>> pending;
  bool dirty = true;
  /* InsertionSortCollider */
  std::vector<Bounds> BB[3];
  std::vector<double> minima, maxima;
  std::vector<CPtr> makeContacts, removeContacts;
  /* OpenMP build: per-thread queues of the parallel insertion sort (mmakeContacts / rremoveContacts,
   * InsertionSortCollider.hpp:95-113) */
  std::vector<std::vector<CPtr>> makeT, removeT;
  long sortPasses = 0;        /* passes of the last parallel insertion sort (diagnostics) */
  double verletDist = -0.05;  /* resolved on first run */
  long nFullRuns = 0;
  int sortAxis = 0;
  /* options */
  int canonicalOrient = 0;
  int applyOrder = 0;
  int updatePhys = 0;
  Energy E;
  std::string err;
  int lastRunFull = 0;
  int parallel = 0;   /* OpenMP contact/node loops with a per-particle lock (reference's OpenMP build) */
  int detParallel = 0; /* OpenMP threads that reproduce the serial results bit for bit (long parity runs) */
  bool anyEll = false; /* an ellipsoid among the particles */
  bool periodic = false;
  Cell cell;
  double stress[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  long ellEvals = 0, ellSolves = 0;   /* contact-function evaluations / solves of the ellipsoid functors */
  /* DynDt as a PeriodicEngine (Engine.hpp:130-160): stepLast, stepPrev; Scene.nextDt; last critical step */
  long dynStepLast = -1, dynStepPrev = -1;
  double nextDt = NaN, dynDtCrit = NaN;
#ifdef _OPENMP
  std::vector<omp_lock_t> locks;
  ~Scene() { for (auto& l : locks) omp_destroy_lock(&l); }
#endif
};

/* ------------------------------------------------------------------ ContactContainer */
/* ContactContainer::addMaybe_fast (ContactContainer.cpp:51-58) */
static void addMaybe_fast(Scene& S, const CPtr& c) {
  Particle& A = S.par[c->pA];
  Particle& B = S.par[c->pB];
  if (A.contacts.count(B.id) == 1) return;
  A.contacts[B.id] = c;
  B.contacts[A.id] = c;
  S.linView.push_back(c);
  c->linIx = S.linView.size() - 1;
}
/* ContactContainer::linView_remove (ContactContainer.cpp:69-80) */
static void linView_remove(Scene& S, size_t ix) {
  if (ix < S.linView.size() - 1) {
    S.linView[ix] = S.linView.back();
    S.linView[ix]->linIx = ix;
  }
  S.linView.resize(S.linView.size() - 1);
}
/* ContactContainer::removeMaybe_fast (ContactContainer.cpp:60-67) */
static void removeMaybe_fast(Scene& S, const CPtr& c) {
  Particle& A = S.par[c->pA];
  Particle& B = S.par[c->pB];
  auto iA = A.contacts.find(B.id);
  if (iA == A.contacts.end()) return;
  A.contacts.erase(iA);
  B.contacts.erase(B.contacts.find(A.id));
  linView_remove(S, c->linIx);
}
/* ContactContainer::remove (ContactContainer.cpp:82-137), particles never vanish here */
static bool removeContact(Scene& S, const CPtr& c) {
  Particle& A = S.par[c->pA];
  Particle& B = S.par[c->pB];
  auto iA = A.contacts.find(B.id);
  if (iA == A.contacts.end()) return false;
  A.contacts.erase(iA);
  auto iB = B.contacts.find(A.id);
  if (iB != B.contacts.end()) B.contacts.erase(iB);
  linView_remove(S, c->linIx);
  return true;
}
static CPtr findContact(Scene& S, int a, int b) {
  auto I = S.par[a].contacts.find(b);
  if (I == S.par[a].contacts.end()) return CPtr();
  return I->second;
}
/* ContactContainer::requestRemoval (ContactContainer.cpp:164-174) + Contact::reset (Contact.cpp:141-145) */
static void requestRemoval(Scene& S, const CPtr& c, bool force = false) {
  c->geom = false; c->phys = false;
  /* Contact::reset drops the CGeom/CPhys objects: a new contact later starts from default values */
  Contact fresh;
  c->gvel = fresh.gvel; c->gangVel = fresh.gangVel; c->uN = fresh.uN; c->lens[0] = c->lens[1] = 0; c->contA = NaN;
  c->trsf = fresh.trsf; c->contPt = V3(); c->gori = Quat();
  c->force = V3(); c->torque = V3(); c->kn = c->kt = c->tanPhi = NaN;
  c->kt0 = c->alpha_sqrtMK = c->R = c->K = c->gamma = c->alpha = c->contRad = 0;
  S.pending.push_back(std::make_pair(c, force));
}

/* ------------------------------------------------------------------ collider */
/* Collider::mayCollide (Collision.cpp:21-43); no shared nodes and no clumps in this model */
static bool mayCollide(const Scene& S, const Particle& A, const Particle& B) {
  if (A.id == B.id) return false;
  if (!(A.mask & B.mask)) return false;
  if ((A.mask & B.mask & S.P.loneMask) != 0) return false;
  return true;
}
/* InsertionSortCollider::spatialOverlap (InsertionSortCollider.cpp:67-73) */
static bool spatialOverlap(const Scene& S, int id1, int id2) {
  const double* mn = S.minima.data();
  const double* mx = S.maxima.data();
  return (mn[3 * id1 + 0] <= mx[3 * id2 + 0]) && (mx[3 * id1 + 0] >= mn[3 * id2 + 0]) &&
         (mn[3 * id1 + 1] <= mx[3 * id2 + 1]) && (mx[3 * id1 + 1] >= mn[3 * id2 + 1]) &&
         (mn[3 * id1 + 2] <= mx[3 * id2 + 2]) && (mx[3 * id1 + 2] >= mn[3 * id2 + 2]);
}
/* makeContactLater (InsertionSortCollider.hpp:106-113) */
/* tid >= 0: the queue of that OpenMP thread (parallel insertion sort); -1: the serial queue */
static void makeContactLater(Scene& S, int a, int b, int tid = -1) {
  CPtr C = std::make_shared<Contact>();
  if (S.canonicalOrient && S.par[a].shape == S.par[b].shape && a > b) std::swap(a, b);
  C->pA = a; C->pB = b; C->stepCreated = (int)S.step;
  (tid < 0 ? S.makeContacts : S.makeT[tid]).push_back(C);
}
/* handleBoundInversion (InsertionSortCollider.cpp:78-113); the container is only read here (additions
 * and removals are queued), so the OpenMP threads of the parallel sort may call it concurrently */
static void handleBoundInversion(Scene& S, int id1, int id2, bool separating, int tid = -1) {
  bool overlap = separating ? false : spatialOverlap(S, id1, id2);
  CPtr C = findContact(S, id1, id2);
  bool hasCon = (bool)C;
  if (!overlap && !hasCon) return;
  if (overlap && hasCon) return;
  if (overlap) {
    if (!mayCollide(S, S.par[id1], S.par[id2])) return;
    makeContactLater(S, id1, id2, tid);
    return;
  }
  if (!C->isReal()) (tid < 0 ? S.removeContacts : S.removeT[tid]).push_back(C);
}
/* insertionSort_part, serial form (InsertionSortCollider.cpp:189-223) */
static void insertionSort(Scene& S, std::vector<Bounds>& v, bool doCollide) {
  long n = (long)v.size();
  for (long i = 1; i < n; i++) {
    if (!(v[i - 1] > v[i])) continue;
    const Bounds viInit = v[i];
    long j = i - 1;
    const bool viInitBB = viInit.hasBB, viInitIsMin = viInit.isMin;
    while (j >= 0 && v[j] > viInit) {
      v[j + 1] = v[j];
      if (viInitIsMin != v[j].isMin && doCollide && viInitBB && v[j].hasBB && viInit.id != v[j].id)
        handleBoundInversion(S, viInit.id, v[j].id, !viInitIsMin);
      j--;
    }
    v[j + 1] = viInit;
  }
}
#ifdef _OPENMP
/* insertionSort_part (InsertionSortCollider.cpp:189-223): sort v[iBegin, iEnd) starting at iStart; when
 * iStart > iBegin (a later pass) it stops at the first ordered couple */
static void insertionSortPart(Scene& S, std::vector<Bounds>& v, bool doCollide, long iBegin, long iEnd, long iStart,
                              int tid) {
  const bool earlyStop = (iBegin != iStart);
  for (long i = std::max(iStart, iBegin + 1); i < iEnd; i++) {
    if (!(v[i - 1] > v[i])) {
      if (earlyStop) return;
      continue;
    }
    const Bounds viInit = v[i];
    long j = i - 1;
    const bool viInitBB = viInit.hasBB, viInitIsMin = viInit.isMin;
    while (j >= iBegin && v[j] > viInit) {
      v[j + 1] = v[j];
      if (viInitIsMin != v[j].isMin && doCollide && viInitBB && v[j].hasBB && viInit.id != v[j].id)
        handleBoundInversion(S, viInit.id, v[j].id, !viInitIsMin, tid);
      j--;
    }
    v[j + 1] = viInit;
  }
}
/* InsertionSortCollider::insertionSort, OpenMP form (InsertionSortCollider.cpp:124-186) with the default
 * ompTuneSort = (1, 1000, 0) and maxSortPass = -100 (InsertionSortCollider.hpp:291,295): the bounds are cut
 * into one chunk per thread (at least 2000 bounds each, rounded to a multiple of the thread count); the
 * chunks are sorted in parallel, alternately between the split points and between the mid-chunk points,
 * until every split point is ordered.  Inversions go to per-thread queues. */
static void insertionSortParallel(Scene& S, std::vector<Bounds>& v, bool doCollide) {
  const long size = (long)v.size();
  if (size == 0) return;
  const int TH = omp_get_max_threads();
  const long minPerCore = 2 * 1000;
  long chunks = TH;
  if (size / chunks < minPerCore) chunks = TH * (long)std::ceil(std::max(1L, size / minPerCore) * 1. / TH);
  const long chunkSize = size / chunks;
  if (chunks == 1 || chunkSize < 100) { insertionSort(S, v, doCollide); return; }
  std::vector<long> splits0(chunks + 1), splits1(chunks);
  for (long i = 0; i < chunks; i++) { splits0[i] = i * chunkSize; splits1[i] = i * chunkSize + chunkSize / 2; }
  splits0[chunks] = size;
  const long maxPass = 100L * TH;
  bool isOk = false;
  long pass;
  for (pass = 0; !isOk; pass++) {
    if (pass == maxPass) throw std::runtime_error("InsertionSortCollider: sort not done after the maximum number of partial sort passes");
    const bool even = (pass % 2) == 0;
    const std::vector<long>& sp = even ? splits0 : splits1;
    const long nch = even ? chunks : chunks - 1;
#pragma omp parallel for schedule(static)
    for (long chunk = 0; chunk < nch; chunk++) {
      const long start = pass == 0 ? sp[chunk] : (even ? splits1[chunk] : splits0[chunk + 1]);
      insertionSortPart(S, v, doCollide, sp[chunk], sp[chunk + 1], start, omp_get_thread_num());
    }
    isOk = true;
    for (long chunk = even ? 1 : 0; chunk < chunks; chunk++)
      if (v[sp[chunk] - 1] > v[sp[chunk]]) { isOk = false; break; }
  }
  S.sortPasses = pass;
}
#endif
/* Bo1_Sphere_Aabb::go (Sphere.cpp:52-64), Bo1_Wall_Aabb::go (Wall.cpp:25-38), then the verlet
 * enlargement of AabbCollider::updateAabb (Collision.cpp:125-162) */
/* Ellipsoid::trsfFromUnitSphere (Ellipsoid.cpp:77-82): column i = ori * (semiAxes[i] e_i) */
static M3 ellTrsf(const Particle& p) {
  M3 m;
  m.c[0] = qrot(p.ori, V3(p.semiAxes.x, 0, 0));
  m.c[1] = qrot(p.ori, V3(0, p.semiAxes.y, 0));
  m.c[2] = qrot(p.ori, V3(0, 0, p.semiAxes.z));
  return m;
}
/* half-extents along the global axes: norms of the rows of trsfFromUnitSphere (Ellipsoid.cpp:87-90) */
static V3 ellExtents(const Particle& p) {
  M3 m = ellTrsf(p);
  V3 d;
  for (int i = 0; i < 3; i++) d[i] = std::sqrt(m.c[0][i] * m.c[0][i] + m.c[1][i] * m.c[1][i] + m.c[2][i] * m.c[2][i]);
  return d;
}
static void updateAabb(Scene& S, Particle& p) {
  Aabb& a = p.bound;
  if (p.shape == WDEM_SHAPE_SPHERE) {
    double df = S.P.distFactor;
    double h = (df > 0 ? df : 1.) * p.radius;
    V3 half(h, h, h);
    if (!S.periodic) {
      a.min = p.pos - half;
      a.max = p.pos + half;
    } else {
      /* Bo1_Sphere_Aabb::goGeneric, periodic (Sphere.cpp:66-81): unsheared centre, shear-aligned extents */
      half = S.cell.shearAlignedExtents(half);
      V3 c = mvec(S.cell.unshearTrsf, p.pos);
      a.min = c - half;
      a.max = c + half;
    }
  } else if (p.shape == WDEM_SHAPE_ELLIPSOID) {
    /* Bo1_Ellipsoid_Aabb::go (Ellipsoid.cpp:97-119), aperiodic or unsheared cell: half-extents are the
     * row norms of trsfFromUnitSphere; a new bound starts with maxRot = 0 (rotation-aware verlet) */
    if (S.periodic && S.cell.hasShear) throw std::runtime_error("ellipsoids in a sheared periodic cell are not restated");
    if (!a.has) a.maxRot = 0.;
    V3 delta = ellExtents(p);
    V3 c = S.periodic ? mvec(S.cell.unshearTrsf, p.pos) : p.pos;
    a.min = c - delta;
    a.max = c + delta;
  } else if (p.shape == WDEM_SHAPE_CAPSULE) {
    /* Bo1_Capsule_Aabb::go (Capsule.cpp:97-114) with Capsule::alignedBox (:67-73), aperiodic: the box of the
     * four points pos +- dShaft +- radius (1,1,1), dShaft = ori (shaft/2, 0, 0); a new bound starts with
     * maxRot = 0 (rotation-aware verlet) */
    if (S.periodic) throw std::runtime_error("capsules in a periodic cell are not restated");
    if (!a.has) a.maxRot = 0.;
    const V3 dShaft = qrot(p.ori, V3(.5 * p.shaft, 0, 0));
    a.min = V3(Inf, Inf, Inf);
    a.max = V3(-Inf, -Inf, -Inf);
    for (double sa : {-1., 1.})
      for (double sb : {-1., 1.}) {
        const double br = sb * p.radius;
        const V3 q = (p.pos + sa * dShaft) + V3(br, br, br);
        for (int k = 0; k < 3; k++) {
          a.min[k] = std::min(a.min[k], q[k]);
          a.max[k] = std::max(a.max[k], q[k]);
        }
      }
  } else if (p.shape == WDEM_SHAPE_FACET) {
    /* Bo1_Facet_Aabb::go (Facet.cpp:275-298), aperiodic: the nodes +- halfThick, coefficient-wise min/max */
    if (S.periodic) throw std::runtime_error("facets in a periodic cell are not restated");
    const V3 ht(p.radius, p.radius, p.radius);
    a.min = p.pos - ht;
    a.max = p.pos + ht;
    for (const V3* v : {&p.fv1, &p.fv2}) {
      const V3 lo = *v - ht, hi = *v + ht;
      for (int k = 0; k < 3; k++) {
        a.min[k] = std::min(a.min[k], lo[k]);
        a.max[k] = std::max(a.max[k], hi[k]);
      }
    }
  } else {
    a.min = V3(-Inf, -Inf, -Inf);
    a.max = V3(Inf, Inf, Inf);
    a.min[p.axis] = a.max[p.axis] = p.pos[p.axis];
  }
  a.has = true;
  a.nodeLastPos = p.pos;
  a.nodeLastOri = p.ori;
  a.maxD2 = pow2(S.verletDist);
  if (S.verletDist > 0) {
    /* AabbCollider::updateAabb (Collision.cpp:152-161): rotation limit from the largest half-extent */
    if (a.maxRot >= 0) {
      double maxArm = .5 * maxCoeff(a.max - a.min);
      if (maxArm > 0.) a.maxRot = std::atan(S.verletDist / maxArm);
      else a.maxRot = 0.;
    }
    V3 vd(S.verletDist, S.verletDist, S.verletDist);
    a.max = a.max + vd;
    a.min = a.min - vd;
  }
}
/* Capsule::volume, Capsule::equivRadius (Capsule.cpp:25-31) */
static double capsuleEquivRadius(const Particle& p) {
  const double r = p.radius;
  const double vol = (4 / 3.) * M_PI * (r * r * r) + M_PI * (r * r) * p.shaft;
  return std::cbrt(vol * 3 / (4 * M_PI));
}
/* AabbCollider::setVerletDist (Collision.cpp:164-184) */
static void setVerletDist(Scene& S) {
  if (S.verletDist >= 0) return;
  double minR = Inf;
  for (const Particle& p : S.par) {
    /* Shape::equivRadius: Sphere.radius, Ellipsoid cbrt(abc) (Ellipsoid.cpp:25-28), NaN for walls */
    double r = NaN;
    if (p.shape == WDEM_SHAPE_SPHERE) r = p.radius;
    else if (p.shape == WDEM_SHAPE_ELLIPSOID) r = std::cbrt(p.semiAxes.x * p.semiAxes.y * p.semiAxes.z);
    else if (p.shape == WDEM_SHAPE_CAPSULE) r = capsuleEquivRadius(p);
    if (!std::isnan(r)) minR = std::min(r, minR);
  }
  if (!std::isinf(minR)) S.verletDist = std::abs(S.verletDist) * minR;
  else S.verletDist = 0.0;
}
/* AabbCollider::aabbIsDirty (Collision.cpp:80-123), maxRot<0 for spheres and walls */
static bool aabbIsDirty(const Particle& p) {
  if (!p.bound.has) return true;
  if (std::isnan(absmax(p.bound.min)) || std::isnan(absmax(p.bound.max))) return true;
  double moveDueToRot2 = 0.;
  if (p.bound.maxRot >= 0.) {
    /* rotation since the last update (Collision.cpp:94-110) */
    double rot = std::max(0., std::abs(quatAngle(qmul(qconj(p.bound.nodeLastOri), p.ori))));
    if (rot > p.bound.maxRot) return true;
    moveDueToRot2 = pow2(.5 * maxCoeff(p.bound.max - p.bound.min) * rot);
  }
  double d2 = std::max(0., sqnorm(p.bound.nodeLastPos - p.pos));
  return d2 + moveDueToRot2 > p.bound.maxD2;
}
/* InsertionSortCollider::cellWrapRel (InsertionSortCollider.cpp:624-628) */
static double cellWrapRel(double x, double x0, double x1, int& period) {
  double xNorm = (x - x0) / (x1 - x0);
  period = (int)std::floor(xNorm);
  return (xNorm - std::floor(xNorm)) * (x1 - x0);
}
/* spatialOverlapPeri_axis, the "new algorithm" (InsertionSortCollider.cpp:897-1010) */
static bool spatialOverlapPeriAxis(int id1, int id2, double min1, double max1, double min2, double max2, double dim,
                                   int& period) {
  if (std::isinf(min1) || std::isinf(min2)) { period = 0; return true; }
  int pmn1_2, pmx1_2, pmn2_1, pmx2_1;
  double mn1_2 = cellWrapRel(min1, min2, min2 + dim, pmn1_2); (void)cellWrapRel(max1, min2, min2 + dim, pmx1_2);
  double mn2_1 = cellWrapRel(min2, min1, min1 + dim, pmn2_1); (void)cellWrapRel(max2, min1, min1 + dim, pmx2_1);
  if (pmn1_2 != pmx1_2 && pmn2_1 != pmx2_1)
    throw std::runtime_error("InsertionSortCollider: ambiguous periodic contact ##" + std::to_string(id1) + "+" + std::to_string(id2));
  else if (pmn2_1 == pmx2_1) { period = -pmn2_1; return mn2_1 < (max1 - min1); }
  else { period = pmn1_2; return mn1_2 < (max2 - min2); }
}
/* spatialOverlapPeri (InsertionSortCollider.cpp:1027-1044) */
static bool spatialOverlapPeri(const Scene& S, int id1, int id2, int* periods) {
  for (int ax = 0; ax < 3; ax++)
    if (!spatialOverlapPeriAxis(id1, id2, S.minima[3 * id1 + ax], S.maxima[3 * id1 + ax], S.minima[3 * id2 + ax],
                                S.maxima[3 * id2 + ax], S.cell.size[ax], periods[ax]))
      return false;
  return true;
}
static bool overlapAny(const Scene& S, int a, int b) {
  if (!S.periodic) return spatialOverlap(S, a, b);
  int per[3];
  return spatialOverlapPeri(S, a, b, per);
}
/* Periodic full run: the pair set the periodic insertion sort maintains
 * (InsertionSortCollider.cpp:637-882): every pair overlapping under spatialOverlapPeri with its
 * periods as Contact.cellDist; real contacts stay; non-real ones that stopped overlapping go.
 * Candidates come from a periodic cell list (any complete candidate set gives the same result). */
static void colliderPeriodicFull(Scene& S) {
  const int n = (int)S.par.size();
  /* existing non-real contacts that no longer overlap */
  std::vector<CPtr> cur = S.linView;
  for (auto& C : cur)
    if (!C->isReal() && !overlapAny(S, C->pA, C->pB)) removeMaybe_fast(S, C);
  V3 W;
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) W[k] = std::max(W[k], S.maxima[3 * i + k] - S.minima[3 * i + k]);
  int nc[3];
  double cw[3];
  for (int k = 0; k < 3; k++) {
    nc[k] = (W[k] > 0) ? (int)std::floor(S.cell.size[k] / (W[k] * (1 + 1e-6))) : 1;
    if (nc[k] < 3) nc[k] = 1;
    cw[k] = S.cell.size[k] / nc[k];
  }
  auto cellOf = [&](int i, int* c) {
    for (int k = 0; k < 3; k++) {
      double x = .5 * (S.minima[3 * i + k] + S.maxima[3 * i + k]);
      double w = x - std::floor(x / S.cell.size[k]) * S.cell.size[k];
      int v = (int)std::floor(w / cw[k]);
      c[k] = std::min(std::max(v, 0), nc[k] - 1);
    }
  };
  std::map<long, std::vector<int>> cells;
  std::vector<std::array<int, 3>> cid(n);
  for (int i = 0; i < n; i++) {
    int c[3];
    cellOf(i, c);
    cid[i] = {c[0], c[1], c[2]};
    cells[((long)c[2] * nc[1] + c[1]) * nc[0] + c[0]].push_back(i);
  }
  /* candidate search (read-only), then the new contacts are added in the order of the serial loop: by i,
   * then by neighbour cell; OpenMP threads take contiguous ranges of i (each pair is met once, from its
   * lower id, so additions made during the loop never change a later test) */
  struct NewPair { int i, j, per[3]; };
  auto search = [&](int i0, int i1, std::vector<NewPair>& out) {
    for (int i = i0; i < i1; i++) {
      std::vector<long> seen;
      for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            int c[3] = {cid[i][0] + dx, cid[i][1] + dy, cid[i][2] + dz};
            for (int k = 0; k < 3; k++) c[k] = ((c[k] % nc[k]) + nc[k]) % nc[k];
            long key = ((long)c[2] * nc[1] + c[1]) * nc[0] + c[0];
            if (std::find(seen.begin(), seen.end(), key) != seen.end()) continue;
            seen.push_back(key);
            auto it = cells.find(key);
            if (it == cells.end()) continue;
            for (int j : it->second) {
              if (j <= i) continue;
              NewPair q;
              q.i = i; q.j = j;
              if (!spatialOverlapPeri(S, i, j, q.per)) continue;
              if (findContact(S, i, j)) continue;
              if (!mayCollide(S, S.par[i], S.par[j])) continue;
              out.push_back(q);
            }
          }
    }
  };
  std::vector<std::vector<NewPair>> found;
#ifdef _OPENMP
  if (S.parallel || S.detParallel) {
    const int T = omp_get_max_threads();
    found.assign(T, std::vector<NewPair>());
#pragma omp parallel num_threads(T)
    {
      const int t = omp_get_thread_num(), nt = omp_get_num_threads();
      search((int)((long)n * t / nt), (int)((long)n * (t + 1) / nt), found[t]);
    }
  } else
#endif
  {
    found.assign(1, std::vector<NewPair>());
    search(0, n, found[0]);
  }
  for (auto& part : found)
    for (const NewPair& q : part) {
      CPtr C = std::make_shared<Contact>();
      C->pA = q.i; C->pB = q.j; C->stepCreated = (int)S.step;
      for (int k = 0; k < 3; k++) C->cellDist[k] = q.per[k];
      addMaybe_fast(S, C);
    }
}

#ifdef _OPENMP
/* The pairs of the initial sort's sweep (InsertionSortCollider.cpp:572-587), found through a cell grid by
 * OpenMP threads: the timing build's replacement of the serial sweep along sortAxis, which visits every
 * bound between a box's minimum and maximum (about 4 minutes for a million spheres on one core; it runs
 * once, before any timed step).  The same predicate decides (handleBoundInversion: spatialOverlap,
 * mayCollide, existing contact); a new contact's pA is the particle whose minimum along sortAxis comes
 * first, as in the sweep.  Existing non-real contacts of boxes that meet along sortAxis but do not overlap
 * are removed, as the sweep does. */
static void initialPairsGrid(Scene& S) {
  const long nP = (long)S.par.size();
  const int ax = S.sortAxis;
  const int TH = omp_get_max_threads();
  S.makeT.assign(TH, std::vector<CPtr>());
  S.removeT.assign(TH, std::vector<CPtr>());
  const double* mn = S.minima.data();
  const double* mx = S.maxima.data();
  /* boxes with finite extents go into the grid; the others (walls) are tested against every box */
  double lo[3] = {Inf, Inf, Inf}, hi[3] = {-Inf, -Inf, -Inf}, w = 0;
  std::vector<int> grid, large;
  std::vector<char> inGrid(nP, 0);
  for (long i = 0; i < nP; i++) {
    if (!S.par[i].bound.has) continue;
    bool fin = true;
    for (int k = 0; k < 3; k++) fin = fin && std::isfinite(mn[3 * i + k]) && std::isfinite(mx[3 * i + k]);
    if (!fin) { large.push_back((int)i); continue; }
    inGrid[i] = 1;
    grid.push_back((int)i);
    for (int k = 0; k < 3; k++) {
      lo[k] = std::min(lo[k], mn[3 * i + k]); hi[k] = std::max(hi[k], mx[3 * i + k]);
      w = std::max(w, mx[3 * i + k] - mn[3 * i + k]);
    }
  }
  int nc[3] = {1, 1, 1};
  if (!grid.empty() && w > 0)
    for (int k = 0; k < 3; k++) nc[k] = (int)std::max(1.0, std::min(1024.0, std::floor((hi[k] - lo[k]) / w)));
  auto cellOf = [&](long i, int k) {
    const double c = 0.5 * (mn[3 * i + k] + mx[3 * i + k]);
    int v = (int)std::floor((c - lo[k]) / (hi[k] - lo[k]) * nc[k]);
    return std::min(std::max(v, 0), nc[k] - 1);
  };
  const long ncell = (long)nc[0] * nc[1] * nc[2];
  std::vector<long> start(ncell + 1, 0);
  std::vector<int> cellIx(nP, -1);
  for (int i : grid) { long c = cellOf(i, 0) + nc[0] * (cellOf(i, 1) + (long)nc[1] * cellOf(i, 2)); cellIx[i] = (int)c; start[c + 1]++; }
  for (long c = 0; c < ncell; c++) start[c + 1] += start[c];
  std::vector<int> members(grid.size());
  {
    std::vector<long> fill(start.begin(), start.end() - 1);
    for (int i : grid) members[fill[cellIx[i]]++] = i;
  }
  /* the sweep's order along sortAxis: the bound with the smaller coordinate first (ties by id) */
  auto firstOf = [&](int a, int b) { return (mn[3 * a + ax] < mn[3 * b + ax] || (mn[3 * a + ax] == mn[3 * b + ax] && a < b)); };
  auto consider = [&](int a, int b, int tid) {
    if (!spatialOverlap(S, a, b)) return;
    if (findContact(S, a, b)) return;
    if (!mayCollide(S, S.par[a], S.par[b])) return;
    if (firstOf(a, b)) makeContactLater(S, a, b, tid); else makeContactLater(S, b, a, tid);
  };
#pragma omp parallel for schedule(dynamic, 1024)
  for (long q = 0; q < (long)grid.size(); q++) {
    const int tid = omp_get_thread_num();
    const int i = grid[q];
    const int ci[3] = {cellOf(i, 0), cellOf(i, 1), cellOf(i, 2)};
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          const int cx = ci[0] + dx, cy = ci[1] + dy, cz = ci[2] + dz;
          if (cx < 0 || cy < 0 || cz < 0 || cx >= nc[0] || cy >= nc[1] || cz >= nc[2]) continue;
          const long c = cx + nc[0] * (cy + (long)nc[1] * cz);
          for (long m = start[c]; m < start[c + 1]; m++) if (members[m] > i) consider(i, members[m], tid);
        }
  }
#pragma omp parallel for schedule(dynamic, 1024)
  for (long i = 0; i < nP; i++) {
    if (!S.par[i].bound.has) continue;
    for (int L : large)
      if (L != (int)i && (inGrid[i] || L < (int)i)) consider(std::min((int)i, L), std::max((int)i, L), omp_get_thread_num());
  }
  /* existing non-real contacts met along sortAxis whose boxes no longer overlap */
  const long nl = (long)S.linView.size();
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nl; k++) {
    const CPtr& C = S.linView[k];
    if (C->isReal()) continue;
    const int a = C->pA, b = C->pB;
    const bool meet = !(mx[3 * a + ax] < mn[3 * b + ax] || mx[3 * b + ax] < mn[3 * a + ax]);
    if (meet && !spatialOverlap(S, a, b)) S.removeT[omp_get_thread_num()].push_back(C);
  }
}
#endif

/* InsertionSortCollider::run, aperiodic (InsertionSortCollider.cpp:386-613) */
static void colliderRun(Scene& S) {
  bool fullRun = false;
  if (S.dirty) { fullRun = true; S.dirty = false; }
  long nPar = (long)S.par.size();
  if ((long)S.BB[0].size() != 2 * nPar) fullRun = true;
  /* updateBboxes_doFullRun (:308-358) */
  setVerletDist(S);
  bool recompute = false;
  if (S.verletDist == 0) recompute = true;
  else {
    const long np = (long)S.par.size();
    int dirtyAny = 0;
#ifdef _OPENMP
#pragma omp parallel for reduction(| : dirtyAny) if (S.parallel || S.detParallel)
#endif
    for (long i = 0; i < np; i++) if (aabbIsDirty(S.par[i])) dirtyAny |= 1;
    recompute = dirtyAny != 0;
  }
  if (recompute) {
    const long np = (long)S.par.size();
#ifdef _OPENMP
#pragma omp parallel for if (S.parallel || S.detParallel)
#endif
    for (long i = 0; i < np; i++) updateAabb(S, S.par[i]);
  }
  if (recompute) fullRun = true;
  S.lastRunFull = fullRun;
  if (!fullRun) {
    /* removePending (ContactContainer.hpp:78-93) with shouldBeRemoved (InsertionSortCollider.hpp:213-218) */
    auto pend = S.pending; S.pending.clear();
    for (auto& pc : pend) if (pc.second || !overlapAny(S, pc.first->pA, pc.first->pB)) removeContact(S, pc.first);
    return;
  }
  if (S.periodic) {
    S.nFullRuns++;
    long nP = (long)S.par.size();
    S.minima.assign(3 * nP, 0); S.maxima.assign(3 * nP, 0);
    for (long id = 0; id < nP; id++)
      for (int k = 0; k < 3; k++) { S.minima[3 * id + k] = S.par[id].bound.min[k]; S.maxima[3 * id + k] = S.par[id].bound.max[k]; }
    auto pend = S.pending; S.pending.clear();
    for (auto& pc : pend) if (pc.second || !overlapAny(S, pc.first->pA, pc.first->pB)) removeContact(S, pc.first);
    for (int i = 0; i < 3; i++) S.BB[i].assign(2 * nP, Bounds());  /* marks "initialised" for the size check */
    colliderPeriodicFull(S);
    return;
  }
  S.nFullRuns++;
  bool doInitSort = false;
  if ((long)S.BB[0].size() != 2 * nPar) {
    for (int i = 0; i < 3; i++) S.BB[i].clear();
    doInitSort = true;
    for (int i = 0; i < 3; i++)
      for (long id = 0; id < nPar; id++) {
        S.BB[i].push_back(Bounds(0, (int)id, true));
        S.BB[i].push_back(Bounds(0, (int)id, false));
      }
  }
  S.minima.assign(3 * nPar, 0); S.maxima.assign(3 * nPar, 0);
  /* copy bounds (:457-494; an OpenMP loop over the bound index in the reference) */
  {
    const long nb = 2 * nPar;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (S.parallel)
#endif
    for (long i = 0; i < nb; i++)
      for (int j = 0; j < 3; j++) {
        Bounds& b = S.BB[j][i];
        const Aabb& bv = S.par[b.id].bound;
        b.hasBB = bv.has;
        b.coord = b.hasBB ? (b.isMin ? bv.min[j] : bv.max[j]) : S.par[b.id].pos[j];
      }
  }
  /* minima/maxima (:498-506) */
  for (long id = 0; id < nPar; id++)
    for (int k = 0; k < 3; k++) {
      S.minima[3 * id + k] = S.par[id].bound.min[k];
      S.maxima[3 * id + k] = S.par[id].bound.max[k];
    }
  /* removePending (:517) */
  {
    auto pend = S.pending; S.pending.clear();
    for (auto& pc : pend) if (pc.second || !spatialOverlap(S, pc.first->pA, pc.first->pB)) removeContact(S, pc.first);
  }
  if (!doInitSort) {
#ifdef _OPENMP
    if (S.parallel) {
      const int TH = omp_get_max_threads();
      S.makeT.assign(TH, std::vector<CPtr>());
      S.removeT.assign(TH, std::vector<CPtr>());
      for (int i = 0; i < 3; i++) insertionSortParallel(S, S.BB[i], true);
    } else
#endif
    for (int i = 0; i < 3; i++) insertionSort(S, S.BB[i], true);
  } else {
    /* std::sort(std::execution::par, ...) or __gnu_parallel::sort in the reference's OpenMP build (:540-553) */
#ifdef _OPENMP
    if (S.parallel) for (int i = 0; i < 3; i++) __gnu_parallel::sort(S.BB[i].begin(), S.BB[i].end());
    else
#endif
    for (int i = 0; i < 3; i++) std::sort(S.BB[i].begin(), S.BB[i].end());
#ifdef _OPENMP
    if (S.parallel) { initialPairsGrid(S); goto process; }
#endif
    {
    std::vector<Bounds>& V = S.BB[S.sortAxis];
    long n2 = 2 * nPar;
    for (long i = 0; i < n2; i++) {
      if (!(V[i].isMin && V[i].hasBB)) continue;
      int iid = V[i].id;
      for (long j = i + 1; j < n2 && V[j].id != iid; j++) {
        if (!V[j].isMin) continue;
        handleBoundInversion(S, iid, V[j].id, false);
      }
    }
    }
  }
#ifdef _OPENMP
process:
#endif
  /* makeRemoveContactLater_process (:35-63): removals first, then additions (per-thread queues in
   * thread order in the OpenMP build) */
  for (auto& C : S.removeContacts) removeMaybe_fast(S, C);
  S.removeContacts.clear();
  for (auto& q : S.removeT) { for (auto& C : q) removeMaybe_fast(S, C); q.clear(); }
  for (auto& C : S.makeContacts) addMaybe_fast(S, C);
  S.makeContacts.clear();
  for (auto& q : S.makeT) { for (auto& C : q) addMaybe_fast(S, C); q.clear(); }
}

/* ------------------------------------------------------------------ geometry */
/* L6Geom::setInitialLocalCoords (L6Geom.cpp:25-36) */
static void setInitialLocalCoords(Contact& C, const V3& locX) {
  V3 e = std::abs(locX.y) < std::abs(locX.z) ? V3(0, 1, 0) : V3(0, 0, 1);
  V3 locY = cross(locX, e);
  locY = locY - locX * dot(locY, locX);
  normalize(locY);
  V3 locZ = cross(locX, locY);
  C.trsf.c[0] = locX; C.trsf.c[1] = locY; C.trsf.c[2] = locZ;
}
/* Cg2_Any_Any_L6Geom__Base::handleSpheresLikeContact (L6Geom.cpp:49-216), L6_TRSF_QUATERNION undefined */
static void handleSpheresLikeContact(Scene& S, Contact& C, const V3& pos1, const V3& vel1, const V3& angVel1,
                                     const V3& pos2, const V3& vel2, const V3& angVel2, const V3& normal,
                                     const V3& contPt, double uN, double r1, double r2) {
  const wdem_params& P = S.P;
  if (!C.geom) {
    C.geom = true;
    C.gvel = V3(); C.gangVel = V3();
    setInitialLocalCoords(C, normal);
    C.uN = uN;
    if (P.iniLensTouch) { C.lens[0] = std::abs(r1); C.lens[1] = std::abs(r2); }
    else { C.lens[0] = std::abs(r1) + uN / 2; C.lens[1] = std::abs(r2) + uN / 2; }
    if (C.lens[0] < 0) C.lens[0] = C.lens[1];
    if (C.lens[1] < 0) C.lens[1] = C.lens[0];
    C.contA = M_PI * pow2((r1 > 0 && r2 > 0) ? std::min(r1, r2) : (r1 > 0 ? r1 : r2));
    C.contPt = contPt;
    C.gori = quatFromMatrix(C.trsf);
    return;
  }
  const V3 currNormal = normal;
  const V3 prevNormal = C.trsf.c[0];
  const V3 prevContPt = C.contPt;
  const double dt = P.dt;
  V3 shiftVel2 = S.periodic ? S.cell.intrShiftVel(C.cellDist) : V3();
  V3 normRotVec = cross(prevNormal, currNormal);
  V3 midNormal = (P.approxMask & 1) ? prevNormal : 0.5 * (prevNormal + currNormal);
  if (norm(midNormal) == 0) midNormal = currNormal;
  else if (!(P.approxMask & 2) && !(P.approxMask & 1)) normalize(midNormal);
  V3 normTwistVec = midNormal * dt * 0.5 * dot(midNormal, angVel1 + angVel2);
  const M3 prevTrsf = C.trsf;
  M3 midTrsf;
  if (P.approxMask & 4) { midTrsf.c[0] = prevNormal; midTrsf.c[1] = prevTrsf.c[1]; }
  else { midTrsf.c[0] = midNormal; midTrsf.c[1] = prevTrsf.c[1] - cross(prevTrsf.c[1], normRotVec + normTwistVec) / 2.; }
  midTrsf.c[2] = cross(midTrsf.c[0], midTrsf.c[1]);
  M3 currTrsf;
  currTrsf.c[0] = currNormal;
  currTrsf.c[1] = prevTrsf.c[1] - cross(midTrsf.c[1], normRotVec + normTwistVec);
  currTrsf.c[2] = cross(currTrsf.c[0], currTrsf.c[1]);
  if (P.trsfRenorm > 0 && (S.step % P.trsfRenorm) == 0) {
    normalize(currTrsf.c[0]);
    currTrsf.c[1] = currTrsf.c[1] - currTrsf.c[0] * dot(currTrsf.c[1], currTrsf.c[0]);
    normalize(currTrsf.c[1]);
    currTrsf.c[2] = cross(currTrsf.c[0], currTrsf.c[1]);
  }
  V3 midContPt, midPos1, midPos2;
  if (P.approxMask & 8) { midContPt = contPt; midPos1 = pos1; midPos2 = pos2; }
  else { midContPt = 0.5 * (prevContPt + contPt); midPos1 = pos1 - (dt / 2.) * vel1; midPos2 = pos2 - (dt / 2.) * (vel2 + shiftVel2); }
  V3 c1x = (P.noRatch && r1 > 0) ? r1 * midNormal : midContPt - midPos1;
  V3 c2x = (P.noRatch && r2 > 0) ? -r2 * midNormal : midContPt - midPos2;
  V3 relVel = (vel2 + shiftVel2 + cross(angVel2, c2x)) - (vel1 + cross(angVel1, c1x));
  C.trsf = currTrsf;
  C.gvel = mulT(midTrsf, relVel);
  C.gangVel = mulT(midTrsf, angVel2 - angVel1);
  C.uN = uN;
  C.contPt = contPt;
  C.gori = quatFromMatrix(C.trsf);
}
/* Cg2_Sphere_Sphere_L6Geom::go (Sphere.cpp:92-117) */
static bool cg2SphereSphere(Scene& S, Contact& C, Particle& A, Particle& B, const V3& shift2, bool force) {
  const double r1 = A.radius, r2 = B.radius;
  const double distFactor = S.P.distFactor;
  V3 relPos = B.pos + shift2 - A.pos;
  double unDistSq = sqnorm(relPos) - pow2(std::abs(distFactor) * (r1 + r2));
  if (unDistSq > 0 && !C.isReal() && !force) return false;
  double dist = norm(relPos);
  double uN = dist - (r1 + r2);
  V3 normal = relPos / dist;
  V3 contPt = A.pos + (r1 + 0.5 * uN) * normal;
  handleSpheresLikeContact(S, C, A.pos, A.vel, A.angVel, B.pos + shift2, B.vel, B.angVel, normal, contPt, uN, r1, r2);
  return true;
}
/* Cg2_Wall_Sphere_L6Geom::go (Wall.cpp:50-84) */
static bool cg2WallSphere(Scene& S, Contact& C, Particle& W, Particle& Sp, const V3& shift2, bool force) {
  const double radius = Sp.radius;
  const int ax = W.axis, sense = W.sense;
  const V3 wallPos = W.pos;
  V3 spherePos = Sp.pos + shift2;
  double dist = spherePos[ax] - wallPos[ax];
  if (!C.isReal() && std::abs(dist) > radius && !force) return false;
  V3 contPt = spherePos; contPt[ax] = wallPos[ax];
  V3 normal;
  if (sense == 0) {
    if (!C.geom) normal[ax] = dist > 0 ? 1. : -1.;
    else normal[ax] = C.trsf.c[0][ax];
  } else normal[ax] = (sense == 1 ? 1. : -1);
  double uN = normal[ax] * dist - radius;
  handleSpheresLikeContact(S, C, wallPos, W.vel, W.angVel, spherePos, Sp.vel, Sp.angVel, normal, contPt, uN, -radius, radius);
  return true;
}

/* ------------------------------------------------------------------ facets */
/* CompUtils::closestSegmentPt (CompUtils.cpp:59-65) */
static V3 closestSegmentPt(const V3& P, const V3& A, const V3& B) {
  const V3 BA = B - A;
  if (sqnorm(BA) == 0.) return A;
  const double u = (dot(P, BA) - dot(A, BA)) / sqnorm(BA);
  return A + std::min(1., std::max(0., u)) * BA;
}
/* CompUtils::triangleBarycentrics (CompUtils.cpp:94-112): the 2x2 system by Eigen's closed-form inverse
 * (1/det times the adjugate, det = m00 m11 - m10 m01) */
static V3 triangleBarycentrics(const V3& x, const V3& A, const V3& B, const V3& C) {
  const V3 vB = B - A, vC = C - A, vX = x - A;
  const double m00 = dot(vB, vB), m01 = dot(vC, vB), m10 = dot(vB, vC), m11 = dot(vC, vC);
  const double invdet = 1. / (m00 * m11 - m10 * m01);
  const double i00 = m11 * invdet, i10 = -m10 * invdet, i01 = -m01 * invdet, i11 = m00 * invdet;
  const double b0 = dot(vX, vB), b1 = dot(vX, vC);
  const double u = i00 * b0 + i01 * b1, v = i10 * b0 + i11 * b1;
  return V3(1 - u - v, u, v);
}
/* Cg2_Facet_Sphere_L6Geom::go (Facet.cpp:333-390) for a facet without neighbour angles (n21lim NaN: no
 * boundary adjustment) and without fakeVel; Facet::getNormal, getOuterVectors (Facet.cpp:76-79, 110-116),
 * interpolatePtLinAngVel (Facet.cpp:162-179). */
static bool cg2FacetSphere(Scene& S, Contact& C, Particle& F, Particle& Sp, const V3& shift2, bool force) {
  const V3 n0 = F.pos, n1 = F.fv1, n2 = F.fv2;
  const double ht = F.radius, r = Sp.radius;
  const V3 sC = Sp.pos + shift2;
  V3 fNormal = cross(n1 - n0, n2 - n0);
  normalize(fNormal);
  const double planeDist = dot(sC - n0, fNormal);
  if (std::abs(planeDist) > (r + ht) && !C.isReal() && !force) return false;
  const V3 fC = sC - planeDist * fNormal;
  const V3 nn = cross(n1 - n0, n2 - n0);
  const V3 outVec[3] = {cross(n1 - n0, nn), cross(n2 - n1, nn), cross(n0 - n2, nn)};
  const V3 nodes[3] = {n0, n1, n2};
  double ll[3];
  for (int i = 0; i < 3; i++) ll[i] = dot(outVec[i], fC - nodes[i]);
  const int w = (ll[0] > 0 ? 1 : 0) + (ll[1] > 0 ? 2 : 0) + (ll[2] > 0 ? 4 : 0);
  V3 contPt;
  switch (w) {
    case 0: contPt = fC; break;
    case 1: contPt = closestSegmentPt(fC, n0, n1); break;
    case 2: contPt = closestSegmentPt(fC, n1, n2); break;
    case 4: contPt = closestSegmentPt(fC, n2, n0); break;
    case 3: contPt = n1; break;
    case 5: contPt = n0; break;
    case 6: contPt = n2; break;
    default: throw std::logic_error("Cg2_Facet_Sphere_L6Geom: impossible sphere-facet intersection");
  }
  V3 normal = sC - contPt;
  if (sqnorm(normal) > pow2(r + ht) && !C.isReal() && !force) return false;
  const double dist = norm(normal);
  if (dist != 0) normal = normal / dist;
  else normal = C.geom ? qrot(C.gori, V3(1, 0, 0)) : V3(1, 0, 0);
  if (ht > 0) contPt = contPt + normal * ht;
  const double uN = dist - r - ht;
  /* velocity of the facet at contPt: barycentric interpolation of the nodes' velocities (zero: fixed) */
  const V3 a = triangleBarycentrics(contPt, n0, n1, n2);
  const V3 vv[3] = {F.vel, V3(), V3()};
  const V3 linVel = a[0] * vv[0] + a[1] * vv[1] + a[2] * vv[2];
  const V3 angVel = cross(n0 - contPt, vv[0]) + cross(n1 - contPt, vv[1]) + cross(n2 - contPt, vv[2]);
  handleSpheresLikeContact(S, C, contPt, linVel, angVel, sC, Sp.vel, Sp.angVel, normal, contPt, uN, std::max(ht, r), r);
  return true;
}

/* ------------------------------------------------------------------ capsules */
/* Cg2_Sphere_Capsule_L6Geom::go (Capsule.cpp:198-216): the closest point of the capsule's axis segment */
static bool cg2SphereCapsule(Scene& S, Contact& C, Particle& Sp, Particle& Cap, const V3& shift2, bool force) {
  const V3 spherePos = Sp.pos;
  const V3 capPos = Cap.pos + shift2;
  const double rSum = Sp.radius + Cap.radius;
  const V3 half = qrot(Cap.ori, V3(Cap.shaft / 2., 0, 0));
  const V3 A = capPos - half, B = capPos + half;
  const V3 pt = closestSegmentPt(spherePos, A, B);
  const double distSq = sqnorm(pt - spherePos);
  if (!C.isReal() && distSq > pow2(rSum) && !force) return false;
  const double dist = std::sqrt(distSq);
  const V3 normal = (pt - spherePos) / dist;
  const double uN = dist - rSum;
  const V3 contPt = spherePos + normal * (Sp.radius + .5 * uN);
  handleSpheresLikeContact(S, C, spherePos, Sp.vel, Sp.angVel, capPos, Cap.vel, Cap.angVel, normal, contPt, uN, Sp.radius, Cap.radius);
  return true;
}

/* Cg2_Wall_Capsule_L6Geom::go (Capsule.cpp:116-164): the overlaps of the two end caps with the wall place
 * the contact point (weighted by the overlaps) and give uN */
static bool cg2WallCapsule(Scene& S, Contact& C, Particle& W, Particle& Cap, const V3& shift2, bool force) {
  const V3 wallPos = W.pos;
  const V3 capPos = Cap.pos + shift2;
  const int ax = W.axis, sense = W.sense;
  const V3 half = qrot(Cap.ori, V3(Cap.shaft / 2., 0, 0));
  const V3 AB[2] = {capPos - half, capPos + half};
  const double d0 = AB[0][ax] - wallPos[ax], d1 = AB[1][ax] - wallPos[ax];
  if (!C.isReal() && (std::abs(d0) > Cap.radius && std::abs(d1) > Cap.radius) && !force) return false;
  const double cDist = capPos[ax] - wallPos[ax];
  V3 normal(0, 0, 0);
  if (sense == 0) normal[ax] = C.geom ? C.trsf.c[0][ax] : (cDist > 0 ? 1. : -1.);
  else normal[ax] = (sense == 1 ? 1. : -1);
  const double u0 = d0 * normal[ax] - Cap.radius, u1 = d1 * normal[ax] - Cap.radius;
  V3 contPt;
  double uN;
  if (u0 * u1 < 0) {
    /* the ends on opposite sides: the overlapping one takes all */
    const int q = (u0 < 0 ? 0 : 1);
    contPt = AB[q];
    uN = q == 0 ? u0 : u1;
  } else if (u0 + u1 != 0.) {
    const double sum = u0 + u1;
    double w0 = u0 / sum, w1 = u1 / sum;
    if (u0 > 0) std::swap(w0, w1);  /* no overlap: the end closer to the wall weighs more */
    contPt = w0 * AB[0] + w1 * AB[1];
    uN = w0 * u0 + w1 * u1;
  } else {
    contPt = .5 * (AB[0] + AB[1]);
    uN = 0.;
  }
  contPt[ax] = wallPos[ax];
  handleSpheresLikeContact(S, C, wallPos, W.vel, W.angVel, capPos, Cap.vel, Cap.angVel, normal, contPt, uN, -Cap.radius, Cap.radius);
  return true;
}

/* CompUtils::distSq_SegmentSegment (CompUtils.cpp:260-592): squared distance of two segments given by centre,
 * unit direction and half-length, with the parameters (s0, s1) of the closest points -- D. Eberly's method
 * ("Distance Between Two Line Segments in 3D", Geometric Tools) as the reference has it: the minimum of the
 * quadratic in (s0, s1) is classified into the nine regions of the parameter rectangle; on a side one
 * parameter sits at its bound and the other is minimised and clamped, a corner tries one side and, when the
 * clamp ends on the far bound, the other; nearly parallel segments (|1 - (d0.d1)^2| < 1e-8) take the
 * symmetric average of the two one-sided solutions.  Every region keeps the reference's order of
 * comparisons and of the additions in the distance formulas. */
struct SegSeg {
  double a01, b0, b1, c, e0, e1;
  /* s1 = f, s0 = the clamped minimiser t = -(a01 f + b0); lowFirst: tested as t < -e0, t <= e0, else;
   * otherwise as t > e0, t >= -e0, else.  far: the last branch was taken. */
  double withS1(double f, bool lowFirst, double& s0, double& s1, bool& far) const {
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
  /* s0 = f, s1 = the clamped minimiser t = -(a01 f + b1) */
  double withS0(double f, bool lowFirst, double& s0, double& s1) const {
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
static double distSqSegSeg(const V3& c0, const V3& d0, double e0, const V3& c1, const V3& d1, double e1, double& s0, double& s1) {
  const V3 diff = c0 - c1;
  SegSeg g;
  g.a01 = -dot(d0, d1);
  g.b0 = dot(diff, d0);
  g.b1 = -dot(diff, d1);
  g.c = sqnorm(diff);
  g.e0 = e0;
  g.e1 = e1;
  const double a01 = g.a01, b0 = g.b0, b1 = g.b1, c = g.c;
  const double det = std::abs(1. - a01 * a01);
  double d;
  bool far;
  if (det >= 1e-8) {
    s0 = a01 * b1 - b0;
    s1 = a01 * b0 - b1;
    const double ed0 = e0 * det, ed1 = e1 * det;
    if (s0 >= -ed0) {
      if (s0 <= ed0) {
        if (s1 >= -ed1) {
          if (s1 <= ed1) {                                    /* interior */
            const double inv = 1. / det;
            s0 *= inv;
            s1 *= inv;
            d = s0 * (s0 + a01 * s1 + 2. * b0) + s1 * (a01 * s0 + s1 + 2. * b1) + c;
          } else d = g.withS1(e1, true, s0, s1, far);        /* side s1 = e1 */
        } else d = g.withS1(-e1, true, s0, s1, far);         /* side s1 = -e1 */
      } else {
        if (s1 >= -ed1) {
          if (s1 <= ed1) d = g.withS0(e0, true, s0, s1);     /* side s0 = e0 */
          else {                                             /* corner (e0, e1) */
            d = g.withS1(e1, true, s0, s1, far);
            if (far) d = g.withS0(e0, true, s0, s1);
          }
        } else {                                             /* corner (e0, -e1) */
          d = g.withS1(-e1, true, s0, s1, far);
          if (far) d = g.withS0(e0, false, s0, s1);
        }
      }
    } else {
      if (s1 >= -ed1) {
        if (s1 <= ed1) d = g.withS0(-e0, true, s0, s1);      /* side s0 = -e0 */
        else {                                               /* corner (-e0, e1) */
          d = g.withS1(e1, false, s0, s1, far);
          if (far) d = g.withS0(-e0, true, s0, s1);
        }
      } else {                                               /* corner (-e0, -e1) */
        d = g.withS1(-e1, false, s0, s1, far);
        if (far) d = g.withS0(-e0, true, s0, s1);
      }
    }
  } else {
    /* parallel: the averaged b0 makes the distance symmetric in the two segments */
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

/* Cg2_Capsule_Capsule_L6Geom::go (Capsule.cpp:223-323): uN and the normal from the closest points of the two
 * axis segments; the contact point from the closest points unless two or more end caps overlap the other
 * capsule's axis, in which case the overlapping ends' points (each moved towards its capsule's end by the
 * other's radius share) are averaged with weights rSum - distance */
static bool cg2CapsuleCapsule(Scene& S, Contact& C, Particle& P1, Particle& P2, const V3& shift2, bool force) {
  const V3 pos1 = P1.pos, pos2 = P2.pos + shift2;
  const V3 dir1 = qrot(P1.ori, V3(1, 0, 0)), dir2 = qrot(P2.ori, V3(1, 0, 0));
  const double rSum = P1.radius + P2.radius;
  double u, v;
  const double distSq = distSqSegSeg(pos1, dir1, .5 * P1.shaft, pos2, dir2, .5 * P2.shaft, u, v);
  if (!C.isReal() && distSq > pow2(rSum) && !force) return false;
  const V3 close0 = pos1 + dir1 * u, close1 = pos2 + dir2 * v;
  const V3 ends[2][2] = {{pos1 - .5 * P1.shaft * dir1, pos1 + .5 * P1.shaft * dir1},
                         {pos2 - .5 * P2.shaft * dir2, pos2 + .5 * P2.shaft * dir2}};
  const double dist = std::sqrt(distSq);
  const double uN = dist - (P1.radius + P2.radius);
  const V3 normal = (close1 - close0) / dist;
  int bits = 0, nOver = 0;
  V3 eClose[2][2];
  double eDistSq[2][2];
  for (int a = 0; a < 2; a++) {
    const int b = 1 - a;
    for (int e = 0; e < 2; e++) {
      eClose[a][e] = closestSegmentPt(ends[a][e], ends[b][0], ends[b][1]);
      eDistSq[a][e] = sqnorm(eClose[a][e] - ends[a][e]);
      if (eDistSq[a][e] < pow2(rSum)) { bits |= 1 << (2 * a + e); nOver++; }
    }
  }
  const double r1r = P1.radius / rSum, r2r = P2.radius / rSum;
  /* the overlapping end moved from its closest point on the other axis towards itself by the other's share */
  auto endPoint = [&](int a, int e) { return eClose[a][e] + (ends[a][e] - eClose[a][e]) * (a == 0 ? r2r : r1r); };
  auto endWeight = [&](int a, int e) { return rSum - std::sqrt(eDistSq[a][e]); };
  V3 contPt;
  if (nOver < 2) contPt = close0 + (P1.radius + 0.5 * uN) * normal;
  else if (nOver == 4) {
    V3 pp(0, 0, 0);
    double ww = 0.;
    for (int a = 0; a < 2; a++)
      for (int e = 0; e < 2; e++) {
        const double w = endWeight(a, e);
        pp = pp + w * endPoint(a, e);
        ww += w;
      }
    contPt = pp / ww;
  } else {
    /* two or three overlapping ends (bit 2a+e for end e of capsule a): the two that place the contact; with
     * three, the two ends of the capsule whose both ends overlap (the reference's lookup table) */
    static const int pick[16][2][2] = {
        {{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}, {{0, 0}, {0, 1}},
        {{0, 0}, {0, 0}}, {{0, 0}, {1, 0}}, {{0, 1}, {1, 0}}, {{0, 0}, {0, 1}},
        {{0, 0}, {0, 0}}, {{0, 0}, {1, 1}}, {{0, 1}, {1, 1}}, {{0, 0}, {0, 1}},
        {{1, 0}, {1, 1}}, {{1, 0}, {1, 1}}, {{1, 0}, {1, 1}}, {{0, 0}, {0, 0}}};
    const int (&ix)[2][2] = pick[bits];
    const V3 p0 = endPoint(ix[0][0], ix[0][1]), p1 = endPoint(ix[1][0], ix[1][1]);
    const double w0 = endWeight(ix[0][0], ix[0][1]), w1 = endWeight(ix[1][0], ix[1][1]);
    contPt = (w0 * p0 + w1 * p1) / (w0 + w1);
  }
  handleSpheresLikeContact(S, C, pos1, P1.vel, P1.angVel, pos2, P2.vel, P2.angVel, normal, contPt, uN, P1.radius, P2.radius);
  return true;
}

/* ------------------------------------------------------------------ ellipsoids */
/* Brent's minimisation without derivatives (R. P. Brent, "Algorithms for Minimization without
 * Derivatives", 1973, ch. 5) as boost::math::tools::brent_find_minima performs it (Boost.Math,
 * header-only, not vendored; the reference CI builds against Ubuntu 20.04's libboost 1.71).  Called at
 * Ellipsoid.cpp:309 on [0, 1]: the requested bits are capped at half the mantissa (26 for double),
 * tolerance 2^(1-bits); start at the upper end; a parabolic step through the three best points when it
 * stays inside the bracket and shrinks, else a golden-section step (0.3819660, a float constant);
 * never step by less than the tolerance.  Returns the abscissa and value of the minimum. */
template <class F>
static std::pair<double, double> brentMin(F f, double lo, double hi, int bits, long* evals) {
  bits = std::min(std::numeric_limits<double>::digits / 2, bits);
  const double tol = std::ldexp(1.0, 1 - bits);
  const double golden = (double)0.3819660f;
  double x = hi, w = hi, v = hi;
  double fx = f(x), fw = fx, fv = fx;
  double step = 0, step2 = 0;
  long n = 1;
  for (;;) {
    const double mid = (lo + hi) / 2;
    const double t1 = tol * std::abs(x) + tol / 4;
    const double t2 = 2 * t1;
    if (std::abs(x - mid) <= (t2 - (hi - lo) / 2)) break;
    bool golden_step = true;
    if (std::abs(step2) > t1) {
      double r = (x - w) * (fx - fv);
      double q = (x - v) * (fx - fw);
      double p = (x - v) * q - (x - w) * r;
      q = 2 * (q - r);
      if (q > 0) p = -p;
      q = std::abs(q);
      const double prev = step2;
      step2 = step;
      if (!((std::abs(p) >= std::abs(q * prev / 2)) || (p <= q * (lo - x)) || (p >= q * (hi - x)))) {
        golden_step = false;
        step = p / q;
        const double u = x + step;
        if (((u - lo) < t2) || ((hi - u) < t2)) step = (mid - x) < 0 ? -std::abs(t1) : std::abs(t1);
      }
    }
    if (golden_step) {
      step2 = (x >= mid) ? lo - x : hi - x;
      step = golden * step2;
    }
    const double u = (std::abs(step) >= t1) ? x + step : (step > 0 ? x + std::abs(t1) : x - std::abs(t1));
    const double fu = f(u);
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
  if (evals) *evals += n;
  return std::make_pair(x, fx);
}

/* Perram-Wertheim contact function of two ellipsoids (Ellipsoid.cpp:270-351; Perram & Wertheim 1985,
 * Donev et al. 2005): A = sum u_k u_k^T / a_k^2, S(l) = l (1-l) R^T G(l)^-1 R with G = (1-l) A^-1 + l B^-1. */
struct PwPair {
  Mat Ainv, Binv;
  V3 R;
};
static PwPair pwSetup(const Quat& oa, const V3& a, const Quat& ob, const V3& b, const V3& R) {
  PwPair P;
  Mat A, B;
  const V3 e[3] = {V3(1, 0, 0), V3(0, 1, 0), V3(0, 0, 1)};
  for (int k = 0; k < 3; k++) {
    const V3 u = qrot(oa, e[k]), v = qrot(ob, e[k]);
    const double a2 = pow2(a[k]), b2 = pow2(b[k]);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        A.r[i][j] = A.r[i][j] + (u[i] * u[j]) / a2;
        B.r[i][j] = B.r[i][j] + (v[i] * v[j]) / b2;
      }
  }
  P.Ainv = minv(A);
  P.Binv = minv(B);
  P.R = R;
  return P;
}
static Mat pwG(const PwPair& P, double l) {
  Mat G;
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) G.r[i][j] = (1 - l) * P.Ainv.r[i][j] + l * P.Binv.r[i][j];
  return G;
}
/* the lambda functor of Ellipsoid.cpp:293: -l (1-l) R^T G^-1 R, evaluated left to right */
static double pwNegS(const PwPair& P, double l) {
  const Mat Gi = minv(pwG(P, l));
  const double sc = -l * (1 - l);
  const V3 sR = sc * P.R;
  V3 t;
  for (int j = 0; j < 3; j++) t[j] = sR.x * Gi.r[0][j] + sR.y * Gi.r[1][j] + sR.z * Gi.r[2][j];
  return t.x * P.R.x + t.y * P.R.y + t.z * P.R.z;
}
/* dS/dl = (1-2l) h + l (1-l) h' with h = R^T x, h' = -x^T (B^-1 - A^-1) x, x = G^-1 R */
static double pwDS(const PwPair& P, double l) {
  const Mat Gi = minv(pwG(P, l));
  const V3 x = mvec(Gi, P.R);
  const Mat D = madd(P.Binv, P.Ainv, -1.0);
  const double h = dot(P.R, x);
  const double hp = -dot(x, mvec(D, x));
  return (1 - 2 * l) * h + l * (1 - l) * hp;
}
/* The maximiser of S on [0, 1].  WDEM_ELL_BRENT: Brent on -S as the reference does.  Otherwise (the
 * oracle for the Newton solver): bisection on the sign of dS/dl, which is decreasing because S is
 * concave, to the last representable lambda, so the converged Newton solution is checked against
 * the exact maximiser rather than against Brent's 26-bit answer. */
static void pwSolve(const Scene& S, const PwPair& P, double& L, double& Fab, long* evals) {
  if (S.P.ellSolver == WDEM_ELL_BRENT) {
    auto r = brentMin([&](double l) { return pwNegS(P, l); }, 0., 1., S.P.brentBits, evals);
    L = r.first;
    Fab = -r.second;
    return;
  }
  double lo = 0, hi = 1;
  for (int it = 0; it < 200; it++) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (pwDS(P, mid) > 0) lo = mid; else hi = mid;
  }
  L = 0.5 * (lo + hi);
  Fab = -pwNegS(P, L);
}
/* Cg2_Ellipsoid_Ellipsoid_L6Geom::go_Ellipsoid_or_Sphere (Ellipsoid.cpp:270-351); a sphere enters with
 * semi-axes (r, r, r) and its own orientation (Cg2_Sphere_Ellipsoid_L6Geom::go, :262) */
static bool cg2EllipsoidOrSphere(Scene& S, Contact& C, Particle& A, const V3& a, Particle& B, const V3& b,
                                 const V3& shift2, bool force) {
  const V3 ra = A.pos, rb = B.pos + shift2;
  const V3 R = rb - ra;
  const PwPair P = pwSetup(A.ori, a, B.ori, b, R);
  double L, Fab;
  pwSolve(S, P, L, Fab, S.parallel ? nullptr : &S.ellEvals);
  if (!S.parallel) S.ellSolves++;
  if (Fab > 1 && !C.isReal() && !force) return false;
  const Mat Gi = minv(pwG(P, L));
  const V3 nUnnorm = mvec(Gi, P.R);
  const V3 contPt = ra + mvec(mscale(P.Ainv, 1 - L), nUnnorm);
  const double mu = std::sqrt(Fab);
  const double Rnorm = norm(R);
  V3 nUnit = nUnnorm;
  normalize(nUnit);
  const V3 rUnit = R / Rnorm;
  const double uN = Rnorm * (1 - 1 / mu) * dot(rUnit, nUnit);
  handleSpheresLikeContact(S, C, ra, A.vel, A.angVel, rb, B.vel, B.angVel, nUnit, contPt, uN, norm(contPt - ra),
                           norm(contPt - rb));
  return true;
}
/* Cg2_Wall_Ellipsoid_L6Geom::go (Ellipsoid.cpp:227-257) */
static bool cg2WallEllipsoid(Scene& S, Contact& C, Particle& W, Particle& E, const V3& shift2, bool force) {
  const int ax = W.axis, sense = W.sense;
  const V3 wallPos = W.pos;
  const V3 ellPos = E.pos + shift2;
  const M3 M = ellTrsf(E);
  const double extent = std::sqrt(M.c[0][ax] * M.c[0][ax] + M.c[1][ax] * M.c[1][ax] + M.c[2][ax] * M.c[2][ax]);
  if (((wallPos[ax] < (ellPos[ax] - extent)) || (wallPos[ax] > (ellPos[ax] + extent))) && !C.isReal() && !force) return false;
  const double dist = ellPos[ax] - wallPos[ax];
  int normAxSgn;
  if (sense == 0) normAxSgn = dist > 0 ? 1 : -1;
  else normAxSgn = (sense == 1 ? 1 : -1);
  const V3 normal = (double)normAxSgn * V3(ax == 0 ? 1. : 0., ax == 1 ? 1. : 0., ax == 2 ? 1. : 0.);
  const double uN = normAxSgn * dist - extent;
  /* Mprime = M^T with unit columns; contact point = centre - normAxSgn (M Mprime).col(ax) */
  V3 mp(M.c[0][ax], M.c[1][ax], M.c[2][ax]);   /* column ax of M^T = row ax of M */
  normalize(mp);
  V3 col;
  for (int i = 0; i < 3; i++) col[i] = M.c[0][i] * mp.x + M.c[1][i] * mp.y + M.c[2][i] * mp.z;
  V3 contPt = ellPos + (double)(-normAxSgn) * col;
  contPt[ax] = wallPos[ax];
  const double contR = norm(contPt - ellPos);
  handleSpheresLikeContact(S, C, wallPos, W.vel, W.angVel, ellPos, E.vel, E.angVel, normal, contPt, uN, -contR, contR);
  return true;
}

/* ------------------------------------------------------------------ physics */
/* Cp2_FrictMat_FrictPhys::updateFrictPhys (FrictMat.cpp:20-44), MatchMaker unset -> min tanPhi */
static void cp2Frict(Scene& S, Contact& C, const wdem_material& m1, const wdem_material& m2) {
  C.phys = true;
  double l0 = C.lens[0], l1 = C.lens[1], A = C.contA;
  C.kn = 1 / (1 / (m1.young * A / l0) + 1 / (m2.young * A / l1));
  C.kt = .5 * (m1.ktDivKn + m2.ktDivKn) * C.kn;
  C.tanPhi = std::min(m1.tanPhi, m2.tanPhi);
}
/* Cp2_HertzMat_HertzPhys::go (Hertz.cpp:34-77) */
static void cp2Hertz(Scene& S, Contact& C, const wdem_material& m1, const wdem_material& m2) {
  C.phys = true;
  const double r1 = C.lens[0], r2 = C.lens[1];
  const double E1 = m1.young, E2 = m2.young;
  const double nu1 = S.P.poisson, nu2 = S.P.poisson;
  C.K = (4 / 3.) * 1. / ((1 - nu1 * nu1) / E1 + (1 - nu2 * nu2) / E2);
  C.R = 1. / (1. / r1 + 1. / r2);
  double kn0 = C.K * std::sqrt(C.R);
  C.gamma = std::min(m1.surfEnergy, m2.surfEnergy);
  C.alpha = .5 * (m1.alpha + m2.alpha);
  double G1 = E1 / (2 * (1 + nu1)); double G2 = E2 / (2 * (1 + nu2));
  double G = .5 * (G1 + G2);
  double nu = .5 * (nu1 + nu2);
  C.kt0 = 2 * std::sqrt(4 * C.R) * G / (2 - nu);
  C.tanPhi = std::min(m1.tanPhi, m2.tanPhi);
  double en = S.P.en;
  if (en > 0 && en < 1.) {
    const double ma = S.par[C.pA].mass, mb = S.par[C.pB].mass;
    double mbar = (ma <= 0 && mb > 0) ? mb : ((ma > 0 && mb <= 0) ? ma : (ma * mb) / (ma + mb));
    double viscAlpha = -std::sqrt(5) * std::log(en) / (std::sqrt(pow2(std::log(en)) + pow2(M_PI)));
    C.alpha_sqrtMK = std::max(0., viscAlpha * std::sqrt(mbar * kn0));
  } else C.alpha_sqrtMK = 0.0;
}
/* Law2_L6Geom_FrictPhys_IdealElPl::go (IdealElPl.cpp:15-125), iniEqlb unsupported */
static bool lawIdealElPl(Scene& S, Contact& C) {
  const wdem_params& P = S.P;
  double uN = C.uN;
  if (uN > 0 && !P.noBreak) {
    if (P.noSlip && P.trackEnergy) {
      double Fn = C.kn * uN;
      double ft0 = C.force.y + P.dt * C.kt * C.gvel.y, ft1 = C.force.z + P.dt * C.kt * C.gvel.z;
      S.E.v[WDEM_E_BROKEN] += .5 * (pow2(Fn) / C.kn + (ft0 * ft0 + ft1 * ft1) / C.kt);
    }
    return false;
  }
  C.torque = V3();
  C.force.x = C.kn * uN;
  if (P.noFrict || C.tanPhi == 0.) {
    C.force.y = 0; C.force.z = 0;
  } else {
    const double vt0 = C.gvel.y, vt1 = C.gvel.z;
    /* Ft += dt*kt*velT: the scalar (dt*kt) multiplies the vector */
    double s = P.dt * C.kt;
    C.force.y = C.force.y + s * vt0;
    C.force.z = C.force.z + s * vt1;
    double maxFt = std::abs(C.force.x) * C.tanPhi;
    double ftSq = C.force.y * C.force.y + C.force.z * C.force.z;
    if (ftSq > maxFt * maxFt && !P.noSlip) {
      double FtNorm = std::sqrt(ftSq);
      double ratio = maxFt / FtNorm;
      if (FtNorm == 0.) ratio = 0.;
      if (P.trackEnergy) {
        double dissip = (C.kt != 0. ? (maxFt) * (FtNorm - maxFt) / C.kt : 0.);
        S.E.v[WDEM_E_PLAST] += dissip;
      }
      C.force.y *= ratio; C.force.z *= ratio;
    }
    if (std::isnan(std::max(C.force.x, std::max(C.force.y, C.force.z)))) {
      S.err = "NaN force in contact ##" + std::to_string(C.pA) + "+" + std::to_string(C.pB);
      throw std::runtime_error(S.err);
    }
  }
  if (P.trackEnergy) {
    double ftSq = C.force.y * C.force.y + C.force.z * C.force.z;
    double elast = 0.5 * (pow2(C.force.x) / C.kn + (C.kt != 0. ? ftSq / C.kt : 0.));
    if (std::isnan(elast)) elast = 0.;
    S.E.v[WDEM_E_ELAST] += elast;
  }
  if (P.relRollStiff > 0. && P.rollTanPhi > 0.) {
    double charLen = C.lens[0] + C.lens[1];
    if (charLen <= 0) throw std::runtime_error("charLen<=0");
    double kr = C.kn * charLen;
    if (P.relTwistStiff > 0) {
      C.torque.x = C.torque.x + P.dt * P.relTwistStiff * kr * C.gangVel.x;
      double maxTt = std::abs(C.force.x * P.rollTanPhi * charLen);
      if (std::abs(C.torque.x) > maxTt) C.torque.x = std::copysign(maxTt, C.torque.x);
    }
    double s = P.dt * kr;
    C.torque.y = C.torque.y + s * C.gangVel.y;
    C.torque.z = C.torque.z + s * C.gangVel.z;
    double maxTr = std::max(0., std::abs(C.force.x) * P.rollTanPhi * charLen);
    double trSq = C.torque.y * C.torque.y + C.torque.z * C.torque.z;
    if (trSq > maxTr * maxTr) {
      double TrNorm = std::sqrt(trSq);
      double ratio = maxTr / TrNorm;
      if (TrNorm == 0.) ratio = 0.;
      C.torque.y *= ratio; C.torque.z *= ratio;
    }
  } else C.torque = V3();
  return true;
}
/* Law2_L6Geom_HertzPhys_DMT::go, DMT branch (Hertz.cpp:85-114, 170-210) */
static bool lawHertzDMT(Scene& S, Contact& C) {
  const wdem_params& P = S.P;
  C.torque = V3();
  const double dt = P.dt;
  const double velN = C.gvel.x;
  const double vt0 = C.gvel.y, vt1 = C.gvel.z;
  double kn0 = C.K * std::sqrt(C.R);
  C.kn = (3 / 2.) * kn0 * std::sqrt(-C.uN);
  double Fne, Fna = 0.;
  if (C.alpha == 0. || C.gamma == 0.) {
    if (C.uN > 0) return false;
    Fne = -kn0 * pown(std::sqrt(-C.uN), 3);
    Fna = 4 * M_PI * C.R * C.gamma;
  } else {
    S.err = "Schwarz branch of Law2_L6Geom_HertzPhys_DMT (alpha!=0 and gamma!=0) is not restated";
    throw std::runtime_error(S.err);
  }
  double eta = (C.alpha_sqrtMK > 0 ? C.alpha_sqrtMK * std::sqrt(std::sqrt(std::max(-C.uN, 0.))) : 0.);
  double Fnv = eta * velN;
  if (C.alpha == 0. && P.noAttraction && Fne + Fnv > 0) Fnv = -Fne;
  C.force.x = Fne + Fna + Fnv;
  if (P.trackEnergy) S.E.v[WDEM_E_VISCN] += Fnv * velN * dt;
  C.kt = C.kt0 * std::sqrt(C.uN < 0 ? -C.uN : 0);
  double s = dt * C.kt;
  C.force.y = C.force.y + s * vt0;
  C.force.z = C.force.z + s * vt1;
  double maxFt = std::abs(std::min(0., C.force.x) * C.tanPhi);
  double ftSq = C.force.y * C.force.y + C.force.z * C.force.z;
  if (ftSq > pow2(maxFt)) {
    double FtNorm = std::sqrt(ftSq);
    double ratio = maxFt / FtNorm;
    if (P.trackEnergy) S.E.v[WDEM_E_PLAST] += (.5 * (FtNorm - maxFt) + maxFt) * (FtNorm - maxFt) / C.kt;
    C.force.y *= ratio; C.force.z *= ratio;
  } else {
    C.force.y = C.force.y + eta * vt0;
    C.force.z = C.force.z + eta * vt1;
    if (P.trackEnergy) S.E.v[WDEM_E_VISCT] += eta * (vt0 * vt0 + vt1 * vt1) * dt;
  }
  if (P.trackEnergy && C.uN < 0) {
    double ftSq2 = C.force.y * C.force.y + C.force.z * C.force.z;
    S.E.v[WDEM_E_ELAST] += kn0 * (2 / 5.) * pown(std::sqrt(-C.uN), 5) + 0.5 * ftSq2 / C.kt;
  }
  return true;
}

/* Contact::getForceTorqueBranch (Contact.cpp:24-34) + DemData::addForceTorque (Particle.hpp:249) */
static void applyForceUninodal(Scene& S, const Contact& C, Particle& p) {
  if (p.shape == WDEM_SHAPE_FACET) return;  /* sh->nodes.size() != 1 (ContactLoop.cpp:272) */
  bool isPA = (C.pA == p.id);
  double sign = isPA ? 1 : -1;
  V3 F = qrot(C.gori, C.force) * sign;
  V3 T = (isZero(C.torque) ? V3() : qrot(C.gori, C.torque)) * sign;
  V3 xc = C.contPt - ((!isPA && S.periodic) ? p.pos + S.cell.intrShiftPos(C.cellDist) : p.pos);
  p.force = p.force + F;
  p.torque = p.torque + (cross(xc, F) + T);
}

static bool isSphereLike(int shape) { return shape == WDEM_SHAPE_SPHERE; }

/* The shape pairs with a Cg2 functor and the order each functor wants (FUNCTOR2D of Sphere.hpp,
 * Wall.hpp, Ellipsoid.hpp): Sphere+Sphere, Wall+Sphere, Ellipsoid+Ellipsoid, Sphere+Ellipsoid,
 * Wall+Ellipsoid.  On the first visit of a fresh potential contact the pair is swapped into that order
 * (Contact::swapOrder, Contact.cpp:12-16) and minDist00Sq is set (ContactLoop.cpp:147-153). */
static bool freshContactSetup(Scene& S, Contact& C) {
  const int sa = S.par[C.pA].shape, sb = S.par[C.pB].shape;
  const bool swap = (sa == WDEM_SHAPE_SPHERE && sb == WDEM_SHAPE_WALL) ||
                    (sa == WDEM_SHAPE_ELLIPSOID && sb == WDEM_SHAPE_SPHERE) ||
                    (sa == WDEM_SHAPE_ELLIPSOID && sb == WDEM_SHAPE_WALL) ||
                    (sa == WDEM_SHAPE_SPHERE && sb == WDEM_SHAPE_FACET) ||
                    (sa == WDEM_SHAPE_CAPSULE && sb == WDEM_SHAPE_SPHERE) ||
                    (sa == WDEM_SHAPE_CAPSULE && sb == WDEM_SHAPE_WALL);
  const bool known = swap || (sa == WDEM_SHAPE_SPHERE && sb == WDEM_SHAPE_SPHERE) ||
                     (sa == WDEM_SHAPE_FACET && sb == WDEM_SHAPE_SPHERE) ||
                     (sa == WDEM_SHAPE_SPHERE && sb == WDEM_SHAPE_CAPSULE) ||
                     (sa == WDEM_SHAPE_WALL && sb == WDEM_SHAPE_CAPSULE) ||
                     (sa == WDEM_SHAPE_CAPSULE && sb == WDEM_SHAPE_CAPSULE) ||
                     (sa == WDEM_SHAPE_WALL && sb == WDEM_SHAPE_SPHERE) ||
                     (sa == WDEM_SHAPE_ELLIPSOID && sb == WDEM_SHAPE_ELLIPSOID) ||
                     (sa == WDEM_SHAPE_SPHERE && sb == WDEM_SHAPE_ELLIPSOID) ||
                     (sa == WDEM_SHAPE_WALL && sb == WDEM_SHAPE_ELLIPSOID);
  if (!known) return false;
  if (swap) { std::swap(C.pA, C.pB); for (int k = 0; k < 3; k++) C.cellDist[k] *= -1; }
  const Particle& A = S.par[C.pA];
  const Particle& B = S.par[C.pB];
  if (A.shape == WDEM_SHAPE_SPHERE && B.shape == WDEM_SHAPE_SPHERE)
    C.minDist00Sq = pow2(std::abs(S.P.distFactor * (A.radius + B.radius)));        /* Sphere.cpp:86-89 */
  else if (A.shape == WDEM_SHAPE_ELLIPSOID && B.shape == WDEM_SHAPE_ELLIPSOID)
    C.minDist00Sq = pow2(maxCoeff(A.semiAxes) + maxCoeff(B.semiAxes));            /* Ellipsoid.cpp:265 */
  else if (A.shape == WDEM_SHAPE_SPHERE && B.shape == WDEM_SHAPE_ELLIPSOID)
    C.minDist00Sq = pow2(A.radius + maxCoeff(B.semiAxes));                        /* Ellipsoid.cpp:259 */
  else if (A.shape == WDEM_SHAPE_SPHERE && B.shape == WDEM_SHAPE_CAPSULE)
    C.minDist00Sq = pow2(A.radius + B.radius + .5 * B.shaft);                     /* Capsule.cpp:193-196 */
  else if (A.shape == WDEM_SHAPE_CAPSULE && B.shape == WDEM_SHAPE_CAPSULE)
    C.minDist00Sq = pow2(A.radius + .5 * A.shaft + B.radius + .5 * B.shaft);      /* Capsule.cpp:218-221 */
  else C.minDist00Sq = -1;
  return true;
}
static bool callGeom(Scene& S, Contact& C, Particle& pA, Particle& pB, const V3& shift2) {
  const int sa = pA.shape, sb = pB.shape;
  if (sa == WDEM_SHAPE_SPHERE && sb == WDEM_SHAPE_SPHERE) return cg2SphereSphere(S, C, pA, pB, shift2, false);
  if (sa == WDEM_SHAPE_WALL && sb == WDEM_SHAPE_SPHERE) return cg2WallSphere(S, C, pA, pB, shift2, false);
  if (sa == WDEM_SHAPE_ELLIPSOID && sb == WDEM_SHAPE_ELLIPSOID)
    return cg2EllipsoidOrSphere(S, C, pA, pA.semiAxes, pB, pB.semiAxes, shift2, false);
  if (sa == WDEM_SHAPE_SPHERE && sb == WDEM_SHAPE_ELLIPSOID)
    return cg2EllipsoidOrSphere(S, C, pA, V3(pA.radius, pA.radius, pA.radius), pB, pB.semiAxes, shift2, false);
  if (sa == WDEM_SHAPE_WALL && sb == WDEM_SHAPE_ELLIPSOID) return cg2WallEllipsoid(S, C, pA, pB, shift2, false);
  if (sa == WDEM_SHAPE_FACET && sb == WDEM_SHAPE_SPHERE) return cg2FacetSphere(S, C, pA, pB, shift2, false);
  if (sa == WDEM_SHAPE_SPHERE && sb == WDEM_SHAPE_CAPSULE) return cg2SphereCapsule(S, C, pA, pB, shift2, false);
  if (sa == WDEM_SHAPE_WALL && sb == WDEM_SHAPE_CAPSULE) return cg2WallCapsule(S, C, pA, pB, shift2, false);
  if (sa == WDEM_SHAPE_CAPSULE && sb == WDEM_SHAPE_CAPSULE) return cg2CapsuleCapsule(S, C, pA, pB, shift2, false);
  return false;
}

#ifdef _OPENMP
/* ContactLoop::run as the reference's OpenMP build runs it: guided parallel loop over the
 * contacts (ContactLoop.cpp:134-137), forces added under a per-node lock (DemData::addForceTorque,
 * Particle.hpp:249), removal requests collected per thread.  Used for the timed CPU baseline only. */
static void contactLoopParallel(Scene& S) {
  const wdem_params& P = S.P;
  const long size = (long)S.linView.size();
  std::vector<CPtr> removeAfter, removals;
  bool nanSeen = false;
  std::string nanMsg;
#pragma omp parallel
  {
    std::vector<CPtr> myRemoveAfter, myRemovals;
#pragma omp for schedule(guided)
    for (long i = 0; i < size; i++) {
      const CPtr C = S.linView[i];
      if (!C->isReal() && !C->isColliding()) { myRemoveAfter.push_back(C); continue; }
      bool fresh = (S.step == C->stepCreated);
      if (!C->isReal() && fresh && !freshContactSetup(S, *C)) continue;
      Particle& pA = S.par[C->pA];
      Particle& pB = S.par[C->pB];
      V3 shift2 = S.periodic ? S.cell.intrShiftPos(C->cellDist) : V3();
      if (P.dist00 && !C->isReal() && !fresh && C->minDist00Sq > 0 && sqnorm(pA.pos - (pB.pos + shift2)) > C->minDist00Sq) continue;
      if (!callGeom(S, *C, pA, pB, shift2)) continue;
      if (!C->phys) C->stepCreated = (int)S.step;
      if (!C->phys || S.updatePhys > WDEM_UPDATE_PHYS_NEVER) {
        const wdem_material& m1 = S.mats[pA.mat];
        const wdem_material& m2 = S.mats[pB.mat];
        if (P.cp2 == WDEM_CP2_FRICT) cp2Frict(S, *C, m1, m2); else cp2Hertz(S, *C, m1, m2);
      }
      bool keep = true;
      try {
        keep = (P.law == WDEM_LAW_IDEALELPL) ? lawIdealElPl(S, *C) : lawHertzDMT(S, *C);
      } catch (std::exception& e) {
#pragma omp critical
        { nanSeen = true; nanMsg = e.what(); }
      }
      if (!keep) {
        C->geom = false; C->phys = false;
        myRemovals.push_back(C);
        continue;
      }
      for (Particle* pp : {&pA, &pB}) {
        omp_set_lock(&S.locks[pp->id]);
        applyForceUninodal(S, *C, *pp);
        omp_unset_lock(&S.locks[pp->id]);
      }
    }
#pragma omp critical
    {
      removeAfter.insert(removeAfter.end(), myRemoveAfter.begin(), myRemoveAfter.end());
      removals.insert(removals.end(), myRemovals.begin(), myRemovals.end());
    }
  }
  if (nanSeen) throw std::runtime_error(nanMsg);
  for (auto& c : removals) requestRemoval(S, c);
  for (auto& c : removeAfter) removeContact(S, c);
  if (S.updatePhys == WDEM_UPDATE_PHYS_ONCE) S.updatePhys = WDEM_UPDATE_PHYS_NEVER;
}
#endif

#ifdef _OPENMP
/* The serial loop below computed by OpenMP threads, with its results bit for bit (the long canonical
 * parity runs): a contact's geometry, physics and law read the particles (unchanged during the loop) and
 * write that contact only, so the contacts run in parallel and their outcomes (dropped when not colliding,
 * removal requested by the law) are applied afterwards in container order, as the serial loop applies
 * them; forces are then added in key order.  Not used with energy tracking (the laws add to shared
 * accumulators) or ellipsoids (solver counters). */
static void contactLoopDet(Scene& S) {
  const wdem_params& P = S.P;
  const long size = (long)S.linView.size();
  std::vector<char> outcome(size, 0);  /* 1: removeAfter, 2: requestRemoval */
  long errIdx = -1;
  std::string errMsg;
#pragma omp parallel for schedule(guided)
  for (long i = 0; i < size; i++) {
    const CPtr& C = S.linView[i];
    if (!C->isReal() && !C->isColliding()) { outcome[i] = 1; continue; }
    bool fresh = (S.step == C->stepCreated);
    if (!C->isReal() && fresh && !freshContactSetup(S, *C)) continue;
    Particle& pA = S.par[C->pA];
    Particle& pB = S.par[C->pB];
    V3 shift2 = S.periodic ? S.cell.intrShiftPos(C->cellDist) : V3();
    if (P.dist00 && !C->isReal() && !fresh && C->minDist00Sq > 0 && sqnorm(pA.pos - (pB.pos + shift2)) > C->minDist00Sq) continue;
    bool keep = true;
    try {
      if (!callGeom(S, *C, pA, pB, shift2)) continue;
      if (!C->phys) C->stepCreated = (int)S.step;
      if (!C->phys || S.updatePhys > WDEM_UPDATE_PHYS_NEVER) {
        const wdem_material& m1 = S.mats[pA.mat];
        const wdem_material& m2 = S.mats[pB.mat];
        if (P.cp2 == WDEM_CP2_FRICT) cp2Frict(S, *C, m1, m2);
        else {
          if (m1.kind != WDEM_MAT_HERTZ || m2.kind != WDEM_MAT_HERTZ)
            throw std::runtime_error("ContactLoop: ##" + std::to_string(pA.id) + "+" + std::to_string(pB.id) + ": no Contact.phys created from materials");
          cp2Hertz(S, *C, m1, m2);
        }
      }
      keep = (P.law == WDEM_LAW_IDEALELPL) ? lawIdealElPl(S, *C) : lawHertzDMT(S, *C);
    } catch (std::exception& e) {
#pragma omp critical
      if (errIdx < 0 || i < errIdx) { errIdx = i; errMsg = e.what(); }
      continue;
    }
    if (!keep) outcome[i] = 2;
  }
  if (errIdx >= 0) { S.err = errMsg; throw std::runtime_error(errMsg); }
  std::vector<CPtr> removeAfter;
  for (long i = 0; i < size; i++) {
    if (outcome[i] == 1) removeAfter.push_back(S.linView[i]);
    else if (outcome[i] == 2) requestRemoval(S, S.linView[i]);
  }
  for (auto& c : removeAfter) removeContact(S, c);
  if (P.applyForces) {
    std::vector<CPtr> real;
    for (auto& c : S.linView) if (c->isReal()) real.push_back(c);
    std::sort(real.begin(), real.end(), [](const CPtr& a, const CPtr& b) {
      long ka = ((long)std::min(a->pA, a->pB) << 32) | std::max(a->pA, a->pB);
      long kb = ((long)std::min(b->pA, b->pB) << 32) | std::max(b->pA, b->pB);
      return ka < kb;
    });
    for (auto& c : real) { applyForceUninodal(S, *c, S.par[c->pA]); applyForceUninodal(S, *c, S.par[c->pB]); }
  }
  if (S.updatePhys == WDEM_UPDATE_PHYS_ONCE) S.updatePhys = WDEM_UPDATE_PHYS_NEVER;
}
#endif

/* ContactLoop::run (ContactLoop.cpp:93-268), aperiodic, no hook, no stress */
static void contactLoopRun(Scene& S) {
  const wdem_params& P = S.P;
  /* removeAllPending when no collider ran: pending is empty after the collider */
  if (!S.pending.empty()) {
    auto pend = S.pending; S.pending.clear();
    for (auto& pc : pend) removeContact(S, pc.first);
  }
  std::vector<CPtr> removeAfter;
  size_t size = S.linView.size();
#ifdef _OPENMP
  if (S.parallel && S.applyOrder == 0) { contactLoopParallel(S); return; }
  if (S.detParallel && S.applyOrder == 1 && !P.trackEnergy && !S.anyEll) { contactLoopDet(S); return; }
#endif
  for (size_t i = 0; i < size; i++) {
    const CPtr C = S.linView[i];
    if (!C->isReal() && !C->isColliding()) { removeAfter.push_back(C); continue; }
    bool fresh = (S.step == C->stepCreated);
    if (!C->isReal() && fresh && !freshContactSetup(S, *C)) continue;
    Particle& pA = S.par[C->pA];
    Particle& pB = S.par[C->pB];
    V3 shift2 = S.periodic ? S.cell.intrShiftPos(C->cellDist) : V3();
    if (P.dist00 && !C->isReal() && !fresh && C->minDist00Sq > 0 && sqnorm(pA.pos - (pB.pos + shift2)) > C->minDist00Sq) continue;
    if (!callGeom(S, *C, pA, pB, shift2)) continue;
    if (!C->phys) C->stepCreated = (int)S.step;
    if (!C->phys || S.updatePhys > WDEM_UPDATE_PHYS_NEVER) {
      const wdem_material& m1 = S.mats[pA.mat];
      const wdem_material& m2 = S.mats[pB.mat];
      if (P.cp2 == WDEM_CP2_FRICT) cp2Frict(S, *C, m1, m2);
      else {
        if (m1.kind != WDEM_MAT_HERTZ || m2.kind != WDEM_MAT_HERTZ) {
          S.err = "ContactLoop: ##" + std::to_string(pA.id) + "+" + std::to_string(pB.id) + ": no Contact.phys created from materials";
          throw std::runtime_error(S.err);
        }
        cp2Hertz(S, *C, m1, m2);
      }
    }
    bool keep = (P.law == WDEM_LAW_IDEALELPL) ? lawIdealElPl(S, *C) : lawHertzDMT(S, *C);
    if (!keep) requestRemoval(S, C);
    if (P.applyForces && C->isReal() && S.applyOrder == 0) {
      applyForceUninodal(S, *C, pA);
      applyForceUninodal(S, *C, pB);
    }
  }
  for (auto& c : removeAfter) removeContact(S, c);
  if (P.applyForces && S.applyOrder == 1) {
    std::vector<CPtr> real;
    for (auto& c : S.linView) if (c->isReal()) real.push_back(c);
    std::sort(real.begin(), real.end(), [](const CPtr& a, const CPtr& b) {
      long ka = ((long)std::min(a->pA, a->pB) << 32) | std::max(a->pA, a->pB);
      long kb = ((long)std::min(b->pA, b->pB) << 32) | std::max(b->pA, b->pB);
      return ka < kb;
    });
    for (auto& c : real) { applyForceUninodal(S, *c, S.par[c->pA]); applyForceUninodal(S, *c, S.par[c->pB]); }
  }
  if (S.updatePhys == WDEM_UPDATE_PHYS_ONCE) S.updatePhys = WDEM_UPDATE_PHYS_NEVER;
}

/* ------------------------------------------------------------------ integrator */
/* Leapfrog::DotQ (Leapfrog.cpp:325-331) */
static Quat dotQ(const V3& w, const Quat& Q) {
  Quat d;
  d.w = (-Q.x * w.x - Q.y * w.y - Q.z * w.z) / 2;
  d.x = (Q.w * w.x - Q.z * w.y + Q.y * w.z) / 2;
  d.y = (Q.z * w.x + Q.w * w.y - Q.x * w.z) / 2;
  d.z = (-Q.y * w.x + Q.x * w.y + Q.w * w.z) / 2;
  return d;
}
/* coefficient-wise q1 + f q2 (Woo's quaternion operator+ and scalar operator*, Math.hpp:139-140) */
static Quat qaxpy(const Quat& q1, double f, const Quat& q2) {
  return Quat(q1.w + q2.w * f, q1.x + q2.x * f, q1.y + q2.y * f, q1.z + q2.z * f);
}
/* Leapfrog::leapfrogAsphericalRotate (Leapfrog.cpp:299-322) */
static void leapfrogAsphericalRotate(Scene& S, Particle& p, const V3& M) {
  const double dt = S.P.dt;
  if (std::isnan(minCoeff(p.angMom))) {
    /* inertia.asDiagonal() * ori.conjugate() * angVel: diag(I) R(ori*) applied to angVel */
    const Mat R = quatToMat(qconj(p.ori));
    Mat DR;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) DR.r[i][j] = p.inertia[i] * R.r[i][j];
    p.angMom = mvec(DR, p.angVel);
  }
  const Mat A = quatToMat(qconj(p.ori));
  const V3 l_n = p.angMom + (dt / 2) * M;
  const V3 l_b_n = mvec(A, l_n);
  const V3 angVel_b_n(l_b_n.x / p.inertia.x, l_b_n.y / p.inertia.y, l_b_n.z / p.inertia.z);
  const Quat dotQ_n = dotQ(angVel_b_n, p.ori);
  const Quat Q_half = qaxpy(p.ori, dt / 2, dotQ_n);
  p.angMom = p.angMom + dt * M;
  const V3 l_b_half = mvec(A, p.angMom);
  const V3 angVel_b_half(l_b_half.x / p.inertia.x, l_b_half.y / p.inertia.y, l_b_half.z / p.inertia.z);
  const Quat dotQ_half = dotQ(angVel_b_half, Q_half);
  p.ori = qaxpy(p.ori, dt, dotQ_half);
  p.angVel = qrot(p.ori, angVel_b_half);
  qnormalize(p.ori);
}
/* Leapfrog::run, aperiodic (Leapfrog.cpp:104-255), ForceResetter folded in via reset=True */
static void leapfrogRun(Scene& S) {
  const wdem_params& P = S.P;
  const double dt = P.dt;
  const double damping = P.damping;
  V3 gravity(P.gravity[0], P.gravity[1], P.gravity[2]);
  bool hasGravity = !isZero(gravity);
  const long np = (long)S.par.size();
  /* GRADV2 matrices (Leapfrog.cpp:119-127) */
  const bool peri = S.periodic;
  Mat ImLL4hInv, IpLL4h, LmL;
  V3 deltaSpinVec;
  if (peri) {
    const Mat& pprevL = S.cell.gradV;
    const Mat& nnextL = S.cell.nextGradV;
    Mat q = mscale(mscale(madd(nnextL, pprevL, 1.0), dt), 1. / 4.);   /* dt*(nnextL+pprevL)/4. */
    ImLL4hInv = minv(madd(Mat::I(), q, -1.0));
    IpLL4h = madd(Mat::I(), q, 1.0);
    LmL = madd(nnextL, pprevL, -1.0);
    deltaSpinVec = -.5 * leviCivita(mscale(madd(pprevL, mtrans(pprevL), -1.0), .5)) +
                   .5 * leviCivita(mscale(madd(nnextL, mtrans(nnextL), -1.0), .5));
  }
  /* reallyTrackEnergy (:132): no energy in step 0 of a periodic scene unless gradV is the identity */
  bool gradVI = true;
  for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) gradVI &= (S.cell.gradV.r[i][k] == (i == k ? 1.0 : 0.0));
  const bool eTrack = P.trackEnergy && (!peri || S.step > 0 || gradVI);
#ifdef _OPENMP
#pragma omp parallel for schedule(guided) if ((S.parallel || S.detParallel) && !eTrack)
#endif
  for (long ip = 0; ip < np; ip++) {
    Particle& p = S.par[ip];
    bool damp = (damping != 0. && !(p.flags & WDEM_DAMPING_SKIP));
    V3& f = p.force;
    V3& t = p.torque;
    if (eTrack) {
      if (damp && !(p.flags & WDEM_ENERGY_SKIP)) {
        /* doDampingDissipation (:53-64) */
        V3 av(std::abs(p.vel.x), std::abs(p.vel.y), std::abs(p.vel.z));
        V3 af(std::abs(f.x), std::abs(f.y), std::abs(f.z));
        V3 aw(std::abs(p.angVel.x), std::abs(p.angVel.y), std::abs(p.angVel.z));
        V3 at(std::abs(t.x), std::abs(t.y), std::abs(t.z));
        S.E.v[WDEM_E_NONVISCDAMP] += dot(av, af) * damping * dt + dot(aw, at) * damping * dt;
      }
      if (hasGravity && !(p.flags & WDEM_GRAVITY_SKIP)) {
        /* doGravityWork (:67-74) */
        double gr = 0;
        if (p.isBlockedNone()) gr = -dot(gravity, p.vel) * p.mass * dt;
        else for (int ax = 0; ax < 3; ax++) if (!p.isBlockedAxisDOF(ax, false)) gr -= gravity[ax] * p.vel[ax] * p.mass * dt;
        S.E.v[WDEM_E_GRAV] += gr;
      }
    }
    V3 pprevFluctVel, pprevFluctAngVel;
    bool useAspherical = p.isAspherical() && !p.isBlockedAllRot();
    V3 linAccel, angAccel;
    if (!p.isBlockedAll()) {
      /* computeAccel (:37-42) */
      if (p.isBlockedNone()) linAccel = f / p.mass;
      else for (int i = 0; i < 3; i++) if (!p.isBlockedAxisDOF(i, false)) linAccel[i] += f[i] / p.mass;
      if (peri) {
        /* Cell::pprevFluctVel / pprevFluctAngVel, HOMO_GRADV2 (Cell.cpp:36-57) */
        pprevFluctVel = p.vel - mvec(S.cell.gradV, p.pos - dt / 2 * p.vel);
        pprevFluctAngVel = p.angVel - S.cell.spinVec;
      } else { pprevFluctVel = p.vel; pprevFluctAngVel = p.angVel; }
      /* nonviscDamp2nd (:33-35) */
      if (damp) for (int i = 0; i < 3; i++) linAccel[i] *= 1 - damping * Sign(f[i] * (pprevFluctVel[i] + 0.5 * dt * linAccel[i]));
      if (peri) p.vel = mvec(ImLL4hInv, mvec(LmL, p.pos) + mvec(IpLL4h, p.vel) + linAccel * dt);
      else p.vel = p.vel + dt * linAccel;
      if (!isZero(p.inertia)) {
        if (!useAspherical) {
          if (p.isBlockedNone()) angAccel = V3(t.x / p.inertia.x, t.y / p.inertia.y, t.z / p.inertia.z);
          else for (int i = 0; i < 3; i++) if (!p.isBlockedAxisDOF(i, true)) angAccel[i] += t[i] / p.inertia[i];
          if (damp) for (int i = 0; i < 3; i++) angAccel[i] *= 1 - damping * Sign(t[i] * (pprevFluctAngVel[i] + 0.5 * dt * angAccel[i]));
          p.angVel = p.angVel + dt * angAccel;
          if (peri) p.angVel = p.angVel - deltaSpinVec;
        } else {
          /* aspherical: blocked rotational DOFs zero the torque, then nonviscDamp1st on the torque (:176-179) */
          for (int i = 0; i < 3; i++) if (p.isBlockedAxisDOF(i, true)) t[i] = 0;
          if (damp) for (int i = 0; i < 3; i++) t[i] *= 1 - damping * Sign(t[i] * pprevFluctAngVel[i]);
        }
      }
    } else if (peri) {
      /* fixed particle with GRADV2: velocity correction without acceleration (Leapfrog.cpp:207-211) */
      p.vel = mvec(ImLL4hInv, mvec(LmL, p.pos) + mvec(IpLL4h, p.vel));
    }
    if (eTrack && !(p.flags & WDEM_ENERGY_SKIP)) {
      /* doKineticEnergy (:76-98), spherical */
      V3 cfv = pprevFluctVel + .5 * dt * linAccel, cfa = pprevFluctAngVel + .5 * dt * angAccel;
      double Etrans = .5 * p.mass * sqnorm(cfv);
      double Erot;
      if (p.isAspherical()) {
        /* .5 w^T (T^T diag(I) T) w with T the rotation matrix of ori (:86-89) */
        const Mat T = quatToMat(p.ori);
        Mat mI;
        mI.r[0][0] = p.inertia.x; mI.r[1][1] = p.inertia.y; mI.r[2][2] = p.inertia.z;
        const Mat M = mmul(mmul(mtrans(T), mI), T);
        Erot = .5 * dot(cfa, mvec(M, cfa));
      } else Erot = 0.5 * dot(cfa, V3(p.inertia.x * cfa.x, p.inertia.y * cfa.y, p.inertia.z * cfa.z));
      if (std::isnan(Erot) || std::isinf(absmax(p.inertia))) Erot = 0;
      S.E.v[WDEM_E_KINETIC] += Etrans + Erot;
    }
    /* leapfrogTranslate (:275-278) */
    p.pos = p.pos + p.vel * dt;
    if (useAspherical) {
      if (isZero(p.inertia)) throw std::runtime_error("Leapfrog: zero inertia of a node using the aspherical integrator");
      leapfrogAsphericalRotate(S, p, t);
    } else {
    /* leapfrogSphericalRotate (:280-297) */
    V3 axis = p.angVel;
    if (!isZero(axis)) {
      double angle = norm(axis);
      axis = axis / angle;
      double ha = 0.5 * (angle * dt);
      double sh = std::sin(ha);
      Quat q(std::cos(ha), sh * axis.x, sh * axis.y, sh * axis.z);
      p.ori = qmul(q, p.ori);
    }
    qnormalize(p.ori);
    }
    if (P.reset) {
      p.force = (hasGravity && !(p.flags & WDEM_GRAVITY_SKIP)) ? p.mass * gravity : V3();
      p.torque = V3();
    }
  }
}

/* DemFuncs::pWaveDt (Funcs.cpp:151-175) */
static double pWaveDt(const Scene& S) {
  double dt = Inf;
  for (const Particle& p : S.par) {
    double radius;
    if (p.shape == WDEM_SHAPE_SPHERE) radius = p.radius;
    else if (p.shape == WDEM_SHAPE_ELLIPSOID) radius = minCoeff(p.semiAxes);
    else if (p.shape == WDEM_SHAPE_CAPSULE) radius = p.radius;
    else continue;
    const wdem_material& m = S.mats[p.mat];
    dt = std::min(dt, radius / (1. * std::sqrt(m.young / m.density)));
  }
  return dt;
}

/* Scene::doOneStep (Scene.cpp:366-467) with engines [Leapfrog, InsertionSortCollider, ContactLoop] */
/* DynDt::nodalCritDtSq (DynDt.cpp:46-63) with nodalStiffAdd (DynDt.cpp:16-38); the contact normal is
 * the contact node's orientation applied to the x axis; Eigen's n.array().pow(2) is taken as n*n */
static double nodalCritDtSq(const Scene& S, int i) {
  const Particle& q = S.par[i];
  if (q.isBlockedAll()) return Inf;
  V3 ktrans(0, 0, 0), krot(0, 0, 0);
  for (const auto& kv : q.contacts) {
    const Contact& C = *kv.second;
    if (!C.isReal()) continue;
    const int ix = (C.pA == i) ? 0 : 1;
    const V3 n = qrot(C.gori, V3(1, 0, 0));
    const V3 n2(n.x * n.x, n.y * n.y, n.z * n.z);
    const double knt = C.kn - C.kt;
    ktrans = V3(ktrans.x + (n2.x * knt + C.kt), ktrans.y + (n2.y * knt + C.kt), ktrans.z + (n2.z * knt + C.kt));
    const double sc = (C.lens[ix] * C.lens[ix]) * C.kt;  /* pow2(lens[ix]) * kt */
    krot = V3(krot.x + sc * (n2.y + n2.z), krot.y + sc * (n2.z + n2.x), krot.z + sc * (n2.x + n2.y));
  }
  double ret = Inf;
  const double kt[3] = {ktrans.x, ktrans.y, ktrans.z}, kr[3] = {krot.x, krot.y, krot.z};
  const double in[3] = {q.inertia.x, q.inertia.y, q.inertia.z};
  for (int k = 0; k < 3; k++) if (kt[k] != 0 && q.mass > 0. && !q.isBlockedAxisDOF(k, false)) ret = std::min(ret, q.mass / std::abs(kt[k]));
  for (int k = 0; k < 3; k++) if (kr[k] != 0 && in[k] > 0. && !q.isBlockedAxisDOF(k, true)) ret = std::min(ret, in[k] / std::abs(kr[k]));
  return 2 * ret;
}

/* DynDt::run (DynDt.cpp:86-113), when PeriodicEngine::isActivated (Engine.cpp:170-196: stepPeriod with
 * stepModulo, initRun) says so; the new dt takes effect after the step (Scene.cpp:432) */
static void dynDtRun(Scene& S) {
  const long per = S.P.dynDtPeriod;
  if (per <= 0) return;
  const long s = S.step;
  if (S.dynStepLast < 0) S.dynStepLast = s;
  if (!((s - S.dynStepLast >= per) || (s % per == 0))) return;
  S.dynStepPrev = S.dynStepLast;
  S.dynStepLast = s;
  double ret = Inf;  /* DynDt::critDt_stiffness */
  for (size_t i = 0; i < S.par.size(); i++) ret = std::min(ret, nodalCritDtSq(S, (int)i));
  const double crDt = std::sqrt(ret);
  S.dynDtCrit = crDt;
  if (std::isinf(crDt)) return;
  const long nSteps = S.step - S.dynStepPrev;
  const double maxNewDt = S.P.dt * pown(1. + S.P.dynDtMaxRelInc, (unsigned)nSteps);
  const double nextDt = std::min(crDt * S.P.dtSafety, maxNewDt);
  if (nextDt != S.P.dt) S.nextDt = nextDt;
}

static void doOneStep(Scene& S) {
  if (S.periodic) S.cell.integrateAndUpdate(S.P.dt);
  if (S.P.trackEnergy) S.E.resetResettables();
  leapfrogRun(S);
  colliderRun(S);
  contactLoopRun(S);
  dynDtRun(S);
  if (S.periodic) S.cell.setNextGradV();
  S.step++;
  S.time += S.P.dt;
  S.P.step = S.step;
  if (!std::isnan(S.nextDt)) { S.P.dt = S.nextDt; S.nextDt = NaN; }
}

}  // namespace orc

/* ====================================================================== C ABI for tests */
using namespace orc;

/* ------------------------------------------------------------------ scene generator
 * The seeded random sequential addition that builds the benchmark packings (the engine library's
 * wdem_make_cloud / wdem_make_cloud_radii), restated so that the CPU arm of the benchmark builds the same
 * packing without loading the engine library; tests/test_oracle_pack.py checks that both give identical
 * arrays.  Radii (given, or drawn uniformly in [rMin, rMax] from a SplitMix64 stream) are placed largest
 * first, each at the first of maxAttempts uniformly random centres that overlaps no placed sphere
 * (nearest periodic image in a periodic box); candidates are found in a grid of cells at least 2 rMax wide. */
static uint64_t packNext(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double packUniform(uint64_t& s) { return (double)(packNext(s) >> 11) * (1.0 / 9007199254740992.0); }

/* wdem_make_cloud: uniform radii, aperiodic box, cells of exactly 2 rMax from lo */
static int64_t packCloud(const double* lo, const double* hi, double rMin, double rMax, int64_t n, uint64_t seed,
                         int32_t maxAttempts, double* centers, double* radii) {
  uint64_t rs = seed;
  std::vector<double> r(n);
  for (int64_t i = 0; i < n; i++) r[i] = (rMax > rMin) ? rMin + (rMax - rMin) * packUniform(rs) : rMin;
  std::sort(r.begin(), r.end(), [](double a, double b) { return a > b; });
  const double cell = 2 * rMax;
  int nc[3];
  for (int k = 0; k < 3; k++) nc[k] = std::max(1, (int)std::ceil((hi[k] - lo[k]) / cell));
  std::vector<int64_t> head((size_t)nc[0] * nc[1] * nc[2], -1), next;
  std::vector<double> c, rr;
  auto cellIdx = [&](const double* x) {
    int64_t idx[3];
    for (int k = 0; k < 3; k++) idx[k] = std::min(std::max((int)std::floor((x[k] - lo[k]) / cell), 0), nc[k] - 1);
    return idx[0] + nc[0] * (idx[1] + (int64_t)nc[1] * idx[2]);
  };
  for (int64_t i = 0; i < n; i++) {
    const double ri = r[i];
    double x[3];
    bool ok = false;
    for (int a = 0; a < maxAttempts && !ok; a++) {
      for (int k = 0; k < 3; k++) x[k] = lo[k] + ri + (hi[k] - lo[k] - 2 * ri) * packUniform(rs);
      int ci[3];
      for (int k = 0; k < 3; k++) ci[k] = std::min(std::max((int)std::floor((x[k] - lo[k]) / cell), 0), nc[k] - 1);
      ok = true;
      for (int dz = -1; dz <= 1 && ok; dz++)
        for (int dy = -1; dy <= 1 && ok; dy++)
          for (int dx = -1; dx <= 1 && ok; dx++) {
            const int cx = ci[0] + dx, cy = ci[1] + dy, cz = ci[2] + dz;
            if (cx < 0 || cy < 0 || cz < 0 || cx >= nc[0] || cy >= nc[1] || cz >= nc[2]) continue;
            for (int64_t j = head[cx + nc[0] * (cy + (int64_t)nc[1] * cz)]; j >= 0; j = next[j]) {
              const double d0 = x[0] - c[3 * j], d1 = x[1] - c[3 * j + 1], d2 = x[2] - c[3 * j + 2];
              const double sr = ri + rr[j];
              if (d0 * d0 + d1 * d1 + d2 * d2 < sr * sr) { ok = false; break; }
            }
          }
    }
    if (!ok) continue;
    const int64_t ci = cellIdx(x);
    next.push_back(head[ci]);
    head[ci] = (int64_t)rr.size();
    c.insert(c.end(), x, x + 3);
    rr.push_back(ri);
  }
  std::copy(c.begin(), c.end(), centers);
  std::copy(rr.begin(), rr.end(), radii);
  return (int64_t)rr.size();
}

/* wdem_make_cloud_radii: given radii, optionally periodic; cells L/floor(L / 2 rMax) wide */
static int64_t packCloudRadii(const double* lo, const double* hi, int periodic, int64_t n, const double* rIn,
                              uint64_t seed, int32_t maxAttempts, double* centers, double* radii) {
  std::vector<double> r(rIn, rIn + n);
  for (double v : r) if (!(v > 0)) return WDEM_ERR_ARG;
  std::sort(r.begin(), r.end(), [](double a, double b) { return a > b; });
  uint64_t rs = seed;
  const double cell = 2 * (n > 0 ? r[0] : 1.0);
  double L[3];
  int nc[3];
  for (int k = 0; k < 3; k++) { L[k] = hi[k] - lo[k]; nc[k] = std::max(1, (int)std::floor(L[k] / cell)); }
  std::vector<int64_t> head((size_t)nc[0] * nc[1] * nc[2], -1), next;
  std::vector<double> c, rr;
  auto cellOf = [&](const double* x, int* ci) {
    for (int k = 0; k < 3; k++) ci[k] = std::min(std::max((int)std::floor((x[k] - lo[k]) / L[k] * nc[k]), 0), nc[k] - 1);
  };
  for (int64_t i = 0; i < n; i++) {
    const double ri = r[i];
    double x[3];
    bool ok = false;
    for (int a = 0; a < maxAttempts && !ok; a++) {
      for (int k = 0; k < 3; k++)
        x[k] = periodic ? lo[k] + L[k] * packUniform(rs) : lo[k] + ri + (L[k] - 2 * ri) * packUniform(rs);
      int ci[3];
      cellOf(x, ci);
      ok = true;
      int span[3];
      for (int k = 0; k < 3; k++) span[k] = nc[k] >= 2 ? 1 : 0;
      for (int dz = -span[2]; dz <= span[2] && ok; dz++)
        for (int dy = -span[1]; dy <= span[1] && ok; dy++)
          for (int dx = -span[0]; dx <= span[0] && ok; dx++) {
            if (periodic && ((nc[0] == 2 && dx == 1) || (nc[1] == 2 && dy == 1) || (nc[2] == 2 && dz == 1))) continue;
            int cx = ci[0] + dx, cy = ci[1] + dy, cz = ci[2] + dz;
            if (periodic) { cx = (cx + nc[0]) % nc[0]; cy = (cy + nc[1]) % nc[1]; cz = (cz + nc[2]) % nc[2]; }
            else if (cx < 0 || cy < 0 || cz < 0 || cx >= nc[0] || cy >= nc[1] || cz >= nc[2]) continue;
            for (int64_t j = head[cx + nc[0] * (cy + (int64_t)nc[1] * cz)]; j >= 0; j = next[j]) {
              double d[3];
              for (int k = 0; k < 3; k++) {
                d[k] = x[k] - c[3 * j + k];
                if (periodic) d[k] -= L[k] * std::nearbyint(d[k] / L[k]);
              }
              const double sr = ri + rr[j];
              if (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] < sr * sr) { ok = false; break; }
            }
          }
    }
    if (!ok) continue;
    int ci[3];
    cellOf(x, ci);
    const int64_t cidx = ci[0] + nc[0] * (ci[1] + (int64_t)nc[1] * ci[2]);
    next.push_back(head[cidx]);
    head[cidx] = (int64_t)rr.size();
    c.insert(c.end(), x, x + 3);
    rr.push_back(ri);
  }
  std::copy(c.begin(), c.end(), centers);
  std::copy(rr.begin(), rr.end(), radii);
  return (int64_t)rr.size();
}

struct orc_handle { Scene S; };

extern "C" {

orc_handle* orc_create(void) { return new orc_handle(); }
void orc_destroy(orc_handle* h) { delete h; }
const char* orc_last_error(orc_handle* h) { return h->S.err.c_str(); }

int orc_set_params(orc_handle* h, const wdem_params* p) {
  Scene& S = h->S;
  S.P = *p;
  S.mats.assign(p->materials, p->materials + p->nMaterials);
  S.P.materials = nullptr;
  S.step = p->step;
  S.updatePhys = p->updatePhys;
  if (S.nFullRuns == 0 && S.BB[0].empty()) S.verletDist = p->verletDist;
  return 0;
}

/* OpenMP loops (only in the liborc_omp.so build); forces are then added in thread order. */
int orc_set_parallel(orc_handle* h, int on) {
#ifdef _OPENMP
  Scene& S = h->S;
  for (auto& l : S.locks) omp_destroy_lock(&l);
  S.locks.assign(S.par.size(), omp_lock_t());
  for (auto& l : S.locks) omp_init_lock(&l);
  S.parallel = on;
  if (on) S.applyOrder = 0;
  return 0;
#else
  (void)h; (void)on;
  return -1;
#endif
}

/* Deterministic OpenMP loops (liborc_omp.so only): the serial oracle's results bit for bit, canonical mode. */
int orc_set_det_parallel(orc_handle* h, int on) {
#ifdef _OPENMP
  h->S.detParallel = on;
  return 0;
#else
  (void)h; (void)on;
  return -1;
#endif
}

int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int orc_set_mode(orc_handle* h, int canonicalOrient, int applyOrder, int sortAxis) {
  h->S.canonicalOrient = canonicalOrient; h->S.applyOrder = applyOrder; h->S.sortAxis = sortAxis;
  return 0;
}

int orc_upload_particles(orc_handle* h, const wdem_particles* p) {
  Scene& S = h->S;
  S.par.assign(p->n, Particle());
  for (int i = 0; i < p->n; i++) {
    Particle& q = S.par[i];
    q.id = i;
    q.shape = p->shape[i];
    q.radius = p->radius[i];
    q.axis = p->wallAxis ? p->wallAxis[i] : 0;
    q.sense = p->wallSense ? p->wallSense[i] : 0;
    q.mat = p->material[i];
    q.mask = p->mask[i];
    q.flags = p->flags[i];
    q.mass = p->mass[i];
    q.inertia = V3(p->inertia[3 * i], p->inertia[3 * i + 1], p->inertia[3 * i + 2]);
    q.pos = V3(p->pos[3 * i], p->pos[3 * i + 1], p->pos[3 * i + 2]);
    q.ori = Quat(p->ori[4 * i], p->ori[4 * i + 1], p->ori[4 * i + 2], p->ori[4 * i + 3]);
    q.vel = V3(p->vel[3 * i], p->vel[3 * i + 1], p->vel[3 * i + 2]);
    q.angVel = V3(p->angVel[3 * i], p->angVel[3 * i + 1], p->angVel[3 * i + 2]);
    q.force = V3(p->force[3 * i], p->force[3 * i + 1], p->force[3 * i + 2]);
    q.torque = V3(p->torque[3 * i], p->torque[3 * i + 1], p->torque[3 * i + 2]);
    if (p->semiAxes) q.semiAxes = V3(p->semiAxes[3 * i], p->semiAxes[3 * i + 1], p->semiAxes[3 * i + 2]);
    if (p->angMom) q.angMom = V3(p->angMom[3 * i], p->angMom[3 * i + 1], p->angMom[3 * i + 2]);
    if (q.shape == WDEM_SHAPE_CAPSULE) {
      if (!p->shaft) { S.err = "capsules need wdem_particles.shaft"; return WDEM_ERR_ARG; }
      q.shaft = p->shaft[i];
      /* Capsule::selfTest (Capsule.cpp:19-23) */
      if (!(q.radius > 0.) || !(q.shaft >= 0.)) { S.err = "Capsule: radius must be positive and shaft non-negative"; return WDEM_ERR_ARG; }
    }
    if (q.shape == WDEM_SHAPE_FACET) {
      if (!p->facetVerts) { S.err = "facets need wdem_particles.facetVerts"; return WDEM_ERR_ARG; }
      q.fv1 = V3(p->facetVerts[9 * i + 3], p->facetVerts[9 * i + 4], p->facetVerts[9 * i + 5]);
      q.fv2 = V3(p->facetVerts[9 * i + 6], p->facetVerts[9 * i + 7], p->facetVerts[9 * i + 8]);
    }
    if (q.shape == WDEM_SHAPE_ELLIPSOID && !(minCoeff(q.semiAxes) > 0)) {
      S.err = "Ellipsoid #" + std::to_string(i) + ": all semi-axes must be positive";
      return WDEM_ERR_ARG;
    }
  }
  S.linView.clear(); S.pending.clear();
  for (int i = 0; i < 3; i++) S.BB[i].clear();
  S.dirty = true;
  S.verletDist = S.P.verletDist;
  S.anyEll = false;
  for (const Particle& q : S.par) if (q.shape == WDEM_SHAPE_ELLIPSOID || q.shape == WDEM_SHAPE_CAPSULE) S.anyEll = true;
  return 0;
}

int orc_upload_contacts(orc_handle* h, const wdem_contacts* c) {
  Scene& S = h->S;
  for (Particle& p : S.par) p.contacts.clear();
  S.linView.clear(); S.pending.clear();
  for (long i = 0; i < c->n; i++) {
    CPtr C = std::make_shared<Contact>();
    C->pA = c->idA[i]; C->pB = c->idB[i];
    if (c->cellDist) for (int k = 0; k < 3; k++) C->cellDist[k] = c->cellDist[3 * i + k];
    C->stepCreated = c->stepCreated[i];
    C->minDist00Sq = c->minDist00Sq ? c->minDist00Sq[i] : -1;
    if (c->real[i]) {
      C->geom = C->phys = true;
      for (int k = 0; k < 3; k++) C->trsf.c[k] = V3(c->trsf[9 * i + 3 * k], c->trsf[9 * i + 3 * k + 1], c->trsf[9 * i + 3 * k + 2]);
      C->contPt = V3(c->contPt[3 * i], c->contPt[3 * i + 1], c->contPt[3 * i + 2]);
      C->gori = quatFromMatrix(C->trsf);
      C->force = V3(c->force[3 * i], c->force[3 * i + 1], c->force[3 * i + 2]);
      C->torque = V3(c->torque[3 * i], c->torque[3 * i + 1], c->torque[3 * i + 2]);
      C->kn = c->kn[i]; C->kt = c->kt[i]; C->tanPhi = c->tanPhi[i];
      /* lens/contA for iniLensTouch=true; Hertz constants recomputed from the materials */
      const Particle& a = S.par[C->pA];
      const Particle& b = S.par[C->pB];
      /* the radii handleSpheresLikeContact got: -r for walls, max(halfThick, r) for facets */
      double r1 = a.shape == WDEM_SHAPE_WALL ? -b.radius : a.shape == WDEM_SHAPE_FACET ? std::max(a.radius, b.radius) : a.radius;
      double r2 = b.radius;
      C->lens[0] = std::abs(r1); C->lens[1] = std::abs(r2);
      C->contA = M_PI * pow2((r1 > 0 && r2 > 0) ? std::min(r1, r2) : (r1 > 0 ? r1 : r2));
      if (S.P.cp2 == WDEM_CP2_HERTZ) {
        double kn = C->kn, kt = C->kt, tp = C->tanPhi;
        cp2Hertz(S, *C, S.mats[a.mat], S.mats[b.mat]);
        C->kn = kn; C->kt = kt; C->tanPhi = tp;
      }
    }
    addMaybe_fast(S, C);
  }
  return 0;
}

int orc_step(orc_handle* h, int n) {
  try {
    for (int i = 0; i < n; i++) doOneStep(h->S);
  } catch (std::exception& e) {
    h->S.err = e.what();
    return WDEM_ERR_NAN;
  }
  return 0;
}

/* Time nSteps steps on the host, returning wall seconds (CPU baseline leg). */
double orc_step_timed(orc_handle* h, int n) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = orc_step(h, n);
  auto t1 = std::chrono::steady_clock::now();
  if (rc) return -1;
  return std::chrono::duration<double>(t1 - t0).count();
}

int orc_download_particles(orc_handle* h, wdem_particles* p) {
  Scene& S = h->S;
  for (int i = 0; i < p->n && i < (int)S.par.size(); i++) {
    const Particle& q = S.par[i];
    if (p->pos) { p->pos[3 * i] = q.pos.x; p->pos[3 * i + 1] = q.pos.y; p->pos[3 * i + 2] = q.pos.z; }
    if (p->ori) { p->ori[4 * i] = q.ori.w; p->ori[4 * i + 1] = q.ori.x; p->ori[4 * i + 2] = q.ori.y; p->ori[4 * i + 3] = q.ori.z; }
    if (p->vel) { p->vel[3 * i] = q.vel.x; p->vel[3 * i + 1] = q.vel.y; p->vel[3 * i + 2] = q.vel.z; }
    if (p->angVel) { p->angVel[3 * i] = q.angVel.x; p->angVel[3 * i + 1] = q.angVel.y; p->angVel[3 * i + 2] = q.angVel.z; }
    if (p->force) { p->force[3 * i] = q.force.x; p->force[3 * i + 1] = q.force.y; p->force[3 * i + 2] = q.force.z; }
    if (p->torque) { p->torque[3 * i] = q.torque.x; p->torque[3 * i + 1] = q.torque.y; p->torque[3 * i + 2] = q.torque.z; }
    if (p->angMom) { p->angMom[3 * i] = q.angMom.x; p->angMom[3 * i + 1] = q.angMom.y; p->angMom[3 * i + 2] = q.angMom.z; }
  }
  return 0;
}

long orc_contact_count(orc_handle* h) { return (long)h->S.linView.size(); }

/* Scene.dt for the next step and DynDt's last critical step */
double orc_get_dt(orc_handle* h) { return h->S.P.dt; }
double orc_dyndt_crit(orc_handle* h) { return h->S.dynDtCrit; }

/* contacts sorted by (min id, max id) */
int orc_download_contacts(orc_handle* h, wdem_contacts* c) {
  Scene& S = h->S;
  std::vector<CPtr> v = S.linView;
  std::sort(v.begin(), v.end(), [](const CPtr& a, const CPtr& b) {
    long ka = ((long)std::min(a->pA, a->pB) << 32) | std::max(a->pA, a->pB);
    long kb = ((long)std::min(b->pA, b->pB) << 32) | std::max(b->pA, b->pB);
    return ka < kb;
  });
  for (long i = 0; i < (long)v.size() && i < c->n; i++) {
    const Contact& C = *v[i];
    if (c->idA) c->idA[i] = C.pA;
    if (c->idB) c->idB[i] = C.pB;
    if (c->cellDist) for (int k = 0; k < 3; k++) c->cellDist[3 * i + k] = C.cellDist[k];
    if (c->real) c->real[i] = C.isReal();
    if (c->stepCreated) c->stepCreated[i] = C.stepCreated;
    if (c->minDist00Sq) c->minDist00Sq[i] = C.minDist00Sq;
    if (c->trsf) for (int k = 0; k < 3; k++) { c->trsf[9 * i + 3 * k] = C.trsf.c[k].x; c->trsf[9 * i + 3 * k + 1] = C.trsf.c[k].y; c->trsf[9 * i + 3 * k + 2] = C.trsf.c[k].z; }
    if (c->contPt) { c->contPt[3 * i] = C.contPt.x; c->contPt[3 * i + 1] = C.contPt.y; c->contPt[3 * i + 2] = C.contPt.z; }
    if (c->geomOri) { c->geomOri[4 * i] = C.gori.w; c->geomOri[4 * i + 1] = C.gori.x; c->geomOri[4 * i + 2] = C.gori.y; c->geomOri[4 * i + 3] = C.gori.z; }
    if (c->geomVel) { c->geomVel[3 * i] = C.gvel.x; c->geomVel[3 * i + 1] = C.gvel.y; c->geomVel[3 * i + 2] = C.gvel.z; }
    if (c->geomAngVel) { c->geomAngVel[3 * i] = C.gangVel.x; c->geomAngVel[3 * i + 1] = C.gangVel.y; c->geomAngVel[3 * i + 2] = C.gangVel.z; }
    if (c->uN) c->uN[i] = C.uN;
    if (c->force) { c->force[3 * i] = C.force.x; c->force[3 * i + 1] = C.force.y; c->force[3 * i + 2] = C.force.z; }
    if (c->torque) { c->torque[3 * i] = C.torque.x; c->torque[3 * i + 1] = C.torque.y; c->torque[3 * i + 2] = C.torque.z; }
    if (c->kn) c->kn[i] = C.kn;
    if (c->kt) c->kt[i] = C.kt;
    if (c->tanPhi) c->tanPhi[i] = C.tanPhi;
  }
  return 0;
}

double orc_crit_dt(orc_handle* h) { return pWaveDt(h->S); }

int orc_get_energy(orc_handle* h, double* e, int n) {
  for (int i = 0; i < n && i < WDEM_E_COUNT; i++) e[i] = h->S.E.v[i];
  return 0;
}
int orc_reset_energy(orc_handle* h) { for (int i = 0; i < WDEM_E_COUNT; i++) h->S.E.v[i] = 0; return 0; }

long orc_nfullruns(orc_handle* h) { return h->S.nFullRuns; }
int64_t orc_make_cloud(const double* lo, const double* hi, double rMin, double rMax, int64_t n, uint64_t seed,
                       int32_t maxAttempts, double* centers, double* radii) {
  if (!lo || !hi || !centers || !radii || n < 0 || rMin <= 0 || rMax < rMin) return WDEM_ERR_ARG;
  return packCloud(lo, hi, rMin, rMax, n, seed, maxAttempts, centers, radii);
}
int64_t orc_make_cloud_radii(const double* lo, const double* hi, int32_t periodic, int64_t n, const double* rIn,
                             uint64_t seed, int32_t maxAttempts, double* centers, double* radii) {
  if (!lo || !hi || !rIn || !centers || !radii || n < 0) return WDEM_ERR_ARG;
  return packCloudRadii(lo, hi, periodic, n, rIn, seed, maxAttempts, centers, radii);
}

int orc_sort_passes(orc_handle* h) { return (int)h->S.sortPasses; }

/* ellipsoid functor statistics: solves and contact-function evaluations so far */
int orc_ell_stats(orc_handle* h, long* solves, long* evals) { *solves = h->S.ellSolves; *evals = h->S.ellEvals; return 0; }
double orc_verlet_dist(orc_handle* h) { return h->S.verletDist; }
long orc_step_count(orc_handle* h) { return h->S.step; }
int orc_set_update_phys(orc_handle* h, int up) { h->S.updatePhys = up; return 0; }
int orc_set_young(orc_handle* h, int mat, double young) { h->S.mats[mat].young = young; return 0; }

/* Periodic cell: row-major hSize, trsf, gradV, nextGradV (4 x 9 doubles); homoDeform GRADV2.
 * Sets Cell like Cell.setHSize + nextGradV assignment (Cell.hpp:108, Cell.cpp:19-21). */
int orc_set_cell(orc_handle* h, int periodic, const double* m) {
  Scene& S = h->S;
  S.periodic = periodic != 0;
  if (!S.periodic) return 0;
  Mat mats[4];
  for (int q = 0; q < 4; q++) for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) mats[q].r[i][k] = m[9 * q + 3 * i + k];
  S.cell.hSize = mats[0]; S.cell.pprevHsize = mats[0]; S.cell.trsf = mats[1];
  S.cell.gradV = mats[2]; S.cell.nextGradV = mats[3];
  S.cell.W = mscale(madd(S.cell.gradV, mtrans(S.cell.gradV), -1.0), .5);
  S.cell.spinVec = .5 * leviCivita(S.cell.W);
  S.cell.integrateAndUpdate(0);
  return 0;
}
int orc_get_cell(orc_handle* h, double* m) {
  const Cell& c = h->S.cell;
  const Mat* mats[5] = {&c.hSize, &c.trsf, &c.gradV, &c.nextGradV, &c.pprevHsize};
  for (int q = 0; q < 5; q++) for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) m[9 * q + 3 * i + k] = mats[q]->r[i][k];
  return 0;
}
/* ContactLoop stress (ContactLoop.cpp:218-229, 243-244): sum over real contacts of F (global, on pA)
 * times the branch dPos = pB - pA (+ cell shift), divided by the cell volume; row-major 3x3. */
int orc_stress(orc_handle* h, double* out) {
  Scene& S = h->S;
  double st[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (auto& C : S.linView) {
    if (!C->isReal()) continue;
    V3 branch = S.par[C->pB].pos - S.par[C->pA].pos;
    if (S.periodic) branch = branch + S.cell.intrShiftPos(C->cellDist);
    V3 F = qrot(C->gori, C->force);
    for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) st[i][k] = st[i][k] + F[i] * branch[k];
  }
  double vol = S.periodic ? mdet(S.cell.hSize) : 1.0;
  for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) out[3 * i + k] = st[i][k] / vol;
  return 0;
}

/* InsertionSortCollider initial sort + sweep (InsertionSortCollider.cpp:536-605) over given boxes,
 * with spatialOverlap and mayCollide; writes pairs (min id, max id) sorted. */
long orc_collide_boxes(int n, const double* mins, const double* maxs, const uint32_t* mask, uint32_t loneMask,
                       int sortAxis, int32_t* pairs, long maxPairs) {
  Scene S;
  S.P.loneMask = loneMask;
  S.par.assign(n, Particle());
  for (int i = 0; i < n; i++) {
    Particle& p = S.par[i];
    p.id = i; p.mask = mask[i];
    p.bound.has = true;
    p.bound.min = V3(mins[3 * i], mins[3 * i + 1], mins[3 * i + 2]);
    p.bound.max = V3(maxs[3 * i], maxs[3 * i + 1], maxs[3 * i + 2]);
  }
  S.minima.assign(3 * n, 0); S.maxima.assign(3 * n, 0);
  for (int i = 0; i < n; i++) for (int k = 0; k < 3; k++) { S.minima[3 * i + k] = mins[3 * i + k]; S.maxima[3 * i + k] = maxs[3 * i + k]; }
  for (int j = 0; j < 3; j++) {
    for (int id = 0; id < n; id++) {
      Bounds a(mins[3 * id + j], id, true); a.hasBB = true;
      Bounds b(maxs[3 * id + j], id, false); b.hasBB = true;
      S.BB[j].push_back(a); S.BB[j].push_back(b);
    }
    std::sort(S.BB[j].begin(), S.BB[j].end());
  }
  std::vector<Bounds>& V = S.BB[sortAxis];
  long n2 = 2L * n;
  for (long i = 0; i < n2; i++) {
    if (!(V[i].isMin && V[i].hasBB)) continue;
    int iid = V[i].id;
    for (long j = i + 1; j < n2 && V[j].id != iid; j++) {
      if (!V[j].isMin) continue;
      handleBoundInversion(S, iid, V[j].id, false);
    }
  }
  for (auto& C : S.makeContacts) addMaybe_fast(S, C);
  std::vector<long> keys;
  for (auto& c : S.linView) keys.push_back(((long)std::min(c->pA, c->pB) << 32) | std::max(c->pA, c->pB));
  std::sort(keys.begin(), keys.end());
  long cnt = (long)keys.size();
  for (long i = 0; i < cnt && i < maxPairs; i++) { pairs[2 * i] = (int32_t)(keys[i] >> 32); pairs[2 * i + 1] = (int32_t)(keys[i] & 0xffffffffL); }
  return cnt;
}

/* Incremental collider check: run the insertion-sort collider over a sequence of box sets
 * (nFrames x n boxes), as InsertionSortCollider does between steps (:524-531), and return the
 * pair count after the last frame plus the sorted pairs.  All pairs are potential (non-real). */
long orc_collide_frames(int n, int nFrames, const double* mins, const double* maxs, const uint32_t* mask,
                        uint32_t loneMask, int32_t* pairs, long maxPairs) {
  Scene S;
  S.P.loneMask = loneMask;
  S.par.assign(n, Particle());
  for (int i = 0; i < n; i++) { S.par[i].id = i; S.par[i].mask = mask[i]; S.par[i].bound.has = true; }
  for (int f = 0; f < nFrames; f++) {
    const double* mn = mins + (size_t)3 * n * f;
    const double* mx = maxs + (size_t)3 * n * f;
    bool init = S.BB[0].empty();
    if (init)
      for (int j = 0; j < 3; j++)
        for (int id = 0; id < n; id++) { S.BB[j].push_back(Bounds(0, id, true)); S.BB[j].push_back(Bounds(0, id, false)); }
    for (int j = 0; j < 3; j++)
      for (Bounds& b : S.BB[j]) { b.hasBB = true; b.coord = b.isMin ? mn[3 * b.id + j] : mx[3 * b.id + j]; }
    S.minima.assign(mn, mn + 3 * n); S.maxima.assign(mx, mx + 3 * n);
    if (!init) { for (int j = 0; j < 3; j++) insertionSort(S, S.BB[j], true); }
    else {
      for (int j = 0; j < 3; j++) std::sort(S.BB[j].begin(), S.BB[j].end());
      std::vector<Bounds>& V = S.BB[0];
      long n2 = 2L * n;
      for (long i = 0; i < n2; i++) {
        if (!(V[i].isMin && V[i].hasBB)) continue;
        int iid = V[i].id;
        for (long j = i + 1; j < n2 && V[j].id != iid; j++) { if (!V[j].isMin) continue; handleBoundInversion(S, iid, V[j].id, false); }
      }
    }
    for (auto& C : S.removeContacts) removeMaybe_fast(S, C);
    S.removeContacts.clear();
    for (auto& C : S.makeContacts) addMaybe_fast(S, C);
    S.makeContacts.clear();
  }
  std::vector<long> keys;
  for (auto& c : S.linView) keys.push_back(((long)std::min(c->pA, c->pB) << 32) | std::max(c->pA, c->pB));
  std::sort(keys.begin(), keys.end());
  long cnt = (long)keys.size();
  for (long i = 0; i < cnt && i < maxPairs; i++) { pairs[2 * i] = (int32_t)(keys[i] >> 32); pairs[2 * i + 1] = (int32_t)(keys[i] & 0xffffffffL); }
  return cnt;
}

}  /* extern "C" */
