// wdem_api.cu -- host runtime of the GB300 DEM engine and its C ABI (include/wdem.h).
//
// The handle owns all device memory and one CUDA stream.  One wdem_step runs, per step, the same
// engine order as Woo's Scene::doOneStep with [Leapfrog, InsertionSortCollider, ContactLoop]
// (src/core/Scene.cpp:420-427):
//   1. k_leapfrog      forces gathered through the contact CSR, integration, verlet trigger
//   2. collider        only when a particle left its verlet box (or after an upload): boxes, grid,
//                      radix sort, sweep, contact history carried over through the old CSR's
//                      sorted keys, real contacts compacted to the front, CSR
//   3. k_contacts      fused Cg2 + Cp2 + Law2 over the contact list
#include "wdem_internal.h"
#include "../../include/wdem.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

using namespace wdem;

namespace wdem {
long long g_kernel_launches = 0;
}

namespace {

const char* kPhaseNames[] = {"leapfrog", "collider", "contacts"};
enum { PH_LEAPFROG = 0, PH_COLLIDER = 1, PH_CONTACTS = 2, PH_COUNT = 3 };

struct ContactBuf {
  Contacts c;
  long long cap = 0;
  bool hertz = false;
  bool geom = false;
  bool peri = false;
  bool ell = false;
};

// Periodic cell on the host (Cell, src/core/Cell.hpp / Cell.cpp), homoDeform GRADV2; row-major 3x3.
struct M3 {
  double r[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  static M3 I() { M3 m; m.r[0][0] = m.r[1][1] = m.r[2][2] = 1; return m; }
};
M3 mul(const M3& a, const M3& b) {
  M3 c;
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) c.r[i][k] = a.r[i][0] * b.r[0][k] + a.r[i][1] * b.r[1][k] + a.r[i][2] * b.r[2][k];
  return c;
}
M3 addScaled(const M3& a, const M3& b, double sb) {
  M3 c;
  for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) c.r[i][k] = a.r[i][k] + sb * b.r[i][k];
  return c;
}
M3 scaled(const M3& a, double s) { M3 c; for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) c.r[i][k] = a.r[i][k] * s; return c; }
M3 transposed(const M3& a) { M3 c; for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) c.r[i][k] = a.r[k][i]; return c; }
// Eigen's 3x3 determinant: expansion along row 0
double det3(const M3& m) {
  const double (*a)[3] = m.r;
  return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
         a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
}
// Eigen's 3x3 inverse: adjugate x (1 / det), det from the cofactors of column 0
M3 inv3(const M3& m) {
  const double (*a)[3] = m.r;
  M3 c;
  c.r[0][0] = a[1][1] * a[2][2] - a[1][2] * a[2][1];
  c.r[0][1] = a[0][2] * a[2][1] - a[0][1] * a[2][2];
  c.r[0][2] = a[0][1] * a[1][2] - a[0][2] * a[1][1];
  c.r[1][0] = a[1][2] * a[2][0] - a[1][0] * a[2][2];
  c.r[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0];
  c.r[1][2] = a[0][2] * a[1][0] - a[0][0] * a[1][2];
  c.r[2][0] = a[1][0] * a[2][1] - a[1][1] * a[2][0];
  c.r[2][1] = a[0][1] * a[2][0] - a[0][0] * a[2][1];
  c.r[2][2] = a[0][0] * a[1][1] - a[0][1] * a[1][0];
  const double d = c.r[0][0] * a[0][0] + c.r[0][1] * a[1][0] + c.r[0][2] * a[2][0];
  const double invdet = 1.0 / d;
  for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) c.r[i][k] = c.r[i][k] * invdet;
  return c;
}
void leviCivita(const M3& m, double* v) { v[0] = m.r[1][2] - m.r[2][1]; v[1] = m.r[2][0] - m.r[0][2]; v[2] = m.r[0][1] - m.r[1][0]; }

struct HostCell {
  M3 trsf = M3::I(), hSize = M3::I(), pprevHsize = M3::I(), gradV, nextGradV, W, shearTrsf = M3::I(), unshearTrsf = M3::I();
  double spinVec[3] = {0, 0, 0}, size[3] = {1, 1, 1}, cos[3] = {1, 1, 1};
  bool hasShear = false;
  // Cell::integrateAndUpdate (Cell.cpp:81-120)
  bool integrateAndUpdate(double dt) {
    M3 trsfInc = scaled(gradV, dt);
    trsf = addScaled(trsf, mul(trsfInc, trsf), 1.0);
    M3 prev = hSize;
    M3 g2 = scaled(scaled(gradV, dt), 1. / 2.);
    hSize = mul(mul(inv3(addScaled(M3::I(), g2, -1.0)), addScaled(M3::I(), g2, 1.0)), hSize);
    pprevHsize = scaled(addScaled(prev, hSize, 1.0), .5);
    if (det3(hSize) == 0) return false;
    M3 Hn;
    for (int i = 0; i < 3; i++) {
      double b[3] = {hSize.r[0][i], hSize.r[1][i], hSize.r[2][i]};
      size[i] = std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
      for (int k = 0; k < 3; k++) Hn.r[k][i] = b[k] / size[i];
    }
    for (int i = 0; i < 3; i++) {
      int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      double a[3] = {Hn.r[0][i1], Hn.r[1][i1], Hn.r[2][i1]}, b[3] = {Hn.r[0][i2], Hn.r[1][i2], Hn.r[2][i2]};
      double c0 = a[1] * b[2] - a[2] * b[1], c1 = a[2] * b[0] - a[0] * b[2], c2 = a[0] * b[1] - a[1] * b[0];
      cos[i] = c0 * c0 + c1 * c1 + c2 * c2;
    }
    shearTrsf = Hn;
    unshearTrsf = inv3(Hn);
    const double (*h)[3] = hSize.r;
    hasShear = (h[0][1] != 0 || h[0][2] != 0 || h[1][0] != 0 || h[1][2] != 0 || h[2][0] != 0 || h[2][1] != 0);
    return true;
  }
  // Cell::setNextGradV (Cell.cpp:60-66)
  void setNextGradV() {
    gradV = nextGradV;
    W = scaled(addScaled(gradV, transposed(gradV), -1.0), .5);
    double v[3];
    leviCivita(W, v);
    for (int k = 0; k < 3; k++) spinVec[k] = .5 * v[k];
  }
};

void put9(double* dst, const M3& m) { for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) dst[3 * i + k] = m.r[i][k]; }
M3 get9(const double* src) { M3 m; for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) m.r[i][k] = src[3 * i + k]; return m; }

}  // namespace

struct wdem_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  int N = 0;   // capacity
  int n = 0;   // particles
  Particles d{};
  // host copies of static per-particle data (radius, shape, material) for pWaveDt and checks
  std::vector<int> shape, mat;
  std::vector<double> radius;
  std::vector<int> smallIds, largeIds;
  int* dSmall = nullptr;
  ContactBuf buf[2];
  int cur = 0;
  long long nContacts = 0;
  Csr csr{};
  long long csrCap = 0;
  ColliderScratch cs{};
  DeviceStatus* dst = nullptr;
  DeviceStatus* hst = nullptr;  // pinned
  unsigned* hcounts = nullptr;  // pinned, 4 entries
  wdem_params raw{};
  std::vector<wdem_material> mats;
  StepParams P{};
  bool paramsSet = false;
  bool particlesSet = false;
  bool forcesInArrays = true;
  bool needRebuild = true;
  bool keepGeom = false;
  long long step = 0;
  long long seq = 0;            // contact passes run so far (stamps of the force records; never reset)
  long long nFullRuns = 0;
  int lastRunFull = 0;
  // queued steps (runQueued): depth limit (0 or 1: every step checked on the host), mean steps between
  // rebuilds, steps since the last one
  bool actValid = false;  // the cull's active list matches the container (a full cull ran since the rebuild)
  bool denseTouch = false;  // real contacts were at least n/8 at the end of the last queue that ran through
  int maxAhead = 32;
  double rebuildInterval = 16;
  int sinceRebuild = 0;
  // queued steps replayed from CUDA graphs: one executable graph per (queue length, first cull full or
  // not), valid while the launch arguments it was captured with (sig) are unchanged; the steps' numbers
  // come from DeviceStatus.stepBase/seqBase, written before each replay
  struct StepGraph {
    std::vector<unsigned char> sig;
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;  // kernel nodes of the graph
  };
  std::map<int, StepGraph> graphs;
  int graphMode = WDEM_GRAPHS_OFF;
  long long graphCaptures = 0, graphReplays = 0;
  // DynDt as a PeriodicEngine (Engine.hpp:130-160): stepLast / stepPrev, Scene.nextDt, last critical step
  long long dynStepLast = -1, dynStepPrev = -1;
  double nextDt = std::numeric_limits<double>::quiet_NaN();
  double dynDtCrit = std::numeric_limits<double>::quiet_NaN();
  double timeSum = 0;  // sum of dt over the steps run
  int updatePhys = 0;
  double verletDistResolved = 0;
  bool verletResolved = false;
  // timing
  bool timing = false;
  std::vector<cudaEvent_t> evPool;
  size_t evUsed = 0;
  std::vector<std::pair<int, std::pair<size_t, size_t>>> evMarks;  // phase, (start, stop) indices
  double phaseMs[PH_COUNT] = {0, 0, 0};
  int phaseLaunches[PH_COUNT] = {0, 0, 0};
  std::string err;
  double* staging = nullptr;    // 13 n doubles for wdem_write_state / wdem_read_state
  long long stagingCap = 0;
  bool periodic = false;
  bool hasEll = false;          // ellipsoids or aspherical nodes: per-particle rotation state allocated
  bool hasFacets = false;       // facets among the particles (their contacts take the FP64 law)
  // facet + wall / facet + facet pairs of one scene whose masks share bits (facet, other, mask & mask); none may
  // survive loneMask at a step
  std::vector<int4> facetPairs;
  unsigned facetsChecked = ~0u;  // loneMask the pairs were last checked against (~0: not yet)
  long long matsChecked = -1;   // material-table size the particle material indices were checked against
  bool gravAccDirty = true;     // angw.w (cached gravity acceleration) needs recomputing
  double* dMatDt = nullptr;     // batched scenes: dt per material
  int matDtCap = 0;
  bool useMatDt = false;
  std::vector<double> semi;     // host copy of the semi-axes (3n; spheres r, r, r)
  float* ellLog = nullptr;      // training records of the ellipsoid solves, when logging
  unsigned long long* ellLogCount = nullptr;
  long long ellLogCap = 0;
  HostCell cell;
  // learned warm start: FP32 master weights (padded layout), BF16 copy, Adam moments, gradient
  float *mlpW = nullptr, *mlpM = nullptr, *mlpV = nullptr, *mlpGrad = nullptr, *mlpLoss = nullptr;
  uint16_t* mlpWbf = nullptr;
  bool mlpReady = false;
  long long mlpT = 0;
  double* dStress = nullptr;    // 9 stress components + scratch for the terms
  double* stressTerms = nullptr;
  long long stressCap = 0;
  std::vector<DevMaterial> devMats;  // the materials table in the kernels' layout
  long long contactLimit = 0;        // wdem_set_contact_limit (0: none)
  wdem_launch_shape launchShape{128, 0, 256, 256, 0, 0};  // launch shape of the step kernels
  int numSMs = 152;
  // particle removal / insertion (wdem_remove_particles, wdem_add_particles): per-particle flags, id list,
  // park positions and the packed records of inserted particles
  uint8_t* editGone = nullptr;
  int* editIds = nullptr;
  double* editPark = nullptr;
  double4_32a* editRec = nullptr;
  int4* editMeta = nullptr;
  long long editCap = 0;
  double* dEnergy = nullptr;    // WDEM_E_COUNT accumulators
  double* ePartials = nullptr;  // block partials of the energy sums
  long long ePartialsCap = 0;
};

namespace {

// The materials table lives in constant memory, one per device and kernel variant, shared by the handles
// of the process: the handle that last uploaded it is recorded, and a step of another handle uploads its
// own table first.
const wdem_handle* g_matsOwner[64] = {nullptr};
void uploadMaterials(wdem_handle* h) {
  upload_materials(h->devMats.data(), (int)h->devMats.size());
  contracted::upload_materials(h->devMats.data(), (int)h->devMats.size());
  if (h->device >= 0 && h->device < 64) g_matsOwner[h->device] = h;
}

int fail(wdem_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

#define CK(call)                                                                            \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return fail(h, WDEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
  } while (0)

template <class T>
cudaError_t dalloc(T*& p, size_t count) {
  if (p) { cudaFree(p); p = nullptr; }
  if (count == 0) count = 1;
  return cudaMalloc((void**)&p, align256(count * sizeof(T)));
}

void freeContacts(ContactBuf& b) {
  Contacts& c = b.c;
  cudaFree(c.ids); cudaFree(c.state); cudaFree(c.act); cudaFree(c.step0); cudaFree(c.tanPhi);
  for (int k = 0; k < HIST_COUNT; k++) cudaFree(c.hist[k]);
  cudaFree(c.out); cudaFree(c.slot); cudaFree(c.rowBit);
  for (int k = 0; k < 7; k++) cudaFree(c.geom[k]);
  for (int k = 0; k < EC_COUNT; k++) cudaFree(c.energy[k]);
  cudaFree(c.cdist);
  cudaFree(c.work);
  cudaFree(c.lam);
  cudaFree(c.lam0);
  memset(&c, 0, sizeof(c));
  b.cap = 0;
}

// (Re)allocate one contact buffer for `cap` contacts, keeping nothing.
cudaError_t allocContacts(ContactBuf& b, long long cap, bool hertz, bool geom, bool peri, bool ell) {
  freeContacts(b);
  Contacts& c = b.c;
  cudaError_t e;
  if ((e = dalloc(c.ids, cap))) return e;
  if ((e = dalloc(c.state, cap))) return e;
  if ((e = dalloc(c.step0, cap))) return e;
  if ((e = dalloc(c.tanPhi, cap))) return e;
  int nh = hertz ? (int)HIST_COUNT : (int)HIST_FRICT;
  for (int k = 0; k < nh; k++) if ((e = dalloc(c.hist[k], cap))) return e;
  // two CSR entries per contact; stamps start at -1 (no pass has written them)
  if ((e = dalloc(c.out, (size_t)OUT_RECORDS * 2 * cap))) return e;
  if ((e = cudaMemset(c.out, 0xff, (size_t)OUT_RECORDS * 2 * cap * sizeof(double4_32a)))) return e;
  if ((e = dalloc(c.slot, cap))) return e;
  if ((e = dalloc(c.rowBit, cap))) return e;
  if (geom) for (int k = 0; k < 7; k++) if ((e = dalloc(c.geom[k], cap))) return e;
  for (int k = 0; k < EC_COUNT; k++) if ((e = dalloc(c.energy[k], cap))) return e;
  if ((e = dalloc(c.work, cap))) return e;
  if ((e = dalloc(c.act, cap))) return e;
  if (peri && (e = dalloc(c.cdist, cap))) return e;
  if (ell && ((e = dalloc(c.lam, cap)) || (e = dalloc(c.lam0, cap)))) return e;
  b.cap = cap;
  b.peri = peri;
  b.ell = ell;
  b.hertz = hertz;
  b.geom = geom;
  return cudaSuccess;
}

// Copy the first n contacts of src into dst (both device), used when a buffer grows in place.

size_t evNext(wdem_handle* h) {
  if (h->evUsed >= h->evPool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    h->evPool.push_back(e);
  }
  return h->evUsed++;
}

struct PhaseTimer {
  wdem_handle* h;
  int ph;
  size_t a = 0;
  PhaseTimer(wdem_handle* h_, int ph_) : h(h_), ph(ph_) {
    if (h->timing) { a = evNext(h); cudaEventRecord(h->evPool[a], h->stream); }
  }
  ~PhaseTimer() {
    if (h->timing) {
      size_t b = evNext(h);
      cudaEventRecord(h->evPool[b], h->stream);
      h->evMarks.push_back(std::make_pair(ph, std::make_pair(a, b)));
    }
  }
};

void collectTimes(wdem_handle* h) {
  if (!h->timing || h->evMarks.empty()) return;
  cudaStreamSynchronize(h->stream);
  for (auto& m : h->evMarks) {
    float ms = 0;
    cudaEventElapsedTime(&ms, h->evPool[m.second.first], h->evPool[m.second.second]);
    h->phaseMs[m.first] += ms;
    h->phaseLaunches[m.first] += 1;
  }
  h->evMarks.clear();
  h->evUsed = 0;
}

// Scratch for the collider sized for nSmall particles and up to nc contacts.
int ensureScratch(wdem_handle* h, long long nc) {
  ColliderScratch& cs = h->cs;
  long long needSort = std::max<long long>((long long)h->smallIds.size(), 2 * nc) + 16;
  if (needSort > cs.sortCap) {
    long long cap = std::max<long long>(needSort, cs.sortCap * 3 / 2);
    CK(dalloc(cs.keys, cap)); CK(dalloc(cs.keysAlt, cap));
    CK(dalloc(cs.vals, cap)); CK(dalloc(cs.valsAlt, cap));
    cs.sortCap = cap;
    cs.histCap = radix_scratch_words(cap);
    CK(dalloc(cs.hist, cs.histCap));
  }
  if (h->periodic && (long long)h->smallIds.size() + 1 > cs.periCap) {
    long long cap = (long long)h->smallIds.size() + 1;
    CK(dalloc(cs.periC, cap)); CK(dalloc(cs.periH, cap));
    CK(dalloc(cs.periCi, (size_t)h->N + 1)); CK(dalloc(cs.periHi, (size_t)h->N + 1));
    cs.periCap = cap;
  }
  // the counting sweep's pair buffer (not used by the periodic collider)
  const long long nSweepT = sweepThreads((int)h->smallIds.size(), cs.nLarge);
  if (!h->periodic && nSweepT > cs.sweepBufCap) {
    const long long cap = std::max<long long>(nSweepT, cs.sweepBufCap * 5 / 4);
    CK(dalloc(cs.sweepBuf, (size_t)cap * SWEEP_BUF));
    cs.sweepBufCap = cap;
  }
  long long needRetain = std::max<long long>(h->nContacts, nc) + 2;
  if (needRetain > cs.retainCap) {
    long long cap = std::max<long long>(needRetain, cs.retainCap * 3 / 2);
    CK(dalloc(cs.retainFlag, cap));
    cs.retainCap = cap;
  }
  // scan scratch: level sums of the longest scan (histograms, pair counts, retain flags)
  long long longest = std::max<long long>(std::max<long long>(cs.histCap, (long long)h->N + 2), cs.retainCap);
  long long needSums = 64 + 2 * (longest / 1024 + 64) + 4096;
  if (needSums > cs.blockSumsCap) {
    CK(dalloc(cs.blockSums, needSums));
    cs.blockSumsCap = needSums;
  }
  return WDEM_OK;
}

// periodic candidate buffers for n candidates (flags scanned in place: n + 1 entries), and the scan
// scratch for a scan of that length
int ensureCand(wdem_handle* h, long long n) {
  ColliderScratch& cs = h->cs;
  if (n + 1 > cs.candCap) {
    long long cap = std::max<long long>(n + n / 4 + 1024, cs.candCap);
    CK(dalloc(cs.cand, cap)); CK(dalloc(cs.candPer, cap)); CK(dalloc(cs.candFlag, cap + 1));
    cs.candCap = cap;
  }
  long long needSums = 64 + 2 * ((n + 1) / 1024 + 64) + 4096;
  if (needSums > cs.blockSumsCap) {
    CK(dalloc(cs.blockSums, needSums));
    cs.blockSumsCap = needSums;
  }
  return WDEM_OK;
}

int ensureCsr(wdem_handle* h, long long nc) {
  if (2 * nc + 1 > h->csrCap) {
    long long cap = std::max<long long>(2 * nc + 1, h->csrCap * 3 / 2);
    CK(dalloc(h->csr.ent, cap));
    CK(dalloc(h->csr.keys, cap));
    h->csrCap = cap;
  }
  return WDEM_OK;
}

int ensurePartials(wdem_handle* h, long long n) {
  long long need = n / 2048 + 16;
  if (need > h->ePartialsCap) {
    CK(dalloc(h->ePartials, need));
    h->ePartialsCap = need;
  }
  return WDEM_OK;
}

int checkDeviceStatus(wdem_handle* h) {
  if (h->hst->code != 0) {
    int code = h->hst->code;
    std::string m;
    if (code == WDEM_ERR_NAN) m = "NaN in the state or in a contact force (particle #" + std::to_string(h->hst->detail) + ")";
    else if (code == WDEM_ERR_OVERFLOW) m = "a device table ran out of capacity";
    else if (code == WDEM_ERR_TOO_BIG)
      m = "ambiguous periodic contact of particle #" + std::to_string(h->hst->detail) +
          ": the boxes overlap across more than one period (a particle larger than half of the cell)";
    else if (code == WDEM_ERR_UNSUPPORTED)
      m = "sphere-facet contact with the projected centre outside all three edges of Facet #" +
          std::to_string(h->hst->detail) + " (degenerate facet)";
    else if (code == WDEM_ERR_TIMEOUT && h->hst->detail == -1)
      m = "the tensor-core warm-start network did not complete within its wait limit";
    else if (code == WDEM_ERR_TIMEOUT)
      m = "a bounded device loop hit its iteration limit (contact solver, particle #" + std::to_string(h->hst->detail) + ")";
    else m = "device error " + std::to_string(code);
    return fail(h, code, m);
  }
  return WDEM_OK;
}

// Collider rebuild: InsertionSortCollider full run (InsertionSortCollider.cpp:407-612).
int rebuild(wdem_handle* h) {
  cudaStream_t s = h->stream;
  const int n = h->n;
  const int nSmall = (int)h->smallIds.size();
  ColliderScratch& cs = h->cs;
  int rc;
  if ((rc = ensureScratch(h, h->nContacts))) return rc;
  launch_bboxes(s, h->P, h->d, n);
  const int nSweep = sweepThreads(nSmall, cs.nLarge);
  const unsigned* totalSrc = cs.counts + nSweep;
  long long nCand = 0;
  if (h->periodic) {
    col_periodic_cand(s, h->P, h->d, h->dSmall, nSmall, cs, false);
    CK(cudaMemcpyAsync(&h->hcounts[0], cs.counts + nSmall + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    nCand = h->hcounts[0];
    if ((rc = ensureCand(h, nCand))) return rc;
    col_periodic_cand(s, h->P, h->d, h->dSmall, nSmall, cs, true);
    col_periodic_exact(s, h->P, h->d, cs, nCand, h->dst);
    totalSrc = cs.candFlag + nCand;
  } else {
    col_extents_and_grid(s, h->d, h->dSmall, nSmall, cs);
    col_sort(s, h->d, h->dSmall, nSmall, cs);
    col_sweep(s, h->d, nSmall, h->P.loneMask, cs, nullptr, 0, false, h->dst);
    exclusive_scan_u32(s, cs.counts, nSweep, cs);
  }
  ContactBuf& old = h->buf[h->cur];
  ContactBuf& neu = h->buf[1 - h->cur];
  const long long nOld = h->nContacts;
  col_retain_flags(s, h->P, h->d, old.c, nOld, cs);
  CK(cudaMemcpyAsync(&h->hcounts[0], totalSrc, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&h->hcounts[1], cs.retainFlag + nOld, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const long long total = h->hcounts[0];
  const long long retained = h->hcounts[1];
  const long long nNew = total + retained;
  if (h->contactLimit > 0 && nNew > h->contactLimit)
    return fail(h, WDEM_ERR_OVERFLOW, "collider: " + std::to_string(nNew) + " contacts exceed the limit of " +
                                          std::to_string(h->contactLimit) + " (wdem_set_contact_limit)");
  const bool hertz = (h->P.cp2 == WDEM_CP2_HERTZ);
  if (nNew > neu.cap || neu.hertz != hertz || neu.geom != h->keepGeom || neu.peri != h->periodic || neu.ell != h->hasEll) {
    long long cap = std::max<long long>(nNew + nNew / 4 + 1024, neu.cap);
    CK(allocContacts(neu, cap, hertz, h->keepGeom, h->periodic, h->hasEll));
  }
  if (h->periodic) col_periodic_emit(s, cs, nCand, neu.c.ids, neu.c.cdist, neu.cap);
  else col_sweep(s, h->d, nSmall, h->P.loneMask, cs, neu.c.ids, neu.cap, true, h->dst);
  col_retain_write(s, old.c, nOld, cs, neu.c.ids, total, neu.cap);
  if (h->periodic && old.c.cdist) col_retain_write_dist(s, old.c, nOld, cs, neu.c.cdist, total, neu.cap);
  const int side = 1 - h->cur;
  // history carried over (each new pair found in the old container through the old CSR's sorted keys),
  // contacts real before the rebuild compacted to the front (the sort scratch, sized for 2 nNew entries,
  // holds the temporaries); then the new container's CSR
  if ((rc = ensureScratch(h, nNew))) return rc;
  Csr oldCsr = h->csr;
  if (nOld <= 0) oldCsr.n = 0;
  col_carry_compact(s, h->d, neu.c, nNew, old.c, oldCsr, h->step, (hertz && old.hertz) ? (int)HIST_COUNT : (int)HIST_FRICT, cs);
  if ((rc = ensureCsr(h, nNew))) return rc;
  col_csr(s, neu.c, nNew, n, h->csr, cs);
  h->cur = side;
  h->nContacts = nNew;
  h->nFullRuns++;
  h->needRebuild = false;
  h->actValid = false;
  return WDEM_OK;
}

void fillStepParams(wdem_handle* h) {
  const wdem_params& r = h->raw;
  StepParams& P = h->P;
  P.dt = r.dt;
  P.step = h->step;
  P.shContactsBlock = h->launchShape.contactsBlock; P.shContactsPerSM = h->launchShape.contactsPerSM;
  P.shCullBlock = h->launchShape.cullBlock; P.shLeapBlock = h->launchShape.integratorBlock; P.shListsPerSM = h->launchShape.listsPerSM;
  P.numSMs = h->numSMs;
  for (int k = 0; k < 3; k++) P.gravity[k] = r.gravity[k];
  P.hasGravity = !(r.gravity[0] == 0 && r.gravity[1] == 0 && r.gravity[2] == 0);
  {
    int nz = 0, ax = -1;
    for (int k = 0; k < 3; k++) if (r.gravity[k] != 0) { nz++; ax = k; }
    P.gravAxis = (nz == 1) ? ax : -1;
    h->gravAccDirty = true;  // recomputed before the next step (parameters change rarely)
  }
  P.distFactor = r.distFactor;
  P.distFactorF = (float)std::fabs(r.distFactor);
  P.bboxFactor = r.distFactor > 0 ? r.distFactor : 1.;
  P.loneMask = r.loneMask;
  P.damping = r.damping;
  P.verletDist = h->verletDistResolved;
  P.maxD2 = h->verletDistResolved * h->verletDistResolved;
  P.verletLoF = (float)(h->verletDistResolved * (1 - 1e-6));
  P.verletHiF = (float)(h->verletDistResolved * (1 + 1e-6));
  P.dampM = 1.0 - r.damping * 1.0;
  P.dampP = 1.0 - r.damping * -1.0;
  P.dampOn = r.damping != 0. ? 1 : 0;
  P.noRatch = r.noRatch; P.iniLensTouch = r.iniLensTouch; P.trsfRenorm = r.trsfRenorm; P.approxMask = r.approxMask;
  P.updatePhysNow = (h->updatePhys != WDEM_UPDATE_PHYS_NEVER);
  P.cp2 = r.cp2; P.law = r.law;
  P.dw = r.arith == WDEM_ARITH_DW ? 1 : 0;
  P.noSlip = r.noSlip; P.noBreak = r.noBreak; P.noFrict = r.noFrict;
  P.relRollStiff = r.relRollStiff; P.relTwistStiff = r.relTwistStiff; P.rollTanPhi = r.rollTanPhi;
  P.noAttraction = r.noAttraction;
  P.poisson = r.poisson; P.en = r.en;
  // Cp2_HertzMat_HertzPhys (Hertz.cpp:70): the same for every contact, so evaluated once here
  double en = r.en;
  P.viscAlpha = (en > 0 && en < 1.) ? -std::sqrt(5) * std::log(en) / (std::sqrt(std::log(en) * std::log(en) + M_PI * M_PI)) : 0.;
  P.trackEnergy = r.trackEnergy;
  P.lfEnergy = r.trackEnergy;
  P.nMaterials = (int)h->mats.size();
  P.periodic = h->periodic ? 1 : 0;
  P.matDt = h->useMatDt ? h->dMatDt : nullptr;
  P.hasEll = h->hasEll ? 1 : 0;
  P.hasFacets = h->hasFacets ? 1 : 0;
  P.ellSolver = r.ellSolver;
  P.brentTol = std::ldexp(1.0, 1 - std::min(std::numeric_limits<double>::digits / 2, (int)r.brentBits));
  P.newtonTol = r.newtonTol;
  P.warmStart = r.warmStart;
  P.fallbackIters = r.fallbackIters;
  P.ellLog = h->ellLog;
  P.ellLogCount = h->ellLogCount;
  P.ellLogCap = h->ellLogCap;
}

// Cell-dependent parameters of one step: shifts, unshear, Leapfrog GRADV2 matrices (Leapfrog.cpp:119-127)
// MCLS_* class of each entry of a row-major 3x3 matrix, 2 bits per entry
int entryClasses(const double* m) {
  int c = 0;
  for (int k = 0; k < 9; k++) {
    unsigned long long b;
    std::memcpy(&b, &m[k], 8);
    int e = MCLS_GEN;
    if (b == 0) e = MCLS_PZERO;
    else if (b == 0x8000000000000000ull) e = MCLS_NZERO;
    else if (m[k] == 1.0) e = MCLS_ONE;
    c |= e << (2 * k);
  }
  return c;
}

void fillCellParams(wdem_handle* h) {
  StepParams& P = h->P;
  const HostCell& c = h->cell;
  const double dt = P.dt;
  put9(P.hS, c.hSize);
  put9(P.shv, mul(c.gradV, c.pprevHsize));
  put9(P.unsh, c.unshearTrsf);
  for (int k = 0; k < 3; k++) { P.csize[k] = c.size[k]; P.sae[k] = 1 / c.cos[k] - 1; P.spinVec[k] = c.spinVec[k]; }
  P.hasShear = c.hasShear ? 1 : 0;
  put9(P.gradV, c.gradV);
  M3 q = scaled(scaled(addScaled(c.nextGradV, c.gradV, 1.0), dt), 1. / 4.);
  put9(P.ImLL4hInv, inv3(addScaled(M3::I(), q, -1.0)));
  put9(P.IpLL4h, addScaled(M3::I(), q, 1.0));
  put9(P.LmL, addScaled(c.nextGradV, c.gradV, -1.0));
  double a[3], b[3];
  leviCivita(scaled(addScaled(c.gradV, transposed(c.gradV), -1.0), .5), a);
  leviCivita(scaled(addScaled(c.nextGradV, transposed(c.nextGradV), -1.0), .5), b);
  for (int k = 0; k < 3; k++) P.dSpin[k] = -.5 * a[k] + .5 * b[k];
  P.clsGradV = entryClasses(P.gradV);
  P.clsImLL4hInv = entryClasses(P.ImLL4hInv);
  P.clsIpLL4h = entryClasses(P.IpLL4h);
  P.clsLmL = entryClasses(P.LmL);
  unsigned long long sb[3];
  std::memcpy(sb, P.dSpin, sizeof sb);
  P.dSpinZero = (sb[0] | sb[1] | sb[2]) == 0 ? 1 : 0;
}

// AabbCollider::setVerletDist (Collision.cpp:164-184): negative -> |verletDist| * min sphere radius
void resolveVerlet(wdem_handle* h) {
  double vd = h->raw.verletDist;
  if (vd >= 0) { h->verletDistResolved = vd; return; }
  double minR = std::numeric_limits<double>::infinity();
  for (int i = 0; i < h->n; i++) {
    // Shape::equivRadius: Sphere.radius, Ellipsoid cbrt(abc) (Ellipsoid.cpp:25-28), Capsule the radius of the
    // sphere of its volume (Capsule.cpp:25-31); NaN for walls and facets
    double r = std::numeric_limits<double>::quiet_NaN();
    if (h->shape[i] == WDEM_SHAPE_SPHERE) r = h->radius[i];
    else if (h->shape[i] == WDEM_SHAPE_ELLIPSOID) r = std::cbrt(h->semi[3 * i] * h->semi[3 * i + 1] * h->semi[3 * i + 2]);
    else if (h->shape[i] == WDEM_SHAPE_CAPSULE) {
      const double rc = h->radius[i], vol = (4 / 3.) * M_PI * (rc * rc * rc) + M_PI * (rc * rc) * h->semi[3 * i + 1];
      r = std::cbrt(vol * 3 / (4 * M_PI));
    }
    if (!std::isnan(r)) minR = std::min(r, minR);
  }
  h->verletDistResolved = std::isinf(minR) ? 0.0 : std::abs(vd) * minR;
}

}  // namespace

extern "C" {

int wdem_abi_version(void) { return WDEM_ABI_VERSION; }

int wdem_create(int device, int32_t maxParticles, wdem_handle** out) {
  if (!out || maxParticles <= 0) return WDEM_ERR_ARG;
  *out = nullptr;
  wdem_handle* h = new wdem_handle();
  h->device = device;
  h->N = maxParticles;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete h; return WDEM_ERR_CUDA; }
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) { delete h; return WDEM_ERR_CUDA; }
  {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && sms > 0) h->numSMs = sms;
    h->P.numSMs = h->numSMs;
    h->P.shContactsBlock = 128; h->P.shCullBlock = 256; h->P.shLeapBlock = 256;
  }
  int N = maxParticles;
  Particles& d = h->d;
  bool ok = true;
  ok &= dalloc(d.posr, N) == cudaSuccess;
  ok &= dalloc(d.velm, N) == cudaSuccess;
  ok &= dalloc(d.angw, N) == cudaSuccess;
  ok &= dalloc(d.inert, N) == cudaSuccess;
  ok &= dalloc(d.ori, N) == cudaSuccess;
  ok &= dalloc(d.lastPos, N) == cudaSuccess;
  ok &= dalloc(d.bbmin, N) == cudaSuccess;
  ok &= dalloc(d.bbmax, N) == cudaSuccess;
  ok &= dalloc(d.force, N) == cudaSuccess;
  ok &= dalloc(d.torque, N) == cudaSuccess;
  ok &= dalloc(d.meta, N) == cudaSuccess;
  ok &= dalloc(d.posf, N) == cudaSuccess;
  ok &= dalloc(d.lastPosf, N) == cudaSuccess;
  ok &= dalloc(d.touched, N) == cudaSuccess;
  ok &= dalloc(d.rowMask, N) == cudaSuccess;
  ok &= dalloc(d.rotList, N) == cudaSuccess;
  ok &= dalloc(d.touchList, N) == cudaSuccess;
  for (int k = 0; k < 3; k++) ok &= dalloc(d.energy[k], N) == cudaSuccess;
  ok &= dalloc(h->dEnergy, WDEM_E_COUNT) == cudaSuccess;
  ok &= dalloc(h->dSmall, N) == cudaSuccess;
  ok &= dalloc(h->cs.large, N) == cudaSuccess;
  ok &= dalloc(h->cs.counts, (size_t)N + 2) == cudaSuccess;
  ok &= dalloc(h->cs.srec, 2 * (size_t)N + 2) == cudaSuccess;
  ok &= dalloc(h->cs.grid, 1) == cudaSuccess;
  ok &= dalloc(h->csr.rowptr, (size_t)N + 1) == cudaSuccess;
  ok &= dalloc(h->csr.cursor, (size_t)N) == cudaSuccess;
  unsigned long long* tmp = nullptr;
  ok &= dalloc(tmp, 64) == cudaSuccess;
  h->cs.temp = tmp;
  // column budget: enough for a fine grid without letting cellStart dominate memory
  h->cs.maxCols = std::max(1024, std::min(1 << 24, 2 * N));
  ok &= dalloc(h->cs.cellStart, (size_t)h->cs.maxCols + 2) == cudaSuccess;
  ok &= dalloc(h->dst, 1) == cudaSuccess;
  h->cs.st = h->dst;
  ok &= cudaMallocHost((void**)&h->hst, sizeof(DeviceStatus)) == cudaSuccess;
  ok &= cudaMallocHost((void**)&h->hcounts, 4 * sizeof(unsigned)) == cudaSuccess;
  if (!ok) { wdem_destroy(h); return WDEM_ERR_CUDA; }
  cudaMemset(h->dst, 0, sizeof(DeviceStatus));
  cudaMemset(h->dEnergy, 0, sizeof(double) * WDEM_E_COUNT);
  cudaMemset(h->csr.rowptr, 0, sizeof(int) * ((size_t)N + 1));
  memset(h->hst, 0, sizeof(DeviceStatus));
  // an empty contact buffer on the current side
  if (allocContacts(h->buf[0], 1024, false, false, false, false) != cudaSuccess) { wdem_destroy(h); return WDEM_ERR_CUDA; }
  if (ensureScratch(h, 0)) { wdem_destroy(h); return WDEM_ERR_CUDA; }
  *out = h;
  return WDEM_OK;
}

int wdem_destroy(wdem_handle* h) {
  if (!h) return WDEM_ERR_ARG;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->device >= 0 && h->device < 64 && g_matsOwner[h->device] == h) g_matsOwner[h->device] = nullptr;
  Particles& d = h->d;
  cudaFree(d.semi); cudaFree(d.angMom); cudaFree(d.lastOri); cudaFree(d.maxRot);
  cudaFree(d.fv1); cudaFree(d.fv2);
  cudaFree(h->ellLog); cudaFree(h->ellLogCount);
  cudaFree(h->dMatDt); cudaFree(h->cs.sceneWall);
  cudaFree(h->mlpW); cudaFree(h->mlpM); cudaFree(h->mlpV); cudaFree(h->mlpGrad); cudaFree(h->mlpLoss); cudaFree(h->mlpWbf);
  cudaFree(d.posr); cudaFree(d.velm); cudaFree(d.angw); cudaFree(d.inert); cudaFree(d.ori);
  cudaFree(d.lastPos); cudaFree(d.bbmin); cudaFree(d.bbmax); cudaFree(d.force); cudaFree(d.torque); cudaFree(d.meta); cudaFree(d.posf); cudaFree(d.lastPosf); cudaFree(d.touched); cudaFree(d.rowMask); cudaFree(d.rotList); cudaFree(d.touchList);
  for (int k = 0; k < 3; k++) cudaFree(d.energy[k]);
  cudaFree(h->dEnergy); cudaFree(h->ePartials); cudaFree(h->dStress); cudaFree(h->stressTerms);
  cudaFree(h->dSmall);
  freeContacts(h->buf[0]); freeContacts(h->buf[1]);
  cudaFree(h->csr.rowptr); cudaFree(h->csr.ent); cudaFree(h->csr.cursor); cudaFree(h->csr.keys);
  ColliderScratch& cs = h->cs;
  cudaFree(cs.keys); cudaFree(cs.keysAlt); cudaFree(cs.vals); cudaFree(cs.valsAlt); cudaFree(cs.hist);
  cudaFree(cs.blockSums); cudaFree(cs.cellStart); cudaFree(cs.counts); cudaFree(cs.large); cudaFree(cs.grid); cudaFree(cs.srec);
  cudaFree(cs.retainFlag); cudaFree(cs.temp); cudaFree(cs.periC); cudaFree(cs.periH); cudaFree(cs.periCi); cudaFree(cs.periHi);
  cudaFree(cs.cand); cudaFree(cs.candPer); cudaFree(cs.candFlag); cudaFree(cs.sweepBuf);
  cudaFree(h->dst);
  cudaFree(h->staging);
  cudaFree(h->editGone); cudaFree(h->editIds); cudaFree(h->editPark); cudaFree(h->editRec); cudaFree(h->editMeta);
  if (h->hst) cudaFreeHost(h->hst);
  if (h->hcounts) cudaFreeHost(h->hcounts);
  for (auto e : h->evPool) cudaEventDestroy(e);
  for (auto& g : h->graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return WDEM_OK;
}

const char* wdem_last_error(wdem_handle* h) { return h ? h->err.c_str() : "null handle"; }

int wdem_set_params(wdem_handle* h, const wdem_params* p) {
  if (h) h->actValid = false;  // the far-pair screen depends on verletDist and distFactor
  if (!h || !p) return WDEM_ERR_ARG;
  if (!p->reset) return fail(h, WDEM_ERR_UNSUPPORTED, "Leapfrog.reset=False is not supported (ForceResetter is folded into the GPU engine)");
  if (p->iniEqlb) return fail(h, WDEM_ERR_UNSUPPORTED, "Law2_L6Geom_FrictPhys_IdealElPl.iniEqlb is not supported");
  if (!p->iniLensTouch) return fail(h, WDEM_ERR_UNSUPPORTED, "Cg2_*_L6Geom.iniLensTouch=False is not supported");
  if (!p->applyForces) return fail(h, WDEM_ERR_UNSUPPORTED, "ContactLoop.applyForces=False is not supported");
  if (p->arith != WDEM_ARITH_EXACT && p->arith != WDEM_ARITH_FMA && p->arith != WDEM_ARITH_DW)
    return fail(h, WDEM_ERR_ARG, "arith must be WDEM_ARITH_EXACT, WDEM_ARITH_FMA or WDEM_ARITH_DW");
  if (p->nMaterials <= 0 || !p->materials || p->nMaterials > MAX_MATERIALS) return fail(h, WDEM_ERR_ARG, "materials table missing or larger than 1024");
  if (p->law == WDEM_LAW_HERTZ_DMT && p->cp2 != WDEM_CP2_HERTZ)
    return fail(h, WDEM_ERR_UNSUPPORTED, "Law2_L6Geom_HertzPhys_DMT needs Cp2_HertzMat_HertzPhys");
  if (p->law == WDEM_LAW_IDEALELPL && p->cp2 != WDEM_CP2_FRICT)
    return fail(h, WDEM_ERR_UNSUPPORTED, "Law2_L6Geom_FrictPhys_IdealElPl is supported with Cp2_FrictMat_FrictPhys only");
  if (p->cp2 == WDEM_CP2_HERTZ) {
    for (int a = 0; a < p->nMaterials; a++)
      for (int b = 0; b < p->nMaterials; b++) {
        const wdem_material &m1 = p->materials[a], &m2 = p->materials[b];
        double alpha = .5 * (m1.alpha + m2.alpha), gamma = std::min(m1.surfEnergy, m2.surfEnergy);
        if (alpha != 0. && gamma != 0.)
          return fail(h, WDEM_ERR_UNSUPPORTED, "Schwarz model of Law2_L6Geom_HertzPhys_DMT (alpha!=0 and surfEnergy!=0) is not supported");
      }
  }
  if (h->paramsSet && h->nContacts > 0 && (p->cp2 != h->raw.cp2 || p->law != h->raw.law))
    return fail(h, WDEM_ERR_STATE, "Cp2/Law2 functors cannot change while contacts exist; re-upload the particles");
  bool updatePhysChanged = (h->raw.updatePhys != p->updatePhys) || !h->paramsSet;
  h->raw = *p;
  h->raw.materials = nullptr;
  h->mats.assign(p->materials, p->materials + p->nMaterials);
  h->step = p->step;
  if (updatePhysChanged) h->updatePhys = p->updatePhys;
  std::vector<DevMaterial> dm(h->mats.size());  // the table of both kernel variants (constant memory)
  for (size_t k = 0; k < h->mats.size(); k++) {
    const wdem_material& m = h->mats[k];
    dm[k].kind = m.kind; dm[k].density = m.density; dm[k].young = m.young; dm[k].ktDivKn = m.ktDivKn;
    dm[k].tanPhi = m.tanPhi; dm[k].surfEnergy = m.surfEnergy; dm[k].alpha = m.alpha;
  }
  cudaSetDevice(h->device);
  h->devMats = dm;
  uploadMaterials(h);
  if (p->materialDt) {
    for (int k = 0; k < p->nMaterials; k++)
      if (!(p->materialDt[k] >= 0)) return fail(h, WDEM_ERR_ARG, "materialDt must be non-negative");
    if (h->matDtCap < p->nMaterials) {
      cudaFree(h->dMatDt);
      h->dMatDt = nullptr;
      CK(dalloc(h->dMatDt, (size_t)p->nMaterials));
      h->matDtCap = p->nMaterials;
    }
    CK(cudaMemcpy(h->dMatDt, p->materialDt, p->nMaterials * sizeof(double), cudaMemcpyHostToDevice));
    h->useMatDt = true;
  } else h->useMatDt = false;
  if (h->particlesSet) resolveVerlet(h);
  fillStepParams(h);
  h->paramsSet = true;
  return WDEM_OK;
}

int wdem_upload_particles(wdem_handle* h, const wdem_particles* p) {
  if (!h || !p) return WDEM_ERR_ARG;
  if (p->n < 0 || p->n > h->N) return fail(h, WDEM_ERR_ARG, "particle count exceeds the handle capacity");
  if (!p->shape || !p->radius || !p->material || !p->mask || !p->flags || !p->mass || !p->inertia || !p->pos || !p->ori ||
      !p->vel || !p->angVel || !p->force || !p->torque)
    return fail(h, WDEM_ERR_ARG, "null particle array");
  const int n = p->n;
  h->n = n;
  h->shape.assign(p->shape, p->shape + n);
  h->mat.assign(p->material, p->material + n);
  h->radius.assign(p->radius, p->radius + n);
  h->smallIds.clear(); h->largeIds.clear();
  std::vector<double4_32a> posr(n), velm(n), angw(n), inert(n), ori(n), force(n), torque(n);
  std::vector<int4> meta(n);
  std::vector<double> semi(3 * (size_t)n, 0.0);
  bool anyEll = false;
  int nScenes = 1;
  std::vector<double4_32a> fv1, fv2;
  std::vector<int> facetIds;
  std::vector<int4> facetPairs;
  std::vector<int2> capMasks;  // (mask, scene) of every capsule
  for (int i = 0; i < n; i++) {
    int sh = p->shape[i];
    if (sh != WDEM_SHAPE_SPHERE && sh != WDEM_SHAPE_WALL && sh != WDEM_SHAPE_ELLIPSOID && sh != WDEM_SHAPE_FACET &&
        sh != WDEM_SHAPE_CAPSULE)
      return fail(h, WDEM_ERR_UNSUPPORTED, "unsupported shape of particle #" + std::to_string(i));
    if (sh == WDEM_SHAPE_CAPSULE) {
      if (!p->shaft) return fail(h, WDEM_ERR_ARG, "capsules need wdem_particles.shaft");
      // Capsule::selfTest (Capsule.cpp:19-23)
      if (!(p->radius[i] > 0.) || !(p->shaft[i] >= 0.))
        return fail(h, WDEM_ERR_ARG, "Capsule #" + std::to_string(i) + ": radius must be positive and shaft non-negative");
      if (h->periodic) return fail(h, WDEM_ERR_UNSUPPORTED, "capsules in a periodic cell are not supported");
      capMasks.push_back(make_int2((int)p->mask[i], p->scene ? p->scene[i] : 0));
    }
    if (sh == WDEM_SHAPE_FACET) {
      // fixed facets: nodes 1 and 2 are not integrated, so node 0 may not move either
      const std::string fid = "Facet #" + std::to_string(i);
      if (!p->facetVerts) return fail(h, WDEM_ERR_ARG, "facets need wdem_particles.facetVerts");
      if (h->periodic) return fail(h, WDEM_ERR_UNSUPPORTED, "facets in a periodic cell are not supported");
      if ((p->flags[i] & 63u) != 63u) return fail(h, WDEM_ERR_UNSUPPORTED, fid + ": facets must have all DOFs blocked");
      for (int k = 0; k < 3; k++)
        if (p->vel[3 * i + k] != 0 || p->angVel[3 * i + k] != 0)
          return fail(h, WDEM_ERR_UNSUPPORTED, fid + ": moving facets are not supported (velocity must be zero)");
      if (!(p->radius[i] >= 0) || !std::isfinite(p->radius[i])) return fail(h, WDEM_ERR_ARG, fid + ": bad halfThick");
      const double* v = p->facetVerts + 9 * (size_t)i;
      for (int k = 0; k < 9; k++)
        if (!std::isfinite(v[k])) return fail(h, WDEM_ERR_ARG, fid + ": non-finite node position");
      if (fv1.empty()) { fv1.assign(n, make_double4_32a(0, 0, 0, 0)); fv2.assign(n, make_double4_32a(0, 0, 0, 0)); }
      fv1[i] = make_double4_32a(v[3], v[4], v[5], 0);
      fv2[i] = make_double4_32a(v[6], v[7], v[8], 0);
      facetIds.push_back(i);
    }
    if (sh == WDEM_SHAPE_ELLIPSOID) {
      if (!p->semiAxes) return fail(h, WDEM_ERR_ARG, "ellipsoids need wdem_particles.semiAxes");
      const double* sa = p->semiAxes + 3 * i;
      if (!(sa[0] > 0 && sa[1] > 0 && sa[2] > 0))
        return fail(h, WDEM_ERR_ARG, "Ellipsoid #" + std::to_string(i) + ": all semi-axes must be positive");
      if (h->periodic) return fail(h, WDEM_ERR_UNSUPPORTED, "ellipsoids in a periodic cell are not supported");
    }
    if (sh == WDEM_SHAPE_WALL && h->periodic) return fail(h, WDEM_ERR_UNSUPPORTED, "walls in a periodic cell are not supported");
    if (p->material[i] < 0 || (h->paramsSet && p->material[i] >= (int)h->mats.size()))
      return fail(h, WDEM_ERR_ARG, "material index out of range for particle #" + std::to_string(i));
    const double* in = p->inertia + 3 * i;
    unsigned fl = p->flags[i];
    if (fl & (WDEM_CLUMP_CLUMP | WDEM_CLUMP_CLUMPED)) return fail(h, WDEM_ERR_UNSUPPORTED, "clumps are not supported");
    // DemData::useAsphericalLeapfrog: unequal inertia and a free rotational DOF (Particle.hpp:275-277)
    const bool asph = !(in[0] == in[1] && in[1] == in[2]) && (fl & 56u) != 56u;
    if (asph && h->periodic) return fail(h, WDEM_ERR_UNSUPPORTED, "aspherical nodes in a periodic cell are not supported");
    int ax = p->wallAxis ? p->wallAxis[i] : 0, sense = p->wallSense ? p->wallSense[i] : 0;
    if (sh == WDEM_SHAPE_WALL && (ax < 0 || ax > 2 || sense < -1 || sense > 1)) return fail(h, WDEM_ERR_ARG, "bad wall axis/sense");
    double r = (sh == WDEM_SHAPE_SPHERE || sh == WDEM_SHAPE_FACET) ? p->radius[i] : 0.0;  // facets: halfThick
    if (sh == WDEM_SHAPE_CAPSULE) r = p->radius[i] + .5 * p->shaft[i];                    // bounding radius
    if (sh == WDEM_SHAPE_ELLIPSOID) {
      // bounding radius: the largest semi-axis (FP32 cull and minDist00Sq of the ellipsoid functors)
      const double* sa = p->semiAxes + 3 * i;
      r = sa[0]; if (sa[1] > r) r = sa[1]; if (sa[2] > r) r = sa[2];
    }
    if (sh == WDEM_SHAPE_ELLIPSOID) { semi[3 * i] = p->semiAxes[3 * i]; semi[3 * i + 1] = p->semiAxes[3 * i + 1]; semi[3 * i + 2] = p->semiAxes[3 * i + 2]; }
    else if (sh == WDEM_SHAPE_SPHERE) { semi[3 * i] = semi[3 * i + 1] = semi[3 * i + 2] = r; }
    else if (sh == WDEM_SHAPE_CAPSULE) { semi[3 * i] = p->radius[i]; semi[3 * i + 1] = p->shaft[i]; semi[3 * i + 2] = 0; }
    anyEll |= (sh == WDEM_SHAPE_ELLIPSOID) || (sh == WDEM_SHAPE_CAPSULE) || asph;
    posr[i] = make_double4_32a(p->pos[3 * i], p->pos[3 * i + 1], p->pos[3 * i + 2], r);
    velm[i] = make_double4_32a(p->vel[3 * i], p->vel[3 * i + 1], p->vel[3 * i + 2], p->mass[i]);
    angw[i] = make_double4_32a(p->angVel[3 * i], p->angVel[3 * i + 1], p->angVel[3 * i + 2], 0);
    inert[i] = make_double4_32a(in[0], in[1], in[2], 0);
    ori[i] = make_double4_32a(p->ori[4 * i], p->ori[4 * i + 1], p->ori[4 * i + 2], p->ori[4 * i + 3]);
    force[i] = make_double4_32a(p->force[3 * i], p->force[3 * i + 1], p->force[3 * i + 2], 0);
    torque[i] = make_double4_32a(p->torque[3 * i], p->torque[3 * i + 1], p->torque[3 * i + 2], 0);
    auto posInert = [](double x) { return x > 0; };
    const bool ipos = posInert(in[0]) && posInert(in[1]) && posInert(in[2]);
    const int sc = p->scene ? p->scene[i] : 0;
    if (sc < 0 || sc >= MAX_SCENES) return fail(h, WDEM_ERR_ARG, "scene index out of range for particle #" + std::to_string(i));
    nScenes = std::max(nScenes, sc + 1);
    meta[i] = make_int4(sh | (ax << 4) | ((sense + 1) << 8) | (asph ? META_ASPH : 0) | (ipos ? META_IPOS : 0) |
                            (sc << META_SCENE_SHIFT),
                        p->material[i], (int)p->mask[i], (int)fl);
    // walls and facets go to the collider's list of large bodies, tested against every box of their scene
    if (sh != WDEM_SHAPE_WALL && sh != WDEM_SHAPE_FACET) h->smallIds.push_back(i); else h->largeIds.push_back(i);
  }
  if (nScenes > 1 && h->periodic) return fail(h, WDEM_ERR_UNSUPPORTED, "batched scenes in a periodic cell are not supported");
  // walls grouped by scene (stable: ids ascending within a scene); per-scene ranges
  std::vector<int> sceneWall(nScenes + 1, 0);
  if (nScenes > 1) {
    std::stable_sort(h->largeIds.begin(), h->largeIds.end(),
                     [&](int x, int y) { return (p->scene ? p->scene[x] : 0) < (p->scene ? p->scene[y] : 0); });
    for (int id : h->largeIds) sceneWall[(p->scene ? p->scene[id] : 0) + 1]++;
    for (int k = 0; k < nScenes; k++) sceneWall[k + 1] += sceneWall[k];
  }
  h->semi = semi;
  h->hasEll = anyEll;
  h->hasFacets = !facetIds.empty();
  for (int f : facetIds)
    for (int j : h->largeIds) {
      const unsigned mm = p->mask[f] & p->mask[j];
      if (j != f && mm != 0 && (p->scene ? p->scene[f] == p->scene[j] : true)) facetPairs.push_back(make_int4(f, j, (int)mm, 0));
    }
  // facet + capsule pairs (no Cg2_Facet_Capsule_L6Geom here) are refused like facet + wall: y = -1
  if (!facetIds.empty() && !capMasks.empty()) {
    std::sort(capMasks.begin(), capMasks.end(), [](int2 x, int2 y) { return x.x != y.x ? x.x < y.x : x.y < y.y; });
    capMasks.erase(std::unique(capMasks.begin(), capMasks.end(), [](int2 x, int2 y) { return x.x == y.x && x.y == y.y; }),
                   capMasks.end());
    for (int f : facetIds)
      for (const int2& cm : capMasks) {
        const unsigned mm = p->mask[f] & (unsigned)cm.x;
        if (mm != 0 && (p->scene ? p->scene[f] : 0) == cm.y) facetPairs.push_back(make_int4(f, -1, (int)mm, 0));
      }
  }
  h->facetPairs = facetPairs;
  h->facetsChecked = ~0u;
  h->matsChecked = -1;
  h->gravAccDirty = true;
  cudaSetDevice(h->device);
  cudaStream_t s = h->stream;
  if (n > 0) {
    CK(cudaMemcpyAsync(h->d.posr, posr.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.velm, velm.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.angw, angw.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.inert, inert.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.ori, ori.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.force, force.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.torque, torque.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.meta, meta.data(), n * sizeof(int4), cudaMemcpyHostToDevice, s));
  }
  if (h->hasEll) {
    // rotation state of ellipsoid / aspherical scenes
    if (!h->d.semi) {
      CK(dalloc(h->d.semi, h->N)); CK(dalloc(h->d.angMom, h->N)); CK(dalloc(h->d.lastOri, h->N)); CK(dalloc(h->d.maxRot, h->N));
    }
    std::vector<double4_32a> sv(n), am(n);
    const double nan = std::numeric_limits<double>::quiet_NaN();
    for (int i = 0; i < n; i++) {
      sv[i] = make_double4_32a(semi[3 * i], semi[3 * i + 1], semi[3 * i + 2], 0);
      if (p->angMom) am[i] = make_double4_32a(p->angMom[3 * i], p->angMom[3 * i + 1], p->angMom[3 * i + 2], 0);
      else am[i] = make_double4_32a(nan, nan, nan, 0);
    }
    if (n > 0) {
      CK(cudaMemcpyAsync(h->d.semi, sv.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(h->d.angMom, am.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    }
    CK(cudaStreamSynchronize(s));  // host vectors go out of scope
  }
  if (!facetIds.empty()) {
    if (!h->d.fv1) { CK(dalloc(h->d.fv1, h->N)); CK(dalloc(h->d.fv2, h->N)); }
    CK(cudaMemcpyAsync(h->d.fv1, fv1.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.fv2, fv2.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // host vectors go out of scope
  }
  if (!h->smallIds.empty())
    CK(cudaMemcpyAsync(h->dSmall, h->smallIds.data(), h->smallIds.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  if (!h->largeIds.empty())
    CK(cudaMemcpyAsync(h->cs.large, h->largeIds.data(), h->largeIds.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  h->cs.nLarge = (int)h->largeIds.size();
  cudaFree(h->cs.sceneWall);
  h->cs.sceneWall = nullptr;
  h->cs.nScenes = nScenes;
  if (nScenes > 1) {
    CK(dalloc(h->cs.sceneWall, (size_t)nScenes + 1));
    CK(cudaMemcpyAsync(h->cs.sceneWall, sceneWall.data(), (nScenes + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
  }
  launch_refresh_posf(s, h->d, n);
  if (n > 0) CK(cudaMemsetAsync(h->d.touched, 0, n, s));
  if (n > 0) CK(cudaMemsetAsync(h->d.rowMask, 0, n * sizeof(unsigned), s));
  CK(cudaStreamSynchronize(s));
  h->nContacts = 0;
  h->forcesInArrays = true;
  h->needRebuild = true;
  h->particlesSet = true;
  resolveVerlet(h);
  fillStepParams(h);
  return WDEM_OK;
}

int wdem_upload_contacts(wdem_handle* h, const wdem_contacts* c) {
  if (!h || !c) return WDEM_ERR_ARG;
  if (!h->particlesSet || !h->paramsSet) return fail(h, WDEM_ERR_STATE, "upload particles and params before contacts");
  const long long nc = c->n;
  if (nc < 0) return WDEM_ERR_ARG;
  if (h->contactLimit > 0 && nc > h->contactLimit)
    return fail(h, WDEM_ERR_OVERFLOW, "upload: " + std::to_string(nc) + " contacts exceed the limit of " +
                                          std::to_string(h->contactLimit) + " (wdem_set_contact_limit)");
  if (nc > 0 && (!c->idA || !c->idB || !c->real || !c->stepCreated)) return fail(h, WDEM_ERR_ARG, "null contact id/state array");
  cudaSetDevice(h->device);
  cudaStream_t s = h->stream;
  const bool hertz = (h->P.cp2 == WDEM_CP2_HERTZ);
  ContactBuf& b = h->buf[h->cur];
  if (nc > b.cap || b.hertz != hertz || b.geom != h->keepGeom || b.peri != h->periodic || b.ell != h->hasEll)
    CK(allocContacts(b, std::max<long long>(nc + 1024, 1024), hertz, h->keepGeom, h->periodic, h->hasEll));
  std::vector<int2> ids(nc);
  std::vector<uint8_t> state(nc);
  std::vector<int> step0(nc);
  std::vector<double> hist[HIST_FRICT], tanPhi(nc, 0.0);
  std::vector<int4> cdist(nc, make_int4(0, 0, 0, 0));
  for (int k = 0; k < HIST_FRICT; k++) hist[k].assign(nc, 0.0);
  for (long long i = 0; i < nc; i++) {
    int a = c->idA[i], bb = c->idB[i];
    if (a < 0 || a >= h->n || bb < 0 || bb >= h->n || a == bb) return fail(h, WDEM_ERR_ARG, "bad contact ids");
    bool swapped = false;
    if (pairSwaps(h->shape[a], h->shape[bb])) { std::swap(a, bb); swapped = true; }
    ids[i] = make_int2(a, bb);
    if (c->cellDist) {
      int sg = swapped ? -1 : 1;
      cdist[i] = make_int4(sg * c->cellDist[3 * i], sg * c->cellDist[3 * i + 1], sg * c->cellDist[3 * i + 2], 0);
    }
    bool real = c->real[i] != 0;
    state[i] = (uint8_t)((real ? CS_REAL : CS_POTENTIAL) | pairShapeBits(h->shape[a], h->shape[bb]));
    step0[i] = c->stepCreated[i];
    if (real) {
      if (!c->trsf || !c->contPt || !c->force || !c->kn || !c->kt || !c->tanPhi) return fail(h, WDEM_ERR_ARG, "real contact without history arrays");
      for (int k = 0; k < 3; k++) { hist[HIST_T0X + k][i] = c->trsf[9 * i + k]; hist[HIST_T1X + k][i] = c->trsf[9 * i + 3 + k]; }
      for (int k = 0; k < 3; k++) { hist[HIST_CX + k][i] = c->contPt[3 * i + k]; hist[HIST_FX + k][i] = c->force[3 * i + k]; }
      hist[HIST_KN][i] = c->kn[i]; hist[HIST_KT][i] = c->kt[i];
      tanPhi[i] = c->tanPhi[i];
    }
  }
  if (nc > 0) {
    CK(cudaMemcpyAsync(b.c.ids, ids.data(), nc * sizeof(int2), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.c.state, state.data(), nc, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.c.step0, step0.data(), nc * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.c.tanPhi, tanPhi.data(), nc * sizeof(double), cudaMemcpyHostToDevice, s));
    for (int k = 0; k < HIST_FRICT; k++) CK(cudaMemcpyAsync(b.c.hist[k], hist[k].data(), nc * sizeof(double), cudaMemcpyHostToDevice, s));
    if (b.c.cdist) CK(cudaMemcpyAsync(b.c.cdist, cdist.data(), nc * sizeof(int4), cudaMemcpyHostToDevice, s));
    // no solver history in the container: all-ones bytes are NaN, i.e. "cold start"
    if (b.c.lam) CK(cudaMemsetAsync(b.c.lam, 0xFF, nc * sizeof(double), s));
    if (b.c.lam0) CK(cudaMemsetAsync(b.c.lam0, 0xFF, nc * sizeof(float), s));
  }
  (h->raw.arith != WDEM_ARITH_EXACT ? contracted::launch_init_uploaded : launch_init_uploaded)(s, h->P, h->d, b.c, nc);
  int rc;
  // the uploaded container's CSR: the next rebuild carries the history of its contacts through it
  if ((rc = ensureScratch(h, nc))) return rc;
  if ((rc = ensureCsr(h, nc))) return rc;
  col_csr(s, b.c, nc, h->n, h->csr, h->cs);
  CK(cudaStreamSynchronize(s));
  h->nContacts = nc;
  h->needRebuild = true;
  return WDEM_OK;
}

// Steps queued without a host check in between.  Every step of Woo's loop ends its integrator with the
// collider trigger (Collision.cpp:80-184), and the contact pass must not start before a triggered rebuild;
// checking on the host costs a device round trip per step.  Instead `ahead` steps are queued at once and
// their kernels guard themselves (haltedIntegrator / haltedContacts): when the integrator of step k raises
// the trigger, the contact pass of k and all later queued kernels return at once.  The host then sees
// haltAt, rebuilds and runs the contact pass of step k, exactly the sequence of the one-step path.  Only
// the configurations whose host-side per-step work is none are queued: no periodic cell (integrated on
// the host each step), no energy tracking (host-launched reductions), no updatePhys='once', no phase
// timing.
// pown (src/supp/base/Math.hpp:166-175): x^n by squaring, x^n = (x^2)^(n/2) x^(n%2)
static double powUint(double x, unsigned n) {
  const unsigned d = n >> 1, r = n & 1;
  const double x2d = d == 0 ? 1 : powUint(x * x, d);
  const double xr = r == 0 ? 1 : x;
  return x2d * xr;
}

// PeriodicEngine::isActivated for a step period with stepModulo (Engine.cpp:170-196), from the second
// call on (the first call only records stepLast, see wdem_step)
static bool dynDtDue(const wdem_handle* h, long long s) {
  const long long per = h->raw.dynDtPeriod;
  return per > 0 && ((s - h->dynStepLast >= per) || (s % per == 0));
}
// the first step >= s at which DynDt runs
static long long dynDtNext(const wdem_handle* h, long long s) {
  const long long per = h->raw.dynDtPeriod;
  if (per <= 0) return std::numeric_limits<long long>::max();
  const long long mult = (s + per - 1) / per * per;
  return std::min(mult, std::max(s, h->dynStepLast + per));
}
// DynDt::run (DynDt.cpp:86-113) after the contact pass of step s, when due
static int dynDtAfterContacts(wdem_handle* h, long long s) {
  if (!dynDtDue(h, s)) return WDEM_OK;
  h->dynStepPrev = h->dynStepLast;
  h->dynStepLast = s;
  cudaStream_t st = h->stream;
  CK(cudaMemsetAsync(&h->dst->dynNotMin, 0, sizeof(unsigned long long), st));
  launch_dyndt(st, h->P, h->d, h->n, h->buf[h->cur].c, h->csr, h->dst);
  unsigned long long v = 0;
  CK(cudaMemcpyAsync(h->hcounts + 2, &h->dst->dynNotMin, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::memcpy(&v, h->hcounts + 2, sizeof v);
  double sq = std::numeric_limits<double>::infinity();
  if (v != 0) { const unsigned long long b = ~v; std::memcpy(&sq, &b, sizeof sq); }
  const double crDt = std::sqrt(sq);  // DynDt::critDt_stiffness
  h->dynDtCrit = crDt;
  if (std::isinf(crDt)) return WDEM_OK;  // no timestep computed, keep the current one
  const long long nSteps = s - h->dynStepPrev;
  const double dt = h->raw.dt;
  const double maxNewDt = dt * powUint(1. + h->raw.dynDtMaxRelInc, (unsigned)nSteps);
  const double nextDt = std::min(crDt * h->raw.dtSafety, maxNewDt);
  if (nextDt != dt) h->nextDt = nextDt;
  return WDEM_OK;
}
// Scene::doOneStep epilogue (Scene.cpp:432): a new dt from DynDt takes effect for the next step
static void applyNextDt(wdem_handle* h) {
  if (std::isnan(h->nextDt)) return;
  h->raw.dt = h->nextDt;
  h->P.dt = h->nextDt;
  h->nextDt = std::numeric_limits<double>::quiet_NaN();
}

// steps may run queued (no host-side per-step work, queue depth not set to 1)
static bool queueEligible(const wdem_handle* h) {
  return !(h->timing || h->periodic || h->P.trackEnergy || h->needRebuild || h->forcesInArrays ||
           h->verletDistResolved == 0 || h->updatePhys == WDEM_UPDATE_PHYS_ONCE || h->maxAhead < 2);
}

static int queueDepth(wdem_handle* h, int left) {
  if (left < 2 || !queueEligible(h)) return 1;
  // expected steps between rebuilds r: a queue of sqrt(3 r) balances the wasted no-op launches behind a
  // trigger against the round trips saved
  int q = (int)std::lround(std::sqrt(3.0 * h->rebuildInterval));
  q = std::max(2, std::min(q, h->maxAhead));
  q = std::min(q, left);
  // DynDt runs on the host side of its step: the queue ends there
  const long long toDyn = dynDtNext(h, h->step) - h->step + 1;
  if (toDyn < q) q = (int)std::max<long long>(1, toDyn);
  return q;
}

// The kernels of `ahead` queued steps (integrator, then contact pass), with the step numbers of P.step and
// P.seq (absolute, or offsets when P.stepDev); the first contact pass culls the whole container if full.
static void launchQueue(wdem_handle* h, StepParams P, int ahead, bool full, bool warm) {
  cudaStream_t s = h->stream;
  const long long step0 = P.step, seq0 = P.seq;
  for (int g = 0; g < ahead; g++) {
    P.step = step0 + g;
    P.seq = seq0 + 1 + g;
    (h->raw.arith != WDEM_ARITH_EXACT ? contracted::launch_leapfrog : launch_leapfrog)(s, P, h->d, h->n, 0, h->buf[h->cur].c, h->csr, h->dst);
    (h->raw.arith != WDEM_ARITH_EXACT ? contracted::launch_contacts : launch_contacts)(s, P, h->d, h->buf[h->cur].c, h->nContacts, h->dst, g == 0 && full,
                    warm ? h->mlpWbf : nullptr, warm ? h->mlpW : nullptr);
  }
}

// The queue as one CUDA graph launch.  The graph is captured with P.stepDev (steps numbered from the
// replay's bases) and kept with the bytes of every launch argument it holds: parameters, particle, contact
// and CSR arrays, counts, status word and network weights.  A replay whose arguments differ (after a
// rebuild, an upload, new parameters or a regrown array) captures again; with graphMode AUTO a capture is
// made only when at least eight replays are expected before the next rebuild (a capture and instantiation
// cost several times the host time of the launches it replaces).  Returns 1 if the queue was
// launched, 0 if the caller launches it kernel by kernel, or a negative error code.
static int replayQueue(wdem_handle* h, int ahead, bool full, bool warm) {
  if (h->graphMode == WDEM_GRAPHS_OFF) return 0;
  cudaStream_t s = h->stream;
  StepParams P = h->P;
  P.stepDev = 1;
  P.step = 0;
  P.seq = 0;
  std::vector<unsigned char> sig;
  auto put = [&sig](const void* x, size_t nb) {
    const unsigned char* b = (const unsigned char*)x;
    sig.insert(sig.end(), b, b + nb);
  };
  const int n = h->n, arith = h->raw.arith;
  const void* wp[2] = {warm ? (const void*)h->mlpWbf : nullptr, warm ? (const void*)h->mlpW : nullptr};
  put(&P, sizeof P); put(&h->d, sizeof h->d); put(&h->buf[h->cur].c, sizeof(Contacts)); put(&h->csr, sizeof h->csr);
  put(&h->nContacts, sizeof h->nContacts); put(&n, sizeof n); put(&arith, sizeof arith); put(&h->dst, sizeof h->dst);
  put(wp, sizeof wp);
  const int key = 2 * ahead + (full ? 1 : 0);
  auto it = h->graphs.find(key);
  const bool valid = it != h->graphs.end() && it->second.exec && it->second.sig == sig;
  if (!valid && h->graphMode == WDEM_GRAPHS_AUTO && h->rebuildInterval < 8.0 * ahead) return 0;
  wdem_handle::StepGraph& g = h->graphs[key];
  if (!valid) {
    const long long k0 = ::wdem::g_kernel_launches;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    launchQueue(h, P, ahead, full, warm);
    const cudaError_t e = cudaStreamEndCapture(s, &graph);
    const long long kernels = ::wdem::g_kernel_launches - k0;
    ::wdem::g_kernel_launches = k0;  // captured, not launched
    if (e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return fail(h, WDEM_ERR_CUDA, std::string("capturing the queued steps: ") + cudaGetErrorString(e));
    }
    if (g.exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(g.exec, graph, &info) != cudaSuccess) {
        cudaGetLastError();  // a topology change: instantiate anew
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
      }
    }
    cudaError_t ie = cudaSuccess;
    if (!g.exec) ie = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
      g.exec = nullptr;
      return fail(h, WDEM_ERR_CUDA, std::string("instantiating the queued steps: ") + cudaGetErrorString(ie));
    }
    g.sig.swap(sig);
    g.kernels = kernels;
    h->graphCaptures++;
  }
  // the replay's step numbers: stepBase + g and seqBase + 1 + g for its g-th step
  h->hst->stepBase = h->step;
  h->hst->seqBase = h->seq;
  CK(cudaMemcpyAsync(&h->dst->stepBase, &h->hst->stepBase, 2 * sizeof(long long), cudaMemcpyHostToDevice, s));
  CK(cudaGraphLaunch(g.exec, s));
  ::wdem::g_kernel_launches += g.kernels;
  h->graphReplays++;
  return 1;
}

// Runs up to `ahead` queued steps; `statusCurrent` tells whether the host's status word is still the
// device's (no kernel that may raise an error ran after it was read back).
static int runQueued(wdem_handle* h, int ahead, int& done, bool& statusCurrent) {
  cudaStream_t s = h->stream;
  const long long s0 = h->step;
  h->P.updatePhysNow = (h->updatePhys != WDEM_UPDATE_PHYS_NEVER);
  const bool warm = h->hasEll && h->P.ellSolver == WDEM_ELL_NEWTON && (h->P.warmStart == WDEM_WARM_MLP || h->P.warmStart == WDEM_WARM_HISTORY_MLP);
  const long long q0 = h->seq;
  const bool full = !h->actValid;
  h->P.denseTouch = h->denseTouch ? 1 : 0;
  const int viaGraph = replayQueue(h, ahead, full, warm);
  if (viaGraph < 0) return viaGraph;
  if (viaGraph == 0) {
    StepParams P = h->P;
    P.step = s0;
    P.seq = q0;
    launchQueue(h, P, ahead, full, warm);
  }
  h->actValid = true;
  CK(cudaMemcpyAsync(h->hst, h->dst, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int rc;
  if ((rc = checkDeviceStatus(h))) return rc;
  const long long halt = h->hst->haltAt;
  statusCurrent = (halt == 0);
  if (halt == 0) {
    // a halted queue's last contact pass did not run (its count is zero): the choice stays
    h->denseTouch = 8ull * h->hst->workCount >= (unsigned long long)h->n;
    h->sinceRebuild += ahead;
    done = ahead;
    h->lastRunFull = 0;
  } else {
    const long long k = halt - 1;  // steps s0 .. k-1 are complete, step k has been integrated
    if (k < s0 || k >= s0 + ahead) return fail(h, WDEM_ERR_STATE, "queued steps: trigger outside the queue");
    h->step = k;
    h->P.step = k;
    h->P.seq = q0 + 1 + (k - s0);
    h->raw.step = k;
    CK(cudaMemsetAsync(&h->dst->dirty, 0, sizeof(int), s));
    CK(cudaMemsetAsync(&h->dst->haltAt, 0, sizeof(long long), s));
    if ((rc = rebuild(h))) return rc;
    (h->raw.arith != WDEM_ARITH_EXACT ? contracted::launch_contacts : launch_contacts)(s, h->P, h->d, h->buf[h->cur].c, h->nContacts, h->dst, !h->actValid, warm ? h->mlpWbf : nullptr,
                    warm ? h->mlpW : nullptr);
    h->actValid = true;
    h->sinceRebuild += (int)(k - s0) + 1;
    h->rebuildInterval = 0.75 * h->rebuildInterval + 0.25 * h->sinceRebuild;
    h->sinceRebuild = 0;
    done = (int)(k - s0) + 1;
    h->lastRunFull = 1;
  }
  // the queue ends at or before the next DynDt step: run it if the last completed step is due
  if ((rc = dynDtAfterContacts(h, s0 + done - 1))) return rc;
  h->seq = q0 + done;
  h->step = s0 + done;
  h->P.step = h->step;
  h->raw.step = h->step;
  for (int k = 0; k < done; k++) h->timeSum += h->raw.dt;  // Scene.time += dt per step
  applyNextDt(h);
  return WDEM_OK;
}

int wdem_step(wdem_handle* h, int32_t nSteps) {
  if (!h || nSteps < 0) return WDEM_ERR_ARG;
  if (!h->particlesSet || !h->paramsSet) return fail(h, WDEM_ERR_STATE, "wdem_step before particles and params were set");
  if (h->matsChecked != (long long)h->mats.size()) {
    // material indices against the current table (once per table size: uploads re-check their own)
    for (int i = 0; i < h->n; i++)
      if (h->mat[i] < 0 || h->mat[i] >= (int)h->mats.size())
        return fail(h, WDEM_ERR_ARG, "material index out of range for particle #" + std::to_string(i));
    h->matsChecked = (long long)h->mats.size();
  }
  if (h->hasEll && (h->P.law != WDEM_LAW_IDEALELPL || h->P.cp2 != WDEM_CP2_FRICT))
    return fail(h, WDEM_ERR_UNSUPPORTED,
                "ellipsoids and aspherical nodes run with Cp2_FrictMat_FrictPhys + Law2_L6Geom_FrictPhys_IdealElPl only");
  if (!h->facetPairs.empty() && h->facetsChecked != h->P.loneMask) {
    // Cg2_Facet_Facet_L6Geom and Cg2_Wall_Facet_L6Geom are not implemented: such pairs must be excluded by
    // the masks (Collider::mayCollide), as DemField.defaultBoundaryMask with DemField.loneMask does
    for (const int4& q : h->facetPairs)
      if (((unsigned)q.z & h->P.loneMask) == 0) {
        if (q.y < 0)
          return fail(h, WDEM_ERR_UNSUPPORTED, "Facet #" + std::to_string(q.x) +
                                                   " may collide with capsules: facet-capsule contacts are not implemented");
        return fail(h, WDEM_ERR_UNSUPPORTED, "Facet #" + std::to_string(q.x) + " may collide with " +
                                                 (h->shape[q.y] == WDEM_SHAPE_WALL ? "Wall #" : "Facet #") + std::to_string(q.y) +
                                                 ": facet-facet and wall-facet contacts are not implemented (give the "
                                                 "boundaries a common loneMask bit)");
      }
    h->facetsChecked = h->P.loneMask;
  }
  if (h->device >= 0 && h->device < 64 && g_matsOwner[h->device] != h) {
    cudaSetDevice(h->device);
    uploadMaterials(h);  // another handle of this process uploaded its table since
  }
  if (h->hasEll && h->P.ellSolver != WDEM_ELL_BRENT && h->P.ellSolver != WDEM_ELL_NEWTON)
    return fail(h, WDEM_ERR_ARG, "unknown ellipsoid solver");
  if (h->hasEll && h->P.ellSolver == WDEM_ELL_NEWTON && !(h->P.newtonTol > 0))
    return fail(h, WDEM_ERR_ARG, "newtonTol must be positive");
  if (h->hasEll && h->P.ellSolver == WDEM_ELL_NEWTON && (h->P.warmStart == WDEM_WARM_MLP || h->P.warmStart == WDEM_WARM_HISTORY_MLP) && !h->mlpReady)
    return fail(h, WDEM_ERR_STATE, "warmStart=MLP needs a network (wdem_warm_init / wdem_warm_set_weights / wdem_warm_train)");
  if (h->raw.dynDtPeriod > 0 && (h->hasEll || h->raw.materialDt))
    return fail(h, WDEM_ERR_UNSUPPORTED, "DynDt runs with sphere and wall scenes of one dt only");
  if (h->raw.dynDtPeriod > 0 && !(1. + h->raw.dynDtMaxRelInc != 1.))
    return fail(h, WDEM_ERR_ARG, "DynDt: maxRelInc too small (1.0+maxRelInc==1.0)");
  // PeriodicEngine::isActivated, first call: counting starts at this step
  if (h->raw.dynDtPeriod > 0 && h->dynStepLast < 0) h->dynStepLast = h->step;
  cudaSetDevice(h->device);
  cudaStream_t s = h->stream;
  for (int k = 0; k < 3; k++) { h->phaseMs[k] = 0; h->phaseLaunches[k] = 0; }
  h->evMarks.clear(); h->evUsed = 0;
  if (h->gravAccDirty) {
    launch_grav_acc(s, h->P, h->d, h->n);
    h->gravAccDirty = false;
  }
  // the integrator's rotation-list counter starts every call at zero (within a call the contact pass
  // clears it for the next step)
  CK(cudaMemsetAsync(&h->dst->rotCount, 0, sizeof(unsigned), s));
  CK(cudaMemsetAsync(&h->dst->touchCount, 0, sizeof(unsigned), s));
  // true while the status word on the host is the one the last queue read back (nothing launched since)
  bool statusRead = false;
  for (int it = 0; it < nSteps; it++) {
    const int ahead = queueDepth(h, nSteps - it);
    if (queueEligible(h)) {
      // also a single step: the integrator and the guarded contact pass go out together and the host reads
      // the status once (a trigger halts the contact pass on the device; the host then rebuilds and runs it),
      // one round trip per call instead of a check between the two kernels and another at the end
      int done = 0, rc;
      if ((rc = runQueued(h, ahead, done, statusRead))) return rc;
      it += done - 1;
      continue;
    }
    statusRead = false;
    h->P.step = h->step;
    h->P.seq = ++h->seq;
    h->P.updatePhysNow = (h->updatePhys != WDEM_UPDATE_PHYS_NEVER);
    if (h->periodic) {
      // Scene::doOneStep prologue: cell->integrateAndUpdate(dt) (Scene.cpp:411)
      if (!h->cell.integrateAndUpdate(h->P.dt)) return fail(h, WDEM_ERR_STATE, "Cell is degenerate (zero volume).");
      fillCellParams(h);
      // Leapfrog's reallyTrackEnergy (Leapfrog.cpp:132): no energy in step 0 with a non-zero gradient
      bool gradVI = true;
      for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) gradVI &= (h->cell.gradV.r[i][k] == (i == k ? 1.0 : 0.0));
      h->P.lfEnergy = h->raw.trackEnergy && (h->step > 0 || gradVI);
    }
    {
      PhaseTimer t(h, PH_LEAPFROG);
      (h->raw.arith != WDEM_ARITH_EXACT ? contracted::launch_leapfrog : launch_leapfrog)(s, h->P, h->d, h->n, h->forcesInArrays ? 1 : 0, h->buf[h->cur].c, h->csr, h->dst);
    }
    if (h->P.trackEnergy && !h->P.lfEnergy) {
      // kinetic is resettable (EnergyTracker::resetResettables at the start of the step)
      CK(cudaMemsetAsync(h->dEnergy + WDEM_E_KINETIC, 0, sizeof(double), s));
    }
    if (h->P.lfEnergy) {
      int rc0;
      if ((rc0 = ensurePartials(h, std::max<long long>(h->n, h->nContacts)))) return rc0;
      energy_accumulate(s, h->d.energy[EP_GRAV], h->n, h->ePartials, h->dEnergy + WDEM_E_GRAV, false);
      energy_accumulate(s, h->d.energy[EP_DAMP], h->n, h->ePartials, h->dEnergy + WDEM_E_NONVISCDAMP, false);
      energy_accumulate(s, h->d.energy[EP_KIN], h->n, h->ePartials, h->dEnergy + WDEM_E_KINETIC, true);
    }
    h->forcesInArrays = false;
    CK(cudaMemcpyAsync(h->hst, h->dst, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    int rc;
    if ((rc = checkDeviceStatus(h))) return rc;
    bool full = h->needRebuild || h->hst->dirty || h->verletDistResolved == 0;
    h->lastRunFull = full;
    h->sinceRebuild++;
    if (full) {
      h->rebuildInterval = 0.75 * h->rebuildInterval + 0.25 * h->sinceRebuild;
      h->sinceRebuild = 0;
    }
    if (full) {
      CK(cudaMemsetAsync(&h->dst->dirty, 0, sizeof(int), s));
      CK(cudaMemsetAsync(&h->dst->haltAt, 0, sizeof(long long), s));
      PhaseTimer t(h, PH_COLLIDER);
      if ((rc = rebuild(h))) return rc;
    }
    if (h->P.trackEnergy && h->nContacts > 0) {
      for (int k = 0; k < EC_COUNT; k++)
        CK(cudaMemsetAsync(h->buf[h->cur].c.energy[k], 0, sizeof(double) * h->nContacts, s));
    }
    {
      PhaseTimer t(h, PH_CONTACTS);
      const bool warm = h->hasEll && h->P.ellSolver == WDEM_ELL_NEWTON && (h->P.warmStart == WDEM_WARM_MLP || h->P.warmStart == WDEM_WARM_HISTORY_MLP);
      (h->raw.arith != WDEM_ARITH_EXACT ? contracted::launch_contacts : launch_contacts)(s, h->P, h->d, h->buf[h->cur].c, h->nContacts, h->dst, !h->actValid, warm ? h->mlpWbf : nullptr,
                      warm ? h->mlpW : nullptr);
      h->actValid = true;
    }
    if (h->P.trackEnergy) {
      int rc0;
      if ((rc0 = ensurePartials(h, std::max<long long>(h->n, h->nContacts)))) return rc0;
      const Contacts& cc = h->buf[h->cur].c;
      const long long nc = h->nContacts;
      energy_accumulate(s, cc.energy[EC_ELAST], nc, h->ePartials, h->dEnergy + WDEM_E_ELAST, true);
      energy_accumulate(s, cc.energy[EC_PLAST], nc, h->ePartials, h->dEnergy + WDEM_E_PLAST, false);
      energy_accumulate(s, cc.energy[EC_VISCN], nc, h->ePartials, h->dEnergy + WDEM_E_VISCN, false);
      energy_accumulate(s, cc.energy[EC_VISCT], nc, h->ePartials, h->dEnergy + WDEM_E_VISCT, false);
      energy_accumulate(s, cc.energy[EC_BROKEN], nc, h->ePartials, h->dEnergy + WDEM_E_BROKEN, false);
    }
    if (h->updatePhys == WDEM_UPDATE_PHYS_ONCE) { h->updatePhys = WDEM_UPDATE_PHYS_NEVER; h->raw.updatePhys = WDEM_UPDATE_PHYS_NEVER; }
    if ((rc = dynDtAfterContacts(h, h->step))) return rc;  // DynDt, the engine after ContactLoop
    if (h->periodic) h->cell.setNextGradV();  // epilogue (Scene.cpp:430)
    h->step++;
    h->P.step = h->step;
    h->raw.step = h->step;
    h->timeSum += h->raw.dt;
    applyNextDt(h);
  }
  if (!statusRead) {
    CK(cudaMemcpyAsync(h->hst, h->dst, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  collectTimes(h);
  CK(cudaGetLastError());
  return checkDeviceStatus(h);
}

int wdem_download_particles(wdem_handle* h, wdem_particles* p) {
  if (!h || !p) return WDEM_ERR_ARG;
  cudaSetDevice(h->device);
  cudaStream_t s = h->stream;
  const int n = std::min(h->n, p->n);
  if (!h->forcesInArrays) {
    StepParams P = h->P;
    P.seq = h->seq + 1;  // the records of the last contact pass
    launch_reduce_forces(s, P, h->d, h->n, h->buf[h->cur].c, h->csr);
  }
  std::vector<double4_32a> posr(n), velm(n), angw(n), ori(n), force(n), torque(n);
  if (n > 0) {
    CK(cudaMemcpyAsync(posr.data(), h->d.posr, n * sizeof(double4_32a), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(velm.data(), h->d.velm, n * sizeof(double4_32a), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(angw.data(), h->d.angw, n * sizeof(double4_32a), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ori.data(), h->d.ori, n * sizeof(double4_32a), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(force.data(), h->d.force, n * sizeof(double4_32a), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(torque.data(), h->d.torque, n * sizeof(double4_32a), cudaMemcpyDeviceToHost, s));
  }
  std::vector<double4_32a> am;
  if (h->hasEll && p->angMom && n > 0) {
    am.resize(n);
    CK(cudaMemcpyAsync(am.data(), h->d.angMom, n * sizeof(double4_32a), cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  for (int i = 0; i < n; i++) {
    if (!am.empty()) { p->angMom[3 * i] = am[i].x; p->angMom[3 * i + 1] = am[i].y; p->angMom[3 * i + 2] = am[i].z; }
    if (p->pos) { p->pos[3 * i] = posr[i].x; p->pos[3 * i + 1] = posr[i].y; p->pos[3 * i + 2] = posr[i].z; }
    if (p->vel) { p->vel[3 * i] = velm[i].x; p->vel[3 * i + 1] = velm[i].y; p->vel[3 * i + 2] = velm[i].z; }
    if (p->angVel) { p->angVel[3 * i] = angw[i].x; p->angVel[3 * i + 1] = angw[i].y; p->angVel[3 * i + 2] = angw[i].z; }
    if (p->ori) { p->ori[4 * i] = ori[i].x; p->ori[4 * i + 1] = ori[i].y; p->ori[4 * i + 2] = ori[i].z; p->ori[4 * i + 3] = ori[i].w; }
    if (p->force) { p->force[3 * i] = force[i].x; p->force[3 * i + 1] = force[i].y; p->force[3 * i + 2] = force[i].z; }
    if (p->torque) { p->torque[3 * i] = torque[i].x; p->torque[3 * i + 1] = torque[i].y; p->torque[3 * i + 2] = torque[i].z; }
  }
  return WDEM_OK;
}

namespace {
struct HostContacts {
  std::vector<int2> ids;
  std::vector<uint8_t> state;
  std::vector<int> step0;
  std::vector<double> hist[HIST_COUNT], tanPhi, geom[7];
  std::vector<int4> cdist;
};
int fetchContacts(wdem_handle* h, HostContacts& hc) {
  cudaStream_t s = h->stream;
  const long long nc = h->nContacts;
  const ContactBuf& b = h->buf[h->cur];
  hc.ids.resize(nc); hc.state.resize(nc); hc.step0.resize(nc); hc.tanPhi.resize(nc);
  if (nc > 0) {
    CK(cudaMemcpyAsync(hc.ids.data(), b.c.ids, nc * sizeof(int2), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hc.state.data(), b.c.state, nc, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hc.step0.data(), b.c.step0, nc * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hc.tanPhi.data(), b.c.tanPhi, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
    int nh = b.hertz ? (int)HIST_COUNT : (int)HIST_FRICT;
    for (int k = 0; k < nh; k++) {
      hc.hist[k].resize(nc);
      CK(cudaMemcpyAsync(hc.hist[k].data(), b.c.hist[k], nc * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    if (b.c.cdist) {
      hc.cdist.resize(nc);
      CK(cudaMemcpyAsync(hc.cdist.data(), b.c.cdist, nc * sizeof(int4), cudaMemcpyDeviceToHost, s));
    }
    if (b.geom)
      for (int k = 0; k < 7; k++) {
        hc.geom[k].resize(nc);
        CK(cudaMemcpyAsync(hc.geom[k].data(), b.c.geom[k], nc * sizeof(double), cudaMemcpyDeviceToHost, s));
      }
  }
  CK(cudaStreamSynchronize(s));
  return WDEM_OK;
}
// rotation matrix columns -> quaternion (same method as the device code)
void quatFromColsHost(const double* c0, const double* c1, const double* c2, double* q) {
  double m[3][3] = {{c0[0], c1[0], c2[0]}, {c0[1], c1[1], c2[1]}, {c0[2], c1[2], c2[2]}};
  double t = m[0][0] + m[1][1] + m[2][2];
  double w, v[3];
  if (t > 0) {
    t = std::sqrt(t + 1.0);
    w = 0.5 * t;
    t = 0.5 / t;
    v[0] = (m[2][1] - m[1][2]) * t;
    v[1] = (m[0][2] - m[2][0]) * t;
    v[2] = (m[1][0] - m[0][1]) * t;
  } else {
    int i = 0;
    if (m[1][1] > m[0][0]) i = 1;
    if (m[2][2] > m[i][i]) i = 2;
    int j = (i + 1) % 3, k = (j + 1) % 3;
    t = std::sqrt(m[i][i] - m[j][j] - m[k][k] + 1.0);
    v[i] = 0.5 * t;
    t = 0.5 / t;
    w = (m[k][j] - m[j][k]) * t;
    v[j] = (m[j][i] + m[i][j]) * t;
    v[k] = (m[k][i] + m[i][k]) * t;
  }
  q[0] = w; q[1] = v[0]; q[2] = v[1]; q[3] = v[2];
}
}  // namespace

int wdem_contact_count(wdem_handle* h, int64_t* n) {
  if (!h || !n) return WDEM_ERR_ARG;
  cudaSetDevice(h->device);
  std::vector<uint8_t> st(h->nContacts);
  if (h->nContacts > 0) {
    CK(cudaMemcpy(st.data(), h->buf[h->cur].c.state, h->nContacts, cudaMemcpyDeviceToHost));
  }
  long long k = 0;
  for (auto v : st) if ((v & CS_MASK) != CS_DEAD) k++;
  *n = k;
  return WDEM_OK;
}

int wdem_download_contacts(wdem_handle* h, wdem_contacts* c) {
  if (!h || !c) return WDEM_ERR_ARG;
  cudaSetDevice(h->device);
  HostContacts hc;
  int rc;
  if ((rc = fetchContacts(h, hc))) return rc;
  std::vector<long long> order;
  for (long long i = 0; i < (long long)hc.ids.size(); i++) if ((hc.state[i] & CS_MASK) != CS_DEAD) order.push_back(i);
  auto key = [&](long long i) {
    unsigned a = (unsigned)std::min(hc.ids[i].x, hc.ids[i].y), b = (unsigned)std::max(hc.ids[i].x, hc.ids[i].y);
    return ((unsigned long long)a << 32) | b;
  };
  std::sort(order.begin(), order.end(), [&](long long x, long long y) { return key(x) < key(y); });
  const bool hertz = h->buf[h->cur].hertz;
  const double nan = std::numeric_limits<double>::quiet_NaN();
  for (long long o = 0; o < (long long)order.size() && o < c->n; o++) {
    long long i = order[o];
    bool real = (hc.state[i] & CS_MASK) == CS_REAL;
    int a = hc.ids[i].x, b = hc.ids[i].y;
    if (c->idA) c->idA[o] = a;
    if (c->idB) c->idB[o] = b;
    if (c->cellDist) {
      int4 d = hc.cdist.empty() ? make_int4(0, 0, 0, 0) : hc.cdist[i];
      c->cellDist[3 * o] = d.x; c->cellDist[3 * o + 1] = d.y; c->cellDist[3 * o + 2] = d.z;
    }
    if (c->real) c->real[o] = real ? 1 : 0;
    if (c->stepCreated) c->stepCreated[o] = hc.step0[i];
    if (c->minDist00Sq) {
      bool ss = h->shape[a] == WDEM_SHAPE_SPHERE && h->shape[b] == WDEM_SHAPE_SPHERE;
      double t = std::abs(h->raw.distFactor * (h->radius[a] + h->radius[b]));
      c->minDist00Sq[o] = ss ? t * t : -1;
    }
    double c0[3], c1[3], c2[3];
    if (real) {
      for (int k = 0; k < 3; k++) { c0[k] = hc.hist[HIST_T0X + k][i]; c1[k] = hc.hist[HIST_T1X + k][i]; }
      c2[0] = c0[1] * c1[2] - c0[2] * c1[1];
      c2[1] = c0[2] * c1[0] - c0[0] * c1[2];
      c2[2] = c0[0] * c1[1] - c0[1] * c1[0];
    } else {
      c0[0] = 1; c0[1] = 0; c0[2] = 0; c1[0] = 0; c1[1] = 1; c1[2] = 0; c2[0] = 0; c2[1] = 0; c2[2] = 1;
    }
    if (c->trsf) for (int k = 0; k < 3; k++) { c->trsf[9 * o + k] = c0[k]; c->trsf[9 * o + 3 + k] = c1[k]; c->trsf[9 * o + 6 + k] = c2[k]; }
    if (c->geomOri) {
      if (real) quatFromColsHost(c0, c1, c2, c->geomOri + 4 * o);
      else { c->geomOri[4 * o] = 1; c->geomOri[4 * o + 1] = 0; c->geomOri[4 * o + 2] = 0; c->geomOri[4 * o + 3] = 0; }
    }
    if (c->contPt) for (int k = 0; k < 3; k++) c->contPt[3 * o + k] = real ? hc.hist[HIST_CX + k][i] : 0.0;
    if (c->force) for (int k = 0; k < 3; k++) c->force[3 * o + k] = real ? hc.hist[HIST_FX + k][i] : 0.0;
    if (c->torque) for (int k = 0; k < 3; k++) c->torque[3 * o + k] = 0.0;
    if (c->kn) c->kn[o] = real ? hc.hist[HIST_KN][i] : nan;
    if (c->kt) c->kt[o] = real ? hc.hist[HIST_KT][i] : nan;
    if (c->tanPhi) c->tanPhi[o] = real ? hc.tanPhi[i] : nan;
    bool g = !hc.geom[0].empty();
    if (c->uN) c->uN[o] = (real && g) ? hc.geom[0][i] : nan;
    if (c->geomVel) for (int k = 0; k < 3; k++) c->geomVel[3 * o + k] = (real && g) ? hc.geom[1 + k][i] : (real ? nan : 0.0);
    if (c->geomAngVel) for (int k = 0; k < 3; k++) c->geomAngVel[3 * o + k] = (real && g) ? hc.geom[4 + k][i] : (real ? nan : 0.0);
    (void)hertz;
  }
  return WDEM_OK;
}

int wdem_crit_dt(wdem_handle* h, double* dt) {
  if (!h || !dt) return WDEM_ERR_ARG;
  double r = std::numeric_limits<double>::infinity();
  for (int i = 0; i < h->n; i++) {
    double radius;
    if (h->shape[i] == WDEM_SHAPE_SPHERE || h->shape[i] == WDEM_SHAPE_CAPSULE) radius = h->radius[i];
    else if (h->shape[i] == WDEM_SHAPE_ELLIPSOID) {
      const double* sa = &h->semi[3 * i];
      radius = sa[0]; if (sa[1] < radius) radius = sa[1]; if (sa[2] < radius) radius = sa[2];
    } else continue;
    if (h->mat[i] < 0 || h->mat[i] >= (int)h->mats.size()) return fail(h, WDEM_ERR_STATE, "materials not set");
    const wdem_material& m = h->mats[h->mat[i]];
    r = std::min(r, radius / (1. * std::sqrt(m.young / m.density)));
  }
  *dt = r;
  return WDEM_OK;
}

int wdem_get_energy(wdem_handle* h, double* e, int32_t n) {
  if (!h || !e || n < 0) return WDEM_ERR_ARG;
  cudaSetDevice(h->device);
  double v[WDEM_E_COUNT];
  CK(cudaMemcpyAsync(v, h->dEnergy, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < n; k++) e[k] = k < WDEM_E_COUNT ? v[k] : 0.0;
  return WDEM_OK;
}
int wdem_reset_energy(wdem_handle* h) {
  if (!h) return WDEM_ERR_ARG;
  cudaSetDevice(h->device);
  CK(cudaMemsetAsync(h->dEnergy, 0, sizeof(double) * WDEM_E_COUNT, h->stream));
  return WDEM_OK;
}

int wdem_get_status(wdem_handle* h, wdem_status* st) {
  if (!h || !st) return WDEM_ERR_ARG;
  cudaSetDevice(h->device);
  CK(cudaMemcpyAsync(h->hst, h->dst, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  memset(st, 0, sizeof(*st));
  st->code = h->hst->code;
  st->detail = h->hst->detail;
  st->step = h->step;
  std::vector<uint8_t> s(h->nContacts);
  if (h->nContacts > 0) CK(cudaMemcpy(s.data(), h->buf[h->cur].c.state, h->nContacts, cudaMemcpyDeviceToHost));
  long long live = 0, real = 0;
  for (auto v : s) { if ((v & CS_MASK) != CS_DEAD) live++; if ((v & CS_MASK) == CS_REAL) real++; }
  st->nContacts = live;
  st->nReal = real;
  st->nFullRuns = h->nFullRuns;
  st->capacity = h->buf[h->cur].cap;
  st->lastRunFull = h->lastRunFull;
  st->ellSolves = (int64_t)h->hst->ellSolves;
  st->ellIters = (int64_t)h->hst->ellIters;
  st->ellFallbacks = (int64_t)h->hst->ellFallbacks;
  st->dt = h->raw.dt;
  st->dynDtCrit = h->dynDtCrit;
  st->timeSum = h->timeSum;
  return WDEM_OK;
}

int wdem_collide_boxes(wdem_handle* h, int32_t n, const double* mins, const double* maxs, const uint32_t* mask,
                       uint32_t loneMask, int32_t* pairs, int64_t maxPairs, int64_t* nPairs) {
  if (!h || !mins || !maxs || !mask || !nPairs || n < 0 || n > h->N) return WDEM_ERR_ARG;
  cudaSetDevice(h->device);
  cudaStream_t s = h->stream;
  // Boxes go straight into the handle's box arrays; finite boxes are "small", others "large".
  std::vector<double4_32a> mn(n), mx(n), posr(n);
  std::vector<int4> meta(n);
  h->smallIds.clear(); h->largeIds.clear();
  h->shape.assign(n, WDEM_SHAPE_SPHERE);
  h->radius.assign(n, 0.0);
  h->mat.assign(n, 0);
  for (int i = 0; i < n; i++) {
    mn[i] = make_double4_32a(mins[3 * i], mins[3 * i + 1], mins[3 * i + 2], 0);
    mx[i] = make_double4_32a(maxs[3 * i], maxs[3 * i + 1], maxs[3 * i + 2], 0);
    bool finite = true;
    for (int k = 0; k < 3; k++) finite &= std::isfinite(mins[3 * i + k]) && std::isfinite(maxs[3 * i + k]);
    posr[i] = finite ? make_double4_32a(.5 * (mn[i].x + mx[i].x), .5 * (mn[i].y + mx[i].y), .5 * (mn[i].z + mx[i].z), 0)
                     : make_double4_32a(0, 0, 0, 0);
    meta[i] = make_int4(finite ? WDEM_SHAPE_SPHERE : WDEM_SHAPE_WALL, 0, (int)mask[i], 63);
    if (finite) h->smallIds.push_back(i); else { h->largeIds.push_back(i); h->shape[i] = WDEM_SHAPE_WALL; }
  }
  h->n = n;
  if (n > 0) {
    CK(cudaMemcpyAsync(h->d.bbmin, mn.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.bbmax, mx.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.posr, posr.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->d.meta, meta.data(), n * sizeof(int4), cudaMemcpyHostToDevice, s));
  }
  if (!h->smallIds.empty()) CK(cudaMemcpyAsync(h->dSmall, h->smallIds.data(), h->smallIds.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  if (!h->largeIds.empty()) CK(cudaMemcpyAsync(h->cs.large, h->largeIds.data(), h->largeIds.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  h->cs.nScenes = 1;
  h->cs.nLarge = (int)h->largeIds.size();
  h->nContacts = 0;
  int rc;
  if ((rc = ensureScratch(h, 0))) return rc;
  const int nSmall = (int)h->smallIds.size();
  ColliderScratch& cs = h->cs;
  col_extents_and_grid(s, h->d, h->dSmall, nSmall, cs);
  col_sort(s, h->d, h->dSmall, nSmall, cs);
  col_sweep(s, h->d, nSmall, loneMask, cs, nullptr, 0, false, h->dst);
  const int nSweep = sweepThreads(nSmall, cs.nLarge);
  exclusive_scan_u32(s, cs.counts, nSweep, cs);
  CK(cudaMemcpyAsync(&h->hcounts[0], cs.counts + nSweep, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  long long total = h->hcounts[0];
  int2* dpairs = nullptr;
  CK(dalloc(dpairs, (size_t)total + 1));
  col_sweep(s, h->d, nSmall, loneMask, cs, dpairs, total, true, h->dst);
  std::vector<int2> hp(total);
  if (total > 0) CK(cudaMemcpyAsync(hp.data(), dpairs, total * sizeof(int2), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  cudaFree(dpairs);
  std::vector<unsigned long long> keys(total);
  for (long long i = 0; i < total; i++) {
    unsigned a = (unsigned)std::min(hp[i].x, hp[i].y), b = (unsigned)std::max(hp[i].x, hp[i].y);
    keys[i] = ((unsigned long long)a << 32) | b;
  }
  std::sort(keys.begin(), keys.end());
  for (long long i = 0; i < total && i < maxPairs; i++) {
    pairs[2 * i] = (int32_t)(keys[i] >> 32);
    pairs[2 * i + 1] = (int32_t)(keys[i] & 0xffffffffu);
  }
  *nPairs = total;
  h->particlesSet = false;  // the particle arrays no longer hold a scene
  return WDEM_OK;
}

namespace {
// device buffers for an edit of m particles (the per-particle flags cover the capacity)
int ensureEdit(wdem_handle* h, long long m) {
  if (!h->editGone) {
    CK(dalloc(h->editGone, (size_t)h->N));
    CK(cudaMemset(h->editGone, 0, (size_t)h->N));
  }
  if (m > h->editCap) {
    const long long cap = std::max<long long>(m, 1024);
    CK(dalloc(h->editIds, cap)); CK(dalloc(h->editPark, 3 * cap));
    CK(dalloc(h->editRec, (size_t)EDIT_RECORDS * cap)); CK(dalloc(h->editMeta, cap));
    h->editCap = cap;
  }
  return WDEM_OK;
}
// the forces of the step just run into the particle arrays, for the next integration: the contact
// container changes before it, but those forces were applied in the step that ran (ContactLoop, then the
// host engines)
void materialiseForces(wdem_handle* h) {
  if (!h->forcesInArrays) {
    StepParams P = h->P;
    P.seq = h->seq + 1;  // the records of the last contact pass
    launch_reduce_forces(h->stream, P, h->d, h->n, h->buf[h->cur].c, h->csr);
    h->forcesInArrays = true;
  }
}
}  // namespace

int wdem_remove_particles(wdem_handle* h, int32_t m, const int32_t* ids, const double* park) {
  if (!h || m < 0 || (m > 0 && !ids)) return WDEM_ERR_ARG;
  if (!h->particlesSet || !h->paramsSet) return fail(h, WDEM_ERR_STATE, "remove particles after particles and params were set");
  std::vector<char> seen(h->n, 0);
  for (int k = 0; k < m; k++) {
    if (ids[k] < 0 || ids[k] >= h->n) return fail(h, WDEM_ERR_ARG, "particle id " + std::to_string(ids[k]) + " out of range");
    if (seen[ids[k]]) return fail(h, WDEM_ERR_ARG, "particle id " + std::to_string(ids[k]) + " given twice");
    seen[ids[k]] = 1;
  }
  if (m == 0) return WDEM_OK;
  cudaSetDevice(h->device);
  int rc;
  if ((rc = ensureEdit(h, m))) return rc;
  cudaStream_t s = h->stream;
  materialiseForces(h);
  CK(cudaMemcpyAsync(h->editIds, ids, m * sizeof(int), cudaMemcpyHostToDevice, s));
  if (park) CK(cudaMemcpyAsync(h->editPark, park, 3 * (size_t)m * sizeof(double), cudaMemcpyHostToDevice, s));
  launch_kill(s, h->d, h->n, h->editIds, m, park ? h->editPark : nullptr, h->editGone, h->buf[h->cur].c, h->nContacts);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  h->needRebuild = true;
  h->actValid = false;
  // a removed facet (mask 0) no longer pairs with the other boundaries
  h->facetPairs.erase(std::remove_if(h->facetPairs.begin(), h->facetPairs.end(),
                                     [&](const int4& q) { return seen[q.x] || seen[q.y]; }),
                      h->facetPairs.end());
  return WDEM_OK;
}

int wdem_add_particles(wdem_handle* h, const wdem_particles* p, const int32_t* ids) {
  if (!h || !p || p->n < 0 || (p->n > 0 && !ids)) return WDEM_ERR_ARG;
  if (!h->particlesSet || !h->paramsSet) return fail(h, WDEM_ERR_STATE, "add particles after particles and params were set");
  const int m = p->n;
  if (m == 0) return WDEM_OK;
  if (!p->shape || !p->radius || !p->material || !p->mask || !p->flags || !p->mass || !p->inertia || !p->pos || !p->ori ||
      !p->vel || !p->angVel || !p->force || !p->torque)
    return fail(h, WDEM_ERR_ARG, "null particle array");
  int newN = h->n;
  for (int k = 0; k < m; k++) {
    if (ids[k] < 0 || ids[k] >= h->N) return fail(h, WDEM_ERR_ARG, "slot " + std::to_string(ids[k]) + " outside the handle capacity");
    newN = std::max(newN, ids[k] + 1);
  }
  std::vector<char> seen(newN, 0);
  for (int k = 0; k < m; k++) {
    if (seen[ids[k]]) return fail(h, WDEM_ERR_ARG, "slot " + std::to_string(ids[k]) + " given twice");
    seen[ids[k]] = 1;
  }
  for (int i = h->n; i < newN; i++)
    if (!seen[i]) return fail(h, WDEM_ERR_ARG, "new slots must extend the particle count contiguously (slot " + std::to_string(i) + " missing)");
  for (int k = 0; k < m; k++)
    if (ids[k] < h->n && (h->shape[ids[k]] == WDEM_SHAPE_WALL || h->shape[ids[k]] == WDEM_SHAPE_FACET))
      return fail(h, WDEM_ERR_ARG, "slot " + std::to_string(ids[k]) + " belongs to a wall or facet and is not reused");
  std::vector<double4_32a> rec((size_t)EDIT_RECORDS * m);
  std::vector<int4> meta(m);
  const double nan = std::numeric_limits<double>::quiet_NaN();
  for (int k = 0; k < m; k++) {
    const int sh = p->shape[k];
    if (sh == WDEM_SHAPE_WALL) return fail(h, WDEM_ERR_UNSUPPORTED, "walls are added through wdem_upload_particles");
    if (sh != WDEM_SHAPE_SPHERE && sh != WDEM_SHAPE_ELLIPSOID && sh != WDEM_SHAPE_CAPSULE)
      return fail(h, WDEM_ERR_UNSUPPORTED, "unsupported shape");
    if (sh == WDEM_SHAPE_CAPSULE && (!p->shaft || !(p->radius[k] > 0.) || !(p->shaft[k] >= 0.)))
      return fail(h, WDEM_ERR_ARG, "capsules need a positive radius and a non-negative wdem_particles.shaft");
    if (p->material[k] < 0 || p->material[k] >= (int)h->mats.size())
      return fail(h, WDEM_ERR_ARG, "material index out of range for an added particle");
    const unsigned fl = p->flags[k];
    if (fl & (WDEM_CLUMP_CLUMP | WDEM_CLUMP_CLUMPED)) return fail(h, WDEM_ERR_UNSUPPORTED, "clumps are not supported");
    const double* in = p->inertia + 3 * k;
    const bool asph = !(in[0] == in[1] && in[1] == in[2]) && (fl & 56u) != 56u;
    if ((sh == WDEM_SHAPE_ELLIPSOID || sh == WDEM_SHAPE_CAPSULE || asph) && !h->hasEll)
      return fail(h, WDEM_ERR_UNSUPPORTED, "ellipsoids or aspherical nodes in a handle without them: use wdem_upload_particles");
    if ((sh == WDEM_SHAPE_ELLIPSOID || sh == WDEM_SHAPE_CAPSULE || asph) && h->periodic)
      return fail(h, WDEM_ERR_UNSUPPORTED, "ellipsoids and aspherical nodes in a periodic cell are not supported");
    const int sc = p->scene ? p->scene[k] : 0;
    if (sc < 0 || sc >= std::max(1, h->cs.nScenes)) return fail(h, WDEM_ERR_ARG, "scene index out of range for an added particle");
    double r = p->radius[k];
    double sa[3] = {r, r, r};
    if (sh == WDEM_SHAPE_ELLIPSOID) {
      if (!p->semiAxes) return fail(h, WDEM_ERR_ARG, "ellipsoids need wdem_particles.semiAxes");
      for (int q = 0; q < 3; q++) sa[q] = p->semiAxes[3 * k + q];
      if (!(sa[0] > 0 && sa[1] > 0 && sa[2] > 0)) return fail(h, WDEM_ERR_ARG, "ellipsoid semi-axes must be positive");
      r = std::max(sa[0], std::max(sa[1], sa[2]));
    }
    if (sh == WDEM_SHAPE_CAPSULE) { sa[0] = p->radius[k]; sa[1] = p->shaft[k]; sa[2] = 0; r = p->radius[k] + .5 * p->shaft[k]; }
    double4_32a* q = rec.data() + (size_t)EDIT_RECORDS * k;
    q[0] = make_double4_32a(p->pos[3 * k], p->pos[3 * k + 1], p->pos[3 * k + 2], r);
    q[1] = make_double4_32a(p->vel[3 * k], p->vel[3 * k + 1], p->vel[3 * k + 2], p->mass[k]);
    q[2] = make_double4_32a(p->angVel[3 * k], p->angVel[3 * k + 1], p->angVel[3 * k + 2], 0);
    q[3] = make_double4_32a(in[0], in[1], in[2], 0);
    q[4] = make_double4_32a(p->ori[4 * k], p->ori[4 * k + 1], p->ori[4 * k + 2], p->ori[4 * k + 3]);
    q[5] = make_double4_32a(p->force[3 * k], p->force[3 * k + 1], p->force[3 * k + 2], 0);
    q[6] = make_double4_32a(p->torque[3 * k], p->torque[3 * k + 1], p->torque[3 * k + 2], 0);
    q[7] = make_double4_32a(sa[0], sa[1], sa[2], 0);
    q[8] = p->angMom ? make_double4_32a(p->angMom[3 * k], p->angMom[3 * k + 1], p->angMom[3 * k + 2], 0)
                     : make_double4_32a(nan, nan, nan, 0);
    const bool ipos = in[0] > 0 && in[1] > 0 && in[2] > 0;
    meta[k] = make_int4(sh | (1 << 8) | (asph ? META_ASPH : 0) | (ipos ? META_IPOS : 0) | (sc << META_SCENE_SHIFT),
                        p->material[k], (int)p->mask[k], (int)fl);
  }
  cudaSetDevice(h->device);
  int rc;
  if ((rc = ensureEdit(h, m))) return rc;
  cudaStream_t s = h->stream;
  materialiseForces(h);
  CK(cudaMemcpyAsync(h->editIds, ids, m * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(h->editRec, rec.data(), rec.size() * sizeof(double4_32a), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(h->editMeta, meta.data(), m * sizeof(int4), cudaMemcpyHostToDevice, s));
  launch_put(s, h->d, h->editIds, m, h->editRec, h->editMeta, h->hasEll);
  CK(cudaGetLastError());
  // host copies of the static data; the new slots join the collider's sorted set
  const int oldN = h->n;
  h->shape.resize(newN); h->mat.resize(newN); h->radius.resize(newN); h->semi.resize(3 * (size_t)newN);
  for (int k = 0; k < m; k++) {
    const int i = ids[k];
    h->shape[i] = p->shape[k]; h->mat[i] = p->material[k]; h->radius[i] = p->radius[k];
    const double4_32a sv = rec[(size_t)EDIT_RECORDS * k + 7];
    h->semi[3 * i] = sv.x; h->semi[3 * i + 1] = sv.y; h->semi[3 * i + 2] = sv.z;
  }
  if (newN > oldN) {
    const size_t first = h->smallIds.size();
    for (int i = oldN; i < newN; i++) h->smallIds.push_back(i);
    CK(cudaMemcpyAsync(h->dSmall + first, h->smallIds.data() + first, (h->smallIds.size() - first) * sizeof(int),
                       cudaMemcpyHostToDevice, s));
  }
  CK(cudaStreamSynchronize(s));
  h->n = newN;
  h->matsChecked = -1;
  h->gravAccDirty = true;
  h->needRebuild = true;
  h->actValid = false;
  resolveVerlet(h);
  fillStepParams(h);
  return WDEM_OK;
}

namespace {
bool shapeValid(const wdem_launch_shape& s) {
  auto in = [](int v, std::initializer_list<int> ok) { for (int o : ok) if (v == o) return true; return false; };
  return in(s.contactsBlock, {64, 128, 256}) && s.contactsPerSM >= 0 && s.contactsPerSM <= 64 &&
         in(s.cullBlock, {128, 256, 512}) && in(s.integratorBlock, {128, 256, 512}) && s.listsPerSM >= 0 &&
         s.listsPerSM <= 64;
}
}  // namespace

int wdem_set_launch_shape(wdem_handle* h, const wdem_launch_shape* shape) {
  if (!h || !shape) return WDEM_ERR_ARG;
  if (!shapeValid(*shape)) return fail(h, WDEM_ERR_ARG, "launch shape: block sizes 64/128/256 (contacts), 128/256/512 (cull, integrator); blocks per SM 0..64");
  h->launchShape = *shape;
  h->launchShape._pad = 0;
  fillStepParams(h);
  return WDEM_OK;
}

int wdem_get_launch_shape(wdem_handle* h, wdem_launch_shape* shape) {
  if (!h || !shape) return WDEM_ERR_ARG;
  *shape = h->launchShape;
  return WDEM_OK;
}

int wdem_autotune(wdem_handle* h, int32_t stepsPerCandidate, wdem_launch_shape* best, double* msBest, double* msStart) {
  if (!h || stepsPerCandidate <= 0) return WDEM_ERR_ARG;
  if (!h->particlesSet || !h->paramsSet) return fail(h, WDEM_ERR_STATE, "autotune after particles and params were set");
  const bool timingWas = h->timing;
  h->timing = true;
  // cost of a shape: per-phase device time of the integrator and the contact pass per step
  auto cost = [&](const wdem_launch_shape& s, double& ms) -> int {
    h->launchShape = s;
    fillStepParams(h);
    int rc = wdem_step(h, 2);
    if (rc) return rc;
    if ((rc = wdem_step(h, stepsPerCandidate))) return rc;
    ms = (h->phaseMs[PH_LEAPFROG] + h->phaseMs[PH_CONTACTS]) / stepsPerCandidate;
    return WDEM_OK;
  };
  wdem_launch_shape cur = h->launchShape;
  double curMs = 0;
  int rc = cost(cur, curMs);
  const double startMs = curMs;
  const std::vector<std::pair<int wdem_launch_shape::*, std::vector<int>>> knobs = {
      {&wdem_launch_shape::contactsBlock, {64, 128, 256}},
      {&wdem_launch_shape::contactsPerSM, {0, 1, 2, 4, 8, 16}},
      {&wdem_launch_shape::cullBlock, {128, 256, 512}},
      {&wdem_launch_shape::integratorBlock, {128, 256, 512}},
      {&wdem_launch_shape::listsPerSM, {0, 1, 2, 4}}};
  for (const auto& kv : knobs) {
    if (rc) break;
    for (int v : kv.second) {
      if (cur.*(kv.first) == v) continue;
      wdem_launch_shape c = cur;
      c.*(kv.first) = v;
      if (!shapeValid(c)) continue;
      double ms = 0;
      if ((rc = cost(c, ms))) break;
      if (ms < curMs) { cur = c; curMs = ms; }
    }
  }
  h->timing = timingWas;
  h->launchShape = cur;
  fillStepParams(h);
  if (rc) return rc;
  if (best) *best = cur;
  if (msBest) *msBest = curMs;
  if (msStart) *msStart = startMs;
  return WDEM_OK;
}

int wdem_set_contact_limit(wdem_handle* h, int64_t maxContacts) {
  if (!h || maxContacts < 0) return WDEM_ERR_ARG;
  h->contactLimit = maxContacts;
  return WDEM_OK;
}

int wdem_set_queue_depth(wdem_handle* h, int32_t depth) {
  if (!h || depth < 0 || depth > 4096) return WDEM_ERR_ARG;
  h->maxAhead = depth;
  return WDEM_OK;
}

int wdem_set_step_graphs(wdem_handle* h, int32_t mode) {
  if (!h || mode < WDEM_GRAPHS_OFF || mode > WDEM_GRAPHS_ON) return WDEM_ERR_ARG;
  h->graphMode = mode;
  return WDEM_OK;
}

int wdem_graph_stats(wdem_handle* h, int64_t* captures, int64_t* replays) {
  if (!h || !captures || !replays) return WDEM_ERR_ARG;
  *captures = h->graphCaptures;
  *replays = h->graphReplays;
  return WDEM_OK;
}

int wdem_set_timing(wdem_handle* h, int32_t enable) {
  if (!h) return WDEM_ERR_ARG;
  h->timing = enable != 0;
  return WDEM_OK;
}

int wdem_kernel_times(wdem_handle* h, const char** names, double* ms, int32_t* launches, int32_t n, int32_t* count) {
  if (!h || !count) return WDEM_ERR_ARG;
  for (int k = 0; k < PH_COUNT && k < n; k++) {
    if (names) names[k] = kPhaseNames[k];
    if (ms) ms[k] = h->phaseMs[k];
    if (launches) launches[k] = h->phaseLaunches[k];
  }
  *count = PH_COUNT;
  return WDEM_OK;
}

int wdem_set_cell(wdem_handle* h, const wdem_cell* c) {
  if (!h || !c) return WDEM_ERR_ARG;
  // a full collider run follows only a change of periodicity (InsertionSortCollider::prologue_doFullRun,
  // InsertionSortCollider.cpp:377-382); new cell matrices alone do not trigger one
  if (!c->periodic) {
    if (h->periodic) h->needRebuild = true;
    h->periodic = false; h->P.periodic = 0;
    return WDEM_OK;
  }
  if (c->homoDeform != 4) return fail(h, WDEM_ERR_UNSUPPORTED, "Cell.homoDeform other than gradV2 (4) is not supported");
  for (int s : h->shape)
    if (s != WDEM_SHAPE_SPHERE)
      return fail(h, WDEM_ERR_UNSUPPORTED, std::string(s == WDEM_SHAPE_FACET ? "facets" : s == WDEM_SHAPE_WALL ? "walls" :
                                                       s == WDEM_SHAPE_CAPSULE ? "capsules" : "ellipsoids") +
                                               " in a periodic cell are not supported");
  if (h->nContacts > 0 && !h->periodic) return fail(h, WDEM_ERR_STATE, "set the cell before uploading contacts");
  if (h->cs.nScenes > 1) return fail(h, WDEM_ERR_UNSUPPORTED, "batched scenes in a periodic cell are not supported");
  HostCell& hc = h->cell;
  // Cell.setHSize / trsf / nextGradV (Cell.hpp:108-111) then postLoad -> integrateAndUpdate(0)
  hc.hSize = get9(c->hSize);
  hc.pprevHsize = hc.hSize;
  hc.trsf = get9(c->trsf);
  hc.gradV = get9(c->gradV);
  hc.nextGradV = get9(c->nextGradV);
  hc.W = scaled(addScaled(hc.gradV, transposed(hc.gradV), -1.0), .5);
  double v[3];
  leviCivita(hc.W, v);
  for (int k = 0; k < 3; k++) hc.spinVec[k] = .5 * v[k];
  if (!hc.integrateAndUpdate(0)) return fail(h, WDEM_ERR_ARG, "Cell is degenerate (zero volume).");
  if (!h->periodic) h->needRebuild = true;
  h->periodic = true;
  h->P.periodic = 1;
  fillCellParams(h);
  return WDEM_OK;
}

int wdem_get_cell(wdem_handle* h, wdem_cell* c) {
  if (!h || !c) return WDEM_ERR_ARG;
  c->periodic = h->periodic ? 1 : 0;
  c->homoDeform = 4;
  put9(c->hSize, h->cell.hSize);
  put9(c->trsf, h->cell.trsf);
  put9(c->gradV, h->cell.gradV);
  put9(c->nextGradV, h->cell.nextGradV);
  put9(c->pprevHsize, h->cell.pprevHsize);
  return WDEM_OK;
}

int wdem_get_stress(wdem_handle* h, double* stress) {
  if (!h || !stress) return WDEM_ERR_ARG;
  cudaSetDevice(h->device);
  cudaStream_t s = h->stream;
  const long long nc = h->nContacts;
  if (9 * std::max<long long>(nc, 1) > h->stressCap) {
    CK(dalloc(h->stressTerms, (size_t)(9 * std::max<long long>(nc, 1))));
    h->stressCap = 9 * std::max<long long>(nc, 1);
  }
  if (!h->dStress) CK(dalloc(h->dStress, 9));
  int rc;
  if ((rc = ensurePartials(h, std::max<long long>(nc, 1)))) return rc;
  if (h->periodic) fillCellParams(h);
  launch_stress(s, h->P, h->d, h->buf[h->cur].c, nc, h->stressTerms, h->ePartials, h->dStress);
  double v[9];
  CK(cudaMemcpyAsync(v, h->dStress, sizeof(v), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const double vol = h->periodic ? det3(h->cell.hSize) : 1.0;
  for (int k = 0; k < 9; k++) stress[k] = v[k] / vol;
  return WDEM_OK;
}

int wdem_get_stress_noalloc(wdem_handle* h, double* stress) {
  if (!h || !stress) return WDEM_ERR_ARG;
  const long long nc = h->nContacts;
  if (nc > stress_noalloc_max_contacts())
    return fail(h, WDEM_ERR_NO_ALLOC, "wdem_get_stress_noalloc: " + std::to_string(nc) +
                " contacts exceed its fixed scratch (at most " + std::to_string(stress_noalloc_max_contacts()) +
                " contacts); use wdem_get_stress");
  CK(cudaSetDevice(h->device));
  void* scratch = nullptr;
  CK(noalloc_scratch(h->device, &scratch));
  if (h->periodic) fillCellParams(h);
  double v[9];
  CK(launch_stress_noalloc(h->stream, h->P, h->d, h->buf[h->cur].c, nc, scratch, v));
  CK(cudaStreamSynchronize(h->stream));
  const double vol = h->periodic ? det3(h->cell.hSize) : 1.0;
  for (int k = 0; k < 9; k++) stress[k] = v[k] / vol;
  return WDEM_OK;
}

namespace {
int mlpEnsure(wdem_handle* h) {
  if (h->mlpW) return WDEM_OK;
  const int n = mlp_npad();
  CK(mlp_prepare_kernels());
  CK(dalloc(h->mlpW, n)); CK(dalloc(h->mlpM, n)); CK(dalloc(h->mlpV, n)); CK(dalloc(h->mlpGrad, n)); CK(dalloc(h->mlpLoss, 1));
  CK(dalloc(h->mlpWbf, n));
  CK(cudaMemsetAsync(h->mlpGrad, 0, n * sizeof(float), h->stream));
  return WDEM_OK;
}
int mlpUpload(wdem_handle* h, const std::vector<float>& pad) {
  const int n = mlp_npad();
  CK(cudaMemcpyAsync(h->mlpW, pad.data(), n * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemsetAsync(h->mlpM, 0, n * sizeof(float), h->stream));
  CK(cudaMemsetAsync(h->mlpV, 0, n * sizeof(float), h->stream));
  mlp_to_bf16(h->stream, h->mlpW, h->mlpWbf);
  CK(cudaStreamSynchronize(h->stream));
  h->mlpT = 0;
  h->mlpReady = true;
  return WDEM_OK;
}
unsigned long long splitmix64(unsigned long long& x) {
  unsigned long long z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform01(unsigned long long& x) { return (double)(splitmix64(x) >> 11) * (1.0 / 9007199254740992.0); }
}  // namespace

int wdem_warm_init(wdem_handle* h, uint64_t seed) {
  if (!h) return WDEM_ERR_ARG;
  CK(cudaSetDevice(h->device));
  int rc;
  if ((rc = mlpEnsure(h))) return rc;
  // He-uniform weights (fan-in), zero biases
  std::vector<float> pub(WDEM_WARM_NPARAM, 0.f);
  unsigned long long st = seed;
  const int fin[4] = {13, 64, 64, 64}, fout[4] = {64, 64, 64, 4};
  size_t q = 0;
  for (int l = 0; l < 4; l++) {
    const double lim = std::sqrt(6.0 / fin[l]);
    for (int k = 0; k < fin[l] * fout[l]; k++) pub[q++] = (float)((2 * uniform01(st) - 1) * lim);
    q += fout[l];
  }
  std::vector<float> pad(mlp_npad());
  mlp_unpack(pub.data(), pad.data());
  return mlpUpload(h, pad);
}

int wdem_warm_set_weights(wdem_handle* h, const float* w, int64_t n) {
  if (!h || !w || n != WDEM_WARM_NPARAM) return WDEM_ERR_ARG;
  CK(cudaSetDevice(h->device));
  int rc;
  if ((rc = mlpEnsure(h))) return rc;
  std::vector<float> pad(mlp_npad());
  mlp_unpack(w, pad.data());
  return mlpUpload(h, pad);
}

int wdem_warm_get_weights(wdem_handle* h, float* w, int64_t n) {
  if (!h || !w || n != WDEM_WARM_NPARAM) return WDEM_ERR_ARG;
  if (!h->mlpReady) return fail(h, WDEM_ERR_STATE, "no warm-start network");
  std::vector<float> pad(mlp_npad());
  CK(cudaMemcpyAsync(pad.data(), h->mlpW, pad.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  mlp_pack(pad.data(), w);
  return WDEM_OK;
}

int wdem_warm_predict(wdem_handle* h, const float* x, int64_t n, float* y) {
  if (!h || (n > 0 && (!x || !y)) || n < 0) return WDEM_ERR_ARG;
  if (!h->mlpReady) return fail(h, WDEM_ERR_STATE, "no warm-start network");
  if (n == 0) return WDEM_OK;
  CK(cudaSetDevice(h->device));
  float *dx = nullptr, *dy = nullptr;
  CK(dalloc(dx, (size_t)n * WDEM_WARM_INPUTS));
  if (dalloc(dy, (size_t)n * WDEM_WARM_OUTPUTS) != cudaSuccess) { cudaFree(dx); return fail(h, WDEM_ERR_CUDA, "out of memory"); }
  cudaMemcpyAsync(dx, x, (size_t)n * WDEM_WARM_INPUTS * sizeof(float), cudaMemcpyHostToDevice, h->stream);
  mlp_launch_predict(h->stream, dx, n, dy, h->mlpWbf, h->mlpW, h->dst);
  cudaMemcpyAsync(y, dy, (size_t)n * WDEM_WARM_OUTPUTS * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
  cudaMemcpyAsync(h->hst, h->dst, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  cudaFree(dx); cudaFree(dy);
  if (e != cudaSuccess) return fail(h, WDEM_ERR_CUDA, cudaGetErrorString(e));
  int rc;
  if ((rc = checkDeviceStatus(h))) return rc;
  return WDEM_OK;
}

int wdem_warm_grad(wdem_handle* h, const float* records, int64_t n, float* grad, float* loss) {
  if (!h || !records || !grad || !loss || n <= 0) return WDEM_ERR_ARG;
  if (!h->mlpReady) return fail(h, WDEM_ERR_STATE, "no warm-start network");
  CK(cudaSetDevice(h->device));
  float* dr = nullptr;
  CK(dalloc(dr, (size_t)n * WDEM_WARM_RECORD));
  cudaMemcpyAsync(dr, records, (size_t)n * WDEM_WARM_RECORD * sizeof(float), cudaMemcpyHostToDevice, h->stream);
  cudaMemsetAsync(h->mlpGrad, 0, mlp_npad() * sizeof(float), h->stream);
  cudaMemsetAsync(h->mlpLoss, 0, sizeof(float), h->stream);
  mlp_launch_grad(h->stream, dr, nullptr, n, h->mlpWbf, h->mlpW, h->mlpGrad, h->mlpLoss, h->dst, h->numSMs);
  std::vector<float> pad(mlp_npad());
  cudaMemcpyAsync(pad.data(), h->mlpGrad, pad.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
  cudaMemcpyAsync(loss, h->mlpLoss, sizeof(float), cudaMemcpyDeviceToHost, h->stream);
  cudaMemsetAsync(h->mlpGrad, 0, mlp_npad() * sizeof(float), h->stream);
  cudaMemcpyAsync(h->hst, h->dst, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  cudaFree(dr);
  if (e != cudaSuccess) return fail(h, WDEM_ERR_CUDA, cudaGetErrorString(e));
  int rc;
  if ((rc = checkDeviceStatus(h))) return rc;
  mlp_pack(pad.data(), grad);
  return WDEM_OK;
}

int wdem_warm_train(wdem_handle* h, const float* records, int64_t n, int32_t epochs, int32_t batch, float lr,
                    uint64_t seed, float* lossPerEpoch) {
  if (!h || !records || n <= 0 || epochs < 0 || batch <= 0 || !(lr > 0)) return WDEM_ERR_ARG;
  if (n > (int64_t)INT32_MAX) return fail(h, WDEM_ERR_ARG, "too many training records");
  CK(cudaSetDevice(h->device));
  int rc;
  if (!h->mlpReady && (rc = wdem_warm_init(h, seed))) return rc;
  cudaStream_t s = h->stream;
  float* dr = nullptr;
  int* didx = nullptr;
  CK(dalloc(dr, (size_t)n * WDEM_WARM_RECORD));
  if (dalloc(didx, (size_t)n) != cudaSuccess) { cudaFree(dr); return fail(h, WDEM_ERR_CUDA, "out of memory"); }
  cudaMemcpyAsync(dr, records, (size_t)n * WDEM_WARM_RECORD * sizeof(float), cudaMemcpyHostToDevice, s);
  std::vector<int> perm(n);
  unsigned long long st = seed ^ 0x5DEECE66Dull;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const long long totalSteps = (long long)epochs * ((n + batch - 1) / batch);
  long long step = 0;
  cudaError_t e = cudaSuccess;
  for (int ep = 0; ep < epochs && e == cudaSuccess; ep++) {
    for (int64_t k = 0; k < n; k++) perm[k] = (int)k;
    for (int64_t k = n - 1; k > 0; k--) std::swap(perm[k], perm[(int64_t)(splitmix64(st) % (unsigned long long)(k + 1))]);
    cudaMemcpyAsync(didx, perm.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(h->mlpLoss, 0, sizeof(float), s);
    long long nb = 0;
    for (int64_t b0 = 0; b0 < n; b0 += batch, nb++, step++) {
      const long long m = std::min<long long>(batch, n - b0);
      mlp_launch_grad(s, dr, didx + b0, m, h->mlpWbf, h->mlpW, h->mlpGrad, h->mlpLoss, h->dst, h->numSMs);
      h->mlpT++;
      const float c1 = 1.f - std::pow(b1, (float)h->mlpT), c2 = 1.f - std::pow(b2, (float)h->mlpT);
      // half-cosine decay from lr to lr/100 over all steps of this call
      const double frac = totalSteps > 1 ? (double)step / (double)(totalSteps - 1) : 0.0;
      const float lrt = (float)(lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(M_PI * frac))));
      mlp_launch_adam(s, h->mlpW, h->mlpM, h->mlpV, h->mlpGrad, h->mlpWbf, lrt, b1, b2, c1, c2, eps);
    }
    float l = 0;
    cudaMemcpyAsync(&l, h->mlpLoss, sizeof(float), cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (lossPerEpoch) lossPerEpoch[ep] = l / (float)nb;
  }
  cudaFree(dr); cudaFree(didx);
  if (e != cudaSuccess) return fail(h, WDEM_ERR_CUDA, cudaGetErrorString(e));
  CK(cudaMemcpyAsync(h->hst, h->dst, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return checkDeviceStatus(h);
}

int wdem_ell_log(wdem_handle* h, int64_t capRecords) {
  if (!h || capRecords < 0) return WDEM_ERR_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  cudaFree(h->ellLog); cudaFree(h->ellLogCount);
  h->ellLog = nullptr; h->ellLogCount = nullptr; h->ellLogCap = 0;
  if (capRecords > 0) {
    CK(dalloc(h->ellLog, (size_t)capRecords * WDEM_WARM_RECORD));
    CK(dalloc(h->ellLogCount, 1));
    CK(cudaMemsetAsync(h->ellLogCount, 0, sizeof(unsigned long long), h->stream));
    h->ellLogCap = capRecords;
  }
  fillStepParams(h);
  return WDEM_OK;
}

int wdem_ell_log_read(wdem_handle* h, float* out, int64_t cap, int64_t* n) {
  if (!h || !n || cap < 0 || (cap > 0 && !out)) return WDEM_ERR_ARG;
  *n = 0;
  if (!h->ellLog) return WDEM_OK;
  unsigned long long cnt = 0;
  CK(cudaMemcpyAsync(&cnt, h->ellLogCount, sizeof(cnt), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  long long m = std::min<long long>((long long)cnt, h->ellLogCap);
  m = std::min<long long>(m, cap);
  if (m > 0) {
    CK(cudaMemcpyAsync(out, h->ellLog, (size_t)m * WDEM_WARM_RECORD * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  *n = m;
  return WDEM_OK;
}

int wdem_get_stream(wdem_handle* h, void** stream) {
  if (!h || !stream) return WDEM_ERR_ARG;
  *stream = (void*)h->stream;
  return WDEM_OK;
}

static int ensureStaging(wdem_handle* h, long long n) {
  if (13 * n > h->stagingCap) {
    CK(dalloc(h->staging, (size_t)(13 * n)));
    h->stagingCap = 13 * n;
  }
  return WDEM_OK;
}

int wdem_write_state(wdem_handle* h, int32_t n, const double* pos, const double* vel, const double* angVel,
                     const double* ori) {
  if (!h || n < 0 || n > h->n) return WDEM_ERR_ARG;
  if (n == 0) return WDEM_OK;
  cudaSetDevice(h->device);
  int rc;
  if ((rc = ensureStaging(h, n))) return rc;
  cudaStream_t s = h->stream;
  double *dp = nullptr, *dv = nullptr, *dw = nullptr, *dq = nullptr;
  double* st = h->staging;
  if (pos) { dp = st; CK(cudaMemcpyAsync(dp, pos, 3 * sizeof(double) * n, cudaMemcpyHostToDevice, s)); }
  if (vel) { dv = st + 3 * (size_t)n; CK(cudaMemcpyAsync(dv, vel, 3 * sizeof(double) * n, cudaMemcpyHostToDevice, s)); }
  if (angVel) { dw = st + 6 * (size_t)n; CK(cudaMemcpyAsync(dw, angVel, 3 * sizeof(double) * n, cudaMemcpyHostToDevice, s)); }
  if (ori) { dq = st + 9 * (size_t)n; CK(cudaMemcpyAsync(dq, ori, 4 * sizeof(double) * n, cudaMemcpyHostToDevice, s)); }
  launch_state_in(s, h->d, n, dp, dv, dw, dq);
  return WDEM_OK;
}

int wdem_read_state(wdem_handle* h, int32_t n, double* pos, double* vel, double* angVel, double* ori) {
  if (!h || n < 0 || n > h->n) return WDEM_ERR_ARG;
  if (n == 0) return WDEM_OK;
  cudaSetDevice(h->device);
  int rc;
  if ((rc = ensureStaging(h, n))) return rc;
  cudaStream_t s = h->stream;
  double* st = h->staging;
  launch_state_out(s, h->d, n, pos ? st : nullptr, vel ? st + 3 * (size_t)n : nullptr, angVel ? st + 6 * (size_t)n : nullptr,
                   ori ? st + 9 * (size_t)n : nullptr);
  if (pos) CK(cudaMemcpyAsync(pos, st, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (vel) CK(cudaMemcpyAsync(vel, st + 3 * (size_t)n, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (angVel) CK(cudaMemcpyAsync(angVel, st + 6 * (size_t)n, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (ori) CK(cudaMemcpyAsync(ori, st + 9 * (size_t)n, 4 * sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return WDEM_OK;
}

int wdem_fp64_peak(wdem_handle* h, double* gflops) {
  if (!h || !gflops) return WDEM_ERR_ARG;
  cudaSetDevice(h->device);
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
  int rc;
  if ((rc = ensureStaging(h, std::max(64, sms * 8)))) return rc;
  *gflops = fp64_probe(h->stream, h->staging, sms, nullptr);
  CK(cudaGetLastError());
  return WDEM_OK;
}

int wdem_launch_count(wdem_handle* h, int64_t* count) {
  if (!h || !count) return WDEM_ERR_ARG;
  *count = ::wdem::g_kernel_launches;
  return WDEM_OK;
}

/* Keep L6Geom.uN/vel/angVel of every real contact for download (off by default; tests turn it on). */
int wdem_keep_geom(wdem_handle* h, int32_t enable) {
  if (!h) return WDEM_ERR_ARG;
  h->keepGeom = enable != 0;
  return WDEM_OK;
}

}  // extern "C"
