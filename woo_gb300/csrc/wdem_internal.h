// wdem_internal.h -- device-side layout of the GB300 DEM engine and the launchers that the host
// runtime (wdem_api.cu) calls.  Shared by the kernel translation units; not part of the C ABI.
//
// HBM layout (all arrays 256-byte aligned, structure-of-arrays):
//   particles, capacity N:
//     posr    double4_32a  (x, y, z, radius)            radius = 0 for walls
//     velm    double4_32a  (vx, vy, vz, mass)
//     angw    double4_32a  (wx, wy, wz, unused)
//     inert   double4_32a  (ix, iy, iz, unused)
//     ori     double4_32a  (w, x, y, z)
//     meta    int4     (shape | wallAxis<<4 | (wallSense+1)<<8, material, mask, flags)
//     posf    float4   FP32 copy of posr, read by the contact kernel's conservative distance cull
//     lastPos double4_32a  position at the last collider rebuild (Aabb.nodeLastPos)
//     bbmin, bbmax double4_32a  verlet-enlarged boxes of the last rebuild (minima/maxima)
//     force, torque double4_32a  DemData.force/torque when materialised (upload, download)
//   contacts, capacity C, double-buffered across collider rebuilds:
//     ids     int2     (pA, pB)
//     state   uint8    CS_POTENTIAL / CS_REAL / CS_PENDING / CS_DEAD
//     step0   int32    Contact.stepCreated
//     hist    double x 14 SoA: trsf col0 (3), trsf col1 (3), contPt (3), force (3, local), kn, kt
//             (+4 for HertzPhys: kn0, kt0, alpha_sqrtMK, adhesion force)
//     tanPhi  double
//     slot    int2     the contact's two entries in the CSR (pA's, pB's)
//     out     2 double4_32a records per CSR entry (one 32-byte sector each), written by the contact pass at
//             the entry's position: (force on the entry's particle, pass stamp), (torque, unused); a particle's
//             records are contiguous, so the integrator's gather reads its CSR row as one run
//   CSR over particles: rowptr[N+1], entries[2C] = contact index | (isB << 31), rows sorted
//   by the partner's id key so that sums run in the order of the sorted contact keys.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/wdem.h"

namespace wdem {

// kernels launched by the library in this process (incremented at every launch site)
extern long long g_kernel_launches;

// contact state byte: bits 0-1 the lifecycle state, bit 2 "pA is a wall", bit 3 "pB is a wall", bits 4-5
// "pA / pB is an ellipsoid", bit 7 "pA is a facet" (pB then is a sphere).  A pair without a geometry
// functor (wall + wall, facet + ellipsoid) carries both wall bits and is never evaluated.
enum ContactState : uint8_t { CS_POTENTIAL = 0, CS_REAL = 1, CS_PENDING = 2, CS_DEAD = 3 };
enum : uint8_t { CS_MASK = 3, CS_WALL_A = 4, CS_WALL_B = 8, CS_ELL_A = 16, CS_ELL_B = 32, CS_ELL = 48, CS_FACET = 128,
                 CS_SHAPES = 188 };
// a potential pair that cannot touch before the next collider run (set by the contact cull, dropped by
// the rebuild's carry): every particle stays within verletDist of its position at the last rebuild,
// so two bounding spheres come closer by at most 4 verletDist between any two steps without a rebuild
enum : uint8_t { CS_FAR = 64 };
// meta.x: shape (bits 0-3), wall axis (4-5), wall sense + 1 (8-9), aspherical Leapfrog (bit 12)
// META_ORI_FIXED: the orientation is not rotating and normalising it is the identity (set and cleared by the
// integrator); META_IPOS: all inertia components are positive (set at upload)
enum { META_ASPH = 1 << 12, META_ORI_FIXED = 1 << 13, META_IPOS = 1 << 14 };
// meta.x bits 16..27: scene index of batched independent scenes
enum { META_SCENE_SHIFT = 16, MAX_SCENES = 4096 };
__host__ __device__ __forceinline__ int sceneOf(int metax) { return (metax >> META_SCENE_SHIFT) & (MAX_SCENES - 1); }
// threads (and pair-count entries) of the collider's sweep: one per small box, one per large body (at least
// one); the exclusive scan of the counts leaves the pair total at counts[sweepThreads]
__host__ __device__ __forceinline__ int sweepThreads(int nSmall, int nLarge) { return nSmall + (nLarge > 0 ? nLarge : 1); }
// pairs of one sweep thread kept by the counting pass for the writing pass (a thread with more walks again)
constexpr int SWEEP_BUF = 8;
// Pair orientation as the geometry functors take it (GeomDispatcher::getFunctor2D swaps a fresh contact,
// ContactLoop.cpp:144-150): the pair (lower id, higher id) is swapped when its shapes come in the order
// Sphere+Wall, Ellipsoid+Sphere, Ellipsoid+Wall or Sphere+Facet.
__host__ __device__ __forceinline__ bool pairSwaps(int sa, int sb) {
  return (sa == WDEM_SHAPE_SPHERE && sb == WDEM_SHAPE_WALL) || (sa == WDEM_SHAPE_ELLIPSOID && sb == WDEM_SHAPE_SPHERE) ||
         (sa == WDEM_SHAPE_ELLIPSOID && sb == WDEM_SHAPE_WALL) || (sa == WDEM_SHAPE_SPHERE && sb == WDEM_SHAPE_FACET) ||
         (sa == WDEM_SHAPE_CAPSULE && sb == WDEM_SHAPE_SPHERE) || (sa == WDEM_SHAPE_CAPSULE && sb == WDEM_SHAPE_WALL);
}
// shape bits of the state byte of an oriented pair: capsules count as aspherical (the ellipsoid bits, the
// contact kernel tells them apart by the shapes); pairs with no functor (wall + wall, facet + anything but a
// sphere, capsule + ellipsoid) get both wall bits and are skipped
__host__ __device__ __forceinline__ uint8_t pairShapeBits(int sa, int sb) {
  if (sa == WDEM_SHAPE_FACET || sb == WDEM_SHAPE_FACET)
    return (uint8_t)((sa == WDEM_SHAPE_FACET && sb == WDEM_SHAPE_SPHERE) ? CS_FACET : (CS_WALL_A | CS_WALL_B));
  if ((sa == WDEM_SHAPE_CAPSULE && sb == WDEM_SHAPE_ELLIPSOID) || (sa == WDEM_SHAPE_ELLIPSOID && sb == WDEM_SHAPE_CAPSULE))
    return (uint8_t)(CS_WALL_A | CS_WALL_B);
  const bool aspA = sa == WDEM_SHAPE_ELLIPSOID || sa == WDEM_SHAPE_CAPSULE;
  const bool aspB = sb == WDEM_SHAPE_ELLIPSOID || sb == WDEM_SHAPE_CAPSULE;
  return (uint8_t)((sa == WDEM_SHAPE_WALL ? CS_WALL_A : 0) | (sb == WDEM_SHAPE_WALL ? CS_WALL_B : 0) |
                   (aspA ? CS_ELL_A : 0) | (aspB ? CS_ELL_B : 0));
}
enum { HIST_T0X = 0, HIST_T0Y, HIST_T0Z, HIST_T1X, HIST_T1Y, HIST_T1Z, HIST_CX, HIST_CY, HIST_CZ,
       HIST_FX, HIST_FY, HIST_FZ, HIST_KN, HIST_KT,
       HIST_E0, HIST_E1, HIST_E2, HIST_E3,   // HertzPhys constants: kn0, kt0, alpha_sqrtMK, DMT adhesion force
       HIST_COUNT };
enum { HIST_FRICT = HIST_E0 };  // FrictPhys contacts carry the first 14 history arrays
// records of one CSR entry in Contacts.out: the force with the stamp of the contact pass that wrote it in w
// (its StepParams.seq; a record whose stamp is not the previous pass's is stale and skipped), the torque
enum { OUT_F = 0, OUT_T = 1, OUT_RECORDS = 2 };
enum { MAX_MATERIALS = 1024 };  // 1024 x 56 B fits the 64 KB constant bank

struct DevMaterial {
  int kind;
  double density, young, ktDivKn, tanPhi, surfEnergy, alpha;
};

// classes of a matrix entry: +0, -0, exactly 1, anything else
enum { MCLS_PZERO = 0, MCLS_NZERO = 1, MCLS_ONE = 2, MCLS_GEN = 3 };

// Engine + functor attributes as the kernels see them.
struct StepParams {
  double dt;
  long long step;
  long long seq;            // number of this step's contact pass (never reset); stamps the pass's force records
  int dw;                   // the contact law of real sphere/wall contacts in double-word FP32 (WDEM_ARITH_DW)
  int hasFacets;            // the scene has facets
  int stepDev;              // 1: step and seq are offsets from DeviceStatus.stepBase/seqBase (steps replayed
                            // from a CUDA graph, whose kernel arguments are fixed at capture)
  int denseTouch;           // 1: real contacts were at least n/8 in the last step the host saw; the
                            // integrator's first pass then compacts each block's untouched particles
  double gravity[3];
  int hasGravity;
  double distFactor;        // DemField.distFactor
  double bboxFactor;        // distFactor > 0 ? distFactor : 1  (Bo1_Sphere_Aabb)
  unsigned loneMask;
  double damping;
  double verletDist;        // resolved, >= 0
  double maxD2;             // verletDist^2
  float verletLoF;          // FP32 lower bound of verletDist (FP32 verlet trigger)
  float verletHiF;          // FP32 upper bound of verletDist (far-pair screen of the contact cull)
  double dampM, dampP;      // 1 - damping * 1 and 1 - damping * (-1), the nonviscDamp2nd factors
  int dampOn;               // damping != 0
  float distFactorF;        // |distFactor| in FP32 (contact cull)
  int gravAxis;             // the only non-zero gravity component, or -1 (angw.w then holds RN(RN(m g)/m))
  int noRatch, iniLensTouch, trsfRenorm, approxMask;
  int updatePhysNow;        // Cp2 runs on existing contacts this step (updatePhys always/once)
  int cp2, law;
  int noSlip, noBreak, noFrict;
  double relRollStiff, relTwistStiff, rollTanPhi;
  int noAttraction;
  double poisson, en, viscAlpha;  // viscAlpha from en, computed once on the host
  int trackEnergy;
  int lfEnergy;       // Leapfrog's reallyTrackEnergy: trackEnergy, off in step 0 of a cell with gradV != I
  int nMaterials;
  // periodic cell (Cell, homoDeform GRADV2), row-major 3x3
  int periodic;
  int hasShear;
  double hS[9];        // Cell.hSize: Contact shift = hSize * cellDist
  double shv[9];       // Cell.gradV * Cell.pprevHsize: shift velocity = shv * cellDist
  double unsh[9];      // Cell unshear transformation (box centres)
  double csize[3];     // cell lengths (periodic collider)
  double sae[3];       // 1/cos[ax] - 1 of Cell::shearAlignedExtents
  double gradV[9];     // Cell.gradV (pprevFluctVel)
  double spinVec[3];
  double ImLL4hInv[9], IpLL4h[9], LmL[9];  // Leapfrog GRADV2 matrices
  double dSpin[3];     // Leapfrog.deltaSpinVec
  // entry classes of gradV, ImLL4hInv, IpLL4h, LmL (2 bits per entry, row-major: MCLS_* below), for
  // products that skip bit-exactly what a zero or a unit entry contributes
  int clsGradV, clsImLL4hInv, clsIpLL4h, clsLmL;
  int dSpinZero;       // every dSpin component is +0
  // ellipsoids: Cg2_Ellipsoid_Ellipsoid_L6Geom solver
  int hasEll;
  int ellSolver;       // WDEM_ELL_*
  double brentTol;     // 2^(1 - min(brentBits, 26))
  double newtonTol;
  int warmStart;       // WDEM_WARM_*
  int fallbackIters;
  const double* matDt;               // batched scenes: dt per material (device), or null (all use dt)
  float* ellLog;                     // training records of solved pairs (17 floats each), or null
  unsigned long long* ellLogCount;
  long long ellLogCap;
  // launch shape (host-side choices carried with the parameters; the kernels do not read them): block
  // sizes of the contact FP64 pass, the contact cull and the integrator's first pass; resident blocks per
  // SM of the contact FP64 pass and of the integrator's list pass (0: as many as fit); SMs of the device
  int shContactsBlock, shContactsPerSM, shCullBlock, shLeapBlock, shListsPerSM;
  int numSMs;
};

// time step of a particle (batched scenes: its material's scene dt)
__device__ __forceinline__ double dtOf(const StepParams& P, int material) { return P.matDt ? P.matDt[material] : P.dt; }

struct Particles {
  double4_32a *posr, *velm, *angw, *inert, *ori, *lastPos, *bbmin, *bbmax, *force, *torque;
  // scenes with ellipsoids (else null): semi-axes (a, b, c, 0; spheres r, r, r), DemData.angMom
  // (NaN = not initialised), Aabb.nodeLastOri and Aabb.maxRot (< 0: rotation ignored)
  double4_32a *semi, *angMom, *lastOri;
  double* maxRot;
  float4* lastPosf;   // FP32 shadow of lastPos (truncated), for the verlet trigger
  double4_32a *fv1, *fv2;  // facets: nodes 1 and 2 (node 0 is posr); null when the scene has no facets
  uint8_t* touched;   // 1 when a real contact of the last contact pass involves the particle
  unsigned* rowMask;  // positions in the particle's CSR row that the last contact pass stamped: bit k for
                      // entry rowptr + k (k < 31), bit 31 for any entry from rowptr + 31 on
  unsigned* rotList;    // untouched spinning spheres, rotated by the integrator's list pass this step
  unsigned* touchList;  // particles with contact forces this step (integrated by the list pass)
  int4* meta;
  float4* posf;  // FP32 shadow of posr (x, y, z, radius), refreshed whenever posr changes
  double* energy[3];  // per-particle energy terms of this step (grav, nonviscDamp, kinetic) when tracked
};
enum { EP_GRAV = 0, EP_DAMP = 1, EP_KIN = 2 };
enum { EC_ELAST = 0, EC_PLAST = 1, EC_VISCN = 2, EC_VISCT = 3, EC_BROKEN = 4, EC_COUNT = 5 };

struct Contacts {
  int2* ids;
  uint8_t* state;
  int* step0;
  double* hist[HIST_COUNT];
  double* tanPhi;
  int2* slot;        // CSR entries of the contact: (pA's, pB's)
  uchar2* rowBit;    // the same entries as positions in their rows, min(position, 31)
  double4_32a* out;  // OUT_RECORDS records per CSR entry e: out[OUT_RECORDS * e + OUT_F / OUT_T] (capacity 2C entries)
  double* geom[7];  // optional (download): L6Geom.uN, vel (3), angVel (3); null when not kept
  double* energy[EC_COUNT];  // per-contact energy terms of this step when tracked (else null)
  int4* cdist;      // periodic: Contact.cellDist (x, y, z, unused); null otherwise
  unsigned* work;   // indices of the contacts the heavy pass processes this step (capacity = contacts)
  unsigned* act;    // contacts the cull walks until the next rebuild (not dead, not wall + wall, not far)
  double* lam;      // ellipsoid pairs: maximiser lambda of the last solve (NaN = none); null otherwise
  float* lam0;      // learned warm start of this step's solve (NaN = none); null unless used
};

struct Csr {
  int* rowptr;    // N+1
  unsigned* ent;  // 2C
  int* cursor;    // N (scratch for filling)
  unsigned long long* keys;  // 2C: the entries' sort keys, row << idBits | partner (the next rebuild's carry
                             // finds each old contact in them)
  int idBits;     // bits of a particle id in keys
  int n;          // particles the rows cover (0: no rows)
};

// Uniform-grid / sweep parameters computed on the device at each rebuild.
struct GridParams {
  int sweepAxis, ax1, ax2;
  int ncx, ncy;
  double lo1, lo2, cell;
  double loS, invQ;  // quantisation along the sweep axis
  double invCell;    // 1 / cell (column binning)
  int qbits;         // sweep key: column << qbits | quantised lower bound (qbits chosen by the host so that the
  unsigned qmax;     //   whole key fits the fewest 8-bit radix passes), qmax = 2^qbits - 1
  int nSmall;        // spheres in the sort
  int ok;
};

struct DeviceStatus {
  int code;
  int detail;
  int dirty;          // set by the integrator when a particle left its verlet box
  int overflow;
  long long haltAt;   // 0, or 1 + the step whose integrator raised the collider trigger (see haltedIntegrator)
  unsigned long long pairTotal;
  unsigned long long ellSolves, ellIters, ellFallbacks;  // ellipsoid solves / Newton iterations (Brent: evaluations) / MLP fallbacks
  unsigned workCount;  // contact work list of this step: real contacts at work[0 .. workCount)
  unsigned workPot;    //   potential pairs near touching at work[nc - workPot .. nc), in reverse
  unsigned rotCount;   // length of the rotation list of this step
  unsigned touchCount; // length of the touched-particle list of this step
  unsigned long long dynNotMin;  // DynDt: ~bits of the smallest nodal critical step^2 (0: none yet)
  unsigned actCount;   // length of the contact cull's active list
  double ext[12];     // box extents reduction scratch (as ordered ints)
  long long stepBase;  // graph replays: Scene.step of the replay's first step
  long long seqBase;   //   and the contact-pass number before it
};

#ifdef __CUDACC__
// The work list: real contacts from the front, potential pairs from the back (so that the warps of the
// FP64 pass run either the full geometry + law path or the short rejection, not both); wc points to
// DeviceStatus.workCount (followed by workPot).
__device__ __forceinline__ unsigned workLen(const unsigned* wc) { return wc[0] + wc[1]; }
__device__ __forceinline__ unsigned workItem(const unsigned* work, const unsigned* wc, long long nc, unsigned k) {
  return k < wc[0] ? work[k] : work[nc - 1 - (k - wc[0])];
}

// Steps queued ahead of the host's collider check.  The integrator of step s that raises the collider
// trigger also stores haltAt = s + 1; from then on the contact pass of step s and every kernel of the
// later steps return at once, until the host has rebuilt the pair set, cleared the trigger and run the
// contact pass of step s itself.  With one step per check (haltAt cleared before the contact pass) the
// guards never fire.  The word is read with a plain (L1-cached) load: the values that matter were
// written by earlier kernels, and a store by the running integrator (step + 1) does not halt it; a
// volatile load per warp would send every warp of the grid to the same L2 line.
// the step number and contact-pass number of the running kernel (StepParams.stepDev)
__device__ __forceinline__ long long stepOf(const StepParams& P, const DeviceStatus* st) {
  return P.stepDev ? st->stepBase + P.step : P.step;
}
__device__ __forceinline__ long long seqOf(const StepParams& P, const DeviceStatus* st) {
  return P.stepDev ? st->seqBase + P.seq : P.seq;
}
__device__ __forceinline__ bool haltedIntegrator(const DeviceStatus* st, long long step) {
  const long long h = st->haltAt;
  return h != 0 && h <= step;
}
__device__ __forceinline__ bool haltedContacts(const DeviceStatus* st, long long step) {
  const long long h = st->haltAt;
  return h != 0 && h <= step + 1;
}
#endif

// ---- launchers (k_leapfrog.cu) ----
void launch_leapfrog(cudaStream_t s, const StepParams& P, Particles p, int n, int fromArrays,
                     Contacts c, Csr csr, DeviceStatus* st);
void launch_reduce_forces(cudaStream_t s, const StepParams& P, Particles p, int n, Contacts c, Csr csr);
// DynDt: the smallest nodal critical step^2 into st->dynNotMin (as ~bits; cleared by the caller)
void launch_dyndt(cudaStream_t s, const StepParams& P, Particles p, int n, Contacts c, Csr csr, DeviceStatus* st);
void launch_state_in(cudaStream_t s, Particles p, int n, const double* pos, const double* vel, const double* angVel,
                     const double* ori);
void launch_state_out(cudaStream_t s, Particles p, int n, double* pos, double* vel, double* angVel, double* ori);
double fp64_probe(cudaStream_t s, double* scratch, int sms, float* msOut);
void launch_refresh_posf(cudaStream_t s, Particles p, int n);
// angw.w = RN(RN(m g[gravAxis]) / m), the acceleration of a particle under gravity alone
void launch_grav_acc(cudaStream_t s, const StepParams& P, Particles p, int n);
// deterministic sum of x[0..n) added to *acc (or stored, when reset): fixed-order block trees
void energy_accumulate(cudaStream_t s, const double* x, long long n, double* partials, double* acc, bool reset);
// ---- the contracted variant of k_leapfrog.cu and k_contact.cu (compiled with WDEM_FMA, wdem_variant.h):
// the same launchers, FP64 multiply-adds contracted, one reciprocal per vector division
namespace contracted {
void launch_leapfrog(cudaStream_t s, const StepParams& P, Particles p, int n, int fromArrays,
                     Contacts c, Csr csr, DeviceStatus* st);
void upload_materials(const DevMaterial* m, int n);
void launch_contacts(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc, DeviceStatus* st,
                     bool full, const uint16_t* warmBf = nullptr, const float* warmF = nullptr);
void launch_init_uploaded(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc);
}  // namespace contracted
// ---- launchers (k_contact.cu) ----
void upload_materials(const DevMaterial* m, int n);
// warm: BF16 and FP32 weights of the learned warm start, run between the cull and the FP64 pass (or null)
void launch_contacts(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc, DeviceStatus* st,
                     bool full, const uint16_t* warmBf = nullptr, const float* warmF = nullptr);
void launch_init_uploaded(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc);
// ---- collider (k_collider.cu) ----
struct ColliderScratch {
  unsigned long long *keys, *keysAlt;   // sort keys (particles, then CSR entries)
  unsigned *vals, *valsAlt;             // sort payloads
  long long sortCap;                    // capacity of the four sort arrays
  unsigned* hist;                       // radix histograms (+1 for the scan total)
  long long histCap;
  unsigned* blockSums;                  // scan scratch
  long long blockSumsCap;
  int* cellStart;                       // maxCols + 1
  float4* srec;                         // sweep records in sort order: 2 per particle (N capacity)
  int2* sweepBuf;                       // the counting sweep's first SWEEP_BUF pairs of each thread
  long long sweepBufCap;                //   (threads)
  int maxCols;
  unsigned* counts;                     // nSmall+2 pair counts per sorted particle, scanned in place
  int* large;                           // ids of walls (unbounded boxes), grouped by scene
  int nLarge;
  int* sceneWall;                       // scene s owns large[sceneWall[s] .. sceneWall[s+1])
  int nScenes;
  GridParams* grid;
  unsigned* retainFlag;                 // old contacts retained (scanned in place)
  long long retainCap;
  float4 *periC, *periH;                // periodic: wrapped FP32 box centres / half-widths in cell order
  float4 *periCi, *periHi;              //   the same by particle id
  long long periCap;
  int2* cand;                           // periodic: FP32 candidate pairs, their exact-test flags
  int4* candPer;                        //   (scanned in place) and cellDist
  unsigned* candFlag;
  long long candCap;
  void* temp;                           // small scratch (extent reduction)
  DeviceStatus* st;                     // the handle's status word (bounded waits report there)
  long long launches;                   // kernels launched by the collider (counted on the host)
};
void launch_bboxes(cudaStream_t s, const StepParams& P, Particles p, int n);
void col_extents_and_grid(cudaStream_t s, Particles p, const int* small, int nSmall, ColliderScratch& cs);
void col_sort(cudaStream_t s, Particles p, const int* small, int nSmall, ColliderScratch& cs);
long long radix_scratch_words(long long n);  // radix-sort scratch (cs.hist) for n keys
void col_sweep(cudaStream_t s, Particles p, int nSmall, unsigned loneMask, ColliderScratch& cs, int2* out,
               long long cap, bool write, DeviceStatus* st);
// periodic collider: 3-D cell grid, FP32 candidates, exact spatialOverlapPeri, emission
void col_periodic_cand(cudaStream_t s, const StepParams& P, Particles p, const int* small, int nSmall,
                       ColliderScratch& cs, bool write);
void col_periodic_exact(cudaStream_t s, const StepParams& P, Particles p, ColliderScratch& cs, long long nCand,
                        DeviceStatus* st);
void col_periodic_emit(cudaStream_t s, ColliderScratch& cs, long long nCand, int2* out, int4* outDist, long long cap);
void col_retain_write_dist(cudaStream_t s, Contacts old, long long nOld, ColliderScratch& cs, int4* out, long long base,
                           long long cap);
// k_mlp.cu: learned warm start of the ellipsoid solve
int mlp_npad();
void mlp_unpack(const float* pub, float* pad);
void mlp_pack(const float* pad, float* pub);
cudaError_t mlp_prepare_kernels();
void mlp_to_bf16(cudaStream_t s, const float* w, uint16_t* wbf);
void mlp_launch_warm(cudaStream_t s, Particles p, Contacts c, long long nc, const unsigned* work, const unsigned* count,
                     const uint16_t* wbf, const float* wf, bool onlyFresh, DeviceStatus* st, int numSMs);
void mlp_launch_predict(cudaStream_t s, const float* X, long long n, float* Y, const uint16_t* wbf, const float* wf,
                        DeviceStatus* st);
void mlp_launch_grad(cudaStream_t s, const float* rec, const int* idx, long long n, const uint16_t* wbf, const float* wf,
                     float* grad, float* loss, DeviceStatus* st, int numSMs);
void mlp_launch_adam(cudaStream_t s, float* w, float* m, float* v, float* grad, uint16_t* wbf, float lr, float b1,
                     float b2, float c1, float c2, float eps);
// k_edit.cu: particle removal and insertion between steps
enum { EDIT_RECORDS = 9 };  // double4 records per inserted particle (posr .. torque, semi, angMom)
void launch_kill(cudaStream_t s, Particles p, int n, const int* ids, int m, const double* park, uint8_t* gone,
                 Contacts c, long long nc);
void launch_put(cudaStream_t s, Particles p, const int* ids, int m, const double4_32a* rec, const int4* meta, bool withRot);
// k_noalloc.cu: the stress sum with its scratch in a fixed device array (no allocation)
long long stress_noalloc_max_contacts();
cudaError_t noalloc_scratch(int device, void** addr);
cudaError_t launch_stress_noalloc(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc,
                                  void* scratch, double* out9);
void launch_stress(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc, double* scratch9,
                   double* partials, double* out9);
void col_retain_flags(cudaStream_t s, const StepParams& P, Particles p, Contacts old, long long nOld, ColliderScratch& cs);
void col_retain_write(cudaStream_t s, Contacts old, long long nOld, ColliderScratch& cs, int2* out, long long base,
                      long long cap);
void col_csr(cudaStream_t s, Contacts c, long long nc, int n, Csr& csr, ColliderScratch& cs);
// history carry-over with compaction: contacts that were real before the rebuild first (in emission order),
// then the others; uses the sort scratch (sized for 2 nNew) as temporary storage
long long col_carry_compact(cudaStream_t s, Particles p, Contacts neu, long long nNew, Contacts old, Csr oldCsr,
                            long long step, int nHist, ColliderScratch& cs);
// exclusive scan of a[0..n) in place; a[n] receives the total (the array holds n+1 entries)
void exclusive_scan_u32(cudaStream_t s, unsigned* a, long long n, ColliderScratch& cs);
int sort_passes_for(int nSmallBits);

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace wdem
