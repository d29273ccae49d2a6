/*
 * wdem.h -- C ABI of the GB300 DEM timestep engine (libwdem.so).
 *
 * One handle runs Woo's DEM timestep for one scene on one GPU.  It replaces the engine trio
 *   Leapfrog(reset=True) -> InsertionSortCollider([Bo1_*_Aabb]) -> ContactLoop([Cg2_*],[Cp2_*],[Law2_*])
 * that woo.utils.defaultEngines / DemField.minimalEngines return (py/utils.py:94-129 of woodem/woo).
 *
 * Conventions
 *  - Plain C structs of pointers and counts.  The caller owns every host array; the library owns
 *    all device memory and never keeps a pointer to a caller array after a call returns.
 *  - Every function returns WDEM_OK (0) or a negative WDEM_ERR_* code; wdem_last_error() gives the
 *    message.  No C++ exception crosses this boundary.
 *  - A handle is not thread-safe.  It owns one CUDA stream; calls are serialised on it.
 *  - Particle ids are indices 0..n-1 (Woo's Particle::id_t, src/dem/ParticleContainer.hpp:43).
 *  - Vectors are stored xyz-interleaved (3 doubles per item), quaternions as (w,x,y,z).
 *  - L6Geom.trsf is stored as its three columns (local x, y, z axes in global coordinates),
 *    9 doubles per contact: col0.xyz, col1.xyz, col2.xyz.
 */
#ifndef WDEM_H
#define WDEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WDEM_ABI_VERSION 2

/* ---- error codes ---------------------------------------------------------------------------- */
enum {
  WDEM_OK = 0,
  WDEM_ERR_ARG = -1,           /* invalid argument (null pointer, bad size, unknown enum) */
  WDEM_ERR_CUDA = -2,          /* a CUDA runtime call failed */
  WDEM_ERR_NAN = -3,           /* NaN force in a contact (Woo: IdealElPl.cpp:79-83 throws) */
  WDEM_ERR_OVERFLOW = -4,      /* a device table ran out of capacity and could not be regrown */
  WDEM_ERR_UNSUPPORTED = -5,   /* a functor/attribute combination the GPU engine does not implement */
  WDEM_ERR_NO_PHYS = -6,       /* no Cp2 functor for a material pair (Woo: ContactLoop.cpp:181) */
  WDEM_ERR_TOO_BIG = -7,       /* particle larger than half the periodic cell (Woo: InsertionSortCollider.cpp:286-290) */
  WDEM_ERR_TIMEOUT = -8,       /* a bounded device loop hit its iteration limit */
  WDEM_ERR_STATE = -9,         /* call out of order (e.g. step before particles were uploaded) */
  WDEM_ERR_NO_ALLOC = -10      /* the input exceeds the fixed scratch of an allocation-free entry point */
};

/* ---- enums mirroring Woo class names -------------------------------------------------------- */
/* Facet (src/dem/Facet.hpp): a triangle of three nodes; node 0 is the particle's pos, nodes 1 and 2 come in
 * wdem_particles.facetVerts; radius holds Facet.halfThick.  Facets are fixed (all DOFs blocked, no
 * velocity), contact spheres through Cg2_Facet_Sphere_L6Geom and receive no contact force from the
 * contact loop (ContactLoop::applyForceUninodal skips shapes with more than one node). */
/* Capsule (src/dem/Capsule.hpp:8-35): a cylinder of length shaft along the node's local x axis with
 * hemispherical caps; radius in wdem_particles.radius, the shaft in wdem_particles.shaft.  Capsules are
 * aspherical (they take the ellipsoids' rotation state and their laws: FrictMat + IdealElPl) and contact
 * spheres, walls and other capsules (Cg2_Sphere_Capsule_L6Geom, Cg2_Wall_Capsule_L6Geom,
 * Cg2_Capsule_Capsule_L6Geom). */
enum { WDEM_SHAPE_SPHERE = 0, WDEM_SHAPE_WALL = 1, WDEM_SHAPE_ELLIPSOID = 2, WDEM_SHAPE_FACET = 3, WDEM_SHAPE_CAPSULE = 4 };
/* Cg2_Ellipsoid_Ellipsoid_L6Geom solver: brent=True (Ellipsoid.hpp:57-59) or Newton-Raphson on dS/dlambda = 0
 * (the reference's brent=False branch, which it leaves unimplemented, Ellipsoid.cpp:311-322) */
enum { WDEM_ELL_BRENT = 0, WDEM_ELL_NEWTON = 1 };
/* initial lambda of the Newton solve: lambda0 = max(a)/(max(a)+max(b)) (the reference's draft guess,
 * Ellipsoid.cpp:314), the learned warm start, the converged lambda of the previous step, or the previous
 * step's lambda where the pair has one and the learned warm start for pairs solved for the first time */
enum { WDEM_WARM_COLD = 0, WDEM_WARM_MLP = 1, WDEM_WARM_HISTORY = 2, WDEM_WARM_HISTORY_MLP = 3 };
enum { WDEM_MAT_FRICT = 0, WDEM_MAT_HERTZ = 1 };                 /* FrictMat, HertzMat */
enum { WDEM_CP2_FRICT = 0, WDEM_CP2_HERTZ = 1 };                 /* Cp2_FrictMat_FrictPhys, Cp2_HertzMat_HertzPhys */
enum { WDEM_LAW_IDEALELPL = 0, WDEM_LAW_HERTZ_DMT = 1 };         /* Law2_L6Geom_FrictPhys_IdealElPl, Law2_L6Geom_HertzPhys_DMT */
enum { WDEM_UPDATE_PHYS_NEVER = 0, WDEM_UPDATE_PHYS_ALWAYS = 1, WDEM_UPDATE_PHYS_ONCE = 2 };
/* wdem_params.arith: the arithmetic of the contact and integrator kernels (no counterpart in the reference) */
enum { WDEM_ARITH_EXACT = 0, WDEM_ARITH_FMA = 1, WDEM_ARITH_DW = 2 };

/* DemData.flags bits (src/dem/Particle.hpp:197-200) */
enum {
  WDEM_DOF_X = 1, WDEM_DOF_Y = 2, WDEM_DOF_Z = 4, WDEM_DOF_RX = 8, WDEM_DOF_RY = 16, WDEM_DOF_RZ = 32,
  WDEM_CLUMP_CLUMPED = 64, WDEM_CLUMP_CLUMP = 128, WDEM_ENERGY_SKIP = 256, WDEM_GRAVITY_SKIP = 512,
  WDEM_TRACER_SKIP = 1024, WDEM_DAMPING_SKIP = 2048
};

/* Energy slots, in this order, returned by wdem_get_energy (names of EnergyTracker, src/core/EnergyTracker.cpp:26). */
enum {
  WDEM_E_KINETIC = 0, WDEM_E_GRAV = 1, WDEM_E_NONVISCDAMP = 2, WDEM_E_ELAST = 3, WDEM_E_PLAST = 4,
  WDEM_E_VISCN = 5, WDEM_E_VISCT = 6, WDEM_E_BROKEN = 7, WDEM_E_COUNT = 8
};

/* ---- materials: FrictMat / HertzMat attributes (src/dem/FrictMat.hpp:6-28, src/dem/Hertz.hpp:5-14) */
typedef struct wdem_material {
  int32_t kind;          /* WDEM_MAT_* */
  int32_t _pad;
  double density;        /* Material.density */
  double young;          /* ElastMat.young */
  double ktDivKn;        /* FrictMat.ktDivKn */
  double tanPhi;         /* FrictMat.tanPhi */
  double surfEnergy;     /* HertzMat.surfEnergy */
  double alpha;          /* HertzMat.alpha */
} wdem_material;

/* ---- engine + functor attributes -------------------------------------------------------------- */
typedef struct wdem_params {
  double dt;              /* Scene.dt (resolved; Scene.dtSafety*critDt when Woo's dt is NaN) */
  int64_t step;           /* Scene.step at the start of the next wdem_step */
  double gravity[3];      /* DemField.gravity */
  double distFactor;      /* DemField.distFactor (negative = 1) */
  uint32_t loneMask;      /* DemField.loneMask */
  int32_t trackEnergy;    /* Scene.trackEnergy */
  /* Leapfrog (src/dem/Leapfrog.hpp:42-61) */
  double damping;
  int32_t reset;          /* must be 1 (ForceResetter folded in) */
  int32_t kinSplit;
  /* InsertionSortCollider / AabbCollider */
  double verletDist;      /* absolute; a negative value means |verletDist| x min sphere radius (Collision.cpp:164-184) */
  /* Cg2_Any_Any_L6Geom__Base (src/dem/L6Geom.hpp:28-49) */
  int32_t noRatch;
  int32_t iniLensTouch;
  int32_t trsfRenorm;
  int32_t approxMask;
  /* ContactLoop (src/dem/ContactLoop.hpp:110-130) */
  int32_t updatePhys;     /* WDEM_UPDATE_PHYS_* */
  int32_t applyForces;
  int32_t dist00;
  /* Cp2 */
  int32_t cp2;            /* WDEM_CP2_* */
  double poisson;         /* Cp2_HertzMat_HertzPhys.poisson */
  double en;              /* Cp2_HertzMat_HertzPhys.en */
  /* Law2 */
  int32_t law;            /* WDEM_LAW_* */
  int32_t noSlip, noBreak, noFrict, iniEqlb;
  double relRollStiff, relTwistStiff, rollTanPhi;
  int32_t noAttraction;   /* Law2_L6Geom_HertzPhys_DMT.noAttraction */
  int32_t _pad;
  /* materials table */
  int32_t nMaterials;
  int32_t _pad2;
  const wdem_material* materials;
  /* Cg2_Ellipsoid_Ellipsoid_L6Geom / Cg2_Sphere_Ellipsoid_L6Geom (Ellipsoid.hpp:52-60) */
  int32_t ellSolver;      /* WDEM_ELL_* */
  int32_t brentBits;      /* Cg2_Ellipsoid_Ellipsoid_L6Geom.brentBits (default 4*sizeof(Real) = 32) */
  double newtonTol;       /* Newton: converged when |delta lambda| <= newtonTol */
  int32_t warmStart;      /* WDEM_WARM_* */
  int32_t fallbackIters;  /* MLP warm start: Newton iterations before falling back to the cold start */
  /* Batched scenes: Scene.dt of each material's scene (nMaterials values), used instead of dt for the
   * particles and contacts of that material; NULL = every particle steps with dt */
  const double* materialDt;
  /* DynDt (src/dem/DynDt.hpp:5-27) after ContactLoop in each step where it is activated as a
   * PeriodicEngine with stepPeriod = dynDtPeriod (stepModulo, initRun; Engine.cpp:170-196); 0 = no DynDt.
   * The critical step from the contact stiffnesses times dtSafety (Scene.dtSafety), capped by the
   * growth dt (1 + dynDtMaxRelInc)^(steps since the previous run), becomes Scene.dt after the step
   * (Scene.cpp:432).  Sphere and wall scenes with one dt (materialDt NULL). */
  int32_t dynDtPeriod;
  int32_t _pad3;
  double dynDtMaxRelInc;  /* DynDt.maxRelInc (default 1e-4) */
  double dtSafety;        /* Scene.dtSafety (default .9) */
  /* Arithmetic of the contact and integrator kernels (no counterpart in the reference):
   * WDEM_ARITH_EXACT (0) = the reference's IEEE FP64 operations in its order, results equal to the CPU
   * restatement bit for bit; WDEM_ARITH_FMA (1) = FP64 multiply-adds contracted into FMAs and one
   * reciprocal per division of a vector by a scalar (per-contact forces within 1e-12 relative of the exact
   * ones after one step from the same state; the collider's pair set is unchanged for the same boxes);
   * WDEM_ARITH_DW (2) = as FMA, and the update of real sphere and wall contacts (frame, law, force
   * rotation, branch torques) in double-word FP32 arithmetic of 48 significant bits, positions, overlaps,
   * contact points and the differences they cancel in kept in FP64 (the same 1e-12 bar). */
  int32_t arith;
  int32_t _pad4;
} wdem_params;

/* ---- particle state, SoA; all arrays have n (or 3n / 4n) items --------------------------------- */
typedef struct wdem_particles {
  int32_t n;
  int32_t _pad;
  int32_t* shape;         /* WDEM_SHAPE_* */
  double* radius;         /* Sphere.radius (unused for walls) */
  int32_t* wallAxis;      /* Wall.axis (unused for spheres) */
  int32_t* wallSense;     /* Wall.sense */
  int32_t* material;      /* index into wdem_params.materials */
  uint32_t* mask;         /* Particle.mask */
  uint32_t* flags;        /* DemData.flags */
  double* mass;           /* DemData.mass */
  double* inertia;        /* 3n DemData.inertia */
  double* pos;            /* 3n Node.pos */
  double* ori;            /* 4n Node.ori (w,x,y,z) */
  double* vel;            /* 3n DemData.vel */
  double* angVel;         /* 3n DemData.angVel */
  double* force;          /* 3n DemData.force */
  double* torque;         /* 3n DemData.torque */
  double* semiAxes;       /* 3n Ellipsoid.semiAxes (NULL when there are no ellipsoids) */
  double* angMom;         /* 3n DemData.angMom, NaN = not initialised (aspherical Leapfrog); may be NULL */
  int32_t* scene;         /* batched independent scenes: scene index of each particle (0..4095); particles of
                             different scenes never interact; NULL = one scene */
  double* facetVerts;     /* 9n: Facet node positions 0, 1, 2 (node 0 equal to pos); NULL when there are no facets */
  double* shaft;          /* n: Capsule.shaft; NULL when there are no capsules */
} wdem_particles;

/* ---- contact state, SoA; n contacts ---------------------------------------------------------- */
typedef struct wdem_contacts {
  int64_t n;
  int32_t* idA;           /* Contact.pA id */
  int32_t* idB;           /* Contact.pB id */
  int32_t* real;          /* Contact.isReal(): geom && phys */
  int32_t* stepCreated;   /* Contact.stepCreated */
  double* minDist00Sq;    /* Contact.minDist00Sq */
  double* trsf;           /* 9n L6Geom.trsf columns */
  double* contPt;         /* 3n L6Geom.node.pos */
  double* geomOri;        /* 4n L6Geom.node.ori, download only */
  double* geomVel;        /* 3n L6Geom.vel, download only */
  double* geomAngVel;     /* 3n L6Geom.angVel, download only */
  double* uN;             /* L6Geom.uN, download only */
  double* force;          /* 3n CPhys.force (local) */
  double* torque;         /* 3n CPhys.torque (local) */
  double* kn;             /* FrictPhys.kn */
  double* kt;             /* FrictPhys.kt */
  double* tanPhi;          /* FrictPhys.tanPhi */
  int32_t* cellDist;       /* 3n Contact.cellDist (periodic cell offset of pB) */
} wdem_contacts;

/* ---- periodic cell (Cell, src/core/Cell.hpp:22-187), row-major 3x3 matrices ---------------------- */
typedef struct wdem_cell {
  int32_t periodic;        /* Scene.isPeriodic */
  int32_t homoDeform;      /* Cell.homoDeform; only 4 (HOMO_GRADV2, the default) is supported */
  double hSize[9];         /* Cell.hSize (columns = cell base vectors) */
  double trsf[9];          /* Cell.trsf */
  double gradV[9];         /* Cell.gradV (at t - dt/2) */
  double nextGradV[9];     /* Cell.nextGradV (applied from the next step) */
  double pprevHsize[9];    /* Cell.pprevHsize, output only */
} wdem_cell;

/* ---- status ----------------------------------------------------------------------------------- */
typedef struct wdem_status {
  int32_t code;            /* first error seen on the device, or WDEM_OK */
  int32_t detail;          /* e.g. particle id of a NaN or oversized particle */
  int64_t step;            /* Scene.step after the last wdem_step */
  int64_t nContacts;       /* contacts in the container (real + potential) */
  int64_t nReal;           /* real contacts */
  int64_t nFullRuns;       /* collider rebuilds since creation (InsertionSortCollider.nFullRuns) */
  int64_t capacity;        /* current contact capacity */
  int32_t lastRunFull;     /* 1 if the last step rebuilt the collider */
  int32_t _pad;
  int64_t ellSolves;       /* ellipsoid contact-function maximisations since creation */
  int64_t ellIters;        /* their Newton iterations (Brent: function evaluations) */
  int64_t ellFallbacks;    /* learned warm starts that fell back to the cold start */
  double dt;               /* Scene.dt for the next step (DynDt may have changed it) */
  double dynDtCrit;        /* critical step of DynDt's last run (DynDt::critDt_stiffness), NaN before */
  double timeSum;          /* sum of dt over the steps run by this handle (Scene.time advances by it) */
} wdem_status;

typedef struct wdem_handle wdem_handle;

/* Library ABI version (WDEM_ABI_VERSION).  No counterpart in the reference, whose engines live in the
 * same binary as the Python module; a binding checks it once after loading the library. */
int wdem_abi_version(void);

/* Create a handle for up to maxParticles particles on CUDA device `device`.
 * Replaces constructing Leapfrog + InsertionSortCollider + ContactLoop and appending them to
 * Scene.engines (py/utils.py:122-129; engine base src/core/Engine.hpp:19-104). */
int wdem_create(int device, int32_t maxParticles, wdem_handle** out);

/* Release all device memory and the stream; replaces removing the three engines from Scene.engines
 * (their destructors, src/core/Engine.hpp:19-104). */
int wdem_destroy(wdem_handle* h);

/* Set engine/functor attributes (Leapfrog, InsertionSortCollider, ContactLoop, Cg2/Cp2/Law2 attrs,
 * DemField.gravity/distFactor/loneMask, Scene.dt/step).  Mirrors setting those attributes from
 * Python (src/dem/ContactLoop.cpp:52-66 functor lists; attrs in the *.hpp CLASS_BASE_DOC_ATTRS). */
int wdem_set_params(wdem_handle* h, const wdem_params* p);

/* Upload particle state.  Marks the contact container dirty, so the next step rebuilds the
 * collider from scratch, as after ContactContainer.clear() / prologue_doFullRun
 * (src/dem/InsertionSortCollider.cpp:360-384). */
int wdem_upload_particles(wdem_handle* h, const wdem_particles* p);

/* Upload the contact container (real contacts with their L6Geom/FrictPhys history and potential
 * contacts).  Replaces ContactContainer::add for each contact (src/dem/ContactContainer.cpp:18-38). */
int wdem_upload_contacts(wdem_handle* h, const wdem_contacts* c);

/* Run nSteps steps of Leapfrog -> collider -> ContactLoop; replaces Scene::doOneStep's engine loop
 * (src/core/Scene.cpp:420-427) for the three engines.  Scene.step advances by nSteps. */
int wdem_step(wdem_handle* h, int32_t nSteps);

/* Download particle state (pos, ori, vel, angVel, force, torque; the other arrays may be null).
 * force/torque are DemData.force/torque as Woo has them after ContactLoop: m*g + contact forces. */
int wdem_download_particles(wdem_handle* h, wdem_particles* p);

/* Number of contacts in the container (real + potential), as len(S.dem.con)
 * (ContactContainer.__len__, src/dem/ContactContainer.hpp:61,121). */
int wdem_contact_count(wdem_handle* h, int64_t* n);

/* Download the contact container; c->n must be >= wdem_contact_count.  Contacts come sorted by
 * (min id, max id).  Null arrays are skipped.  Replaces iterating S.dem.con from Python
 * (ContactContainer::pyIter / pyNth, src/dem/ContactContainer.cpp:219-233). */
int wdem_download_contacts(wdem_handle* h, wdem_contacts* c);

/* Critical timestep of the field, DemFuncs::pWaveDt (src/dem/Funcs.cpp:151-175), via DemField::critDt
 * (src/dem/Particle.cpp:399-404): min over spheres of r/sqrt(E/rho). */
int wdem_crit_dt(wdem_handle* h, double* dt);

/* Energies accumulated since the last reset, in WDEM_E_* order: the entries ContactLoop and Leapfrog
 * add to Scene.energy (EnergyTracker::add, src/core/EnergyTracker.hpp:29-61; Scene.energy
 * src/core/Scene.hpp:223).  wdem_reset_energy is EnergyTracker.clear (EnergyTracker.hpp:60). */
int wdem_get_energy(wdem_handle* h, double* e, int32_t n);
int wdem_reset_energy(wdem_handle* h);

/* Device status: the first error flagged by any kernel, counters.  Like Woo's exceptions surfacing
 * as RuntimeError after the engine run (src/core/Scene.cpp:91-118). */
int wdem_get_status(wdem_handle* h, wdem_status* s);

/* Message of the last error on this handle (valid until the next call). */
const char* wdem_last_error(wdem_handle* h);

/* Collider alone: compute the candidate pair set for the given axis-aligned boxes, as
 * InsertionSortCollider's initial sort + sweep does (src/dem/InsertionSortCollider.cpp:536-605)
 * with the closed-interval test spatialOverlap (:67-73) and Collider::mayCollide
 * (src/dem/Collision.cpp:21-43).  Boxes may hold +-inf (walls).  Pairs are written as
 * (min id, max id), sorted; *nPairs gets the count; at most maxPairs are written. */
int wdem_collide_boxes(wdem_handle* h, int32_t n, const double* mins, const double* maxs,
                       const uint32_t* mask, uint32_t loneMask,
                       int32_t* pairs, int64_t maxPairs, int64_t* nPairs);

/* Per-kernel device time of the last wdem_step call, in milliseconds, summed over its steps.
 * Counterpart of Engine.execTime / execCount under Master.timingEnabled (src/core/Engine.hpp:92-93),
 * per kernel instead of per engine.
 * names[i] (static strings) and ms[i], up to n entries; *count gets the number of entries. */
int wdem_kernel_times(wdem_handle* h, const char** names, double* ms, int32_t* launches, int32_t n, int32_t* count);

/* Enable/disable per-kernel CUDA-event timing inside wdem_step (off by default), as
 * Master.timingEnabled switches Engine.execTime accounting (src/core/Engine.hpp:92-94). */
int wdem_set_timing(wdem_handle* h, int32_t enable);

/* Steps that wdem_step may queue on the device before it checks the collider trigger on the host
 * (default 32; 0 or 1 = check after every integrator pass).  Queued kernels guard themselves: once
 * the integrator of a step raises the trigger, the rest of the queue does nothing, and the host
 * rebuilds and finishes that step exactly as with one step per check, so results do not depend on
 * the depth.  No counterpart in the reference, whose loop checks in every step
 * (InsertionSortCollider::run, InsertionSortCollider.cpp:386-400). */
int wdem_set_queue_depth(wdem_handle* h, int32_t depth);

/* How the queued steps reach the GPU: WDEM_GRAPHS_OFF (default) launches every kernel of the queue
 * from the host; WDEM_GRAPHS_ON captures the queue's kernels once as a CUDA graph and launches that
 * graph for every later queue with the same launch arguments (same parameters, arrays and contact
 * count; a rebuild or an upload captures again); WDEM_GRAPHS_AUTO captures only when at least eight
 * replays are expected before the next collider rebuild.  Results do not depend on the mode.  No
 * counterpart in the reference, whose Scene::doOneStep calls each engine's run() in turn
 * (src/core/Scene.cpp:420-426). */
enum { WDEM_GRAPHS_OFF = 0, WDEM_GRAPHS_AUTO = 1, WDEM_GRAPHS_ON = 2 };
int wdem_set_step_graphs(wdem_handle* h, int32_t mode);

/* Graph captures and graph launches of queued steps since the handle was created. */
int wdem_graph_stats(wdem_handle* h, int64_t* captures, int64_t* replays);

/* Keep L6Geom.uN, L6Geom.vel and L6Geom.angVel of every real contact so that
 * wdem_download_contacts can return them (off by default: they are per-step values that Woo keeps
 * in the contact's CGeom object, L6Geom.vel/angVel/uN at src/dem/L6Geom.hpp:16-18; storing them
 * costs 56 bytes per contact per step). */
int wdem_keep_geom(wdem_handle* h, int32_t enable);

/* Periodic cell: Scene.isPeriodic + Cell.hSize/trsf/gradV/nextGradV (src/core/Cell.hpp:22-187), set
 * like Cell.setHSize and Cell.nextGradV from Python; homoDeform gradV2 only.  Call after
 * wdem_upload_particles and before wdem_upload_contacts.  The cell advances every step
 * (Cell::integrateAndUpdate at the start, Cell::setNextGradV at the end, src/core/Scene.cpp:411,430). */
int wdem_set_cell(wdem_handle* h, const wdem_cell* c);
int wdem_get_cell(wdem_handle* h, wdem_cell* c);

/* Stress tensor of the contact network, row-major 3x3: sum over real contacts of the global contact
 * force times the branch vector (pB image - pA) divided by the cell volume (ContactLoop.evalStress,
 * src/dem/ContactLoop.cpp:218-229, 243-244); volume 1 for aperiodic scenes. */
int wdem_get_stress(wdem_handle* h, double* stress);

/* ---- learned warm start of the ellipsoid solve (no counterpart in the reference) -------------------
 * A 13 -> 64 -> 64 -> 64 -> 4 ReLU network, BF16 on the tensor cores with FP32 accumulation, predicts
 * the maximiser lambda of the Perram-Wertheim contact function (and the contact point) of an ellipsoid
 * pair from WDEM_WARM_INPUTS features; with warmStart = WDEM_WARM_MLP its lambda starts the Newton solve,
 * which falls back to the cold start after fallbackIters iterations.  A record is the features followed
 * by the solver's converged lambda and contact point (WDEM_WARM_RECORD floats): features = centre offset
 * of B in A's frame (3), orientation of B relative to A with w >= 0 (4), semi-axes of A (3) and of B (3),
 * lengths divided by max(a) + max(b); targets = lambda, contact point in A's frame / (max(a) + max(b)).
 * Weights (WDEM_WARM_NPARAM floats): W1 (13 x 64, row = input), b1 (64), W2 (64 x 64), b2, W3, b3,
 * W4 (64 x 4), b4 (4). */
#define WDEM_WARM_INPUTS 13
#define WDEM_WARM_OUTPUTS 4
#define WDEM_WARM_RECORD 17
#define WDEM_WARM_NPARAM 9476
int wdem_warm_init(wdem_handle* h, uint64_t seed);                     /* He-uniform weights, zero biases */
int wdem_warm_set_weights(wdem_handle* h, const float* w, int64_t n);  /* n == WDEM_WARM_NPARAM */
int wdem_warm_get_weights(wdem_handle* h, float* w, int64_t n);
/* outputs (n x 4) of feature rows (n x 13) */
int wdem_warm_predict(wdem_handle* h, const float* x, int64_t n, float* y);
/* gradient (WDEM_WARM_NPARAM) and value of the mean weighted squared error over n records
 * (output weights 1, 0.1, 0.1, 0.1) */
int wdem_warm_grad(wdem_handle* h, const float* records, int64_t n, float* grad, float* loss);
/* Adam training on n records: epochs over a seeded shuffle, mini-batches of `batch`, learning rate lr
 * decayed along a half cosine to lr/100 over the run; lossPerEpoch (epochs floats, may be NULL)
 * receives the mean training loss of each epoch. */
int wdem_warm_train(wdem_handle* h, const float* records, int64_t n, int32_t epochs, int32_t batch, float lr,
                    uint64_t seed, float* lossPerEpoch);
/* Log a record for every ellipsoid pair solved in the following steps, up to capRecords (0 stops and
 * frees the log); wdem_ell_log_read copies up to cap logged records out and sets *n. */
int wdem_ell_log(wdem_handle* h, int64_t capRecords);
int wdem_ell_log_read(wdem_handle* h, float* out, int64_t cap, int64_t* n);

/* wdem_get_stress without any device memory allocation.  No counterpart in the reference: it exists
 * for callers that must not touch the CUDA allocator at the moment they ask for the stress, e.g. a
 * controller running between steps of a serving loop whose memory is fully reserved up front, where
 * cudaMalloc can fail, or where the implicit device-wide synchronisation of cudaFree would stall other
 * streams.  wdem_get_stress grows per-handle buffers on demand; this call instead uses one fixed
 * 295,424-byte array in device memory, shared by all handles of the library on a device.
 * - at most 16,777,216 contacts (WDEM_ERR_NO_ALLOC beyond that; wdem_get_stress has no such limit);
 * - the result equals wdem_get_stress up to the order of the additions (relative ~1e-15), and is
 *   itself deterministic;
 * - the first call on each device looks the array's address up (this may load the module): make that
 *   first call before capturing any stream;
 * - the array is shared: calls that overlap in time on one device (several host threads, or handles
 *   on different streams) race on it and give undefined results; serialise them per device.
 * Synchronises the handle's stream before returning. */
int wdem_get_stress_noalloc(wdem_handle* h, double* stress);

/* Remove particles between steps, on the device (DemField::removeParticle, src/dem/Particle.cpp:483-530,
 * as Outlet::run calls it, src/dem/Outlet.cpp:15-116): the m slots `ids` become inert (mask 0, so that
 * Collider::mayCollide never pairs them; all DOFs blocked; zero velocity) and are parked at park[3k..3k+2]
 * when park is not NULL; every contact of a removed particle dies with its history.  The forces of the step
 * just run (removed contacts included, as the reference applied them before the outlet ran) are kept for the
 * next integration; the collider runs in full at the next step.  Only the ids, the park positions and the
 * contact states are touched: nothing is copied back to the host. */
int wdem_remove_particles(wdem_handle* h, int32_t m, const int32_t* ids, const double* park);

/* Insert particles between steps, on the device (particles added by RandomInlet::run,
 * src/dem/Inlet.cpp:228-515): the p->n particles of p go to the slots ids[0 .. p->n) -- slots of removed
 * particles (below the current count) or new slots that extend the particle count contiguously, up to the
 * handle's capacity.  Spheres and ellipsoids (the latter when the handle already holds ellipsoids); walls
 * go through wdem_upload_particles.  The other particles and the contact container stay on the device; the
 * collider runs in full at the next step. */
int wdem_add_particles(wdem_handle* h, const wdem_particles* p, const int32_t* ids);

/* Launch shape of the step kernels (no counterpart in the reference, which has none): threads per block of
 * the contact pass's FP64 kernel (64, 128, 256), its resident blocks per SM (0 = as many as fit), threads
 * per block of the contact cull (128, 256, 512) and of the integrator's first pass (128, 256, 512), blocks
 * per SM of the integrator's list pass (0 = as many as fit).  Results do not depend on the shape (every
 * contact and particle is computed alone; sums run in fixed orders): only the speed does. */
typedef struct wdem_launch_shape {
  int32_t contactsBlock;
  int32_t contactsPerSM;
  int32_t cullBlock;
  int32_t integratorBlock;
  int32_t listsPerSM;
  int32_t _pad;
} wdem_launch_shape;
int wdem_set_launch_shape(wdem_handle* h, const wdem_launch_shape* shape);
int wdem_get_launch_shape(wdem_handle* h, wdem_launch_shape* shape);

/* Autotuner of the launch shape (no counterpart in the reference): runs the simulation forward, each
 * candidate shape for stepsPerCandidate steps (after 2 untimed ones) with the per-phase CUDA-event times of
 * the integrator and the contact pass as its cost, by coordinate descent over the five knobs starting from
 * the current shape; keeps and returns the fastest shape and its cost and that of the starting shape (ms per
 * step).  The run advances by the steps it takes (results are those of the same steps run untuned). */
int wdem_autotune(wdem_handle* h, int32_t stepsPerCandidate, wdem_launch_shape* best, double* msBest, double* msStart);

/* Upper bound on the contact container (real and potential pairs) for callers that budget device memory;
 * 0 (the default) = grow as needed.  No counterpart in the reference, whose container grows without
 * bound.  A collider run or a contact upload that needs more than maxContacts stops with
 * WDEM_ERR_OVERFLOW before it allocates or changes the container; the step that hit the limit is left
 * half done (its integrator ran), so the caller re-uploads the state (or raises the limit and restarts
 * from its own copy) before stepping on. */
int wdem_set_contact_limit(wdem_handle* h, int64_t maxContacts);

/* The CUDA stream (cudaStream_t) every kernel of this handle is launched on, for callers that
 * record CUDA events around wdem_step.  No counterpart in the reference (CPU only). */
int wdem_get_stream(wdem_handle* h, void** stream);

/* Overwrite / read the kinematic state of the first n particles in place, without touching the
 * contact container (as editing S.dem.par[i].pos/vel/angVel between steps in Woo: the Particle
 * properties of src/dem/Particle.hpp:100-104).  Caller host buffers
 * (pinned memory gives full copy bandwidth); null arrays are skipped; pos/vel/angVel are 3n, ori 4n. */
int wdem_write_state(wdem_handle* h, int32_t n, const double* pos, const double* vel, const double* angVel,
                     const double* ori);
int wdem_read_state(wdem_handle* h, int32_t n, double* pos, double* vel, double* angVel, double* ori);

/* Measured FP64 fused-multiply-add throughput of the device in GFLOP/s (2 flops per FMA): the
 * ceiling of the FP64-issue-bound kernels, reported beside the HBM roofline.  No counterpart in the
 * reference. */
int wdem_fp64_peak(wdem_handle* h, double* gflops);

/* Number of CUDA kernels launched by the library in this process (every launch site counts).  No
 * counterpart in the reference. */
int wdem_launch_count(wdem_handle* h, int64_t* count);

/* Seeded random sequential addition of n non-overlapping spheres, radii uniform in [rMin, rMax],
 * inside the box [lo, hi]: the synthetic-input counterpart of Woo's SpherePack::makeCloud
 * (src/supp/sphere-pack/SpherePack.cpp:140-).  Host only, no GPU needed.  Returns the number placed
 * (<= n; largest radii first) or a negative WDEM_ERR_*. */
int64_t wdem_make_cloud(const double* lo, const double* hi, double rMin, double rMax, int64_t n, uint64_t seed,
                        int32_t maxAttempts, double* centers, double* radii);
/* The same for n caller-given radii rIn (placed largest first); periodic != 0 fills the periodic box
 * [lo, hi) with no overlap across its faces either (nearest-image test). */
int64_t wdem_make_cloud_radii(const double* lo, const double* hi, int32_t periodic, int64_t n, const double* rIn,
                              uint64_t seed, int32_t maxAttempts, double* centers, double* radii);

#ifdef __cplusplus
}
#endif
#endif /* WDEM_H */
