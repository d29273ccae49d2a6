// k_collider.cu -- GPU collider for the DEM engine: the GB300 replacement of Woo's
// InsertionSortCollider (src/dem/InsertionSortCollider.cpp:386-613) and AabbCollider's verlet
// boxes (src/dem/Collision.cpp:80-184).
//
// A rebuild runs whenever a particle left its verlet box (aabbIsDirty).  It produces the same
// candidate set as the reference collider on the same boxes: every pair whose closed boxes overlap
// on all three axes (spatialOverlap, InsertionSortCollider.cpp:67-73) and that mayCollide
// (Collision.cpp:21-43), plus every real contact carried over from before (the reference never
// removes real contacts in the collider).  Instead of an incremental insertion sort, the rebuild
//   1. sorts small particles by (grid column in the two long axes, quantised box minimum along the
//      shortest axis) with an LSD radix sort written here (one kernel per digit, decoupled look-back),
//   2. sweeps each particle forward along the sweep axis in its own and the 8 neighbouring columns,
//      testing the exact FP64 closed-interval overlap (grid cell >= widest box, so no pair is missed),
//   3. tests walls, facets and other large boxes against every particle of their scene,
//   4. writes the pairs in a deterministic order (count pass with each particle's first pairs buffered,
//      exclusive scan, write pass),
//   5. carries contact history over, finding each pair's old contact by a binary search in the old
//      CSR's sorted keys (row of the lower id, keyed by the partner),
//   6. builds the per-particle contact CSR with rows ordered by the partner id.
#include "wdem_internal.h"
#include "wdem_math.cuh"
#include "wdem_peri.cuh"
#include "../../include/wdem.h"
#include <cstdio>

namespace wdem {

// columns of the sweep grid at most (keys of 20 column bits and 12 or more quantisation bits: 4 radix passes)
static const int SWEEP_MAX_COLS = (1 << 20) - 2;

// ------------------------------------------------------------------------------------------ boxes
// Bo1_Sphere_Aabb::go / Bo1_Wall_Aabb::go + AabbCollider::updateAabb: pos +- bboxFactor*r,
// walls unbounded except along their axis; both enlarged by verletDist; nodeLastPos = pos.
__global__ void k_bboxes(StepParams P, Particles p, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4_32a pr = p.posr[i];
  int sh = p.meta[i].x & 15;
  double4_32a mn, mx;
  if (sh == WDEM_SHAPE_SPHERE) {
    double h = P.bboxFactor * pr.w;
    if (!P.periodic) {
      mn = make_double4_32a(pr.x - h, pr.y - h, pr.z - h, 0);
      mx = make_double4_32a(pr.x + h, pr.y + h, pr.z + h, 0);
    } else {
      // periodic (Sphere.cpp:66-81): unsheared centre, extents enlarged by Cell::shearAlignedExtents
      double hx = h, hy = h, hz = h;
      if (P.hasShear) {
        double e[3] = {h, h, h};
        for (int ax = 0; ax < 3; ax++) {
          int ax1 = (ax + 1) % 3, ax2 = (ax + 2) % 3;
          e[ax1] = e[ax1] + .5 * h * P.sae[ax];
          e[ax2] = e[ax2] + .5 * h * P.sae[ax];
        }
        hx = e[0]; hy = e[1]; hz = e[2];
      }
      const d3 c = mvec(P.unsh, mk(pr.x, pr.y, pr.z));
      mn = make_double4_32a(c.x - hx, c.y - hy, c.z - hz, 0);
      mx = make_double4_32a(c.x + hx, c.y + hy, c.z + hz, 0);
    }
  } else if (sh == WDEM_SHAPE_ELLIPSOID) {
    // Bo1_Ellipsoid_Aabb::go (Ellipsoid.cpp:97-107): half-extents = row norms of trsfFromUnitSphere
    const double4_32a sa = p.semi[i], o4 = p.ori[i];
    qd q;
    q.w = o4.x; q.x = o4.y; q.y = o4.z; q.z = o4.w;
    const d3 c0 = qrot(q, mk(sa.x, 0, 0)), c1 = qrot(q, mk(0, sa.y, 0)), c2 = qrot(q, mk(0, 0, sa.z));
    const double hx = sqrt(c0.x * c0.x + c1.x * c1.x + c2.x * c2.x);
    const double hy = sqrt(c0.y * c0.y + c1.y * c1.y + c2.y * c2.y);
    const double hz = sqrt(c0.z * c0.z + c1.z * c1.z + c2.z * c2.z);
    mn = make_double4_32a(pr.x - hx, pr.y - hy, pr.z - hz, 0);
    mx = make_double4_32a(pr.x + hx, pr.y + hy, pr.z + hz, 0);
  } else if (sh == WDEM_SHAPE_CAPSULE) {
    // Bo1_Capsule_Aabb::go (Capsule.cpp:97-114) with Capsule::alignedBox (:67-73): the box of the four points
    // pos +- dShaft +- radius (1,1,1), dShaft = ori (shaft/2, 0, 0), min/max as Eigen's AlignedBox::extend
    const double4_32a cs = p.semi[i], o4 = p.ori[i];
    qd q;
    q.w = o4.x; q.x = o4.y; q.y = o4.z; q.z = o4.w;
    const d3 ds = qrot(q, mk(.5 * cs.y, 0, 0));
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    mn = make_double4_32a(inf, inf, inf, 0);
    mx = make_double4_32a(-inf, -inf, -inf, 0);
    for (int sa = -1; sa <= 1; sa += 2)
      for (int sb = -1; sb <= 1; sb += 2) {
        const double br = (double)sb * cs.x;
        const d3 e = mk(pr.x, pr.y, pr.z) + (double)sa * ds;
        const double x = e.x + br, y = e.y + br, z = e.z + br;
        mn.x = (x < mn.x) ? x : mn.x; mn.y = (y < mn.y) ? y : mn.y; mn.z = (z < mn.z) ? z : mn.z;
        mx.x = (mx.x < x) ? x : mx.x; mx.y = (mx.y < y) ? y : mx.y; mx.z = (mx.z < z) ? z : mx.z;
      }
  } else if (sh == WDEM_SHAPE_FACET) {
    // Bo1_Facet_Aabb::go (Facet.cpp:275-298), aperiodic: the three nodes +- halfThick (posr.w), coefficient-wise
    // min/max in the order of Eigen's array().min()/max() (std::min/std::max semantics)
    const double ht = pr.w;
    mn = make_double4_32a(pr.x - ht, pr.y - ht, pr.z - ht, 0);
    mx = make_double4_32a(pr.x + ht, pr.y + ht, pr.z + ht, 0);
    const double4_32a v[2] = {p.fv1[i], p.fv2[i]};
    for (int k = 0; k < 2; k++) {
      const double lx = v[k].x - ht, ly = v[k].y - ht, lz = v[k].z - ht;
      const double ux = v[k].x + ht, uy = v[k].y + ht, uz = v[k].z + ht;
      mn.x = (lx < mn.x) ? lx : mn.x; mn.y = (ly < mn.y) ? ly : mn.y; mn.z = (lz < mn.z) ? lz : mn.z;
      mx.x = (mx.x < ux) ? ux : mx.x; mx.y = (mx.y < uy) ? uy : mx.y; mx.z = (mx.z < uz) ? uz : mx.z;
    }
  } else {
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    int ax = (p.meta[i].x >> 4) & 3;
    mn = make_double4_32a(-inf, -inf, -inf, 0);
    mx = make_double4_32a(inf, inf, inf, 0);
    double c = ax == 0 ? pr.x : (ax == 1 ? pr.y : pr.z);
    if (ax == 0) { mn.x = c; mx.x = c; } else if (ax == 1) { mn.y = c; mx.y = c; } else { mn.z = c; mx.z = c; }
  }
  if (p.maxRot) {
    // Aabb.maxRot: -1 (ignored) for spheres and walls; ellipsoids start at 0 and get
    // atan(verletDist / largest half-extent) when verletDist > 0 (Collision.cpp:152-158)
    double mr = -1.;
    if (sh == WDEM_SHAPE_ELLIPSOID || sh == WDEM_SHAPE_CAPSULE) {
      mr = 0.;
      if (P.verletDist > 0) {
        const double arm = .5 * dmax3(mk(mx.x - mn.x, mx.y - mn.y, mx.z - mn.z));
        mr = (arm > 0.) ? atan(P.verletDist / arm) : 0.;
      }
    }
    p.maxRot[i] = mr;
    p.lastOri[i] = p.ori[i];
  }
  if (P.verletDist > 0) {
    double vd = P.verletDist;
    mx.x = mx.x + vd; mx.y = mx.y + vd; mx.z = mx.z + vd;
    mn.x = mn.x - vd; mn.y = mn.y - vd; mn.z = mn.z - vd;
  }
  p.bbmin[i] = mn;
  p.bbmax[i] = mx;
  p.lastPos[i] = make_double4_32a(pr.x, pr.y, pr.z, 0);
  if (p.lastPosf) p.lastPosf[i] = make_float4(truncF(pr.x), truncF(pr.y), truncF(pr.z), 0.f);
}

void launch_bboxes(cudaStream_t s, const StepParams& P, Particles p, int n) {
  if (n <= 0) return;
  (k_bboxes<<<(n + 255) / 256, 256, 0, s>>>(P, p, n), ++::wdem::g_kernel_launches);
}

// ------------------------------------------------------------------------------------ grid setup
// Order-preserving map double -> unsigned 64 for atomic min/max.
__device__ __forceinline__ unsigned long long ordKey(double d) {
  unsigned long long u = (unsigned long long)__double_as_longlong(d);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double ordVal(unsigned long long k) {
  unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

// ext layout (ordered keys): [0..2] min centre, [3..5] max centre (stored as ~key for max via min),
// [6..8] min box lower bound, [9..11] max box upper bound, [12..14] max box width
struct ExtAcc { unsigned long long v[15]; };

__global__ void k_extents_init(unsigned long long* ext) {
  int t = threadIdx.x;
  if (t < 15) ext[t] = ~0ull;  // all stored as "min" accumulators
}

__global__ void k_extents(Particles p, const int* small, int nSmall, unsigned long long* ext) {
  __shared__ unsigned long long sh[15];
  if (threadIdx.x < 15) sh[threadIdx.x] = ~0ull;
  __syncthreads();
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nSmall) {
    int i = small[k];
    double4_32a pr = p.posr[i];
    double4_32a mn = p.bbmin[i], mx = p.bbmax[i];
    double c[3] = {pr.x, pr.y, pr.z};
    double lo[3] = {mn.x, mn.y, mn.z};
    double hi[3] = {mx.x, mx.y, mx.z};
    for (int a = 0; a < 3; a++) {
      atomicMin(&sh[a], ordKey(c[a]));
      atomicMin(&sh[3 + a], ~ordKey(c[a]));
      atomicMin(&sh[6 + a], ordKey(lo[a]));
      atomicMin(&sh[9 + a], ~ordKey(hi[a]));
      atomicMin(&sh[12 + a], ~ordKey(hi[a] - lo[a]));
    }
  }
  __syncthreads();
  if (threadIdx.x < 15) atomicMin(&ext[threadIdx.x], sh[threadIdx.x]);
}

__global__ void k_grid_setup(const unsigned long long* ext, int nSmall, int maxCols, int qbits, GridParams* g) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  GridParams G;
  G.nSmall = nSmall;
  G.qbits = qbits;
  G.qmax = (1u << qbits) - 1;
  if (nSmall == 0) { G.ok = 0; G.sweepAxis = 0; G.ax1 = 1; G.ax2 = 2; G.ncx = G.ncy = 1; G.lo1 = G.lo2 = 0; G.cell = 1; G.invCell = 1; G.loS = 0; G.invQ = 0; *g = G; return; }
  double cmin[3], cmax[3], bmin[3], bmax[3], w[3];
  for (int a = 0; a < 3; a++) {
    cmin[a] = ordVal(ext[a]);
    cmax[a] = ordVal(~ext[3 + a]);
    bmin[a] = ordVal(ext[6 + a]);
    bmax[a] = ordVal(~ext[9 + a]);
    w[a] = ordVal(~ext[12 + a]);
  }
  // the sweep runs along the shortest extent of the box centres and the columns tile the two longest: the
  // most columns for the cap, so the fewest boxes per column and the shortest binary searches into them
  // (a row of batched scenes along one axis would otherwise put all scenes into the same few long columns)
  int ax = 0;
  for (int a = 1; a < 3; a++) if (cmax[a] - cmin[a] < cmax[ax] - cmin[ax]) ax = a;
  int a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
  double W = fmax(w[a1], w[a2]);
  double cell = W * (1.0 + 1e-6) + 1e-300;
  double e1 = cmax[a1] - cmin[a1], e2 = cmax[a2] - cmin[a2];
  // cap the column count; a larger cell stays correct (only the cell >= W bound matters)
  for (int it = 0; it < 64; it++) {
    double n1 = floor(e1 / cell) + 1, n2 = floor(e2 / cell) + 1;
    if (n1 * n2 <= (double)maxCols) break;
    cell *= 1.25;
  }
  // non-finite extents (NaN or infinite positions) or a grid still too fine: one column
  if (!(e1 >= 0 && e2 >= 0 && e1 < 1e300 && e2 < 1e300 && cell > 0 && cell < 1e300) ||
      (floor(e1 / cell) + 1) * (floor(e2 / cell) + 1) > (double)maxCols) {
    e1 = 0; e2 = 0; cell = 1e300;
    cmin[a1] = 0; cmin[a2] = 0;
  }
  G.sweepAxis = ax; G.ax1 = a1; G.ax2 = a2;
  G.cell = cell;
  G.invCell = 1.0 / cell;
  G.lo1 = cmin[a1]; G.lo2 = cmin[a2];
  G.ncx = (int)(floor(e1 / cell) + 1);
  G.ncy = (int)(floor(e2 / cell) + 1);
  G.loS = bmin[ax];
  double span = bmax[ax] - bmin[ax];
  G.invQ = (span > 0 && span < 1e300) ? (double)(G.qmax - 1) / span : 0.0;
  if (!(G.invQ == G.invQ)) G.invQ = 0.0;
  if (!(G.loS == G.loS)) G.loS = 0.0;
  G.ok = 1;
  *g = G;
}

__device__ __forceinline__ double cmp3(const double4_32a& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// monotone non-decreasing quantisation along the sweep axis (any such map gives the same pair set: ties
// are ordered by particle id; coarser steps only lengthen the walks a little)
__device__ __forceinline__ unsigned quant(double x, const GridParams& G) {
  double t = (x - G.loS) * G.invQ;
  if (!(t > 0)) return 0;                 // also NaN
  if (t >= (double)G.qmax) return G.qmax;
  return (unsigned)t;                      // truncation == floor for t >= 0
}

__device__ __forceinline__ void columnOf(const double4_32a& pr, const GridParams& G, int& cx, int& cy) {
  // multiplying by the rounded reciprocal moves a centre at most a few ulp across a column edge: two centres
  // closer than the widest box (cell = widest box x (1 + 1e-6)) still fall into the same or adjacent columns
  double t1 = floor((cmp3(pr, G.ax1) - G.lo1) * G.invCell);
  double t2 = floor((cmp3(pr, G.ax2) - G.lo2) * G.invCell);
  cx = (int)fmin(fmax(t1, 0.0), (double)(G.ncx - 1));
  cy = (int)fmin(fmax(t2, 0.0), (double)(G.ncy - 1));
}

__global__ void k_make_keys(Particles p, const int* small, int nSmall, const GridParams* g,
                            unsigned long long* keys, unsigned* vals) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nSmall) return;
  GridParams G = *g;
  int i = small[k];
  int cx, cy;
  columnOf(p.posr[i], G, cx, cy);
  unsigned long long col = (unsigned long long)cx + (unsigned long long)G.ncx * cy;
  unsigned q = quant(cmp3(p.bbmin[i], G.sweepAxis), G);
  keys[k] = (col << G.qbits) | q;
  vals[k] = (unsigned)i;
}


// ------------------------------------------------------------------------------------ scan
// Exclusive scan of a[0..n) in place, a[n] <- total.  Block-wise scan, recursive on block sums.
static const int SCAN_T = 256, SCAN_I = 4, SCAN_TILE = SCAN_T * SCAN_I;

__global__ void k_scan_tiles(unsigned* a, long long n, unsigned* sums) {
  __shared__ unsigned s[SCAN_T];
  long long base = (long long)blockIdx.x * SCAN_TILE;
  unsigned v[SCAN_I];
  unsigned tsum = 0;
  for (int k = 0; k < SCAN_I; k++) {
    long long idx = base + threadIdx.x * SCAN_I + k;
    v[k] = idx < n ? a[idx] : 0;
    tsum += v[k];
  }
  s[threadIdx.x] = tsum;
  __syncthreads();
  for (int off = 1; off < SCAN_T; off <<= 1) {
    unsigned t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  unsigned run = s[threadIdx.x] - tsum;  // exclusive prefix of this thread
  for (int k = 0; k < SCAN_I; k++) {
    long long idx = base + threadIdx.x * SCAN_I + k;
    if (idx < n) a[idx] = run;
    run += v[k];
  }
  if (threadIdx.x == SCAN_T - 1) sums[blockIdx.x] = s[SCAN_T - 1];
}



// Exclusive scan of a[0..n) in place with the total written to a[n]: tile scans, the tile sums scanned by
// the same routine (which leaves their total at sums[nb]), then the sums added back; with one tile the
// tile kernel writes the total itself.
__global__ void k_scan_add(unsigned* a, long long n, const unsigned* sums, long long nb) {
  long long base = (long long)blockIdx.x * SCAN_TILE;
  unsigned add = sums[blockIdx.x];
  for (int k = 0; k < SCAN_I; k++) {
    long long idx = base + threadIdx.x * SCAN_I + k;
    if (idx < n) a[idx] += add;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a[n] = sums[nb];
}

static void scan_rec(cudaStream_t s, unsigned* a, long long n, unsigned* scratch) {
  long long nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb == 0) {
    cudaMemsetAsync(a, 0, sizeof(unsigned), s);  // empty: total 0
    return;
  }
  unsigned* sums = scratch;  // nb + 1 entries
  (k_scan_tiles<<<(unsigned)nb, SCAN_T, 0, s>>>(a, n, nb == 1 ? a + n : sums), ++::wdem::g_kernel_launches);
  if (nb > 1) {
    scan_rec(s, sums, nb, scratch + ((nb + 1 + 63) & ~63ll));
    (k_scan_add<<<(unsigned)nb, SCAN_T, 0, s>>>(a, n, sums, nb), ++::wdem::g_kernel_launches);
  }
}

void exclusive_scan_u32(cudaStream_t s, unsigned* a, long long n, ColliderScratch& cs) {
  scan_rec(s, a, n, cs.blockSums + 64);
}

// ------------------------------------------------------------------------------------ radix sort
// LSD radix sort, 8-bit digits, keys u64 with u32 payload, one kernel per digit (Merrill & Garland's
// single-pass prefix scan with decoupled look-back, applied per digit as in "Onesweep", Adinets & Merrill
// 2022).  Before the passes, one kernel counts the digits of every pass over the whole input (the global
// digit starts do not depend on the order) and one block scans them.  A pass kernel takes its tile in
// acquisition order (atomic counter, so every earlier tile is running or done), counts the tile's digits,
// publishes them (aggregate), looks back over earlier tiles for the digit's exclusive prefix (stopping at
// the first inclusive prefix), publishes its own inclusive prefix, ranks the tile's keys stably (round,
// warp, lane order) into shared memory and writes each digit's run contiguously.  Every look-back wait is
// bounded; a wait that gives up sets WDEM_ERR_TIMEOUT.
static const int RS_T = 256, RS_R = 8, RS_TILE = RS_T * RS_R;
static const int RS_MAX_PASSES = 8;
static const unsigned RS_AGG = 1u << 30, RS_PRE = 2u << 30, RS_VAL = (1u << 30) - 1;
static const long long RS_SPIN = 1ll << 22;

// global digit counts of all passes: gcount[p][d]
__global__ void __launch_bounds__(RS_T) k_rs_count(const unsigned long long* keys, long long n, int passes, unsigned* gcount) {
  __shared__ unsigned h[RS_MAX_PASSES][256];
  for (int p = 0; p < passes; p++) h[p][threadIdx.x] = 0;
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = keys[i];
    for (int p = 0; p < passes; p++) atomicAdd(&h[p][(k >> (8 * p)) & 255], 1u);
  }
  __syncthreads();
  for (int p = 0; p < passes; p++)
    if (h[p][threadIdx.x]) atomicAdd(&gcount[p * 256 + threadIdx.x], h[p][threadIdx.x]);
}
// exclusive scan of each pass's 256 counts (one block, thread = digit)
__global__ void __launch_bounds__(RS_T) k_rs_starts(unsigned* gcount, int passes) {
  __shared__ unsigned s[256];
  for (int p = 0; p < passes; p++) {
    const unsigned c = gcount[p * 256 + threadIdx.x];
    s[threadIdx.x] = c;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
      const unsigned t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    gcount[p * 256 + threadIdx.x] = s[threadIdx.x] - c;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(RS_T) k_rs_pass(const unsigned long long* kin, const unsigned* vin, unsigned long long* kout,
                                                  unsigned* vout, long long n, int shift, const unsigned* digitStart,
                                                  unsigned* status, unsigned* tileCounter, DeviceStatus* st) {
  __shared__ unsigned tileS;
  __shared__ unsigned cnt[256];      // the tile's digit counts
  __shared__ unsigned lstart[256];   // exclusive prefix of cnt: the digit's run in the tile's staging
  __shared__ unsigned goff[256];     // the digit's first position in the output
  __shared__ unsigned runBase[256];
  __shared__ unsigned wc[RS_T / 32][256];
  __shared__ unsigned long long skey[RS_TILE];
  __shared__ unsigned sval[RS_TILE];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  if (t == 0) tileS = atomicAdd(tileCounter, 1u);
  cnt[t] = 0;
  runBase[t] = 0;
  __syncthreads();
  const long long tile = tileS;
  const long long base = tile * RS_TILE;
  unsigned long long k[RS_R];
  unsigned v[RS_R];
#pragma unroll
  for (int r = 0; r < RS_R; r++) {
    const long long idx = base + r * RS_T + t;
    k[r] = idx < n ? kin[idx] : 0;
    v[r] = idx < n ? vin[idx] : 0;
    if (idx < n) atomicAdd(&cnt[(k[r] >> shift) & 255], 1u);
  }
  __syncthreads();
  // thread t: digit t.  Aggregate first, then the look-back, then the inclusive prefix.
  const unsigned c = cnt[t];
  volatile unsigned* mine = status + tile * 256;
  unsigned excl = 0;
  if (tile == 0) {
    mine[t] = RS_PRE | c;
  } else {
    mine[t] = RS_AGG | c;
    for (long long j = tile - 1; j >= 0; j--) {
      volatile unsigned* pr = status + j * 256;
      unsigned w = pr[t];
      long long it = 0;
      while ((w & ~RS_VAL) == 0) {
        if (++it > RS_SPIN) {
          atomicCAS(&st->code, 0, WDEM_ERR_TIMEOUT);
          w = RS_PRE;
          break;
        }
        __nanosleep(32);
        w = pr[t];
      }
      excl += w & RS_VAL;
      if ((w & ~RS_VAL) == RS_PRE) break;
    }
    mine[t] = RS_PRE | (excl + c);
  }
  goff[t] = digitStart[t] + excl;
  // exclusive scan of the tile's counts: where each digit's run starts in the staging arrays
  {
    unsigned* sc = &wc[0][0];  // free until the ranking rounds
    sc[t] = c;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
      const unsigned u = t >= off ? sc[t - off] : 0;
      __syncthreads();
      sc[t] += u;
      __syncthreads();
    }
    lstart[t] = sc[t] - c;
    __syncthreads();
  }
  // stable ranking into the staging arrays: round r, then warp, then lane
  for (int r = 0; r < RS_R; r++) {
    for (int w = 0; w < RS_T / 32; w++) wc[w][t] = 0;
    __syncthreads();
    const long long idx = base + r * RS_T + t;
    const bool valid = idx < n;
    const unsigned d = valid ? (unsigned)((k[r] >> shift) & 255) : 256u + lane;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned rankInWarp = __popc(peers & ((1u << lane) - 1));
    if (valid && lane == __ffs(peers) - 1) wc[warp][d] = __popc(peers);
    __syncthreads();
    unsigned dsum = 0;
    for (int w = 0; w < RS_T / 32; w++) { const unsigned cc = wc[w][t]; wc[w][t] = dsum; dsum += cc; }
    __syncthreads();
    if (valid) {
      const unsigned pos = lstart[d] + runBase[d] + wc[warp][d] + rankInWarp;
      skey[pos] = k[r];
      sval[pos] = v[r];
    }
    __syncthreads();
    runBase[t] += dsum;
  }
  __syncthreads();
  // each digit's run written contiguously
  const long long m = n - base < RS_TILE ? n - base : RS_TILE;
  for (int j = t; j < m; j += RS_T) {
    const unsigned long long kk = skey[j];
    const unsigned d = (unsigned)((kk >> shift) & 255);
    const unsigned pos = goff[d] + (unsigned)j - lstart[d];
    kout[pos] = kk;
    vout[pos] = sval[j];
  }
}

// scratch of one sort: status words of every pass (passes x tiles x 256), then the per-pass tile counters
// and global digit starts (passes x 256), cleared by one memset
static void radix_sort(cudaStream_t s, unsigned long long*& keys, unsigned*& vals, unsigned long long*& keysAlt,
                       unsigned*& valsAlt, long long n, int bits, ColliderScratch& cs) {
  DeviceStatus* st = cs.st;
  if (n <= 1) return;
  const long long nTiles = (n + RS_TILE - 1) / RS_TILE;
  const int passes = (bits + 7) / 8;
  unsigned* status = cs.hist;
  unsigned* starts = status + (size_t)passes * nTiles * 256;
  unsigned* counters = starts + passes * 256;
  cudaMemsetAsync(status, 0, ((size_t)passes * nTiles * 256 + passes * 256 + passes) * sizeof(unsigned), s);
  const unsigned cb = (unsigned)std::min<long long>((n + RS_T - 1) / RS_T, 152 * 8);
  (k_rs_count<<<cb, RS_T, 0, s>>>(keys, n, passes, starts), ++::wdem::g_kernel_launches);
  (k_rs_starts<<<1, RS_T, 0, s>>>(starts, passes), ++::wdem::g_kernel_launches);
  for (int p = 0; p < passes; p++) {
    (k_rs_pass<<<(unsigned)nTiles, RS_T, 0, s>>>(keys, vals, keysAlt, valsAlt, n, 8 * p, starts + p * 256,
                                                  status + (size_t)p * nTiles * 256, counters + p, st),
     ++::wdem::g_kernel_launches);
    unsigned long long* tk = keys; keys = keysAlt; keysAlt = tk;
    unsigned* tv = vals; vals = valsAlt; valsAlt = tv;
  }
}
// words of radix-sort scratch for n keys
long long radix_scratch_words(long long n) {
  const long long nTiles = (n + RS_TILE - 1) / RS_TILE;
  return (long long)RS_MAX_PASSES * nTiles * 256 + RS_MAX_PASSES * 257 + 64;
}

// ------------------------------------------------------------------------------------ sort small
__global__ void k_cell_start(const unsigned long long* keys, int nSmall, const GridParams* g, int* cellStart) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int ncols = g->ncx * g->ncy;
  if (nSmall == 0) {
    for (int k = s; k <= ncols; k += gridDim.x * blockDim.x) cellStart[k] = 0;
    return;
  }
  if (s >= nSmall) return;
  const int qb = g->qbits;
  long long c = (long long)(keys[s] >> qb);
  long long cp = s > 0 ? (long long)(keys[s - 1] >> qb) : -1;
  for (long long k = cp + 1; k <= c; k++) cellStart[k] = s;
  if (s == nSmall - 1)
    for (long long k = c + 1; k <= ncols; k++) cellStart[k] = nSmall;
}


// ------------------------------------------------------------------------------------ sweep
__device__ __forceinline__ bool overlap3(const double4_32a& mn1, const double4_32a& mx1, const double4_32a& mn2, const double4_32a& mx2) {
  return (mn1.x <= mx2.x) && (mx1.x >= mn2.x) && (mn1.y <= mx2.y) && (mx1.y >= mn2.y) && (mn1.z <= mx2.z) && (mx1.z >= mn2.z);
}
__device__ __forceinline__ bool mayCollide(unsigned m1, unsigned m2, unsigned lone) {
  return (m1 & m2) != 0 && (m1 & m2 & lone) == 0;
}
// contact orientation: same shape -> (lower id, higher id); otherwise the order of the Cg2 functor
// (Wall+Sphere, Facet+Sphere, Sphere+Ellipsoid, Wall+Ellipsoid)
__device__ __forceinline__ int2 orient(int i, int j, int shi, int shj) {
  int a = min(i, j), b = max(i, j);
  int sa = (a == i) ? shi : shj, sb = (a == i) ? shj : shi;
  if (pairSwaps(sa, sb)) {
    int t = a; a = b; b = t;
  }
  return make_int2(a, b);
}

// Sweep records, two float4 per particle in sort order: the box in FP32 with the minimum rounded down and
// the maximum rounded up (every pair of FP64 boxes that overlap overlaps in FP32 too, so a pair the FP32
// test rejects needs no FP64 test), the mask (lo.w) and meta.x with shape and scene (hi.w).  The sweep
// walks these contiguous records instead of gathering meta, bbmin and bbmax by particle id.
__global__ void k_sweep_records(Particles p, const unsigned* vals, int nSmall, float4* rec) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nSmall) return;
  const int i = (int)vals[s];
  const double4_32a mn = p.bbmin[i], mx = p.bbmax[i];
  const int4 m = p.meta[i];
  rec[2 * s] = make_float4(__double2float_rd(mn.x), __double2float_rd(mn.y), __double2float_rd(mn.z), __uint_as_float((unsigned)m.z));
  rec[2 * s + 1] = make_float4(__double2float_ru(mx.x), __double2float_ru(mx.y), __double2float_ru(mx.z), __int_as_float(m.x));
}
__device__ __forceinline__ bool overlapF(const float4& mn1, const float4& mx1, const float4& mn2, const float4& mx2) {
  return (mn1.x <= mx2.x) && (mx1.x >= mn2.x) && (mn1.y <= mx2.y) && (mx1.y >= mn2.y) && (mn1.z <= mx2.z) && (mx1.z >= mn2.z);
}

struct SweepArgs {
  const float4* rec;
  const unsigned long long* keys;
  const unsigned* vals;
  const int* cellStart;
  const int* large;
  int nLarge;
  int nSmall;
  unsigned loneMask;
  const int* sceneWall;  // per-scene ranges of the large list (null: one scene)
  int2* buf;             // SWEEP_BUF pairs per thread, written by the counting pass (null: none kept)
};

// The sweep runs twice: counting (WRITE false) and writing at the scanned offsets (WRITE true).  With a
// buffer, the counting pass keeps each thread's first SWEEP_BUF pairs in walk order and the writing pass
// copies them, walking again only for threads that found more: the output is the same, in the same order.
template <bool WRITE>
__global__ void k_sweep(Particles p, SweepArgs A, const GridParams* g, unsigned* counts, int2* out, long long cap,
                        DeviceStatus* st) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= sweepThreads(A.nSmall, A.nLarge)) return;
  unsigned cnt = 0;
  unsigned long long base = WRITE ? counts[s] : 0;
  if (WRITE && A.buf) {
    const unsigned found = counts[s + 1] - counts[s];
    if (found <= (unsigned)SWEEP_BUF) {
      const int2* b = A.buf + (long long)s * SWEEP_BUF;
      for (unsigned k = 0; k < found; k++)
        if (base + k < (unsigned long long)cap) out[base + k] = b[k];
      return;
    }
  }
  auto emit = [&](int2 pr) {
    if (WRITE) {
      const unsigned long long o = base + cnt;
      if (o < (unsigned long long)cap) out[o] = pr;
    } else if (A.buf && cnt < (unsigned)SWEEP_BUF) {
      A.buf[(long long)s * SWEEP_BUF + cnt] = pr;
    }
    cnt++;
  };
  if (s >= A.nSmall) {
    // large-large pairs, one thread per large body a: the bodies after it in the large list up to the
    // first one of another scene (the list is grouped by scene)
    const int a = s - A.nSmall;
    if (a < A.nLarge) {
      const int i = A.large[a];
      const int4 mi = p.meta[i];
      const double4_32a mn = p.bbmin[i], mx = p.bbmax[i];
      for (int b = a + 1; b < A.nLarge; b++) {
        const int j = A.large[b];
        const int4 mj = p.meta[j];
        if (sceneOf(mi.x) != sceneOf(mj.x)) break;
        if (!mayCollide((unsigned)mi.z, (unsigned)mj.z, A.loneMask)) continue;
        if (!overlap3(mn, mx, p.bbmin[j], p.bbmax[j])) continue;
        emit(orient(i, j, mi.x & 15, mj.x & 15));
      }
    }
    if (!WRITE) counts[s] = cnt;
    return;
  }
  GridParams G = *g;
  unsigned long long key = A.keys[s];
  int i = (int)A.vals[s];
  int4 mi = p.meta[i];
  double4_32a mn = p.bbmin[i], mx = p.bbmax[i];
  const float4 fmn = A.rec[2 * s], fmx = A.rec[2 * s + 1];
  unsigned qi = (unsigned)(key & G.qmax);
  unsigned qmax = quant(cmp3(mx, G.sweepAxis), G);
  long long col = (long long)(key >> G.qbits);
  int cx = (int)(col % G.ncx), cy = (int)(col / G.ncx);
  for (int dy = -1; dy <= 1; dy++) {
    int y = cy + dy;
    if (y < 0 || y >= G.ncy) continue;
    for (int dx = -1; dx <= 1; dx++) {
      int x = cx + dx;
      if (x < 0 || x >= G.ncx) continue;
      long long c2 = (long long)x + (long long)G.ncx * y;
      int beg = A.cellStart[c2], end = A.cellStart[c2 + 1];
      int q;
      if (c2 == col) q = s + 1;
      else {
        unsigned long long target = ((unsigned long long)c2 << G.qbits) | qi;
        int lo = beg, hi = end;
        while (lo < hi) { int mid = (lo + hi) >> 1; if (A.keys[mid] < target) lo = mid + 1; else hi = mid; }
        q = lo;
        while (q < end && A.keys[q] == target && (int)A.vals[q] < i) q++;
      }
      for (; q < end; q++) {
        unsigned long long kq = A.keys[q];
        if ((unsigned)(kq & G.qmax) > qmax) break;
        const float4 gmn = A.rec[2 * q], gmx = A.rec[2 * q + 1];
        const unsigned maskj = __float_as_uint(gmn.w);
        const int metaxj = __float_as_int(gmx.w);
        if (!mayCollide((unsigned)mi.z, maskj, A.loneMask)) continue;
        if (sceneOf(mi.x) != sceneOf(metaxj)) continue;
        if (!overlapF(fmn, fmx, gmn, gmx)) continue;
        int j = (int)A.vals[q];
        if (!overlap3(mn, mx, p.bbmin[j], p.bbmax[j])) continue;
        emit(orient(i, j, mi.x & 15, metaxj & 15));
      }
    }
  }
  const int sc = sceneOf(mi.x);
  const int a0 = A.sceneWall ? A.sceneWall[sc] : 0, a1 = A.sceneWall ? A.sceneWall[sc + 1] : A.nLarge;
  for (int a = a0; a < a1; a++) {
    int j = A.large[a];
    int4 mj = p.meta[j];
    if (!mayCollide((unsigned)mi.z, (unsigned)mj.z, A.loneMask)) continue;
    if (!overlap3(mn, mx, p.bbmin[j], p.bbmax[j])) continue;
    emit(orient(i, j, mi.x & 15, mj.x & 15));
  }
  if (!WRITE) counts[s] = cnt;
}

// ------------------------------------------------------------------------------------ retain
// Real contacts whose new boxes no longer overlap stay in the container (the reference collider
// removes only non-real contacts on separation, InsertionSortCollider.cpp:107-110).
__global__ void k_retain_flag(StepParams P, Particles p, Contacts old, long long nOld, unsigned* flag,
                              const float4* pci, const float4* phi) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nOld) return;
  unsigned f = 0;
  if ((old.state[c] & CS_MASK) == CS_REAL) {
    int2 id = old.ids[c];
    bool ov;
    if (P.periodic) {
      // boxes that overlap on every axis by more than the FP32 margin (both narrow: no ambiguity) overlap
      // in the exact test too (the FP32 copies of this rebuild, k_peri_sorted)
      const float4 c1 = pci[id.x], h1 = phi[id.x], c2 = pci[id.y], h2 = phi[id.y];
      const float L0 = (float)P.csize[0], L1 = (float)P.csize[1], L2 = (float)P.csize[2];
      if (h1.w == 0.f && h2.w == 0.f && periNear(c1.x, h1.x, c2.x, h2.x, L0, 1.f / L0) &&
          periNear(c1.y, h1.y, c2.y, h2.y, L1, 1.f / L1) && periNear(c1.z, h1.z, c2.z, h2.z, L2, 1.f / L2))
        ov = true;
      else {
        int4 per; bool amb = false;
        ov = overlapPeri(p.bbmin[id.x], p.bbmax[id.x], p.bbmin[id.y], p.bbmax[id.y], P.csize, per, amb);
      }
    } else ov = overlap3(p.bbmin[id.x], p.bbmax[id.x], p.bbmin[id.y], p.bbmax[id.y]);
    if (!ov) f = 1;
  }
  flag[c] = f;
}
__global__ void k_retain_write_dist(Contacts old, long long nOld, const unsigned* flagScan, int4* out, long long base, long long cap) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nOld) return;
  if (flagScan[c + 1] != flagScan[c]) {
    long long o = base + flagScan[c];
    if (o < cap) out[o] = old.cdist[c];
  }
}
__global__ void k_retain_write(Contacts old, long long nOld, const unsigned* flagScan, int2* out, long long base, long long cap) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nOld) return;
  if (flagScan[c + 1] != flagScan[c]) {
    long long o = base + flagScan[c];
    if (o < cap) out[o] = old.ids[c];
  }
}

// ------------------------------------------------------------------------------------ old-contact lookup
// The contact of the pair (a, b) in the container whose CSR is `csr` (built at the last rebuild or upload):
// binary search of the partner in the row of the lower id, whose keys are sorted by partner; -1 if none.
__device__ __forceinline__ long long csrFind(const Csr& csr, int a, int b) {
  const int lo = min(a, b), hi = max(a, b);
  if (lo < 0 || hi >= csr.n) return -1;  // ids the rows do not cover (appended since) had no contact
  const unsigned long long key = ((unsigned long long)(unsigned)lo << csr.idBits) | (unsigned)hi;
  int l = csr.rowptr[lo], r = csr.rowptr[lo + 1];
  while (l < r) {
    const int m = (l + r) >> 1;
    if (csr.keys[m] < key) l = m + 1; else r = m;
  }
  if (l < csr.rowptr[lo + 1] && csr.keys[l] == key) return (long long)(csr.ent[l] & 0x7fffffffu);
  return -1;
}

// ------------------------------------------------------------------------------------ carry-over
// History of pairs already in the container is copied; new pairs start as potential contacts
// created in this step (InsertionSortCollider.hpp:106-113 stepCreated=scene->step).  A contact that
// the law broke in the previous step (pending) becomes potential: removePending in a full run keeps
// it only when its new boxes overlap, which holds for every pair the sweep emitted.
// Compaction: the pairs that were real contacts before the rebuild go to the front of the new container,
// in emission order (the role of ContactLoop's reorderContacts, ContactLoop.cpp:75-91), so that the real
// contacts the contact pass and the force gather touch every step are dense in every per-contact array.
// Pass 1 finds each new pair's old index (or none) and flags the real ones; after a scan of the flags,
// pass 2 writes each contact at its place: real ones at their rank, the others after them in order.
__global__ void k_part_flag(Contacts neu, long long nNew, Contacts old, Csr oldCsr, unsigned long long* tmpIds,
                            unsigned* tmpJ, unsigned* flag, int4* tmpDist) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nNew) return;
  const int2 id = neu.ids[c];
  tmpIds[c] = ((unsigned long long)(unsigned)id.y << 32) | (unsigned)id.x;
  if (tmpDist) tmpDist[c] = neu.cdist[c];
  const long long j = csrFind(oldCsr, id.x, id.y);
  unsigned jj = 0xffffffffu, f = 0;
  if (j >= 0) {
    const uint8_t os = old.state[j] & CS_MASK;
    if (os != CS_DEAD) { jj = (unsigned)j; f = (os == CS_REAL) ? 1u : 0u; }
  }
  tmpJ[c] = jj;
  flag[c] = f;
}
__global__ void k_carry_compact(Particles p, Contacts neu, long long nNew, Contacts old, const unsigned long long* tmpIds,
                                const unsigned* tmpJ, const unsigned* scan, const int4* tmpDist, long long step, int nHist) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nNew) return;
  const unsigned before = scan[c];
  const bool wasReal = scan[c + 1] != before;
  const long long d = wasReal ? (long long)before : (long long)scan[nNew] + (c - (long long)before);
  const unsigned long long t = tmpIds[c];
  const int2 id = make_int2((int)(unsigned)(t & 0xffffffffu), (int)(unsigned)(t >> 32));
  const unsigned jj = tmpJ[c];
  if (jj == 0xffffffffu) {
    const uint8_t sb = pairShapeBits(p.meta[id.x].x & 15, p.meta[id.y].x & 15);
    neu.ids[d] = id;
    if (neu.cdist) neu.cdist[d] = tmpDist[c];
    neu.state[d] = CS_POTENTIAL | sb;
    neu.step0[d] = (int)step;
    if (neu.lam) neu.lam[d] = __longlong_as_double(0x7ff8000000000000ll);
    return;
  }
  const long long j = jj;
  if (neu.lam && old.lam) neu.lam[d] = old.lam[j];
  else if (neu.lam) neu.lam[d] = __longlong_as_double(0x7ff8000000000000ll);
  neu.ids[d] = old.ids[j];  // keep the stored orientation (and, periodic, the stored cellDist)
  if (neu.cdist) neu.cdist[d] = old.cdist ? old.cdist[j] : tmpDist[c];
  neu.state[d] = (wasReal ? CS_REAL : CS_POTENTIAL) | (old.state[j] & CS_SHAPES);
  neu.step0[d] = old.step0[j];
  if (wasReal) {
    for (int h = 0; h < nHist; h++) neu.hist[h][d] = old.hist[h][j];
    neu.tanPhi[d] = old.tanPhi[j];
  }
}

// ------------------------------------------------------------------------------------ CSR
__global__ void k_csr_entries(Contacts c, long long nc, int idBits, unsigned long long* keys, unsigned* vals) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nc) return;
  int2 id = c.ids[e];
  keys[2 * e] = ((unsigned long long)(unsigned)id.x << idBits) | (unsigned)id.y;
  vals[2 * e] = (unsigned)e;
  keys[2 * e + 1] = ((unsigned long long)(unsigned)id.y << idBits) | (unsigned)id.x;
  vals[2 * e + 1] = (unsigned)e | 0x80000000u;
}
// the sorted entries, and each contact's two entry positions (where the contact pass writes its shares)
// with their positions in the rows (which bit of the row's mask the contact pass sets)
__global__ void k_csr_ent_slots(const unsigned* vals, const unsigned long long* keys, int idBits, const int* rowptr,
                                long long ne, unsigned* ent, int2* slot, uchar2* rowBit) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const unsigned v = vals[e];
  ent[e] = v;
  const unsigned ci = v & 0x7fffffffu;
  const long long k = e - rowptr[keys[e] >> idBits];
  const unsigned char bit = (unsigned char)(k < 31 ? k : 31);
  if (v >> 31) { slot[ci].y = (int)e; rowBit[ci].y = bit; }
  else { slot[ci].x = (int)e; rowBit[ci].x = bit; }
}
__global__ void k_csr_rows(const unsigned long long* keys, long long ne, int idBits, int n, int* rowptr) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) {
    if (ne == 0 && e <= n) rowptr[e] = 0;
    return;
  }
  long long r = (long long)(keys[e] >> idBits);
  long long rp = e > 0 ? (long long)(keys[e - 1] >> idBits) : -1;
  for (long long k = rp + 1; k <= r; k++) rowptr[k] = (int)e;
  if (e == ne - 1)
    for (long long k = r + 1; k <= n; k++) rowptr[k] = (int)ne;
}

// ------------------------------------------------------------------------------------ periodic grid
// Cells of the periodic box (unsheared coordinates), at least as wide as the widest box per axis, so
// overlapping periodic images of two boxes lie in neighbouring cells (with wrap-around).  Axes with
// fewer than 3 cells get one cell.  Candidates are then decided by the exact spatialOverlapPeri.
struct PeriGrid {
  int nc[3];
  double cw[3];
  int ok;
};

__global__ void k_grid_peri(const unsigned long long* ext, StepParams P, int maxCells, PeriGrid* g) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  PeriGrid G;
  long long tot = 1;
  for (int k = 0; k < 3; k++) {
    double W = ordVal(~ext[12 + k]);
    int n = (W > 0 && W < 1e300) ? (int)floor(P.csize[k] / (W * (1 + 1e-6))) : 1;
    if (n < 3) n = 1;
    if (n > 1024) n = 1024;
    G.nc[k] = n;
    tot *= n;
  }
  while (tot > maxCells) {
    int kmax = 0;
    for (int k = 1; k < 3; k++) if (G.nc[k] > G.nc[kmax]) kmax = k;
    G.nc[kmax] = G.nc[kmax] * 3 / 4;
    if (G.nc[kmax] < 3) G.nc[kmax] = 1;
    tot = (long long)G.nc[0] * G.nc[1] * G.nc[2];
  }
  for (int k = 0; k < 3; k++) G.cw[k] = P.csize[k] / G.nc[k];
  G.ok = 1;
  *g = G;
}

__device__ __forceinline__ void periCell(const double4_32a& mn, const double4_32a& mx, const StepParams& P,
                                         const PeriGrid& G, int* c) {
  const double ctr[3] = {.5 * (mn.x + mx.x), .5 * (mn.y + mx.y), .5 * (mn.z + mx.z)};
  for (int k = 0; k < 3; k++) {
    double w = ctr[k] - floor(ctr[k] / P.csize[k]) * P.csize[k];
    double v = floor(w / G.cw[k]);
    c[k] = (int)fmin(fmax(v, 0.0), (double)(G.nc[k] - 1));
  }
}

__global__ void k_keys_peri(StepParams P, Particles p, const int* small, int nSmall, const PeriGrid* g,
                            unsigned long long* keys, unsigned* vals) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nSmall) return;
  const PeriGrid G = *g;
  const int i = small[k];
  int c[3];
  periCell(p.bbmin[i], p.bbmax[i], P, G, c);
  keys[k] = ((unsigned long long)c[2] * G.nc[1] + c[1]) * G.nc[0] + c[0];
  vals[k] = (unsigned)i;
}

// cellStart[c] = first sorted position of cell c, for the grid's own cells (nc0 nc1 nc2 + 1 entries)
__global__ void k_cell_start_plain(const unsigned long long* keys, int nSmall, const PeriGrid* g, int* cellStart) {
  const long long ncells = (long long)g->nc[0] * g->nc[1] * g->nc[2];
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (nSmall == 0) {
    for (long long k = s; k <= ncells; k += (long long)gridDim.x * blockDim.x) cellStart[k] = 0;
    return;
  }
  if (s >= nSmall) return;
  long long c = (long long)keys[s];
  long long cp = s > 0 ? (long long)keys[s - 1] : -1;
  for (long long k = cp + 1; k <= c; k++) cellStart[k] = s;
  if (s == nSmall - 1)
    for (long long k = c + 1; k <= ncells; k++) cellStart[k] = nSmall;
}

// FP32 copies, in cell order, of each box's centre wrapped into the cell and of its half-widths: the
// candidate loop rejects with them the pairs whose minimum-image centre distance exceeds the sum of
// the half-widths by more than the rounding of these copies on some axis.  Such boxes are disjoint on
// that axis for every period shift, so spatialOverlapPeri rejects them too, and it is evaluated (in
// FP64, as the reference does) only for the survivors.  Boxes wider than a quarter of the cell skip
// the filter (there the exact test may find an ambiguous contact, which is an error to report).
__global__ void k_peri_sorted(StepParams P, Particles p, const unsigned* vals, int nSmall, float4* pc, float4* ph,
                              float4* pci, float4* phi) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nSmall) return;
  const int i = (int)vals[q];
  const double4_32a mn = p.bbmin[i], mx = p.bbmax[i];
  const double lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
  float c[3], h[3];
  bool wide = false;
  for (int k = 0; k < 3; k++) {
    const double L = P.csize[k];
    const double ctr = .5 * (lo[k] + hi[k]), half = .5 * (hi[k] - lo[k]);
    const double w = ctr - floor(ctr / L) * L;
    c[k] = (float)w;
    h[k] = (float)half;
    wide |= !(half < .25 * L);  // also catches infinite and NaN extents
  }
  pc[q] = make_float4(c[0], c[1], c[2], 0.f);
  ph[q] = make_float4(h[0], h[1], h[2], wide ? 1.f : 0.f);
  pci[i] = pc[q];
  phi[i] = ph[q];
}



// Candidate pass: thread q takes the q-th box in cell order and runs the FP32 filter against the boxes
// of the 27 neighbouring cells (wrapped, each cell once) with a larger particle id; it counts (WRITE
// false) or writes (WRITE true, at its scanned offset) the survivors.  The exact FP64 test runs in a
// separate dense pass (k_peri_exact): inside this loop the survivors of one warp's 32 boxes differ per
// lane, and the FP64 test would run with a few lanes at a time.
template <bool WRITE>
__global__ void k_peri_cand(StepParams P, int nSmall, const PeriGrid* g, const unsigned long long* keys,
                            const unsigned* vals, const float4* pc, const float4* ph, const int* cellStart,
                            unsigned* counts, int2* cand, long long cap) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q > nSmall) return;
  if (q == nSmall) { if (!WRITE) counts[q] = 0; return; }
  const PeriGrid G = *g;
  const int i = (int)vals[q];
  const float4 c1 = pc[q], h1 = ph[q];
  const float L0 = (float)P.csize[0], L1 = (float)P.csize[1], L2 = (float)P.csize[2];
  const float iL0 = 1.f / L0, iL1 = 1.f / L1, iL2 = 1.f / L2;
  const long long key0 = (long long)keys[q];
  int c[3];
  c[0] = (int)(key0 % G.nc[0]);
  c[1] = (int)((key0 / G.nc[0]) % G.nc[1]);
  c[2] = (int)(key0 / ((long long)G.nc[0] * G.nc[1]));
  // neighbouring cells per axis, each index once (axes of one or two cells have fewer)
  int nbr[3][3], nn[3];
  for (int a = 0; a < 3; a++) {
    nn[a] = 0;
    for (int d = -1; d <= 1; d++) {
      const int v = ((c[a] + d) % G.nc[a] + G.nc[a]) % G.nc[a];
      bool dup = false;
      for (int b = 0; b < nn[a]; b++) dup |= (nbr[a][b] == v);
      if (!dup) nbr[a][nn[a]++] = v;
    }
  }
  unsigned cnt = 0;
  const unsigned long long base = WRITE ? counts[q] : 0;
  for (int az = 0; az < nn[2]; az++)
    for (int ay = 0; ay < nn[1]; ay++)
      for (int ax = 0; ax < nn[0]; ax++) {
        const long long key = ((long long)nbr[2][az] * G.nc[1] + nbr[1][ay]) * G.nc[0] + nbr[0][ax];
        const int beg = cellStart[key], end = cellStart[key + 1];
        for (int q2 = beg; q2 < end; q2++) {
          const int j = (int)vals[q2];
          if (j <= i) continue;
          const float4 h2 = ph[q2];
          if (h1.w == 0.f && h2.w == 0.f) {
            const float4 c2 = pc[q2];
            if (periFar(c1.x, h1.x, c2.x, h2.x, L0, iL0) || periFar(c1.y, h1.y, c2.y, h2.y, L1, iL1) ||
                periFar(c1.z, h1.z, c2.z, h2.z, L2, iL2))
              continue;
          }
          if (WRITE) {
            const unsigned long long o = base + cnt;
            if (o < (unsigned long long)cap) cand[o] = make_int2(i, j);
          }
          cnt++;
        }
      }
  if (!WRITE) counts[q] = cnt;
}

// Exact pass, one thread per candidate: spatialOverlapPeri (FP64, the reference's operations; an
// ambiguous contact is an error) and Collider::mayCollide.
__global__ void k_peri_exact(StepParams P, Particles p, const int2* cand, long long nc, unsigned* flag, int4* per,
                             DeviceStatus* st) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const int2 ij = cand[k];
  int4 pr = make_int4(0, 0, 0, 0);
  bool amb = false;
  bool ok = overlapPeri(p.bbmin[ij.x], p.bbmax[ij.x], p.bbmin[ij.y], p.bbmax[ij.y], P.csize, pr, amb);
  if (amb) { if (atomicCAS(&st->code, 0, WDEM_ERR_TOO_BIG) == 0) st->detail = ij.x; ok = false; }
  if (ok) ok = mayCollide((unsigned)p.meta[ij.x].z, (unsigned)p.meta[ij.y].z, P.loneMask);
  flag[k] = ok ? 1u : 0u;
  per[k] = pr;
}

// the accepted candidates, in candidate order, with their cellDist
__global__ void k_peri_emit(const int2* cand, const int4* per, const unsigned* flagScan, long long nc, int2* out,
                            int4* outDist, long long cap) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc || flagScan[k + 1] == flagScan[k]) return;
  const long long o = flagScan[k];
  if (o < cap) { out[o] = cand[k]; outDist[o] = per[k]; }
}

// ------------------------------------------------------------------------------------ stress
// ContactLoop stress (ContactLoop.cpp:218-229): F (global, on pA) x branch (pB image - pA) per real
// contact; the nine components are summed by the deterministic energy reduction.
__global__ void k_stress_terms(StepParams P, Particles p, Contacts c, long long nc, double* terms) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if ((c.state[i] & CS_MASK) == CS_REAL) {
    const int2 id = c.ids[i];
    d3 branch = xyz(p.posr[id.y]) - xyz(p.posr[id.x]);
    if (P.periodic) {
      const int4 cd = c.cdist[i];
      branch = branch + mvec(P.hS, mk((double)cd.x, (double)cd.y, (double)cd.z));
    }
    const double4_32a f4 = c.out[OUT_RECORDS * (long long)c.slot[i].x + OUT_F];  // pA's entry: the force on pA
    const double F[3] = {f4.x, f4.y, f4.z};
    const double b[3] = {branch.x, branch.y, branch.z};
    for (int r = 0; r < 3; r++) for (int q = 0; q < 3; q++) v[3 * r + q] = F[r] * b[q];
  }
  for (int q = 0; q < 9; q++) terms[(long long)q * nc + i] = v[q];
}

}  // namespace wdem

// ============================================================================== host orchestration
namespace wdem {


static int bitsFor(unsigned long long v) { int b = 0; while ((1ull << b) < v) b++; return b < 1 ? 1 : b; }
// the sweep grid's column cap and the quantisation bits of its keys: column bits + qbits fill 32, 40 or 48
// bits (4, 5 or 6 radix passes), with at least 12 quantisation bits and at most 24
static int sweepCols(const ColliderScratch& cs) { return std::min(cs.maxCols, SWEEP_MAX_COLS); }
static int sweepQbits(const ColliderScratch& cs) {
  const int cb = bitsFor((unsigned long long)sweepCols(cs) + 1);
  int total = 32;
  while (total - cb < 12) total += 8;
  return std::min(24, total - cb);
}

// The collider sub-steps are called from wdem_api.cu through these thin wrappers.
void col_extents_and_grid(cudaStream_t s, Particles p, const int* small, int nSmall, ColliderScratch& cs) {
  unsigned long long* ext = (unsigned long long*)cs.temp;
  (k_extents_init<<<1, 32, 0, s>>>(ext), ++::wdem::g_kernel_launches);
  if (nSmall > 0) (k_extents<<<(nSmall + 255) / 256, 256, 0, s>>>(p, small, nSmall, ext), ++::wdem::g_kernel_launches);
  (k_grid_setup<<<1, 1, 0, s>>>(ext, nSmall, sweepCols(cs), sweepQbits(cs), cs.grid), ++::wdem::g_kernel_launches);
}

void col_sort(cudaStream_t s, Particles p, const int* small, int nSmall, ColliderScratch& cs) {
  if (nSmall > 0) (k_make_keys<<<(nSmall + 255) / 256, 256, 0, s>>>(p, small, nSmall, cs.grid, cs.keys, cs.vals), ++::wdem::g_kernel_launches);
  int bits = sweepQbits(cs) + bitsFor((unsigned long long)sweepCols(cs) + 1);
  radix_sort(s, cs.keys, cs.vals, cs.keysAlt, cs.valsAlt, nSmall, bits, cs);
  int threads = nSmall > 0 ? nSmall : (cs.maxCols + 1);
  (k_cell_start<<<(threads + 255) / 256, 256, 0, s>>>(cs.keys, nSmall, cs.grid, cs.cellStart), ++::wdem::g_kernel_launches);
  if (nSmall > 0) (k_sweep_records<<<(nSmall + 255) / 256, 256, 0, s>>>(p, cs.vals, nSmall, cs.srec), ++::wdem::g_kernel_launches);
}

void col_sweep(cudaStream_t s, Particles p, int nSmall, unsigned loneMask, ColliderScratch& cs, int2* out, long long cap,
               bool write, DeviceStatus* st) {
  SweepArgs A;
  A.rec = cs.srec;
  A.keys = cs.keys; A.vals = cs.vals; A.cellStart = cs.cellStart; A.large = cs.large; A.nLarge = cs.nLarge;
  A.nSmall = nSmall; A.loneMask = loneMask;
  A.sceneWall = cs.nScenes > 1 ? cs.sceneWall : nullptr;
  A.buf = cs.sweepBufCap >= sweepThreads(nSmall, cs.nLarge) ? cs.sweepBuf : nullptr;
  const int threads = sweepThreads(nSmall, cs.nLarge);
  if (write) (k_sweep<true><<<(threads + 127) / 128, 128, 0, s>>>(p, A, cs.grid, cs.counts, out, cap, st), ++::wdem::g_kernel_launches);
  else (k_sweep<false><<<(threads + 127) / 128, 128, 0, s>>>(p, A, cs.grid, cs.counts, out, cap, st), ++::wdem::g_kernel_launches);
}

void col_retain_write_dist(cudaStream_t s, Contacts old, long long nOld, ColliderScratch& cs, int4* out, long long base,
                           long long cap) {
  if (nOld > 0) (k_retain_write_dist<<<(unsigned)((nOld + 255) / 256), 256, 0, s>>>(old, nOld, cs.retainFlag, out, base, cap), ++::wdem::g_kernel_launches);
}

void col_retain_flags(cudaStream_t s, const StepParams& P, Particles p, Contacts old, long long nOld, ColliderScratch& cs) {
  if (nOld > 0) (k_retain_flag<<<(unsigned)((nOld + 255) / 256), 256, 0, s>>>(P, p, old, nOld, cs.retainFlag, cs.periCi, cs.periHi), ++::wdem::g_kernel_launches);
  exclusive_scan_u32(s, cs.retainFlag, nOld, cs);
}
void col_retain_write(cudaStream_t s, Contacts old, long long nOld, ColliderScratch& cs, int2* out, long long base, long long cap) {
  if (nOld > 0) (k_retain_write<<<(unsigned)((nOld + 255) / 256), 256, 0, s>>>(old, nOld, cs.retainFlag, out, base, cap), ++::wdem::g_kernel_launches);
}

// periodic pair search, part 1: grid, cell sort, FP32 candidates counted (write false; counts
// scanned, total at counts[nSmall + 1]) or written (write true)
void col_periodic_cand(cudaStream_t s, const StepParams& P, Particles p, const int* small, int nSmall,
                       ColliderScratch& cs, bool write) {
  PeriGrid* g = (PeriGrid*)((char*)cs.temp + 256);
  const int threads = nSmall + 1;
  if (!write) {
    unsigned long long* ext = (unsigned long long*)cs.temp;
    (k_extents_init<<<1, 32, 0, s>>>(ext), ++::wdem::g_kernel_launches);
    if (nSmall > 0) (k_extents<<<(nSmall + 255) / 256, 256, 0, s>>>(p, small, nSmall, ext), ++::wdem::g_kernel_launches);
    (k_grid_peri<<<1, 1, 0, s>>>(ext, P, cs.maxCols, g), ++::wdem::g_kernel_launches);
    if (nSmall > 0) (k_keys_peri<<<(nSmall + 255) / 256, 256, 0, s>>>(P, p, small, nSmall, g, cs.keys, cs.vals), ++::wdem::g_kernel_launches);
    radix_sort(s, cs.keys, cs.vals, cs.keysAlt, cs.valsAlt, nSmall, bitsFor((unsigned long long)cs.maxCols + 1), cs);
    int t = nSmall > 0 ? nSmall : (cs.maxCols + 1);
    (k_cell_start_plain<<<(t + 255) / 256, 256, 0, s>>>(cs.keys, nSmall, g, cs.cellStart), ++::wdem::g_kernel_launches);
    if (nSmall > 0) (k_peri_sorted<<<(nSmall + 255) / 256, 256, 0, s>>>(P, p, cs.vals, nSmall, cs.periC, cs.periH, cs.periCi, cs.periHi), ++::wdem::g_kernel_launches);
    (k_peri_cand<false><<<(threads + 127) / 128, 128, 0, s>>>(P, nSmall, g, cs.keys, cs.vals, cs.periC, cs.periH, cs.cellStart, cs.counts, nullptr, 0), ++::wdem::g_kernel_launches);
    exclusive_scan_u32(s, cs.counts, nSmall + 1, cs);
  } else {
    (k_peri_cand<true><<<(threads + 127) / 128, 128, 0, s>>>(P, nSmall, g, cs.keys, cs.vals, cs.periC, cs.periH, cs.cellStart, cs.counts, cs.cand, cs.candCap), ++::wdem::g_kernel_launches);
  }
}

// part 2: the exact test of nCand candidates; flags scanned, accepted total at candFlag[nCand]
void col_periodic_exact(cudaStream_t s, const StepParams& P, Particles p, ColliderScratch& cs, long long nCand,
                        DeviceStatus* st) {
  if (nCand > 0) (k_peri_exact<<<(unsigned)((nCand + 255) / 256), 256, 0, s>>>(P, p, cs.cand, nCand, cs.candFlag, cs.candPer, st), ++::wdem::g_kernel_launches);
  exclusive_scan_u32(s, cs.candFlag, nCand, cs);
}

// part 3: accepted pairs and their cellDist into the new container
void col_periodic_emit(cudaStream_t s, ColliderScratch& cs, long long nCand, int2* out, int4* outDist, long long cap) {
  if (nCand > 0) (k_peri_emit<<<(unsigned)((nCand + 255) / 256), 256, 0, s>>>(cs.cand, cs.candPer, cs.candFlag, nCand, out, outDist, cap), ++::wdem::g_kernel_launches);
}

void launch_stress(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc, double* scratch9,
                   double* partials, double* out9) {
  if (nc > 0) (k_stress_terms<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(P, p, c, nc, scratch9), ++::wdem::g_kernel_launches);
  for (int q = 0; q < 9; q++) energy_accumulate(s, scratch9 + (long long)q * nc, nc, partials, out9 + q, true);
}

long long col_carry_compact(cudaStream_t s, Particles p, Contacts neu, long long nNew, Contacts old, Csr oldCsr,
                            long long step, int nHist, ColliderScratch& cs) {
  if (nNew <= 0) return 0;
  unsigned long long* tmpIds = cs.keys;
  unsigned* tmpJ = cs.vals;
  unsigned* flag = cs.valsAlt;
  int4* tmpDist = neu.cdist ? reinterpret_cast<int4*>(cs.keysAlt) : nullptr;
  const unsigned blocks = (unsigned)((nNew + 255) / 256);
  (k_part_flag<<<blocks, 256, 0, s>>>(neu, nNew, old, oldCsr, tmpIds, tmpJ, flag, tmpDist), ++::wdem::g_kernel_launches);
  exclusive_scan_u32(s, flag, nNew, cs);
  (k_carry_compact<<<blocks, 256, 0, s>>>(p, neu, nNew, old, tmpIds, tmpJ, flag, tmpDist, step, nHist), ++::wdem::g_kernel_launches);
  return nNew;
}

void col_csr(cudaStream_t s, Contacts c, long long nc, int n, Csr& csr, ColliderScratch& cs) {
  int idBits = bitsFor((unsigned long long)n + 1);
  long long ne = 2 * nc;
  if (nc > 0) (k_csr_entries<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(c, nc, idBits, cs.keys, cs.vals), ++::wdem::g_kernel_launches);
  radix_sort(s, cs.keys, cs.vals, cs.keysAlt, cs.valsAlt, ne, 2 * idBits, cs);
  // the sorted keys stay with the CSR for the next rebuild's carry (cs.keys is the sort's scratch)
  if (ne > 0) cudaMemcpyAsync(csr.keys, cs.keys, (size_t)ne * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s);
  csr.idBits = idBits;
  csr.n = n;
  long long threads = ne > 0 ? ne : (long long)n + 1;
  (k_csr_rows<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(cs.keys, ne, idBits, n, csr.rowptr), ++::wdem::g_kernel_launches);
  if (ne > 0)
    (k_csr_ent_slots<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(cs.vals, cs.keys, idBits, csr.rowptr, ne, csr.ent, c.slot, c.rowBit),
     ++::wdem::g_kernel_launches);
}

}  // namespace wdem
