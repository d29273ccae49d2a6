// wdem_pack.cu -- seeded random sequential addition of non-overlapping spheres in a box: the
// synthetic-input generator used in place of Woo's SpherePack::makeCloud
// (src/supp/sphere-pack/SpherePack.cpp:140-) for the benchmark scenes.  Host code only.
//
// Radii are drawn uniformly in [rMin, rMax] (or all rMin when equal), placed largest first; each
// sphere gets up to maxAttempts uniformly random centres inside the box shrunk by its radius and is
// kept at the first centre that overlaps no placed sphere (uniform grid of cell 2*rMax).  The
// random stream is SplitMix64 (Steele, Lea, Flood 2014), so a seed gives the same cloud on every
// machine.
#include "../../include/wdem.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
};

}  // namespace

extern "C" int64_t wdem_make_cloud(const double* lo, const double* hi, double rMin, double rMax, int64_t n,
                                   uint64_t seed, int32_t maxAttempts, double* centers, double* radii) {
  if (!lo || !hi || !centers || !radii || n < 0 || rMin <= 0 || rMax < rMin) return WDEM_ERR_ARG;
  SplitMix64 rng(seed);
  std::vector<double> r(n);
  for (int64_t i = 0; i < n; i++) r[i] = (rMax > rMin) ? rMin + (rMax - rMin) * rng.uniform() : rMin;
  std::sort(r.begin(), r.end(), [](double a, double b) { return a > b; });
  const double cell = 2 * rMax;
  int nc[3];
  for (int k = 0; k < 3; k++) nc[k] = std::max(1, (int)std::ceil((hi[k] - lo[k]) / cell));
  const int64_t ncells = (int64_t)nc[0] * nc[1] * nc[2];
  std::vector<int64_t> head(ncells, -1);
  std::vector<int64_t> next;
  next.reserve(n);
  std::vector<double> c;
  c.reserve(3 * n);
  std::vector<double> rr;
  rr.reserve(n);
  auto cellOf = [&](const double* x, int* ci) {
    for (int k = 0; k < 3; k++) {
      int v = (int)std::floor((x[k] - lo[k]) / cell);
      ci[k] = std::min(std::max(v, 0), nc[k] - 1);
    }
  };
  int64_t placed = 0;
  for (int64_t i = 0; i < n; i++) {
    const double ri = r[i];
    bool ok = false;
    double x[3];
    for (int a = 0; a < maxAttempts && !ok; a++) {
      for (int k = 0; k < 3; k++) x[k] = lo[k] + ri + (hi[k] - lo[k] - 2 * ri) * rng.uniform();
      int ci[3];
      cellOf(x, ci);
      ok = true;
      for (int dz = -1; dz <= 1 && ok; dz++)
        for (int dy = -1; dy <= 1 && ok; dy++)
          for (int dx = -1; dx <= 1 && ok; dx++) {
            int cx = ci[0] + dx, cy = ci[1] + dy, cz = ci[2] + dz;
            if (cx < 0 || cy < 0 || cz < 0 || cx >= nc[0] || cy >= nc[1] || cz >= nc[2]) continue;
            for (int64_t j = head[((int64_t)cz * nc[1] + cy) * nc[0] + cx]; j >= 0; j = next[j]) {
              double d0 = x[0] - c[3 * j], d1 = x[1] - c[3 * j + 1], d2 = x[2] - c[3 * j + 2];
              double s = ri + rr[j];
              if (d0 * d0 + d1 * d1 + d2 * d2 < s * s) { ok = false; break; }
            }
          }
    }
    if (!ok) continue;
    int ci[3];
    cellOf(x, ci);
    int64_t cidx = ((int64_t)ci[2] * nc[1] + ci[1]) * nc[0] + ci[0];
    c.push_back(x[0]); c.push_back(x[1]); c.push_back(x[2]);
    rr.push_back(ri);
    next.push_back(head[cidx]);
    head[cidx] = placed;
    placed++;
  }
  for (int64_t j = 0; j < placed; j++) {
    centers[3 * j] = c[3 * j]; centers[3 * j + 1] = c[3 * j + 1]; centers[3 * j + 2] = c[3 * j + 2];
    radii[j] = rr[j];
  }
  return placed;
}

// The same random sequential addition for caller-given radii (placed largest first), optionally in a
// periodic box: centres anywhere in [lo, hi), overlaps tested against the nearest periodic image and
// grid cells wrapped, so that the packing has no overlap across the faces either.
extern "C" int64_t wdem_make_cloud_radii(const double* lo, const double* hi, int32_t periodic, int64_t n,
                                         const double* rIn, uint64_t seed, int32_t maxAttempts, double* centers,
                                         double* radii) {
  if (!lo || !hi || !rIn || !centers || !radii || n < 0) return WDEM_ERR_ARG;
  std::vector<double> r(rIn, rIn + n);
  for (double v : r) if (!(v > 0)) return WDEM_ERR_ARG;
  std::sort(r.begin(), r.end(), [](double a, double b) { return a > b; });
  SplitMix64 rng(seed);
  const double rMax = n > 0 ? r[0] : 1.0;
  const double cell = 2 * rMax;
  double L[3];
  int nc[3];
  for (int k = 0; k < 3; k++) {
    L[k] = hi[k] - lo[k];
    nc[k] = std::max(1, (int)std::floor(L[k] / cell));  // cells at least 2 rMax wide
  }
  const int64_t ncells = (int64_t)nc[0] * nc[1] * nc[2];
  std::vector<int64_t> head(ncells, -1), next;
  next.reserve(n);
  std::vector<double> c, rr;
  c.reserve(3 * n);
  rr.reserve(n);
  auto cellOf = [&](const double* x, int* ci) {
    for (int k = 0; k < 3; k++) {
      int v = (int)std::floor((x[k] - lo[k]) / L[k] * nc[k]);
      ci[k] = std::min(std::max(v, 0), nc[k] - 1);
    }
  };
  int64_t placed = 0;
  for (int64_t i = 0; i < n; i++) {
    const double ri = r[i];
    bool ok = false;
    double x[3];
    for (int a = 0; a < maxAttempts && !ok; a++) {
      for (int k = 0; k < 3; k++)
        x[k] = periodic ? lo[k] + L[k] * rng.uniform() : lo[k] + ri + (L[k] - 2 * ri) * rng.uniform();
      int ci[3];
      cellOf(x, ci);
      ok = true;
      const int span[3] = {nc[0] >= 3 ? 1 : (nc[0] == 2 ? 1 : 0), nc[1] >= 3 ? 1 : (nc[1] == 2 ? 1 : 0),
                           nc[2] >= 3 ? 1 : (nc[2] == 2 ? 1 : 0)};
      for (int dz = -span[2]; dz <= span[2] && ok; dz++)
        for (int dy = -span[1]; dy <= span[1] && ok; dy++)
          for (int dx = -span[0]; dx <= span[0] && ok; dx++) {
            // periodic with two cells: -1 and +1 are the same neighbour
            if (periodic && nc[0] == 2 && dx == 1) continue;
            if (periodic && nc[1] == 2 && dy == 1) continue;
            if (periodic && nc[2] == 2 && dz == 1) continue;
            int cx = ci[0] + dx, cy = ci[1] + dy, cz = ci[2] + dz;
            if (periodic) {
              cx = (cx + nc[0]) % nc[0]; cy = (cy + nc[1]) % nc[1]; cz = (cz + nc[2]) % nc[2];
            } else if (cx < 0 || cy < 0 || cz < 0 || cx >= nc[0] || cy >= nc[1] || cz >= nc[2]) continue;
            for (int64_t j = head[((int64_t)cz * nc[1] + cy) * nc[0] + cx]; j >= 0; j = next[j]) {
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
    const int64_t cidx = ((int64_t)ci[2] * nc[1] + ci[1]) * nc[0] + ci[0];
    c.push_back(x[0]); c.push_back(x[1]); c.push_back(x[2]);
    rr.push_back(ri);
    next.push_back(head[cidx]);
    head[cidx] = placed;
    placed++;
  }
  for (int64_t j = 0; j < placed; j++) {
    centers[3 * j] = c[3 * j]; centers[3 * j + 1] = c[3 * j + 1]; centers[3 * j + 2] = c[3 * j + 2];
    radii[j] = rr[j];
  }
  return placed;
}
