// k_noalloc.cu -- stress tensor of the contact network with no device allocation.
//
// Same sum as k_stress_terms + the deterministic reductions (sum over real contacts of the global
// contact force times the branch vector pB image - pA, ContactLoop.cpp:218-229), but all scratch
// lives in one fixed file-scope device array: one block reduces a fixed chunk of NA_CHUNK contacts
// into 9 partial sums, and the last block to finish adds the partials in block order.  The result is
// deterministic (fixed chunks, fixed tree, fixed final order) and differs from the per-handle
// reduction only in the order of the additions.
//
// The array is shared by every handle on a device: two calls that overlap in time on one device
// (two host threads, or two streams) race on it and both results are undefined.  Calls must be
// serialised per device by the caller.
#include <mutex>

#include "wdem_internal.h"
#include "wdem_math.cuh"

namespace wdem {

namespace {

constexpr int NA_THREADS = 256;
constexpr long long NA_CHUNK = 4096;                     // contacts reduced by one block
constexpr int NA_MAX_BLOCKS = 4096;                      // partial-sum slots in the scratch array
constexpr size_t NA_PARTIAL_BYTES = sizeof(double) * 9 * NA_MAX_BLOCKS;   // 294,912 B
constexpr size_t NA_RESULT_OFFSET = NA_PARTIAL_BYTES;                     // 9 doubles
constexpr size_t NA_DONE_OFFSET = NA_PARTIAL_BYTES + 256;                 // block-completion counter
constexpr size_t NA_SCRATCH_BYTES = NA_PARTIAL_BYTES + 512;               // 295,424 B in all
static_assert(NA_RESULT_OFFSET + 9 * sizeof(double) <= NA_DONE_OFFSET, "scratch layout");
static_assert(NA_DONE_OFFSET + sizeof(unsigned) <= NA_SCRATCH_BYTES, "scratch layout");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_SCRATCH_BYTES];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
void* g_na_addr[NA_MAX_DEVICES] = {};

__global__ void __launch_bounds__(NA_THREADS)
k_stress_noalloc(StepParams P, Particles p, Contacts c, long long nc, unsigned char* scratch) {
  double* partial = (double*)scratch;
  double* result = (double*)(scratch + NA_RESULT_OFFSET);
  unsigned* done = (unsigned*)(scratch + NA_DONE_OFFSET);
  __shared__ double red[9][NA_THREADS];
  __shared__ bool last;
  const int t = threadIdx.x;
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const long long base = (long long)blockIdx.x * NA_CHUNK;
  const long long end = base + NA_CHUNK < nc ? base + NA_CHUNK : nc;
  for (long long i = base + t; i < end; i += NA_THREADS) {
    if ((c.state[i] & CS_MASK) != CS_REAL) continue;
    const int2 id = c.ids[i];
    d3 branch = xyz(p.posr[id.y]) - xyz(p.posr[id.x]);
    if (P.periodic) {
      const int4 cd = c.cdist[i];
      branch = branch + mvec(P.hS, mk((double)cd.x, (double)cd.y, (double)cd.z));
    }
    const double4_32a f4 = c.out[OUT_RECORDS * (long long)c.slot[i].x + OUT_F];  // pA's entry: the force on pA
    const double F[3] = {f4.x, f4.y, f4.z};
    const double b[3] = {branch.x, branch.y, branch.z};
    for (int r = 0; r < 3; r++)
      for (int q = 0; q < 3; q++) v[3 * r + q] = v[3 * r + q] + F[r] * b[q];
  }
  for (int q = 0; q < 9; q++) red[q][t] = v[q];
  __syncthreads();
  for (int s = NA_THREADS / 2; s > 0; s >>= 1) {
    if (t < s)
      for (int q = 0; q < 9; q++) red[q][t] = red[q][t] + red[q][t + s];
    __syncthreads();
  }
  if (t == 0) {
    for (int q = 0; q < 9; q++) partial[9 * blockIdx.x + q] = red[q][0];
    __threadfence();  // partials visible device-wide before the block counts itself done
    last = (atomicAdd(done, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last && t < 9) {
    __threadfence();
    double sum = 0;
    for (unsigned blk = 0; blk < gridDim.x; blk++) sum = sum + __ldcg(&partial[9 * blk + t]);
    result[t] = sum;
  }
}

}  // namespace

long long stress_noalloc_max_contacts() { return NA_CHUNK * NA_MAX_BLOCKS; }

// Device address of the scratch array, looked up once per device (cudaGetSymbolAddress may load the
// module on first use under lazy loading, so the first call on a device belongs outside any stream
// capture).  The address is kept for the life of the process: a cudaDeviceReset, which also invalidates
// every handle on that device, invalidates it too, and the library must not be used on that device again.
cudaError_t noalloc_scratch(int device, void** addr) {
  if (device < 0 || device >= NA_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_addr[device]) {
    void* a = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_na_addr[device] = a;
  }
  *addr = g_na_addr[device];
  return cudaSuccess;
}

// Clears the completion counter, reduces, and copies the 9 sums to out9 (host memory); asynchronous
// on s: the caller synchronises before reading out9.
cudaError_t launch_stress_noalloc(cudaStream_t s, const StepParams& P, Particles p, Contacts c, long long nc,
                                  void* scratch, double* out9) {
  unsigned char* sc = (unsigned char*)scratch;
  cudaError_t e = cudaMemsetAsync(sc + NA_DONE_OFFSET, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  const unsigned blocks = nc > 0 ? (unsigned)((nc + NA_CHUNK - 1) / NA_CHUNK) : 1u;
  if (blocks > (unsigned)NA_MAX_BLOCKS) return cudaErrorInvalidValue;
  (k_stress_noalloc<<<blocks, NA_THREADS, 0, s>>>(P, p, c, nc, sc), ++::wdem::g_kernel_launches);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return cudaMemcpyAsync(out9, sc + NA_RESULT_OFFSET, 9 * sizeof(double), cudaMemcpyDeviceToHost, s);
}

}  // namespace wdem
