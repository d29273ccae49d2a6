// k_mlp.cu -- the learned warm start of the ellipsoid contact solve.
//
// A 13 -> 64 -> 64 -> 64 -> 4 multilayer perceptron (ReLU hidden layers) maps the state of an
// ellipsoid pair (centre offset in A's frame, relative orientation, both semi-axis triples; lengths
// divided by max(a) + max(b)) to the maximiser lambda of the Perram-Wertheim contact function and the
// contact point in A's frame.  Its lambda starts the Newton solve (WDEM_WARM_MLP); the solve falls
// back to the cold start when it has not converged after fallbackIters iterations.
//
// Arithmetic: BF16 operands, FP32 accumulation, on the 5th-generation tensor cores (tcgen05.mma with the
// accumulators in tensor memory).  Rounding points, which the CPU reference of the network follows:
// inputs, weights and post-ReLU activations are rounded to BF16, and so are the dZ operands of the
// backward products; biases, pre-activations, outputs and bias gradients stay FP32.  Inference (the warm
// start of the contact pass and wdem_warm_predict) is k_mlp_tc; training (k_mlp_grad_tc) runs forward,
// backward and the weight-gradient products of tiles of 128 records, and Adam (Kingma & Ba 2015) updates
// FP32 master weights (k_adam).
//
// Parameter layout on the device (padded): W1[16][64] (input rows 13..15 zero), b1[64], W2[64][64],
// b2[64], W3[64][64], b3[64], W4[64][8] (output columns 4..7 zero), b4[8]; W[l][in][out] row-major.
#include <cuda_bf16.h>
#include <cstdint>
#include <vector>

#include "wdem_internal.h"
#include "wdem_math.cuh"
#include "wdem_ell.cuh"
#include "../../include/wdem.h"

namespace wdem {

namespace {

constexpr int H = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + 16 * H, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H, OFF_W3 = OFF_B2 + H,
              OFF_B3 = OFF_W3 + H * H, OFF_W4 = OFF_B3 + H, OFF_B4 = OFF_W4 + H * 8, NPAD = OFF_B4 + 8;
// loss weights of the four outputs: lambda, contact point x, y, z
__constant__ float c_lossW[4] = {1.0f, 0.1f, 0.1f, 0.1f};

__device__ __forceinline__ uint16_t bf(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }
__device__ __forceinline__ float fbf(uint16_t u) { return __bfloat162float(__ushort_as_bfloat16(u)); }
__device__ __forceinline__ uint32_t pk(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }

// Adam (Kingma & Ba 2015) on the FP32 master weights; refreshes the BF16 copy and clears the gradient.
__global__ void k_adam(float* w, float* m, float* v, float* grad, uint16_t* wbf, int n, float lr, float b1, float b2,
                       float c1, float c2, float eps) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float gk = grad[k];
  const float mk_ = b1 * m[k] + (1.f - b1) * gk;
  const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
  m[k] = mk_;
  v[k] = vk;
  const float mh = mk_ / c1, vh = vk / c2;
  const float wk = w[k] - lr * mh / (sqrtf(vh) + eps);
  w[k] = wk;
  wbf[k] = bf(wk);
  grad[k] = 0.f;
}

__global__ void k_to_bf16(const float* w, uint16_t* wbf, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) wbf[k] = bf(w[k]);
}

// ------------------------------------------------------------------------------ inference on tcgen05
// The same network for tiles of 128 samples on the 5th-generation tensor cores: one CTA of 4 warps per
// tile (thread t owns sample t), BF16 operands in shared memory, FP32 accumulators in tensor memory (TMEM),
// one elected thread issuing tcgen05.mma (M = 128, N = 64 or 16, K = 16 per instruction) and committing to
// an mbarrier; the epilogue of each layer (bias, ReLU, BF16 rounding) reads the accumulator rows back with
// tcgen05.ld and writes the next layer's A operand.  Rounding points as listed at the top of this file.
//
// Operand layout: the canonical K-major layout without swizzling, 8 x 16-byte core matrices; element
// (r, k) of an R x K operand at (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2 bytes, with
// LBO = 128 (core matrices adjacent along K) and SBO = K / 8 * 128 (the next 8 rows).  A holds the
// samples (rows) x inputs, B the outputs (rows) x inputs, i.e. W transposed.
constexpr int TC_M = 128;            // samples per tile
constexpr int TC_N4 = 16;            // output layer padded to the smallest N for M = 128
constexpr int TC_W1 = 0;                          // B of layer 1: 64 x 16
constexpr int TC_W2 = TC_W1 + H * 16 * 2;         // B of layer 2: 64 x 64
constexpr int TC_W3 = TC_W2 + H * H * 2;          // B of layer 3
constexpr int TC_W4 = TC_W3 + H * H * 2;          // B of layer 4: 16 x 64
constexpr int TC_X = TC_W4 + TC_N4 * H * 2;       // A of layer 1: 128 x 16
constexpr int TC_H = TC_X + TC_M * 16 * 2;        // A of layers 2-4: 128 x 64
constexpr int TC_B = TC_H + TC_M * H * 2;         // biases, FP32: b1, b2, b3 (64 each), b4 (16)
constexpr int TC_BAR = TC_B + (3 * H + TC_N4) * 4;  // mbarrier (8 bytes)
constexpr int TC_TMEM = TC_BAR + 8;               // TMEM base address written by tcgen05.alloc
constexpr size_t SMEM_TC = TC_TMEM + 8 + 1024;    // + alignment slack of the dynamic base
constexpr unsigned TC_COLS = 64;                  // TMEM columns: one 128 x 64 FP32 accumulator
constexpr long long TC_SPIN = 1ll << 26;          // bounded mbarrier wait

__device__ __forceinline__ uint32_t kmajorOff(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
// tcgen05 shared-memory matrix descriptor: start >> 4 (bits 0-13), LBO >> 4 (16-29), SBO >> 4 (32-45),
// the fixed 0b001 at bits 46-48, base offset 0, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t tcDesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9 and 10-12 = 1), both
// K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
__host__ __device__ constexpr uint32_t tcIdesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tcMma(uint32_t dTmem, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dTmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void tcCommit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// waits for the mbarrier phase `parity` to complete; false after TC_SPIN polls
__device__ __forceinline__ bool tcWait(uint32_t bar, unsigned parity) {
  for (long long it = 0; it < TC_SPIN; it++) {
    unsigned done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void tcFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tcFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxyFence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive accumulator columns of this thread's row (warp w reads TMEM lanes 32 w .. 32 w + 31)
__device__ __forceinline__ void tcLoad16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

// one layer: D = A (128 x K, at aOff) x B^T (N x K, at bOff), issued by thread 0, waited for by all;
// false when the wait gave up
template <int K, int N>
__device__ __forceinline__ bool tcLayer(unsigned char* sm, int aOff, int bOff, uint32_t dTmem, uint32_t bar,
                                        unsigned& phase) {
  proxyFence();  // this thread's st.shared of the operands, visible to the tensor core
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (threadIdx.x == 0) {
    const uint32_t a0 = smemAddr(sm + aOff), b0 = smemAddr(sm + bOff);
#pragma unroll
    for (int ks = 0; ks < K / 16; ks++)
      tcMma(dTmem, tcDesc(a0 + 256 * ks, 128, K / 8 * 128), tcDesc(b0 + 256 * ks, 128, K / 8 * 128), tcIdesc(TC_M, N),
            ks > 0 ? 1 : 0);
    tcCommit(smemAddr(sm + TC_BAR));
  }
  const bool ok = tcWait(bar, phase);
  phase ^= 1u;
  tcFenceAfter();
  return __syncthreads_and(ok) != 0;  // the same answer in every thread: all leave the tile loop together
}

// hidden-layer epilogue: this thread's accumulator row + bias, ReLU, BF16, into row t of the 128 x 64 A tile
// at dst (default: the inference kernel's activation tile)
__device__ __forceinline__ void tcHidden(unsigned char* sm, uint32_t tRow, const float* bias, int t, int dst = TC_H) {
#pragma unroll
  for (int c = 0; c < H; c += 16) {
    float v[16];
    tcLoad16(tRow + c, v);
    uint32_t w[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
      w[k] = pk(bf(fmaxf(v[2 * k] + bias[c + 2 * k], 0.f)), bf(fmaxf(v[2 * k + 1] + bias[c + 2 * k + 1], 0.f)));
    *reinterpret_cast<uint4*>(sm + dst + kmajorOff(t, c, H)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(sm + dst + kmajorOff(t, c + 8, H)) = make_uint4(w[4], w[5], w[6], w[7]);
  }
}

// The network over tiles of 128 samples.  WORK: the samples are the contact work list (features from the
// particle state of each ellipsoid pair that the contact pass may solve; lam0 written, NaN = cold start;
// with onlyFresh, pairs that carry the previous step's maximiser get NaN too, and a tile whose 128 pairs all
// carry one skips the network); otherwise feature rows X -> output rows Y.
template <bool WORK>
__global__ void __launch_bounds__(128, 1) k_mlp_tc(Particles p, Contacts c, const unsigned* work, const unsigned* count,
                                                   long long ncon, const float* X, long long nx, float* Y,
                                                   const uint16_t* wbf, const float* wf, int onlyFresh,
                                                   DeviceStatus* st) {
  extern __shared__ unsigned char smRaw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smRaw) + 1023) & ~uintptr_t(1023));
  const int t = threadIdx.x, warp = t >> 5;
  // weights as B operands (W transposed: output rows, input columns), biases
  for (int e = t; e < H * 16; e += blockDim.x) {
    const int n = e / 16, k = e % 16;
    *reinterpret_cast<uint16_t*>(sm + TC_W1 + kmajorOff(n, k, 16)) = wbf[OFF_W1 + k * H + n];
  }
  for (int e = t; e < H * H; e += blockDim.x) {
    const int n = e / H, k = e % H;
    *reinterpret_cast<uint16_t*>(sm + TC_W2 + kmajorOff(n, k, H)) = wbf[OFF_W2 + k * H + n];
    *reinterpret_cast<uint16_t*>(sm + TC_W3 + kmajorOff(n, k, H)) = wbf[OFF_W3 + k * H + n];
  }
  for (int e = t; e < TC_N4 * H; e += blockDim.x) {
    const int n = e / H, k = e % H;
    *reinterpret_cast<uint16_t*>(sm + TC_W4 + kmajorOff(n, k, H)) = n < 8 ? wbf[OFF_W4 + k * 8 + n] : (uint16_t)0;
  }
  float* bias = reinterpret_cast<float*>(sm + TC_B);
  for (int e = t; e < 3 * H + TC_N4; e += blockDim.x) {
    const int l = e / H, j = e % H;
    bias[e] = l == 0 ? wf[OFF_B1 + j] : (l == 1 ? wf[OFF_B2 + j] : (l == 2 ? wf[OFF_B3 + j] : (j < 8 ? wf[OFF_B4 + j] : 0.f)));
  }
  const uint32_t bar = smemAddr(sm + TC_BAR);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(sm + TC_TMEM)),
                 "r"(TC_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + TC_TMEM);
  const uint32_t tRow = tmem + ((uint32_t)(32 * warp) << 16);  // this thread's accumulator row (lane 32 w + lane)
  unsigned phase = 0;
  bool ok = true;
  const long long n = WORK ? (long long)workLen(count) : nx;
  for (long long base = (long long)blockIdx.x * TC_M; base < n && ok; base += (long long)gridDim.x * TC_M) {
    const long long s = base + t;
    long long i = -1;
    bool use = false;
    float f[16];
#pragma unroll
    for (int k = 0; k < 16; k++) f[k] = 0.f;
    if (WORK) {
      i = s < n ? (long long)workItem(work, count, ncon, (unsigned)s) : -1;
      if (i >= 0) {
        const uint8_t sb = c.state[i] & CS_SHAPES;
        const bool hasLam = onlyFresh && c.lam && c.lam[i] > 0 && c.lam[i] < 1;
        const int2 id = c.ids[i];
        const bool ellPair = (p.meta[id.x].x & 15) != WDEM_SHAPE_CAPSULE && (p.meta[id.y].x & 15) != WDEM_SHAPE_CAPSULE;
        if ((sb & CS_ELL) && !(sb & CS_WALL_A) && ellPair && (c.state[i] & CS_MASK) != CS_DEAD && !hasLam) {
          const double4_32a OA = p.ori[id.x], OB = p.ori[id.y];
          qd oa, ob;
          oa.w = OA.x; oa.x = OA.y; oa.y = OA.z; oa.z = OA.w;
          ob.w = OB.x; ob.x = OB.y; ob.y = OB.z; ob.z = OB.w;
          const d3 R = xyz(p.posr[id.y]) - xyz(p.posr[id.x]);
          ellFeatures(oa, xyz(p.semi[id.x]), ob, xyz(p.semi[id.y]), R, f);
          use = true;
        }
      }
    } else if (s < n) {
      for (int k = 0; k < ELL_FEATURES; k++) f[k] = X[s * ELL_FEATURES + k];
      use = true;
    }
    // a tile none of whose pairs needs the network: cold starts only
    if (!__syncthreads_or(use)) {
      if (WORK && i >= 0) c.lam0[i] = __int_as_float(0x7fffffff);
      continue;
    }
    uint32_t xw[8];
#pragma unroll
    for (int k = 0; k < 8; k++) xw[k] = pk(bf(f[2 * k]), bf(f[2 * k + 1]));
    *reinterpret_cast<uint4*>(sm + TC_X + kmajorOff(t, 0, 16)) = make_uint4(xw[0], xw[1], xw[2], xw[3]);
    *reinterpret_cast<uint4*>(sm + TC_X + kmajorOff(t, 8, 16)) = make_uint4(xw[4], xw[5], xw[6], xw[7]);
    if (!(ok = tcLayer<16, H>(sm, TC_X, TC_W1, tmem, bar, phase))) break;
    tcHidden(sm, tRow, bias, t);
    if (!(ok = tcLayer<H, H>(sm, TC_H, TC_W2, tmem, bar, phase))) break;
    tcHidden(sm, tRow, bias + H, t);
    if (!(ok = tcLayer<H, H>(sm, TC_H, TC_W3, tmem, bar, phase))) break;
    tcHidden(sm, tRow, bias + 2 * H, t);
    if (!(ok = tcLayer<H, TC_N4>(sm, TC_H, TC_W4, tmem, bar, phase))) break;
    float o[16];
    tcLoad16(tRow, o);
    if (WORK) {
      if (i >= 0) {
        const float l = fminf(fmaxf(o[0] + bias[3 * H], 1e-3f), 1.f - 1e-3f);
        c.lam0[i] = use ? l : __int_as_float(0x7fffffff);
      }
    } else if (s < n) {
      for (int k = 0; k < ELL_TARGETS; k++) Y[s * ELL_TARGETS + k] = o[k] + bias[3 * H + k];
    }
    tcFenceBefore();  // the accumulator reads are done before the next tile's first MMA overwrites it
  }
  // a round that timed out may still have MMAs running: wait for its commit once more (bounded) before the
  // accumulator columns and the barrier's shared memory are given up
  if (!ok) tcWait(bar, phase ^ 1u);
  if (!ok && t == 0) {
    atomicCAS(&st->code, 0, WDEM_ERR_TIMEOUT);
    st->detail = -1;
  }
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_COLS) : "memory");
}

// ------------------------------------------------------------------------------ training on tcgen05
// Forward, backward and weight gradients of tiles of 128 records on the tensor cores.  Per tile: the four
// forward layers as in k_mlp_tc (activations H1..H3 kept in shared memory), the output error dZ4, then per
// layer l = 4..1: dW_l += H_{l-1}^T dZ_l (M = inputs padded to 128, N = outputs, K = the 128 samples; the
// accumulators stay in TMEM across all tiles of the CTA) and dA_{l-1} = dZ_l W_l^T (M = 128 samples, N = 64
// inputs, K = outputs), whose epilogue masks by ReLU' (H_{l-1} > 0) and rounds to BF16 the next dZ.  The
// transposed operands (H^T, dZ^T: samples along K) are written by each thread into its sample's column.
// Bias gradients and the loss are summed from the FP32 values (warp shuffles, then shared atomics), as in
// the warp-level kernel; the CTA adds everything to the global gradient once, at the end.
constexpr int TT_FW1 = 0;                          // forward B operands (W^T: outputs x inputs)
constexpr int TT_FW2 = TT_FW1 + H * 16 * 2;
constexpr int TT_FW3 = TT_FW2 + H * H * 2;
constexpr int TT_FW4 = TT_FW3 + H * H * 2;         // 16 x 64
constexpr int TT_BW4 = TT_FW4 + TC_N4 * H * 2;     // backward B operands (W: inputs x outputs): 64 x 16
constexpr int TT_BW3 = TT_BW4 + H * TC_N4 * 2;     // 64 x 64
constexpr int TT_BW2 = TT_BW3 + H * H * 2;
constexpr int TT_X = TT_BW2 + H * H * 2;           // 128 x 16
constexpr int TT_H1 = TT_X + TC_M * 16 * 2;        // 128 x 64 each
constexpr int TT_H2 = TT_H1 + TC_M * H * 2;
constexpr int TT_H3 = TT_H2 + TC_M * H * 2;
constexpr int TT_DZ = TT_H3 + TC_M * H * 2;        // dZ as the A operand of dA (128 x 64, or x 16 for dZ4)
constexpr int TT_AT = TT_DZ + TC_M * H * 2;        // H^T or X^T: 128 (inputs, zero-padded) x 128 samples
constexpr int TT_DZT = TT_AT + TC_M * TC_M * 2;    // dZ^T: 64 (outputs) x 128 samples
constexpr int TT_BIAS = TT_DZT + H * TC_M * 2;     // b1, b2, b3, b4 (FP32)
constexpr int TT_GB = TT_BIAS + (3 * H + TC_N4) * 4;  // bias-gradient sums of the CTA
constexpr int TT_LOSS = TT_GB + (3 * H + TC_N4) * 4;
constexpr int TT_BAR = TT_LOSS + 8;
constexpr int TT_TMEM = TT_BAR + 8;
constexpr size_t SMEM_TC_TRAIN = TT_TMEM + 8 + 1024;
constexpr unsigned TT_COLS = 512;                  // TMEM: scratch 0..63, dW4 64..79, dW3 128.., dW2 192.., dW1 256..
constexpr uint32_t TT_DW4 = 64, TT_DW3 = 128, TT_DW2 = 192, TT_DW1 = 256;

// all threads: operands visible, one barrier; thread 0 runs `issue` (its MMAs) and commits; all wait.  The
// same answer in every thread (false: the wait gave up).
template <class F>
__device__ __forceinline__ bool tcRound(unsigned char* sm, uint32_t bar, unsigned& phase, F issue) {
  proxyFence();
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (threadIdx.x == 0) {
    issue();
    tcCommit(bar);
  }
  const bool ok = tcWait(bar, phase);
  phase ^= 1u;
  tcFenceAfter();
  return __syncthreads_and(ok) != 0;
}
// D (TMEM) (+)= A (128 x K at aOff) x B^T (N x K at bOff), K-major operands
template <int K, int N>
__device__ __forceinline__ void tcIssue(unsigned char* sm, int aOff, int bOff, uint32_t d, bool accumulate) {
  const uint32_t a0 = smemAddr(sm + aOff), b0 = smemAddr(sm + bOff);
#pragma unroll
  for (int ks = 0; ks < K / 16; ks++)
    tcMma(d, tcDesc(a0 + 256 * ks, 128, K / 8 * 128), tcDesc(b0 + 256 * ks, 128, K / 8 * 128), tcIdesc(TC_M, N),
          (ks > 0 || accumulate) ? 1 : 0);
}
// column sums of the warp (FP32, shuffles) added to the CTA's sums
__device__ __forceinline__ void warpColumnAdd(float* dst, const float* v, int cols) {
  for (int c = 0; c < cols; c++) {
    float x = v[c];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&dst[c], x);
  }
}
// the sample's column of a transposed operand: element (r, t) of an R x 128 K-major tile, r = 0 .. cols-1
__device__ __forceinline__ void putColumn(unsigned char* sm, int off, int t, const uint16_t* v, int cols) {
  for (int r = 0; r < cols; r++) *reinterpret_cast<uint16_t*>(sm + off + kmajorOff(r, t, TC_M)) = v[r];
}
// this thread's row of a 128 x 64 activation tile
__device__ __forceinline__ void getRow64(const unsigned char* sm, int off, int t, uint16_t* v) {
  for (int c = 0; c < H; c += 8) {
    const uint4 q = *reinterpret_cast<const uint4*>(sm + off + kmajorOff(t, c, H));
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
    for (int k = 0; k < 4; k++) { v[c + 2 * k] = (uint16_t)(w[k] & 0xffff); v[c + 2 * k + 1] = (uint16_t)(w[k] >> 16); }
  }
}
// dZ_prev = dA (this thread's accumulator row) masked by ReLU' of the activation row hv; bias-gradient sums;
// dZ_prev as the next A operand (row t) and as the transposed B operand (column t)
__device__ __forceinline__ void backEpilogue(unsigned char* sm, uint32_t tRow, const uint16_t* hv, float* gb, int t) {
  float z[H];
#pragma unroll
  for (int c = 0; c < H; c += 16) tcLoad16(tRow + c, z + c);
  uint16_t zb[H];
#pragma unroll
  for (int c = 0; c < H; c++) {
    z[c] = fbf(hv[c]) > 0.f ? z[c] : 0.f;
    zb[c] = bf(z[c]);
  }
  warpColumnAdd(gb, z, H);
  for (int c = 0; c < H; c += 8) {
    uint32_t w[4];
    for (int k = 0; k < 4; k++) w[k] = pk(zb[c + 2 * k], zb[c + 2 * k + 1]);
    *reinterpret_cast<uint4*>(sm + TT_DZ + kmajorOff(t, c, H)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  putColumn(sm, TT_DZT, t, zb, H);
}

__global__ void __launch_bounds__(128, 1) k_mlp_grad_tc(const float* rec, const int* idx, long long n, float invN,
                                                        const uint16_t* wbf, const float* wf, float* grad, float* loss,
                                                        DeviceStatus* st) {
  extern __shared__ unsigned char smRaw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smRaw) + 1023) & ~uintptr_t(1023));
  const int t = threadIdx.x, warp = t >> 5;
  // weights: forward B (W^T) and backward B (W), biases; the padded rows of H^T stay zero
  for (int e = t; e < H * 16; e += blockDim.x) {
    const int nn = e / 16, k = e % 16;
    *reinterpret_cast<uint16_t*>(sm + TT_FW1 + kmajorOff(nn, k, 16)) = wbf[OFF_W1 + k * H + nn];
  }
  for (int e = t; e < H * H; e += blockDim.x) {
    const int a = e / H, b = e % H;
    *reinterpret_cast<uint16_t*>(sm + TT_FW2 + kmajorOff(a, b, H)) = wbf[OFF_W2 + b * H + a];
    *reinterpret_cast<uint16_t*>(sm + TT_FW3 + kmajorOff(a, b, H)) = wbf[OFF_W3 + b * H + a];
    *reinterpret_cast<uint16_t*>(sm + TT_BW3 + kmajorOff(a, b, H)) = wbf[OFF_W3 + a * H + b];
    *reinterpret_cast<uint16_t*>(sm + TT_BW2 + kmajorOff(a, b, H)) = wbf[OFF_W2 + a * H + b];
  }
  for (int e = t; e < TC_N4 * H; e += blockDim.x) {
    const int a = e / H, b = e % H;  // forward: output a, input b
    *reinterpret_cast<uint16_t*>(sm + TT_FW4 + kmajorOff(a, b, H)) = a < 8 ? wbf[OFF_W4 + b * 8 + a] : (uint16_t)0;
    const int i = e / TC_N4, o = e % TC_N4;  // backward: input i, output o
    *reinterpret_cast<uint16_t*>(sm + TT_BW4 + kmajorOff(i, o, TC_N4)) = o < 8 ? wbf[OFF_W4 + i * 8 + o] : (uint16_t)0;
  }
  for (int e = t; e < TC_M * TC_M / 8; e += blockDim.x) reinterpret_cast<uint4*>(sm + TT_AT)[e] = make_uint4(0, 0, 0, 0);
  float* bias = reinterpret_cast<float*>(sm + TT_BIAS);
  float* gb = reinterpret_cast<float*>(sm + TT_GB);
  for (int e = t; e < 3 * H + TC_N4; e += blockDim.x) {
    const int l = e / H, j = e % H;
    bias[e] = l == 0 ? wf[OFF_B1 + j] : (l == 1 ? wf[OFF_B2 + j] : (l == 2 ? wf[OFF_B3 + j] : (j < 8 ? wf[OFF_B4 + j] : 0.f)));
    gb[e] = 0.f;
  }
  if (t == 0) *reinterpret_cast<float*>(sm + TT_LOSS) = 0.f;
  const uint32_t bar = smemAddr(sm + TT_BAR);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(sm + TT_TMEM)),
                 "r"(TT_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + TT_TMEM);
  const uint32_t lane0 = (uint32_t)(32 * warp) << 16;
  const uint32_t tRow = tmem + lane0;
  unsigned phase = 0;
  bool ok = true, first = true;
  float myLoss = 0.f;
  for (long long base = (long long)blockIdx.x * TC_M; base < n && ok; base += (long long)gridDim.x * TC_M) {
    const long long s = base + t;
    const bool valid = s < n;
    const float* r = valid ? rec + (long long)(idx ? idx[s] : s) * ELL_RECORD : nullptr;
    float f[16];
    for (int k = 0; k < 16; k++) f[k] = (valid && k < ELL_FEATURES) ? r[k] : 0.f;
    uint16_t xb[16];
    for (int k = 0; k < 16; k++) xb[k] = bf(f[k]);
    {
      uint32_t xw[8];
      for (int k = 0; k < 8; k++) xw[k] = pk(xb[2 * k], xb[2 * k + 1]);
      *reinterpret_cast<uint4*>(sm + TT_X + kmajorOff(t, 0, 16)) = make_uint4(xw[0], xw[1], xw[2], xw[3]);
      *reinterpret_cast<uint4*>(sm + TT_X + kmajorOff(t, 8, 16)) = make_uint4(xw[4], xw[5], xw[6], xw[7]);
    }
    // forward
    if (!(ok = tcRound(sm, bar, phase, [&] { tcIssue<16, H>(sm, TT_X, TT_FW1, tmem, false); }))) break;
    tcHidden(sm, tRow, bias, t, TT_H1);
    if (!(ok = tcRound(sm, bar, phase, [&] { tcIssue<H, H>(sm, TT_H1, TT_FW2, tmem, false); }))) break;
    tcHidden(sm, tRow, bias + H, t, TT_H2);
    if (!(ok = tcRound(sm, bar, phase, [&] { tcIssue<H, H>(sm, TT_H2, TT_FW3, tmem, false); }))) break;
    tcHidden(sm, tRow, bias + 2 * H, t, TT_H3);
    if (!(ok = tcRound(sm, bar, phase, [&] { tcIssue<H, TC_N4>(sm, TT_H3, TT_FW4, tmem, false); }))) break;
    // output error: dZ4 = 2 w (o - y) / n (zero for padded samples), its bias gradient, the loss
    {
      float o[16], d[16];
      tcLoad16(tRow, o);
      for (int k = 0; k < 16; k++) d[k] = 0.f;
      if (valid)
        for (int k = 0; k < ELL_TARGETS; k++) {
          const float e = o[k] + bias[3 * H + k] - r[ELL_FEATURES + k];
          myLoss += c_lossW[k] * e * e * invN;
          d[k] = 2.f * c_lossW[k] * e * invN;
        }
      warpColumnAdd(gb + 3 * H, d, ELL_TARGETS);
      uint16_t db[16];
      for (int k = 0; k < 16; k++) db[k] = bf(d[k]);
      uint32_t w[8];
      for (int k = 0; k < 8; k++) w[k] = pk(db[2 * k], db[2 * k + 1]);
      *reinterpret_cast<uint4*>(sm + TT_DZ + kmajorOff(t, 0, TC_N4)) = make_uint4(w[0], w[1], w[2], w[3]);
      *reinterpret_cast<uint4*>(sm + TT_DZ + kmajorOff(t, 8, TC_N4)) = make_uint4(w[4], w[5], w[6], w[7]);
      putColumn(sm, TT_DZT, t, db, TC_N4);
      uint16_t hv[H];
      getRow64(sm, TT_H3, t, hv);
      putColumn(sm, TT_AT, t, hv, H);
    }
    const bool acc = !first;
    // layer 4: dW4, dA3
    if (!(ok = tcRound(sm, bar, phase, [&] {
          tcIssue<TC_M, TC_N4>(sm, TT_AT, TT_DZT, tmem + TT_DW4, acc);
          tcIssue<TC_N4, H>(sm, TT_DZ, TT_BW4, tmem, false);
        })))
      break;
    {
      uint16_t hv[H];
      getRow64(sm, TT_H3, t, hv);
      backEpilogue(sm, tRow, hv, gb + 2 * H, t);
      getRow64(sm, TT_H2, t, hv);
      putColumn(sm, TT_AT, t, hv, H);
    }
    // layer 3: dW3, dA2
    if (!(ok = tcRound(sm, bar, phase, [&] {
          tcIssue<TC_M, H>(sm, TT_AT, TT_DZT, tmem + TT_DW3, acc);
          tcIssue<H, H>(sm, TT_DZ, TT_BW3, tmem, false);
        })))
      break;
    {
      uint16_t hv[H];
      getRow64(sm, TT_H2, t, hv);
      backEpilogue(sm, tRow, hv, gb + H, t);
      getRow64(sm, TT_H1, t, hv);
      putColumn(sm, TT_AT, t, hv, H);
    }
    // layer 2: dW2, dA1
    if (!(ok = tcRound(sm, bar, phase, [&] {
          tcIssue<TC_M, H>(sm, TT_AT, TT_DZT, tmem + TT_DW2, acc);
          tcIssue<H, H>(sm, TT_DZ, TT_BW2, tmem, false);
        })))
      break;
    {
      uint16_t hv[H];
      getRow64(sm, TT_H1, t, hv);
      backEpilogue(sm, tRow, hv, gb, t);
      // X^T in rows 0..15 of the transposed operand, zeros over the rows of H1^T above them
      uint16_t xv[H];
      for (int k = 0; k < H; k++) xv[k] = k < 16 ? xb[k] : (uint16_t)0;
      putColumn(sm, TT_AT, t, xv, H);
    }
    // layer 1: dW1
    if (!(ok = tcRound(sm, bar, phase, [&] { tcIssue<TC_M, H>(sm, TT_AT, TT_DZT, tmem + TT_DW1, acc); }))) break;
    first = false;
  }
  if (!ok) tcWait(bar, phase ^ 1u);  // as in k_mlp_tc: the timed-out round's MMAs, before TMEM is freed
  if (!ok && t == 0) {
    atomicCAS(&st->code, 0, WDEM_ERR_TIMEOUT);
    st->detail = -1;
  }
  // the CTA's sums into the global gradient: weight rows are TMEM lanes (inputs), columns the outputs
  if (ok && !first) {
    const int m = 32 * warp + (t & 31);  // this thread's input row
    for (int c = 0; c < TC_N4; c += 16) {
      float v[16];
      tcLoad16(tmem + lane0 + TT_DW4 + c, v);
      if (m < H)
        for (int k = 0; k < 8; k++) if (v[k] != 0.f) atomicAdd(&grad[OFF_W4 + m * 8 + k], v[k]);
    }
    for (int c = 0; c < H; c += 16) {
      float v3[16], v2[16], v1[16];
      tcLoad16(tmem + lane0 + TT_DW3 + c, v3);
      tcLoad16(tmem + lane0 + TT_DW2 + c, v2);
      tcLoad16(tmem + lane0 + TT_DW1 + c, v1);
      for (int k = 0; k < 16; k++) {
        if (m < H && v3[k] != 0.f) atomicAdd(&grad[OFF_W3 + m * H + c + k], v3[k]);
        if (m < H && v2[k] != 0.f) atomicAdd(&grad[OFF_W2 + m * H + c + k], v2[k]);
        if (m < 16 && v1[k] != 0.f) atomicAdd(&grad[OFF_W1 + m * H + c + k], v1[k]);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) myLoss += __shfl_xor_sync(0xffffffffu, myLoss, o);
  if ((t & 31) == 0) atomicAdd(reinterpret_cast<float*>(sm + TT_LOSS), myLoss);
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (ok && !first) {
    for (int e = t; e < 3 * H + ELL_TARGETS; e += blockDim.x) {
      const int l = e / H, j = e % H;
      const int off = l == 0 ? OFF_B1 + j : (l == 1 ? OFF_B2 + j : (l == 2 ? OFF_B3 + j : OFF_B4 + j));
      if (gb[e] != 0.f) atomicAdd(&grad[off], gb[e]);
    }
    if (t == 0) atomicAdd(loss, *reinterpret_cast<float*>(sm + TT_LOSS));
  }
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TT_COLS) : "memory");
}


}  // namespace

// ------------------------------------------------------------------------------ host side
int mlp_npad() { return NPAD; }

// public layout (W1 13x64, b1, W2, b2, W3, b3, W4 64x4, b4) <-> padded device layout
void mlp_unpack(const float* pub, float* pad) {
  for (int k = 0; k < NPAD; k++) pad[k] = 0.f;
  const float* q = pub;
  for (int i = 0; i < ELL_FEATURES; i++) for (int j = 0; j < H; j++) pad[OFF_W1 + i * H + j] = *q++;
  for (int j = 0; j < H; j++) pad[OFF_B1 + j] = *q++;
  for (int i = 0; i < H; i++) for (int j = 0; j < H; j++) pad[OFF_W2 + i * H + j] = *q++;
  for (int j = 0; j < H; j++) pad[OFF_B2 + j] = *q++;
  for (int i = 0; i < H; i++) for (int j = 0; j < H; j++) pad[OFF_W3 + i * H + j] = *q++;
  for (int j = 0; j < H; j++) pad[OFF_B3 + j] = *q++;
  for (int i = 0; i < H; i++) for (int j = 0; j < ELL_TARGETS; j++) pad[OFF_W4 + i * 8 + j] = *q++;
  for (int j = 0; j < ELL_TARGETS; j++) pad[OFF_B4 + j] = *q++;
}
void mlp_pack(const float* pad, float* pub) {
  float* q = pub;
  for (int i = 0; i < ELL_FEATURES; i++) for (int j = 0; j < H; j++) *q++ = pad[OFF_W1 + i * H + j];
  for (int j = 0; j < H; j++) *q++ = pad[OFF_B1 + j];
  for (int i = 0; i < H; i++) for (int j = 0; j < H; j++) *q++ = pad[OFF_W2 + i * H + j];
  for (int j = 0; j < H; j++) *q++ = pad[OFF_B2 + j];
  for (int i = 0; i < H; i++) for (int j = 0; j < H; j++) *q++ = pad[OFF_W3 + i * H + j];
  for (int j = 0; j < H; j++) *q++ = pad[OFF_B3 + j];
  for (int i = 0; i < H; i++) for (int j = 0; j < ELL_TARGETS; j++) *q++ = pad[OFF_W4 + i * 8 + j];
  for (int j = 0; j < ELL_TARGETS; j++) *q++ = pad[OFF_B4 + j];
}

cudaError_t mlp_prepare_kernels() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_mlp_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TC))) return e;
  if ((e = cudaFuncSetAttribute(k_mlp_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TC))) return e;
  if ((e = cudaFuncSetAttribute(k_mlp_grad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TC_TRAIN))) return e;
  return cudaSuccess;
}

void mlp_to_bf16(cudaStream_t s, const float* w, uint16_t* wbf) {
  (k_to_bf16<<<(NPAD + 255) / 256, 256, 0, s>>>(w, wbf, NPAD), ++::wdem::g_kernel_launches);
}

void mlp_launch_warm(cudaStream_t s, Particles p, Contacts c, long long nc, const unsigned* work, const unsigned* count,
                     const uint16_t* wbf, const float* wf, bool onlyFresh, DeviceStatus* st, int numSMs) {
  if (nc <= 0) return;
  long long blocks = (nc + TC_M - 1) / TC_M;
  const long long cap = 2ll * (numSMs > 0 ? numSMs : 152);  // persistent blocks: weights staged once per block
  if (blocks > cap) blocks = cap;
  (k_mlp_tc<true><<<(unsigned)blocks, 128, SMEM_TC, s>>>(p, c, work, count, nc, nullptr, 0, nullptr, wbf, wf,
                                                          onlyFresh ? 1 : 0, st),
   ++::wdem::g_kernel_launches);
}

void mlp_launch_predict(cudaStream_t s, const float* X, long long n, float* Y, const uint16_t* wbf, const float* wf,
                        DeviceStatus* st) {
  if (n <= 0) return;
  long long blocks = (n + TC_M - 1) / TC_M;
  if (blocks > 152 * 4) blocks = 152 * 4;
  (k_mlp_tc<false><<<(unsigned)blocks, 128, SMEM_TC, s>>>(Particles{}, Contacts{}, nullptr, nullptr, 0, X, n, Y, wbf, wf,
                                                           0, st),
   ++::wdem::g_kernel_launches);
}

void mlp_launch_grad(cudaStream_t s, const float* rec, const int* idx, long long n, const uint16_t* wbf, const float* wf,
                     float* grad, float* loss, DeviceStatus* st, int numSMs) {
  if (n <= 0) return;
  long long blocks = (n + TC_M - 1) / TC_M;
  const long long sms = numSMs > 0 ? numSMs : 152;  // one CTA per SM: it holds 512 TMEM columns
  if (blocks > sms) blocks = sms;
  (k_mlp_grad_tc<<<(unsigned)blocks, 128, SMEM_TC_TRAIN, s>>>(rec, idx, n, 1.0f / (float)n, wbf, wf, grad, loss, st),
   ++::wdem::g_kernel_launches);
}

void mlp_launch_adam(cudaStream_t s, float* w, float* m, float* v, float* grad, uint16_t* wbf, float lr, float b1,
                     float b2, float c1, float c2, float eps) {
  (k_adam<<<(NPAD + 255) / 256, 256, 0, s>>>(w, m, v, grad, wbf, NPAD, lr, b1, b2, c1, c2, eps), ++::wdem::g_kernel_launches);
}

}  // namespace wdem
