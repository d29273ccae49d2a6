// k_mlp.cu -- the learned warm start of the ellipsoid contact solve.
//
// A 13 -> 64 -> 64 -> 64 -> 4 multilayer perceptron (ReLU hidden layers) maps the state of an
// ellipsoid pair (centre offset in A's frame, relative orientation, both semi-axis triples; lengths
// divided by max(a) + max(b)) to the maximiser lambda of the Perram-Wertheim contact function and the
// contact point in A's frame.  Its lambda starts the Newton solve (WDEM_WARM_MLP); the solve falls
// back to the cold start when it has not converged after fallbackIters iterations.
//
// Arithmetic: BF16 operands, FP32 accumulation, on the tensor cores.  Rounding points, which the CPU
// reference of the network follows: inputs, weights and post-ReLU activations are rounded to BF16;
// biases, pre-activations and outputs stay FP32.  Inference (the warm start of the contact pass and
// wdem_warm_predict) runs on the 5th-generation tensor cores (tcgen05.mma, accumulators in tensor
// memory, k_mlp_tc).  Training runs forward and backward with warp-level mma.sync.m16n8k16 (one warp =
// 16 samples, activations in shared memory; BF16 operands: activations, dZ, weights), sums the gradient
// of a mini-batch per block in shared memory, and applies Adam (Kingma & Ba 2015) to FP32 master weights.
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
constexpr int WARPS = 4;             // warps per block, 16 samples each
constexpr int SAMPLES = 16 * WARPS;  // samples per block
// loss weights of the four outputs: lambda, contact point x, y, z
__constant__ float c_lossW[4] = {1.0f, 0.1f, 0.1f, 0.1f};

// per-warp shared buffers (BF16 bits as uint16): x[16][16], a1..a3[16][64], dz[16][64]; out[16][8] fp32
struct WarpSmem {
  uint16_t x[16 * 16];
  uint16_t a[3][16 * H];
  uint16_t dz[16 * H];
  uint16_t dz4[16 * 16];
  float out[16 * 8];
};
// weights: BF16 copy of the padded parameter vector; biases FP32 (b1 at 0, b2 at 64, b3 at 128, b4 at 192)
constexpr int SB1 = 0, SB2 = 64, SB3 = 128, SB4 = 192, NB = 200;
struct NetSmem {
  uint16_t w[NPAD];
  float b[NB];
};

__device__ __forceinline__ uint16_t bf(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }
__device__ __forceinline__ float fbf(uint16_t u) { return __bfloat162float(__ushort_as_bfloat16(u)); }
__device__ __forceinline__ uint32_t pk(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Fragment loaders for m16n8k16 (row.col): lane = 4 * g + t.  A (16 x 16): rows g, g+8; columns 2t, 2t+1
// and 2t+8, 2t+9.  B (16 x 8): rows (k) 2t, 2t+1 and 2t+8, 2t+9; column (n) g.  C: rows g, g+8; columns
// 2t, 2t+1.
// A from a row-major tile T[16][ld] at column k0
__device__ __forceinline__ void fragA(const uint16_t* T, int ld, int k0, int g, int t, uint32_t* a) {
  a[0] = pk(T[g * ld + k0 + 2 * t], T[g * ld + k0 + 2 * t + 1]);
  a[1] = pk(T[(g + 8) * ld + k0 + 2 * t], T[(g + 8) * ld + k0 + 2 * t + 1]);
  a[2] = pk(T[g * ld + k0 + 2 * t + 8], T[g * ld + k0 + 2 * t + 9]);
  a[3] = pk(T[(g + 8) * ld + k0 + 2 * t + 8], T[(g + 8) * ld + k0 + 2 * t + 9]);
}
// A = S^T for S row-major [16 samples][ld]: A[m][k] = S[k][m0 + m]
__device__ __forceinline__ void fragAT(const uint16_t* S, int ld, int m0, int g, int t, uint32_t* a) {
  a[0] = pk(S[(2 * t) * ld + m0 + g], S[(2 * t + 1) * ld + m0 + g]);
  a[1] = pk(S[(2 * t) * ld + m0 + g + 8], S[(2 * t + 1) * ld + m0 + g + 8]);
  a[2] = pk(S[(2 * t + 8) * ld + m0 + g], S[(2 * t + 9) * ld + m0 + g]);
  a[3] = pk(S[(2 * t + 8) * ld + m0 + g + 8], S[(2 * t + 9) * ld + m0 + g + 8]);
}
// B from W row-major [K][ld]: B[k][n] = W[k0 + k][n0 + n]
__device__ __forceinline__ void fragB(const uint16_t* W, int ld, int k0, int n0, int g, int t, uint32_t* b) {
  b[0] = pk(W[(k0 + 2 * t) * ld + n0 + g], W[(k0 + 2 * t + 1) * ld + n0 + g]);
  b[1] = pk(W[(k0 + 2 * t + 8) * ld + n0 + g], W[(k0 + 2 * t + 9) * ld + n0 + g]);
}
// B = W^T for W row-major [N][ld] with only kmax valid k: B[k][n] = W[n0 + n][k0 + k] (0 for k >= kmax)
__device__ __forceinline__ void fragBT(const uint16_t* W, int ld, int k0, int n0, int kmax, int g, int t, uint32_t* b) {
  const uint16_t* r = W + (n0 + g) * ld;
  const int k = k0 + 2 * t;
  b[0] = pk(k < kmax ? r[k] : 0, k + 1 < kmax ? r[k + 1] : 0);
  b[1] = pk(k + 8 < kmax ? r[k + 8] : 0, k + 9 < kmax ? r[k + 9] : 0);
}

// One dense layer of the warp's 16 samples: Out = act(In[16][K] W[K][N] + b)
template <int K, int N, bool RELU>
__device__ __forceinline__ void layer(const uint16_t* In, const uint16_t* W, const float* b, uint16_t* OutBf,
                                      float* OutF, int g, int t) {
#pragma unroll
  for (int nt = 0; nt < N / 8; nt++) {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int ks = 0; ks < K / 16; ks++) {
      uint32_t a[4], bb[2];
      fragA(In, K, ks * 16, g, t, a);
      fragB(W, N, ks * 16, nt * 8, g, t, bb);
      mma16816(acc, a, bb);
    }
    const int col = nt * 8 + 2 * t;
    const float z00 = acc[0] + b[col], z01 = acc[1] + b[col + 1], z10 = acc[2] + b[col], z11 = acc[3] + b[col + 1];
    if (RELU) {
      OutBf[g * N + col] = bf(fmaxf(z00, 0.f)); OutBf[g * N + col + 1] = bf(fmaxf(z01, 0.f));
      OutBf[(g + 8) * N + col] = bf(fmaxf(z10, 0.f)); OutBf[(g + 8) * N + col + 1] = bf(fmaxf(z11, 0.f));
    } else {
      OutF[g * N + col] = z00; OutF[g * N + col + 1] = z01;
      OutF[(g + 8) * N + col] = z10; OutF[(g + 8) * N + col + 1] = z11;
    }
  }
  __syncwarp();
}

__device__ __forceinline__ void forward(const NetSmem& net, WarpSmem& ws, int g, int t) {
  layer<16, H, true>(ws.x, net.w + OFF_W1, net.b + SB1, ws.a[0], nullptr, g, t);
  layer<H, H, true>(ws.a[0], net.w + OFF_W2, net.b + SB2, ws.a[1], nullptr, g, t);
  layer<H, H, true>(ws.a[1], net.w + OFF_W3, net.b + SB3, ws.a[2], nullptr, g, t);
  layer<H, 8, false>(ws.a[2], net.w + OFF_W4, net.b + SB4, nullptr, ws.out, g, t);
}

__device__ __forceinline__ void loadNet(NetSmem& net, const uint16_t* wbf, const float* wf) {
  const uint32_t* src = reinterpret_cast<const uint32_t*>(wbf);
  uint32_t* dst = reinterpret_cast<uint32_t*>(net.w);
  for (int k = threadIdx.x; k < NPAD / 2; k += blockDim.x) dst[k] = src[k];
  for (int k = threadIdx.x; k < NB; k += blockDim.x) {
    const int off = k < 64 ? OFF_B1 + k : (k < 128 ? OFF_B2 + k - 64 : (k < 192 ? OFF_B3 + k - 128 : OFF_B4 + k - 192));
    net.b[k] = wf[off];
  }
  __syncthreads();
}

// ------------------------------------------------------------------------------ training
// dW[in][out] += S^T dZ over the warp's 16 samples (S: [16][ldS] BF16 activations, dZ: [16][ldZ]),
// accumulated into the block's shared gradient with shared-memory atomics.
template <int M, int N>
__device__ __forceinline__ void gradW(const uint16_t* S, int ldS, const uint16_t* dZ, int ldZ, float* gW, int g, int t) {
#pragma unroll
  for (int mt = 0; mt < M / 16; mt++)
#pragma unroll
    for (int nt = 0; nt < N / 8; nt++) {
      uint32_t a[4], b[2];
      fragAT(S, ldS, mt * 16, g, t, a);
      // B[k = sample][n] = dZ[sample][nt*8 + n]
      b[0] = pk(dZ[(2 * t) * ldZ + nt * 8 + g], dZ[(2 * t + 1) * ldZ + nt * 8 + g]);
      b[1] = pk(dZ[(2 * t + 8) * ldZ + nt * 8 + g], dZ[(2 * t + 9) * ldZ + nt * 8 + g]);
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      mma16816(d, a, b);
      const int r0 = mt * 16 + g, col = nt * 8 + 2 * t;
      atomicAdd(&gW[r0 * N + col], d[0]); atomicAdd(&gW[r0 * N + col + 1], d[1]);
      atomicAdd(&gW[(r0 + 8) * N + col], d[2]); atomicAdd(&gW[(r0 + 8) * N + col + 1], d[3]);
    }
}

// dA[16][K] = dZ[16][N] W^T (W: [K][N]) then dZ_prev = dA * (A > 0), stored as BF16; bias grad of the
// previous layer from the FP32 values.
template <int K, int N>
__device__ __forceinline__ void backLayer(const uint16_t* dZ, const uint16_t* W, const uint16_t* A, uint16_t* dZprev,
                                          float* gb, int g, int t) {
#pragma unroll
  for (int nt = 0; nt < K / 8; nt++) {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    constexpr int KS = (N + 15) / 16;
#pragma unroll
    for (int ks = 0; ks < KS; ks++) {
      uint32_t a[4], b[2];
      // A[s][j] = dZ[s][ks*16 + j]  (dZ rows have stride max(N,16); padded columns are zero)
      constexpr int ldz = N < 16 ? 16 : N;
      fragA(dZ, ldz, ks * 16, g, t, a);
      // B[j][k] = W[nt*8 + k][ks*16 + j]
      fragBT(W, N, ks * 16, nt * 8, N, g, t, b);
      mma16816(acc, a, b);
    }
    const int col = nt * 8 + 2 * t;
    float z[4];
    z[0] = fbf(A[g * K + col]) > 0.f ? acc[0] : 0.f;
    z[1] = fbf(A[g * K + col + 1]) > 0.f ? acc[1] : 0.f;
    z[2] = fbf(A[(g + 8) * K + col]) > 0.f ? acc[2] : 0.f;
    z[3] = fbf(A[(g + 8) * K + col + 1]) > 0.f ? acc[3] : 0.f;
    dZprev[g * K + col] = bf(z[0]); dZprev[g * K + col + 1] = bf(z[1]);
    dZprev[(g + 8) * K + col] = bf(z[2]); dZprev[(g + 8) * K + col + 1] = bf(z[3]);
    atomicAdd(&gb[col], z[0] + z[2]);
    atomicAdd(&gb[col + 1], z[1] + z[3]);
  }
  __syncwarp();
}

// Gradient of the mean weighted squared error over the records idx[0..n) (or 0..n when idx is null),
// summed into grad (padded layout, FP32) and loss (sum over the batch / n).
__global__ void __launch_bounds__(128) k_mlp_grad(const float* rec, const int* idx, long long n, float invN,
                                                  const uint16_t* wbf, const float* wf, float* grad, float* loss) {
  extern __shared__ __align__(16) unsigned char smem[];
  NetSmem& net = *reinterpret_cast<NetSmem*>(smem);
  WarpSmem* wsAll = reinterpret_cast<WarpSmem*>(smem + sizeof(NetSmem));
  float* gsum = reinterpret_cast<float*>(smem + sizeof(NetSmem) + WARPS * sizeof(WarpSmem));
  for (int k = threadIdx.x; k < NPAD; k += blockDim.x) gsum[k] = 0.f;
  loadNet(net, wbf, wf);  // includes __syncthreads
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  WarpSmem& ws = wsAll[warp];
  float myLoss = 0.f;
  for (long long base = (long long)blockIdx.x * SAMPLES + warp * 16; base < n; base += (long long)gridDim.x * SAMPLES) {
    const long long s = base + (lane & 15);
    const bool valid = s < n;
    const float* r = valid ? rec + (long long)(idx ? idx[s] : s) * ELL_RECORD : nullptr;
    if (lane < 16)
      for (int k = 0; k < 16; k++) ws.x[lane * 16 + k] = bf((valid && k < ELL_FEATURES) ? r[k] : 0.f);
    __syncwarp();
    forward(net, ws, g, t);
    // dZ4 = 2 w (o - y) / n, padded to 16 columns of zeros
    if (lane < 16) {
      for (int k = 0; k < 16; k++) {
        float d = 0.f;
        if (valid && k < ELL_TARGETS) {
          const float e = ws.out[lane * 8 + k] - r[ELL_FEATURES + k];
          myLoss += c_lossW[k] * e * e * invN;
          d = 2.f * c_lossW[k] * e * invN;
          atomicAdd(&gsum[OFF_B4 + k], d);
        }
        ws.dz4[lane * 16 + k] = bf(d);
      }
    }
    __syncwarp();
    gradW<H, 8>(ws.a[2], H, ws.dz4, 16, gsum + OFF_W4, g, t);
    backLayer<H, 8>(ws.dz4, net.w + OFF_W4, ws.a[2], ws.dz, gsum + OFF_B3, g, t);
    gradW<H, H>(ws.a[1], H, ws.dz, H, gsum + OFF_W3, g, t);
    // dz is both input and output of the next back step: route through dz4-sized staging? use a[2] as
    // scratch for the new dZ (a3 is no longer needed)
    backLayer<H, H>(ws.dz, net.w + OFF_W3, ws.a[1], ws.a[2], gsum + OFF_B2, g, t);
    gradW<H, H>(ws.a[0], H, ws.a[2], H, gsum + OFF_W2, g, t);
    backLayer<H, H>(ws.a[2], net.w + OFF_W2, ws.a[0], ws.dz, gsum + OFF_B1, g, t);
    gradW<16, H>(ws.x, 16, ws.dz, H, gsum + OFF_W1, g, t);
    __syncwarp();
  }
  for (int o = 16; o > 0; o >>= 1) myLoss += __shfl_xor_sync(0xffffffffu, myLoss, o);
  if (lane == 0) atomicAdd(loss, myLoss);
  __syncthreads();
  for (int k = threadIdx.x; k < NPAD; k += blockDim.x)
    if (gsum[k] != 0.f) atomicAdd(&grad[k], gsum[k]);
}

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
// tcgen05.ld and writes the next layer's A operand.  Rounding points as in the mma.sync path; only the
// order of the FP32 additions inside the tensor core may differ.
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
__device__ __forceinline__ void tcHidden(unsigned char* sm, uint32_t tRow, const float* bias, int t) {
#pragma unroll
  for (int c = 0; c < H; c += 16) {
    float v[16];
    tcLoad16(tRow + c, v);
    uint32_t w[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
      w[k] = pk(bf(fmaxf(v[2 * k] + bias[c + 2 * k], 0.f)), bf(fmaxf(v[2 * k + 1] + bias[c + 2 * k + 1], 0.f)));
    *reinterpret_cast<uint4*>(sm + TC_H + kmajorOff(t, c, H)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(sm + TC_H + kmajorOff(t, c + 8, H)) = make_uint4(w[4], w[5], w[6], w[7]);
  }
}

// The network over tiles of 128 samples.  WORK: the samples are the contact work list (features from the
// particle state, as k_mlp_warm; lam0 written); otherwise feature rows X -> output rows Y.
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

constexpr size_t SMEM_INFER = sizeof(NetSmem) + WARPS * sizeof(WarpSmem);
constexpr size_t SMEM_TRAIN = SMEM_INFER + NPAD * sizeof(float);

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
  return cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TRAIN);
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
                     float* grad, float* loss) {
  if (n <= 0) return;
  long long blocks = (n + SAMPLES - 1) / SAMPLES;
  if (blocks > 152 * 2) blocks = 152 * 2;
  (k_mlp_grad<<<(unsigned)blocks, 128, SMEM_TRAIN, s>>>(rec, idx, n, 1.0f / (float)n, wbf, wf, grad, loss),
   ++::wdem::g_kernel_launches);
}

void mlp_launch_adam(cudaStream_t s, float* w, float* m, float* v, float* grad, uint16_t* wbf, float lr, float b1,
                     float b2, float c1, float c2, float eps) {
  (k_adam<<<(NPAD + 255) / 256, 256, 0, s>>>(w, m, v, grad, wbf, NPAD, lr, b1, b2, c1, c2, eps), ++::wdem::g_kernel_launches);
}

}  // namespace wdem
