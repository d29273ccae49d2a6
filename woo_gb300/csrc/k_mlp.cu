// k_mlp.cu -- the learned warm start of the ellipsoid contact solve.
//
// A 13 -> 64 -> 64 -> 64 -> 4 multilayer perceptron (ReLU hidden layers) maps the state of an
// ellipsoid pair (centre offset in A's frame, relative orientation, both semi-axis triples; lengths
// divided by max(a) + max(b)) to the maximiser lambda of the Perram-Wertheim contact function and the
// contact point in A's frame.  Its lambda starts the Newton solve (WDEM_WARM_MLP); the solve falls
// back to the cold start when it has not converged after fallbackIters iterations.
//
// Arithmetic: BF16 operands, FP32 accumulation, on the tensor cores through mma.sync.m16n8k16 (one
// warp = 16 samples; activations stay in shared memory between layers).  Rounding points, which the
// CPU reference of the network follows: inputs, weights and post-ReLU activations are rounded to BF16;
// biases, pre-activations and outputs stay FP32.  Training runs the backward pass with the same
// fragments (BF16 operands: activations, dZ, weights; FP32 accumulation), sums the gradient of a
// mini-batch per block in shared memory, and applies Adam (Kingma & Ba 2015) to FP32 master weights.
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

// ------------------------------------------------------------------------------ inference
// lam0 of every ellipsoid pair (sphere + ellipsoid included; walls excluded) that the contact kernel
// may solve this step; other entries are NaN (cold start).  onlyFresh: pairs that carry the previous
// step's maximiser (c.lam in (0, 1)) get NaN as well (the solve starts from that), and a warp whose 16
// pairs all carry one skips the network.
__global__ void __launch_bounds__(128) k_mlp_warm(Particles p, Contacts c, const unsigned* work, const unsigned* count,
                                                  long long ncon, const uint16_t* wbf, const float* wf, int onlyFresh) {
  extern __shared__ __align__(16) unsigned char smem[];
  NetSmem& net = *reinterpret_cast<NetSmem*>(smem);
  WarpSmem* wsAll = reinterpret_cast<WarpSmem*>(smem + sizeof(NetSmem));
  loadNet(net, wbf, wf);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  WarpSmem& ws = wsAll[warp];
  const long long nw = workLen(count);
  for (long long base = (long long)blockIdx.x * SAMPLES + warp * 16; base < nw; base += (long long)gridDim.x * SAMPLES) {
    const long long kw = base + (lane & 15);
    const long long i = kw < nw ? (long long)workItem(work, count, ncon, (unsigned)kw) : -1;
    bool use = false;
    if (lane < 16) {
      float f[ELL_FEATURES];
      for (int k = 0; k < ELL_FEATURES; k++) f[k] = 0.f;
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
      for (int k = 0; k < 16; k++) ws.x[(lane & 15) * 16 + k] = bf(k < ELL_FEATURES ? f[k] : 0.f);
    }
    __syncwarp();
    if (__ballot_sync(0xffffffffu, use) == 0) {
      // no pair of this warp needs the network
      if (lane < 16 && i >= 0) c.lam0[i] = __int_as_float(0x7fffffff);
      __syncwarp();
      continue;
    }
    forward(net, ws, g, t);
    if (lane < 16 && i >= 0) {
      float l = ws.out[(lane & 15) * 8 + 0];
      l = fminf(fmaxf(l, 1e-3f), 1.f - 1e-3f);
      c.lam0[i] = use ? l : __int_as_float(0x7fffffff);
    }
    __syncwarp();
  }
}

// Arbitrary feature rows (n x 13) -> outputs (n x 4), for tests and tools.
__global__ void __launch_bounds__(128) k_mlp_predict(const float* X, long long n, float* Y, const uint16_t* wbf,
                                                     const float* wf) {
  extern __shared__ __align__(16) unsigned char smem[];
  NetSmem& net = *reinterpret_cast<NetSmem*>(smem);
  WarpSmem* wsAll = reinterpret_cast<WarpSmem*>(smem + sizeof(NetSmem));
  loadNet(net, wbf, wf);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  WarpSmem& ws = wsAll[warp];
  for (long long base = (long long)blockIdx.x * SAMPLES + warp * 16; base < n; base += (long long)gridDim.x * SAMPLES) {
    const long long i = base + (lane & 15);
    if (lane < 16)
      for (int k = 0; k < 16; k++) ws.x[lane * 16 + k] = bf((i < n && k < ELL_FEATURES) ? X[i * ELL_FEATURES + k] : 0.f);
    __syncwarp();
    forward(net, ws, g, t);
    if (lane < 16 && i < n)
      for (int k = 0; k < ELL_TARGETS; k++) Y[i * ELL_TARGETS + k] = ws.out[lane * 8 + k];
    __syncwarp();
  }
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
  if ((e = cudaFuncSetAttribute(k_mlp_warm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_INFER))) return e;
  if ((e = cudaFuncSetAttribute(k_mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_INFER))) return e;
  return cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TRAIN);
}

void mlp_to_bf16(cudaStream_t s, const float* w, uint16_t* wbf) {
  (k_to_bf16<<<(NPAD + 255) / 256, 256, 0, s>>>(w, wbf, NPAD), ++::wdem::g_kernel_launches);
}

void mlp_launch_warm(cudaStream_t s, Particles p, Contacts c, long long nc, const unsigned* work, const unsigned* count,
                     const uint16_t* wbf, const float* wf, bool onlyFresh) {
  if (nc <= 0) return;
  long long blocks = (nc + SAMPLES - 1) / SAMPLES;
  if (blocks > 152 * 2) blocks = 152 * 2;  // persistent blocks: the weights are loaded once per block
  (k_mlp_warm<<<(unsigned)blocks, 128, SMEM_INFER, s>>>(p, c, work, count, nc, wbf, wf, onlyFresh ? 1 : 0),
   ++::wdem::g_kernel_launches);
}

void mlp_launch_predict(cudaStream_t s, const float* X, long long n, float* Y, const uint16_t* wbf, const float* wf) {
  if (n <= 0) return;
  long long blocks = (n + SAMPLES - 1) / SAMPLES;
  if (blocks > 152 * 8) blocks = 152 * 8;
  (k_mlp_predict<<<(unsigned)blocks, 128, SMEM_INFER, s>>>(X, n, Y, wbf, wf), ++::wdem::g_kernel_launches);
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
