// Kernels of the learned join proposal: a 32-256-256-128-1 ReLU MLP with
// BF16 weights and activations and FP32 accumulation (no counterpart in the
// reference; it orders the candidate joins of a search pass).
//
// k_gemm: C = op(A) op(B) (+ bias, ReLU) on tensor cores through inline PTX
// mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32.  A warp owns a 16x32
// tile of C (four m16n8 accumulators); fragments are gathered straight from
// global/L2 memory following the documented m16n8k16 register layout
// (groupID = lane / 4 selects rows / columns, threadID_in_group = lane % 4
// selects the k pairs).  The layers are tiny (K <= 256), so the kernel is
// latency- not bandwidth-shaped; the exact DP dominates the search.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include "poyd_internal.h"

namespace poyd {
namespace {

__device__ __forceinline__ float ld_bf(const __nv_bfloat16 *p, int64_t i, bool ok) {
  return ok ? __bfloat162float(p[i]) : 0.f;
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

// C[M,N] = op(A)[M,K] . op(B)[K,N];  op(A)[m,k] = tA ? A[k*lda+m] : A[m*lda+k],
// op(B)[k,n] = tB ? B[n*ldb+k] : B[k*ldb+n].  Epilogue: + bias[n] (fp32),
// ReLU, then fp32 and/or bf16 stores.
__global__ void __launch_bounds__(128) k_gemm(const __nv_bfloat16 *A, int lda, int tA,
                                              const __nv_bfloat16 *B, int ldb, int tB, int M,
                                              int N, int K, const float *bias, int relu,
                                              float *C32, __nv_bfloat16 *C16, int ldc,
                                              int accumulate) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int m0 = (blockIdx.y * 4 + warp) * 16;
  const int n0 = blockIdx.x * 32;
  if (m0 >= M) return;
  float acc[4][4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[j][q] = 0.f;
  auto a_at = [&](int m, int k) -> float {
    const bool ok = m < M && k < K;
    return ld_bf(A, tA ? (int64_t)k * lda + m : (int64_t)m * lda + k, ok);
  };
  auto b_at = [&](int k, int n) -> float {
    const bool ok = k < K && n < N;
    return ld_bf(B, tB ? (int64_t)n * ldb + k : (int64_t)k * ldb + n, ok);
  };
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint32_t a[4];
    a[0] = pack2(a_at(m0 + g, k0 + 2 * t), a_at(m0 + g, k0 + 2 * t + 1));
    a[1] = pack2(a_at(m0 + g + 8, k0 + 2 * t), a_at(m0 + g + 8, k0 + 2 * t + 1));
    a[2] = pack2(a_at(m0 + g, k0 + 2 * t + 8), a_at(m0 + g, k0 + 2 * t + 9));
    a[3] = pack2(a_at(m0 + g + 8, k0 + 2 * t + 8), a_at(m0 + g + 8, k0 + 2 * t + 9));
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + 8 * j + g;
      uint32_t b0 = pack2(b_at(k0 + 2 * t, n), b_at(k0 + 2 * t + 1, n));
      uint32_t b1 = pack2(b_at(k0 + 2 * t + 8, n), b_at(k0 + 2 * t + 9, n));
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
          "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
          : "+f"(acc[j][0]), "+f"(acc[j][1]), "+f"(acc[j][2]), "+f"(acc[j][3])
          : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int m = m0 + g + (q >= 2 ? 8 : 0);
      const int n = n0 + 8 * j + 2 * t + (q & 1);
      if (m >= M || n >= N) continue;
      float v = acc[j][q];
      if (accumulate && C32) v += C32[(int64_t)m * ldc + n];
      if (bias) v += bias[n];
      if (relu) v = v > 0.f ? v : 0.f;
      if (C32) C32[(int64_t)m * ldc + n] = v;
      if (C16) C16[(int64_t)m * ldc + n] = __float2bfloat16_rn(v);
    }
}

// ---------------------------------------------------------------------------
// Fused inference of the 32-256-256-128-1 MLP: a block takes 64 rows and
// runs the three hidden layers and the head with the activations in shared
// memory.  Each layer is the same arithmetic as k_gemm (mma.sync m16n8k16
// over k chunks in ascending order, + bias, ReLU, bf16 rounding) and the
// head that of k_head_forward (lane-strided sums, then the xor butterfly),
// so the predictions equal the layer-by-layer path's bit for bit.  The
// weights come in transposed (Wt[n][k]), so every B fragment is one 32-bit
// load from L2; activation rows are padded by 8 elements so that the A
// fragment loads hit 32 distinct banks.
// ---------------------------------------------------------------------------
constexpr int kFRows = 64;
constexpr int kFPadX = 32 + 8, kFPadH = 256 + 8;
constexpr int kFSmem = (kFRows * kFPadX + 2 * kFRows * kFPadH) * 2;

template <int K, int N, int LDI, int LDO>
__device__ __forceinline__ void fwd_layer(const __nv_bfloat16 *in,
                                          const __nv_bfloat16 *__restrict__ Wt,
                                          const float *__restrict__ bias, __nv_bfloat16 *out,
                                          int warp, int lane) {
  constexpr int NT = N / 64;  // n8 tiles of each of the 8 warps
  const int g = lane >> 2, t = lane & 3;
  const int nb = warp * (N / 8);
  float acc[4][NT][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
#pragma unroll 2
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint32_t a[4][4];
#pragma unroll
    for (int mt = 0; mt < 4; ++mt) {
      const __nv_bfloat16 *r0 = in + (mt * 16 + g) * LDI + k0 + 2 * t;
      const __nv_bfloat16 *r1 = r0 + 8 * LDI;
      a[mt][0] = *reinterpret_cast<const uint32_t *>(r0);
      a[mt][1] = *reinterpret_cast<const uint32_t *>(r1);
      a[mt][2] = *reinterpret_cast<const uint32_t *>(r0 + 8);
      a[mt][3] = *reinterpret_cast<const uint32_t *>(r1 + 8);
    }
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const __nv_bfloat16 *w = Wt + (int64_t)(nb + nt * 8 + g) * K + k0 + 2 * t;
      const uint32_t b0 = *reinterpret_cast<const uint32_t *>(w);
      const uint32_t b1 = *reinterpret_cast<const uint32_t *>(w + 8);
#pragma unroll
      for (int mt = 0; mt < 4; ++mt)
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
            "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
            : "+f"(acc[mt][nt][0]), "+f"(acc[mt][nt][1]), "+f"(acc[mt][nt][2]),
              "+f"(acc[mt][nt][3])
            : "r"(a[mt][0]), "r"(a[mt][1]), "r"(a[mt][2]), "r"(a[mt][3]), "r"(b0), "r"(b1));
    }
  }
#pragma unroll
  for (int mt = 0; mt < 4; ++mt)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int m = mt * 16 + g + (q >= 2 ? 8 : 0);
        const int n = nb + nt * 8 + 2 * t + (q & 1);
        float v = acc[mt][nt][q] + bias[n];
        v = v > 0.f ? v : 0.f;
        out[m * LDO + n] = __float2bfloat16_rn(v);
      }
}

__global__ void __launch_bounds__(256) k_mlp_forward(const __nv_bfloat16 *__restrict__ X, int M,
                                                     const __nv_bfloat16 *__restrict__ W1t,
                                                     const float *__restrict__ b1,
                                                     const __nv_bfloat16 *__restrict__ W2t,
                                                     const float *__restrict__ b2,
                                                     const __nv_bfloat16 *__restrict__ W3t,
                                                     const float *__restrict__ b3,
                                                     const __nv_bfloat16 *__restrict__ w4,
                                                     const float *__restrict__ b4, float *y) {
  extern __shared__ __align__(16) unsigned char mlp_dsm[];
  __nv_bfloat16 *xs = reinterpret_cast<__nv_bfloat16 *>(mlp_dsm);
  __nv_bfloat16 *h1 = xs + kFRows * kFPadX;
  __nv_bfloat16 *h2 = h1 + kFRows * kFPadH;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t m0 = (int64_t)blockIdx.x * kFRows;
  // the block's 64 input rows (32 bf16 each), zero past M
  for (int e = threadIdx.x; e < kFRows * 4; e += blockDim.x) {
    const int r = e >> 2, c = (e & 3) * 8;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (m0 + r < M) v = *reinterpret_cast<const uint4 *>(X + (m0 + r) * 32 + c);
    *reinterpret_cast<uint4 *>(xs + r * kFPadX + c) = v;
  }
  __syncthreads();
  fwd_layer<32, 256, kFPadX, kFPadH>(xs, W1t, b1, h1, warp, lane);
  __syncthreads();
  fwd_layer<256, 256, kFPadH, kFPadH>(h1, W2t, b2, h2, warp, lane);
  __syncthreads();
  fwd_layer<256, 128, kFPadH, kFPadH>(h2, W3t, b3, h1, warp, lane);
  __syncthreads();
  // the head, k_head_forward's order: 8 rows per warp
  for (int rr = 0; rr < kFRows / 8; ++rr) {
    const int r = warp * (kFRows / 8) + rr;
    float sacc = 0.f;
    for (int k = lane; k < 128; k += 32)
      sacc += __bfloat162float(h1[r * kFPadH + k]) * __bfloat162float(w4[k]);
    for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
    if (lane == 0 && m0 + r < M) y[m0 + r] = sacc + b4[0];
  }
}

// dZ = dH * (H > 0), bf16 in / out
__global__ void k_relu_grad(const __nv_bfloat16 *dH, const __nv_bfloat16 *H, __nv_bfloat16 *dZ,
                            int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dZ[i] = __bfloat162float(H[i]) > 0.f ? dH[i] : __float2bfloat16_rn(0.f);
}

// out[n] = sum_m X[m, n] (fp32 accumulation of bf16 rows)
__global__ void k_colsum(const __nv_bfloat16 *X, int M, int N, float *out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += __bfloat162float(X[(int64_t)m * N + n]);
  out[n] = s;
}

// y[m] = H[m,:] . w + b (the 128 -> 1 output layer), fp32 accumulate
__global__ void k_head_forward(const __nv_bfloat16 *H, const __nv_bfloat16 *w, const float *b,
                               int M, int K, float *y) {
  const int lane = threadIdx.x & 31;
  const int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (m >= M) return;
  float s = 0.f;
  for (int k = lane; k < K; k += 32)
    s += __bfloat162float(H[(int64_t)m * K + k]) * __bfloat162float(w[k]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[m] = s + b[0];
}

// MSE head: dy = 2 (y - target) / M; dH = dy w (masked by H > 0);
// dw = H^T dy; db = sum dy; loss = mean (y - target)^2 (atomic)
__global__ void k_head_backward(const __nv_bfloat16 *H, const __nv_bfloat16 *w, const float *y,
                                const float *target, int M, int K, __nv_bfloat16 *dZ, float *dw,
                                float *db, float *loss) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < K) {
    float s = 0.f;
    for (int m = 0; m < M; ++m) {
      const float dy = 2.f * (y[m] - target[m]) / (float)M;
      s += __bfloat162float(H[(int64_t)m * K + k]) * dy;
    }
    dw[k] = s;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    float s = 0.f, l = 0.f;
    for (int m = 0; m < M; ++m) {
      const float e = y[m] - target[m];
      s += 2.f * e / (float)M;
      l += e * e;
    }
    db[0] = s;
    loss[0] = l / (float)M;
  }
  const int64_t total = (int64_t)M * K;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(i / K), kk = (int)(i % K);
    const float dy = 2.f * (y[m] - target[m]) / (float)M;
    const float h = __bfloat162float(H[i]);
    dZ[i] = __float2bfloat16_rn(h > 0.f ? dy * __bfloat162float(w[kk]) : 0.f);
  }
}

// Adam on fp32 master weights, refreshing the bf16 copy.
__global__ void k_adam(float *w, __nv_bfloat16 *w16, const float *g, float *mo, float *ve,
                       int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float m = b1 * mo[i] + (1.f - b1) * gi;
  const float v = b2 * ve[i] + (1.f - b2) * gi * gi;
  mo[i] = m;
  ve[i] = v;
  const float upd = lr * (m / c1) / (sqrtf(v / c2) + eps);
  w[i] -= upd;
  if (w16) w16[i] = __float2bfloat16_rn(w[i]);
}

__global__ void k_to_bf16(const float *x, __nv_bfloat16 *y, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace
}  // namespace poyd

using namespace poyd;

#define MLP_LAUNCH_CHECK()                                   \
  do {                                                       \
    cudaError_t e_ = cudaGetLastError();                     \
    if (e_ != cudaSuccess) return cuda_fail(e_, "mlp kernel"); \
  } while (0)

extern "C" int poyd_gemm_bf16(const void *A, int32_t lda, int32_t tA, const void *B, int32_t ldb,
                              int32_t tB, int32_t M, int32_t N, int32_t K, const float *bias,
                              int32_t relu, float *C32, void *C16, int32_t ldc,
                              int32_t accumulate, void *stream) {
  if (M < 0 || N < 0 || K < 0 || !A || !B || (!C32 && !C16))
    return fail(POYD_EINVAL, "poyd_gemm_bf16: bad arguments");
  if (M == 0 || N == 0) return POYD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid(nblk(N, 32), nblk(M, 64));
  ProfScope ps("mlp_gemm", st);
  k_gemm<<<grid, 128, 0, st>>>((const __nv_bfloat16 *)A, lda, tA, (const __nv_bfloat16 *)B, ldb,
                               tB, M, N, K, bias, relu, C32, (__nv_bfloat16 *)C16, ldc,
                               accumulate);
  MLP_LAUNCH_CHECK();
  return POYD_OK;
}

extern "C" int poyd_relu_grad_bf16(const void *dH, const void *H, void *dZ, int64_t n,
                                   void *stream) {
  if (n <= 0) return POYD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps("mlp_relu_grad", st);
  k_relu_grad<<<nblk(n, 256), 256, 0, st>>>((const __nv_bfloat16 *)dH, (const __nv_bfloat16 *)H,
                                            (__nv_bfloat16 *)dZ, n);
  MLP_LAUNCH_CHECK();
  return POYD_OK;
}

extern "C" int poyd_colsum_bf16(const void *X, int32_t M, int32_t N, float *out, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps("mlp_colsum", st);
  k_colsum<<<nblk(N, 128), 128, 0, st>>>((const __nv_bfloat16 *)X, M, N, out);
  MLP_LAUNCH_CHECK();
  return POYD_OK;
}

extern "C" int poyd_mlp_head_forward(const void *H, const void *w, const float *b, int32_t M,
                                     int32_t K, float *y, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps("mlp_head_fwd", st);
  k_head_forward<<<nblk((int64_t)M * 32, 256), 256, 0, st>>>(
      (const __nv_bfloat16 *)H, (const __nv_bfloat16 *)w, b, M, K, y);
  MLP_LAUNCH_CHECK();
  return POYD_OK;
}

extern "C" int poyd_mlp_head_backward(const void *H, const void *w, const float *y,
                                      const float *target, int32_t M, int32_t K, void *dZ,
                                      float *dw, float *db, float *loss, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps("mlp_head_bwd", st);
  k_head_backward<<<nblk((int64_t)M * K, 256) < 1024 ? nblk((int64_t)M * K, 256) : 1024, 256, 0,
                    st>>>((const __nv_bfloat16 *)H, (const __nv_bfloat16 *)w, y, target, M, K,
                          (__nv_bfloat16 *)dZ, dw, db, loss);
  MLP_LAUNCH_CHECK();
  return POYD_OK;
}

extern "C" int poyd_adam_step(float *w, void *w16, const float *g, float *m, float *v, int64_t n,
                              float lr, float b1, float b2, float eps, int32_t step,
                              void *stream) {
  if (n <= 0) return POYD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  ProfScope ps("mlp_adam", st);
  k_adam<<<nblk(n, 256), 256, 0, st>>>(w, (__nv_bfloat16 *)w16, g, m, v, n, lr, b1, b2, eps, c1,
                                       c2);
  MLP_LAUNCH_CHECK();
  return POYD_OK;
}

extern "C" int poyd_to_bf16(const float *x, void *y, int64_t n, void *stream) {
  if (n <= 0) return POYD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps("mlp_to_bf16", st);
  k_to_bf16<<<nblk(n, 256), 256, 0, st>>>(x, (__nv_bfloat16 *)y, n);
  MLP_LAUNCH_CHECK();
  return POYD_OK;
}

extern "C" int poyd_mlp_forward(const void *X, int32_t M, const void *W1t, const float *b1,
                                const void *W2t, const float *b2, const void *W3t,
                                const float *b3, const void *w4, const float *b4, float *y,
                                void *stream) {
  if (M < 0) return fail(POYD_EINVAL, "negative size");
  if (M == 0) return POYD_OK;
  if (!X || !W1t || !b1 || !W2t || !b2 || !W3t || !b3 || !w4 || !b4 || !y)
    return fail(POYD_EINVAL, "poyd_mlp_forward: null argument");
  if (((uintptr_t)X & 15) || ((uintptr_t)W1t & 3) || ((uintptr_t)W2t & 3) || ((uintptr_t)W3t & 3))
    return fail(POYD_EINVAL, "poyd_mlp_forward: X must be 16-byte aligned, weights 4-byte aligned");
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr[dev & 63]) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kFSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_mlp_forward)");
    attr[dev & 63] = true;
  }
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps("mlp_forward", st);
  k_mlp_forward<<<nblk(M, kFRows), 256, kFSmem, st>>>(
      (const __nv_bfloat16 *)X, M, (const __nv_bfloat16 *)W1t, b1, (const __nv_bfloat16 *)W2t, b2,
      (const __nv_bfloat16 *)W3t, b3, (const __nv_bfloat16 *)w4, b4, y);
  MLP_LAUNCH_CHECK();
  return POYD_OK;
}
