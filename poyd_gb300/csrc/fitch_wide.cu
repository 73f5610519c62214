// Fitch on 16- and 32-bit state sets: NonaddCS16 / NonaddCS32, which the
// reference builds from nonaddCSc.c with CHARSIZE 16 / 32 under the
// nonadd16_ / nonadd32_ names (myocamlbuild.ml.in:262-289), for characters
// of 9-16 and 17-32 states.
//
// Same layout and launch shape as the 8-bit kernels: one warp per
// candidate, each lane moving one 16-byte vector per load, which now holds
// 8 (16-bit) or 4 (32-bit) characters.  Only the per-character zero test
// and the containment compare change width.  The rules are those of
// nonadd_median (nonaddCSc.c:422-462), nonadd_median_3 (472-544) and
// char_nonadd_CAML_distance (1076-1105).
#include <cuda_runtime.h>
#include <cstdint>
#include "poyd_internal.h"

namespace poyd {
namespace {

constexpr unsigned kFullW = 0xffffffffu;

// all-ones in every W-bit character of x that is zero
template <int W>
__device__ __forceinline__ uint32_t zero_lanes(uint32_t x);
template <>
__device__ __forceinline__ uint32_t zero_lanes<16>(uint32_t x) { return __vcmpeq2(x, 0u); }
template <>
__device__ __forceinline__ uint32_t zero_lanes<32>(uint32_t x) { return x == 0u ? kFullW : 0u; }

// all-ones in every W-bit character where x equals y
template <int W>
__device__ __forceinline__ uint32_t eq_lanes(uint32_t x, uint32_t y);
template <>
__device__ __forceinline__ uint32_t eq_lanes<16>(uint32_t x, uint32_t y) { return __vcmpeq2(x, y); }
template <>
__device__ __forceinline__ uint32_t eq_lanes<32>(uint32_t x, uint32_t y) {
  return x == y ? kFullW : 0u;
}

// word `word` of a 16-byte vector with its bytes at index >= valid_bytes
// set (valid_bytes clamped to 0..16 by the caller)
__device__ __forceinline__ uint32_t tail_bytes(int valid_bytes, int word) {
  const int v = valid_bytes - 4 * word;
  if (v >= 4) return 0u;
  if (v <= 0) return kFullW;
  return kFullW << (8 * v);
}

// bytes of vector v that hold characters below len
template <int W>
__device__ __forceinline__ int valid_bytes(int len, int v) {
  constexpr int kPer = 128 / W;
  const int left = len - v * kPer;
  return left >= kPer ? 16 : left * (W / 8);
}

template <int W>
__global__ void k_fitch_wide_distance(const uint8_t *nodes, int64_t stride, int len, int n,
                                      const int32_t *ai, const int32_t *bi, int64_t *dist) {
  constexpr int kPer = 128 / W;
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= n) return;
  const uint4 *a = (const uint4 *)(nodes + (int64_t)ai[c] * stride);
  const uint4 *b = (const uint4 *)(nodes + (int64_t)bi[c] * stride);
  const int nv = (len + kPer - 1) / kPer;
  unsigned cnt = 0;
  for (int v = lane; v < nv; v += 32) {
    const uint4 x = a[v], y = b[v];
    const int vb = valid_bytes<W>(len, v);
    cnt += __popc(zero_lanes<W>(x.x & y.x) & ~tail_bytes(vb, 0)) / W;
    cnt += __popc(zero_lanes<W>(x.y & y.y) & ~tail_bytes(vb, 1)) / W;
    cnt += __popc(zero_lanes<W>(x.z & y.z) & ~tail_bytes(vb, 2)) / W;
    cnt += __popc(zero_lanes<W>(x.w & y.w) & ~tail_bytes(vb, 3)) / W;
  }
  cnt = __reduce_add_sync(kFullW, cnt);
  if (lane == 0) dist[c] = cnt;
}

template <int W>
__device__ __forceinline__ uint32_t median_word(uint32_t x, uint32_t y, uint32_t tail,
                                                unsigned &cnt) {
  const uint32_t i = x & y;
  const uint32_t z = zero_lanes<W>(i);
  cnt += __popc(z & ~tail) / W;
  return i | (z & (x | y));
}

template <int W>
__global__ void k_fitch_wide_median(const uint8_t *nodes, int64_t stride, int len, int n,
                                    const int32_t *ai, const int32_t *bi, uint8_t *out,
                                    int64_t *added) {
  constexpr int kPer = 128 / W;
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= n) return;
  const uint4 *a = (const uint4 *)(nodes + (int64_t)ai[c] * stride);
  const uint4 *b = (const uint4 *)(nodes + (int64_t)bi[c] * stride);
  uint4 *r = (uint4 *)(out + (int64_t)c * stride);
  const int nv = (len + kPer - 1) / kPer;
  unsigned cnt = 0;
  for (int v = lane; v < nv; v += 32) {
    const uint4 x = a[v], y = b[v];
    const int vb = valid_bytes<W>(len, v);
    uint4 o;
    o.x = median_word<W>(x.x, y.x, tail_bytes(vb, 0), cnt);
    o.y = median_word<W>(x.y, y.y, tail_bytes(vb, 1), cnt);
    o.z = median_word<W>(x.z, y.z, tail_bytes(vb, 2), cnt);
    o.w = median_word<W>(x.w, y.w, tail_bytes(vb, 3), cnt);
    r[v] = o;
  }
  cnt = __reduce_add_sync(kFullW, cnt);
  if (lane == 0 && added) added[c] = cnt;
}

template <int W>
__device__ __forceinline__ uint32_t fitch3_word(uint32_t A, uint32_t N, uint32_t D1, uint32_t D2) {
  // nonadd_median_3 (nonaddCSc.c:499-527), 32 / W characters at a time
  uint32_t inter = N | (A & (D1 | D2));
  uint32_t temp = inter;
  const uint32_t was_union = zero_lanes<W>(D1 & D2);
  inter = (inter | A) & was_union;
  temp |= inter;
  const uint32_t contained = eq_lanes<W>(A & N, A);
  const uint32_t f = contained & A;
  temp &= ~contained;
  return f | temp;
}

template <int W>
__global__ void k_fitch_wide_median3(const uint8_t *nodes, int64_t stride, int len, int n,
                                     const int32_t *anc, const int32_t *pre, const int32_t *d1,
                                     const int32_t *d2, uint8_t *out) {
  constexpr int kPer = 128 / W;
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= n) return;
  const uint4 *A = (const uint4 *)(nodes + (int64_t)anc[c] * stride);
  const uint4 *N = (const uint4 *)(nodes + (int64_t)pre[c] * stride);
  const uint4 *X = (const uint4 *)(nodes + (int64_t)d1[c] * stride);
  const uint4 *Y = (const uint4 *)(nodes + (int64_t)d2[c] * stride);
  uint4 *r = (uint4 *)(out + (int64_t)c * stride);
  const int nv = (len + kPer - 1) / kPer;
  for (int v = lane; v < nv; v += 32) {
    const uint4 a = A[v], p = N[v], x = X[v], y = Y[v];
    uint4 o;
    o.x = fitch3_word<W>(a.x, p.x, x.x, y.x);
    o.y = fitch3_word<W>(a.y, p.y, x.y, y.y);
    o.z = fitch3_word<W>(a.z, p.z, x.z, y.z);
    o.w = fitch3_word<W>(a.w, p.w, x.w, y.w);
    r[v] = o;
  }
}

// Rows of len W-bit characters at a 16-byte aligned base, stride a
// multiple of 16 bytes and at least the row's bytes rounded up to 16.
int check_wide_rows(const void *nodes, int64_t stride, int len, int n, int width) {
  if (n < 0 || len < 0) return fail(POYD_EINVAL, "negative size");
  if (n > 0 && !nodes) return fail(POYD_EINVAL, "null node array");
  const int64_t row = ((int64_t)len * (width / 8) + 15) / 16 * 16;
  if (stride % 16 || stride < row || ((uintptr_t)nodes & 15))
    return fail(POYD_EINVAL,
                "node rows must be 16-byte aligned with stride >= len x %d bytes rounded to 16",
                width / 8);
  return POYD_OK;
}

unsigned warp_blocks(int32_t n) { return (unsigned)(((int64_t)n * 32 + 255) / 256); }

#define FW_CK(call)                                       \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

template <int W>
int wide_distance(const void *nodes, int64_t stride, int32_t len, int32_t n, const int32_t *ai,
                  const int32_t *bi, int64_t *dist, void *stream) {
  int rc = check_wide_rows(nodes, stride, len, n, W);
  if (rc) return rc;
  if (n == 0) return POYD_OK;
  if (!ai || !bi || !dist) return fail(POYD_EINVAL, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps(W == 16 ? "fitch16_distance" : "fitch32_distance", st);
  k_fitch_wide_distance<W><<<warp_blocks(n), 256, 0, st>>>((const uint8_t *)nodes, stride, len, n,
                                                            ai, bi, dist);
  FW_CK(cudaGetLastError());
  return POYD_OK;
}

template <int W>
int wide_median(const void *nodes, int64_t stride, int32_t len, int32_t n, const int32_t *ai,
                const int32_t *bi, void *out, int64_t *added, void *stream) {
  int rc = check_wide_rows(nodes, stride, len, n, W);
  if (rc) return rc;
  if (n == 0) return POYD_OK;
  if (!ai || !bi) return fail(POYD_EINVAL, "null argument");
  if (!out || ((uintptr_t)out & 15)) return fail(POYD_EINVAL, "output rows must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps(W == 16 ? "fitch16_median" : "fitch32_median", st);
  k_fitch_wide_median<W><<<warp_blocks(n), 256, 0, st>>>((const uint8_t *)nodes, stride, len, n,
                                                          ai, bi, (uint8_t *)out, added);
  FW_CK(cudaGetLastError());
  return POYD_OK;
}

template <int W>
int wide_median3(const void *nodes, int64_t stride, int32_t len, int32_t n, const int32_t *anc,
                 const int32_t *pre, const int32_t *d1, const int32_t *d2, void *out,
                 void *stream) {
  int rc = check_wide_rows(nodes, stride, len, n, W);
  if (rc) return rc;
  if (n == 0) return POYD_OK;
  if (!anc || !pre || !d1 || !d2) return fail(POYD_EINVAL, "null argument");
  if (!out || ((uintptr_t)out & 15)) return fail(POYD_EINVAL, "output rows must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps(W == 16 ? "fitch16_median3" : "fitch32_median3", st);
  k_fitch_wide_median3<W><<<warp_blocks(n), 256, 0, st>>>((const uint8_t *)nodes, stride, len, n,
                                                           anc, pre, d1, d2, (uint8_t *)out);
  FW_CK(cudaGetLastError());
  return POYD_OK;
}

}  // namespace
}  // namespace poyd

using namespace poyd;

#define POYD_FITCH_WIDE(W)                                                                      \
  extern "C" int poyd_nonadd##W##_distance_batch(const void *nodes, int64_t stride, int32_t len, \
                                                 int32_t n, const int32_t *a_idx,               \
                                                 const int32_t *b_idx, int64_t *dist,            \
                                                 void *stream) {                                \
    return wide_distance<W>(nodes, stride, len, n, a_idx, b_idx, dist, stream);                \
  }                                                                                             \
  extern "C" int poyd_nonadd##W##_median_batch(const void *nodes, int64_t stride, int32_t len,   \
                                               int32_t n, const int32_t *a_idx,                 \
                                               const int32_t *b_idx, void *out,                 \
                                               int64_t *added_cost, void *stream) {             \
    return wide_median<W>(nodes, stride, len, n, a_idx, b_idx, out, added_cost, stream);       \
  }                                                                                             \
  extern "C" int poyd_nonadd##W##_median_3_batch(                                               \
      const void *nodes, int64_t stride, int32_t len, int32_t n, const int32_t *anc,            \
      const int32_t *prelim, const int32_t *d1, const int32_t *d2, void *out, void *stream) {   \
    return wide_median3<W>(nodes, stride, len, n, anc, prelim, d1, d2, out, stream);           \
  }
POYD_FITCH_WIDE(16)
POYD_FITCH_WIDE(32)
