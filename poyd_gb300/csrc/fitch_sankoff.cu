// Fitch (non-additive, 8-bit state sets) and Sankoff character kernels.
//
// Fitch restates nonadd_median (nonaddCSc.c:422-462), nonadd_median_3
// (nonaddCSc.c:472-544) and char_nonadd_CAML_distance
// (nonaddCSc.c:1076-1105) for NonaddCS8 (2-8 states).  One warp handles one
// candidate; each lane moves 16 bytes (16 characters) per load, so a node
// row of `len` characters is read with coalesced 128-bit loads and the
// empty-intersection count is a per-lane byte compare + popcount + warp
// reduction.  Bytes past `len` in the last vector never count, like the
// reference's VCOUNT bound (nonaddCSc.c:56-62).
//
// Sankoff restates SankCS.elt_median / distance (sankCS.ml:302-377) with
// int32 costs and the saturating infinity of sankCS.ml:34-67 mapped to
// POYD_SANK_INF: one thread per (candidate, character), k <= 8 states,
// tcm in shared memory.
#include <cuda_runtime.h>
#include <cstdint>
#include "poyd_internal.h"

namespace poyd {
namespace {

constexpr unsigned kFullF = 0xffffffffu;

// 0xff in every byte of x that is zero
__device__ __forceinline__ uint32_t zbytes(uint32_t x) { return __vcmpeq4(x, 0u); }

// bytes at index >= valid (0..16) of a 16-byte vector forced to 0xff
__device__ __forceinline__ uint32_t tailmask(int valid, int word) {
  const int v = valid - 4 * word;
  if (v >= 4) return 0u;
  if (v <= 0) return 0xffffffffu;
  return 0xffffffffu << (8 * v);
}

__global__ void k_fitch_distance(const uint8_t *nodes, int64_t stride, int len, int n,
                                 const int32_t *ai, const int32_t *bi, int64_t *dist) {
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= n) return;
  const uint4 *a = (const uint4 *)(nodes + (int64_t)ai[c] * stride);
  const uint4 *b = (const uint4 *)(nodes + (int64_t)bi[c] * stride);
  const int nv = (len + 15) >> 4;
  unsigned cnt = 0;
  for (int v = lane; v < nv; v += 32) {
    const uint4 x = a[v], y = b[v];
    const int valid = len - v * 16;
    uint32_t z0 = zbytes(x.x & y.x) & ~tailmask(valid, 0);
    uint32_t z1 = zbytes(x.y & y.y) & ~tailmask(valid, 1);
    uint32_t z2 = zbytes(x.z & y.z) & ~tailmask(valid, 2);
    uint32_t z3 = zbytes(x.w & y.w) & ~tailmask(valid, 3);
    cnt += (__popc(z0) + __popc(z1) + __popc(z2) + __popc(z3)) >> 3;
  }
  cnt = __reduce_add_sync(kFullF, cnt);
  if (lane == 0) dist[c] = cnt;
}

__global__ void k_fitch_median(const uint8_t *nodes, int64_t stride, int len, int n,
                               const int32_t *ai, const int32_t *bi, uint8_t *out,
                               int64_t *added) {
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= n) return;
  const uint4 *a = (const uint4 *)(nodes + (int64_t)ai[c] * stride);
  const uint4 *b = (const uint4 *)(nodes + (int64_t)bi[c] * stride);
  uint4 *r = (uint4 *)(out + (int64_t)c * stride);
  const int nv = (len + 15) >> 4;
  unsigned cnt = 0;
  for (int v = lane; v < nv; v += 32) {
    const uint4 x = a[v], y = b[v];
    const int valid = len - v * 16;
    uint4 o;
    uint32_t i, z;
    i = x.x & y.x; z = zbytes(i); o.x = i | (z & (x.x | y.x)); cnt += __popc(z & ~tailmask(valid, 0)) >> 3;
    i = x.y & y.y; z = zbytes(i); o.y = i | (z & (x.y | y.y)); cnt += __popc(z & ~tailmask(valid, 1)) >> 3;
    i = x.z & y.z; z = zbytes(i); o.z = i | (z & (x.z | y.z)); cnt += __popc(z & ~tailmask(valid, 2)) >> 3;
    i = x.w & y.w; z = zbytes(i); o.w = i | (z & (x.w | y.w)); cnt += __popc(z & ~tailmask(valid, 3)) >> 3;
    r[v] = o;
  }
  cnt = __reduce_add_sync(kFullF, cnt);
  if (lane == 0 && added) added[c] = cnt;
}

__device__ __forceinline__ uint32_t fitch3(uint32_t A, uint32_t N, uint32_t D1, uint32_t D2) {
  // nonadd_median_3 (nonaddCSc.c:499-527), four characters at a time
  uint32_t inter = N | (A & (D1 | D2));
  uint32_t temp = inter;
  const uint32_t was_union = zbytes(D1 & D2);
  inter = (inter | A) & was_union;
  temp |= inter;
  const uint32_t contained = __vcmpeq4(A & N, A);
  const uint32_t f = contained & A;
  temp &= ~contained;
  return f | temp;
}

__global__ void k_fitch_median3(const uint8_t *nodes, int64_t stride, int len, int n,
                                const int32_t *anc, const int32_t *pre, const int32_t *d1,
                                const int32_t *d2, uint8_t *out) {
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= n) return;
  const uint4 *A = (const uint4 *)(nodes + (int64_t)anc[c] * stride);
  const uint4 *N = (const uint4 *)(nodes + (int64_t)pre[c] * stride);
  const uint4 *X = (const uint4 *)(nodes + (int64_t)d1[c] * stride);
  const uint4 *Y = (const uint4 *)(nodes + (int64_t)d2[c] * stride);
  uint4 *r = (uint4 *)(out + (int64_t)c * stride);
  const int nv = (len + 15) >> 4;
  for (int v = lane; v < nv; v += 32) {
    const uint4 a = A[v], p = N[v], x = X[v], y = Y[v];
    uint4 o;
    o.x = fitch3(a.x, p.x, x.x, y.x);
    o.y = fitch3(a.y, p.y, x.y, y.y);
    o.z = fitch3(a.z, p.z, x.z, y.z);
    o.w = fitch3(a.w, p.w, x.w, y.w);
    r[v] = o;
  }
}

// ---- Sankoff ---------------------------------------------------------------
constexpr int kSInf = POYD_SANK_INF;

__device__ __forceinline__ int sadd(int a, int b) {
  return (a >= kSInf || b >= kSInf) ? kSInf : a + b;
}

// elt_median for one character; returns min c and (optionally) writes rows.
template <int K>
__device__ __forceinline__ void sank_char(const int *tcm, const int *as, const int *bs, int *c,
                                          int *e, int *beta, int &minc, int &mina, int &minb) {
  minc = kSInf; mina = kSInf; minb = kSInf;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    mina = (as[i] < mina) ? as[i] : mina;
    minb = (bs[i] < minb) ? bs[i] : minb;
  }
#pragma unroll
  for (int i = 0; i < K; ++i) {
    // min over (j,k) of tcm[i][j] + tcm[i][k] + a.s[j] + b.s[k] separates
    // into two independent minima (all terms non-negative integers)
    int ma = kSInf, mb = kSInf;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const int x = sadd(tcm[i * K + j], as[j]);
      const int y = sadd(tcm[i * K + j], bs[j]);
      ma = x < ma ? x : ma;
      mb = y < mb ? y : mb;
    }
    c[i] = sadd(ma, mb);
    minc = c[i] < minc ? c[i] : minc;
  }
#pragma unroll
  for (int i = 0; i < K; ++i) e[i] = (c[i] >= kSInf) ? kSInf : (minc >= kSInf ? 0 : c[i] - minc);
#pragma unroll
  for (int s = 0; s < K; ++s) {
    int best = kSInf;
#pragma unroll
    for (int x = 0; x < K; ++x) {
      const int v = sadd(tcm[s * K + x], e[x]);
      best = v < best ? v : best;
    }
    beta[s] = best;
  }
}

template <int K>
__global__ void k_sank_median(const int32_t *nodes, int nchar, const int32_t *tcm_g, int n,
                              const int32_t *ai, const int32_t *bi, int32_t *out_s,
                              int32_t *out_e, int32_t *out_b) {
  __shared__ int tcm[K * K];
  for (int t = threadIdx.x; t < K * K; t += blockDim.x) tcm[t] = tcm_g[t];
  __syncthreads();
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (int64_t)n * nchar) return;
  const int c = (int)(g / nchar), ch = (int)(g % nchar);
  const int32_t *a = nodes + ((int64_t)ai[c] * nchar + ch) * K;
  const int32_t *b = nodes + ((int64_t)bi[c] * nchar + ch) * K;
  int as[K], bs[K], cc[K], e[K], beta[K], minc, mina, minb;
#pragma unroll
  for (int i = 0; i < K; ++i) { as[i] = a[i]; bs[i] = b[i]; }
  sank_char<K>(tcm, as, bs, cc, e, beta, minc, mina, minb);
  const int64_t o = ((int64_t)c * nchar + ch) * K;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    out_s[o + i] = cc[i];
    if (out_e) out_e[o + i] = e[i];
    if (out_b) out_b[o + i] = beta[i];
  }
}

// Goloboff's beta of a preliminary cost vector: e = s - min s (an infinite
// state stays infinite; canonize, sankCS.ml:254-271, and elt_median's e,
// whose max_int is infinite under +$), beta[y] = min_x tcm[y][x] +$ e[x].
template <int K>
__device__ __forceinline__ void sank_beta(const int *tcm, const int *s, int *beta) {
  int mn = kSInf, e[K];
#pragma unroll
  for (int i = 0; i < K; ++i) mn = s[i] < mn ? s[i] : mn;
#pragma unroll
  for (int i = 0; i < K; ++i) e[i] = s[i] >= kSInf ? kSInf : s[i] - mn;
#pragma unroll
  for (int y = 0; y < K; ++y) {
    int best = kSInf;
#pragma unroll
    for (int x = 0; x < K; ++x) {
      const int v = sadd(tcm[y * K + x], e[x]);
      best = v < best ? v : best;
    }
    beta[y] = best;
  }
}

// elt_median_3 (sankCS.ml:402-452) for one (node, character): the node's
// final e and best states from its ancestor's final (e, best-state bits),
// its preliminary s and its children's preliminary s (their beta).
template <int K>
__global__ void k_sank_median3(const int32_t *nodes, const int32_t *fin_e,
                               const int32_t *fin_best, int nchar, const int32_t *tcm_g, int n,
                               const int32_t *anc, const int32_t *node, const int32_t *left,
                               const int32_t *right, int32_t *out_e, int32_t *out_best) {
  __shared__ int tcm[K * K];
  for (int t = threadIdx.x; t < K * K; t += blockDim.x) tcm[t] = tcm_g[t];
  __syncthreads();
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (int64_t)n * nchar) return;
  const int c = (int)(g / nchar), ch = (int)(g % nchar);
  const int32_t *ae_p = fin_e + ((int64_t)anc[c] * nchar + ch) * K;
  const int32_t *ns_p = nodes + ((int64_t)node[c] * nchar + ch) * K;
  const int32_t *ls_p = nodes + ((int64_t)left[c] * nchar + ch) * K;
  const int32_t *rs_p = nodes + ((int64_t)right[c] * nchar + ch) * K;
  const uint32_t abest = (uint32_t)fin_best[(int64_t)anc[c] * nchar + ch];
  int ae[K], ns[K], ls[K], rs[K], lb[K], rb[K], bst[K];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    ae[i] = ae_p[i];
    ns[i] = ns_p[i];
    ls[i] = ls_p[i];
    rs[i] = rs_p[i];
  }
  sank_beta<K>(tcm, ls, lb);
  sank_beta<K>(tcm, rs, rb);
#pragma unroll
  for (int i = 0; i < K; ++i) {  // init_d': best over x for ancestor state i
    int b = kSInf;
#pragma unroll
    for (int x = 0; x < K; ++x) {
      const int v = sadd(sadd(tcm[i * K + x], lb[x]), rb[x]);
      b = v < b ? v : b;
    }
    bst[i] = b;
  }
  const int64_t o = ((int64_t)c * nchar + ch) * K;
#pragma unroll
  for (int s = 0; s < K; ++s) {  // init_e: min over ancestor states of d'[i][s]
    int b = kSInf;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int d = sadd(sadd(sadd(ae[i], tcm[i * K + s]), lb[s]), rb[s]);
      // -$: an infinite minuend is infinite here, an infinite subtrahend gives 0
      const int v = d >= kSInf ? kSInf : (bst[i] >= kSInf ? 0 : d - bst[i]);
      b = v < b ? v : b;
    }
    out_e[o + s] = b;
  }
  // best states: the node's states cheapest against the ancestor's best
  // states (plain + and min from infinity; every final has a best state)
  int best_cost = kSInf;
  uint32_t mine = 0;
#pragma unroll
  for (int pos = 0; pos < K; ++pos) {
    int mc = kSInf;
#pragma unroll
    for (int x = 0; x < K; ++x)
      if ((abest >> x) & 1u) {
        const int v = ns[pos] + tcm[pos * K + x];
        mc = v < mc ? v : mc;
      }
    if (mc == best_cost) mine |= 1u << pos;
    else if (mc < best_cost) {
      best_cost = mc;
      mine = 1u << pos;
    }
  }
  out_best[(int64_t)c * nchar + ch] = (int32_t)mine;
}

template <int K>
__global__ void k_sank_distance(const int32_t *nodes, int nchar, const int32_t *tcm_g, int n,
                                const int32_t *ai, const int32_t *bi, int64_t *dist) {
  __shared__ int tcm[K * K];
  for (int t = threadIdx.x; t < K * K; t += blockDim.x) tcm[t] = tcm_g[t];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= n) return;
  long long acc = 0;
  for (int ch = lane; ch < nchar; ch += 32) {
    const int32_t *a = nodes + ((int64_t)ai[c] * nchar + ch) * K;
    const int32_t *b = nodes + ((int64_t)bi[c] * nchar + ch) * K;
    int as[K], bs[K], cc[K], e[K], beta[K], minc, mina, minb;
#pragma unroll
    for (int i = 0; i < K; ++i) { as[i] = a[i]; bs[i] = b[i]; }
    sank_char<K>(tcm, as, bs, cc, e, beta, minc, mina, minb);
    acc += (long long)minc - mina - minb;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(kFullF, acc, o);
  if (lane == 0) dist[c] = acc;
}

#define FS_CK(call)                                       \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

int check_rows(const void *nodes, int64_t stride, int len, int n) {
  if (n < 0 || len < 0) return fail(POYD_EINVAL, "negative size");
  if (n > 0 && !nodes) return fail(POYD_EINVAL, "null node array");
  if (stride % 16 || stride < ((len + 15) / 16) * 16 || ((uintptr_t)nodes & 15))
    return fail(POYD_EINVAL, "node rows must be 16-byte aligned with stride >= len rounded to 16");
  return POYD_OK;
}

}  // namespace
}  // namespace poyd

using namespace poyd;

extern "C" int poyd_nonadd8_distance_batch(const uint8_t *nodes, int64_t stride, int32_t len,
                                           int32_t n, const int32_t *a_idx,
                                           const int32_t *b_idx, int64_t *dist, void *stream) {
  int rc = check_rows(nodes, stride, len, n);
  if (rc) return rc;
  if (n == 0) return POYD_OK;
  if (!a_idx || !b_idx || !dist) return fail(POYD_EINVAL, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps("fitch_distance", st);
  k_fitch_distance<<<(unsigned)(((int64_t)n * 32 + 255) / 256), 256, 0, st>>>(
      nodes, stride, len, n, a_idx, b_idx, dist);
  FS_CK(cudaGetLastError());
  return POYD_OK;
}

extern "C" int poyd_nonadd8_median_batch(const uint8_t *nodes, int64_t stride, int32_t len,
                                         int32_t n, const int32_t *a_idx, const int32_t *b_idx,
                                         uint8_t *out, int64_t *added_cost, void *stream) {
  int rc = check_rows(nodes, stride, len, n);
  if (rc) return rc;
  if (n == 0) return POYD_OK;
  if (!a_idx || !b_idx) return fail(POYD_EINVAL, "null argument");
  if (!out || ((uintptr_t)out & 15)) return fail(POYD_EINVAL, "output rows must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps("fitch_median", st);
  k_fitch_median<<<(unsigned)(((int64_t)n * 32 + 255) / 256), 256, 0, st>>>(
      nodes, stride, len, n, a_idx, b_idx, out, added_cost);
  FS_CK(cudaGetLastError());
  return POYD_OK;
}

extern "C" int poyd_nonadd8_median_3_batch(const uint8_t *nodes, int64_t stride, int32_t len,
                                           int32_t n, const int32_t *anc, const int32_t *prelim,
                                           const int32_t *d1, const int32_t *d2, uint8_t *out,
                                           void *stream) {
  int rc = check_rows(nodes, stride, len, n);
  if (rc) return rc;
  if (n == 0) return POYD_OK;
  if (!anc || !prelim || !d1 || !d2) return fail(POYD_EINVAL, "null argument");
  if (!out || ((uintptr_t)out & 15)) return fail(POYD_EINVAL, "output rows must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps("fitch_median3", st);
  k_fitch_median3<<<(unsigned)(((int64_t)n * 32 + 255) / 256), 256, 0, st>>>(
      nodes, stride, len, n, anc, prelim, d1, d2, out);
  FS_CK(cudaGetLastError());
  return POYD_OK;
}

#define SANK_DISPATCH(KV, launch) \
  case KV: launch(KV); break;

extern "C" int poyd_sank_median_batch(const int32_t *nodes, int32_t nchar, int32_t k,
                                      const int32_t *tcm, int32_t n, const int32_t *a_idx,
                                      const int32_t *b_idx, int32_t *out_s, int32_t *out_e,
                                      int32_t *out_beta, void *stream) {
  if (k < 2 || k > 8) return fail(POYD_EUNSUP, "Sankoff characters need 2..8 states");
  if (n < 0 || nchar < 0) return fail(POYD_EINVAL, "negative size");
  if (n == 0 || nchar == 0) return POYD_OK;
  if (!nodes || !tcm || !a_idx || !b_idx || !out_s) return fail(POYD_EINVAL, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t total = (int64_t)n * nchar;
  const unsigned blocks = (unsigned)((total + 255) / 256);
  ProfScope ps("sank_median", st);
#define L(KV) k_sank_median<KV><<<blocks, 256, 0, st>>>(nodes, nchar, tcm, n, a_idx, b_idx, out_s, out_e, out_beta)
  switch (k) {
    SANK_DISPATCH(2, L) SANK_DISPATCH(3, L) SANK_DISPATCH(4, L) SANK_DISPATCH(5, L)
    SANK_DISPATCH(6, L) SANK_DISPATCH(7, L) SANK_DISPATCH(8, L)
  }
#undef L
  FS_CK(cudaGetLastError());
  return POYD_OK;
}

extern "C" int poyd_sank_distance_batch(const int32_t *nodes, int32_t nchar, int32_t k,
                                        const int32_t *tcm, int32_t n, const int32_t *a_idx,
                                        const int32_t *b_idx, int64_t *dist, void *stream) {
  if (k < 2 || k > 8) return fail(POYD_EUNSUP, "Sankoff characters need 2..8 states");
  if (n < 0 || nchar < 0) return fail(POYD_EINVAL, "negative size");
  if (n == 0) return POYD_OK;
  if (!nodes || !tcm || !a_idx || !b_idx || !dist) return fail(POYD_EINVAL, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)(((int64_t)n * 32 + 255) / 256);
  ProfScope ps("sank_distance", st);
#define L(KV) k_sank_distance<KV><<<blocks, 256, 0, st>>>(nodes, nchar, tcm, n, a_idx, b_idx, dist)
  switch (k) {
    SANK_DISPATCH(2, L) SANK_DISPATCH(3, L) SANK_DISPATCH(4, L) SANK_DISPATCH(5, L)
    SANK_DISPATCH(6, L) SANK_DISPATCH(7, L) SANK_DISPATCH(8, L)
  }
#undef L
  FS_CK(cudaGetLastError());
  return POYD_OK;
}

extern "C" int poyd_sank_median_3_batch(const int32_t *nodes, const int32_t *fin_e,
                                        const int32_t *fin_best, int32_t nchar, int32_t k,
                                        const int32_t *tcm, int32_t n, const int32_t *anc,
                                        const int32_t *node, const int32_t *left,
                                        const int32_t *right, int32_t *out_e,
                                        int32_t *out_best, void *stream) {
  if (k < 2 || k > 8) return fail(POYD_EUNSUP, "Sankoff characters need 2..8 states");
  if (n < 0 || nchar < 0) return fail(POYD_EINVAL, "negative size");
  if (n == 0 || nchar == 0) return POYD_OK;
  if (!nodes || !fin_e || !fin_best || !tcm || !anc || !node || !left || !right || !out_e ||
      !out_best)
    return fail(POYD_EINVAL, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t total = (int64_t)n * nchar;
  const unsigned blocks = (unsigned)((total + 255) / 256);
  ProfScope ps("sank_median3", st);
#define L(KV)                                                                              \
  k_sank_median3<KV><<<blocks, 256, 0, st>>>(nodes, fin_e, fin_best, nchar, tcm, n, anc, node, \
                                             left, right, out_e, out_best)
  switch (k) {
    SANK_DISPATCH(2, L) SANK_DISPATCH(3, L) SANK_DISPATCH(4, L) SANK_DISPATCH(5, L)
    SANK_DISPATCH(6, L) SANK_DISPATCH(7, L) SANK_DISPATCH(8, L)
  }
#undef L
  FS_CK(cudaGetLastError());
  return POYD_OK;
}

namespace poyd {
namespace {

// One block per pair of a level (see LevelPost): the Fitch median
// (k_fitch_median's arithmetic, its count summed over the block), the
// Sankoff medians (k_sank_median's), and by thread 0 the DO median's place:
// the fourth sequence of the pair's result slot.
template <int K>
__global__ void __launch_bounds__(128) k_level_post(LevelPost P) {
  __shared__ int tcm[64];
  __shared__ unsigned wsum[4];
  const int i = blockIdx.x;
  if (K > 0)
    for (int t = threadIdx.x; t < K * K; t += blockDim.x) tcm[t] = P.tcm[t];
  const int ia = P.a[i], ib = P.b[i], io = P.out[i];
  unsigned cnt = 0;
  if (P.fitch_len > 0) {
    const uint4 *fa = (const uint4 *)(P.fitch + (int64_t)ia * P.stride);
    const uint4 *fb = (const uint4 *)(P.fitch + (int64_t)ib * P.stride);
    uint4 *r = (uint4 *)(P.fitch + (int64_t)io * P.stride);
    const int nv = (P.fitch_len + 15) >> 4;
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
      const uint4 x = fa[v], y = fb[v];
      const int valid = P.fitch_len - v * 16;
      uint4 o;
      uint32_t in, z;
      in = x.x & y.x; z = zbytes(in); o.x = in | (z & (x.x | y.x)); cnt += __popc(z & ~tailmask(valid, 0)) >> 3;
      in = x.y & y.y; z = zbytes(in); o.y = in | (z & (x.y | y.y)); cnt += __popc(z & ~tailmask(valid, 1)) >> 3;
      in = x.z & y.z; z = zbytes(in); o.z = in | (z & (x.z | y.z)); cnt += __popc(z & ~tailmask(valid, 2)) >> 3;
      in = x.w & y.w; z = zbytes(in); o.w = in | (z & (x.w | y.w)); cnt += __popc(z & ~tailmask(valid, 3)) >> 3;
      r[v] = o;
    }
  }
  __syncthreads();  // tcm
  if (K > 0) {
    for (int ch = threadIdx.x; ch < P.nchar; ch += blockDim.x) {
      const int32_t *sa = P.sank + ((int64_t)ia * P.nchar + ch) * K;
      const int32_t *sb = P.sank + ((int64_t)ib * P.nchar + ch) * K;
      int as[K > 0 ? K : 1], bs[K > 0 ? K : 1], cc[K > 0 ? K : 1], e[K > 0 ? K : 1],
          beta[K > 0 ? K : 1], minc, mina, minb;
#pragma unroll
      for (int q = 0; q < K; ++q) { as[q] = sa[q]; bs[q] = sb[q]; }
      sank_char<K>(tcm, as, bs, cc, e, beta, minc, mina, minb);
      int32_t *so = P.sank + ((int64_t)io * P.nchar + ch) * K;
#pragma unroll
      for (int q = 0; q < K; ++q) so[q] = cc[q];
    }
  }
  cnt = __reduce_add_sync(kFullF, cnt);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned fc = wsum[0] + wsum[1] + wsum[2] + wsum[3];
    const int nm = P.out_len[2 * i + 1];
    if (nm < 0) {
      atomicOr(P.err, 1);
      P.node_off[io] = P.slot_off[i];
      P.node_len[io] = 0;
    } else {
      P.node_off[io] = P.slot_off[i] + 4 * slot_cap(P.a_len[i], P.b_len[i]) - nm;
      P.node_len[io] = nm;
    }
    P.costs[2 * i] = P.cost[i];
    P.costs[2 * i + 1] = P.fitch_len > 0 ? (int64_t)fc : 0;
  }
}

}  // namespace

int launch_level_post(const LevelPost &P, cudaStream_t st) {
  if (P.n == 0) return POYD_OK;
  const int k = P.nchar > 0 ? P.k : 0;
  if (k != 0 && (k < 2 || k > 8)) return fail(POYD_EUNSUP, "Sankoff characters need 2..8 states");
  ProfScope ps("level_post", st);
#define L(KV) k_level_post<KV><<<(unsigned)P.n, 128, 0, st>>>(P)
  switch (k) {
    case 0: L(0); break;
    SANK_DISPATCH(2, L) SANK_DISPATCH(3, L) SANK_DISPATCH(4, L) SANK_DISPATCH(5, L)
    SANK_DISPATCH(6, L) SANK_DISPATCH(7, L) SANK_DISPATCH(8, L)
  }
#undef L
  FS_CK(cudaGetLastError());
  return POYD_OK;
}

}  // namespace poyd
