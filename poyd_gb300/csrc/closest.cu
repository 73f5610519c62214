// Batched Sequence.Align.closest (sequence.ml:967-1033) as DOS.to_single
// calls it (seqCS.ml:730-745): the final ("single") sequence of a node from
// its parent's single sequence and its own preliminary median.
//
// The pairs (parent, node) are first aligned by the batched align_2 (the
// linear or affine driver, outputs in the caller's slots).  Then one warp
// per pair walks the aligned columns: each column of the node becomes its
// state closest to the parent's column (Cost_matrix.Two_D.get_closest,
// cost_matrix.ml:681-698), gaps are dropped and the leading gap is put back.
// Identical sequences skip the alignment in the reference: their columns
// are the sequences themselves with the gap bit cleared past position 0.
// The result lands right-aligned in the slot's fourth segment, where
// align_2 leaves the median.
#include <climits>

#include "poyd_internal.h"

namespace poyd {

// get_closest a b: states of b tried lowest bit first, first strict
// minimum of cost[a][state]; -1 when b has no state.
__device__ __forceinline__ int closest_state(const int32_t *cost, int a, int b, int gap,
                                             int nbits) {
  if (a != gap && b != gap) b = ((a & gap) && (b & gap)) ? gap : (b & ~gap);
  int best = -1, bc = INT_MAX;
  for (int x = 0; x < nbits; ++x) {
    const int v = 1 << x;
    if (b & v) {
      const int c = cost[(a << 5) | v];
      if (best < 0 || c < bc) {
        best = v;
        bc = c;
      }
    }
  }
  return best;
}

__device__ __forceinline__ bool warp_all_gap(const uint8_t *s, int len, int gap, int lane) {
  bool ok = true;
  for (int i = lane; i < len; i += 32) ok &= (s[i] == gap);
  return __all_sync(0xffffffffu, ok);
}

__device__ __forceinline__ bool warp_equal(const uint8_t *a, const uint8_t *b, int len,
                                           int lane) {
  bool ok = true;
  for (int i = lane; i < len; i += 32) ok &= (a[i] == b[i]);
  return __all_sync(0xffffffffu, ok);
}

// Column i of the pair as get_closest sees it.
__device__ __forceinline__ int column_state(const int32_t *cost, const uint8_t *A,
                                            const uint8_t *B, int64_t i, bool mask, int gap,
                                            int nbits) {
  int a = A[i], b = B[i];
  if (mask && i > 0) {
    a &= ~gap;
    b &= ~gap;
  }
  return closest_state(cost, a, b, gap, nbits);
}

__global__ void __launch_bounds__(256) k_closest(int32_t n, const uint8_t *seq,
                                                 const int64_t *p_off, const int32_t *p_len,
                                                 const int64_t *m_off, const int32_t *m_len,
                                                 uint8_t *out, const int64_t *out_off,
                                                 int32_t *out_len, const DevTables *tab, int gap,
                                                 int nbits, int dos_empty) {
  __shared__ int32_t cost[1024];
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) cost[i] = tab->cost[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (id >= n) return;
  int lp = p_len[id];
  const int lm = m_len[id];
  const uint8_t *P = seq + p_off[id];
  const uint8_t *M = seq + m_off[id];
  const int64_t cap = slot_cap(lp, lm);
  uint8_t *slot = out + out_off[id];
  uint8_t *end = slot + 4 * cap;
  if (warp_all_gap(M, lm, gap, lane)) {  // closest returns the node itself
    for (int i = lane; i < lm; i += 32) end[i - lm] = M[i];
    if (lane == 0) out_len[2 * id + 1] = lm;
    return;
  }
  if (dos_empty && warp_all_gap(P, lp, gap, lane)) {  // DOS.to_single: parent := node
    P = M;
    lp = lm;
  }
  const bool same = lp == lm && warp_equal(P, M, lm, lane);
  const uint8_t *A, *B;
  int64_t L;
  if (same) {
    A = P;
    B = M;
    L = lm;
  } else {
    L = out_len[2 * id];
    if (L < 0 || L > cap) {  // the alignment failed: propagate
      if (lane == 0) out_len[2 * id + 1] = -1;
      return;
    }
    A = slot + cap - L;
    B = slot + 2 * cap - L;
  }
  // pass 1: how many columns keep a state (the result is right-aligned)
  int count = 0;
  bool bad = false;
  for (int64_t base = 0; base < L; base += 32) {
    const int64_t i = base + lane;
    const int v = i < L ? column_state(cost, A, B, i, same, gap, nbits) : gap;
    bad |= v < 0;
    count += __popc(__ballot_sync(0xffffffffu, v >= 0 && v != gap));
  }
  if (__any_sync(0xffffffffu, bad)) {
    if (lane == 0) out_len[2 * id + 1] = -2;
    return;
  }
  uint8_t *o = end - (1 + count);
  if (lane == 0) o[0] = (uint8_t)gap;
  int pos = 1;
  for (int64_t base = 0; base < L; base += 32) {
    const int64_t i = base + lane;
    const int v = i < L ? column_state(cost, A, B, i, same, gap, nbits) : gap;
    const bool keep = v != gap;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) o[pos + __popc(m & ((1u << lane) - 1))] = (uint8_t)v;
    pos += __popc(m);
  }
  if (lane == 0) out_len[2 * id + 1] = 1 + count;
}

}  // namespace poyd

using namespace poyd;

extern "C" int poyd_closest_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                                  const int64_t *p_off, const int32_t *p_len,
                                  const int64_t *m_off, const int32_t *m_len, int32_t *cost,
                                  uint8_t *out, const int64_t *out_off, int32_t *out_len,
                                  int32_t flags, void *stream) {
  if (!cm) return fail(POYD_EINVAL, "poyd_closest_batch: null cost matrix");
  if (!cm->combinations)
    return fail(POYD_EUNSUP, "poyd_closest_batch: alphabets without combinations");
  if (cm->lcm < 1 || cm->lcm > 5)
    return fail(POYD_EUNSUP, "poyd_closest_batch: states must fit 5 bits");
  int rc = poyd_align_2_batch(cm, n, seq, p_off, p_len, m_off, m_len, cost, out, out_off,
                              out_len, nullptr, 0, stream);
  if (rc || n == 0) return rc;
  DevTables *tabs = nullptr;
  rc = upload_tables(cm, &tabs, stream);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int threads = 256;
  const int64_t blocks = ((int64_t)n * 32 + threads - 1) / threads;
  {
    ProfScope ps("closest", st);
    k_closest<<<(unsigned)blocks, threads, 0, st>>>(n, seq, p_off, p_len, m_off, m_len, out,
                                                    out_off, out_len, tabs, cm->gap, cm->lcm,
                                                    (flags & POYD_FLAG_DOS_EMPTY) ? 1 : 0);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_closest");
  return POYD_OK;
}
