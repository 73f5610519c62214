// Column operations on pairs that are already aligned (equal lengths): the
// externals of sequence.ml:453-758 that need no DP, batched.
//
//   median_2_with_gaps  algn_get_median_2d_with_gaps (algn.c:4011-4024):
//                       the median of every column
//   median_2_no_gaps    algn_get_median_2d_no_gaps (algn.c:4031-4046): the
//                       medians that are not gaps, after one leading gap
//   ancestor_2          algn_ancestor_2 (algn.c:4126-4147): non-gap
//                       medians with the leading gap; for an affine matrix
//                       with combinations every median, corrected by
//                       algn_correct_blocks_affine (algn.c:4080-4119) and
//                       stripped of gaps (algn_remove_gaps, algn.c:4048-4066)
//   worst_2 / verify_2  algn_calculate_from_2_aligned (algn.c:3316-3370)
//                       with the worst / cost table: the alignment's cost,
//                       gap openings charged per block
//
// One thread per pair: these are single passes over a few thousand bytes,
// negligible beside the DP, and the block correction and the gap-opening
// count are sequential state machines.  A sequence result lands
// right-aligned in the pair's slot (out + out_off[i], len[i] + 1 bytes),
// as the reference's seq_prepend leaves it.
#include "poyd_internal.h"

namespace poyd {

namespace {

enum ColOp { kMedianWg = 0, kMedianNoGaps = 1, kAncestor = 2, kWorst = 3, kVerify = 4 };

struct ColArgs {
  int n;
  const uint8_t *seq;
  const int64_t *a_off, *b_off;
  const int32_t *len;
  const DevTables *tab;
  int gap, combinations, affine, go;
  uint8_t *out;
  const int64_t *out_off;
  int32_t *out_len;
  int32_t *value;
};

// Block correction state of algn_correct_blocks_affine.
struct BlockFix {
  int extending = 0, inside = 0, prev = 0;
  __device__ int step(int gap, int ab, int bb, int sb) {
    const bool ga = ab & gap, gb = bb & gap;
    if (!inside && (!ga || !gb)) inside = 0;
    else if (inside && (!ga || !gb)) inside = 0;
    else if ((ga || gb) && (ab != gap || bb != gap)) inside = 1;
    else inside = 0;
    if ((ga || gb) && !(sb & gap) && !extending) {
      prev = inside;
      extending = 1;
    } else if (ga && gb && (sb & gap) && sb != gap && extending && inside && !prev) {
      sb &= ~gap;
      prev = 0;
    } else if (ga && gb && extending == 1) {
      prev = inside;
      extending = 0;
    }
    return sb;
  }
};

template <int OP>
__global__ void __launch_bounds__(128) k_columns(ColArgs A) {
  __shared__ uint8_t med[1024];
  __shared__ int32_t tab[1024];
  for (int t = threadIdx.x; t < 1024; t += blockDim.x) {
    med[t] = A.tab->median[t];
    tab[t] = OP == kWorst ? A.tab->worst[t] : A.tab->cost[t];
  }
  __syncthreads();
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= A.n) return;
  const uint8_t *a = A.seq + A.a_off[id];
  const uint8_t *b = A.seq + A.b_off[id];
  const int len = A.len[id];
  const int gap = A.gap;
  if (OP == kWorst || OP == kVerify) {
    // gap openings: one per block of gaps in either sequence; a leading
    // gap column is skipped
    const bool comb = A.combinations;
    auto isg = [&](int x) { return comb ? (x & gap) != 0 : x == gap; };
    int res = 0, row = 0, i = 0;
    if (len > 0 && isg(a[0]) && isg(b[0])) i = 1;
    for (; i < len; ++i) {
      const int x = a[i], y = b[i];
      const bool gx = isg(x), gy = isg(y);
      if (row == 0) {
        if (gx && (!comb || !gy)) { res += A.go; row = 1; }
        else if (gy && (!comb || !gx)) { res += A.go; row = 2; }
      } else if (row == 1) {
        if (!gx) {
          if (gy) { res += A.go; row = 2; }
          else row = 0;
        }
      } else {
        if (!gy) {
          if (gx) { res += A.go; row = 1; }
          else row = 0;
        }
      }
      res += tab[(x << 5) | y];
    }
    A.value[id] = res;
    return;
  }
  uint8_t *end = A.out + A.out_off[id] + len + 1;
  if (OP == kMedianWg) {
    for (int i = 0; i < len; ++i) end[i - len] = med[(a[i] << 5) | b[i]];
    A.out_len[id] = len;
    return;
  }
  const bool fix = OP == kAncestor && A.combinations && A.affine;
  // pass 1: the result's length; pass 2: its bytes after the leading gap
  int count = 0;
  BlockFix F;
  for (int i = 0; i < len; ++i) {
    int v = med[(a[i] << 5) | b[i]];
    if (fix) v = F.step(gap, a[i], b[i], v);
    count += v != gap;
  }
  uint8_t *o = end - (count + 1);
  o[0] = (uint8_t)gap;
  int k = 1;
  BlockFix G;
  for (int i = 0; i < len; ++i) {
    int v = med[(a[i] << 5) | b[i]];
    if (fix) v = G.step(gap, a[i], b[i], v);
    if (v != gap) o[k++] = (uint8_t)v;
  }
  A.out_len[id] = count + 1;
}

int columns(int op, const poyd_cm *cm, int32_t n, const uint8_t *seq, const int64_t *a_off,
            const int64_t *b_off, const int32_t *len, uint8_t *out, const int64_t *out_off,
            int32_t *out_len, int32_t *value, void *stream) {
  if (!cm) return fail(POYD_EINVAL, "column operation: null cost matrix");
  const bool seq_op = op <= kAncestor;
  if (n < 0 || (n > 0 && (!seq || !a_off || !b_off || !len ||
                          (seq_op ? (!out || !out_off || !out_len) : !value))))
    return fail(POYD_EINVAL, "column operation: null argument");
  if (n == 0) return POYD_OK;
  DevTables *tabs = nullptr;
  int rc = upload_tables(cm, &tabs, stream);
  if (rc) return rc;
  ColArgs A;
  A.n = n; A.seq = seq; A.a_off = a_off; A.b_off = b_off; A.len = len; A.tab = tabs;
  A.gap = cm->gap; A.combinations = cm->combinations; A.affine = cm->cost_model == 1;
  A.go = cm->gap_open;  // cm_get_gap_opening_parameter: 0 for a linear matrix
  A.out = out; A.out_off = out_off; A.out_len = out_len; A.value = value;
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned blocks = (unsigned)(((int64_t)n + 127) / 128);
  ProfScope ps("columns", st);
  switch (op) {
    case kMedianWg: k_columns<kMedianWg><<<blocks, 128, 0, st>>>(A); break;
    case kMedianNoGaps: k_columns<kMedianNoGaps><<<blocks, 128, 0, st>>>(A); break;
    case kAncestor: k_columns<kAncestor><<<blocks, 128, 0, st>>>(A); break;
    case kWorst: k_columns<kWorst><<<blocks, 128, 0, st>>>(A); break;
    default: k_columns<kVerify><<<blocks, 128, 0, st>>>(A); break;
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? POYD_OK : cuda_fail(e, "k_columns");
}

// Single-pair form over host buffers: upload, one launch, download.
int columns_host(int op, const uint8_t *a, const uint8_t *b, int32_t len, const poyd_cm *cm,
                 uint8_t *out, int32_t *out_len, int32_t *value) {
  if (!a || !b || len < 0 || (op <= kAncestor ? (!out || !out_len) : !value))
    return fail(POYD_EINVAL, "column operation: null argument");
  Workspace *w = workspace();
  const size_t L = (size_t)len;
  // [a | b | out slot] then {a_off, b_off, out_off, len, out_len, value}
  uint8_t *buf = (uint8_t *)ws_buffer(w, WS_SEQ, 3 * L + 64);
  int64_t *meta = (int64_t *)ws_buffer(w, WS_META, 64);
  if (!buf || !meta) return fail(POYD_ENOMEM, "column operation: workspace");
  const int64_t hm[3] = {0, (int64_t)L, (int64_t)(2 * L)};
  int32_t *m32 = (int32_t *)(meta + 3);
  cudaError_t e = cudaMemcpy(buf, a, L, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(buf + L, b, L, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(meta, hm, sizeof hm, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m32, &len, sizeof len, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "column operation upload");
  int rc = columns(op, cm, 1, buf, meta, meta + 1, m32, buf, meta + 2, m32 + 1, m32 + 2, nullptr);
  if (rc) return rc;
  int32_t res[2] = {0, 0};
  e = cudaMemcpy(res, m32 + 1, sizeof res, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "column operation");
  if (op <= kAncestor) {
    *out_len = res[0];
    e = cudaMemcpy(out, buf + 2 * L + L + 1 - res[0], (size_t)res[0], cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "column operation");
  } else {
    *value = res[1];
  }
  return POYD_OK;
}

}  // namespace

}  // namespace poyd

using namespace poyd;

#define POYD_COLUMN_BATCH(name, op)                                                           \
  extern "C" int name(const poyd_cm *cm, int32_t n, const uint8_t *seq, const int64_t *a_off, \
                      const int64_t *b_off, const int32_t *len, uint8_t *out,                 \
                      const int64_t *out_off, int32_t *out_len, void *stream) {               \
    return columns(op, cm, n, seq, a_off, b_off, len, out, out_off, out_len, nullptr, stream); \
  }
POYD_COLUMN_BATCH(poyd_median_2_with_gaps_batch, kMedianWg)
POYD_COLUMN_BATCH(poyd_median_2_no_gaps_batch, kMedianNoGaps)
POYD_COLUMN_BATCH(poyd_ancestor_2_batch, kAncestor)

extern "C" int poyd_worst_2_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                                  const int64_t *a_off, const int64_t *b_off, const int32_t *len,
                                  int32_t *value, void *stream) {
  return columns(kWorst, cm, n, seq, a_off, b_off, len, nullptr, nullptr, nullptr, value, stream);
}

extern "C" int poyd_verify_2_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                                   const int64_t *a_off, const int64_t *b_off, const int32_t *len,
                                   int32_t *value, void *stream) {
  return columns(kVerify, cm, n, seq, a_off, b_off, len, nullptr, nullptr, nullptr, value, stream);
}

extern "C" int poyd_algn_median_2_with_gaps(const uint8_t *a, const uint8_t *b, int32_t len,
                                            const poyd_cm *cm, uint8_t *out, int32_t *out_len) {
  return columns_host(kMedianWg, a, b, len, cm, out, out_len, nullptr);
}
extern "C" int poyd_algn_median_2_no_gaps(const uint8_t *a, const uint8_t *b, int32_t len,
                                          const poyd_cm *cm, uint8_t *out, int32_t *out_len) {
  return columns_host(kMedianNoGaps, a, b, len, cm, out, out_len, nullptr);
}
extern "C" int poyd_algn_ancestor_2(const uint8_t *a, const uint8_t *b, int32_t len,
                                    const poyd_cm *cm, uint8_t *out, int32_t *out_len) {
  return columns_host(kAncestor, a, b, len, cm, out, out_len, nullptr);
}
extern "C" int poyd_algn_worst_2(const uint8_t *a, const uint8_t *b, int32_t len,
                                 const poyd_cm *cm, int32_t *value) {
  return columns_host(kWorst, a, b, len, cm, nullptr, nullptr, value);
}
extern "C" int poyd_algn_verify_2(const uint8_t *a, const uint8_t *b, int32_t len,
                                  const poyd_cm *cm, int32_t *value) {
  return columns_host(kVerify, a, b, len, cm, nullptr, nullptr, value);
}
