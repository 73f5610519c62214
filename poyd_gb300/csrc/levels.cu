// poyd_median_levels: downpass levels with the node data resident on the
// device.
//
// A downpass level is one batch of median pairs (DOS.median, seqCS.ml:747-776;
// NonaddCS8.median and SankCS.median through Node.median, node.ml:272/333),
// and every level waits on the ones below it.  Driven from the host one
// batched call per level, each level pays a round trip for the output
// lengths before the next level's batch can be laid out.  Here the whole
// list of levels runs on one stream: per level
//   1. k_lvl_gather builds the pair batch from the device node table (the
//      places of the inputs) and lays the result slots out in the pool;
//   2. the batched align_2 (plan, order, DP with fused traceback) writes
//      every pair's four result sequences into its slot;
//   3. one launch (launch_level_post) writes the Fitch and Sankoff medians
//      into the output nodes' own rows and points every output node at its
//      median (the fourth sequence of its slot), recording the costs.
// The host waits once per level (the align_2 plan read-back) and once at the
// end, when the output nodes' places and the costs come back.
#include <cuda_runtime.h>
#include <algorithm>
#include <vector>
#include "poyd_internal.h"

namespace poyd {
namespace {

#define LV_CK(call)                                       \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

constexpr int kLvlThreads = 1024;

// Pair batch of one level from the node table, and its result slots: slot
// i starts at the running pool top plus the sizes of slots 0..i-1 (4 *
// slot_cap bytes each); the top advances past the level, rounded to 128
// bytes so that no cache line holds both this level's results and the next
// level's.  One block: levels are small, and the scan is sequential over
// chunks of kLvlThreads pairs.
__global__ void __launch_bounds__(kLvlThreads) k_lvl_gather(
    int n, const int32_t *a, const int32_t *b, const int64_t *node_off, const int32_t *node_len,
    int64_t *a_off, int32_t *a_len, int64_t *b_off, int32_t *b_len, int64_t *slot_off,
    int64_t *top) {
  __shared__ int64_t warp_sum[kLvlThreads / 32];
  __shared__ int64_t base;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) base = *top;
  __syncthreads();
  for (int c0 = 0; c0 < n; c0 += kLvlThreads) {
    const int i = c0 + threadIdx.x;
    int64_t sz = 0;
    if (i < n) {
      const int ia = a[i], ib = b[i];
      const int la = node_len[ia], lb = node_len[ib];
      a_off[i] = node_off[ia];
      a_len[i] = la;
      b_off[i] = node_off[ib];
      b_len[i] = lb;
      sz = 4 * slot_cap(la, lb);
    }
    int64_t x = sz;  // inclusive warp scan
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int64_t w = warp_sum[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warp_sum[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const int64_t before = (wid ? warp_sum[wid - 1] : 0) + x - sz;
    if (i < n) slot_off[i] = base + before;
    __syncthreads();
    if (threadIdx.x == 0) base += warp_sum[kLvlThreads / 32 - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *top = (base + 127) & ~(int64_t)127;
}

// The output nodes' places, pair order: res[2i] = offset, res[2i+1] = length.
__global__ void k_lvl_collect(int n, const int32_t *out, const int64_t *node_off,
                              const int32_t *node_len, int64_t *res) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  res[2 * i] = node_off[out[i]];
  res[2 * i + 1] = node_len[out[i]];
}

template <typename T>
T *carve(unsigned char *&p, size_t count) {
  T *r = (T *)p;
  p += (count * sizeof(T) + 255) / 256 * 256;
  return r;
}

}  // namespace
}  // namespace poyd

using namespace poyd;

extern "C" int poyd_median_levels(const poyd_cm *cm, const poyd_node_store *store,
                                  int32_t n_nodes, int64_t *node_off, int32_t *node_len,
                                  int32_t n_levels, const int32_t *level_start, const int32_t *a,
                                  const int32_t *b, const int32_t *out, int64_t *pool_top,
                                  int64_t *need, int64_t *costs, void *stream) {
  if (!cm || !store || !node_off || !node_len || !level_start || !pool_top)
    return fail(POYD_EINVAL, "poyd_median_levels: null argument");
  if (n_nodes < 0 || n_levels < 0) return fail(POYD_EINVAL, "negative size");
  if (n_levels == 0) return POYD_OK;
  if (level_start[0] != 0) return fail(POYD_EINVAL, "level_start[0] must be 0");
  for (int l = 0; l < n_levels; ++l)
    if (level_start[l + 1] < level_start[l]) return fail(POYD_EINVAL, "level_start must not decrease");
  const int32_t np = level_start[n_levels];
  if (np == 0) return POYD_OK;
  if (!a || !b || !out || !store->pool) return fail(POYD_EINVAL, "poyd_median_levels: null argument");
  if (store->fitch_len < 0 || store->sank_nchar < 0) return fail(POYD_EINVAL, "negative size");
  if (store->fitch_len > 0 &&
      (!store->fitch || store->fitch_stride % 16 || store->fitch_stride < (store->fitch_len + 15) / 16 * 16 ||
       ((uintptr_t)store->fitch & 15)))
    return fail(POYD_EINVAL, "Fitch rows must be 16-byte aligned with stride >= len rounded to 16");
  if (store->sank_nchar > 0 && (!store->sank || !store->sank_tcm))
    return fail(POYD_EINVAL, "null Sankoff rows or matrix");
  if (store->sank_nchar > 0 && (store->sank_k < 2 || store->sank_k > 8))
    return fail(POYD_EUNSUP, "Sankoff characters need 2..8 states");

  // Ids, the write-once rule and a host bound of the pool bytes: a median
  // is at most la + lb long, so its slot is at most 4 * slot_cap of the
  // bounds of its inputs; each level's slots are rounded to 128 bytes.
  std::vector<int32_t> bound(node_len, node_len + n_nodes);
  // written[v]: 0 never an output, else 1 + the level that writes v
  std::vector<int32_t> written((size_t)n_nodes, 0);
  int64_t total = 0;
  for (int l = 0; l < n_levels; ++l) {
    int64_t lvl = 0;
    for (int32_t i = level_start[l]; i < level_start[l + 1]; ++i) {
      const int32_t v = out[i];
      if (v < 0 || v >= n_nodes) return fail(POYD_EINVAL, "node id out of range");
      if (written[(size_t)v]) return fail(POYD_EINVAL, "node %d is an output twice", v);
      written[(size_t)v] = 1 + l;
    }
    for (int32_t i = level_start[l]; i < level_start[l + 1]; ++i) {
      const int32_t x = a[i], y = b[i];
      if (x < 0 || x >= n_nodes || y < 0 || y >= n_nodes)
        return fail(POYD_EINVAL, "node id out of range");
      // the Fitch and Sankoff kernels read inputs and write outputs of a
      // level in one launch
      if (written[(size_t)x] == 1 + l || written[(size_t)y] == 1 + l)
        return fail(POYD_EINVAL, "an output of a level is an input of the same level");
      if (bound[x] < 1 || bound[y] < 1) return fail(POYD_EINVAL, "input node without a sequence");
      lvl += 4 * slot_cap(bound[x], bound[y]);
    }
    // outputs take their bounds after the whole level (no input of the
    // level is an output of it)
    for (int32_t i = level_start[l]; i < level_start[l + 1]; ++i) {
      const int32_t v = out[i];
      const int64_t bv = (int64_t)bound[a[i]] + bound[b[i]];
      if (bv >= (1 << 30)) return fail(POYD_ERANGE, "sequence length bound overflows");
      bound[v] = (int32_t)bv;
    }
    total += (lvl + 127) / 128 * 128;
  }
  const int64_t start = (*pool_top + 127) & ~(int64_t)127;
  if (*pool_top < 0 || start + total > store->pool_size) {
    if (need) *need = total + 128;
    return fail(POYD_ESPACE, "sequence pool too small: the levels need up to %lld bytes above "
                "the top, %lld are free", (long long)(total + 128),
                (long long)(store->pool_size - *pool_top));
  }

  cudaStream_t st = (cudaStream_t)stream;
  Workspace *w = workspace(st);
  // device node table (int64 offsets then int32 lengths) and the top
  unsigned char *nd = (unsigned char *)ws_buffer(w, WS_LVL_NODES,
                                                 (size_t)n_nodes * 12 + 2048);
  const size_t per_pair = 3 * 4 + 2 * 8 + 2 * 4 + 8 + 2 * 4 + 4 + 2 * 8 + 2 * 8;
  unsigned char *pp = (unsigned char *)ws_buffer(w, WS_LVL_PAIRS, (size_t)np * per_pair + 16 * 256);
  if (!nd || !pp) return fail(POYD_ENOMEM, "level engine workspace allocation failed");
  unsigned char *q = nd;
  int64_t *d_off = carve<int64_t>(q, (size_t)n_nodes);
  int32_t *d_len = carve<int32_t>(q, (size_t)n_nodes);
  int64_t *d_top = carve<int64_t>(q, 1);
  int32_t *d_err = carve<int32_t>(q, 1);
  q = pp;
  int32_t *d_ids = carve<int32_t>(q, 3 * (size_t)np);  // a, b, out
  int64_t *a_off = carve<int64_t>(q, (size_t)np);
  int64_t *b_off = carve<int64_t>(q, (size_t)np);
  int32_t *a_len = carve<int32_t>(q, (size_t)np);
  int32_t *b_len = carve<int32_t>(q, (size_t)np);
  int64_t *slot_off = carve<int64_t>(q, (size_t)np);
  int32_t *out_len = carve<int32_t>(q, 2 * (size_t)np);
  int32_t *cost = carve<int32_t>(q, (size_t)np);
  int64_t *d_costs = carve<int64_t>(q, 2 * (size_t)np);
  int64_t *d_res = carve<int64_t>(q, 2 * (size_t)np);
  const int32_t *da = d_ids, *db = d_ids + np, *dout = d_ids + 2 * np;

  LV_CK(cudaMemcpyAsync(d_off, node_off, sizeof(int64_t) * (size_t)n_nodes, cudaMemcpyHostToDevice, st));
  LV_CK(cudaMemcpyAsync(d_len, node_len, sizeof(int32_t) * (size_t)n_nodes, cudaMemcpyHostToDevice, st));
  LV_CK(cudaMemcpyAsync(d_ids, a, sizeof(int32_t) * (size_t)np, cudaMemcpyHostToDevice, st));
  LV_CK(cudaMemcpyAsync(d_ids + np, b, sizeof(int32_t) * (size_t)np, cudaMemcpyHostToDevice, st));
  LV_CK(cudaMemcpyAsync(d_ids + 2 * np, out, sizeof(int32_t) * (size_t)np, cudaMemcpyHostToDevice, st));
  LV_CK(cudaMemcpyAsync(d_top, &start, sizeof(int64_t), cudaMemcpyHostToDevice, st));
  LV_CK(cudaMemsetAsync(d_err, 0, sizeof(int32_t), st));

  for (int l = 0; l < n_levels; ++l) {
    const int32_t s = level_start[l], n = level_start[l + 1] - s;
    if (n == 0) continue;
    k_lvl_gather<<<1, kLvlThreads, 0, st>>>(n, da + s, db + s, d_off, d_len, a_off + s, a_len + s,
                                            b_off + s, b_len + s, slot_off + s, d_top);
    LV_CK(cudaGetLastError());
    int rc = poyd_align_2_batch(cm, n, store->pool, a_off + s, a_len + s, b_off + s, b_len + s,
                                cost + s, store->pool, slot_off + s, out_len + 2 * s, nullptr,
                                POYD_FLAG_DOS_EMPTY, st);
    if (rc) return rc;
    LevelPost LP;
    LP.n = n; LP.a = da + s; LP.b = db + s; LP.out = dout + s;
    LP.fitch = store->fitch; LP.stride = store->fitch_stride; LP.fitch_len = store->fitch_len;
    LP.sank = store->sank; LP.nchar = store->sank_nchar; LP.k = store->sank_k;
    LP.tcm = store->sank_tcm;
    LP.slot_off = slot_off + s; LP.a_len = a_len + s; LP.b_len = b_len + s;
    LP.out_len = out_len + 2 * s; LP.cost = cost + s;
    LP.node_off = d_off; LP.node_len = d_len; LP.costs = d_costs + 2 * s; LP.err = d_err;
    rc = launch_level_post(LP, st);
    if (rc) return rc;
    LV_CK(cudaGetLastError());
  }
  k_lvl_collect<<<(np + 127) / 128, 128, 0, st>>>(np, dout, d_off, d_len, d_res);
  LV_CK(cudaGetLastError());
  std::vector<int64_t> res(2 * (size_t)np), cst(costs ? 0 : 2 * (size_t)np);
  int64_t top = 0;
  int32_t err = 0;
  LV_CK(cudaMemcpyAsync(res.data(), d_res, sizeof(int64_t) * 2 * (size_t)np, cudaMemcpyDeviceToHost, st));
  LV_CK(cudaMemcpyAsync(costs ? costs : cst.data(), d_costs, sizeof(int64_t) * 2 * (size_t)np,
                        cudaMemcpyDeviceToHost, st));
  LV_CK(cudaMemcpyAsync(&top, d_top, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  LV_CK(cudaMemcpyAsync(&err, d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  LV_CK(cudaStreamSynchronize(st));
  for (int32_t i = 0; i < np; ++i) {
    node_off[out[i]] = res[2 * (size_t)i];
    node_len[out[i]] = (int32_t)res[2 * (size_t)i + 1];
  }
  *pool_top = top;
  if (err) return fail(POYD_ERANGE, "traceback left the band (a median could not be built)");
  return POYD_OK;
}
