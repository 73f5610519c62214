// Host runtime: error reporting, per-device grow-only workspace, cost-table
// upload, and the batched / single-pair C entry points of the linear and
// affine DO path.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <tuple>
#include <vector>
#include "poyd_internal.h"
#include "linear_kernels.cuh"
#include "affine_kernels.cuh"

namespace poyd {

static thread_local char g_err[512] = "";

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(int err, const char *what) {
  return fail(POYD_ECUDA, "%s: %s", what, cudaGetErrorString((cudaError_t)err));
}

#define CK(call)                                          \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

struct Workspace {
  void *ptr[WS_NSLOTS] = {};
  size_t size[WS_NSLOTS] = {};
  poyd_cm last_cm;
  bool have_cm = false;
};

static std::mutex g_ws_mu;
static std::map<std::pair<int, cudaStream_t>, Workspace *> g_ws;

// One workspace per (device, stream): batches issued on different streams
// may be in flight together without sharing scratch.
Workspace *workspace(cudaStream_t st) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_ws_mu);
  Workspace *&w = g_ws[std::make_pair(dev, st)];
  if (!w) w = new Workspace();
  return w;
}

// Frees every cached buffer of the current device's workspaces (the grow-
// only scratch of all entry points); the next call allocates again.
extern "C" int poyd_workspace_release(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cuda_fail(cudaGetLastError(), "cudaGetDevice");
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceSynchronize");
  std::lock_guard<std::mutex> lk(g_ws_mu);
  for (auto &kv : g_ws) {
    if (kv.first.first != dev) continue;
    Workspace *w = kv.second;
    for (int k = 0; k < WS_NSLOTS; ++k) {
      if (w->ptr[k]) cudaFree(w->ptr[k]);
      w->ptr[k] = nullptr;
      w->size[k] = 0;
    }
    w->have_cm = false;
  }
  return POYD_OK;
}

void *ws_buffer(Workspace *w, int slot, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (w->size[slot] >= bytes) return w->ptr[slot];
  if (w->ptr[slot]) {
    cudaDeviceSynchronize();
    cudaFree(w->ptr[slot]);
    w->ptr[slot] = nullptr;
    w->size[slot] = 0;
  }
  size_t want = bytes + bytes / 4;
  void *p = nullptr;
  if (cudaMalloc(&p, want) != cudaSuccess) {
    cudaGetLastError();
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    want = bytes;
  }
  w->ptr[slot] = p;
  w->size[slot] = want;
  return p;
}

// Checks the matrix is one the GPU path implements: the combinations
// alphabet with lcm 5 and gap 16, tail[x] = cost[x][gap] and
// prepend[x] = cost[gap][x] (fill_default_prepend_tail, cost_matrix.ml:397-403),
// which lets the kernels fold the first-row, first-column and last-column
// special cells (algn.c:548-620) into the ordinary cell rule.
static int check_cm(const poyd_cm *cm, int *maxc) {
  if (!cm) return fail(POYD_EINVAL, "null cost matrix");
  if (cm->lcm != 5 || cm->gap != 16 || !cm->combinations)
    return fail(POYD_EUNSUP, "only the 5-bit combinations alphabet (DNA with ambiguity codes) is supported");
  int mx = 0;
  for (int a = 1; a < 32; ++a) {
    if (cm->tail[a] != cm->cost[(a << 5) | 16] || cm->prepend[a] != cm->cost[(16 << 5) | a])
      return fail(POYD_EUNSUP, "tail/prepend costs differ from the gap column/row of the cost table");
    for (int b = 1; b < 32; ++b) {
      const int c = cm->cost[(a << 5) | b];
      if (c < 0) return fail(POYD_ERANGE, "negative transformation cost");
      mx = std::max(mx, c);
    }
  }
  if (mx >= 65536) return fail(POYD_ERANGE, "transformation costs must be below 65536");
  if (cm->cost_model == 1 && (cm->gap_open < 0 || cm->gap_open >= 65536))
    return fail(POYD_ERANGE, "gap opening cost out of range");
  *maxc = mx;
  return POYD_OK;
}

void longest_first(const std::vector<int64_t> &work, std::vector<int32_t> &order) {
  // a stable two-pass radix sort on a descending 24-bit key (work / 128),
  // linear in n
  const int32_t n = (int32_t)work.size();
  std::vector<int32_t> tmp((size_t)n);
  std::vector<uint32_t> key((size_t)n);
  order.assign((size_t)n, 0);
  for (int32_t i = 0; i < n; ++i) {
    const int64_t q = std::min<int64_t>(work[i] >> 7, (1 << 24) - 1);
    key[i] = (uint32_t)((1 << 24) - 1 - q);
    tmp[i] = i;
  }
  for (int pass = 0; pass < 2; ++pass) {
    const int sh = 12 * pass;
    std::vector<int32_t> cnt((1 << 12) + 1, 0);
    for (int32_t i = 0; i < n; ++i) ++cnt[((key[tmp[i]] >> sh) & 4095) + 1];
    for (int b = 0; b < (1 << 12); ++b) cnt[b + 1] += cnt[b];
    for (int32_t i = 0; i < n; ++i) order[cnt[(key[tmp[i]] >> sh) & 4095]++] = tmp[i];
    if (pass == 0) std::swap(order, tmp);
  }
}

int upload_tables(const poyd_cm *cm, DevTables **dev, void *stream) {
  return upload_tables_ws(workspace((cudaStream_t)stream), cm, dev, stream);
}

int upload_tables_ws(Workspace *w, const poyd_cm *cm, DevTables **dev, void *stream) {
  DevTables *d = (DevTables *)ws_buffer(w, WS_TABLES, sizeof(DevTables));
  if (!d) return fail(POYD_ENOMEM, "table allocation failed");
  if (!w->have_cm || std::memcmp(&w->last_cm, cm, sizeof(poyd_cm)) != 0) {
    static thread_local DevTables h;
    for (int a = 0; a < 32; ++a)
      for (int b = 0; b < 32; ++b)
        h.packed[(a << 5) | b] = (uint32_t)(cm->cost[(a << 5) | b] & 0xffff) |
                                 ((uint32_t)(cm->cost[(16 << 5) | b] & 0xffff) << 16);
    std::memcpy(h.median, cm->median, sizeof(h.median));
    std::memcpy(h.cost, cm->cost, sizeof(h.cost));
    std::memcpy(h.worst, cm->worst, sizeof(h.worst));
    CK(cudaMemcpyAsync(d, &h, sizeof(DevTables), cudaMemcpyHostToDevice, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    w->last_cm = *cm;
    w->have_cm = true;
  }
  *dev = d;
  return POYD_OK;
}

// Shared driver of poyd_cost_2_batch (want_align = false) and
// poyd_align_2_batch (want_align = true) for the linear model.
constexpr int kTuneMax = 8;  // variants timed per batch (poyd_tune_result)

// ---------------------------------------------------------------------------
// Autotuner (no counterpart in the reference, whose C code has one kernel per
// operation).  The batched linear DP has several implementations that give
// identical results: the packed kernel (k_lin_dp4, when the plan finds every
// value fits 16 bits) or the 32-bit one (k_lin_dp), a persistent grid of 1 to
// the kernel's maximum resident blocks per SM, and, for batches with a warp
// per pair, the whole-warp small-batch walk or the batched one.  Which is
// fastest depends on the batch's shape; poyd_autotune_batch times each on a
// caller's batch and records the winner for the batch's shape class (device,
// mode, log2 of the pair count, log2 of the widest band), and every later
// batch of that class launches it.  Without an entry the defaults apply
// (packed when eligible, the maximum resident grid, the solo walk when
// every pair has its own warp).  The band itself is always the reference's.
// ---------------------------------------------------------------------------
struct LinVariant {
  int packed;         // 1 packed when eligible, 0 the 32-bit kernel, -1 default
  int blocks_per_sm;  // 0: the maximum resident
  int solo;           // 1 / 0 small-batch walk on / off, -1 default
};
using TuneKey = std::tuple<int, int, int, int>;  // device, align, lg pairs, lg width
static std::mutex g_tune_mu;
static std::map<TuneKey, LinVariant> g_tune;
static thread_local const LinVariant *g_force = nullptr;  // set while tuning
static thread_local TuneKey g_last_key{-1, -1, -1, -1};  // class of the last batch
static thread_local bool g_last_eligible = false;         // ... packed-eligible

static int ilog2_64(int64_t x) {
  int r = 0;
  while (x > 1) {
    x >>= 1;
    ++r;
  }
  return r;
}

static int linear_batch(Workspace *w, const poyd_cm *cm, int maxc, int32_t n, const uint8_t *seq,
                        const int64_t *a_off, const int32_t *a_len, const int64_t *b_off,
                        const int32_t *b_len, int32_t policy, const int32_t *deltaw,
                        int32_t *cost, int64_t *cells, bool want_align, int32_t flags,
                        uint8_t *out, const int64_t *out_off, int32_t *out_len,
                        cudaStream_t st, LinStream *ls = nullptr) {
  DevTables *tabs = nullptr;
  int rc = upload_tables_ws(w, cm, &tabs, st);
  if (rc) return rc;
  LinPlan *plans = (LinPlan *)ws_buffer(w, WS_PLANS, sizeof(LinPlan) * (size_t)n);
  int64_t *dmw = (int64_t *)ws_buffer(w, WS_DMWORDS, sizeof(int64_t) * 2 * (size_t)n);
  int32_t *wdb = (int32_t *)ws_buffer(w, WS_WD, sizeof(int32_t) * 2 * (size_t)n + 16);
  LinOrderScratch *os = (LinOrderScratch *)ws_buffer(w, WS_ORDSCR, sizeof(LinOrderScratch));
  int32_t *dord = (int32_t *)ws_buffer(w, WS_ORDER, sizeof(int32_t) * (size_t)n);
  int *counter = (int *)ws_buffer(w, WS_COUNTER, 64);
  if (!plans || !dmw || !wdb || !os || !dord || !counter)
    return fail(POYD_ENOMEM, "plan allocation failed");
  int32_t *err = &os->pad;  // the plan's error bits travel with the order totals
  CK(cudaMemsetAsync(os, 0, sizeof(LinOrderScratch), st));
  LinPlanArgs PA;
  PA.n = n; PA.seq = seq; PA.a_off = a_off; PA.a_len = a_len; PA.b_off = b_off; PA.b_len = b_len;
  PA.policy = policy; PA.deltaw = deltaw; PA.gap = cm->gap; PA.maxc = maxc;
  // The batched align_2 knows backtrack_2d's priority before the fill and
  // keeps only the chosen moves (values x4 must fit the 16-bit profile); the
  // single-pair protocol (out == nullptr) keeps the full direction sets.
  const int mode = !want_align ? kDpCost : ((out && maxc < 16384) ? kDpChoice : kDpSets);
  PA.with_dm = mode; PA.dos_empty = (flags & POYD_FLAG_DOS_EMPTY) ? 1 : 0;
  PA.plans = plans; PA.dm_words = dmw; PA.wd_out = wdb; PA.cells = cells; PA.err = err;
  { ProfScope ps("lin_plan", st); launch_lin_plan(PA, st); }
  CK(cudaGetLastError());

  // Pair order (longest first by log2 buckets) and direction-matrix
  // offsets on the device; one small read-back brings the plan's error bits,
  // the widest band and the direction-matrix size.
  int64_t *doff = dmw + n;
  // Batched align_2 with backtrack moves: the traceback runs inside the DP
  // kernel, batch by batch as their fills complete.
  const bool fuse = want_align && out && mode == kDpChoice;
  const int nbatch = (int)(((int64_t)n + kLanes - 1) / kLanes);
  int *batch_done = nullptr;
  if (fuse) {
    batch_done = (int *)ws_buffer(w, WS_BATCH, sizeof(int) * (size_t)nbatch);
    if (!batch_done) return fail(POYD_ENOMEM, "batch counter allocation failed");
  }
  // small batches take pairs in id order (the kernel also zeroes the DP's
  // counters); the others the bucketed longest-first order
  const bool small = n <= kOrderSmall && !ls;
  {
    ProfScope ps("lin_order", st);
    if (small) launch_lin_order_small(n, plans, dmw, doff, os, counter, batch_done, nbatch, st);
    else launch_lin_order(n, plans, dmw, doff, os, dord, st);
  }
  CK(cudaGetLastError());
  struct {
    unsigned long long total;
    int maxwd, err;
  } tl;
  static_assert(sizeof(tl) == 16, "order read-back");
  CK(cudaMemcpyAsync(&tl, &os->total, sizeof tl, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (tl.err & 1) return fail(POYD_EINVAL, "sequences must have length >= 1 (the leading gap)");
  if (tl.err & 2) return fail(POYD_ERANGE, "alignment costs could exceed the 2^24 range of the kernels");
  if (tl.err & 4) return fail(POYD_EINVAL, "sequence codes must be below 32 (5-bit element masks)");
  const int maxwd = std::max(1, tl.maxwd);
  const int64_t need = want_align ? (int64_t)tl.total : 0;
  // Waves: consecutive runs of a longest-first order whose direction
  // matrices fit the device-memory budget, one persistent launch each; one
  // wave, with the device order, when the whole batch fits (the usual
  // case).  The single-pair protocol (out == nullptr) keeps its one matrix
  // for the later backtrack.
  int64_t budget = INT64_MAX;
  if (want_align && out) {
    if (const char *e = std::getenv("POYD_DM_BUDGET_BYTES")) {
      budget = std::max<int64_t>(std::atoll(e) / 4, 1);
    } else if ((size_t)need * 4 > w->size[WS_DM]) {
      size_t freeb = 0, totb = 0;
      cudaMemGetInfo(&freeb, &totb);
      budget = std::max<int64_t>((int64_t)((double)(freeb + w->size[WS_DM]) * 0.8) / 4, 1);
    }
  }
  const bool host_waves = need > budget;
  std::vector<int32_t> order;
  std::vector<int64_t> hw;
  std::vector<int32_t> wave_at{0, n};
  int64_t max_words = std::max<int64_t>(need, 1);
  if (host_waves) {
    // too large for one launch: waves of a longest-first order built here
    hw.resize((size_t)n);
    CK(cudaMemcpyAsync(hw.data(), dmw, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    longest_first(hw, order);
    wave_at.assign(1, 0);
    int64_t wave_words = 0;
    max_words = 1;
    for (int32_t p = 0; p < n; ++p) {
      const int64_t x = hw[order[p]];
      if (p > wave_at.back() && wave_words + x > budget) {
        wave_at.push_back(p);
        wave_words = 0;
      }
      wave_words += x;
      max_words = std::max(max_words, wave_words);
    }
    wave_at.push_back(n);
    CK(cudaMemcpyAsync(dord, order.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, st));
  } else if (ls) {
    order.resize((size_t)n);
    CK(cudaMemcpyAsync(order.data(), dord, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  if (ls) {  // output slots in DP order
    int64_t o = 0;
    for (int32_t p = 0; p < n; ++p) {
      const int32_t id = order[p];
      ls->out_off_host[id] = o;
      o += 4 * slot_cap(ls->a_len_h[id], ls->b_len_h[id]);
    }
    CK(cudaMemcpyAsync(ls->out_off_dev, ls->out_off_host, sizeof(int64_t) * (size_t)n,
                       cudaMemcpyHostToDevice, st));
    out_off = ls->out_off_dev;
    ls->order = order;
    ls->waves = (int)wave_at.size() - 1;
  }
  uint32_t *dm = nullptr;
  if (want_align) {
    dm = (uint32_t *)ws_buffer(w, WS_DM, sizeof(uint32_t) * (size_t)max_words);
    if (!dm) return fail(POYD_ENOMEM, "direction matrix allocation (%lld bytes) failed",
                         (long long)(max_words * 4));
  }
  // The packed kernel (four rows per lane in 16-bit halves) runs the batch
  // when the plan found every pair's values to fit (no err bit 16);
  // POYD_PACKED=0 keeps the 32-bit kernel.
  bool packed = !(tl.err & 16) && mode != kDpSets;
  if (const char *e = std::getenv("POYD_PACKED")) packed = packed && std::atoi(e) != 0;
  // the launch variant of this batch's shape class (autotuner)
  LinVariant var{-1, 0, -1};
  {
    int dev = 0;
    cudaGetDevice(&dev);
    g_last_key = TuneKey(dev, mode == kDpChoice ? 1 : 0, ilog2_64(n), ilog2_64(maxwd));
    g_last_eligible = packed;
    if (g_force) {
      var = *g_force;
    } else if (mode != kDpSets) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tune.find(g_last_key);
      if (it != g_tune.end()) var = it->second;
    }
  }
  if (var.packed == 0) packed = false;
  int blocks = packed ? lin_dp4_blocks(mode) : lin_dp_blocks(mode);
  if (var.blocks_per_sm > 0) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    blocks = std::min(blocks, var.blocks_per_sm * std::max(sms, 1));
  }
  const int warps = packed ? lin_dp4_warps() : kDpWarps;
  const int64_t slab = maxwd + 64;
  int *scratch = (int *)ws_buffer(w, WS_SCRATCH, sizeof(int) * (size_t)slab * (size_t)blocks * warps);
  if (!scratch) return fail(POYD_ENOMEM, "scratch allocation failed");
  std::vector<int64_t> off(host_waves ? (size_t)n : 0, 0);
  for (size_t v = 0; v + 1 < wave_at.size(); ++v) {
    const int32_t p0 = wave_at[v], p1 = wave_at[v + 1], m = p1 - p0;
    if (host_waves) {  // this wave's matrices from the start of the buffer
      int64_t total = 0;
      for (int32_t p = p0; p < p1; ++p) {
        off[order[p]] = total;
        total += hw[order[p]];
      }
      CK(cudaMemcpyAsync(doff, off.data(), sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice, st));
    }
    const bool id_order = small && !host_waves;  // k_order_small zeroed the counters
    if (!id_order) {
      CK(cudaMemsetAsync(counter, 0, 4, st));
      if (fuse) CK(cudaMemsetAsync(batch_done, 0, sizeof(int) * (((size_t)m + kLanes - 1) / kLanes), st));
    }
    LinTbArgs TA;
    TA.n = m; TA.seq = seq; TA.plans = plans; TA.dm_off = doff; TA.dm = dm; TA.tables = tabs;
    TA.gap = cm->gap; TA.out = out; TA.out_off = out_off; TA.out_len = out_len;
    TA.swaped = -1; TA.mode = mode; TA.order = id_order ? nullptr : dord + p0;
    LinDpArgs DA;
    DA.n = m; DA.seq = seq; DA.plans = plans; DA.dm_off = doff; DA.order = id_order ? nullptr : dord + p0;
    DA.tables = tabs; DA.gap = cm->gap; DA.counter = counter; DA.scratch = scratch;
    DA.slab = slab; DA.dm = dm; DA.cost = cost; DA.swaped = -1;
    DA.fuse_tb = fuse ? 1 : 0; DA.batch_done = batch_done; DA.tb = TA; DA.k = dp_constants();
    DA.done = (ls && fuse && wave_at.size() == 2) ? ls->done : nullptr;
    DA.tb_solo = (fuse && packed && !DA.done && (int64_t)m <= (int64_t)blocks * warps &&
                  var.solo != 0) ? 1 : 0;
    {
      ProfScope ps(want_align ? "lin_dp_dm" : "lin_dp_cost", st);
      if (packed) launch_lin_dp4(DA, mode, blocks, st);
      else launch_lin_dp(DA, mode, blocks, st);
    }
    CK(cudaGetLastError());
    if (want_align && out && !fuse) {
      { ProfScope ps("lin_traceback", st); launch_lin_traceback(TA, st); }
      CK(cudaGetLastError());
    }
  }
  return POYD_OK;
}

}  // namespace poyd

using namespace poyd;

extern "C" const char *poyd_last_error(void) { return g_err; }

extern "C" int poyd_pack_alignments(int32_t n, const uint8_t *out, const int64_t *out_off,
                                    const int32_t *a_len, const int32_t *b_len,
                                    const int32_t *out_len, uint8_t *packed,
                                    const int64_t *packed_off, void *stream) {
  if (n < 0 || (n > 0 && (!out || !out_off || !a_len || !b_len || !out_len || !packed ||
                          !packed_off)))
    return fail(POYD_EINVAL, "poyd_pack_alignments: null argument");
  if (n == 0) return POYD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  { ProfScope ps("pack_alignments", st); launch_pack_alignments(n, out, out_off, a_len, b_len, out_len, packed, packed_off, st); }
  CK(cudaGetLastError());
  return POYD_OK;
}
extern "C" int poyd_version(void) { return 1; }

extern "C" int poyd_cost_2_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                                 const int64_t *a_off, const int32_t *a_len,
                                 const int64_t *b_off, const int32_t *b_len,
                                 int32_t deltaw_policy, const int32_t *deltaw, int32_t *cost,
                                 int64_t *band_cells, void *stream) {
  int maxc = 0;
  int rc = check_cm(cm, &maxc);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!seq || !a_off || !a_len || !b_off || !b_len || !cost)))
    return fail(POYD_EINVAL, "poyd_cost_2_batch: null argument");
  if (deltaw_policy == POYD_DELTAW_EXPLICIT && !deltaw)
    return fail(POYD_EINVAL, "explicit deltaw policy needs the deltaw array");
  if (n == 0) return POYD_OK;
  if (cm->cost_model == 1)
    return affine_batch(cm, maxc, n, seq, a_off, a_len, b_off, b_len, cost, band_cells, false,
                        0, nullptr, nullptr, nullptr, (cudaStream_t)stream);
  return linear_batch(workspace((cudaStream_t)stream), cm, maxc, n, seq, a_off, a_len, b_off, b_len, deltaw_policy, deltaw, cost,
                      band_cells, false, 0, nullptr, nullptr, nullptr, (cudaStream_t)stream);
}

extern "C" int poyd_align_2_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                                  const int64_t *a_off, const int32_t *a_len,
                                  const int64_t *b_off, const int32_t *b_len, int32_t *cost,
                                  uint8_t *out, const int64_t *out_off, int32_t *out_len,
                                  int64_t *band_cells, int32_t flags, void *stream) {
  int maxc = 0;
  int rc = check_cm(cm, &maxc);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!seq || !a_off || !a_len || !b_off || !b_len || !cost || !out ||
                          !out_off || !out_len)))
    return fail(POYD_EINVAL, "poyd_align_2_batch: null argument");
  if (n == 0) return POYD_OK;
  if (cm->cost_model == 1)
    return affine_batch(cm, maxc, n, seq, a_off, a_len, b_off, b_len, cost, band_cells, true,
                        flags, out, out_off, out_len, (cudaStream_t)stream);
  return linear_batch(workspace((cudaStream_t)stream), cm, maxc, n, seq, a_off, a_len, b_off, b_len, POYD_DELTAW_DEFAULT,
                      nullptr, cost, band_cells, true, flags, out, out_off, out_len,
                      (cudaStream_t)stream);
}

int poyd::align_2_streamed(const poyd_cm *cm, int32_t n, const uint8_t *seq, const int64_t *a_off,
                     const int32_t *a_len, const int64_t *b_off, const int32_t *b_len,
                     int32_t *cost, uint8_t *out, int32_t *out_len, int32_t flags,
                     LinStream *ls, cudaStream_t st) {
  int maxc = 0;
  int rc = check_cm(cm, &maxc);
  if (rc) return rc;
  if (cm->cost_model == 1) return fail(POYD_EUNSUP, "streamed align_2: linear model only");
  return linear_batch(workspace(st), cm, maxc, n, seq, a_off, a_len, b_off, b_len,
                      POYD_DELTAW_DEFAULT, nullptr, cost, nullptr, true, flags, out, nullptr,
                      out_len, st, ls);
}

// ---------------------------------------------------------------------------
// Single-pair drop-ins.  A poyd_matrix owns its own workspace so that the
// direction matrix of algn_CAML_simple_2 survives until the matching
// algn_CAML_backtrack_2d, as Matrix.m does (algn.c:3908-3924).
// ---------------------------------------------------------------------------
struct poyd_matrix {
  Workspace ws;
  int32_t l1 = -1, l2 = -1;  // pair whose DM is held
  cudaStream_t st = nullptr;
};

extern "C" poyd_matrix *poyd_matrix_create(void) { return new poyd_matrix(); }

extern "C" void poyd_matrix_free(poyd_matrix *m) {
  if (!m) return;
  for (int s = 0; s < WS_NSLOTS; ++s)
    if (m->ws.ptr[s]) cudaFree(m->ws.ptr[s]);
  delete m;
}

// Copies one pair (a, b) to the device and lays out its batch-of-one
// metadata: seq, a_off, a_len, b_off, b_len, deltaw, cost.
struct OnePair {
  uint8_t *seq;
  int64_t *off;
  int32_t *len;
  int32_t *dw;
  int32_t *cost;
};

static int stage_pair(Workspace *w, const uint8_t *a, int32_t la, const uint8_t *b, int32_t lb,
                      int32_t deltaw, OnePair *P, cudaStream_t st) {
  uint8_t *seq = (uint8_t *)ws_buffer(w, WS_SEQ, (size_t)la + lb + 64);
  unsigned char *meta = (unsigned char *)ws_buffer(w, WS_META, 256);
  if (!seq || !meta) return fail(POYD_ENOMEM, "pair staging allocation failed");
  struct {
    int64_t off[2];
    int32_t len[2];
    int32_t dw;
    int32_t cost;
  } h = {{0, la}, {la, lb}, deltaw, 0};
  CK(cudaMemcpyAsync(seq, a, (size_t)la, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(seq + la, b, (size_t)lb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(meta, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  P->seq = seq;
  P->off = (int64_t *)meta;
  P->len = (int32_t *)(meta + 16);
  P->dw = (int32_t *)(meta + 24);
  P->cost = (int32_t *)(meta + 28);
  return POYD_OK;
}

extern "C" int poyd_algn_simple_2(const uint8_t *s1, int32_t l1, const uint8_t *s2, int32_t l2,
                                  const poyd_cm *cm, poyd_matrix *mat, int32_t deltawh,
                                  int32_t *cost) {
  int maxc = 0;
  int rc = check_cm(cm, &maxc);
  if (rc) return rc;
  if (!s1 || !s2 || !mat || !cost) return fail(POYD_EINVAL, "poyd_algn_simple_2: null argument");
  if (l2 < 1 || l1 < l2) return fail(POYD_EINVAL, "algn_CAML_simple_2 needs len(s1) >= len(s2) >= 1");
  if (cm->cost_model != 0) return fail(POYD_EINVAL, "algn_CAML_simple_2 is the linear model");
  OnePair P;
  rc = stage_pair(&mat->ws, s1, l1, s2, l2, deltawh, &P, mat->st);
  if (rc) return rc;
  // want_align without an output buffer: DP + direction matrix, kept in mat
  rc = linear_batch(&mat->ws, cm, maxc, 1, P.seq, P.off, P.len, P.off + 1, P.len + 1,
                    POYD_DELTAW_RAW, P.dw, P.cost, nullptr, true, 0, nullptr, nullptr, nullptr,
                    mat->st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(cost, P.cost, sizeof(int32_t), cudaMemcpyDeviceToHost, mat->st));
  CK(cudaStreamSynchronize(mat->st));
  mat->l1 = l1;
  mat->l2 = l2;
  return POYD_OK;
}

extern "C" int poyd_algn_backtrack_2d(const uint8_t *s1, int32_t l1, const uint8_t *s2,
                                      int32_t l2, uint8_t *s1p, uint8_t *s2p, int32_t cap,
                                      int32_t *len, poyd_matrix *mat, const poyd_cm *cm,
                                      int32_t swaped) {
  (void)s1;
  (void)s2;
  if (!mat || !s1p || !s2p || !len || !cm) return fail(POYD_EINVAL, "poyd_algn_backtrack_2d: null argument");
  if (mat->l1 != l1 || mat->l2 != l2)
    return fail(POYD_EINVAL, "backtrack_2d needs the direction matrix of the preceding simple_2 on this pair");
  Workspace *w = &mat->ws;
  DevTables *tabs = nullptr;
  int rc = upload_tables_ws(w, cm, &tabs, mat->st);
  if (rc) return rc;
  const int64_t slot = slot_cap(l1, l2);
  const size_t tail = ((size_t)4 * slot + 63) & ~(size_t)63;
  uint8_t *out = (uint8_t *)ws_buffer(w, WS_OUT, tail + 64);
  if (!out) return fail(POYD_ENOMEM, "backtrack output allocation failed");
  int32_t *olen = (int32_t *)(out + tail);
  int64_t *ooff = (int64_t *)(out + tail + 16);
  const int64_t zero = 0;
  CK(cudaMemcpyAsync(ooff, &zero, sizeof(zero), cudaMemcpyHostToDevice, mat->st));
  LinTbArgs TA;
  TA.n = 1;
  TA.seq = (const uint8_t *)w->ptr[WS_SEQ];
  TA.plans = (const LinPlan *)w->ptr[WS_PLANS];
  TA.dm_off = ((const int64_t *)w->ptr[WS_DMWORDS]) + 1;
  TA.dm = (const uint32_t *)w->ptr[WS_DM];
  TA.tables = tabs;
  TA.gap = cm->gap;
  TA.out = out;
  TA.out_off = ooff;
  TA.out_len = olen;
  TA.swaped = swaped ? 1 : 0;
  TA.mode = kDpSets;
  TA.order = nullptr;
  {
    ProfScope ps("lin_traceback", mat->st);
    launch_lin_traceback(TA, mat->st);
  }
  CK(cudaGetLastError());
  int32_t hl[2];
  CK(cudaMemcpyAsync(hl, olen, sizeof(hl), cudaMemcpyDeviceToHost, mat->st));
  CK(cudaStreamSynchronize(mat->st));
  if (hl[0] < 0) return fail(POYD_ERANGE, "traceback left the band");
  if (hl[0] > cap) return fail(POYD_ERANGE, "output capacity %d below the aligned length %d", cap, hl[0]);
  CK(cudaMemcpy(s1p + cap - hl[0], out + slot - hl[0], (size_t)hl[0], cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(s2p + cap - hl[0], out + 2 * slot - hl[0], (size_t)hl[0], cudaMemcpyDeviceToHost));
  *len = hl[0];
  return POYD_OK;
}

extern "C" int poyd_algn_align_2d(const uint8_t *s1, int32_t l1, const uint8_t *s2, int32_t l2,
                                  const poyd_cm *cm, poyd_matrix *mat, uint8_t *s1p,
                                  uint8_t *s2p, int32_t cap, int32_t *len, int32_t deltawh,
                                  int32_t swaped, int32_t *cost) {
  const int rc = poyd_algn_simple_2(s1, l1, s2, l2, cm, mat, deltawh, cost);
  if (rc) return rc;
  return poyd_algn_backtrack_2d(s1, l1, s2, l2, s1p, s2p, cap, len, mat, cm, swaped);
}

static int affine_one(const uint8_t *si, int32_t li, const uint8_t *sj, int32_t lj,
                      const poyd_cm *cm, bool align, uint8_t *resi, uint8_t *resj,
                      uint8_t *median, uint8_t *medianwg, int32_t cap, int32_t *lens,
                      int32_t *cost) {
  int maxc = 0;
  int rc = check_cm(cm, &maxc);
  if (rc) return rc;
  if (cm->cost_model != 1) return fail(POYD_EINVAL, "the affine entry points need an affine matrix");
  if (!si || !sj || !cost || li < 1 || lj < 1) return fail(POYD_EINVAL, "affine: bad pair");
  Workspace *w = workspace();
  cudaStream_t st = nullptr;
  OnePair P;
  rc = stage_pair(w, si, li, sj, lj, 0, &P, st);
  if (rc) return rc;
  const int64_t slot = slot_cap(li, lj);
  uint8_t *out = nullptr;
  int32_t *olen = nullptr;
  int64_t *ooff = nullptr;
  if (align) {
    if (cap < (int64_t)li + lj + 2) return fail(POYD_ERANGE, "output capacity below len(si) + len(sj) + 2");
    const size_t tail = ((size_t)4 * slot + 63) & ~(size_t)63;
    out = (uint8_t *)ws_buffer(w, WS_OUT, tail + 64);
    if (!out) return fail(POYD_ENOMEM, "affine output allocation failed");
    olen = (int32_t *)(out + tail);
    ooff = (int64_t *)(out + tail + 16);
    const int64_t zero = 0;
    CK(cudaMemcpyAsync(ooff, &zero, sizeof(zero), cudaMemcpyHostToDevice, st));
  }
  rc = affine_batch(cm, maxc, 1, P.seq, P.off, P.len, P.off + 1, P.len + 1, P.cost, nullptr,
                    align, 0, out, ooff, olen, st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(cost, P.cost, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (!align) return POYD_OK;
  int32_t hl[2];
  CK(cudaMemcpy(hl, olen, sizeof(hl), cudaMemcpyDeviceToHost));
  if (hl[0] < 0) return fail(POYD_ERANGE, "affine traceback left the band");
  // outputs right-aligned in buffers of capacity cap, like the reference's seq
  uint8_t *dst[4] = {resi, resj, medianwg, median};
  const int32_t ln[4] = {hl[0], hl[0], hl[0], hl[1]};
  for (int k = 0; k < 4; ++k)
    if (dst[k])
      CK(cudaMemcpy(dst[k] + cap - ln[k], out + (k + 1) * slot - ln[k], (size_t)ln[k],
                    cudaMemcpyDeviceToHost));
  if (lens) {
    lens[0] = hl[0];
    lens[1] = hl[1];
    lens[2] = hl[0];
  }
  return POYD_OK;
}

extern "C" int poyd_algn_cost_affine_3(const uint8_t *si, int32_t li, const uint8_t *sj,
                                       int32_t lj, const poyd_cm *cm, int32_t *cost) {
  return affine_one(si, li, sj, lj, cm, false, nullptr, nullptr, nullptr, nullptr, 0, nullptr,
                    cost);
}

extern "C" int poyd_algn_align_affine_3(const uint8_t *si, int32_t li, const uint8_t *sj,
                                        int32_t lj, const poyd_cm *cm, uint8_t *resi,
                                        uint8_t *resj, uint8_t *median, uint8_t *medianwg,
                                        int32_t cap, int32_t *lens, int32_t *cost) {
  return affine_one(si, li, sj, lj, cm, true, resi, resj, median, medianwg, cap, lens, cost);
}

// ---------------------------------------------------------------------------
// Autotuner entry points (see LinVariant above).
// ---------------------------------------------------------------------------
extern "C" int poyd_autotune_set(int32_t device, int32_t align, int32_t lg_pairs,
                                 int32_t lg_width, int32_t packed, int32_t blocks_per_sm,
                                 int32_t solo) {
  if (packed < -1 || packed > 1 || solo < -1 || solo > 1 || blocks_per_sm < 0)
    return fail(POYD_EINVAL, "autotune: packed and solo are -1, 0 or 1; blocks_per_sm >= 0");
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[TuneKey(device, align ? 1 : 0, lg_pairs, lg_width)] = LinVariant{packed, blocks_per_sm, solo};
  return POYD_OK;
}

extern "C" int poyd_autotune_get(int32_t device, int32_t align, int32_t lg_pairs,
                                 int32_t lg_width, int32_t *packed, int32_t *blocks_per_sm,
                                 int32_t *solo) {
  if (!packed || !blocks_per_sm || !solo) return fail(POYD_EINVAL, "autotune: null argument");
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(TuneKey(device, align ? 1 : 0, lg_pairs, lg_width));
  if (it == g_tune.end()) return 0;
  *packed = it->second.packed;
  *blocks_per_sm = it->second.blocks_per_sm;
  *solo = it->second.solo;
  return 1;
}

extern "C" int poyd_autotune_clear(void) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
  return POYD_OK;
}

namespace {
struct ForceGuard {  // the forced variant lasts for one scope only
  explicit ForceGuard(const LinVariant *v) { g_force = v; }
  ~ForceGuard() { g_force = nullptr; }
};
}  // namespace

extern "C" int poyd_autotune_batch(const poyd_cm *cm, int32_t align, int32_t n,
                                   const uint8_t *seq, const int64_t *a_off, const int32_t *a_len,
                                   const int64_t *b_off, const int32_t *b_len,
                                   int32_t deltaw_policy, int32_t *cost, uint8_t *out,
                                   const int64_t *out_off, int32_t *out_len, int32_t flags,
                                   int32_t reps, poyd_tune_result *res, void *stream) {
  int maxc = 0;
  int rc = check_cm(cm, &maxc);
  if (rc) return rc;
  if (cm->cost_model != 0) return fail(POYD_EUNSUP, "autotune: linear model only");
  if (n <= 0 || !seq || !a_off || !a_len || !b_off || !b_len || !cost || !res ||
      (align && (!out || !out_off || !out_len)))
    return fail(POYD_EINVAL, "poyd_autotune_batch: null argument or empty batch");
  if (deltaw_policy == POYD_DELTAW_EXPLICIT || deltaw_policy == POYD_DELTAW_RAW)
    return fail(POYD_EINVAL, "autotune: deltaw policies with a per-pair array are not tuned");
  cudaStream_t st = (cudaStream_t)stream;
  auto run = [&]() -> int {
    return align ? poyd_align_2_batch(cm, n, seq, a_off, a_len, b_off, b_len, cost, out, out_off,
                                      out_len, nullptr, flags, stream)
                 : poyd_cost_2_batch(cm, n, seq, a_off, a_len, b_off, b_len, deltaw_policy,
                                     nullptr, cost, nullptr, stream);
  };
  // the defaults first: the batch's class, and the results every variant
  // must reproduce
  const LinVariant dflt{-1, 0, -1};
  {
    ForceGuard g(&dflt);
    rc = run();
  }
  if (rc) return rc;
  const TuneKey key = g_last_key;
  const bool eligible = g_last_eligible;
  std::vector<int32_t> ref_cost((size_t)n), ref_len(align ? 2 * (size_t)n : 0), chk;
  CK(cudaMemcpyAsync(ref_cost.data(), cost, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, st));
  if (align)
    CK(cudaMemcpyAsync(ref_len.data(), out_len, sizeof(int32_t) * 2 * (size_t)n,
                       cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  sms = std::max(sms, 1);
  const int mode = align ? kDpChoice : kDpCost;
  std::vector<LinVariant> cands;
  for (int pk = eligible ? 1 : 0; pk >= 0; --pk) {
    const int maxb = (pk ? lin_dp4_blocks(mode) : lin_dp_blocks(mode)) / sms;
    for (int b = std::max(maxb, 1); b >= 1 && (int)cands.size() < kTuneMax; --b) {
      const bool small = align && pk && (int64_t)n <= (int64_t)b * sms * lin_dp4_warps();
      cands.push_back(LinVariant{pk, b, small ? 1 : -1});
      if (small && (int)cands.size() < kTuneMax) cands.push_back(LinVariant{pk, b, 0});
    }
  }
  reps = std::max(reps, 1);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int best = -1;
  float best_ms = 0.f;
  res->n_variants = (int32_t)cands.size();
  for (size_t c = 0; c < cands.size(); ++c) {
    ForceGuard g(&cands[c]);
    rc = run();  // warm-up, and the result check below
    if (!rc) {
      CK(cudaEventRecord(e0, st));
      for (int r = 0; r < reps && !rc; ++r) rc = run();
      CK(cudaEventRecord(e1, st));
    }
    if (rc) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    ms /= (float)reps;
    chk.resize((size_t)n);
    CK(cudaMemcpy(chk.data(), cost, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost));
    bool same = chk == ref_cost;
    if (same && align) {
      chk.resize(2 * (size_t)n);
      CK(cudaMemcpy(chk.data(), out_len, sizeof(int32_t) * 2 * (size_t)n, cudaMemcpyDeviceToHost));
      same = chk == ref_len;
    }
    if (!same) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return fail(POYD_ERANGE, "autotune: variant %d (packed %d, %d blocks per SM, solo %d) "
                  "changed the results", (int)c, cands[c].packed, cands[c].blocks_per_sm,
                  cands[c].solo);
    }
    res->ms[c] = ms;
    res->variant[c][0] = cands[c].packed;
    res->variant[c][1] = cands[c].blocks_per_sm;
    res->variant[c][2] = cands[c].solo;
    if (best < 0 || ms < best_ms) {
      best = (int)c;
      best_ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = cands[(size_t)best];
  }
  res->packed = cands[(size_t)best].packed;
  res->blocks_per_sm = cands[(size_t)best].blocks_per_sm;
  res->solo = cands[(size_t)best].solo;
  res->lg_pairs = std::get<2>(key);
  res->lg_width = std::get<3>(key);
  return POYD_OK;
}
