// poyd_cost_2_batch_noalloc: the batched linear cost_2 for callers that
// cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at all: an OCaml servant whose C stub
// runs inside a host that owns the CUDA context and its memory pool, or a
// process with a fixed device-memory budget that forbids growth after
// start-up.  For them this entry point runs the same
// plan and band-DP kernels as poyd_cost_2_batch, but every scratch byte
// those kernels need -- per-pair plans, the launch counter and error
// flags, the staged cost tables and the per-warp boundary-row slabs --
// lives in one file-scope __device__ array of fixed size, which every GPU
// that loads this library keeps until the process exits.  The caller still
// provides the inputs and the cost output.
//
// Limits: at most kNaMaxPairs pairs per call and band widths up to
// kNaSlabInts - 64 diagonals; larger requests are refused with POYD_ERANGE
// before any DP kernel runs.  The array is shared by every call: calls
// that overlap on the GPU (different streams or host threads) race on it,
// so callers must serialise them.  The counter and error flags are
// cleared on every call; the rest is fully rewritten before it is read.
//
// The call waits for its stream once, to read the plan's error flags back
// before the DP launch; a stream that is being captured cannot be waited
// on, so such a stream is refused with POYD_EUNSUP before anything is
// enqueued.  The first call on each device looks up the array's device
// address with cudaGetSymbolAddress (the name of a __device__ variable is
// only a host-side handle, not a device pointer); make that first call
// outside any stream capture.
#include <cuda_runtime.h>
#include <cstring>
#include <mutex>
#include "poyd_internal.h"
#include "linear_kernels.cuh"

namespace poyd {
namespace {

constexpr int kNaMaxPairs = 65536;
constexpr int kNaSlabInts = 2048;   // per-warp boundary row: wd <= 1984
constexpr int kNaWarps = 2432;      // persistent warps (304 blocks of kDpWarps = 8)
constexpr size_t kNaHeader = 256;   // counter + error flags
constexpr size_t kNaTables = (sizeof(DevTables) + 255) / 256 * 256;
constexpr size_t kNaPlans = sizeof(LinPlan) * (size_t)kNaMaxPairs;
constexpr size_t kNaWords = sizeof(int64_t) * (size_t)kNaMaxPairs;
constexpr size_t kNaWd = sizeof(int32_t) * (size_t)kNaMaxPairs;
constexpr size_t kNaSlabs = sizeof(int) * (size_t)kNaSlabInts * (size_t)kNaWarps;
constexpr size_t kNaBytes = kNaHeader + kNaTables + kNaPlans + kNaWords + kNaWd + kNaSlabs;

// Fixed scratch of the no-allocation entry point (about 24 MiB).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

std::mutex g_na_mu;
unsigned char *g_na_ptr[64] = {};

// Device address of g_noalloc_scratch on the current device (looked up
// once per device).
int na_scratch(unsigned char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(POYD_EINVAL, "device index out of range");
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_na_ptr[dev] = (unsigned char *)p;
  }
  *out = g_na_ptr[dev];
  return POYD_OK;
}

// Rejects plans whose band would overflow a fixed per-warp slab.
__global__ void k_na_check(const int32_t *wd, int n, int limit, int32_t *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && wd[i] > limit) atomicOr(err, 8);
}

int na_check_cm(const poyd_cm *cm, int *maxc) {
  if (!cm) return fail(POYD_EINVAL, "null cost matrix");
  if (cm->lcm != 5 || cm->gap != 16 || !cm->combinations)
    return fail(POYD_EUNSUP, "only the 5-bit combinations alphabet is supported");
  if (cm->cost_model != 0)
    return fail(POYD_EUNSUP, "the no-allocation entry point implements the linear model only");
  int mx = 0;
  for (int a = 1; a < 32; ++a) {
    if (cm->tail[a] != cm->cost[(a << 5) | 16] || cm->prepend[a] != cm->cost[(16 << 5) | a])
      return fail(POYD_EUNSUP, "tail/prepend costs differ from the gap column/row");
    for (int b = 1; b < 32; ++b) {
      const int c = cm->cost[(a << 5) | b];
      if (c < 0 || c >= 65536) return fail(POYD_ERANGE, "transformation cost out of range");
      if (c > mx) mx = c;
    }
  }
  *maxc = mx;
  return POYD_OK;
}

#define NA_CK(call)                                       \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

}  // namespace
}  // namespace poyd

using namespace poyd;

extern "C" int poyd_cost_2_batch_noalloc(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                                         const int64_t *a_off, const int32_t *a_len,
                                         const int64_t *b_off, const int32_t *b_len,
                                         int32_t deltaw_policy, const int32_t *deltaw,
                                         int32_t *cost, void *stream) {
  int maxc = 0;
  int rc = na_check_cm(cm, &maxc);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!seq || !a_off || !a_len || !b_off || !b_len || !cost)))
    return fail(POYD_EINVAL, "poyd_cost_2_batch_noalloc: null argument");
  if (n > kNaMaxPairs)
    return fail(POYD_ERANGE, "poyd_cost_2_batch_noalloc: %d pairs exceed the fixed limit of %d",
                n, kNaMaxPairs);
  if (deltaw_policy == POYD_DELTAW_EXPLICIT && !deltaw)
    return fail(POYD_EINVAL, "explicit deltaw policy needs the deltaw array");
  if (n == 0) return POYD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  NA_CK(cudaStreamIsCapturing(st, &cap));
  if (cap != cudaStreamCaptureStatusNone)
    return fail(POYD_EUNSUP, "poyd_cost_2_batch_noalloc waits for its stream (error flags are "
                             "read back), which a stream under capture cannot do");
  unsigned char *base = nullptr;
  rc = na_scratch(&base);
  if (rc) return rc;
  int *counter = (int *)base;
  int32_t *err = (int32_t *)(base + 64);
  DevTables *tabs = (DevTables *)(base + kNaHeader);
  LinPlan *plans = (LinPlan *)(base + kNaHeader + kNaTables);
  int64_t *words = (int64_t *)((unsigned char *)plans + kNaPlans);
  int32_t *wd = (int32_t *)((unsigned char *)words + kNaWords);
  int *slabs = (int *)((unsigned char *)wd + kNaWd);

  // cost tables staged from a stack buffer (no allocation)
  DevTables h;
  for (int a = 0; a < 32; ++a)
    for (int b = 0; b < 32; ++b)
      h.packed[(a << 5) | b] = (uint32_t)(cm->cost[(a << 5) | b] & 0xffff) |
                               ((uint32_t)(cm->cost[(16 << 5) | b] & 0xffff) << 16);
  std::memcpy(h.median, cm->median, sizeof(h.median));
  std::memcpy(h.cost, cm->cost, sizeof(h.cost));
  std::memcpy(h.worst, cm->worst, sizeof(h.worst));
  NA_CK(cudaMemcpyAsync(tabs, &h, sizeof(DevTables), cudaMemcpyHostToDevice, st));
  NA_CK(cudaMemsetAsync(base, 0, kNaHeader, st));

  LinPlanArgs PA;
  PA.n = n; PA.seq = seq; PA.a_off = a_off; PA.a_len = a_len; PA.b_off = b_off; PA.b_len = b_len;
  PA.policy = deltaw_policy; PA.deltaw = deltaw; PA.gap = cm->gap; PA.maxc = maxc;
  PA.with_dm = 0; PA.dos_empty = 0;
  PA.plans = plans; PA.dm_words = words; PA.wd_out = wd; PA.cells = nullptr; PA.err = err;
  launch_lin_plan(PA, st);
  NA_CK(cudaGetLastError());
  k_na_check<<<(n + 255) / 256, 256, 0, st>>>(wd, n, kNaSlabInts - 64, err);
  NA_CK(cudaGetLastError());
  int32_t herr = 0;
  NA_CK(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
  if (herr & 1) return fail(POYD_EINVAL, "sequences must have length >= 1 (the leading gap)");
  if (herr & 2) return fail(POYD_ERANGE, "alignment costs could exceed the 2^24 range of the kernels");
  if (herr & 4) return fail(POYD_EINVAL, "sequence codes must be below 32 (5-bit element masks)");
  if (herr & 8)
    return fail(POYD_ERANGE, "a band is wider than the %d diagonals the fixed scratch holds",
                kNaSlabInts - 64);

  LinDpArgs DA;
  DA.n = n; DA.seq = seq; DA.plans = plans; DA.dm_off = nullptr; DA.order = nullptr;
  DA.tables = tabs; DA.gap = cm->gap; DA.counter = counter; DA.scratch = slabs;
  DA.slab = kNaSlabInts; DA.dm = nullptr; DA.cost = cost; DA.swaped = -1;
  DA.fuse_tb = 0; DA.batch_done = nullptr; DA.done = nullptr; DA.tb_solo = 0; DA.tb = LinTbArgs{};
  DA.k = dp_constants();
  launch_lin_dp(DA, kDpCost, kNaWarps / kDpWarps, st);
  NA_CK(cudaGetLastError());
  return POYD_OK;
}
