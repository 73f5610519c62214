// Internal declarations shared by the host runtime and the kernels.
#pragma once
#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>
#include <vector>
#include "poyd_gb300.h"

namespace poyd {

// Record a failure message (poyd_last_error) and return the code.
int fail(int code, const char *fmt, ...);
int cuda_fail(int err, const char *what);

// Cells outside the band hold this value; every real DP value must stay
// below kMaxCost so that kInf plus a cost never collides with one.
constexpr int kInf = 1 << 25;
constexpr int kMaxCost = 1 << 24;
constexpr int kLanes = 32;      // lanes per pair
constexpr int kRows = 64;       // rows per strip: two per lane
constexpr int kLag = 3;         // steps between consecutive lanes
constexpr int kStepBlock = 32;  // steps per queue block and per direction word
constexpr int kDpWarps = 8;     // warps per k_lin_dp block
constexpr int kMinPeriod = 160; // shortest strip period (boundary flush-to-prefetch distance)
// k_lin_dp modes: costs only; full direction sets; backtrack moves (values x4)
constexpr int kDpCost = 0, kDpSets = 1, kDpChoice = 2;
constexpr int kInfChoice = 3 << 25;  // out-of-band value of kDpChoice (x4 scale)
// direction-matrix words per (strip, 32-step block) of each mode
__host__ __device__ constexpr int lin_dm_words(int mode) {
  return mode == kDpSets ? 3 * kRows : (mode == kDpChoice ? 2 * kRows : 0);
}

// Capacity of each of the four right-aligned output sequences of a batched
// align_2 pair: la + lb + 2 (the longest alignment plus the leading gap),
// rounded up to a multiple of 4 so that every pair's outputs are word
// aligned alike (the tracebacks' word-buffered writers then flush in step
// across a warp).
__host__ __device__ inline int64_t slot_cap(int64_t la, int64_t lb) {
  return (la + lb + 2 + 3) & ~(int64_t)3;
}

// Streamed download of a batched linear align_2 (poyd_align_2_host): the
// output slots are laid out in the DP's longest-first order, so that the
// slots of finished batches form a growing prefix the caller downloads
// while the DP runs.
struct LinStream {
  const int32_t *a_len_h, *b_len_h;  // host copies of the lengths
  int64_t *out_off_host;             // out: slot offset of every pair
  int64_t *out_off_dev;              // device array receiving the same
  int *done;                         // device pointer to host-mapped batch flags
  std::vector<int32_t> order;        // out: the DP order
  int waves = 0;                     // out: launches (flags are set for one wave only)
};
int align_2_streamed(const poyd_cm *cm, int32_t n, const uint8_t *seq, const int64_t *a_off,
                     const int32_t *a_len, const int64_t *b_off, const int32_t *b_len,
                     int32_t *cost, uint8_t *out, int32_t *out_len, int32_t flags,
                     LinStream *ls, cudaStream_t st);

// Per-pair plan of the linear banded DP, produced on the device.
struct LinPlan {
  int64_t s1_off, s2_off;  // rows (longer) and columns sequences
  int64_t dm_off;          // 32-bit word offset of the direction matrix
  int32_t l1, l2;          // rows / columns lengths
  int32_t dlo, wd;         // band diagonals [dlo, dlo + wd)
  int32_t swap;            // 1: rows are the caller's b
  int32_t nstrips;         // ceil(l1 / 64)
  int32_t sblocks;         // strip period W in 32-step blocks
  int32_t deltaw;          // width extension used
  int32_t empty;           // DOS.median empty rule: 1 = a empty, 2 = b empty
  int32_t nblk;            // 32-step blocks of the whole sweep
};
static_assert(sizeof(LinPlan) == 64, "LinPlan layout");

// Packed cost table staged in shared memory: entry (a<<5)+b holds
// cost[a][b] in the low 16 bits and cost[gap][b] in the high 16 bits.
struct DevTables {
  uint32_t packed[1024];
  uint8_t median[1024];
  int32_t cost[1024];
  int32_t worst[1024];
};

struct Workspace;
Workspace *workspace(cudaStream_t st = nullptr);  // per (current device, stream)
// Grow-only device buffer `slot` of at least `bytes`; returns nullptr on failure.
void *ws_buffer(Workspace *w, int slot, size_t bytes);
enum WsSlot {
  WS_TABLES = 0, WS_PLANS, WS_DMWORDS, WS_WD, WS_ORDER, WS_DM, WS_SCRATCH,
  WS_COUNTER, WS_CELLS, WS_AFF, WS_ERR, WS_SEQ, WS_META, WS_OUT, WS_BATCH, WS_ORDSCR,
  WS_LVL_NODES, WS_LVL_PAIRS, WS_P3_RING, WS_P3_DIR, WS_P3_META, WS_P3_IO, WS_NSLOTS
};

int upload_tables(const poyd_cm *cm, DevTables **dev, void *stream);
// Pair order for the persistent DP kernels: largest work first (stable).
void longest_first(const std::vector<int64_t> &work, std::vector<int32_t> &order);
int upload_tables_ws(Workspace *w, const poyd_cm *cm, DevTables **dev, void *stream);

// Launch accounting (profile.cu): bracket one kernel launch on `st`.
void prof_begin(const char *name, cudaStream_t st, void **token);
void prof_end(void *token, cudaStream_t st);
struct ProfScope {
  void *tok;
  cudaStream_t st;
  ProfScope(const char *name, cudaStream_t s) : st(s) { prof_begin(name, s, &tok); }
  ~ProfScope() { prof_end(tok, st); }
};

// The rest of one level of the level engine after its DO alignments
// (fitch_sankoff.cu), in one launch: per pair, the Fitch and Sankoff medians
// of the input nodes' rows into the output node's rows and the placement of
// the DO median (the output node's place in the pool, the pair's costs).
struct LevelPost {
  int n;
  const int32_t *a, *b, *out;     // node ids of the level's pairs
  uint8_t *fitch;                 // Fitch rows (fitch_len 0: none)
  int64_t stride;
  int fitch_len;
  int32_t *sank;                  // Sankoff rows (nchar 0: none)
  int nchar, k;
  const int32_t *tcm;
  const int64_t *slot_off;        // the align_2 result slots
  const int32_t *a_len, *b_len, *out_len, *cost;
  int64_t *node_off;              // the device node table
  int32_t *node_len;
  int64_t *costs;                 // per pair: DO cost, Fitch cost
  int32_t *err;                   // bit 0: a failed traceback
};
int launch_level_post(const LevelPost &P, cudaStream_t st);

}  // namespace poyd
