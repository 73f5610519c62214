// Argument blocks and launchers of the linear-gap kernels (linear.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "poyd_internal.h"

namespace poyd {

struct LinPlanArgs {
  int n;
  const uint8_t *seq;
  const int64_t *a_off;
  const int32_t *a_len;
  const int64_t *b_off;
  const int32_t *b_len;
  int policy;
  const int32_t *deltaw;
  int gap;
  int maxc;
  int with_dm;  // kDpCost, kDpSets or kDpChoice: sizes the direction matrix
  int dos_empty;
  LinPlan *plans;
  int64_t *dm_words;
  int32_t *wd_out;
  int64_t *cells;
  int32_t *err;
};

struct LinTbArgs {
  int n;
  const uint8_t *seq;
  const LinPlan *plans;
  const int64_t *dm_off;
  const uint32_t *dm;
  const DevTables *tables;
  int gap;
  uint8_t *out;
  const int64_t *out_off;
  int32_t *out_len;
  int swaped;  // -1: derive from the orientation, else backtrack_2d's flag
  int mode;    // kDpSets or kDpChoice: how the direction matrix was written
  const int32_t *order;  // k_lin_traceback: thread t walks pair order[t] (nullable)
};

// Runtime multipliers of the DP's multiply-add arithmetic (see linear.cu).
struct DpK {
  int one, m1, four, m64k;
};
inline DpK dp_constants() { return DpK{1, -1, 4, -65536}; }

struct LinDpArgs {
  int n;
  const uint8_t *seq;
  const LinPlan *plans;
  const int64_t *dm_off;
  const int32_t *order;
  const DevTables *tables;
  int gap;
  int *counter;
  int *scratch;   // per-warp boundary-row slabs
  int64_t slab;   // ints per slab
  uint32_t *dm;
  int32_t *cost;
  int swaped;  // kDpChoice priority: -1 derives it from the orientation
  // kDpChoice with fuse_tb: the warp finishing the last DP of 32 consecutive
  // pairs (order positions 32b..32b+31, counted in batch_done[b]) runs their
  // traceback with `tb`
  int fuse_tb;
  int *batch_done;
  // with fuse_tb: done[b] = 1 once batch b's results are written (host-mapped
  // memory a caller polls to download finished slots early; may be null)
  int *done;
  // with fuse_tb, packed kernel: every pair has its own warp (n <= warps of
  // the grid) and no done flags are kept, so the warp that filled a pair
  // walks it at once, all lanes together (latency of small batches)
  int tb_solo;
  LinTbArgs tb;
  DpK k;  // multiplier constants (1, -1, 4, -65536)
};

// Device-side pair order and direction-matrix offsets (one launch wave):
// pairs are bucketed by log2 of their lane-steps (32 buckets per octave,
// longest first) and given disjoint direction-matrix regions.
struct LinOrderScratch {
  int hist[1024];           // pairs per bucket, then the scatter cursors
  int base[1024];           // first order position of each bucket
  unsigned long long total; // direction-matrix words of the batch
  int maxwd;                // widest band
  int pad;
};
void launch_lin_order(int n, const LinPlan *plans, const int64_t *dm_words, int64_t *dm_off,
                      LinOrderScratch *os, int32_t *order, cudaStream_t st);
constexpr int kOrderSmall = 1024;  // batches up to this size use k_order_small
void launch_lin_order_small(int n, const LinPlan *plans, const int64_t *dm_words,
                            int64_t *dm_off, LinOrderScratch *os, int *counter, int *batch_done,
                            int nbatch, cudaStream_t st);

void launch_lin_plan(const LinPlanArgs &A, cudaStream_t st);
int lin_dp_blocks(int mode);
void launch_lin_dp(const LinDpArgs &A, int mode, int blocks, cudaStream_t st);
// Packed DP (linear4.cu): four rows per lane in 16-bit halves, kDpCost or
// kDpChoice, for batches the plan marks eligible (no err bit 16).
int lin_dp4_blocks(int mode);
int lin_dp4_warps();
void launch_lin_dp4(const LinDpArgs &A, int mode, int blocks, cudaStream_t st);
void launch_lin_traceback(const LinTbArgs &A, cudaStream_t st);
void launch_pack_alignments(int n, const uint8_t *out, const int64_t *out_off,
                            const int32_t *a_len, const int32_t *b_len,
                            const int32_t *out_len, uint8_t *packed,
                            const int64_t *packed_off, cudaStream_t st);

}  // namespace poyd
