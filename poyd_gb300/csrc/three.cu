// Three-sequence alignment of the Iterative (ThreeD) cost mode.
//
// Sequence.Align.readjust_3d (sequence.ml:1117-1140) re-estimates a node's
// median from its two children and its parent with align_3_powell_inter
// (sequence.ml:1089-1115), which aligns the three sequences with
// powell_3D_align (ukkCommon.c:111-143): Powell's three-way generalisation
// of Ukkonen's algorithm over 16 column states, with check-pointing
// (ukk.checkp.c).  Its cost is the optimum of a fixed cost model
// (alignmentCost, ukkCommon.c:345-391), which does not depend on how the
// optimum is searched.  Here each triple is one dynamic program over the
// full (la x lb x lc) cube and the 16 states, swept by hyperplanes
// h = i + j + k (a cell depends only on the three hyperplanes before it):
//   * one block per triple (a cluster of 2-8 blocks for small batches),
//     persistent over a largest-first queue; a warp takes a row (fixed i)
//     of the hyperplane, a lane one cell of it;
//   * a thread computes all 16 states of its cell: every state reads one
//     neighbour cell (the one its column consumes from), so a cell loads 7
//     neighbours of 16 values; values are stored x16 with a state number
//     in the low 4 bits, so that one add-min per (previous, next) state
//     pair keeps the least cost and, on ties, the lowest-numbered previous
//     state; by default two states per 32-bit word (16-bit halves), the
//     32-bit values as the fallback for large costs;
//   * the last four hyperplanes' values in a ring in global memory
//     ([h & 3][i][j][state]); the 16 choices of a cell (4 bits each) in
//     one 64-bit word of a per-triple cube laid out [i][j + k][j] so that
//     a hyperplane's cells of one i are contiguous;
//   * then one thread walks the choices back and writes the three aligned
//     rows and the column medians (Cost_matrix.Three_D.median) right-aligned
//     into the triple's slot.
// Among equally cheap alignments the walk keeps the lowest-numbered final
// state and at every column the lowest-numbered previous state; Powell's
// recursion may return another of the optimal alignments.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "poyd_internal.h"

#define CK3(call)                                         \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

namespace poyd {

constexpr int kP3States = 16;
constexpr int kP3Threads = 256;
constexpr int kP3Inf = 1 << 30;      // x16 domain
constexpr int kP3MaxLen = 4096;

// Powell's column states (ukkCommon.c:206-262): per sequence match (M),
// delete (D) or insert (I), at least one M and at most one I, numbered in
// increasing order of x0 + 3 x1 + 9 x2 (M 0, D 1, I 2), MMM first.  A
// state without I consumes a character of each M sequence; a state with I
// consumes one of the I sequence only.  ngo[s][t] counts the gap openings
// of a step from s to t (ukkCommon.c:263-290): the sequences in D or I in
// t that were not in that same state in s.
struct P3States {
  int code[kP3States], adv[kP3States], ins[kP3States], ndel[kP3States];
  int ngo[kP3States][kP3States];
};

__host__ __device__ constexpr P3States p3_states() {
  P3States S{};
  int n = 0;
  for (int c = 0; c < 27; ++c) {
    const int x0 = c % 3, x1 = c / 3 % 3, x2 = c / 9 % 3;
    const int nm = (x0 == 0) + (x1 == 0) + (x2 == 0);
    const int ni = (x0 == 2) + (x1 == 2) + (x2 == 2);
    if (nm == 0 || ni > 1) continue;
    S.code[n] = c;
    S.ins[n] = ni;
    S.ndel[n] = 3 - nm - ni;
    S.adv[n] = ni ? ((x0 == 2) | (x1 == 2) << 1 | (x2 == 2) << 2)
                  : ((x0 == 0) | (x1 == 0) << 1 | (x2 == 0) << 2);
    ++n;
  }
  for (int s = 0; s < kP3States; ++s)
    for (int t = 0; t < kP3States; ++t) {
      int k = 0, cs = S.code[s], ct = S.code[t];
      for (int q = 0; q < 3; ++q, cs /= 3, ct /= 3)
        if (ct % 3 != 0 && ct % 3 != cs % 3) ++k;
      S.ngo[s][t] = k;
    }
  return S;
}

// The same tables for indices known only at run time (traceback, table
// setup): constant memory rather than a local copy.
__constant__ P3States c_p3 = p3_states();

struct P3Args {
  int n, mode;            // mode 1: readjust_3d's early returns and changed flags
  const uint8_t *seq;
  const int64_t *off[4];  // a, b, c; m (mode 1)
  const int32_t *len[4];
  int32_t *cost;
  uint8_t *out;
  const int64_t *out_off;
  int32_t *out_len;
  int32_t *changed;
  const int32_t *order;
  int32_t *counter;
  int32_t *err;
  int32_t *ring;
  int64_t ring_stride;    // int32 per block
  uint64_t *dir;
  int64_t dir_stride;     // words per block
  int mm, go, ge, gap, has_med, smax;
  uint8_t med[128];       // Three_D.median of (x, y, z) over A C G T gap, 25 x + 5 y + z
};

// Offset of the (j + k = s) row in an i-slice of the choice cube:
// the sum over s' < s of the row lengths min(nb, s') - max(0, s' - nc) + 1.
__device__ __forceinline__ int64_t p3_soff(int s, int nb, int nc) {
  int64_t f;
  if (s <= nb + 1) f = (int64_t)s * (s + 1) / 2;
  else f = (int64_t)(nb + 1) * (nb + 2) / 2 + (int64_t)(s - nb - 1) * (nb + 1);
  if (s > nc + 1) {
    const int64_t m = s - nc - 1;
    f -= m * (m + 1) / 2;
  }
  return f;
}

__device__ __forceinline__ int p3_code(int x) {  // copySequence: lowest of A C G T
  return (x & 1) ? 1 : (x & 2) ? 2 : (x & 4) ? 4 : (x & 8) ? 8 : 0;
}
__device__ __forceinline__ int p3_ix(int x) { return __ffs(x) - 1; }  // 1 2 4 8 16 -> 0..4

// One cell (a, b, c) of hyperplane h: its 16 values (x16, into the ring)
// and its 64-bit choice word (returned).
__device__ __forceinline__ uint64_t p3_cell(int32_t *ring, int64_t pl, int nb, int h, int a,
                                            int b, int c, const int *g16, const int *col16) {
  constexpr P3States S = p3_states();
  int best[kP3States];
#pragma unroll
  for (int t = 0; t < kP3States; ++t) best[t] = kP3Inf;
#pragma unroll
  for (int d = 1; d < 8; ++d) {  // the neighbour cell one column of step d back
    const int da = d & 1, db = d >> 1 & 1, dc = d >> 2 & 1;
    if (a < da || b < db || c < dc) continue;
    const int hs = h - da - db - dc;
    const int4 *p = reinterpret_cast<const int4 *>(
        ring + ((int64_t)(hs & 3) * pl + (int64_t)(a - da) * (nb + 1) + (b - db)) * kP3States);
    int w[kP3States];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int4 u = p[q];
      w[4 * q] = u.x + 4 * q;  // the previous state in the low bits
      w[4 * q + 1] = u.y + 4 * q + 1;
      w[4 * q + 2] = u.z + 4 * q + 2;
      w[4 * q + 3] = u.w + 4 * q + 3;
    }
#pragma unroll
    for (int t = 0; t < kP3States; ++t) {
      if (S.adv[t] != d) continue;
#pragma unroll
      for (int s = 0; s < kP3States; ++s) best[t] = __viaddmin_s32(w[s], g16[S.ngo[s][t]], best[t]);
    }
  }
  int4 *o = reinterpret_cast<int4 *>(
      ring + ((int64_t)(h & 3) * pl + (int64_t)a * (nb + 1) + b) * kP3States);
  uint64_t word = 0;
  int v[kP3States];
#pragma unroll
  for (int t = 0; t < kP3States; ++t) {
    const bool fin = best[t] < kP3Inf;
    // an I column costs one extension; otherwise one per D plus the
    // mismatches of the matched characters
    const int col = S.ins[t] ? g16[4] : col16[S.adv[t]] + S.ndel[t] * g16[4];
    v[t] = fin ? (best[t] & ~15) + col : kP3Inf;
    word |= (uint64_t)(fin ? best[t] & 15 : 0) << (4 * t);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) o[q] = make_int4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  return word;
}

// The same cell with two values per 32-bit word, for batches whose costs
// stay small: x16 values in 16-bit halves of a uint16 ring, each value
// carrying its own state number in the low 4 bits, so that a value loaded
// as a previous state already holds its rank, and one __viaddmin_u16x2
// tries two previous states.  Infinity is 0xC000; every value is clamped
// to it and every addend stays below 0x4000, so no half wraps.  A value
// that reaches the clamp is not exact; a triple whose optimum reaches it is
// redone by the 32-bit cell (the cells of an optimal path never exceed the
// optimum, so a smaller optimum is exact).  Neighbours outside the cube
// are read from a constant infinite cell, so the 14 loads of a cell issue
// before any of its arithmetic.
constexpr unsigned kP3Inf2 = 0xC000C000u;
// min per half (measured: the fused add-min with a zero addend in its
// place executes 365 instructions per cell instead of 331; sharing one
// 16-way minimum among the next states of a step when go = 0 let the
// loads interleave with the arithmetic again and ran 1.5x slower)
__device__ __forceinline__ unsigned p3_min2(unsigned a, unsigned b) { return __vminu2(a, b); }
template <bool GO0, bool CL>
__device__ __forceinline__ uint64_t p3_cell16(const uint16_t *const *src, uint16_t *dst,
                                              const unsigned *gg, const uint4 ca,
                                              const uint4 cb) {
  constexpr P3States S = p3_states();
  uint4 u[7][2];
#pragma unroll
  for (int d = 0; d < 7; ++d) {
    const uint4 *p = reinterpret_cast<const uint4 *>(src[d]);
    // a cluster's blocks write each other's neighbours: read them from L2
    u[d][0] = CL ? __ldcg(p) : p[0];
    u[d][1] = CL ? __ldcg(p + 1) : p[1];
  }
  unsigned best[kP3States];
#pragma unroll
  for (int t = 0; t < kP3States; ++t) best[t] = kP3Inf2;
#pragma unroll
  for (int d = 1; d < 8; ++d) {
    const unsigned w[8] = {u[d - 1][0].x, u[d - 1][0].y, u[d - 1][0].z, u[d - 1][0].w,
                           u[d - 1][1].x, u[d - 1][1].y, u[d - 1][1].z, u[d - 1][1].w};
#pragma unroll
    for (int t = 0; t < kP3States; ++t) {
      if (S.adv[t] != d) continue;
#pragma unroll
      for (int q = 0; q < 8; ++q)
        best[t] = GO0 ? p3_min2(w[q], best[t])
                      : __viaddmin_u16x2(w[q], gg[4 * S.ngo[2 * q][t] + S.ngo[2 * q + 1][t]],
                                         best[t]);
    }
  }
  const unsigned col2[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
  uint64_t word = 0;
  unsigned v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {  // states 2k (low half) and 2k + 1 (high half)
    const unsigned lo = __byte_perm(best[2 * k], best[2 * k + 1], 0x5410);
    const unsigned hi = __byte_perm(best[2 * k], best[2 * k + 1], 0x7632);
    const unsigned m = p3_min2(lo, hi);
    const unsigned own = (unsigned)(2 * k) | (unsigned)(2 * k + 1) << 16;
    v[k] = p3_min2((m & 0xFFF0FFF0u) + col2[k], kP3Inf2 + own);
    word |= (uint64_t)(m & 15u) << (8 * k) | (uint64_t)(m >> 16 & 15u) << (8 * k + 4);
  }
  uint4 *o = reinterpret_cast<uint4 *>(dst);
  o[0] = make_uint4(v[0], v[1], v[2], v[3]);
  o[1] = make_uint4(v[4], v[5], v[6], v[7]);
  return word;
}

// Column costs of the packed cell (x16, each state's own number added):
// state pairs (2k, 2k + 1) for the characters x0, x1, x2 (0: none) of a
// cell; an entry whose state needs a missing character is never used.
__device__ __forceinline__ unsigned p3_col2(int k, int x0, int x1, int x2, int mm16, int ge16) {
  const P3States &S = c_p3;
  unsigned r = 0;
  for (int h = 0; h < 2; ++h) {
    const int t = 2 * k + h, d = S.adv[t];
    const int ch = ((d & 1) ? x0 : 0) | ((d & 2) ? x1 : 0) | ((d & 4) ? x2 : 0);
    const int col = S.ins[t] ? ge16 : mm16 * max(__popc(ch) - 1, 0) + S.ndel[t] * ge16;
    r |= (unsigned)(col + t) << (16 * h);
  }
  return r;
}

// CL: a thread-block cluster per triple (small batches): the rows of a
// hyperplane are spread over the cluster's blocks and a cluster barrier
// ends each hyperplane; block 0 of the cluster takes the jobs, writes the
// early-return outputs and walks the choices back.  Every branch depends
// only on data all blocks read alike, so all blocks reach every barrier.
template <bool PACKED, bool GO0, bool CL>
__global__ void __launch_bounds__(kP3Threads) k_p3(const __grid_constant__ P3Args A) {
  namespace cg = cooperative_groups;
  constexpr P3States S = p3_states();
  extern __shared__ uint8_t p3_sm[];
  __shared__ int s_job;
  const int rank = CL ? (int)cg::this_cluster().block_rank() : 0;
  const int csz = CL ? (int)cg::this_cluster().num_blocks() : 1;
  const bool lead = rank == 0;
  auto bar = [&]() {
    if (CL) cg::this_cluster().sync();
    else __syncthreads();
  };
  const uint8_t *sq[3] = {p3_sm, p3_sm + A.smax, p3_sm + 2 * A.smax};
  uint8_t *sqw[3] = {p3_sm, p3_sm + A.smax, p3_sm + 2 * A.smax};
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int kWarps = kP3Threads / 32;
  // x16 costs: g16[k] = k gap openings, g16[4] = one extension
  const int g16[5] = {0, 16 * A.go, 32 * A.go, 48 * A.go, 16 * A.ge};
  const int64_t slot = CL ? blockIdx.x / csz : blockIdx.x;  // the block's (cluster's) scratch
  int32_t *ring = A.ring + slot * A.ring_stride;
  // packed: [infinite cell | ring]; the column-cost table after the
  // sequences in shared memory, 8 words per (x0, x1, x2), each 0..4
  uint16_t *const infc = reinterpret_cast<uint16_t *>(ring);
  uint16_t *const ring16 = infc + kP3States;
  uint4 *const ctab = reinterpret_cast<uint4 *>(p3_sm + 3 * A.smax);
  unsigned gg[16];  // packed opening costs of two previous states
#pragma unroll
  for (int k = 0; k < 16; ++k) gg[k] = (unsigned)g16[k >> 2] | (unsigned)g16[k & 3] << 16;
  if (PACKED) {
    if (lead && tid < 2)
      reinterpret_cast<uint4 *>(infc)[tid] = make_uint4(kP3Inf2, kP3Inf2, kP3Inf2, kP3Inf2);
    for (int e = tid; e < 125 * 8; e += kP3Threads) {
      const int cmb = e >> 3, k = e & 7;
      const int i0 = cmb / 25, i1 = cmb / 5 % 5, i2 = cmb % 5;
      reinterpret_cast<unsigned *>(ctab)[e] =
          p3_col2(k, i0 ? 1 << (i0 - 1) : 0, i1 ? 1 << (i1 - 1) : 0, i2 ? 1 << (i2 - 1) : 0,
                  16 * A.mm, g16[4]);
    }
  }
  uint64_t *dir = A.dir + slot * A.dir_stride;

  for (;;) {
    if (lead && tid == 0) s_job = atomicAdd(A.counter, 1);
    bar();
    const int job = CL ? *cg::this_cluster().map_shared_rank(&s_job, 0) : s_job;
    if (CL) cg::this_cluster().sync();  // every block has read block 0's s_job
    if (job >= A.n) break;
    const int i = A.order[job];
    const int la = A.len[0][i], lb = A.len[1][i], lc = A.len[2][i];
    const uint8_t *src[3] = {A.seq + A.off[0][i], A.seq + A.off[1][i], A.seq + A.off[2][i]};
    const int cap = (la + lb + lc + 3) & ~3;
    uint8_t *o = A.out + A.out_off[i];

    if (A.mode == 1) {
      // readjust_3d's early returns (sequence.ml:1118-1129); is_empty is
      // sequence.ml:442-450
      const int lm = A.len[3][i];
      const uint8_t *m = A.seq + A.off[3][i];
      int keep = 0;  // 1 m, 2 b, 3 a, 4 c
      if (la == lb && lm == lc && la == lm) {
        keep = 1;
      } else {
        bool e[3] = {true, true, true};
        for (int q = 0; q < 3; ++q) {
          const int l = q == 0 ? la : q == 1 ? lb : lc;
          bool all = true;
          for (int x = tid; x < l; x += kP3Threads) all &= src[q][x] == A.gap;
          e[q] = __syncthreads_and(all);
        }
        keep = (e[0] && !e[1]) ? 2 : (e[1] && !e[0]) ? 3 : e[2] ? 4 : 0;
      }
      if (keep) {
        const uint8_t *k = keep == 1 ? m : keep == 2 ? src[1] : keep == 3 ? src[0] : src[2];
        const int lk = keep == 1 ? lm : keep == 2 ? lb : keep == 3 ? la : lc;
        bool diff = lk != lm;
        for (int x = tid; x < lk; x += kP3Threads) {
          if (lead) o[4 * cap - lk + x] = k[x];
          if (lk == lm) diff |= k[x] != m[x];
        }
        diff = __syncthreads_or(diff);
        if (lead && tid == 0) {
          A.cost[i] = 0;
          A.out_len[2 * i] = 0;
          A.out_len[2 * i + 1] = lk;
          A.changed[i] = diff ? 1 : 0;
        }
        bar();
        continue;
      }
    }

    // the characters Powell's code aligns (copySequence, ukkCommon.c:84-105)
    bool bad = false;
    for (int q = 0; q < 3; ++q) {
      const int l = q == 0 ? la : q == 1 ? lb : lc;
      for (int x = 1 + tid; x < l; x += kP3Threads) {
        const int c = p3_code(src[q][x]);
        bad |= c == 0;
        sqw[q][x] = (uint8_t)c;
      }
    }
    if (__syncthreads_or(bad)) {
      if (lead && tid == 0) {
        A.cost[i] = -1;
        A.out_len[2 * i] = -1;
        A.out_len[2 * i + 1] = -1;
        if (A.mode == 1) A.changed[i] = 0;
        atomicOr(A.err, 1);
      }
      bar();
      continue;
    }

    const int na = la - 1, nb = lb - 1, nc = lc - 1, H = na + nb + nc;
    const int64_t pl = (int64_t)(na + 1) * (nb + 1);  // ring plane (cells)
    const int64_t bcs = (int64_t)(nb + 1) * (nc + 1); // choice-cube i-slice
    for (int h = 0; h <= H; ++h) {
      const int a_lo = max(0, h - nb - nc), a_hi = min(na, h);
      for (int a = a_lo + rank * kWarps + warp; a <= a_hi; a += kWarps * csz) {  // a warp per row
        const int s = h - a, blo = max(0, s - nc), bhi = min(nb, s);
        const int64_t drow = (int64_t)a * bcs + p3_soff(s, nb, nc) - blo;
        if (PACKED && h > 0) {
          // row bases (uint16 units) of the 7 neighbours and of the cell
          int rb[7];
#pragma unroll
          for (int d = 1; d < 8; ++d) {
            const int da = d & 1, db = d >> 1 & 1, dc = d >> 2 & 1;
            rb[d - 1] = (((h - da - db - dc) & 3) * (int)pl + (a - da) * (nb + 1) - db) * kP3States;
          }
          const int ob = ((h & 3) * (int)pl + a * (nb + 1)) * kP3States;
          const int i0 = a ? __ffs(sq[0][a]) : 0;
          for (int b = blo + lane; b <= bhi; b += 32) {
            const int c = s - b, b16 = b * kP3States;
            const uint16_t *src[7];
#pragma unroll
            for (int d = 1; d < 8; ++d) {
              const bool ok = (a >= (d & 1)) && (b >= (d >> 1 & 1)) && (c >= (d >> 2 & 1));
              src[d - 1] = ok ? ring16 + rb[d - 1] + b16 : infc;
            }
            const int cmb = (i0 * 5 + (b ? __ffs(sq[1][b]) : 0)) * 5 + (c ? __ffs(sq[2][c]) : 0);
            dir[drow + b] = p3_cell16<GO0, CL>(src, ring16 + ob + b16, gg, ctab[2 * cmb],
                                           ctab[2 * cmb + 1]);
          }
          continue;
        }
        for (int b = blo + lane; b <= bhi; b += 32) {
          const int c = s - b;
          uint64_t word = 0;
          if (h == 0) {  // the start: MMM at cost 0
            if (PACKED) {
              uint4 *r = reinterpret_cast<uint4 *>(ring16);
              // every value carries its own state number
              r[0] = make_uint4(0xC0010000u, 0xC003C002u, 0xC005C004u, 0xC007C006u);
              r[1] = make_uint4(0xC009C008u, 0xC00BC00Au, 0xC00DC00Cu, 0xC00FC00Eu);
            } else {
              int4 *r = reinterpret_cast<int4 *>(ring);
              r[0] = make_int4(0, kP3Inf, kP3Inf, kP3Inf);
              for (int q = 1; q < 4; ++q) r[q] = make_int4(kP3Inf, kP3Inf, kP3Inf, kP3Inf);
            }
          } else {
            // alignmentCost's mismatches (ukkCommon.c:381-389), x16, by the
            // sequences a column consumes: mm per extra distinct character
            const int x0 = a ? sq[0][a] : 0, x1 = b ? sq[1][b] : 0, x2 = c ? sq[2][c] : 0;
            int col16[8];
            col16[0] = 0;
#pragma unroll
            for (int d = 1; d < 8; ++d) {
              const int ch = ((d & 1) ? x0 : 0) | ((d & 2) ? x1 : 0) | ((d & 4) ? x2 : 0);
              col16[d] = 16 * A.mm * (__popc(ch) - 1);
            }
            word = p3_cell(ring, pl, nb, h, a, b, c, g16, col16);
          }
          dir[drow + b] = word;
        }
      }
      bar();
    }

    if (lead && tid == 0) {
      const int64_t fo = ((int64_t)(H & 3) * pl + (int64_t)na * (nb + 1) + nb) * kP3States;
      const int inf = PACKED ? 0xC000 : kP3Inf;
      int best = inf, st = 0;
      for (int s = 0; s < kP3States; ++s) {
        const int f = PACKED ? (int)(__ldcg(ring16 + fo + s) & 0xFFF0u) : __ldcg(ring + fo + s);
        if (f < best) best = f, st = s;
      }
      if (PACKED && best >= inf) {  // the optimum reached the clamp: redo in 32 bits
        if (tid == 0) atomicOr(A.err, 4);
      }
      int a = na, b = nb, c = nc, n = 0, nm = 0;
      bool okw = best < inf;
      while (okw && (a | b | c)) {
        const int s = b + c;
        const uint64_t wd =
            __ldcg(dir + (int64_t)a * bcs + p3_soff(s, nb, nc) + (b - max(0, s - nc)));
        const int prev = (int)(wd >> (4 * st) & 15);
        const int ad = c_p3.adv[st];
        if ((ad & 1) > a || (ad >> 1 & 1) > b || (ad >> 2 & 1) > c) {
          okw = false;  // cannot happen for a finite optimum; kept as a guard
          break;
        }
        const int ca = (ad & 1) ? sq[0][a] : 16, cb = (ad & 2) ? sq[1][b] : 16,
                  cc = (ad & 4) ? sq[2][c] : 16;
        ++n;
        o[cap - n] = (uint8_t)ca;
        o[2 * cap - n] = (uint8_t)cb;
        o[3 * cap - n] = (uint8_t)cc;
        const int md = A.med[25 * p3_ix(ca) + 5 * p3_ix(cb) + p3_ix(cc)];
        if (A.has_med && md != A.gap) o[4 * cap - ++nm] = (uint8_t)md;
        a -= ad & 1;
        b -= ad >> 1 & 1;
        c -= ad >> 2 & 1;
        st = prev;
      }
      ++n;  // the leading gap column (printTraceBack, ukk.checkp.c)
      o[cap - n] = o[2 * cap - n] = o[3 * cap - n] = 16;
      if (A.has_med) o[4 * cap - ++nm] = (uint8_t)A.gap;
      if (!okw) {
        if (!PACKED) atomicOr(A.err, 2);
        n = nm = -1;
      }
      A.cost[i] = okw ? best >> 4 : -1;
      A.out_len[2 * i] = n;
      A.out_len[2 * i + 1] = A.has_med ? nm : 0;
      if (A.mode == 1) {
        const int lm = A.len[3][i];
        const uint8_t *m = A.seq + A.off[3][i];
        bool diff = nm != lm;
        for (int x = 0; !diff && x < lm; ++x) diff = o[4 * cap - nm + x] != m[x];
        A.changed[i] = diff ? 1 : 0;
      }
    }
    bar();
  }
}

// Host side shared by the two batched entry points.
static int p3_run(int mode, int32_t n, const uint8_t *seq, const int64_t *const off[4],
                  const int32_t *const len[4], int mm, int go, int ge, int gap,
                  const uint8_t *median3, int32_t *cost, uint8_t *out, const int64_t *out_off,
                  int32_t *out_len, int32_t *changed, cudaStream_t st) {
  if (n < 0) return fail(POYD_EINVAL, "three-sequence batch: n < 0");
  if (n == 0) return POYD_OK;
  if (!seq || !cost || !out || !out_off || !out_len || (mode == 1 && !changed))
    return fail(POYD_EINVAL, "three-sequence batch: null argument");
  if (mm <= 0 || go < 0 || ge <= 0)
    return fail(POYD_EINVAL, "powell_3D_align needs mm > 0, go >= 0, ge > 0 (ukkCommon.c:130)");
  const int nq = mode == 1 ? 4 : 3;
  for (int q = 0; q < nq; ++q)
    if (!off[q] || !len[q]) return fail(POYD_EINVAL, "three-sequence batch: null argument");
  std::vector<int32_t> hl[4];
  for (int q = 0; q < nq; ++q) {
    hl[q].resize(n);
    CK3(cudaMemcpyAsync(hl[q].data(), len[q], sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  }
  CK3(cudaStreamSynchronize(st));
  int64_t ring_max = 0, dir_max = 0;
  int smax = 16;
  std::vector<int64_t> work(n);
  const int64_t step_max = 2LL * go + 2LL * ge + 2LL * mm;
  for (int32_t i = 0; i < n; ++i) {
    const int64_t la = hl[0][i], lb = hl[1][i], lc = hl[2][i];
    if (la < 1 || lb < 1 || lc < 1 || (mode == 1 && hl[3][i] < 0))
      return fail(POYD_EINVAL, "triple %d: every sequence holds at least its leading gap", i);
    if (la > kP3MaxLen || lb > kP3MaxLen || lc > kP3MaxLen)
      return fail(POYD_ERANGE, "triple %d: sequences longer than %d", i, kP3MaxLen);
    if ((la + lb + lc) * step_max * 16 >= kP3Inf / 2)
      return fail(POYD_ERANGE, "triple %d: costs could reach the DP's infinity", i);
    ring_max = std::max(ring_max, 4 * la * lb * kP3States);
    dir_max = std::max(dir_max, la * lb * lc);
    smax = std::max<int>(smax, (int)std::max(la, std::max(lb, lc)));
    work[i] = la * lb * lc;
  }
  smax = (smax + 15) & ~15;
  std::vector<int32_t> order;
  longest_first(work, order);

  int dev = 0, sms = 0;
  CK3(cudaGetDevice(&dev));
  CK3(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  size_t fr = 0, tot = 0;
  CK3(cudaMemGetInfo(&fr, &tot));
  const int64_t per_block = ring_max * 4 + dir_max * 8;
  // the choice cubes dominate: one per resident block, sized for the
  // largest triple; by default at most 60 % of the free memory, 120 GiB
  int64_t budget = std::min<int64_t>((int64_t)(fr * 0.6), 120LL << 30);
  if (const char *e = getenv("POYD_P3_BUDGET_MB")) budget = std::max<int64_t>(1, atoll(e)) << 20;
  int64_t blocks = std::min<int64_t>({(int64_t)n, 3LL * sms, std::max<int64_t>(1, budget / per_block)});

  Workspace *w = workspace(st);
  int32_t *ring = (int32_t *)ws_buffer(w, WS_P3_RING, (size_t)(ring_max * 4 * blocks));
  uint64_t *dirp = (uint64_t *)ws_buffer(w, WS_P3_DIR, (size_t)(dir_max * 8 * blocks));
  int32_t *meta = (int32_t *)ws_buffer(w, WS_P3_META, sizeof(int32_t) * ((size_t)n + 4));
  if (!ring || !dirp || !meta) return fail(POYD_ENOMEM, "three-sequence workspace (%lld blocks)", (long long)blocks);
  order.push_back(0);  // counter
  order.push_back(0);  // err
  CK3(cudaMemcpyAsync(meta, order.data(), sizeof(int32_t) * ((size_t)n + 2), cudaMemcpyHostToDevice, st));

  P3Args A;
  std::memset(&A, 0, sizeof(A));
  A.n = n;
  A.mode = mode;
  A.seq = seq;
  for (int q = 0; q < nq; ++q) {
    A.off[q] = off[q];
    A.len[q] = len[q];
  }
  A.cost = cost;
  A.out = out;
  A.out_off = out_off;
  A.out_len = out_len;
  A.changed = changed;
  A.order = meta;
  A.counter = meta + n;
  A.err = meta + n + 1;
  A.ring = ring;
  A.ring_stride = ring_max;
  A.dir = dirp;
  A.dir_stride = dir_max;
  A.mm = mm;
  A.go = go;
  A.ge = ge;
  A.gap = gap;
  A.has_med = median3 ? 1 : 0;
  {
    static const int st5[5] = {1, 2, 4, 8, 16};
    for (int x = 0; x < 5; ++x)
      for (int y = 0; y < 5; ++y)
        for (int z = 0; z < 5; ++z)
          A.med[25 * x + 5 * y + z] =
              median3 ? median3[(st5[x] << 10) | (st5[y] << 5) | st5[z]] : (uint8_t)gap;
  }
  A.smax = smax;
  const size_t smem = 3 * (size_t)smax + 125 * 8 * sizeof(unsigned);
  // 16-bit halves while every addend of a half stays below 0x4000
  // (openings, column costs); a triple whose optimum reaches the clamp
  // sets err bit 4 and the batch is redone in 32 bits
  const char *pk = getenv("POYD_P3_PACKED");
  bool packed = !(pk && pk[0] == '0') && 48LL * go + 15 < 0x4000 &&
                16LL * (2LL * mm + 3LL * ge) < 0x4000;
  // small batches: a cluster of up to 8 blocks per triple, so that the
  // batch still covers the SMs (POYD_P3_CLUSTER=0: one block per triple)
  int csize = 1;
  {
    const char *ce = getenv("POYD_P3_CLUSTER");
    const int64_t want = 3LL * sms / std::max<int64_t>(blocks, 1);
    if (!(ce && ce[0] == '0'))
      while (csize < 8 && 2 * csize <= want) csize *= 2;
  }
  for (;;) {
    auto kern = packed ? (go == 0 ? k_p3<true, true, false> : k_p3<true, false, false>)
                       : k_p3<false, false, false>;
    auto kcl = go == 0 ? k_p3<true, true, true> : k_p3<true, false, true>;
    bool launched = false;
    if (packed && csize > 1) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)csize;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3((unsigned)(blocks * csize));
      cfg.blockDim = dim3(kP3Threads);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = st;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      if (smem > 48 * 1024)
        CK3(cudaFuncSetAttribute(kcl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      int ncl = 0;
      if (cudaOccupancyMaxActiveClusters(&ncl, kcl, &cfg) == cudaSuccess && ncl > 0) {
        ProfScope ps("p3", st);
        CK3(cudaLaunchKernelEx(&cfg, kcl, A));
        launched = true;
      } else {
        cudaGetLastError();
        csize = 1;
      }
    }
    if (!launched) {
      if (smem > 48 * 1024)
        CK3(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      ProfScope ps("p3", st);
      kern<<<(unsigned)blocks, kP3Threads, smem, st>>>(A);
    }
    CK3(cudaGetLastError());
    int32_t herr = 0;
    CK3(cudaMemcpyAsync(&herr, A.err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK3(cudaStreamSynchronize(st));
    if (herr & 1)
      return fail(POYD_EINVAL, "an element holds none of A, C, G, T (powell_3D_align fails, "
                               "ukkCommon.c:101): its triple has cost -1");
    if (herr & 2) return fail(POYD_ERANGE, "three-sequence traceback left the cube");
    if (!(herr & 4)) return POYD_OK;
    packed = false;  // some optimum reached the 16-bit clamp
    const int32_t zero2[2] = {0, 0};
    CK3(cudaMemcpyAsync(A.counter, zero2, sizeof(zero2), cudaMemcpyHostToDevice, st));
  }
}

// Cost_matrix.Three_D.of_two_dim_comb (cost_matrix.ml:803-851): the median
// of (i, j, k) is the lowest single state l with the least
// cost[l][i] + cost[l][j] + cost[l][k]; the gap takes part only for metric
// matrices or when two of i, j, k hold it.  The reference seeds each entry
// with OCaml's max_int, which fits a C int on a 32-bit OCaml only (on a
// 64-bit one it truncates to -1 and no entry is ever set); this follows the
// 32-bit reading.
static void median3_table(const poyd_cm *cm, uint8_t *tab) {
  std::memset(tab, 0, 32768);
  for (int i = 1; i < 32; ++i)
    for (int j = 1; j < 32; ++j)
      for (int k = 1; k < 32; ++k) {
        int64_t best = INT64_MAX;
        int med = 0;
        for (int l = 0; l < cm->lcm; ++l) {
          const int x = 1 << l;
          const int shared = ((i & x) != 0) + ((j & x) != 0) + ((k & x) != 0);
          int64_t c = INT64_MAX;
          if (cm->is_metric || shared >= 2 || x != cm->gap)
            c = (int64_t)cm->cost[(x << 5) + i] + cm->cost[(x << 5) + j] + cm->cost[(x << 5) + k];
          if (c < best) {
            best = c;
            med = x;
          } else if (c == best) {
            med |= x;
          }
        }
        tab[(i << 10) | (j << 5) | k] = (uint8_t)(med & -med);
      }
}

}  // namespace poyd

using namespace poyd;

extern "C" int poyd_cm_median3(const poyd_cm *cm, uint8_t *tab) {
  if (!cm || !tab) return fail(POYD_EINVAL, "poyd_cm_median3: null argument");
  if (!cm->combinations || cm->lcm < 1 || cm->lcm > 5)
    return fail(POYD_EUNSUP, "poyd_cm_median3: combination alphabets of at most 5 states");
  median3_table(cm, tab);
  return POYD_OK;
}

extern "C" int poyd_powell_3d_batch(int32_t n, const uint8_t *seq, const int64_t *a_off,
                                    const int32_t *a_len, const int64_t *b_off,
                                    const int32_t *b_len, const int64_t *c_off,
                                    const int32_t *c_len, int32_t mm, int32_t go, int32_t ge,
                                    const uint8_t *median3, int32_t *cost, uint8_t *out,
                                    const int64_t *out_off, int32_t *out_len, void *stream) {
  const int64_t *off[4] = {a_off, b_off, c_off, nullptr};
  const int32_t *len[4] = {a_len, b_len, c_len, nullptr};
  return p3_run(0, n, seq, off, len, mm, go, ge, 16, median3, cost, out, out_off, out_len,
                nullptr, (cudaStream_t)stream);
}

extern "C" int poyd_readjust_3d_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                                      const int64_t *s1_off, const int32_t *s1_len,
                                      const int64_t *s2_off, const int32_t *s2_len,
                                      const int64_t *m_off, const int32_t *m_len,
                                      const int64_t *p_off, const int32_t *p_len,
                                      int32_t *cost, uint8_t *out, const int64_t *out_off,
                                      int32_t *out_len, int32_t *changed, void *stream) {
  if (!cm) return fail(POYD_EINVAL, "poyd_readjust_3d_batch: null cost matrix");
  if (!cm->combinations || cm->lcm != 5 || cm->gap != 16)
    return fail(POYD_EUNSUP, "poyd_readjust_3d_batch: the DNA alphabet with combinations");
  // align_3_powell_inter's parameters (sequence.ml:1091-1102)
  const int mm = cm->cost[(1 << 5) + 2], ge = cm->cost[(1 << 5) + 16];
  const int go = cm->cost_model == 1 ? cm->gap_open : 0;
  static thread_local uint8_t tab[32768];
  median3_table(cm, tab);
  const int64_t *off[4] = {s1_off, s2_off, p_off, m_off};
  const int32_t *len[4] = {s1_len, s2_len, p_len, m_len};
  return p3_run(1, n, seq, off, len, mm, go, ge, cm->gap, tab, cost, out, out_off, out_len,
                changed, (cudaStream_t)stream);
}

extern "C" int poyd_powell_3D_align(const uint8_t *sa, int32_t la, const uint8_t *sb,
                                    int32_t lb, const uint8_t *sc, int32_t lc, uint8_t *ra,
                                    uint8_t *rb, uint8_t *rc, int32_t cap, int32_t *len,
                                    int32_t mm, int32_t go, int32_t ge, int32_t *cost) {
  if (!sa || !sb || !sc || !ra || !rb || !rc || !len || !cost)
    return fail(POYD_EINVAL, "poyd_powell_3D_align: null argument");
  if (la < 1 || lb < 1 || lc < 1) return fail(POYD_EINVAL, "poyd_powell_3D_align: empty sequence");
  if ((int64_t)cap < (int64_t)la + lb + lc - 2)
    return fail(POYD_ERANGE, "output capacity below len(a) + len(b) + len(c) - 2");
  Workspace *w = workspace();
  cudaStream_t st = nullptr;
  // staging: [offsets x4 | lengths x3, cost, out_len x2 | a b c | slot]
  const int64_t slot = ((int64_t)la + lb + lc + 3) & ~(int64_t)3;
  const size_t in = ((size_t)la + lb + lc + 63) & ~(size_t)63;
  uint8_t *buf = (uint8_t *)ws_buffer(w, WS_P3_IO, 64 + in + 4 * (size_t)slot);
  if (!buf) return fail(POYD_ENOMEM, "poyd_powell_3D_align: staging allocation failed");
  int64_t *meta = (int64_t *)buf;
  int32_t *m32 = (int32_t *)(buf + 32);
  uint8_t *sq = buf + 64, *o = buf + 64 + in;
  const int64_t hmeta[4] = {0, la, (int64_t)la + lb, 0};
  const int32_t hlen[3] = {la, lb, lc};
  CK3(cudaMemcpyAsync(sq, sa, la, cudaMemcpyHostToDevice, st));
  CK3(cudaMemcpyAsync(sq + la, sb, lb, cudaMemcpyHostToDevice, st));
  CK3(cudaMemcpyAsync(sq + la + lb, sc, lc, cudaMemcpyHostToDevice, st));
  CK3(cudaMemcpyAsync(meta, hmeta, sizeof(hmeta), cudaMemcpyHostToDevice, st));
  CK3(cudaMemcpyAsync(m32, hlen, sizeof(hlen), cudaMemcpyHostToDevice, st));
  int rc_ = poyd_powell_3d_batch(1, sq, meta, m32, meta + 1, m32 + 1, meta + 2, m32 + 2, mm, go,
                                 ge, nullptr, m32 + 3, o, meta + 3, m32 + 4, st);
  if (rc_) return rc_;
  int32_t res[3];
  CK3(cudaMemcpy(res, m32 + 3, sizeof(res), cudaMemcpyDeviceToHost));
  const int n = res[1];
  if (n > cap) return fail(POYD_ERANGE, "poyd_powell_3D_align: alignment longer than cap");
  uint8_t *dst[3] = {ra, rb, rc};
  for (int k = 0; k < 3; ++k)
    CK3(cudaMemcpy(dst[k] + cap - n, o + (k + 1) * slot - n, (size_t)n, cudaMemcpyDeviceToHost));
  *len = n;
  *cost = res[0];
  return POYD_OK;
}
