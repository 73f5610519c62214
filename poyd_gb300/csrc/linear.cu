// Linear-gap banded direct-optimization DP on sm_103a.
//
// Restates algn_fill_plane_2 / algn_fill_plane (algn.c:812-968) with the
// per-cell rule of algn_fill_row (algn.c:375-453) and the band-edge cells of
// algn.c:461-620, plus backtrack_2d (algn.c:3551-3666), ancestor_2
// (algn.c:4126-4147) and median_2_with_gaps (algn.c:4011-4024).
//
// Layout on the GPU.  One warp owns one pair.  Lane k owns DP row
// r = 32*strip + k of a 32-row strip; the warp sweeps the band in diagonal
// coordinates d = j - r, which makes the band edges of every row the same
// two diagonals [dlo, dlo+wd) (the reference's ukk left/right cells).  Lane
// k handles diagonal d at step s = d - dlo + 2k: the value of row r-1 at
// (d+1) -- the "delete" predecessor -- arrives from lane k-1 by one shuffle
// that also carries the column character s2[r+d]; the previous shuffle's
// value is the "align" predecessor and the lane's own previous value is the
// "insert" predecessor.  Lane 0 is fed the previous strip's last row from a
// register queue that rotates one lane per step and is refilled / flushed
// with one coalesced 128-byte load / store every 32 steps (the boundary row
// lives in a per-warp global scratch slab of wd ints).  Cells outside the
// band or the matrix hold kInf, which removes exactly the moves the
// reference's edge cells omit.  The direction set of every cell (ALIGN 1,
// INSERT 2, DELETE 4; matrices.h:22-27) is packed 8 cells per 32-bit word
// and stored with one coalesced store per 8 steps; the traceback addresses
// it by (strip, step/8, lane).
#include <cuda_runtime.h>
#include <cstdint>
#include "poyd_internal.h"
#include "linear_kernels.cuh"

namespace poyd {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// Plan: orientation, deltaw, band geometry, DM size and band cell count.
// ---------------------------------------------------------------------------
__global__ void k_lin_plan(LinPlanArgs A) {
  const int lane = threadIdx.x & 31;
  const int id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (id >= A.n) return;
  const int la = A.a_len[id], lb = A.b_len[id];
  const int64_t ao = A.a_off[id], bo = A.b_off[id];
  const int gap = A.gap;
  unsigned ga = 0, gb = 0, na = 0, nb = 0;
  for (int x = lane; x < la; x += 32) {
    const int c = A.seq[ao + x];
    ga += (c & gap) != 0;
    na += c != gap;
  }
  for (int x = lane; x < lb; x += 32) {
    const int c = A.seq[bo + x];
    gb += (c & gap) != 0;
    nb += c != gap;
  }
  ga = __reduce_add_sync(kFull, ga);
  gb = __reduce_add_sync(kFull, gb);
  na = __reduce_add_sync(kFull, na);
  nb = __reduce_add_sync(kFull, nb);

  const int swap = la < lb;
  const int l1 = swap ? lb : la, l2 = swap ? la : lb;
  // deltaw (sequence.ml:691-713); seq_CAML_count counts positions sharing
  // a bit with the gap (seq.c:571-581).
  const int gaps = (int)(ga > gb ? ga : gb);
  const int dif = l1 - l2;
  const int lower = (int)((double)l1 * 0.10);
  int dwc;
  if (A.policy == POYD_DELTAW_RAW) {
    dwc = A.deltaw[id] - gaps;  // deltawh passed straight to algn_nw
  } else if (A.policy == POYD_DELTAW_DEFAULT) {
    dwc = (dif < lower) ? lower / 2 : 2;
  } else {
    int v = (A.policy == POYD_DELTAW_EXPLICIT) ? A.deltaw[id] : (dif > 8 ? dif : 8);
    dwc = (dif < lower) ? lower : v;
  }
  const int dw = gaps + dwc;
  // algn_fill_plane_2 band cases (algn.c:880-937)
  int width = 50 + dw, height = dif + 50 + dw;
  if (width > l2) width = l2;
  if (height > l1) height = l1;
  int full = 0, delta = 0;
  if (__fmul_rn(1.5f, (float)l2) <= (float)l1) full = 1;
  else if (2 * height < l1) delta = 1;
  else if (8 >= l1 - height) full = 1;
  int dlo, dhi;
  if (full) { dlo = -(l1 - 1); dhi = l2 - 1; }
  else { dlo = delta - height; dhi = width - 1; }
  const int wd = dhi - dlo + 1;

  // DP cells the reference evaluates: row r covers diagonals
  // [max(dlo, -r), min(dhi, l2-1-r)].
  long long cells = 0;
  for (int r = lane; r < l1; r += 32) {
    const int lo = dlo > -r ? dlo : -r;
    const int hi = dhi < l2 - 1 - r ? dhi : l2 - 1 - r;
    if (hi >= lo) cells += hi - lo + 1;
  }
  for (int o = 16; o > 0; o >>= 1) cells += __shfl_xor_sync(kFull, cells, o);

  if (lane == 0) {
    LinPlan P;
    P.s1_off = swap ? bo : ao;
    P.s2_off = swap ? ao : bo;
    P.dm_off = 0;
    P.l1 = l1; P.l2 = l2;
    P.dlo = dlo; P.wd = wd;
    P.swap = swap;
    P.nstrips = (l1 + kRows - 1) / kRows;
    const int S = wd + kLag * (kLanes - 1) + 1;
    const int Spad = (S + kStepBlock - 1) / kStepBlock * kStepBlock;
    P.sblocks = Spad / 8;
    P.deltaw = dw;
    P.empty = 0;
    if (A.dos_empty) {
      if (na == 0) P.empty = 1;
      else if (nb == 0) P.empty = 2;
    }
    P.pad_ = 0;
    A.plans[id] = P;
    // direction-matrix words; also the work estimate used to order pairs
    A.dm_words[id] = (int64_t)P.nstrips * P.sblocks * kRows;
    A.wd_out[id] = wd;
    if (A.cells) A.cells[id] = cells;
    if (la < 1 || lb < 1) atomicOr(A.err, 1);
    if ((long long)A.maxc * (l1 + l2 + 2) >= kMaxCost) atomicOr(A.err, 2);
  }
}

// ---------------------------------------------------------------------------
// Band DP.  DM = true also writes the direction matrix.
// ---------------------------------------------------------------------------
struct LinStrip {
  int HA, HB, diag, Pk, q;
  uint32_t wA, wB;
  int result;
};

// 32 steps of one strip.  Each lane owns two rows: row A = r0 + 2k handles
// diagonal d at step s = d - dlo + 3k, row B = row A + 1 handles d - 1 in
// the same step, so row B's delete predecessor is row A's value computed
// just before and both cells use the same column character.  MASK applies
// the per-row band/matrix validity (needed only in blocks where some row is
// outside its band); CAP records the final cell (last strip only).
template <bool DM, bool MASK, bool CAP>
__device__ __forceinline__ void lin_block(LinStrip &S, const int2 *trowA, const int2 *trowB,
                                          int cDA, int cDB, int vbA, int cntA, int vbB, int cntB,
                                          int finA, int finB, uint2 *dmw, int lane) {
#pragma unroll
  for (int u = 0; u < kStepBlock; ++u) {
    int up = __shfl_up_sync(kFull, S.Pk, 1);
    if (lane == 0) up = S.q;
    S.q = __shfl_sync(kFull, S.q, (lane + 1) & 31);
    const int c = up & 31;
    const int hup = up >> 5;
    const int2 TA = trowA[c];  // {cost[a][c], cost[gap][c]}
    const int2 TB = trowB[c];
    // row A: delete from the lane above, align from its previous value
    const int Av = S.diag + TA.x;
    const int Dv = hup + cDA;
    const int Iv = S.HA + TA.y;
    int ha = min(min(Av, Dv), Iv);
    if (MASK) ha = ((unsigned)(vbA + u) < (unsigned)cntA) ? ha : kInf;
    // row B: delete from row A now, align from row A's previous value
    const int Av2 = S.HA + TB.x;
    const int Dv2 = ha + cDB;
    const int Iv2 = S.HB + TB.y;
    int hb = min(min(Av2, Dv2), Iv2);
    if (MASK) hb = ((unsigned)(vbB + u) < (unsigned)cntB) ? hb : kInf;
    if (DM) {
      const uint32_t fa = (uint32_t)(Av == ha) | ((uint32_t)(Iv == ha) << 1) |
                          ((uint32_t)(Dv == ha) << 2);
      const uint32_t fb = (uint32_t)(Av2 == hb) | ((uint32_t)(Iv2 == hb) << 1) |
                          ((uint32_t)(Dv2 == hb) << 2);
      S.wA = (S.wA << 4) | fa;
      S.wB = (S.wB << 4) | fb;
      if ((u & 7) == 7) dmw[(u >> 3) * kLanes] = make_uint2(S.wA, S.wB);
    }
    if (CAP) {
      if (u == finA) S.result = ha;
      if (u == finB) S.result = hb;
    }
    S.Pk = (int)(((unsigned)hb << 5) | (unsigned)c);
    if (lane == 31) S.q = S.Pk;
    S.diag = hup;
    S.HA = ha;
    S.HB = hb;
  }
}

template <bool DM>
__device__ __forceinline__ void lin_pair(const LinDpArgs &A, const int2 *tab,
                                         const LinPlan &P, int64_t dm_off, int id,
                                         int *bnd, int lane) {
  const uint8_t *s1 = A.seq + P.s1_off;
  const uint8_t *s2 = A.seq + P.s2_off;
  const int L1 = P.l1, L2 = P.l2, dlo = P.dlo, wd = P.wd;
  const int gap = A.gap;

  for (int x = lane; x < wd; x += 32) bnd[x] = kInf;
  __syncwarp();
  if (lane == 0) bnd[-dlo] = -tab[(s1[0] << 5) | s2[0]].x;
  __syncwarp();

  const int Spad = P.sblocks * 8;
  const int r_last = L1 - 1;
  const int d_last = L2 - L1;
  LinStrip S;
  S.result = 0;
  uint32_t *dm = DM ? A.dm + dm_off : nullptr;

  for (int strip = 0; strip < P.nstrips; ++strip) {
    const int r0 = strip * kRows;
    const int rA = r0 + 2 * lane, rB = rA + 1;
    const bool okA = rA < L1, okB = rB < L1;
    const bool last = strip == P.nstrips - 1;
    const int aA = okA ? s1[rA] : 0, aB = okB ? s1[rB] : 0;
    const int2 *trowA = tab + (aA << 5), *trowB = tab + (aB << 5);
    const int cDA = tab[(aA << 5) | gap].x, cDB = tab[(aB << 5) | gap].x;
    const int offA = (-dlo - rA) > 0 ? (-dlo - rA) : 0;
    const int offB = (-dlo - rB) > 0 ? (-dlo - rB) : 0;
    const int lowerA = kLag * lane + offA, lowerB = kLag * lane + 1 + offB;
    const int cntA = okA ? wd - offA : 0, cntB = okB ? wd - offB : 0;
    const int sfinA = (rA == r_last) ? (d_last - dlo + kLag * lane) : -1000000;
    const int sfinB = (rB == r_last) ? (d_last - dlo + kLag * lane + 1) : -1000000;
    // steps where both rows of every lane are inside their bands
    const int lo = lowerA > lowerB ? lowerA : lowerB;
    const int hi = (lowerA + cntA) < (lowerB + cntB) ? (lowerA + cntA) : (lowerB + cntB);
    const int all_lo = (int)__reduce_max_sync(kFull, (unsigned)lo);
    const int all_hi = (int)__reduce_min_sync(kFull, (unsigned)hi);
    S.HA = kInf;
    S.HB = kInf;
    S.diag = kInf;
    S.Pk = (int)((unsigned)kInf << 5);
    S.wA = 0;
    S.wB = 0;
    auto qload = [&](int s0) -> int {
      const int x = s0 + lane + 1;
      const int hv = (x < wd) ? bnd[x] : kInf;
      const int j = r0 + dlo + s0 + lane;
      const int c = (j >= 0 && j < L2) ? s2[j] : 0;
      return (int)(((unsigned)hv << 5) | (unsigned)c);
    };
    S.q = qload(0);
    if (lane == 0) S.diag = bnd[0];
    uint2 *dmrow = DM ? (uint2 *)(dm + (int64_t)strip * P.sblocks * kRows) + lane : nullptr;
    for (int s0 = 0; s0 < Spad; s0 += kStepBlock) {
      const int qn = (s0 + kStepBlock < Spad) ? qload(s0 + kStepBlock) : 0;
      uint2 *dmw = DM ? dmrow + (s0 >> 3) * kLanes : nullptr;
      const int vbA = s0 - lowerA, vbB = s0 - lowerB;
      if (last) {
        lin_block<DM, true, true>(S, trowA, trowB, cDA, cDB, vbA, cntA, vbB, cntB, sfinA - s0,
                                  sfinB - s0, dmw, lane);
      } else if (s0 >= all_lo && s0 + kStepBlock <= all_hi) {
        lin_block<DM, false, false>(S, trowA, trowB, cDA, cDB, vbA, cntA, vbB, cntB, -1, -1, dmw,
                                    lane);
      } else {
        lin_block<DM, true, false>(S, trowA, trowB, cDA, cDB, vbA, cntA, vbB, cntB, -1, -1, dmw,
                                   lane);
      }
      const int x = s0 + lane - (kLag * 31 + 1);
      if (x >= 0 && x < wd) bnd[x] = S.q >> 5;
      S.q = qn;
    }
    __syncwarp();
  }
  const int src = (r_last % kRows) >> 1;
  const int result = __shfl_sync(kFull, S.result, src);
  if (lane == 0) A.cost[id] = result;
}

template <bool DM>
__global__ void __launch_bounds__(256, 4) k_lin_dp(LinDpArgs A) {
  __shared__ int2 tab[1024];  // {cost[a][b], cost[gap][b]}
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
    const uint32_t p = A.tables->packed[i];
    tab[i] = make_int2((int)(p & 0xffffu), (int)(p >> 16));
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int *bnd = A.scratch + gw * A.slab;
  for (;;) {
    int p = 0;
    if (lane == 0) p = atomicAdd(A.counter, 1);
    p = __shfl_sync(kFull, p, 0);
    if (p >= A.n) break;
    const int id = A.order ? A.order[p] : p;
    const LinPlan P = A.plans[id];
    if (P.empty) {
      if (lane == 0) A.cost[id] = 0;
      continue;
    }
    lin_pair<DM>(A, tab, P, DM ? A.dm_off[id] : 0, id, bnd, lane);
  }
}

// ---------------------------------------------------------------------------
// Traceback + medians: one thread per pair.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_lin_traceback(LinTbArgs A) {
  __shared__ uint8_t med[1024];
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) med[i] = A.tables->median[i];
  __syncthreads();
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= A.n) return;
  const LinPlan P = A.plans[id];
  const int gap = A.gap;
  const int la = P.swap ? P.l2 : P.l1, lb = P.swap ? P.l1 : P.l2;
  const int64_t cap = (int64_t)la + lb + 2;
  uint8_t *oa = A.out + A.out_off[id];
  uint8_t *ob = oa + cap, *ow = ob + cap, *om = ow + cap;
  const uint8_t *s1 = A.seq + P.s1_off, *s2 = A.seq + P.s2_off;
  if (P.empty) {
    // DOS.median: the non-empty (or second) sequence is the median.
    const bool a_empty = P.empty == 1;
    const uint8_t *src = (a_empty != (bool)P.swap) ? s2 : s1;  // caller's b if a empty
    const int len = a_empty ? lb : la;
    for (int i = 0; i < len; ++i) om[cap - len + i] = src[i];
    A.out_len[2 * id] = 0;
    A.out_len[2 * id + 1] = len;
    return;
  }
  const uint32_t *dm = A.dm + A.dm_off[id];
  const int L2 = P.l2, dlo = P.dlo, sb = P.sblocks;
  // backtrack priority (algn.c:3605-3666): the caller's first argument is
  // the rows sequence unless the pair was swapped
  const bool swaped = A.swaped < 0 ? !P.swap : (A.swaped != 0);
  int r = P.l1 - 1, j = L2 - 1;
  int64_t n = 0, nm = 0;
  const int spad = sb * 8;
  bool bad = false;
  while ((int64_t)r * L2 + j >= 0) {
    const int k = (r & (kRows - 1)) >> 1, strip = r / kRows;
    const int s = (j - r) - dlo + kLag * k + (r & 1);
    if (r < 0 || j < 0 || s < 0 || s >= spad || n + 2 >= cap) {  // left the band: a bug
      bad = true;
      break;
    }
    const uint32_t w = dm[((int64_t)strip * sb + (s >> 3)) * kRows + (r & (kRows - 1))];
    const uint32_t f = (w >> (4 * (7 - (s & 7)))) & 15u;
    int cr, cc;
    if (f & 1u) { cr = s1[r]; cc = s2[j]; --r; --j; }
    else if (swaped ? (f & 2u) : !(f & 4u)) { cr = gap; cc = s2[j]; --j; }
    else { cr = s1[r]; cc = gap; --r; }
    const int ca = P.swap ? cc : cr, cb = P.swap ? cr : cc;
    const int m = med[(ca << 5) | cb];
    oa[cap - 1 - n] = (uint8_t)ca;
    ob[cap - 1 - n] = (uint8_t)cb;
    ow[cap - 1 - n] = (uint8_t)m;
    if (m != gap) om[cap - 1 - nm++] = (uint8_t)m;
    ++n;
  }
  // ancestor_2 ends with the leading gap (algn.c:4140-4141)
  om[cap - 1 - nm++] = (uint8_t)gap;
  A.out_len[2 * id] = bad ? -1 : (int32_t)n;
  A.out_len[2 * id + 1] = bad ? -1 : (int32_t)nm;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_lin_plan(const LinPlanArgs &A, cudaStream_t st) {
  const int threads = 256;
  const int64_t blocks = ((int64_t)A.n * 32 + threads - 1) / threads;
  k_lin_plan<<<(unsigned)blocks, threads, 0, st>>>(A);
}

int lin_dp_blocks(bool dm) {
  static int cache[2][64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  int &c = cache[dm ? 1 : 0][dev & 63];
  if (!c) {
    int per_sm = 0, sms = 0;
    if (dm) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lin_dp<true>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lin_dp<false>, 256, 0);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    c = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  return c;
}

void launch_lin_dp(const LinDpArgs &A, bool dm, int blocks, cudaStream_t st) {
  if (dm) k_lin_dp<true><<<blocks, 256, 0, st>>>(A);
  else k_lin_dp<false><<<blocks, 256, 0, st>>>(A);
}

void launch_lin_traceback(const LinTbArgs &A, cudaStream_t st) {
  const int threads = 128;
  k_lin_traceback<<<(A.n + threads - 1) / threads, threads, 0, st>>>(A);
}

}  // namespace poyd
