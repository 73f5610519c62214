// Linear-gap banded direct-optimization DP on sm_103a.
//
// Restates algn_fill_plane_2 / algn_fill_plane (algn.c:812-968) with the
// per-cell rule of algn_fill_row (algn.c:375-453) and the band-edge cells of
// algn.c:461-620, plus backtrack_2d (algn.c:3551-3666), ancestor_2
// (algn.c:4126-4147) and median_2_with_gaps (algn.c:4011-4024).
//
// Layout on the GPU.  One warp owns one pair (persistent grid, pairs taken
// longest-first).  Lane k owns DP rows 64t + 2k and 64t + 2k + 1 of strip t;
// the warp sweeps the band in diagonal coordinates d = j - r, which makes
// the band edges of every row the same two diagonals [dlo, dlo+wd) (the
// reference's ukk left/right cells).  Strips follow one another without a
// pipeline ramp (the schedule is described at the band DP below): lane k's
// first row is at band index i at step tW + 3k + i and its second row at
// i - 1 in the same step.  The value of the row above at (d+1) -- the
// "delete" predecessor -- arrives from lane k-1 by one shuffle; the previous
// shuffle's value is the "align" predecessor and the lane's own previous
// value the "insert" predecessor.  Lane 0 is fed the previous strip's last
// row from a register queue that rotates one lane per step and is refilled /
// flushed with one coalesced 128-byte load / store every 32 steps (the
// boundary row lives in a per-warp global slab of wd ints).  Cells outside
// the band or the matrix hold an out-of-band value that removes exactly the
// moves the reference's edge cells omit.  Column characters come from
// per-warp shared windows, costs from a per-lane profile in shared memory
// (both row characters' costs against every column character in one word,
// laid out [char][lane] so a step's 32 lookups hit 32 banks).  Direction
// information is written per 32-step block with one coalesced store (see
// the mode notes below); the traceback addresses it by (global block, lane).
#include <cuda_runtime.h>
#include <cstdint>
#include "poyd_internal.h"
#include "linear_kernels.cuh"
#include "back_writer.cuh"

namespace poyd {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// Plan: orientation, deltaw, band geometry, DM size and band cell count.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128, 16) k_lin_plan(LinPlanArgs A) {
  const int lane = threadIdx.x & 31;
  const int id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (id >= A.n) return;
  const int la = A.a_len[id], lb = A.b_len[id];
  const int64_t ao = A.a_off[id], bo = A.b_off[id];
  const int gap = A.gap;
  unsigned ga = 0, gb = 0, na = 0, nb = 0, wide = 0, zero = 0;
  for (int x = lane; x < la; x += 32) {
    const int c = A.seq[ao + x];
    ga += (c & gap) != 0;
    na += c != gap;
    wide |= (unsigned)c >> 5;
    zero |= c == 0;
  }
  for (int x = lane; x < lb; x += 32) {
    const int c = A.seq[bo + x];
    gb += (c & gap) != 0;
    nb += c != gap;
    wide |= (unsigned)c >> 5;
    zero |= c == 0;
  }
  wide = __reduce_or_sync(kFull, wide);
  zero = __reduce_or_sync(kFull, zero);
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
    // strip period W (see the DP schedule) and the pair's 32-step blocks
    int W = (wd + 2 + kStepBlock - 1) / kStepBlock * kStepBlock;
    if (W < kMinPeriod) W = kMinPeriod;
    P.sblocks = W / kStepBlock;
    P.nblk = ((P.nstrips - 1) * W + kLag * (kLanes - 1) + 1 + wd + kStepBlock - 1) / kStepBlock;
    P.deltaw = dw;
    P.empty = 0;
    if (A.dos_empty) {
      if (na == 0) P.empty = 1;
      else if (nb == 0) P.empty = 2;
    }
    A.plans[id] = P;
    // direction-matrix words; also the work estimate used to order pairs
    int64_t words = (int64_t)P.nblk * lin_dm_words(A.with_dm == kDpChoice ? kDpChoice : kDpSets);
    // The packed kernel (linear4.cu): 128-row strips, period
    // max(roundup32(wd + 4), 288), eight words per lane and 32-step block.
    // It holds every value in 16 bits when sc * maxc * (max(l1, l2) + 260)
    // + 6 < 0xC000 (sc = 4 with backtrack moves), byte costs fit its profile
    // and no code 0 (whose table entries are unbounded) occurs; else err
    // bit 16 keeps the batch on this file's kernel.
    {
      const int W4 = max((wd + 4 + 31) / 32 * 32, 288), T4 = (l1 + 127) >> 7;
      const int64_t nblk4 = ((int64_t)(T4 - 1) * W4 + 221 + wd + 31) >> 5;
      if (A.with_dm == kDpChoice && nblk4 * 256 > words) words = nblk4 * 256;
      const int sc4 = A.with_dm == kDpChoice ? 4 : 1;
      const int lim = A.with_dm == kDpChoice ? 31 : 127;
      const long long need = (long long)sc4 * A.maxc * ((l1 > l2 ? l1 : l2) + 260) + 6;
      if (zero || A.maxc > lim || need >= 0xC000 || A.with_dm == kDpSets) atomicOr(A.err, 16);
    }
    A.dm_words[id] = words;
    A.wd_out[id] = wd;
    if (A.cells) A.cells[id] = cells;
    if (la < 1 || lb < 1) atomicOr(A.err, 1);
    if (wide) atomicOr(A.err, 4);  // codes index 32-entry table rows
    if ((long long)A.maxc * (l1 + l2 + 2) >= kMaxCost) atomicOr(A.err, 2);
  }
}

// ---------------------------------------------------------------------------
// Traceback + medians of one pair by one thread.  Run by k_lin_traceback
// (one thread per pair) or, for batched align_2, inside k_lin_dp by the warp
// that finishes the last DP of a 32-pair batch (one lane per pair).
// ---------------------------------------------------------------------------
template <int MODE>
__device__ __noinline__ void tb_pair(const LinTbArgs &A, const uint8_t *med, int id) {
  const LinPlan P = A.plans[id];
  const int gap = A.gap;
  const int la = P.swap ? P.l2 : P.l1, lb = P.swap ? P.l1 : P.l2;
  const int64_t cap = slot_cap(la, lb);
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
  int n = 0, nm = 0;
  const int wdt = P.wd;
  bool bad = false;
  // kDpChoice: the four words of one (block, lane) -- both rows of the lane,
  // 32 steps -- form one 16-byte group; the walk keeps the current group
  // (eight lanes' groups share a 128-byte line, so the next ones are
  // usually L1 hits).
  const uint4 *dm4 = (const uint4 *)dm;
  uint4 cur = make_uint4(0, 0, 0, 0);
  int cur_key = -1;
  // aligned a, aligned b and median with gaps advance together; their slots
  // are cap apart (a multiple of 4), so one writer serves the three
  BackWriter3 wabw(oa + cap - 1, ob + cap - 1, ow + cap - 1);
  BackWriter wm(om + cap - 1);
  // cell (r, j) ends the walk once r * L2 + j < 0
  while (r > 0 || (r == 0 && j >= 0)) {
    const int k = (r & (kRows - 1)) >> 1, strip = r >> 6;
    const int s = (j - r) - dlo + kLag * k + (r & 1);
    const int blk = strip * sb + (s >> 5);  // global step strip * W + s
    const int bi = (j - r) - dlo;           // band index
    if (j < 0 || bi < 0 || bi >= wdt || blk >= P.nblk || n + 2 >= cap) {  // left the band: a bug
      bad = true;
      break;
    }
    int move;  // 0 align, 1 insert (s2 against a gap), 2 delete
    if (MODE == kDpChoice) {
      const int key = blk * kLanes + k;
      if (key != cur_key) {
        cur = dm4[key];
        cur_key = key;
      }
      // 2-bit rank per step, 16 steps per word (row A: x, y; row B: z, w);
      // step s of a word is bits 2*(15 - s%16); rank 1 is insert when
      // swaped, else delete
      const uint32_t lo = (r & 1) ? cur.z : cur.x, hi = (r & 1) ? cur.w : cur.y;
      const uint32_t w = (s & 16) ? hi : lo;
      const uint32_t code = (w >> (30 - 2 * (s & 15))) & 3u;
      move = code == 0 ? 0 : (((code == 1u) == swaped) ? 1 : 2);
    } else {
      // three bit planes (align, insert, delete); step s of a block is bit 31 - s%32
      const uint32_t *w = dm + (int64_t)blk * (3 * kRows) + (r & (kRows - 1));
      const int sh = 31 - (s & 31);
      const uint32_t f = ((w[0] >> sh) & 1u) | (((w[kRows] >> sh) & 1u) << 1) |
                         (((w[2 * kRows] >> sh) & 1u) << 2);
      move = (f & 1u) ? 0 : ((swaped ? (f & 2u) : !(f & 4u)) ? 1 : 2);
    }
    const bool dr = move != 1, dj = move != 2;  // consumes a row / a column
    const int cr = dr ? (int)s1[r] : gap, cc = dj ? (int)s2[j] : gap;
    r -= dr;
    j -= dj;
    const int ca = P.swap ? cc : cr, cb = P.swap ? cr : cc;
    const int m = med[(ca << 5) | cb];
    wabw.put((uint32_t)ca, (uint32_t)cb, (uint32_t)m);
    if (m != gap) {
      wm.put((uint32_t)m);
      ++nm;
    }
    ++n;
  }
  // ancestor_2 ends with the leading gap (algn.c:4140-4141)
  wm.put((uint32_t)gap);
  ++nm;
  wabw.flush();
  wm.flush();
  A.out_len[2 * id] = bad ? -1 : (int32_t)n;
  A.out_len[2 * id + 1] = bad ? -1 : (int32_t)nm;
}

__global__ void __launch_bounds__(128) k_lin_traceback(LinTbArgs A) {
  __shared__ uint8_t med[1024];
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) med[i] = A.tables->median[i];
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.n) return;
  const int id = A.order ? A.order[t] : t;
  if (A.mode == kDpChoice) tb_pair<kDpChoice>(A, med, id);
  else tb_pair<kDpSets>(A, med, id);
}

// ---------------------------------------------------------------------------
// Band DP.
//
// Three modes share one sweep:
//   kDpCost    costs only;
//   kDpSets    also the full direction set of every cell, three bit planes
//              (align, insert, delete), for the single-pair simple_2 /
//              backtrack_2d protocol where the backtrack priority is chosen
//              after the fill;
//   kDpChoice  the move backtrack_2d will take from every cell, two bits,
//              when the priority is known before the fill (batched align_2).
//              Values are kept times four with the move's rank in the low two
//              bits (align 0; then insert 1, delete 2 when swaped, else
//              delete 1, insert 2), so one add-min chain yields the minimum
//              and, among tied moves, the one of highest priority.
// Every value is biased by cost[s1[0]][s2[0]] (cell (0,0) holds it instead
// of 0) so that all values stay non-negative; the bias is removed from the
// result.
//
// Schedule.  Lane k works on its rows 64t + 2k and 64t + 2k + 1 of strip t
// during the steps [tW + 3k, tW + 3k + W) of the pair, strip after strip
// with no pipeline ramp in between; at step tW + 3k + i its first row is at
// band index i (diagonal dlo + i) and its second row at index i - 1.
// W = max(roundup32(wd + 2), 160): the two padding diagonals put a lane's
// last steps of a strip out of band (the values it receives there from a
// lane that has moved on are never used), and 160 steps leave two blocks
// between lane 31's flush of a boundary value and lane 0's prefetch of it.
// In the 32-step block at offset o of period t (steps tW + o .. tW + o + 31)
// lane k switches from strip t-1 to strip t at step 3k - o when o < 96;
// from o = 96 on every lane is in strip t and the next strip's profile and
// parameters are prepared.  Column characters do not travel with the
// values: each block stages, per strip present, the 64 columns its lanes
// read in a per-warp window (lane k reads window[32 + u - k] at step u).
// ---------------------------------------------------------------------------
struct LinStrip {
  int HA, HB, diag, Pk, q;
  uint32_t a0, a1, a2;  // row A direction words
  uint32_t b0, b1, b2;  // row B
  int result;
};

// Per-lane parameters of one strip.
struct StripParams {
  int baseA, cntA;  // first row valid at steps [baseA, baseA + cntA)
  int baseB, cntB;  // second row likewise
  int cDA, cDB;     // delete costs of the two row characters (+ rank)
  const uint32_t *col;  // this lane's profile column
};

// Shared memory of one k_lin_dp block (dynamic: above the 48 KB static limit).
struct LinSmem {
  uint32_t ctab[32 * 33];                  // cost[a][b] at a*33 + b (rows padded one bank)
  int gcost[3][32];                        // cost[gap][b]; 4*cost[gap][b] + 1; ... + 2
  uint32_t prof[kDpWarps][2][32][kLanes];  // by strip parity, per lane: cost[aA][c] | cost[aB][c] << 16 (x4 in kDpChoice)
  uint8_t win[kDpWarps][2][64];            // column windows of a block: strip t, strip t-1
  uint8_t med[1024];                       // median table (fused traceback)
};

template <int MODE>
struct DpMode {
  static constexpr int kScale = MODE == kDpChoice ? 4 : 1;
  static constexpr int kInfV = MODE == kDpChoice ? kInfChoice : kInf;
};

// Integer work of the DP splits over two pipes that issue side by side, each
// at half a warp instruction per clock: min / select / logic / shifts run on
// the ALU pipe, while the adds, the field extraction and the packing are
// issued as multiply-adds (IMAD on the FMA pipe) through imad().  The
// multipliers are kernel arguments (DpK: 1, -1, 4, -65536), so the compiler
// cannot fold them back into ALU adds and shifts.
__device__ __forceinline__ int imad(int a, int b, int c) {
  int d;
  asm("mad.lo.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

// Appends one direction bit: (plane << 1) | [cand == h].  h is the minimum
// of the candidates, so cand - h - 1 is negative exactly when cand == h.
__device__ __forceinline__ uint32_t dir_bit(uint32_t plane, int cand, int h) {
  return __funnelshift_l((uint32_t)(cand - h - 1), plane, 1);
}

// This lane's parameters of strip s (cnt 0 outside 0 <= s < T); builds its
// profile column when asked.
template <int MODE>
__device__ __forceinline__ StripParams strip_params(const LinSmem &sm, uint32_t *col,
                                                    const uint8_t *s1, int L1, int T, int s,
                                                    int W, int dlo, int wd, int gap, int rank_d,
                                                    bool build, int lane) {
  constexpr int kScale = DpMode<MODE>::kScale;
  StripParams p;
  const int rA = s * kRows + 2 * lane, rB = rA + 1;
  const bool in = s >= 0 && s < T;
  const bool okA = in && rA < L1, okB = in && rB < L1;
  const int aA = okA ? s1[rA] : 0, aB = okB ? s1[rB] : 0;
  if (build) {
    // read back only by this lane: no warp synchronisation needed
#pragma unroll 8
    for (int c = 0; c < 32; ++c)
      col[c * kLanes] = kScale * (sm.ctab[aA * 33 + c] | (sm.ctab[aB * 33 + c] << 16));
  }
  p.cDA = kScale * (int)sm.ctab[aA * 33 + gap] + rank_d;
  p.cDB = kScale * (int)sm.ctab[aB * 33 + gap] + rank_d;
  const int offA = (-dlo - rA) > 0 ? (-dlo - rA) : 0;
  const int offB = (-dlo - rB) > 0 ? (-dlo - rB) : 0;
  p.baseA = s * W + kLag * lane + offA;
  p.cntA = okA ? wd - offA : 0;
  p.baseB = s * W + kLag * lane + 1 + offB;
  p.cntB = okB ? wd - offB : 0;
  p.col = col;
  return p;
}

// 32 steps of one block, as two runs of 16 unrolled steps (the code of the
// block variants stays small enough for the instruction cache).  KIND 0:
// every lane in strip t and inside its band for all steps; KIND 2: lane k
// uses strip t-1 (parameters Pp, window wp) before step uc and strip t (Pc,
// window wc) from it, with per-step band masks (uc = 0, Pp = Pc for a
// masked block inside one strip).  Each lane owns two rows: the first
// handles index i at a step, the second index i - 1 in the same step, so the
// second row's delete predecessor is the first row's value computed just
// before and both cells share the column character.  CAP records the final
// cell.
template <int MODE, int KIND, bool CAP>
__device__ __forceinline__ void lin_block(LinStrip &S, const StripParams &Pc,
                                          const StripParams &Pp, const uint8_t *wc,
                                          const uint8_t *wp, int uc, int G0, const int *gcost,
                                          const DpK &K, int finA, int finB, uint32_t *dmw,
                                          int lane) {
  constexpr int kInfV = DpMode<MODE>::kInfV;
  constexpr int kHalf = kStepBlock / 2;
#pragma unroll 1
  for (int e = 0; e < 2; ++e) {
    const int u0 = e * kHalf;
    const int vbAc = G0 + u0 - Pc.baseA, vbBc = G0 + u0 - Pc.baseB;
    const int vbAp = G0 + u0 - Pp.baseA, vbBp = G0 + u0 - Pp.baseB;
    const int ue = uc - u0, fA = finA - u0, fB = finB - u0;
    const uint8_t *wce = wc + u0, *wpe = wp + u0;
    uint32_t accA = 0, accB = 0;  // kDpChoice: 2-bit moves of this half
#pragma unroll
    for (int v = 0; v < kHalf; ++v) {
      int up = __shfl_up_sync(kFull, S.Pk, 1);
      if (lane == 0) up = S.q;
      S.q = __shfl_sync(kFull, S.q, (lane + 1) & 31);
      const bool nw = KIND != 2 || v >= ue;
      const int c = (nw ? wce : wpe)[v];
      const uint32_t *pcol = nw ? Pc.col : Pp.col;
      const int cDA = nw ? Pc.cDA : Pp.cDA, cDB = nw ? Pc.cDB : Pp.cDB;
      bool okA = true, okB = true;
      if (KIND == 2) {
        okA = nw ? (unsigned)(vbAc + v) < (unsigned)Pc.cntA : (unsigned)(vbAp + v) < (unsigned)Pp.cntA;
        okB = nw ? (unsigned)(vbBc + v) < (unsigned)Pc.cntB : (unsigned)(vbBp + v) < (unsigned)Pp.cntB;
      }
      const uint32_t pr = pcol[c * kLanes];  // {cost[aA][c], cost[aB][c]}
      const int g = gcost[c];                // cost[gap][c] (+ rank)
      int ha, hb;
      if (MODE == kDpSets) {
        // first row: delete from the lane above, align from its previous value
        const int Av = S.diag + (int)(pr & 0xffffu);
        const int Dv = up + cDA;
        const int Iv = S.HA + g;
        ha = min(min(Av, Dv), Iv);
        if (KIND != 0) ha = okA ? ha : kInfV;
        // second row: delete from the first row now, align from its previous value
        const int Av2 = S.HA + (int)(pr >> 16);
        const int Dv2 = ha + cDB;
        const int Iv2 = S.HB + g;
        hb = min(min(Av2, Dv2), Iv2);
        if (KIND != 0) hb = okB ? hb : kInfV;
        S.a0 = dir_bit(S.a0, Av, ha);
        S.a1 = dir_bit(S.a1, Iv, ha);
        S.a2 = dir_bit(S.a2, Dv, ha);
        S.b0 = dir_bit(S.b0, Av2, hb);
        S.b1 = dir_bit(S.b1, Iv2, hb);
        S.b2 = dir_bit(S.b2, Dv2, hb);
      } else {
        const int hi = (int)(pr >> 16);  // cost[aB][c]
        const int Av = imad(hi, K.m64k, imad((int)pr, K.one, S.diag));
        const int Iv = imad(g, K.one, S.HA);
        ha = __viaddmin_s32(up, cDA, min(Av, Iv));
        if (MODE == kDpChoice) {
          // acc * 4 + (ha & 3) as acc * 4 + ha - (ha & ~3), exact mod 2^32
          const int hc = ha & ~3;
          accA = (uint32_t)imad(hc, K.m1, imad((int)accA, K.four, ha));
          ha = hc;
        }
        if (KIND != 0) ha = okA ? ha : kInfV;
        const int Av2 = imad(hi, K.one, S.HA);
        const int Iv2 = imad(g, K.one, S.HB);
        hb = __viaddmin_s32(ha, cDB, min(Av2, Iv2));
        if (MODE == kDpChoice) {
          const int hc = hb & ~3;
          accB = (uint32_t)imad(hc, K.m1, imad((int)accB, K.four, hb));
          hb = hc;
        }
        if (KIND != 0) hb = okB ? hb : kInfV;
      }
      if (CAP) {
        if (v == fA) S.result = ha;
        if (v == fB) S.result = hb;
      }
      S.Pk = hb;
      if (lane == 31) S.q = hb;
      S.diag = up;
      S.HA = ha;
      S.HB = hb;
    }
    if (MODE == kDpChoice) {
      if (e == 0) {
        S.a0 = accA;
        S.b0 = accB;
      } else {
        S.a1 = accA;
        S.b1 = accB;
      }
    }
  }
  if (MODE == kDpSets) {
    uint2 *w = (uint2 *)dmw;
    w[0] = make_uint2(S.a0, S.b0);
    w[kLanes] = make_uint2(S.a1, S.b1);
    w[2 * kLanes] = make_uint2(S.a2, S.b2);
  } else if (MODE == kDpChoice) {
    *(uint4 *)dmw = make_uint4(S.a0, S.a1, S.b0, S.b1);
  }
}

template <int MODE>
__device__ __forceinline__ void lin_pair(const LinDpArgs &A, const LinSmem &sm, int warp,
                                         const LinPlan &P, int64_t dm_off, int id, int *bnd,
                                         int lane) {
  constexpr int kScale = DpMode<MODE>::kScale, kInfV = DpMode<MODE>::kInfV;
  constexpr int kWords = lin_dm_words(MODE);  // DM words per 32-step block
  const uint8_t *s1 = A.seq + P.s1_off;
  const uint8_t *s2 = A.seq + P.s2_off;
  const int L1 = P.l1, L2 = P.l2, dlo = P.dlo, wd = P.wd;
  const int T = P.nstrips, W = P.sblocks * kStepBlock, nblk = P.nblk;
  const int gap = A.gap;
  // backtrack priority (algn.c:3605-3666): insert before delete when swaped
  const bool swaped = A.swaped < 0 ? !P.swap : (A.swaped != 0);
  const int rank_i = MODE == kDpChoice ? (swaped ? 1 : 2) : 0;
  const int rank_d = MODE == kDpChoice ? 3 - rank_i : 0;
  const int *gcost = sm.gcost[rank_i];
  uint32_t *col0 = const_cast<uint32_t *>(&sm.prof[warp][0][0][lane]);
  uint32_t *col1 = const_cast<uint32_t *>(&sm.prof[warp][1][0][lane]);
  uint8_t *win = const_cast<uint8_t *>(&sm.win[warp][0][0]);
  // this lane's read position in the windows of strip t and strip t-1
  const uint8_t *wc = win + 32 - lane, *wp = win + 64 + 32 - lane;
  const int bias = kScale * (int)sm.ctab[s1[0] * 33 + s2[0]];

  for (int x = lane; x < wd; x += 32) bnd[x] = (x == -dlo) ? 0 : kInfV;
  __syncwarp();

  // the final cell (L1-1, L2-1): owner lane, row and step
  const int r_last = L1 - 1, d_last = L2 - L1;
  const int kf = (r_last & (kRows - 1)) >> 1, hf = r_last & 1;
  const int G_fin = (T - 1) * W + kLag * kf + (d_last - dlo) + hf;
  LinStrip S;
  S.result = 0;
  S.HA = kInfV;
  S.HB = kInfV;
  S.diag = kInfV;
  S.Pk = kInfV;
  S.a0 = S.a1 = S.a2 = S.b0 = S.b1 = S.b2 = 0;
  if (lane == 0) S.diag = bnd[0];
  uint32_t *dm = MODE != kDpCost ? A.dm + dm_off : nullptr;

  StripParams Pp = strip_params<MODE>(sm, col1, s1, L1, T, -1, W, dlo, wd, gap, rank_d, false, lane);
  StripParams Pc = strip_params<MODE>(sm, col0, s1, L1, T, 0, W, dlo, wd, gap, rank_d, true, lane);
  StripParams Pn = Pp;
  auto unmasked_range = [&](const StripParams &p, int &lo, int &hi) {
    const int l = p.baseA > p.baseB ? p.baseA : p.baseB;
    const int h = (p.baseA + p.cntA) < (p.baseB + p.cntB) ? (p.baseA + p.cntA) : (p.baseB + p.cntB);
    lo = __reduce_max_sync(kFull, l);
    hi = __reduce_min_sync(kFull, h);
  };
  int all_lo, all_hi;
  unmasked_range(Pc, all_lo, all_hi);

  // lane 0's inputs of a block: the row above its strip (the previous
  // strip's last row, from the boundary slab) at index i + 1; index W reads
  // slot 0, the new strip's first align predecessor
  // (blocks are addressed by period t and offset o: G0 = t * W + o)
  auto qload = [&](int o) -> int {
    int x = o + lane + 1;
    if (x == W) x = 0;
    return (x < wd) ? bnd[x] : kInfV;
  };
  // this lane's two bytes of the column windows of the block at (t, o)
  auto wload = [&](int t, int o, uint32_t &cw, uint32_t &pw) {
    const int jc = t * kRows + dlo + o - 32 + lane;  // strip t
    const int jp = jc - kRows + W;                   // strip t-1
    const int c0 = (jc >= 0 && jc < L2) ? s2[jc] : 0;
    const int c1 = (jc + 32 >= 0 && jc + 32 < L2) ? s2[jc + 32] : 0;
    const int p0 = (jp >= 0 && jp < L2) ? s2[jp] : 0;
    const int p1 = (jp + 32 >= 0 && jp + 32 < L2) ? s2[jp + 32] : 0;
    cw = (uint32_t)c0 | ((uint32_t)c1 << 8);
    pw = (uint32_t)p0 | ((uint32_t)p1 << 8);
  };
  auto wstore = [&](uint32_t cw, uint32_t pw) {
    __syncwarp();
    win[lane] = (uint8_t)cw;
    win[lane + 32] = (uint8_t)(cw >> 8);
    win[64 + lane] = (uint8_t)pw;
    win[64 + lane + 32] = (uint8_t)(pw >> 8);
    __syncwarp();
  };
  S.q = qload(0);
  {
    uint32_t cw, pw;
    wload(0, 0, cw, pw);
    wstore(cw, pw);
  }

  int t0 = 0, o = 0;
  for (int b = 0; b < nblk; ++b, o += kStepBlock) {
    if (o == W) {
      o = 0;
      ++t0;
    }
    const int G0 = b * kStepBlock;
    if (b > 0 && o == 0) {  // a new period: strip t0 becomes current
      Pp = Pc;
      Pc = Pn;
      unmasked_range(Pc, all_lo, all_hi);
    }
    if (o == 96)  // every lane is in strip t0: prepare strip t0 + 1
      Pn = strip_params<MODE>(sm, ((t0 + 1) & 1) ? col1 : col0, s1, L1, T, t0 + 1, W, dlo, wd,
                              gap, rank_d, t0 + 1 < T, lane);
    const int o1 = (o + kStepBlock == W) ? 0 : o + kStepBlock;  // the next block
    const int t1 = (o1 == 0) ? t0 + 1 : t0;
    const int qn = qload(o1);
    uint32_t cw, pw;
    wload(t1, o1, cw, pw);
    uint32_t *dmw = MODE == kDpCost ? nullptr
                  : dm + (int64_t)b * kWords + (MODE == kDpSets ? 2 * lane : 4 * lane);
    const bool cap = G_fin >= G0 && G_fin < G0 + kStepBlock;
    const int finA = (cap && lane == kf && hf == 0) ? G_fin - G0 : -1;
    const int finB = (cap && lane == kf && hf == 1) ? G_fin - G0 : -1;
    if (o < 96) {
      const int uc = kLag * lane - o;
      if (cap)
        lin_block<MODE, 2, true>(S, Pc, Pp, wc, wp, uc, G0, gcost, A.k, finA, finB, dmw, lane);
      else
        lin_block<MODE, 2, false>(S, Pc, Pp, wc, wp, uc, G0, gcost, A.k, -1, -1, dmw, lane);
    } else if (cap) {
      lin_block<MODE, 2, true>(S, Pc, Pc, wc, wc, 0, G0, gcost, A.k, finA, finB, dmw, lane);
    } else if (G0 >= all_lo && G0 + kStepBlock <= all_hi) {
      lin_block<MODE, 0, false>(S, Pc, Pc, wc, wc, 0, G0, gcost, A.k, -1, -1, dmw, lane);
    } else {
      lin_block<MODE, 2, false>(S, Pc, Pc, wc, wc, 0, G0, gcost, A.k, -1, -1, dmw, lane);
    }
    // lane 31's second-row values of this block (lane L holds step G0 + L)
    // become the boundary row of the next strip
    {
      const int pA = G0 + lane - kLag * 31;  // lane 31's first-row position
      const int x = (pA >= t0 * W ? pA - t0 * W : pA - (t0 - 1) * W) - 1;
      if (pA >= 0 && x >= 0 && x < wd) bnd[x] = S.q;
    }
    S.q = qn;
    wstore(cw, pw);
  }
  const int result = __shfl_sync(kFull, S.result, kf);
  if (lane == 0) A.cost[id] = (result - bias) / kScale;
}

template <int MODE>
__global__ void __launch_bounds__(kDpWarps * 32, 3) k_lin_dp(LinDpArgs A) {
  extern __shared__ __align__(16) unsigned char lin_dsm[];
  LinSmem &sm = *reinterpret_cast<LinSmem *>(lin_dsm);
  for (int i = threadIdx.x; i < 1024; i += blockDim.x)
    sm.ctab[(i >> 5) * 33 + (i & 31)] = A.tables->packed[i] & 0xffffu;
  if (MODE == kDpChoice && A.fuse_tb)
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) sm.med[i] = A.tables->median[i];
  if (threadIdx.x < 32) {
    const int g = (int)(A.tables->packed[threadIdx.x] >> 16);
    sm.gcost[0][threadIdx.x] = g;
    sm.gcost[1][threadIdx.x] = 4 * g + 1;
    sm.gcost[2][threadIdx.x] = 4 * g + 2;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
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
    } else {
      lin_pair<MODE>(A, sm, warp, P, MODE != kDpCost ? A.dm_off[id] : 0, id, bnd, lane);
    }
    if (MODE == kDpChoice && A.fuse_tb) {
      // Publish this pair's direction matrix; the warp completing the batch
      // (no waiting: the count tells) walks all of its pairs, one per lane.
      __syncwarp();
      const int b = p / kLanes;
      const int size = min(kLanes, A.n - b * kLanes);
      int last = 0;
      if (lane == 0) {
        __threadfence();
        last = atomicAdd(A.batch_done + b, 1) == size - 1;
      }
      if (__shfl_sync(kFull, last, 0)) {
        __threadfence();
        if (lane < size)
          tb_pair<kDpChoice>(A.tb, sm.med, A.order ? A.order[b * kLanes + lane] : b * kLanes + lane);
        if (A.done) {
          // every lane's results visible to the host before the flag
          __threadfence_system();
          __syncwarp();
          if (lane == 0) *(volatile int *)(A.done + b) = 1;
        }
        __syncwarp();
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Packing of batched align_2 results: one warp per pair copies the used tail
// of each of its four right-aligned slots back to back.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128, 16) k_pack_alignments(int n, const uint8_t *out, const int64_t *out_off,
                                  const int32_t *a_len, const int32_t *b_len,
                                  const int32_t *out_len, uint8_t *packed,
                                  const int64_t *packed_off) {
  const int lane = threadIdx.x & 31;
  const int64_t id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (id >= n) return;
  const int64_t cap = slot_cap(a_len[id], b_len[id]);
  const int64_t na = out_len[2 * id], nm = out_len[2 * id + 1];
  const uint8_t *src = out + out_off[id];
  uint8_t *dst = packed + packed_off[id];
  for (int k = 0; k < 4; ++k) {
    const int64_t len = k < 3 ? na : nm;
    const uint8_t *s = src + (k + 1) * cap - len;
    uint8_t *d = dst + (k < 3 ? k * na : 3 * na);
    for (int64_t x = lane; x < len; x += 32) d[x] = s[x];
  }
}

void launch_pack_alignments(int n, const uint8_t *out, const int64_t *out_off,
                            const int32_t *a_len, const int32_t *b_len,
                            const int32_t *out_len, uint8_t *packed,
                            const int64_t *packed_off, cudaStream_t st) {
  // 128-thread blocks (<= 32 registers each) fit in the registers a
  // resident k_lin_dp grid leaves free on every SM, so a pipelined caller's
  // pack runs beside the next chunk's DP instead of after it
  const int threads = 128;
  const int64_t blocks = ((int64_t)n * 32 + threads - 1) / threads;
  k_pack_alignments<<<(unsigned)blocks, threads, 0, st>>>(n, out, out_off, a_len, b_len,
                                                          out_len, packed, packed_off);
}

// ---------------------------------------------------------------------------
// Device-side ordering: longest first by log2 buckets, disjoint direction
// matrices (their placement does not follow the order: each pair's DP
// writes only its own region).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int order_bucket(const LinPlan &P) {
  const unsigned long long work = (unsigned long long)P.nstrips * (unsigned)P.sblocks + 1;
  const int lz = __clzll((long long)work);
  const int lg = 63 - lz;                                     // floor(log2(work))
  const int frac = (int)((work << lz) >> 58) & 31;            // next 5 bits
  const int b = min(lg * 32 + frac, 1023);
  return 1023 - b;                                            // most work first
}

__global__ void __launch_bounds__(128, 16) k_order_count(int n, const LinPlan *plans,
                                                        const int64_t *dm_words, int64_t *dm_off,
                                                        LinOrderScratch *os) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool ok = id < n;
  int wd = 0;
  unsigned long long w = 0;
  if (ok) {
    const LinPlan P = plans[id];
    atomicAdd(&os->hist[order_bucket(P)], 1);
    wd = P.wd;
    w = (unsigned long long)dm_words[id];
  }
  // warp-aggregated region allocation and widest band
  unsigned long long incl = w;
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long x = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += x;
  }
  unsigned long long base = 0;
  if (lane == 31) base = atomicAdd(&os->total, incl);
  base = __shfl_sync(0xffffffffu, base, 31);
  if (ok) dm_off[id] = (int64_t)(base + incl - w);
  for (int d = 16; d > 0; d >>= 1) wd = max(wd, __shfl_xor_sync(0xffffffffu, wd, d));
  if (lane == 0) atomicMax(&os->maxwd, wd);
}

__global__ void __launch_bounds__(1024) k_order_scan(LinOrderScratch *os) {
  __shared__ int part[32];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int v = os->hist[t];
  int incl = v;
  for (int d = 1; d < 32; d <<= 1) {
    const int x = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += x;
  }
  if (lane == 31) part[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int p = part[lane];
    for (int d = 1; d < 32; d <<= 1) {
      const int x = __shfl_up_sync(0xffffffffu, p, d);
      if (lane >= d) p += x;
    }
    part[lane] = p;  // inclusive over warps
  }
  __syncthreads();
  os->base[t] = (warp ? part[warp - 1] : 0) + incl - v;
  os->hist[t] = 0;  // now the scatter cursor
}

__global__ void __launch_bounds__(128, 16) k_order_scatter(int n, const LinPlan *plans,
                                                          LinOrderScratch *os, int32_t *order) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= n) return;
  const int b = order_bucket(plans[id]);
  order[os->base[b] + atomicAdd(&os->hist[b], 1)] = id;
}

// Small batches (at most 1,024 pairs; every pair has its own warp, so the
// longest-first order buys nothing): one block lays the direction matrices
// out in id order, finds the widest band and zeroes the DP's counters, in
// place of the bucketed order's three launches and two memsets.
__global__ void __launch_bounds__(1024) k_order_small(int n, const LinPlan *plans,
                                                      const int64_t *dm_words, int64_t *dm_off,
                                                      LinOrderScratch *os, int *counter,
                                                      int *batch_done, int nbatch) {
  __shared__ unsigned long long part[32];
  __shared__ int wmax[32];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const unsigned long long w = t < n ? (unsigned long long)dm_words[t] : 0ull;
  int wd = t < n ? plans[t].wd : 0;
  unsigned long long incl = w;
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long x = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += x;
  }
  for (int d = 16; d > 0; d >>= 1) wd = max(wd, __shfl_xor_sync(0xffffffffu, wd, d));
  if (lane == 31) part[warp] = incl;
  if (lane == 0) wmax[warp] = wd;
  __syncthreads();
  if (warp == 0) {
    unsigned long long p = part[lane];
    int m = wmax[lane];
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long x = __shfl_up_sync(0xffffffffu, p, d);
      if (lane >= d) p += x;
    }
    for (int d = 16; d > 0; d >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, d));
    part[lane] = p;  // inclusive over warps
    if (lane == 0) wmax[0] = m;
  }
  __syncthreads();
  if (t < n) dm_off[t] = (int64_t)((warp ? part[warp - 1] : 0ull) + incl - w);
  if (t == 0) {
    os->total = part[31];
    os->maxwd = wmax[0];
    *counter = 0;
  }
  if (batch_done)
    for (int i = t; i < nbatch; i += blockDim.x) batch_done[i] = 0;
}

void launch_lin_order_small(int n, const LinPlan *plans, const int64_t *dm_words,
                            int64_t *dm_off, LinOrderScratch *os, int *counter, int *batch_done,
                            int nbatch, cudaStream_t st) {
  k_order_small<<<1, 1024, 0, st>>>(n, plans, dm_words, dm_off, os, counter, batch_done, nbatch);
}

void launch_lin_order(int n, const LinPlan *plans, const int64_t *dm_words, int64_t *dm_off,
                      LinOrderScratch *os, int32_t *order, cudaStream_t st) {
  const int threads = 128;
  const unsigned blocks = (unsigned)(((int64_t)n + threads - 1) / threads);
  k_order_count<<<blocks, threads, 0, st>>>(n, plans, dm_words, dm_off, os);
  k_order_scan<<<1, 1024, 0, st>>>(os);
  k_order_scatter<<<blocks, threads, 0, st>>>(n, plans, os, order);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_lin_plan(const LinPlanArgs &A, cudaStream_t st) {
  const int threads = 128;  // fits beside a resident k_lin_dp grid (see above)
  const int64_t blocks = ((int64_t)A.n * 32 + threads - 1) / threads;
  k_lin_plan<<<(unsigned)blocks, threads, 0, st>>>(A);
}

// Opts k_lin_dp<MODE> in to its dynamic shared memory (once per device).
template <int MODE>
static void lin_dp_optin(int dev) {
  static int done[64] = {};
  if (!done[dev & 63]) {
    cudaFuncSetAttribute(k_lin_dp<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(LinSmem));
    done[dev & 63] = 1;
  }
}

template <int MODE>
static int lin_dp_prepare(int dev) {
  lin_dp_optin<MODE>(dev);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lin_dp<MODE>, kDpWarps * 32,
                                                sizeof(LinSmem));
  return per_sm;
}

int lin_dp_blocks(int mode) {
  static int cache[3][64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  int &c = cache[mode][dev & 63];
  if (!c) {
    int per_sm = mode == kDpSets ? lin_dp_prepare<kDpSets>(dev)
               : mode == kDpChoice ? lin_dp_prepare<kDpChoice>(dev) : lin_dp_prepare<kDpCost>(dev);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    c = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  return c;
}

void launch_lin_dp(const LinDpArgs &A, int mode, int blocks, cudaStream_t st) {
  const size_t sm = sizeof(LinSmem);
  int dev = 0;
  cudaGetDevice(&dev);
  if (mode == kDpSets) lin_dp_optin<kDpSets>(dev);
  else if (mode == kDpChoice) lin_dp_optin<kDpChoice>(dev);
  else lin_dp_optin<kDpCost>(dev);
  if (mode == kDpSets) k_lin_dp<kDpSets><<<blocks, kDpWarps * 32, sm, st>>>(A);
  else if (mode == kDpChoice) k_lin_dp<kDpChoice><<<blocks, kDpWarps * 32, sm, st>>>(A);
  else k_lin_dp<kDpCost><<<blocks, kDpWarps * 32, sm, st>>>(A);
}

void launch_lin_traceback(const LinTbArgs &A, cudaStream_t st) {
  const int threads = 128;
  k_lin_traceback<<<(A.n + threads - 1) / threads, threads, 0, st>>>(A);
}

}  // namespace poyd
