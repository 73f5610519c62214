// Affine-gap ("3 matrix", 4-state) banded DO on sm_103a.
//
// Restates algn_fill_plane_3_aff_nobt / algn_fill_plane_3_aff
// (algn.c:2287-2548) with the FILL_* cell rules (algn.c:1740-1977) and
// ASSIGN_MINIMUM (algn.c:2251-2280), initialize_matrices_affine[_nobt]
// (algn.c:2124-2248) and backtrace_affine (algn.c:1983-2097), as run by
// algn_CAML_cost_affine_3 / algn_CAML_align_affine_3 (algn.c:2551-2680):
// rows are the shorter sequence si, columns the longer sj.
//
// The band of row i is columns [max(1, i-39), min(e0+i-1, lenj)] with a
// vertical boundary cell just left of it and, while the band has not
// reached lenj, a HIGH_NUM boundary cell just right of it.  In diagonal
// coordinates d = j - i that is d in [-40, e0] for every row.  A group of
// kAffRows lanes sweeps one pair's band (a warp runs 32 / kAffRows pairs
// side by side): lane k of the group owns row kAffRows*strip+k and handles
// diagonal d at step d + 40 + 2k.  The four states (EH, EV, EB, CB) of row
// i-1 at column j arrive from lane k-1 by shuffles; the column quantities
// come from a shared window staged per 32-step block; lane 0 of the group
// reads the previous strip's last row from a per-group global slab of
// 16-byte records.  The bt variant packs the bits backtrace_affine reads
// into one byte per cell (4 cells per word, kAffRows words per strip and
// 4-step column).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <numeric>
#include <vector>
#include "affine_kernels.cuh"
#include "back_writer.cuh"

namespace poyd {

namespace {

constexpr unsigned kFullA = 0xffffffffu;
constexpr int kHigh = 1000000;  // HIGH_NUM (algn.c:38)
constexpr int kStart = 40;      // start_v (algn.c:2291)
constexpr int kDlo = -40;
// Rows per strip: one per lane of a lane group; a warp runs kAffGroups
// pairs side by side, one per group (the strips' pipeline ramp is
// 2 * (kAffRows - 1) steps, against an ~85-diagonal band).
constexpr int kAffRows = 8;
constexpr int kAffGroups = 32 / kAffRows;  // pairs per warp
constexpr int kAffWarps = 4;                // warps per block (24 per SM)

// One-byte direction code: bits 0-1 the m_todo choice (0 H, 1 A, 2 V, 3 D:
// DO_HORIZONTAL > DO_ALIGN > DO_VERTICAL > DO_DIAGONAL, algn.c:2005-2012),
// bit 2 END_VERTICAL, bit 3 END_HORIZONTAL, bit 4 END_BLOCK, bits 5-6 the
// m_align choice (0 H, 1 D, 2 V, 3 none: ALIGN_TO_HORIZONTAL >
// ALIGN_TO_DIAGONAL > ALIGN_TO_VERTICAL, algn.c:2049-2051).
constexpr uint32_t kCodeLeft = 2u | 4u | (3u << 5);   // DO_VERTICAL | END_VERTICAL
constexpr uint32_t kCodeRight = 0u | 8u | (3u << 5);  // DO_HORIZONTAL | END_HORIZONTAL

struct AffPlan {
  int64_t si_off, sj_off;
  int32_t leni, lenj;  // rows 0..leni (si), columns 0..lenj (sj)
  int32_t e0, wd;
  int32_t swap;        // 1: rows are the caller's b
  int32_t nstrips, sblocks;  // sblocks: 4-step DM words per lane per strip
  int32_t empty;
  int32_t pad_[4];
};
static_assert(sizeof(AffPlan) == 64, "AffPlan layout");

struct AffPlanArgs {
  int n;
  const uint8_t *seq;
  const int64_t *a_off;
  const int32_t *a_len;
  const int64_t *b_off;
  const int32_t *b_len;
  int gap;
  int dos_empty;
  long long maxc;
  AffPlan *plans;
  int64_t *dm_words;
  int32_t *wd_out;
  int64_t *cells;
  int32_t *err;
};

struct AffDpArgs {
  int n;
  const uint8_t *seq;
  const AffPlan *plans;
  const int64_t *dm_off;
  const int32_t *order;
  const DevTables *tables;
  int go;
  int *counter;
  int4 *scratch;
  int64_t slab;
  uint32_t *dm;
  int32_t *cost;
  int32_t *err;  // k_aff_dp2: bit 8 when a final cost is past its exact range
};

struct AffTbArgs {
  int n;
  const uint8_t *seq;
  const AffPlan *plans;
  const int64_t *dm_off;
  const uint32_t *dm;
  const DevTables *tables;
  uint8_t *out;
  const int64_t *out_off;
  int32_t *out_len;
};

__global__ void k_aff_plan(AffPlanArgs A) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= A.n) return;
  const int la = A.a_len[id], lb = A.b_len[id];
  const int64_t ao = A.a_off[id], bo = A.b_off[id];
  const int swap = la > lb;  // rows = shorter (algn.c:2595-2617)
  const int li = swap ? lb : la, lj = swap ? la : lb;
  const int leni = li - 1, lenj = lj - 1;
  int e0 = (lenj - leni) + 8;
  if (e0 < 40) e0 = 40;
  if (e0 > lenj) e0 = lenj;
  AffPlan P;
  P.si_off = swap ? bo : ao;
  P.sj_off = swap ? ao : bo;
  P.leni = leni; P.lenj = lenj; P.e0 = e0;
  P.wd = e0 - kDlo + 1;
  P.swap = swap;
  P.nstrips = (leni + 1 + kAffRows - 1) / kAffRows;
  const int S = P.wd + 2 * (kAffRows - 1);
  const int Spad = (S + 15) / 16 * 16;  // whole 16-step half blocks
  P.sblocks = Spad / 4;
  P.empty = 0;
  if (A.dos_empty) {
    bool ea = true, eb = true;
    for (int x = 0; x < la && ea; ++x) ea = A.seq[ao + x] == A.gap;
    for (int x = 0; x < lb && eb; ++x) eb = A.seq[bo + x] == A.gap;
    P.empty = ea ? 1 : (eb ? 2 : 0);
  }
  for (int t = 0; t < 4; ++t) P.pad_[t] = 0;
  A.plans[id] = P;
  A.dm_words[id] = (int64_t)P.nstrips * P.sblocks * kAffRows;
  A.wd_out[id] = P.wd;
  if (A.cells) {
    long long c = lenj + 1;
    for (int i = 1; i <= leni; ++i) {
      const int s = i > kStart ? i - kStart + 1 : 1;
      int e = e0 + i - 1;
      if (e > lenj) e = lenj;
      c += e - s + 1;
    }
    A.cells[id] = c;
  }
  if (la < 1 || lb < 1) atomicOr(A.err, 1);
  unsigned wide = 0;  // codes index 32-entry table rows
  for (int x = 0; x < la; ++x) wide |= A.seq[ao + x];
  for (int x = 0; x < lb; ++x) wide |= A.seq[bo + x];
  if (wide >> 5) atomicOr(A.err, 4);
  // real costs must stay clear of the HIGH_NUM sentinel arithmetic
  if (A.maxc * (long long)(la + lb + 2) >= (1 << 22)) atomicOr(A.err, 2);
}

// Shared memory of one k_aff_dp block.
struct AffSmem {
  uint32_t tab[1024];            // packed {cost[a][b], cost[gap][b]}
  uint16_t cost[1024];           // cost[a][b]
  int4 col[kAffWarps][kAffGroups][64];   // per lane group: the columns of a 32-step block (AffCol)
  int4 ring_in[kAffWarps][kAffGroups][32];   // per lane group: its first lane's inputs of the block
  int4 ring_out[kAffWarps][kAffGroups][32];  // per lane group: its last lane's states of the block
};

// Column quantities of column j (algn.c:2321-2328 / 2451-2457), computed
// once per column when a block's window is staged:
//   x = hext: the horizontal extension cost into column j
//   y = sj_open + sj_ext: the horizontal opening cost
//   z = sj_open
//   w = sj[j]
__device__ __forceinline__ int4 aff_column(const uint32_t *tab, int jc, int jp, int j, int go) {
  const int sj_ext = (int)(tab[jc] >> 16);  // prepend[jc] = cost[gap][jc]
  const int sj_open = (!(jp & 16) && (jc & 16)) ? 0 : go;
  const int hext = (j == 1) ? sj_ext : (((jp & 16) && !(jc & 16)) ? sj_open + sj_ext : sj_ext);
  return make_int4(hext, sj_open + sj_ext, sj_open, jc);
}

// 16 steps of one strip of a lane group (`lane` is the lane in the group,
// the row in the strip): cells (i, j = i + d) with d = kDlo + s - 2 * lane at
// step s = s0 + u.  The four states of row i-1 at column j come from lane
// k-1 by shuffles (lane 0: from ring_in, the previous strip's last row), the
// column characters from the block's window, and lane 31's states go to
// ring_out.  The cell rules restate FILL_EXTEND_HORIZONTAL / _VERTICAL /
// _BLOCK_DIAGONAL[_NOBT], FILL_CLOSE_BLOCK_DIAGONAL and ASSIGN_MINIMUM
// (algn.c:1740-1977, 2251-2280); the boundary cells restate
// initialize_matrices_affine[_nobt] and the band edges of
// algn_fill_plane_3_aff[_nobt] (algn.c:2124-2248, 2309-2400).
struct AffRow {
  int ic, ip, si_ext, si_open, si_vext, i;
  int icg;                 // ic has the gap bit: all ones, else 0
  const uint16_t *srow;    // cost[ic & 15][.]
  int uL, uR, uF;  // steps (relative to the half block) of the left / right boundary cell and of the final cell
};
struct AffState {
  int eh_l, cb_l;                  // this row's previous cell (horizontal predecessor)
  int eh_d, ev_d, eb_d, cb_d;      // row above, previous column (diagonal predecessor)
  int m_eh, m_ev, m_eb, m_cb;      // this row's last cell, for the lane below
  uint32_t word;
  int result;
};

// ENDS: the strip holds row 0 or the last row (their boundary rules and the
// final cell are checked only there).
template <bool BT, bool ENDS>
__device__ __forceinline__ void aff_half(AffState &S, const AffRow &R, const AffSmem &sm,
                                         const int4 *clane, const int4 *rin, int4 *rout,
                                         int s0, int go, uint32_t *dmb, int lane) {
  const int v_open = R.si_open + R.si_ext;
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    int u_eh = __shfl_up_sync(kFullA, S.m_eh, 1, kAffRows);
    int u_ev = __shfl_up_sync(kFullA, S.m_ev, 1, kAffRows);
    int u_eb = __shfl_up_sync(kFullA, S.m_eb, 1, kAffRows);
    int u_cb = __shfl_up_sync(kFullA, S.m_cb, 1, kAffRows);
    if (lane == 0) {
      const int4 v = rin[u];
      u_eh = v.x; u_ev = v.y; u_eb = v.z; u_cb = v.w;
    }
    const int4 D = clane[u];  // this lane's column at this step
    const int jc = D.w, sj_open = D.z;
    // FILL_EXTEND_HORIZONTAL
    const int e1 = S.eh_l + D.x, e2 = S.cb_l + D.y;
    int eh = min(e1, e2);
    // FILL_EXTEND_VERTICAL
    const int v1 = u_ev + R.si_vext, v2 = u_cb + v_open;
    int ev = min(v1, v2);
    // FILL_EXTEND_BLOCK_DIAGONAL[_NOBT]; _NOBT's open cost is 2 * go when
    // both characters carry the gap bit (its no-open case needs sj[j] without it)
    const bool both = R.icg && (jc & 16);
    const int dg = both ? 0 : kHigh;
    const int od = BT ? dg : (both ? 2 * go : kHigh);
    const int b1 = S.eb_d + dg, b2 = S.cb_d + od;
    int eb = min(b1, b2);
    // FILL_CLOSE_BLOCK_DIAGONAL
    const int cdiag = (int)R.srow[jc & 15];
    const int extra = max(sj_open, R.si_open);
    const int fa = S.cb_d + cdiag;
    const int fv = S.ev_d + cdiag + (sj_open & R.icg);
    const int fh = S.eh_d + cdiag + ((jc & 16) ? R.si_open : 0);
    const int fd = S.eb_d + cdiag + extra;
    int cb = min(min(fa, fv), min(fh, fd));
    // ASSIGN_MINIMUM
    int f = min(min(eh, ev), min(eb, cb));
    uint32_t code = 0;
    if (BT) {
      // among tied states: DO_HORIZONTAL > DO_ALIGN > DO_VERTICAL > DO_DIAGONAL
      // (algn.c:2005-2012); ALIGN_TO_HORIZONTAL > _DIAGONAL > _VERTICAL
      // (algn.c:2049-2051)
      const uint32_t todo = eh == f ? 0u : (cb == f ? 1u : (ev == f ? 2u : 3u));
      const uint32_t achoice = fh == cb ? 0u : (fd == cb ? 1u : (fv == cb ? 2u : 3u));
      code = todo | (v1 < v2 ? 0u : 4u) | (e1 < e2 ? 0u : 8u) | (b1 < b2 ? 0u : 16u) |
             (achoice << 5);
    }
    if (ENDS && R.i == 0) {  // initialize_matrices_affine row 0 (j = d there)
      if (kDlo + s0 + u - 2 * lane == 0) { eh = go; ev = go; eb = 0; cb = 0; f = 0; }
      else { eh = S.eh_l + (D.y - sj_open); cb = eh; eb = kHigh; ev = kHigh; f = eh; }
    } else if (u == R.uL) {  // vertical boundary cell left of the band
      eh = kHigh; cb = kHigh; eb = kHigh; ev = v1; f = ev;
      code = kCodeLeft;
    } else if (u == R.uR) {  // HIGH_NUM cell right of the band
      eh = kHigh; ev = kHigh; eb = kHigh; cb = kHigh;
      code = kCodeRight;
    }
    if (ENDS && u == R.uF) S.result = f;
    if (BT) {
      S.word = (S.word << 8) | code;
      if ((u & 3) == 3 && dmb) dmb[(u >> 2) * kAffRows] = S.word;
    }
    S.m_eh = eh; S.m_ev = ev; S.m_eb = eb; S.m_cb = cb;
    if (lane == kAffRows - 1) rout[u] = make_int4(eh, ev, eb, cb);
    S.eh_d = u_eh; S.ev_d = u_ev; S.eb_d = u_eb; S.cb_d = u_cb;
    S.eh_l = eh; S.cb_l = cb;
  }
}

// kAffGroups pairs per warp, one per group of kAffRows lanes (kAffRows-row
// strips).  Every group runs the same strip / block / half-block loop, to
// the largest pair's bounds; a group whose pair has no strip or step left
// computes cells that nothing reads and writes no direction word, boundary
// record or cost.
template <bool BT>
__device__ __forceinline__ void aff_pair(const AffDpArgs &A, AffSmem &sm, int warp,
                                         const AffPlan &P, bool has, int64_t dm_off, int id,
                                         int4 *bnd, int lane) {
  const int h = lane / kAffRows, k = lane & (kAffRows - 1);
  const uint8_t *si = A.seq + P.si_off;
  const uint8_t *sj = A.seq + P.sj_off;
  const int leni = P.leni, lenj = P.lenj, e0 = P.e0, wd = P.wd, go = A.go;
  const int Th = has ? P.nstrips : 0, Sh = has ? P.sblocks * 4 : 0;
  const int T = __reduce_max_sync(kFullA, Th);  // the largest pair of the warp
  int4 *win = sm.col[warp][h];
  int4 *rin = sm.ring_in[warp][h], *rout = sm.ring_out[warp][h];
  // this lane's column j at block step u is window index 16 + u - k
  const int4 *wl = win + kAffRows - k;
  const int4 kHigh4 = make_int4(kHigh, kHigh, kHigh, kHigh);
  AffState S;
  S.result = 0;
  uint32_t *dm = BT ? A.dm + dm_off : nullptr;

  for (int strip = 0; strip < T; ++strip) {
    const bool act = strip < Th;
    const int Spad = __reduce_max_sync(kFullA, act ? Sh : 0);  // the same in every group
    const bool ends = __any_sync(kFullA, strip == 0 || strip == Th - 1);
    const int r0 = strip * kAffRows;
    AffRow R;
    R.i = r0 + k;
    const bool rowok = act && R.i <= leni;
    R.ic = rowok ? si[R.i] : 0;
    R.ip = (rowok && R.i > 0) ? si[R.i - 1] : 0;
    R.si_ext = (int)(sm.tab[(R.ic << 5) | 16] & 0xffffu);
    R.si_open = (!(R.ip & 16) && (R.ic & 16)) ? 0 : go;
    R.si_vext = (R.i > 1 && (R.ip & 16) && !(R.ic & 16)) ? R.si_open + R.si_ext : R.si_ext;
    R.srow = sm.cost + ((R.ic & 15) << 5);
    R.icg = (R.ic & 16) ? -1 : 0;
    const int d_lb = (-R.i > kDlo) ? -R.i : kDlo;
    const bool has_rb = e0 <= lenj - R.i;
    const int sL = d_lb - kDlo + 2 * k;
    const int sR = has_rb ? e0 - kDlo + 2 * k : -1000000;
    const int sF = (act && R.i == leni) ? (lenj - leni) - kDlo + 2 * k : -1000000;

    S.eh_l = kHigh; S.cb_l = kHigh;
    S.eh_d = kHigh; S.ev_d = kHigh; S.eb_d = kHigh; S.cb_d = kHigh;
    S.m_eh = kHigh; S.m_ev = kHigh; S.m_eb = kHigh; S.m_cb = kHigh;
    S.word = 0;
    if (k == 0 && act && strip > 0) {
      const int4 v = bnd[0];
      S.eh_d = v.x; S.ev_d = v.y; S.eb_d = v.z; S.cb_d = v.w;
    }
    for (int s0 = 0; s0 < Spad; s0 += 32) {
      // stage the block: the first lane's inputs bnd[s + 1], the 64 columns
      // r0 - 40 + s0 - 16 + x (x = 0..63); the last lane's states go to ring_out
      __syncwarp();
      {
        auto chr = [&](int j) { return (j >= 0 && j <= lenj) ? (int)sj[j] : 0; };
        const int jb = r0 + kDlo + s0 - kAffRows;
#pragma unroll
        for (int e = k; e < 32; e += kAffRows) {
          const int x = s0 + e + 1;
          rin[e] = (act && strip > 0 && x < wd) ? bnd[x] : kHigh4;
        }
        // window index 0 is read only as the predecessor of index 1
#pragma unroll
        for (int x = k; x < 64; x += kAffRows)
          win[x] = aff_column(sm.tab, chr(jb + x), chr(jb + x - 1), jb + x, go);
      }
      __syncwarp();
      uint32_t *dmb = (BT && act) ? dm + ((int64_t)strip * P.sblocks + (s0 >> 2)) * kAffRows + k
                                  : nullptr;
#pragma unroll 1
      for (int hh = 0; hh < 2; ++hh) {
        const int hs = s0 + 16 * hh;
        if (hs >= Spad) break;  // a strip may end on a half block; the last
                                // lane's positions past the band are not copied out
        R.uL = sL - hs;
        R.uR = sR - hs;
        R.uF = sF - hs;
        uint32_t *dmh = (dmb && hs < Sh) ? dmb + 4 * kAffRows * hh : nullptr;
        if (ends)
          aff_half<BT, true>(S, R, sm, wl + 16 * hh, rin + 16 * hh, rout + 16 * hh, hs, go, dmh, k);
        else
          aff_half<BT, false>(S, R, sm, wl + 16 * hh, rin + 16 * hh, rout + 16 * hh, hs, go, dmh, k);
      }
      __syncwarp();
#pragma unroll
      for (int e = k; e < 32; e += kAffRows) {
        const int x = s0 + e - 2 * (kAffRows - 1);  // the last lane's band index at block step e
        if (act && x >= 0 && x < wd) bnd[x] = rout[e];
      }
    }
    __syncwarp();
  }
  const int r = __shfl_sync(kFullA, S.result, h * kAffRows + (leni & (kAffRows - 1)));
  if (k == 0 && has) A.cost[id] = r;
}

// ---------------------------------------------------------------------------
// Packed affine DP (k_aff_dp2): two pairs per lane group, pair A in the low
// 16-bit half of every register and pair B in the high half, so one
// instruction advances two cells.  Values are kept times four with the two
// low bits free: every minimum takes its candidates tagged with the rank
// the reference's tie rule gives them, so the winner's rank is the choice
// and clearing the bits gives the value:
//   todo   = min(EH|0, CB|1, EV|2, EB|3)         (DO_HORIZONTAL > DO_ALIGN >
//                                                 DO_VERTICAL > DO_DIAGONAL)
//   achoice = min(fh|0, fd|1, fv|2, fa|3)        (ALIGN_TO_HORIZONTAL >
//                                                 _DIAGONAL > _VERTICAL)
//   END_x  = the opening candidate (rank 0) wins ties against the
//            extension (rank 1): `ext < open ? 0 : END` of the cell rules.
// HIGH_NUM becomes the 16-bit infinity 0xC000: every add of a cost
// saturates there (__viaddmin_u16x2 with the infinity as the bound; a cost
// is far below the 0x4000 headroom), and where the reference adds HIGH_NUM
// itself the infinity is selected instead.  Exactness: the
// values on a pair's optimal path are at most its final cost, and every
// choice the traceback reads at a path cell compares a path value with
// candidates that are either exact or saturated above it.  So the results
// are the reference's whenever the final cost is below kAffPackLim (every
// path value x4 plus one step's largest add stays below the infinity); a
// pair above it sets error bit 8 and the host runs the batch again on the
// 32-bit kernel.  The direction bytes have k_aff_dp's layout, per pair, so
// k_aff_traceback reads them unchanged.
// ---------------------------------------------------------------------------
constexpr uint32_t kInfA2 = 0xC000C000u;   // the infinity in both halves
constexpr uint32_t kLo1 = 0x00010001u;
constexpr uint32_t kRk = 0x00030003u;      // the rank bits of both halves
constexpr int kAffPackLim = 12000;         // final costs below this are exact

struct AffSmem2 {
  uint32_t tab[1024];            // packed {cost[a][b], cost[gap][b]}
  uint16_t cost4[1024];          // 4 * cost[a][b]
  uint4 col[kAffWarps][kAffGroups][64];   // both pairs' columns (x4 costs, characters)
  uint4 ring_in[kAffWarps][kAffGroups][32];
  uint4 ring_out[kAffWarps][kAffGroups][32];
};

__device__ __forceinline__ uint32_t am2(uint32_t a, uint32_t b) {
  return __viaddmin_u16x2(a, b, kInfA2);  // saturating add, both halves
}
// min / max per half (measured: the plain SIMD forms run the 65,536-pair DP
// in 46.7-47.1 ms, the fused add-min / add-max with a zero addend in 48.8)
__device__ __forceinline__ uint32_t mn2(uint32_t a, uint32_t b) { return __vminu2(a, b); }
__device__ __forceinline__ uint32_t mx2(uint32_t a, uint32_t b) { return __vmaxu2(a, b); }
// selects b where m is all ones, else a (m: 0 / 0xFFFF per half)
__device__ __forceinline__ uint32_t sel2(uint32_t a, uint32_t b, uint32_t m) {
  return (a & ~m) | (b & m);
}

// Column quantities of both pairs (aff_column, times four), one half each.
__device__ __forceinline__ uint4 aff_column2(const uint32_t *tab, int jca, int jpa, int jcb,
                                            int jpb, int j, int go) {
  const int4 a = aff_column(tab, jca, jpa, j, go), b = aff_column(tab, jcb, jpb, j, go);
  return make_uint4((uint32_t)(4 * a.x) | ((uint32_t)(4 * b.x) << 16),
                    (uint32_t)(4 * a.y) | ((uint32_t)(4 * b.y) << 16),
                    (uint32_t)(4 * a.z) | ((uint32_t)(4 * b.z) << 16),
                    (uint32_t)a.w | ((uint32_t)b.w << 16));
}

struct AffRow2 {
  uint32_t vext, vopen, sopen;  // 4 * si_vext, 4 * (si_open + si_ext), 4 * si_open
  uint32_t icg;                 // 0xFFFF in a half whose row character has the gap bit
  const uint16_t *srowA, *srowB;  // 4 * cost[ic & 15][.] of each pair
  int i;
  uint32_t specL, specRA, specRB;  // bit u: step u of the half block is a boundary cell
  uint32_t spec;                   // any of the three
  int uFA, uFB;                    // step of each pair's final cell in the half block
};
struct AffState2 {
  uint32_t eh_l, cb_l;
  uint32_t eh_d, ev_d, eb_d, cb_d;
  uint32_t m_eh, m_ev, m_eb, m_cb;
  uint32_t wA, wB;
  int resA, resB;
};

// ENDS: the strip holds row 0 or a pair's last row.  Boundary cells (left
// and right of the band) are handled under a per-step test of the lane's
// bits.  Measured alternatives: computing the masks on every step, 4 %
// slower; a second copy of the half block without them, chosen per half
// block by a warp vote or by a per-strip mask, 35-50 % slower (both large
// unrolled copies are then hot at once).
template <bool BT, bool ENDS>
__device__ __forceinline__ void aff2_half(AffState2 &S, const AffRow2 &R, const uint4 *clane,
                                          const uint4 *rin, uint4 *rout, int s0, uint32_t go4,
                                          uint32_t go8, uint32_t *dmA, uint32_t *dmB, int lane) {
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    uint32_t u_eh = __shfl_up_sync(kFullA, S.m_eh, 1, kAffRows);
    uint32_t u_ev = __shfl_up_sync(kFullA, S.m_ev, 1, kAffRows);
    uint32_t u_eb = __shfl_up_sync(kFullA, S.m_eb, 1, kAffRows);
    uint32_t u_cb = __shfl_up_sync(kFullA, S.m_cb, 1, kAffRows);
    if (lane == 0) {
      const uint4 v = rin[u];
      u_eh = v.x; u_ev = v.y; u_eb = v.z; u_cb = v.w;
    }
    const uint4 D = clane[u];  // {hext, sj_open + sj_ext, sj_open} x4, characters
    const uint32_t jg = ((D.w >> 4) & kLo1) * 0xFFFFu;  // column character has the gap bit
    // FILL_EXTEND_HORIZONTAL: extension (rank 1) against opening (rank 0)
    const uint32_t ehr = mn2(am2(S.eh_l, D.x) | kLo1, am2(S.cb_l, D.y));
    // FILL_EXTEND_VERTICAL
    const uint32_t v1 = am2(u_ev, R.vext);
    const uint32_t evr = mn2(v1 | kLo1, am2(u_cb, R.vopen));
    // FILL_EXTEND_BLOCK_DIAGONAL[_NOBT]: the HIGH_NUM terms are selected,
    // not added (an infinite operand plus the infinity would wrap)
    const uint32_t both = R.icg & jg;
    const uint32_t b2 = sel2(kInfA2, BT ? S.cb_d : am2(S.cb_d, go8), both);
    const uint32_t ebr = mn2(sel2(kInfA2, S.eb_d, both) | kLo1, b2);
    // FILL_CLOSE_BLOCK_DIAGONAL, achoice ranks fh 0, fd 1, fv 2, fa 3
    const uint32_t cd = (uint32_t)R.srowA[D.w & 15u] | ((uint32_t)R.srowB[(D.w >> 16) & 15u] << 16);
    const uint32_t fh = am2(S.eh_d, cd + (R.sopen & jg));
    const uint32_t fd = am2(S.eb_d, cd + mx2(D.z, R.sopen)) | kLo1;
    const uint32_t fv = am2(S.ev_d, cd + (D.z & R.icg)) | (2u * kLo1);
    const uint32_t fa = am2(S.cb_d, cd) | kRk;
    const uint32_t cbr = mn2(mn2(fh, fd), mn2(fv, fa));
    uint32_t eh = ehr & ~kRk, ev = evr & ~kRk, eb = ebr & ~kRk, cb = cbr & ~kRk;
    // ASSIGN_MINIMUM, todo ranks EH 0, CB 1, EV 2, EB 3
    uint32_t f = mn2(mn2(eh, cb | kLo1), mn2(ev | (2u * kLo1), eb | kRk));
    uint32_t code = 0;
    if (BT)
      code = (f & kRk) | ((~evr & kLo1) << 2) | ((~ehr & kLo1) << 3) | ((~ebr & kLo1) << 4) |
             ((cbr & kRk) << 5);
    f &= ~kRk;
    bool row0 = false;
    if (ENDS && R.i == 0) {  // initialize_matrices_affine row 0 (both pairs: j = d)
      row0 = true;
      if (kDlo + s0 + u - 2 * lane == 0) {
        eh = go4; ev = go4; eb = 0; cb = 0; f = 0;
      } else {
        eh = am2(S.eh_l, D.y - D.z);
        cb = eh; eb = kInfA2; ev = kInfA2; f = eh;
      }
    }
    if (!row0 && ((R.spec >> u) & 1u)) {
      // the vertical boundary cell left of the band (the same step in both
      // pairs: one row) and each pair's HIGH_NUM cell right of it
      const uint32_t mL = (R.specL >> u) & 1u ? 0xFFFFFFFFu : 0u;
      const uint32_t mR = ((R.specRA >> u) & 1u ? 0xFFFFu : 0u) |
                          ((R.specRB >> u) & 1u ? 0xFFFF0000u : 0u);
      const uint32_t mLR = mL | mR;
      eh = sel2(eh, kInfA2, mLR);
      cb = sel2(cb, kInfA2, mLR);
      eb = sel2(eb, kInfA2, mLR);
      ev = sel2(sel2(ev, v1, mL), kInfA2, mR);
      f = sel2(f, ev, mL);
      if (BT)
        code = sel2(code, (kCodeLeft * kLo1 & mL) | (kCodeRight * kLo1 & mR), mLR & 0x00FF00FFu);
    }
    if (ENDS) {
      if (u == R.uFA) S.resA = (int)(f & 0xFFFFu);
      if (u == R.uFB) S.resB = (int)(f >> 16);
    }
    if (BT) {
      S.wA = __byte_perm(S.wA, code, 0x2104);  // (wA << 8) | code byte 0
      S.wB = __byte_perm(S.wB, code, 0x2106);  // (wB << 8) | code byte 2
      if ((u & 3) == 3) {
        if (dmA) dmA[(u >> 2) * kAffRows] = S.wA;
        if (dmB) dmB[(u >> 2) * kAffRows] = S.wB;
      }
    }
    S.m_eh = eh; S.m_ev = ev; S.m_eb = eb; S.m_cb = cb;
    if (lane == kAffRows - 1) rout[u] = make_uint4(eh, ev, eb, cb);
    S.eh_d = u_eh; S.ev_d = u_ev; S.eb_d = u_eb; S.cb_d = u_cb;
    S.eh_l = eh; S.cb_l = cb;
  }
}

// Bit u of the mask: step s0 + u is in [st, st + 16) at st.
__device__ __forceinline__ uint32_t step_bit(int st, int hs) {
  const int u = st - hs;
  return (u >= 0 && u < 16) ? (1u << u) : 0u;
}

// Two pairs per lane group (A low half, B high half), kAffGroups groups per
// warp; the warp runs its strips, blocks and half blocks to the largest
// pair's bounds, like aff_pair.
template <bool BT>
__device__ __forceinline__ void aff2_pairs(const AffDpArgs &A, AffSmem2 &sm, int warp,
                                           const AffPlan &PA, const AffPlan &PB, bool hasA,
                                           bool hasB, int64_t offA, int64_t offB, int idA,
                                           int idB, uint4 *bnd, int lane) {
  const int h = lane / kAffRows, k = lane & (kAffRows - 1);
  const uint8_t *siA = A.seq + PA.si_off, *sjA = A.seq + PA.sj_off;
  const uint8_t *siB = A.seq + PB.si_off, *sjB = A.seq + PB.sj_off;
  const int go = A.go;
  const uint32_t go4 = 4u * (uint32_t)go * kLo1, go8 = 8u * (uint32_t)go * kLo1;
  const int ThA = hasA ? PA.nstrips : 0, ThB = hasB ? PB.nstrips : 0;
  const int ShA = hasA ? PA.sblocks * 4 : 0, ShB = hasB ? PB.sblocks * 4 : 0;
  const int T = __reduce_max_sync(kFullA, max(ThA, ThB));
  uint4 *win = sm.col[warp][h];
  uint4 *rin = sm.ring_in[warp][h], *rout = sm.ring_out[warp][h];
  const uint4 *wl = win + kAffRows - k;
  const uint4 kInf4 = make_uint4(kInfA2, kInfA2, kInfA2, kInfA2);
  AffState2 S;
  S.resA = S.resB = 0;
  uint32_t *dmbaseA = (BT && hasA) ? A.dm + offA : nullptr;
  uint32_t *dmbaseB = (BT && hasB) ? A.dm + offB : nullptr;

  for (int strip = 0; strip < T; ++strip) {
    const bool actA = strip < ThA, actB = strip < ThB;
    const int Spad = __reduce_max_sync(kFullA, max(actA ? ShA : 0, actB ? ShB : 0));
    const bool ends = __any_sync(kFullA, strip == 0 || (actA && strip == ThA - 1) ||
                                             (actB && strip == ThB - 1));
    const int r0 = strip * kAffRows;
    AffRow2 R;
    R.i = r0 + k;
    const bool okA = actA && R.i <= PA.leni, okB = actB && R.i <= PB.leni;
    const int icA = okA ? siA[R.i] : 0, ipA = (okA && R.i > 0) ? siA[R.i - 1] : 0;
    const int icB = okB ? siB[R.i] : 0, ipB = (okB && R.i > 0) ? siB[R.i - 1] : 0;
    auto rowq = [&](int ic, int ip, uint32_t &vext, uint32_t &vopen, uint32_t &sopen) {
      const int si_ext = (int)(sm.tab[(ic << 5) | 16] & 0xffffu);
      const int si_open = (!(ip & 16) && (ic & 16)) ? 0 : go;
      const int si_vext = (R.i > 1 && (ip & 16) && !(ic & 16)) ? si_open + si_ext : si_ext;
      vext = 4u * (uint32_t)si_vext;
      vopen = 4u * (uint32_t)(si_open + si_ext);
      sopen = 4u * (uint32_t)si_open;
    };
    uint32_t xa, ya, za, xb, yb, zb;
    rowq(icA, ipA, xa, ya, za);
    rowq(icB, ipB, xb, yb, zb);
    R.vext = xa | (xb << 16);
    R.vopen = ya | (yb << 16);
    R.sopen = za | (zb << 16);
    R.icg = ((icA & 16) ? 0xFFFFu : 0u) | ((icB & 16) ? 0xFFFF0000u : 0u);
    R.srowA = sm.cost4 + ((icA & 15) << 5);
    R.srowB = sm.cost4 + ((icB & 15) << 5);
    // the boundary cells' steps in the strip (aff_pair's sL, sR, sF)
    const int d_lb = (-R.i > kDlo) ? -R.i : kDlo;
    const int sL = d_lb - kDlo + 2 * k;
    const int sRA = (PA.e0 <= PA.lenj - R.i) ? PA.e0 - kDlo + 2 * k : -1000000;
    const int sRB = (PB.e0 <= PB.lenj - R.i) ? PB.e0 - kDlo + 2 * k : -1000000;
    const int sFA = (actA && R.i == PA.leni) ? (PA.lenj - PA.leni) - kDlo + 2 * k : -1000000;
    const int sFB = (actB && R.i == PB.leni) ? (PB.lenj - PB.leni) - kDlo + 2 * k : -1000000;

    S.eh_l = kInfA2; S.cb_l = kInfA2;
    S.eh_d = kInfA2; S.ev_d = kInfA2; S.eb_d = kInfA2; S.cb_d = kInfA2;
    S.m_eh = kInfA2; S.m_ev = kInfA2; S.m_eb = kInfA2; S.m_cb = kInfA2;
    S.wA = S.wB = 0;
    if (k == 0 && strip > 0) {
      // a pair past its last strip reads an infinite record
      const uint4 v = bnd[0];
      const uint32_t keep = (actA ? 0xFFFFu : 0u) | (actB ? 0xFFFF0000u : 0u);
      S.eh_d = sel2(kInfA2, v.x, keep); S.ev_d = sel2(kInfA2, v.y, keep);
      S.eb_d = sel2(kInfA2, v.z, keep); S.cb_d = sel2(kInfA2, v.w, keep);
    }
    for (int s0 = 0; s0 < Spad; s0 += 32) {
      __syncwarp();
      {
        auto chrA = [&](int j) { return (actA && j >= 0 && j <= PA.lenj) ? (int)sjA[j] : 0; };
        auto chrB = [&](int j) { return (actB && j >= 0 && j <= PB.lenj) ? (int)sjB[j] : 0; };
        const int jb = r0 + kDlo + s0 - kAffRows;
#pragma unroll
        for (int e = k; e < 32; e += kAffRows) {
          const int x = s0 + e + 1;
          uint4 v = kInf4;
          const bool inA = actA && strip > 0 && x < PA.wd, inB = actB && strip > 0 && x < PB.wd;
          if (inA || inB) {
            const uint4 b = bnd[x];
            const uint32_t keep = (inA ? 0xFFFFu : 0u) | (inB ? 0xFFFF0000u : 0u);
            v = make_uint4(sel2(kInfA2, b.x, keep), sel2(kInfA2, b.y, keep),
                           sel2(kInfA2, b.z, keep), sel2(kInfA2, b.w, keep));
          }
          rin[e] = v;
        }
#pragma unroll
        for (int x = k; x < 64; x += kAffRows)
          win[x] = aff_column2(sm.tab, chrA(jb + x), chrA(jb + x - 1), chrB(jb + x),
                               chrB(jb + x - 1), jb + x, go);
      }
      __syncwarp();
      uint32_t *dmbA = (BT && actA) ? dmbaseA + ((int64_t)strip * PA.sblocks + (s0 >> 2)) * kAffRows + k
                                    : nullptr;
      uint32_t *dmbB = (BT && actB) ? dmbaseB + ((int64_t)strip * PB.sblocks + (s0 >> 2)) * kAffRows + k
                                    : nullptr;
#pragma unroll 1
      for (int hh = 0; hh < 2; ++hh) {
        const int hs = s0 + 16 * hh;
        if (hs >= Spad) break;
        R.specL = step_bit(sL, hs);
        R.specRA = step_bit(sRA, hs);
        R.specRB = step_bit(sRB, hs);
        R.uFA = sFA - hs;
        R.uFB = sFB - hs;
        uint32_t *dmhA = (dmbA && hs < ShA) ? dmbA + 4 * kAffRows * hh : nullptr;
        uint32_t *dmhB = (dmbB && hs < ShB) ? dmbB + 4 * kAffRows * hh : nullptr;
        R.spec = R.specL | R.specRA | R.specRB;
        const uint4 *cl = wl + 16 * hh, *ri = rin + 16 * hh;
        uint4 *ro = rout + 16 * hh;
        if (ends)
          aff2_half<BT, true>(S, R, cl, ri, ro, hs, go4, go8, dmhA, dmhB, k);
        else
          aff2_half<BT, false>(S, R, cl, ri, ro, hs, go4, go8, dmhA, dmhB, k);
      }
      __syncwarp();
      const int wdm = max(actA ? PA.wd : 0, actB ? PB.wd : 0);
#pragma unroll
      for (int e = k; e < 32; e += kAffRows) {
        const int x = s0 + e - 2 * (kAffRows - 1);
        if (x >= 0 && x < wdm) bnd[x] = rout[e];
      }
    }
    __syncwarp();
  }
  const int rA = __shfl_sync(kFullA, S.resA, h * kAffRows + (PA.leni & (kAffRows - 1)));
  const int rB = __shfl_sync(kFullA, S.resB, h * kAffRows + (PB.leni & (kAffRows - 1)));
  if (k == 0) {
    if (hasA) {
      A.cost[idA] = rA >> 2;
      if ((rA >> 2) >= kAffPackLim) atomicOr(A.err, 8);
    }
    if (hasB) {
      A.cost[idB] = rB >> 2;
      if ((rB >> 2) >= kAffPackLim) atomicOr(A.err, 8);
    }
  }
}

template <bool BT>
__global__ void __launch_bounds__(kAffWarps * 32, 5) k_aff_dp2(AffDpArgs A) {
  __shared__ AffSmem2 sm;
  for (int t = threadIdx.x; t < 1024; t += blockDim.x) {
    sm.tab[t] = A.tables->packed[t];
    sm.cost4[t] = (uint16_t)(4u * (A.tables->packed[t] & 0xffffu));
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int h = lane / kAffRows;
  uint4 *bnd = (uint4 *)A.scratch + (gw * kAffGroups + h) * A.slab;  // one slab per lane group
  for (;;) {
    int p = 0;
    if (lane == 0) p = atomicAdd(A.counter, 2 * kAffGroups);  // consecutive pairs: similar sizes
    p = __shfl_sync(kFullA, p, 0);
    if (p >= A.n) break;
    AffPlan P2[2];
    bool has2[2];
    int id2[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int ph = p + 2 * h + q;
      has2[q] = ph < A.n;
      id2[q] = has2[q] ? (A.order ? A.order[ph] : ph) : 0;
      P2[q] = AffPlan{};
      P2[q].leni = P2[q].lenj = -1;
      if (has2[q]) {
        const AffPlan Q = A.plans[id2[q]];
        if (Q.empty) {
          if ((lane & (kAffRows - 1)) == 0) A.cost[id2[q]] = 0;
          has2[q] = false;
        } else {
          P2[q] = Q;
        }
      }
    }
    aff2_pairs<BT>(A, sm, warp, P2[0], P2[1], has2[0], has2[1],
                   (BT && has2[0]) ? A.dm_off[id2[0]] : 0, (BT && has2[1]) ? A.dm_off[id2[1]] : 0,
                   id2[0], id2[1], bnd, lane);
  }
}

template <bool BT>
__global__ void __launch_bounds__(kAffWarps * 32, 24 / kAffWarps) k_aff_dp(AffDpArgs A) {
  __shared__ AffSmem sm;
  for (int t = threadIdx.x; t < 1024; t += blockDim.x) {
    sm.tab[t] = A.tables->packed[t];
    sm.cost[t] = (uint16_t)(A.tables->packed[t] & 0xffffu);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int h = lane / kAffRows;
  int4 *bnd = A.scratch + (gw * kAffGroups + h) * A.slab;  // one boundary slab per lane group
  for (;;) {
    int p = 0;
    if (lane == 0) p = atomicAdd(A.counter, kAffGroups);  // consecutive pairs: similar sizes
    p = __shfl_sync(kFullA, p, 0);
    if (p >= A.n) break;
    const int ph = p + h;
    bool has = ph < A.n;
    const int id = has ? (A.order ? A.order[ph] : ph) : 0;
    AffPlan P = {};
    P.leni = P.lenj = -1;
    if (has) {
      const AffPlan Q = A.plans[id];
      if (Q.empty) {
        if ((lane & (kAffRows - 1)) == 0) A.cost[id] = 0;
        has = false;
      } else {
        P = Q;
      }
    }
    aff_pair<BT>(A, sm, warp, P, has, (BT && has) ? A.dm_off[id] : 0, id, bnd, lane);
  }
}

__global__ void __launch_bounds__(128) k_aff_traceback(AffTbArgs A) {
  __shared__ uint8_t med[1024];
  for (int t = threadIdx.x; t < 1024; t += blockDim.x) med[t] = A.tables->median[t];
  __syncthreads();
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= A.n) return;
  const AffPlan P = A.plans[id];
  const int li = P.leni + 1, lj = P.lenj + 1;
  const int la = P.swap ? lj : li, lb = P.swap ? li : lj;
  const int64_t cap = slot_cap(la, lb);
  uint8_t *oa = A.out + A.out_off[id];
  uint8_t *ob = oa + cap, *ow = ob + cap, *om = ow + cap;
  const uint8_t *si = A.seq + P.si_off, *sj = A.seq + P.sj_off;
  if (P.empty) {
    const bool a_empty = P.empty == 1;
    const uint8_t *src = (a_empty != (bool)P.swap) ? sj : si;
    const int len = a_empty ? lb : la;
    for (int t = 0; t < len; ++t) om[cap - len + t] = src[t];
    A.out_len[2 * id] = 0;
    A.out_len[2 * id + 1] = len;
    return;
  }
  // resi / resj of backtrace_affine in caller order
  uint8_t *ri = P.swap ? ob : oa, *rj = P.swap ? oa : ob;
  const uint32_t *dm = A.dm + A.dm_off[id];
  const int sb = P.sblocks, e0 = P.e0, lenj = P.lenj;
  int i = P.leni, j = P.lenj;
  int ic = si[i], jc = sj[j];
  int64_t nr = 0, nm = 0;
  // the four outputs are written backwards through word-buffered writers
  BackWriter wri(ri + cap - 1), wrj(rj + cap - 1), wow(ow + cap - 1), wom(om + cap - 1);
  int last_m = -1;  // the median byte written last (its position cap - nm)
  auto put_r = [&](int x, int y) {  // one column of resi / resj
    wri.put((uint32_t)x);
    wrj.put((uint32_t)y);
    ++nr;
  };
  auto put_m = [&](int x) {
    wom.put((uint32_t)x);
    last_m = x;
    ++nm;
  };
  int mode = 0;  // 0 todo, 1 vertical, 2 horizontal, 3 diagonal, 4 align
  bool bad = false;
  while (i != 0 && j != 0) {
    const int d = j - i;
    const int d_lb = (-i > kDlo) ? -i : kDlo;
    if (d < d_lb || d > e0 || (d == e0 && !(e0 <= lenj - i))) { bad = true; break; }
    const int k = i & (kAffRows - 1), strip = i / kAffRows;
    const int s = d - kDlo + 2 * k;
    const uint32_t w = dm[((int64_t)strip * sb + (s >> 2)) * kAffRows + k];
    const uint32_t c = (w >> (8 * (3 - (s & 3)))) & 0xffu;
    if (mode == 0) {
      const uint32_t t = c & 3u;
      mode = t == 0 ? 2 : t == 1 ? 4 : t == 2 ? 1 : 3;
    } else if (mode == 1) {
      if (c & 4u) mode = 0;
      if (!(ic & 16)) { put_m(ic | 16); wow.put(ic | 16); }
      else wow.put(16);
      put_r(ic, 16);
      --i; ic = si[i];
    } else if (mode == 2) {
      if (c & 8u) mode = 0;
      if (!(jc & 16)) { put_m(jc | 16); wow.put(jc | 16); }
      else wow.put(16);
      put_r(16, jc);
      --j; jc = sj[j];
    } else if (mode == 3) {
      if (c & 16u) mode = 0;
      put_r(ic, jc);
      wow.put(16);
      --i; --j; jc = sj[j]; ic = si[i];
    } else {
      const uint32_t a = (c >> 5) & 3u;
      if (a == 0) mode = 2;
      else if (a == 1) mode = 3;
      else if (a == 2) mode = 1;
      const int m = med[((ic & 15) << 5) | (jc & 15)];
      put_m(m); wow.put(m);
      put_r(ic, jc);
      --i; --j; jc = sj[j]; ic = si[i];
    }
    if (nr + 4 >= cap) { bad = true; break; }
  }
  while (!bad && i != 0) {
    if (!(ic & 16)) { put_m(ic | 16); wow.put(ic | 16); }
    else wow.put(16);
    put_r(ic, 16);
    --i; ic = si[i];
  }
  while (!bad && j != 0) {
    if (!(jc & 16)) { put_m(jc | 16); wow.put(jc | 16); }
    else wow.put(16);
    put_r(16, jc);
    --j; jc = sj[j];
  }
  put_r(16, 16);
  wow.put(16);
  // an empty median has no position 0 in the reference; treated as not a gap
  if (nm == 0 || last_m != 16) put_m(16);
  wri.flush();
  wrj.flush();
  wow.flush();
  wom.flush();
  A.out_len[2 * id] = bad ? -1 : (int32_t)nr;
  A.out_len[2 * id + 1] = bad ? -1 : (int32_t)nm;
}

int aff_blocks(bool bt, bool packed) {
  static int cache[4][64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  int &c = cache[(bt ? 1 : 0) + (packed ? 2 : 0)][dev & 63];
  if (!c) {
    int per_sm = 0, sms = 0;
    if (packed && bt) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_aff_dp2<true>, kAffWarps * 32, 0);
    else if (packed) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_aff_dp2<false>, kAffWarps * 32, 0);
    else if (bt) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_aff_dp<true>, kAffWarps * 32, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_aff_dp<false>, kAffWarps * 32, 0);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    c = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  return c;
}

#define CKA(call)                                         \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

}  // namespace

int affine_batch(const poyd_cm *cm, int maxc, int32_t n, const uint8_t *seq,
                 const int64_t *a_off, const int32_t *a_len, const int64_t *b_off,
                 const int32_t *b_len, int32_t *cost, int64_t *cells, bool want_align,
                 int32_t flags, uint8_t *out, const int64_t *out_off, int32_t *out_len,
                 cudaStream_t st) {
  Workspace *w = workspace(st);
  DevTables *tabs = nullptr;
  int rc = upload_tables_ws(w, cm, &tabs, st);
  if (rc) return rc;
  AffPlan *plans = (AffPlan *)ws_buffer(w, WS_AFF, sizeof(AffPlan) * (size_t)n);
  int64_t *dmw = (int64_t *)ws_buffer(w, WS_DMWORDS, sizeof(int64_t) * 2 * (size_t)n);
  int32_t *wdb = (int32_t *)ws_buffer(w, WS_WD, sizeof(int32_t) * 2 * (size_t)n + 16);
  int32_t *err = (int32_t *)ws_buffer(w, WS_ERR, 64);
  if (!plans || !dmw || !wdb || !err) return fail(POYD_ENOMEM, "plan allocation failed");
  CKA(cudaMemsetAsync(err, 0, 4, st));
  AffPlanArgs PA;
  PA.n = n; PA.seq = seq; PA.a_off = a_off; PA.a_len = a_len; PA.b_off = b_off;
  PA.b_len = b_len; PA.gap = cm->gap; PA.dos_empty = (flags & POYD_FLAG_DOS_EMPTY) ? 1 : 0;
  PA.maxc = std::max(maxc, cm->gap_open);
  PA.plans = plans; PA.dm_words = dmw; PA.wd_out = wdb; PA.cells = cells; PA.err = err;
  {
    ProfScope ps("aff_plan", st);
    k_aff_plan<<<(n + 127) / 128, 128, 0, st>>>(PA);
  }
  CKA(cudaGetLastError());
  std::vector<int64_t> hw((size_t)n);
  std::vector<int32_t> hwd((size_t)n + 1);
  CKA(cudaMemcpyAsync(hw.data(), dmw, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost, st));
  CKA(cudaMemcpyAsync(hwd.data(), wdb, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, st));
  CKA(cudaMemcpyAsync(hwd.data() + n, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CKA(cudaStreamSynchronize(st));
  if (hwd[n] & 1) return fail(POYD_EINVAL, "sequences must have length >= 1 (the leading gap)");
  if (hwd[n] & 2) return fail(POYD_ERANGE, "affine costs could reach the HIGH_NUM sentinel range");
  if (hwd[n] & 4) return fail(POYD_EINVAL, "sequence codes must be below 32 (5-bit element masks)");
  std::vector<int64_t> off((size_t)n);
  int64_t total = 0;
  int maxwd = 1;
  for (int32_t t = 0; t < n; ++t) {
    off[t] = total;
    if (want_align) total += hw[t];
    maxwd = std::max(maxwd, hwd[t]);
  }
  std::vector<int32_t> order;
  longest_first(hw, order);
  int64_t *doff = dmw + n;
  int32_t *dord = (int32_t *)ws_buffer(w, WS_ORDER, sizeof(int32_t) * (size_t)n);
  int *counter = (int *)ws_buffer(w, WS_COUNTER, 64);
  if (!dord || !counter) return fail(POYD_ENOMEM, "order allocation failed");
  CKA(cudaMemcpyAsync(doff, off.data(), sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice, st));
  CKA(cudaMemcpyAsync(dord, order.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, st));
  CKA(cudaMemsetAsync(counter, 0, 4, st));
  uint32_t *dm = nullptr;
  if (want_align) {
    dm = (uint32_t *)ws_buffer(w, WS_DM, sizeof(uint32_t) * (size_t)std::max<int64_t>(total, 1));
    if (!dm) return fail(POYD_ENOMEM, "affine direction matrix allocation failed");
  }
  // The packed kernel runs when one step's largest add stays far below its
  // 16-bit infinity (small cost tables; POYD_AFF_PACKED=0 keeps the 32-bit
  // kernel); a pair whose final cost is past its exact range sends the
  // whole batch to the 32-bit kernel afterwards.
  bool packed = 4LL * (PA.maxc + 2LL * cm->gap_open + 1) < 0x3000;
  if (const char *e = std::getenv("POYD_AFF_PACKED")) packed = packed && std::atoi(e) != 0;
  for (int attempt = 0; attempt < 2; ++attempt) {
    const int blocks = aff_blocks(want_align, packed);
    const int64_t slab = maxwd + 8;
    int4 *scratch = (int4 *)ws_buffer(w, WS_SCRATCH,
                                      sizeof(int4) * (size_t)slab * (size_t)blocks * kAffWarps *
                                          kAffGroups);
    if (!scratch) return fail(POYD_ENOMEM, "scratch allocation failed");
    AffDpArgs DA;
    DA.n = n; DA.seq = seq; DA.plans = plans; DA.dm_off = doff; DA.order = dord; DA.tables = tabs;
    DA.go = cm->gap_open; DA.counter = counter; DA.scratch = scratch; DA.slab = slab; DA.dm = dm;
    DA.cost = cost; DA.err = err;
    if (attempt) CKA(cudaMemsetAsync(counter, 0, 4, st));
    {
      ProfScope ps(want_align ? "aff_dp_dm" : "aff_dp_cost", st);
      if (packed && want_align) k_aff_dp2<true><<<blocks, kAffWarps * 32, 0, st>>>(DA);
      else if (packed) k_aff_dp2<false><<<blocks, kAffWarps * 32, 0, st>>>(DA);
      else if (want_align) k_aff_dp<true><<<blocks, kAffWarps * 32, 0, st>>>(DA);
      else k_aff_dp<false><<<blocks, kAffWarps * 32, 0, st>>>(DA);
    }
    CKA(cudaGetLastError());
    if (want_align) {
      AffTbArgs TA;
      TA.n = n; TA.seq = seq; TA.plans = plans; TA.dm_off = doff; TA.dm = dm; TA.tables = tabs;
      TA.out = out; TA.out_off = out_off; TA.out_len = out_len;
      {
        ProfScope ps("aff_traceback", st);
        k_aff_traceback<<<(n + 127) / 128, 128, 0, st>>>(TA);
      }
      CKA(cudaGetLastError());
    }
    if (!packed) break;
    int32_t e = 0;
    CKA(cudaMemcpyAsync(&e, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CKA(cudaStreamSynchronize(st));
    if (!(e & 8)) break;
    packed = false;  // a cost past the packed range: the 32-bit kernel, again
  }
  return POYD_OK;
}

}  // namespace poyd
