// Packed linear-gap banded DP on sm_103a: four DP rows per lane, two cells
// per 32-bit register in unsigned 16-bit halves.
//
// Restates the same recurrence as linear.cu (algn_fill_plane_2 /
// algn_fill_plane, algn.c:812-968, cell rule algn_fill_row algn.c:375-453,
// band-edge cells algn.c:461-620) and the same backtrack priorities
// (backtrack_2d, algn.c:3551-3666), for batches whose every in-band value
// fits 16 bits.
//
// Layout.  One warp owns one pair (persistent grid, longest first).  Lane k
// owns rows 128t + 4k + m (m = 0..3) of strip t.  Row m runs lam[m] =
// (0, 1, 3, 4) steps behind the lane's row 0 and lane k runs 7k steps
// behind lane 0, so row 4k+m of strip t is at band index i (diagonal
// dlo + i) at step tW + 7k + lam[m] + i.  Lane k-1's row 3 value that lane
// k's row 0 needs is computed two steps earlier, so the shuffle carrying it
// is issued a step ahead and stays off the step's dependency chain.  Rows
// 0 and 2 share register X (low, high half), rows 1 and 3 register Y:
//   * X's rows never depend on each other within a step (row 2 reads row 1
//     of the previous steps), so one __viaddmin_u16x2 updates both;
//   * Y's rows read X's fresh values as their delete predecessors (rows 1
//     and 3 run one step behind rows 0 and 2), so D_Y = X and A_Y = the
//     previous X, with no permute;
//   * X's delete predecessors are {row above row 0 (lane k-1's row 3),
//     row 1} = one byte permute of the shuffled Y and the lane's own Y;
//   * per register, min(align, insert) is formed first (it needs no value
//     of the step) and the delete term enters with one add-min.
// Rows 0 and 1 read column c(u) at step u, rows 2 and 3 column c(u-1): one
// profile word per step holds four byte costs (one per row) and the cost
// operands are byte permutes of this step's and the previous step's word
// (with the permute's sign-replicate mode writing zero bytes).  Values are
// biased by cost[s1[0]][s2[0]] and kept x4 with the move rank in the low
// two bits in kDpChoice, as in linear.cu.
//
// Out-of-band cells.  Strips follow one another with period W =
// max(roundup32(wd + 4), 288): each row spends W - wd >= 4 steps out of the
// band between strips, so every strip-dependent input of a lane (column
// window, profile, delete costs) can switch at one step.  The cell of each
// row at band index wd is forced to INF (the reference's right-edge cell
// has no delete move); every later out-of-band cell then stays >= INF.
// Cells left of column 0 (the band's top-left triangle) and rows before
// their first step are forced to INF by a second table.  Forcing is one
// LOP3 per register with a 16x2 bit mask read from small shared tables
// indexed by the lane's step offset.  Blocks of 32 steps come in four
// kinds: plain (no lane switches strips or meets a forced cell), mixed
// (strip switches and right-edge forcing), slow (also the first strips'
// masks) and slow with the final-cell capture.
//
// Why 16 bits hold: every in-band cell (r, j) with j <= L2 is at most
// bias + max(r, j) * maxc; the host only launches this kernel when
// sc * maxc * (max(L1, L2) + 260) + 6 < INF16 = 0xC000 for every pair, so
// real values never reach INF16 and INF16 plus a cost never wraps.  Adds
// of two packed halves as one 32-bit add (the insert candidates) carry
// from the low half only where the low row is past the matrix edge, and
// then the high row is too.
#include <cuda_runtime.h>
#include <cstdint>
#include "poyd_internal.h"
#include "linear_kernels.cuh"
#include "back_writer.cuh"

namespace poyd {
namespace {

constexpr unsigned kFull4 = 0xffffffffu;
constexpr int k4Warps = 8;          // warps per block
constexpr int k4Lag = 7;            // steps between consecutive lanes
constexpr int k4R3 = 7 * 31 + 4;    // lane 31's row 3 behind lane 0's row 0
constexpr int k4MinPeriod = 288;    // boundary row flush-to-prefetch distance
constexpr int k4WinBase = 3 * 31;   // window position of lane 31's step-0 column
constexpr int k4Win = 128;          // window entries per strip (positions 0..124)
constexpr uint32_t kInf16 = 0xC000u;
constexpr uint32_t kInf2 = 0xC000C000u;
constexpr int kEdgeOff = 40, kEdgeN = 112;  // right-edge masks, offsets [-40, 72)
constexpr int kTriOff = 40, kTriN = 80;     // first-strip masks, offsets [-40, 40)

// Shared memory, in bytes from a 128-byte aligned base.
constexpr uint32_t kSmProf = 0;                        // [warp][parity][c][lane] u32
constexpr uint32_t kSmWin = kSmProf + k4Warps * 8192;  // [warp][new, old][k4Win] uint2
constexpr uint32_t kSmCtab = kSmWin + k4Warps * 2 * k4Win * 8;  // cost[a][b] at a*33+b (u32)
constexpr uint32_t kSmGt = kSmCtab + 32 * 33 * 4;      // insert costs [rank 0,1,2][c] (u32)
constexpr uint32_t kSmEdge = kSmGt + 3 * 32 * 4;       // [kEdgeN] {X mask, Y mask}
constexpr uint32_t kSmTri = kSmEdge + kEdgeN * 8;      // [4][kTriN] {X mask, Y mask}
constexpr uint32_t kSmMed = kSmTri + 4 * kTriN * 8;    // median table (u8)
constexpr uint32_t kSmBytes = kSmMed + 1024 + 128;     // + alignment slack

constexpr int kPlain = 0, kMixed = 1, kSlow = 2, kSlowCap = 3;

__device__ __forceinline__ uint32_t lds32(uint32_t a) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ uint2 lds64(uint32_t a) {
  uint2 v;
  asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(a));
  return v;
}
__device__ __forceinline__ void sts32(uint32_t a, uint32_t v) {
  asm volatile("st.shared.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void sts64(uint32_t a, uint32_t x, uint32_t y) {
  asm volatile("st.shared.v2.u32 [%0], {%1, %2};" ::"r"(a), "r"(x), "r"(y) : "memory");
}
// prmt in its default mode: a selector nibble with bit 3 set replicates the
// sign bit of the selected byte (a zero byte when that byte is below 128).
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t s) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(s));
  return d;
}
// A 32-bit add kept on the multiply-add pipe (the ALU pipe is the busier one).
__device__ __forceinline__ uint32_t add_fma(uint32_t a, uint32_t b, uint32_t one) {
  uint32_t d;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(one), "r"(b));
  return d;
}
// Halves selected by m (0xffff per half) become exactly INF16.
__device__ __forceinline__ uint32_t force_inf(uint32_t x, uint32_t m) {
  return (x & ~m) | (kInf2 & m);
}

// Geometry of one pair in the packed schedule.
struct Geo4 {
  int L1, L2, dlo, wd, W, G, T, nblk, tri_last;
};

__device__ __forceinline__ Geo4 geo4(const LinPlan &P) {
  Geo4 g;
  g.L1 = P.l1;
  g.L2 = P.l2;
  g.dlo = P.dlo;
  g.wd = P.wd;
  g.W = max((P.wd + 4 + 31) / 32 * 32, k4MinPeriod);
  g.G = g.W - P.wd;
  g.T = (P.l1 + 127) >> 7;
  g.nblk = ((g.T - 1) * g.W + k4R3 + P.wd + 31) >> 5;
  g.tri_last = (-P.dlo - 1) >= 0 ? (-P.dlo - 1) >> 7 : 0;
  return g;
}

// Per-lane inputs of one 16-step half block.
struct Half4 {
  uint32_t wn, wo;                  // window read address of step 0 (new / old strip)
  uint32_t cdXn, cdYn, cdXo, cdYo;  // delete costs (x scale + rank), new / old strip
  uint32_t fe, ft;                  // mask table addresses of step 0
  int sw;                           // steps >= sw use the new strip
  int tg;                           // steps >= tg take the first-strip masks
  int fv;                           // step of the final cell (kSlowCap), else -1
};

struct State4 {
  uint32_t X, Y, DXp, q, prp, res;
  uint32_t up;  // the row above of row 0 for the next step (shuffled a step ahead)
};

// Multiplier constants passed at run time, so that the adds stay
// multiply-adds on the FMA pipe (DpK: 1, -1, 4).
struct K4 {
  uint32_t one, m1, four;
};

// 16 steps of one block half.  Per step: the shuffle of the row above for
// the next step, the queue rotation, the window-word and profile-word
// loads, four byte permutes, and per register one 32-bit add (insert
// candidate, both halves) and two 16x2 add-mins: min(align, insert) first,
// then the delete term.  In kDpChoice the 2-bit ranks of both halves go
// into the direction words (eight steps per word) and are cleared from the
// values.
template <int MODE, int KIND>
__device__ __forceinline__ void l4_half(State4 &S, const Half4 &H, uint32_t lane4, int lane,
                                         int qsrc, bool capY, const K4 &K, uint32_t &ax0,
                                         uint32_t &ax1, uint32_t &ay0, uint32_t &ay1) {
  // The shared loads run ahead of their step (the asm loads keep source
  // order): window words two steps ahead, profile and mask words one.
  auto waddr = [&](int v) -> uint32_t {
    return ((KIND == kPlain || v >= H.sw) ? H.wn : H.wo) + 8 * v;
  };
  uint2 wq0 = lds64(waddr(0)), wq1 = lds64(waddr(1));
  uint32_t pq0 = lds32(add_fma(wq0.x, lane4, K.one));
  uint2 fq = make_uint2(0, 0), tq = make_uint2(0, 0);
  if (KIND >= kMixed) fq = lds64(H.fe);
  if (KIND >= kSlow) tq = lds64(H.ft);
#pragma unroll
  for (int v = 0; v < 16; ++v) {
    const uint2 w = wq0;
    const uint32_t pr = pq0;
    const uint2 fe = fq, ft = tq;
    wq0 = wq1;
    if (v + 2 < 16) wq1 = lds64(waddr(v + 2));
    if (v + 1 < 16) {
      pq0 = lds32(add_fma(wq0.x, lane4, K.one));
      if (KIND >= kMixed) fq = lds64(H.fe + 8 * (v + 1));
      if (KIND >= kSlow) tq = lds64(H.ft + 8 * (v + 1));
    }
    const uint32_t up = S.up;
    // lane k-1's current Y feeds lane k's row 0 at the next step; lane 0
    // takes the boundary queue's next value after the rotation
    const uint32_t recv = __shfl_up_sync(kFull4, S.Y, 1);
    S.q = __shfl_sync(kFull4, S.q, qsrc);
    S.up = (lane == 0) ? S.q : recv;
    const bool nw = KIND == kPlain || v >= H.sw;
    const uint32_t caX = prmt(pr, S.prp, 0xE680);  // {row 0 vs c(u), row 2 vs c(u-1)}
    const uint32_t caY = prmt(pr, S.prp, 0xF791);  // {row 1 vs c(u), row 3 vs c(u-1)}
    const uint32_t ci = w.y;                       // {g(c(u)), g(c(u-1))}
    const uint32_t cdX = nw ? H.cdXn : H.cdXo, cdY = nw ? H.cdYn : H.cdYo;
    uint32_t mX = 0, mY = 0;
    if (KIND >= kMixed) {
      mX = fe.x;
      mY = fe.y;
    }
    if (KIND >= kSlow) {
      const bool on = v >= H.tg;
      mX |= on ? ft.x : 0u;
      mY |= on ? ft.y : 0u;
    }
    // X = {row 0, row 2}: align from the previous delete operand, insert
    // from the own previous value; Y = {row 1, row 3}: align from the
    // previous X, insert from the own previous value
    const uint32_t tX = __viaddmin_u16x2(S.DXp, caX, add_fma(S.X, ci, K.one));
    const uint32_t tY = __viaddmin_u16x2(S.X, caY, add_fma(S.Y, ci, K.one));
    const uint32_t DX = prmt(up, S.Y, 0x5432);  // {row above row 0, row 1}
    uint32_t Xn = __viaddmin_u16x2(DX, cdX, tX);
    if (MODE == kDpChoice) {
      // clear the rank bits (one LOP on the dependency chain); the rank
      // itself, old - cleared, and its accumulation stay on the FMA pipe
      const uint32_t Xc = Xn & 0xFFFCFFFCu;
      uint32_t r;
      asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(Xc), "r"(K.m1), "r"(Xn));
      if (v < 8) {
        asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(ax0) : "r"(ax0), "r"(K.four), "r"(r));
      } else {
        asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(ax1) : "r"(ax1), "r"(K.four), "r"(r));
      }
      Xn = Xc;
    }
    if (KIND >= kMixed) Xn = force_inf(Xn, mX);
    // Y's delete predecessors are X's fresh values
    uint32_t Yn = __viaddmin_u16x2(Xn, cdY, tY);
    if (MODE == kDpChoice) {
      // clear the rank bits (one LOP on the dependency chain); the rank
      // itself, old - cleared, and its accumulation stay on the FMA pipe
      const uint32_t Yc = Yn & 0xFFFCFFFCu;
      uint32_t r;
      asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(Yc), "r"(K.m1), "r"(Yn));
      if (v < 8) {
        asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(ay0) : "r"(ay0), "r"(K.four), "r"(r));
      } else {
        asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(ay1) : "r"(ay1), "r"(K.four), "r"(r));
      }
      Yn = Yc;
    }
    if (KIND >= kMixed) Yn = force_inf(Yn, mY);
    if (KIND == kSlowCap && v == H.fv) S.res = capY ? Yn : Xn;
    if (lane == 31) S.q = Yn;
    S.DXp = DX;
    S.X = Xn;
    S.Y = Yn;
    S.prp = pr;
  }
}

// Row m's step lag behind row 0 of its lane: (0, 1, 3, 4).
__device__ __forceinline__ int lam4(int m) { return m + (m >> 1); }

// Builds lane `lane`'s cost profile of strip t into parity buffer t & 1
// (word [c] = four byte costs sc * cost[a_m][c], rows m = 0..3; the lane
// alone reads its column) and returns the strip's packed delete costs
// {row 0, row 2} and {row 1, row 3}.  Rows past the matrix (or strips out
// of range) use the gap character: their cells are never read.
template <int MODE>
__device__ __forceinline__ void build4(uint32_t sb, uint32_t prof0, const uint8_t *s1,
                                       const Geo4 &g, int t, int lane, int gap, int rank_d,
                                       bool profile, uint32_t &cdX, uint32_t &cdY) {
  constexpr int sc = MODE == kDpChoice ? 4 : 1;
  int a[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int r = 128 * t + 4 * lane + m;
    a[m] = (t >= 0 && t < g.T && r < g.L1) ? (int)s1[r] : gap;
  }
  const uint32_t ct = sb + kSmCtab;
  if (profile) {
    const uint32_t dst = prof0 + (uint32_t)(t & 1) * 4096u + 4u * lane;
#pragma unroll 4
    for (int c = 0; c < 32; ++c) {
      uint32_t wv = 0;
#pragma unroll
      for (int m = 0; m < 4; ++m) wv |= (sc * lds32(ct + 4 * (a[m] * 33 + c))) << (8 * m);
      sts32(dst + 128u * c, wv);
    }
  }
  uint32_t cd[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) cd[m] = sc * lds32(ct + 4 * (a[m] * 33 + gap)) + rank_d;
  cdX = cd[0] | (cd[2] << 16);
  cdY = cd[1] | (cd[3] << 16);
}

// Window entry of the column a lane reads at window position p of the
// block at offset o of period t0, in strip ts (t0 or t0 - 1): {shared
// address of profile row c of the strip's parity buffer, the insert costs
// g(c_p) | g(c_{p-1}) << 16 of this column and the one before, which are
// the row pairs' insert operands of that step}.  Column j = 128 ts + dlo +
// (t0 - ts) W + o - 93 + p; lane k reads p = v - 3k + 93 at step v (8-byte
// entries 24 bytes apart: no bank conflict within a half warp).
__device__ __forceinline__ int win_col(const Geo4 &g, int ts, int t0, int o, int p) {
  return 128 * ts + g.dlo + (t0 - ts) * g.W + o - k4WinBase + p;
}

template <int MODE>
__device__ __forceinline__ void lin4_pair(const LinDpArgs &A, uint32_t sb, int warp, int lane,
                                          const LinPlan &P, int64_t dm_off, int id,
                                          uint32_t *bnd) {
  constexpr int sc = MODE == kDpChoice ? 4 : 1;
  const Geo4 g = geo4(P);
  const uint8_t *s1 = A.seq + P.s1_off, *s2 = A.seq + P.s2_off;
  const int gap = A.gap;
  // backtrack priority (algn.c:3605-3666): insert before delete when swaped
  const bool swaped = A.swaped < 0 ? !P.swap : (A.swaped != 0);
  const int rank_i = MODE == kDpChoice ? (swaped ? 1 : 2) : 0;
  const int rank_d = MODE == kDpChoice ? 3 - rank_i : 0;
  const uint32_t gt = sb + kSmGt + 128u * rank_i;
  const uint32_t prof0 = sb + kSmProf + 8192u * warp;
  const uint32_t win0 = sb + kSmWin + 16u * k4Win * warp;
  const uint32_t lane4 = 4u * lane;
  const int qsrc = (lane + 1) & 31;
  const K4 K{(uint32_t)A.k.one, (uint32_t)A.k.m1, (uint32_t)A.k.four};
  const int bias = sc * (int)lds32(sb + kSmCtab + 4 * (s1[0] * 33 + s2[0]));

  // the row above strip 0: INF, except the seed of cell (0, 0)
  for (int x = lane; x < g.wd; x += 32) bnd[x] = (x == -g.dlo) ? 0u : (kInf16 << 16);
  uint32_t cdXc, cdYc, cdXp, cdYp, cdXn = 0, cdYn = 0;
  build4<MODE>(sb, prof0, s1, g, 0, lane, gap, rank_d, true, cdXc, cdYc);
  build4<MODE>(sb, prof0, s1, g, -1, lane, gap, rank_d, false, cdXp, cdYp);
  __syncwarp();

  // boundary input of lane L at the step 32b + L: the row above at band
  // index i + 1 (index W wraps to 0: the next strip's first align input)
  auto qload = [&](int t1, int o1) -> uint32_t {
    int x = o1 + lane + 1;
    if (x == g.W) x = 0;
    return x < g.wd ? bnd[x] : (kInf16 << 16);
  };
  // window chars of the block at (t0, o): positions lane + 32 i of the new
  // strip (t0) and of the old one (t0 - 1)
  // (chars of positions p and p - 1: ch[i][0..1] new strip, ch[i][2..3] old)
  auto wchars = [&](int t0, int o, int (&ch)[4][4]) {
    auto col = [&](int j) { return (j >= 0 && j < g.L2) ? (int)s2[j] : gap; };
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int p = lane + 32 * i;
      const int jn = win_col(g, t0, t0, o, p), jo = win_col(g, t0 - 1, t0, o, p);
      ch[i][0] = col(jn);
      ch[i][1] = col(jn - 1);
      ch[i][2] = col(jo);
      ch[i][3] = col(jo - 1);
    }
  };
  auto wstore = [&](int t0, const int (&ch)[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int p = lane + 32 * i;
#pragma unroll
      for (int h = 0; h < 2; ++h) {  // new strip t0, old strip t0 - 1
        const int c = ch[i][2 * h], cp = ch[i][2 * h + 1];
        const uint32_t pa = prof0 + (uint32_t)((t0 - h) & 1) * 4096u + 128u * c;
        sts64(win0 + 8u * (h * k4Win + p), pa, lds32(gt + 4 * c) | (lds32(gt + 4 * cp) << 16));
      }
    }
  };

  State4 S;
  S.X = S.Y = kInf2;
  S.DXp = lane == 0 ? ((kInf16 << 16) | (bnd[0] >> 16)) : kInf2;
  S.prp = 0;
  S.res = 0;
  S.q = qload(0, 0);
  S.up = lane == 0 ? S.q : kInf2;
  {
    int ch[4][4];
    wchars(0, 0, ch);
    wstore(0, ch);
  }
  __syncwarp();

  // the final cell (L1 - 1, L2 - 1): owner lane, register, half and step
  const int rf = g.L1 - 1;
  const int kf = (rf & 127) >> 2, mf = rf & 3;
  const int Gf = (rf >> 7) * g.W + k4Lag * kf + lam4(mf) + (g.L2 - 1 - rf - g.dlo);
  const bool capY = (mf & 1) != 0;
  uint32_t *dm = MODE == kDpChoice ? A.dm + dm_off : nullptr;
  const int slow_end0 = max(-g.dlo + (k4Lag - 4) * 31 + 1, k4R3);

  int t0 = 0, o = 0;
  for (int b = 0; b < g.nblk; ++b, o += 32) {
    if (o == g.W) {  // a new period: strip t0 becomes the lanes' new strip
      o = 0;
      ++t0;
      cdXp = cdXc;
      cdYp = cdYc;
      cdXc = cdXn;
      cdYc = cdYn;
    }
    const int G0 = 32 * b;
    // every lane is in strip t0 from step 217 on: its parity buffer's
    // other half (strip t0 - 1) is free for strip t0 + 1
    if (o == 224) build4<MODE>(sb, prof0, s1, g, t0 + 1, lane, gap, rank_d, true, cdXn, cdYn);
    const int o1 = (o + 32 == g.W) ? 0 : o + 32, t1 = (o1 == 0) ? t0 + 1 : t0;
    const uint32_t qn = qload(t1, o1);
    int ch[4][4];
    wchars(t1, o1, ch);

    int kind = kPlain;
    if (o + 31 >= g.W - g.G || o <= k4R3) kind = kMixed;
    if (t0 <= g.tri_last && o <= max(slow_end0 - 128 * t0, k4R3)) kind = kSlow;
    if ((Gf >> 5) == b) kind = kSlowCap;

    Half4 H;
    H.sw = k4Lag * lane - o;  // t0 W + 7k - G0
    H.wn = win0 + 8u * (uint32_t)(k4WinBase - 3 * lane);
    H.wo = H.wn + 8u * k4Win;
    H.cdXn = cdXc;
    H.cdYn = cdYc;
    H.cdXo = cdXp;
    H.cdYo = cdYp;
    {
      int ee = o - k4Lag * lane + g.G;  // steps past the lane's right-edge window
      if (ee > (g.W >> 1)) ee -= g.W;
      ee = min(max(ee, -40), 40);
      H.fe = sb + kSmEdge + 8u * (uint32_t)(ee + kEdgeOff);
    }
    H.ft = sb + kSmTri;
    H.tg = 0;
    if (kind >= kSlow) {
      const int off0 = -g.dlo - 128 * t0 - 4 * lane;  // row 0's first in-matrix band index
      const int var = min(max(off0, 0), 3);
      const int d0 = o - k4Lag * lane;
      int et = var == 3 ? d0 - off0 : d0;
      et = min(max(et, -40), 8);
      H.ft = sb + kSmTri + 8u * (uint32_t)(var * kTriN + et + kTriOff);
      H.tg = t0 == 0 ? -64 : H.sw;
    }
    H.fv = lane == kf ? Gf - G0 : -1;
#pragma unroll 1
    for (int e = 0; e < 2; ++e) {
      uint32_t ax0 = 0, ax1 = 0, ay0 = 0, ay1 = 0;
      if (kind == kPlain)
        l4_half<MODE, kPlain>(S, H, lane4, lane, qsrc, capY, K, ax0, ax1, ay0, ay1);
      else if (kind == kMixed)
        l4_half<MODE, kMixed>(S, H, lane4, lane, qsrc, capY, K, ax0, ax1, ay0, ay1);
      else if (kind == kSlow)
        l4_half<MODE, kSlow>(S, H, lane4, lane, qsrc, capY, K, ax0, ax1, ay0, ay1);
      else
        l4_half<MODE, kSlowCap>(S, H, lane4, lane, qsrc, capY, K, ax0, ax1, ay0, ay1);
      if (MODE == kDpChoice)
        *(uint4 *)(dm + ((int64_t)b * 32 + lane) * 8 + 4 * e) = make_uint4(ax0, ax1, ay0, ay1);
      H.sw -= 16;
      H.tg -= 16;
      H.fv -= 16;
      H.wn += 128u;  // 16 window positions
      H.wo += 128u;
      H.fe += 128u;
      H.ft += 128u;
    }
    // lane 31's row-3 values of this block (lane L holds step G0 + L)
    // become the boundary row of the next strip
    {
      int x = o + lane - k4R3;
      const int pstep = G0 + lane - k4R3;
      if (x < 0) x += g.W;
      if (pstep >= 0 && x < g.wd) bnd[x] = S.q;
    }
    S.q = qn;
    if (lane == 0) S.up = qn;  // lane 0's first input of the next block
    __syncwarp();
    wstore(t1, ch);
    __syncwarp();
  }
  const uint32_t res = __shfl_sync(kFull4, S.res, kf);
  if (lane == 0) A.cost[id] = ((int)((res >> (16 * (mf >> 1))) & 0xFFFFu) - bias) / sc;
}

// ---------------------------------------------------------------------------
// Traceback + medians of one pair by one thread, from the packed layout's
// 2-bit moves (backtrack_2d, algn.c:3551-3666; ancestor_2, algn.c:4126-4147;
// median_2_with_gaps, algn.c:4011-4024).  Direction words of (block, lane):
// half e holds {row 0/2 steps 0-7, steps 8-15, row 1/3 steps 0-7, 8-15},
// row 2 and 3 in the high halves.
// ---------------------------------------------------------------------------
__device__ __noinline__ void tb_pair4(const LinTbArgs &A, const uint8_t *med, int id) {
  const LinPlan P = A.plans[id];
  const int gap = A.gap;
  const int la = P.swap ? P.l2 : P.l1, lb = P.swap ? P.l1 : P.l2;
  const int64_t cap = slot_cap(la, lb);
  uint8_t *oa = A.out + A.out_off[id];
  uint8_t *ob = oa + cap, *ow = ob + cap, *om = ow + cap;
  const uint8_t *__restrict__ s1 = A.seq + P.s1_off;
  const uint8_t *__restrict__ s2 = A.seq + P.s2_off;
  if (P.empty) {
    // DOS.median: the non-empty (or second) sequence is the median
    const bool a_empty = P.empty == 1;
    const uint8_t *src = (a_empty != (bool)P.swap) ? s2 : s1;
    const int len = a_empty ? lb : la;
    for (int i = 0; i < len; ++i) om[cap - len + i] = src[i];
    A.out_len[2 * id] = 0;
    A.out_len[2 * id + 1] = len;
    return;
  }
  const Geo4 g = geo4(P);
  const uint4 *dm4 = (const uint4 *)(A.dm + A.dm_off[id]);
  const bool swaped = A.swaped < 0 ? !P.swap : (A.swaped != 0);
  int r = P.l1 - 1, j = P.l2 - 1;
  int n = 0, nm = 0;
  bool bad = false;
  uint4 cur = make_uint4(0, 0, 0, 0);
  int cur_key = -1;
  BackWriter3 wabw(oa + cap - 1, ob + cap - 1, ow + cap - 1);
  BackWriter wm(om + cap - 1);
  while (r > 0 || (r == 0 && j >= 0)) {
    const int k = (r & 127) >> 2, m = r & 3;
    const int bi = (j - r) - g.dlo;  // band index
    const int G = (r >> 7) * g.W + k4Lag * k + lam4(m) + bi;
    const int blk = G >> 5, vv = G & 31;
    if (j < 0 || bi < 0 || bi >= g.wd || blk >= g.nblk || n + 2 >= cap) {  // left the band: a bug
      bad = true;
      break;
    }
    const int key = (blk * 32 + k) * 2 + (vv >> 4);
    // both characters are read whatever the move (r, j >= 0 here), off the
    // read-only path, so that the loads issue ahead of the move's decode
    const int c1 = __ldg(s1 + r), c2 = __ldg(s2 + j);
    if (key != cur_key) {
      cur = dm4[key];
      cur_key = key;
    }
    const uint32_t w = (m & 1) ? ((vv & 8) ? cur.w : cur.z) : ((vv & 8) ? cur.y : cur.x);
    const uint32_t code = (w >> (2 * (7 - (vv & 7)) + 16 * (m >> 1))) & 3u;
    // rank 1 is insert when swaped, else delete
    const int move = code == 0 ? 0 : (((code == 1u) == swaped) ? 1 : 2);
    const bool dr = move != 1, dj = move != 2;  // consumes a row / a column
    const int cr = dr ? c1 : gap, cc = dj ? c2 : gap;
    r -= dr;
    j -= dj;
    const int ca = P.swap ? cc : cr, cb = P.swap ? cr : cc;
    const int md = med[(ca << 5) | cb];
    wabw.put((uint32_t)ca, (uint32_t)cb, (uint32_t)md);
    if (md != gap) {
      wm.put((uint32_t)md);
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

// The same traceback by the pair's whole warp, for small batches where
// every pair has its own warp.  tb_pair4's walk is one dependent chain of
// index arithmetic (a few hundred cycles per step for a lone warp); here the
// lanes read a stretch of the path at once.  Most moves are diagonal, so
// lane i reads the move of cell (r - i, j - i) on the current diagonal (the
// same band index); a ballot finds the first cell whose move is not
// diagonal, and the warp takes the diagonal run up to it plus that cell's
// move in one iteration, each lane writing its own column of the outputs
// (the gap-free median by a ballot prefix count).  The path and the bytes
// written are those of tb_pair4.  The direction words come from an 8-block
// window of the pair's direction matrix that all lanes load together into
// the warp's profile buffer (free once its fill is done); step positions
// never increase along the walk (a diagonal move or a delete lowers the
// row part of G by at least as much as the band index rises; an insert
// lowers the band index), so the window slides down.
__device__ __noinline__ void tb_pair4_solo(const LinTbArgs &A, const uint8_t *med, int id,
                                           uint4 *win, int lane) {
  const LinPlan P = A.plans[id];
  const int gap = A.gap;
  const int la = P.swap ? P.l2 : P.l1, lb = P.swap ? P.l1 : P.l2;
  const int64_t cap = slot_cap(la, lb);
  uint8_t *oa = A.out + A.out_off[id];
  uint8_t *ob = oa + cap, *ow = ob + cap, *om = ow + cap;
  const uint8_t *__restrict__ s1 = A.seq + P.s1_off;
  const uint8_t *__restrict__ s2 = A.seq + P.s2_off;
  if (P.empty) {
    // DOS.median: the non-empty (or second) sequence is the median
    const bool a_empty = P.empty == 1;
    const uint8_t *src = (a_empty != (bool)P.swap) ? s2 : s1;
    const int len = a_empty ? lb : la;
    for (int i = lane; i < len; i += 32) om[cap - len + i] = src[i];
    if (lane == 0) {
      A.out_len[2 * id] = 0;
      A.out_len[2 * id + 1] = len;
    }
    return;
  }
  const Geo4 g = geo4(P);
  const uint4 *dm4 = (const uint4 *)(A.dm + A.dm_off[id]);
  const int nq = g.nblk * 64;  // 16-byte words of the pair's direction matrix
  const bool swaped = A.swaped < 0 ? !P.swap : (A.swaped != 0);
  int r = P.l1 - 1, j = P.l2 - 1;  // the walk's cell (the same on every lane)
  int n = 0, nm = 0;
  int wlo = g.nblk;  // the window holds blocks [wlo, wlo + 8)
  bool bad = false;
  while (r > 0 || (r == 0 && j >= 0)) {
    const int bi = (j - r) - g.dlo;  // band index, constant along the diagonal
    const int G0 = (r >> 7) * g.W + k4Lag * ((r & 127) >> 2) + lam4(r & 3) + bi;
    const int blk0 = G0 >> 5;
    if (j < 0 || bi < 0 || bi >= g.wd || blk0 >= g.nblk || n + 2 >= cap) {  // left the band: a bug
      bad = true;
      break;
    }
    if (blk0 < wlo || blk0 >= wlo + 8) {
      wlo = max(blk0 - 7, 0);
      __syncwarp();
      for (int i = lane; i < 8 * 64; i += 32) {
        const int q = wlo * 64 + i;
        if (q < nq) win[i] = dm4[q];
      }
      __syncwarp();
    }
    // lane i: the move of cell (r - i, j - i); 4 = not read (the run stops
    // before this cell: outside the matrix, the output slot or the window)
    const int ri = r - lane, ji = j - lane;
    uint32_t code = 4;
    if (ri >= 0 && ji >= 0 && n + lane + 2 < cap) {
      const int k = (ri & 127) >> 2, m = ri & 3;
      const int G = (ri >> 7) * g.W + k4Lag * k + lam4(m) + bi;
      const int blk = G >> 5, vv = G & 31;
      if (blk >= wlo) {
        const uint4 cur = win[(blk - wlo) * 64 + k * 2 + (vv >> 4)];
        const uint32_t w = (m & 1) ? ((vv & 8) ? cur.w : cur.z) : ((vv & 8) ? cur.y : cur.x);
        code = (w >> (2 * (7 - (vv & 7)) + 16 * (m >> 1))) & 3u;
      }
    }
    const uint32_t stop = __ballot_sync(kFull4, code != 0);
    const int f = stop ? __ffs(stop) - 1 : 32;  // lanes below f move diagonally
    const uint32_t cf = __shfl_sync(kFull4, code, f & 31);
    const bool step_f = f < 32 && cf != 4;  // lane f's cell was read: its move too
    // rank 1 is insert when swaped, else delete
    const int move_f = step_f ? (((cf == 1u) == swaped) ? 1 : 2) : 0;
    const bool writes = lane < f || (lane == f && step_f);
    int md = gap;
    if (writes) {
      const bool dr = lane < f || move_f != 1, dj = lane < f || move_f != 2;
      const int cr = dr ? (int)__ldg(s1 + ri) : gap, cc = dj ? (int)__ldg(s2 + ji) : gap;
      const int ca = P.swap ? cc : cr, cb = P.swap ? cr : cc;
      md = med[(ca << 5) | cb];
      const int64_t pos = cap - 1 - (n + lane);
      oa[pos] = (uint8_t)ca;
      ob[pos] = (uint8_t)cb;
      ow[pos] = (uint8_t)md;
    }
    const bool keep = writes && md != gap;
    const uint32_t kb = __ballot_sync(kFull4, keep);
    if (keep) om[cap - 1 - (nm + __popc(kb & ((1u << lane) - 1u)))] = (uint8_t)md;
    n += f + (step_f ? 1 : 0);
    nm += __popc(kb);
    r -= f + ((step_f && move_f != 1) ? 1 : 0);
    j -= f + ((step_f && move_f != 2) ? 1 : 0);
  }
  if (lane == 0) {
    // ancestor_2 ends with the leading gap (algn.c:4140-4141)
    if (!bad) om[cap - 1 - nm] = (uint8_t)gap;
    A.out_len[2 * id] = bad ? -1 : (int32_t)n;
    A.out_len[2 * id + 1] = bad ? -1 : (int32_t)(nm + 1);
  }
  __syncwarp();
}

template <int MODE>
__global__ void __launch_bounds__(k4Warps * 32, 2) k_lin_dp4(LinDpArgs A) {
  extern __shared__ __align__(128) unsigned char lin4_dsm[];
  const uint32_t raw = (uint32_t)__cvta_generic_to_shared(lin4_dsm);
  const uint32_t sb = (raw + 127u) & ~127u;
  uint8_t *med = lin4_dsm + (sb - raw) + kSmMed;
  constexpr int sc = MODE == kDpChoice ? 4 : 1;
  // cost table, insert costs per rank, mask tables, median table
  for (int i = threadIdx.x; i < 32 * 33; i += blockDim.x) {
    const int a = i / 33, b = i - 33 * a;
    sts32(sb + kSmCtab + 4 * i, b < 32 ? (A.tables->packed[(a << 5) | b] & 0xffffu) : 0u);
  }
  if (threadIdx.x < 96) {
    // insert cost of column char c: cost[gap][c] (the high half of any
    // packed entry of column c), scaled, plus the insert rank 0, 1 or 2
    const int rk = threadIdx.x >> 5, c = threadIdx.x & 31;
    sts32(sb + kSmGt + 4 * threadIdx.x,
          sc * (A.tables->packed[c] >> 16) + (MODE == kDpChoice ? rk : 0));
  }
  for (int i = threadIdx.x; i < kEdgeN; i += blockDim.x) {
    const int e = i - kEdgeOff;
    const uint32_t mx = (e == 0 ? 0xFFFFu : 0u) | (e == 3 ? 0xFFFF0000u : 0u);
    const uint32_t my = (e == 1 ? 0xFFFFu : 0u) | (e == 4 ? 0xFFFF0000u : 0u);
    sts64(sb + kSmEdge + 8 * i, mx, my);
  }
  for (int i = threadIdx.x; i < 4 * kTriN; i += blockDim.x) {
    const int var = i / kTriN, e = i - var * kTriN - kTriOff;
    // thresholds of rows 0..3 (row 0's first in-matrix index clipped to 3)
    const int th0 = var == 3 ? 0 : var, th1 = var == 3 ? 0 : max(var, 1);
    const int th2 = var == 3 ? 1 : 3, th3 = var == 3 ? 1 : 4;
    const uint32_t mx = (e < th0 ? 0xFFFFu : 0u) | (e < th2 ? 0xFFFF0000u : 0u);
    const uint32_t my = (e < th1 ? 0xFFFFu : 0u) | (e < th3 ? 0xFFFF0000u : 0u);
    sts64(sb + kSmTri + 8 * i, mx, my);
  }
  if (MODE == kDpChoice && A.fuse_tb)
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) med[i] = A.tables->median[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  uint32_t *bnd = (uint32_t *)A.scratch + gw * A.slab;
  // Every warp's first pair is fixed by position, warp-major over the
  // blocks (consecutive pairs on different blocks, so on different SMs):
  // a small batch then runs one pair per SM instead of sharing schedulers.
  // Later pairs come from the counter, past the first wave.
  const int nwarps = (int)gridDim.x * k4Warps;
  int p = warp * (int)gridDim.x + (int)blockIdx.x;
  for (;; p = __shfl_sync(kFull4, lane == 0 ? atomicAdd(A.counter, 1) + nwarps : 0, 0)) {
    if (p >= A.n) break;
    const int id = A.order ? A.order[p] : p;
    const LinPlan P = A.plans[id];
    if (P.empty) {
      if (lane == 0) A.cost[id] = 0;
    } else {
      lin4_pair<MODE>(A, sb, warp, lane, P, MODE == kDpChoice ? A.dm_off[id] : 0, id, bnd);
    }
    if (MODE == kDpChoice && A.fuse_tb && A.tb_solo) {
      __syncwarp();  // the fill's direction words and profile reads are done
      tb_pair4_solo(A.tb, med, id,
                    (uint4 *)(lin4_dsm + (sb - raw) + kSmProf + warp * 8192), lane);
    } else if (MODE == kDpChoice && A.fuse_tb) {
      // Publish this pair's direction matrix; the warp completing the batch
      // (no waiting: the count tells) walks all of its pairs, one per lane.
      __syncwarp();
      const int bt = p / kLanes;
      const int size = min(kLanes, A.n - bt * kLanes);
      int last = 0;
      if (lane == 0) {
        __threadfence();
        last = atomicAdd(A.batch_done + bt, 1) == size - 1;
      }
      if (__shfl_sync(kFull4, last, 0)) {
        __threadfence();
        if (lane < size)
          tb_pair4(A.tb, med, A.order ? A.order[bt * kLanes + lane] : bt * kLanes + lane);
        if (A.done) {
          __threadfence_system();
          __syncwarp();
          if (lane == 0) *(volatile int *)(A.done + bt) = 1;
        }
        __syncwarp();
      }
    }
  }
}

template <int MODE>
int lin_dp4_prepare(int dev) {
  static int done[64] = {};
  if (!done[dev & 63]) {
    cudaFuncSetAttribute(k_lin_dp4<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmBytes);
    done[dev & 63] = 1;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lin_dp4<MODE>, k4Warps * 32,
                                                kSmBytes);
  return per_sm;
}

}  // namespace

int lin_dp4_blocks(int mode) {
  static int cache[3][64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  int &c = cache[mode == kDpChoice ? 1 : 0][dev & 63];
  if (!c) {
    const int per_sm = mode == kDpChoice ? lin_dp4_prepare<kDpChoice>(dev)
                                         : lin_dp4_prepare<kDpCost>(dev);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    c = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  return c;
}

int lin_dp4_warps() { return k4Warps; }

void launch_lin_dp4(const LinDpArgs &A, int mode, int blocks, cudaStream_t st) {
  if (mode == kDpChoice) k_lin_dp4<kDpChoice><<<blocks, k4Warps * 32, kSmBytes, st>>>(A);
  else k_lin_dp4<kDpCost><<<blocks, k4Warps * 32, kSmBytes, st>>>(A);
}

}  // namespace poyd
