/*
 * poyd_gb300 -- C ABI of the GB300 (sm_103a) direct-optimization scoring path.
 *
 * Plain pointers and sizes only.  Sequences use POY's bitmask alphabet (DNA:
 * A=1, C=2, G=4, T=8, gap=16, ambiguity codes are unions) and start with the
 * leading gap at position 0, exactly like the reference's `struct seq`
 * contents (seq.h:46-54).  Output sequences are written the way the reference
 * prepends into a `seq`: right-aligned at the END of a caller-provided slot,
 * so element i of a result of length n sits at slot[cap - n + i].
 *
 * Every entry point returns 0 on success or a negative POYD_E* code; the
 * reference instead raises an OCaml exception through failwith
 * (matrices.c:107-113, cm.c:345-358), which an OCaml stub over this ABI
 * would do on a non-zero return.  poyd_last_error() gives the message.
 *
 * Device pointers are CUDA global-memory pointers; `stream` is a
 * cudaStream_t (NULL = legacy default stream).
 *
 * Threads: the library keeps one grow-only scratch workspace per (device,
 * stream).  Calls from several host threads are safe when each thread uses
 * its own stream; calls that share a stream must not overlap in time (the
 * same rule as a cuBLAS handle).  The single-pair affine and column entry
 * points (poyd_algn_*_affine_3, poyd_algn_median_2_*, ancestor_2, worst_2,
 * verify_2) run on the legacy default stream and count as calls on it.
 * poyd_algn_simple_2 / backtrack_2d / align_2d work in the poyd_matrix they
 * are given, so two threads need two matrices, as two OCaml domains would
 * need two Matrix.m.  poyd_align_2_host serialises itself per device.  The
 * message of poyd_last_error() is per thread.
 */
#ifndef POYD_GB300_H
#define POYD_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define POYD_OK 0
#define POYD_EINVAL -1   /* bad argument */
#define POYD_ECUDA -2    /* CUDA runtime error */
#define POYD_ERANGE -3   /* costs or lengths outside the supported range */
#define POYD_ENOMEM -4   /* device allocation failed */
#define POYD_EUNSUP -5   /* cost matrix form the GPU path does not implement */

/*
 * Two-dimensional transformation cost matrix over the bitmask alphabet,
 * restricted to lcm <= 5 (struct cm, cm.h:29-43).  Tables are indexed
 * (a << 5) + b.  Built by poyd_cm_dna / poyd_cm_of_matrix5, which restate
 * Cost_matrix.Two_D's constructors (cost_matrix.ml:520-656).
 */
typedef struct poyd_cm {
    int32_t lcm;
    int32_t gap;
    int32_t a_sz;
    int32_t combinations;
    int32_t cost_model; /* 0 linear, 1 affine (Cost_matrix.cost_model) */
    int32_t gap_open;
    int32_t is_metric;
    int32_t all_elements;
    int32_t cost[1024];
    int32_t worst[1024];
    int32_t prepend[32];
    int32_t tail[32];
    uint8_t median[1024];
} poyd_cm;

const char *poyd_last_error(void);
int poyd_version(void);
/* Frees the device scratch the library keeps between calls (grow-only, per
 * device and stream; the three-sequence choice cubes can reach tens of GB)
 * for the current device.  No call of the library may be in flight on that
 * device.  No reference counterpart (the reference frees its matrices with
 * the OCaml custom block). */
int poyd_workspace_release(void);

/* Replaces Cost_matrix.Two_D.of_transformations_and_gaps true 5 sub indel 31
 * (cost_matrix.ml:645-656) followed, for gap_open >= 0, by
 * Cost_matrix.Two_D.set_affine (cost_matrix.ml:405-416).  gap_open < 0 keeps
 * the linear model (Cost_matrix.Two_D.default is poyd_cm_dna(m, 1, 2, -1)). */
int poyd_cm_dna(poyd_cm *m, int32_t sub, int32_t indel, int32_t gap_open);
/* Replaces Cost_matrix.Two_D.of_list ~use_comb:true over a 5x5 matrix
 * (A, C, G, T, gap) (cost_matrix.ml:559-563, 520-538), then set_affine as
 * above. */
int poyd_cm_of_matrix5(poyd_cm *m, const int32_t *mat25, int32_t gap_open);

/* ---------------------------------------------------------------------
 * Batched pairwise direct optimization (device-resident inputs).
 *
 * `seq` is one device buffer holding every sequence; pair i is
 * a = seq[a_off[i] .. a_off[i]+a_len[i]) and b likewise, in the caller's
 * argument order (the order Sequence.Align.cost_2/align_2 receive).  All
 * per-pair arrays are device arrays of length n.
 * ------------------------------------------------------------------- */

/* deltaw policies for the linear band (sequence.ml:691-713) */
#define POYD_DELTAW_DEFAULT 0 /* cost_2 without ?deltaw (align_2, median) */
#define POYD_DELTAW_EXPLICIT 1 /* cost_2 ~deltaw:deltaw[i] */
#define POYD_DELTAW_DOS_DISTANCE 2 /* DOS.distance: max(|la-lb|, 8) (seqCS.ml:856-866) */
#define POYD_DELTAW_RAW 3 /* deltaw[i] is algn_CAML_simple_2's deltawh as is */

/* Batched Sequence.Align.cost_2 (sequence.ml:716-723): for each pair the
 * linear banded cost algn_CAML_simple_2 (algn.c:3409-3427) with the deltaw
 * policy above, or, for an affine matrix, algn_CAML_cost_affine_3
 * (algn.c:2628-2680).  cost[i] receives the result.  band_cells, when not
 * NULL, receives the number of DP cells the reference's band evaluates for
 * each pair (the unit of the GCUPS metric). */
int poyd_cost_2_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                      const int64_t *a_off, const int32_t *a_len,
                      const int64_t *b_off, const int32_t *b_len,
                      int32_t deltaw_policy, const int32_t *deltaw,
                      int32_t *cost, int64_t *band_cells, void *stream);

/* poyd_cost_2_batch for callers that cannot allocate device memory.  It has
 * no counterpart in the reference (whose C code mallocs host scratch per
 * call).  Some callers cannot call cudaMalloc: a C stub running inside a
 * host that owns the CUDA context and its memory pool, or a service with a
 * fixed device-memory budget.  This entry point allocates nothing: its
 * scratch (plans, counters,
 * cost tables, per-warp boundary rows) is one fixed ~24 MiB __device__ array
 * in the library, held by every GPU that loads the library until exit.
 * Linear model only; at most 65,536 pairs per call and bands up to 1,984
 * diagonals, else POYD_ERANGE before any DP kernel runs.  All calls share the
 * array, so calls that overlap on the GPU race and must be serialised by the
 * caller.  The call waits for its stream once (it reads the plan's error
 * flags back before the DP launch), so a stream that is being captured is
 * refused with POYD_EUNSUP.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress); make that first call before
 * any stream capture. */
int poyd_cost_2_batch_noalloc(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                              const int64_t *a_off, const int32_t *a_len,
                              const int64_t *b_off, const int32_t *b_len,
                              int32_t deltaw_policy, const int32_t *deltaw,
                              int32_t *cost, void *stream);

/* Batched DOS.median composition (seqCS.ml:747-776) with its pieces:
 *   linear: align_2 (cost_2 + backtrack_2d, sequence.ml:849-869,
 *           algn.c:3551-3666), ancestor_2 (algn.c:4126-4147) and
 *           median_2_with_gaps (algn.c:4011-4024);
 *   affine: align_affine_3 (algn.c:2551-2619).
 * Pair i owns the device slot out + out_off[i] of 4*cap_i bytes,
 * cap_i = a_len[i] + b_len[i] + 2 rounded up to a multiple of 4 (the longest
 * alignment plus the leading gap; the rounding keeps every pair's outputs
 * word aligned alike when out_off[i] is a multiple of 4), split in four
 * right-aligned sequences:
 *   [0, cap)      aligned a         (align_2's s1p / affine resi)
 *   [cap, 2cap)   aligned b         (s2p / resj)
 *   [2cap, 3cap)  median with gaps  (median_2_with_gaps / medianwg)
 *   [3cap, 4cap)  median            (ancestor_2 / affine median)
 * out_len[2i] = aligned length, out_len[2i+1] = median length.
 * With POYD_FLAG_DOS_EMPTY, a pair whose a (or b) is all gaps returns cost 0
 * and median = the other sequence, as DOS.median does (seqCS.ml:749-752). */
#define POYD_FLAG_DOS_EMPTY 1
int poyd_align_2_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                       const int64_t *a_off, const int32_t *a_len,
                       const int64_t *b_off, const int32_t *b_len,
                       int32_t *cost, uint8_t *out, const int64_t *out_off,
                       int32_t *out_len, int64_t *band_cells, int32_t flags,
                       void *stream);

/* Packs the results of poyd_align_2_batch for a download (no reference
 * counterpart: the reference hands back one seq block per call).  Pair i's
 * aligned a, aligned b and median with gaps (out_len[2i] bytes each) and its
 * median (out_len[2i+1] bytes) are copied back to back, in that order, to
 * packed + packed_off[i], where packed_off[i] is the sum over j < i of
 * 3 * out_len[2j] + out_len[2j+1].  Device pointers; asynchronous on
 * `stream`.  POYD_ERANGE is not checked here: pass only out_len >= 0. */
int poyd_pack_alignments(int32_t n, const uint8_t *out, const int64_t *out_off,
                         const int32_t *a_len, const int32_t *b_len,
                         const int32_t *out_len, uint8_t *packed,
                         const int64_t *packed_off, void *stream);

/* Column operations on aligned pairs (a_i and b_i both len[i] bytes, the
 * output of an alignment), the DP-free externals of sequence.ml:453-758:
 *   median_2_with_gaps: algn_CAML_median_2_with_gaps (algn.c:4011-4024)
 *   median_2_no_gaps:   algn_CAML_median_2_no_gaps (algn.c:4031-4046)
 *   ancestor_2:         algn_CAML_ancestor_2 (algn.c:4126-4147, with the
 *                       affine block correction algn.c:4080-4119)
 *   worst_2, verify_2:  algn_CAML_worst_2 / algn_CAML_verify_2, the cost of
 *                       the alignment under the worst / cost table with gap
 *                       openings per block (algn.c:3316-3370)
 * Batched forms: device pointers, asynchronous on `stream`; pair i's result
 * is right-aligned in out + out_off[i] (capacity len[i] + 1), its length in
 * out_len[i]; worst/verify write value[i].  Single-pair forms (poyd_algn_*):
 * host pointers, synchronous; the result is written from out[0]. */
int poyd_median_2_with_gaps_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                                  const int64_t *a_off, const int64_t *b_off,
                                  const int32_t *len, uint8_t *out, const int64_t *out_off,
                                  int32_t *out_len, void *stream);
int poyd_median_2_no_gaps_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                                const int64_t *a_off, const int64_t *b_off,
                                const int32_t *len, uint8_t *out, const int64_t *out_off,
                                int32_t *out_len, void *stream);
int poyd_ancestor_2_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                          const int64_t *a_off, const int64_t *b_off, const int32_t *len,
                          uint8_t *out, const int64_t *out_off, int32_t *out_len,
                          void *stream);
int poyd_worst_2_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                       const int64_t *a_off, const int64_t *b_off, const int32_t *len,
                       int32_t *value, void *stream);
int poyd_verify_2_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                        const int64_t *a_off, const int64_t *b_off, const int32_t *len,
                        int32_t *value, void *stream);
int poyd_algn_median_2_with_gaps(const uint8_t *a, const uint8_t *b, int32_t len,
                                 const poyd_cm *cm, uint8_t *out, int32_t *out_len);
int poyd_algn_median_2_no_gaps(const uint8_t *a, const uint8_t *b, int32_t len,
                               const poyd_cm *cm, uint8_t *out, int32_t *out_len);
int poyd_algn_ancestor_2(const uint8_t *a, const uint8_t *b, int32_t len,
                         const poyd_cm *cm, uint8_t *out, int32_t *out_len);
int poyd_algn_worst_2(const uint8_t *a, const uint8_t *b, int32_t len,
                      const poyd_cm *cm, int32_t *value);
int poyd_algn_verify_2(const uint8_t *a, const uint8_t *b, int32_t len,
                       const poyd_cm *cm, int32_t *value);

/* Host-buffer form of poyd_align_2_batch for a caller whose sequences live
 * in host memory (an OCaml stub over seq blocks, which the reference aligns
 * one pair per call, sequence.ml:849-869).  seq, a_off, a_len, b_off, b_len
 * are host arrays (seq in page-locked memory for a fast upload).  The batch
 * runs as one DP launch.  Its output slots (4*cap_i bytes each, the layout
 * of poyd_align_2_batch) are laid out in the order the DP finishes them, so
 * they are downloaded while the DP runs.  The library sets out_off[i]: pair
 * i's slot starts at out + out_off[i].  out (host, page-locked for overlap)
 * must hold out_cap >= sum of 4 * cap_i bytes (POYD_ERANGE otherwise).
 * Synchronous: on return cost[n], out_len[2n] and the slots are in host
 * memory.  Linear matrices stream; affine ones download after the DP.
 * Calls on one device are serialised. */
int poyd_align_2_host(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                      const int64_t *a_off, const int32_t *a_len,
                      const int64_t *b_off, const int32_t *b_len,
                      int32_t *cost, uint8_t *out, int64_t out_cap,
                      int64_t *out_off, int32_t *out_len, int32_t flags);

/* Batched Sequence.Align.closest (sequence.ml:967-1033), the final-state
 * step of DOS.to_single (seqCS.ml:730-745) that AllDirChar.assign_single
 * runs from the root outwards (allDirChar.ml:288-328): for pair i, the
 * single sequence of node m_i given its parent's single sequence p_i.
 * The pair is aligned as by poyd_align_2_batch (same slots, cap_i from
 * p_len[i] and m_len[i]; cost[i] = that alignment's cost), then every
 * column of m_i takes its state closest to p_i's column
 * (Cost_matrix.Two_D.get_closest, cost_matrix.ml:681-698: lowest state
 * bit among the cheapest), gaps are dropped and the leading gap kept.
 * Identical sequences are not aligned: their gap bits past position 0
 * are cleared instead (sequence.ml:1003-1013).  The single sequence is
 * written right-aligned in the slot's fourth segment [3cap, 4cap) with
 * its length in out_len[2i+1]; out_len[2i+1] = -1 if the alignment
 * failed, -2 if a column has no state.  m_i all gaps gives m_i.  With
 * POYD_FLAG_DOS_EMPTY, a parent that is all gaps is replaced by m_i
 * (DOS.to_single's rule).  Needs a matrix with combinations. */
int poyd_closest_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                       const int64_t *p_off, const int32_t *p_len,
                       const int64_t *m_off, const int32_t *m_len,
                       int32_t *cost, uint8_t *out, const int64_t *out_off,
                       int32_t *out_len, int32_t flags, void *stream);

/* ---------------------------------------------------------------------
 * Single-pair drop-ins with the OCaml externals' argument order
 * (sequence.ml:453-466, 731-758).  Host pointers; each call runs the
 * device path on one pair and synchronises.  A poyd_matrix plays the role
 * of Matrix.m: algn_CAML_simple_2 leaves the direction matrix of its pair
 * in it and algn_CAML_backtrack_2d reads it back (algn.c:3908-3924).
 * ------------------------------------------------------------------- */
typedef struct poyd_matrix poyd_matrix;
poyd_matrix *poyd_matrix_create(void);
void poyd_matrix_free(poyd_matrix *m);

/* algn_CAML_simple_2(s1, s2, cm, mat, deltawh): s1 is the longer sequence
 * (algn.c:3281); returns the cost through *cost. */
int poyd_algn_simple_2(const uint8_t *s1, int32_t l1, const uint8_t *s2,
                       int32_t l2, const poyd_cm *cm, poyd_matrix *mat,
                       int32_t deltawh, int32_t *cost);
/* algn_CAML_backtrack_2d(s1, s2, s1p, s2p, mat, cm, swap): prepends into
 * s1p/s2p (capacity cap each, right-aligned) and sets their lengths. */
int poyd_algn_backtrack_2d(const uint8_t *s1, int32_t l1, const uint8_t *s2,
                           int32_t l2, uint8_t *s1p, uint8_t *s2p,
                           int32_t cap, int32_t *len, poyd_matrix *mat,
                           const poyd_cm *cm, int32_t swaped);
/* algn_CAML_align_2d(s1, s2, cm, mat, s1p, s2p, deltawh, swaped)
 * (algn.c:3987-3996): poyd_algn_simple_2 then poyd_algn_backtrack_2d. */
int poyd_algn_align_2d(const uint8_t *s1, int32_t l1, const uint8_t *s2,
                       int32_t l2, const poyd_cm *cm, poyd_matrix *mat,
                       uint8_t *s1p, uint8_t *s2p, int32_t cap, int32_t *len,
                       int32_t deltawh, int32_t swaped, int32_t *cost);
/* algn_CAML_cost_affine_3(si, sj, cm, mat). */
int poyd_algn_cost_affine_3(const uint8_t *si, int32_t li, const uint8_t *sj,
                            int32_t lj, const poyd_cm *cm, int32_t *cost);
/* algn_CAML_align_affine_3(si, sj, cm, mat, resi, resj, median, medianwg):
 * four right-aligned outputs of capacity cap = li + lj + 2 each. */
int poyd_algn_align_affine_3(const uint8_t *si, int32_t li, const uint8_t *sj,
                             int32_t lj, const poyd_cm *cm, uint8_t *resi,
                             uint8_t *resj, uint8_t *median, uint8_t *medianwg,
                             int32_t cap, int32_t *lens /* [3]: res, median, medianwg */,
                             int32_t *cost);

/* ---------------------------------------------------------------------
 * Three-sequence alignment of the Iterative (ThreeD) cost mode
 * (sequence.ml:1075-1140, ukkCommon.c, ukk.checkp.c).  Sequences carry
 * their leading gap; every other element must hold one of A, C, G, T
 * (the lowest such bit is the character aligned, as powell_3D_align's
 * copySequence does, ukkCommon.c:84-105).  The cost is Powell's optimum
 * (alignmentCost, ukkCommon.c:345-391); among equally cheap alignments the
 * GPU keeps, from the end, the lowest-numbered final state and at every
 * column the lowest-numbered previous state (Powell's recursion can return
 * another optimal one).  Each sequence is at most 4,096 elements; the
 * choice cube needs 8 bytes per cell of la x lb x lc.
 * ------------------------------------------------------------------- */
/* powell_3D_align(sa, sb, sc, ra, rb, rc, mm, go, ge) (ukkCommon.c:111-143)
 * with host buffers: the aligned rows, leading gap column first, are
 * written right-aligned into ra/rb/rc of capacity cap (at least
 * la + lb + lc - 2), their length to *len, the cost to *cost. */
int poyd_powell_3D_align(const uint8_t *sa, int32_t la, const uint8_t *sb, int32_t lb,
                         const uint8_t *sc, int32_t lc, uint8_t *ra, uint8_t *rb, uint8_t *rc,
                         int32_t cap, int32_t *len, int32_t mm, int32_t go, int32_t ge,
                         int32_t *cost);
/* Cost_matrix.Three_D.median over a DNA combination matrix
 * (Three_D.of_two_dim_comb, cost_matrix.ml:803-851) into a host table of
 * 32,768 bytes indexed (i << 10) | (j << 5) | k. */
int poyd_cm_median3(const poyd_cm *cm, uint8_t *tab);
/* Batched align_3_powell (sequence.ml:1078-1087) with the median of
 * align_3_powell_inter (sequence.ml:1103-1115) when median3 (a host table
 * from poyd_cm_median3) is given.  Device arrays.  Triple i owns the slot
 * out + out_off[i] of 4*cap_i bytes, cap_i = a_len + b_len + c_len rounded
 * up to a multiple of 4, split in four right-aligned sequences: aligned a,
 * aligned b, aligned c, median.  out_len[2i] = aligned length (with the
 * leading gap column), out_len[2i+1] = median length (0 without median3).
 * A triple with an element lacking A, C, G and T gets cost -1 and the call
 * returns POYD_EINVAL after finishing the others. */
int poyd_powell_3d_batch(int32_t n, const uint8_t *seq, const int64_t *a_off,
                         const int32_t *a_len, const int64_t *b_off, const int32_t *b_len,
                         const int64_t *c_off, const int32_t *c_len, int32_t mm, int32_t go,
                         int32_t ge, const uint8_t *median3, int32_t *cost, uint8_t *out,
                         const int64_t *out_off, int32_t *out_len, void *stream);
/* Batched Sequence.Align.readjust_3d s1 s2 m cm cm3 p with first_gap true
 * (sequence.ml:1117-1140): the early returns (equal lengths keep m; an
 * empty child or parent gives the other sequence), otherwise the median of
 * align_3_powell_inter (s1, s2, p) with mm = cost 1 2, go = the affine
 * opening (0 for the linear model), ge = cost 1 16 and cm3 =
 * Three_D.of_two_dim cm.  Slots as poyd_powell_3d_batch with c = p; the
 * new median is the fourth sequence (out_len[2i] = 0 for an early return);
 * cost[i] is the returned cost and changed[i] = (new median <> m). */
int poyd_readjust_3d_batch(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                           const int64_t *s1_off, const int32_t *s1_len,
                           const int64_t *s2_off, const int32_t *s2_len,
                           const int64_t *m_off, const int32_t *m_len,
                           const int64_t *p_off, const int32_t *p_len, int32_t *cost,
                           uint8_t *out, const int64_t *out_off, int32_t *out_len,
                           int32_t *changed, void *stream);

/* ---------------------------------------------------------------------
 * Fitch non-additive characters, 8-bit state masks (NonaddCS8).
 * Batched over candidate pairs: row k of the result uses node rows
 * a_idx[k] and b_idx[k] of `nodes` (device, n_nodes x len bytes, row
 * stride `stride` bytes, a multiple of 16).
 * ------------------------------------------------------------------- */
/* char_nonadd8_CAML_distance (nonaddCSc.c:1076-1105) per candidate. */
int poyd_nonadd8_distance_batch(const uint8_t *nodes, int64_t stride,
                                int32_t len, int32_t n, const int32_t *a_idx,
                                const int32_t *b_idx, int64_t *dist,
                                void *stream);
/* nonadd_median (nonaddCSc.c:422-462) per candidate: median rows into
 * `out` (n x stride) and added_cost[k]. */
int poyd_nonadd8_median_batch(const uint8_t *nodes, int64_t stride,
                              int32_t len, int32_t n, const int32_t *a_idx,
                              const int32_t *b_idx, uint8_t *out,
                              int64_t *added_cost, void *stream);
/* nonadd_median_3 (nonaddCSc.c:472-544) per node: final states. */
int poyd_nonadd8_median_3_batch(const uint8_t *nodes, int64_t stride,
                                int32_t len, int32_t n, const int32_t *anc,
                                const int32_t *prelim, const int32_t *d1,
                                const int32_t *d2, uint8_t *out, void *stream);

/* Fitch on 16- and 32-bit state sets (NonaddCS16 / NonaddCS32: nonaddCSc.c
 * built with CHARSIZE 16 / 32, characters of 9-16 / 17-32 states).  The
 * same three operations and arguments as the 8-bit batches, with node rows
 * of `len` characters of 2 / 4 bytes (host byte order): stride a multiple
 * of 16 bytes and at least len x 2 (x 4) rounded up to 16. */
int poyd_nonadd16_distance_batch(const void *nodes, int64_t stride,
                                 int32_t len, int32_t n, const int32_t *a_idx,
                                 const int32_t *b_idx, int64_t *dist,
                                 void *stream);
int poyd_nonadd16_median_batch(const void *nodes, int64_t stride, int32_t len,
                               int32_t n, const int32_t *a_idx,
                               const int32_t *b_idx, void *out,
                               int64_t *added_cost, void *stream);
int poyd_nonadd16_median_3_batch(const void *nodes, int64_t stride,
                                 int32_t len, int32_t n, const int32_t *anc,
                                 const int32_t *prelim, const int32_t *d1,
                                 const int32_t *d2, void *out, void *stream);
int poyd_nonadd32_distance_batch(const void *nodes, int64_t stride,
                                 int32_t len, int32_t n, const int32_t *a_idx,
                                 const int32_t *b_idx, int64_t *dist,
                                 void *stream);
int poyd_nonadd32_median_batch(const void *nodes, int64_t stride, int32_t len,
                               int32_t n, const int32_t *a_idx,
                               const int32_t *b_idx, void *out,
                               int64_t *added_cost, void *stream);
int poyd_nonadd32_median_3_batch(const void *nodes, int64_t stride,
                                 int32_t len, int32_t n, const int32_t *anc,
                                 const int32_t *prelim, const int32_t *d1,
                                 const int32_t *d2, void *out, void *stream);

/* ---------------------------------------------------------------------
 * Sankoff characters (SankCS, sankCS.ml:302-377).  k states per character
 * (k <= 8), nchar characters per node; per-node data int32
 * [nchar][k] with the sentinel POYD_SANK_INF standing for OCaml's
 * max_int/4 (saturating arithmetic, sankCS.ml:34-67).  tcm: device
 * [k][k].
 * ------------------------------------------------------------------- */
#define POYD_SANK_INF (1 << 30)
/* elt_median over all characters for each candidate (a_idx[i], b_idx[i]):
 * writes s (c), e and beta rows of the median and, when cost != NULL, the
 * node's median cost sum_char min_s c (SankCS.median + cost). */
int poyd_sank_median_batch(const int32_t *nodes, int32_t nchar, int32_t k,
                           const int32_t *tcm, int32_t n, const int32_t *a_idx,
                           const int32_t *b_idx, int32_t *out_s,
                           int32_t *out_e, int32_t *out_beta, void *stream);
/* SankCS.median_3 / elt_median_3 (sankCS.ml:402-452, called by the
 * uppass, node.ml:478 and allDirChar.ml:1399-1424), per pair i and
 * character: the final e row and best-state bits of node node[i] from its
 * ancestor's final (fin_e / fin_best rows anc[i]: int32 [nchar][k] and
 * [nchar], a bit per state), its preliminary s row (nodes[node[i]]) and its
 * children's preliminary s rows (nodes[left[i]], nodes[right[i]]; a leaf
 * passes itself).  An ancestor's best-state bits must be non-zero (the
 * root's final holds its cheapest states).  Writes out_e [n][nchar][k] and
 * out_best [n][nchar]. */
int poyd_sank_median_3_batch(const int32_t *nodes, const int32_t *fin_e,
                             const int32_t *fin_best, int32_t nchar, int32_t k,
                             const int32_t *tcm, int32_t n, const int32_t *anc,
                             const int32_t *node, const int32_t *left, const int32_t *right,
                             int32_t *out_e, int32_t *out_best, void *stream);
/* SankCS.distance (sankCS.ml:371-377) per candidate as the integer sum of
 * per-character (min c - min a.s - min b.s); dist[i] is int64. */
int poyd_sank_distance_batch(const int32_t *nodes, int32_t nchar, int32_t k,
                             const int32_t *tcm, int32_t n,
                             const int32_t *a_idx, const int32_t *b_idx,
                             int64_t *dist, void *stream);

/* ---------------------------------------------------------------------
 * Downpass levels with the node data resident on the device.
 *
 * The downpass (AllDirChar.internal_downpass, allDirChar.ml:722-790) makes
 * every interior vertex's preliminary data the median of its two
 * children's (Node.median, node.ml:638: DOS.median, seqCS.ml:747-776, for
 * the sequence; NonaddCS8.median, node.ml:272; SankCS.median, node.ml:333)
 * in a post-order visit.  Vertices of one height are independent, so a
 * downpass -- or the re-diagnosis of the vertices a tree move changes --
 * is a list of levels, each one batch of median pairs whose inputs are
 * existing nodes or outputs of earlier levels.
 *
 * Node store (device memory, owned by the caller):
 *   pool: the sequences' bytes; node v's sequence is pool[node_off[v] ..
 *         + node_len[v]) (the leading gap included);
 *   fitch: rows [node][fitch_stride] of fitch_len NonaddCS8 characters
 *         (16-byte aligned; fitch_len 0: none);
 *   sank: rows [node][sank_nchar][sank_k] int32 (POYD_SANK_INF as above),
 *         sank_tcm [k][k] (sank_nchar 0: none).
 * ------------------------------------------------------------------- */
typedef struct poyd_node_store {
  uint8_t *pool;
  int64_t pool_size;
  uint8_t *fitch;
  int64_t fitch_stride;
  int32_t fitch_len;
  int32_t sank_nchar;
  int32_t *sank;
  const int32_t *sank_tcm;
  int32_t sank_k;
  int32_t pad;
} poyd_node_store;

#define POYD_ESPACE -6  /* the caller's pool is too small (poyd_median_levels) */

/* ---------------------------------------------------------------------
 * Autotuner (no counterpart in the reference).  The batched linear DP
 * (poyd_cost_2_batch, poyd_align_2_batch, poyd_align_2_host and every
 * caller of them) has launch variants with identical results: the packed
 * kernel when its 16-bit bound holds or the 32-bit kernel, a persistent
 * grid of 1 to the maximum resident blocks per SM, and for batches with a
 * warp per pair the whole-warp or the batched traceback walk.  A variant
 * is kept per shape class: (device, align 0/1, floor(log2 pairs),
 * floor(log2 widest band)).  Without an entry the defaults apply (packed
 * when it can, the maximum grid, the whole-warp walk when every pair has
 * its own warp).  The band is always the reference's.
 * ------------------------------------------------------------------- */
typedef struct poyd_tune_result {
  int32_t packed, blocks_per_sm, solo; /* the variant kept (-1: default) */
  int32_t lg_pairs, lg_width;          /* its class */
  int32_t n_variants;
  float ms[8];                         /* mean time of each variant tried */
  int32_t variant[8][3];               /* {packed, blocks_per_sm, solo} */
} poyd_tune_result;
/* Times every variant on this batch (one warm-up, then `reps` runs each;
 * the arguments of poyd_align_2_batch when align != 0, else of
 * poyd_cost_2_batch with `deltaw_policy`), checks that each gives the
 * default's costs (and lengths), and keeps the fastest for the batch's
 * class.  The outputs hold the batch's results on return.  Returns
 * POYD_ERANGE if a variant's results differ (a bug, reported). */
int poyd_autotune_batch(const poyd_cm *cm, int32_t align, int32_t n, const uint8_t *seq,
                        const int64_t *a_off, const int32_t *a_len, const int64_t *b_off,
                        const int32_t *b_len, int32_t deltaw_policy, int32_t *cost,
                        uint8_t *out, const int64_t *out_off, int32_t *out_len, int32_t flags,
                        int32_t reps, poyd_tune_result *res, void *stream);
/* Sets / reads (returns 1 when present, else 0) / clears the kept variants
 * (host tables only: no CUDA call). */
int poyd_autotune_set(int32_t device, int32_t align, int32_t lg_pairs, int32_t lg_width,
                      int32_t packed, int32_t blocks_per_sm, int32_t solo);
int poyd_autotune_get(int32_t device, int32_t align, int32_t lg_pairs, int32_t lg_width,
                      int32_t *packed, int32_t *blocks_per_sm, int32_t *solo);
int poyd_autotune_clear(void);

/* Levels l = 0 .. n_levels-1 of median pairs, pairs
 * [level_start[l], level_start[l+1]): node out[i] becomes the median of
 * nodes a[i] and b[i] (DOS.median with Sequence.is_empty's all-gap rule,
 * as poyd_align_2_batch with POYD_FLAG_DOS_EMPTY, plus the Fitch and
 * Sankoff medians of its rows).  Every out[i] is distinct and none is an
 * input of its own or an earlier level.  The medians are written into the
 * pool from *pool_top upwards (the four-sequence result slots of
 * poyd_align_2_batch; node out[i] points at the fourth, the median).
 *
 * node_off / node_len are HOST arrays over all n_nodes node ids, in and
 * out: the call reads the inputs' places and writes the outputs'.
 * level_start, a, b, out are host arrays too; everything else stays on the
 * device, and the call waits for the stream once per level (the align_2
 * plan) and once at the end.  costs (host, may be NULL) receives per pair
 * the DO cost and the Fitch median cost (int64 pairs).  Before any launch
 * the call bounds the bytes it can need (a median is at most as long as
 * its two inputs together); when *pool_top + that bound exceeds pool_size
 * it writes the bound to *need (may be NULL) and returns POYD_ESPACE,
 * leaving everything unchanged, so that the caller can compact or grow its
 * pool and call again.  *pool_top returns the first unused byte. */
int poyd_median_levels(const poyd_cm *cm, const poyd_node_store *store, int32_t n_nodes,
                       int64_t *node_off, int32_t *node_len, int32_t n_levels,
                       const int32_t *level_start, const int32_t *a, const int32_t *b,
                       const int32_t *out, int64_t *pool_top, int64_t *need, int64_t *costs,
                       void *stream);

/* ---------------------------------------------------------------------
 * Learned join proposal (no counterpart in the reference): building blocks
 * of the 32-256-256-128-1 ReLU MLP with BF16 weights/activations and FP32
 * accumulation on tensor cores.  Matrices are row-major bf16 (uint16
 * storage); op(A)[m,k] = tA ? A[k*lda+m] : A[m*lda+k], likewise B.
 * ------------------------------------------------------------------- */
/* C[M,N] = op(A) op(B) (+ bias[n]) (ReLU) -> C32 (fp32, optional, added to
 * when accumulate) and/or C16 (bf16), row stride ldc. */
int poyd_gemm_bf16(const void *A, int32_t lda, int32_t tA, const void *B, int32_t ldb,
                   int32_t tB, int32_t M, int32_t N, int32_t K, const float *bias,
                   int32_t relu, float *C32, void *C16, int32_t ldc, int32_t accumulate,
                   void *stream);
/* dZ = dH * (H > 0) over n bf16 elements */
int poyd_relu_grad_bf16(const void *dH, const void *H, void *dZ, int64_t n, void *stream);
/* out[n] = sum_m X[m, n] */
int poyd_colsum_bf16(const void *X, int32_t M, int32_t N, float *out, void *stream);
/* y[m] = H[m,:] . w + b[0] (the 128 -> 1 output layer) */
int poyd_mlp_head_forward(const void *H, const void *w, const float *b, int32_t M, int32_t K,
                          float *y, void *stream);
/* mean-squared-error head: dZ = (2(y-t)/M) w masked by H > 0, dw = H^T dy,
 * db = sum dy, loss = mean (y-t)^2 */
int poyd_mlp_head_backward(const void *H, const void *w, const float *y, const float *target,
                           int32_t M, int32_t K, void *dZ, float *dw, float *db, float *loss,
                           void *stream);
/* Adam on fp32 master weights (step >= 1), refreshing the bf16 copy w16 */
int poyd_adam_step(float *w, void *w16, const float *g, float *m, float *v, int64_t n, float lr,
                   float b1, float b2, float eps, int32_t step, void *stream);
int poyd_to_bf16(const float *x, void *y, int64_t n, void *stream);
/* The whole 32-256-256-128-1 forward for inference in one launch: y[m] for
 * the M rows of X ([M][32] bf16, 16-byte aligned) with the weights
 * transposed (W1t [256][32], W2t [256][256], W3t [128][256] bf16), biases
 * fp32, the output layer w4 [128] bf16 and b4 [1]; the same values as the
 * layer-by-layer poyd_gemm_bf16 + poyd_mlp_head_forward path, bit for bit. */
int poyd_mlp_forward(const void *X, int32_t M, const void *W1t, const float *b1,
                     const void *W2t, const float *b2, const void *W3t, const float *b3,
                     const void *w4, const float *b4, float *y, void *stream);

/* ---------------------------------------------------------------------
 * Measurement helpers (no counterpart in the reference, which has no
 * device).  While profiling is on, every kernel the library launches is
 * bracketed by CUDA events on its own stream; poyd_profile_read sums the
 * recorded durations of kernels named `name` (NULL = all) in ms and
 * returns how many launches matched.  poyd_launch_count counts every
 * kernel launch since load.  poyd_int_pipe_rate measures integer issue
 * (Gop/s) with independent chains: mode 0 fused add-min (2 ops per
 * instruction, ALU pipe), mode 1 adds issued as multiply-adds (1 op, FMA
 * pipe), mode 2 the two interleaved (both pipes).  poyd_int32_peak is
 * mode 2, the denominator of the DP roofline: the DP issues its mins and
 * logic on the ALU pipe and its adds on the FMA pipe.
 * ------------------------------------------------------------------- */
int poyd_profile_enable(int on);
int poyd_profile_read(const char *name, double *ms_total, int clear);
long long poyd_launch_count(void);
int poyd_int_pipe_rate(int mode, double *gops, double *ms);
int poyd_int32_peak(double *gops, double *ms);

#ifdef __cplusplus
}
#endif
#endif
