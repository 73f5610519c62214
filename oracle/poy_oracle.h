/*
 * CPU oracle for the POY direct-optimization scoring path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * algorithms, used by tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference arm of bench.py to check and time the CUDA path.  Nothing in the
 * poyd_gb300 package links, imports or calls it.
 *
 * Parity pin: the restatement is checked against the reference's own C
 * kernels (algn.c, nonaddCSc.c, ukkCommon.c / ukk.checkp.c) compiled from
 * source by oracle/build_ref.sh
 * into oracle/_ref/, and against golden vectors in tests/golden/ produced by
 * that compiled reference (tests/golden/make_golden.py).
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project's src/ directory).
 */
#ifndef POY_ORACLE_H
#define POY_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Direction-set bits of the linear DP (matrices.h:22-27). */
#define OR_ALIGN 1
#define OR_INSERT 2
#define OR_DELETE 4

/* Affine direction bits (algn.c:1695-1708). */
#define OR_ALIGN_TO_ALIGN 1
#define OR_ALIGN_TO_VERTICAL 2
#define OR_ALIGN_TO_HORIZONTAL 4
#define OR_ALIGN_TO_DIAGONAL 8
#define OR_BEGIN_BLOCK 16
#define OR_END_BLOCK 32
#define OR_BEGIN_VERTICAL 64
#define OR_END_VERTICAL 128
#define OR_BEGIN_HORIZONTAL 256
#define OR_END_HORIZONTAL 512
#define OR_DO_ALIGN 1024
#define OR_DO_VERTICAL 2048
#define OR_DO_HORIZONTAL 4096
#define OR_DO_DIAGONAL 8192
#define OR_HIGH_NUM 1000000 /* algn.c:38 */

/* Two-dimensional transformation cost matrix with the bitmask alphabet
 * (struct cm, cm.h:29-43), restricted to lcm <= 5 (DNA with ambiguity
 * codes: 31 combinations of A, C, G, T and gap).  Tables are indexed
 * (a << 5) + b. */
typedef struct or_cm {
    int32_t lcm;
    int32_t gap;
    int32_t a_sz;
    int32_t combinations;
    int32_t cost_model; /* 0 linear, 1 affine */
    int32_t gap_open;
    int32_t is_metric;
    int32_t all_elements;
    int32_t cost[1024];
    int32_t worst[1024];
    int32_t prepend[32];
    int32_t tail[32];
    uint8_t median[1024];
} or_cm;

/* ---- cost_matrix.ml restatement ---- */
/* of_transformations_and_gaps true 5 sub indel 31 (cost_matrix.ml:645-656),
 * followed, when gap_open >= 0, by set_affine (cost_matrix.ml:405-416);
 * gap_open < 0 keeps the linear model. */
void or_cm_dna(or_cm *m, int sub, int indel, int gap_open);
/* of_list with an arbitrary 5x5 matrix over A,C,G,T,gap (cost_matrix.ml:559-563). */
void or_cm_of_matrix5(or_cm *m, const int32_t *mat25, int gap_open);

/* ---- Sequence.Align.cost_2 band policy (sequence.ml:687-723) ---- */
int or_count_gaps(const uint8_t *s, int len, int gap);
/* deltaw passed to algn_CAML_simple_2 for cost_2 s1 s2 (ls1 >= ls2 oriented);
 * has_deltaw/deltaw model the optional ?deltaw argument. */
int or_cost2_deltaw(const uint8_t *s1, int l1, const uint8_t *s2, int l2,
                    int gap, int has_deltaw, int deltaw);
/* DOS.distance's explicit deltaw: max(|la-lb|, 8) (seqCS.ml:856-866). */
int or_dos_distance_deltaw(int la, int lb);

/* ---- linear banded DP (algn.c:584-968, 3246-3283) ---- */
/* Cost of s1 (rows, len l1 >= l2) against s2 with width extension deltawh;
 * when dm != NULL the direction set of every band cell is written into dm,
 * row-major with stride l2 (the reference's DM layout). */
int or_simple_2(const uint8_t *s1, int l1, const uint8_t *s2, int l2,
                const or_cm *m, int deltawh, uint16_t *dm);
/* Number of DP cells the reference's band evaluates (row 0 included). */
int64_t or_band_cells_linear(int l1, int l2, int deltawh);
/* backtrack_2d, linear branch (algn.c:3551-3666).  Writes the aligned rows
 * sequence into r1 and columns sequence into r2 (both of capacity l1+l2);
 * returns the aligned length. */
int or_backtrack_2d(const uint8_t *s1, int l1, const uint8_t *s2, int l2,
                    const uint16_t *dm, const or_cm *m, int swaped,
                    uint8_t *r1, uint8_t *r2);
/* Sequence.Align.align_2 with first_gap = true (sequence.ml:849-869) for the
 * linear model: cost_2 (default deltaw) + create_edited_2.  a and b in caller
 * order; outputs aligned a' and b' (capacity la+lb), returns cost and writes
 * aligned length. */
int or_align_2(const uint8_t *a, int la, const uint8_t *b, int lb,
               const or_cm *m, uint8_t *ra, uint8_t *rb, int *alen);
/* cost_2 (sequence.ml:716-723): linear with deltaw policy, affine -> nobt. */
int or_cost_2(const uint8_t *a, int la, const uint8_t *b, int lb,
              const or_cm *m, int has_deltaw, int deltaw);

/* ---- medians of aligned pairs (algn.c:4011-4147) ---- */
int or_median_2_with_gaps(const uint8_t *a, const uint8_t *b, int len,
                          const or_cm *m, uint8_t *out);
int or_median_2_no_gaps(const uint8_t *a, const uint8_t *b, int len,
                        const or_cm *m, uint8_t *out);
int or_ancestor_2(const uint8_t *a, const uint8_t *b, int len,
                  const or_cm *m, uint8_t *out);
int or_worst_2(const uint8_t *a, const uint8_t *b, int len, const or_cm *m);
int or_verify_2(const uint8_t *a, const uint8_t *b, int len, const or_cm *m);
void or_union(const uint8_t *a, const uint8_t *b, int len, uint8_t *out);

/* ---- affine (algn.c:1695-2680) ---- */
int or_cost_affine_3(const uint8_t *si, int li, const uint8_t *sj, int lj,
                     const or_cm *m);
/* algn_CAML_align_affine_3: outputs median, medianwg, resi, resj (capacity
 * li+lj+2 each) and their lengths; returns the cost. */
int or_align_affine_3(const uint8_t *si, int li, const uint8_t *sj, int lj,
                      const or_cm *m, uint8_t *median, int *lmed,
                      uint8_t *medianwg, int *lmedwg, uint8_t *resi,
                      uint8_t *resj, int *lres);
int64_t or_band_cells_affine(int li, int lj);

/* ---- DOS.median composition (seqCS.ml:747-776) ---- */
/* Returns cost; writes median (seqm), aligned children and medianwg. */
int or_dos_median(const uint8_t *a, int la, const uint8_t *b, int lb,
                  const or_cm *m, uint8_t *seqm, int *lm, uint8_t *ra,
                  uint8_t *rb, uint8_t *medwg, int *lal);

/* ---- DOS.to_single (seqCS.ml:730-745) / Sequence.Align.closest
 * (sequence.ml:967-1033) ---- */
/* Single sequence of `mine` given its parent's; writes `out` (capacity
 * lp + lm + 2), returns its length or -1 (a column without states). */
int or_closest(const uint8_t *parent, int lp, const uint8_t *mine, int lm,
               const or_cm *m, int dos_empty, uint8_t *out);

/* DOS.median on pairs idx[0..n) of a packed batch (CPU timing driver);
 * returns the total band cells, writes each pair's cost. */
int64_t or_dos_median_many(const uint8_t *seq, const int64_t *a_off, const int32_t *a_len,
                           const int64_t *b_off, const int32_t *b_len, const int32_t *idx,
                           int n, const or_cm *m, int32_t *cost);

/* Results of a batched align_2 computed elsewhere (host copies): per pair
 * cost, lengths (aligned, median) and a slot of four right-aligned
 * sequences at out + off[i]. */
typedef struct {
    const int32_t *cost;
    const uint8_t *out;
    const int64_t *off;
    const int32_t *len;
} or_result_set;

/* or_dos_median_many plus a comparison of every output with nset result
 * sets; bad[t] has bit k set where set k differs on pair idx[t]. */
int64_t or_dos_median_check_many(const uint8_t *seq, const int64_t *a_off, const int32_t *a_len,
                                 const int64_t *b_off, const int32_t *b_len, const int32_t *idx,
                                 int n, const or_cm *m, int32_t *cost, int nset,
                                 const or_result_set *sets, int32_t *bad);

/* Candidate-join scores DOS.distance + Fitch + Sankoff (CPU timing driver). */
void or_candidate_scores(const uint8_t *seq, const int64_t *off, const int32_t *len,
                         const uint8_t *fitch, int nf, const int64_t *sank, int ns, int k,
                         const int64_t *tcm, const int32_t *a, const int32_t *b, int n,
                         const or_cm *m, int64_t *out);

/* ---- Fitch non-additive characters, 8-bit lanes (nonaddCSc.c) ---- */
int64_t or_nonadd_median(const uint8_t *a, const uint8_t *b, int len, uint8_t *res);
int64_t or_nonadd_distance(const uint8_t *a, const uint8_t *b, int len);
void or_nonadd_median_3(const uint8_t *A, const uint8_t *N, const uint8_t *D1,
                        const uint8_t *D2, int len, uint8_t *F);
int64_t or_nonadd_dist_2(const uint8_t *a, const uint8_t *b, const uint8_t *c, int len);
int64_t or_nonadd16_median(const uint16_t *a, const uint16_t *b, int len, uint16_t *res);
int64_t or_nonadd16_distance(const uint16_t *a, const uint16_t *b, int len);
void or_nonadd16_median_3(const uint16_t *A, const uint16_t *N, const uint16_t *D1,
                          const uint16_t *D2, int len, uint16_t *F);
int64_t or_nonadd32_median(const uint32_t *a, const uint32_t *b, int len, uint32_t *res);
int64_t or_nonadd32_distance(const uint32_t *a, const uint32_t *b, int len);
void or_nonadd32_median_3(const uint32_t *A, const uint32_t *N, const uint32_t *D1,
                          const uint32_t *D2, int len, uint32_t *F);

/* ---- Sankoff characters (sankCS.ml) ---- */
#define OR_SANK_INF ((int64_t)(((uint64_t)1 << 62) - 1) / 4) /* max_int/4, 63-bit */
/* elt_median over k states: a_s, b_s -> c (s), e, beta; tcm is k x k. */
void or_sank_elt_median(int k, const int64_t *tcm, const int64_t *a_s,
                        const int64_t *b_s, int64_t *c, int64_t *e, int64_t *beta);
/* elt_median_3 (sankCS.ml:402-452): final e and best-state bits of a node
 * from its ancestor's final (a_e, a_best; a_best 0: the ancestor's cheapest
 * states of a_s), its preliminary s and its children's preliminary s. */
void or_sank_elt_median_3(int k, const int64_t *tcm, const int64_t *a_s, const int64_t *a_e,
                          uint32_t a_best, const int64_t *n_s, const int64_t *l_s,
                          const int64_t *r_s, int64_t *e_out, uint32_t *best_out);
/* elt_distance as a float (sankCS.ml:347-354). */
double or_sank_elt_distance(int k, const int64_t *tcm, const int64_t *a_s,
                            const int64_t *b_s);


/* ---- Three-sequence alignment of the Iterative (ThreeD) mode ---- */
#define OR_P3_STATES 16
/* powell_3D_align (ukkCommon.c:111-143): optimal cost of aligning three
 * sequences (each with its leading gap) under Powell's state model with
 * mismatch mm, gap opening go and extension ge.  Writes the aligned rows
 * (characters reduced to one base, 16 for gaps, leading gap first) to
 * oa/ob/oc (capacity la + lb + lc) and their length to *olen.  Returns -1
 * for an element with none of A, C, G, T. */
int or_powell_3d(const uint8_t *a, int la, const uint8_t *b, int lb, const uint8_t *c, int lc,
                 int mm, int go, int ge, uint8_t *oa, uint8_t *ob, uint8_t *oc, int *olen);
/* The least alignmentCost (ukkCommon.c:345-391) of a given alignment. */
int or_powell_alignment_cost(const uint8_t *oa, const uint8_t *ob, const uint8_t *oc, int n,
                             int mm, int go, int ge);
/* Cost_matrix.Three_D median table from a 2-D matrix (cost_matrix.ml:803-851),
 * 32768 bytes indexed (i << 10) | (j << 5) | k. */
void or_median3_table(const or_cm *m, uint8_t *tab);
/* Sequence.Align.readjust_3d (sequence.ml:1117-1140): new median of a node
 * from its children s1, s2, its current median cm_ and its parent p. */
int or_readjust_3d(const uint8_t *s1, int l1, const uint8_t *s2, int l2, const uint8_t *cm_,
                   int lm, const uint8_t *p, int lp, const or_cm *m, const uint8_t *tab3,
                   uint8_t *res, int *lres, int *changed);

#ifdef __cplusplus
}
#endif
#endif
