/*
 * CPU oracle for the POY direct-optimization scoring path (restatement).
 *
 * TEST INFRASTRUCTURE ONLY: results the CUDA path is checked against, never
 * shipped.
 * See poy_oracle.h for the parity pin.  File:line citations are relative to
 * the reference project's src/ directory.
 */
#include "poy_oracle.h"
#include <stdlib.h>
#include <string.h>

#define TBL(a, b) (((a) << 5) + (b))

/* ------------------------------------------------------------------------ */
/* cost_matrix.ml                                                           */
/* ------------------------------------------------------------------------ */

/* cost_matrix.ml:39: max_int is overridden to Int32.max_int lsr 1. */
#define OR_CM_MAX_INT 1073741823

static int popc5(int x) { return __builtin_popcount((unsigned)x & 31u); }

/* fill_best_cost_and_median_for_all_combinations (cost_matrix.ml:323-354):
 * cost of an ambiguity pair = min over members a in i, b in j and a single
 * intermediate state v of cost(a,v)+cost(v,b); median = OR of all tied v. */
static void fill_metric(or_cm *m) {
    int i, j, a, b, k;
    for (i = 1; i <= 31; i++) {
        for (j = 1; j <= 31; j++) {
            int best = 0, c = OR_CM_MAX_INT, w = 0;
            for (a = 1; a <= 16; a <<= 1) {
                if (!(i & a)) continue;
                for (b = 1; b <= 16; b <<= 1) {
                    if (!(j & b)) continue;
                    for (k = 0; k < 5; k++) {
                        int v = 1 << k;
                        int goa = (m->cost_model == 1 && v == m->gap &&
                                   (a & m->gap) && (b & m->gap)) ? m->gap_open : 0;
                        int tc = m->cost[TBL(a, v)] + m->cost[TBL(v, b)] + goa;
                        if (tc < c) { c = tc; best = v; }
                        else if (tc == c) best |= v;
                    }
                    if (m->cost[TBL(a, b)] > w) w = m->cost[TBL(a, b)];
                }
            }
            if (popc5(i) == 1 && popc5(j) == 1) {
                m->median[TBL(i, j)] = (uint8_t)(i | j);
            } else {
                m->cost[TBL(i, j)] = c;
                /* cleanup (cost_matrix.ml:246-255) is the identity unless the
                 * matrix is already affine when this fill runs. */
                if (m->cost_model == 1 && best != m->gap && (best & m->gap))
                    best = m->gap;
                m->median[TBL(i, j)] = (uint8_t)best;
            }
            m->worst[TBL(i, j)] = w;
        }
    }
}

/* fill_best_cost_and_median_for_all_combinations_bitwise
 * (cost_matrix.ml:270-321): overlapping sets cost 0 with median = shared
 * bits; disjoint sets take the cheapest member pair in either order, median =
 * OR of the tied pairs; worst = max over both orders. */
static void fill_bitwise(or_cm *m) {
    int i, j, a, b;
    for (i = 1; i <= 31; i++) {
        for (j = 1; j <= 31; j++) {
            if (popc5(i) == 1 && popc5(j) == 1) {
                m->median[TBL(i, j)] = (uint8_t)(i | j);
                m->worst[TBL(i, j)] = m->cost[TBL(i, j)];
                continue;
            }
            int best = OR_CM_MAX_INT, med = 0, worst = 0, pass;
            for (pass = 0; pass < 2; pass++) {
                int x = pass == 0 ? j : i, y = pass == 0 ? i : j;
                for (a = 1; a <= 16; a <<= 1) {
                    if (!(x & a)) continue;
                    for (b = 1; b <= 16; b <<= 1) {
                        if (!(y & b)) continue;
                        int c = m->cost[TBL(a, b)];
                        if (c < best) { best = c; med = a | b; }
                        else if (c == best) med |= a | b;
                        if (c > worst) worst = c;
                    }
                }
            }
            if (i & j) {
                m->median[TBL(i, j)] = (uint8_t)(i & j);
                m->cost[TBL(i, j)] = 0;
                m->worst[TBL(i, j)] = worst;
            } else {
                m->median[TBL(i, j)] = (uint8_t)med;
                m->cost[TBL(i, j)] = best;
                m->worst[TBL(i, j)] = worst;
            }
        }
    }
}

/* fill_default_prepend_tail (cost_matrix.ml:397-403). */
static void fill_prepend_tail(or_cm *m) {
    int i;
    m->tail[0] = 0;
    m->prepend[0] = 0;
    for (i = 1; i <= 31; i++) {
        m->tail[i] = m->cost[TBL(i, m->gap)];
        m->prepend[i] = m->cost[TBL(m->gap, i)];
    }
}

/* input_is_metric (cost_matrix.ml:512-517) on the 5x5 input. */
static int input_is_metric(const int32_t *l) {
    int i, j, k;
    for (i = 0; i < 25; i++) if (l[i] < 0) return 0;
    for (i = 0; i < 5; i++) for (j = 0; j < 5; j++) if (l[i * 5 + j] != l[j * 5 + i]) return 0;
    for (i = 0; i < 5; i++) for (j = 0; j < 5; j++) for (k = 0; k < 5; k++)
        if (l[i * 5 + j] > l[i * 5 + k] + l[k * 5 + j]) return 0;
    for (i = 0; i < 5; i++) if (l[i * 5 + i] != 0) return 0;
    return 1;
}

void or_cm_of_matrix5(or_cm *m, const int32_t *mat25, int gap_open) {
    int i, j;
    memset(m, 0, sizeof(*m));
    /* cm_set_val with combinations (cm.c:318-361) */
    m->gap = 16; m->a_sz = 31; m->lcm = 5; m->combinations = 1;
    m->all_elements = 31; m->cost_model = 0; m->gap_open = 0;
    /* store_input_list_in_cost_matrix_all_combinations (cost_matrix.ml:157-177) */
    for (i = 0; i < 5; i++) for (j = 0; j < 5; j++)
        m->cost[TBL(1 << i, 1 << j)] = mat25[i * 5 + j];
    /* fill_cost_matrix (cost_matrix.ml:520-538) */
    if (input_is_metric(mat25)) { m->is_metric = 1; fill_metric(m); }
    else fill_bitwise(m);
    fill_prepend_tail(m);
    if (gap_open >= 0) {
        /* set_affine (cost_matrix.ml:405-416) with Affine gap_open; a
         * negative gap_open keeps the linear model. */
        m->cost_model = 1; m->gap_open = gap_open;
        fill_bitwise(m);
        fill_prepend_tail(m);
    }
}

void or_cm_dna(or_cm *m, int sub, int indel, int gap_open) {
    /* of_transformations_and_gaps (cost_matrix.ml:645-656) */
    int32_t l[25];
    int x, y;
    for (x = 0; x < 5; x++) for (y = 0; y < 5; y++)
        l[x * 5 + y] = (x == y) ? 0 : ((y == 4 || x == 4) ? indel : sub);
    or_cm_of_matrix5(m, l, gap_open);
}

/* ------------------------------------------------------------------------ */
/* sequence.ml cost_2 band policy                                            */
/* ------------------------------------------------------------------------ */

int or_count_gaps(const uint8_t *s, int len, int gap) {
    /* seq_CAML_count (seq.c:571-581): positions sharing a bit with gap */
    int i, c = 0;
    for (i = 0; i < len; i++) if (s[i] & gap) c++;
    return c;
}

int or_cost2_deltaw(const uint8_t *s1, int l1, const uint8_t *s2, int l2,
                    int gap, int has_deltaw, int deltaw) {
    /* sequence.ml:691-713 */
    int g1 = or_count_gaps(s1, l1, gap), g2 = or_count_gaps(s2, l2, gap);
    int gaps = g1 > g2 ? g1 : g2;
    int big = l1 >= l2 ? l1 : l2, small = l1 >= l2 ? l2 : l1;
    int dif = big - small;
    int lower = (int)((double)big * 0.10);
    int dw;
    if (!has_deltaw) dw = (dif < lower) ? lower / 2 : 2;
    else dw = (dif < lower) ? lower : deltaw;
    return gaps + dw;
}

int or_dos_distance_deltaw(int la, int lb) {
    int d = la > lb ? la - lb : lb - la;
    return d > 8 ? d : 8;
}

/* ------------------------------------------------------------------------ */
/* Linear banded DP                                                          */
/* ------------------------------------------------------------------------ */

/* Band geometry of algn_fill_plane_2 (algn.c:872-968), restated as per-row
 * column intervals.  Every row r >= 1 covers columns [lo, hi]:
 *   full plane (case 1, or case 3 with <= 8 leftover rows): lo = 0, hi = L2-1;
 *   otherwise lo = max(0, r - height + delta), hi = min(r + width - 1, L2-1)
 *   with delta = 1 in case 2 (2*height < L1) and 0 in case 3.
 * The left cell is "first" (delete only) when lo = 0, else it has no insert
 * (algn_fill_ukk_left_cell, algn.c:507-541).  The right cell has no delete
 * while r + width - 1 <= L2 - 1 (algn_fill_ukk_right_cell, algn.c:461-500),
 * otherwise it is a normal cell re-checked against the tail cost
 * (algn_fill_last_column, algn.c:548-560).  Row 0 covers [0, width-1]. */
typedef struct { int full, width, height, delta; } or_band;

static or_band band_plan(int l1, int l2, int deltawh) {
    or_band b;
    int width = 50 + deltawh, height = (l1 - l2) + 50 + deltawh;
    if (width > l2) width = l2;
    if (height > l1) height = l1;
    b.width = width; b.height = height; b.delta = 0; b.full = 0;
    if (((float)l1) >= (((float)((float)3 / (float)2) * (float)l2))) b.full = 1;
    else if ((2 * height) < l1) b.delta = 1;
    else if (8 >= (l1 - height)) b.full = 1;
    if (b.full) { b.width = l2; b.height = l1 + 1; b.delta = 0; }
    return b;
}

static void band_row(const or_band *b, int r, int l2, int *lo, int *hi, int *right_open) {
    int x = r - b->height + b->delta;
    int y = r + b->width - 1;
    *lo = x > 0 ? x : 0;
    *hi = y < l2 - 1 ? y : l2 - 1;
    *right_open = (y <= l2 - 1); /* right cell without delete */
}

int64_t or_band_cells_linear(int l1, int l2, int deltawh) {
    or_band b = band_plan(l1, l2, deltawh);
    int64_t n = b.width;
    int r, lo, hi, ro;
    for (r = 1; r < l1; r++) { band_row(&b, r, l2, &lo, &hi, &ro); n += hi - lo + 1; }
    return n;
}

int or_simple_2(const uint8_t *s1, int l1, const uint8_t *s2, int l2,
                const or_cm *m, int deltawh, uint16_t *dm) {
    or_band b = band_plan(l1, l2, deltawh);
    int *pm = (int *)malloc(sizeof(int) * (size_t)(l2 + 1));
    int *mm = (int *)malloc(sizeof(int) * (size_t)(l2 + 1));
    const int gap = m->gap;
    int r, j, lo, hi, ro, res;
    /* first row (algn_fill_first_row, algn.c:584-607): prepend costs */
    pm[0] = 0;
    if (dm) dm[0] = OR_ALIGN;
    for (j = 1; j < b.width; j++) {
        pm[j] = pm[j - 1] + m->prepend[s2[j]];
        if (dm) dm[j] = OR_INSERT;
    }
    for (r = 1; r < l1; r++) {
        const int a = s1[r];
        const int cdel = m->cost[TBL(a, gap)];
        const int ctail = m->tail[a];
        uint16_t *drow = dm ? dm + (size_t)r * (size_t)l2 : NULL;
        band_row(&b, r, l2, &lo, &hi, &ro);
        for (j = lo; j <= hi; j++) {
            int h, d;
            if (j == 0) {
                /* algn_fill_first_cell / algn_fill_full_row */
                h = pm[0] + (b.full ? cdel : ctail);
                d = OR_DELETE;
            } else if (j == lo) {
                int D = pm[j] + cdel, A = pm[j - 1] + m->cost[TBL(a, s2[j])];
                h = D < A ? D : A;
                d = (D == h ? OR_DELETE : 0) | (A == h ? OR_ALIGN : 0);
            } else if (j == hi && ro) {
                int I = mm[j - 1] + m->cost[TBL(gap, s2[j])];
                int A = pm[j - 1] + m->cost[TBL(a, s2[j])];
                h = I < A ? I : A;
                d = (I == h ? OR_INSERT : 0) | (A == h ? OR_ALIGN : 0);
            } else {
                int D = pm[j] + cdel;
                int I = mm[j - 1] + m->cost[TBL(gap, s2[j])];
                int A = pm[j - 1] + m->cost[TBL(a, s2[j])];
                h = D < I ? D : I;
                if (A < h) h = A;
                d = (A == h ? OR_ALIGN : 0) | (I == h ? OR_INSERT : 0) | (D == h ? OR_DELETE : 0);
            }
            if (j == hi && !ro && j > 0) {
                int cst = ctail + pm[j];
                if (cst < h) { h = cst; d = OR_DELETE; }
                else if (cst == h) d |= OR_DELETE;
            }
            mm[j] = h;
            if (drow) drow[j] = (uint16_t)d;
        }
        { int *t = pm; pm = mm; mm = t; }
    }
    res = pm[l2 - 1];
    free(pm); free(mm);
    return res;
}

int or_backtrack_2d(const uint8_t *s1, int l1, const uint8_t *s2, int l2,
                    const uint16_t *dm, const or_cm *m, int swaped,
                    uint8_t *r1, uint8_t *r2) {
    /* Walk from the last cell; the reference loops while the DM pointer is
     * at or after its start, i.e. r*L2 + j >= 0, which ends right after the
     * align move out of cell (0,0).  Output is prepended. */
    int cap = l1 + l2, n = 0;
    int r = l1 - 1, j = l2 - 1;
    uint8_t *t1 = (uint8_t *)malloc((size_t)cap + 1), *t2 = (uint8_t *)malloc((size_t)cap + 1);
    while ((long)r * l2 + j >= 0) {
        int d = dm[(size_t)r * l2 + j];
        int mv;
        if (d & OR_ALIGN) mv = 0;
        else if (swaped) mv = (d & OR_INSERT) ? 1 : 2;
        else mv = (d & OR_DELETE) ? 2 : 1;
        if (mv == 0) { t1[n] = s1[r]; t2[n] = s2[j]; r--; j--; }
        else if (mv == 1) { t1[n] = (uint8_t)m->gap; t2[n] = s2[j]; j--; }
        else { t1[n] = s1[r]; t2[n] = (uint8_t)m->gap; r--; }
        n++;
        if (n > cap) break;
    }
    for (r = 0; r < n; r++) { r1[r] = t1[n - 1 - r]; r2[r] = t2[n - 1 - r]; }
    free(t1); free(t2);
    return n;
}

int or_cost_2(const uint8_t *a, int la, const uint8_t *b, int lb,
              const or_cm *m, int has_deltaw, int deltaw) {
    if (m->cost_model == 1) return or_cost_affine_3(a, la, b, lb, m);
    int dw = or_cost2_deltaw(a, la, b, lb, m->gap, has_deltaw, deltaw);
    if (la >= lb) return or_simple_2(a, la, b, lb, m, dw, NULL);
    return or_simple_2(b, lb, a, la, m, dw, NULL);
}

int or_align_2(const uint8_t *a, int la, const uint8_t *b, int lb,
               const or_cm *m, uint8_t *ra, uint8_t *rb, int *alen) {
    /* sequence.ml:849-869 (first_gap = true), linear model:
     * cost_2 then create_edited_2 (sequence.ml:813-823). */
    /* One grow-only direction matrix per thread, reused across calls like
     * the reference's Matrix.default arena (matrices.c:77-120); it is not
     * cleared between calls. */
    static __thread uint16_t *dm_arena = NULL;
    static __thread size_t dm_cap = 0;
    size_t need = (size_t)la * (size_t)lb;
    int dw = or_cost2_deltaw(a, la, b, lb, m->gap, 0, 0);
    int cost;
    if (need > dm_cap) {
        free(dm_arena);
        dm_arena = (uint16_t *)malloc(sizeof(uint16_t) * need);
        dm_cap = need;
    }
    if (la >= lb) {
        cost = or_simple_2(a, la, b, lb, m, dw, dm_arena);
        *alen = or_backtrack_2d(a, la, b, lb, dm_arena, m, 1, ra, rb);
    } else {
        cost = or_simple_2(b, lb, a, la, m, dw, dm_arena);
        *alen = or_backtrack_2d(b, lb, a, la, dm_arena, m, 0, rb, ra);
    }
    return cost;
}

/* ------------------------------------------------------------------------ */
/* Medians of aligned pairs                                                  */
/* ------------------------------------------------------------------------ */

int or_median_2_with_gaps(const uint8_t *a, const uint8_t *b, int len,
                          const or_cm *m, uint8_t *out) {
    /* algn_get_median_2d_with_gaps (algn.c:4011-4024) */
    int i;
    for (i = 0; i < len; i++) out[i] = m->median[TBL(a[i], b[i])];
    return len;
}

int or_median_2_no_gaps(const uint8_t *a, const uint8_t *b, int len,
                        const or_cm *m, uint8_t *out) {
    /* algn_get_median_2d_no_gaps (algn.c:4031-4046): non-gap medians with
     * one leading gap */
    int i, n = 1;
    out[0] = (uint8_t)m->gap;
    for (i = 0; i < len; i++) {
        int v = m->median[TBL(a[i], b[i])];
        if (v != m->gap) out[n++] = (uint8_t)v;
    }
    return n;
}

/* algn_remove_gaps (algn.c:4048-4066) on a buffer in place. */
static int remove_gaps(int gap, uint8_t *s, int len) {
    int i, n = 0;
    uint8_t *tmp = (uint8_t *)malloc((size_t)len + 1);
    for (i = 0; i < len; i++) if (s[i] != gap) tmp[n++] = s[i];
    s[0] = (uint8_t)gap;
    memcpy(s + 1, tmp, (size_t)n);
    free(tmp);
    return n + 1;
}

/* algn_correct_blocks_affine (algn.c:4068-4110). */
static int correct_blocks_affine(int gap, uint8_t *s, int len, const uint8_t *a, const uint8_t *b) {
    int i, extending_gap = 0, inside_block = 0, prev_block = 0;
    for (i = 0; i < len; i++) {
        int ab = a[i], bb = b[i], sb = s[i];
        if (!inside_block && (!(ab & gap) || !(bb & gap))) inside_block = 0;
        else if (inside_block && ((!(ab & gap)) || (!(bb & gap)))) inside_block = 0;
        else if (((ab & gap) || (bb & gap)) && ((ab != gap) || (bb != gap))) inside_block = 1;
        else inside_block = 0;
        if (((gap & ab) || (gap & bb)) && (!(sb & gap)) && !extending_gap) {
            prev_block = inside_block;
            extending_gap = 1;
        } else if ((gap & ab) && (gap & bb) && (sb & gap) && (sb != gap) &&
                   extending_gap && inside_block && !prev_block) {
            sb = (~gap) & sb;
            prev_block = 0;
        } else if ((gap & ab) && (gap & bb) && (1 == extending_gap)) {
            prev_block = inside_block;
            extending_gap = 0;
        }
        s[i] = (uint8_t)sb;
    }
    return remove_gaps(gap, s, len);
}

int or_ancestor_2(const uint8_t *a, const uint8_t *b, int len,
                  const or_cm *m, uint8_t *out) {
    /* algn_ancestor_2 (algn.c:4117-4147) */
    int i, n = 0, gap = m->gap;
    int keep_gaps = m->combinations && m->cost_model == 1;
    uint8_t *tmp = (uint8_t *)malloc((size_t)len + 2);
    for (i = 0; i < len; i++) {
        int v = m->median[TBL(a[i], b[i])];
        if (keep_gaps || v != gap) tmp[n++] = (uint8_t)v;
    }
    if (!m->combinations || (m->cost_model != 1 && (n == 0 || tmp[0] != gap))) {
        /* an empty result has no position 0 in the reference (an
         * out-of-range read there); it is treated here as "not a gap". */
        out[0] = (uint8_t)gap;
        memcpy(out + 1, tmp, (size_t)n);
        n++;
    } else {
        memcpy(out, tmp, (size_t)n);
        n = correct_blocks_affine(gap, out, n, a, b);
    }
    free(tmp);
    return n;
}

/* algn_calculate_from_2_aligned (algn.c:3316-3370). */
static int calc_from_aligned(const uint8_t *s1, const uint8_t *s2, int len,
                             const or_cm *c, const int32_t *matrix) {
    int i, res = 0, gap_row = 0, gap = c->gap, go = c->gap_open;
    int s1b = s1[0], s2b = s2[0];
    if ((c->combinations && (gap & s1b) && (gap & s2b)) ||
        (!c->combinations && (gap == s1b) && (gap == s2b))) i = 1;
    else i = 0;
    for (; i < len; i++) {
        s1b = s1[i]; s2b = s2[i];
        if (0 == gap_row) {
            if ((c->combinations && (s1b & gap) && !(s2b & gap)) || (!c->combinations && s1b == gap)) {
                res += go; gap_row = 1;
            } else if ((c->combinations && (s2b & gap) && !(s1b & gap)) || (!c->combinations && s2b == gap)) {
                res += go; gap_row = 2;
            }
        } else if (1 == gap_row) {
            if ((c->combinations && !(s1b & gap)) || (!c->combinations && s1b != gap)) {
                if ((c->combinations && (s2b & gap) && !(s1b & gap)) || (!c->combinations && s2b == gap)) {
                    res += go; gap_row = 2;
                } else gap_row = 0;
            }
        } else {
            if ((c->combinations && !(s2b & gap)) || (!c->combinations && s2b != gap)) {
                if ((c->combinations && (s1b & gap)) || (!c->combinations && s1b == gap)) {
                    res += go; gap_row = 1;
                } else gap_row = 0;
            }
        }
        res += matrix[TBL(s1b, s2b)];
    }
    return res;
}

int or_worst_2(const uint8_t *a, const uint8_t *b, int len, const or_cm *m) {
    return calc_from_aligned(a, b, len, m, m->worst);
}
int or_verify_2(const uint8_t *a, const uint8_t *b, int len, const or_cm *m) {
    return calc_from_aligned(a, b, len, m, m->cost);
}
void or_union(const uint8_t *a, const uint8_t *b, int len, uint8_t *out) {
    int i;
    for (i = 0; i < len; i++) out[i] = a[i] | b[i];
}

/* ------------------------------------------------------------------------ */
/* Affine ("3 matrix") DP: algn.c:1695-2680                                  */
/* ------------------------------------------------------------------------ */

#define AFF_START_V 40
#define TMPGAP 16
#define NTMPGAP 15

static int has_gap_opening(int prev, int curr, int gap, int go) {
    /* HAS_GAP_OPENING (algn.c:1730-1733) */
    return ((!(gap & prev)) && (gap & curr)) ? 0 : go;
}

/* Band of the affine fill (algn.c:2309-2400): row i (1..leni) computes
 * columns [start(i), end(i)], start = max(1, i - 39), end = min(e0 + i - 1,
 * lenj) with e0 = clamp(max(lenj - leni + 8, 40), <= lenj).  Column start-1
 * holds a vertical boundary cell and, while end < lenj, column end+1 holds a
 * boundary cell of HIGH_NUM values. */
static int aff_e0(int leni, int lenj) {
    int e = (lenj - leni) + 8;
    if (e < 40) e = 40;
    if (e > lenj) e = lenj;
    return e;
}

int64_t or_band_cells_affine(int li, int lj) {
    int leni = li - 1, lenj = lj - 1;
    int64_t n;
    int i, e0;
    if (leni > lenj) { int t = leni; leni = lenj; lenj = t; }
    n = lenj + 1; /* row 0 of the rows = shorter orientation */
    e0 = aff_e0(leni, lenj);
    for (i = 1; i <= leni; i++) {
        int s = i > AFF_START_V ? i - AFF_START_V + 1 : 1;
        int e = e0 + i - 1; if (e > lenj) e = lenj;
        n += e - s + 1;
    }
    return n;
}

/* One affine plane fill.  si is the shorter sequence (rows), sj the longer.
 * bt selects algn_fill_plane_3_aff (with the FILL_EXTEND_BLOCK_DIAGONAL open
 * cost quirk, algn.c:1863-1880) over the _nobt variant (algn.c:1840-1860). */
static int aff_fill(const uint8_t *si, int leni, const uint8_t *sj, int lenj,
                    const or_cm *c, int bt, uint16_t *dm) {
    const int gap = c->gap, go = c->gap_open, W = lenj + 1;
    int *EH[2], *EV[2], *EB[2], *CB[2];
    int *gop = (int *)malloc(sizeof(int) * (size_t)W);
    int *hext = (int *)malloc(sizeof(int) * (size_t)W);
    int i, j, k, res, fc_last = 0;
    int e0 = aff_e0(leni, lenj), end_pos = e0, start_pos = 1;
    for (k = 0; k < 2; k++) {
        EH[k] = (int *)malloc(sizeof(int) * (size_t)(W + 1));
        EV[k] = (int *)malloc(sizeof(int) * (size_t)(W + 1));
        EB[k] = (int *)malloc(sizeof(int) * (size_t)(W + 1));
        CB[k] = (int *)malloc(sizeof(int) * (size_t)(W + 1));
    }
    /* initialize_matrices_affine[_nobt] (algn.c:2124-2248), row 0 */
    CB[0][0] = 0; EB[0][0] = 0; EH[0][0] = go; EV[0][0] = go;
    if (dm) dm[0] = 0xFFFF;
    for (j = 1; j <= lenj; j++) {
        int r = EH[0][j - 1] + c->prepend[sj[j]];
        EH[0][j] = r; CB[0][j] = r; EB[0][j] = OR_HIGH_NUM; EV[0][j] = OR_HIGH_NUM;
        if (dm) dm[j] = OR_DO_HORIZONTAL | OR_END_HORIZONTAL;
    }
    if (lenj == 0) fc_last = 0; else fc_last = EH[0][lenj];
    for (j = 1; j <= lenj; j++) {
        gop[j] = has_gap_opening(sj[j - 1], sj[j], gap, go);
        if ((sj[j - 1] & gap) && !(sj[j] & gap)) hext[j] = gop[j] + c->prepend[sj[j]];
        else hext[j] = c->prepend[sj[j]];
    }
    if (lenj >= 1) hext[1] = c->prepend[sj[1]];
    for (i = 1; i <= leni; i++) {
        int *peh = EH[(i - 1) & 1], *pev = EV[(i - 1) & 1], *peb = EB[(i - 1) & 1], *pcb = CB[(i - 1) & 1];
        int *eh = EH[i & 1], *ev = EV[i & 1], *eb = EB[i & 1], *cb = CB[i & 1];
        int ic = si[i], ip = si[i - 1];
        int si_ext = c->cost[TBL(ic, gap)];
        int si_open = has_gap_opening(ip, ic, gap, go);
        int si_ng = NTMPGAP & ic;
        int si_vext = (i > 1 && (ip & gap) && !(ic & gap)) ? si_open + si_ext : si_ext;
        uint16_t *drow = dm ? dm + (size_t)i * W : NULL;
        int jc, jp;
        if (i > AFF_START_V) start_pos++;
        {
            int s = start_pos - 1;
            int r = pev[s] + si_vext;
            eh[s] = OR_HIGH_NUM; cb[s] = OR_HIGH_NUM; eb[s] = OR_HIGH_NUM; ev[s] = r;
            if (s == lenj) fc_last = r;
            if (drow) drow[s] = OR_DO_VERTICAL | OR_END_VERTICAL;
        }
        jc = sj[start_pos - 1];
        for (j = start_pos; j <= end_pos; j++) {
            int sj_ng, sj_ext, sj_open, v, ext, open, flag, diag, odiag, algn, fv, fh, fd, extra;
            int d = 0;
            jp = jc; jc = sj[j];
            sj_ng = NTMPGAP & jc;
            sj_ext = c->prepend[jc];
            sj_open = gop[j];
            /* FILL_EXTEND_HORIZONTAL (algn.c:1762-1788) */
            ext = eh[j - 1] + hext[j];
            open = cb[j - 1] + sj_open + sj_ext;
            if (ext < open) { eh[j] = ext; d |= OR_BEGIN_HORIZONTAL; }
            else { eh[j] = open; d |= OR_END_HORIZONTAL; }
            /* FILL_EXTEND_VERTICAL (algn.c:1807-1828) */
            ext = pev[j] + si_vext;
            open = pcb[j] + si_open + si_ext;
            if (ext < open) { ev[j] = ext; d |= OR_BEGIN_VERTICAL; }
            else { ev[j] = open; d |= OR_END_VERTICAL; }
            /* FILL_EXTEND_BLOCK_DIAGONAL[_NOBT] (algn.c:1835-1882) */
            flag = (TMPGAP & ic) && (TMPGAP & jc);
            diag = flag ? 0 : OR_HIGH_NUM;
            if (bt) odiag = diag; /* the bt variant adds diag to the open cost */
            else odiag = flag ? (((!(TMPGAP & ip)) && (!(TMPGAP & jc))) ? 0 : 2 * go) : OR_HIGH_NUM;
            ext = peb[j - 1] + diag;
            open = pcb[j - 1] + odiag;
            if (ext < open) { eb[j] = ext; d |= OR_BEGIN_BLOCK; }
            else { eb[j] = open; d |= OR_END_BLOCK; }
            /* FILL_CLOSE_BLOCK_DIAGONAL (algn.c:1884-1977) */
            diag = c->cost[TBL(si_ng, sj_ng)];
            extra = (sj_open < si_open) ? si_open : sj_open;
            algn = pcb[j - 1] + diag;
            fv = pev[j - 1] + diag + (ic == si_ng ? 0 : sj_open);
            fh = peh[j - 1] + diag + (jc == sj_ng ? 0 : si_open);
            fd = peb[j - 1] + diag + extra;
            {
                int cur = algn, mask = OR_ALIGN_TO_ALIGN;
                if (cur >= fv) { if (cur > fv) { cur = fv; mask = OR_ALIGN_TO_VERTICAL; } else mask |= OR_ALIGN_TO_VERTICAL; }
                if (cur >= fh) { if (cur > fh) { cur = fh; mask = OR_ALIGN_TO_HORIZONTAL; } else mask |= OR_ALIGN_TO_HORIZONTAL; }
                if (cur >= fd) { if (cur > fd) { cur = fd; mask = OR_ALIGN_TO_DIAGONAL; } else mask |= OR_ALIGN_TO_DIAGONAL; }
                cb[j] = cur;
                d |= mask;
            }
            /* ASSIGN_MINIMUM (algn.c:2251-2280) */
            {
                int f = eh[j], mask = OR_DO_HORIZONTAL;
                if (f >= ev[j]) { if (f > ev[j]) { f = ev[j]; mask = OR_DO_VERTICAL; } else mask |= OR_DO_VERTICAL; }
                if (f >= eb[j]) { if (f > eb[j]) { f = eb[j]; mask = OR_DO_DIAGONAL; } else mask |= OR_DO_DIAGONAL; }
                if (f >= cb[j]) { if (f > cb[j]) { f = cb[j]; mask = OR_DO_ALIGN; } else mask |= OR_DO_ALIGN; }
                d |= mask;
                if (j == lenj) fc_last = f;
            }
            v = d;
            if (drow) drow[j] = (uint16_t)v;
        }
        if (end_pos < lenj) {
            end_pos++;
            ev[end_pos] = OR_HIGH_NUM; cb[end_pos] = OR_HIGH_NUM;
            eh[end_pos] = OR_HIGH_NUM; eb[end_pos] = OR_HIGH_NUM;
            if (drow) drow[end_pos] = OR_DO_HORIZONTAL | OR_END_HORIZONTAL;
        }
    }
    if (bt) res = fc_last;
    else {
        int t = leni & 1;
        res = EH[t][lenj];
        if (res > EV[t][lenj]) res = EV[t][lenj];
        if (res > EB[t][lenj]) res = EB[t][lenj];
        if (res > CB[t][lenj]) res = CB[t][lenj];
    }
    for (k = 0; k < 2; k++) { free(EH[k]); free(EV[k]); free(EB[k]); free(CB[k]); }
    free(gop); free(hext);
    return res;
}

int or_cost_affine_3(const uint8_t *si, int li, const uint8_t *sj, int lj, const or_cm *m) {
    /* algn_CAML_cost_affine_3 (algn.c:2628-2680): rows = shorter */
    if (li <= lj) return aff_fill(si, li - 1, sj, lj - 1, m, 0, NULL);
    return aff_fill(sj, lj - 1, si, li - 1, m, 0, NULL);
}

/* Prepend buffer: data grows towards the front. */
typedef struct { uint8_t *buf; int cap; int head; } pbuf;
static void pb_init(pbuf *p, int cap) { p->buf = (uint8_t *)malloc((size_t)cap + 1); p->cap = cap; p->head = cap; }
static void pb_pre(pbuf *p, int v) { if (p->head > 0) p->buf[--p->head] = (uint8_t)v; }
static int pb_len(const pbuf *p) { return p->cap - p->head; }
static void pb_out(pbuf *p, uint8_t *out) { memcpy(out, p->buf + p->head, (size_t)pb_len(p)); free(p->buf); }

/* backtrace_affine (algn.c:1983-2097). */
static void aff_backtrace(const uint16_t *dm, const uint8_t *si, int li, const uint8_t *sj, int lj,
                          const or_cm *c, pbuf *median, pbuf *medianwg, pbuf *resi, pbuf *resj) {
    enum { M_TODO, M_VERT, M_HORZ, M_DIAG, M_ALIGN } mode = M_TODO;
    int i = li - 1, j = lj - 1, lenj = lj - 1;
    int ic = si[i], jc = sj[j];
    long p = (long)(li) * (lenj + 1) - 1;
    while (i != 0 && j != 0) {
        int f = dm[p];
        if (mode == M_TODO) {
            if (f & OR_DO_HORIZONTAL) mode = M_HORZ;
            else if (f & OR_DO_ALIGN) mode = M_ALIGN;
            else if (f & OR_DO_VERTICAL) mode = M_VERT;
            else mode = M_DIAG;
        } else if (mode == M_VERT) {
            if (f & OR_END_VERTICAL) mode = M_TODO;
            if (!(ic & TMPGAP)) { pb_pre(median, ic | TMPGAP); pb_pre(medianwg, ic | TMPGAP); }
            else pb_pre(medianwg, TMPGAP);
            pb_pre(resi, ic); pb_pre(resj, TMPGAP);
            i--; p -= (lenj + 1); ic = si[i];
        } else if (mode == M_HORZ) {
            if (f & OR_END_HORIZONTAL) mode = M_TODO;
            if (!(jc & TMPGAP)) { pb_pre(median, jc | TMPGAP); pb_pre(medianwg, jc | TMPGAP); }
            else pb_pre(medianwg, TMPGAP);
            pb_pre(resi, TMPGAP); pb_pre(resj, jc);
            j--; p -= 1; jc = sj[j];
        } else if (mode == M_DIAG) {
            if (f & OR_END_BLOCK) mode = M_TODO;
            pb_pre(resi, ic); pb_pre(resj, jc); pb_pre(medianwg, TMPGAP);
            i--; j--; p -= (lenj + 2); jc = sj[j]; ic = si[i];
        } else {
            int prep;
            if (f & OR_ALIGN_TO_HORIZONTAL) mode = M_HORZ;
            else if (f & OR_ALIGN_TO_DIAGONAL) mode = M_DIAG;
            else if (f & OR_ALIGN_TO_VERTICAL) mode = M_VERT;
            prep = c->median[TBL(ic & NTMPGAP, jc & NTMPGAP)];
            pb_pre(median, prep); pb_pre(medianwg, prep);
            pb_pre(resi, ic); pb_pre(resj, jc);
            i--; j--; p -= (lenj + 2); jc = sj[j]; ic = si[i];
        }
    }
    while (i != 0) {
        if (!(ic & TMPGAP)) { pb_pre(median, ic | TMPGAP); pb_pre(medianwg, ic | TMPGAP); }
        else pb_pre(medianwg, TMPGAP);
        pb_pre(resi, ic); pb_pre(resj, TMPGAP);
        i--; ic = si[i];
    }
    while (j != 0) {
        if (!(jc & TMPGAP)) { pb_pre(median, jc | TMPGAP); pb_pre(medianwg, jc | TMPGAP); }
        else pb_pre(medianwg, TMPGAP);
        pb_pre(resi, TMPGAP); pb_pre(resj, jc);
        j--; jc = sj[j];
    }
    pb_pre(resi, TMPGAP); pb_pre(resj, TMPGAP); pb_pre(medianwg, TMPGAP);
    /* an empty median has no position 0 in the reference (out-of-range
     * read); treated here as "not a gap". */
    if (pb_len(median) == 0 || median->buf[median->head] != TMPGAP) pb_pre(median, TMPGAP);
}

int or_align_affine_3(const uint8_t *si, int li, const uint8_t *sj, int lj,
                      const or_cm *m, uint8_t *median, int *lmed,
                      uint8_t *medianwg, int *lmedwg, uint8_t *resi,
                      uint8_t *resj, int *lres) {
    /* algn_CAML_align_affine_3 (algn.c:2551-2619) */
    int cap = li + lj + 2, res;
    pbuf pm, pw, pi, pj;
    uint16_t *dm = (uint16_t *)malloc(sizeof(uint16_t) * (size_t)li * (size_t)lj);
    pb_init(&pm, cap); pb_init(&pw, cap); pb_init(&pi, cap); pb_init(&pj, cap);
    if (li <= lj) {
        res = aff_fill(si, li - 1, sj, lj - 1, m, 1, dm);
        aff_backtrace(dm, si, li, sj, lj, m, &pm, &pw, &pi, &pj);
    } else {
        res = aff_fill(sj, lj - 1, si, li - 1, m, 1, dm);
        aff_backtrace(dm, sj, lj, si, li, m, &pm, &pw, &pj, &pi);
    }
    free(dm);
    *lmed = pb_len(&pm); *lmedwg = pb_len(&pw); *lres = pb_len(&pi);
    pb_out(&pm, median); pb_out(&pw, medianwg); pb_out(&pi, resi); pb_out(&pj, resj);
    return res;
}

/* ------------------------------------------------------------------------ */
/* DOS.median (seqCS.ml:747-776)                                             */
/* ------------------------------------------------------------------------ */

static int is_empty(const uint8_t *s, int len, int gap) {
    /* Sequence.is_empty (sequence.ml:442-450) */
    int i;
    for (i = 0; i < len; i++) if (s[i] != gap) return 0;
    return 1;
}

int or_dos_median(const uint8_t *a, int la, const uint8_t *b, int lb,
                  const or_cm *m, uint8_t *seqm, int *lm, uint8_t *ra,
                  uint8_t *rb, uint8_t *medwg, int *lal) {
    if (is_empty(a, la, m->gap)) { memcpy(seqm, b, (size_t)lb); *lm = lb; *lal = 0; return 0; }
    if (is_empty(b, lb, m->gap)) { memcpy(seqm, a, (size_t)la); *lm = la; *lal = 0; return 0; }
    if (m->cost_model == 1) {
        int lw;
        return or_align_affine_3(a, la, b, lb, m, seqm, lm, medwg, &lw, ra, rb, lal);
    } else {
        int cost = or_align_2(a, la, b, lb, m, ra, rb, lal);
        *lm = or_ancestor_2(ra, rb, *lal, m, seqm);
        or_median_2_with_gaps(ra, rb, *lal, m, medwg);
        return cost;
    }
}

/* ------------------------------------------------------------------------ */
/* DOS.to_single (seqCS.ml:730-745) over Sequence.Align.closest             */
/* (sequence.ml:967-1033), combinations on (combine = 1)                    */
/* ------------------------------------------------------------------------ */

/* Cost_matrix.Two_D.get_closest (cost_matrix.ml:681-698): the state of b
 * closest to a; the states are tried lowest bit first (list_of_bits is
 * built high bit first and reversed) and the first strict minimum wins.
 * Returns -1 where b has no state ("No bits on?"). */
static int or_get_closest(const or_cm *m, int a, int b) {
    int gap = m->gap, best = a, bc = 0, found = 0, x;
    if (a != gap && b != gap) b = ((a & gap) && (b & gap)) ? gap : (b & ~gap);
    for (x = 0; x < m->lcm; x++) {
        int v = 1 << x;
        if (b & v) {
            int c = m->cost[TBL(a, v)];
            if (!found || c < bc) { best = v; bc = c; found = 1; }
        }
    }
    return found ? best : -1;
}

/* The single sequence of `mine` given its parent's single `parent`.
 * dos_empty selects DOS.to_single's rules (mine all gaps -> mine; parent
 * all gaps -> closest(mine, mine)); without it, Sequence.Align.closest's
 * (mine all gaps -> mine).  Returns the length written to `out`
 * (capacity lp + lm + 2), or -1 on a column without states. */
int or_closest(const uint8_t *parent, int lp, const uint8_t *mine, int lm,
               const or_cm *m, int dos_empty, uint8_t *out) {
    int gap = m->gap, n, i, k = 0;
    uint8_t *ra, *rb;
    if (is_empty(mine, lm, gap)) { memcpy(out, mine, (size_t)lm); return lm; }
    if (dos_empty && is_empty(parent, lp, gap)) { parent = mine; lp = lm; }
    ra = (uint8_t *)malloc((size_t)lp + lm + 2);
    rb = (uint8_t *)malloc((size_t)lp + lm + 2);
    if (lp == lm && memcmp(parent, mine, (size_t)lm) == 0) {
        /* identical: no alignment, the gap bit cleared past position 0 */
        n = lm;
        for (i = 0; i < n; i++) {
            ra[i] = (uint8_t)(i > 0 ? (parent[i] & ~gap) : parent[i]);
            rb[i] = (uint8_t)(i > 0 ? (mine[i] & ~gap) : mine[i]);
        }
    } else if (m->cost_model == 1) {
        uint8_t *md = (uint8_t *)malloc((size_t)lp + lm + 2);
        uint8_t *mw = (uint8_t *)malloc((size_t)lp + lm + 2);
        int lmd, lmw;
        or_align_affine_3(parent, lp, mine, lm, m, md, &lmd, mw, &lmw, ra, rb, &n);
        free(md);
        free(mw);
    } else {
        or_align_2(parent, lp, mine, lm, m, ra, rb, &n);
    }
    out[k++] = (uint8_t)gap;
    for (i = 0; i < n; i++) {
        int v = or_get_closest(m, ra[i], rb[i]);
        if (v < 0) { k = -1; break; }
        if (v != gap) out[k++] = (uint8_t)v;
    }
    free(ra);
    free(rb);
    return k;
}

/* ------------------------------------------------------------------------ */
/* Fitch (nonaddCSc.c, CHARSIZE 8)                                          */
/* ------------------------------------------------------------------------ */

int64_t or_nonadd_median(const uint8_t *a, const uint8_t *b, int len, uint8_t *res) {
    /* nonadd_median (nonaddCSc.c:422-462) */
    int64_t cost = 0;
    int i;
    for (i = 0; i < len; i++) {
        uint8_t in = a[i] & b[i];
        if (!in) { cost++; res[i] = a[i] | b[i]; }
        else res[i] = in;
    }
    return cost;
}

int64_t or_nonadd_distance(const uint8_t *a, const uint8_t *b, int len) {
    /* char_nonadd_CAML_distance (nonaddCSc.c:1076-1105) */
    int64_t cost = 0;
    int i;
    for (i = 0; i < len; i++) if (!(a[i] & b[i])) cost++;
    return cost;
}

void or_nonadd_median_3(const uint8_t *A, const uint8_t *N, const uint8_t *D1,
                        const uint8_t *D2, int len, uint8_t *F) {
    /* nonadd_median_3 (nonaddCSc.c:472-544) */
    int i;
    for (i = 0; i < len; i++) {
        uint8_t a = A[i], n = N[i], d1 = D1[i], d2 = D2[i];
        uint8_t inter = (uint8_t)(n | (a & (d1 | d2)));
        uint8_t temp = inter;
        uint8_t was_union = (uint8_t)((d1 & d2) == 0 ? 0xFF : 0);
        uint8_t contained, f;
        inter = (uint8_t)((inter | a) & was_union);
        temp |= inter;
        contained = (uint8_t)(((a & n) == a) ? 0xFF : 0);
        f = (uint8_t)(contained & a);
        contained = (uint8_t)(contained == 0 ? 0xFF : 0);
        temp &= contained;
        F[i] = (uint8_t)(f | temp);
    }
}

int64_t or_nonadd_dist_2(const uint8_t *a, const uint8_t *b, const uint8_t *c, int len) {
    /* char_nonadd_CAML_dist_2 (nonaddCSc.c:1349-1376) */
    int64_t d = 0;
    int i;
    for (i = 0; i < len; i++) if (!(a[i] & b[i]) && !(a[i] & c[i])) d++;
    return d;
}

/* NonaddCS16 / NonaddCS32: the same three rules on 16- and 32-bit state
 * sets (nonaddCSc.c built with CHARSIZE 16 / 32 under the nonadd16_ /
 * nonadd32_ names, myocamlbuild.ml.in:262-289).  Arrays hold len elements
 * of the width in host byte order. */
#define OR_NONADD_WIDE(W, T)                                                     \
int64_t or_nonadd##W##_median(const T *a, const T *b, int len, T *res) {          \
    int64_t cost = 0;                                                            \
    int i;                                                                       \
    for (i = 0; i < len; i++) {                                                  \
        T in = (T)(a[i] & b[i]);                                                 \
        if (!in) { cost++; res[i] = (T)(a[i] | b[i]); }                          \
        else res[i] = in;                                                        \
    }                                                                            \
    return cost;                                                                 \
}                                                                                \
int64_t or_nonadd##W##_distance(const T *a, const T *b, int len) {                \
    int64_t cost = 0;                                                            \
    int i;                                                                       \
    for (i = 0; i < len; i++) if (!(a[i] & b[i])) cost++;                        \
    return cost;                                                                 \
}                                                                                \
void or_nonadd##W##_median_3(const T *A, const T *N, const T *D1, const T *D2,    \
                             int len, T *F) {                                    \
    int i;                                                                       \
    for (i = 0; i < len; i++) {                                                  \
        T a = A[i], n = N[i], d1 = D1[i], d2 = D2[i];                            \
        T inter = (T)(n | (a & (d1 | d2)));                                      \
        T temp = inter;                                                          \
        T was_union = (T)((d1 & d2) == 0 ? ~(T)0 : 0);                           \
        T contained, f;                                                          \
        inter = (T)((inter | a) & was_union);                                    \
        temp |= inter;                                                           \
        contained = (T)(((a & n) == a) ? ~(T)0 : 0);                             \
        f = (T)(contained & a);                                                  \
        contained = (T)(contained == 0 ? ~(T)0 : 0);                             \
        temp &= contained;                                                       \
        F[i] = (T)(f | temp);                                                    \
    }                                                                            \
}
OR_NONADD_WIDE(16, uint16_t)
OR_NONADD_WIDE(32, uint32_t)

/* ------------------------------------------------------------------------ */
/* Sankoff (sankCS.ml)                                                       */
/* ------------------------------------------------------------------------ */

static int s_isinf(int64_t x) { return x >= OR_SANK_INF; }
static int64_t s_plus(int64_t a, int64_t b) { return (s_isinf(a) || s_isinf(b)) ? OR_SANK_INF : a + b; }
static int64_t s_minus(int64_t a, int64_t b) {
    /* cost_minus (sankCS.ml:50-55): an infinite minuend gives max_int */
    if (s_isinf(a)) return (int64_t)(((uint64_t)1 << 62) - 1);
    if (s_isinf(b)) return 0;
    return a - b;
}
static int s_less(int64_t a, int64_t b) { if (s_isinf(a)) return 0; if (s_isinf(b)) return 1; return a < b; }

void or_sank_elt_median(int k, const int64_t *tcm, const int64_t *a_s,
                        const int64_t *b_s, int64_t *c, int64_t *e, int64_t *beta) {
    /* elt_median (sankCS.ml:302-338) */
    int i, j, l, x;
    int64_t min_cost = OR_SANK_INF;
    for (i = 0; i < k; i++) {
        int64_t best = OR_SANK_INF;
        for (j = k - 1; j >= 0; j--) for (l = k - 1; l >= 0; l--) {
            int64_t cc = tcm[i * k + j] + tcm[i * k + l];
            cc = s_plus(s_plus(cc, a_s[j]), b_s[l]);
            if (s_less(cc, best)) best = cc;
        }
        if (s_less(best, min_cost)) min_cost = best;
        c[i] = best;
    }
    for (i = 0; i < k; i++) e[i] = s_minus(c[i], min_cost);
    for (i = 0; i < k; i++) {
        int64_t best = OR_SANK_INF;
        for (x = k - 1; x >= 0; x--) {
            int64_t v = s_plus(tcm[i * k + x], e[x]);
            if (s_less(v, best)) best = v;
        }
        beta[i] = best;
    }
}

/* Goloboff's beta of a preliminary cost vector s: e = s - min s with an
 * infinite state staying infinite (canonize, sankCS.ml:254-271, and
 * elt_median's e, whose max_int for an infinite state is infinite under
 * +$), then beta[y] = min_x tcm[y][x] +$ e[x]. */
static void or_sank_beta(int k, const int64_t *tcm, const int64_t *s, int64_t *beta) {
    int64_t e[64], mn = OR_SANK_INF;
    int x, y;
    for (x = 0; x < k; x++) if (s_less(s[x], mn)) mn = s[x];
    for (x = 0; x < k; x++) e[x] = s_isinf(s[x]) ? OR_SANK_INF : s_minus(s[x], mn);
    for (y = 0; y < k; y++) {
        int64_t best = OR_SANK_INF;
        for (x = k - 1; x >= 0; x--) {
            int64_t v = s_isinf(e[x]) ? e[x] : s_plus(e[x], tcm[y * k + x]);
            if (s_less(v, best)) best = v;
        }
        beta[y] = best;
    }
}

/* elt_median_3 (sankCS.ml:402-452): the final e and best states of node n
 * from its ancestor's final (a_e; a_best, a bit per state, 0 when the
 * ancestor has none, then its cheapest states of a_s are used), the node's
 * preliminary s (n_s) and the children's preliminary cost vectors (their
 * beta as in or_sank_beta).  Writes e_out[k] and the best-state bits. */
void or_sank_elt_median_3(int k, const int64_t *tcm, const int64_t *a_s, const int64_t *a_e,
                          uint32_t a_best, const int64_t *n_s, const int64_t *l_s,
                          const int64_t *r_s, int64_t *e_out, uint32_t *best_out) {
    int64_t lb[64], rb[64], bst[64];
    int i, s, x, pos;
    uint32_t abest = a_best, mine = 0;
    int64_t best_cost = OR_SANK_INF;
    or_sank_beta(k, tcm, l_s, lb);
    or_sank_beta(k, tcm, r_s, rb);
    for (i = 0; i < k; i++) {  /* init_d': the best over x for ancestor state i */
        int64_t b = OR_SANK_INF;
        for (x = k - 1; x >= 0; x--) {
            int64_t v = s_plus(s_plus(tcm[i * k + x], lb[x]), rb[x]);
            if (s_less(v, b)) b = v;
        }
        bst[i] = b;
    }
    for (s = 0; s < k; s++) {  /* init_e: min over ancestor states of d'[i][s] */
        int64_t b = OR_SANK_INF;
        for (x = k - 1; x >= 0; x--) {
            int64_t d = s_minus(s_plus(s_plus(s_plus(a_e[x], tcm[x * k + s]), lb[s]), rb[s]), bst[x]);
            if (s_less(d, b)) b = d;
        }
        e_out[s] = b;
    }
    if (!abest) {  /* the ancestor's cheapest states (plain comparisons) */
        int64_t c = OR_SANK_INF;
        for (pos = 0; pos < k; pos++) {
            if (c == a_s[pos]) abest |= 1u << pos;
            else if (c > a_s[pos]) { c = a_s[pos]; abest = 1u << pos; }
        }
    }
    for (pos = 0; pos < k; pos++) {  /* mybest: plain + and min, from infinity */
        int64_t mc = OR_SANK_INF;
        for (x = 0; x < k; x++)
            if ((abest >> x) & 1u) {
                int64_t v = n_s[pos] + tcm[pos * k + x];
                if (v < mc) mc = v;
            }
        if (mc == best_cost) mine |= 1u << pos;
        else if (mc < best_cost) { best_cost = mc; mine = 1u << pos; }
    }
    *best_out = mine;
}

double or_sank_elt_distance(int k, const int64_t *tcm, const int64_t *a_s, const int64_t *b_s) {
    /* elt_distance (sankCS.ml:347-354) */
    int64_t c[64], e[64], beta[64];
    int64_t mc = OR_SANK_INF, ma = OR_SANK_INF, mb = OR_SANK_INF;
    int i;
    or_sank_elt_median(k, tcm, a_s, b_s, c, e, beta);
    for (i = 0; i < k; i++) {
        if (s_less(c[i], mc)) mc = c[i];
        if (s_less(a_s[i], ma)) ma = a_s[i];
        if (s_less(b_s[i], mb)) mb = b_s[i];
    }
    {
        double fm = s_isinf(mc) ? __builtin_inf() : (double)mc;
        double fa = s_isinf(ma) ? __builtin_inf() : (double)ma;
        double fb = s_isinf(mb) ? __builtin_inf() : (double)mb;
        return fm - fa - fb;
    }
}

/* ------------------------------------------------------------------------ */
/* Batch driver for timing the CPU restatement (bench.py's CPU arms): runs   */
/* DOS.median's linear pieces (align_2, ancestor_2, median_2_with_gaps) or   */
/* the affine align_affine_3 on pairs idx[0..n) of a packed batch.           */
/* ------------------------------------------------------------------------ */
int64_t or_dos_median_many(const uint8_t *seq, const int64_t *a_off, const int32_t *a_len,
                           const int64_t *b_off, const int32_t *b_len, const int32_t *idx,
                           int n, const or_cm *m, int32_t *cost) {
    static __thread uint8_t *buf = NULL;
    static __thread size_t cap = 0;
    int64_t cells = 0;
    int t;
    for (t = 0; t < n; t++) {
        int i = idx[t];
        const uint8_t *a = seq + a_off[i], *b = seq + b_off[i];
        int la = a_len[i], lb = b_len[i], lm, lal;
        size_t need = (size_t)(la + lb + 4) * 4;
        if (need > cap) { free(buf); buf = (uint8_t *)malloc(need); cap = need; }
        {
            uint8_t *sm = buf, *ra = buf + (la + lb + 4), *rb = ra + (la + lb + 4), *wg = rb + (la + lb + 4);
            cost[t] = or_dos_median(a, la, b, lb, m, sm, &lm, ra, rb, wg, &lal);
        }
        if (m->cost_model == 1) cells += or_band_cells_affine(la, lb);
        else cells += or_band_cells_linear(la >= lb ? la : lb, la >= lb ? lb : la,
                                           or_cost2_deltaw(a, la, b, lb, m->gap, 0, 0));
    }
    return cells;
}

/* One result tail of a right-aligned slot: the last len bytes before end. */
static int or_tail_eq(const uint8_t *end, int32_t len, const uint8_t *want, int wlen) {
    return len == wlen && memcmp(end - len, want, (size_t)len) == 0;
}

/* or_dos_median_many that also checks batches computed elsewhere against
 * the restatement's outputs.  Each of the nset result sets holds, per pair
 * i of the batch, the cost cost[i], the lengths len[2i] (aligned pair and
 * median with gaps) and len[2i+1] (median), and a slot at out + off[i] of
 * four right-aligned sequences (aligned a, aligned b, median with gaps,
 * median), each cap = (la + lb + 5) & ~3 bytes: the layout batched align_2
 * writes.  bad[t] gets a bit per set whose pair idx[t] differs anywhere. */
int64_t or_dos_median_check_many(const uint8_t *seq, const int64_t *a_off, const int32_t *a_len,
                                 const int64_t *b_off, const int32_t *b_len, const int32_t *idx,
                                 int n, const or_cm *m, int32_t *cost, int nset,
                                 const or_result_set *sets, int32_t *bad) {
    static __thread uint8_t *buf = NULL;
    static __thread size_t cap = 0;
    int64_t cells = 0;
    int t, k;
    for (t = 0; t < n; t++) {
        int i = idx[t];
        const uint8_t *a = seq + a_off[i], *b = seq + b_off[i];
        int la = a_len[i], lb = b_len[i], lm = 0, lal = 0;
        size_t need = (size_t)(la + lb + 4) * 4;
        int64_t sc = ((int64_t)la + lb + 2 + 3) / 4 * 4;
        uint8_t *sm, *ra, *rb, *wg;
        if (need > cap) { free(buf); buf = (uint8_t *)malloc(need); cap = need; }
        sm = buf; ra = buf + (la + lb + 4); rb = ra + (la + lb + 4); wg = rb + (la + lb + 4);
        cost[t] = or_dos_median(a, la, b, lb, m, sm, &lm, ra, rb, wg, &lal);
        bad[t] = 0;
        for (k = 0; k < nset; k++) {
            const or_result_set *S = &sets[k];
            const uint8_t *slot = S->out + S->off[i];
            int32_t n0 = S->len[2 * i], n1 = S->len[2 * i + 1];
            int ok = S->cost[i] == cost[t] && n0 == lal && n1 == lm &&
                     or_tail_eq(slot + sc, n0, ra, lal) && or_tail_eq(slot + 2 * sc, n0, rb, lal) &&
                     or_tail_eq(slot + 4 * sc, n1, sm, lm);
            /* the median with gaps is defined for the linear model's
             * median_2_with_gaps and affine's medianwg alike */
            if (ok && lal > 0) ok = or_tail_eq(slot + 3 * sc, n0, wg, lal);
            if (!ok) bad[t] |= 1 << k;
        }
        if (m->cost_model == 1) cells += or_band_cells_affine(la, lb);
        else cells += or_band_cells_linear(la >= lb ? la : lb, la >= lb ? lb : la,
                                           or_cost2_deltaw(a, la, b, lb, m->gap, 0, 0));
    }
    return cells;
}

/* Candidate-join scores for the CPU timing of a search pass: for pairs
 * (a[t], b[t]) of nodes, DOS.distance (seqCS.ml:819-867) + Fitch distance
 * (nonaddCSc.c:1076-1105) + Sankoff distance (sankCS.ml:371-377).  Node
 * data: sequences in a packed buffer, Fitch rows [node][nf], Sankoff cost
 * vectors [node][ns][k] (int64, OR_SANK_INF = infinity). */
void or_candidate_scores(const uint8_t *seq, const int64_t *off, const int32_t *len,
                         const uint8_t *fitch, int nf, const int64_t *sank, int ns, int k,
                         const int64_t *tcm, const int32_t *a, const int32_t *b, int n,
                         const or_cm *m, int64_t *out) {
    int t, ch;
    for (t = 0; t < n; t++) {
        const uint8_t *x = seq + off[a[t]], *y = seq + off[b[t]];
        int lx = len[a[t]], ly = len[b[t]];
        int64_t s = or_cost_2(x, lx, y, ly, m, 1, or_dos_distance_deltaw(lx, ly));
        if (nf) s += or_nonadd_distance(fitch + (int64_t)a[t] * nf, fitch + (int64_t)b[t] * nf, nf);
        {
            double tot = 0.0;
            for (ch = 0; ch < ns; ch++)
                tot += or_sank_elt_distance(k, tcm, sank + ((int64_t)a[t] * ns + ch) * k,
                                            sank + ((int64_t)b[t] * ns + ch) * k);
            s += (int64_t)tot;
        }
        out[t] = s;
    }
}

/* ------------------------------------------------------------------------ */
/* Three-sequence alignment of the Iterative (ThreeD) mode:                  */
/* Sequence.Align.readjust_3d (sequence.ml:1117-1140) over                   */
/* align_3_powell_inter (sequence.ml:1089-1115) and powell_3D_align          */
/* (ukkCommon.c:111-143, ukk.checkp.c).                                      */
/* ------------------------------------------------------------------------ */

/* Powell's column states (ukkCommon.c setup, lines 206-262): one of match
 * (M), delete (D) or insert (I) per sequence, at least one M and at most
 * one I; code x0 + 3 x1 + 9 x2 with M 0, D 1, I 2, numbered in increasing
 * code order (16 states, MMM first).  A state without I advances its M
 * sequences; a state with I advances only the I sequence. */
typedef struct {
    int n;
    int code[OR_P3_STATES];
    int adv[OR_P3_STATES];   /* bit i: sequence i consumes a character */
    int gapm[OR_P3_STATES];  /* bit i: sequence i is in D or I */
    int ins[OR_P3_STATES];
    int ndel[OR_P3_STATES];
    int trans[OR_P3_STATES][OR_P3_STATES]; /* opening cost from s to t */
} p3_states;

static void p3_setup(p3_states *S, int go) {
    int code, s, t, i;
    S->n = 0;
    for (code = 0; code < 27; code++) {
        int x[3] = {code % 3, (code / 3) % 3, (code / 9) % 3};
        int nm = 0, ni = 0, nd = 0, adv = 0, gm = 0;
        for (i = 0; i < 3; i++) {
            nm += x[i] == 0; nd += x[i] == 1; ni += x[i] == 2;
            if (x[i] != 0) gm |= 1 << i;
        }
        if (nm == 0 || ni > 1) continue;
        for (i = 0; i < 3; i++)
            if (ni ? x[i] == 2 : x[i] == 0) adv |= 1 << i;
        S->code[S->n] = code; S->adv[S->n] = adv; S->gapm[S->n] = gm;
        S->ins[S->n] = ni; S->ndel[S->n] = nd;
        S->n++;
    }
    /* transition cost (ukkCommon.c:263-290): go for every sequence that
     * is in D or I in the new state and was not in that same state */
    for (s = 0; s < S->n; s++)
        for (t = 0; t < S->n; t++) {
            int c = 0;
            for (i = 0; i < 3; i++) {
                int xs = (S->code[s] / (i == 0 ? 1 : i == 1 ? 3 : 9)) % 3;
                int xt = (S->code[t] / (i == 0 ? 1 : i == 1 ? 3 : 9)) % 3;
                if (xt != 0 && xt != xs) c += go;
            }
            S->trans[s][t] = c;
        }
}

/* Column cost of state t over the characters its M (or I) sequences
 * consume (alignmentCost, ukkCommon.c:345-391): ge for an insert column;
 * otherwise ge per D plus mm per mismatch among the matched characters
 * (three matched: 0 all equal, 1 two equal, 2 all different). */
static int p3_col(const p3_states *S, int t, int mm, int ge, const int *ch) {
    int v[3], n = 0, i;
    if (S->ins[t]) return ge;
    for (i = 0; i < 3; i++) if (S->adv[t] >> i & 1) v[n++] = ch[i];
    {
        int c = ge * S->ndel[t];
        if (n == 2) c += (v[0] != v[1]) ? mm : 0;
        if (n == 3) {
            if (v[0] == v[1] && v[1] == v[2]) ;
            else if (v[0] == v[1] || v[0] == v[2] || v[1] == v[2]) c += mm;
            else c += 2 * mm;
        }
        return c;
    }
}

/* The character Powell's code aligns for a sequence element
 * (copySequence, ukkCommon.c:84-105): the lowest of the A, C, G, T bits;
 * -1 for an element with none (the reference fails). */
static int p3_base(int x) {
    if (x & 1) return 1;
    if (x & 2) return 2;
    if (x & 4) return 4;
    if (x & 8) return 8;
    return -1;
}

#define P3_INF (1 << 29)

int or_powell_3d(const uint8_t *a, int la, const uint8_t *b, int lb, const uint8_t *c, int lc,
                 int mm, int go, int ge, uint8_t *oa, uint8_t *ob, uint8_t *oc, int *olen) {
    /* The optimum of Powell's cost model by plain dynamic programming over
     * the (la x lb x lc) cube and the 16 states, instead of Powell's
     * furthest-reaching recursion: cell (i, j, k) holds, per state, the
     * least cost of aligning a[1..i], b[1..j], c[1..k] with that state in
     * the last column; the start (0, 0, 0) is MMM at cost 0 (the state
     * before the first column, ukkCommon.c:351 and ukk.checkp.c:99-107).
     * The cost equals powell_3D_align's; among equally cheap alignments
     * this one keeps, from the end, the lowest-numbered final state and at
     * every column the lowest-numbered previous state. */
    p3_states S;
    int na = la - 1, nb = lb - 1, nc = lc - 1, i, j, k, t, s;
    int64_t plane = (int64_t)lb * lc;
    int *V0, *V1;
    uint64_t *P;
    int best = P3_INF, bt = 0, cost;
    uint8_t *A = (uint8_t *)malloc((size_t)la + 1), *B = (uint8_t *)malloc((size_t)lb + 1),
            *C = (uint8_t *)malloc((size_t)lc + 1);
    if (la < 1 || lb < 1 || lc < 1) { free(A); free(B); free(C); return -1; }
    for (i = 1; i < la; i++) if ((A[i] = (uint8_t)p3_base(a[i])) == 0xff) { free(A); free(B); free(C); return -1; }
    for (i = 1; i < lb; i++) if ((B[i] = (uint8_t)p3_base(b[i])) == 0xff) { free(A); free(B); free(C); return -1; }
    for (i = 1; i < lc; i++) if ((C[i] = (uint8_t)p3_base(c[i])) == 0xff) { free(A); free(B); free(C); return -1; }
    p3_setup(&S, go);
    V0 = (int *)malloc(sizeof(int) * (size_t)plane * OR_P3_STATES);
    V1 = (int *)malloc(sizeof(int) * (size_t)plane * OR_P3_STATES);
    P = (uint64_t *)calloc((size_t)plane * la, sizeof(uint64_t));
    for (i = 0; i <= na; i++) {
        int *cur = (i & 1) ? V1 : V0, *prv = (i & 1) ? V0 : V1;
        for (j = 0; j <= nb; j++)
            for (k = 0; k <= nc; k++) {
                int *v = cur + ((int64_t)j * lc + k) * OR_P3_STATES;
                uint64_t pw = 0;
                for (t = 0; t < S.n; t++) {
                    int di = S.adv[t] & 1, dj = S.adv[t] >> 1 & 1, dk = S.adv[t] >> 2 & 1;
                    const int *u;
                    int ch[3], col, bv = P3_INF, bs = 0;
                    v[t] = P3_INF;
                    if (i == 0 && j == 0 && k == 0) { if (t == 0) v[t] = 0; continue; }
                    if (i < di || j < dj || k < dk) continue;
                    u = (di ? prv : cur) + ((int64_t)(j - dj) * lc + (k - dk)) * OR_P3_STATES;
                    ch[0] = A[i]; ch[1] = B[j]; ch[2] = C[k];
                    col = p3_col(&S, t, mm, ge, ch);
                    for (s = 0; s < S.n; s++) {
                        if (u[s] >= P3_INF) continue;
                        if (u[s] + S.trans[s][t] < bv) { bv = u[s] + S.trans[s][t]; bs = s; }
                    }
                    if (bv < P3_INF) { v[t] = bv + col; pw |= (uint64_t)bs << (4 * t); }
                }
                P[(int64_t)i * plane + (int64_t)j * lc + k] = pw;
            }
    }
    {
        const int *v = ((na & 1) ? V1 : V0) + ((int64_t)nb * lc + nc) * OR_P3_STATES;
        for (t = 0; t < S.n; t++) if (v[t] < best) { best = v[t]; bt = t; }
    }
    cost = best;
    /* traceback, writing the columns right-aligned then moving them left */
    {
        int cap = na + nb + nc + 1, n = 0;
        i = na; j = nb; k = nc; t = bt;
        while (i || j || k) {
            int di = S.adv[t] & 1, dj = S.adv[t] >> 1 & 1, dk = S.adv[t] >> 2 & 1;
            int s2 = (int)(P[(int64_t)i * plane + (int64_t)j * lc + k] >> (4 * t) & 15);
            n++;
            oa[cap - n] = di ? A[i] : 16;
            ob[cap - n] = dj ? B[j] : 16;
            oc[cap - n] = dk ? C[k] : 16;
            i -= di; j -= dj; k -= dk; t = s2;
        }
        n++;
        oa[cap - n] = ob[cap - n] = oc[cap - n] = 16;  /* the leading gap */
        memmove(oa, oa + cap - n, (size_t)n);
        memmove(ob, ob + cap - n, (size_t)n);
        memmove(oc, oc + cap - n, (size_t)n);
        *olen = n;
    }
    free(V0); free(V1); free(P); free(A); free(B); free(C);
    return cost;
}

int or_powell_alignment_cost(const uint8_t *oa, const uint8_t *ob, const uint8_t *oc, int n,
                             int mm, int go, int ge) {
    /* alignmentCost (ukkCommon.c:345-391) of an alignment whose columns
     * carry no states: each column takes the cheapest state that
     * consumes exactly its non-gap rows, given the previous column's
     * state (the all-gap leading column is skipped).  Exhaustive over
     * state sequences by dynamic programming on the column index. */
    p3_states S;
    int cur[OR_P3_STATES], nxt[OR_P3_STATES], x, t, s, best = P3_INF;
    p3_setup(&S, go);
    for (t = 0; t < S.n; t++) cur[t] = t == 0 ? 0 : P3_INF;
    for (x = 1; x < n; x++) {
        int adv = (oa[x] != 16) | (ob[x] != 16) << 1 | (oc[x] != 16) << 2;
        int ch[3] = {oa[x], ob[x], oc[x]};
        for (t = 0; t < S.n; t++) {
            nxt[t] = P3_INF;
            if (S.adv[t] != adv) continue;
            for (s = 0; s < S.n; s++)
                if (cur[s] < P3_INF && cur[s] + S.trans[s][t] < nxt[t]) nxt[t] = cur[s] + S.trans[s][t];
            if (nxt[t] < P3_INF) nxt[t] += p3_col(&S, t, mm, ge, ch);
        }
        memcpy(cur, nxt, sizeof(cur));
    }
    for (t = 0; t < S.n; t++) if (cur[t] < best) best = cur[t];
    return best;
}

void or_median3_table(const or_cm *m, uint8_t *tab) {
    /* Cost_matrix.Three_D.of_two_dim_comb (cost_matrix.ml:803-851): the
     * median of (i, j, k) is the lowest single state l minimising
     * cost[l][i] + cost[l][j] + cost[l][k]; the gap state takes part only
     * for metric matrices or when at least two of i, j, k hold the gap.
     * The reference seeds each entry with OCaml's max_int, which fits a C
     * int on a 32-bit OCaml; on a 64-bit one it becomes -1 and the table
     * keeps no median at all.  This follows the 32-bit reading.  Indexed
     * (i << 10) | (j << 5) | k. */
    int i, j, k, l;
    memset(tab, 0, 32768);
    for (i = 1; i < 32; i++)
        for (j = 1; j < 32; j++)
            for (k = 1; k < 32; k++) {
                int64_t best = INT64_MAX;
                int med = 0;
                for (l = 0; l < m->lcm; l++) {
                    int inter = 1 << l;
                    int shared = ((i & inter) != 0) + ((j & inter) != 0) + ((k & inter) != 0);
                    int64_t c;
                    if (m->is_metric || shared >= 2 || inter != m->gap)
                        c = (int64_t)m->cost[(inter << 5) + i] + m->cost[(inter << 5) + j] +
                            m->cost[(inter << 5) + k];
                    else
                        c = INT64_MAX;
                    if (c < best) { best = c; med = inter; }
                    else if (c == best) med |= inter;
                }
                tab[(i << 10) | (j << 5) | k] = (uint8_t)(med & -med);
            }
}

int or_readjust_3d(const uint8_t *s1, int l1, const uint8_t *s2, int l2, const uint8_t *cm_,
                   int lm, const uint8_t *p, int lp, const or_cm *m, const uint8_t *tab3,
                   uint8_t *res, int *lres, int *changed) {
    /* Sequence.Align.readjust_3d with first_gap = true
     * (sequence.ml:1117-1140): the early returns, then
     * align_3_powell_inter (sequence.ml:1089-1115) with mm = cost 1 2,
     * go = the affine opening (0 for the linear model) and ge = cost 1 16;
     * the median keeps the non-gap column medians behind one leading gap.
     * cm_ is the node's current median m.  Returns the cost, or -1 where
     * the reference fails (an element without A, C, G or T). */
    int gap = m->gap, cost, n, x, q;
    const uint8_t *keep = NULL;
    int lkeep = 0;
    if (l1 == l2 && lm == lp && l1 == lm) { keep = cm_; lkeep = lm; cost = 0; }
    else if (is_empty(s1, l1, gap) && !is_empty(s2, l2, gap)) { keep = s2; lkeep = l2; cost = 0; }
    else if (is_empty(s2, l2, gap) && !is_empty(s1, l1, gap)) { keep = s1; lkeep = l1; cost = 0; }
    else if (is_empty(p, lp, gap)) { keep = p; lkeep = lp; cost = 0; }
    if (keep) {
        memcpy(res, keep, (size_t)lkeep);
        *lres = lkeep;
    } else {
        int cap = l1 + l2 + lp;
        uint8_t *oa = (uint8_t *)malloc((size_t)cap), *ob = (uint8_t *)malloc((size_t)cap),
                *oc = (uint8_t *)malloc((size_t)cap);
        int mmc = m->cost[(1 << 5) + 2], ge = m->cost[(1 << 5) + 16];
        int go = m->cost_model == 1 ? m->gap_open : 0;
        cost = or_powell_3d(s1, l1, s2, l2, p, lp, mmc, go, ge, oa, ob, oc, &n);
        if (cost < 0) { free(oa); free(ob); free(oc); return -1; }
        q = 0;
        res[q++] = (uint8_t)gap;
        for (x = 0; x < n; x++) {
            int md = tab3[(oa[x] << 10) | (ob[x] << 5) | oc[x]];
            if (md != gap) res[q++] = (uint8_t)md;
        }
        *lres = q;
        free(oa); free(ob); free(oc);
    }
    *changed = (*lres != lm) || memcmp(res, cm_, (size_t)lm) != 0;
    return cost;
}
