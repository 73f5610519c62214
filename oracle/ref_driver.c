/*
 * Plain-C driver around the reference's own compiled C kernels (algn.c,
 * nonaddCSc.c built by oracle/build_ref.sh).  TEST INFRASTRUCTURE ONLY: it
 * gives the tests and the CPU reference arm of bench.py pointer-and-size entry
 * points into the reference code, emulating the OCaml custom blocks the
 * reference expects (struct seq with its data at the end of the buffer,
 * seq.h:29-54; struct cm, cm.h:29-43; struct matrices, matrices.h:44-56).
 *
 * Built only where the reference sources are present; never shipped.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <caml/mlvalues.h>
#include <caml/bigarray.h>
#include <caml/custom.h>
#include "seq.h"
#include "cm.h"
#include "matrices.h"
#include "poy_oracle.h"

/* reference entry points (algn.c, nonaddCSc.c after the 8-bit rename) */
value algn_CAML_simple_2(value s1, value s2, value c, value a, value deltawh);
value algn_CAML_backtrack_2d(value s1, value s2, value s1p, value s2p, value a, value c, value swap);
value algn_CAML_cost_affine_3(value si, value sj, value cm, value am);
value algn_CAML_align_affine_3(value si, value sj, value cm, value am, value resi,
                               value resj, value median, value medianwg);
value algn_CAML_ancestor_2(value s1, value s2, value m, value sm);
value algn_CAML_median_2_with_gaps(value s1, value s2, value m, value sm);
value algn_CAML_median_2_no_gaps(value s1, value s2, value m, value sm);
value algn_CAML_worst_2(value s1, value s2, value c);
value algn_CAML_verify_2(value s1, value s2, value c);
value char_nonadd8_CAML_basic_median(value v, value a, value b);
value char_nonadd8_CAML_distance(value a, value b);
value char_nonadd8_CAML_median_3(value v, value vA, value vN, value vD1, value vD2);
value char_nonadd8_CAML_dist_2(value va, value vb, value vc);
value char_nonadd16_CAML_basic_median(value v, value a, value b);
value char_nonadd16_CAML_distance(value a, value b);
value char_nonadd16_CAML_median_3(value v, value vA, value vN, value vD1, value vD2);
value char_nonadd32_CAML_basic_median(value v, value a, value b);
value char_nonadd32_CAML_distance(value a, value b);
value char_nonadd32_CAML_median_3(value v, value vA, value vN, value vD1, value vD2);

/* ---- runtime stand-ins declared by the stub headers ---- */
value oracle_alloc_custom(struct custom_operations *ops, uintptr_t size, uintptr_t mem, uintptr_t max) {
    (void)ops; (void)mem; (void)max;
    return (value)calloc(1, size);
}
value oracle_copy_double(double d) {
    static __thread double slot;
    slot = d;
    return (value)&slot;
}
value oracle_alloc(uintptr_t n, int tag) { (void)tag; return (value)calloc(n + 1, sizeof(value)); }
value oracle_alloc_bigarray(int flags, int ndims, void *data, intptr_t *dims) {
    (void)flags; (void)ndims; (void)dims;
    struct caml_ba_array *b = calloc(1, sizeof(*b));
    b->data = data;
    return (value)b;
}

/* ---- custom-block emulation ---- */
typedef struct { struct seq s; } seq_hdr;

static value make_seq(int cap, const uint8_t *data, int len) {
    struct seq *sq = (struct seq *)calloc(1, sizeof(struct seq) + (size_t)cap + 16);
    sq->magic_number = POY_SEQ_MAGIC_NUMBER;
    sq->cap = cap;
    sq->len = len;
    sq->head = (SEQT *)(sq + 1);
    sq->end = sq->head + cap - 1;
    sq->begin = sq->end - len + 1;
    if (len) memcpy(sq->begin, data, (size_t)len);
    return (value)sq;
}
static int seq_out(value v, uint8_t *out) {
    struct seq *sq = (struct seq *)v;
    SEQT *head = (SEQT *)(sq + 1);
    SEQT *end = head + sq->cap - 1;
    SEQT *begin = end - sq->len + 1;
    if (out && sq->len) memcpy(out, begin, (size_t)sq->len);
    return sq->len;
}

static __thread struct matrices *tl_mat;
static struct matrices *mat(void) {
    if (!tl_mat) tl_mat = (struct matrices *)calloc(1, sizeof(struct matrices));
    return tl_mat;
}

/* struct cm built from the oracle's table layout (tables indexed (a<<5)+b;
 * the reference allocates 2*(1<<lcm)^2 entries, cm.c:340-352). */
void *ref_cm_new(const or_cm *m) {
    struct cm *c = (struct cm *)calloc(1, sizeof(struct cm));
    size_t n = 2 * 32 * 32;
    c->a_sz = m->a_sz; c->lcm = m->lcm; c->gap = m->gap;
    c->cost_model_type = m->cost_model; c->combinations = m->combinations;
    c->gap_open = m->gap_open; c->is_metric = m->is_metric;
    c->all_elements = m->all_elements;
    c->cost = (int *)calloc(n, sizeof(int));
    c->worst = (int *)calloc(n, sizeof(int));
    c->prepend_cost = (int *)calloc(n, sizeof(int));
    c->tail_cost = (int *)calloc(n, sizeof(int));
    c->median = (SEQT *)calloc(n, sizeof(SEQT));
    memcpy(c->cost, m->cost, sizeof(m->cost));
    memcpy(c->worst, m->worst, sizeof(m->worst));
    memcpy(c->prepend_cost, m->prepend, sizeof(m->prepend));
    memcpy(c->tail_cost, m->tail, sizeof(m->tail));
    memcpy(c->median, m->median, sizeof(m->median));
    return c;
}
void ref_cm_free(void *p) {
    struct cm *c = (struct cm *)p;
    free(c->cost); free(c->worst); free(c->prepend_cost); free(c->tail_cost); free(c->median);
    free(c);
}

int ref_simple_2(const uint8_t *s1, int l1, const uint8_t *s2, int l2, void *cm, int deltaw) {
    value a = make_seq(l1, s1, l1), b = make_seq(l2, s2, l2);
    int r = Int_val(algn_CAML_simple_2(a, b, (value)cm, (value)mat(), Val_int(deltaw)));
    free((void *)a); free((void *)b);
    return r;
}

/* Sequence.Align.align_2 (sequence.ml:849-869) for the linear model, with
 * the caller-computed deltaw: cost_2 followed by create_edited_2. */
int ref_align_2(const uint8_t *s1, int l1, const uint8_t *s2, int l2, void *cm, int deltaw,
                uint8_t *o1, uint8_t *o2, int *olen) {
    value a = make_seq(l1, s1, l1), b = make_seq(l2, s2, l2);
    value p1 = make_seq(l1 + l2, NULL, 0), p2 = make_seq(l1 + l2, NULL, 0);
    int r;
    if (l1 >= l2) {
        r = Int_val(algn_CAML_simple_2(a, b, (value)cm, (value)mat(), Val_int(deltaw)));
        algn_CAML_backtrack_2d(a, b, p1, p2, (value)mat(), (value)cm, Val_true);
    } else {
        r = Int_val(algn_CAML_simple_2(b, a, (value)cm, (value)mat(), Val_int(deltaw)));
        algn_CAML_backtrack_2d(b, a, p2, p1, (value)mat(), (value)cm, Val_false);
    }
    *olen = seq_out(p1, o1);
    seq_out(p2, o2);
    free((void *)a); free((void *)b); free((void *)p1); free((void *)p2);
    return r;
}

int ref_cost_affine_3(const uint8_t *s1, int l1, const uint8_t *s2, int l2, void *cm) {
    value a = make_seq(l1, s1, l1), b = make_seq(l2, s2, l2);
    int r = Int_val(algn_CAML_cost_affine_3(a, b, (value)cm, (value)mat()));
    free((void *)a); free((void *)b);
    return r;
}

int ref_align_affine_3(const uint8_t *s1, int l1, const uint8_t *s2, int l2, void *cm,
                       uint8_t *med, int *lmed, uint8_t *medwg, int *lmedwg,
                       uint8_t *r1, uint8_t *r2, int *lres) {
    int cap = l1 + l2 + 2;
    value a = make_seq(l1, s1, l1), b = make_seq(l2, s2, l2);
    value ri = make_seq(cap, NULL, 0), rj = make_seq(cap, NULL, 0);
    value m = make_seq(cap, NULL, 0), mw = make_seq(cap, NULL, 0);
    int r = Int_val(algn_CAML_align_affine_3(a, b, (value)cm, (value)mat(), ri, rj, m, mw));
    *lmed = seq_out(m, med); *lmedwg = seq_out(mw, medwg);
    *lres = seq_out(ri, r1); seq_out(rj, r2);
    free((void *)a); free((void *)b); free((void *)ri); free((void *)rj);
    free((void *)m); free((void *)mw);
    return r;
}

int ref_ancestor_2(const uint8_t *s1, const uint8_t *s2, int len, void *cm, uint8_t *out) {
    value a = make_seq(len, s1, len), b = make_seq(len, s2, len), o = make_seq(len + 1, NULL, 0);
    int n;
    algn_CAML_ancestor_2(a, b, (value)cm, o);
    n = seq_out(o, out);
    free((void *)a); free((void *)b); free((void *)o);
    return n;
}

int ref_median_2_with_gaps(const uint8_t *s1, const uint8_t *s2, int len, void *cm, uint8_t *out) {
    value a = make_seq(len, s1, len), b = make_seq(len, s2, len), o = make_seq(len, NULL, 0);
    int n;
    algn_CAML_median_2_with_gaps(a, b, (value)cm, o);
    n = seq_out(o, out);
    free((void *)a); free((void *)b); free((void *)o);
    return n;
}

int ref_median_2_no_gaps(const uint8_t *s1, const uint8_t *s2, int len, void *cm, uint8_t *out) {
    value a = make_seq(len, s1, len), b = make_seq(len, s2, len), o = make_seq(len + 1, NULL, 0);
    int n;
    algn_CAML_median_2_no_gaps(a, b, (value)cm, o);
    n = seq_out(o, out);
    free((void *)a); free((void *)b); free((void *)o);
    return n;
}

int ref_worst_2(const uint8_t *s1, const uint8_t *s2, int len, void *cm) {
    value a = make_seq(len, s1, len), b = make_seq(len, s2, len);
    int r = Int_val(algn_CAML_worst_2(a, b, (value)cm));
    free((void *)a); free((void *)b);
    return r;
}

int ref_verify_2(const uint8_t *s1, const uint8_t *s2, int len, void *cm) {
    value a = make_seq(len, s1, len), b = make_seq(len, s2, len);
    int r = Int_val(algn_CAML_verify_2(a, b, (value)cm));
    free((void *)a); free((void *)b);
    return r;
}

/* ---- Fitch (8-bit), struct _naca_t layout (nonaddCSc.c:293-300) ---- */
struct ref_naca { long len, heur, code, added_cost; void *data; };

/* len elements of eb bytes each */
static value make_naca_w(const void *d, int len, int eb) {
    size_t sz = sizeof(struct ref_naca) + (size_t)len * eb + 64;
    struct ref_naca *n = (struct ref_naca *)calloc(1, sz);
    n->len = len;
    n->data = (void *)(n + 1);
    if (d) memcpy(n + 1, d, (size_t)len * eb);
    return (value)n;
}
static value make_naca(const uint8_t *d, int len) { return make_naca_w(d, len, 1); }

long ref_nonadd8_median(const uint8_t *a, const uint8_t *b, int len, uint8_t *res) {
    value va = make_naca(a, len), vb = make_naca(b, len), vr = make_naca(NULL, len);
    long c;
    char_nonadd8_CAML_basic_median(vr, va, vb);
    memcpy(res, (struct ref_naca *)vr + 1, (size_t)len);
    c = ((struct ref_naca *)vr)->added_cost;
    free((void *)va); free((void *)vb); free((void *)vr);
    return c;
}

long ref_nonadd8_distance(const uint8_t *a, const uint8_t *b, int len) {
    value va = make_naca(a, len), vb = make_naca(b, len);
    long c = Long_val(char_nonadd8_CAML_distance(va, vb));
    free((void *)va); free((void *)vb);
    return c;
}

void ref_nonadd8_median_3(const uint8_t *A, const uint8_t *N, const uint8_t *D1,
                          const uint8_t *D2, int len, uint8_t *F) {
    value va = make_naca(A, len), vn = make_naca(N, len), v1 = make_naca(D1, len),
          v2 = make_naca(D2, len), vf = make_naca(NULL, len);
    char_nonadd8_CAML_median_3(vf, va, vn, v1, v2);
    memcpy(F, (struct ref_naca *)vf + 1, (size_t)len);
    free((void *)va); free((void *)vn); free((void *)v1); free((void *)v2); free((void *)vf);
}

long ref_nonadd8_dist_2(const uint8_t *a, const uint8_t *b, const uint8_t *c, int len) {
    value va = make_naca(a, len), vb = make_naca(b, len), vc = make_naca(c, len);
    long d = Long_val(char_nonadd8_CAML_dist_2(va, vb, vc));
    free((void *)va); free((void *)vb); free((void *)vc);
    return d;
}

/* ---- Fitch on 16- and 32-bit state sets (nonaddCSc.c with CHARSIZE 16 / 32) ---- */
#define REF_NONADD_WIDE(W, EB)                                                        \
long ref_nonadd##W##_median(const void *a, const void *b, int len, void *res) {       \
    value va = make_naca_w(a, len, EB), vb = make_naca_w(b, len, EB),                 \
          vr = make_naca_w(NULL, len, EB);                                            \
    long c;                                                                           \
    char_nonadd##W##_CAML_basic_median(vr, va, vb);                                   \
    memcpy(res, (struct ref_naca *)vr + 1, (size_t)len * EB);                         \
    c = ((struct ref_naca *)vr)->added_cost;                                          \
    free((void *)va); free((void *)vb); free((void *)vr);                             \
    return c;                                                                         \
}                                                                                     \
long ref_nonadd##W##_distance(const void *a, const void *b, int len) {                \
    value va = make_naca_w(a, len, EB), vb = make_naca_w(b, len, EB);                 \
    long c = Long_val(char_nonadd##W##_CAML_distance(va, vb));                        \
    free((void *)va); free((void *)vb);                                               \
    return c;                                                                         \
}                                                                                     \
void ref_nonadd##W##_median_3(const void *A, const void *N, const void *D1,           \
                              const void *D2, int len, void *F) {                     \
    value va = make_naca_w(A, len, EB), vn = make_naca_w(N, len, EB),                 \
          v1 = make_naca_w(D1, len, EB), v2 = make_naca_w(D2, len, EB),               \
          vf = make_naca_w(NULL, len, EB);                                            \
    char_nonadd##W##_CAML_median_3(vf, va, vn, v1, v2);                               \
    memcpy(F, (struct ref_naca *)vf + 1, (size_t)len * EB);                           \
    free((void *)va); free((void *)vn); free((void *)v1); free((void *)v2);           \
    free((void *)vf);                                                                 \
}
REF_NONADD_WIDE(16, 2)
REF_NONADD_WIDE(32, 4)

/* powell_3D_align (ukkCommon.c:111-143) through its OCaml external: three
 * sequences with their leading gap, the aligned rows prepended into seqs
 * of capacity la + lb + lc (align_3_powell, sequence.ml:1078-1087). */
value powell_3D_align(value sa, value sb, value sc, value ra, value rb, value rc,
                      value mm, value go, value ge);
int ref_powell_3d(const uint8_t *a, int la, const uint8_t *b, int lb, const uint8_t *c, int lc,
                  int mm, int go, int ge, uint8_t *oa, uint8_t *ob, uint8_t *oc, int *olen) {
    int cap = la + lb + lc;
    value va = make_seq(la, a, la), vb = make_seq(lb, b, lb), vc = make_seq(lc, c, lc);
    value pa = make_seq(cap, NULL, 0), pb = make_seq(cap, NULL, 0), pc = make_seq(cap, NULL, 0);
    int r = Int_val(powell_3D_align(va, vb, vc, pa, pb, pc, Val_int(mm), Val_int(go), Val_int(ge)));
    *olen = seq_out(pa, oa);
    seq_out(pb, ob);
    seq_out(pc, oc);
    free((void *)va); free((void *)vb); free((void *)vc);
    free((void *)pa); free((void *)pb); free((void *)pc);
    return r;
}
