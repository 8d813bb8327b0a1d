/*
 * ish_oracle.c -- CPU restatement of ish's striped alignment-scoring path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA path and the timed
 * CPU baseline.  The product never links or calls this file.
 *
 * Citations are to the ish repository (Mojo, v1.4.0).  The lane loops below
 * restate the reference's SIMD vectors lane by lane; with W fixed at compile
 * time (8 / 16) GCC vectorises them again.
 */
#include "ish_oracle.h"

#include <stdlib.h>
#include <string.h>

#define ISH_O_MAXW 64

/* ------------------------------------------------------------------------ */
/* Matrices and encodings: scoring_matrix.mojo:9-172 (tables), 328-391       */
/* (constructors), 403-416 (encode + optimal score).                          */
/* ------------------------------------------------------------------------ */

/* BLOSUM62 in the residue order A R N D C Q E G H I L K M F P S T W Y V B Z X *
 * (scoring_matrix.mojo:98-124, the parasail ordering). */
static const int8_t O_BLOSUM62[24 * 24] = {
    4, -1, -2, -2, 0, -1, -1, 0, -2, -1, -1, -1, -1, -2, -1, 1, 0, -3, -2, 0, -2, -1, 0, -4,
    -1, 5, 0, -2, -3, 1, 0, -2, 0, -3, -2, 2, -1, -3, -2, -1, -1, -3, -2, -3, -1, 0, -1, -4,
    -2, 0, 6, 1, -3, 0, 0, 0, 1, -3, -3, 0, -2, -3, -2, 1, 0, -4, -2, -3, 3, 0, -1, -4,
    -2, -2, 1, 6, -3, 0, 2, -1, -1, -3, -4, -1, -3, -3, -1, 0, -1, -4, -3, -3, 4, 1, -1, -4,
    0, -3, -3, -3, 9, -3, -4, -3, -3, -1, -1, -3, -1, -2, -3, -1, -1, -2, -2, -1, -3, -3, -2, -4,
    -1, 1, 0, 0, -3, 5, 2, -2, 0, -3, -2, 1, 0, -3, -1, 0, -1, -2, -1, -2, 0, 3, -1, -4,
    -1, 0, 0, 2, -4, 2, 5, -2, 0, -3, -3, 1, -2, -3, -1, 0, -1, -3, -2, -2, 1, 4, -1, -4,
    0, -2, 0, -1, -3, -2, -2, 6, -2, -4, -4, -2, -3, -3, -2, 0, -2, -2, -3, -3, -1, -2, -1, -4,
    -2, 0, 1, -1, -3, 0, 0, -2, 8, -3, -3, -1, -2, -1, -2, -1, -2, -2, 2, -3, 0, 0, -1, -4,
    -1, -3, -3, -3, -1, -3, -3, -4, -3, 4, 2, -3, 1, 0, -3, -2, -1, -3, -1, 3, -3, -3, -1, -4,
    -1, -2, -3, -4, -1, -2, -3, -4, -3, 2, 4, -2, 2, 0, -3, -2, -1, -2, -1, 1, -4, -3, -1, -4,
    -1, 2, 0, -1, -3, 1, 1, -2, -1, -3, -2, 5, -1, -3, -1, 0, -1, -3, -2, -2, 0, 1, -1, -4,
    -1, -1, -2, -3, -1, 0, -2, -3, -2, 1, 2, -1, 5, 0, -2, -1, -1, -1, -1, 1, -3, -1, -1, -4,
    -2, -3, -3, -3, -2, -3, -3, -3, -1, 0, 0, -3, 0, 6, -4, -2, -2, 1, 3, -1, -3, -3, -1, -4,
    -1, -2, -2, -1, -3, -1, -1, -2, -2, -3, -3, -1, -2, -4, 7, -1, -1, -4, -3, -2, -2, -1, -2, -4,
    1, -1, 1, 0, -1, 0, 0, 0, -1, -2, -2, 0, -1, -2, -1, 4, 1, -3, -2, -2, 0, 0, 0, -4,
    0, -1, 0, -1, -1, -1, -1, -2, -2, -1, -1, -1, -1, -2, -1, 1, 5, -2, -2, 0, -1, -1, 0, -4,
    -3, -3, -4, -4, -2, -2, -3, -2, -2, -3, -2, -3, -1, 1, -4, -3, -2, 11, 2, -3, -4, -3, -2, -4,
    -2, -2, -2, -3, -2, -1, -2, -3, 2, -1, -1, -2, -1, 3, -3, -2, -2, 2, 7, -1, -3, -2, -1, -4,
    0, -3, -3, -3, -1, -2, -2, -3, -3, 3, 1, -2, 1, -1, -2, -2, 0, -3, -1, 4, -3, -2, -1, -4,
    -2, -1, 3, 4, -3, 0, 1, -1, 0, -3, -4, 0, -3, -3, -2, 0, -1, -4, -3, -3, 4, 1, -1, -4,
    -1, 0, 0, 1, -3, 3, 4, -2, 0, -3, -3, 1, -1, -3, -1, 0, -1, -3, -2, -2, 1, 4, -1, -4,
    0, -1, -1, -1, -2, -1, -1, -1, -1, -1, -1, -1, -1, -1, -2, 0, 0, -2, -1, -1, -1, -1, -1, -4,
    -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, 1,
};
/* ACTGN (scoring_matrix.mojo:156-163): +2 on the diagonal, -2 off it, N (code
 * 4) scores +2 against everything.  ACTGN0 (165-172): N scores 0. */
static const int8_t O_ACTGN[25] = {2, -2, -2, -2, 2, -2, 2, -2, -2, 2, -2, -2, 2,
                                   -2, 2, -2, -2, -2, 2, 2, 2, 2, 2, 2, 2};
static const int8_t O_ACTGN0[25] = {2, -2, -2, -2, 0, -2, 2, -2, -2, 0, -2, -2, 2,
                                    -2, 0, -2, -2, -2, 2, 0, 0, 0, 0, 0, 0};
static int8_t O_ASCII[256 * 256];
static uint8_t O_AA_TO_NUM[256], O_NT_TO_NUM[256], O_IDENT[256];
static const uint8_t O_NUM_TO_AA[24] = {'A', 'R', 'N', 'D', 'C', 'Q', 'E', 'G', 'H', 'I', 'L', 'K',
                                        'M', 'F', 'P', 'S', 'T', 'W', 'Y', 'V', 'B', 'Z', 'X', '*'};
static const uint8_t O_NUM_TO_NT[5] = {'A', 'C', 'G', 'T', 'N'};
static int o_tables_ready = 0;

static void o_tables(void) {
    if (o_tables_ready) return;
    /* ScoringMatrix._default_matrix(256): match 2, mismatch -2 (379-391). */
    for (int i = 0; i < 256; i++)
        for (int j = 0; j < 256; j++) O_ASCII[i * 256 + j] = (i == j) ? 2 : -2;
    for (int i = 0; i < 256; i++) O_IDENT[i] = (uint8_t)i;
    /* AA_TO_NUM (9-27): unknown bytes map to 23 ('*'); upper and lower case
     * letters map to the index of the letter in O_NUM_TO_AA, J O U -> 23. */
    for (int i = 0; i < 256; i++) O_AA_TO_NUM[i] = 23;
    for (int c = 0; c < 24; c++) {
        uint8_t a = O_NUM_TO_AA[c];
        if (a >= 'A' && a <= 'Z') {
            O_AA_TO_NUM[a] = (uint8_t)c;
            O_AA_TO_NUM[a + 32] = (uint8_t)c;
        }
    }
    /* NT_TO_NUM (131-149): A/a 0, C/c 1, G/g 2, T/t U/u 3, anything else 4. */
    for (int i = 0; i < 256; i++) O_NT_TO_NUM[i] = 4;
    O_NT_TO_NUM['A'] = O_NT_TO_NUM['a'] = 0;
    O_NT_TO_NUM['C'] = O_NT_TO_NUM['c'] = 1;
    O_NT_TO_NUM['G'] = O_NT_TO_NUM['g'] = 2;
    O_NT_TO_NUM['T'] = O_NT_TO_NUM['t'] = 3;
    O_NT_TO_NUM['U'] = O_NT_TO_NUM['u'] = 3;
    o_tables_ready = 1;
}

int ish_o_matrix(int kind, const int8_t **values, const uint8_t **a2c, const uint8_t **c2a) {
    o_tables();
    switch (kind) {
    case ISH_O_ASCII:
        *values = O_ASCII; *a2c = O_IDENT; *c2a = O_IDENT;
        return 256;
    case ISH_O_ACTGN:
        *values = O_ACTGN; *a2c = O_NT_TO_NUM; *c2a = O_NUM_TO_NT;
        return 5;
    case ISH_O_ACTGN0:
        *values = O_ACTGN0; *a2c = O_NT_TO_NUM; *c2a = O_NUM_TO_NT;
        return 5;
    case ISH_O_BLOSUM62:
        *values = O_BLOSUM62; *a2c = O_AA_TO_NUM; *c2a = O_NUM_TO_AA;
        return 24;
    default:
        return -1;
    }
}

int32_t ish_o_encode_and_score(int kind, const uint8_t *ascii, size_t n, uint8_t *out) {
    const int8_t *M; const uint8_t *a2c, *c2a;
    int size = ish_o_matrix(kind, &M, &a2c, &c2a);
    int32_t score = 0;
    for (size_t i = 0; i < n; i++) {
        uint8_t c = a2c[ascii[i]];
        score += M[c * size + c];
        out[i] = c;
    }
    return score;
}

void ish_o_encode(int kind, const uint8_t *ascii, size_t n, uint8_t *out) {
    const int8_t *M; const uint8_t *a2c, *c2a;
    ish_o_matrix(kind, &M, &a2c, &c2a);
    for (size_t i = 0; i < n; i++) out[i] = a2c[ascii[i]];
}

void ish_o_matrix_minmax(const int8_t *M, int size, int8_t *mn, int8_t *mx) {
    /* Profile.__init__ (semi_global_aln/striped.mojo:62-71): starts at 0. */
    int8_t lo = 0, hi = 0;
    for (int i = 0; i < size * size; i++) {
        if (M[i] < lo) lo = M[i];
        if (M[i] > hi) hi = M[i];
    }
    *mn = lo;
    *mx = hi;
}

uint8_t ish_o_sw_bias(const int8_t *M, int size) {
    /* local_aln/striped.mojo:81-85: bias = |min(0, min M)|. */
    int8_t lo = 0;
    for (int i = 0; i < size * size; i++)
        if (M[i] < lo) lo = M[i];
    return (uint8_t)(lo < 0 ? -lo : lo);
}

/* ------------------------------------------------------------------------ */
/* Query profiles: semi_global_aln/striped.mojo:92-118, local 110-139.       */
/* ------------------------------------------------------------------------ */
void ish_o_sg_profile_i16(const uint8_t *q, int Q, const int8_t *M, int size, int W, int16_t *out) {
    int seg = (Q + W - 1) / W;
    int t = 0;
    for (int nt = 0; nt < size; nt++)
        for (int i = 0; i < seg; i++, t++) {
            int j = i;
            for (int k = 0; k < W; k++, j += seg)
                out[t * W + k] = (int16_t)(j >= Q ? 0 : M[nt * size + q[j]]);
        }
}

void ish_o_sg_profile_i8(const uint8_t *q, int Q, const int8_t *M, int size, int W, int8_t *out) {
    int seg = (Q + W - 1) / W;
    int t = 0;
    for (int nt = 0; nt < size; nt++)
        for (int i = 0; i < seg; i++, t++) {
            int j = i;
            for (int k = 0; k < W; k++, j += seg)
                out[t * W + k] = (int8_t)(j >= Q ? 0 : M[nt * size + q[j]]);
        }
}

void ish_o_sw_profile_u8(const uint8_t *q, int Q, const int8_t *M, int size, int W, uint8_t bias,
                         uint8_t *out) {
    int seg = (Q + W - 1) / W;
    int t = 0;
    for (int nt = 0; nt < size; nt++)
        for (int i = 0; i < seg; i++, t++) {
            int j = i;
            for (int k = 0; k < W; k++, j += seg)
                out[t * W + k] =
                    j >= Q ? bias : (uint8_t)(int8_t)(M[nt * size + q[j]] + (int8_t)bias);
        }
}

void ish_o_sw_profile_u16(const uint8_t *q, int Q, const int8_t *M, int size, int W, uint8_t bias,
                          uint16_t *out) {
    int seg = (Q + W - 1) / W;
    int t = 0;
    for (int nt = 0; nt < size; nt++)
        for (int i = 0; i < seg; i++, t++) {
            int j = i;
            for (int k = 0; k < W; k++, j += seg)
                out[t * W + k] = (uint16_t)(
                    j >= Q ? bias : (uint8_t)(int8_t)(M[nt * size + q[j]] + (int8_t)bias));
        }
}

/* ------------------------------------------------------------------------ */
/* Saturating lane arithmetic: striped_utils.mojo:7-40 (llvm.*add.sat /     */
/* llvm.*sub.sat).                                                           */
/* ------------------------------------------------------------------------ */
#define O_CLAMP(x, lo, hi) ((x) < (lo) ? (lo) : ((x) > (hi) ? (hi) : (x)))
#define O_MAX(a, b) ((a) > (b) ? (a) : (b))

/* ------------------------------------------------------------------------ */
/* semi_global_aln (semi_global_aln/striped.mojo:252-498), do_saturation_    */
/* check=False as the matcher calls it (striped_semi_global_matcher.mojo:   */
/* 232).  TY is the lane type; every scalar expression of the reference that */
/* is evaluated in the lane type (boundary rows, lazy-F insert) wraps modulo */
/* 2^bits exactly like the Mojo SIMD scalars do.                             */
/* ------------------------------------------------------------------------ */
#define O_DEFINE_SG(NAME, TY, TMIN, TMAX)                                                      \
    static inline __attribute__((always_inline)) ish_o_end NAME##_impl(                       \
        const uint8_t *rec, int T, int Q, int open_i, int ext_i, const TY *prof, const int W, \
        int8_t max_s, int8_t min_s, int ends) {                                               \
        ish_o_end res = {0, 0, 0};                                                             \
        (void)max_s;                                                                           \
        if (Q == 0 || T == 0) return res; /* 275-276 */                                       \
        const int qs = ends & ISH_O_QS, qe = ends & ISH_O_QE;                                  \
        const int ts = ends & ISH_O_TS, te = ends & ISH_O_TE;                                  \
        const TY open = (TY)open_i, ext = (TY)ext_i;                                           \
        int end_query = Q - 1, end_ref = -1;                                                   \
        const int seg = (Q + W - 1) / W;                                                       \
        const int offset = (Q - 1) % seg;                                                      \
        const int position = (W - 1) - (Q - 1) / seg;                                          \
        const int mask_lane = (Q - 1) / seg; /* lane selected by v_pos_mask (285) */          \
        TY *hs = (TY *)calloc((size_t)seg * W, sizeof(TY));                                    \
        TY *hl = (TY *)calloc((size_t)seg * W, sizeof(TY));                                    \
        TY *pe = (TY *)calloc((size_t)seg * W, sizeof(TY));                                    \
        TY *bnd = (TY *)malloc(((size_t)T + 1) * sizeof(TY));                                  \
        /* Initial H and E (298-314). */                                                       \
        for (int i = 0; i < seg; i++)                                                          \
            for (int k = 0; k < W; k++) {                                                      \
                TY idx = (TY)(k * seg + i);                                                    \
                TY tmp = qs ? (TY)0 : (TY)(-(int64_t)open - (int64_t)ext * idx);               \
                hs[i * W + k] = tmp;                                                           \
                pe[i * W + k] = (TY)(tmp - open);                                              \
            }                                                                                  \
        /* Record-side boundary (316-324). */                                                  \
        bnd[0] = 0;                                                                            \
        for (int i = 1; i <= T; i++)                                                           \
            bnd[i] = ts ? (TY)0 : (TY)(-(int64_t)open - (int64_t)ext * (TY)(i - 1));           \
        TY neg; /* v_neg_limit (329-334) */                                                    \
        if ((TY)(-open) < (TY)min_s)                                                           \
            neg = (TY)(TMIN + open + 1);                                                       \
        else                                                                                   \
            neg = (TY)(TMIN - (TY)min_s + 1);                                                  \
        TY score = neg;                                                                        \
        TY vmaxh = neg; /* only the v_pos_mask lane of v_max_h is ever read */                \
        TY vf[ISH_O_MAXW], vh[ISH_O_MAXW], th[ISH_O_MAXW];                                     \
        for (int i = 0; i < T; i++) {                                                          \
            for (int k = 0; k < W; k++) vf[k] = neg;                                           \
            /* v_h = pv_h_store[seg-1].shift_right[1]() (352-353) */                           \
            vh[0] = 0;                                                                         \
            for (int k = 1; k < W; k++) vh[k] = hs[(seg - 1) * W + k - 1];                     \
            const TY *p = prof + (size_t)rec[i] * seg * W;                                     \
            TY *sw_tmp = hl; hl = hs; hs = sw_tmp; /* swap(load, store) (358) */             \
            vh[0] = bnd[i];                                                                    \
            for (int j = 0; j < seg; j++) { /* 364-394 */                                      \
                for (int k = 0; k < W; k++) {                                                  \
                    int32_t h = O_CLAMP((int32_t)vh[k] + p[j * W + k], TMIN, TMAX);            \
                    TY e = pe[j * W + k];                                                      \
                    h = O_MAX(h, e);                                                           \
                    h = O_MAX(h, vf[k]);                                                       \
                    hs[j * W + k] = (TY)h;                                                     \
                    int32_t hm = O_CLAMP(h - open, TMIN, TMAX);                                \
                    int32_t e2 = O_CLAMP((int32_t)e - ext, TMIN, TMAX);                        \
                    pe[j * W + k] = (TY)O_MAX(e2, hm);                                         \
                    int32_t f2 = O_CLAMP((int32_t)vf[k] - ext, TMIN, TMAX);                    \
                    vf[k] = (TY)O_MAX(f2, hm);                                                 \
                    vh[k] = hl[j * W + k];                                                     \
                }                                                                              \
            }                                                                                  \
            /* lazy_f (396-434) */                                                             \
            for (int kk = 0; kk < W; kk++) {                                                   \
                TY ins = ts ? (TY)(0 - open) : (TY)(bnd[i + 1] - open);                        \
                for (int k = W - 1; k > 0; k--) vf[k] = vf[k - 1];                             \
                vf[0] = ins;                                                                   \
                for (int j = 0; j < seg; j++) {                                                \
                    int any = 0;                                                               \
                    for (int k = 0; k < W; k++) {                                              \
                        TY h = O_MAX(hs[j * W + k], vf[k]);                                    \
                        hs[j * W + k] = h;                                                     \
                        th[k] = (TY)O_CLAMP((int32_t)h - open, TMIN, TMAX);                    \
                        vf[k] = (TY)O_CLAMP((int32_t)vf[k] - ext, TMIN, TMAX);                 \
                        any |= vf[k] > th[k];                                                  \
                    }                                                                          \
                    if (!any) goto lazy_done;                                                  \
                }                                                                              \
            }                                                                                  \
        lazy_done:;                                                                            \
            /* last query row tracking (436-441) */                                            \
            TY last = hs[offset * W + mask_lane];                                              \
            if (last > vmaxh) end_ref = i;                                                     \
            vmaxh = O_MAX(last, vmaxh);                                                        \
        }                                                                                      \
        (void)position;                                                                        \
        if (te) { /* 446-450: lane (Q-1)/seg of v_max_h after `position` shifts */            \
            score = vmaxh;                                                                     \
            end_query = Q - 1;                                                                 \
        }                                                                                      \
        if (qe) { /* 453-468 */                                                                \
            for (int i = 0; i < seg; i++)                                                      \
                for (int j = 0; j < W; j++) {                                                  \
                    int temp = i + j * seg;                                                    \
                    if (temp >= Q) continue;                                                   \
                    TY v = hs[i * W + j];                                                      \
                    if (v > score) {                                                           \
                        score = v;                                                             \
                        end_query = temp;                                                      \
                        end_ref = T - 1;                                                       \
                    } else if (v == score && end_ref == T - 1 && temp < end_query) {           \
                        end_query = temp;                                                      \
                    }                                                                          \
                }                                                                              \
        }                                                                                      \
        if (!te && !qe) { /* 471-477 */                                                        \
            score = hs[offset * W + mask_lane];                                                \
            end_ref = T - 1;                                                                   \
            end_query = Q - 1;                                                                 \
        }                                                                                      \
        free(hs); free(hl); free(pe); free(bnd);                                               \
        res.score = score;                                                                     \
        res.reference = end_ref;                                                               \
        res.query = end_query;                                                                 \
        return res;                                                                            \
    }

O_DEFINE_SG(o_sg_i16, int16_t, -32768, 32767)
O_DEFINE_SG(o_sg_i8, int8_t, -128, 127)

static int o_use_vectors = 1;
void ish_o_set_vectors(int on) { o_use_vectors = on; }
int ish_o_vectors(void) { return o_use_vectors && ish_o_neon_available(); }

ish_o_end ish_o_sg_aln_i16(const uint8_t *rec, int T, int Q, int open, int ext, const int16_t *prof,
                           int W, int8_t max_s, int8_t min_s, int ends) {
#if defined(__aarch64__) && !defined(ISH_O_NO_NEON)
    if (W == 8 && o_use_vectors) return ish_o_neon_sg_i16(rec, T, Q, open, ext, prof, max_s, min_s, ends);
#endif
    switch (W) {
    case 8: return o_sg_i16_impl(rec, T, Q, open, ext, prof, 8, max_s, min_s, ends);
    case 16: return o_sg_i16_impl(rec, T, Q, open, ext, prof, 16, max_s, min_s, ends);
    default: return o_sg_i16_impl(rec, T, Q, open, ext, prof, W, max_s, min_s, ends);
    }
}

ish_o_end ish_o_sg_aln_i8(const uint8_t *rec, int T, int Q, int open, int ext, const int8_t *prof,
                          int W, int8_t max_s, int8_t min_s, int ends) {
    switch (W) {
    case 16: return o_sg_i8_impl(rec, T, Q, open, ext, prof, 16, max_s, min_s, ends);
    default: return o_sg_i8_impl(rec, T, Q, open, ext, prof, W, max_s, min_s, ends);
    }
}

/* semi_global_aln_start_end (striped.mojo:121-191). */
int ish_o_sg_start_end_i16(const uint8_t *rec, int T, int Q, int open, int ext, const int16_t *prof,
                           const int16_t *rprof, int W, int8_t max_s, int8_t min_s, int ends,
                           float cutoff, ish_o_start_end *out) {
    ish_o_end fwd = ish_o_sg_aln_i16(rec, T, Q, open, ext, prof, W, max_s, min_s, ends);
    if ((float)fwd.score < cutoff) return 0; /* 157-158 */
    int rlen = fwd.reference + 1;            /* reference[0 : end + 1]; the slice clamps to T */
    if (rlen < 0) rlen = 0;
    if (rlen > T) rlen = T;
    uint8_t *rev = (uint8_t *)malloc(rlen > 0 ? (size_t)rlen : 1);
    for (int i = 0; i < rlen; i++) rev[i] = rec[rlen - 1 - i];
    /* swapped free ends (178-182) */
    int sw_ends = ((ends & ISH_O_QE) ? ISH_O_QS : 0) | ((ends & ISH_O_QS) ? ISH_O_QE : 0) |
                  ((ends & ISH_O_TE) ? ISH_O_TS : 0) | ((ends & ISH_O_TS) ? ISH_O_TE : 0);
    ish_o_end bwd = ish_o_sg_aln_i16(rev, rlen, Q, open, ext, rprof, W, max_s, min_s, sw_ends);
    free(rev);
    out->score = fwd.score;
    out->query_start = Q - bwd.query - 1;
    out->query_end = fwd.query;
    out->target_start = rlen - bwd.reference - 1;
    out->target_end = fwd.reference;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* sw (local_aln/striped.mojo:272-434).                                      */
/* ------------------------------------------------------------------------ */
#define O_DEFINE_SW(NAME, TY, TMAX)                                                             \
    static inline __attribute__((always_inline)) ish_o_end NAME##_impl(                        \
        const uint8_t *rec, int T, int reverse, int Q, TY open, TY ext, const TY *prof,        \
        const int W, TY terminate, TY bias) {                                                  \
        ish_o_end res;                                                                          \
        const int seg = (Q + W - 1) / W; /* ProfileVectors.__init__ (123-124) */             \
        TY *hs = (TY *)calloc((size_t)seg * W + 1, sizeof(TY));                                \
        TY *hl = (TY *)calloc((size_t)seg * W + 1, sizeof(TY));                                \
        TY *pe = (TY *)calloc((size_t)seg * W + 1, sizeof(TY));                                \
        TY *hm = (TY *)calloc((size_t)seg * W + 1, sizeof(TY));                                \
        TY max_score = 0;                                                                       \
        int end_query = Q - 1, end_ref = -1;                                                    \
        TY vmax_score[ISH_O_MAXW], vmax_mark[ISH_O_MAXW], vf[ISH_O_MAXW], vh[ISH_O_MAXW];        \
        TY vcol[ISH_O_MAXW], th[ISH_O_MAXW];                                                    \
        for (int k = 0; k < W; k++) vmax_score[k] = vmax_mark[k] = 0;                          \
        int begin = 0, end = T, step = 1;                                                       \
        if (reverse) { begin = T - 1; end = -1; step = -1; }                                    \
        int i = begin;                                                                          \
        while (i != end) {                                                                      \
            for (int k = 0; k < W; k++) { vf[k] = 0; vcol[k] = 0; }                             \
            vh[0] = 0;                                                                          \
            for (int k = 1; k < W; k++) vh[k] = hs[(seg - 1) * W + k - 1];                      \
            const TY *p = prof + (size_t)rec[i] * seg * W;                                      \
            TY *sw_tmp = hl; hl = hs; hs = sw_tmp;                                              \
            for (int j = 0; j < seg; j++) { /* 346-371 */                                       \
                for (int k = 0; k < W; k++) {                                                   \
                    int32_t h = O_CLAMP((int32_t)vh[k] + p[j * W + k], 0, TMAX);                \
                    h = O_CLAMP(h - (int32_t)bias, 0, TMAX);                                    \
                    TY e = pe[j * W + k];                                                       \
                    h = O_MAX(h, e);                                                            \
                    h = O_MAX(h, vf[k]);                                                        \
                    vcol[k] = (TY)O_MAX(vcol[k], h);                                            \
                    hs[j * W + k] = (TY)h;                                                      \
                    int32_t hm2 = O_CLAMP(h - (int32_t)open, 0, TMAX);                          \
                    int32_t e2 = O_CLAMP((int32_t)e - ext, 0, TMAX);                            \
                    pe[j * W + k] = (TY)O_MAX(e2, hm2);                                         \
                    int32_t f2 = O_CLAMP((int32_t)vf[k] - ext, 0, TMAX);                        \
                    vf[k] = (TY)O_MAX(f2, hm2);                                                 \
                    vh[k] = hl[j * W + k];                                                      \
                }                                                                               \
            }                                                                                   \
            /* lazy_f (374-393) */                                                              \
            for (int kk = 0; kk < W; kk++) {                                                    \
                for (int k = W - 1; k > 0; k--) vf[k] = vf[k - 1];                              \
                vf[0] = 0;                                                                      \
                int stop = 0;                                                                   \
                for (int j = 0; j < seg; j++) {                                                 \
                    int any = 0;                                                                \
                    for (int k = 0; k < W; k++) {                                               \
                        TY h = O_MAX(hs[j * W + k], vf[k]);                                     \
                        vcol[k] = O_MAX(vcol[k], h);                                            \
                        hs[j * W + k] = h;                                                      \
                        th[k] = (TY)O_CLAMP((int32_t)h - (int32_t)open, 0, TMAX);               \
                        vf[k] = (TY)O_CLAMP((int32_t)vf[k] - (int32_t)ext, 0, TMAX);            \
                        any |= vf[k] > th[k];                                                   \
                    }                                                                           \
                    if (!any) { stop = 1; break; }                                              \
                }                                                                               \
                if (stop) break;                                                                \
            }                                                                                   \
            /* new max check (395-411) */                                                       \
            int all_eq = 1;                                                                     \
            for (int k = 0; k < W; k++) {                                                       \
                vmax_score[k] = O_MAX(vmax_score[k], vcol[k]);                                  \
                all_eq &= vmax_mark[k] == vmax_score[k];                                        \
            }                                                                                   \
            if (!all_eq) {                                                                      \
                TY temp = 0;                                                                    \
                for (int k = 0; k < W; k++) {                                                   \
                    temp = O_MAX(temp, vmax_score[k]);                                          \
                    vmax_mark[k] = vmax_score[k];                                               \
                }                                                                               \
                if (temp > max_score) {                                                         \
                    max_score = temp;                                                           \
                    if ((TY)(max_score + bias) >= (TY)TMAX) break;                              \
                    end_ref = i;                                                                \
                    memcpy(hm, hs, (size_t)seg * W * sizeof(TY));                               \
                }                                                                               \
            }                                                                                   \
            TY colmax = 0; /* 414-416 */                                                        \
            for (int k = 0; k < W; k++) colmax = O_MAX(colmax, vcol[k]);                        \
            if (colmax >= terminate) break;                                                     \
            i += step;                                                                          \
        }                                                                                       \
        for (int s = 0; s < seg; s++) /* 423-428 */                                             \
            for (int k = 0; k < W; k++)                                                         \
                if (hm[s * W + k] == max_score) {                                               \
                    int temp = s + k * seg;                                                     \
                    if (temp < end_query) end_query = temp;                                     \
                }                                                                               \
        free(hs); free(hl); free(pe); free(hm);                                                 \
        res.score = max_score;                                                                  \
        res.reference = end_ref;                                                                \
        res.query = end_query;                                                                  \
        return res;                                                                             \
    }

O_DEFINE_SW(o_sw_u8, uint8_t, 255)
O_DEFINE_SW(o_sw_u16, uint16_t, 65535)

ish_o_end ish_o_sw_u8(const uint8_t *rec, int T, int reverse, int Q, uint8_t open, uint8_t ext,
                      const uint8_t *prof, int W, uint8_t terminate, uint8_t bias) {
#if defined(__aarch64__) && !defined(ISH_O_NO_NEON)
    if (W == 16 && o_use_vectors) return ish_o_neon_sw_u8(rec, T, reverse, Q, open, ext, prof, terminate, bias);
#endif
    if (W == 16) return o_sw_u8_impl(rec, T, reverse, Q, open, ext, prof, 16, terminate, bias);
    return o_sw_u8_impl(rec, T, reverse, Q, open, ext, prof, W, terminate, bias);
}

ish_o_end ish_o_sw_u16(const uint8_t *rec, int T, int reverse, int Q, uint16_t open, uint16_t ext,
                       const uint16_t *prof, int W, uint16_t terminate, uint16_t bias) {
#if defined(__aarch64__) && !defined(ISH_O_NO_NEON)
    if (W == 8 && o_use_vectors) return ish_o_neon_sw_u16(rec, T, reverse, Q, open, ext, prof, terminate, bias);
#endif
    if (W == 8) return o_sw_u16_impl(rec, T, reverse, Q, open, ext, prof, 8, terminate, bias);
    return o_sw_u16_impl(rec, T, reverse, Q, open, ext, prof, W, terminate, bias);
}

/* ssw_align (local_aln/striped.mojo:142-269) with ScoreSize.Adaptive. */
int ish_o_ssw_align(const uint8_t *rec, int T, int Q, const uint8_t *prof8, const uint16_t *prof16,
                    const uint8_t *rprof8, const uint16_t *rprof16, int W8, int W16, uint8_t bias,
                    uint8_t open, uint8_t ext, float cutoff, ish_o_alignment *out) {
    ish_o_end b = ish_o_sw_u8(rec, T, 0, Q, open, ext, prof8, W8, (uint8_t)255, bias);
    int used_word = 0;
    if (b.score + (int32_t)bias >= 255) { /* 174-189 */
        b = ish_o_sw_u16(rec, T, 0, Q, open, ext, prof16, W16, (uint16_t)65535, bias);
        used_word = 1;
    }
    if ((float)b.score <= cutoff) return 0; /* 215-217 */
    out->score1 = b.score;
    out->ref_end1 = b.reference;
    out->read_end1 = b.query;
    out->used_word = used_word;
    if (b.reference <= 0 || b.query <= 0) { /* 223-230 */
        out->ref_begin1 = -1;
        out->read_begin1 = -1;
        return 1;
    }
    ish_o_end r; /* 233-258 */
    if (!used_word)
        r = ish_o_sw_u8(rec, b.reference + 1, 1, Q, open, ext, rprof8, W8, (uint8_t)255, bias);
    else
        r = ish_o_sw_u16(rec, b.reference + 1, 1, Q, open, ext, rprof16, W16, (uint16_t)65535,
                         bias);
    out->ref_begin1 = r.reference;
    out->read_begin1 = b.query - r.query;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Matchers.                                                                 */
/* ------------------------------------------------------------------------ */
struct ish_o_matcher {
    int algo, kind, Q, ends, w_sg, w_u8, w_u16, size;
    int open, ext;
    int32_t max_score;
    float thr;
    const int8_t *M;
    uint8_t *q, *rq;
    int8_t mmin, mmax;
    uint8_t bias;
    int16_t *sg, *rsg;
    uint8_t *p8, *rp8;
    uint16_t *p16, *rp16;
};

ish_o_matcher *ish_o_matcher_new(int algo, int kind, const uint8_t *enc, int Q, int32_t max_score,
                                 float thr, int gap_open, int gap_extend, int ends, int w_sg,
                                 int w_u8, int w_u16) {
    const uint8_t *a2c, *c2a;
    ish_o_matcher *m = (ish_o_matcher *)calloc(1, sizeof(*m));
    m->algo = algo;
    m->kind = kind;
    m->Q = Q;
    m->ends = ends;
    m->w_sg = w_sg;
    m->w_u8 = w_u8;
    m->w_u16 = w_u16;
    m->max_score = max_score;
    m->thr = thr;
    m->size = ish_o_matrix(kind, &m->M, &a2c, &c2a);
    m->q = (uint8_t *)malloc(Q + 1);
    m->rq = (uint8_t *)malloc(Q + 1);
    memcpy(m->q, enc, Q);
    for (int i = 0; i < Q; i++) m->rq[i] = enc[Q - 1 - i]; /* create_reversed */
    ish_o_matrix_minmax(m->M, m->size, &m->mmin, &m->mmax);
    if (algo == ISH_O_SEMI_GLOBAL) {
        /* Matcher arguments are UInt; the int16 path truncates them. */
        m->open = (int16_t)gap_open;
        m->ext = (int16_t)gap_extend;
        int seg = (Q + w_sg - 1) / w_sg;
        size_t n = (size_t)m->size * (seg ? seg : 1) * w_sg;
        m->sg = (int16_t *)calloc(n, sizeof(int16_t));
        m->rsg = (int16_t *)calloc(n, sizeof(int16_t));
        ish_o_sg_profile_i16(m->q, Q, m->M, m->size, w_sg, m->sg);
        ish_o_sg_profile_i16(m->rq, Q, m->M, m->size, w_sg, m->rsg);
    } else {
        /* ssw_align takes UInt8 gap penalties. */
        m->open = (uint8_t)gap_open;
        m->ext = (uint8_t)gap_extend;
        m->bias = ish_o_sw_bias(m->M, m->size);
        int s8 = (Q + w_u8 - 1) / w_u8, s16 = (Q + w_u16 - 1) / w_u16;
        size_t n8 = (size_t)m->size * (s8 ? s8 : 1) * w_u8;
        size_t n16 = (size_t)m->size * (s16 ? s16 : 1) * w_u16;
        m->p8 = (uint8_t *)calloc(n8, 1);
        m->rp8 = (uint8_t *)calloc(n8, 1);
        m->p16 = (uint16_t *)calloc(n16, 2);
        m->rp16 = (uint16_t *)calloc(n16, 2);
        ish_o_sw_profile_u8(m->q, Q, m->M, m->size, w_u8, m->bias, m->p8);
        ish_o_sw_profile_u8(m->rq, Q, m->M, m->size, w_u8, m->bias, m->rp8);
        ish_o_sw_profile_u16(m->q, Q, m->M, m->size, w_u16, m->bias, m->p16);
        ish_o_sw_profile_u16(m->rq, Q, m->M, m->size, w_u16, m->bias, m->rp16);
    }
    return m;
}

void ish_o_matcher_free(ish_o_matcher *m) {
    if (!m) return;
    free(m->q); free(m->rq); free(m->sg); free(m->rsg);
    free(m->p8); free(m->rp8); free(m->p16); free(m->rp16);
    free(m);
}

ish_o_end ish_o_matcher_forward(const ish_o_matcher *m, const uint8_t *rec, int T) {
    if (m->algo == ISH_O_SEMI_GLOBAL)
        return ish_o_sg_aln_i16(rec, T, m->Q, m->open, m->ext, m->sg, m->w_sg, m->mmax, m->mmin,
                                m->ends);
    ish_o_end b = ish_o_sw_u8(rec, T, 0, m->Q, (uint8_t)m->open, (uint8_t)m->ext, m->p8, m->w_u8,
                              (uint8_t)255, m->bias);
    if (b.score + (int32_t)m->bias >= 255)
        b = ish_o_sw_u16(rec, T, 0, m->Q, (uint16_t)(uint8_t)m->open, (uint16_t)(uint8_t)m->ext,
                         m->p16, m->w_u16, (uint16_t)65535, m->bias);
    return b;
}

int ish_o_matcher_first_match(const ish_o_matcher *m, const uint8_t *rec, int T, int64_t *start,
                              int64_t *end) {
    float maxf = (float)m->max_score;
    if (m->algo == ISH_O_SEMI_GLOBAL) {
        /* striped_semi_global_matcher.mojo:227-257 */
        float cutoff = maxf * m->thr;
        ish_o_start_end r;
        if (!ish_o_sg_start_end_i16(rec, T, m->Q, m->open, m->ext, m->sg, m->rsg, m->w_sg, m->mmax,
                                    m->mmin, m->ends, cutoff, &r))
            return 0;
        if (!((float)r.score / maxf >= m->thr)) return 0;
        *start = r.target_start;
        *end = (int64_t)r.target_end + 1;
        return 1;
    }
    /* striped_local_matcher.mojo:61-90 */
    float cutoff = m->thr * maxf;
    ish_o_alignment a;
    if (!ish_o_ssw_align(rec, T, m->Q, m->p8, m->p16, m->rp8, m->rp16, m->w_u8, m->w_u16, m->bias,
                         (uint8_t)m->open, (uint8_t)m->ext, cutoff, &a))
        return 0;
    if (!(a.ref_begin1 >= 0 && a.ref_end1 >= 0 && (float)a.score1 / maxf >= m->thr)) return 0;
    *start = a.ref_begin1;
    *end = (int64_t)a.ref_end1 + 1;
    return 1;
}

int64_t ish_o_sg_find_start(const ish_o_matcher *m, const uint8_t *rec, int n) {
    /* striped_semi_global_matcher.mojo:259-276 */
    uint8_t *rev = (uint8_t *)malloc(n > 0 ? (size_t)n : 1);
    for (int i = 0; i < n; i++) rev[i] = rec[n - 1 - i];
    int e = m->ends;
    int sw_ends = ((e & ISH_O_QE) ? ISH_O_QS : 0) | ((e & ISH_O_QS) ? ISH_O_QE : 0) |
                  ((e & ISH_O_TE) ? ISH_O_TS : 0) | ((e & ISH_O_TS) ? ISH_O_TE : 0);
    ish_o_end r = ish_o_sg_aln_i16(rev, n, m->Q, m->open, m->ext, m->rsg, m->w_sg, m->mmax,
                                   m->mmin, sw_ends);
    free(rev);
    return (int64_t)n - r.reference - 1;
}

void ish_o_matcher_batch(const ish_o_matcher *m, const uint8_t *recs, const uint64_t *off,
                         int64_t n, int threads, int32_t *score, int32_t *qend, int32_t *tend,
                         uint8_t *hit, int64_t *mstart, int64_t *mend) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads > 0 ? threads : 1)
    for (int64_t i = 0; i < n; i++) {
        const uint8_t *r = recs + off[i];
        int T = (int)(off[i + 1] - off[i]);
        if (score || qend || tend) {
            ish_o_end f = ish_o_matcher_forward(m, r, T);
            if (score) score[i] = f.score;
            if (qend) qend[i] = f.query;
            if (tend) tend[i] = f.reference;
        }
        if (hit || mstart || mend) {
            int64_t s = -1, e = -1;
            int h = ish_o_matcher_first_match(m, r, T, &s, &e);
            if (hit) hit[i] = (uint8_t)h;
            if (mstart) mstart[i] = h ? s : -1;
            if (mend) mend[i] = h ? e : -1;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Equivalence model: the striped semi-global / local passes restated as a   */
/* per-cell recurrence over the query in natural order.  Exact integers (no  */
/* saturation), valid while no lane value of the striped pass saturates and  */
/* gap_open > gap_extend (then lazy-F's early exit never skips an update).    */
/*                                                                            */
/* Per record row i and query position q = l*seg + j (lane l, stripe slot j): */
/*   Hd  = Hprev[q-1] + P[rec[i]][q]           (Hprev[-1] = boundary[i])      */
/*   Fp  = neg_limit at j == 0, else the in-stripe F chain                     */
/*   H1  = max(Hd, E[q], Fp)                                                   */
/*   v   = H1 - open;  E[q] = max(E[q] - ext, v);  Fp' = max(Fp - ext, v)      */
/*   X_l = F chain entering lane l from lanes < l (lazy-F), decays by ext      */
/*   H   = max(H1, X_l - j*ext)                                                */
/* E never sees X: the reference's lazy-F loop does not update E.             */
/* ------------------------------------------------------------------------ */
ish_o_end ish_o_sg_model(const uint8_t *rec, int T, const uint8_t *q, int Q, const int8_t *M,
                         int size, int open, int ext, int W, int ends) {
    ish_o_end res = {0, 0, 0};
    if (Q == 0 || T == 0) return res;
    const int qs = ends & ISH_O_QS, qe = ends & ISH_O_QE, ts = ends & ISH_O_TS,
              te = ends & ISH_O_TE;
    int8_t mn, mx;
    ish_o_matrix_minmax(M, size, &mn, &mx);
    const int seg = (Q + W - 1) / W;
    const int nl = (Q + seg - 1) / seg; /* lanes holding real positions */
    const int neg = (-open < mn) ? (-32768 + open + 1) : (-32768 - mn + 1);
    int64_t *H = (int64_t *)malloc(sizeof(int64_t) * Q);
    int64_t *H1 = (int64_t *)malloc(sizeof(int64_t) * Q);
    int64_t *E = (int64_t *)malloc(sizeof(int64_t) * Q);
    int64_t Fo[ISH_O_MAXW], X[ISH_O_MAXW];
    for (int p = 0; p < Q; p++) {
        H[p] = qs ? 0 : -(int64_t)open - (int64_t)ext * p;
        E[p] = H[p] - open;
    }
    int64_t best = neg;
    int end_ref = -1, end_query = Q - 1;
    for (int i = 0; i < T; i++) {
        int64_t Bi = (i == 0 || ts) ? 0 : -(int64_t)open - (int64_t)ext * (i - 1);
        int64_t Bn = ts ? 0 : -(int64_t)open - (int64_t)ext * i;
        int64_t hdiag = Bi, Fp = neg;
        for (int p = 0; p < Q; p++) {
            int j = p % seg, l = p / seg;
            if (j == 0) Fp = neg;
            int64_t hd = hdiag + M[rec[i] * size + q[p]];
            hdiag = H[p];
            int64_t u = hd > Fp ? hd : Fp;
            if (E[p] > u) u = E[p];
            int64_t v = u - open;
            E[p] = (E[p] - ext) > v ? (E[p] - ext) : v;
            Fp = (Fp - ext) > v ? (Fp - ext) : v;
            H1[p] = u;
            if (j == seg - 1) Fo[l] = Fp;
        }
        X[0] = Bn - open;
        for (int l = 1; l < nl; l++) {
            int64_t d = X[l - 1] - (int64_t)seg * ext;
            X[l] = Fo[l - 1] > d ? Fo[l - 1] : d;
        }
        for (int p = 0; p < Q; p++) {
            int64_t x = X[p / seg] - (int64_t)(p % seg) * ext;
            H[p] = H1[p] > x ? H1[p] : x;
        }
        if (H[Q - 1] > best) {
            best = H[Q - 1];
            end_ref = i;
        }
    }
    int64_t score = neg;
    if (te) score = best;
    if (qe) {
        /* Scan order of the striped epilogue: slot-major, lane-minor. */
        for (int s = 0; s < seg; s++)
            for (int l = 0; l < W; l++) {
                int t = s + l * seg;
                if (t >= Q) continue;
                if (H[t] > score) {
                    score = H[t];
                    end_query = t;
                    end_ref = T - 1;
                } else if (H[t] == score && end_ref == T - 1 && t < end_query) {
                    end_query = t;
                }
            }
    }
    if (!te && !qe) {
        score = H[Q - 1];
        end_ref = T - 1;
        end_query = Q - 1;
    }
    free(H); free(H1); free(E);
    res.score = (int32_t)score;
    res.reference = end_ref;
    res.query = end_query;
    return res;
}

ish_o_end ish_o_sw_model(const uint8_t *rec, int T, const uint8_t *q, int Q, const int8_t *M,
                         int size, int open, int ext, int W) {
    ish_o_end res;
    const int seg = (Q + W - 1) / W;
    const int nl = (Q + seg - 1) / seg;
    int64_t *H = (int64_t *)calloc(Q + 1, sizeof(int64_t));
    int64_t *H1 = (int64_t *)calloc(Q + 1, sizeof(int64_t));
    int64_t *E = (int64_t *)calloc(Q + 1, sizeof(int64_t));
    int64_t *Hb = (int64_t *)calloc(Q + 1, sizeof(int64_t));
    int64_t Fo[ISH_O_MAXW], X[ISH_O_MAXW];
    int64_t best = 0;
    int end_ref = -1;
    for (int i = 0; i < T; i++) {
        int64_t hdiag = 0, Fp = 0, col = 0;
        for (int p = 0; p < Q; p++) {
            int j = p % seg, l = p / seg;
            if (j == 0) Fp = 0;
            int64_t hd = hdiag + M[rec[i] * size + q[p]];
            if (hd < 0) hd = 0;
            hdiag = H[p];
            int64_t u = hd > Fp ? hd : Fp;
            if (E[p] > u) u = E[p];
            int64_t v = u - open > 0 ? u - open : 0;
            int64_t e2 = E[p] - ext > 0 ? E[p] - ext : 0;
            E[p] = e2 > v ? e2 : v;
            int64_t f2 = Fp - ext > 0 ? Fp - ext : 0;
            Fp = f2 > v ? f2 : v;
            H1[p] = u;
            if (j == seg - 1) Fo[l] = Fp;
        }
        X[0] = 0;
        for (int l = 1; l < nl; l++) {
            int64_t d = X[l - 1] - (int64_t)seg * ext;
            if (d < 0) d = 0;
            X[l] = Fo[l - 1] > d ? Fo[l - 1] : d;
        }
        for (int p = 0; p < Q; p++) {
            int64_t x = X[p / seg] - (int64_t)(p % seg) * ext;
            H[p] = H1[p] > x ? H1[p] : x;
            if (H[p] > col) col = H[p];
        }
        if (col > best) {
            best = col;
            end_ref = i;
            memcpy(Hb, H, sizeof(int64_t) * Q);
        }
    }
    int end_query = Q - 1;
    for (int p = 0; p < Q; p++)
        if (Hb[p] == best && p < end_query) {
            end_query = p;
            break;
        }
    if (best == 0) end_query = 0;
    free(H); free(H1); free(E); free(Hb);
    res.score = (int32_t)best;
    res.reference = end_ref;
    res.query = end_query;
    return res;
}
