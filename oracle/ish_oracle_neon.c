/* CPU oracle: the striped passes of the reference on 128-bit NEON vectors.
 *
 * TEST INFRASTRUCTURE ONLY (the timed CPU baseline of bench.py and a checker).
 *
 * The reference runs its striped passes on SIMD[int16, 8] / SIMD[uint8, 16] /
 * SIMD[uint16, 8] vectors, which a Grace host executes as 128-bit NEON with
 * saturating adds and subtracts in one instruction each.  The scalar lane
 * loops of ish_oracle.c restate the same arithmetic lane by lane; this file
 * restates it vector by vector for the reference's own lane counts (W = 8
 * int16, 16 uint8, 8 uint16), so that the CPU baseline runs the
 * instruction mix ish runs on the same host.  Results are identical to the
 * lane loops (tests/test_oracle_neon.py compares them on the GPU machine, the
 * aarch64 host this compiles for).  Elsewhere the file is empty.
 *
 *   semi_global_aln: ishlib/matcher/alignment/semi_global_aln/striped.mojo:252-498
 *   sw:              ishlib/matcher/alignment/local_aln/striped.mojo:272-434
 */
#include "ish_oracle.h"

#if defined(__aarch64__) && !defined(ISH_O_NO_NEON)
#include <arm_neon.h>
#include <stdlib.h>
#include <string.h>

/* shift lanes up by one, lane 0 = x (the reference's shift_right[1] + insert) */
static inline int16x8_t sh_in_s16(int16x8_t v, int16_t x) { return vextq_s16(vdupq_n_s16(x), v, 7); }
static inline uint8x16_t sh_in_u8(uint8x16_t v, uint8_t x) { return vextq_u8(vdupq_n_u8(x), v, 15); }
static inline uint16x8_t sh_in_u16(uint16x8_t v, uint16_t x) { return vextq_u16(vdupq_n_u16(x), v, 7); }

/* semi_global_aln[int16, 8] (striped.mojo:252-498), as ish_o_sg_aln_i16 with W = 8. */
ish_o_end ish_o_neon_sg_i16(const uint8_t *rec, int T, int Q, int open_i, int ext_i, const int16_t *prof,
                            int8_t max_s, int8_t min_s, int ends) {
    enum { W = 8 };
    ish_o_end res = {0, 0, 0};
    (void)max_s;
    if (Q == 0 || T == 0) return res;
    const int qs = ends & ISH_O_QS, qe = ends & ISH_O_QE;
    const int ts = ends & ISH_O_TS, te = ends & ISH_O_TE;
    const int16_t open = (int16_t)open_i, ext = (int16_t)ext_i;
    int end_query = Q - 1, end_ref = -1;
    const int seg = (Q + W - 1) / W;
    const int offset = (Q - 1) % seg;
    const int mask_lane = (Q - 1) / seg;
    int16_t *hs = (int16_t *)calloc((size_t)seg * W, sizeof(int16_t));
    int16_t *hl = (int16_t *)calloc((size_t)seg * W, sizeof(int16_t));
    int16_t *pe = (int16_t *)calloc((size_t)seg * W, sizeof(int16_t));
    int16_t *bnd = (int16_t *)malloc(((size_t)T + 1) * sizeof(int16_t));
    for (int i = 0; i < seg; i++)
        for (int k = 0; k < W; k++) {
            int16_t idx = (int16_t)(k * seg + i);
            int16_t tmp = qs ? (int16_t)0 : (int16_t)(-(int64_t)open - (int64_t)ext * idx);
            hs[i * W + k] = tmp;
            pe[i * W + k] = (int16_t)(tmp - open);
        }
    bnd[0] = 0;
    for (int i = 1; i <= T; i++) bnd[i] = ts ? (int16_t)0 : (int16_t)(-(int64_t)open - (int64_t)ext * (int16_t)(i - 1));
    int16_t neg;
    if ((int16_t)(-open) < (int16_t)min_s)
        neg = (int16_t)(-32768 + open + 1);
    else
        neg = (int16_t)(-32768 - (int16_t)min_s + 1);
    int16_t vmaxh = neg;
    const int16x8_t vopen = vdupq_n_s16(open), vext = vdupq_n_s16(ext), vneg = vdupq_n_s16(neg);
    for (int i = 0; i < T; i++) {
        int16x8_t vf = vneg;
        int16x8_t vh = sh_in_s16(vld1q_s16(hs + (size_t)(seg - 1) * W), bnd[i]);
        const int16_t *p = prof + (size_t)rec[i] * seg * W;
        int16_t *sw_tmp = hl;
        hl = hs;
        hs = sw_tmp;
        for (int j = 0; j < seg; j++) {
            int16x8_t h = vqaddq_s16(vh, vld1q_s16(p + (size_t)j * W));
            const int16x8_t e = vld1q_s16(pe + (size_t)j * W);
            h = vmaxq_s16(vmaxq_s16(h, e), vf);
            vst1q_s16(hs + (size_t)j * W, h);
            const int16x8_t hm = vqsubq_s16(h, vopen);
            vst1q_s16(pe + (size_t)j * W, vmaxq_s16(vqsubq_s16(e, vext), hm));
            vf = vmaxq_s16(vqsubq_s16(vf, vext), hm);
            vh = vld1q_s16(hl + (size_t)j * W);
        }
        for (int kk = 0; kk < W; kk++) { /* lazy_f (396-434) */
            const int16_t ins = ts ? (int16_t)(0 - open) : (int16_t)(bnd[i + 1] - open);
            vf = sh_in_s16(vf, ins);
            int stop = 0;
            for (int j = 0; j < seg; j++) {
                const int16x8_t h = vmaxq_s16(vld1q_s16(hs + (size_t)j * W), vf);
                vst1q_s16(hs + (size_t)j * W, h);
                const int16x8_t th = vqsubq_s16(h, vopen);
                vf = vqsubq_s16(vf, vext);
                if (vmaxvq_u16(vcgtq_s16(vf, th)) == 0) {
                    stop = 1;
                    break;
                }
            }
            if (stop) break;
        }
        const int16_t last = hs[offset * W + mask_lane]; /* 436-441 */
        if (last > vmaxh) end_ref = i;
        if (last > vmaxh) vmaxh = last;
    }
    int16_t score = neg;
    if (te) {
        score = vmaxh;
        end_query = Q - 1;
    }
    if (qe) { /* 453-468 */
        for (int i = 0; i < seg; i++)
            for (int j = 0; j < W; j++) {
                const int temp = i + j * seg;
                if (temp >= Q) continue;
                const int16_t v = hs[i * W + j];
                if (v > score) {
                    score = v;
                    end_query = temp;
                    end_ref = T - 1;
                } else if (v == score && end_ref == T - 1 && temp < end_query) {
                    end_query = temp;
                }
            }
    }
    if (!te && !qe) {
        score = hs[offset * W + mask_lane];
        end_ref = T - 1;
        end_query = Q - 1;
    }
    free(hs);
    free(hl);
    free(pe);
    free(bnd);
    res.score = score;
    res.reference = end_ref;
    res.query = end_query;
    return res;
}

/* sw (local_aln/striped.mojo:272-434) on NL-lane vectors of type TY: the
 * same steps as the lane loops of ish_oracle.c, one vector per stripe. */
#define O_NEON_SW(NAME, TY, VT, NL, TMAX, LD, ST, DUP, QADD, QSUB, MAX, CGT, MAXV, SHIN)                   \
    ish_o_end NAME(const uint8_t *rec, int T, int reverse, int Q, TY open, TY ext, const TY *prof,          \
                   TY terminate, TY bias) {                                                                \
        ish_o_end res;                                                                                      \
        const int W = NL;                                                                                   \
        const int seg = (Q + W - 1) / W;                                                                    \
        TY *hs = (TY *)calloc((size_t)seg * W + 1, sizeof(TY));                                            \
        TY *hl = (TY *)calloc((size_t)seg * W + 1, sizeof(TY));                                            \
        TY *pe = (TY *)calloc((size_t)seg * W + 1, sizeof(TY));                                            \
        TY *hmx = (TY *)calloc((size_t)seg * W + 1, sizeof(TY));                                           \
        TY max_score = 0;                                                                                   \
        int end_query = Q - 1, end_ref = -1;                                                                \
        VT vmax_score = DUP(0), vmax_mark = DUP(0);                                                         \
        const VT vopen = DUP(open), vext = DUP(ext), vbias = DUP(bias);                                     \
        int begin = 0, end = T, step = 1;                                                                   \
        if (reverse) {                                                                                      \
            begin = T - 1;                                                                                  \
            end = -1;                                                                                       \
            step = -1;                                                                                      \
        }                                                                                                   \
        int i = begin;                                                                                      \
        while (i != end) {                                                                                  \
            VT vf = DUP(0), vcol = DUP(0);                                                                  \
            VT vh = SHIN(LD(hs + (size_t)(seg - 1) * W), 0);                                                \
            const TY *p = prof + (size_t)rec[i] * seg * W;                                                  \
            TY *sw_tmp = hl;                                                                                \
            hl = hs;                                                                                        \
            hs = sw_tmp;                                                                                    \
            for (int j = 0; j < seg; j++) {                                                                 \
                VT h = QSUB(QADD(vh, LD(p + (size_t)j * W)), vbias);                                        \
                const VT e = LD(pe + (size_t)j * W);                                                        \
                h = MAX(MAX(h, e), vf);                                                                     \
                vcol = MAX(vcol, h);                                                                        \
                ST(hs + (size_t)j * W, h);                                                                  \
                const VT hm2 = QSUB(h, vopen);                                                              \
                ST(pe + (size_t)j * W, MAX(QSUB(e, vext), hm2));                                            \
                vf = MAX(QSUB(vf, vext), hm2);                                                              \
                vh = LD(hl + (size_t)j * W);                                                                \
            }                                                                                               \
            for (int kk = 0; kk < W; kk++) { /* lazy_f (374-393) */                                         \
                vf = SHIN(vf, 0);                                                                           \
                int stop = 0;                                                                               \
                for (int j = 0; j < seg; j++) {                                                             \
                    const VT h = MAX(LD(hs + (size_t)j * W), vf);                                           \
                    vcol = MAX(vcol, h);                                                                    \
                    ST(hs + (size_t)j * W, h);                                                              \
                    const VT th = QSUB(h, vopen);                                                           \
                    vf = QSUB(vf, vext);                                                                    \
                    if (MAXV(CGT(vf, th)) == 0) {                                                           \
                        stop = 1;                                                                           \
                        break;                                                                              \
                    }                                                                                       \
                }                                                                                           \
                if (stop) break;                                                                            \
            }                                                                                               \
            vmax_score = MAX(vmax_score, vcol); /* 395-411 */                                               \
            TY ms[NL], mk[NL];                                                                              \
            ST(ms, vmax_score);                                                                             \
            ST(mk, vmax_mark);                                                                              \
            if (memcmp(ms, mk, sizeof ms) != 0) {                                                           \
                const TY temp = (TY)MAXV(vmax_score);                                                       \
                vmax_mark = vmax_score;                                                                     \
                if (temp > max_score) {                                                                     \
                    max_score = temp;                                                                       \
                    if ((TY)(max_score + bias) >= (TY)TMAX) break;                                          \
                    end_ref = i;                                                                            \
                    memcpy(hmx, hs, (size_t)seg * W * sizeof(TY));                                          \
                }                                                                                           \
            }                                                                                               \
            if ((TY)MAXV(vcol) >= terminate) break; /* 414-416 */                                           \
            i += step;                                                                                      \
        }                                                                                                   \
        for (int s = 0; s < seg; s++) /* 423-428 */                                                         \
            for (int k = 0; k < W; k++)                                                                     \
                if (hmx[s * W + k] == max_score) {                                                          \
                    const int temp = s + k * seg;                                                           \
                    if (temp < end_query) end_query = temp;                                                 \
                }                                                                                           \
        free(hs);                                                                                           \
        free(hl);                                                                                           \
        free(pe);                                                                                           \
        free(hmx);                                                                                          \
        res.score = max_score;                                                                              \
        res.reference = end_ref;                                                                            \
        res.query = end_query;                                                                              \
        return res;                                                                                         \
    }

O_NEON_SW(ish_o_neon_sw_u8, uint8_t, uint8x16_t, 16, 255, vld1q_u8, vst1q_u8, vdupq_n_u8, vqaddq_u8, vqsubq_u8,
          vmaxq_u8, vcgtq_u8, vmaxvq_u8, sh_in_u8)
O_NEON_SW(ish_o_neon_sw_u16, uint16_t, uint16x8_t, 8, 65535, vld1q_u16, vst1q_u16, vdupq_n_u16, vqaddq_u16,
          vqsubq_u16, vmaxq_u16, vcgtq_u16, vmaxvq_u16, sh_in_u16)

int ish_o_neon_available(void) { return 1; }

#else

int ish_o_neon_available(void) { return 0; }

#endif
