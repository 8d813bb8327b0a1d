/*
 * ish_oracle.h -- CPU restatement of ish's striped alignment-scoring path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * path in ish_gb300/csrc and the timed CPU baseline of bench.py.  Nothing in
 * the product (libish_gpu.so, the ish_gb300 package) links, loads or calls it.
 *
 * Every function restates the reference algorithm line by line; the citations
 * are relative to the ish repository (Mojo sources, v1.4.0):
 *
 *   scoring matrices / encodings  ishlib/matcher/alignment/scoring_matrix.mojo
 *   striped semi-global           ishlib/matcher/alignment/semi_global_aln/striped.mojo
 *   striped local (SSW)           ishlib/matcher/alignment/local_aln/striped.mojo
 *   saturating lane ops           ishlib/matcher/alignment/striped_utils.mojo:7-40
 *   matcher decisions             ishlib/matcher/striped_semi_global_matcher.mojo:227-276
 *                                 ishlib/matcher/striped_local_matcher.mojo:61-90
 *   GPU-path epilogue             ishlib/cpu/process_batch.mojo:37-68
 *
 * "W" is the SIMD lane count of the reference build.  The reference picks it
 * with simd_width_of[dtype]() (ishlib/matcher/__init__.mojo:11-30), so a host
 * with 128-bit vectors (NEON on Grace, SSE) runs 8 x int16 / 16 x uint8 lanes.
 * The result of the striped algorithm depends on W in rare cases (an E gap is
 * never opened from an F gap that crossed a stripe boundary), which is why W is
 * an explicit argument everywhere.
 */
#ifndef ISH_ORACLE_H
#define ISH_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ISH_O_ASCII = 0, ISH_O_ACTGN = 1, ISH_O_ACTGN0 = 2, ISH_O_BLOSUM62 = 3 };
enum { ISH_O_SEMI_GLOBAL = 0, ISH_O_LOCAL = 1 };
/* ends-free bits: (query_start, query_end, target_start, target_end) */
enum { ISH_O_QS = 1, ISH_O_QE = 2, ISH_O_TS = 4, ISH_O_TE = 8 };

typedef struct {
    int32_t score;
    int32_t reference; /* 0-based inclusive end on the record, -1 if none */
    int32_t query;     /* 0-based inclusive end on the query */
} ish_o_end;

/* ---- matrices and encodings (scoring_matrix.mojo:9-172, 328-416) ---- */
/* Returns the edge length of the square matrix and points at its values,
 * the ascii->code table and the code->ascii table. */
int ish_o_matrix(int kind, const int8_t **values, const uint8_t **ascii_to_code,
                 const uint8_t **code_to_ascii);
/* convert_ascii_to_encoding_and_score: encodes `n` bytes into `out` and
 * returns the optimal score sum(M[c][c]). */
int32_t ish_o_encode_and_score(int kind, const uint8_t *ascii, size_t n, uint8_t *out);
void ish_o_encode(int kind, const uint8_t *ascii, size_t n, uint8_t *out);

/* ---- striped semi-global (semi_global_aln/striped.mojo) ---- */
/* Profile.generate_query_profile: out[(c*seg + i)*W + k] = M[c][q[i+k*seg]] or 0. */
void ish_o_sg_profile_i16(const uint8_t *q, int Q, const int8_t *M, int size, int W, int16_t *out);
void ish_o_sg_profile_i8(const uint8_t *q, int Q, const int8_t *M, int size, int W, int8_t *out);
void ish_o_matrix_minmax(const int8_t *M, int size, int8_t *mn, int8_t *mx);

/* semi_global_aln[int16, W, do_saturation_check=False] (striped.mojo:252-498) */
ish_o_end ish_o_sg_aln_i16(const uint8_t *rec, int T, int Q, int open, int ext,
                           const int16_t *prof, int W, int8_t max_s, int8_t min_s, int ends);
/* semi_global_aln[int8, W, do_saturation_check=False] */
ish_o_end ish_o_sg_aln_i8(const uint8_t *rec, int T, int Q, int open, int ext,
                          const int8_t *prof, int W, int8_t max_s, int8_t min_s, int ends);

typedef struct {
    int32_t score, query_start, query_end, target_start, target_end;
} ish_o_start_end;

/* semi_global_aln_start_end (striped.mojo:121-191): returns 1 and fills `out`
 * when the forward score passes `cutoff`, else 0. */
int ish_o_sg_start_end_i16(const uint8_t *rec, int T, int Q, int open, int ext,
                           const int16_t *prof, const int16_t *rprof, int W,
                           int8_t max_s, int8_t min_s, int ends, float cutoff,
                           ish_o_start_end *out);

/* ---- striped local (local_aln/striped.mojo) ---- */
void ish_o_sw_profile_u8(const uint8_t *q, int Q, const int8_t *M, int size, int W,
                         uint8_t bias, uint8_t *out);
void ish_o_sw_profile_u16(const uint8_t *q, int Q, const int8_t *M, int size, int W,
                          uint8_t bias, uint16_t *out);
uint8_t ish_o_sw_bias(const int8_t *M, int size);
/* sw[uint8, W] / sw[uint16, W] (local_aln/striped.mojo:272-434).  `reverse`
 * walks the record from its end; terminate is the type-cast value (-1 -> MAX). */
ish_o_end ish_o_sw_u8(const uint8_t *rec, int T, int reverse, int Q, uint8_t open,
                      uint8_t ext, const uint8_t *prof, int W, uint8_t terminate,
                      uint8_t bias);
ish_o_end ish_o_sw_u16(const uint8_t *rec, int T, int reverse, int Q, uint16_t open,
                       uint16_t ext, const uint16_t *prof, int W, uint16_t terminate,
                       uint16_t bias);

typedef struct {
    int32_t score1, ref_begin1, ref_end1, read_begin1, read_end1;
    int32_t used_word;
} ish_o_alignment;

/* ssw_align (local_aln/striped.mojo:142-269) with both profiles present
 * (ScoreSize.Adaptive).  Returns 1 and fills `out`, or 0 for None. */
int ish_o_ssw_align(const uint8_t *rec, int T, int Q,
                    const uint8_t *prof8, const uint16_t *prof16,
                    const uint8_t *rprof8, const uint16_t *rprof16,
                    int W8, int W16, uint8_t bias, uint8_t open, uint8_t ext,
                    float cutoff, ish_o_alignment *out);

/* ---- matchers ---- */
typedef struct ish_o_matcher ish_o_matcher;

/* StripedSemiGlobalMatcher / StripedLocalMatcher construction from an
 * already-encoded pattern.  w_sg: int16 lanes of the semi-global path,
 * w_u8 / w_u16: lanes of the local byte / word passes. */
ish_o_matcher *ish_o_matcher_new(int algo, int kind, const uint8_t *enc_pattern, int Q,
                                 int32_t max_score, float threshold, int gap_open,
                                 int gap_extend, int ends, int w_sg, int w_u8, int w_u16);
void ish_o_matcher_free(ish_o_matcher *m);

/* Forward pass exactly as the matcher runs it (semi_global_aln / the adaptive
 * u8->u16 sw of ssw_align): score and 0-based inclusive ends. */
ish_o_end ish_o_matcher_forward(const ish_o_matcher *m, const uint8_t *rec, int T);

/* first_match: returns 1 for a hit with [start, end) filled, else 0. */
int ish_o_matcher_first_match(const ish_o_matcher *m, const uint8_t *rec, int T,
                              int64_t *start, int64_t *end);

/* StripedSemiGlobalMatcher.find_start on haystack[0:end_exclusive]. */
int64_t ish_o_sg_find_start(const ish_o_matcher *m, const uint8_t *rec, int end_exclusive);

/* Batch over records rec[off[i]:off[i+1]] with `threads` OpenMP threads.
 * Any output pointer may be NULL.  hit[i] is 1 for first_match hits. */
void ish_o_matcher_batch(const ish_o_matcher *m, const uint8_t *recs, const uint64_t *off,
                         int64_t n, int threads, int32_t *score, int32_t *qend,
                         int32_t *tend, uint8_t *hit, int64_t *mstart, int64_t *mend);

/* ---- equivalence model ----
 * A sequential (non-striped) statement of what the striped semi-global pass
 * computes, cell by cell, in exact integer arithmetic.  It is the recurrence
 * the CUDA kernels implement; tests check it against ish_o_sg_aln_i16. */
ish_o_end ish_o_sg_model(const uint8_t *rec, int T, const uint8_t *q, int Q, const int8_t *M,
                         int size, int open, int ext, int W, int ends);
ish_o_end ish_o_sw_model(const uint8_t *rec, int T, const uint8_t *q, int Q, const int8_t *M,
                         int size, int open, int ext, int W);

/* ---- vector passes (ish_oracle_neon.c) ----
 * On an aarch64 host the striped passes at the reference's own lane counts
 * (semi-global int16 x 8, local uint8 x 16 and uint16 x 8) run on NEON
 * vectors, as the reference runs them there; ish_o_set_vectors(0) selects the
 * lane loops instead (for comparing the two).  ish_o_vectors() reports
 * whether the vector passes are in use. */
ish_o_end ish_o_neon_sg_i16(const uint8_t *rec, int T, int Q, int open, int ext, const int16_t *prof,
                            int8_t max_s, int8_t min_s, int ends);
ish_o_end ish_o_neon_sw_u8(const uint8_t *rec, int T, int reverse, int Q, uint8_t open, uint8_t ext,
                           const uint8_t *prof, uint8_t terminate, uint8_t bias);
ish_o_end ish_o_neon_sw_u16(const uint8_t *rec, int T, int reverse, int Q, uint16_t open, uint16_t ext,
                            const uint16_t *prof, uint16_t terminate, uint16_t bias);
int ish_o_neon_available(void);
void ish_o_set_vectors(int on);
int ish_o_vectors(void);

#ifdef __cplusplus
}
#endif
#endif
