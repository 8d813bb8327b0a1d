/*
 * ish_gpu.h -- C ABI of libish_gpu.so, the GB300 (sm_103a) alignment-scoring
 * engine behind ish's GPU matcher plugin.
 *
 * The entry points replace the device layer that ish drives through its
 * `GpuMatcher` trait (ishlib/matcher/__init__.mojo:79-121) and
 * `SearcherDevice` (ishlib/gpu/searcher_device.mojo:98-519), as called from
 * `gpu/process_batch.parallel_starts_ends` (ishlib/gpu/process_batch.mojo:27-163)
 * and `cpu/process_batch.parallel_starts` (ishlib/cpu/process_batch.mojo:37-68).
 *
 * Conventions
 *   - Every function returns 0 on success or a negative errno-style status
 *     (ISH_E*).  Nothing aborts and no device code traps; the text of the last
 *     failure is available from ish_gpu_last_error().
 *   - Records and queries are ENCODED (codes < alphabet size), exactly what the
 *     reference runners hand to the matcher after convert_ascii_to_encoding
 *     (ishlib/parallel_line_search_runner.mojo:90-94).
 *   - Record sets are given as one concatenated byte array plus n+1 offsets:
 *     record i is records[offsets[i] .. offsets[i+1]).
 *   - Coordinates are 0-based and inclusive, as in the reference's
 *     AlignmentEnd (ishlib/matcher/alignment/striped_utils.mojo:103-108).
 *   - One context per host thread.  The caller owns every host array; the
 *     library owns device memory and pinned staging.
 */
#ifndef ISH_GPU_H
#define ISH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define ISH_API __attribute__((visibility("default")))
#else
#define ISH_API
#endif

#define ISH_GPU_ABI_VERSION 1

/* status codes */
#define ISH_OK 0
#define ISH_EINVAL (-22)    /* bad argument, unknown id, record code >= alphabet */
#define ISH_ENOMEM (-12)    /* device or pinned allocation failed */
#define ISH_EOVERFLOW (-75) /* query longer than the engine supports */
#define ISH_ENODEV (-19)    /* no usable CUDA device */
#define ISH_EDEVICE (-5)    /* CUDA runtime error (text in ish_gpu_last_error) */
#define ISH_EAGAIN (-11)    /* serving: result not ready yet */
#define ISH_ETIMEDOUT (-110) /* a bounded device wait gave up */

/* MatrixKind (ishlib/matcher/alignment/scoring_matrix.mojo:178-183) */
#define ISH_MATRIX_ASCII 0
#define ISH_MATRIX_ACTGN 1
#define ISH_MATRIX_ACTGN0 2
#define ISH_MATRIX_BLOSUM62 3

/* --match-algo (ishlib/searcher_settings.mojo:104-114) */
#define ISH_ALGO_SEMI_GLOBAL 0 /* striped-semi-global */
#define ISH_ALGO_LOCAL 1       /* striped-local */

/* --sg-ends-free bits (SemiGlobalEndsFreeness, ishlib/searcher_settings.mojo:288-414) */
#define ISH_FREE_QUERY_START 1u
#define ISH_FREE_QUERY_END 2u
#define ISH_FREE_TARGET_START 4u
#define ISH_FREE_TARGET_END 8u

/* kernel choice for ish_gpu_set_option(ISH_OPT_KERNEL, ...) */
#define ISH_KERNEL_AUTO 0  /* wavefront engine, exact fallback where needed */
#define ISH_KERNEL_PLAIN 1 /* one thread per record (the reference GPU design) */
#define ISH_KERNEL_EXACT 2 /* per-record emulation of the striped CPU algorithm */

#define ISH_OPT_KERNEL 1      /* value: ISH_KERNEL_* */
#define ISH_OPT_SG_LANES 2    /* int16 lanes of the reference CPU build (default 8) */
#define ISH_OPT_SW_U8_LANES 3 /* uint8 lanes of the local byte pass (default 16) */
#define ISH_OPT_SW_U16_LANES 4 /* uint16 lanes of the local word pass (default 8) */
#define ISH_OPT_WAVE_GROUP 5  /* force threads per record pair (0 = autotuned) */
#define ISH_OPT_WAVE_K 6      /* force query columns per thread (0 = autotuned) */

typedef struct ish_ctx ish_ctx;

ISH_API int ish_gpu_abi_version(void);

/* Open a context on CUDA device `device` (SearcherDevice.create_devices,
 * ishlib/gpu/searcher_device.mojo:153-174).  *out is NULL on failure. */
ISH_API int ish_gpu_open(int device, ish_ctx **out);
ISH_API void ish_gpu_close(ish_ctx *ctx);
/* Text of the last failure on this context ("" if none).  Valid until the
 * next call on the context.  ctx may be NULL (then: the last open failure). */
ISH_API const char *ish_gpu_last_error(const ish_ctx *ctx);
ISH_API int ish_gpu_set_option(ish_ctx *ctx, int option, int64_t value);

/* Register a query: the matcher state of StripedSemiGlobalMatcher.__init__
 * (ishlib/matcher/striped_semi_global_matcher.mojo:41-75) or
 * StripedLocalMatcher.__init__ (ishlib/matcher/striped_local_matcher.mojo:31-57).
 *   matrix:   alphabet*alphabet int8 values, row = record code, column = query
 *             code (GpuMatcher.matrix_bytes/matrix_len).
 *   max_score: Matcher.max_alignment_score (the optimal score of the query).
 *   threshold: Matcher.score_threshold (--score).
 *   ends_free: ISH_FREE_* bits, used by the semi-global algorithm only.
 * gap_open / gap_ext are the positive penalties of --gap-open/--gap-extend. */
ISH_API int ish_gpu_set_query(ish_ctx *ctx, const uint8_t *enc_query, uint32_t qlen, int matrix_kind,
                      const int8_t *matrix, uint32_t alphabet, int algo, uint32_t gap_open,
                      uint32_t gap_ext, uint32_t ends_free, int32_t max_score, float threshold,
                      int32_t *query_id);
ISH_API int ish_gpu_free_query(ish_ctx *ctx, int32_t query_id);

/* One-shot scoring of host records against one query
 * (gpu/process_batch.parallel_starts_ends + the threshold of
 * cpu/process_batch.parallel_starts).  Per record i (any output may be NULL):
 *   score[i], query_end[i], target_end[i]: the forward pass of the matcher
 *       (semi_global_aln / the adaptive sw of ssw_align);
 *   hit[i]: 1 iff first_match() of the CPU matcher returns a match;
 *   hit_idx[0 .. *n_hits): the hits in ascending record order. */
ISH_API int ish_gpu_score(ish_ctx *ctx, int32_t query_id, const uint8_t *records, const uint64_t *offsets,
                  uint32_t n, int32_t *score, int32_t *query_end, int32_t *target_end, uint8_t *hit,
                  uint32_t *hit_idx, uint32_t *n_hits);

/* Device-resident record sets (kept in HBM across queries). */
ISH_API int ish_gpu_records_load(ish_ctx *ctx, const uint8_t *records, const uint64_t *offsets, uint32_t n,
                         int32_t *set_id);
ISH_API int ish_gpu_records_free(ish_ctx *ctx, int32_t set_id);
/* Number of records and total residue bytes of a resident set. */
ISH_API int ish_gpu_records_info(ish_ctx *ctx, int32_t set_id, uint32_t *n, uint64_t *total_bytes);

/* Score one query against a resident set; outputs as for ish_gpu_score. */
ISH_API int ish_gpu_score_set(ish_ctx *ctx, int32_t query_id, int32_t set_id, int32_t *score,
                      int32_t *query_end, int32_t *target_end, uint8_t *hit, uint32_t *hit_idx,
                      uint32_t *n_hits);

/* Score records that are already in device memory, into device outputs,
 * without allocating anything.  No counterpart in the reference: this serves
 * callers that cannot allocate device memory when they score (device memory
 * owned by another allocator or arena, hosts that forbid cudaMalloc/cudaFree
 * from worker threads, an exhausted device-memory budget).
 *   d_records / records_bytes: device bytes of the encoded records;
 *   d_offsets: device uint64[n+1], record i = d_records[d_offsets[i] .. d_offsets[i+1]);
 *   enc_query, matrix: HOST arrays, as for ish_gpu_set_query;
 *   d_score, d_query_end, d_target_end, d_hit: device outputs (any may be NULL),
 *       same values as ish_gpu_score, in record order;
 *   stream: cudaStream_t to run on (NULL = the legacy default stream);
 *   err: optional buffer for a message (err_len bytes).
 * Working memory is a fixed 32 MiB __device__ array inside the library that
 * every GPU loading the library holds until exit; a query needing more
 * (2*alphabet*qlen bytes of profile plus 1 KiB per query column) is rejected
 * with ISH_EOVERFLOW.  All calls share that array: calls that overlap on the
 * GPU race and must be serialised by the caller.  The first call on a device
 * (with that device current) resolves the array's address; make it before
 * any stream capture.  Blocks until the work on `stream` is done. */
ISH_API int ish_gpu_score_noalloc(const uint8_t *d_records, uint64_t records_bytes, const uint64_t *d_offsets,
                                  uint32_t n, const uint8_t *enc_query, uint32_t qlen, const int8_t *matrix,
                                  uint32_t alphabet, int algo, uint32_t gap_open, uint32_t gap_ext,
                                  uint32_t ends_free, int32_t max_score, float threshold, int32_t *d_score,
                                  int32_t *d_query_end, int32_t *d_target_end, uint8_t *d_hit, void *stream,
                                  char *err, size_t err_len);

/* Device-side timing of the last scoring call on this context: milliseconds
 * from the first scoring kernel to the end of the hit compaction (CUDA events
 * on the engine's stream; excludes host<->device copies). */
ISH_API int ish_gpu_last_kernel_ms(ish_ctx *ctx, double *ms);

/* Throughput of the packed 16-bit DPX add-max instruction on this device,
 * measured now (instructions per second; each covers two 16-bit lanes).  The
 * integer cell-update roofline of the engine is derived from it.  No
 * counterpart in the reference: measurement support for the engine. */
ISH_API int ish_gpu_calibrate(ish_ctx *ctx, double *dpx_ops_per_s);

#ifdef __cplusplus
}
#endif
#endif
