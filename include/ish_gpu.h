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
/* one thread per record with int16 per-thread H/E arrays, 15,000 threads in
 * blocks of 32: the reference GPU kernel's storage and launch shape
 * (ishlib/matcher/alignment/semi_global_aln/basic.mojo:305-306,
 * ishlib/gpu/searcher_device.mojo:477-497); queries up to 2048 residues,
 * longer ones run as ISH_KERNEL_PLAIN */
#define ISH_KERNEL_PLAIN16 3

#define ISH_OPT_KERNEL 1      /* value: ISH_KERNEL_* */
#define ISH_OPT_SG_LANES 2    /* int16 lanes of the reference CPU build (default 8) */
#define ISH_OPT_SW_U8_LANES 3 /* uint8 lanes of the local byte pass (default 16) */
#define ISH_OPT_SW_U16_LANES 4 /* uint16 lanes of the local word pass (default 8) */
#define ISH_OPT_WAVE_GROUP 5  /* force threads per record pair (0 = autotuned) */
#define ISH_OPT_WAVE_K 6      /* force query columns per thread (0 = autotuned) */
#define ISH_OPT_PROFILE_LAYOUT 7 /* force the profile layout: -1 auto, 0 16-bit, 1 pair, 2 32-bit */
#define ISH_OPT_WAVE_BLOCKS 8 /* cap wavefront blocks per SM (0 = as many as fit) */
#define ISH_OPT_WINDOWS 10    /* 1 (default): window long records when they would bound the pass; 0: never */
#define ISH_OPT_WAVE_LEAN 9   /* 34 <= K <= 48: -1 measured default, 0 128x3 blocks, 1 128x2 (more registers) */
#define ISH_OPT_SERVE_STEP_CELLS 13 /* serving: cells a step aims at per query (default 1.25e11); a query takes
                                    * cells/that steps, 1..chunks; 0: every query takes `chunks` steps */
/* Fault injection for testing a caller's error paths (no counterpart in the
 * reference).  ISH_OPT_STEP_BUDGET: 0 (default) lets every wavefront and
 * batched launch of this context run to the end of its work; n > 0 caps each
 * warp at n pipeline steps, so a launch with more work stops early and the call
 * (or, in the serving loop, the queries of that step) fails with
 * ISH_ETIMEDOUT -- the device-side bound every wavefront launch carries, made
 * to run out.  ISH_OPT_FAULT_ALLOC: n >= 0 makes the (n+1)-th device allocation
 * the library attempts from now on fail as if device memory were exhausted
 * (ISH_ENOMEM); it applies to every context of the process and disarms after
 * firing; -1 disarms it.  Neither changes results when left at its default. */
#define ISH_OPT_STEP_BUDGET 11
#define ISH_OPT_FAULT_ALLOC 12

typedef struct ish_ctx ish_ctx;

ISH_API int ish_gpu_abi_version(void);

/* Open a context on CUDA device `device` (SearcherDevice.create_devices,
 * ishlib/gpu/searcher_device.mojo:153-174).  *out is NULL on failure. */
ISH_API int ish_gpu_open(int device, ish_ctx **out);
ISH_API void ish_gpu_close(ish_ctx *ctx);
/* Text of the last failure on this context ("" if none).  Valid until the
 * next call on the context.  ctx may be NULL (then: the last open failure). */
ISH_API const char *ish_gpu_last_error(const ish_ctx *ctx);
/* Sets one of the ISH_OPT_* options.  Refused (ISH_EINVAL) while the serving
 * loop runs: its thread reads them. */
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
 *   hit_idx[0 .. *n_hits): the hits in ascending record order (room for n
 *       entries: the call may write past *n_hits, those entries mean nothing).
 * Outputs in pinned host memory (cudaHostAlloc) come back at full copy speed;
 * pageable ones are staged by the CUDA driver. */
ISH_API int ish_gpu_score(ish_ctx *ctx, int32_t query_id, const uint8_t *records, const uint64_t *offsets,
                  uint32_t n, int32_t *score, int32_t *query_end, int32_t *target_end, uint8_t *hit,
                  uint32_t *hit_idx, uint32_t *n_hits);

/* Device-resident record sets (kept in HBM across queries). */
ISH_API int ish_gpu_records_load(ish_ctx *ctx, const uint8_t *records, const uint64_t *offsets, uint32_t n,
                         int32_t *set_id);
ISH_API int ish_gpu_records_free(ish_ctx *ctx, int32_t set_id);
/* As ish_gpu_records_load, but returns as soon as the upload and packing are
 * queued on the context's load stream, so that they overlap the scoring of
 * another set: load batch k + 1 with this call, then score batch k.  One load
 * is in flight per context: it completes (the call waits for it) when its set
 * is first used, when another load starts, and in ish_gpu_close.  `records`
 * and `offsets` must stay valid and unchanged until then (pinned host memory
 * is read by the copy engine while the call has already returned).  Replaces
 * the synchronous per-batch upload of ishlib/gpu/process_batch.mojo:112-132,
 * where the CPU packs the next batch while the device scores. */
ISH_API int ish_gpu_records_load_async(ish_ctx *ctx, const uint8_t *records, const uint64_t *offsets, uint32_t n,
                                       int32_t *set_id);
/* Number of records and total residue bytes of a resident set. */
ISH_API int ish_gpu_records_info(ish_ctx *ctx, int32_t set_id, uint32_t *n, uint64_t *total_bytes);

/* Load a resident set from RAW bytes: records as for ish_gpu_records_load, but
 * not yet encoded; the device encodes them with ish's table for matrix_kind
 * (convert_ascii_to_encoding: ishlib/matcher/alignment/scoring_matrix.mojo:
 * 9-27 AA_TO_NUM, 131-149 NT_TO_NUM, identity for ascii) while packing,
 * replacing the runners' per-byte host loop
 * (ishlib/parallel_line_search_runner.mojo:90-94, 344-348). */
ISH_API int ish_gpu_records_load_raw(ish_ctx *ctx, const uint8_t *raw, const uint64_t *offsets, uint32_t n,
                                     int matrix_kind, int32_t *set_id);

/* Load the LINES of a text buffer as a resident set: split at '\n' on the
 * device exactly as ish's line reader does (ishlib/vendor/kseq.mojo:270-330:
 * a trailing '\r' is dropped from lines longer than one byte, a last line
 * without '\n' is a record, empty lines are records), encoded on the device as
 * for ish_gpu_records_load_raw.  Record i is line i of the text. */
ISH_API int ish_gpu_records_load_lines(ish_ctx *ctx, const uint8_t *text, uint64_t bytes, int matrix_kind,
                                       int32_t *set_id, uint32_t *n_records);

/* Load the FASTA/FASTQ records of a text buffer as a resident set: split on
 * the device exactly as ish's FASTX runners read a file
 * (ishlib/vendor/kseq.mojo:370-461, FastxReader[read_comment=False].read, in
 * the loop of ishlib/parallel_fastx_search_runner.mojo:93-121): text before
 * the first '>' or '@' is skipped, a record's sequence lines are joined with
 * one trailing '\r' dropped from each, an empty line appends a '\n' and the
 * whole next line, and reading stops at the first record whose read returns
 * 0 or less (an empty sequence, a FASTQ quality of another length, a missing
 * quality line).  Sequences are encoded on the device as for
 * ish_gpu_records_load_raw; record i is the i-th record of the text.
 *   bounds (may be NULL): 4 entries per record, byte offsets into `text`:
 *     name [bounds[4i], bounds[4i+1]) (the header line after its '>'/'@',
 *     as the reader keeps it), quality [bounds[4i+2], bounds[4i+3]) (both 0
 *     for a FASTA record).  If more than bounds_cap records are read the call
 *     fails with ISH_EOVERFLOW and loads nothing.
 * A FASTQ quality that continues on the next line (legal for kseq, which
 * reads quality lines until the quality is as long as the sequence) is not
 * split on the device: ISH_EINVAL. */
ISH_API int ish_gpu_records_load_fastx(ish_ctx *ctx, const uint8_t *text, uint64_t bytes, int matrix_kind,
                                       int32_t *set_id, uint32_t *n_records, uint64_t *bounds, uint64_t bounds_cap);

/* Copy records [first, first + count) of a resident set back to the host, in
 * record order, as the set holds them (encoded codes): codes receives them
 * concatenated (capacity codes_cap bytes), offsets count + 1 entries
 * (record i of the range is codes[offsets[i] .. offsets[i + 1])).  What a
 * runner prints for a match when the device parsed the file (the FASTX
 * runners keep every record's sequence for their output,
 * ishlib/parallel_fastx_search_runner.mojo:306-331).  ISH_EOVERFLOW if the
 * codes do not fit (offsets are still filled). */
ISH_API int ish_gpu_records_get(ish_ctx *ctx, int32_t set_id, uint32_t first, uint32_t count, uint8_t *codes,
                                uint64_t codes_cap, uint64_t *offsets);

/* Score one query against a resident set; outputs as for ish_gpu_score. */
ISH_API int ish_gpu_score_set(ish_ctx *ctx, int32_t query_id, int32_t set_id, int32_t *score,
                      int32_t *query_end, int32_t *target_end, uint8_t *hit, uint32_t *hit_idx,
                      uint32_t *n_hits);

/* Score several queries against one resident set in one batched launch.
 * Replaces the reference's per-query launch loop over a record set
 * (benchmarking/ish_bench_aligner_gpu.mojo:1616-1888 with 2039-2297: one
 * launch per query, kernels instantiated per query-length bin).  Queries are
 * grouped by kernel shape; each group runs as one persistent kernel whose
 * blocks steal record pairs of the group's queries from per-query work
 * counters, and the groups, the hit compaction and the counter resets form one
 * CUDA graph, captured on the first call for a (query list, set, requested
 * outputs) combination and replayed after.
 *   score, query_end, target_end, hit: query-major arrays of n_queries * n
 *     entries (n = records in the set): entry [i * n + r] is query
 *     query_ids[i] against record r.  Any may be NULL.
 *   hit_offsets: n_queries + 1 entries (may be NULL); query i's hits are
 *     hit_idx[hit_offsets[i] .. hit_offsets[i + 1]), ascending record indices.
 *   hit_idx: capacity hit_cap (may be NULL).  If the hits do not fit, nothing
 *     is written to it, hit_offsets is still filled and ISH_EOVERFLOW returned.
 * Results are identical to ish_gpu_score_set for every query. */
ISH_API int ish_gpu_score_multi(ish_ctx *ctx, const int32_t *query_ids, uint32_t n_queries, int32_t set_id,
                                int32_t *score, int32_t *query_end, int32_t *target_end, uint8_t *hit,
                                uint32_t *hit_idx, uint64_t hit_cap, uint64_t *hit_offsets);

/* Autotuner: for each query, times the candidate kernel shapes (threads per
 * record pair, query columns per thread, profile layout) on a sample of a
 * resident set and keeps the fastest for every later launch (single and
 * batched) of a query with the same algorithm, alphabet and length.  group /
 * cols (may be NULL) receive the shape each query now uses.  Options
 * ISH_OPT_WAVE_GROUP / ISH_OPT_WAVE_K still override.  No counterpart in the
 * reference (its kernels are instantiated per query-length bin,
 * ish_bench_aligner_gpu.mojo:2039-2297, with a fixed launch shape,
 * ishlib/gpu/searcher_device.mojo:477-497). */
ISH_API int ish_gpu_autotune(ish_ctx *ctx, int32_t set_id, const int32_t *query_ids, uint32_t n_queries,
                             int32_t *group, int32_t *cols);

/* Match starts of hits, computed on the device: for hit i (record hit_idx[i]
 * of a resident set, forward target end target_end[i] as returned by the
 * scoring calls) start[i] is the target start the CPU matcher reports, i.e.
 * MatchResult(start, target_end + 1).  Replaces the per-hit CPU find_start of
 * ishlib/cpu/process_batch.mojo:56-61 (StripedSemiGlobalMatcher.find_start,
 * ishlib/matcher/striped_semi_global_matcher.mojo:259-276; the reverse pass of
 * semi_global_aln_start_end, semi_global_aln/striped.mojo:160-191; for local
 * alignment the reverse sw of ssw_align, local_aln/striped.mojo:232-259). */
ISH_API int ish_gpu_match_starts(ish_ctx *ctx, int32_t query_id, int32_t set_id, const uint32_t *hit_idx,
                                 const int32_t *target_end, uint32_t n_hits, int64_t *start);

/* ---- serving loop: continuous batching against a resident set ----
 * Replaces the reference's synchronous per-batch device round trip
 * (ishlib/gpu/process_batch.mojo:27-163 driving SearcherDevice,
 * ishlib/gpu/searcher_device.mojo:419-519) for callers that keep one record set
 * on the device and score queries as they arrive.  A scheduler thread owned by
 * the context admits waiting queries while fewer than max_active run and the
 * device memory their outputs need (29 bytes per record of the set) fits
 * mem_budget (0: half of the free device memory), and runs steps: each step
 * scores the next chunk of the set for every admitted query in one batched
 * launch, so queries that arrive while others run join at the next step and
 * share the device with them.  A query takes between 1 and `chunks` steps,
 * as many as keep a step near ISH_OPT_SERVE_STEP_CELLS cells (its chunk c of
 * m: every m-th record pair of the set's longest-first order, from pair c).  Results are
 * identical to ish_gpu_score_set.  submit and poll may be called from any
 * thread; the other calls on the context stay on one thread. */
ISH_API int ish_gpu_serve_start(ish_ctx *ctx, int32_t set_id, uint32_t max_active, uint64_t mem_budget,
                                uint32_t chunks);
/* Queue query query_id (its parameters are copied; the query may be freed
 * afterwards).  *ticket identifies the result. */
ISH_API int ish_gpu_submit(ish_ctx *ctx, int32_t query_id, uint64_t *ticket);
/* Result of a ticket: ISH_EAGAIN while it runs (after waiting up to wait_ms);
 * else the hits (ascending record indices, with score, query end and target
 * end of each; any pointer may be NULL), their number and the latency from
 * submit to completion.  If the hits exceed cap, ISH_EOVERFLOW is returned with
 * *n_hits set and the result kept.  A query that could not run returns its
 * error.  A result is delivered once. */
ISH_API int ish_gpu_poll(ish_ctx *ctx, uint64_t ticket, uint32_t *hit_idx, int32_t *hit_score, int32_t *hit_qend,
                         int32_t *hit_tend, uint32_t cap, uint32_t *n_hits, double *latency_ms, int32_t wait_ms);
/* Finish every queued and running query, then stop the scheduler. */
ISH_API int ish_gpu_serve_stop(ish_ctx *ctx);
/* Completed queries, cells scored, device time of the steps, the largest
 * number of queries that shared a step, and the number of steps. */
ISH_API int ish_gpu_serve_stats(ish_ctx *ctx, uint64_t *completed, double *cells, double *device_ms,
                                uint32_t *max_active_seen, uint64_t *steps);

/* Score records that are already in device memory, into device outputs,
 * without allocating anything.  No counterpart in the reference: this serves
 * callers that cannot allocate device memory when they score (device memory
 * owned by another allocator or arena, hosts that forbid cudaMalloc/cudaFree
 * from worker threads, an exhausted device-memory budget).
 *   d_records / records_bytes: device bytes of the encoded records;
 *   d_offsets: device uint64[n+1], record i = d_records[d_offsets[i] .. d_offsets[i+1]);
 *   enc_query, matrix: HOST arrays, as for ish_gpu_set_query;
 *   d_score, d_query_end, d_target_end, d_hit: device outputs (any may be NULL),
 *       same values as ish_gpu_score, in record order, for every request it
 *       accepts.  It has no lane-exact fallback: parameters outside the
 *       exact-integer regime (gap_open <= gap_extend, scores that could leave
 *       int16) and, with a fixed target start, records too long for the int16
 *       boundary row are refused with ISH_EINVAL where ish_gpu_score would
 *       switch to its exact kernels;
 *   stream: cudaStream_t to run on (NULL = the legacy default stream);
 *   err: optional buffer for a message (err_len bytes).
 * Working memory is a fixed 32 MiB __device__ array inside the library that
 * every GPU loading the library holds until exit; a query needing more
 * (2*alphabet*qlen bytes of profile plus 1 KiB per query column) is rejected
 * with ISH_EOVERFLOW.  All calls share that array: calls that overlap on the
 * GPU race and must be serialised by the caller.  The first call on a device
 * (with that device current) resolves the array's address; make it before
 * any stream capture, and do not use the entry point after a cudaDeviceReset
 * (or a release of the device's primary context) in the same process: the
 * address kept from the first call would be stale.  Blocks until the work on
 * `stream` is done. */
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

/* Phases of the last record load (ish_gpu_records_load*): upload_ms, device
 * time from the start of the host-to-device copy to the start of packing
 * (for text loads this includes the splitting kernels); pack_ms, device time
 * of the sort and pack kernels; wall_ms, host time of the whole call.  When
 * the records' bytes are uploaded on the copy stream (concatenated records:
 * ish_gpu_records_load, _async, _raw and ish_gpu_score), the sort kernels run
 * during that upload, upload_ms ends with the upload and pack_ms is the time
 * after it, so the two add up to the load's device time.  Any pointer may be
 * NULL.  No counterpart in the reference: measurement support for the
 * engine. */
ISH_API int ish_gpu_last_load_ms(ish_ctx *ctx, double *upload_ms, double *pack_ms, double *wall_ms);

/* Throughput of the packed 16-bit DPX add-max instruction on this device,
 * measured now (instructions per second; each covers two 16-bit lanes).  The
 * integer cell-update roofline of the engine is derived from it.  No
 * counterpart in the reference: measurement support for the engine. */
ISH_API int ish_gpu_calibrate(ish_ctx *ctx, double *dpx_ops_per_s);

/* Local-alignment cell updates per second on packed lanes, measured now with
 * no memory traffic: two 16-bit lanes per word with DPX add-max (the
 * wavefront kernel's form) and four 8-bit lanes per word with the saturating
 * SIMD byte add/subtract/max on a biased profile (the form of the reference's
 * uint8 pass, local_aln/striped.mojo:162-196).  No counterpart in the
 * reference: it measures this engine's choice of lane width. */
ISH_API int ish_gpu_calibrate_lanes(ish_ctx *ctx, double *s16x2_cells_per_s, double *u8x4_cells_per_s);

/* Number of CUDA kernels the library has launched on this context (a batched
 * launch counts the kernel nodes of its graph).  No counterpart in the
 * reference: measurement support. */
ISH_API int ish_gpu_launch_count(ish_ctx *ctx, uint64_t *count);

/* Windows the last single-query scoring call cut its longest records into
 * (0: the set was scored record by record).  With a free target start the
 * best alignment spans a bounded number of record rows, so long records are
 * scored as overlapping windows and folded per record, with results identical
 * to whole-record scoring (see ISH_OPT_WINDOWS).  No counterpart in the
 * reference: measurement support. */
ISH_API int ish_gpu_last_windows(ish_ctx *ctx, uint32_t *windows);

#ifdef __cplusplus
}
#endif
#endif
