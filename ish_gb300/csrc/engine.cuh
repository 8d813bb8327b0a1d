// engine.cuh -- shared definitions of the GB300 alignment-scoring engine.
//
// Scores are exact integers.  In the regime the engine runs its fast kernels
// in (gap_open > gap_extend and no int16 lane of the reference saturating,
// checked on the host), the striped passes of the reference compute the same
// H matrix as plain Gotoh: an E gap opened from an F gap that crossed a stripe
// boundary (which the lazy-F loop of
// ishlib/matcher/alignment/semi_global_aln/striped.mojo:396-434 never allows)
// can always be swapped for the E-then-F path of equal score, which the striped
// pass does allow.  The kernels therefore evaluate plain Gotoh and reproduce
// the reference's end-coordinate and tie rules exactly.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ish {

enum Mode : int { SG = 0, SW = 1 };

// Sentinel used for "minus infinity" lanes; far below every value the safe
// regime admits (|value| < 30000) and far from wrapping when a penalty is
// added to it.
constexpr int NEG_BIG = -20000;

// Layouts of the wavefront profile in shared memory (for code c, thread t
// and the thread's column j):
//   PROF_S16:  16-bit scores, [c][t][j]; a record pair's word is assembled
//              with one PRMT per column (large alphabets x long queries);
//   PROF_PAIR: packed 32-bit words for every (code A, code B) pair,
//              [cA][cB][t][j] (small alphabets);
//   PROF_S32:  32-bit words with the score in the low half, [c][t][j]; the
//              pair's word is one IMAD (the default).
enum ProfLayout : int { PROF_S16 = 0, PROF_PAIR = 1, PROF_S32 = 2 };

// Control word of the wavefront pipeline (one per row step).
constexpr uint32_t CTL_NEW = 1u << 16;   // row 0 of a new record pair
constexpr uint32_t CTL_IDLE = 1u << 17;  // no work in this slot
constexpr int CTL_SEQ_SHIFT = 18;        // 5-bit pair sequence number

struct Decision {
  int32_t max_score;
  float threshold;
};

// Record set in HBM, sorted by descending length.  Record bytes of sorted
// entry s live at codes[off[s] .. off[s] + len[s]), 16-byte aligned.
struct RecordsDev {
  const uint8_t *codes;
  const uint64_t *off;
  const uint32_t *len;
  const uint32_t *orig;  // original record index of sorted entry s
  uint32_t n;
};

// Per-record outputs, indexed by the ORIGINAL record index.
struct OutDev {
  int32_t *score;
  int32_t *qend;
  int32_t *tend;
  uint8_t *hit;
};

struct WaveParams {
  const uint4 *prof;       // wavefront profile (see build_wave_profile)
  uint32_t prof_bytes;     // bytes copied into shared memory
  int Q, G, K, d, kp;      // query length, threads per group, columns per thread, front padding, profile stride
  int alphabet;            // profile rows (codes map to rows through the remap table when remap_off != 0)
  uint32_t remap_off;      // byte offset of the 256-entry code -> row table in the profile, 0: none
  int layout;              // PROF_S16, PROF_PAIR or PROF_S32 (see below)
  uint32_t lane_mul;       // 65536: b * lane_mul + a packs two PROF_S32 words
  int open, ext, ends;
  int neg_limit;           // v_neg_limit of the reference (semi_global_aln/striped.mojo:329-334)
  int hleft, fin;          // left boundary value and F entering the padding
  int frame_mask;          // semi-global: R - 1, rows between frame resets (R * ext <= 2048)
  // packed 16-bit pairs of values used every row, precomputed on the host so
  // that the kernel reads them as operands instead of deriving them
  uint32_t pk_nopen;       // (-open, -open)
  uint32_t pk_next;        // (-ext, -ext)
  uint32_t pk_eopen;       // (ext - open, ext - open): the framed E update
  uint32_t pk_fsin;        // (fin + open, fin + open): F + open entering the padding
  uint32_t pk_ext;         // (ext, ext) for semi-global, 0 for local: one row's frame step
  uint32_t pk_drop;        // (-R * ext, -R * ext): a frame reset
  uint32_t row_bytes;      // profile bytes between consecutive codes' rows ((G * kp) words)
  const int16_t *hinit;    // H(-1, q) for q in [-d, Q), index q + d
  uint32_t first, count;   // sorted entries [first, first + count) are scored
  uint32_t pair_stride, pair_phase;  // of those, record pairs phase, phase + stride, ... (stride 0: every pair)
  uint32_t *counter;       // work counter (record pairs), zeroed before launch
  uint64_t max_steps;      // hard bound on pipeline steps per warp
  int *error;              // bit 0: record code >= alphabet; bit 1: step budget exceeded
  RecordsDev rec;
  OutDev out;
  Decision dec;
};

// One work range of the batched launch: sorted entries [first, first + count)
// of the record set (every stride-th record pair from phase, if `pairs` says
// so) scored against query q of the launch, handed out pair by pair by its own
// counter.
struct BatchTile {
  uint32_t q, first, count;
  uint32_t pairs;  // (stride << 16) | phase: the tile's record pairs, as WaveParams (0: every pair)
};

struct BatchParams {
  const WaveParams *queries;  // per query of the launch: layout, outputs, decision
  const BatchTile *tiles;
  uint32_t ntiles;
  uint32_t *tile_counter;     // one pair counter per tile, zeroed before launch
  uint32_t prof_area;         // shared-memory bytes reserved for the largest profile (16-byte multiple)
  uint32_t slot_words;        // slot words per block: 32 per group at the class's smallest G
  uint64_t step_cap;          // nonzero: pipeline steps per warp and tile (ISH_OPT_STEP_BUDGET)
};

struct PlainParams {
  const int16_t *prof;     // natural profile [code][Q]
  uint32_t prof_bytes;
  int use_smem;
  int Q, alphabet, open, ext, ends, neg_limit;
  const int16_t *hinit;    // H(-1, q), q in [0, Q)
  int32_t *scratch;        // 2 * Q * nthreads int32: H and E columns, interleaved by thread
  uint32_t nthreads;
  uint32_t first, count;
  int *error;
  RecordsDev rec;
  OutDev out;
  Decision dec;
};

// ---- packed 16-bit helpers (DPX on sm_90+) ----
__device__ __forceinline__ uint32_t dup16(int v) { return __byte_perm((uint32_t)v, 0u, 0x1010); }
// the same on the host
inline uint32_t dup16_host(int v) {
  const uint32_t u = (uint32_t)v & 0xffffu;
  return u | (u << 16);
}
__device__ __forceinline__ int lo16(uint32_t w) { return (int)(int16_t)(w & 0xffff); }
__device__ __forceinline__ int hi16(uint32_t w) { return (int)(int16_t)(w >> 16); }

// Hit decision of the CPU matchers.  Float32 arithmetic with round-to-nearest,
// exactly as Mojo's Float32 ops.
//  semi-global: striped_semi_global_matcher.mojo:245-251 together with the
//               cutoff test of semi_global_aln_start_end (striped.mojo:157-158);
//  local:       striped_local_matcher.mojo:514-533 with ssw_align's strict
//               cutoff (local_aln/striped.mojo:215-217) and its end sanity
//               check (223-230).
__device__ __forceinline__ uint8_t decide(int mode, int32_t score, int32_t qend, int32_t tend,
                                          const Decision &d) {
  float maxf = (float)d.max_score;
  float s = (float)score;
  if (mode == SG) {
    float cutoff = __fmul_rn(maxf, d.threshold);
    if (s < cutoff) return 0;
    return __fdiv_rn(s, maxf) >= d.threshold ? 1 : 0;
  }
  float cutoff = __fmul_rn(d.threshold, maxf);
  if (s <= cutoff) return 0;
  if (tend <= 0 || qend <= 0) return 0;
  return __fdiv_rn(s, maxf) >= d.threshold ? 1 : 0;
}

}  // namespace ish
