// kernels.cuh -- declarations shared by the kernel translation units and the
// host engine.
#pragma once

#include "engine.cuh"

namespace ish {

constexpr uint32_t NBUCKETS = 65536;     // length buckets of the record sort
constexpr uint32_t SCAN_TILE = 4096;     // values per block of k_scan64_block (1024 threads)
constexpr uint32_t HIT_TILE = 8192;      // records per block of the hit compaction
constexpr uint32_t SMEM_BUCKETS = 4096;  // length buckets counted in shared memory by k_lengths / k_scatter

constexpr uint32_t LINE_TILE = 65536;    // text bytes per block of the line splitter
__global__ void k_zero2(uint32_t *a, uint32_t na, uint32_t *b, uint32_t nb);
__global__ void k_lengths(const uint64_t *off, const uint64_t *end, uint32_t n, uint32_t *len, uint64_t *tile_sum,
                          uint32_t *hist, uint32_t *max_bucket, uint32_t *summary);
__global__ void k_scan_slots(const uint32_t *len, uint32_t n, const uint64_t *tile_sum, uint64_t *poff);
constexpr uint32_t BUCKET_BLOCKS = NBUCKETS / 1024;  // blocks of the bucket cursor kernel
__global__ void k_bucket_cursors(const uint32_t *hist, const uint32_t *max_bucket, uint32_t *cursor,
                                 uint32_t *summary);
__global__ void k_scatter(const uint32_t *len, const uint64_t *poff, uint32_t n, uint32_t *cursor, uint32_t *len_s,
                          uint64_t *off_s, uint32_t *orig_s, uint32_t *hist, uint32_t *max_bucket,
                          const uint32_t *summary);
__global__ void k_pack(const uint8_t *src, uint64_t src_bytes, const uint64_t *off, const uint64_t *end,
                       const uint64_t *poff, uint32_t n, const uint32_t *len_s, const uint32_t *orig_s,
                       uint32_t *long_counter, const uint8_t *enc, uint8_t *dst, uint32_t *max_code, uint32_t gw);
__global__ void k_count_newlines(const uint8_t *text, uint64_t bytes, uint32_t *block_counts);
__global__ void k_write_newlines(const uint8_t *text, uint64_t bytes, const uint32_t *block_offsets, uint64_t *pos);
__global__ void k_line_bounds(const uint8_t *text, uint64_t bytes, const uint64_t *nl, uint32_t n_nl, uint32_t n_lines,
                              uint64_t *start, uint64_t *end, unsigned long long *total);
__global__ void k_scan64_block(const uint64_t *in, uint64_t *out, uint32_t n, uint64_t *block_sums);
__global__ void k_scan64_add(uint64_t *out, uint32_t n, const uint64_t *block_offsets);
__global__ void k_trivial(RecordsDev rec, uint32_t first, uint32_t count, int mode, int qlen, OutDev out, Decision dec);
typedef void (*PlainFn)(const PlainParams);
// plain_kernel<mode, qmax>: qmax 0 (int32 columns in global scratch) or a
// power of two 64..2048 (int16 per-thread columns); nullptr otherwise
PlainFn plain_fn(int mode, int qmax);
constexpr int PLAIN16_QMAX = 2048;     // longest query of the int16 plain kernel
constexpr int PLAIN16_THREADS = 15000; // its launch: 15,000 threads in blocks of 32
__global__ void k_count_hits(const uint8_t *hit, uint32_t n, uint32_t *block_counts);
__global__ void k_scan_counts(uint32_t *counts, uint32_t nb, uint32_t *total);
__global__ void k_dpx_peak(uint32_t *out, int iters, uint32_t b, uint32_t c);
// k_lane_rows<u8>: local-alignment rows on 2 x 16-bit or 4 x 8-bit lanes
// (ish_gpu_calibrate_lanes)
typedef void (*LaneFn)(uint32_t *out, int rows, uint32_t p0, uint32_t popen, uint32_t pext, uint32_t bias);
LaneFn lane_rows_fn(bool u8);
__global__ void k_write_hits(const uint8_t *hit, uint32_t n, const uint32_t *block_offsets, uint32_t *idx);
__global__ void k_gather_hits(const uint32_t *idx, const uint32_t *count, const int32_t *score, const int32_t *qend,
                              const int32_t *tend, int32_t *hit_score, int32_t *hit_qend, int32_t *hit_tend);

// Rows a wavefront thread computes per pipeline step.  A record's codes arrive
// four to a 32-bit word, and everything beside the recurrence itself -- the
// pipeline shuffles and control word, thread 0's work grab, the code refill,
// the frame reset, the end-of-record test and the target-end maximum -- runs
// once per step instead of once per row.  A pair's rows are rounded up to a
// multiple of the rows per step (the rows past both records' ends feed nothing).
// Semi-global row frames reset only at step boundaries, so the fast regime
// keeps R >= WAVE_RPS_SG rows per frame period (gap_extend <= 512 at 4).
// Chosen per mode from measurements (protein, K = 38): semi-global 4, local 2
// (local alignment's per-row maximum and dominance state make four rows per
// step cost more registers than they save).
#ifndef WAVE_RPS_SG
#define WAVE_RPS_SG 4
#endif
#ifndef WAVE_RPS_SW
#define WAVE_RPS_SW 2
#endif

// Wavefront kernels are instantiated for K = 2, 4, ..., WAVE_KMAX columns per
// thread, both modes and both profile layouts.
constexpr int WAVE_KMAX = 64;
// Threads per block and blocks per SM (the register budget): 256 x 2 up to
// K = 32 columns per thread, 128 x 3 up to K = 48 (12 warps per SM for wide
// rows), above that 128 x 2 for semi-global and 256 x 1 for local alignment
// (whose long-query profiles and saved rows would otherwise fit only one
// 128-thread block per SM: +46 % at Q = 1900).
__host__ __device__ constexpr int wave_block_threads(int K, int mode) {
  return K <= 32 ? 256 : (K <= 48 ? 128 : (mode == 1 ? 256 : 128));
}
__host__ __device__ constexpr int wave_blocks_per_sm(int K, int mode) {
  return K <= 32 ? 2 : (K <= 48 ? 3 : (mode == 1 ? 1 : 2));
}
// Register-lean builds trade warps for registers per thread: for
// 25 <= K <= 32, 128 x 3 (12 warps, 170 registers) instead of 256 x 2 (16
// warps, 128); for 34 <= K <= 48, 128 x 2 instead of 128 x 3 (168).  Which
// build runs is chosen per (K, mode) from measurements (wave_lean, batch_lean).
constexpr int WAVE_LEAN_KMIN = 25, WAVE_LEAN_KMAX = 48;
__host__ __device__ constexpr bool wave_has_lean(int K) { return K >= WAVE_LEAN_KMIN && K <= WAVE_LEAN_KMAX && K != 33; }
__host__ __device__ constexpr int wave_threads_lean(int K, int mode, int lean) {
  return (lean && wave_has_lean(K) && K <= 32) ? 128 : wave_block_threads(K, mode);
}
__host__ __device__ constexpr int wave_blocks_lean(int K, int mode, int lean) {
  return (lean && wave_has_lean(K)) ? (K <= 32 ? 3 : 2) : wave_blocks_per_sm(K, mode);
}
// wave_kernel reads its parameters from a shared-memory copy for these
// (K, mode, lean build) (see wave.cuh).  Measured on the protein search
// (400k records, G = 8, Q = 8K - 2): semi-global at K = 9..32 +1 to +12 %;
// local at K = 12..32 mostly +1.4 to +9.7 %; the 128 x 3 builds of K = 34..48
// +5 to +10 % (semi-global), -1 to +10 % (local); K = 58..64 +1.5 to +6.6 %
// and local K = 50 +3 % (K = 52..56: -2.6 to +0.2 %).  The register-lean
// builds of K >= 34 keep the parameter bank.
#ifndef WAVE_PARAMS_SMEM
#define WAVE_PARAMS_SMEM(K, MODE, LEAN)                                              \
  (((MODE) == 0 && (K) >= 9 && (K) <= 32) || ((MODE) == 1 && (K) >= 12 && (K) <= 32) || \
   (!(LEAN) && (K) >= 34 && (K) <= 48) || (K) >= 58 || ((MODE) == 1 && (K) == 50))
#endif
// Local alignment keeps, per thread, the H row of each lane's last
// improvement as 16-bit values: two arrays of K (rounded up to 8) halves,
// strided by an odd number of 16-byte units.
__host__ __device__ constexpr int wave_save_words(int K) { return ((((K + 7) & ~7) / 4) | 1) * 4; }
typedef void (*WaveFn)(const WaveParams);
// Returns the kernel for (K, mode, profile layout, lean variant) or nullptr.
WaveFn wave_fn(int K, int mode, int layout, int lean = 0);
typedef void (*BatchFn)(const BatchParams);
BatchFn batch_fn(int K, int mode, int layout, int lean = 0);  // batch_kernel<K, mode, layout, lean> or nullptr

// The splitting kernels take the text in tiles of LINE_TILE bytes per
// 1024-thread block; warp w of a block covers LINE_WARP consecutive bytes of
// its tile, 128 per step and 4 per lane, so no block-wide barrier runs inside
// a loop.  The text lies in a buffer with at least 3 bytes of slack past its
// end (every 4-byte word that starts inside it can be loaded) and starts
// 4-byte aligned.
constexpr uint32_t LINE_WARP = LINE_TILE / 32;

// Bit k set where byte k of the 4 at text[i] (i < bytes, i % 4 == 0) is c and
// lies inside the text.
__device__ __forceinline__ uint32_t byte_bits(const uint8_t *text, uint64_t bytes, uint64_t i, uint32_t c) {
  const uint32_t w = *reinterpret_cast<const uint32_t *>(text + i);
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) m |= (uint32_t)(((w >> (8 * k)) & 0xffu) == c) << k;
  const uint64_t left = bytes - i;
  return left >= 4 ? m : m & ((1u << left) - 1u);
}

// Newlines of the warp's segment starting at byte w0 (every lane gets the count).
__device__ __forceinline__ uint32_t warp_newlines(const uint8_t *text, uint64_t bytes, uint64_t w0, uint32_t lane) {
  uint32_t c = 0;
#pragma unroll 4
  for (uint32_t k = 0; k < LINE_WARP; k += 128) {
    const uint64_t i = w0 + k + 4 * lane;
    if (i < bytes) c += __popc(byte_bits(text, bytes, i, '\n'));
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  return c;
}

// Newlines before each warp's segment: block_offsets (exclusive scan of the
// per-tile counts) plus the tile's earlier warps.
__device__ __forceinline__ uint32_t warp_newline_base(const uint8_t *text, uint64_t bytes,
                                                      const uint32_t *block_offsets, uint64_t w0, uint32_t lane,
                                                      uint32_t wid, uint32_t *wsum) {
  const uint32_t c = warp_newlines(text, bytes, w0, lane);
  if (lane == 0) wsum[wid] = c;
  __syncthreads();
  uint32_t x = wsum[lane];
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  return block_offsets[blockIdx.x] + __shfl_sync(0xffffffffu, x, wid) - c;
}

}  // namespace ish
