// host.h -- internal types of the host engine (not part of the C ABI): device
// buffers, query and record-set state, the context, and the helpers shared by
// the translation units of libish_gpu.so.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ish_gpu.h"
#include "kernels.cuh"

namespace ish {
namespace host {

// Injected allocation failure (ISH_OPT_FAULT_ALLOC): -1 disarmed, else the
// number of device allocations still to succeed before one fails.
extern std::atomic<int64_t> g_alloc_fault;
inline bool alloc_fault_fires() {
  if (g_alloc_fault.load(std::memory_order_relaxed) < 0) return false;
  return g_alloc_fault.fetch_sub(1) == 0;
}

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    if (alloc_fault_fires()) return cudaErrorMemoryAllocation;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T *as() const { return reinterpret_cast<T *>(p); }
};

struct WaveLayout {
  int G = 0, K = 0, d = 0, kp = 0, layout = 0;
  uint32_t prof_bytes = 0;  // profile rows, then (if remapped) the 256-byte code -> row table
  uint32_t remap_off = 0;   // byte offset of that table, 0: codes are rows
  DevBuf prof, hinit;
};

struct Query {
  int algo = 0, kind = 0, alphabet = 0, Q = 0, open = 0, ext = 0, ends = 0;
  int32_t max_score = 0;
  float thr = 0.f;
  std::vector<int8_t> M;
  std::vector<uint8_t> q;
  int mmin = 0, mmax = 0;
  int neg_limit = 0;
  // Profile rows: codes whose matrix rows agree on every query column share
  // one row (for ascii, every byte that is not in the query); rowmap[c] is the
  // row of code c, rep[r] a code of row r.
  int rows = 0;
  std::vector<uint8_t> rowmap, rep;
  DevBuf plain_prof, plain_hinit;
  bool plain_ready = false;
  std::map<long, WaveLayout> layouts;
  std::unique_ptr<Query> reverse;  // reversed query with swapped free ends (start finding)
  std::unique_ptr<Query> fixed_start;  // the query with its start fixed (windows past row 0, windows.cu)
  std::map<long, DevBuf> exact_prof;  // striped profiles of the exact kernels (exact.cu)
};

// Parameters and sequence of a query without its device state.
void compute_rows(Query &q);
inline void clone_params(const Query &src, Query &dst) {
  dst.algo = src.algo;
  dst.kind = src.kind;
  dst.alphabet = src.alphabet;
  dst.Q = src.Q;
  dst.open = src.open;
  dst.ext = src.ext;
  dst.ends = src.ends;
  dst.max_score = src.max_score;
  dst.thr = src.thr;
  dst.M = src.M;
  dst.q = src.q;
  dst.mmin = src.mmin;
  dst.mmax = src.mmax;
  dst.neg_limit = src.neg_limit;
  dst.rows = src.rows;
  dst.rowmap = src.rowmap;
  dst.rep = src.rep;
}

// Window view of a record set (windows.cu): its long records cut into
// overlapping windows, the rest whole, longest first.
struct WindowView {
  uint64_t W = 0, O = 0;      // window stride and overlap (rows)
  uint32_t entries = 0;       // sorted entries covered
  uint32_t nw = 0;            // windows (slots)
  uint32_t n_first = 0;       // view entries [0, n_first) start at record row 0, the rest later
  uint64_t total = 0;         // rows over all windows
  uint32_t max_len = 0;
  DevBuf off, len, slot;      // per view entry (longest first): code offset, rows, slot
  DevBuf start, cs;           // per slot: first record row; per entry: first slot (n + 1)
  void release() {
    DevBuf *b[] = {&off, &len, &slot, &start, &cs};
    for (DevBuf *x : b) x->release();
    nw = 0;
  }
};

// Per-window results of the last windowed pass (windows.cu).
struct WindowOut {
  DevBuf score, qend, tend, hit;
  void release() {
    score.release();
    qend.release();
    tend.release();
    hit.release();
  }
};

struct RecordSet {
  bool pending = false;  // loaded asynchronously: its host-side summary is not read back yet
  uint32_t n = 0;
  uint64_t total = 0;
  uint32_t max_len = 0;
  DevBuf codes, off_s, len_s, orig_s;
  std::vector<uint32_t> hist;  // length-bucket histogram (host copy) up to the largest bucket used
  uint32_t n_empty = 0;
  uint32_t max_code = 0;       // largest record code in the set
  DevBuf inv;                  // sorted entry of each original record (built on first use)
  WindowView windows;          // built on first windowed pass
};

// The largest length bucket a set's histogram holds (the buckets above it
// have no records).
inline uint32_t top_bucket(const RecordSet &rs) { return rs.hist.empty() ? 0u : (uint32_t)rs.hist.size() - 1; }

struct Regime {
  bool fast = false;
  uint64_t max_safe_len = 0;  // records longer than this need the exact path
};

// Scratch, rerun flags and work counter of the exact kernels (exact.cu); a
// batched plan and the serving loop own theirs, so captured graphs and
// concurrent steps never share them.
struct ExactRes {
  DevBuf scratch, redo, counter;
  void release() {
    scratch.release();
    redo.release();
    counter.release();
  }
};

// Scratch of the FASTA/FASTQ splitter (fastx.cu): per line, per record.
struct FastxScratch {
  DevBuf hc, len, src, hdr, pos, rec, role, tiles, scan, totals, rec_off, bounds, flags, seq;
  void release() {
    DevBuf *b[] = {&hc, &len, &src, &hdr, &pos, &rec, &role, &tiles, &scan, &totals, &rec_off, &bounds, &flags, &seq};
    for (DevBuf *x : b) x->release();
  }
};

struct MultiPlan;  // multi.cu
struct Server;     // serve.cu
struct Tuned {
  int G = 0, K = 0, layout = -1;  // layout: -1 = the layout rule (choose_layout), else forced
};

}  // namespace host
}  // namespace ish

struct ish_ctx {
  int device = 0;
  int num_sms = 0;
  size_t mem_total = 0;  // device memory (bytes)
  cudaStream_t stream = nullptr;
  cudaStream_t load_stream = nullptr;  // asynchronous record loads (ish_gpu_records_load_async)
  cudaEvent_t load_done = nullptr;     // end of the asynchronous load in flight
  uint32_t *h_summary = nullptr;       // pinned: its largest code, largest bucket, then the histogram
  uint64_t *h_small = nullptr;         // pinned: small results read back by a call (error flags, counts)
  int32_t pending_set = 0;             // the set whose asynchronous load is in flight (0: none)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t load_ev[3] = {nullptr, nullptr, nullptr};  // last load: start, packing start, end
  double last_load_ms[3] = {0, 0, 0};                    // upload (+ splitting), packing, host wall
  // a load's records' bytes travel on copy_stream, after its offsets
  // (off_ev), while the packing kernels that need only the offsets run;
  // raw_ev marks the end of that upload
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t raw_ev = nullptr;
  cudaEvent_t off_ev = nullptr;  // the offsets are on the device
  bool raw_overlapped = false;  // the last load used copy_stream
  std::string err;
  int kernel = ISH_KERNEL_AUTO;
  int sg_lanes = 8, sw_u8_lanes = 16, sw_u16_lanes = 8;
  int force_G = 0, force_K = 0, force_layout = -1;
  int force_blocks = 0;  // cap on wavefront blocks per SM (0: occupancy limit)
  int force_lean = -1;   // lean kernel variant: -1 per (K, mode) default, 0 off, 1 on
  int windows_on = 1;    // window long records (windows.cu)
  double serve_step_cells = 1.25e11;  // ISH_OPT_SERVE_STEP_CELLS
  uint64_t step_budget = 0;  // ISH_OPT_STEP_BUDGET: cap on pipeline steps per warp (0: the launch's own bound)
  std::map<int32_t, ish::host::Query> queries;
  int32_t next_query = 1;
  std::map<int32_t, ish::host::RecordSet> sets;
  // device buffers of recently freed record sets, reused by the next load
  // (a load/score/free cycle per batch then allocates nothing)
  std::vector<ish::host::RecordSet> spare_sets;
  int32_t next_set = 1;
  // scratch
  ish::host::DevBuf raw, off_in, len_tmp, poff_tmp, hist, scan_tmp, summary;
  bool pack_dirty = true;  // the packing accumulators need clearing before the next load
  ish::host::DevBuf counter, error, out_score, out_qend, out_tend, out_hit, hit_idx, block_counts, nhits;
  ish::host::DevBuf plain_scratch;
  ish::host::DevBuf enc_tables, nl_pos, line_end;  // encoding tables; line splitting scratch
  ish::host::FastxScratch fastx;                    // FASTA/FASTQ splitting scratch (fastx.cu)
  ish::host::ExactRes exact;                        // exact kernels (exact.cu)
  ish::host::WindowOut window_out;                  // windowed passes (windows.cu)
  uint32_t last_windows = 0;                        // windows of the last windowed pass
  float last_ms = 0.f;
  // batched launches (multi.cu): plans cached per (queries, set, outputs)
  std::map<std::string, ish::host::MultiPlan *> plans;
  // autotuner results: (mode, alphabet, query length) -> shape
  std::map<uint64_t, ish::host::Tuned> tuned;
  // the serving loop (serve.cu), if started
  ish::host::Server *server = nullptr;
  // kernels launched by the library on this context (graph replays count
  // their kernel nodes; the serving thread adds its own)
  std::atomic<uint64_t> launches{0};
};


namespace ish {
namespace host {

int fail(ish_ctx *c, int code, const char *fmt, ...);
extern thread_local std::string g_open_error;

// Host wall time of a record-load call, kept for ish_gpu_last_load_ms.
struct LoadTimer {
  ish_ctx *ctx;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  explicit LoadTimer(ish_ctx *c) : ctx(c) {}
  ~LoadTimer() {
    ctx->last_load_ms[2] =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
};

// A failed runtime call also leaves the runtime's last-error state set;
// it is cleared here so that the next call does not report it again.
#define CU(call)                                                                                   \
  do {                                                                                             \
    cudaError_t _e = (call);                                                                       \
    if (_e != cudaSuccess) {                                                                       \
      (void)cudaGetLastError();                                                                    \
      return ::ish::host::fail(ctx, _e == cudaErrorMemoryAllocation ? ISH_ENOMEM : ISH_EDEVICE,     \
                               "%s: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__); \
    }                                                                                              \
  } while (0)

inline uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

int frame_rows(int ext);
int wave_lean(const ish_ctx *ctx, int K, int mode, int G);
int batch_lean(const ish_ctx *ctx, int K, int mode, int G);
uint64_t window_overlap(const Query &q);
int launch_windows(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t nonempty, OutDev out, cudaStream_t s, bool *done);
uint64_t window_stride(const ish_ctx *ctx, const RecordSet &rs, uint64_t O, int G, int K, int mode);
int build_window_view(ish_ctx *ctx, const RecordSet &rs, uint32_t nonempty, uint64_t W, uint64_t O, WindowView &V,
                      cudaStream_t s);
RecordSet window_set(const RecordSet &rs, const WindowView &V);
int merge_windows(ish_ctx *ctx, const RecordSet &rs, uint32_t nonempty, const WindowView &V, const Query &q,
                  const int32_t *ws, const int32_t *wq, const int32_t *wt, OutDev out, cudaStream_t s,
                  uint32_t *kernels);
bool windowable_whole(const Query &q);  // the query runs windows past row 0 as it is (no fixed-start twin)
Regime regime(const Query &q, int qpad);
void release_query(Query &q);
void release_set(RecordSet &rs);
void recycle_set(ish_ctx *ctx, RecordSet &rs);
void take_spare_set(ish_ctx *ctx, RecordSet &rs, size_t codes_bytes);
int wave_k_available(int k);
// Shape of the wavefront kernel for a query: the autotuner's choice when one
// exists, else the cost model; forced options override both.
void pick_shape(ish_ctx *ctx, const Query &q, int *G, int *K, int *layout);
void choose_shape(int Q, int force_G, int force_K, int *G, int *K);
uint64_t tune_key(int mode, int alphabet, int Q);
int layout_stride(int layout, int K);
size_t layout_bytes(int layout, int alphabet, int G, int K);
int choose_layout(int alphabet, int G, int K, int mode);
int build_wave_layout(ish_ctx *ctx, Query &q, int G, int K, int layout, WaveLayout **out);
int load_records(ish_ctx *ctx, const uint8_t *records, const uint64_t *offsets, uint32_t n, RecordSet &rs,
                 const uint8_t *enc, cudaStream_t s = nullptr, bool defer = false);
// Sorts and packs the n records in ctx->raw ([off_in[i], end[i]) or, with end
// NULL, [off_in[i], off_in[i + 1])) into rs on stream s (NULL: the context's
// stream).  defer: the host-side summary of the set (histogram, largest code)
// is read back when the set is first used (finish_pending_load), not now.
int pack_set(ish_ctx *ctx, uint32_t n, uint64_t raw_bytes, const uint64_t *end, const uint8_t *enc, RecordSet &rs,
             cudaStream_t s = nullptr, bool defer = false, bool raw_pending = false);
// Device phases of the last load (ish_gpu_last_load_ms).
void load_phase_times(ish_ctx *ctx);
// A set's host-side summary from {largest code, largest bucket, counts}.
void set_summary(RecordSet &rs, const uint32_t *h);
// Completes an asynchronous load in flight (ish_gpu_records_load_async), if any.
int finish_pending_load(ish_ctx *ctx);
// The set, with its asynchronous load completed; nullptr (and the error) if
// the id is unknown or the load failed.
RecordSet *use_set(ish_ctx *ctx, int32_t set_id, int *rc);
int load_lines(ish_ctx *ctx, const uint8_t *text, uint64_t bytes, RecordSet &rs, const uint8_t *enc, uint32_t *n_out);
int device_encoding(ish_ctx *ctx, int kind, const uint8_t **out);
void encoding_table(int kind, uint8_t t[256]);
uint32_t count_longer(const RecordSet &rs, uint64_t len);
// Checks that query q may run on the wavefront kernels against set rs with
// shape (G, K): 0 or a status with the reason in msg.  check_fast picks the
// shape and records the reason as the context's error.
int fast_check(const Query &q, const RecordSet &rs, int G, int K, char *msg, size_t len);
int check_fast(ish_ctx *ctx, const Query &q, const RecordSet &rs);
// Fills the per-query part of the wavefront parameters (not first/count/counter).
void wave_params(const Query &q, const WaveLayout &L, const RecordSet &rs, OutDev out, int *error, WaveParams *p);
int launch_wave_range(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t first, uint32_t count, OutDev out, int G, int K,
                      int layout, cudaStream_t s);
bool wave_fits(const Query &q, int G, int K, int layout);
// Whether the wavefront kernels compute the reference's exact results for q on
// rs (the safe regime); the exact kernels (exact.cu) take the rest.
bool fast_regime(ish_ctx *ctx, const Query &q, const RecordSet &rs);
int launch_exact(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t first, uint32_t count, OutDev out, cudaStream_t s);
int exact_prepare(ish_ctx *ctx, Query &q, uint32_t count, ExactRes &res);
int exact_enqueue(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t first, uint32_t count, OutDev out, cudaStream_t s,
                  ExactRes &res, uint32_t *launches);
int launch_range(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t first, uint32_t count, OutDev out, cudaStream_t s);
void drop_plans(ish_ctx *ctx, int32_t query_id, int32_t set_id);  // multi.cu
void free_plans(ish_ctx *ctx);                                   // multi.cu
void stop_server(ish_ctx *ctx);                                  // serve.cu
bool server_uses_set(const ish_ctx *ctx, int32_t set_id);        // serve.cu
size_t wave_smem(uint32_t prof_area, int threads, int G, int K, int mode);

}  // namespace host
}  // namespace ish
