// ish_gpu.cu -- host side of libish_gpu.so: the C ABI declared in
// include/ish_gpu.h.  It owns device memory, pinned staging and the engine
// stream, packs record sets in HBM, builds query profiles and picks and
// launches the scoring kernels.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "host.h"

using namespace ish;

using namespace ish::host;

namespace ish {
namespace host {

thread_local std::string g_open_error;
std::atomic<int64_t> g_alloc_fault{-1};

int fail(ish_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  else g_open_error = buf;
  return code;
}

void release_query(Query &q) {
  q.plain_prof.release();
  q.plain_hinit.release();
  for (auto &l : q.layouts) {
    l.second.prof.release();
    l.second.hinit.release();
  }
  q.layouts.clear();
  for (auto &kv : q.exact_prof) kv.second.release();
  q.exact_prof.clear();
  if (q.reverse) release_query(*q.reverse);
  q.reverse.reset();
  if (q.fixed_start) release_query(*q.fixed_start);
  q.fixed_start.reset();
}

void release_set(RecordSet &rs) {
  DevBuf *b[] = {&rs.codes, &rs.off_s, &rs.len_s, &rs.orig_s, &rs.inv};
  for (DevBuf *x : b) x->release();
  rs.windows.release();
}

// Freed sets keep their device buffers for the next load: at most two sets,
// each with packed codes under a sixteenth of device memory (at least 1 GiB),
// so the cache stays small next to HBM; an allocation that fails gives the
// cached buffers back first (pack_set).
static constexpr size_t kSpareSets = 2;
static size_t spare_codes_max(const ish_ctx *ctx) { return std::max<size_t>(size_t(1) << 30, ctx->mem_total / 16); }

void recycle_set(ish_ctx *ctx, RecordSet &rs) {
  rs.inv.release();  // rebuilt on first use by the next set
  rs.windows.release();
  if (!rs.codes.p || rs.codes.cap > spare_codes_max(ctx)) {
    release_set(rs);
    return;
  }
  if (ctx->spare_sets.size() >= kSpareSets) {
    release_set(ctx->spare_sets.front());
    ctx->spare_sets.erase(ctx->spare_sets.begin());
  }
  RecordSet keep;
  keep.codes = rs.codes;
  keep.off_s = rs.off_s;
  keep.len_s = rs.len_s;
  keep.orig_s = rs.orig_s;
  ctx->spare_sets.push_back(keep);
  rs.codes = rs.off_s = rs.len_s = rs.orig_s = DevBuf{};
}

// Hands `rs` the spare buffers with the smallest code area that holds
// codes_bytes (buffers that are still too small grow in DevBuf::ensure).
void take_spare_set(ish_ctx *ctx, RecordSet &rs, size_t codes_bytes) {
  if (rs.codes.p || ctx->spare_sets.empty()) return;
  size_t pick = ctx->spare_sets.size();
  for (size_t i = 0; i < ctx->spare_sets.size(); ++i) {
    const size_t cap = ctx->spare_sets[i].codes.cap;
    if (cap >= codes_bytes && (pick == ctx->spare_sets.size() || cap < ctx->spare_sets[pick].codes.cap)) pick = i;
  }
  if (pick == ctx->spare_sets.size()) return;
  RecordSet &sp = ctx->spare_sets[pick];
  rs.codes = sp.codes;
  rs.off_s = sp.off_s;
  rs.len_s = sp.len_s;
  rs.orig_s = sp.orig_s;
  ctx->spare_sets.erase(ctx->spare_sets.begin() + pick);
}

void compute_rows(Query &q) {
  const int A = q.alphabet;
  q.rowmap.assign(256, 0);
  q.rep.clear();
  std::map<std::vector<int8_t>, int> seen;
  std::vector<int8_t> key(q.Q);
  for (int c = 0; c < A; ++c) {
    for (int j = 0; j < q.Q; ++j) key[j] = q.M[(size_t)c * A + q.q[j]];
    auto it = seen.find(key);
    if (it == seen.end()) {
      it = seen.emplace(key, (int)q.rep.size()).first;
      q.rep.push_back((uint8_t)c);
    }
    q.rowmap[c] = (uint8_t)it->second;
  }
  q.rows = (int)q.rep.size();
}

int matrix_alphabet_ok(uint32_t alphabet) { return alphabet >= 1 && alphabet <= 256; }

// Safe-regime checks (see engine.cuh): the fast kernels evaluate plain Gotoh
// in 16-bit lanes; the result equals the reference's striped int16 pass when
// gap_open > gap_extend and no lane value of the reference can saturate or
// wrap.  Bounds are conservative.

// Semi-global rows are held in frames that rise by ext per row and drop back
// to 0 every R rows, R a power of two with R * ext <= 2048 (the headroom the
// regime keeps above the largest score).
// Whether (K, mode) runs the lean kernel variant (128 x 2 blocks with more
// registers instead of 128 x 3, whose parameters come from shared memory),
// as measured on GB300 for the protein search (blosum62, 400k records,
// G = 8, Q = 8K - 2): lean is ahead for semi-global at K = 34..40 (+0.5 to
// +5.7 %) and local at 34..38 (+1.3 to +2.4 %), behind from there on (up to
// -15 %).
int wave_lean(const ish_ctx *ctx, int K, int mode, int G) {
  if (!wave_has_lean(K)) return 0;
  if (ctx->force_lean >= 0) return ctx->force_lean;
  // Measured per K (protein records, Q = G * K - 2).  G <= 8 (200k records):
  // the 128 x 3 build beats 256 x 2 from K = 27 (semi-global) / 30 (local)
  // on, by up to 16 %; from K = 34 the 128 x 3 default build beats the 128 x
  // 2 lean one by 3-19 % up to K = 44, and loses at 46-48.  Wider groups
  // (300k records): at G = 32 the 256 x 2 build wins up to K = 30 (by 7-20 %)
  // and ties at K = 32; at G = 16 the lean build wins from K = 44
  // (semi-global, +7 %) / 40 (local, +15 %; 2.6x at K = 48).
  if (G <= 8) {
    if (K <= 32) return mode == SW ? K >= 30 : K >= 27;
    return K >= 46;
  }
  if (K <= 32) return mode == SG && K == 32 && G >= 32;
  return mode == SW ? K >= 40 : K >= 44;
}

// The same choice for the batched kernel (parameters in shared memory, one
// more live pointer), measured the same way through ish_gpu_score_multi.
// G <= 8: the 128 x 3 build wins everywhere but local alignment at K = 36
// (+2.0 %) and K = 48 (+6.7 %); the lean build loses 12-17 % from K = 38 on.
// Wider groups: at G = 32 the lean build wins semi-global K = 32 (+10 %),
// the default one K = 26-30; at G = 16 the lean build wins from K = 44
// (semi-global) / 36 (local, 2.9x at K = 48).  G is the class's narrowest.
int batch_lean(const ish_ctx *ctx, int K, int mode, int G) {
  if (!wave_has_lean(K)) return 0;
  if (ctx->force_lean >= 0) return ctx->force_lean;
  if (G <= 8) {
    if (K <= 32) return 0;
    return mode == SW && (K == 36 || K == 48);
  }
  if (K <= 32) return mode == SG && K == 32 && G >= 32;
  return mode == SW ? K >= 36 : K >= 44;
}

int frame_rows(int ext) {
  int R = 1;
  while (R < (1 << 20) && (long)2 * R * std::max(ext, 1) <= 2048) R *= 2;
  return R;
}

Regime regime(const Query &q, int qpad) {
  Regime r;
  if (q.Q == 0) return r;
  if (!(q.open > q.ext) || q.ext < 0) return r;
  const long top = (long)(q.Q + 1) * std::max(q.mmax, 1);
  if (top > 30000) return r;
  if (q.algo == ISH_ALGO_LOCAL) {
    r.fast = true;
    r.max_safe_len = ~0ull;
    return r;
  }
  if (q.open + q.ext > 10000) return r;
  if (frame_rows(q.ext) < WAVE_RPS_SG) return r;  // row frames reset at step boundaries (see frame_rows)
  const long base = 2L * q.open + (long)q.ext * (qpad + 3) + std::abs(q.mmin) + 64;
  if (base > 30000) return r;
  r.fast = true;
  if (q.ends & ISH_FREE_TARGET_START) {
    r.max_safe_len = ~0ull;
  } else {
    const long room = 30000 - base - q.open;
    r.max_safe_len = q.ext > 0 ? (uint64_t)(room / q.ext) : ~0ull;
  }
  return r;
}

int neg_limit_of(int open, int mmin) {
  // v_neg_limit (ishlib/matcher/alignment/semi_global_aln/striped.mojo:329-334)
  const int16_t o = (int16_t)open;
  if ((int16_t)(-o) < (int16_t)mmin) return (int16_t)(-32768 + o + 1);
  return (int16_t)(-32768 - mmin + 1);
}

// Columns per thread (K) and threads per group (G) for a query length: the
// smallest modelled cost with G*K >= Q + 1.  Per thread-row the kernel spends
// about five DPX instructions per column plus ~50 instructions of fixed work
// (pipeline, codes, tracking), i.e. ROW_OVERHEAD column-equivalents; K <= 48
// keeps 12-16 warps per SM, wider rows run at 8 (charged 25% more).  Kernels
// exist for every K <= 32 and even K up to 64.
int wave_k_available(int k) { return (k >= 1 && k <= 32) || (k > 32 && k <= WAVE_KMAX && !(k & 1)); }

void choose_shape(int Q, int force_G, int force_K, int *G, int *K) {
  const double ROW_OVERHEAD = 8.0;
  double bestc = 1e30;
  int bg = 0, bk = 0;
  for (int g = 1; g <= 32; g <<= 1) {
    if (force_G && g != force_G) continue;
    int k = force_K ? force_K : (Q + 1 + g - 1) / g;
    if (!force_K && k > 32) k = (k + 1) & ~1;
    if (!wave_k_available(k) || g * k < Q + 1) continue;
    double c = (double)g * k * (1.0 + ROW_OVERHEAD / k);
    if (k > 48) c *= 1.25;
    if (c < bestc) {
      bestc = c;
      bg = g;
      bk = k;
    }
  }
  *G = bg;
  *K = bk;
}

// Autotuner key: mode, profile rows (the profile's size) and query length.
uint64_t tune_key(int mode, int rows, int Q) { return ((uint64_t)mode << 48) | ((uint64_t)rows << 32) | (uint32_t)Q; }

// Row stride (in words) of a profile layout.  Strides are an odd number of
// 16-byte units: the eight threads of a quarter-warp read consecutive rows
// with 16-byte loads, and an odd stride spreads them over all 32 banks.
int layout_stride(int layout, int K) {
  if (layout == PROF_S16) {
    int kp = (K + 7) & ~7;
    return ((kp / 8) & 1) ? kp : kp + 8;
  }
  int kp = (K + 3) & ~3;
  return ((kp / 4) & 1) ? kp : kp + 4;
}

size_t layout_bytes(int layout, int alphabet, int G, int K) {
  const size_t kp = (size_t)layout_stride(layout, K);
  if (layout == PROF_PAIR) return (size_t)alphabet * alphabet * G * kp * 4;
  if (layout == PROF_S32) return (size_t)alphabet * G * kp * 4;
  return (size_t)alphabet * G * kp * 2;
}

// The pair layout (no per-column work to assemble a record pair's word) when
// it takes at most 64 KB; else 32-bit single-code words (one IMAD per column)
// when a block still fits twice on an SM; else 16-bit words (one PRMT).
int choose_layout(int alphabet, int G, int K, int mode) {
  if (layout_bytes(PROF_PAIR, alphabet, G, K) <= 64 * 1024) return PROF_PAIR;
  if (wave_smem((uint32_t)layout_bytes(PROF_S32, alphabet, G, K), wave_block_threads(K, mode), G, K, mode) <= 112 * 1024)
    return PROF_S32;
  return PROF_S16;
}

void pick_shape(ish_ctx *ctx, const Query &q, int *G, int *K, int *layout) {
  const int mode = q.algo == ISH_ALGO_LOCAL ? SW : SG;
  auto it = ctx->tuned.find(tune_key(mode, q.rows, q.Q));
  if (!ctx->force_G && !ctx->force_K && ctx->force_layout < 0 && it != ctx->tuned.end()) {
    *G = it->second.G;
    *K = it->second.K;
    *layout = it->second.layout >= 0 ? it->second.layout : choose_layout(q.rows, *G, *K, mode);
    return;
  }
  choose_shape(q.Q, ctx->force_G, ctx->force_K, G, K);
  *layout = ctx->force_layout >= 0 ? ctx->force_layout : (*G ? choose_layout(q.rows, *G, *K, mode) : PROF_S16);
}

int build_wave_layout(ish_ctx *ctx, Query &q, int G, int K, int layout, WaveLayout **out) {
  const long key = ((long)G << 20) | ((long)K << 8) | layout;
  auto it = q.layouts.find(key);
  if (it != q.layouts.end()) {
    *out = &it->second;
    return ISH_OK;
  }
  WaveLayout L;
  L.G = G;
  L.K = K;
  L.d = G * K - q.Q;
  L.layout = layout;
  L.kp = layout_stride(layout, K);
  // profile rows: one per class of codes with equal scores against the
  // query (q.rep), addressed through q.rowmap when the classes merge codes
  const int A = q.rows;
  const bool sg = q.algo == ISH_ALGO_SEMI_GLOBAL;
  const int ppad = (sg && !(q.ends & ISH_FREE_TARGET_START)) ? -(q.open + q.ext) : 0;
  // semi-global scores carry +ext: with row frames rising by ext per row,
  // H(i-1) in frame(i-1) plus P + ext lands in frame(i)
  const int pext = sg ? q.ext : 0;
  auto P = [&](int r, int col) -> int {
    if (col < 0) return ppad + pext;
    return q.M[(size_t)q.rep[r] * q.alphabet + q.q[col]] + pext;
  };
  std::vector<uint8_t> host;
  if (layout == PROF_PAIR) {
    std::vector<uint32_t> w((size_t)A * A * G * L.kp, 0u);
    for (int a = 0; a < A; ++a)
      for (int b = 0; b < A; ++b)
        for (int t = 0; t < G; ++t)
          for (int j = 0; j < K; ++j) {
            const int col = t * K + j - L.d;
            w[((size_t)(a * A + b) * G + t) * L.kp + j] =
                ((uint32_t)P(a, col) & 0xffffu) | ((uint32_t)(P(b, col) & 0xffff) << 16);
          }
    host.resize(w.size() * 4);
    memcpy(host.data(), w.data(), host.size());
  } else if (layout == PROF_S32) {
    std::vector<uint32_t> w((size_t)A * G * L.kp, 0u);
    for (int a = 0; a < A; ++a)
      for (int t = 0; t < G; ++t)
        for (int j = 0; j < K; ++j) w[((size_t)a * G + t) * L.kp + j] = (uint32_t)P(a, t * K + j - L.d) & 0xffffu;
    host.resize(w.size() * 4);
    memcpy(host.data(), w.data(), host.size());
  } else {
    std::vector<int16_t> w((size_t)A * G * L.kp, 0);
    for (int a = 0; a < A; ++a)
      for (int t = 0; t < G; ++t)
        for (int j = 0; j < K; ++j) w[((size_t)a * G + t) * L.kp + j] = (int16_t)P(a, t * K + j - L.d);
    host.resize(w.size() * 2);
    memcpy(host.data(), w.data(), host.size());
  }
  L.prof_bytes = (uint32_t)((host.size() + 15) & ~(size_t)15);
  host.resize(L.prof_bytes, 0);
  if (q.rows < q.alphabet) {
    L.remap_off = L.prof_bytes;
    host.insert(host.end(), q.rowmap.begin(), q.rowmap.end());
    L.prof_bytes += 256;
  }
  std::vector<int16_t> hin((size_t)G * K, 0);
  for (int c = 0; c < G * K; ++c) {
    const int col = c - L.d;
    int v = 0;
    if (sg && col >= 0 && !(q.ends & ISH_FREE_QUERY_START)) v = -q.open - q.ext * col;
    hin[c] = (int16_t)v;
  }
  CU(L.prof.ensure(L.prof_bytes));
  CU(L.hinit.ensure(hin.size() * 2));
  CU(cudaMemcpy(L.prof.p, host.data(), L.prof_bytes, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(L.hinit.p, hin.data(), hin.size() * 2, cudaMemcpyHostToDevice));
  auto res = q.layouts.emplace(key, std::move(L));
  *out = &res.first->second;
  return ISH_OK;
}

int build_plain(ish_ctx *ctx, Query &q) {
  if (q.plain_ready) return ISH_OK;
  const int A = q.alphabet;
  std::vector<int16_t> prof((size_t)A * q.Q + 8, 0);
  for (int c = 0; c < A; ++c)
    for (int col = 0; col < q.Q; ++col) prof[(size_t)c * q.Q + col] = q.M[(size_t)c * A + q.q[col]];
  std::vector<int16_t> hin(q.Q + 1, 0);
  if (q.algo == ISH_ALGO_SEMI_GLOBAL && !(q.ends & ISH_FREE_QUERY_START))
    for (int col = 0; col < q.Q; ++col) hin[col] = (int16_t)(-q.open - q.ext * col);
  CU(q.plain_prof.ensure(prof.size() * 2));
  CU(q.plain_hinit.ensure(hin.size() * 2));
  CU(cudaMemcpy(q.plain_prof.p, prof.data(), prof.size() * 2, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(q.plain_hinit.p, hin.data(), hin.size() * 2, cudaMemcpyHostToDevice));
  q.plain_ready = true;
  return ISH_OK;
}

// Byte -> code tables of ish's encodings (convert_ascii_to_encoding,
// ishlib/matcher/alignment/scoring_matrix.mojo:9-27 AA_TO_NUM, 131-149
// NT_TO_NUM): ascii is the identity; actgn / actgn0 map A/a C/c G/g T/t/U/u to
// 0-3 and everything else to 4 (N); blosum62 maps the 23 letters of its
// residue order (either case) to their index and everything else to 23 ('*').
void encoding_table(int kind, uint8_t t[256]) {
  if (kind == ISH_MATRIX_ASCII) {
    for (int i = 0; i < 256; ++i) t[i] = (uint8_t)i;
  } else if (kind == ISH_MATRIX_ACTGN || kind == ISH_MATRIX_ACTGN0) {
    memset(t, 4, 256);
    const char *groups[4] = {"Aa", "Cc", "Gg", "TtUu"};
    for (int code = 0; code < 4; ++code)
      for (const char *c = groups[code]; *c; ++c) t[(uint8_t)*c] = (uint8_t)code;
  } else {
    memset(t, 23, 256);
    const char *order = "ARNDCQEGHILKMFPSTWYVBZX*";
    for (int code = 0; order[code]; ++code) {
      const uint8_t c = (uint8_t)order[code];
      if (c >= 'A' && c <= 'Z') {
        t[c] = (uint8_t)code;
        t[c + 32] = (uint8_t)code;
      }
    }
  }
}

// Device copy of the encoding table of a matrix kind (nullptr: records are
// already encoded).
int device_encoding(ish_ctx *ctx, int kind, const uint8_t **out) {
  if (kind < ISH_MATRIX_ASCII || kind > ISH_MATRIX_BLOSUM62) return fail(ctx, ISH_EINVAL, "unknown matrix kind %d", kind);
  if (!ctx->enc_tables.p) {
    uint8_t t[4 * 256];
    for (int k = 0; k < 4; ++k) encoding_table(k, t + 256 * k);
    CU(ctx->enc_tables.ensure(sizeof t));
    CU(cudaMemcpy(ctx->enc_tables.p, t, sizeof t, cudaMemcpyHostToDevice));
  }
  *out = ctx->enc_tables.as<uint8_t>() + 256 * kind;
  return ISH_OK;
}

// Device phases of the last load for ish_gpu_last_load_ms: upload (with the
// splitting of a text load) and packing.  When the records' bytes travelled on
// the copy stream, the packing kernels that need only the offsets ran during
// the upload, and packing counts from the end of the upload.
void load_phase_times(ish_ctx *ctx) {
  float a = 0.f, b = 0.f;
  cudaEvent_t mid = ctx->raw_overlapped ? ctx->raw_ev : ctx->load_ev[1];
  if (cudaEventElapsedTime(&a, ctx->load_ev[0], mid) == cudaSuccess) ctx->last_load_ms[0] = a;
  if (cudaEventElapsedTime(&b, mid, ctx->load_ev[2]) == cudaSuccess) ctx->last_load_ms[1] = b;
  (void)cudaGetLastError();
}

// Sort and pack n records held in ctx->raw (raw_bytes bytes): record i is
// raw[off_in[i] .. end[i]) with `end` on the device, or raw[off_in[i] ..
// off_in[i + 1]) without; `enc` (device, may be null) encodes bytes on the way
// (see k_lengths .. k_pack in kernels.cu).  rs.total must hold the residue
// count.  The kernels run on s; with raw_pending the records' bytes are still
// on their way on the copy stream and only k_pack waits for them (raw_ev).
// With defer the host summary is copied into pinned staging and read when the
// set is first used (finish_pending_load).
int pack_set(ish_ctx *ctx, uint32_t n, uint64_t raw_bytes, const uint64_t *end, const uint8_t *enc, RecordSet &rs,
             cudaStream_t s, bool defer, bool raw_pending) {
  if (!s) s = ctx->stream;
  rs.n = n;
  const uint32_t tiles = ceil_div(n, SCAN_TILE);
  if (tiles > SCAN_TILE) return fail(ctx, ISH_EINVAL, "too many records in one set (%u)", n);
  CU(ctx->len_tmp.ensure((size_t)n * 4));
  CU(ctx->poff_tmp.ensure((size_t)n * 8));
  CU(ctx->scan_tmp.ensure((size_t)tiles * 8));
  // counts [NBUCKETS], descending cursors [NBUCKETS], the largest bucket and
  // the pack's long-record counter
  CU(ctx->hist.ensure((size_t)NBUCKETS * 4 * 2 + 16));
  uint32_t *counts = ctx->hist.as<uint32_t>(), *cursor = counts + NBUCKETS, *max_bucket = cursor + NBUCKETS;
  // what the host reads back: largest code, largest bucket, counts
  CU(ctx->summary.ensure((size_t)(2 + NBUCKETS) * 4));
  uint32_t *summary = ctx->summary.as<uint32_t>();
  CU(cudaEventRecord(ctx->load_ev[1], s));
  if (ctx->pack_dirty) {  // first load, or the last one stopped before k_scatter cleared the accumulators
    k_zero2<<<64, 1024, 0, s>>>(counts, NBUCKETS, max_bucket, 2);
    ++ctx->launches;
  }
  ctx->pack_dirty = true;
  uint64_t *tile_sum = ctx->scan_tmp.as<uint64_t>();
  k_lengths<<<tiles, 1024, 0, s>>>(ctx->off_in.as<uint64_t>(), end, n, ctx->len_tmp.as<uint32_t>(), tile_sum, counts,
                                   max_bucket, summary);
  ++ctx->launches;
  k_scan_slots<<<tiles, 1024, 0, s>>>(ctx->len_tmp.as<uint32_t>(), n, tile_sum, ctx->poff_tmp.as<uint64_t>());
  ++ctx->launches;
  k_bucket_cursors<<<BUCKET_BLOCKS, 1024, 0, s>>>(counts, max_bucket, cursor, summary);
  ++ctx->launches;
  const uint64_t packed = rs.total + 16ull * n + 16;
  take_spare_set(ctx, rs, packed);
  CU(rs.len_s.ensure((size_t)n * 4));
  CU(rs.off_s.ensure((size_t)n * 8));
  CU(rs.orig_s.ensure((size_t)n * 4));
  k_scatter<<<ceil_div(n, 1024), 1024, 0, s>>>(ctx->len_tmp.as<uint32_t>(), ctx->poff_tmp.as<uint64_t>(), n, cursor,
                                               rs.len_s.as<uint32_t>(), rs.off_s.as<uint64_t>(),
                                               rs.orig_s.as<uint32_t>(), counts, max_bucket, summary);
  ++ctx->launches;
  CU(cudaGetLastError());
  ctx->pack_dirty = false;
  {
    cudaError_t e = rs.codes.ensure(packed);
    if (e == cudaErrorMemoryAllocation && !ctx->spare_sets.empty()) {  // give the cached buffers back first
      (void)cudaGetLastError();
      for (RecordSet &sp : ctx->spare_sets) release_set(sp);
      ctx->spare_sets.clear();
      e = rs.codes.ensure(packed);
    }
    CU(e);
  }
  // lanes per record: the power of two nearest above the average 16-byte
  // chunks per record, 4 to 32
  uint32_t gw = 4;
  while (gw < 32 && (uint64_t)gw * 16 * n < rs.total) gw <<= 1;
  ctx->raw_overlapped = raw_pending;
  if (raw_pending) CU(cudaStreamWaitEvent(s, ctx->raw_ev, 0));  // the records' bytes are on the device
  // one group per record, or a block per 64 KB for sets of long records
  const uint32_t pb = (uint32_t)std::min<uint64_t>(
      std::max<uint64_t>(ceil_div((uint64_t)n * gw, 256), (rs.total >> 16) + 1), (uint64_t)ctx->num_sms * 3);
  k_pack<<<pb, 256, 0, s>>>(ctx->raw.as<uint8_t>(), raw_bytes, ctx->off_in.as<uint64_t>(), end,
                            ctx->poff_tmp.as<uint64_t>(), n, rs.len_s.as<uint32_t>(), rs.orig_s.as<uint32_t>(),
                            max_bucket + 1, enc, rs.codes.as<uint8_t>(), summary, gw);
  ++ctx->launches;
  CU(cudaGetLastError());
  CU(cudaEventRecord(ctx->load_ev[2], s));
  if (defer) {
    // the summary the host needs, read back when the set is first used
    CU(cudaMemcpyAsync(ctx->h_summary, summary, (size_t)(2 + NBUCKETS) * 4, cudaMemcpyDeviceToHost, s));
    CU(cudaEventRecord(ctx->load_done, s));
    rs.pending = true;
    return ISH_OK;
  }
  // host copy of the summary: the largest code and bucket and the counts of
  // the buckets of lengths below HIST_HEAD in one round trip, the rest (long
  // records only) after it
  constexpr uint32_t HIST_HEAD = 8192;
  uint32_t *h = ctx->h_summary;
  CU(cudaMemcpyAsync(h, summary, (size_t)(2 + HIST_HEAD) * 4, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  const uint32_t maxb = std::min<uint32_t>(h[1], NBUCKETS - 1);
  if (maxb >= HIST_HEAD) {
    CU(cudaMemcpyAsync(h + 2 + HIST_HEAD, summary + 2 + HIST_HEAD, (size_t)(maxb + 1 - HIST_HEAD) * 4,
                       cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
  }
  set_summary(rs, h);
  load_phase_times(ctx);
  return ISH_OK;
}

// A set's host-side summary from the device's {largest code, largest bucket,
// counts}; counts above the largest bucket are not read (they are zero).
void set_summary(RecordSet &rs, const uint32_t *h) {
  rs.max_code = h[0];
  const uint32_t maxb = std::min<uint32_t>(h[1], NBUCKETS - 1);
  rs.hist.assign(h + 2, h + 2 + maxb + 1);
  rs.n_empty = rs.hist[0];
  rs.max_len = maxb < 32768 ? maxb : (uint32_t)(32768 + ((uint64_t)(maxb - 32768) << 5) + 31);
}

// Upload and pack a record set given as concatenated records + n+1 offsets.
int load_records(ish_ctx *ctx, const uint8_t *records, const uint64_t *offsets, uint32_t n, RecordSet &rs,
                 const uint8_t *enc, cudaStream_t stream, bool defer) {
  if (n == 0) {
    rs.n = 0;
    rs.total = 0;
    return ISH_OK;
  }
  if (!offsets) return fail(ctx, ISH_EINVAL, "offsets is NULL");
  const uint64_t base = offsets[0], end = offsets[n];
  if (end < base) return fail(ctx, ISH_EINVAL, "offsets are not monotone");
  const uint64_t bytes = end - base;
  if (bytes && !records) return fail(ctx, ISH_EINVAL, "records is NULL");
  rs.total = bytes;
  cudaStream_t s = stream ? stream : ctx->stream;
  // The offsets go first on s; the records' bytes (+16 slack for the
  // realigning pack loads) follow on the copy stream once the offsets are in
  // (everything before this load on s, which includes the previous pack's
  // reads of the same buffer, is before that point too), while s computes
  // lengths, packed offsets and sorted positions.
  CU(ctx->raw.ensure(bytes + 32));
  CU(ctx->off_in.ensure((size_t)(n + 1) * 8));
  CU(cudaEventRecord(ctx->load_ev[0], s));
  std::vector<uint64_t> rebased;
  if (base) {
    rebased.assign(offsets, offsets + n + 1);
    for (auto &v : rebased) v -= base;
  }
  CU(cudaMemcpyAsync(ctx->off_in.p, base ? rebased.data() : offsets, (size_t)(n + 1) * 8, cudaMemcpyHostToDevice, s));
  CU(cudaEventRecord(ctx->off_ev, s));
  {
    cudaStream_t c = ctx->copy_stream;
    cudaError_t oe = cudaStreamWaitEvent(c, ctx->off_ev, 0);
    if (oe == cudaSuccess && bytes) oe = cudaMemcpyAsync(ctx->raw.p, records + base, bytes, cudaMemcpyHostToDevice, c);
    if (oe == cudaSuccess) oe = cudaEventRecord(ctx->raw_ev, c);
    if (oe != cudaSuccess) {
      cudaStreamSynchronize(c);  // the caller's buffers are free again on return
      cudaStreamSynchronize(s);
      CU(oe);
    }
  }
  if (base) CU(cudaEventSynchronize(ctx->off_ev));  // the rebased offsets are a temporary
  const int rc = pack_set(ctx, n, bytes, nullptr, enc, rs, s, defer, bytes != 0);
  if (rc && bytes) cudaStreamSynchronize(ctx->copy_stream);
  return rc;
}

// Completes the asynchronous load in flight: waits for its stream's work and
// fills the set's host-side summary from the pinned staging copy.
int finish_pending_load(ish_ctx *ctx) {
  if (!ctx->pending_set) return ISH_OK;
  const int32_t id = ctx->pending_set;
  ctx->pending_set = 0;
  auto it = ctx->sets.find(id);
  const cudaError_t e = cudaEventSynchronize(ctx->load_done);
  if (it == ctx->sets.end()) return ISH_OK;
  RecordSet &rs = it->second;
  rs.pending = false;
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    release_set(rs);
    ctx->sets.erase(it);
    return fail(ctx, ISH_EDEVICE, "asynchronous load of record set %d failed: %s (the set is gone)", id,
                cudaGetErrorString(e));
  }
  set_summary(rs, ctx->h_summary);
  load_phase_times(ctx);
  return ISH_OK;
}

RecordSet *use_set(ish_ctx *ctx, int32_t set_id, int *rc) {
  auto it = ctx->sets.find(set_id);
  if (it == ctx->sets.end()) {
    *rc = fail(ctx, ISH_EINVAL, "unknown record set %d", set_id);
    return nullptr;
  }
  if (it->second.pending) {
    *rc = finish_pending_load(ctx);
    if (*rc) return nullptr;
  }
  *rc = ISH_OK;
  return &it->second;
}

// Upload a text buffer, split it into lines on the device and pack the lines
// as records (see k_count_newlines .. k_line_bounds in kernels.cu).
int load_lines(ish_ctx *ctx, const uint8_t *text, uint64_t bytes, RecordSet &rs, const uint8_t *enc, uint32_t *n_out) {
  *n_out = 0;
  rs.n = 0;
  rs.total = 0;
  if (bytes == 0) return ISH_OK;
  if (!text) return fail(ctx, ISH_EINVAL, "text is NULL");
  cudaStream_t s = ctx->stream;
  CU(ctx->raw.ensure(bytes + 32));
  CU(cudaEventRecord(ctx->load_ev[0], s));
  CU(cudaMemcpyAsync(ctx->raw.p, text, bytes, cudaMemcpyHostToDevice, s));
  const uint64_t tiles64 = (bytes + LINE_TILE - 1) / LINE_TILE;
  if (tiles64 > 0x7fffffffull) return fail(ctx, ISH_EINVAL, "text too large");
  const uint32_t tiles = (uint32_t)tiles64;
  CU(ctx->block_counts.ensure((size_t)tiles * 4 + 8));
  CU(ctx->nhits.ensure(16));
  k_count_newlines<<<tiles, 1024, 0, s>>>(ctx->raw.as<uint8_t>(), bytes, ctx->block_counts.as<uint32_t>());
  ++ctx->launches;
  k_scan_counts<<<1, 1024, 0, s>>>(ctx->block_counts.as<uint32_t>(), tiles, ctx->nhits.as<uint32_t>());
  ++ctx->launches;
  uint32_t *hs = reinterpret_cast<uint32_t *>(ctx->h_small);
  CU(cudaMemcpyAsync(hs, ctx->nhits.p, 4, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  const uint32_t n_nl = hs[0];
  const uint8_t last = text[bytes - 1];
  const uint64_t lines = (uint64_t)n_nl + (last != '\n' ? 1 : 0);
  if (lines >= 0xffffffffull) return fail(ctx, ISH_EINVAL, "too many lines (%llu)", (unsigned long long)lines);
  const uint32_t n = (uint32_t)lines;
  CU(ctx->nl_pos.ensure((size_t)n_nl * 8 + 8));
  CU(ctx->off_in.ensure((size_t)(n + 1) * 8));
  CU(ctx->line_end.ensure((size_t)n * 8 + 8));
  k_write_newlines<<<tiles, 1024, 0, s>>>(ctx->raw.as<uint8_t>(), bytes, ctx->block_counts.as<uint32_t>(),
                                          ctx->nl_pos.as<uint64_t>());
  ++ctx->launches;
  CU(cudaMemsetAsync(ctx->nhits.p, 0, 16, s));
  k_line_bounds<<<std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(n, 256), (uint32_t)ctx->num_sms * 16)), 256, 0,
                  s>>>(ctx->raw.as<uint8_t>(), bytes, ctx->nl_pos.as<uint64_t>(), n_nl, n, ctx->off_in.as<uint64_t>(),
                       ctx->line_end.as<uint64_t>(), reinterpret_cast<unsigned long long *>(ctx->nhits.p));
  ++ctx->launches;
  CU(cudaGetLastError());
  // residues: the text minus the newlines and the dropped carriage returns
  CU(cudaMemcpyAsync(ctx->h_small, ctx->nhits.p, 8, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  rs.total = ctx->h_small[0];
  *n_out = n;
  return pack_set(ctx, n, bytes, ctx->line_end.as<uint64_t>(), enc, rs);
}

// Number of records (a prefix of the descending order) whose length bucket
// may exceed `len`.
uint32_t count_longer(const RecordSet &rs, uint64_t len) {
  uint64_t cnt = 0;
  for (uint32_t b = top_bucket(rs); b > 0; --b) {
    const uint64_t lo = b < 32768 ? b : 32768 + ((uint64_t)(b - 32768) << 5);
    const uint64_t hi = b < 32768 ? b : lo + 31;
    if (hi <= len) break;
    (void)lo;
    cnt += rs.hist[b];
  }
  return (uint32_t)cnt;
}

int ensure_outputs(ish_ctx *ctx, uint32_t n) {
  CU(ctx->out_score.ensure((size_t)n * 4 + 4));
  CU(ctx->out_qend.ensure((size_t)n * 4 + 4));
  CU(ctx->out_tend.ensure((size_t)n * 4 + 4));
  CU(ctx->out_hit.ensure((size_t)n + 16));
  CU(ctx->counter.ensure(64));
  CU(ctx->error.ensure(64));
  return ISH_OK;
}

void wave_params(const Query &q, const WaveLayout &L, const RecordSet &rs, OutDev out, int *error, WaveParams *pp) {
  WaveParams &p = *pp;
  p = WaveParams{};
  const int mode = q.algo == ISH_ALGO_LOCAL ? SW : SG;
  p.prof = L.prof.as<const uint4>();
  p.prof_bytes = L.prof_bytes;
  p.Q = q.Q;
  p.G = L.G;
  p.K = L.K;
  p.d = L.d;
  p.kp = L.kp;
  p.alphabet = q.rows;
  p.remap_off = L.remap_off;
  p.layout = L.layout;
  p.lane_mul = 65536u;
  p.open = q.open;
  p.ext = q.ext;
  p.ends = q.ends;
  p.neg_limit = q.neg_limit;
  const bool sg = mode == SG;
  p.hleft = (sg && !(q.ends & ISH_FREE_TARGET_START)) ? NEG_BIG : 0;
  p.fin = sg ? NEG_BIG : 0;
  p.frame_mask = sg ? frame_rows(q.ext) - 1 : 0x3fffffff;
  p.pk_nopen = dup16_host(-q.open);
  p.pk_next = dup16_host(-q.ext);
  p.pk_eopen = dup16_host(q.ext - q.open);
  p.pk_fsin = dup16_host(p.fin + q.open);
  p.pk_ext = sg ? (uint32_t)q.ext * 0x10001u : 0u;
  p.pk_drop = sg ? dup16_host(-(p.frame_mask + 1) * q.ext) : 0u;
  p.row_bytes = (uint32_t)(L.G * L.kp * (L.layout == PROF_S16 ? 2 : 4));
  p.hinit = L.hinit.as<const int16_t>();
  p.error = error;
  p.rec = RecordsDev{rs.codes.as<const uint8_t>(), rs.off_s.as<const uint64_t>(), rs.len_s.as<const uint32_t>(),
                     rs.orig_s.as<const uint32_t>(), rs.n};
  p.out = out;
  p.dec = Decision{q.max_score, q.thr};
}

// Shared memory of a wavefront block: the profile, 32 slot words per group,
// and (local alignment) wave_save_words(K) save words per thread (see wave.cuh).
size_t wave_smem(uint32_t prof_area, int threads, int G, int K, int mode) {
  const size_t save = mode == SW ? (size_t)threads * wave_save_words(K) * 4 : 0;
  return prof_area + (size_t)(threads / G) * 32 * 4 + save;
}

int launch_wave_range(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t first, uint32_t count, OutDev out, int G, int K,
                      int layout, cudaStream_t s) {
  if (count == 0) return ISH_OK;
  if (!G || G * K < q.Q + 1) return fail(ctx, ISH_EOVERFLOW, "no wavefront shape for a query of %d residues", q.Q);
  WaveLayout *L = nullptr;
  int rc = build_wave_layout(ctx, q, G, K, layout, &L);
  if (rc) return rc;
  const int mode = q.algo == ISH_ALGO_LOCAL ? SW : SG;
  const int lean = wave_lean(ctx, K, mode, G);
  WaveFn fn = wave_fn(K, mode, L->layout, lean);
  if (!fn) return fail(ctx, ISH_EOVERFLOW, "no wavefront kernel for K=%d", K);
  const int threads = wave_threads_lean(K, mode, lean);
  const int groups = threads / G;
  const size_t smem = wave_smem((L->prof_bytes + 15) & ~15u, threads, G, K, mode);
  {
    const cudaError_t e = cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      cudaFuncAttributes a{};
      const cudaError_t ea = cudaFuncGetAttributes(&a, (const void *)fn);
      (void)cudaGetLastError();
      return fail(ctx, ISH_EDEVICE,
                  "wavefront kernel K=%d mode=%d layout=%d: dynamic shared memory %zu bytes refused (%s); kernel "
                  "attributes (%s): static %zu, max dynamic %d, %d registers",
                  K, mode, L->layout, smem, cudaGetErrorString(e), cudaGetErrorString(ea), a.sharedSizeBytes,
                  a.maxDynamicSharedSizeBytes, a.numRegs);
    }
  }
  int per_sm = 0;
  CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)fn, threads, smem));
  if (per_sm < 1) return fail(ctx, ISH_EOVERFLOW, "wavefront kernel K=%d does not fit (smem %zu)", K, smem);
  if (ctx->force_blocks) per_sm = std::min(per_sm, ctx->force_blocks);
  const uint32_t pairs = (count + 1) / 2;
  const uint32_t want = ceil_div(pairs, groups);
  const uint32_t grid = std::max<uint32_t>(1, std::min<uint32_t>(want, (uint32_t)(per_sm * ctx->num_sms)));
  WaveParams p;
  wave_params(q, *L, rs, out, ctx->error.as<int>(), &p);
  p.first = first;
  p.count = count;
  p.counter = ctx->counter.as<uint32_t>();
  p.max_steps = ctx->step_budget ? ctx->step_budget : rs.total + 2ull * count + 1024;
  CU(cudaMemsetAsync(ctx->counter.p, 0, 4, s));
  fn<<<grid, threads, smem, s>>>(p);
  ++ctx->launches;
  CU(cudaGetLastError());
  return ISH_OK;
}

int launch_plain(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t first, uint32_t count, OutDev out) {
  if (count == 0) return ISH_OK;
  int rc = build_plain(ctx, q);
  if (rc) return rc;
  // the int16 form (the reference kernel's per-thread arrays and launch shape)
  // when asked for and the query fits its largest array; else int32 columns
  int qmax = 0;
  if (ctx->kernel == ISH_KERNEL_PLAIN16 && q.Q <= PLAIN16_QMAX)
    for (qmax = 64; qmax < q.Q; qmax <<= 1) {
    }
  const int threads = qmax ? 32 : 128;
  const uint32_t blocks =
      qmax ? ceil_div(PLAIN16_THREADS, threads)
           : std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(count, threads), (uint32_t)ctx->num_sms * 4));
  const uint32_t nth = qmax ? PLAIN16_THREADS : blocks * threads;
  if (!qmax) CU(ctx->plain_scratch.ensure((size_t)2 * q.Q * nth * 4 + 16));
  PlainParams p{};
  p.prof = q.plain_prof.as<const int16_t>();
  p.prof_bytes = (uint32_t)(((size_t)q.alphabet * q.Q * 2 + 15) & ~(size_t)15);
  p.use_smem = p.prof_bytes <= 96 * 1024;
  p.Q = q.Q;
  p.alphabet = q.alphabet;
  p.open = q.open;
  p.ext = q.ext;
  p.ends = q.ends;
  p.neg_limit = q.neg_limit;
  p.hinit = q.plain_hinit.as<const int16_t>();
  p.scratch = ctx->plain_scratch.as<int32_t>();
  p.nthreads = nth;
  p.first = first;
  p.count = count;
  p.error = ctx->error.as<int>();
  p.rec = RecordsDev{rs.codes.as<const uint8_t>(), rs.off_s.as<const uint64_t>(), rs.len_s.as<const uint32_t>(),
                     rs.orig_s.as<const uint32_t>(), rs.n};
  p.out = out;
  p.dec = Decision{q.max_score, q.thr};
  const size_t smem = p.use_smem ? p.prof_bytes : 0;
  PlainFn fn = plain_fn(q.algo == ISH_ALGO_LOCAL ? SW : SG, qmax);
  CU(cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(smem, 1)));
  fn<<<blocks, threads, smem, ctx->stream>>>(p);
  ++ctx->launches;
  CU(cudaGetLastError());
  return ISH_OK;
}

int fast_check(const Query &q, const RecordSet &rs, int G, int K, char *msg, size_t len) {
  Regime r = regime(q, G ? G * K : q.Q + 64);
  if (!r.fast) {
    snprintf(msg, len,
             "parameters outside the exact-integer fast regime (gap_open must exceed gap_extend and scores must stay "
             "within int16)");
    return ISH_EINVAL;
  }
  const uint32_t nonempty = rs.n - rs.n_empty;
  const uint32_t n_long = r.max_safe_len == ~0ull ? 0 : std::min(count_longer(rs, r.max_safe_len), nonempty);
  if (n_long) {
    snprintf(msg, len, "%u records are longer than %llu residues with a non-free target start", n_long,
             (unsigned long long)r.max_safe_len);
    return ISH_EINVAL;
  }
  if (rs.max_code >= (uint32_t)q.alphabet) {
    snprintf(msg, len, "a record contains code %u >= the alphabet size %d of the query", rs.max_code, q.alphabet);
    return ISH_EINVAL;
  }
  if (!G || G * K < q.Q + 1) {
    snprintf(msg, len, "no wavefront shape for a query of %d residues", q.Q);
    return ISH_EOVERFLOW;
  }
  return ISH_OK;
}

bool fast_regime(ish_ctx *ctx, const Query &q, const RecordSet &rs) {
  int G, K, layout;
  pick_shape(ctx, q, &G, &K, &layout);
  char msg[256];
  return fast_check(q, rs, G, K, msg, sizeof msg) == ISH_OK;
}

int check_fast(ish_ctx *ctx, const Query &q, const RecordSet &rs) {
  int G, K, layout;
  pick_shape(ctx, q, &G, &K, &layout);
  char msg[256];
  const int rc = fast_check(q, rs, G, K, msg, sizeof msg);
  return rc ? fail(ctx, rc, "%s", msg) : ISH_OK;
}

// Whether the wavefront kernel's shared memory (profile, code -> row table,
// slots, saved rows) fits in a block for this shape and layout.
bool wave_fits(const Query &q, int G, int K, int layout) {
  if (!G) return false;
  const int mode = q.algo == ISH_ALGO_LOCAL ? SW : SG;
  size_t prof = (layout_bytes(layout, q.rows, G, K) + 15) & ~(size_t)15;
  if (q.rows < q.alphabet) prof += 256;
  return wave_smem((uint32_t)prof, wave_block_threads(K, mode), G, K, mode) <= 227 * 1024;
}

// The wavefront kernel, or the plain kernel when the wavefront profile does
// not fit in shared memory (long queries over large alphabets) or the plain
// kernel was asked for.
int launch_range(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t first, uint32_t count, OutDev out, cudaStream_t s) {
  int G, K, layout;
  pick_shape(ctx, q, &G, &K, &layout);
  if (ctx->kernel == ISH_KERNEL_PLAIN || ctx->kernel == ISH_KERNEL_PLAIN16 || !wave_fits(q, G, K, layout)) {
    if (s != ctx->stream) return fail(ctx, ISH_EINVAL, "the plain kernel runs on the context stream only");
    return launch_plain(ctx, q, rs, first, count, out);
  }
  return launch_wave_range(ctx, q, rs, first, count, out, G, K, layout, s);
}

// Score query q against set rs into the context's device output buffers.
int run_scoring(ish_ctx *ctx, Query &q, RecordSet &rs) {
  const uint32_t n = rs.n;
  int rc = ensure_outputs(ctx, n);
  if (rc) return rc;
  cudaStream_t s = ctx->stream;
  CU(cudaMemsetAsync(ctx->error.p, 0, 4, s));
  OutDev out{ctx->out_score.as<int32_t>(), ctx->out_qend.as<int32_t>(), ctx->out_tend.as<int32_t>(),
             ctx->out_hit.as<uint8_t>()};
  const int mode = q.algo == ISH_ALGO_LOCAL ? SW : SG;
  const uint32_t n_empty = (q.Q == 0) ? n : rs.n_empty;
  const uint32_t nonempty = n - n_empty;
  CU(cudaEventRecord(ctx->ev0, s));
  if (n_empty) {
    k_trivial<<<std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(n_empty, 256), 1024)), 256, 0, s>>>(
        RecordsDev{rs.codes.as<const uint8_t>(), rs.off_s.as<const uint64_t>(), rs.len_s.as<const uint32_t>(),
                   rs.orig_s.as<const uint32_t>(), rs.n},
        nonempty, n_empty, mode, q.Q, out, Decision{q.max_score, q.thr});
    ++ctx->launches;
    CU(cudaGetLastError());
  }
  if (nonempty) {
    if (rs.max_code >= (uint32_t)q.alphabet)
      return fail(ctx, ISH_EINVAL, "a record contains code %u >= the alphabet size %d of the query", rs.max_code,
                  q.alphabet);
    if (ctx->kernel == ISH_KERNEL_EXACT || !fast_regime(ctx, q, rs)) {
      rc = launch_exact(ctx, q, rs, 0, nonempty, out, s);
    } else {
      bool windowed = false;
      ctx->last_windows = 0;
      rc = launch_windows(ctx, q, rs, nonempty, out, s, &windowed);
      if (!rc && !windowed) rc = launch_range(ctx, q, rs, 0, nonempty, out, s);
    }
    if (rc) return rc;
  }
  return ISH_OK;
}

int fetch_outputs(ish_ctx *ctx, uint32_t n, int32_t *score, int32_t *qend, int32_t *tend, uint8_t *hit,
                  uint32_t *hit_idx, uint32_t *n_hits) {
  cudaStream_t s = ctx->stream;
  const bool compact = (hit_idx || n_hits) && n;
  if (compact) {
    const uint32_t nb = ceil_div(n, HIT_TILE);
    CU(ctx->block_counts.ensure((size_t)nb * 4 + 8));
    CU(ctx->hit_idx.ensure((size_t)n * 4 + 4));
    CU(ctx->nhits.ensure(16));
    k_count_hits<<<nb, 1024, 0, s>>>(ctx->out_hit.as<uint8_t>(), n, ctx->block_counts.as<uint32_t>());
    ++ctx->launches;
    k_scan_counts<<<1, 1024, 0, s>>>(ctx->block_counts.as<uint32_t>(), nb, ctx->nhits.as<uint32_t>());
    ++ctx->launches;
    k_write_hits<<<nb, 1024, 0, s>>>(ctx->out_hit.as<uint8_t>(), n, ctx->block_counts.as<uint32_t>(),
                                     ctx->hit_idx.as<uint32_t>());
    ++ctx->launches;
    CU(cudaGetLastError());
  }
  CU(cudaEventRecord(ctx->ev1, s));
  if (n && score) CU(cudaMemcpyAsync(score, ctx->out_score.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  if (n && qend) CU(cudaMemcpyAsync(qend, ctx->out_qend.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  if (n && tend) CU(cudaMemcpyAsync(tend, ctx->out_tend.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  if (n && hit) CU(cudaMemcpyAsync(hit, ctx->out_hit.p, (size_t)n, cudaMemcpyDeviceToHost, s));
  // error flags and hit count into pinned staging, so that every copy of the
  // call stays asynchronous until the one synchronisation below
  uint32_t *hs = reinterpret_cast<uint32_t *>(ctx->h_small);
  hs[1] = 0;
  CU(cudaMemcpyAsync(hs, ctx->error.p, 4, cudaMemcpyDeviceToHost, s));
  if (compact) CU(cudaMemcpyAsync(hs + 1, ctx->nhits.p, 4, cudaMemcpyDeviceToHost, s));
  // the first hit indices travel with the count (hit_idx holds n entries, so
  // the prefix fits whatever the count); the rest, if any, after it
  constexpr uint32_t HIT_PREFIX = 4096;
  const uint32_t prefix = std::min<uint32_t>(n, HIT_PREFIX);
  if (hit_idx && compact) CU(cudaMemcpyAsync(hit_idx, ctx->hit_idx.p, (size_t)prefix * 4, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  const int herr = (int)hs[0];
  const uint32_t total = hs[1];
  if (hit_idx && total > prefix) {
    CU(cudaMemcpyAsync(hit_idx + prefix, ctx->hit_idx.as<uint32_t>() + prefix, (size_t)(total - prefix) * 4,
                       cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
  }
  if (n_hits) *n_hits = total;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) ctx->last_ms = ms;
  if (herr & 2) return fail(ctx, ISH_ETIMEDOUT, "wavefront kernel exceeded its step budget (internal error)");
  if (herr) return fail(ctx, ISH_EINVAL, "a record contains a code >= the alphabet size of the query");
  return ISH_OK;
}

}  // namespace host
}  // namespace ish

extern "C" {

int ish_gpu_abi_version(void) { return ISH_GPU_ABI_VERSION; }

int ish_gpu_open(int device, ish_ctx **out) {
  if (!out) return fail(nullptr, ISH_EINVAL, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(nullptr, ISH_ENODEV, "no CUDA device: %s", e == cudaSuccess ? "count is 0" : cudaGetErrorString(e));
  if (device < 0 || device >= ndev) return fail(nullptr, ISH_EINVAL, "device %d out of range (%d devices)", device, ndev);
  ish_ctx *ctx = new ish_ctx();
  ctx->device = device;
  auto bail = [&](cudaError_t err, const char *what) {
    g_open_error = std::string(what) + ": " + cudaGetErrorString(err);
    delete ctx;
    return ISH_EDEVICE;
  };
  if ((e = cudaSetDevice(device)) != cudaSuccess) return bail(e, "cudaSetDevice");
  if ((e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
    return bail(e, "cudaDeviceGetAttribute");
  {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) ctx->mem_total = total_b;
    (void)cudaGetLastError();
  }
  if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(e, "cudaStreamCreate");
  if ((e = cudaEventCreate(&ctx->ev0)) != cudaSuccess) return bail(e, "cudaEventCreate");
  if ((e = cudaEventCreate(&ctx->ev1)) != cudaSuccess) return bail(e, "cudaEventCreate");
  for (cudaEvent_t &ev : ctx->load_ev)
    if ((e = cudaEventCreate(&ev)) != cudaSuccess) return bail(e, "cudaEventCreate");
  if ((e = cudaStreamCreateWithFlags(&ctx->load_stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(e, "cudaStreamCreate");
  if ((e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(e, "cudaStreamCreate");
  if ((e = cudaEventCreate(&ctx->raw_ev)) != cudaSuccess) return bail(e, "cudaEventCreate");
  if ((e = cudaEventCreateWithFlags(&ctx->off_ev, cudaEventDisableTiming)) != cudaSuccess)
    return bail(e, "cudaEventCreate");
  if ((e = cudaEventCreateWithFlags(&ctx->load_done, cudaEventDisableTiming)) != cudaSuccess)
    return bail(e, "cudaEventCreate");
  if ((e = cudaHostAlloc((void **)&ctx->h_summary, (size_t)(2 + NBUCKETS) * 4, cudaHostAllocDefault)) != cudaSuccess)
    return bail(e, "cudaHostAlloc");
  if ((e = cudaHostAlloc((void **)&ctx->h_small, 64 * 8, cudaHostAllocDefault)) != cudaSuccess)
    return bail(e, "cudaHostAlloc");
  *out = ctx;
  return ISH_OK;
}

void ish_gpu_close(ish_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  stop_server(ctx);
  (void)finish_pending_load(ctx);
  cudaStreamSynchronize(ctx->stream);
  free_plans(ctx);
  for (auto &kv : ctx->queries) release_query(kv.second);
  for (auto &kv : ctx->sets) release_set(kv.second);
  for (RecordSet &sp : ctx->spare_sets) release_set(sp);
  DevBuf *bufs[] = {&ctx->raw, &ctx->off_in, &ctx->len_tmp, &ctx->poff_tmp, &ctx->hist, &ctx->summary,
                    &ctx->scan_tmp, &ctx->counter, &ctx->error, &ctx->out_score, &ctx->out_qend, &ctx->out_tend,
                    &ctx->out_hit, &ctx->hit_idx, &ctx->block_counts, &ctx->nhits, &ctx->plain_scratch,
                    &ctx->enc_tables, &ctx->nl_pos, &ctx->line_end};
  for (DevBuf *b : bufs) b->release();
  ctx->exact.release();
  ctx->window_out.release();
  ctx->fastx.release();
  cudaEventDestroy(ctx->ev0);
  cudaEventDestroy(ctx->ev1);
  cudaEventDestroy(ctx->load_done);
  cudaStreamDestroy(ctx->load_stream);
  if (ctx->raw_ev) cudaEventDestroy(ctx->raw_ev);
  if (ctx->off_ev) cudaEventDestroy(ctx->off_ev);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  cudaFreeHost(ctx->h_summary);
  if (ctx->h_small) cudaFreeHost(ctx->h_small);
  for (cudaEvent_t ev : ctx->load_ev) cudaEventDestroy(ev);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char *ish_gpu_last_error(const ish_ctx *ctx) { return ctx ? ctx->err.c_str() : g_open_error.c_str(); }

int ish_gpu_set_option(ish_ctx *ctx, int option, int64_t value) {
  if (!ctx) return ISH_EINVAL;
  // the serving thread reads the options for every step
  if (ctx->server) return fail(ctx, ISH_EINVAL, "options cannot change while the serving loop runs");
  switch (option) {
  case ISH_OPT_KERNEL:
    if (value < ISH_KERNEL_AUTO || value > ISH_KERNEL_PLAIN16)
      return fail(ctx, ISH_EINVAL, "bad kernel %lld", (long long)value);
    ctx->kernel = (int)value;
    return ISH_OK;
  case ISH_OPT_SG_LANES:
  case ISH_OPT_SW_U8_LANES:
  case ISH_OPT_SW_U16_LANES:
    if (value < 1 || value > 64) return fail(ctx, ISH_EINVAL, "lane count must be in 1..64");
    (option == ISH_OPT_SG_LANES ? ctx->sg_lanes : option == ISH_OPT_SW_U8_LANES ? ctx->sw_u8_lanes : ctx->sw_u16_lanes) =
        (int)value;
    return ISH_OK;
  case ISH_OPT_WAVE_GROUP:
    if (value != 0 && (value < 1 || value > 32 || (value & (value - 1))))
      return fail(ctx, ISH_EINVAL, "group size must be 0 or a power of two <= 32");
    ctx->force_G = (int)value;
    drop_plans(ctx, 0, 0);
    return ISH_OK;
  case ISH_OPT_PROFILE_LAYOUT:
    if (value < -1 || value > PROF_S32) return fail(ctx, ISH_EINVAL, "profile layout must be -1, 0, 1 or 2");
    ctx->force_layout = (int)value;
    drop_plans(ctx, 0, 0);
    return ISH_OK;
  case ISH_OPT_WAVE_K:
    if (value != 0 && !wave_k_available((int)value))
      return fail(ctx, ISH_EINVAL, "K must be 0, 1..32 or even up to %d", WAVE_KMAX);
    ctx->force_K = (int)value;
    drop_plans(ctx, 0, 0);
    return ISH_OK;
  case ISH_OPT_WINDOWS:
    if (value != 0 && value != 1) return fail(ctx, ISH_EINVAL, "windows must be 0 or 1");
    if (ctx->windows_on != (int)value) free_plans(ctx);  // batched plans window the set or not
    ctx->windows_on = (int)value;
    return ISH_OK;
  case ISH_OPT_WAVE_LEAN:
    if (value < -1 || value > 1) return fail(ctx, ISH_EINVAL, "lean variant must be -1, 0 or 1");
    ctx->force_lean = (int)value;
    drop_plans(ctx, 0, 0);
    return ISH_OK;
  case ISH_OPT_STEP_BUDGET:
    if (value < 0) return fail(ctx, ISH_EINVAL, "step budget must be >= 0");
    ctx->step_budget = (uint64_t)value;
    drop_plans(ctx, 0, 0);
    return ISH_OK;
  case ISH_OPT_SERVE_STEP_CELLS:
    if (value < 0) return fail(ctx, ISH_EINVAL, "serving step cells must be >= 0");
    ctx->serve_step_cells = (double)value;
    return ISH_OK;
  case ISH_OPT_FAULT_ALLOC:
    if (value < -1) return fail(ctx, ISH_EINVAL, "allocation fault countdown must be >= -1");
    g_alloc_fault.store(value);
    return ISH_OK;
  case ISH_OPT_WAVE_BLOCKS:
    if (value < 0 || value > 32) return fail(ctx, ISH_EINVAL, "blocks per SM must be in 0..32");
    ctx->force_blocks = (int)value;
    drop_plans(ctx, 0, 0);
    return ISH_OK;
  default:
    return fail(ctx, ISH_EINVAL, "unknown option %d", option);
  }
}

int ish_gpu_set_query(ish_ctx *ctx, const uint8_t *enc_query, uint32_t qlen, int matrix_kind, const int8_t *matrix,
                      uint32_t alphabet, int algo, uint32_t gap_open, uint32_t gap_ext, uint32_t ends_free,
                      int32_t max_score, float threshold, int32_t *query_id) {
  if (!ctx || !query_id) return ctx ? fail(ctx, ISH_EINVAL, "query_id is NULL") : ISH_EINVAL;
  if (algo != ISH_ALGO_SEMI_GLOBAL && algo != ISH_ALGO_LOCAL) return fail(ctx, ISH_EINVAL, "unknown algorithm %d", algo);
  if (matrix_kind < ISH_MATRIX_ASCII || matrix_kind > ISH_MATRIX_BLOSUM62)
    return fail(ctx, ISH_EINVAL, "unknown matrix kind %d", matrix_kind);
  if (!matrix || !matrix_alphabet_ok(alphabet)) return fail(ctx, ISH_EINVAL, "matrix must be alphabet^2 int8, alphabet 1..256");
  if (qlen && !enc_query) return fail(ctx, ISH_EINVAL, "enc_query is NULL");
  if (qlen > 32767) return fail(ctx, ISH_EOVERFLOW, "query of %u residues is longer than 32767", qlen);
  if (ends_free > 15) return fail(ctx, ISH_EINVAL, "ends_free has bits above ISH_FREE_TARGET_END");
  Query q;
  q.algo = algo;
  q.kind = matrix_kind;
  q.alphabet = (int)alphabet;
  q.Q = (int)qlen;
  // The matchers hand UInt penalties to lanes of the pass type: int16 for the
  // semi-global pass (striped_semi_global_matcher.mojo:232-245), uint8 for
  // ssw_align (local_aln/striped.mojo:151-152).
  if (algo == ISH_ALGO_SEMI_GLOBAL) {
    q.open = (int16_t)gap_open;
    q.ext = (int16_t)gap_ext;
  } else {
    q.open = (uint8_t)gap_open;
    q.ext = (uint8_t)gap_ext;
  }
  q.ends = algo == ISH_ALGO_SEMI_GLOBAL ? (int)ends_free : 0;
  q.max_score = max_score;
  q.thr = threshold;
  q.M.assign(matrix, matrix + (size_t)alphabet * alphabet);
  q.q.assign(enc_query, enc_query + qlen);
  for (uint32_t i = 0; i < qlen; ++i)
    if (q.q[i] >= alphabet) return fail(ctx, ISH_EINVAL, "query code %u at %u >= alphabet %u", q.q[i], i, alphabet);
  q.mmin = 0;
  q.mmax = 0;
  for (int8_t v : q.M) {
    q.mmin = std::min<int>(q.mmin, v);
    q.mmax = std::max<int>(q.mmax, v);
  }
  q.neg_limit = neg_limit_of(q.open, q.mmin);
  compute_rows(q);
  cudaSetDevice(ctx->device);
  const int32_t id = ctx->next_query++;
  ctx->queries.emplace(id, std::move(q));
  *query_id = id;
  return ISH_OK;
}

int ish_gpu_free_query(ish_ctx *ctx, int32_t query_id) {
  if (!ctx) return ISH_EINVAL;
  auto it = ctx->queries.find(query_id);
  if (it == ctx->queries.end()) return fail(ctx, ISH_EINVAL, "unknown query %d", query_id);
  cudaStreamSynchronize(ctx->stream);
  drop_plans(ctx, query_id, 0);
  release_query(it->second);
  ctx->queries.erase(it);
  return ISH_OK;
}

int ish_gpu_records_load(ish_ctx *ctx, const uint8_t *records, const uint64_t *offsets, uint32_t n, int32_t *set_id) {
  if (!ctx || !set_id) return ctx ? fail(ctx, ISH_EINVAL, "set_id is NULL") : ISH_EINVAL;
  if (int rc0 = finish_pending_load(ctx)) return rc0;
  LoadTimer timer(ctx);
  cudaSetDevice(ctx->device);
  RecordSet rs;
  int rc = load_records(ctx, records, offsets, n, rs, nullptr);
  if (rc) {
    release_set(rs);
    return rc;
  }
  const int32_t id = ctx->next_set++;
  ctx->sets.emplace(id, std::move(rs));
  *set_id = id;
  return ISH_OK;
}

int ish_gpu_records_load_async(ish_ctx *ctx, const uint8_t *records, const uint64_t *offsets, uint32_t n,
                               int32_t *set_id) {
  if (!ctx || !set_id) return ctx ? fail(ctx, ISH_EINVAL, "set_id is NULL") : ISH_EINVAL;
  // one load in flight: the previous one completes first (its scratch is reused)
  if (int rc0 = finish_pending_load(ctx)) return rc0;
  LoadTimer timer(ctx);
  cudaSetDevice(ctx->device);
  RecordSet rs;
  // the load stream starts after the work already queued on the context's
  // stream (a set freed just before may still be read there)
  CU(cudaEventRecord(ctx->load_ev[0], ctx->stream));
  CU(cudaStreamWaitEvent(ctx->load_stream, ctx->load_ev[0], 0));
  int rc = load_records(ctx, records, offsets, n, rs, nullptr, ctx->load_stream, true);
  if (rc) {
    cudaStreamSynchronize(ctx->load_stream);
    release_set(rs);
    return rc;
  }
  const int32_t id = ctx->next_set++;
  const bool pending = rs.pending;
  ctx->sets.emplace(id, std::move(rs));
  if (pending) ctx->pending_set = id;
  *set_id = id;
  return ISH_OK;
}

int ish_gpu_records_load_raw(ish_ctx *ctx, const uint8_t *raw, const uint64_t *offsets, uint32_t n, int matrix_kind,
                             int32_t *set_id) {
  if (!ctx || !set_id) return ctx ? fail(ctx, ISH_EINVAL, "set_id is NULL") : ISH_EINVAL;
  if (int rc0 = finish_pending_load(ctx)) return rc0;
  LoadTimer timer(ctx);
  cudaSetDevice(ctx->device);
  const uint8_t *enc = nullptr;
  int rc = device_encoding(ctx, matrix_kind, &enc);
  if (rc) return rc;
  RecordSet rs;
  rc = load_records(ctx, raw, offsets, n, rs, enc);
  if (rc) {
    release_set(rs);
    return rc;
  }
  const int32_t id = ctx->next_set++;
  ctx->sets.emplace(id, std::move(rs));
  *set_id = id;
  return ISH_OK;
}

int ish_gpu_records_load_lines(ish_ctx *ctx, const uint8_t *text, uint64_t bytes, int matrix_kind, int32_t *set_id,
                               uint32_t *n_records) {
  if (!ctx || !set_id) return ctx ? fail(ctx, ISH_EINVAL, "set_id is NULL") : ISH_EINVAL;
  if (int rc0 = finish_pending_load(ctx)) return rc0;
  LoadTimer timer(ctx);
  cudaSetDevice(ctx->device);
  const uint8_t *enc = nullptr;
  int rc = device_encoding(ctx, matrix_kind, &enc);
  if (rc) return rc;
  RecordSet rs;
  uint32_t n = 0;
  rc = load_lines(ctx, text, bytes, rs, enc, &n);
  if (rc) {
    release_set(rs);
    return rc;
  }
  const int32_t id = ctx->next_set++;
  ctx->sets.emplace(id, std::move(rs));
  *set_id = id;
  if (n_records) *n_records = n;
  return ISH_OK;
}

int ish_gpu_records_free(ish_ctx *ctx, int32_t set_id) {
  if (!ctx) return ISH_EINVAL;
  int urc = ISH_OK;
  RecordSet *it_set = use_set(ctx, set_id, &urc);
  if (!it_set) return urc;
  if (server_uses_set(ctx, set_id)) return fail(ctx, ISH_EINVAL, "record set %d is used by the serving loop", set_id);
  auto it = ctx->sets.find(set_id);
  cudaStreamSynchronize(ctx->stream);
  drop_plans(ctx, 0, set_id);
  recycle_set(ctx, it->second);
  ctx->sets.erase(it);
  return ISH_OK;
}

int ish_gpu_records_info(ish_ctx *ctx, int32_t set_id, uint32_t *n, uint64_t *total_bytes) {
  if (!ctx) return ISH_EINVAL;
  int urc = ISH_OK;
  RecordSet *it_set = use_set(ctx, set_id, &urc);
  if (!it_set) return urc;
  if (n) *n = it_set->n;
  if (total_bytes) *total_bytes = it_set->total;
  return ISH_OK;
}

int ish_gpu_score_set(ish_ctx *ctx, int32_t query_id, int32_t set_id, int32_t *score, int32_t *query_end,
                      int32_t *target_end, uint8_t *hit, uint32_t *hit_idx, uint32_t *n_hits) {
  if (!ctx) return ISH_EINVAL;
  auto qi = ctx->queries.find(query_id);
  if (qi == ctx->queries.end()) return fail(ctx, ISH_EINVAL, "unknown query %d", query_id);
  int urc = ISH_OK;
  RecordSet *si_set = use_set(ctx, set_id, &urc);
  if (!si_set) return urc;
  cudaSetDevice(ctx->device);
  int rc = run_scoring(ctx, qi->second, *si_set);
  if (rc) {
    cudaStreamSynchronize(ctx->stream);
    return rc;
  }
  return fetch_outputs(ctx, si_set->n, score, query_end, target_end, hit, hit_idx, n_hits);
}

int ish_gpu_score(ish_ctx *ctx, int32_t query_id, const uint8_t *records, const uint64_t *offsets, uint32_t n,
                  int32_t *score, int32_t *query_end, int32_t *target_end, uint8_t *hit, uint32_t *hit_idx,
                  uint32_t *n_hits) {
  if (!ctx) return ISH_EINVAL;
  auto qi = ctx->queries.find(query_id);
  if (qi == ctx->queries.end()) return fail(ctx, ISH_EINVAL, "unknown query %d", query_id);
  cudaSetDevice(ctx->device);
  if (int rc0 = finish_pending_load(ctx)) return rc0;
  RecordSet rs;
  int rc = load_records(ctx, records, offsets, n, rs, nullptr);
  if (!rc) rc = run_scoring(ctx, qi->second, rs);
  if (!rc) rc = fetch_outputs(ctx, n, score, query_end, target_end, hit, hit_idx, n_hits);
  cudaStreamSynchronize(ctx->stream);
  recycle_set(ctx, rs);  // the next call's set takes these buffers
  return rc;
}

int ish_gpu_calibrate(ish_ctx *ctx, double *dpx_ops_per_s) {
  if (!ctx || !dpx_ops_per_s) return ISH_EINVAL;
  cudaSetDevice(ctx->device);
  CU(ctx->counter.ensure(64));
  const int blocks = ctx->num_sms * 8, threads = 256, iters = 8192;
  cudaStream_t s = ctx->stream;
  k_dpx_peak<<<blocks, threads, 0, s>>>(ctx->counter.as<uint32_t>(), 256, 0x00010001u, 0xfffbfffbu);  // warm-up
  CU(cudaEventRecord(ctx->ev0, s));
  ++ctx->launches;
  k_dpx_peak<<<blocks, threads, 0, s>>>(ctx->counter.as<uint32_t>(), iters, 0x00010001u, 0xfffbfffbu);
  ++ctx->launches;
  CU(cudaEventRecord(ctx->ev1, s));
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(s));
  float ms = 0.f;
  CU(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  *dpx_ops_per_s = (double)blocks * threads * iters * 8 / (ms * 1e-3);
  return ISH_OK;
}

int ish_gpu_calibrate_lanes(ish_ctx *ctx, double *s16x2_cells_per_s, double *u8x4_cells_per_s) {
  if (!ctx) return ISH_EINVAL;
  if (!s16x2_cells_per_s || !u8x4_cells_per_s) return fail(ctx, ISH_EINVAL, "NULL output");
  cudaSetDevice(ctx->device);
  CU(ctx->counter.ensure(64));
  const int blocks = ctx->num_sms * 8, threads = 256, rows = 4096;
  cudaStream_t s = ctx->stream;
  for (int u8 = 0; u8 < 2; ++u8) {
    const LaneFn fn = lane_rows_fn(u8 != 0);
    const uint32_t open = u8 ? 0x0a0a0a0au : 10u, ext = u8 ? 0x01010101u : 1u;
    fn<<<blocks, threads, 0, s>>>(ctx->counter.as<uint32_t>(), 64, 0x03020104u, open, ext, 0x04040404u);  // warm-up
    CU(cudaEventRecord(ctx->ev0, s));
    fn<<<blocks, threads, 0, s>>>(ctx->counter.as<uint32_t>(), rows, 0x03020104u, open, ext, 0x04040404u);
    CU(cudaEventRecord(ctx->ev1, s));
    ctx->launches += 2;
    CU(cudaGetLastError());
    CU(cudaStreamSynchronize(s));
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    // 16 words per thread and row, 2 or 4 cells per word
    const double cells = (double)blocks * threads * rows * 16 * (u8 ? 4 : 2);
    (u8 ? *u8x4_cells_per_s : *s16x2_cells_per_s) = cells / (ms * 1e-3);
  }
  return ISH_OK;
}

int ish_gpu_launch_count(ish_ctx *ctx, uint64_t *count) {
  if (!ctx || !count) return ISH_EINVAL;
  *count = ctx->launches.load();
  return ISH_OK;
}

int ish_gpu_last_windows(ish_ctx *ctx, uint32_t *windows) {
  if (!ctx || !windows) return ISH_EINVAL;
  *windows = ctx->last_windows;
  return ISH_OK;
}

int ish_gpu_last_kernel_ms(ish_ctx *ctx, double *ms) {
  if (!ctx || !ms) return ISH_EINVAL;
  *ms = ctx->last_ms;
  return ISH_OK;
}

int ish_gpu_last_load_ms(ish_ctx *ctx, double *upload_ms, double *pack_ms, double *wall_ms) {
  if (!ctx) return ISH_EINVAL;
  if (upload_ms) *upload_ms = ctx->last_load_ms[0];
  if (pack_ms) *pack_ms = ctx->last_load_ms[1];
  if (wall_ms) *wall_ms = ctx->last_load_ms[2];
  return ISH_OK;
}

}  // extern "C"

// Dispatch over the instantiation files.
namespace ish {
WaveFn wave_fn_a(int, int, int);
WaveFn wave_fn_b(int, int, int);
WaveFn wave_fn_c(int, int, int);
WaveFn wave_fn_d(int, int, int);
WaveFn wave_fn_e(int, int, int);
WaveFn wave_fn_f(int, int, int);
WaveFn wave_fn_g(int, int, int);
BatchFn batch_fn_g(int, int, int);
WaveFn wave_fn_h(int, int, int);
BatchFn batch_fn_h(int, int, int);
WaveFn wave_fn(int K, int mode, int layout, int lean) {
  if (K < 1) return nullptr;
  if (lean && wave_has_lean(K)) return K <= 32 ? wave_fn_h(K, mode, layout) : wave_fn_g(K, mode, layout);
  if (K <= 8) return wave_fn_a(K, mode, layout);
  if (K <= 16) return wave_fn_b(K, mode, layout);
  if (K <= 24) return wave_fn_c(K, mode, layout);
  if (K <= 32) return wave_fn_d(K, mode, layout);
  if (K <= 48) return wave_fn_e(K, mode, layout);
  return wave_fn_f(K, mode, layout);
}
BatchFn batch_fn_a(int, int, int);
BatchFn batch_fn_b(int, int, int);
BatchFn batch_fn_c(int, int, int);
BatchFn batch_fn_d(int, int, int);
BatchFn batch_fn_e(int, int, int);
BatchFn batch_fn_f(int, int, int);
BatchFn batch_fn(int K, int mode, int layout, int lean) {
  if (K < 1) return nullptr;
  if (lean && wave_has_lean(K)) return K <= 32 ? batch_fn_h(K, mode, layout) : batch_fn_g(K, mode, layout);
  if (K <= 8) return batch_fn_a(K, mode, layout);
  if (K <= 16) return batch_fn_b(K, mode, layout);
  if (K <= 24) return batch_fn_c(K, mode, layout);
  if (K <= 32) return batch_fn_d(K, mode, layout);
  if (K <= 48) return batch_fn_e(K, mode, layout);
  return batch_fn_f(K, mode, layout);
}
}  // namespace ish
