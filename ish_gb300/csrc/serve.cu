// serve.cu -- the serving loop: continuous batching of queries against one
// resident record set (ish_gpu_serve_start / submit / poll / stop / stats).
//
// A scheduler thread owned by the context runs steps.  Before each step it
// admits waiting requests while an active slot is free and the device memory
// their outputs need fits the budget (profiles live in shared memory and DP
// rows in registers, so outputs are what a request costs).  A step scores the
// next chunk of the record set (chunk c of n: every n-th record pair of the
// descending length order from pair c) for EVERY active request, in one
// batched launch: one persistent batch_kernel per shape class, whose blocks steal
// record pairs from per-(request, chunk) counters, so the work of all active
// requests overlaps on the device.  A request that has run its last chunk is
// compacted (hit list, scores and ends of the hits) and handed to poll; new
// requests join at the next step.  Results do not depend on the mix: every
// (request, record) cell is computed by the same kernel code as a single
// query launch.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <set>
#include <thread>
#include <vector>

#include "host.h"

namespace ish {
namespace host {

using Clock = std::chrono::steady_clock;

// Device buffers of one admitted request.  Every request of a server scores
// the same set, so bundles have one size and are pooled.
struct Bundle {
  DevBuf score, qend, tend, hit, idx, counts, nhits, hs, hq, ht;
  void release() {
    DevBuf *b[] = {&score, &qend, &tend, &hit, &idx, &counts, &nhits, &hs, &hq, &ht};
    for (DevBuf *x : b) x->release();
  }
};

// A window view of the served set, shared by the requests that score it and
// released with the last of them.
struct SharedView {
  WindowView V;
  ~SharedView() { V.release(); }
};

struct Request {
  uint64_t ticket = 0;
  Query q;  // private copy: parameters and sequence (its layouts belong to the scheduler)
  int G = 0, K = 0, layout = 0, mode = 0;
  WaveLayout *L = nullptr;
  bool exact = false;  // scored by the lane-exact kernels (outside the wavefront kernels' regime)
  Bundle *b = nullptr;
  // long records: the request scores the windows of `view` into wout, folded
  // into its outputs after its last chunk
  std::shared_ptr<SharedView> view;
  DevBuf wscore, wqend, wtend, whit;
  WaveParams params{};
  uint32_t next_chunk = 0;
  uint32_t nch = 0;  // chunks (steps) of this request
  Clock::time_point t_submit, t_done;
  int status = ISH_OK;
  std::string err;
  std::vector<uint32_t> hit_idx;
  std::vector<int32_t> hit_score, hit_qend, hit_tend;
};

struct Server {
  ish_ctx *ctx = nullptr;
  int32_t set_id = 0;
  RecordSet *rs = nullptr;
  uint32_t max_active = 0;
  uint64_t mem_budget = 0;
  std::vector<std::pair<uint32_t, uint32_t>> chunks;  // (first, count) of sorted entries
  std::vector<double> chunk_residues;
  std::thread th;
  // shared with the API threads (under mu)
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> pending;
  std::map<uint64_t, Request *> finished;
  std::set<uint64_t> live;
  uint64_t next_ticket = 1;
  bool stopping = false;
  uint64_t completed = 0, steps = 0;
  double cells = 0, device_ms = 0;
  uint32_t max_active_seen = 0;
  // scheduler thread only
  std::vector<Request *> active;
  std::shared_ptr<SharedView> view;  // the newest window view (overlap view->V.O)
  cudaStream_t s = nullptr;
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> join;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, fork = nullptr;
  std::vector<Bundle *> pool;
  uint32_t bundles = 0;
  size_t bundle_bytes = 0;
  DevBuf step_params, step_tiles, step_counters, error;
  ExactRes exact;         // exact kernels' resources, shared by the exact requests (one stream)
  uint32_t max_chunk = 0;  // records in the largest chunk
  WaveParams *h_params = nullptr;  // pinned staging
  BatchTile *h_tiles = nullptr;
  uint32_t *h_nhits = nullptr;
};

namespace {

inline uint64_t bucket_len(uint32_t b) { return b < 32768 ? b : 32768 + ((uint64_t)(b - 32768) << 5) + 31; }

// Splits the set's non-empty sorted entries into `n` chunks of about equal
// residue count.
void make_chunks(Server &S, uint32_t n) {
  const RecordSet &rs = *S.rs;
  double total = 0;
  for (uint32_t b = 1; b <= top_bucket(rs); ++b) total += (double)rs.hist[b] * (double)bucket_len(b);
  const double per = total / std::max<uint32_t>(n, 1);
  uint32_t pos = 0, first = 0;
  double acc = 0;
  for (uint32_t b = top_bucket(rs); b >= 1; --b) {
    uint64_t c = rs.hist[b];
    const double L = (double)bucket_len(b);
    while (c) {
      uint64_t take = c;
      if (S.chunks.size() + 1 < n && L > 0) {
        const double room = per * (S.chunks.size() + 1) - acc;
        take = std::min<uint64_t>(c, (uint64_t)std::max(1.0, std::ceil(room / L)));
      }
      pos += (uint32_t)take;
      c -= take;
      acc += (double)take * L;
      if (S.chunks.size() + 1 < n && acc >= per * (S.chunks.size() + 1)) {
        S.chunks.push_back({first, pos - first});
        S.chunk_residues.push_back(0);
        first = pos;
      }
    }
  }
  if (pos > first || S.chunks.empty()) {
    S.chunks.push_back({first, pos - first});
    S.chunk_residues.push_back(0);
  }
  // residues per chunk (for the cell count)
  uint32_t ci = 0;
  uint64_t at = 0;
  for (uint32_t b = top_bucket(rs); b >= 1 && ci < S.chunks.size(); --b) {
    uint64_t c = rs.hist[b];
    while (c && ci < S.chunks.size()) {
      const uint64_t end = (uint64_t)S.chunks[ci].first + S.chunks[ci].second;
      const uint64_t take = std::min<uint64_t>(c, end - at);
      S.chunk_residues[ci] += (double)take * (double)bucket_len(b);
      at += take;
      c -= take;
      if (at >= end) ++ci;
    }
  }
}

void finish(Server &S, Request *r) {
  r->t_done = Clock::now();
  release_query(r->q);
  r->view.reset();
  r->wscore.release();
  r->wqend.release();
  r->wtend.release();
  r->whit.release();
  r->L = nullptr;
  if (r->b) {
    S.pool.push_back(r->b);
    r->b = nullptr;
  }
  std::lock_guard<std::mutex> lk(S.mu);
  S.finished.emplace(r->ticket, r);
  ++S.completed;
  if (r->status == ISH_OK) S.cells += (double)r->q.Q * (double)S.rs->total;
  S.cv_done.notify_all();
}

#define SCU(call)                                                                  \
  do {                                                                             \
    cudaError_t _e = (call);                                                       \
    if (_e != cudaSuccess) {                                                       \
      (void)cudaGetLastError();                                                    \
      snprintf(msg, 256, "%s: %s", #call, cudaGetErrorString(_e));                 \
      return _e == cudaErrorMemoryAllocation ? ISH_ENOMEM : ISH_EDEVICE;           \
    }                                                                              \
  } while (0)

// Admission work on the scheduler thread: shape check, profile, outputs.
int admit(Server &S, Request *r, char *msg, size_t) {
  const RecordSet &rs = *S.rs;
  const uint32_t n = rs.n;
  if (r->q.Q > 0 && rs.n > rs.n_empty) {
    if (rs.max_code >= (uint32_t)r->q.alphabet) {
      snprintf(msg, 256, "a record contains code %u >= the alphabet size %d of the query", rs.max_code, r->q.alphabet);
      return ISH_EINVAL;
    }
    char why[256];
    if (fast_check(r->q, rs, r->G, r->K, why, sizeof why) == ISH_OK && wave_fits(r->q, r->G, r->K, r->layout)) {
      int rc = build_wave_layout(S.ctx, r->q, r->G, r->K, r->layout, &r->L);
      if (rc) {
        snprintf(msg, 256, "profile upload failed");
        return rc;
      }
      r->layout = r->L->layout;
    } else {
      // outside the wavefront kernels' exact regime, or a profile that fits
      // no layout: the lane-exact kernels score its chunks
      int rc = exact_prepare(S.ctx, r->q, S.max_chunk, S.exact);
      if (rc) {
        snprintf(msg, 256, "exact kernel resources: %s", ish_gpu_last_error(S.ctx));
        return rc;
      }
      r->exact = true;
    }
  }
  if (S.pool.empty()) {
    Bundle *b = new Bundle();
    const uint32_t nb = std::max<uint32_t>(1, ceil_div(n, HIT_TILE));
    cudaError_t e = cudaSuccess;
    auto grab = [&](DevBuf &d, size_t bytes) {
      if (e == cudaSuccess) e = d.ensure(bytes);
    };
    grab(b->score, (size_t)n * 4 + 4);
    grab(b->qend, (size_t)n * 4 + 4);
    grab(b->tend, (size_t)n * 4 + 4);
    grab(b->hit, (size_t)n + 16);
    grab(b->idx, (size_t)n * 4 + 4);
    grab(b->counts, (size_t)nb * 4 + 8);
    grab(b->nhits, 16);
    grab(b->hs, (size_t)n * 4 + 4);
    grab(b->hq, (size_t)n * 4 + 4);
    grab(b->ht, (size_t)n * 4 + 4);
    if (e != cudaSuccess) {
      b->release();
      delete b;
      snprintf(msg, 256, "device memory for a request: %s", cudaGetErrorString(e));
      return ISH_ENOMEM;
    }
    S.pool.push_back(b);
    ++S.bundles;
  }
  r->b = S.pool.back();
  S.pool.pop_back();
  if (r->L) {
    OutDev out{r->b->score.as<int32_t>(), r->b->qend.as<int32_t>(), r->b->tend.as<int32_t>(),
               r->b->hit.as<uint8_t>()};
    // long records that would bound the request's steps: it scores a window
    // view (free target start, no free query start), shared with the other
    // requests whose overlap it covers; a request that needs a larger overlap
    // gets a new view (the old one lives on with the requests using it)
    const uint64_t O = S.ctx->windows_on && S.ctx->kernel == ISH_KERNEL_AUTO && windowable_whole(r->q)
                           ? window_overlap(r->q) : 0;
    const uint32_t nonempty = rs.n - rs.n_empty;
    const int mode = r->q.algo == ISH_ALGO_LOCAL ? SW : SG;
    const uint64_t W = (O && nonempty <= (1u << 22)) ? window_stride(S.ctx, rs, O, r->G, r->K, mode) : 0;
    if (W) {
      if (!S.view || S.view->V.O < O) {
        auto v = std::make_shared<SharedView>();
        const uint64_t Ov = S.view ? std::max<uint64_t>(O, S.view->V.O) : O;
        const uint64_t Wv = std::max<uint64_t>(W, 8 * Ov);
        int rc = build_window_view(S.ctx, rs, nonempty, (Wv + 15) & ~15ull, Ov, v->V, S.s);
        if (rc) {
          snprintf(msg, 256, "window view: %s", ish_gpu_last_error(S.ctx));
          return rc;
        }
        S.view = v;
      }
      r->view = S.view;
      const uint32_t nw = r->view->V.nw;
      cudaError_t e = r->wscore.ensure((size_t)nw * 4);
      if (e == cudaSuccess) e = r->wqend.ensure((size_t)nw * 4);
      if (e == cudaSuccess) e = r->wtend.ensure((size_t)nw * 4);
      if (e == cudaSuccess) e = r->whit.ensure((size_t)nw + 16);
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        snprintf(msg, 256, "device memory for a request's windows: %s", cudaGetErrorString(e));
        return ISH_ENOMEM;
      }
      OutDev wout{r->wscore.as<int32_t>(), r->wqend.as<int32_t>(), r->wtend.as<int32_t>(), r->whit.as<uint8_t>()};
      wave_params(r->q, *r->L, window_set(rs, r->view->V), wout, S.error.as<int>(), &r->params);
    } else {
      wave_params(r->q, *r->L, rs, out, S.error.as<int>(), &r->params);
    }
  }
  // steps per request: the exact kernels take the set's contiguous chunks; a
  // wavefront request takes as many interleaved chunks as keep its steps near
  // ISH_OPT_SERVE_STEP_CELLS cells (short queries finish in one or two steps
  // instead of paying a host round trip per chunk), at most the server's
  // chunk count
  const double step_cells = S.ctx->serve_step_cells;  // default 1.25e11: ~25 ms at 5 TCUPS
  if (r->exact) {
    r->nch = (uint32_t)S.chunks.size();
  } else if (r->L) {
    const double cells = (double)r->q.Q * (double)rs.total;
    r->nch = step_cells > 0 ? (uint32_t)std::min<double>((double)S.chunks.size(),
                                                         std::max(1.0, std::round(cells / step_cells)))
                            : (uint32_t)S.chunks.size();
  } else {
    r->nch = 0;
  }
  r->next_chunk = 0;
  return ISH_OK;
}

// One step: the next chunk of every active request in one batched launch,
// then completion of the requests that ran their last chunk.
int step(Server &S, char *msg) {
  const RecordSet &rs = *S.rs;
  const uint32_t n = rs.n;
  cudaStream_t s = S.s;
  // ---- classes of this step ----
  struct Cls {
    int K, mode, layout, Gmin = 32;
    uint32_t prof_area = 0, first = 0, count = 0;
  };
  std::vector<Cls> cls;
  std::vector<std::vector<Request *>> members;
  for (Request *r : S.active) {
    if (r->next_chunk >= r->nch || r->exact) continue;
    size_t c = 0;
    for (; c < cls.size(); ++c)
      if (cls[c].K == r->K && cls[c].mode == r->mode && cls[c].layout == r->layout) break;
    if (c == cls.size()) {
      cls.push_back(Cls{r->K, r->mode, r->layout});
      members.emplace_back();
    }
    cls[c].Gmin = std::min(cls[c].Gmin, r->G);
    cls[c].prof_area = std::max(cls[c].prof_area, (r->L->prof_bytes + 15u) & ~15u);
    members[c].push_back(r);
  }
  uint32_t k = 0;
  for (size_t c = 0; c < cls.size(); ++c) {
    cls[c].first = k;
    for (Request *r : members[c]) {
      S.h_params[k] = r->params;
      // the wavefront requests' chunk c is every nch-th record pair of the
      // set from pair c: each step meets the whole length distribution
      // (longest pairs first), so its kernels end as evenly as a pass over
      // the whole set (contiguous chunks of the longest-first order made the
      // steps of the long records end on a few long pairs)
      const uint32_t nch = r->nch;
      const uint32_t entries = r->view ? r->view->V.nw : rs.n - rs.n_empty;  // windows or records
      S.h_tiles[k] = BatchTile{k - cls[c].first, 0, entries, nch > 1 ? (nch << 16) | r->next_chunk : 0u};
      ++k;
    }
    cls[c].count = k - cls[c].first;
  }
  SCU(cudaEventRecord(S.ev0, s));
  if (k) {
    SCU(cudaMemcpyAsync(S.step_params.p, S.h_params, (size_t)k * sizeof(WaveParams), cudaMemcpyHostToDevice, s));
    SCU(cudaMemcpyAsync(S.step_tiles.p, S.h_tiles, (size_t)k * sizeof(BatchTile), cudaMemcpyHostToDevice, s));
    SCU(cudaMemsetAsync(S.step_counters.p, 0, (size_t)k * 4, s));
    if (cls.size() > 1) SCU(cudaEventRecord(S.fork, s));
    while (S.side.size() + 1 < cls.size()) {
      cudaStream_t st;
      cudaEvent_t e;
      SCU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      SCU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      S.side.push_back(st);
      S.join.push_back(e);
    }
    for (size_t c = 0; c < cls.size(); ++c) {
      const Cls &C = cls[c];
      const int lean = batch_lean(S.ctx, C.K, C.mode, C.Gmin);
      BatchFn fn = batch_fn(C.K, C.mode, C.layout, lean);
      if (!fn) {
        snprintf(msg, 256, "no batch kernel for K=%d", C.K);
        return ISH_EOVERFLOW;
      }
      const int threads = wave_threads_lean(C.K, C.mode, lean);
      const size_t slot_words = (size_t)(threads / C.Gmin) * 32;
      const size_t save = C.mode == SW ? (size_t)threads * wave_save_words(C.K) * 4 : 0;
      const size_t smem = C.prof_area + slot_words * 4 + save;
      SCU(cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      int per_sm = 0;
      SCU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)fn, threads, smem));
      if (per_sm < 1) {
        snprintf(msg, 256, "batch kernel K=%d does not fit (smem %zu)", C.K, smem);
        return ISH_EOVERFLOW;
      }
      BatchParams b{};
      b.queries = S.step_params.as<const WaveParams>() + C.first;
      b.tiles = S.step_tiles.as<const BatchTile>() + C.first;
      b.ntiles = C.count;
      b.tile_counter = S.step_counters.as<uint32_t>() + C.first;
      b.prof_area = C.prof_area;
      b.slot_words = (uint32_t)slot_words;
      b.step_cap = S.ctx->step_budget;
      cudaStream_t cs = c == 0 ? s : S.side[c - 1];
      if (c > 0) SCU(cudaStreamWaitEvent(cs, S.fork, 0));
      fn<<<per_sm * S.ctx->num_sms, threads, smem, cs>>>(b);
      ++S.ctx->launches;
      SCU(cudaGetLastError());
      if (c > 0) {
        SCU(cudaEventRecord(S.join[c - 1], cs));
        SCU(cudaStreamWaitEvent(s, S.join[c - 1], 0));
      }
    }
  }
  // ---- requests on the exact kernels: their chunk, after the batched launch ----
  for (Request *r : S.active) {
    if (!r->exact || r->next_chunk >= r->nch) continue;
    const auto &ch = S.chunks[r->next_chunk];
    OutDev out{r->b->score.as<int32_t>(), r->b->qend.as<int32_t>(), r->b->tend.as<int32_t>(), r->b->hit.as<uint8_t>()};
    uint32_t nl = 0;
    if (exact_enqueue(S.ctx, r->q, *S.rs, ch.first, ch.second, out, s, S.exact, &nl)) {
      snprintf(msg, 256, "exact kernel launch failed");
      return ISH_EDEVICE;
    }
    S.ctx->launches += nl;
  }
  // ---- completion of requests past their last chunk ----
  std::vector<Request *> done;
  const RecordsDev rec{rs.codes.as<const uint8_t>(), rs.off_s.as<const uint64_t>(), rs.len_s.as<const uint32_t>(),
                       rs.orig_s.as<const uint32_t>(), rs.n};
  for (Request *r : S.active) {
    if (r->next_chunk < r->nch) ++r->next_chunk;
    if (r->next_chunk < r->nch) continue;
    Bundle &b = *r->b;
    OutDev out{b.score.as<int32_t>(), b.qend.as<int32_t>(), b.tend.as<int32_t>(), b.hit.as<uint8_t>()};
    if (r->view) {
      int rc = merge_windows(S.ctx, rs, rs.n - rs.n_empty, r->view->V, r->q, r->wscore.as<const int32_t>(),
                             r->wqend.as<const int32_t>(), r->wtend.as<const int32_t>(), out, s, nullptr);
      if (rc) {
        snprintf(msg, 256, "window fold: %s", ish_gpu_last_error(S.ctx));
        return rc;
      }
    }
    const uint32_t n_empty = (r->q.Q == 0) ? n : rs.n_empty;
    if (n_empty) {
      k_trivial<<<std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(n_empty, 256), 1024)), 256, 0, s>>>(
          rec, n - n_empty, n_empty, r->mode, r->q.Q, out, Decision{r->q.max_score, r->q.thr});
      ++S.ctx->launches;
    }
    const uint32_t nb = std::max<uint32_t>(1, ceil_div(n, HIT_TILE));
    if (n) {
      k_count_hits<<<nb, 1024, 0, s>>>(b.hit.as<uint8_t>(), n, b.counts.as<uint32_t>());
      ++S.ctx->launches;
      k_scan_counts<<<1, 1024, 0, s>>>(b.counts.as<uint32_t>(), nb, b.nhits.as<uint32_t>());
      ++S.ctx->launches;
      k_write_hits<<<nb, 1024, 0, s>>>(b.hit.as<uint8_t>(), n, b.counts.as<uint32_t>(), b.idx.as<uint32_t>());
      ++S.ctx->launches;
      k_gather_hits<<<S.ctx->num_sms * 4, 256, 0, s>>>(b.idx.as<uint32_t>(), b.nhits.as<uint32_t>(),
                                                      b.score.as<int32_t>(), b.qend.as<int32_t>(),
                                                      b.tend.as<int32_t>(), b.hs.as<int32_t>(), b.hq.as<int32_t>(),
                                                      b.ht.as<int32_t>());
      ++S.ctx->launches;
      SCU(cudaGetLastError());
      SCU(cudaMemcpyAsync(&S.h_nhits[done.size()], b.nhits.p, 4, cudaMemcpyDeviceToHost, s));
    } else {
      S.h_nhits[done.size()] = 0;
    }
    done.push_back(r);
  }
  int herr = 0;
  SCU(cudaMemcpyAsync(&S.h_nhits[S.max_active], S.error.p, 4, cudaMemcpyDeviceToHost, s));
  SCU(cudaEventRecord(S.ev1, s));
  SCU(cudaEventSynchronize(S.ev1));
  herr = (int)S.h_nhits[S.max_active];
  float ms = 0.f;
  cudaEventElapsedTime(&ms, S.ev0, S.ev1);
  {
    std::lock_guard<std::mutex> lk(S.mu);
    S.device_ms += ms;
    ++S.steps;
  }
  if (herr) {
    snprintf(msg, 256, herr & 2 ? "batch kernel exceeded its step budget (internal error)"
                                : "a record contains a code >= the alphabet size of a query");
    return herr & 2 ? ISH_ETIMEDOUT : ISH_EINVAL;
  }
  for (size_t i = 0; i < done.size(); ++i) {
    Request *r = done[i];
    const uint32_t nh = S.h_nhits[i];
    r->hit_idx.resize(nh);
    r->hit_score.resize(nh);
    r->hit_qend.resize(nh);
    r->hit_tend.resize(nh);
    if (nh) {
      SCU(cudaMemcpyAsync(r->hit_idx.data(), r->b->idx.p, (size_t)nh * 4, cudaMemcpyDeviceToHost, s));
      SCU(cudaMemcpyAsync(r->hit_score.data(), r->b->hs.p, (size_t)nh * 4, cudaMemcpyDeviceToHost, s));
      SCU(cudaMemcpyAsync(r->hit_qend.data(), r->b->hq.p, (size_t)nh * 4, cudaMemcpyDeviceToHost, s));
      SCU(cudaMemcpyAsync(r->hit_tend.data(), r->b->ht.p, (size_t)nh * 4, cudaMemcpyDeviceToHost, s));
    }
  }
  if (!done.empty()) SCU(cudaStreamSynchronize(s));
  for (Request *r : done) {
    S.active.erase(std::find(S.active.begin(), S.active.end(), r));
    finish(S, r);
  }
  return ISH_OK;
}

void fail_all(Server &S, int rc, const char *msg) {
  for (Request *r : S.active) {
    r->status = rc;
    r->err = msg;
    finish(S, r);
  }
  S.active.clear();
}

void scheduler(Server *Sp) {
  Server &S = *Sp;
  cudaSetDevice(S.ctx->device);
  char msg[256];
  while (true) {
    std::vector<Request *> admit_now;
    {
      std::unique_lock<std::mutex> lk(S.mu);
      S.cv_work.wait(lk, [&] { return S.stopping || !S.pending.empty() || !S.active.empty(); });
      if (S.stopping && S.pending.empty() && S.active.empty()) break;
      while (!S.pending.empty() && S.active.size() + admit_now.size() < S.max_active) {
        const bool fresh = S.pool.size() <= admit_now.size();
        const uint64_t used = (uint64_t)S.bundles * S.bundle_bytes;
        const bool nothing_running = S.active.empty() && admit_now.empty();
        if (fresh && used + S.bundle_bytes > S.mem_budget && !nothing_running) break;
        admit_now.push_back(S.pending.front());
        S.pending.pop_front();
      }
    }
    for (Request *r : admit_now) {
      msg[0] = 0;
      const int rc = admit(S, r, msg, sizeof msg);
      if (rc) {
        r->status = rc;
        r->err = msg;
        if (r->b) {
          S.pool.push_back(r->b);
          r->b = nullptr;
        }
        finish(S, r);
      } else {
        S.active.push_back(r);
      }
    }
    {
      std::lock_guard<std::mutex> lk(S.mu);
      S.max_active_seen = std::max<uint32_t>(S.max_active_seen, (uint32_t)S.active.size());
    }
    if (S.active.empty()) continue;
    msg[0] = 0;
    const int rc = step(S, msg);
    if (rc) {
      cudaStreamSynchronize(S.s);
      fail_all(S, rc, msg);
      cudaMemsetAsync(S.error.p, 0, 4, S.s);
      cudaStreamSynchronize(S.s);
    }
  }
}

}  // namespace

bool server_uses_set(const ish_ctx *ctx, int32_t set_id) { return ctx->server && ctx->server->set_id == set_id; }

void stop_server(ish_ctx *ctx) {
  Server *S = ctx->server;
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stopping = true;
  }
  S->cv_work.notify_all();
  if (S->th.joinable()) S->th.join();
  // (a serve_start that failed part-way may have created only some of these)
  if (S->s) cudaStreamSynchronize(S->s);
  for (Bundle *b : S->pool) {
    b->release();
    delete b;
  }
  for (auto &kv : S->finished) delete kv.second;
  for (auto st : S->side) cudaStreamDestroy(st);
  for (auto e : S->join) cudaEventDestroy(e);
  if (S->ev0) cudaEventDestroy(S->ev0);
  if (S->ev1) cudaEventDestroy(S->ev1);
  if (S->fork) cudaEventDestroy(S->fork);
  if (S->s) cudaStreamDestroy(S->s);
  S->step_params.release();
  S->step_tiles.release();
  S->step_counters.release();
  S->error.release();
  S->exact.release();
  cudaFreeHost(S->h_params);
  cudaFreeHost(S->h_tiles);
  cudaFreeHost(S->h_nhits);
  delete S;
  ctx->server = nullptr;
}

}  // namespace host
}  // namespace ish

using namespace ish;
using namespace ish::host;

extern "C" {

int ish_gpu_serve_start(ish_ctx *ctx, int32_t set_id, uint32_t max_active, uint64_t mem_budget, uint32_t chunks) {
  if (!ctx) return ISH_EINVAL;
  if (ctx->server) return fail(ctx, ISH_EINVAL, "the serving loop is already running");
  int urc = ISH_OK;
  RecordSet *si_set = use_set(ctx, set_id, &urc);
  if (!si_set) return urc;
  if (max_active == 0 || max_active > 4096) return fail(ctx, ISH_EINVAL, "max_active must be in 1..4096");
  if (chunks == 0 || chunks > 1024) return fail(ctx, ISH_EINVAL, "chunks must be in 1..1024");
  cudaSetDevice(ctx->device);
  Server *S = new Server();
  S->ctx = ctx;
  S->set_id = set_id;
  S->rs = si_set;
  S->max_active = max_active;
  const uint32_t n = S->rs->n;
  const uint32_t nb = std::max<uint32_t>(1, ceil_div(n, HIT_TILE));
  S->bundle_bytes = (size_t)n * 29 + (size_t)nb * 4 + 256;  // see Bundle
  if (mem_budget == 0) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    mem_budget = fr / 2;
  }
  S->mem_budget = mem_budget;
  make_chunks(*S, chunks);
  for (const auto &ch : S->chunks) S->max_chunk = std::max(S->max_chunk, ch.second);
  auto bail = [&](cudaError_t e) {
    (void)cudaGetLastError();
    ctx->server = S;
    stop_server(ctx);
    return fail(ctx, e == cudaErrorMemoryAllocation ? ISH_ENOMEM : ISH_EDEVICE, "serve_start: %s",
                cudaGetErrorString(e));
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&S->s, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
  if ((e = cudaEventCreate(&S->ev0)) != cudaSuccess) return bail(e);
  if ((e = cudaEventCreate(&S->ev1)) != cudaSuccess) return bail(e);
  if ((e = cudaEventCreateWithFlags(&S->fork, cudaEventDisableTiming)) != cudaSuccess) return bail(e);
  if ((e = S->step_params.ensure((size_t)max_active * sizeof(WaveParams))) != cudaSuccess) return bail(e);
  if ((e = S->step_tiles.ensure((size_t)max_active * sizeof(BatchTile))) != cudaSuccess) return bail(e);
  if ((e = S->step_counters.ensure((size_t)max_active * 4)) != cudaSuccess) return bail(e);
  if ((e = S->error.ensure(64)) != cudaSuccess) return bail(e);
  if ((e = cudaMemset(S->error.p, 0, 64)) != cudaSuccess) return bail(e);
  if ((e = cudaMallocHost((void **)&S->h_params, (size_t)max_active * sizeof(WaveParams))) != cudaSuccess)
    return bail(e);
  if ((e = cudaMallocHost((void **)&S->h_tiles, (size_t)max_active * sizeof(BatchTile))) != cudaSuccess)
    return bail(e);
  if ((e = cudaMallocHost((void **)&S->h_nhits, (size_t)(max_active + 1) * 4)) != cudaSuccess) return bail(e);
  ctx->server = S;
  S->th = std::thread(scheduler, S);
  return ISH_OK;
}

int ish_gpu_submit(ish_ctx *ctx, int32_t query_id, uint64_t *ticket) {
  if (!ctx || !ticket) return ctx ? fail(ctx, ISH_EINVAL, "ticket is NULL") : ISH_EINVAL;
  Server *S = ctx->server;
  if (!S) return fail(ctx, ISH_EINVAL, "the serving loop is not running");
  auto qi = ctx->queries.find(query_id);
  if (qi == ctx->queries.end()) return fail(ctx, ISH_EINVAL, "unknown query %d", query_id);
  Request *r = new Request();
  clone_params(qi->second, r->q);
  pick_shape(ctx, r->q, &r->G, &r->K, &r->layout);
  r->mode = r->q.algo == ISH_ALGO_LOCAL ? SW : SG;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stopping) {
      delete r;
      return fail(ctx, ISH_EINVAL, "the serving loop is stopping");
    }
    r->ticket = S->next_ticket++;
    S->live.insert(r->ticket);
    S->pending.push_back(r);
  }
  S->cv_work.notify_one();
  *ticket = r->ticket;
  return ISH_OK;
}

int ish_gpu_poll(ish_ctx *ctx, uint64_t ticket, uint32_t *hit_idx, int32_t *hit_score, int32_t *hit_qend,
                 int32_t *hit_tend, uint32_t cap, uint32_t *n_hits, double *latency_ms, int32_t wait_ms) {
  if (!ctx) return ISH_EINVAL;
  Server *S = ctx->server;
  if (!S) return fail(ctx, ISH_EINVAL, "the serving loop is not running");
  std::unique_lock<std::mutex> lk(S->mu);
  if (!S->live.count(ticket)) return fail(ctx, ISH_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
  auto ready = [&] { return S->finished.count(ticket) > 0; };
  if (!ready() && wait_ms > 0) S->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), ready);
  auto it = S->finished.find(ticket);
  if (it == S->finished.end()) return ISH_EAGAIN;
  Request *r = it->second;
  if (r->status != ISH_OK) {
    const int rc = r->status;
    const std::string err = r->err;
    S->finished.erase(it);
    S->live.erase(ticket);
    delete r;
    return fail(ctx, rc, "%s", err.c_str());
  }
  const uint32_t nh = (uint32_t)r->hit_idx.size();
  if (n_hits) *n_hits = nh;
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  const bool want = hit_idx || hit_score || hit_qend || hit_tend;
  if (want && nh > cap) return fail(ctx, ISH_EOVERFLOW, "%u hits do not fit (capacity %u)", nh, cap);
  if (hit_idx && nh) memcpy(hit_idx, r->hit_idx.data(), (size_t)nh * 4);
  if (hit_score && nh) memcpy(hit_score, r->hit_score.data(), (size_t)nh * 4);
  if (hit_qend && nh) memcpy(hit_qend, r->hit_qend.data(), (size_t)nh * 4);
  if (hit_tend && nh) memcpy(hit_tend, r->hit_tend.data(), (size_t)nh * 4);
  S->finished.erase(it);
  S->live.erase(ticket);
  delete r;
  return ISH_OK;
}

int ish_gpu_serve_stop(ish_ctx *ctx) {
  if (!ctx) return ISH_EINVAL;
  if (!ctx->server) return fail(ctx, ISH_EINVAL, "the serving loop is not running");
  stop_server(ctx);
  return ISH_OK;
}

int ish_gpu_serve_stats(ish_ctx *ctx, uint64_t *completed, double *cells, double *device_ms, uint32_t *max_active_seen,
                        uint64_t *steps) {
  if (!ctx) return ISH_EINVAL;
  Server *S = ctx->server;
  if (!S) return fail(ctx, ISH_EINVAL, "the serving loop is not running");
  std::lock_guard<std::mutex> lk(S->mu);
  if (completed) *completed = S->completed;
  if (cells) *cells = S->cells;
  if (device_ms) *device_ms = S->device_ms;
  if (max_active_seen) *max_active_seen = S->max_active_seen;
  if (steps) *steps = S->steps;
  return ISH_OK;
}

}  // extern "C"
