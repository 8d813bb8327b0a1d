// multi.cu -- batched multi-query launches (ish_gpu_score_multi) and the
// kernel-shape autotuner (ish_gpu_autotune).
//
// A batched launch scores every query of a list against one resident record
// set.  Queries are grouped into shape classes (columns per thread K, mode,
// profile layout); each class runs as ONE persistent batch_kernel whose blocks
// steal record pairs of its queries from per-query counters (wave.cuh).  The classes run
// as parallel branches of one CUDA graph, followed by the hit compaction of
// all queries; the graph is captured on the first call for a (queries, set,
// outputs) combination and replayed on later calls.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "host.h"

namespace ish {
namespace host {

struct MultiClass {
  int K = 0, mode = 0, layout = 0, threads = 0, Gmin = 32;
  BatchFn fn = nullptr;
  size_t smem = 0;
  uint32_t grid = 0, ntiles = 0, prof_area = 0, counter_base = 0;
  std::vector<uint32_t> members;  // positions in the launch's query list
  DevBuf params, tiles;
};

struct MultiPlan {
  std::vector<int32_t> qids;
  int32_t set_id = 0;
  unsigned want = 0;
  uint32_t n = 0, nq = 0, nb = 0, n_counters = 0;
  uint32_t kernels = 0;  // kernel nodes of the graph
  std::vector<MultiClass> classes;
  DevBuf counters, score, qend, tend, hit, block_counts, hit_idx, nhits;
  std::vector<uint32_t> exact_q;  // positions of the queries the exact kernels score
  ExactRes exact;
  // long records: the queries at positions win_q score the plan's window view
  // (results per window in wscore.., window k of query w at [w * view.nw + k])
  // and are folded into their outputs after the batched kernels
  WindowView view;
  std::vector<uint32_t> win_q;
  DevBuf wscore, wqend, wtend, whit;
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> events;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t last_use = 0;

  void release() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    for (auto s : side) cudaStreamDestroy(s);
    for (auto e : events) cudaEventDestroy(e);
    side.clear();
    events.clear();
    for (auto &c : classes) {
      c.params.release();
      c.tiles.release();
    }
    view.release();
    win_q.clear();
    DevBuf *bufs[] = {&counters, &score, &qend, &tend, &hit, &block_counts, &hit_idx, &nhits, &wscore, &wqend,
                      &wtend, &whit};
    for (DevBuf *b : bufs) b->release();
    exact.release();
  }
};

enum : unsigned { W_SCORE = 1, W_QEND = 2, W_TEND = 4, W_HIT = 8, W_COMPACT = 16 };

namespace {

uint64_t g_use_clock = 0;
constexpr size_t MAX_PLANS = 8;

// Length of the records in histogram bucket b (buckets above 32767 hold 32
// lengths; their upper end is used, which only affects tile sizing).
inline uint64_t bucket_len(uint32_t b) { return b < 32768 ? b : 32768 + ((uint64_t)(b - 32768) << 5) + 31; }

std::string plan_key(const int32_t *qids, uint32_t nq, int32_t set_id, unsigned want) {
  std::string k = std::to_string(set_id) + ":" + std::to_string(want) + ":";
  k.append(reinterpret_cast<const char *>(qids), (size_t)nq * sizeof(int32_t));
  return k;
}

void evict_one(ish_ctx *ctx) {
  auto victim = ctx->plans.end();
  for (auto it = ctx->plans.begin(); it != ctx->plans.end(); ++it)
    if (victim == ctx->plans.end() || it->second->last_use < victim->second->last_use) victim = it;
  if (victim != ctx->plans.end()) {
    cudaStreamSynchronize(ctx->stream);
    victim->second->release();
    delete victim->second;
    ctx->plans.erase(victim);
  }
}

// Builds (but does not capture) a plan: shapes, layouts, parameters, tiles,
// output buffers.
int build_plan(ish_ctx *ctx, const int32_t *qids, uint32_t nq, int32_t set_id, RecordSet &rs, unsigned want,
               MultiPlan &P) {
  P.qids.assign(qids, qids + nq);
  P.set_id = set_id;
  P.want = want;
  P.n = rs.n;
  P.nq = nq;
  const uint32_t n = rs.n;
  const size_t total = (size_t)nq * n;
  if ((want & W_SCORE)) CU(P.score.ensure(total * 4 + 4));
  if ((want & W_QEND)) CU(P.qend.ensure(total * 4 + 4));
  if ((want & W_TEND)) CU(P.tend.ensure(total * 4 + 4));
  if ((want & (W_HIT | W_COMPACT))) CU(P.hit.ensure(total + 16));
  CU(ctx->error.ensure(64));
  const uint32_t nonempty = n - rs.n_empty;

  // ---- shape classes ----
  struct Member {
    uint32_t pos;
    int G, K, layout, mode;
    WaveLayout *L;
  };
  std::vector<Member> members;
  for (uint32_t i = 0; i < nq; ++i) {
    Query &q = ctx->queries.at(qids[i]);
    if (q.Q == 0 || nonempty == 0) continue;
    if (rs.max_code >= (uint32_t)q.alphabet)
      return fail(ctx, ISH_EINVAL, "a record contains code %u >= the alphabet size %d of query %d", rs.max_code,
                  q.alphabet, qids[i]);
    Member m;
    m.pos = i;
    pick_shape(ctx, q, &m.G, &m.K, &m.layout);
    m.mode = q.algo == ISH_ALGO_LOCAL ? SW : SG;
    if (!fast_regime(ctx, q, rs) || !wave_fits(q, m.G, m.K, m.layout)) {
      // outside the wavefront kernels' exact regime, or a profile that fits
      // no layout: the lane-exact kernels score this query in the same graph
      int rc = exact_prepare(ctx, q, nonempty, P.exact);
      if (rc) return rc;
      P.exact_q.push_back(i);
      continue;
    }
    int rc = build_wave_layout(ctx, q, m.G, m.K, m.layout, &m.L);
    if (rc) return rc;
    m.layout = m.L->layout;
    members.push_back(m);
  }
  // ---- windows: when the set's longest records would bound the pass, the
  // members whose window fold is exact (free target start; no free query
  // start, whose windows past row 0 would need a second profile) score a
  // window view with the largest overlap any of them needs ----
  std::vector<char> windowed(nq, 0);
  if (ctx->windows_on && ctx->kernel == ISH_KERNEL_AUTO && nonempty > 0 && nonempty <= (1u << 22)) {
    uint64_t O = 0, W = 0;
    for (const Member &m : members) {
      const Query &q = ctx->queries.at(qids[m.pos]);
      if (windowable_whole(q)) O = std::max(O, window_overlap(q));
    }
    if (O) {
      for (const Member &m : members) {
        const Query &q = ctx->queries.at(qids[m.pos]);
        if (windowable_whole(q) && window_overlap(q)) W = std::max(W, window_stride(ctx, rs, O, m.G, m.K, m.mode));
      }
    }
    if (W) {
      int rc = build_window_view(ctx, rs, nonempty, W, O, P.view, ctx->stream);
      if (rc) return rc;
      for (const Member &m : members) {
        const Query &q = ctx->queries.at(qids[m.pos]);
        if (windowable_whole(q) && window_overlap(q)) {
          windowed[m.pos] = 1;
          P.win_q.push_back(m.pos);
        }
      }
      const size_t nwq = (size_t)P.win_q.size() * P.view.nw;
      CU(P.wscore.ensure(nwq * 4 + 4));
      CU(P.wqend.ensure(nwq * 4 + 4));
      CU(P.wtend.ensure(nwq * 4 + 4));
      CU(P.whit.ensure(nwq + 16));
    }
  }
  const RecordSet view = P.view.nw ? window_set(rs, P.view) : RecordSet{};

  std::map<long, size_t> cls_of;
  for (const Member &m : members) {
    const long key = ((long)m.K << 8) | (m.mode << 4) | m.layout;
    auto it = cls_of.find(key);
    if (it == cls_of.end()) {
      MultiClass c;
      c.K = m.K;
      c.mode = m.mode;
      c.layout = m.layout;
      it = cls_of.emplace(key, P.classes.size()).first;
      P.classes.push_back(std::move(c));
    }
    MultiClass &c = P.classes[it->second];
    c.members.push_back(m.pos);
    c.Gmin = std::min(c.Gmin, m.G);
    c.prof_area = std::max(c.prof_area, (m.L->prof_bytes + 15u) & ~15u);
  }

  // ---- per class: kernel, occupancy, parameters, tiles ----
  for (MultiClass &c : P.classes) {
    const int lean = batch_lean(ctx, c.K, c.mode, c.Gmin);
    c.fn = batch_fn(c.K, c.mode, c.layout, lean);
    if (!c.fn) return fail(ctx, ISH_EOVERFLOW, "no batch kernel for K=%d", c.K);
    c.threads = wave_threads_lean(c.K, c.mode, lean);
    const size_t slot_words = (size_t)(c.threads / c.Gmin) * 32;
    const size_t save = c.mode == SW ? (size_t)c.threads * wave_save_words(c.K) * 4 : 0;
    c.smem = c.prof_area + slot_words * 4 + save;
    CU(cudaFuncSetAttribute((const void *)c.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem));
    int per_sm = 0;
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)c.fn, c.threads, c.smem));
    if (per_sm < 1) return fail(ctx, ISH_EOVERFLOW, "batch kernel K=%d does not fit (smem %zu)", c.K, c.smem);
    if (ctx->force_blocks) per_sm = std::min(per_sm, ctx->force_blocks);
    c.grid = (uint32_t)(per_sm * ctx->num_sms);

    std::vector<WaveParams> params(c.members.size());
    std::vector<BatchTile> tiles;
    for (size_t j = 0; j < c.members.size(); ++j) {
      const uint32_t pos = c.members[j];
      const Member &m = *std::find_if(members.begin(), members.end(), [&](const Member &x) { return x.pos == pos; });
      Query &q = ctx->queries.at(qids[pos]);
      OutDev out{(want & W_SCORE) ? P.score.as<int32_t>() + (size_t)pos * n : nullptr,
                 (want & W_QEND) ? P.qend.as<int32_t>() + (size_t)pos * n : nullptr,
                 (want & W_TEND) ? P.tend.as<int32_t>() + (size_t)pos * n : nullptr,
                 (want & (W_HIT | W_COMPACT)) ? P.hit.as<uint8_t>() + (size_t)pos * n : nullptr};
      if (windowed[pos]) {
        const size_t w = std::find(P.win_q.begin(), P.win_q.end(), pos) - P.win_q.begin();
        const size_t at = w * P.view.nw;
        OutDev wout{P.wscore.as<int32_t>() + at, P.wqend.as<int32_t>() + at, P.wtend.as<int32_t>() + at,
                    P.whit.as<uint8_t>() + at};
        wave_params(q, *m.L, view, wout, ctx->error.as<int>(), &params[j]);
        tiles.push_back(BatchTile{(uint32_t)j, 0, P.view.nw, 0});
      } else {
        wave_params(q, *m.L, rs, out, ctx->error.as<int>(), &params[j]);
        tiles.push_back(BatchTile{(uint32_t)j, 0, nonempty, 0});
      }
    }
    // the longest queries first: blocks that start on them finish with the rest
    std::stable_sort(tiles.begin(), tiles.end(), [&](const BatchTile &x, const BatchTile &y) {
      return params[x.q].Q > params[y.q].Q;
    });
    c.ntiles = (uint32_t)tiles.size();
    c.counter_base = P.n_counters;
    P.n_counters += c.ntiles;
    CU(c.params.ensure(params.size() * sizeof(WaveParams)));
    CU(c.tiles.ensure(std::max<size_t>(1, tiles.size()) * sizeof(BatchTile)));
    CU(cudaMemcpy(c.params.p, params.data(), params.size() * sizeof(WaveParams), cudaMemcpyHostToDevice));
    if (!tiles.empty()) CU(cudaMemcpy(c.tiles.p, tiles.data(), tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice));
  }
  CU(P.counters.ensure((size_t)std::max<uint32_t>(1, P.n_counters) * 4 + 16));
  if (want & W_COMPACT) {
    P.nb = std::max<uint32_t>(1, ceil_div(n, HIT_TILE));
    CU(P.block_counts.ensure((size_t)P.nb * nq * 4 + 8));
    CU(P.hit_idx.ensure(total * 4 + 4));
    CU(P.nhits.ensure(16));
  }
  for (size_t i = 1; i < P.classes.size(); ++i) {
    cudaStream_t st;
    CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    P.side.push_back(st);
  }
  for (size_t i = 0; i < P.classes.size() + 1; ++i) {
    cudaEvent_t e;
    CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    P.events.push_back(e);
  }
  return ISH_OK;
}

// Enqueues the whole batched launch on stream s (captured into the graph).
int enqueue_plan(ish_ctx *ctx, MultiPlan &P, RecordSet &rs, cudaStream_t s) {
  const uint32_t n = P.n;
  CU(cudaMemsetAsync(ctx->error.p, 0, 4, s));
  CU(cudaMemsetAsync(P.counters.p, 0, (size_t)std::max<uint32_t>(1, P.n_counters) * 4, s));
  if (P.classes.size() > 1) CU(cudaEventRecord(P.events[0], s));
  for (size_t i = 0; i < P.classes.size(); ++i) {
    MultiClass &c = P.classes[i];
    cudaStream_t cs = i == 0 ? s : P.side[i - 1];
    if (i > 0) CU(cudaStreamWaitEvent(cs, P.events[0], 0));
    BatchParams b{};
    b.queries = c.params.as<const WaveParams>();
    b.tiles = c.tiles.as<const BatchTile>();
    b.ntiles = c.ntiles;
    b.tile_counter = P.counters.as<uint32_t>() + c.counter_base;
    b.prof_area = c.prof_area;
    b.slot_words = (uint32_t)((c.threads / c.Gmin) * 32);
    b.step_cap = ctx->step_budget;
    if (c.ntiles) c.fn<<<c.grid, c.threads, c.smem, cs>>>(b);
    if (c.ntiles) ++P.kernels;
    CU(cudaGetLastError());
    if (i > 0) {
      CU(cudaEventRecord(P.events[i], cs));
      CU(cudaStreamWaitEvent(s, P.events[i], 0));
    }
  }
  // windowed queries: fold their window results into their outputs
  for (size_t w = 0; w < P.win_q.size(); ++w) {
    const uint32_t i = P.win_q[w];
    const Query &q = ctx->queries.at(P.qids[i]);
    OutDev out{(P.want & W_SCORE) ? P.score.as<int32_t>() + (size_t)i * n : nullptr,
               (P.want & W_QEND) ? P.qend.as<int32_t>() + (size_t)i * n : nullptr,
               (P.want & W_TEND) ? P.tend.as<int32_t>() + (size_t)i * n : nullptr,
               (P.want & (W_HIT | W_COMPACT)) ? P.hit.as<uint8_t>() + (size_t)i * n : nullptr};
    const size_t at = w * P.view.nw;
    int rc = merge_windows(ctx, rs, n - rs.n_empty, P.view, q, P.wscore.as<const int32_t>() + at,
                           P.wqend.as<const int32_t>() + at, P.wtend.as<const int32_t>() + at, out, s, &P.kernels);
    if (rc) return rc;
  }
  // queries the lane-exact kernels score
  for (uint32_t i : P.exact_q) {
    Query &q = ctx->queries.at(P.qids[i]);
    OutDev out{(P.want & W_SCORE) ? P.score.as<int32_t>() + (size_t)i * n : nullptr,
               (P.want & W_QEND) ? P.qend.as<int32_t>() + (size_t)i * n : nullptr,
               (P.want & W_TEND) ? P.tend.as<int32_t>() + (size_t)i * n : nullptr,
               (P.want & (W_HIT | W_COMPACT)) ? P.hit.as<uint8_t>() + (size_t)i * n : nullptr};
    int rc = exact_enqueue(ctx, q, rs, 0, n - rs.n_empty, out, s, P.exact, &P.kernels);
    if (rc) return rc;
  }
  // empty records and empty queries
  const RecordsDev rec{rs.codes.as<const uint8_t>(), rs.off_s.as<const uint64_t>(), rs.len_s.as<const uint32_t>(),
                       rs.orig_s.as<const uint32_t>(), rs.n};
  for (uint32_t i = 0; i < P.nq; ++i) {
    const Query &q = ctx->queries.at(P.qids[i]);
    const uint32_t n_empty = (q.Q == 0) ? n : rs.n_empty;
    if (!n_empty) continue;
    OutDev out{(P.want & W_SCORE) ? P.score.as<int32_t>() + (size_t)i * n : nullptr,
               (P.want & W_QEND) ? P.qend.as<int32_t>() + (size_t)i * n : nullptr,
               (P.want & W_TEND) ? P.tend.as<int32_t>() + (size_t)i * n : nullptr,
               (P.want & (W_HIT | W_COMPACT)) ? P.hit.as<uint8_t>() + (size_t)i * n : nullptr};
    k_trivial<<<std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(n_empty, 256), 1024)), 256, 0, s>>>(
        rec, n - n_empty, n_empty, q.algo == ISH_ALGO_LOCAL ? SW : SG, q.Q, out, Decision{q.max_score, q.thr});
    ++P.kernels;
    CU(cudaGetLastError());
  }
  if (P.want & W_COMPACT) {
    const dim3 g(P.nb, P.nq);
    k_count_hits<<<g, 1024, 0, s>>>(P.hit.as<uint8_t>(), n, P.block_counts.as<uint32_t>());
    ++P.kernels;
    k_scan_counts<<<1, 1024, 0, s>>>(P.block_counts.as<uint32_t>(), P.nb * P.nq, P.nhits.as<uint32_t>());
    ++P.kernels;
    k_write_hits<<<g, 1024, 0, s>>>(P.hit.as<uint8_t>(), n, P.block_counts.as<uint32_t>(), P.hit_idx.as<uint32_t>());
    ++P.kernels;
    CU(cudaGetLastError());
  }
  return ISH_OK;
}

int capture_plan(ish_ctx *ctx, MultiPlan &P, RecordSet &rs) {
  cudaStream_t s = ctx->stream;
  CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_plan(ctx, P, rs, s);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail(ctx, ISH_EDEVICE, "graph capture: %s", cudaGetErrorString(e));
  P.graph = g;
  CU(cudaGraphInstantiate(&P.exec, P.graph, 0));
  return ISH_OK;
}

}  // namespace

void drop_plans(ish_ctx *ctx, int32_t query_id, int32_t set_id) {
  bool synced = false;
  for (auto it = ctx->plans.begin(); it != ctx->plans.end();) {
    MultiPlan *P = it->second;
    const bool hit = (set_id && P->set_id == set_id) ||
                     (query_id && std::find(P->qids.begin(), P->qids.end(), query_id) != P->qids.end());
    if (hit || (!query_id && !set_id)) {
      if (!synced) cudaStreamSynchronize(ctx->stream);
      synced = true;
      P->release();
      delete P;
      it = ctx->plans.erase(it);
    } else {
      ++it;
    }
  }
}

void free_plans(ish_ctx *ctx) { drop_plans(ctx, 0, 0); }

}  // namespace host
}  // namespace ish

using namespace ish;
using namespace ish::host;

extern "C" {

int ish_gpu_score_multi(ish_ctx *ctx, const int32_t *query_ids, uint32_t n_queries, int32_t set_id, int32_t *score,
                        int32_t *query_end, int32_t *target_end, uint8_t *hit, uint32_t *hit_idx, uint64_t hit_cap,
                        uint64_t *hit_offsets) {
  if (!ctx) return ISH_EINVAL;
  if (n_queries && !query_ids) return fail(ctx, ISH_EINVAL, "query_ids is NULL");
  int urc = ISH_OK;
  RecordSet *si_set = use_set(ctx, set_id, &urc);
  if (!si_set) return urc;
  for (uint32_t i = 0; i < n_queries; ++i)
    if (!ctx->queries.count(query_ids[i])) return fail(ctx, ISH_EINVAL, "unknown query %d", query_ids[i]);
  RecordSet &rs = *si_set;
  const uint32_t n = rs.n;
  if (n_queries == 0 || n == 0) {
    if (hit_offsets)
      for (uint32_t i = 0; i <= n_queries; ++i) hit_offsets[i] = 0;
    ctx->last_ms = 0.f;
    return ISH_OK;
  }
  if (n_queries > 65535) return fail(ctx, ISH_EINVAL, "at most 65535 queries per batched launch (%u)", n_queries);
  if ((uint64_t)n_queries * n >= (1ull << 32))
    return fail(ctx, ISH_EOVERFLOW, "%u queries x %u records exceed 2^32 results per batched launch", n_queries, n);
  cudaSetDevice(ctx->device);
  const unsigned want = (score ? W_SCORE : 0) | (query_end ? W_QEND : 0) | (target_end ? W_TEND : 0) |
                        (hit ? W_HIT : 0) | ((hit_idx || hit_offsets) ? W_COMPACT : 0);
  const std::string key = plan_key(query_ids, n_queries, set_id, want);
  MultiPlan *P = nullptr;
  auto pit = ctx->plans.find(key);
  if (pit != ctx->plans.end()) {
    P = pit->second;
  } else {
    while (ctx->plans.size() >= MAX_PLANS) evict_one(ctx);
    P = new MultiPlan();
    int rc = build_plan(ctx, query_ids, n_queries, set_id, rs, want, *P);
    if (!rc) rc = capture_plan(ctx, *P, rs);
    if (rc) {
      cudaStreamSynchronize(ctx->stream);
      P->release();
      delete P;
      return rc;
    }
    ctx->plans.emplace(key, P);
  }
  P->last_use = ++g_use_clock;
  cudaStream_t s = ctx->stream;
  CU(cudaEventRecord(ctx->ev0, s));
  CU(cudaGraphLaunch(P->exec, s));
  ctx->launches += P->kernels;
  CU(cudaEventRecord(ctx->ev1, s));
  const size_t total = (size_t)n_queries * n;
  if (score) CU(cudaMemcpyAsync(score, P->score.p, total * 4, cudaMemcpyDeviceToHost, s));
  if (query_end) CU(cudaMemcpyAsync(query_end, P->qend.p, total * 4, cudaMemcpyDeviceToHost, s));
  if (target_end) CU(cudaMemcpyAsync(target_end, P->tend.p, total * 4, cudaMemcpyDeviceToHost, s));
  if (hit) CU(cudaMemcpyAsync(hit, P->hit.p, total, cudaMemcpyDeviceToHost, s));
  std::vector<uint32_t> offs;
  uint32_t *hs = reinterpret_cast<uint32_t *>(ctx->h_small);  // pinned: error flags, hit count
  hs[1] = 0;
  CU(cudaMemcpyAsync(hs, ctx->error.p, 4, cudaMemcpyDeviceToHost, s));
  if (want & W_COMPACT) {
    offs.resize((size_t)P->nb * n_queries);
    CU(cudaMemcpyAsync(offs.data(), P->block_counts.p, offs.size() * 4, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(hs + 1, P->nhits.p, 4, cudaMemcpyDeviceToHost, s));
  }
  CU(cudaStreamSynchronize(s));
  const int herr = (int)hs[0];
  const uint32_t nh = hs[1];
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) ctx->last_ms = ms;
  if (herr & 2) return fail(ctx, ISH_ETIMEDOUT, "batch kernel exceeded its step budget (internal error)");
  if (herr) return fail(ctx, ISH_EINVAL, "a record contains a code >= the alphabet size of a query");
  if (want & W_COMPACT) {
    if (hit_offsets) {
      for (uint32_t i = 0; i < n_queries; ++i) hit_offsets[i] = offs[(size_t)i * P->nb];
      hit_offsets[n_queries] = nh;
    }
    if (hit_idx) {
      if (nh > hit_cap) return fail(ctx, ISH_EOVERFLOW, "%u hits do not fit hit_idx (capacity %llu)", nh,
                                    (unsigned long long)hit_cap);
      if (nh) {
        CU(cudaMemcpyAsync(hit_idx, P->hit_idx.p, (size_t)nh * 4, cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
      }
    }
  }
  return ISH_OK;
}

int ish_gpu_autotune(ish_ctx *ctx, int32_t set_id, const int32_t *query_ids, uint32_t n_queries, int32_t *group,
                     int32_t *cols) {
  if (!ctx) return ISH_EINVAL;
  if (n_queries && !query_ids) return fail(ctx, ISH_EINVAL, "query_ids is NULL");
  int urc = ISH_OK;
  RecordSet *si_set = use_set(ctx, set_id, &urc);
  if (!si_set) return urc;
  RecordSet &rs = *si_set;
  cudaSetDevice(ctx->device);
  const uint32_t nonempty = rs.n - rs.n_empty;
  CU(ctx->out_score.ensure((size_t)rs.n * 4 + 4));
  CU(ctx->out_qend.ensure((size_t)rs.n * 4 + 4));
  CU(ctx->out_tend.ensure((size_t)rs.n * 4 + 4));
  CU(ctx->out_hit.ensure((size_t)rs.n + 16));
  CU(ctx->counter.ensure(64));
  CU(ctx->error.ensure(64));
  OutDev out{ctx->out_score.as<int32_t>(), ctx->out_qend.as<int32_t>(), ctx->out_tend.as<int32_t>(),
             ctx->out_hit.as<uint8_t>()};
  cudaStream_t s = ctx->stream;
  int rc = ISH_OK;
  for (uint32_t i = 0; i < n_queries && rc == ISH_OK; ++i) {
    auto qi = ctx->queries.find(query_ids[i]);
    if (qi == ctx->queries.end()) {
      rc = fail(ctx, ISH_EINVAL, "unknown query %d", query_ids[i]);
      break;
    }
    Query &q = qi->second;
    const int mode = q.algo == ISH_ALGO_LOCAL ? SW : SG;
    const uint64_t key = tune_key(mode, q.rows, q.Q);
    // (queries outside the wavefront kernels' exact regime run on the exact
    // kernels, which have no shapes to tune)
    if (q.Q > 0 && nonempty > 0 && !ctx->tuned.count(key) && fast_regime(ctx, q, rs)) {
      // candidates: every group size whose modelled cost is within 1.6x of
      // the best, each with its profile layout and the alternative one
      struct Cand {
        int G, K, layout;
        double model;
      };
      std::vector<Cand> cands;
      double best_model = 1e30;
      for (int g = 1; g <= 32; g <<= 1) {
        int k = (q.Q + 1 + g - 1) / g;
        if (k > 32) k = (k + 1) & ~1;
        if (!wave_k_available(k)) continue;
        const double m = (double)g * (k + 8) * (k > 48 ? 1.25 : 1.0);
        best_model = std::min(best_model, m);
        // the layout rule's pick, and the 16/32-bit alternative to it (the
        // 32-bit profile saves an ALU instruction per column but can cost
        // occupancy)
        const int pick = choose_layout(q.rows, g, k, mode);
        cands.push_back({g, k, pick, m});
        const int other = pick == PROF_S32 ? PROF_S16 : (pick == PROF_S16 ? PROF_S32 : -1);
        if (other >= 0 &&
            wave_smem((uint32_t)layout_bytes(other, q.rows, g, k), wave_block_threads(k, mode), g, k, mode) <= 227 * 1024)
          cands.push_back({g, k, other, m});
      }
      cands.erase(std::remove_if(cands.begin(), cands.end(), [&](const Cand &c) { return c.model > 1.6 * best_model; }),
                  cands.end());
      // sample: a run of sorted entries from the middle of the length order
      // holding about 4e9 cells
      const double want_res = 4e9 / std::max(q.Q, 1);
      uint32_t first = nonempty / 4, count = 0;
      {
        uint64_t pos = 0;
        double res = 0;
        for (uint32_t b = top_bucket(rs); b >= 1 && count == 0; --b) {
          const uint64_t c = rs.hist[b];
          if (pos + c > first) {
            const uint64_t from = std::max<uint64_t>(first, pos);
            for (uint64_t r = from; r < pos + c; ++r) {
              res += (double)bucket_len(b);
              if (res >= want_res) {
                count = (uint32_t)(r + 1 - first);
                break;
              }
            }
          }
          pos += c;
        }
        if (count == 0) count = nonempty - first;
      }
      double best_t = 1e30;
      Tuned best{};
      for (const Cand &c : cands) {
        float t = 1e30f;
        for (int rep = 0; rep < 3 && rc == ISH_OK; ++rep) {
          CU(cudaEventRecord(ctx->ev0, s));
          rc = launch_wave_range(ctx, q, rs, first, count, out, c.G, c.K, c.layout, s);
          CU(cudaEventRecord(ctx->ev1, s));
          CU(cudaStreamSynchronize(s));
          float ms = 0.f;
          CU(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
          if (rep > 0) t = std::min(t, ms);
        }
        if (rc) break;
        if (t < best_t) {
          best_t = t;
          best = Tuned{c.G, c.K, c.layout};
        }
      }
      if (rc) break;
      if (best.G) ctx->tuned[key] = best;
    }
    if (group || cols) {
      int G = 0, K = 0, layout = 0;
      if (q.Q > 0) pick_shape(ctx, q, &G, &K, &layout);
      if (group) group[i] = G;
      if (cols) cols[i] = K;
    }
  }
  drop_plans(ctx, 0, 0);  // batched plans were built with the old shapes
  return rc;
}

}  // extern "C"
