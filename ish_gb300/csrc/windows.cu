// windows.cu -- long records scored as overlapping windows.
//
// With a free target start, the best alignment of a query against a long
// record never spans more than a bounded number of record rows: a path over S
// rows makes at most Q diagonal steps, so at least S - Q rows are a gap in the
// query, and its score is at most Q * mmax - open - (S - Q - 1) * ext, while
// the best score is at least the full-query diagonal's Q * mmin (semi-global)
// or positive (local).  So S <= O = Q + 1 + (Q * mmax - open - M_min) / ext.
//
// A window of a record that starts at row s runs the same recurrence from a
// top boundary that only holds paths the whole record also has: for s = 0 the
// query's own, for s > 0 the fixed-query-start one, H(s-1, j) = -(open +
// ext*j) -- a start on the free left boundary at row s-1 followed by a query
// gap.  (A free query start may begin a path at any query column on row 0
// only; letting a later window begin one there would invent alignments.)  It
// then scores every cell at most as high as the whole record does (its paths
// are a subset), and exactly as high at every cell whose best path starts
// inside the window.  Windows that
// overlap by O rows therefore hold, for the record's best cell (the first
// row, then the smallest column, of its maximum), that cell's exact value in
// some window, and no cell before it reaches that value in any window.  The
// record's result is the window result with the largest score, then the
// smallest record row, then the smallest query column -- exactly the
// whole-record result, end coordinates and tie rules included:
//   semi-global with free target start and end and a fixed query end (the
//     target-end maximum of semi_global_aln/striped.mojo:436-450);
//   local alignment (local_aln/striped.mojo:395-428).
//
// The point is load balance: a pass over records of very unequal lengths is
// bound by its longest record pairs, one group each, however many groups
// finish early.  Windows of equal length spread those records over all
// groups.  This file decides when to window, builds the window view of the
// set (windows of the long records plus the other records whole, longest
// first), scores it with the wavefront kernel into per-window results, and
// folds them per record on the device.
#include <algorithm>
#include <numeric>
#include <vector>

#include "host.h"

namespace ish {

// One thread per sorted entry: fold the entry's window results (slots
// [cs[e], cs[e+1]), window w starting at record row start[w]) into its outputs.
__global__ void k_merge_windows(const uint32_t *orig_s, uint32_t n, const uint32_t *cs, const uint32_t *start,
                                const int32_t *ws, const int32_t *wq, const int32_t *wt, int mode, OutDev out,
                                Decision dec) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const uint32_t a = cs[e], b = cs[e + 1];
    int bs = ws[a], bq = wq[a];
    long long bt = wt[a] >= 0 ? (long long)wt[a] + start[a] : -1;
    for (uint32_t w = a + 1; w < b; ++w) {
      const int sc = ws[w], tq = wq[w];
      const long long tt = wt[w] >= 0 ? (long long)wt[w] + start[w] : -1;
      // equal scores carry rows of the same kind (all -1 when nothing beat
      // the initial best), so the row and column order the ties
      if (sc > bs || (sc == bs && tt >= 0 && (tt < bt || (tt == bt && tq < bq)))) {
        bs = sc;
        bq = tq;
        bt = tt;
      }
    }
    const uint32_t o = orig_s[e];
    if (out.score) out.score[o] = bs;
    if (out.qend) out.qend[o] = bq;
    if (out.tend) out.tend[o] = (int32_t)bt;
    if (out.hit) out.hit[o] = decide(mode, bs, bq, (int)bt, dec);
  }
}

namespace host {

// The query as windows past row 0 run it: its start fixed.
static Query &fixed_start_of(Query &q) {
  if (!(q.algo == ISH_ALGO_SEMI_GLOBAL && (q.ends & ISH_FREE_QUERY_START))) return q;
  if (!q.fixed_start) {
    q.fixed_start.reset(new Query());
    clone_params(q, *q.fixed_start);
    q.fixed_start->ends = q.ends & ~ISH_FREE_QUERY_START;
  }
  return *q.fixed_start;
}

bool windowable_whole(const Query &q) { return !(q.algo == ISH_ALGO_SEMI_GLOBAL && (q.ends & ISH_FREE_QUERY_START)); }

// Rows two windows of a record must share (see above), or 0 when no bound
// holds for this query.
uint64_t window_overlap(const Query &q) {
  const int mode = q.algo == ISH_ALGO_LOCAL ? SW : SG;
  if (q.ext < 1 || q.Q == 0) return 0;
  if (mode == SG && !((q.ends & ISH_FREE_TARGET_START) && (q.ends & ISH_FREE_TARGET_END) &&
                      !(q.ends & ISH_FREE_QUERY_END)))
    return 0;
  const long long mmin = mode == SG ? std::min(q.mmin, 0) : 0;
  const long long min_best = mode == SG ? (long long)q.Q * mmin : 0;
  const long long top = (long long)q.Q * std::max(q.mmax, 0) - q.open - min_best;
  const long long o = (long long)q.Q + 2 + std::max(0LL, (top + q.ext - 1) / q.ext);
  return (uint64_t)((o + 15) & ~15LL);
}

// Windows pay when the longest record exceeds ISH_WINDOW_QUARTERS / 4 of the
// rows a group scores on average: its pair alone would then outlast the pass.
// Measured on 10,000 records of 10 kb-1 Mb (1,000-nt query, 32-thread groups,
// 589k rows per group on average, 1M rows in the longest record): no windows
// at 2x (5,112-5,336 GCUPS), windows at 1.25x and 1x (6,794 / 6,803).
#ifndef ISH_WINDOW_QUARTERS
#define ISH_WINDOW_QUARTERS 5
#endif

// The window stride for scoring `rs` with groups of the given shape, or 0
// when windows would not help: the longest records must exceed twice the
// rows a group scores on average (they would bound the pass) and one window.
uint64_t window_stride(const ish_ctx *ctx, const RecordSet &rs, uint64_t O, int G, int K, int mode) {
  const int lean = wave_lean(ctx, K, mode, G);
  // groups in flight and the rows each would score on average (two records
  // per pair share their rows)
  const uint64_t groups =
      (uint64_t)ctx->num_sms * wave_blocks_lean(K, mode, lean) * (wave_threads_lean(K, mode, lean) / G);
  const uint64_t avg_rows = rs.total / 2 / std::max<uint64_t>(groups, 1);
  // window stride: about four pairs of windows per group, and at least 8x
  // the overlap so that windowing adds at most an eighth of the work
  uint64_t W = std::max<uint64_t>(8 * O, rs.total / std::max<uint64_t>(8 * groups, 1));
  W = (W + 15) & ~15ull;
  if (rs.max_len * 4 <= avg_rows * ISH_WINDOW_QUARTERS || rs.max_len <= W + O) return 0;
  return W;
}

// Builds the window view of sorted entries [0, nonempty) of rs (stride W,
// overlap O) into V, unless V already holds it.
int build_window_view(ish_ctx *ctx, const RecordSet &rs, uint32_t nonempty, uint64_t W, uint64_t O, WindowView &V,
                      cudaStream_t s) {
  if (V.nw && V.W == W && V.O == O && V.entries == nonempty) return ISH_OK;
  V.release();
  std::vector<uint32_t> len(nonempty);
  std::vector<uint64_t> off(nonempty);
  CU(cudaStreamSynchronize(s));
  CU(cudaMemcpy(len.data(), rs.len_s.p, (size_t)nonempty * 4, cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(off.data(), rs.off_s.p, (size_t)nonempty * 8, cudaMemcpyDeviceToHost));
  // slots: the windows of entry e are [cs[e], cs[e+1]); each has a first
  // record row, a length and a code offset
  std::vector<uint32_t> cs(nonempty + 1), wstart, wlen;
  std::vector<uint64_t> woff;
  for (uint32_t e = 0; e < nonempty; ++e) {
    cs[e] = (uint32_t)wstart.size();
    const uint64_t L = len[e];
    if (L <= W + O) {
      wstart.push_back(0);
      wlen.push_back((uint32_t)L);
      woff.push_back(off[e]);
      continue;
    }
    for (uint64_t k = 0; k * W < L; ++k) {
      const uint64_t st = k == 0 ? 0 : ((k * W - O) & ~15ull);
      const uint64_t en = std::min<uint64_t>(L, (k + 1) * W);
      wstart.push_back((uint32_t)st);
      wlen.push_back((uint32_t)(en - st));
      woff.push_back(off[e] + st);
    }
  }
  const uint32_t nw = (uint32_t)wstart.size();
  cs[nonempty] = nw;
  // the view: windows that start at record row 0 first, then the others,
  // each group longest first (pairs of similar length)
  std::vector<uint32_t> order(nw);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
    if ((wstart[a] == 0) != (wstart[b] == 0)) return wstart[a] == 0;
    return wlen[a] > wlen[b];
  });
  uint32_t n_first = 0;
  while (n_first < nw && wstart[order[n_first]] == 0) ++n_first;
  std::vector<uint32_t> vlen(nw), vslot(nw);
  std::vector<uint64_t> voff(nw);
  uint64_t vtotal = 0;
  for (uint32_t i = 0; i < nw; ++i) {
    vlen[i] = wlen[order[i]];
    voff[i] = woff[order[i]];
    vslot[i] = order[i];
    vtotal += vlen[i];
  }
  CU(V.off.ensure((size_t)nw * 8));
  CU(V.len.ensure((size_t)nw * 4));
  CU(V.slot.ensure((size_t)nw * 4));
  CU(V.start.ensure((size_t)nw * 4));
  CU(V.cs.ensure((size_t)(nonempty + 1) * 4));
  CU(cudaMemcpy(V.off.p, voff.data(), (size_t)nw * 8, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(V.len.p, vlen.data(), (size_t)nw * 4, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(V.slot.p, vslot.data(), (size_t)nw * 4, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(V.start.p, wstart.data(), (size_t)nw * 4, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(V.cs.p, cs.data(), (size_t)(nonempty + 1) * 4, cudaMemcpyHostToDevice));
  V.W = W;
  V.O = O;
  V.entries = nonempty;
  V.nw = nw;
  V.n_first = n_first;
  V.total = vtotal;
  V.max_len = *std::max_element(vlen.begin(), vlen.end());
  return ISH_OK;
}

// A record set over rs's codes whose entries are the windows of V (the
// buffers are borrowed: the view is never released).
RecordSet window_set(const RecordSet &rs, const WindowView &V) {
  RecordSet view;
  view.n = V.nw;
  view.total = V.total;
  view.max_len = V.max_len;
  view.codes = rs.codes;
  view.off_s = V.off;
  view.len_s = V.len;
  view.orig_s = V.slot;
  return view;
}

// Folds per-window results into the records' outputs.
int merge_windows(ish_ctx *ctx, const RecordSet &rs, uint32_t nonempty, const WindowView &V, const Query &q,
                  const int32_t *ws, const int32_t *wq, const int32_t *wt, OutDev out, cudaStream_t s,
                  uint32_t *kernels) {
  const int mode = q.algo == ISH_ALGO_LOCAL ? SW : SG;
  const uint32_t nb = std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(nonempty, 256), (uint32_t)ctx->num_sms * 8));
  k_merge_windows<<<nb, 256, 0, s>>>(rs.orig_s.as<const uint32_t>(), nonempty, V.cs.as<const uint32_t>(),
                                     V.start.as<const uint32_t>(), ws, wq, wt, mode, out,
                                     Decision{q.max_score, q.thr});
  if (kernels)
    ++*kernels;  // a captured launch: the caller counts it per replay
  else
    ++ctx->launches;
  CU(cudaGetLastError());
  return ISH_OK;
}

// Scores sorted entries [0, nonempty) of rs through the window view when its
// longest records would bound the pass; *done is false when it did nothing.
// The view is built once per (set, stride, overlap) and kept with the set.
int launch_windows(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t nonempty, OutDev out, cudaStream_t s,
                   bool *done) {
  *done = false;
  if (!ctx->windows_on || ctx->kernel != ISH_KERNEL_AUTO || nonempty == 0 || nonempty > (1u << 22)) return ISH_OK;
  const uint64_t O = window_overlap(q);
  if (!O) return ISH_OK;
  const int mode = q.algo == ISH_ALGO_LOCAL ? SW : SG;
  int G, K, layout;
  pick_shape(ctx, q, &G, &K, &layout);
  if (!G || !wave_fits(q, G, K, layout)) return ISH_OK;
  const uint64_t W = window_stride(ctx, rs, O, G, K, mode);
  if (!W) return ISH_OK;
  WindowView &V = rs.windows;
  int rc = build_window_view(ctx, rs, nonempty, W, O, V, s);
  if (rc) return rc;
  const uint32_t nw = V.nw;
  WindowOut &R = ctx->window_out;
  CU(R.score.ensure((size_t)nw * 4));
  CU(R.qend.ensure((size_t)nw * 4));
  CU(R.tend.ensure((size_t)nw * 4));
  CU(R.hit.ensure((size_t)nw));
  RecordSet view = window_set(rs, V);
  OutDev wout{R.score.as<int32_t>(), R.qend.as<int32_t>(), R.tend.as<int32_t>(), R.hit.as<uint8_t>()};
  Query &qc = fixed_start_of(q);
  if (&qc == &q) {
    rc = launch_wave_range(ctx, q, view, 0, nw, wout, G, K, layout, s);
  } else {
    rc = launch_wave_range(ctx, q, view, 0, V.n_first, wout, G, K, layout, s);
    if (!rc && nw > V.n_first) rc = launch_wave_range(ctx, qc, view, V.n_first, nw - V.n_first, wout, G, K, layout, s);
  }
  if (!rc)
    rc = merge_windows(ctx, rs, nonempty, V, q, R.score.as<const int32_t>(), R.qend.as<const int32_t>(),
                       R.tend.as<const int32_t>(), out, s, nullptr);
  if (rc) return rc;
  ctx->last_windows = nw;
  *done = true;
  return ISH_OK;
}

}  // namespace host
}  // namespace ish
