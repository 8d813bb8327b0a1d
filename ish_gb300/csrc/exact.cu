// exact.cu -- lane-exact emulation of the reference's striped CPU passes on
// the device, for the parameters the wavefront kernels do not take:
// gap_open <= gap_extend (where the lazy-F pass's early exit makes results
// depend on the lane count) and int16 boundary rows that wrap (non-free target
// start on very long records).  It also serves ISH_KERNEL_EXACT on request.
//
// One tile of W threads emulates one W-lane SIMD vector of the reference and
// scores one record at a time: thread k is lane k.  Lane k only ever touches
// the stripe elements [j][k] of the H, E (and saved-H) arrays, which live in
// a per-tile slice of a global scratch buffer; the two cross-lane steps of the
// algorithm -- shifting a vector by one lane, and the lazy-F loop's "any lane"
// test -- are tile shuffles and votes.
//   semi_global_aln[int16, W]: ishlib/matcher/alignment/semi_global_aln/striped.mojo:252-498
//   sw[uint8 | uint16, W]:      ishlib/matcher/alignment/local_aln/striped.mojo:272-434
//   ssw_align's adaptive width (uint8 pass, uint16 rerun on saturation): 162-196
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include <algorithm>
#include <vector>

#include "host.h"

namespace cg = cooperative_groups;

namespace ish {

struct ExactParams {
  const void *prof;      // striped profile [code][seg][W] of the lane type
  int Q, seg;
  int open, ext, ends;   // penalties as the lane type holds them
  int min_s;             // smallest matrix entry (semi-global v_neg_limit)
  int bias;              // local alignment bias
  RecordsDev rec;
  uint32_t first, count;
  uint32_t *counter;
  void *scratch;         // per tile: 4 arrays of seg * W lane values
  size_t tile_stride;    // lane values per tile
  const uint8_t *redo;   // local uint16 pass: only entries with redo[s - first] set
  uint8_t *redo_out;     // local uint8 pass: flags entries whose score + bias >= 255
  OutDev out;
  Decision dec;
};

namespace {

__device__ __forceinline__ int sat16(int x) { return x < -32768 ? -32768 : (x > 32767 ? 32767 : x); }
template <int TMAX>
__device__ __forceinline__ int satu(int x) { return x < 0 ? 0 : (x > TMAX ? TMAX : x); }

// H(0, j) and the record-side boundary of semi_global_aln (striped.mojo:298-324),
// in the lane type: values wrap modulo 2^16 like the reference's scalars.
__device__ __forceinline__ int16_t sg_boundary(int i, bool ts, int16_t open, int16_t ext) {
  if (i == 0 || ts) return 0;
  return (int16_t)(-(long long)open - (long long)ext * (int16_t)(i - 1));
}

template <int W>
__global__ void __launch_bounds__(256) exact_sg_kernel(const __grid_constant__ ExactParams p) {
  auto tile = cg::tiled_partition<W>(cg::this_thread_block());
  const int k = tile.thread_rank();
  const size_t gid = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / W;
  const int seg = p.seg, Q = p.Q;
  int16_t *hs = reinterpret_cast<int16_t *>(p.scratch) + gid * p.tile_stride;
  int16_t *hl = hs + (size_t)seg * W;
  int16_t *pe = hl + (size_t)seg * W;
  const int16_t *prof = reinterpret_cast<const int16_t *>(p.prof);
  const bool qs = p.ends & 1, qe = p.ends & 2, ts = p.ends & 4, te = p.ends & 8;
  const int16_t open = (int16_t)p.open, ext = (int16_t)p.ext;
  // v_neg_limit (striped.mojo:329-334)
  const int16_t neg = ((int16_t)(-open) < (int16_t)p.min_s) ? (int16_t)(-32768 + open + 1)
                                                             : (int16_t)(-32768 - p.min_s + 1);
  const int offset = Q > 0 ? (Q - 1) % seg : 0;
  const int mask_lane = Q > 0 ? (Q - 1) / seg : 0;
  while (true) {
    uint32_t r = 0;
    if (k == 0) r = atomicAdd(p.counter, 1u);
    r = tile.shfl(r, 0);
    if (r >= p.count) break;
    const uint32_t s = p.first + r;
    const int T = (int)p.rec.len[s];
    const uint8_t *rec = p.rec.codes + p.rec.off[s];
    int score = 0, end_ref = 0, end_query = 0;
    if (Q > 0 && T > 0) {
      end_query = Q - 1;
      end_ref = -1;
      int16_t hlast = 0, hoff = 0;
      for (int i = 0; i < seg; ++i) {
        const int16_t idx = (int16_t)(k * seg + i);
        const int16_t tmp = qs ? (int16_t)0 : (int16_t)(-(long long)open - (long long)ext * idx);
        hs[(size_t)i * W + k] = tmp;
        pe[(size_t)i * W + k] = (int16_t)(tmp - open);
        if (i == seg - 1) hlast = tmp;
        if (i == offset) hoff = tmp;
      }
      int16_t vmaxh = neg;
      for (int i = 0; i < T; ++i) {
        int vf = neg;
        int vh = tile.shfl_up((int)hlast, 1);
        if (k == 0) vh = sg_boundary(i, ts, open, ext);
        int16_t *t = hl;
        hl = hs;
        hs = t;
        const int16_t *pr = prof + (size_t)rec[i] * seg * W;
        for (int j = 0; j < seg; ++j) {  // 364-394
          const size_t x = (size_t)j * W + k;
          int h = sat16(vh + pr[x]);
          const int e = pe[x];
          h = max(h, e);
          h = max(h, vf);
          hs[x] = (int16_t)h;
          const int hm = sat16(h - open);
          pe[x] = (int16_t)max(sat16(e - ext), hm);
          vf = max(sat16(vf - ext), hm);
          vh = hl[x];
          if (j == seg - 1) hlast = (int16_t)h;
          if (j == offset) hoff = (int16_t)h;
        }
        // lazy_f (396-434)
        bool stop = false;
        for (int kk = 0; kk < W && !stop; ++kk) {
          const int16_t ins = ts ? (int16_t)(0 - open) : (int16_t)(sg_boundary(i + 1, ts, open, ext) - open);
          vf = tile.shfl_up(vf, 1);
          if (k == 0) vf = ins;
          for (int j = 0; j < seg; ++j) {
            const size_t x = (size_t)j * W + k;
            const int h = max((int)hs[x], vf);
            hs[x] = (int16_t)h;
            if (j == seg - 1) hlast = (int16_t)h;
            if (j == offset) hoff = (int16_t)h;
            const int th = sat16(h - open);
            vf = sat16(vf - ext);
            if (!tile.any(vf > th)) {
              stop = true;
              break;
            }
          }
        }
        // last query row (436-441)
        const int16_t last = (int16_t)tile.shfl((int)hoff, mask_lane);
        if (last > vmaxh) end_ref = i;
        vmaxh = max(last, vmaxh);
      }
      score = neg;
      if (te) {  // 446-450
        score = vmaxh;
        end_query = Q - 1;
      }
      if (qe) {  // 453-468, as an order-free reduction
        int vmax = -32769, tmin = 0x7fffffff;
        for (int i = 0; i < seg; ++i) {
          const int temp = i + k * seg;
          if (temp >= Q) continue;
          const int v = hs[(size_t)i * W + k];
          if (v > vmax) {
            vmax = v;
            tmin = temp;
          } else if (v == vmax && temp < tmin) {
            tmin = temp;
          }
        }
        const int gmax = cg::reduce(tile, vmax, cg::greater<int>());
        const int gt = cg::reduce(tile, vmax == gmax ? tmin : 0x7fffffff, cg::less<int>());
        if (gmax > score) {
          score = gmax;
          end_query = gt;
          end_ref = T - 1;
        } else if (gmax == score && end_ref == T - 1 && gt < end_query) {
          end_query = gt;
        }
      }
      if (!te && !qe) {  // 471-477
        score = tile.shfl((int)hoff, mask_lane);
        end_ref = T - 1;
        end_query = Q - 1;
      }
    }
    if (k == 0) {
      const uint32_t orig = p.rec.orig[s];
      if (p.out.score) p.out.score[orig] = score;
      if (p.out.qend) p.out.qend[orig] = end_query;
      if (p.out.tend) p.out.tend[orig] = end_ref;
      if (p.out.hit) p.out.hit[orig] = decide(SG, score, end_query, end_ref, p.dec);
    }
  }
}

// sw[TY, W] (local_aln/striped.mojo:272-434), forward, terminate = type max.
template <int W, typename TY, int TMAX>
__global__ void __launch_bounds__(256) exact_sw_kernel(const __grid_constant__ ExactParams p) {
  auto tile = cg::tiled_partition<W>(cg::this_thread_block());
  const int k = tile.thread_rank();
  const size_t gid = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / W;
  const int seg = p.seg, Q = p.Q;
  TY *hs = reinterpret_cast<TY *>(p.scratch) + gid * p.tile_stride;
  TY *hl = hs + (size_t)seg * W;
  TY *pe = hl + (size_t)seg * W;
  TY *hm = pe + (size_t)seg * W;
  const TY *prof = reinterpret_cast<const TY *>(p.prof);
  const int open = p.open, ext = p.ext, bias = p.bias;
  while (true) {
    uint32_t r = 0;
    if (k == 0) r = atomicAdd(p.counter, 1u);
    r = tile.shfl(r, 0);
    if (r >= p.count) break;
    const uint32_t s = p.first + r;
    if (p.redo && !p.redo[r]) continue;
    const int T = (int)p.rec.len[s];
    const uint8_t *rec = p.rec.codes + p.rec.off[s];
    for (int j = 0; j < seg; ++j) {  // fresh vectors (the reference allocates them zeroed)
      const size_t x = (size_t)j * W + k;
      hs[x] = hl[x] = pe[x] = hm[x] = 0;
    }
    int max_score = 0, end_ref = -1, end_query = Q - 1;
    int vmax_score = 0, vmax_mark = 0;
    TY hlast = 0;
    for (int i = 0; i < T; ++i) {
      int vf = 0, vcol = 0;
      int vh = tile.shfl_up((int)hlast, 1);
      if (k == 0) vh = 0;
      TY *t = hl;
      hl = hs;
      hs = t;
      const TY *pr = prof + (size_t)rec[i] * seg * W;
      for (int j = 0; j < seg; ++j) {  // 346-371
        const size_t x = (size_t)j * W + k;
        int h = satu<TMAX>(vh + pr[x]);
        h = satu<TMAX>(h - bias);
        const int e = pe[x];
        h = max(h, e);
        h = max(h, vf);
        vcol = max(vcol, h);
        hs[x] = (TY)h;
        const int hm2 = satu<TMAX>(h - open);
        pe[x] = (TY)max(satu<TMAX>(e - ext), hm2);
        vf = max(satu<TMAX>(vf - ext), hm2);
        vh = hl[x];
        if (j == seg - 1) hlast = (TY)h;
      }
      bool stop = false;  // lazy_f (374-393)
      for (int kk = 0; kk < W && !stop; ++kk) {
        vf = tile.shfl_up(vf, 1);
        if (k == 0) vf = 0;
        for (int j = 0; j < seg; ++j) {
          const size_t x = (size_t)j * W + k;
          const int h = max((int)hs[x], vf);
          vcol = max(vcol, h);
          hs[x] = (TY)h;
          if (j == seg - 1) hlast = (TY)h;
          const int th = satu<TMAX>(h - open);
          vf = satu<TMAX>(vf - ext);
          if (!tile.any(vf > th)) {
            stop = true;
            break;
          }
        }
      }
      // new max check (395-411)
      vmax_score = max(vmax_score, vcol);
      if (!tile.all(vmax_mark == vmax_score)) {
        const int temp = cg::reduce(tile, vmax_score, cg::greater<int>());
        vmax_mark = vmax_score;
        if (temp > max_score) {
          max_score = temp;
          if ((TY)(max_score + bias) >= (TY)TMAX) break;
          end_ref = i;
          for (int j = 0; j < seg; ++j) hm[(size_t)j * W + k] = hs[(size_t)j * W + k];
        }
      }
      const int colmax = cg::reduce(tile, vcol, cg::greater<int>());  // 414-416
      if (colmax >= TMAX) break;
    }
    // 423-428: smallest query position of the maximum in the saved row
    int qmin = 0x7fffffff;
    for (int j = 0; j < seg; ++j)
      if ((int)hm[(size_t)j * W + k] == max_score) qmin = min(qmin, j + k * seg);
    qmin = cg::reduce(tile, qmin, cg::less<int>());
    if (qmin < end_query) end_query = qmin;
    if (k == 0) {
      if (p.redo_out) p.redo_out[r] = max_score + bias >= 255;
      const uint32_t orig = p.rec.orig[s];
      if (p.out.score) p.out.score[orig] = max_score;
      if (p.out.qend) p.out.qend[orig] = end_query;
      if (p.out.tend) p.out.tend[orig] = end_ref;
      if (p.out.hit) p.out.hit[orig] = decide(SW, max_score, end_query, end_ref, p.dec);
    }
  }
}

}  // namespace

namespace host {

namespace {

typedef void (*ExactFn)(const ExactParams);

ExactFn exact_fn(int mode, int W, int word) {
  if (mode == SG) {
    switch (W) {
      case 8: return exact_sg_kernel<8>;
      case 16: return exact_sg_kernel<16>;
      case 32: return exact_sg_kernel<32>;
    }
    return nullptr;
  }
  if (!word) {
    switch (W) {
      case 8: return exact_sw_kernel<8, uint8_t, 255>;
      case 16: return exact_sw_kernel<16, uint8_t, 255>;
      case 32: return exact_sw_kernel<32, uint8_t, 255>;
    }
    return nullptr;
  }
  switch (W) {
    case 8: return exact_sw_kernel<8, uint16_t, 65535>;
    case 16: return exact_sw_kernel<16, uint16_t, 65535>;
    case 32: return exact_sw_kernel<32, uint16_t, 65535>;
  }
  return nullptr;
}

// Striped profile of the reference (semi_global_aln/striped.mojo:92-118,
// local_aln/striped.mojo:110-139): p[code][i][k] = M[code][q[i + k * seg]],
// past the query 0 (semi-global) or the bias (local, biased by the bias).
template <typename TY>
std::vector<TY> striped_profile(const Query &q, int W, bool local, int bias) {
  const int seg = std::max(1, (q.Q + W - 1) / W);
  std::vector<TY> out((size_t)q.alphabet * seg * W);
  for (int c = 0; c < q.alphabet; ++c)
    for (int i = 0; i < seg; ++i)
      for (int k = 0; k < W; ++k) {
        const int j = i + k * seg;
        int v;
        if (!local) v = j >= q.Q ? 0 : q.M[(size_t)c * q.alphabet + q.q[j]];
        else v = j >= q.Q ? bias : (uint8_t)(int8_t)(q.M[(size_t)c * q.alphabet + q.q[j]] + (int8_t)bias);
        out[((size_t)c * seg + i) * W + k] = (TY)v;
      }
  return out;
}

// Lanes, lane type and grid of one pass: one tile per record in flight, each
// with a scratch slice of 4 * seg * W lane values; at most ~1 GB in all.
struct PassShape {
  int mode, W, word, seg;
  size_t tile_stride, tile_bytes;
  uint64_t blocks;
};

PassShape pass_shape(const ish_ctx *ctx, const Query &q, int mode, int W, int word, uint32_t count) {
  PassShape ps;
  ps.mode = mode;
  ps.W = W;
  ps.word = word;
  ps.seg = std::max(1, (q.Q + W - 1) / W);
  const size_t lane_bytes = (mode == SW && !word) ? 1 : 2;
  ps.tile_stride = (size_t)4 * ps.seg * W;
  ps.tile_bytes = ps.tile_stride * lane_bytes;
  const uint32_t tiles_per_block = 256 / W;
  uint64_t blocks = std::min<uint64_t>((uint64_t)ctx->num_sms * 8, ((uint64_t)count + tiles_per_block - 1) / tiles_per_block);
  blocks = std::min<uint64_t>(blocks, std::max<uint64_t>(1, (1ull << 30) / (ps.tile_bytes * tiles_per_block)));
  ps.blocks = std::max<uint64_t>(blocks, 1);
  return ps;
}

std::vector<PassShape> passes_of(const ish_ctx *ctx, const Query &q, uint32_t count) {
  if (q.algo == ISH_ALGO_SEMI_GLOBAL) return {pass_shape(ctx, q, SG, ctx->sg_lanes, 0, count)};
  return {pass_shape(ctx, q, SW, ctx->sw_u8_lanes, 0, count), pass_shape(ctx, q, SW, ctx->sw_u16_lanes, 1, count)};
}

long prof_key(const PassShape &ps) { return ((long)ps.mode << 16) | ((long)ps.word << 8) | ps.W; }

int enqueue_pass(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t first, uint32_t count, OutDev out, cudaStream_t s,
                 const PassShape &ps, ExactRes &res, const uint8_t *redo, uint8_t *redo_out, uint32_t *launches) {
  ExactFn fn = exact_fn(ps.mode, ps.W, ps.word);
  ExactParams p{};
  p.prof = q.exact_prof.at(prof_key(ps)).p;
  p.Q = q.Q;
  p.seg = ps.seg;
  p.open = ps.mode == SG ? q.open : (uint8_t)q.open;
  p.ext = ps.mode == SG ? q.ext : (uint8_t)q.ext;
  p.ends = q.ends;
  p.min_s = q.mmin;
  p.bias = ps.mode == SW ? -std::min(0, q.mmin) : 0;
  p.rec = RecordsDev{rs.codes.as<const uint8_t>(), rs.off_s.as<const uint64_t>(), rs.len_s.as<const uint32_t>(),
                     rs.orig_s.as<const uint32_t>(), rs.n};
  p.first = first;
  p.count = count;
  p.counter = res.counter.as<uint32_t>();
  p.scratch = res.scratch.p;
  p.tile_stride = ps.tile_stride;
  p.redo = redo;
  p.redo_out = redo_out;
  p.out = out;
  p.dec = Decision{q.max_score, q.thr};
  CU(cudaMemsetAsync(res.counter.p, 0, 4, s));
  fn<<<(uint32_t)ps.blocks, 256, 0, s>>>(p);
  ++*launches;
  CU(cudaGetLastError());
  return ISH_OK;
}

}  // namespace

// Uploads the striped profiles q needs and sizes res for passes over up to
// `count` records (no launch; call before a CUDA graph capture).
int exact_prepare(ish_ctx *ctx, Query &q, uint32_t count, ExactRes &res) {
  for (const PassShape &ps : passes_of(ctx, q, count)) {
    if (!exact_fn(ps.mode, ps.W, ps.word))
      return fail(ctx, ISH_EINVAL, "exact kernel: %d lanes are not supported (8, 16 or 32)", ps.W);
    DevBuf &prof = q.exact_prof[prof_key(ps)];
    if (!prof.p) {
      const int bias = ps.mode == SW ? -std::min(0, q.mmin) : 0;
      if (ps.mode == SG) {
        auto v = striped_profile<int16_t>(q, ps.W, false, 0);
        CU(prof.ensure(v.size() * 2));
        CU(cudaMemcpy(prof.p, v.data(), v.size() * 2, cudaMemcpyHostToDevice));
      } else if (!ps.word) {
        auto v = striped_profile<uint8_t>(q, ps.W, true, bias);
        CU(prof.ensure(v.size()));
        CU(cudaMemcpy(prof.p, v.data(), v.size(), cudaMemcpyHostToDevice));
      } else {
        auto v = striped_profile<uint16_t>(q, ps.W, true, bias);
        CU(prof.ensure(v.size() * 2));
        CU(cudaMemcpy(prof.p, v.data(), v.size() * 2, cudaMemcpyHostToDevice));
      }
    }
    CU(res.scratch.ensure(ps.blocks * (256 / ps.W) * ps.tile_bytes + 16));
  }
  CU(res.counter.ensure(64));
  CU(res.redo.ensure((size_t)count + 16));
  return ISH_OK;
}

// The reference's striped passes emulated lane by lane, for sorted entries
// [first, first + count) of rs, with resources from exact_prepare (no
// allocation, graph-capturable).  Local alignment runs the uint8 pass and
// reruns the entries that saturated it with uint16 lanes, as ssw_align does.
int exact_enqueue(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t first, uint32_t count, OutDev out, cudaStream_t s,
                  ExactRes &res, uint32_t *launches) {
  if (count == 0) return ISH_OK;
  const std::vector<PassShape> ps = passes_of(ctx, q, count);
  if (ps.size() == 1) return enqueue_pass(ctx, q, rs, first, count, out, s, ps[0], res, nullptr, nullptr, launches);
  int rc = enqueue_pass(ctx, q, rs, first, count, out, s, ps[0], res, nullptr, res.redo.as<uint8_t>(), launches);
  if (rc) return rc;
  return enqueue_pass(ctx, q, rs, first, count, out, s, ps[1], res, res.redo.as<uint8_t>(), nullptr, launches);
}

int launch_exact(ish_ctx *ctx, Query &q, RecordSet &rs, uint32_t first, uint32_t count, OutDev out, cudaStream_t s) {
  if (count == 0) return ISH_OK;
  int rc = exact_prepare(ctx, q, count, ctx->exact);
  if (rc) return rc;
  uint32_t n = 0;
  rc = exact_enqueue(ctx, q, rs, first, count, out, s, ctx->exact, &n);
  ctx->launches += n;
  return rc;
}

}  // namespace host
}  // namespace ish
