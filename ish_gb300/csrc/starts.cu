// starts.cu -- match starts on the device (ish_gpu_match_starts): the reverse
// pass that the CPU matchers run for every hit.
//
//   semi-global: semi_global_aln_start_end runs semi_global_aln again on the
//     reversed prefix record[0 : target_end + 1] with the reversed query and
//     swapped free ends; start = len(prefix) - reverse.reference - 1
//     (ishlib/matcher/alignment/semi_global_aln/striped.mojo:160-191, and the
//     matcher's find_start, striped_semi_global_matcher.mojo:259-276);
//   local: ssw_align runs sw over record[0 : ref_end + 1] backwards with the
//     reversed query; ref_begin = the record index of that pass's best
//     (ishlib/matcher/alignment/local_aln/striped.mojo:232-259).
//
// Both are the forward pass on reversed inputs, so the device builds the
// reversed prefixes of all hits as a packed record set, scores it with the
// wavefront kernel and the reversed query, and turns the reverse end row j
// into start = len(prefix) - 1 - j.
#include <algorithm>
#include <vector>

#include "host.h"

namespace ish {

__global__ void k_invert(const uint32_t *orig_s, uint32_t n, uint32_t *inv) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) inv[orig_s[s]] = s;
}

// Prefix length and 16-byte slot of every hit (the slot keeps at least one
// zero byte past the prefix and is never empty).
__global__ void k_rev_lengths(const uint32_t *hits, const int32_t *tend, uint32_t nh, const uint32_t *inv,
                              const uint32_t *len_s, uint32_t n, uint32_t *rlen, uint64_t *slot, uint32_t *orig,
                              int *error) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nh; i += gridDim.x * blockDim.x) {
    const uint32_t h = hits[i];
    uint32_t r = 0;
    if (h < n) {
      const int64_t T = len_s[inv[h]];
      int64_t e = (int64_t)tend[i] + 1;
      e = e < 0 ? 0 : e;
      r = (uint32_t)(e < T ? e : T);
    } else {
      atomicOr(error, 4);
    }
    rlen[i] = r;
    slot[i] = ((uint64_t)r + 16) & ~(uint64_t)15;
    orig[i] = i;
  }
}

// One warp per hit: reversed prefix, zero padded to the slot end.
__global__ void k_rev_pack(const uint32_t *hits, uint32_t nh, uint32_t n, const uint32_t *inv, const uint8_t *codes,
                           const uint64_t *off_s, const uint32_t *rlen, const uint64_t *poff, const uint64_t *slot,
                           uint8_t *dst) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nh; i += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t h = hits[i];
    const uint32_t r = rlen[i];
    const uint8_t *src = h < n ? codes + off_s[inv[h]] : codes;
    uint8_t *d = dst + poff[i];
    const uint64_t sz = slot[i];
    for (uint64_t j = lane; j < sz; j += 32) d[j] = j < r ? src[r - 1 - j] : 0;
  }
}

__global__ void k_starts(const uint32_t *rlen, const int32_t *rev_end, uint32_t nh, int64_t *start) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nh; i += gridDim.x * blockDim.x)
    start[i] = (int64_t)rlen[i] - 1 - rev_end[i];
}

namespace host {
namespace {

// The reversed query: sequence reversed, free query/target start and end
// swapped (semi_global_aln_start_end, striped.mojo:165-183).
Query &reverse_of(Query &q) {
  if (!q.reverse) {
    q.reverse.reset(new Query());
    Query &r = *q.reverse;
    clone_params(q, r);
    std::reverse(r.q.begin(), r.q.end());
    if (q.algo == ISH_ALGO_SEMI_GLOBAL) {
      const int e = q.ends;
      r.ends = ((e & ISH_FREE_QUERY_END) ? ISH_FREE_QUERY_START : 0) |
               ((e & ISH_FREE_QUERY_START) ? ISH_FREE_QUERY_END : 0) |
               ((e & ISH_FREE_TARGET_END) ? ISH_FREE_TARGET_START : 0) |
               ((e & ISH_FREE_TARGET_START) ? ISH_FREE_TARGET_END : 0);
    }
  }
  return *q.reverse;
}

}  // namespace
}  // namespace host
}  // namespace ish

using namespace ish;
using namespace ish::host;

extern "C" int ish_gpu_match_starts(ish_ctx *ctx, int32_t query_id, int32_t set_id, const uint32_t *hit_idx,
                                    const int32_t *target_end, uint32_t n_hits, int64_t *start) {
  if (!ctx) return ISH_EINVAL;
  auto qi = ctx->queries.find(query_id);
  if (qi == ctx->queries.end()) return fail(ctx, ISH_EINVAL, "unknown query %d", query_id);
  int urc = ISH_OK;
  RecordSet *si_set = use_set(ctx, set_id, &urc);
  if (!si_set) return urc;
  if (n_hits == 0) return ISH_OK;
  if (!hit_idx || !target_end || !start) return fail(ctx, ISH_EINVAL, "hit_idx, target_end and start are required");
  cudaSetDevice(ctx->device);
  Query &q = qi->second;
  RecordSet &rs = *si_set;
  const uint32_t n = rs.n;
  for (uint32_t i = 0; i < n_hits; ++i)
    if (hit_idx[i] >= n) return fail(ctx, ISH_EINVAL, "hit index %u >= %u records", hit_idx[i], n);
  Query &rq = reverse_of(q);
  // the reverse pass runs where the forward pass ran: the wavefront kernels
  // in their exact regime, else the lane-exact emulation (exact.cu)
  bool fast = rq.Q > 0 && ctx->kernel != ISH_KERNEL_EXACT;
  if (fast) {
    int G, K, layout;
    pick_shape(ctx, rq, &G, &K, &layout);
    Regime r = regime(rq, G ? G * K : rq.Q + 64);
    fast = r.fast && G && G * K >= rq.Q + 1 && (r.max_safe_len == ~0ull || rs.max_len <= r.max_safe_len);
  }
  if (rq.Q > 0 && rs.max_code >= (uint32_t)rq.alphabet)
    return fail(ctx, ISH_EINVAL, "a record contains code %u >= the alphabet size %d of the query", rs.max_code,
                rq.alphabet);
  cudaStream_t s = ctx->stream;
  const uint32_t nb = std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(n, 256), (uint32_t)ctx->num_sms * 8));
  if (!rs.inv.p) {
    CU(rs.inv.ensure((size_t)n * 4));
    k_invert<<<nb, 256, 0, s>>>(rs.orig_s.as<uint32_t>(), n, rs.inv.as<uint32_t>());
    ++ctx->launches;
    CU(cudaGetLastError());
  }
  // scratch: hits, ends, lengths, slots, offsets, identity order, reverse ends, starts
  DevBuf d_hits, d_tend, rlen, slot, poff, orig, rev_end, d_start, scan;
  RecordSet rev;
  auto cleanup = [&] {
    DevBuf *b[] = {&d_hits, &d_tend, &rlen, &slot, &poff, &orig, &rev_end, &d_start, &scan};
    for (DevBuf *x : b) x->release();
    rev.codes.release();
    rev.windows.release();
  };
  int rc = ISH_OK;
  do {
    const uint32_t tiles = ceil_div(n_hits, SCAN_TILE);
    if (tiles > SCAN_TILE) {
      rc = fail(ctx, ISH_EINVAL, "too many hits in one call (%u)", n_hits);
      break;
    }
#define SCU(call)                                                                                  \
  {                                                                                                \
    cudaError_t _e = (call);                                                                       \
    if (_e != cudaSuccess) {                                                                       \
      (void)cudaGetLastError();                                                                    \
      rc = fail(ctx, _e == cudaErrorMemoryAllocation ? ISH_ENOMEM : ISH_EDEVICE, "%s: %s", #call,  \
                cudaGetErrorString(_e));                                                           \
      break;                                                                                       \
    }                                                                                              \
  }
    SCU(d_hits.ensure((size_t)n_hits * 4));
    SCU(d_tend.ensure((size_t)n_hits * 4));
    SCU(rlen.ensure((size_t)n_hits * 4));
    SCU(slot.ensure((size_t)n_hits * 8));
    SCU(poff.ensure((size_t)n_hits * 8 + 8));
    SCU(orig.ensure((size_t)n_hits * 4));
    SCU(rev_end.ensure((size_t)n_hits * 4));
    SCU(d_start.ensure((size_t)n_hits * 8));
    SCU(scan.ensure((size_t)(tiles + 1) * 16));
    SCU(ctx->error.ensure(64));
    SCU(cudaMemsetAsync(ctx->error.p, 0, 4, s));
    SCU(cudaMemcpyAsync(d_hits.p, hit_idx, (size_t)n_hits * 4, cudaMemcpyHostToDevice, s));
    SCU(cudaMemcpyAsync(d_tend.p, target_end, (size_t)n_hits * 4, cudaMemcpyHostToDevice, s));
    const uint32_t hb = std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(n_hits, 256), (uint32_t)ctx->num_sms * 8));
    k_rev_lengths<<<hb, 256, 0, s>>>(d_hits.as<uint32_t>(), d_tend.as<int32_t>(), n_hits, rs.inv.as<uint32_t>(),
                                      rs.len_s.as<uint32_t>(), n, rlen.as<uint32_t>(), slot.as<uint64_t>(),
                                      orig.as<uint32_t>(), ctx->error.as<int>());
    ++ctx->launches;
    uint64_t *bsum = scan.as<uint64_t>();
    uint64_t *boff = bsum + tiles + 1;
    k_scan64_block<<<tiles, 1024, 0, s>>>(slot.as<uint64_t>(), poff.as<uint64_t>(), n_hits, bsum);
    ++ctx->launches;
    if (tiles > 1) {
      k_scan64_block<<<1, 1024, 0, s>>>(bsum, boff, tiles, nullptr);
      ++ctx->launches;
      k_scan64_add<<<tiles, 1024, 0, s>>>(poff.as<uint64_t>(), n_hits, boff);
      ++ctx->launches;
    }
    SCU(cudaGetLastError());
    uint64_t last[2] = {0, 0};
    SCU(cudaMemcpyAsync(&last[0], poff.as<uint64_t>() + n_hits - 1, 8, cudaMemcpyDeviceToHost, s));
    SCU(cudaMemcpyAsync(&last[1], slot.as<uint64_t>() + n_hits - 1, 8, cudaMemcpyDeviceToHost, s));
    SCU(cudaStreamSynchronize(s));
    const uint64_t bytes = last[0] + last[1];
    SCU(rev.codes.ensure(bytes + 16));
    k_rev_pack<<<std::max<uint32_t>(1, std::min<uint32_t>(ceil_div((uint64_t)n_hits * 32, 256),
                                                          (uint32_t)ctx->num_sms * 16)),
                 256, 0, s>>>(d_hits.as<uint32_t>(), n_hits, n, rs.inv.as<uint32_t>(), rs.codes.as<uint8_t>(),
                              rs.off_s.as<uint64_t>(), rlen.as<uint32_t>(), poff.as<uint64_t>(), slot.as<uint64_t>(),
                              rev.codes.as<uint8_t>());
    ++ctx->launches;
    SCU(cudaGetLastError());
    // the reversed prefixes as a record set in hit order (empty prefixes keep
    // reverse end 0, i.e. start -1, as semi_global_aln gives for an empty
    // record)
    rev.n = n_hits;
    rev.total = bytes;
    rev.off_s.p = poff.p;
    rev.len_s.p = rlen.p;
    rev.orig_s.p = orig.p;
    SCU(cudaMemsetAsync(rev_end.p, 0, (size_t)n_hits * 4, s));
    OutDev out{nullptr, nullptr, rev_end.as<int32_t>(), nullptr};
    if (rq.Q > 0 && fast) {
      // long prefixes (hits in long records) go through the window view like
      // a forward pass; it needs the longest prefix
      std::vector<uint32_t> hl(n_hits);
      SCU(cudaMemcpy(hl.data(), rlen.p, (size_t)n_hits * 4, cudaMemcpyDeviceToHost));
      rev.max_len = *std::max_element(hl.begin(), hl.end());
      bool windowed = false;
      rc = launch_windows(ctx, rq, rev, n_hits, out, s, &windowed);
      if (!rc && !windowed) rc = launch_range(ctx, rq, rev, 0, n_hits, out, s);
      if (!rc) SCU(cudaStreamSynchronize(s));
    } else if (rq.Q > 0) {
      rc = launch_exact(ctx, rq, rev, 0, n_hits, out, s);
    }
    rev.off_s.p = rev.len_s.p = rev.orig_s.p = nullptr;  // owned by poff / rlen / orig
    if (rc) break;
    k_starts<<<hb, 256, 0, s>>>(rlen.as<uint32_t>(), rev_end.as<int32_t>(), n_hits, d_start.as<int64_t>());
    ++ctx->launches;
    SCU(cudaGetLastError());
    int herr = 0;
    SCU(cudaMemcpyAsync(start, d_start.p, (size_t)n_hits * 8, cudaMemcpyDeviceToHost, s));
    SCU(cudaMemcpyAsync(&herr, ctx->error.p, 4, cudaMemcpyDeviceToHost, s));
    SCU(cudaStreamSynchronize(s));
    if (herr & 2) rc = fail(ctx, ISH_ETIMEDOUT, "wavefront kernel exceeded its step budget (internal error)");
    else if (herr) rc = fail(ctx, ISH_EINVAL, "bad hit index or record code");
#undef SCU
  } while (0);
  cudaStreamSynchronize(s);
  cleanup();
  return rc;
}
