// fastx.cu -- FASTA/FASTQ records split, encoded and packed on the device.
//
// Replaces the FASTX runners' record reader (ishlib/vendor/kseq.mojo:370-461,
// FastxReader[read_comment=False].read, called in a loop by
// ishlib/parallel_fastx_search_runner.mojo:93-121 and 339-362 until a read
// returns 0 or less).  The reader is a byte-level state machine, but every
// decision it takes is made at a line start, so it is restated here as a
// machine over LINES with four states:
//
//   SEEK  looking for a header: the first '>' or '@' anywhere in the line
//         starts one (kseq.mojo:383-393), the rest of the line is its name;
//   SEQ   a sequence line is expected: leading '\r's are skipped (429-431) and
//         the next byte c decides -- '>' or '@' ends the record and starts the
//         next header at c, '+' starts a FASTQ quality, end of line (the line
//         held only '\r's) appends a '\n' AND the whole next line (read_until
//         is called after pushing c), anything else appends c and the rest of
//         the line;
//   ABS   the line appended whole after such an empty line;
//   QUAL  the quality line after a '+' line; the next line is SEEK again.
//
// A line's effect on the state is a map {SEEK,SEQ,ABS,QUAL} -> state (one
// byte), maps compose associatively, so the state at every line start comes
// from a parallel prefix scan of the lines' maps.  read_until drops one
// trailing '\r' from the buffer it fills when that buffer is longer than one
// byte (kseq.mojo:318-323), which here means: one trailing '\r' of every
// appended sequence line, of a name longer than one byte and of a quality
// longer than one byte.
//
// A FASTQ quality may span several lines in kseq (454-457: lines are read
// until the quality is as long as the sequence).  That depends on lengths,
// not on a finite state, so the device takes one quality line per record and
// refuses a file in which a record's quality continues on the next line
// (ISH_EINVAL) rather than splitting it differently.
#include "host.h"

namespace ish {

namespace {

constexpr uint32_t FX_SEEK = 0, FX_SEQ = 1, FX_ABS = 2, FX_QUAL = 3;
constexpr uint32_t MAP_ID = 0xE4;  // s -> s
constexpr uint32_t FX_TILE = 4096;  // lines per block (1024 threads x 4)
constexpr int FX_PER = 4;
// line roles
constexpr uint8_t R_SKIP = 0, R_HEADER = 1, R_SEQ = 2, R_EMPTY = 3, R_ABS = 4, R_PLUS = 5, R_QUAL = 6, R_END = 7;
// per-record flags
constexpr uint32_t F_PLUS = 1, F_QUAL = 2, F_QUAL_MORE = 4, F_STOP = 8;

__device__ __forceinline__ uint32_t map_apply(uint32_t m, uint32_t s) { return (m >> (2 * s)) & 3u; }
// a first, then b
__device__ __forceinline__ uint32_t map_then(uint32_t a, uint32_t b) {
  uint32_t r = 0;
#pragma unroll
  for (uint32_t s = 0; s < 4; ++s) r |= map_apply(b, map_apply(a, s)) << (2 * s);
  return r;
}

struct Line {
  uint64_t s, e;  // [s, e): the line without its '\n'
  bool nl;        // ends with '\n'
};
__device__ __forceinline__ Line line_at(const uint64_t *nl, uint32_t n_nl, uint64_t bytes, uint32_t i) {
  Line L;
  L.s = i == 0 ? 0 : nl[i - 1] + 1;
  L.nl = i < n_nl;
  L.e = L.nl ? nl[i] : bytes;
  return L;
}

// The byte that decides a line read in state SEQ (after its leading '\r's):
// the byte itself, '\n' for a line of only '\r's, -1 at the end of the file.
__device__ __forceinline__ int seq_char(const uint8_t *text, const Line &L, uint64_t *sp) {
  uint64_t k = L.s;
  while (k < L.e && text[k] == '\r') ++k;
  *sp = k;
  return k < L.e ? (int)text[k] : (L.nl ? '\n' : -1);
}

__device__ __forceinline__ uint32_t line_map(const uint8_t *text, const Line &L, uint64_t hc) {
  uint64_t sp;
  const int c = seq_char(text, L, &sp);
  const uint32_t on_seek = hc < L.e ? FX_SEQ : FX_SEEK;
  const uint32_t on_seq = c == '+' ? FX_QUAL : (c == '\n' ? FX_ABS : FX_SEQ);
  return on_seek | (on_seq << 2) | (FX_SEQ << 4) | (FX_SEEK << 6);
}

// Exclusive scan of one map per thread over a 1024-thread block, in thread
// order; *total receives the composition of all of them.
__device__ uint32_t block_excl_maps(uint32_t m, uint32_t *total) {
  __shared__ uint32_t wt[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t incl = m;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl = map_then(y, incl);
  }
  uint32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
  if (lane == 0) excl = MAP_ID;
  if (lane == 31) wt[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    uint32_t v = lane < nw ? wt[lane] : MAP_ID;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v = map_then(y, v);
    }
    wt[lane] = v;  // inclusive over warps
  }
  __syncthreads();
  const uint32_t wp = wid ? wt[wid - 1] : MAP_ID;
  *total = wt[nw - 1];
  __syncthreads();  // wt is reused by the next call
  return map_then(wp, excl);
}

// First '>' or '@' of every line (the header a SEEK line starts), by
// atomicMin; hc is preset to all ones.  block_offsets: newlines before each
// LINE_TILE-byte tile (exclusive scan of k_count_newlines).
__global__ void __launch_bounds__(1024) k_fx_header_chars(const uint8_t *text, uint64_t bytes,
                                                          const uint32_t *block_offsets, unsigned long long *hc) {
  __shared__ uint32_t wsum[32];
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t w0 = (uint64_t)blockIdx.x * LINE_TILE + (uint64_t)wid * LINE_WARP;
  uint32_t run = warp_newline_base(text, bytes, block_offsets, w0, lane, wid, wsum);
  for (uint32_t k = 0; k < LINE_WARP; k += 128) {
    const uint64_t i = w0 + k + 4 * lane;
    uint32_t nl = 0, h = 0;
    if (i < bytes) {
      nl = byte_bits(text, bytes, i, '\n');
      h = byte_bits(text, bytes, i, '>') | byte_bits(text, bytes, i, '@');
    }
    const uint32_t cnt = __popc(nl);
    uint32_t incl = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    const uint32_t before = run + incl - cnt;  // newlines before this lane's 4 bytes
    while (h) {
      const uint32_t bit = (uint32_t)(__ffs(h) - 1);
      atomicMin(hc + before + __popc(nl & ((1u << bit) - 1u)), (unsigned long long)(i + bit));
      h &= h - 1;
    }
    run += __shfl_sync(0xffffffffu, incl, 31);
  }
}

// Composition of the maps of each tile of FX_TILE lines.
__global__ void k_fx_tile_maps(const uint8_t *text, uint64_t bytes, const uint64_t *nl, uint32_t n_nl, uint32_t n,
                               const unsigned long long *hc, uint32_t *tile_map) {
  const uint32_t first = blockIdx.x * FX_TILE + threadIdx.x * FX_PER;
  uint32_t m = MAP_ID;
  for (int k = 0; k < FX_PER; ++k) {
    const uint32_t i = first + k;
    if (i < n) m = map_then(m, line_map(text, line_at(nl, n_nl, bytes, i), hc[i]));
  }
  uint32_t total;
  (void)block_excl_maps(m, &total);
  if (threadIdx.x == 0) tile_map[blockIdx.x] = total;
}

// State at the first line of every tile, from SEEK at the start of the file
// (one block, sequential chunks of 1024 tiles).
__global__ void k_fx_tile_states(const uint32_t *tile_map, uint32_t tiles, uint8_t *tile_state) {
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = FX_SEEK;
  __syncthreads();
  for (uint32_t base = 0; base < tiles; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    uint32_t total;
    const uint32_t pre = block_excl_maps(i < tiles ? tile_map[i] : MAP_ID, &total);
    const uint32_t c = carry;
    if (i < tiles) tile_state[i] = (uint8_t)map_apply(pre, c);
    __syncthreads();
    if (threadIdx.x == 0) carry = map_apply(total, c);
    __syncthreads();
  }
}

// Role of every line, the bytes it adds to its record's sequence (len) and
// where they start (src), and a header flag for the record numbering.
__global__ void k_fx_roles(const uint8_t *text, uint64_t bytes, const uint64_t *nl, uint32_t n_nl, uint32_t n,
                           const unsigned long long *hc, const uint8_t *tile_state, uint8_t *role, uint64_t *len,
                           uint64_t *src, uint64_t *hdr) {
  const uint32_t first = blockIdx.x * FX_TILE + threadIdx.x * FX_PER;
  uint32_t m = MAP_ID;
  for (int k = 0; k < FX_PER; ++k) {
    const uint32_t i = first + k;
    if (i < n) m = map_then(m, line_map(text, line_at(nl, n_nl, bytes, i), hc[i]));
  }
  uint32_t total;
  const uint32_t pre = block_excl_maps(m, &total);
  uint32_t st = map_apply(pre, tile_state[blockIdx.x]);
  for (int k = 0; k < FX_PER; ++k) {
    const uint32_t i = first + k;
    if (i >= n) break;
    const Line L = line_at(nl, n_nl, bytes, i);
    uint8_t r = R_SKIP;
    uint64_t ln = 0, from = 0;
    if (st == FX_SEEK) {
      if (hc[i] < L.e) {
        r = R_HEADER;
        from = hc[i];
      }
    } else if (st == FX_SEQ) {
      uint64_t sp;
      const int c = seq_char(text, L, &sp);
      if (c < 0) {
        r = R_END;
      } else if (c == '\n') {
        r = R_EMPTY;
        ln = 1;
      } else if (c == '>' || c == '@') {
        r = R_HEADER;
        from = sp;
      } else if (c == '+') {
        r = R_PLUS;
      } else {
        r = R_SEQ;
        from = sp;
        ln = L.e - sp;
        if (ln > 1 && text[L.e - 1] == '\r') --ln;
      }
    } else if (st == FX_ABS) {
      r = R_ABS;
      from = L.s;
      ln = L.e - L.s;
      if (ln >= 1 && text[L.e - 1] == '\r') --ln;  // the buffer already holds the pushed '\n'
    } else {
      r = R_QUAL;
    }
    role[i] = r;
    len[i] = ln;
    src[i] = from;
    hdr[i] = r == R_HEADER;
    st = map_apply(line_map(text, L, hc[i]), st);
  }
}

// Per record: sequence offset, name and quality bounds, FASTQ flags.
// rec_excl: headers before each line; pos: sequence bytes before each line.
__global__ void k_fx_records(const uint8_t *text, uint64_t bytes, const uint64_t *nl, uint32_t n_nl, uint32_t n,
                             const uint8_t *role, const uint64_t *rec_excl, const uint64_t *pos, uint64_t *rec_off,
                             uint64_t *bounds, uint32_t *flags, const uint64_t *src) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint8_t r = role[i];
    if (r == R_HEADER) {
      const uint64_t rec = rec_excl[i];
      const Line L = line_at(nl, n_nl, bytes, i);
      const uint64_t h = src[i];
      uint64_t ne = L.e;
      if (ne - (h + 1) > 1 && text[ne - 1] == '\r') --ne;
      rec_off[rec] = pos[i];
      bounds[4 * rec + 0] = h + 1;  // the quality half stays 0 unless a quality line sets it
      bounds[4 * rec + 1] = ne;
      // a header byte with nothing after it: the name read hits the end of
      // the file and the reader stops (kseq.mojo:416-421)
      if (h + 1 >= bytes) atomicOr(flags + rec, F_STOP);
    } else if (r == R_PLUS) {
      const uint64_t rec = rec_excl[i] - 1;
      const Line L = line_at(nl, n_nl, bytes, i);
      // no newline after '+': -2; no quality line after it: -3 (445-459)
      atomicOr(flags + rec, F_PLUS | ((!L.nl || i + 1 >= n) ? F_STOP : 0u));
    } else if (r == R_QUAL) {
      const uint64_t rec = rec_excl[i] - 1;
      const Line L = line_at(nl, n_nl, bytes, i);
      uint64_t qe = L.e;
      if (qe - L.s > 1 && text[qe - 1] == '\r') --qe;
      bounds[4 * rec + 2] = L.s;
      bounds[4 * rec + 3] = qe;
      atomicOr(flags + rec, F_QUAL | (i + 1 < n ? F_QUAL_MORE : 0u));
    }
  }
}

// The first record at which the reader returns 0 or less (an empty sequence,
// a quality of the wrong length or a missing one), as 2 * record + (1 if the
// cause is a quality continued on the next line, which the device does not
// split); records from there on are not part of the set.
__global__ void k_fx_check(uint32_t nrec, const uint64_t *rec_off, const uint64_t *bounds, const uint32_t *flags,
                           unsigned long long *first_bad) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += gridDim.x * blockDim.x) {
    const uint64_t seqlen = rec_off[r + 1] - rec_off[r];
    const uint32_t f = flags[r];
    bool stop = (f & F_STOP) || seqlen == 0;
    bool unsupported = false;
    if (!stop && (f & F_PLUS)) {
      const uint64_t qlen = (f & F_QUAL) ? bounds[4 * r + 3] - bounds[4 * r + 2] : 0;
      if (!(f & F_QUAL) || qlen > seqlen) stop = true;
      else if (qlen < seqlen) {
        if (f & F_QUAL_MORE) unsupported = true;
        else stop = true;  // the next quality read hits the end of the file: -3
      }
    }
    if (stop || unsupported) atomicMin(first_bad, 2ull * r + (unsupported ? 1ull : 0ull));
  }
}

// Sequence bytes of every line into their records' places: one warp per
// line, lane k copying bytes k, k + 32, ... (coalesced on both sides).
__global__ void k_fx_gather(const uint8_t *text, uint32_t n, const uint8_t *role, const uint64_t *len,
                            const uint64_t *src, const uint64_t *pos, uint8_t *out) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const uint64_t ln = len[i];
    if (!ln) continue;
    uint8_t *d = out + pos[i];
    if (role[i] == R_EMPTY) {
      if (lane == 0) d[0] = '\n';
      continue;
    }
    const uint8_t *s = text + src[i];
    for (uint64_t k = lane; k < ln; k += 32) d[k] = s[k];
  }
}

// rec_off[nrec] = all sequence bytes
__global__ void k_fx_totals(uint32_t n, const uint64_t *len, const uint64_t *pos, const uint64_t *hdr,
                            const uint64_t *rec_excl, uint64_t *rec_off, uint64_t *totals) {
  const uint64_t seq = n ? pos[n - 1] + len[n - 1] : 0;
  const uint64_t nrec = n ? rec_excl[n - 1] + hdr[n - 1] : 0;
  rec_off[nrec] = seq;
  totals[0] = nrec;
  totals[1] = seq;
}

}  // namespace

namespace host {

// Exclusive scan of n uint64 values (any n below 2^32), tile by tile.
int scan_u64(ish_ctx *ctx, const uint64_t *in, uint64_t *out, uint64_t n, DevBuf &tmp, size_t tmp_off = 0) {
  if (n == 0) return ISH_OK;
  cudaStream_t s = ctx->stream;
  const uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  // this level's tile sums and their scan, then deeper levels
  const size_t need = tmp_off + (size_t)(tiles + 1) * 16;
  if (tmp.cap < need) return fail(ctx, ISH_EINVAL, "scan scratch too small");
  uint64_t *bsum = reinterpret_cast<uint64_t *>(static_cast<char *>(tmp.p) + tmp_off);
  uint64_t *boff = bsum + tiles + 1;
  k_scan64_block<<<(uint32_t)tiles, 1024, 0, s>>>(in, out, (uint32_t)n, tiles > 1 ? bsum : nullptr);
  ++ctx->launches;
  if (tiles > 1) {
    int rc = scan_u64(ctx, bsum, boff, tiles, tmp, need);
    if (rc) return rc;
    k_scan64_add<<<(uint32_t)tiles, 1024, 0, s>>>(out, (uint32_t)n, boff);
    ++ctx->launches;
  }
  CU(cudaGetLastError());
  return ISH_OK;
}

size_t scan_u64_scratch(uint64_t n) {
  size_t b = 0;
  while (n > 1) {
    const uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    b += (size_t)(tiles + 1) * 16;
    n = tiles;
  }
  return b + 64;
}

int load_fastx(ish_ctx *ctx, const uint8_t *text, uint64_t bytes, RecordSet &rs, const uint8_t *enc, uint32_t *n_out,
               uint64_t *bounds_out, uint64_t bounds_cap) {
  *n_out = 0;
  rs.n = 0;
  rs.total = 0;
  if (bytes == 0) return ISH_OK;
  if (!text) return fail(ctx, ISH_EINVAL, "text is NULL");
  cudaStream_t s = ctx->stream;
  FastxScratch &fx = ctx->fastx;
  CU(ctx->raw.ensure(bytes + 32));
  CU(cudaEventRecord(ctx->load_ev[0], s));
  CU(cudaMemcpyAsync(ctx->raw.p, text, bytes, cudaMemcpyHostToDevice, s));
  const uint8_t *dtext = ctx->raw.as<uint8_t>();
  // ---- newlines, as for line records ----
  const uint64_t tiles64 = (bytes + LINE_TILE - 1) / LINE_TILE;
  if (tiles64 > 0x7fffffffull) return fail(ctx, ISH_EINVAL, "text too large");
  const uint32_t btiles = (uint32_t)tiles64;
  CU(ctx->block_counts.ensure((size_t)btiles * 4 + 8));
  CU(ctx->nhits.ensure(16));
  k_count_newlines<<<btiles, 1024, 0, s>>>(dtext, bytes, ctx->block_counts.as<uint32_t>());
  ++ctx->launches;
  k_scan_counts<<<1, 1024, 0, s>>>(ctx->block_counts.as<uint32_t>(), btiles, ctx->nhits.as<uint32_t>());
  ++ctx->launches;
  uint32_t n_nl = 0;
  CU(cudaMemcpyAsync(&n_nl, ctx->nhits.p, 4, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  const uint64_t lines64 = (uint64_t)n_nl + (text[bytes - 1] != '\n' ? 1 : 0);
  if (lines64 >= 0xfffff000ull) return fail(ctx, ISH_EINVAL, "too many lines (%llu)", (unsigned long long)lines64);
  const uint32_t n = (uint32_t)lines64;
  const uint32_t ltiles = ceil_div(n, FX_TILE);
  CU(ctx->nl_pos.ensure((size_t)n_nl * 8 + 8));
  CU(fx.hc.ensure((size_t)n * 8 + 8));
  CU(fx.len.ensure((size_t)n * 8 + 8));
  CU(fx.src.ensure((size_t)n * 8 + 8));
  CU(fx.hdr.ensure((size_t)n * 8 + 8));
  CU(fx.pos.ensure((size_t)n * 8 + 8));
  CU(fx.rec.ensure((size_t)n * 8 + 8));
  CU(fx.role.ensure((size_t)n + 16));
  CU(fx.tiles.ensure((size_t)ltiles * 5 + 16));
  CU(fx.scan.ensure(scan_u64_scratch(n)));
  CU(fx.totals.ensure(64));
  k_write_newlines<<<btiles, 1024, 0, s>>>(dtext, bytes, ctx->block_counts.as<uint32_t>(), ctx->nl_pos.as<uint64_t>());
  ++ctx->launches;
  CU(cudaMemsetAsync(fx.hc.p, 0xff, (size_t)n * 8, s));
  k_fx_header_chars<<<btiles, 1024, 0, s>>>(dtext, bytes, ctx->block_counts.as<uint32_t>(),
                                            fx.hc.as<unsigned long long>());
  ++ctx->launches;
  // ---- the reader's state at every line ----
  const uint64_t *nl = ctx->nl_pos.as<uint64_t>();
  const unsigned long long *hc = fx.hc.as<unsigned long long>();
  uint32_t *tile_map = fx.tiles.as<uint32_t>();
  uint8_t *tile_state = reinterpret_cast<uint8_t *>(tile_map + ltiles);
  k_fx_tile_maps<<<ltiles, 1024, 0, s>>>(dtext, bytes, nl, n_nl, n, hc, tile_map);
  ++ctx->launches;
  k_fx_tile_states<<<1, 1024, 0, s>>>(tile_map, ltiles, tile_state);
  ++ctx->launches;
  k_fx_roles<<<ltiles, 1024, 0, s>>>(dtext, bytes, nl, n_nl, n, hc, tile_state, fx.role.as<uint8_t>(),
                                     fx.len.as<uint64_t>(), fx.src.as<uint64_t>(), fx.hdr.as<uint64_t>());
  ++ctx->launches;
  CU(cudaGetLastError());
  // ---- record numbering and sequence offsets ----
  int rc = scan_u64(ctx, fx.len.as<uint64_t>(), fx.pos.as<uint64_t>(), n, fx.scan);
  if (!rc) rc = scan_u64(ctx, fx.hdr.as<uint64_t>(), fx.rec.as<uint64_t>(), n, fx.scan);
  if (rc) return rc;
  // every line could be a header: size the record arrays for n + 1
  CU(fx.rec_off.ensure((size_t)(n + 2) * 8));
  CU(fx.bounds.ensure((size_t)(n + 1) * 32));
  CU(fx.flags.ensure((size_t)(n + 1) * 4));
  k_fx_totals<<<1, 1, 0, s>>>(n, fx.len.as<uint64_t>(), fx.pos.as<uint64_t>(), fx.hdr.as<uint64_t>(),
                              fx.rec.as<uint64_t>(), fx.rec_off.as<uint64_t>(), fx.totals.as<uint64_t>());
  ++ctx->launches;
  CU(cudaMemsetAsync(fx.flags.p, 0, (size_t)(n + 1) * 4, s));
  CU(cudaMemsetAsync(fx.bounds.p, 0, (size_t)(n + 1) * 32, s));
  CU(cudaMemsetAsync(fx.totals.as<uint64_t>() + 2, 0xff, 8, s));
  const uint32_t gb = std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(n, 256), (uint32_t)ctx->num_sms * 16));
  k_fx_records<<<gb, 256, 0, s>>>(dtext, bytes, nl, n_nl, n, fx.role.as<uint8_t>(), fx.rec.as<uint64_t>(),
                                  fx.pos.as<uint64_t>(), fx.rec_off.as<uint64_t>(), fx.bounds.as<uint64_t>(),
                                  fx.flags.as<uint32_t>(), fx.src.as<uint64_t>());
  ++ctx->launches;
  uint64_t tot[3] = {0, 0, 0};
  CU(cudaMemcpyAsync(tot, fx.totals.p, 16, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  const uint64_t nrec = tot[0], seq_bytes = tot[1];
  if (nrec > 0) {
    k_fx_check<<<std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(nrec, 256), (uint32_t)ctx->num_sms * 16)), 256, 0,
                 s>>>((uint32_t)nrec, fx.rec_off.as<uint64_t>(), fx.bounds.as<uint64_t>(), fx.flags.as<uint32_t>(),
                      reinterpret_cast<unsigned long long *>(fx.totals.as<uint64_t>() + 2));
    ++ctx->launches;
  }
  CU(cudaMemcpyAsync(&tot[2], fx.totals.as<uint64_t>() + 2, 8, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  uint64_t keep = nrec;
  if (tot[2] != ~0ull) {
    const uint64_t r = tot[2] >> 1;
    if (tot[2] & 1)
      return fail(ctx, ISH_EINVAL,
                  "FASTQ record %llu: its quality continues on the next line (one quality line per record is "
                  "split on the device)",
                  (unsigned long long)r);
    keep = std::min(keep, r);
  }
  if (keep > 0xffffffffull) return fail(ctx, ISH_EINVAL, "too many records (%llu)", (unsigned long long)keep);
  const uint32_t nr = (uint32_t)keep;
  if (bounds_out) {
    if (nr > bounds_cap) return fail(ctx, ISH_EOVERFLOW, "%u records, bounds capacity %llu", nr,
                                     (unsigned long long)bounds_cap);
    if (nr) CU(cudaMemcpyAsync(bounds_out, fx.bounds.p, (size_t)nr * 32, cudaMemcpyDeviceToHost, s));
  }
  // ---- the kept records' sequences, contiguous, then the common packing ----
  uint64_t used = 0;
  if (nr) CU(cudaMemcpyAsync(&used, fx.rec_off.as<uint64_t>() + nr, 8, cudaMemcpyDeviceToHost, s));
  CU(fx.seq.ensure(seq_bytes + 32));
  const uint32_t gw = std::max<uint32_t>(1, std::min<uint32_t>(ceil_div((uint64_t)n * 32, 256), (uint32_t)ctx->num_sms * 32));
  k_fx_gather<<<gw, 256, 0, s>>>(dtext, n, fx.role.as<uint8_t>(), fx.len.as<uint64_t>(), fx.src.as<uint64_t>(),
                                 fx.pos.as<uint64_t>(), fx.seq.as<uint8_t>());
  ++ctx->launches;
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(s));
  CU(ctx->off_in.ensure((size_t)(nr + 1) * 8));
  if (nr) {
    CU(cudaMemcpyAsync(ctx->raw.p, fx.seq.p, used, cudaMemcpyDeviceToDevice, s));
    CU(cudaMemcpyAsync(ctx->off_in.p, fx.rec_off.p, (size_t)nr * 8, cudaMemcpyDeviceToDevice, s));
  }
  rs.total = used;
  *n_out = nr;
  if (nr == 0) return ISH_OK;
  return pack_set(ctx, nr, used, fx.rec_off.as<uint64_t>() + 1, enc, rs);
}

}  // namespace host
}  // namespace ish

using namespace ish;
using namespace ish::host;

int ish_gpu_records_load_fastx(ish_ctx *ctx, const uint8_t *text, uint64_t bytes, int matrix_kind, int32_t *set_id,
                               uint32_t *n_records, uint64_t *bounds, uint64_t bounds_cap) {
  if (!ctx) return ISH_EINVAL;
  if (!set_id) return fail(ctx, ISH_EINVAL, "set_id is NULL");
  if (int rc0 = finish_pending_load(ctx)) return rc0;
  LoadTimer timer(ctx);
  cudaSetDevice(ctx->device);
  const uint8_t *enc = nullptr;
  int rc = device_encoding(ctx, matrix_kind, &enc);
  if (rc) return rc;
  RecordSet rs;
  uint32_t n = 0;
  rc = load_fastx(ctx, text, bytes, rs, enc, &n, bounds, bounds_cap);
  if (rc) {
    cudaStreamSynchronize(ctx->stream);
    release_set(rs);
    return rc;
  }
  const int32_t id = ctx->next_set++;
  ctx->sets.emplace(id, std::move(rs));
  *set_id = id;
  if (n_records) *n_records = n;
  return ISH_OK;
}
