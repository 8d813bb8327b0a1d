// wave.cuh -- the wavefront scoring kernel.
//
// A group of G threads (G = 1, 2, ..., 32; a sub-warp) scores a PAIR of
// records at once: the low and high 16-bit halves of every register belong to
// record A and record B of the pair.  Thread t of the group owns K consecutive
// query columns [t*K - d, (t+1)*K - d); the query is padded at the front with
// d >= 1 columns whose profile and boundary values make them transparent (see
// build_wave_layout in ish_gpu.cu), so the last query column is always the
// last register of thread G-1.  Rows flow through the group as a software
// pipeline: thread t processes row i of the pair one step after thread t-1
// did, receiving H(i, first column - 1) and F(i, first column) through
// __shfl_up_sync.  G = 1 is "one thread per record pair with packed 16-bit
// lanes" for short queries; G = 32 is a warp-wide anti-diagonal wavefront for
// long queries.
//
// Per cell and record pair (two cells) the recurrence costs five DPX
// instructions (four for semi-global, below), in two in-place passes over the
// thread's columns:
//   backward:  T = max(Hdiag + P, E);  u = T - open;  E = max(E - ext, u);  H := T
//   forward:   H = max(Fs - open, T);  Fs = max(Fs - ext, T)
// with Fs = F + open carried along the row (local alignment floors u at 0,
// which keeps E, T and H non-negative).  E opens from T only, never from F: an
// F-then-E gap pair always has an E-then-F twin of at least the same score,
// which this recurrence keeps, so H is exactly the Gotoh H.  The serial
// dependency along a row is the single Fs instruction per cell, and both passes
// update H and E in place (no register rotation between rows).
//
// Semi-global alignment needs only four: row r is held raised by a frame
// f(r) = (r mod R) * ext, and the profile carries +ext, so H(r-1) + P lands in
// f(r) and the E update E' = max(E - ext, T - open) becomes
// E'(framed) = max(T(framed) + ext - open, E(framed)), one add-max.  Every R
// rows (R * ext <= 2048, headroom the fast regime keeps above the largest
// score) the carried row drops back to frame 0; scores leave the kernel with
// their frame taken off.  Local alignment keeps five: its floor at 0 would
// move with the frame.
//
// End coordinates follow the reference exactly:
//   semi-global, target end free: first row where H(i, Q-1) strictly beats the
//     running maximum (ishlib/matcher/alignment/semi_global_aln/striped.mojo:436-450);
//   semi-global, query end free: smallest query column of the maximum of the
//     last row, with the tie rule of striped.mojo:453-468;
//   local: first row whose column maximum strictly beats every earlier cell,
//     smallest query column of that maximum in that row
//     (ishlib/matcher/alignment/local_aln/striped.mojo:395-428).
#pragma once

#include "kernels.cuh"

namespace ish {

// Scores sorted entries [p.first, p.first + p.count) of the record set: the
// groups of the calling block take record pairs from *counter until none are
// left.  `prof` is the profile in shared memory; `slots_all` holds 32 words per
// group (pair indices in flight), `save_all` wave_save_words(K) words per thread (local
// alignment only).
template <int K, int MODE, int LAYOUT>
__device__ __forceinline__ void wave_rows(const WaveParams &p, const unsigned char *prof, uint32_t *slots_all,
                                          uint32_t *save_all, uint32_t *counter) {
  constexpr int RPS = (MODE == SG) ? WAVE_RPS_SG : WAVE_RPS_SW;
  static_assert(RPS == 2 || RPS == 4, "rows per step: 2 or 4");
  const int tid = threadIdx.x;
  const int G = p.G;
  const int lane = tid & 31;
  const int t = lane & (G - 1);
  const bool t0 = t == 0;
  uint32_t *slots = slots_all + (tid / G) * 32;
  // local alignment: per thread, the H row of the last improvement of each lane
  constexpr int KP8 = (K + 7) & ~7;
  uint16_t *saveA = reinterpret_cast<uint16_t *>(save_all + tid * wave_save_words(K));
  uint16_t *saveB = saveA + KP8;

  const unsigned FULL = 0xffffffffu;
  const uint32_t NOPEN = p.pk_nopen;
  const uint32_t NEXT = p.pk_next;
  const uint32_t VFLOOR = (MODE == SW) ? 0u : 0x80008000u;
  const uint32_t FS_IN = p.pk_fsin;  // F + open entering the padding
  // semi-global row frames: row r is held raised by frame = (r mod R) * ext
  const uint32_t EOPEN = p.pk_eopen;  // E' = max(T + ext - open, E)
  const uint32_t NEGMIN = 0x80008000u;
  const int f0 = (MODE == SG) ? p.ext : 0;  // row -1 sits in frame -ext
  const bool te = (MODE == SG) && (p.ends & 8);
  const bool qe = (MODE == SG) && (p.ends & 2);
  // record pairs of the range: every pair_stride-th from pair_phase
  const uint32_t pstride = p.pair_stride ? p.pair_stride : 1u, pphase = p.pair_stride ? p.pair_phase : 0u;
  const uint32_t npairs_all = (p.count + 1) >> 1;
  const uint32_t npairs = npairs_all > pphase ? (npairs_all - pphase + pstride - 1) / pstride : 0u;
  const int col0 = t * K - p.d;  // query column of register 0
  // parameters read every step, held in registers (the batched kernel's
  // parameters live in shared memory)
  const int kp = p.kp, alpha = p.alphabet, fmask = p.frame_mask, ext = p.ext, hleft = p.hleft;
  const uint32_t remap_off = p.remap_off, lane_mul = p.lane_mul;
  // the frame of a row (always 0 for local alignment)
  auto frame_of = [&](int r) { return (MODE == SG) ? (r & fmask) * ext : 0; };
  // +ext in both 16-bit halves: added to a boundary value hleft + frame
  // (hleft 0 or NEG_BIG, frames <= 2048), the low half never carries
  const uint32_t EXT2 = (MODE == SG) ? p.pk_ext : 0u;
  // this thread's part of every profile row, and the bytes between the rows
  // of consecutive codes: a row's address is one multiply-add
  const unsigned char *prof_t = prof + (uint32_t)(t * kp) * (LAYOUT == PROF_S16 ? 2u : 4u);
  const uint32_t row_bytes = p.row_bytes;

  uint32_t H[K], E[K];
#pragma unroll
  for (int j = 0; j < K; ++j) {
    H[j] = 0;
    E[j] = 0;
  }
  uint32_t prevH = 0;  // H(row above the step's first row, column col0 - 1)
  // per row of the step, passed to thread t+1: H of the last column, F + open
  // leaving it, and (local alignment) the running best of this thread's and
  // all earlier columns
  uint32_t outH[RPS], outF[RPS], outB[RPS];
#pragma unroll
  for (int k = 0; k < RPS; ++k) outH[k] = outF[k] = outB[k] = 0;
  uint32_t outC = CTL_IDLE;
  int q4 = 0, lenA = 0, lenB = 0, lastA_row = -1, lastB_row = -1;  // q4: row of the step's first row
  uint32_t pr = 0;
  // this thread's record streams: 4 codes per 32-bit word, one word ahead
  const uint8_t *pa = nullptr, *pb = nullptr;
  uint32_t wA = 0, wB = 0, nA = 0, nB = 0;
  // tracking
  uint32_t best = 0;         // SG: lane-wise running max of H(i, Q-1); SW: of this thread's cells
  int rowA = -1, rowB = -1;  // first row of the lane's maximum
  uint32_t oR0 = 0, oR1 = 0, oR2 = 0, oR3 = 0;  // last-row partials for thread t+1
  uint32_t iR0 = 0, iR1 = 0, iR2 = 0, iR3 = 0;  // ... and those of thread t-1
  bool has_out = false;
  // thread 0 of the group grabs record pairs: f_left steps of the current pair
  // are still to start, f_ctl is the control word of the next step
  bool f_done = false;
  int f_left = 0;
  uint32_t f_ctl = CTL_IDLE;
  uint32_t f_seq = 31;
  // the next row at which one of this thread's records ends (-3: none)
  int ev_row = -3;
  const bool remap = remap_off != 0;
  uint64_t steps = 0;
  constexpr int CHK = 8 / RPS;  // steps between termination checks
  int chk = CHK;

  // One row of the pair with record codes cA, cB: `diag` is H of the row above
  // at column col0 - 1, `fs` is F + open entering column col0.  Updates H and
  // E in place and returns F + open leaving the thread's last column.
  auto row_step = [&](uint32_t cA, uint32_t cB, uint32_t diag, uint32_t fs) -> uint32_t {
    if (remap) {  // codes that score alike share a profile row
      cA = prof[remap_off + cA];
      cB = prof[remap_off + cB];
    }
    uint32_t P[K];
    if (LAYOUT == PROF_PAIR) {
      const uint4 *r4 = reinterpret_cast<const uint4 *>(prof_t + (cA * alpha + cB) * row_bytes);
#pragma unroll
      for (int v = 0; v < (K + 3) / 4; ++v) {
        const uint4 w = r4[v];
        if (4 * v + 0 < K) P[4 * v + 0] = w.x;
        if (4 * v + 1 < K) P[4 * v + 1] = w.y;
        if (4 * v + 2 < K) P[4 * v + 2] = w.z;
        if (4 * v + 3 < K) P[4 * v + 3] = w.w;
      }
    } else if (LAYOUT == PROF_S32) {
      // 32-bit words holding the 16-bit score in the low half; the packed
      // pair is b * 65536 + a, one integer multiply-add (the multiplier is a
      // runtime value, so this stays an IMAD on the FMA pipe, which the DPX
      // recurrence on the ALU pipe leaves idle)
      const uint4 *ra = reinterpret_cast<const uint4 *>(prof_t + cA * row_bytes);
      const uint4 *rb = reinterpret_cast<const uint4 *>(prof_t + cB * row_bytes);
      const uint32_t mul = lane_mul;
#pragma unroll
      for (int v = 0; v < (K + 3) / 4; ++v) {
        const uint4 a = ra[v], b = rb[v];
        if (4 * v + 0 < K) P[4 * v + 0] = b.x * mul + a.x;
        if (4 * v + 1 < K) P[4 * v + 1] = b.y * mul + a.y;
        if (4 * v + 2 < K) P[4 * v + 2] = b.z * mul + a.z;
        if (4 * v + 3 < K) P[4 * v + 3] = b.w * mul + a.w;
      }
    } else {
      // 16-bit words (profiles too large for the 32-bit layout): one PRMT
      // per packed pair
      const uint4 *ra = reinterpret_cast<const uint4 *>(prof_t + cA * row_bytes);
      const uint4 *rb = reinterpret_cast<const uint4 *>(prof_t + cB * row_bytes);
#pragma unroll
      for (int v = 0; v < (K + 7) / 8; ++v) {
        const uint4 a = ra[v], b = rb[v];
        const uint32_t aw[4] = {a.x, a.y, a.z, a.w}, bw[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          if (8 * v + 2 * m < K) P[8 * v + 2 * m] = __byte_perm(aw[m], bw[m], 0x5410);
          if (8 * v + 2 * m + 1 < K) P[8 * v + 2 * m + 1] = __byte_perm(aw[m], bw[m], 0x7632);
        }
      }
    }
    // backward pass (columns independent), then the F chain
#pragma unroll
    for (int j = K - 1; j >= 0; --j) {
      const uint32_t T = __viaddmax_s16x2(j == 0 ? diag : H[j - 1], P[j], E[j]);
      if (MODE == SG) {
        E[j] = __viaddmax_s16x2(T, EOPEN, E[j]);  // in the row frames (see the header)
      } else {
        const uint32_t u = __viaddmax_s16x2(T, NOPEN, VFLOOR);
        E[j] = __viaddmax_s16x2(E[j], NEXT, u);
      }
      H[j] = T;
    }
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const uint32_t T = H[j];
      H[j] = __viaddmax_s16x2(fs, NOPEN, T);
      fs = __viaddmax_s16x2(fs, NEXT, T);
    }
    return fs;
  };

  // Local alignment, after row `row`: only a row maximum above every cell so
  // far in this thread AND in all columns to its left (`left`, their running
  // best up to this row, passed along the pipeline) can be the first row of
  // the record's maximum at its smallest column; anything else is dominated
  // (smaller, or equal in an earlier row or a smaller column), so only those
  // improvements are recorded.  Returns the running best passed on.
  auto sw_track = [&](int row, uint32_t left) -> uint32_t {
    uint32_t cm = H[0];
#pragma unroll
    for (int j = 1; j + 1 < K; j += 2) cm = __vimax3_s16x2(cm, H[j], H[j + 1]);
    if ((K & 1) == 0 && K > 1) cm = __viaddmax_s16x2(cm, 0u, H[K - 1]);
    const uint32_t thr = __viaddmax_s16x2(best, 0u, left);
    const uint32_t nb = __viaddmax_s16x2(thr, 0u, cm);
    if (nb != thr) {
      // keep this row (shared-memory stores only); the column of the maximum
      // is looked up once, at the record's last row
      const bool upA = lo16(cm) > lo16(thr), upB = hi16(cm) > hi16(thr);
      // the improving lane's halves of the row: one PRMT per two columns
#define ISH_H(j) ((j) < K ? H[(j) < K ? (j) : 0] : 0u)
      if (upA) {
#pragma unroll
        for (int v = 0; v < KP8 / 8; ++v)
          reinterpret_cast<uint4 *>(saveA)[v] =
              make_uint4(__byte_perm(ISH_H(8 * v), ISH_H(8 * v + 1), 0x5410),
                         __byte_perm(ISH_H(8 * v + 2), ISH_H(8 * v + 3), 0x5410),
                         __byte_perm(ISH_H(8 * v + 4), ISH_H(8 * v + 5), 0x5410),
                         __byte_perm(ISH_H(8 * v + 6), ISH_H(8 * v + 7), 0x5410));
      }
      if (upB) {
#pragma unroll
        for (int v = 0; v < KP8 / 8; ++v)
          reinterpret_cast<uint4 *>(saveB)[v] =
              make_uint4(__byte_perm(ISH_H(8 * v), ISH_H(8 * v + 1), 0x7632),
                         __byte_perm(ISH_H(8 * v + 2), ISH_H(8 * v + 3), 0x7632),
                         __byte_perm(ISH_H(8 * v + 4), ISH_H(8 * v + 5), 0x7632),
                         __byte_perm(ISH_H(8 * v + 6), ISH_H(8 * v + 7), 0x7632));
      }
#undef ISH_H
      if (upA) rowA = row;
      if (upB) rowB = row;
      best = ((upA ? cm : best) & 0xffffu) | ((upB ? cm : best) & 0xffff0000u);
    }
    return nb;
  };

  // Semi-global, target end free, one row: the running max of column Q-1
  // (register K-1 of thread G-1); a strict improvement records the row, so
  // the FIRST row of the maximum wins.
  auto te_row = [&](int row) {
    const uint32_t nb = __viaddmax_s16x2(best, 0u, __viaddmax_s16x2(H[K - 1], dup16(-frame_of(row)), NEGMIN));
    if (nb != best) {
      if (lo16(nb) != lo16(best)) rowA = row;
      if (hi16(nb) != hi16(best)) rowB = row;
      best = nb;
    }
  };

  // o takes v's 16-bit half of each lane whose record ends now
  auto put_lanes = [](uint32_t &o, uint32_t v, bool a, bool b) {
    o = (a ? (v & 0xffffu) : (o & 0xffffu)) | (b ? (v & 0xffff0000u) : (o & 0xffff0000u));
  };

  // The last row of one or both records of the pair (H holds it): fold the
  // partial results left to right -- thread t-1's arrived as iR at the start
  // of this step, this thread's leave as oR at the next -- and thread G-1
  // writes the record's outputs.
  auto on_event = [&](int row) {
    const bool lastA = row == lastA_row, lastB = row == lastB_row;
    {  // the other record's end, if it is still ahead
      int nxt = lastA_row > row ? lastA_row : -3;
      if (lastB_row > row && (nxt < 0 || lastB_row < nxt)) nxt = lastB_row;
      ev_row = nxt;
    }
    if (MODE == SG) {
      uint32_t mx = 0, mq = 0;
      if (qe) {
        int bA = -32768, bB = -32768, qA = 0x7fff, qB = 0x7fff;
        uint32_t row_h[K];  // staged as in the local-alignment scan
#pragma unroll
        for (int j = 0; j < K; ++j) row_h[j] = H[j];
#pragma unroll 1
        for (int j = 0; j < K; ++j) {
          if (col0 + j >= 0) {
            const int a = lo16(row_h[j]), b = hi16(row_h[j]);
            if (a > bA) {
              bA = a;
              qA = col0 + j;
            }
            if (b > bB) {
              bB = b;
              qB = col0 + j;
            }
          }
        }
        if (t > 0) {  // columns to the left win ties
          if (!(bA > lo16(iR0))) {
            bA = lo16(iR0);
            qA = (int)(iR1 & 0xffffu);
          }
          if (!(bB > hi16(iR0))) {
            bB = hi16(iR0);
            qB = (int)(iR1 >> 16);
          }
        }
        mx = (uint32_t)(bA & 0xffff) | ((uint32_t)bB << 16);
        mq = (uint32_t)qA | ((uint32_t)qB << 16);
        if (t < G - 1) {
          put_lanes(oR0, mx, lastA, lastB);
          put_lanes(oR1, mq, lastA, lastB);
          has_out = true;
        }
      }
      if (t == G - 1) {
#pragma unroll
        for (int x = 0; x < 2; ++x) {
          if (!(x == 0 ? lastA : lastB)) continue;
          const uint32_t orig = p.rec.orig[p.first + 2 * pr + x];
          const int T = x == 0 ? lenA : lenB;
          int score, er, eq = p.Q - 1;
          if (!te && !qe) {
            score = (x == 0 ? lo16(H[K - 1]) : hi16(H[K - 1])) - frame_of(row);  // this row's H(i, Q-1)
            er = T - 1;
          } else {
            score = te ? (x == 0 ? lo16(best) : hi16(best)) : p.neg_limit;
            er = x == 0 ? rowA : rowB;
            if (qe) {
              const int s1 = (x == 0 ? lo16(mx) : hi16(mx)) - frame_of(row);
              const int t1 = x == 0 ? (int)(mq & 0xffffu) : (int)(mq >> 16);
              if (s1 > score) {
                score = s1;
                er = T - 1;
                eq = t1;
              } else if (s1 == score && er == T - 1 && t1 < eq) {
                eq = t1;
              }
            }
          }
          if (p.out.score) p.out.score[orig] = score;
          if (p.out.qend) p.out.qend[orig] = eq;
          if (p.out.tend) p.out.tend[orig] = er;
          if (p.out.hit) p.out.hit[orig] = decide(SG, score, eq, er, p.dec);
        }
      }
    } else {
      int bA = lo16(best), bB = hi16(best), rA = rowA, rB = rowB, qA = 0x7fff, qB = 0x7fff;
      // smallest column of this thread's maximum in its first row
#pragma unroll 1
      for (int j = K - 1; j >= 0; --j) {
        if (bA > 0 && (int)(int16_t)saveA[j] == bA) qA = col0 + j;
        if (bB > 0 && (int)(int16_t)saveB[j] == bB) qB = col0 + j;
      }
      if (t > 0) {
        const int ia = lo16(iR0), ib = hi16(iR0), ira = (int)iR2, irb = (int)iR3;
        const int iqa = (int)(int16_t)(iR1 & 0xffffu), iqb = (int)(int16_t)(iR1 >> 16);
        if (ia > bA || (ia == bA && (ira < rA || (ira == rA && iqa < qA)))) {
          bA = ia;
          rA = ira;
          qA = iqa;
        }
        if (ib > bB || (ib == bB && (irb < rB || (irb == rB && iqb < qB)))) {
          bB = ib;
          rB = irb;
          qB = iqb;
        }
      }
      if (t < G - 1) {
        put_lanes(oR0, (uint32_t)(bA & 0xffff) | ((uint32_t)bB << 16), lastA, lastB);
        put_lanes(oR1, (uint32_t)(qA & 0xffff) | ((uint32_t)qB << 16), lastA, lastB);
        if (lastA) oR2 = (uint32_t)rA;
        if (lastB) oR3 = (uint32_t)rB;
        has_out = true;
      } else {
#pragma unroll
        for (int x = 0; x < 2; ++x) {
          if (!(x == 0 ? lastA : lastB)) continue;
          const uint32_t orig = p.rec.orig[p.first + 2 * pr + x];
          int score = x == 0 ? bA : bB, er = x == 0 ? rA : rB, eq = x == 0 ? qA : qB;
          if (score == 0) {
            er = -1;
            eq = 0;
          }
          if (p.out.score) p.out.score[orig] = score;
          if (p.out.qend) p.out.qend[orig] = eq;
          if (p.out.tend) p.out.tend[orig] = er;
          if (p.out.hit) p.out.hit[orig] = decide(SW, score, eq, er, p.dec);
        }
      }
    }
  };

  while (true) {
    __syncwarp();
    uint32_t msgH[RPS], msgF[RPS], msgB[RPS];
#pragma unroll
    for (int k = 0; k < RPS; ++k) {
      msgH[k] = __shfl_up_sync(FULL, outH[k], 1, G);
      msgF[k] = __shfl_up_sync(FULL, outF[k], 1, G);
      msgB[k] = (MODE == SW) ? __shfl_up_sync(FULL, outB[k], 1, G) : 0u;
    }
    uint32_t msgC = __shfl_up_sync(FULL, outC, 1, G);
    // partial results of records that ended in thread t-1's previous step
    if (__any_sync(FULL, has_out)) {
      iR0 = __shfl_up_sync(FULL, oR0, 1, G);
      iR1 = __shfl_up_sync(FULL, oR1, 1, G);
      if (MODE == SW) {
        iR2 = __shfl_up_sync(FULL, oR2, 1, G);
        iR3 = __shfl_up_sync(FULL, oR3, 1, G);
      }
      has_out = false;
    }

    if (t0) {
      if (f_left <= 0 && !f_done) {
        const uint32_t nt = atomicAdd(counter, 1u);
        if (nt < npairs) {
          const uint32_t np = nt * pstride + pphase;  // the pair's index in the range
          f_seq = (f_seq + 1) & 31;
          slots[f_seq] = np;
          const uint32_t sA = p.first + 2 * np;
          const int na = (int)p.rec.len[sA];
          const int nb = (2 * np + 1 < p.count) ? (int)p.rec.len[sA + 1] : 0;
          f_left = (max(max(na, nb), 1) + RPS - 1) / RPS;
          f_ctl = CTL_NEW | (f_seq << CTL_SEQ_SHIFT);
        } else {
          f_done = true;
        }
      }
      msgC = f_ctl;
      f_ctl &= ~CTL_NEW;
      if (--f_left <= 0) f_ctl = CTL_IDLE;
    }

    const bool busy = !(msgC & CTL_IDLE);
    if (busy) {
      if (msgC & CTL_NEW) {
        pr = slots[(msgC >> CTL_SEQ_SHIFT) & 31];
        const uint32_t sA = p.first + 2 * pr;
        lenA = (int)p.rec.len[sA];
        pa = p.rec.codes + p.rec.off[sA];
        if (2 * pr + 1 < p.count) {
          lenB = (int)p.rec.len[sA + 1];
          pb = p.rec.codes + p.rec.off[sA + 1];
        } else {
          lenB = 0;
          pb = pa;
        }
        lastA_row = lenA - 1;
        lastB_row = lenB > 0 ? lenB - 1 : -2;
        // the earlier of the two records' last rows (either may be empty)
        ev_row = lastA_row >= 0 ? lastA_row : -3;
        if (lastB_row >= 0 && (ev_row < 0 || lastB_row < ev_row)) ev_row = lastB_row;
        nA = __ldg(reinterpret_cast<const uint32_t *>(pa));
        nB = lenB ? __ldg(reinterpret_cast<const uint32_t *>(pb)) : 0u;
        const int16_t *hi = p.hinit + t * K;
#pragma unroll
        for (int j = 0; j < K; ++j) {
          const int h0 = hi[j];
          H[j] = dup16(h0 - f0);
          E[j] = (MODE == SW) ? 0u : dup16(h0 - p.open);
        }
        prevH = t0 ? dup16(p.hleft - f0) : dup16(p.hinit[t * K - 1] - f0);
        best = (MODE == SW) ? 0u : dup16(p.neg_limit);
        rowA = rowB = -1;
        q4 = 0;
      } else {
        q4 += RPS;
        if (MODE == SG) {
          if ((q4 & fmask) == 0) {
            // frame R*ext -> 0: lower what this step takes from the row above
            const uint32_t FRAME_DROP = p.pk_drop;
#pragma unroll
            for (int j = 0; j < K; ++j) {
              H[j] = __viaddmax_s16x2(H[j], FRAME_DROP, NEGMIN);
              E[j] = __viaddmax_s16x2(E[j], FRAME_DROP, NEGMIN);
            }
            prevH = __viaddmax_s16x2(prevH, FRAME_DROP, NEGMIN);
          }
        }
      }
      // ---- record codes of this step ----
      // Codes were checked against the alphabet when the set was loaded and
      // every record slot is zero-padded to 16 bytes.  Past a record's end the
      // last word repeats: those rows only feed a lane whose result is final.
      if (RPS == 4 || (q4 & 3) == 0) {
        wA = nA;
        wB = nB;
        if (q4 + 4 < lenA) nA = __ldg(reinterpret_cast<const uint32_t *>(pa + q4 + 4));
        if (q4 + 4 < lenB) nB = __ldg(reinterpret_cast<const uint32_t *>(pb + q4 + 4));
        // long records: the codes 256 rows ahead are pulled into L1, so the
        // group's loads hit L1 even when few warps are left to hide latency
        if ((q4 & 127) == 0) {
          if (q4 + 256 < lenA) asm volatile("prefetch.global.L1 [%0];" ::"l"(pa + q4 + 256));
          if (q4 + 256 < lenB) asm volatile("prefetch.global.L1 [%0];" ::"l"(pb + q4 + 256));
        }
      } else {
        wA >>= 16;
        wB >>= 16;
      }
      // thread 0: what enters the padding from the left, H = hleft in the
      // row's frame and F = -infinity (semi-global) / 0 (local)
      if (t0) {
        const uint32_t hf = dup16(hleft + frame_of(q4));
#pragma unroll
        for (int k = 0; k < RPS; ++k) {
          msgH[k] = hf + (uint32_t)k * EXT2;
          msgF[k] = FS_IN;
          msgB[k] = 0u;
        }
      }
    }
    // whether a record of the warp ends in this step's rows (warp-uniform)
    const bool slow = __any_sync(FULL, busy && (unsigned)(ev_row - q4) < (unsigned)RPS);

    if (busy) {
      if (!slow) {
        // ---- the step's rows, no record ending ----
#pragma unroll
        for (int k = 0; k < RPS; ++k) {
          const uint32_t fs = row_step(__byte_perm(wA, 0u, 0x4440 + k), __byte_perm(wB, 0u, 0x4440 + k),
                                       k == 0 ? prevH : msgH[k - 1], msgF[k]);
          outH[k] = H[K - 1];
          outF[k] = fs;
          if (MODE == SW) outB[k] = sw_track(q4 + k, msgB[k]);
        }
        prevH = msgH[RPS - 1];
        if (te) {
          // the largest H(., Q-1) of the step's rows without their frames
          // (frame(q4 + k) = frame(q4) + k * ext): m = max_k outH[k] - k * ext
          uint32_t m = outH[RPS - 1];
#pragma unroll
          for (int k = RPS - 2; k >= 0; --k) m = __viaddmax_s16x2(m, NEXT, outH[k]);
          const uint32_t nb = __viaddmax_s16x2(m, dup16(-frame_of(q4)), best);
          if (nb != best) {
            // the first row reaching the new maximum, per improved lane
            bool dA = lo16(nb) == lo16(best), dB = hi16(nb) == hi16(best);
#pragma unroll
            for (int k = 0; k < RPS; ++k) {
              const uint32_t u = __viaddmax_s16x2(outH[k], dup16(-frame_of(q4 + k)), NEGMIN);
              if (!dA && lo16(u) == lo16(nb)) {
                rowA = q4 + k;
                dA = true;
              }
              if (!dB && hi16(u) == hi16(nb)) {
                rowB = q4 + k;
                dB = true;
              }
            }
            best = nb;
          }
        }
      } else {
        // ---- a record of the warp ends in these rows: one row at a time,
        // with the end-of-record work after its last row ----
        uint32_t d = prevH, sA = wA, sB = wB;
#pragma unroll 1
        for (int k = 0; k < RPS; ++k) {
          const int row = q4 + k;
          const uint32_t fs = row_step(sA & 0xffu, sB & 0xffu, d, msgF[0]);
          sA >>= 8;
          sB >>= 8;
          d = msgH[0];
          const uint32_t left = msgB[0];
#pragma unroll
          for (int j = 0; j + 1 < RPS; ++j) {
            msgH[j] = msgH[j + 1];
            msgF[j] = msgF[j + 1];
            msgB[j] = msgB[j + 1];
            outH[j] = outH[j + 1];
            outF[j] = outF[j + 1];
            outB[j] = outB[j + 1];
          }
          outH[RPS - 1] = H[K - 1];
          outF[RPS - 1] = fs;
          if (MODE == SW) outB[RPS - 1] = sw_track(row, left);
          if (te) te_row(row);
          if (row == ev_row) on_event(row);
        }
        prevH = d;
      }
      outC = msgC;
    } else {
      outC = CTL_IDLE;
    }

    // Every step thread 0 starts reaches thread G-1 within G-1 steps, so the
    // group is done once thread 0 is and no step is in flight.  The step budget
    // (all rows of the range plus the pipeline depth) is a hard stop.
    // (checked every CHK steps; idle extra steps do nothing)
    if (--chk == 0) {
      chk = CHK;
      steps += CHK * RPS;
      const bool more = busy || (t0 && !f_done);
      if (!__any_sync(FULL, more)) break;
      if (steps > p.max_steps) {
        if (lane == 0) atomicOr(p.error, 2);
        break;
      }
    }
  }
}

// Rows with the parameters read from a shared-memory copy, as the batched
// kernel does: kept in the parameter bank, the compiler holds them in
// registers across the row loop, which some shapes pay for in spills
// (WAVE_PARAMS_SMEM).  Only the kernels that call this declare the copy.
template <int K, int MODE, int LAYOUT>
__device__ __forceinline__ void wave_rows_smem_params(const WaveParams &p, const unsigned char *prof,
                                                      uint32_t *slots_all, uint32_t *save_all) {
  __shared__ WaveParams sp;
  if (threadIdx.x == 0) sp = p;
  __syncthreads();
  wave_rows<K, MODE, LAYOUT>(sp, prof, slots_all, save_all, p.counter);
}

// Shared memory of a block: the profile, then 32 slot words per group, then
// (local alignment) wave_save_words(K) save words per thread.
template <int K, int MODE, int LAYOUT, int LEAN = 0>
__global__ void __launch_bounds__(wave_threads_lean(K, MODE, LEAN), wave_blocks_lean(K, MODE, LEAN))
    wave_kernel(const __grid_constant__ WaveParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  {
    const uint4 *src = p.prof;
    uint4 *dst = reinterpret_cast<uint4 *>(smem_raw);
    const uint32_t nvec = p.prof_bytes >> 4;
    for (uint32_t i = threadIdx.x; i < nvec; i += blockDim.x) dst[i] = src[i];
  }
  uint32_t *slots_all = reinterpret_cast<uint32_t *>(smem_raw + ((p.prof_bytes + 15u) & ~15u));
  uint32_t *save_all = slots_all + (blockDim.x / p.G) * 32;
  if constexpr (WAVE_PARAMS_SMEM(K, MODE, LEAN)) {
    wave_rows_smem_params<K, MODE, LAYOUT>(p, smem_raw, slots_all, save_all);
  } else {
    __syncthreads();
    wave_rows<K, MODE, LAYOUT>(p, smem_raw, slots_all, save_all, p.counter);
  }
}

// The batched launch: one persistent kernel for every query of a shape class
// (same K, mode and profile layout; G may differ per query).  Each query's
// record pairs are handed out by its own counter in global memory, in
// descending length order, exactly as in wave_kernel.  A block walks the
// queries of the class starting at its own offset (so the blocks spread over
// the queries) and stays on a query until its counter runs dry; a barrier and
// a profile reload happen only at a query switch, where the pairs left are the
// shortest of the set.  Queries whose counter is already exhausted are skipped.
template <int K, int MODE, int LAYOUT, int LEAN = 0>
__global__ void __launch_bounds__(wave_threads_lean(K, MODE, LEAN), wave_blocks_lean(K, MODE, LEAN))
    batch_kernel(const __grid_constant__ BatchParams b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ WaveParams sp;
  __shared__ int s_skip;
  uint32_t *slots_all = reinterpret_cast<uint32_t *>(smem_raw + b.prof_area);
  uint32_t *save_all = slots_all + b.slot_words;
  const uint32_t start = (uint32_t)(((uint64_t)blockIdx.x * b.ntiles) / gridDim.x);
  for (uint32_t it = 0; it < b.ntiles; ++it) {
    uint32_t tile = start + it;
    if (tile >= b.ntiles) tile -= b.ntiles;
    const BatchTile tl = b.tiles[tile];
    const WaveParams *qp = b.queries + tl.q;
    uint32_t *counter = b.tile_counter + tile;
    if (threadIdx.x == 0) {
      const uint32_t taken = *reinterpret_cast<volatile uint32_t *>(counter);
      const uint32_t stride = tl.pairs >> 16, phase = tl.pairs & 0xffffu, all = (tl.count + 1) / 2;
      const uint32_t mine = stride ? (all > phase ? (all - phase + stride - 1) / stride : 0u) : all;
      s_skip = taken >= mine;
      if (!s_skip) {
        sp = *qp;
        sp.first = tl.first;
        sp.count = tl.count;
        sp.pair_stride = stride;
        sp.pair_phase = phase;
        // every group's steps are bounded by all pairs of the range at its
        // longest length (records are sorted, the first is longest)
        const uint64_t npairs = (tl.count + 1) / 2;
        sp.max_steps = b.step_cap ? b.step_cap : npairs * ((uint64_t)qp->rec.len[tl.first] + 2 * 32 + 8) + 1024;
      }
    }
    __syncthreads();
    if (s_skip) {
      __syncthreads();  // s_skip is rewritten next iteration
      continue;
    }
    {
      const uint4 *src = qp->prof;
      uint4 *dst = reinterpret_cast<uint4 *>(smem_raw);
      const uint32_t nvec = qp->prof_bytes >> 4;
      for (uint32_t i = threadIdx.x; i < nvec; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    wave_rows<K, MODE, LAYOUT>(sp, smem_raw, slots_all, save_all, counter);
    __syncthreads();
  }
}

}  // namespace ish

namespace ish {

// Kernel tables.  Each wave_X.cu instantiates the wavefront and batched
// kernels of one K range (one translation unit per range, so the build
// compiles them in parallel); wave_table / batch_table pick one at run time
// by (K, mode, profile layout).
template <int K, int LEAN>
struct WaveEntry {
  static WaveFn wave(int mode, int layout) {
    static const WaveFn t[2][3] = {
        {wave_kernel<K, SG, PROF_S16, LEAN>, wave_kernel<K, SG, PROF_PAIR, LEAN>, wave_kernel<K, SG, PROF_S32, LEAN>},
        {wave_kernel<K, SW, PROF_S16, LEAN>, wave_kernel<K, SW, PROF_PAIR, LEAN>, wave_kernel<K, SW, PROF_S32, LEAN>}};
    return t[mode == SW][layout];
  }
  static BatchFn batch(int mode, int layout) {
    static const BatchFn t[2][3] = {
        {batch_kernel<K, SG, PROF_S16, LEAN>, batch_kernel<K, SG, PROF_PAIR, LEAN>,
         batch_kernel<K, SG, PROF_S32, LEAN>},
        {batch_kernel<K, SW, PROF_S16, LEAN>, batch_kernel<K, SW, PROF_PAIR, LEAN>,
         batch_kernel<K, SW, PROF_S32, LEAN>}};
    return t[mode == SW][layout];
  }
};

template <int LEAN, int... Ks>
WaveFn wave_table(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  WaveFn f = nullptr;
  ((K == Ks ? (void)(f = WaveEntry<Ks, LEAN>::wave(mode, layout)) : (void)0), ...);
  return f;
}

template <int LEAN, int... Ks>
BatchFn batch_table(int K, int mode, int layout) {
  if (layout < PROF_S16 || layout > PROF_S32) return nullptr;
  BatchFn f = nullptr;
  ((K == Ks ? (void)(f = WaveEntry<Ks, LEAN>::batch(mode, layout)) : (void)0), ...);
  return f;
}

}  // namespace ish
