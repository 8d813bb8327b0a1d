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
  const int tid = threadIdx.x;
  const int G = p.G;
  const int lane = tid & 31;
  const int t = lane & (G - 1);
  uint32_t *slots = slots_all + (tid / G) * 32;
  // local alignment: per thread, the H row of the last improvement of each lane
  constexpr int KP8 = (K + 7) & ~7;
  uint16_t *saveA = reinterpret_cast<uint16_t *>(save_all + tid * wave_save_words(K));
  uint16_t *saveB = saveA + KP8;

  const unsigned FULL = 0xffffffffu;
  const uint32_t NOPEN = dup16(-p.open);
  const uint32_t NEXT = dup16(-p.ext);
  const uint32_t VFLOOR = (MODE == SW) ? 0u : dup16(-32768);
  const uint32_t FS_IN = dup16(p.fin + p.open);  // F + open entering the padding
  // semi-global row frames: row r is held raised by frame = (r mod R) * ext
  const uint32_t EOPEN = dup16(p.ext - p.open);                   // E' = max(T + ext - open, E)
  const uint32_t NEGMIN = dup16(-32768);
  const int f0 = (MODE == SG) ? p.ext : 0;  // row -1 sits in frame -ext
  const bool te = (MODE == SG) && (p.ends & 8);
  const bool qe = (MODE == SG) && (p.ends & 2);
  const uint32_t npairs = (p.count + 1) >> 1;
  const uint16_t *prof16 = reinterpret_cast<const uint16_t *>(prof);
  const uint32_t *prof32 = reinterpret_cast<const uint32_t *>(prof);
  const int col0 = t * K - p.d;  // query column of register 0
  // parameters read every row, held in registers (the batched kernel's
  // parameters live in shared memory)
  const int kp = p.kp, alpha = p.alphabet, fmask = p.frame_mask, ext = p.ext, hleft = p.hleft;
  const uint32_t remap_off = p.remap_off, lane_mul = p.lane_mul;
  // the frame of a row (always 0 for local alignment)
  auto frame_of = [&](int r) { return (MODE == SG) ? (r & fmask) * ext : 0; };

  uint32_t H[K], E[K];
#pragma unroll
  for (int j = 0; j < K; ++j) {
    H[j] = 0;
    E[j] = 0;
  }
  uint32_t prevH = 0, outH = 0, outF = 0, outC = CTL_IDLE;
  uint32_t outBest = 0;  // local alignment: best cell so far in this thread's and all earlier columns
  int row = 0, lenA = 0, lenB = 0, lastA_row = -1, lastB_row = -1;
  uint32_t pr = 0;
  // this thread's record streams: 4 codes per 32-bit word, one word ahead
  const uint8_t *pa = nullptr, *pb = nullptr;
  uint32_t wA = 0, wB = 0, nA = 0, nB = 0;
  // tracking
  uint32_t best = 0;         // SG: lane-wise running max of H(i, Q-1); SW: of this thread's cells
  int rowA = -1, rowB = -1;  // first row of the lane's maximum
  uint32_t oR0 = 0, oR1 = 0, oR2 = 0, oR3 = 0;  // last-row partials for thread t+1
  bool has_out = false;
  // thread 0 of the group grabs record pairs: f_left rows of the current pair
  // are still to start, f_ctl is the control word of the next row
  bool f_done = false;
  int f_left = 0;
  uint32_t f_ctl = CTL_IDLE;
  uint32_t f_seq = 31;
  // the next row at which one of this thread's records ends (-3: none)
  int ev_row = -3;
  const bool remap = remap_off != 0;
  uint64_t steps = 0;
  int chk = 8;

  while (true) {
    __syncwarp();
    const uint32_t msgH = __shfl_up_sync(FULL, outH, 1, G);
    const uint32_t msgF = __shfl_up_sync(FULL, outF, 1, G);
    uint32_t msgC = __shfl_up_sync(FULL, outC, 1, G);
    const uint32_t msgBest = (MODE == SW) ? __shfl_up_sync(FULL, outBest, 1, G) : 0u;

    if (t == 0) {
      if (f_left <= 0 && !f_done) {
        const uint32_t np = atomicAdd(counter, 1u);
        if (np < npairs) {
          f_seq = (f_seq + 1) & 31;
          slots[f_seq] = np;
          const uint32_t sA = p.first + 2 * np;
          const int na = (int)p.rec.len[sA];
          const int nb = (2 * np + 1 < p.count) ? (int)p.rec.len[sA + 1] : 0;
          f_left = max(max(na, nb), 1);
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
        prevH = (t == 0) ? dup16(p.hleft - f0) : dup16(p.hinit[t * K - 1] - f0);
        best = (MODE == SW) ? 0u : dup16(p.neg_limit);
        rowA = rowB = -1;
        row = 0;
      } else {
        ++row;
        if (MODE == SG) {
          if ((row & fmask) == 0) {
            // frame R*ext -> 0: lower what this row takes from the row above
            const uint32_t FRAME_DROP = dup16(-(p.frame_mask + 1) * p.ext);
#pragma unroll
            for (int j = 0; j < K; ++j) {
              H[j] = __viaddmax_s16x2(H[j], FRAME_DROP, NEGMIN);
              E[j] = __viaddmax_s16x2(E[j], FRAME_DROP, NEGMIN);
            }
            prevH = __viaddmax_s16x2(prevH, FRAME_DROP, NEGMIN);
          }
        }
      }

      // ---- record codes of this row ----
      // Codes were checked against the alphabet when the set was loaded and
      // every record slot is zero-padded to 16 bytes.  Past a record's end the
      // last word repeats: those rows only feed a lane whose result is final.
      uint32_t P[K];
      {
        // A new code word every 4 rows.  The threads of a group sit on
        // different rows, so a conditional block here diverges every row;
        // for the shapes where it measured faster the refill is written as
        // selects and guarded loads instead (semi-global K <= 24 and >= 34:
        // +1 to +3.4 %; local K <= 24 and >= 50), elsewhere the extra live
        // registers cost more than the branch saves.
        constexpr bool SELECT_REFILL = (MODE == SG) ? (K <= 24 || K >= 34) : (K <= 24 || K >= 50);
        // long records: the codes 256 rows ahead are pulled into L1, so the
        // group's loads hit L1 even when few warps are left to hide latency
        if constexpr (SELECT_REFILL) {
          const bool refill = (row & 3) == 0;
          wA = refill ? nA : wA;
          wB = refill ? nB : wB;
          if (refill && row + 4 < lenA) nA = __ldg(reinterpret_cast<const uint32_t *>(pa + row + 4));
          if (refill && row + 4 < lenB) nB = __ldg(reinterpret_cast<const uint32_t *>(pb + row + 4));
          const bool pf = (row & 127) == 0;
          if (pf && row + 256 < lenA) asm volatile("prefetch.global.L1 [%0];" ::"l"(pa + row + 256));
          if (pf && row + 256 < lenB) asm volatile("prefetch.global.L1 [%0];" ::"l"(pb + row + 256));
        } else if ((row & 3) == 0) {
          wA = nA;
          wB = nB;
          if (row + 4 < lenA) nA = __ldg(reinterpret_cast<const uint32_t *>(pa + row + 4));
          if (row + 4 < lenB) nB = __ldg(reinterpret_cast<const uint32_t *>(pb + row + 4));
          if ((row & 127) == 0) {
            if (row + 256 < lenA) asm volatile("prefetch.global.L1 [%0];" ::"l"(pa + row + 256));
            if (row + 256 < lenB) asm volatile("prefetch.global.L1 [%0];" ::"l"(pb + row + 256));
          }
        }
        uint32_t cA = wA & 0xffu, cB = wB & 0xffu;
        if (remap) {  // codes that score alike share a profile row
          cA = prof[remap_off + cA];
          cB = prof[remap_off + cB];
        }
        wA >>= 8;
        wB >>= 8;
        if (LAYOUT == PROF_PAIR) {
          const uint4 *r4 = reinterpret_cast<const uint4 *>(prof32 + ((cA * alpha + cB) * G + t) * kp);
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
          // pair is b * 65536 + a, one integer multiply-add (the multiplier is
          // a runtime value, so this stays an IMAD on the FMA pipe, which the
          // DPX recurrence on the ALU pipe leaves idle)
          const uint4 *ra = reinterpret_cast<const uint4 *>(prof32 + (cA * G + t) * kp);
          const uint4 *rb = reinterpret_cast<const uint4 *>(prof32 + (cB * G + t) * kp);
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
          const uint4 *ra = reinterpret_cast<const uint4 *>(prof16 + (cA * G + t) * kp);
          const uint4 *rb = reinterpret_cast<const uint4 *>(prof16 + (cB * G + t) * kp);
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
      }

      // ---- the row: backward pass (columns independent), then the F chain ----
#pragma unroll
      for (int j = K - 1; j >= 0; --j) {
        const uint32_t T = __viaddmax_s16x2(j == 0 ? prevH : H[j - 1], P[j], E[j]);
        if (MODE == SG) {
          E[j] = __viaddmax_s16x2(T, EOPEN, E[j]);  // in the row frames (see the header)
        } else {
          const uint32_t u = __viaddmax_s16x2(T, NOPEN, VFLOOR);
          E[j] = __viaddmax_s16x2(E[j], NEXT, u);
        }
        H[j] = T;
      }
      uint32_t Fs = (t == 0) ? FS_IN : msgF;
#pragma unroll
      for (int j = 0; j < K; ++j) {
        const uint32_t T = H[j];
        H[j] = __viaddmax_s16x2(Fs, NOPEN, T);
        Fs = __viaddmax_s16x2(Fs, NEXT, T);
      }
      prevH = (t == 0) ? dup16(hleft + frame_of(row)) : msgH;  // this row's H left of column 0
      outH = H[K - 1];
      outF = Fs;
      outC = msgC;

      if (MODE == SW) {
        uint32_t cm = H[0];
#pragma unroll
        for (int j = 1; j + 1 < K; j += 2) cm = __vimax3_s16x2(cm, H[j], H[j + 1]);
        if ((K & 1) == 0 && K > 1) cm = __viaddmax_s16x2(cm, 0u, H[K - 1]);
        // Only a row maximum above every cell so far in this thread AND in
        // all columns to its left (`left`, the running best passed along the
        // pipeline for this row) can be the first row of the record's
        // maximum at its smallest column; anything else is dominated
        // (smaller, or equal in an earlier row or a smaller column), so only
        // those improvements are recorded.
        const uint32_t left = (t == 0) ? 0u : msgBest;
        const uint32_t thr = __viaddmax_s16x2(best, 0u, left);
        const uint32_t nb = __viaddmax_s16x2(thr, 0u, cm);
        outBest = nb;
        if (nb != thr) {
          // keep this row (shared-memory stores only); the column of the
          // maximum is looked up once, at the record's last row
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
      }

      if (MODE == SG && te) {
        // running max of column Q-1 (register K-1 of thread G-1); a strict
        // improvement records the row, so the FIRST row of the maximum wins
        const uint32_t nb = __viaddmax_s16x2(best, 0u, __viaddmax_s16x2(H[K - 1], dup16(-frame_of(row)), NEGMIN));
        if (nb != best) {
          if (lo16(nb) != lo16(best)) rowA = row;
          if (hi16(nb) != hi16(best)) rowB = row;
          best = nb;
        }
      }
    } else {
      outC = CTL_IDLE;
    }

    // ---- last row of a record: fold partial results left to right ----
    // (a handled end moves ev_row on, so an idle thread never sees it again)
    const bool ev = row == ev_row;
    if (__any_sync(FULL, ev || has_out)) {
      const bool lastA = ev && row == lastA_row, lastB = ev && row == lastB_row;
      if (ev) {  // the other record's end, if it is still ahead
        int nxt = lastA_row > row ? lastA_row : -3;
        if (lastB_row > row && (nxt < 0 || lastB_row < nxt)) nxt = lastB_row;
        ev_row = nxt;
      }
      const uint32_t iR0 = __shfl_up_sync(FULL, oR0, 1, G);
      const uint32_t iR1 = __shfl_up_sync(FULL, oR1, 1, G);
      uint32_t iR2 = 0, iR3 = 0;
      if (MODE == SW) {
        iR2 = __shfl_up_sync(FULL, oR2, 1, G);
        iR3 = __shfl_up_sync(FULL, oR3, 1, G);
      }
      has_out = false;
      if (lastA || lastB) {
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
              oR0 = mx;
              oR1 = mq;
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
                score = (x == 0 ? lo16(outH) : hi16(outH)) - frame_of(row);  // this row's H(i, Q-1)
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
            oR0 = (uint32_t)(bA & 0xffff) | ((uint32_t)bB << 16);
            oR1 = (uint32_t)(qA & 0xffff) | ((uint32_t)qB << 16);
            oR2 = (uint32_t)rA;
            oR3 = (uint32_t)rB;
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
      }
    }

    // Every row thread 0 starts reaches thread G-1 within G-1 steps, so the
    // group is done once thread 0 is and no row is in flight.  The step budget
    // (all rows of the range plus the pipeline depth) is a hard stop.
    // (checked every 8 steps; idle extra steps do nothing)
    if (--chk == 0) {
      chk = 8;
      steps += 8;
      const bool more = busy || (t == 0 && !f_done);
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
      s_skip = taken >= (tl.count + 1) / 2;
      if (!s_skip) {
        sp = *qp;
        sp.first = tl.first;
        sp.count = tl.count;
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
