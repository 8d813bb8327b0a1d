// wave.cuh -- the wavefront scoring kernel.
//
// A group of G threads (G = 1, 2, ..., 32; a sub-warp) scores a PAIR of
// records at once: the low and high 16-bit halves of every register belong to
// record A and record B of the pair.  Thread t of the group owns K consecutive
// query columns [t*K - d, (t+1)*K - d); the query is padded at the front with
// d >= 1 columns whose profile and boundary values make them transparent (see
// build_wave_profile), so the last query column is always the last register of
// thread G-1.  Records flow through the group as a software pipeline: thread t
// processes row i of the pair one step after thread t-1 did, receiving from it
// H(i, first column - 1), F(i, first column) and the control word (record codes
// of row i) through __shfl_up_sync.  G = 1 is "one thread per record pair with
// packed 16-bit lanes" for short queries; G = 32 is a warp-wide anti-diagonal
// wavefront for long queries.
//
// Per cell and record pair (two cells) the recurrence costs five DPX/SIMD
// instructions:
//   H = max(Hdiag + P, max(E, F));  v = H - open;  E = max(E - ext, v);  F = max(F - ext, v)
// (local alignment floors v at 0, which keeps E, F and H non-negative).
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

#include "engine.cuh"

namespace ish {

template <int K, int MODE, bool PAIR>
__global__ void __launch_bounds__(256) wave_kernel(const WaveParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x;
  {
    const uint4 *src = p.prof;
    uint4 *dst = reinterpret_cast<uint4 *>(smem_raw);
    const uint32_t nvec = p.prof_bytes >> 4;
    for (uint32_t i = tid; i < nvec; i += blockDim.x) dst[i] = src[i];
  }
  const int G = p.G;
  const int lane = tid & 31;
  const int t = lane & (G - 1);
  const int group = tid / G;
  uint32_t *slots = reinterpret_cast<uint32_t *>(smem_raw + ((p.prof_bytes + 15u) & ~15u)) + group * 32;
  __syncthreads();

  const unsigned FULL = 0xffffffffu;
  const uint32_t NOPEN = dup16(-p.open);
  const uint32_t NEXT = dup16(-p.ext);
  const uint32_t VFLOOR = (MODE == SW) ? 0u : dup16(-32768);
  const uint32_t HLEFT = dup16(p.hleft);
  const uint32_t FIN = dup16(p.fin);
  const bool te = (MODE == SG) && (p.ends & 8);
  const bool qe = (MODE == SG) && (p.ends & 2);
  const int qlast_local = K - 1;  // column Q-1 is register K-1 of thread G-1
  const uint32_t npairs = (p.count + 1) >> 1;

  // profile rows
  const uint16_t *prof16 = reinterpret_cast<const uint16_t *>(smem_raw);
  const uint32_t *prof32 = reinterpret_cast<const uint32_t *>(smem_raw);

  uint32_t H[K], E[K];
#pragma unroll
  for (int j = 0; j < K; ++j) { H[j] = 0; E[j] = 0; }
  uint32_t prevH = HLEFT;
  uint32_t outH = 0, outF = 0, outC = CTL_IDLE;
  int row = 0;
  int lenA = 0, lenB = 0;
  uint32_t origA = 0, origB = 0;
  uint64_t steps = 0;

  // tracking (see header comment)
  int bestA = 0, bestB = 0;    // SG: running max of H(i, Q-1); SW: running max of this thread's cells
  int rowA = -1, rowB = -1;    // first row of `best`, per lane
  int mqA = 0, mqB = 0;        // SW: smallest column of `best` in that row
  // last-row reduction messages
  uint32_t oR0 = 0, oR1 = 0, oR2 = 0, oR3 = 0, iR0 = 0, iR1 = 0, iR2 = 0, iR3 = 0;
  bool has_out = false;

  // thread-0 feeder state
  bool f_active = false, f_done = false;
  int f_row = 0, f_rows = 0, f_lenA = 0, f_lenB = 0;
  uint32_t f_seq = 31;
  const uint8_t *f_pa = nullptr, *f_pb = nullptr;
  uint4 f_curA = make_uint4(0, 0, 0, 0), f_nxtA = f_curA, f_curB = f_curA, f_nxtB = f_curA;
  uint32_t f_wA = 0, f_wB = 0;

  while (true) {
    __syncwarp();
    uint32_t msgH = __shfl_up_sync(FULL, outH, 1, G);
    uint32_t msgF = __shfl_up_sync(FULL, outF, 1, G);
    uint32_t msgC = __shfl_up_sync(FULL, outC, 1, G);
    if (__any_sync(FULL, has_out)) {
      iR0 = __shfl_up_sync(FULL, oR0, 1, G);
      iR1 = __shfl_up_sync(FULL, oR1, 1, G);
      if (MODE == SW) {
        iR2 = __shfl_up_sync(FULL, oR2, 1, G);
        iR3 = __shfl_up_sync(FULL, oR3, 1, G);
      }
      has_out = false;
    }

    if (t == 0) {
      // ---- feeder: inject the next row of the current pair ----
      if (!f_active && !f_done) {
        uint32_t pr = atomicAdd(p.counter, 1u);
        if (pr < npairs) {
          f_active = true;
          f_seq = (f_seq + 1) & 31;
          slots[f_seq] = pr;
          uint32_t sA = p.first + 2 * pr, sB = sA + 1;
          f_lenA = (int)p.rec.len[sA];
          f_lenB = (2 * pr + 1 < p.count) ? (int)p.rec.len[sB] : 0;
          f_pa = p.rec.codes + p.rec.off[sA];
          f_pb = f_lenB ? p.rec.codes + p.rec.off[sB] : f_pa;
          f_rows = max(max(f_lenA, f_lenB), 1);
          f_row = 0;
          f_nxtA = __ldg(reinterpret_cast<const uint4 *>(f_pa));
          f_nxtB = f_lenB ? __ldg(reinterpret_cast<const uint4 *>(f_pb)) : make_uint4(0, 0, 0, 0);
        } else {
          f_done = true;
        }
      }
      if (f_active) {
        const int r = f_row;
        if ((r & 15) == 0) {
          f_curA = f_nxtA;
          f_curB = f_nxtB;
          if (r + 16 < f_lenA) f_nxtA = __ldg(reinterpret_cast<const uint4 *>(f_pa + r + 16));
          if (r + 16 < f_lenB) f_nxtB = __ldg(reinterpret_cast<const uint4 *>(f_pb + r + 16));
        }
        if ((r & 3) == 0) {
          const int w = (r >> 2) & 3;
          f_wA = w == 0 ? f_curA.x : w == 1 ? f_curA.y : w == 2 ? f_curA.z : f_curA.w;
          f_wB = w == 0 ? f_curB.x : w == 1 ? f_curB.y : w == 2 ? f_curB.z : f_curB.w;
        }
        uint32_t cA = r < f_lenA ? (f_wA & 0xffu) : 0u;
        uint32_t cB = r < f_lenB ? (f_wB & 0xffu) : 0u;
        f_wA >>= 8;
        f_wB >>= 8;
        if (cA >= (uint32_t)p.alphabet || cB >= (uint32_t)p.alphabet) {
          atomicOr(p.error, 1);
          cA = 0;
          cB = 0;
        }
        msgC = cA | (cB << 8) | (r == 0 ? CTL_NEW : 0u) | (f_seq << CTL_SEQ_SHIFT);
        f_row = r + 1;
        if (f_row >= f_rows) f_active = false;
      } else {
        msgC = CTL_IDLE;
      }
      msgH = HLEFT;
      msgF = FIN;
    }

    const bool busy = !(msgC & CTL_IDLE);
    if (busy) {
      if (msgC & CTL_NEW) {
        const uint32_t pr = slots[(msgC >> CTL_SEQ_SHIFT) & 31];
        const uint32_t sA = p.first + 2 * pr, sB = sA + 1;
        lenA = (int)p.rec.len[sA];
        origA = p.rec.orig[sA];
        if (2 * pr + 1 < p.count) {
          lenB = (int)p.rec.len[sB];
          origB = p.rec.orig[sB];
        } else {
          lenB = 0;
        }
        const int16_t *hi = p.hinit + t * K;
#pragma unroll
        for (int j = 0; j < K; ++j) {
          const int h0 = hi[j];
          H[j] = dup16(h0);
          E[j] = (MODE == SW) ? 0u : dup16(h0 - p.open);
        }
        prevH = (t == 0) ? HLEFT : dup16(p.hinit[t * K - 1]);
        bestA = bestB = (MODE == SW) ? 0 : p.neg_limit;
        rowA = rowB = -1;
        mqA = mqB = 0;
        row = 0;
      } else {
        ++row;
      }

      // ---- profile of this row ----
      const uint32_t cA = msgC & 0xffu, cB = (msgC >> 8) & 0xffu;
      uint32_t P[K];
      if (PAIR) {
        const uint4 *r4 = reinterpret_cast<const uint4 *>(prof32 + ((cA * p.alphabet + cB) * G + t) * p.kp);
#pragma unroll
        for (int v = 0; v < (K + 3) / 4; ++v) {
          const uint4 w = r4[v];
          if (4 * v + 0 < K) P[4 * v + 0] = w.x;
          if (4 * v + 1 < K) P[4 * v + 1] = w.y;
          if (4 * v + 2 < K) P[4 * v + 2] = w.z;
          if (4 * v + 3 < K) P[4 * v + 3] = w.w;
        }
      } else {
        const uint4 *ra = reinterpret_cast<const uint4 *>(prof16 + (cA * G + t) * p.kp);
        const uint4 *rb = reinterpret_cast<const uint4 *>(prof16 + (cB * G + t) * p.kp);
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

      // ---- the row ----
      uint32_t hdiag = prevH;
      uint32_t F = msgF;
#pragma unroll
      for (int j = 0; j < K; ++j) {
        const uint32_t ef = __vmaxs2(E[j], F);
        const uint32_t h = __viaddmax_s16x2(hdiag, P[j], ef);
        hdiag = H[j];
        H[j] = h;
        const uint32_t v = __viaddmax_s16x2(h, NOPEN, VFLOOR);
        E[j] = __viaddmax_s16x2(E[j], NEXT, v);
        F = __viaddmax_s16x2(F, NEXT, v);
      }
      prevH = msgH;
      outH = H[K - 1];
      outF = F;
      outC = msgC;

      const bool lastA = (row == lenA - 1), lastB = (row == lenB - 1);

      if (MODE == SG) {
        if (te) {
          // strict improvement only: the FIRST row of the maximum wins
          const int ha = lo16(H[qlast_local]), hb = hi16(H[qlast_local]);
          if (ha > bestA) { bestA = ha; rowA = row; }
          if (hb > bestB) { bestB = hb; rowB = row; }
        }
        if (lastA || lastB) {
          uint32_t mx = 0;
          uint32_t mq = 0;
          if (qe) {
            // smallest column of the row maximum, this thread's columns
            int bA = -32768, bB = -32768, qA = 0x7fff, qB = 0x7fff;
#pragma unroll
            for (int j = 0; j < K; ++j) {
              const int q = t * K + j - p.d;
              if (q >= 0) {
                const int a = lo16(H[j]), b = hi16(H[j]);
                if (a > bA) { bA = a; qA = q; }
                if (b > bB) { bB = b; qB = q; }
              }
            }
            if (t > 0) {  // fold in columns to the left (thread t-1, previous step)
              const int ia = lo16(iR0), ib = hi16(iR0);
              if (!(bA > ia)) { bA = ia; qA = (int)(iR1 & 0xffffu); }
              if (!(bB > ib)) { bB = ib; qB = (int)(iR1 >> 16); }
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
              const bool fin = x == 0 ? lastA : lastB;
              if (!fin) continue;
              const uint32_t orig = x == 0 ? origA : origB;
              const int T = x == 0 ? lenA : lenB;
              const int hl = x == 0 ? lo16(H[qlast_local]) : hi16(H[qlast_local]);
              int score, er, eq;
              if (!te && !qe) {
                score = hl; er = T - 1; eq = p.Q - 1;
              } else {
                int s0 = x == 0 ? bestA : bestB;
                int r0 = x == 0 ? rowA : rowB;
                score = te ? s0 : p.neg_limit;
                er = te ? r0 : (x == 0 ? rowA : rowB);
                eq = p.Q - 1;
                if (qe) {
                  const int s1 = x == 0 ? lo16(mx) : hi16(mx);
                  const int t1 = x == 0 ? (int)(mq & 0xffffu) : (int)(mq >> 16);
                  if (s1 > score) { score = s1; er = T - 1; eq = t1; }
                  else if (s1 == score && er == T - 1 && t1 < eq) { eq = t1; }
                }
              }
              if (p.out.score) p.out.score[orig] = score;
              if (p.out.qend) p.out.qend[orig] = eq;
              if (p.out.tend) p.out.tend[orig] = er;
              if (p.out.hit) p.out.hit[orig] = decide(SG, score, eq, er, p.dec);
            }
          }
        }
      } else {
        // ---- local: this thread's first strict maximum ----
        uint32_t cm = H[0];
#pragma unroll
        for (int j = 1; j + 1 < K; j += 2) cm = __vimax3_s16x2(cm, H[j], H[j + 1]);
        if ((K & 1) == 0 && K > 1) cm = __vmaxs2(cm, H[K - 1]);
        const int ca = lo16(cm), cb = hi16(cm);
        const bool upA = ca > bestA, upB = cb > bestB;
        if (upA || upB) {
          int qa = 0x7fff, qb = 0x7fff;
#pragma unroll
          for (int j = K - 1; j >= 0; --j) {
            const int q = t * K + j - p.d;
            if (lo16(H[j]) == ca) qa = q;
            if (hi16(H[j]) == cb) qb = q;
          }
          if (upA) { bestA = ca; rowA = row; mqA = qa; }
          if (upB) { bestB = cb; rowB = row; mqB = qb; }
        }
        if (lastA || lastB) {
          int bA = bestA, bB = bestB, rA = rowA, rB = rowB, qA = mqA, qB = mqB;
          if (t > 0) {
            const int ia = lo16(iR0), ib = hi16(iR0);
            const int ira = (int)iR2, irb = (int)iR3;
            const int iqa = (int)(int16_t)(iR1 & 0xffffu), iqb = (int)(int16_t)(iR1 >> 16);
            if (ia > bA || (ia == bA && (ira < rA || (ira == rA && iqa < qA)))) { bA = ia; rA = ira; qA = iqa; }
            if (ib > bB || (ib == bB && (irb < rB || (irb == rB && iqb < qB)))) { bB = ib; rB = irb; qB = iqb; }
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
              const bool fin = x == 0 ? lastA : lastB;
              if (!fin) continue;
              const uint32_t orig = x == 0 ? origA : origB;
              int score = x == 0 ? bA : bB;
              int er = x == 0 ? rA : rB;
              int eq = x == 0 ? qA : qB;
              if (score == 0) { er = -1; eq = 0; }
              if (p.out.score) p.out.score[orig] = score;
              if (p.out.qend) p.out.qend[orig] = eq;
              if (p.out.tend) p.out.tend[orig] = er;
              if (p.out.hit) p.out.hit[orig] = decide(SW, score, eq, er, p.dec);
            }
          }
        }
      }
    } else {
      outC = CTL_IDLE;
    }
    // Every row the feeder injects reaches thread G-1 within G-1 steps, so the
    // group is done once the feeder is and no row is in flight.  The step
    // budget (all rows of the range plus the pipeline depth) is a hard stop.
    const bool more = busy || (t == 0 && !f_done);
    if (!__any_sync(FULL, more)) break;
    if (++steps > p.max_steps) {
      if (lane == 0) atomicOr(p.error, 2);
      break;
    }
  }
}

}  // namespace ish
