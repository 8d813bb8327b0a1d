// noalloc.cu -- ish_gpu_score_noalloc: scoring that allocates nothing.
//
// Who needs it: callers that must not (or cannot) allocate device memory at
// the moment they score -- a host process whose device memory is owned by
// another allocator (a framework's caching pool or a fixed arena it must stay
// inside), plugins whose host forbids cudaMalloc/cudaFree from worker threads
// because they synchronise the device, and services that have to score while a
// hard device-memory budget is already spent.  Every other entry point of this
// library allocates (records are packed and sorted into library-owned HBM); this
// one scores records the caller already holds in device memory, into device
// outputs the caller owns.
//
// Its only working memory is `g_noalloc_scratch`, a file-scope __device__ array
// of NOALLOC_SCRATCH_BYTES (32 MiB) that is part of the library image: every
// GPU that loads this library holds it until the process exits.  It carries the
// error flag, a copy of the scoring matrix and the query, the query profile, the
// boundary row and the H/E columns of the one-thread-per-record kernel (the
// design of the plain kernel in kernels.cu).  Requests whose scratch does not
// fit are rejected with ISH_EOVERFLOW before anything is launched.
//
// Every call shares the array, and a call leaves its contents behind: the
// error flag is cleared at the start of each call, the profile and boundary row
// are rewritten, and each thread initialises its columns per record.  Calls
// whose work overlaps on the GPU (different streams, or different host threads
// on the same device) race on the array and must be serialised by the caller.
//
// The first call on a device, with that device current, resolves the array's
// device address with cudaGetSymbolAddress (the array's name is only a
// host-side stand-in, not a device address) and caches it; make that first
// call before any stream capture begins.
#include <mutex>

#include "../../include/ish_gpu.h"
#include "engine.cuh"

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 32u << 20;
constexpr int NOALLOC_MAX_DEVICES = 64;
constexpr int NA_THREADS = 128;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

struct NoallocDevice {
  unsigned char *base = nullptr;  // device address of g_noalloc_scratch on this device
  int sms = 0;
};

std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[NOALLOC_MAX_DEVICES];

inline size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

struct NaParams {
  const uint8_t *records;
  uint64_t records_bytes;
  const uint64_t *off;
  uint32_t n;
  const int16_t *prof;   // [alphabet][Q]
  const int16_t *hinit;  // [Q]
  int32_t *cols;         // 2 * Q * nthreads
  uint32_t nthreads;
  int Q, alphabet, open, ext, ends, neg_limit;
  long long max_safe_len;  // records longer than this leave the exact regime
  int *error;              // bit 0: code >= alphabet, bit 1: bad offsets, bit 2: record too long
  ish::OutDev out;
  ish::Decision dec;
};

__global__ void na_build_profile(const int8_t *M, const uint8_t *q, int A, int Q, int sg_init, int open, int ext,
                                 int16_t *prof, int16_t *hinit) {
  const int total = A * Q;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total + Q; i += gridDim.x * blockDim.x) {
    if (i < total) {
      const int c = i / Q, col = i - c * Q;
      prof[i] = M[c * A + q[col]];
    } else {
      const int col = i - total;
      hinit[col] = (int16_t)(sg_init ? -open - ext * col : 0);
    }
  }
}

template <int MODE>
__global__ void __launch_bounds__(NA_THREADS) na_plain_kernel(const NaParams p) {
  const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= p.nthreads) return;
  const uint32_t nth = p.nthreads;
  const int Q = p.Q, open = p.open, ext = p.ext;
  const bool ts = p.ends & 4, te = p.ends & 8, qe = p.ends & 2;
  int32_t *Hc = p.cols + gt;
  int32_t *Ec = p.cols + (size_t)Q * nth + gt;
  for (uint32_t r = gt; r < p.n; r += nth) {
    const uint64_t a = p.off[r], b = p.off[r + 1];
    int score = 0, qend = 0, tend = 0;
    if (b < a || b > p.records_bytes) {
      atomicOr(p.error, 2);
    } else if ((long long)(b - a) > p.max_safe_len) {
      atomicOr(p.error, 4);
    } else if (Q == 0 || b == a) {
      // empty query or record (semi_global_aln/striped.mojo:275-276; sw leaves
      // max 0, end -1 and query end 0, or -1 for an empty query)
      if (MODE == ish::SW) {
        tend = -1;
        qend = Q > 0 ? 0 : -1;
      }
    } else {
      const int T = (int)(b - a);
      const uint8_t *codes = p.records + a;
      for (int q = 0; q < Q; ++q) {
        const int h0 = p.hinit[q];
        Hc[(size_t)q * nth] = h0;
        Ec[(size_t)q * nth] = MODE == ish::SW ? 0 : h0 - open;
      }
      int best = MODE == ish::SW ? 0 : p.neg_limit, er = -1, eq = MODE == ish::SW ? 0 : Q - 1, hlast = 0;
      for (int i = 0; i < T; ++i) {
        uint32_t c = codes[i];
        if (c >= (uint32_t)p.alphabet) {
          atomicOr(p.error, 1);
          c = 0;
        }
        const int16_t *prow = p.prof + (size_t)c * Q;
        int hdiag = 0, F = 0;
        if (MODE == ish::SG) {
          hdiag = (i == 0 || ts) ? 0 : -open - ext * (i - 1);
          F = (ts ? 0 : -open - ext * i) - open;
        }
        int colmax = 0, colq = 0, h = 0;
        for (int q = 0; q < Q; ++q) {
          const int e = Ec[(size_t)q * nth];
          const int hold = Hc[(size_t)q * nth];
          h = max(hdiag + prow[q], max(e, F));
          hdiag = hold;
          Hc[(size_t)q * nth] = h;
          int v = h - open;
          if (MODE == ish::SW) v = max(v, 0);
          Ec[(size_t)q * nth] = max(e - ext, v);
          F = max(F - ext, v);
          if (MODE == ish::SW && h > colmax) {
            colmax = h;
            colq = q;
          }
        }
        if (MODE == ish::SW) {
          if (colmax > best) {
            best = colmax;
            er = i;
            eq = colq;
          }
        } else {
          if (h > best) {
            best = h;
            er = i;
          }
          hlast = h;
        }
      }
      if (MODE == ish::SW) {
        score = best;
        tend = best == 0 ? -1 : er;
        qend = best == 0 ? 0 : eq;
      } else if (!te && !qe) {
        score = hlast;
        tend = T - 1;
        qend = Q - 1;
      } else {
        score = te ? best : p.neg_limit;
        tend = er;
        qend = Q - 1;
        if (qe) {
          for (int q = 0; q < Q; ++q) {
            const int v = Hc[(size_t)q * nth];
            if (v > score) {
              score = v;
              qend = q;
              tend = T - 1;
            } else if (v == score && tend == T - 1 && q < qend) {
              qend = q;
            }
          }
        }
      }
    }
    if (p.out.score) p.out.score[r] = score;
    if (p.out.qend) p.out.qend[r] = qend;
    if (p.out.tend) p.out.tend[r] = tend;
    if (p.out.hit) p.out.hit[r] = ish::decide(MODE, score, qend, tend, p.dec);
  }
}

int na_fail(char *err, size_t err_len, int code, const char *msg) {
  if (err && err_len) {
    size_t i = 0;
    for (; msg[i] && i + 1 < err_len; ++i) err[i] = msg[i];
    err[i] = 0;
  }
  return code;
}

}  // namespace

extern "C" int ish_gpu_score_noalloc(const uint8_t *d_records, uint64_t records_bytes, const uint64_t *d_offsets,
                                     uint32_t n, const uint8_t *enc_query, uint32_t qlen, const int8_t *matrix,
                                     uint32_t alphabet, int algo, uint32_t gap_open, uint32_t gap_ext,
                                     uint32_t ends_free, int32_t max_score, float threshold, int32_t *d_score,
                                     int32_t *d_query_end, int32_t *d_target_end, uint8_t *d_hit, void *stream,
                                     char *err, size_t err_len) {
  if (err && err_len) err[0] = 0;
  if (algo != ISH_ALGO_SEMI_GLOBAL && algo != ISH_ALGO_LOCAL)
    return na_fail(err, err_len, ISH_EINVAL, "unknown algorithm");
  if (!matrix || alphabet < 1 || alphabet > 256) return na_fail(err, err_len, ISH_EINVAL, "matrix must be alphabet^2 int8");
  if (qlen && !enc_query) return na_fail(err, err_len, ISH_EINVAL, "enc_query is NULL");
  if (n && !d_offsets) return na_fail(err, err_len, ISH_EINVAL, "d_offsets is NULL");
  if (records_bytes && !d_records) return na_fail(err, err_len, ISH_EINVAL, "d_records is NULL");
  if (ends_free > 15) return na_fail(err, err_len, ISH_EINVAL, "ends_free has bits above ISH_FREE_TARGET_END");
  for (uint32_t i = 0; i < qlen; ++i)
    if (enc_query[i] >= alphabet) return na_fail(err, err_len, ISH_EINVAL, "query code >= alphabet");

  // --- scratch budget (checked before touching the device) ---
  const int Q = (int)qlen, A = (int)alphabet;
  const size_t off_mat = 256, off_q = off_mat + up256((size_t)A * A), off_prof = off_q + up256(qlen ? qlen : 1);
  const size_t off_hinit = off_prof + up256((size_t)A * Q * 2 + 2), off_cols = off_hinit + up256((size_t)Q * 2 + 2);
  if (qlen > 32767 || off_cols >= NOALLOC_SCRATCH_BYTES ||
      (Q > 0 && (NOALLOC_SCRATCH_BYTES - off_cols) / ((size_t)8 * Q) < (size_t)NA_THREADS))
    return na_fail(err, err_len, ISH_EOVERFLOW,
                   "query x alphabet too large for the 32 MiB no-allocation scratch (needs profile 2*A*Q bytes plus "
                   "1 KiB per query column for 128 threads)");

  // --- exact-integer regime of the one-thread-per-record kernel (as ish_gpu_score) ---
  int open, ext;
  if (algo == ISH_ALGO_SEMI_GLOBAL) {
    open = (int16_t)gap_open;
    ext = (int16_t)gap_ext;
  } else {
    open = (uint8_t)gap_open;
    ext = (uint8_t)gap_ext;
  }
  int mmin = 0, mmax = 0;
  for (size_t i = 0; i < (size_t)A * A; ++i) {
    mmin = matrix[i] < mmin ? matrix[i] : mmin;
    mmax = matrix[i] > mmax ? matrix[i] : mmax;
  }
  const int ends = algo == ISH_ALGO_SEMI_GLOBAL ? (int)ends_free : 0;
  long long max_safe_len = 1ll << 62;
  if (Q > 0) {
    const long base = 2L * open + (long)ext * (Q + 2) + (mmin < 0 ? -mmin : mmin) + 64;
    if (!(open > ext) || ext < 0 || (long)(Q + 1) * (mmax > 1 ? mmax : 1) > 30000 ||
        (algo == ISH_ALGO_SEMI_GLOBAL && (open + ext > 10000 || base > 30000)))
      return na_fail(err, err_len, ISH_EINVAL,
                     "parameters outside the exact-integer regime (gap_open must exceed gap_extend and scores must "
                     "stay within int16)");
    if (algo == ISH_ALGO_SEMI_GLOBAL && !(ends & ISH_FREE_TARGET_START) && ext > 0)
      max_safe_len = (30000 - base - open) / ext;
  }
  const int16_t o16 = (int16_t)open;
  const int neg_limit = ((int16_t)(-o16) < (int16_t)mmin) ? (int16_t)(-32768 + o16 + 1) : (int16_t)(-32768 - mmin + 1);

  // --- per-device set-up: the scratch array's device address ---
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return na_fail(err, err_len, ISH_ENODEV, "no current CUDA device");
  NoallocDevice nd;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocDevice &slot = g_noalloc_dev[dev];
    if (!slot.base) {
      void *ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr)
        return na_fail(err, err_len, ISH_EDEVICE, "cudaGetSymbolAddress of the no-allocation scratch failed");
      int sms = 0;
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
        return na_fail(err, err_len, ISH_EDEVICE, "cudaDeviceGetAttribute failed");
      slot.sms = sms;
      slot.base = static_cast<unsigned char *>(ptr);
    }
    nd = slot;
  }

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char *base = nd.base;
  int *d_err = reinterpret_cast<int *>(base);
  int8_t *d_mat = reinterpret_cast<int8_t *>(base + off_mat);
  uint8_t *d_q = base + off_q;
  int16_t *d_prof = reinterpret_cast<int16_t *>(base + off_prof);
  int16_t *d_hinit = reinterpret_cast<int16_t *>(base + off_hinit);
  int32_t *d_cols = reinterpret_cast<int32_t *>(base + off_cols);

  uint32_t blocks = (n + NA_THREADS - 1) / NA_THREADS;
  if (blocks > (uint32_t)nd.sms * 4) blocks = (uint32_t)nd.sms * 4;
  if (Q > 0) {
    const size_t fit = (NOALLOC_SCRATCH_BYTES - off_cols) / ((size_t)8 * Q) / NA_THREADS;
    if (blocks > fit) blocks = (uint32_t)fit;
  }
  if (blocks < 1) blocks = 1;

  cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_mat, matrix, (size_t)A * A, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && qlen) e = cudaMemcpyAsync(d_q, enc_query, qlen, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && Q > 0) {
    na_build_profile<<<64, 256, 0, s>>>(d_mat, d_q, A, Q,
                                        algo == ISH_ALGO_SEMI_GLOBAL && !(ends & ISH_FREE_QUERY_START), open, ext,
                                        d_prof, d_hinit);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && n) {
    NaParams p{};
    p.records = d_records;
    p.records_bytes = records_bytes;
    p.off = d_offsets;
    p.n = n;
    p.prof = d_prof;
    p.hinit = d_hinit;
    p.cols = d_cols;
    p.nthreads = blocks * NA_THREADS;
    p.Q = Q;
    p.alphabet = A;
    p.open = open;
    p.ext = ext;
    p.ends = ends;
    p.neg_limit = neg_limit;
    p.max_safe_len = max_safe_len;
    p.error = d_err;
    p.out = ish::OutDev{d_score, d_query_end, d_target_end, d_hit};
    p.dec = ish::Decision{max_score, threshold};
    if (algo == ISH_ALGO_LOCAL)
      na_plain_kernel<ish::SW><<<blocks, NA_THREADS, 0, s>>>(p);
    else
      na_plain_kernel<ish::SG><<<blocks, NA_THREADS, 0, s>>>(p);
    e = cudaGetLastError();
  }
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return na_fail(err, err_len, ISH_EDEVICE, cudaGetErrorString(e));
  if (herr & 2) return na_fail(err, err_len, ISH_EINVAL, "offsets are not monotone or exceed records_bytes");
  if (herr & 4)
    return na_fail(err, err_len, ISH_EINVAL, "a record is too long for the int16 boundary row (non-free target start)");
  if (herr & 1) return na_fail(err, err_len, ISH_EINVAL, "a record contains a code >= the alphabet size");
  return ISH_OK;
}
