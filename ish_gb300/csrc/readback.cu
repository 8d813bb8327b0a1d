// readback.cu -- records of a resident set copied back to the host in record
// order (ish_gpu_records_get): what a runner prints for its matches when the
// device split the file (ishlib/parallel_fastx_search_runner.mojo:306-331
// keeps every record's sequence for its output).
#include <algorithm>

#include "host.h"

namespace ish {

__global__ void k_invert(const uint32_t *orig_s, uint32_t n, uint32_t *inv);  // starts.cu

namespace {

// Length of each record of the range (record order).
__global__ void k_get_lengths(const uint32_t *inv, const uint32_t *len_s, uint32_t first, uint32_t count,
                              uint64_t *len) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    len[i] = len_s[inv[first + i]];
}

// Codes of each record of the range at its offset.
__global__ void k_get_codes(const uint32_t *inv, const uint32_t *len_s, const uint64_t *off_s, const uint8_t *codes,
                            uint32_t first, uint32_t count, const uint64_t *dst_off, uint8_t *dst) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const uint32_t j = inv[first + i];
    const uint8_t *s = codes + off_s[j];
    uint8_t *d = dst + dst_off[i];
    for (uint32_t k = 0, L = len_s[j]; k < L; ++k) d[k] = s[k];
  }
}

__global__ void k_get_total(const uint64_t *len, const uint64_t *off, uint32_t count, uint64_t *out_off) {
  out_off[count] = count ? off[count - 1] + len[count - 1] : 0;
}

}  // namespace

namespace host {
int scan_u64(ish_ctx *ctx, const uint64_t *in, uint64_t *out, uint64_t n, DevBuf &tmp, size_t tmp_off);
size_t scan_u64_scratch(uint64_t n);
}  // namespace host

}  // namespace ish

using namespace ish;
using namespace ish::host;

int ish_gpu_records_get(ish_ctx *ctx, int32_t set_id, uint32_t first, uint32_t count, uint8_t *codes,
                        uint64_t codes_cap, uint64_t *offsets) {
  if (!ctx) return ISH_EINVAL;
  int urc = ISH_OK;
  RecordSet *it_set = use_set(ctx, set_id, &urc);
  if (!it_set) return urc;
  RecordSet &rs = *it_set;
  if ((uint64_t)first + count > rs.n)
    return fail(ctx, ISH_EINVAL, "records [%u, %llu) outside the set's %u", first,
                (unsigned long long)first + count, rs.n);
  if (!offsets) return fail(ctx, ISH_EINVAL, "offsets is NULL");
  if (count == 0) {
    offsets[0] = 0;
    return ISH_OK;
  }
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const uint32_t nb = std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(rs.n, 256), (uint32_t)ctx->num_sms * 8));
  if (!rs.inv.p) {
    CU(rs.inv.ensure((size_t)rs.n * 4));
    k_invert<<<nb, 256, 0, s>>>(rs.orig_s.as<uint32_t>(), rs.n, rs.inv.as<uint32_t>());
    ++ctx->launches;
  }
  DevBuf len, off, scan, out;
  auto cleanup = [&] {
    cudaStreamSynchronize(s);
    len.release();
    off.release();
    scan.release();
    out.release();
  };
  int rc = ISH_OK;
  do {
    const uint32_t gb = std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(count, 256), (uint32_t)ctx->num_sms * 8));
    cudaError_t e = len.ensure((size_t)count * 8);
    if (e == cudaSuccess) e = off.ensure((size_t)(count + 1) * 8);
    if (e == cudaSuccess) e = scan.ensure(scan_u64_scratch(count));
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      rc = fail(ctx, ISH_ENOMEM, "records_get: %s", cudaGetErrorString(e));
      break;
    }
    k_get_lengths<<<gb, 256, 0, s>>>(rs.inv.as<uint32_t>(), rs.len_s.as<uint32_t>(), first, count,
                                     len.as<uint64_t>());
    ++ctx->launches;
    rc = scan_u64(ctx, len.as<uint64_t>(), off.as<uint64_t>(), count, scan, 0);
    if (rc) break;
    k_get_total<<<1, 1, 0, s>>>(len.as<uint64_t>(), off.as<uint64_t>(), count, off.as<uint64_t>());
    ++ctx->launches;
    e = cudaMemcpyAsync(offsets, off.p, (size_t)(count + 1) * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      rc = fail(ctx, ISH_EDEVICE, "records_get: %s", cudaGetErrorString(e));
      break;
    }
    const uint64_t total = offsets[count];
    if (total > codes_cap || (!codes && total)) {
      rc = fail(ctx, ISH_EOVERFLOW, "records_get: %llu code bytes, capacity %llu", (unsigned long long)total,
                (unsigned long long)codes_cap);
      break;
    }
    if (!total) break;
    e = out.ensure(total);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      rc = fail(ctx, ISH_ENOMEM, "records_get: %s", cudaGetErrorString(e));
      break;
    }
    k_get_codes<<<gb, 256, 0, s>>>(rs.inv.as<uint32_t>(), rs.len_s.as<uint32_t>(), rs.off_s.as<uint64_t>(),
                                   rs.codes.as<uint8_t>(), first, count, off.as<uint64_t>(), out.as<uint8_t>());
    ++ctx->launches;
    e = cudaMemcpyAsync(codes, out.p, total, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      rc = fail(ctx, ISH_EDEVICE, "records_get: %s", cudaGetErrorString(e));
    }
  } while (false);
  cleanup();
  return rc;
}
