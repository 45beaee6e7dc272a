// Key-value multisplit that allocates nothing: its scratch (scan state and
// bucket-count matrix) lives in a fixed array in device global memory that the
// library itself declares.
//
// Who needs it: code that cannot call cudaMalloc at the point where it wants a
// multisplit -- for example a caller inside a region where allocation is
// forbidden (a custom allocator's own bookkeeping, a plugin host that hands out
// only the input and output buffers, real-time paths that pre-size all memory
// at start-up), or a caller with no way to keep a scratch buffer alive between
// calls.  It still passes its own input and output buffers.
//
// Limits and rules:
//   * The array holds GMS_NOALLOC_SCRATCH_BYTES (4 MiB) on every GPU that loads
//     the library, for the life of the process.  A call is accepted when the
//     multisplit's minimum scratch (header, count matrix and scan status, without
//     the optional byte per key) fits: up to 16,764,928 pairs at 256 buckets
//     (4093 tiles of 4096), proportionally more at fewer buckets.  Larger calls
//     are rejected with GMS_ERROR_SCRATCH_TOO_SMALL.  Costly identifiers (range,
//     div, even-float) keep their byte per key in the array only when it also
//     fits, and otherwise evaluate the identifier in both stages; the output is
//     the same either way.  More than 256 buckets take two digit passes whose
//     ping-pong keys and values also live in the array (about 460 thousand pairs
//     at 1000 buckets).
//   * The first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture.
//   * Every call on a device shares the one array and leaves its contents
//     behind.  Each call's prescan rewrites everything the later stages read
//     (error word, scan ticket and status words, the whole count matrix), so no
//     clearing is needed between calls -- but calls whose work overlaps on the
//     GPU (different streams, or different host threads) race on the array and
//     must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/gpumultisplit.h"
#include "ms_host.h"

namespace {

constexpr size_t kNoAllocBytes = GMS_NOALLOC_SCRATCH_BYTES;

// The library-owned scratch.  In host code this name is only a host-side
// stand-in for the symbol, never a device address: the address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// Device address of g_noalloc_scratch on the current device (looked up once per device).
cudaError_t scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_addr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" gms_status gms_multisplit_key_value_noalloc(const uint32_t* d_key_in, const uint32_t* d_value_in,
                                                       uint32_t* d_key_out, uint32_t* d_value_out, uint32_t n,
                                                       const gms_bucket_desc* desc, gms_stream_t stream) {
  if (desc == nullptr) return GMS_ERROR_INVALID_VALUE;
  // Up to 256 buckets the minimum scratch (without the byte per key) is what
  // must fit; a call beyond it is rejected before the device is touched.  The
  // wrapped entry point checks again (and, above 256 buckets, alone), and keeps
  // bucket bytes only when they fit as well.
  if (n != 0 && desc->num_buckets >= 2 && desc->num_buckets <= 256) {
    int logb = 0;
    while ((1u << logb) < desc->num_buckets) ++logb;
    if (gms::make_geometry(n, logb, true).bytes > kNoAllocBytes) return GMS_ERROR_SCRATCH_TOO_SMALL;
  }
  if (n == 0) return gms_multisplit_key_value(d_key_in, d_value_in, d_key_out, d_value_out, 0, desc, nullptr, 0,
                                              nullptr, stream);
  void* scratch = nullptr;
  cudaError_t e = scratch_address(&scratch);
  if (e != cudaSuccess) {
    gms::note_cuda_error(e);
    return GMS_ERROR_CUDA;
  }
  return gms_multisplit_key_value(d_key_in, d_value_in, d_key_out, d_value_out, n, desc, scratch, kNoAllocBytes,
                                  nullptr, stream);
}
