// In-translation-unit path of the drop-in API: a functor type the library has
// no descriptor for is compiled into the library's own kernel templates right
// here (FunctorPolicy), exactly as the reference instantiates its kernels on
// the user functor.  Needs nvcc and -I <repo>/gpumultisplit_gb300/csrc; without
// nvcc such functors are reported as GMS_ERROR_NOT_SUPPORTED.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gpumultisplit.h"

#if defined(__CUDACC__)
#include "ms_dispatch.cuh"

namespace gms {
namespace dropin {

inline bool generic_log2(uint32_t b, int* logb) {
  if (b < 2 || b > 256 || (b & (b - 1)) != 0) return false;
  int l = 0;
  while ((1u << l) < b) ++l;
  *logb = l;
  return true;
}

template <class F, bool KV>
cudaError_t generic_launch(int logb, const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout,
                           uint32_t n, const F& f, unsigned char* scratch, cudaStream_t s, uint8_t* bucket_bytes) {
  switch (logb) {
#define GMS_GENERIC_CASE(L)                                                                                    \
  case L:                                                                                                      \
    return launch_multisplit<FunctorPolicy<F, L>, L, KV>(kin, vin, kout, vout, n, f, scratch, STAGE_ALL, s, \
                                                         bucket_bytes);
    GMS_GENERIC_CASE(1)
    GMS_GENERIC_CASE(2)
    GMS_GENERIC_CASE(3)
    GMS_GENERIC_CASE(4)
    GMS_GENERIC_CASE(5)
    GMS_GENERIC_CASE(6)
    GMS_GENERIC_CASE(7)
    GMS_GENERIC_CASE(8)
#undef GMS_GENERIC_CASE
    default:
      return cudaErrorInvalidValue;
  }
}

// Multisplit with a user functor; same checks, scratch layout and offsets
// export as the C ABI.  vin == nullptr: key-only.
template <class F>
gms_status generic_multisplit(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                              uint32_t num_buckets, const F& f, void* scratch, size_t scratch_bytes,
                              uint32_t* h_offsets, cudaStream_t s) {
  int logb = 0;
  if (!generic_log2(num_buckets, &logb)) return GMS_ERROR_UNSUPPORTED_BUCKETS;
  const bool kv = vin != nullptr;
  if (n == 0) {
    if (h_offsets)
      for (uint32_t b = 0; b < num_buckets; ++b) h_offsets[b] = 0;
    return GMS_SUCCESS;
  }
  if (kin == nullptr || kout == nullptr || scratch == nullptr || (kv && vout == nullptr))
    return GMS_ERROR_INVALID_VALUE;
  const Geometry g = make_geometry(n, logb, kv);
  if (scratch_bytes < g.bytes) return GMS_ERROR_SCRATCH_TOO_SMALL;
  auto* sc = static_cast<unsigned char*>(scratch);
  // A user functor's cost is unknown: with room for a byte per key, its
  // buckets are computed once (prescan) and read back (postscan).
  uint8_t* bb = scratch_bytes >= g.bytes_full ? sc + g.off_buckets : nullptr;
  cudaError_t e = kv ? generic_launch<F, true>(logb, kin, vin, kout, vout, n, f, sc, s, bb)
                     : generic_launch<F, false>(logb, kin, nullptr, kout, nullptr, n, f, sc, s, bb);
  if (e == cudaSuccess && h_offsets) {
    e = cudaMemcpy2DAsync(h_offsets, sizeof(uint32_t), sc + g.off_matrix, size_t(g.num_tiles) * 4, sizeof(uint32_t),
                          num_buckets, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  return e == cudaSuccess ? GMS_SUCCESS : GMS_ERROR_CUDA;
}

// Histogram with a user functor (adds into d_hist).
template <class F>
gms_status generic_histogram(const uint32_t* keys, uint32_t n, uint32_t num_buckets, const F& f, int32_t* d_hist,
                             cudaStream_t s) {
  int logb = 0;
  if (!generic_log2(num_buckets, &logb)) return GMS_ERROR_UNSUPPORTED_BUCKETS;
  if (n == 0) return GMS_SUCCESS;
  cudaError_t e = cudaErrorInvalidValue;
  switch (logb) {
#define GMS_GENERIC_HIST(L)                                                                      \
  case L: {                                                                                      \
    static std::atomic<int> per_sm{0};                                                           \
    auto kern = histogram_kernel<L, FunctorPolicy<F, L>>;                                        \
    const uint32_t grid = persistent_grid(kern, HIST_THREADS, uint32_t((uint64_t(n) + HIST_CHUNK - 1) / HIST_CHUNK), per_sm); \
    kern<<<grid, HIST_THREADS, 0, s>>>(keys, n, d_hist, f, num_buckets);                         \
    e = cudaGetLastError();                                                                      \
    break;                                                                                       \
  }
    GMS_GENERIC_HIST(1)
    GMS_GENERIC_HIST(2)
    GMS_GENERIC_HIST(3)
    GMS_GENERIC_HIST(4)
    GMS_GENERIC_HIST(5)
    GMS_GENERIC_HIST(6)
    GMS_GENERIC_HIST(7)
    GMS_GENERIC_HIST(8)
#undef GMS_GENERIC_HIST
    default:
      break;
  }
  return e == cudaSuccess ? GMS_SUCCESS : GMS_ERROR_CUDA;
}

}  // namespace dropin
}  // namespace gms

#else  // host compiler: only functors with a descriptor are usable

namespace gms {
namespace dropin {
template <class F>
gms_status generic_multisplit(const uint32_t*, const uint32_t*, uint32_t*, uint32_t*, uint32_t, uint32_t, const F&,
                              void*, size_t, uint32_t*, cudaStream_t) {
  return GMS_ERROR_NOT_SUPPORTED;
}
template <class F>
gms_status generic_histogram(const uint32_t*, uint32_t, uint32_t, const F&, int32_t*, cudaStream_t) {
  return GMS_ERROR_NOT_SUPPORTED;
}
}  // namespace dropin
}  // namespace gms

#endif
