// Launchers for one identifier kind: picks the compiled tile instance for
// log2 B and key/value, sets its shared-memory limit once per device, and
// launches prescan -> scan -> postscan on the caller's stream.
// Included by exactly one inst_*.cu per kind (explicit instantiation).
#pragma once

#include <atomic>

#include "batch_kernels.cuh"
#include "histogram_kernels.cuh"
#include "ms_host.h"
#include "multisplit_kernels.cuh"

namespace gms {

// Raise a kernel's dynamic shared-memory limit to `bytes` once per device (bit
// per device id); needed once its static plus dynamic shared memory passes 48 KB.
template <class Kernel>
inline cudaError_t ensure_smem_limit(Kernel k, size_t bytes, std::atomic<uint64_t>& done_mask,
                                     size_t static_bytes = 0) {
  if (bytes + static_bytes <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = 1ull << (dev & 63);
  if (done_mask.load(std::memory_order_acquire) & bit) return cudaSuccess;
  e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (e == cudaSuccess) done_mask.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

// Grid of a persistent kernel: as many blocks as fit on the device at once
// (cached per kernel; the device's SM count is read per call), capped by `work`.
// Postscan L2 prefetch distance, in quarters of a wave of resident blocks (0 = off).
#ifndef GMS_PREFETCH_WAVES
#define GMS_PREFETCH_WAVES 2
#endif

template <class Kernel>
inline uint32_t persistent_grid(Kernel k, int threads, uint32_t work, std::atomic<int>& per_sm_cache,
                                size_t smem = 0) {
  int per_sm = per_sm_cache.load(std::memory_order_relaxed);
  if (per_sm <= 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem) != cudaSuccess || per_sm <= 0)
      per_sm = 1;
    per_sm_cache.store(per_sm, std::memory_order_relaxed);
  }
  const uint64_t cap = uint64_t(device_sm_count()) * uint64_t(per_sm);
  return uint32_t(work < cap ? work : cap);
}

// Stages of one multisplit with identifier policy P (descriptor kinds here;
// user functors from the drop-in C++ headers).  `scratch` is laid out as
// make_geometry(n, LOGB, KV).  bucket_bytes (n bytes, or null): for
// identifiers that are costly to evaluate, the prescan stores every key's
// bucket there and the postscan reads it instead of evaluating the identifier
// a second time; the prescan and postscan of one multisplit must agree on it.
//
// KW / VW: 32-bit words per key / value.  64-bit keys (KW = 2) are identified
// by the prescan only, which stores every key's bucket in bucket_bytes (then
// required); their postscan reads those bytes.
template <int W>
using ElemT = std::conditional_t<W == 2, uint64_t, uint32_t>;

template <class P, int LOGB, bool KV, int KW = 1, int VW = 1>
cudaError_t launch_multisplit(const ElemT<KW>* kin, const ElemT<VW>* vin, ElemT<KW>* kout, ElemT<VW>* vout,
                              uint32_t n, const typename P::Params& params, unsigned char* scratch, int stages,
                              cudaStream_t stream, uint8_t* bucket_bytes = nullptr) {
  if constexpr (P::CHEAP) bucket_bytes = nullptr;
  using S = TileShape<LOGB, KV, KW, VW>;
  using C = TileCfg<LOGB, S::WARPS, S::IPT, KV, KW, VW>;
  const Geometry g = make_geometry(n, LOGB, KV, KW, VW);
  if (g.num_tiles == 0) return cudaSuccess;
  auto* hdr = reinterpret_cast<ScratchHeader*>(scratch);
  auto* status = reinterpret_cast<uint64_t*>(scratch + g.off_status);
  auto* matrix = reinterpret_cast<uint32_t*>(scratch + g.off_matrix);

  if constexpr (KW == 2) {
    if (bucket_bytes == nullptr) return cudaErrorInvalidValue;
    if (stages & STAGE_PRESCAN) {
      static std::atomic<int> per_sm{0};
      auto kern = prescan64_kernel<C, P>;
      const uint32_t grid = persistent_grid(kern, C::THREADS, g.num_tiles, per_sm);
      kern<<<grid, C::THREADS, 0, stream>>>(kin, n, g.num_tiles, matrix, params, hdr, status, g.num_chunks,
                                            bucket_bytes);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    if (stages & STAGE_SCAN) {
      cudaError_t e = run_scan(matrix, g.m, status, hdr, stream);
      if (e != cudaSuccess) return e;
    }
    if (stages & STAGE_POSTSCAN) {
      static std::atomic<uint64_t> smem_done{0};
      static std::atomic<int> per_sm{0};
      auto kern = postscan_kernel<C, P, true>;
      constexpr size_t smem = PostLayout<C, P, true>::BYTES;
      cudaError_t e = ensure_smem_limit(kern, smem, smem_done);
      if (e != cudaSuccess) return e;
      const uint32_t wave = persistent_grid(kern, C::THREADS, g.num_tiles, per_sm, smem);
      const uint32_t dist = (GMS_PREFETCH_WAVES * wave) / 4u;
      return launch_after_previous(kern, dim3(g.num_tiles), dim3(C::THREADS), smem, stream, kin, vin, kout, vout, n,
                                   g.num_tiles, matrix, params, hdr, dist, bucket_bytes);
    }
    return cudaSuccess;
  } else {
  if (stages & STAGE_PRESCAN) {
    static std::atomic<int> per_sm{0};
    auto kern = prescan_kernel<C, P>;
    const uint32_t grid = persistent_grid(kern, C::THREADS, g.num_tiles, per_sm);
    kern<<<grid, C::THREADS, 0, stream>>>(kin, n, g.num_tiles, matrix, params, hdr, status, g.num_chunks,
                                          bucket_bytes);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (stages & STAGE_SCAN) {
    cudaError_t e = run_scan(matrix, g.m, status, hdr, stream);
    if (e != cudaSuccess) return e;
  }
  if constexpr (!P::CHEAP) {
    if ((stages & STAGE_POSTSCAN) && bucket_bytes != nullptr) {
      // Buckets from the prescan: no identifier in the postscan at all.
      static std::atomic<uint64_t> smem_done{0};
      static std::atomic<int> per_sm{0};
      auto kern = postscan_kernel<C, P, true>;
      constexpr size_t smem = PostLayout<C, P, true>::BYTES;
      cudaError_t e = ensure_smem_limit(kern, smem, smem_done);
      if (e != cudaSuccess) return e;
      const uint32_t wave = persistent_grid(kern, C::THREADS, g.num_tiles, per_sm, smem);
      const uint32_t dist = (GMS_PREFETCH_WAVES * wave) / 4u;
      return launch_after_previous(kern, dim3(g.num_tiles), dim3(C::THREADS), smem, stream, kin, vin, kout, vout, n,
                                   g.num_tiles, matrix, params, hdr, dist, bucket_bytes);
    }
  }
  if ((stages & STAGE_POSTSCAN) && P::USES_SMEM) {
    // Identifiers with a shared area: persistent blocks prepare it once.
    static std::atomic<uint64_t> smem_done{0};
    static std::atomic<int> per_sm{0};
    auto kern = postscan_persistent_kernel<C, P>;
    constexpr size_t smem = PostLayout<C, P>::BYTES;
    cudaError_t e = ensure_smem_limit(kern, smem, smem_done);
    if (e != cudaSuccess) return e;
    const uint32_t grid = persistent_grid(kern, C::THREADS, g.num_tiles, per_sm, smem);
    return launch_after_previous(kern, dim3(grid), dim3(C::THREADS), smem, stream, kin, vin, kout, vout, n,
                                 g.num_tiles, matrix, params, hdr);
  }
  if (stages & STAGE_POSTSCAN) {
    static std::atomic<uint64_t> smem_done{0};
    static std::atomic<int> per_sm{0};
    auto kern = postscan_kernel<C, P>;
    constexpr size_t smem = PostLayout<C, P>::BYTES;
    cudaError_t e = ensure_smem_limit(kern, smem, smem_done);
    if (e != cudaSuccess) return e;
    // Prefetch distance: a fraction of the number of blocks resident at once (one wave).
    const uint32_t wave = persistent_grid(kern, C::THREADS, g.num_tiles, per_sm, smem);
    const uint32_t dist = (GMS_PREFETCH_WAVES * wave) / 4u;
    e = launch_after_previous(kern, dim3(g.num_tiles), dim3(C::THREADS), smem, stream, kin, vin, kout, vout, n,
                              g.num_tiles, matrix, params, hdr, dist, static_cast<const uint8_t*>(nullptr));
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
  }
}

template <int KIND, int LOGB, bool KV>
cudaError_t run_multisplit_t(const MsCall& c, int stages) {
  return launch_multisplit<DescPolicy<KIND, LOGB>, LOGB, KV>(c.kin, c.vin, c.kout, c.vout, c.n, c.bp, c.scratch,
                                                             stages, c.stream, c.bucket_bytes);
}

template <int KIND, bool KV>
cudaError_t run_multisplit_kv(const MsCall& c, int stages) {
  switch (c.logb) {
    case 1: return run_multisplit_t<KIND, 1, KV>(c, stages);
    case 2: return run_multisplit_t<KIND, 2, KV>(c, stages);
    case 3: return run_multisplit_t<KIND, 3, KV>(c, stages);
    case 4: return run_multisplit_t<KIND, 4, KV>(c, stages);
    case 5: return run_multisplit_t<KIND, 5, KV>(c, stages);
    case 6: return run_multisplit_t<KIND, 6, KV>(c, stages);
    case 7: return run_multisplit_t<KIND, 7, KV>(c, stages);
    case 8: return run_multisplit_t<KIND, 8, KV>(c, stages);
    default: return cudaErrorInvalidValue;
  }
}

template <int KIND>
cudaError_t run_multisplit(const MsCall& c, int stages) {
  return c.kv ? run_multisplit_kv<KIND, true>(c, stages) : run_multisplit_kv<KIND, false>(c, stages);
}

// 64-bit elements: (key words, value words) = (1, 2), (2, 0), (2, 1), (2, 2).
template <int KIND, int LOGB, bool KV, int KW, int VW>
cudaError_t run_multisplit_wide_t(const MsCallWide& c, int stages) {
  using K = ElemT<KW>;
  using V = ElemT<VW>;
  const K* kin = static_cast<const K*>(c.kin);
  const V* vin = static_cast<const V*>(c.vin);
  K* kout = static_cast<K*>(c.kout);
  V* vout = static_cast<V*>(c.vout);
  if constexpr (KW == 2)
    return launch_multisplit<DescPolicy64<KIND, LOGB>, LOGB, KV, KW, VW>(kin, vin, kout, vout, c.n, c.bp64,
                                                                           c.scratch, stages, c.stream,
                                                                           c.bucket_bytes);
  else
    return launch_multisplit<DescPolicy<KIND, LOGB>, LOGB, KV, KW, VW>(kin, vin, kout, vout, c.n, c.bp, c.scratch,
                                                                         stages, c.stream, c.bucket_bytes);
}

template <int KIND, int LOGB>
cudaError_t run_multisplit_wide_l(const MsCallWide& c, int stages) {
  if (c.kw == 1 && c.kv && c.vw == 2) return run_multisplit_wide_t<KIND, LOGB, true, 1, 2>(c, stages);
  if (c.kw == 2 && !c.kv) return run_multisplit_wide_t<KIND, LOGB, false, 2, 1>(c, stages);
  if (c.kw == 2 && c.kv && c.vw == 1) return run_multisplit_wide_t<KIND, LOGB, true, 2, 1>(c, stages);
  if (c.kw == 2 && c.kv && c.vw == 2) return run_multisplit_wide_t<KIND, LOGB, true, 2, 2>(c, stages);
  return cudaErrorInvalidValue;  // 32-bit keys and values take run_multisplit
}

template <int KIND, int LOGB>
cudaError_t run_histogram64_t(const uint64_t* keys, uint32_t n, const BucketParams64& bp, int32_t* hist,
                              cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  static std::atomic<int> per_sm{0};
  auto kern = histogram64_kernel<LOGB, KIND>;
  const uint32_t grid = persistent_grid(kern, HIST_THREADS, uint32_t((uint64_t(n) + HIST_CHUNK - 1) / HIST_CHUNK),
                                        per_sm);
  kern<<<grid, HIST_THREADS, 0, stream>>>(keys, n, hist, bp, bp.num_buckets);
  return cudaGetLastError();
}

template <int KIND>
cudaError_t run_histogram64(const uint64_t* keys, uint32_t n, int logb, const BucketParams64& bp, int32_t* hist,
                            cudaStream_t stream) {
  switch (logb) {
    case 1: return run_histogram64_t<KIND, 1>(keys, n, bp, hist, stream);
    case 2: return run_histogram64_t<KIND, 2>(keys, n, bp, hist, stream);
    case 3: return run_histogram64_t<KIND, 3>(keys, n, bp, hist, stream);
    case 4: return run_histogram64_t<KIND, 4>(keys, n, bp, hist, stream);
    case 5: return run_histogram64_t<KIND, 5>(keys, n, bp, hist, stream);
    case 6: return run_histogram64_t<KIND, 6>(keys, n, bp, hist, stream);
    case 7: return run_histogram64_t<KIND, 7>(keys, n, bp, hist, stream);
    case 8: return run_histogram64_t<KIND, 8>(keys, n, bp, hist, stream);
    default: return cudaErrorInvalidValue;
  }
}

template <int KIND>
cudaError_t run_multisplit_wide(const MsCallWide& c, int stages) {
  switch (c.logb) {
    case 1: return run_multisplit_wide_l<KIND, 1>(c, stages);
    case 2: return run_multisplit_wide_l<KIND, 2>(c, stages);
    case 3: return run_multisplit_wide_l<KIND, 3>(c, stages);
    case 4: return run_multisplit_wide_l<KIND, 4>(c, stages);
    case 5: return run_multisplit_wide_l<KIND, 5>(c, stages);
    case 6: return run_multisplit_wide_l<KIND, 6>(c, stages);
    case 7: return run_multisplit_wide_l<KIND, 7>(c, stages);
    case 8: return run_multisplit_wide_l<KIND, 8>(c, stages);
    default: return cudaErrorInvalidValue;
  }
}

template <int KIND, int LOGB, bool KV, int V>
cudaError_t run_batch_class_t(const BatchClassLaunch& c, int stage) {
  constexpr int WARPS = kTileVariants[V].warps;
  constexpr int IPT = kTileVariants[V].ipt;
  if constexpr (WARPS * 32 < (1 << LOGB)) {
    return cudaErrorInvalidValue;  // the shape has fewer threads than buckets
  } else {
    using C = TileCfg<LOGB, WARPS, IPT, KV>;
    if (c.class_tiles == 0) return cudaSuccess;
    if (stage == STAGE_PRESCAN) {
      static std::atomic<int> per_sm{0};
      auto kern = batch_prescan_kernel<C, KIND>;
      const uint32_t grid = persistent_grid(kern, C::THREADS, c.class_tiles, per_sm);
      kern<<<grid, C::THREADS, 0, c.stream>>>(c.segs, c.tile_map, c.class_tiles, c.matrix, c.byte_area);
      return cudaGetLastError();
    }
    static std::atomic<uint64_t> smem_done{0};
    using P = DescPolicy<KIND, LOGB>;
    constexpr size_t smem = PostLayout<C, P, !P::CHEAP>::BYTES;
    auto kern = batch_postscan_kernel<C, KIND>;
    cudaError_t e = ensure_smem_limit(kern, smem, smem_done);
    if (e != cudaSuccess) return e;
    kern<<<c.class_tiles, C::THREADS, smem, c.stream>>>(c.segs, c.tile_map, c.matrix, c.hdr, c.byte_area);
    return cudaGetLastError();
  }
}

template <int KIND, bool KV, int V>
cudaError_t run_batch_class_kv(const BatchClassLaunch& c, int stage) {
  switch (c.logb) {
    case 1: return run_batch_class_t<KIND, 1, KV, V>(c, stage);
    case 2: return run_batch_class_t<KIND, 2, KV, V>(c, stage);
    case 3: return run_batch_class_t<KIND, 3, KV, V>(c, stage);
    case 4: return run_batch_class_t<KIND, 4, KV, V>(c, stage);
    case 5: return run_batch_class_t<KIND, 5, KV, V>(c, stage);
    case 6: return run_batch_class_t<KIND, 6, KV, V>(c, stage);
    case 7: return run_batch_class_t<KIND, 7, KV, V>(c, stage);
    case 8: return run_batch_class_t<KIND, 8, KV, V>(c, stage);
    default: return cudaErrorInvalidValue;
  }
}

template <int KIND, int LOGB, bool KV>
cudaError_t run_batch_warp_t(const BatchClassLaunch& c) {
  static_assert(kWarpSegMax == WARP_SEG_MAX, "host and kernel agree on the warp segment size");
  if (c.class_tiles == 0) return cudaSuccess;
  const uint32_t blocks = (c.class_tiles + WARP_SEG_WARPS - 1) / WARP_SEG_WARPS;
  batch_warp_kernel<KIND, LOGB, KV><<<blocks, WARP_SEG_WARPS * 32, 0, c.stream>>>(c.segs, c.seg_ids, c.class_tiles,
                                                                                 c.matrix);
  return cudaGetLastError();
}

template <int KIND>
cudaError_t run_batch_warp(const BatchClassLaunch& c) {
  switch (c.logb) {
    case 1: return c.kv ? run_batch_warp_t<KIND, 1, true>(c) : run_batch_warp_t<KIND, 1, false>(c);
    case 2: return c.kv ? run_batch_warp_t<KIND, 2, true>(c) : run_batch_warp_t<KIND, 2, false>(c);
    case 3: return c.kv ? run_batch_warp_t<KIND, 3, true>(c) : run_batch_warp_t<KIND, 3, false>(c);
    case 4: return c.kv ? run_batch_warp_t<KIND, 4, true>(c) : run_batch_warp_t<KIND, 4, false>(c);
    case 5: return c.kv ? run_batch_warp_t<KIND, 5, true>(c) : run_batch_warp_t<KIND, 5, false>(c);
    case 6: return c.kv ? run_batch_warp_t<KIND, 6, true>(c) : run_batch_warp_t<KIND, 6, false>(c);
    case 7: return c.kv ? run_batch_warp_t<KIND, 7, true>(c) : run_batch_warp_t<KIND, 7, false>(c);
    case 8: return c.kv ? run_batch_warp_t<KIND, 8, true>(c) : run_batch_warp_t<KIND, 8, false>(c);
    default: return cudaErrorInvalidValue;
  }
}

template <int KIND, int V>
cudaError_t run_batch_class_v(const BatchClassLaunch& c, int stage) {
  return c.kv ? run_batch_class_kv<KIND, true, V>(c, stage) : run_batch_class_kv<KIND, false, V>(c, stage);
}

template <int KIND, int LOGB>
cudaError_t run_histogram_t(const uint32_t* keys, uint32_t n, const BucketParams& bp, int32_t* hist,
                            cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  static std::atomic<int> per_sm{0};
  auto kern = histogram_kernel<LOGB, DescPolicy<KIND, LOGB>>;
  const uint32_t grid = persistent_grid(kern, HIST_THREADS, uint32_t((uint64_t(n) + HIST_CHUNK - 1) / HIST_CHUNK), per_sm);
  kern<<<grid, HIST_THREADS, 0, stream>>>(keys, n, hist, bp, bp.num_buckets);
  return cudaGetLastError();
}

template <int KIND>
cudaError_t run_histogram(const uint32_t* keys, uint32_t n, int logb, const BucketParams& bp, int32_t* hist,
                          cudaStream_t stream) {
  switch (logb) {
    case 1: return run_histogram_t<KIND, 1>(keys, n, bp, hist, stream);
    case 2: return run_histogram_t<KIND, 2>(keys, n, bp, hist, stream);
    case 3: return run_histogram_t<KIND, 3>(keys, n, bp, hist, stream);
    case 4: return run_histogram_t<KIND, 4>(keys, n, bp, hist, stream);
    case 5: return run_histogram_t<KIND, 5>(keys, n, bp, hist, stream);
    case 6: return run_histogram_t<KIND, 6>(keys, n, bp, hist, stream);
    case 7: return run_histogram_t<KIND, 7>(keys, n, bp, hist, stream);
    case 8: return run_histogram_t<KIND, 8>(keys, n, bp, hist, stream);
    default: return cudaErrorInvalidValue;
  }
}

// ------------------------------------------- more than 256 buckets
template <int KIND, int LOGB, bool KV>
cudaError_t digit_prescan_scan_t(const DigitPass& c) {
  using S = TileShape<LOGB, KV>;
  using C = TileCfg<LOGB, S::WARPS, S::IPT, KV>;
  const Geometry g = make_geometry(c.n, LOGB, KV);
  if (g.num_tiles == 0) return cudaSuccess;
  if (c.bucket_bytes == nullptr) return cudaErrorInvalidValue;
  auto* hdr = reinterpret_cast<ScratchHeader*>(c.scratch);
  auto* status = reinterpret_cast<uint64_t*>(c.scratch + g.off_status);
  auto* matrix = reinterpret_cast<uint32_t*>(c.scratch + g.off_matrix);
  static std::atomic<int> per_sm{0};
  auto kern = prescan_kernel<C, DigitPolicy<KIND, LOGB>>;
  const uint32_t grid = persistent_grid(kern, C::THREADS, g.num_tiles, per_sm);
  kern<<<grid, C::THREADS, 0, c.stream>>>(c.kin, c.n, g.num_tiles, matrix, c.bp, hdr, status, g.num_chunks,
                                          c.bucket_bytes);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return run_scan(matrix, g.m, status, hdr, c.stream);
}

template <int LOGB, bool KV>
cudaError_t digit_postscan_t(const DigitPass& c) {
  using S = TileShape<LOGB, KV>;
  using C = TileCfg<LOGB, S::WARPS, S::IPT, KV>;
  using P = GivenBytesPolicy;
  const Geometry g = make_geometry(c.n, LOGB, KV);
  if (g.num_tiles == 0) return cudaSuccess;
  if (c.bucket_bytes == nullptr) return cudaErrorInvalidValue;
  auto* hdr = reinterpret_cast<ScratchHeader*>(c.scratch);
  auto* matrix = reinterpret_cast<uint32_t*>(c.scratch + g.off_matrix);
  static std::atomic<uint64_t> smem_done{0};
  static std::atomic<int> per_sm{0};
  auto kern = postscan_kernel<C, P, true>;
  constexpr size_t smem = PostLayout<C, P, true>::BYTES;
  cudaError_t e = ensure_smem_limit(kern, smem, smem_done);
  if (e != cudaSuccess) return e;
  const uint32_t wave = persistent_grid(kern, C::THREADS, g.num_tiles, per_sm, smem);
  const uint32_t dist = (GMS_PREFETCH_WAVES * wave) / 4u;
  return launch_after_previous(kern, dim3(g.num_tiles), dim3(C::THREADS), smem, c.stream, c.kin, c.vin, c.kout,
                               c.vout, c.n, g.num_tiles, matrix, c.bp, hdr, dist, c.bucket_bytes);
}

#define GMS_DIGIT_SWITCH(FN, ...)                                 \
  switch (c.logb) {                                               \
    case 1: return c.kv ? FN<__VA_ARGS__ 1, true>(c) : FN<__VA_ARGS__ 1, false>(c); \
    case 2: return c.kv ? FN<__VA_ARGS__ 2, true>(c) : FN<__VA_ARGS__ 2, false>(c); \
    case 3: return c.kv ? FN<__VA_ARGS__ 3, true>(c) : FN<__VA_ARGS__ 3, false>(c); \
    case 4: return c.kv ? FN<__VA_ARGS__ 4, true>(c) : FN<__VA_ARGS__ 4, false>(c); \
    case 5: return c.kv ? FN<__VA_ARGS__ 5, true>(c) : FN<__VA_ARGS__ 5, false>(c); \
    case 6: return c.kv ? FN<__VA_ARGS__ 6, true>(c) : FN<__VA_ARGS__ 6, false>(c); \
    case 7: return c.kv ? FN<__VA_ARGS__ 7, true>(c) : FN<__VA_ARGS__ 7, false>(c); \
    case 8: return c.kv ? FN<__VA_ARGS__ 8, true>(c) : FN<__VA_ARGS__ 8, false>(c); \
    default: return cudaErrorInvalidValue;                        \
  }

template <int KIND>
cudaError_t run_digit_prescan_scan(const DigitPass& c) {
  GMS_DIGIT_SWITCH(digit_prescan_scan_t, KIND,)
}

template <int KIND>
cudaError_t run_big_histogram(const uint32_t* keys, uint32_t n, const BucketParams& p, uint32_t* hist,
                              cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const uint32_t work = uint32_t((uint64_t(n) / 4 + HIST_THREADS) / HIST_THREADS);  // blocks of 4-key vectors
  if (p.num_buckets <= BIG_HIST_SMEM_BINS) {
    // Per-block shared histograms; the limit and the occupancy query assume the largest size.
    static std::atomic<int> per_sm{0};
    static std::atomic<uint64_t> smem_done{0};
    auto kern = big_histogram_kernel<KIND, true>;
    const size_t smem = size_t(p.num_buckets) * 4;
    cudaError_t e = ensure_smem_limit(kern, size_t(BIG_HIST_SMEM_BINS) * 4, smem_done,
                                      size_t(big_identifier_smem_words<KIND>()) * 4);
    if (e != cudaSuccess) return e;
    const uint32_t grid = persistent_grid(kern, HIST_THREADS, work, per_sm, size_t(BIG_HIST_SMEM_BINS) * 4);
    kern<<<grid, HIST_THREADS, smem, stream>>>(keys, n, p, hist);
    return cudaGetLastError();
  }
  static std::atomic<int> per_sm{0};
  auto kern = big_histogram_kernel<KIND, false>;
  const uint32_t grid = persistent_grid(kern, HIST_THREADS, work, per_sm);
  kern<<<grid, HIST_THREADS, 0, stream>>>(keys, n, p, hist);
  return cudaGetLastError();
}

template <int KIND>
cudaError_t run_big_offsets(const uint32_t* sorted_keys, uint32_t n, const BucketParams& p, uint32_t* starts,
                            cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  static std::atomic<int> per_sm{0};
  auto kern = big_offsets_kernel<KIND>;
  const uint32_t grid = persistent_grid(kern, HIST_THREADS, uint32_t((uint64_t(n) + HIST_THREADS - 1) / HIST_THREADS),
                                        per_sm);
  kern<<<grid, HIST_THREADS, 0, stream>>>(sorted_keys, n, p, starts);
  return cudaGetLastError();
}

}  // namespace gms

#define GMS_INSTANTIATE_KIND(K)                                                                        \
  template cudaError_t gms::run_multisplit<K>(const gms::MsCall&, int);                                \
  template cudaError_t gms::run_histogram<K>(const uint32_t*, uint32_t, int, const gms::BucketParams&, \
                                             int32_t*, cudaStream_t);

#define GMS_INSTANTIATE_BIG(K)                                                           \
  template cudaError_t gms::run_digit_prescan_scan<K>(const gms::DigitPass&);           \
  template cudaError_t gms::run_big_histogram<K>(const uint32_t*, uint32_t, const gms::BucketParams&, uint32_t*, \
                                                 cudaStream_t);                                                 \
  template cudaError_t gms::run_big_offsets<K>(const uint32_t*, uint32_t, const gms::BucketParams&, uint32_t*, \
                                               cudaStream_t);

#define GMS_INSTANTIATE_WIDE(K)                                                                          \
  template cudaError_t gms::run_multisplit_wide<K>(const gms::MsCallWide&, int);                        \
  template cudaError_t gms::run_histogram64<K>(const uint64_t*, uint32_t, int, const gms::BucketParams64&, \
                                               int32_t*, cudaStream_t);

#define GMS_INSTANTIATE_BATCH_WARP(K) template cudaError_t gms::run_batch_warp<K>(const gms::BatchClassLaunch&);

#define GMS_INSTANTIATE_BATCH(K, V) template cudaError_t gms::run_batch_class_v<K, V>(const gms::BatchClassLaunch&, int);
