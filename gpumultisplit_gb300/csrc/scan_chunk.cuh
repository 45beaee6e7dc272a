// One chunk of the single-pass exclusive prefix sum with decoupled look-back,
// in place over a uint32 array (the bucket-count matrix); scan_kernels.cuh
// runs it as one block per chunk, the batch queue as one work item per chunk.
// Replaces the reference's cub::DeviceScan::ExclusiveSum call
// (src/api/multisplit.cuh:141,258).
//
// Every wait is bounded in time; on timeout the chunk records
// DEV_ERR_LOOKBACK_TIMEOUT in the scratch header and still publishes, so no
// successor waits forever.
#pragma once

#include "gms_device.cuh"

namespace gms {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_IPT = GMS_SCAN_IPT;
constexpr uint32_t SCAN_CHUNK = SCAN_THREADS * SCAN_IPT;  // counts per chunk

enum : uint32_t { SCAN_FLAG_AGGREGATE = 1u, SCAN_FLAG_PREFIX = 2u };

__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) v += __shfl_xor_sync(~0u, v, d);
  return v;
}

// Scans chunk `chunk` of data[0, m) in place: exclusive values, offset by the
// sum of every earlier chunk, found by decoupled look-back over status[0,
// chunk).  status[c] = (flag << 32) | value, written once per phase with one
// 64-bit store.  Called by all SCAN_THREADS threads of a block.  The counts
// are read through L2 (`ld.global.cg`): in the batch queue they were written
// by other blocks of the same launch.
__device__ __forceinline__ void scan_chunk(uint32_t* __restrict__ data, uint32_t m, uint32_t chunk,
                                           uint64_t* __restrict__ status, ScratchHeader* hdr) {
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  __shared__ uint32_t s_prefix;

  const uint32_t tid = threadIdx.x;
  const uint32_t lane = tid & 31u;
  const uint32_t warp = tid >> 5;
  const uint32_t first = chunk * SCAN_CHUNK + tid * SCAN_IPT;

  // Load 16 consecutive counts per thread (16-byte vectors when `data` is
  // 16-byte aligned, which every caller arranges; element loads otherwise).
  const bool vec = (reinterpret_cast<uintptr_t>(data) & 15u) == 0;
  uint32_t v[SCAN_IPT];
  if (vec && first + SCAN_IPT <= m) {
#pragma unroll
    for (int k = 0; k < SCAN_IPT / 4; ++k) {
      const uint4 q = __ldcg(reinterpret_cast<const uint4*>(data + first + 4 * k));
      v[4 * k + 0] = q.x;
      v[4 * k + 1] = q.y;
      v[4 * k + 2] = q.z;
      v[4 * k + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) v[k] = (first + k < m) ? __ldcg(data + first + k) : 0u;
  }
  // Inclusive scan inside the thread.
#pragma unroll
  for (int k = 1; k < SCAN_IPT; ++k) v[k] += v[k - 1];
  const uint32_t thread_total = v[SCAN_IPT - 1];

  // Exclusive scan of thread totals across the warp, then across warps.
  uint32_t incl = thread_total;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t t = __shfl_up_sync(~0u, incl, d);
    if (lane >= uint32_t(d)) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  uint32_t warp_prefix = 0, chunk_total = 0;
#pragma unroll
  for (int w = 0; w < SCAN_THREADS / 32; ++w) {
    const uint32_t t = s_warp[w];
    warp_prefix += (uint32_t(w) < warp) ? t : 0u;
    chunk_total += t;
  }

  // Publish, then look back over predecessors 32 at a time.
  if (warp == 0) {
    uint32_t prefix = 0;
    if (chunk == 0) {
      if (lane == 0) st_relaxed_u64(&status[0], (uint64_t(SCAN_FLAG_PREFIX) << 32) | chunk_total);
    } else {
      if (lane == 0) st_relaxed_u64(&status[chunk], (uint64_t(SCAN_FLAG_AGGREGATE) << 32) | chunk_total);
      int64_t pred = int64_t(chunk) - 1;
      const uint64_t t0 = global_timer_ns();
      // After an error elsewhere in the call, give up on the first empty window.
      const uint64_t limit = error_recorded(hdr) ? 0ull : wait_limit_ns(hdr);
      bool timed_out = false;
      while (true) {
        const int64_t idx = pred - int64_t(lane);
        const uint64_t s = (idx >= 0) ? ld_relaxed_u64(&status[idx]) : (uint64_t(SCAN_FLAG_PREFIX) << 32);
        const uint32_t flag = uint32_t(s >> 32);
        if (__any_sync(~0u, flag == 0u)) {
          const bool late = (lane == 0) && (global_timer_ns() - t0 > limit);
          if (__shfl_sync(~0u, late ? 1u : 0u, 0)) {
            timed_out = true;
            break;
          }
          __nanosleep(32);
          continue;
        }
        const uint32_t pmask = __ballot_sync(~0u, flag == SCAN_FLAG_PREFIX);
        uint32_t val = uint32_t(s);
        if (pmask != 0u) {
          const uint32_t nearest = __ffs(pmask) - 1u;  // lane 0 is the closest predecessor
          prefix += warp_sum(lane <= nearest ? val : 0u);
          break;
        }
        prefix += warp_sum(val);
        pred -= 32;
      }
      if (timed_out && lane == 0) record_error(hdr, DEV_ERR_LOOKBACK_TIMEOUT);
      if (lane == 0) st_relaxed_u64(&status[chunk], (uint64_t(SCAN_FLAG_PREFIX) << 32) | (prefix + chunk_total));
    }
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();

  // Exclusive values: element k gets offset + inclusive(k-1).
  const uint32_t offset = s_prefix + warp_prefix + (incl - thread_total);
  uint32_t out[SCAN_IPT];
  out[0] = offset;
#pragma unroll
  for (int k = 1; k < SCAN_IPT; ++k) out[k] = offset + v[k - 1];
  if (vec && first + SCAN_IPT <= m) {
#pragma unroll
    for (int k = 0; k < SCAN_IPT / 4; ++k) {
      *reinterpret_cast<uint4*>(data + first + 4 * k) =
          make_uint4(out[4 * k + 0], out[4 * k + 1], out[4 * k + 2], out[4 * k + 3]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
      if (first + k < m) data[first + k] = out[k];
    }
  }
}

}  // namespace gms
