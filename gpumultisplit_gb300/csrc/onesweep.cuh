// One-sweep LSD radix sort of 32-bit keys (optionally with 32-bit values).
//
// The multisplit sort (src/api/multisplit_sort.cuh:320-364,
// src/api/multisplit_sort_pairs.cuh:21-65) runs prescan -> scan -> postscan for
// every digit.  Here:
//   1. onesweep_hist_kernel counts every digit of the schedule in one read of
//      the keys (a digit's global histogram does not depend on the key order);
//   2. onesweep_bases_kernel turns each digit's histogram into bucket starts;
//   3. per digit, onesweep_pass_kernel claims tiles in order by ticket, stages
//      and ranks a tile exactly as the multisplit postscan does, publishes the
//      tile's per-bucket counts as soon as they are known (after phase 2),
//      sorts the tile in shared memory (phase 3) and only then looks back over
//      the earlier tiles' published counts, per bucket, for its global
//      offsets.  The look-back's memory round trips thus come after the
//      tile's shared-memory reorder rather than in front of it.
// Every digit pass is a stable multisplit, so the output equals the
// multisplit sort's bit for bit.
//
// Status words: one per (tile, bucket) of the current digit, 64 bits,
// (flag << 32) | count, written with single 64-bit stores so flag and count
// are never torn.  flag 1: the tile's own count; flag 2: the count of this
// bucket in this tile and every earlier one (inclusive).
#pragma once

#include "multisplit_kernels.cuh"

namespace gms {

constexpr int OS_MAX_PASSES = 8;            // 32-bit keys, digits of 4 to 8 bits
constexpr uint32_t OS_HIST_STRIDE = 256;    // words per digit in the histogram / bucket starts
constexpr uint32_t OS_HIST_SMEM = 2048;     // shared bins of the histogram kernel
constexpr uint64_t OS_FLAG_AGGREGATE = 1ull << 32;
constexpr uint64_t OS_FLAG_INCLUSIVE = 2ull << 32;
constexpr uint64_t OS_FLAG_MASK = 3ull << 32;

struct OnesweepDigits {
  int passes;
  uint32_t shift[OS_MAX_PASSES];
  uint32_t logb[OS_MAX_PASSES];
};

// Shared layout of the histogram kernel: digit p's bins start at off(p); bins
// of digits narrower than 5 bits are replicated 32/B times (lane l uses
// replica l % R) so few lanes of a warp hit the same word.
__host__ __device__ inline uint32_t os_replicas(uint32_t logb) { return logb >= 5 ? 1u : (32u >> logb); }

__host__ __device__ inline uint32_t os_bins(const OnesweepDigits& d) {
  uint32_t total = 0;
  for (int p = 0; p < d.passes; ++p) total += (1u << d.logb[p]) * os_replicas(d.logb[p]);
  return total;
}

// hist[p * OS_HIST_STRIDE + b] += count of keys whose digit p is b.  hist is
// zeroed by the caller.  Persistent grid; 16-byte vector loads when the keys
// are 16-byte aligned.
__global__ void __launch_bounds__(256) onesweep_hist_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                            OnesweepDigits d, uint32_t* __restrict__ hist) {
  __shared__ uint32_t s_h[OS_HIST_SMEM];
  const uint32_t tid = threadIdx.x;
  const uint32_t lane = tid & 31u;
  const uint32_t bins = os_bins(d);
  for (uint32_t i = tid; i < bins; i += blockDim.x) s_h[i] = 0u;
  // per digit: shift, mask, log2 of the replica count, and this lane's first word
  uint32_t sh[OS_MAX_PASSES], mk[OS_MAX_PASSES], lr[OS_MAX_PASSES], at[OS_MAX_PASSES];
  uint32_t off = 0;
#pragma unroll
  for (int p = 0; p < OS_MAX_PASSES; ++p) {
    const bool on = p < d.passes;
    const uint32_t logb = on ? d.logb[p] : 1u;
    const uint32_t r = os_replicas(logb);
    sh[p] = on ? d.shift[p] : 0u;
    mk[p] = (1u << logb) - 1u;
    lr[p] = logb >= 5 ? 0u : 5u - logb;
    at[p] = off + (lane & (r - 1u));
    off += on ? (1u << logb) * r : 0u;
  }
  __syncthreads();
  auto count = [&](uint32_t key) {
#pragma unroll
    for (int p = 0; p < OS_MAX_PASSES; ++p) {
      if (p < d.passes) atomicAdd(&s_h[at[p] + (((key >> sh[p]) & mk[p]) << lr[p])], 1u);
    }
  };
  const bool vec = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0;
  const uint32_t nv = vec ? n / 4u : 0u;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t v = blockIdx.x * blockDim.x + tid; v < nv; v += stride) {
    const uint4 q = ld_nc_v4(keys + 4u * v);
    count(q.x);
    count(q.y);
    count(q.z);
    count(q.w);
  }
  for (uint32_t i = 4u * nv + blockIdx.x * blockDim.x + tid; i < n; i += stride) count(keys[i]);
  __syncthreads();
  // add the replicas of every bin and the block's counts into the histogram
  uint32_t first = 0;
  for (int p = 0; p < d.passes; ++p) {
    const uint32_t B = 1u << d.logb[p], r = os_replicas(d.logb[p]);
    for (uint32_t b = tid; b < B; b += blockDim.x) {
      uint32_t c = 0;
      for (uint32_t k = 0; k < r; ++k) c += s_h[first + b * r + k];
      if (c != 0u) atomicAdd(&hist[p * OS_HIST_STRIDE + b], c);
    }
    first += B * r;
  }
}

// One block per digit: its histogram becomes the buckets' global starts
// (exclusive scan over B <= 256 buckets), in place.
__global__ void __launch_bounds__(256) onesweep_bases_kernel(uint32_t* __restrict__ hist, OnesweepDigits d) {
  __shared__ uint32_t s_warp[8];
  const uint32_t p = blockIdx.x, tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t B = 1u << d.logb[p];
  const uint32_t c = tid < B ? hist[p * OS_HIST_STRIDE + tid] : 0u;
  uint32_t incl = c;
#pragma unroll
  for (int k = 1; k < 32; k <<= 1) {
    const uint32_t t = __shfl_up_sync(~0u, incl, k);
    if (lane >= uint32_t(k)) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  uint32_t start = incl - c;
  for (uint32_t w = 0; w < warp; ++w) start += s_warp[w];
  if (tid < B) hist[p * OS_HIST_STRIDE + tid] = start;
}

// A tile's global bucket offsets by decoupled look-back over the earlier
// tiles' status words (see GivenOffset for the calls).  Every wait is bounded
// by the call's wait limit; on timeout the error is recorded and the tile
// still publishes, so no later tile waits forever.
struct LookbackOffset {
  static constexpr bool KNOWN_EARLY = false;  // resolved after the shared-memory reorder
  uint64_t* status;  // this digit's words, [tile][B]
  uint32_t tile;
  uint32_t num_buckets;
  uint32_t base;     // start of this thread's bucket over all tiles
  ScratchHeader* hdr;

  __device__ __forceinline__ void aggregate(uint32_t b, uint32_t total) {
    st_relaxed_u64(&status[size_t(tile) * num_buckets + b],
                   (tile == 0 ? OS_FLAG_INCLUSIVE : OS_FLAG_AGGREGATE) | uint64_t(total));
  }

  // The walk reads LOOKBACK_WINDOW predecessors per round trip: tiles start
  // a few nanoseconds apart but a status load takes most of a microsecond, so
  // a tile must look past a few dozen predecessors that have published only
  // their own counts before it meets an inclusive one.
  static constexpr int LOOKBACK_WINDOW = 16;

  __device__ __forceinline__ uint32_t offset(uint32_t b, uint32_t total) {
    if (tile == 0) return base;
    const uint64_t limit = error_recorded(hdr) ? 0ull : wait_limit_ns(hdr);
    uint32_t excl = 0;
    int64_t p = int64_t(tile) - 1;  // nearest tile not yet added
    uint64_t t0 = 0;
    bool waiting = false, timed_out = false;
    while (p >= 0) {
      uint64_t s[LOOKBACK_WINDOW];
#pragma unroll
      for (int i = 0; i < LOOKBACK_WINDOW; ++i)
        s[i] = p - i >= 0 ? ld_relaxed_u64(&status[size_t(p - i) * num_buckets + b]) : OS_FLAG_INCLUSIVE;
      // add the window's counts in order, up to the first inclusive one or
      // the first that is not published yet
      bool done = false, stall = false;
      int used = 0;
#pragma unroll
      for (int i = 0; i < LOOKBACK_WINDOW; ++i) {
        const uint64_t flag = s[i] & OS_FLAG_MASK;
        if (!done && !stall) {
          if (flag == 0ull) {
            stall = true;
          } else {
            excl += uint32_t(s[i]);
            used = i + 1;
            done = flag == OS_FLAG_INCLUSIVE;
          }
        }
      }
      if (done) break;
      p -= used;
      if (stall) {
        if (!waiting) {
          waiting = true;
          t0 = global_timer_ns();
        } else if (global_timer_ns() - t0 > limit) {
          timed_out = true;
          break;
        }
        __nanosleep(128);
      } else {
        waiting = false;
      }
    }
    if (timed_out) record_error(hdr, DEV_ERR_LOOKBACK_TIMEOUT);
    st_relaxed_u64(&status[size_t(tile) * num_buckets + b], OS_FLAG_INCLUSIVE | uint64_t(excl + total));
    return base + excl;
  }
};

// Blocks per SM a pass is register-budgeted for: the multisplit postscan's
// for key-value tiles; four (64 registers) for key-only tiles, whose six-block
// budget spills with the look-back's state.
template <class C, class P>
constexpr int onesweep_min_blocks() {
  return C::KV ? PostLayout<C, P>::MIN_BLOCKS : 4;
}

// One digit pass.  P identifies the digit (KIND_BITS: (key >> shift) & (B-1)).
// ticket: this pass's tile counter (zero before the launch); status: this
// pass's words (zero before the launch); bases: the digit's bucket starts.
template <class C, class P>
__global__ void __launch_bounds__(C::THREADS, (onesweep_min_blocks<C, P>())) onesweep_pass_kernel(
    const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
    uint32_t* __restrict__ vout, uint32_t n, uint32_t num_tiles, typename P::Params bp, ScratchHeader* hdr,
    uint32_t* ticket, uint64_t* status, const uint32_t* __restrict__ bases, uint32_t prefetch_dist) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint32_t s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const TileJob<typename P::Params> job{kin, vin, kout, vout, n, num_tiles, tile, nullptr, 0u,
                                        prefetch_dist != 0 ? tile + prefetch_dist : ~0u, bp, 0u, nullptr};
  postscan_job<C, P, true, false>(job, hdr, smem, nullptr,
                                  [&](const TileJob<typename P::Params>& j, uint32_t tid, uint32_t nb) {
                                    return LookbackOffset{status, j.tile, nb, tid < nb ? bases[tid] : 0u, hdr};
                                  });
}

}  // namespace gms
