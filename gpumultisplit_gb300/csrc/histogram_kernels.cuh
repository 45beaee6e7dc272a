// Device-wide histogram over B <= 256 bins with any bucket identifier.
// Generalises the reference's multisplit2_histogram_even_* / _range_* kernels
// (src/kernels/histogram/multisplit2_histograms.cuh:36-699): a persistent grid
// counts per block (KeyCounter: ballots or replicated shared atomics), then
// adds one global atomicAdd per bin per block into the caller-zeroed int
// histogram.  Unlike the reference, any n is accepted (its kernels have no tail
// guard).
#pragma once

#include "multisplit_kernels.cuh"

namespace gms {

constexpr int HIST_WARPS = 8;
constexpr int HIST_THREADS = HIST_WARPS * 32;
constexpr int HIST_IPT = 16;
constexpr uint32_t HIST_CHUNK = HIST_THREADS * HIST_IPT;

// Persistent grid; block-strided over chunks of HIST_CHUNK keys.  The counts
// run over 2^LOGB bins; only the first num_bins (<= 2^LOGB, the caller's
// array) are written.
template <int LOGB, class P>
__global__ void __launch_bounds__(HIST_THREADS) histogram_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                                 int32_t* __restrict__ hist, typename P::Params bp,
                                                                 uint32_t num_bins) {
  using Counter = KeyCounter<LOGB, typename P::Id>;
  __shared__ uint32_t s_hist[Counter::smem_words(HIST_WARPS)];
  __shared__ uint32_t s_split[P::SMEM_WORDS];
  P::prepare(s_split, bp);
  Counter counter(P::make(bp, s_split), s_hist);
  counter.clear_shared();
  __syncthreads();
  count_tiles<HIST_THREADS, HIST_IPT>(keys, n, blockIdx.x, gridDim.x, counter, [](uint32_t) {});
  const uint32_t total = counter.block_total();
  if (threadIdx.x < num_bins && total) atomicAdd(&hist[threadIdx.x], int32_t(total));
}

// Histogram of 64-bit keys (the 64-bit identifiers, B <= 256): the same
// persistent counting as histogram_kernel, the keys read as 16-byte vectors of
// two when the array is 16-byte aligned.
template <int LOGB, int KIND>
__global__ void __launch_bounds__(HIST_THREADS) histogram64_kernel(const uint64_t* __restrict__ keys, uint32_t n,
                                                                   int32_t* __restrict__ hist, BucketParams64 bp,
                                                                   uint32_t num_bins) {
  using P = DescPolicy64<KIND, LOGB>;
  using Counter = KeyCounter<LOGB, typename P::Id>;
  __shared__ uint32_t s_hist[Counter::smem_words(HIST_WARPS)];
  __shared__ __align__(16) uint32_t s_split[P::SMEM_WORDS];
  P::prepare(s_split, bp);
  Counter counter(P::make(bp, s_split), s_hist);
  counter.clear_shared();
  __syncthreads();
  const bool vec = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0;
  for (uint32_t base = blockIdx.x * HIST_CHUNK; base < n; base += gridDim.x * HIST_CHUNK) {
    if (vec && n - base >= HIST_CHUNK) {
#pragma unroll 4
      for (int k = 0; k < HIST_IPT / 2; ++k) {
        const uint4 q = ld_nc_v4(reinterpret_cast<const uint32_t*>(keys + base + (uint32_t(k) * HIST_THREADS + threadIdx.x) * 2u));
        counter.template add_bucket<0>(counter.ident(uint64_t(q.x) | (uint64_t(q.y) << 32)), true);
        counter.template add_bucket<1>(counter.ident(uint64_t(q.z) | (uint64_t(q.w) << 32)), true);
      }
    } else {
#pragma unroll 4
      for (int k = 0; k < HIST_IPT; ++k) {
        const uint32_t i = base + uint32_t(k) * HIST_THREADS + threadIdx.x;
        const bool valid = i < n;
        counter.add_bucket(counter.ident(valid ? keys[i] : 0ull), valid);
      }
    }
  }
  const uint32_t total = counter.block_total();
  if (threadIdx.x < num_bins && total) atomicAdd(&hist[threadIdx.x], int32_t(total));
}

// Histogram over B > 256 bins (to 65536): the whole bucket id of every key
// (big_bucket_id).  Up to BIG_HIST_SMEM_BINS bins every block counts into a
// shared histogram (dynamic shared memory) and adds its non-zero bins into
// hist[0..B) at the end; above that, one global atomic per key.  Persistent
// grid, strided over keys.
constexpr uint32_t BIG_HIST_SMEM_BINS = 8192;

template <int KIND, bool SHARED>
__global__ void __launch_bounds__(HIST_THREADS) big_histogram_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                                     BucketParams p, uint32_t* __restrict__ hist) {
  __shared__ uint32_t s_split[big_identifier_smem_words<KIND>()];
  extern __shared__ uint32_t s_bins[];  // SHARED: B counters
  const uint32_t B = p.num_buckets;
  if constexpr (SHARED) {
    for (uint32_t b = threadIdx.x; b < B; b += HIST_THREADS) s_bins[b] = 0u;
  }
  prepare_big_identifier<KIND>(s_split, p);
  __syncthreads();
  auto add = [&](uint32_t key) {
    const uint32_t b = big_bucket_id<KIND>(key, p, s_split);
    if constexpr (SHARED)
      atomicAdd(&s_bins[b], 1u);
    else
      atomicAdd(&hist[b], 1u);
  };
  // 16-byte vectors of four keys while whole vectors remain (keys 16-byte
  // aligned), then single keys.
  const uint32_t stride = gridDim.x * HIST_THREADS;
  const uint32_t nv = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0 ? n / 4 : 0u;
  for (uint32_t v = blockIdx.x * HIST_THREADS + threadIdx.x; v < nv; v += stride) {
    const uint4 q = ld_nc_v4(keys + 4 * v);
    add(q.x);
    add(q.y);
    add(q.z);
    add(q.w);
  }
  for (uint32_t i = 4 * nv + blockIdx.x * HIST_THREADS + threadIdx.x; i < n; i += stride) add(keys[i]);
  if constexpr (SHARED) {
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < B; b += HIST_THREADS) {
      const uint32_t c = s_bins[b];
      if (c) atomicAdd(&hist[b], c);
    }
  }
}

// Bucket starts of a multisplit by the whole bucket id, read off its output
// (keys sorted by id, stably): key i starts every bucket b with
// id(key[i-1]) < b <= id(key[i]) (key -1 reading as id -1), and buckets past
// the last key's id start at n.  Every start is written exactly once.
template <int KIND>
__global__ void __launch_bounds__(HIST_THREADS) big_offsets_kernel(const uint32_t* __restrict__ sorted_keys,
                                                                   uint32_t n, BucketParams p,
                                                                   uint32_t* __restrict__ starts) {
  __shared__ uint32_t s_split[big_identifier_smem_words<KIND>()];
  prepare_big_identifier<KIND>(s_split, p);
  __syncthreads();
  const uint32_t B = p.num_buckets;
  const uint32_t stride = gridDim.x * HIST_THREADS;
  for (uint32_t i = blockIdx.x * HIST_THREADS + threadIdx.x; i < n; i += stride) {
    const uint32_t cur = big_bucket_id<KIND>(sorted_keys[i], p, s_split);
    const uint32_t first = i == 0 ? 0u : big_bucket_id<KIND>(sorted_keys[i - 1], p, s_split) + 1u;
    for (uint32_t b = first; b <= cur; ++b) starts[b] = i;
    if (i == n - 1)
      for (uint32_t b = cur + 1; b < B; ++b) starts[b] = n;
  }
}

}  // namespace gms
