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

// Persistent grid; block-strided over chunks of HIST_CHUNK keys.
template <int LOGB, class P>
__global__ void __launch_bounds__(HIST_THREADS) histogram_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                                 int32_t* __restrict__ hist, typename P::Params bp) {
  using Counter = KeyCounter<LOGB, typename P::Id>;
  __shared__ uint32_t s_hist[Counter::smem_words(HIST_WARPS)];
  __shared__ uint32_t s_split[P::SMEM_WORDS];
  P::prepare(s_split, bp);
  Counter counter(P::make(bp, s_split), s_hist);
  counter.clear_shared();
  __syncthreads();
  count_tiles<HIST_THREADS, HIST_IPT>(keys, n, blockIdx.x, gridDim.x, counter, [](uint32_t) {});
  const uint32_t total = counter.block_total();
  if (threadIdx.x < (1u << LOGB) && total) atomicAdd(&hist[threadIdx.x], int32_t(total));
}

// Histogram pass of the one-pass multisplit: global bucket counts into
// hist[0..B) (zeroed by the caller), then the last block to finish (counted in
// hdr->done, zeroed by the caller) writes their exclusive scan, the global
// start of every bucket, into starts[0..B).
template <int LOGB, class P>
__global__ void __launch_bounds__(HIST_THREADS) onepass_histogram_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                                         uint32_t* hist, uint32_t* __restrict__ starts,
                                                                         ScratchHeader* hdr, typename P::Params bp) {
  using Counter = KeyCounter<LOGB, typename P::Id>;
  constexpr uint32_t B = 1u << LOGB;
  __shared__ uint32_t s_hist[Counter::smem_words(HIST_WARPS)];
  __shared__ uint32_t s_split[P::SMEM_WORDS];
  __shared__ uint32_t s_warp[HIST_WARPS];
  __shared__ uint32_t s_last;
  const uint32_t tid = threadIdx.x;
  P::prepare(s_split, bp);
  Counter counter(P::make(bp, s_split), s_hist);
  counter.clear_shared();
  __syncthreads();
  count_tiles<HIST_THREADS, HIST_IPT>(keys, n, blockIdx.x, gridDim.x, counter, [](uint32_t) {});
  const uint32_t total = counter.block_total();
  if (tid < B && total) atomicAdd(&hist[tid], total);
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = atomicAdd(&hdr->done, 1u) == gridDim.x - 1u ? 1u : 0u;
  __syncthreads();
  if (s_last == 0u) return;
  __threadfence();
  // Exclusive scan of the B totals (warp scans, then the warp totals).
  const uint32_t lane = tid & 31u, warp = tid >> 5;
  const uint32_t v = tid < B ? ld_relaxed_u32(&hist[tid]) : 0u;
  uint32_t incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t t = __shfl_up_sync(~0u, incl, d);
    if (lane >= uint32_t(d)) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  uint32_t before = 0;
  for (uint32_t w = 0; w < warp; ++w) before += s_warp[w];
  if (tid < B) starts[tid] = before + incl - v;
}

}  // namespace gms
