// Device-wide histogram over B <= 256 bins with any bucket identifier.
// Generalises the reference's multisplit2_histogram_even_* / _range_* kernels
// (src/kernels/histogram/multisplit2_histograms.cuh:36-699): per-block counts
// (ballots for B <= 32, shared atomics above), then one global atomicAdd per
// bin per block into the caller-zeroed int histogram.  Unlike the reference,
// any n is accepted (its kernels have no tail guard).
#pragma once

#include "multisplit_kernels.cuh"

namespace gms {

constexpr int HIST_WARPS = 8;
constexpr int HIST_THREADS = HIST_WARPS * 32;
constexpr int HIST_IPT = 16;
constexpr uint32_t HIST_CHUNK = HIST_THREADS * HIST_IPT;

// Persistent grid; block-strided over chunks of HIST_CHUNK keys.
template <int LOGB, int KIND>
__global__ void __launch_bounds__(HIST_THREADS) histogram_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                                 int32_t* __restrict__ hist, BucketParams bp) {
  constexpr uint32_t B = 1u << LOGB;
  __shared__ uint32_t s_hist[LOGB <= 5 ? HIST_WARPS * 32 : B];
  __shared__ uint32_t s_split[LOGB <= 5 ? 32 : B];
  const uint32_t tid = threadIdx.x;

  load_splitters<KIND, LOGB>(s_split, bp);
  if constexpr (LOGB > 5) {
    for (uint32_t b = tid; b < B; b += HIST_THREADS) s_hist[b] = 0u;
  }
  __syncthreads();

  const bool vec_ok = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0;
  const Identifier<KIND, LOGB> ident{bp, s_split};
  KeyCounter<LOGB, KIND> counter(ident, s_hist);
  const uint32_t num_chunks = (n + HIST_CHUNK - 1) / HIST_CHUNK;
  for (uint32_t c = blockIdx.x; c < num_chunks; c += gridDim.x) {
    const uint32_t base = c * HIST_CHUNK;
    count_tile<HIST_THREADS, HIST_IPT>(keys, base, min(HIST_CHUNK, n - base), vec_ok, counter);
  }

  if constexpr (LOGB <= 5) {
    const uint32_t lane = tid & 31u, warp = tid >> 5;
    if (lane < B) s_hist[warp * 32 + lane] = counter.lane_cnt;
    __syncthreads();
    if (tid < B) {
      uint32_t total = 0;
#pragma unroll
      for (int w = 0; w < HIST_WARPS; ++w) total += s_hist[w * 32 + tid];
      if (total) atomicAdd(&hist[tid], int32_t(total));
    }
  } else {
    __syncthreads();
    for (uint32_t b = tid; b < B; b += HIST_THREADS) {
      const uint32_t total = s_hist[b];
      if (total) atomicAdd(&hist[b], int32_t(total));
    }
  }
}

}  // namespace gms
