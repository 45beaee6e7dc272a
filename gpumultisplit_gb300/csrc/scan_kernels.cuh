// Single-pass exclusive prefix sum with decoupled look-back, in place over a
// uint32 array (the bucket-count matrix), one block per chunk (scan_chunk.cuh).
// Replaces the reference's cub::DeviceScan::ExclusiveSum call
// (src/api/multisplit.cuh:141,258).
//
// Chunks are claimed through an atomic ticket, so a chunk only ever waits on
// chunks that were claimed (and are therefore running) before it.
#pragma once

#include "scan_chunk.cuh"

namespace gms {

// One chunk per block, claimed through the header's ticket counter.
__global__ void __launch_bounds__(SCAN_THREADS) scan_kernel(uint32_t* __restrict__ data, uint32_t m,
                                                            uint64_t* __restrict__ status, ScratchHeader* hdr) {
  __shared__ uint32_t s_chunk;
  griddep_wait();  // launched while the prescan finishes: the counts and the reset ticket are in place
  griddep_launch_dependents();
  if (threadIdx.x == 0) s_chunk = atomicAdd(&hdr->ticket, 1u);
  __syncthreads();
  const uint32_t chunk = s_chunk;
  // Tickets run from 0 when the prescan reset the counter; a block that draws
  // one past the last chunk (a counter not reset) has nothing to scan.
  if (chunk >= gridDim.x) return;
  scan_chunk(data, m, chunk, status, hdr);
}

}  // namespace gms
