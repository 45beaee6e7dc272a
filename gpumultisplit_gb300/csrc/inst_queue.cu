// The batch queue kernel (batch_queue.cuh) and its launcher: one persistent
// launch, as many blocks as fit on the device.
#include "batch_queue.cuh"
#include "ms_dispatch.cuh"

namespace gms {

static_assert(SCAN_CHUNK == kScanChunk, "host and device agree on the scan chunk");

cudaError_t run_batch_queue(const BatchQueueLaunch& c) {
  if (c.num_items == 0) return cudaSuccess;
  static std::atomic<uint64_t> smem_done{0};
  static std::atomic<int> per_sm{0};
  auto kern = batch_queue_kernel;
  cudaError_t e = ensure_smem_limit(kern, kQueueSmemBytes, smem_done);
  if (e != cudaSuccess) return e;
  const uint32_t grid = persistent_grid(kern, QUEUE_WARPS * 32, c.num_items, per_sm, kQueueSmemBytes);
  const QueueState st{c.state, c.state + 1, c.state + 1 + c.num_segs, c.status};
  kern<<<grid, QUEUE_WARPS * 32, kQueueSmemBytes, c.stream>>>(c.qsegs, c.items, c.num_items, c.matrix, c.byte_area,
                                                               st, c.hdr);
  return cudaGetLastError();
}

}  // namespace gms
