// Batched multisplit kernels: many independent multisplits ("segments") of
// uneven sizes in one launch per stage and segment class.  A class is every
// segment with the same identifier kind, bucket count and key/value shape; a
// device-side tile map sends block t of a class to (segment, tile) and the
// segment descriptor table supplies that segment's arrays and identifier.
//
// All segments' count matrices are laid end to end and scanned as one array,
// so a scanned offset is the segment's start within its scan group (`base`,
// the sum of the n of earlier segments in the group) plus the offset inside
// the segment; the postscan subtracts `base`.
#pragma once

#include "multisplit_kernels.cuh"

namespace gms {

struct SegDesc {
  const uint32_t* kin;
  const uint32_t* vin;  // null for key-only segments
  uint32_t* kout;
  uint32_t* vout;
  uint32_t n;
  uint32_t num_tiles;
  uint32_t matrix_off;  // first count of this segment in the batch count matrix
  uint32_t base;        // start of this segment in its scan group
  BucketParams bp;
};

// Persistent prescan over the tiles of one class.  Tiles of one segment are
// consecutive in the map, so the identifier is re-prepared only when the
// segment changes (all threads of the block see the same tile).
template <class C, int KIND>
__global__ void __launch_bounds__(C::THREADS) batch_prescan_kernel(const SegDesc* __restrict__ segs,
                                                                   const uint2* __restrict__ tile_map,
                                                                   uint32_t class_tiles,
                                                                   uint32_t* __restrict__ matrix) {
  using P = DescPolicy<KIND, C::LOGB>;
  using Counter = KeyCounter<C::LOGB, typename P::Id>;
  __shared__ uint32_t s_hist[Counter::smem_words(C::WARPS)];
  __shared__ uint32_t s_split[P::SMEM_WORDS];
  const uint32_t tid = threadIdx.x;

  SegDesc sd{};
  uint32_t cur = ~0u;
  Counter counter(P::make(BucketParams{}, s_split), s_hist);
  counter.clear_shared();
  __syncthreads();
  for (uint32_t t = blockIdx.x; t < class_tiles; t += gridDim.x) {
    const uint2 m = tile_map[t];
    if (m.x != cur) {
      cur = m.x;
      sd = segs[cur];
      P::prepare(s_split, sd.bp);
      if constexpr (P::USES_SMEM) __syncthreads();
      counter.ident = P::make(sd.bp, s_split);
    }
    const uint32_t base = m.y * C::TILE;
    const uint32_t cnt = min(C::TILE, sd.n - base);
    if (cnt == C::TILE && (reinterpret_cast<uintptr_t>(sd.kin) & 15u) == 0) {
      uint4 v[C::IPT / 4];
      load_tile_v4<C::THREADS, C::IPT>(sd.kin, base, v);
      count_v4<C::THREADS, C::IPT>(v, counter);
    } else {
#pragma unroll 4
      for (int k = 0; k < C::IPT; ++k) {
        const uint32_t i = uint32_t(k) * C::THREADS + tid;
        const bool valid = i < cnt;
        counter.add(valid ? sd.kin[base + i] : 0u, valid);
      }
    }
    const uint32_t total = counter.block_total();
    if (tid < C::B) matrix[sd.matrix_off + tid * sd.num_tiles + m.y] = total;
  }
}

// One block per tile of one class.
template <class C, int KIND>
__global__ void __launch_bounds__(C::THREADS, (PostLayout<C, DescPolicy<KIND, C::LOGB>>::MIN_BLOCKS))
    batch_postscan_kernel(const SegDesc* __restrict__ segs, const uint2* __restrict__ tile_map,
                          const uint32_t* __restrict__ matrix, ScratchHeader* hdr) {
  extern __shared__ __align__(128) unsigned char smem[];
  const uint2 m = tile_map[blockIdx.x];
  const SegDesc& sd = segs[m.x];
  const TileJob<BucketParams> job{sd.kin, sd.vin,  sd.kout, sd.vout, sd.n,  sd.num_tiles,
                                  m.y,    matrix + sd.matrix_off, sd.base, ~0u, sd.bp, m.x};
  postscan_job<C, DescPolicy<KIND, C::LOGB>>(job, hdr, smem);
}

// Persistent form for identifiers with a shared area (RANGE): block b runs a
// contiguous range of the class's tile map and prepares the identifier again
// only when the segment changes.  The prefetch pulls the next tile of the same
// segment into L2.
template <class C, int KIND>
__global__ void __launch_bounds__(C::THREADS, (PostLayout<C, DescPolicy<KIND, C::LOGB>>::MIN_BLOCKS))
    batch_postscan_persistent_kernel(const SegDesc* __restrict__ segs, const uint2* __restrict__ tile_map,
                                     uint32_t class_tiles, const uint32_t* __restrict__ matrix, ScratchHeader* hdr) {
  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t per = (class_tiles + gridDim.x - 1) / gridDim.x;
  const uint32_t first = blockIdx.x * per;
  const uint32_t last = min(first + per, class_tiles);
  postscan_run<C, DescPolicy<KIND, C::LOGB>>(
      first, last, 1u,
      [&](uint32_t t, uint32_t next) {
        const uint2 m = tile_map[t];
        const SegDesc& sd = segs[m.x];
        const uint32_t pf = (next != ~0u && tile_map[next].x == m.x) ? tile_map[next].y : ~0u;
        return TileJob<BucketParams>{sd.kin, sd.vin, sd.kout, sd.vout, sd.n, sd.num_tiles, m.y,
                                     matrix + sd.matrix_off, sd.base, pf, sd.bp, m.x};
      },
      hdr, smem);
}

}  // namespace gms
