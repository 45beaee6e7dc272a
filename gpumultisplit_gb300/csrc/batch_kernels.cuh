// Batched multisplit kernels: many independent multisplits ("segments") of
// uneven sizes in one launch per stage and segment class.  A class is every
// segment with the same identifier kind, bucket count and key/value shape; a
// device-side tile map sends block t of a class to (segment, tile) and the
// segment descriptor table supplies that segment's arrays and identifier.
//
// All segments' count matrices are laid end to end and scanned as one array,
// so a scanned offset is the segment's start within its scan group (`base`,
// the sum of the n of earlier segments in the group) plus the offset inside
// the segment; the postscan subtracts `base`.  Segments whose identifier is
// costly (range, div, even-float) get a byte per key in the batch's byte
// area: the prescan stores each key's bucket there and the postscan reads it.
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
  uint64_t bytes_off;   // costly identifiers: this segment's bucket bytes in the batch's byte area
};

// Persistent prescan over the tiles of one class.  Tiles of one segment are
// consecutive in the map, so the identifier is re-prepared only when the
// segment changes (all threads of the block see the same tile).
template <class C, int KIND>
__global__ void __launch_bounds__(C::THREADS) batch_prescan_kernel(const SegDesc* __restrict__ segs,
                                                                   const uint2* __restrict__ tile_map,
                                                                   uint32_t class_tiles,
                                                                   uint32_t* __restrict__ matrix,
                                                                   uint8_t* __restrict__ byte_area) {
  using P = DescPolicy<KIND, C::LOGB>;
  constexpr bool BYTES = !P::CHEAP;
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
    uint8_t* bytes = BYTES ? byte_area + sd.bytes_off + base : nullptr;
    if (cnt == C::TILE && (reinterpret_cast<uintptr_t>(sd.kin) & 15u) == 0) {
      uint4 v[C::IPT / 4];
      load_tile_v4<C::THREADS, C::IPT>(sd.kin, base, v);
      count_v4<C::THREADS, C::IPT, BYTES>(v, counter, bytes);
    } else {
#pragma unroll 4
      for (int k = 0; k < C::IPT; ++k) {
        const uint32_t i = uint32_t(k) * C::THREADS + tid;
        const bool valid = i < cnt;
        const uint32_t b = counter.ident(valid ? sd.kin[base + i] : 0u);
        counter.add_bucket(b, valid);
        if constexpr (BYTES) {
          if (valid) bytes[i] = uint8_t(b);
        }
      }
    }
    const uint32_t total = counter.block_total();
    if (tid < C::B) matrix[sd.matrix_off + tid * sd.num_tiles + m.y] = total;
  }
}

// One block per tile of one class; costly identifiers read the buckets the
// prescan stored.
template <class C, int KIND>
__global__ void __launch_bounds__(C::THREADS,
                                  (PostLayout<C, DescPolicy<KIND, C::LOGB>, !DescPolicy<KIND, C::LOGB>::CHEAP>::MIN_BLOCKS))
    batch_postscan_kernel(const SegDesc* __restrict__ segs, const uint2* __restrict__ tile_map,
                          const uint32_t* __restrict__ matrix, ScratchHeader* hdr, const uint8_t* byte_area) {
  using P = DescPolicy<KIND, C::LOGB>;
  extern __shared__ __align__(128) unsigned char smem[];
  const uint2 m = tile_map[blockIdx.x];
  const SegDesc& sd = segs[m.x];
  const TileJob<BucketParams> job{sd.kin, sd.vin,  sd.kout, sd.vout, sd.n,  sd.num_tiles,
                                  m.y,    matrix + sd.matrix_off, sd.base, ~0u, sd.bp, m.x,
                                  P::CHEAP ? nullptr : byte_area + sd.bytes_off};
  postscan_job<C, P, true, !P::CHEAP>(job, hdr, smem);
}

}  // namespace gms
