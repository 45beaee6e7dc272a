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

// ------------------------------------------------ one warp per segment
// Segments of at most WARP_SEG_MAX keys are multisplit by one warp each, in
// one launch per class and without a count matrix or a scan: the warp ranks
// its keys as the postscan ranks them within a warp (slot j, lane l holds key
// 32j + l, so ranks follow input order), scans its bucket counts and stores
// every key at its final position.  Such a segment's output spans at most
// WARP_SEG_MAX words, whose sectors merge in L2.  Its bucket starts are also
// written to its 2^LOGB count-matrix entries (as one tile), outside every scan
// group, so they read like the scanned offsets of a tiled segment.
constexpr uint32_t WARP_SEG_SLOTS = 16;
constexpr uint32_t WARP_SEG_MAX = 32 * WARP_SEG_SLOTS;
constexpr int WARP_SEG_WARPS = 4;  // warps per block

// Bucket of a key for the warp path: the descriptor identifiers without a
// shared area; RANGE searches the segment's splitters through the read-only
// cache (segments of one block may carry different splitters).
template <int KIND, int LOGB>
__device__ __forceinline__ uint32_t warp_seg_bucket(uint32_t key, const BucketParams& bp) {
  if constexpr (KIND == KIND_RANGE) {
    uint32_t lo = 0, hi = bp.num_buckets;
    while (lo < hi) {  // upper_bound
      const uint32_t mid = (lo + hi) >> 1;
      if (__ldg(bp.splitters + mid) <= key)
        lo = mid + 1;
      else
        hi = mid;
    }
    return lo == 0u ? bp.num_buckets - 1u : lo - 1u;
  } else {
    return Identifier<KIND, LOGB>{bp, nullptr}(key);
  }
}

template <int KIND, int LOGB, bool KV>
__global__ void __launch_bounds__(WARP_SEG_WARPS * 32) batch_warp_kernel(const SegDesc* __restrict__ segs,
                                                                         const uint32_t* __restrict__ seg_ids,
                                                                         uint32_t count, uint32_t* __restrict__ matrix) {
  constexpr uint32_t B = 1u << LOGB;
  constexpr uint32_t S = WARP_SEG_SLOTS;
  __shared__ uint16_t s_table[WARP_SEG_WARPS][LOGB > 5 ? B : 1];  // per-warp bucket counts, then starts
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t w = blockIdx.x * WARP_SEG_WARPS + warp;
  if (w >= count) return;  // warp-uniform
  const SegDesc sd = segs[seg_ids[w]];
  const uint32_t lt = lanemask_lt();

  uint32_t key[S], val[KV ? S : 1], packed[S];  // packed: bucket << 16 | rank within bucket
#pragma unroll
  for (uint32_t j = 0; j < S; ++j) {
    const uint32_t i = j * 32u + lane;
    key[j] = i < sd.n ? sd.kin[i] : 0u;
    if constexpr (KV) val[j] = i < sd.n ? sd.vin[i] : 0u;
  }
  uint16_t* table = s_table[warp];
  if constexpr (LOGB > 5) {
    for (uint32_t b = lane; b < B; b += 32) table[b] = 0;
    __syncwarp();
  }
  uint32_t my_cnt = 0;  // LOGB <= 5: count of bucket `lane`
  uint32_t xm[LOGB <= 5 ? LOGB : 1];
  if constexpr (LOGB <= 5) {
#pragma unroll
    for (int i = 0; i < LOGB; ++i) xm[i] = ((lane >> i) & 1u) ? 0u : ~0u;
  }
#pragma unroll
  for (uint32_t j = 0; j < S; ++j) {
    if (j * 32u >= sd.n) break;  // warp-uniform
    const bool valid = j * 32u + lane < sd.n;
    const uint32_t b = warp_seg_bucket<KIND, LOGB>(key[j], sd.bp);
    const uint32_t vmask = __ballot_sync(~0u, valid);
    if constexpr (LOGB <= 5) {
      uint32_t m = vmask;
#pragma unroll
      for (int i = 0; i < LOGB; ++i) m &= __ballot_sync(~0u, (b >> i) & 1u) ^ xm[i];
      const uint32_t peers = __shfl_sync(~0u, m, b);
      const uint32_t before = __shfl_sync(~0u, my_cnt, b);
      packed[j] = (b << 16) | (before + __popc(peers & lt));
      my_cnt += __popc(m);
    } else {
      const uint32_t peers = peers_by_ballot<LOGB>(b) & vmask;
      const uint32_t rank = __popc(peers & lt);
      const uint32_t before = valid ? table[b] : 0u;
      __syncwarp();
      if (valid && rank == 0) table[b] = uint16_t(before + __popc(peers));
      __syncwarp();
      packed[j] = (b << 16) | (before + rank);
    }
  }
  // Bucket starts inside the segment: an exclusive scan of the counts.
  uint32_t start = 0;  // LOGB <= 5: start of bucket `lane`
  if constexpr (LOGB <= 5) {
    uint32_t incl = lane < B ? my_cnt : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(~0u, incl, d);
      if (lane >= uint32_t(d)) incl += t;
    }
    start = incl - (lane < B ? my_cnt : 0u);
    if (lane < B) matrix[sd.matrix_off + lane] = sd.base + start;
  } else {
    constexpr uint32_t PER = B / 32;  // consecutive buckets per lane
    uint32_t local = 0;
#pragma unroll
    for (uint32_t k = 0; k < PER; ++k) local += table[lane * PER + k];
    uint32_t incl = local;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(~0u, incl, d);
      if (lane >= uint32_t(d)) incl += t;
    }
    uint32_t run = incl - local;
    __syncwarp();
#pragma unroll
    for (uint32_t k = 0; k < PER; ++k) {
      const uint32_t c = table[lane * PER + k];
      table[lane * PER + k] = uint16_t(run);
      matrix[sd.matrix_off + lane * PER + k] = sd.base + run;
      run += c;
    }
    __syncwarp();
  }
#pragma unroll
  for (uint32_t j = 0; j < S; ++j) {
    if (j * 32u >= sd.n) break;
    const uint32_t b = packed[j] >> 16;
    uint32_t base;
    if constexpr (LOGB <= 5)
      base = __shfl_sync(~0u, start, b);
    else
      base = table[b];
    if (j * 32u + lane < sd.n) {
      const uint32_t pos = base + (packed[j] & 0xFFFFu);
      sd.kout[pos] = key[j];
      if constexpr (KV) sd.vout[pos] = val[j];
    }
  }
}

// ------------------------------------------------ the batch queue
// Records of the one-launch schedule (batch_queue.cuh runs them).
constexpr int QUEUE_WARPS = 8;
constexpr int QUEUE_IPT = 16;
constexpr uint32_t QUEUE_TILE = QUEUE_WARPS * 32u * QUEUE_IPT;
constexpr uint32_t QUEUE_PRE_TILES = 4;  // tiles per PRE item
constexpr int QUEUE_MIN_BLOCKS = 4;                  // 64 registers: the key-value postscan's budget

enum QueueItemType : uint32_t { QITEM_PRE = 0, QITEM_SCAN = 1, QITEM_POST = 2 };
constexpr uint32_t QITEM_SHIFT = 28;

// A segment as the queue sees it.  d uses the queue's layout: num_tiles of
// QUEUE_TILE keys, matrix_off 16-byte aligned, base 0, bytes_off for every
// identifier but delta.
struct QSeg {
  SegDesc d;
  uint32_t meta;        // kind | logb << 8 | kv << 16
  uint32_t chunks;      // scan chunks of its count matrix
  uint32_t status_off;  // first of its chunks' look-back words
  uint32_t pad;
};

// Device state of one run, zeroed before the launch.
struct QueueState {
  uint32_t* ticket;     // next item
  uint32_t* pre_done;   // per segment: tiles counted
  uint32_t* scan_done;  // per segment: chunks scanned
  uint64_t* status;     // look-back words of every segment's chunks
};

}  // namespace gms
