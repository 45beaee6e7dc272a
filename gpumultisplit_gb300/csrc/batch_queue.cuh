// The batched multisplit as one persistent launch over a device-side work
// list.  Every segment of a batch becomes three kinds of items:
//   PRE   counts up to QUEUE_PRE_TILES tiles of the segment (its count-matrix
//         columns) and, for every identifier but delta, stores each key's
//         bucket as one byte;
//   SCAN  scans one chunk of the segment's count matrix with decoupled
//         look-back over the segment's earlier chunks, once every PRE item of
//         the segment has finished;
//   POST  ranks, reorders and scatters one tile, once the segment's scan is
//         complete.
// Blocks claim items through one ticket counter, in the order of the list the
// host built: a segment's PRE items, then its SCAN items, and its POST items a
// fixed number of PRE tiles later.  An item only ever waits on items earlier
// in the list, which were claimed by running blocks, so the launch needs no
// co-residency and cannot deadlock; every wait is bounded by the call's wait
// limit and records DEV_ERR_LOOKBACK_TIMEOUT when it runs out.  Because the
// POST items of a segment follow its PRE items closely, the segment's keys
// (and bucket bytes) are usually still in L2 when the postscan stages them.
//
// Each segment's count matrix is scanned on its own, so its scanned offsets
// start at 0 (no bias).  Every tile is 4096 keys (8 warps x 16 keys).
#pragma once

#include "batch_kernels.cuh"
#include "scan_chunk.cuh"

namespace gms {

static_assert(SCAN_THREADS == QUEUE_WARPS * 32, "a SCAN item runs on the queue's blocks");

template <int LOGB, bool KV>
using QueueCfg = TileCfg<LOGB, QUEUE_WARPS, QUEUE_IPT, KV>;

// Thread 0 waits until *ctr >= target (acquire), bounded by the call's wait
// limit; the block then proceeds either way.  The proxy fence lets bulk copies
// issued afterwards by thread 0 see what the awaited blocks wrote.
__device__ __forceinline__ void queue_wait(const uint32_t* ctr, uint32_t target, ScratchHeader* hdr) {
  if (threadIdx.x == 0) {
    if (ld_acquire_u32(ctr) < target) {
      const uint64_t limit = error_recorded(hdr) ? 0ull : wait_limit_ns(hdr);
      const uint64_t t0 = global_timer_ns();
      while (ld_acquire_u32(ctr) < target) {
        if (global_timer_ns() - t0 > limit) {
          record_error(hdr, DEV_ERR_LOOKBACK_TIMEOUT);
          break;
        }
        __nanosleep(100);
      }
    }
    fence_proxy_async_global();
  }
  __syncthreads();
}

// Every thread's global writes of this item become visible, then thread 0
// adds `v` to the counter other items wait on.
__device__ __forceinline__ void queue_publish(uint32_t* ctr, uint32_t v) {
  __threadfence();
  fence_proxy_async_global();
  __syncthreads();
  if (threadIdx.x == 0) red_release_add_u32(ctr, v);
}

// PRE: tiles [t0, t1) of the segment.  Their counts are gathered in shared
// memory and written bucket by bucket, (t1 - t0) consecutive words each.
template <int KIND, int LOGB>
__device__ __forceinline__ void queue_pre(const QSeg* q, uint32_t item, uint32_t* __restrict__ matrix,
                                       uint8_t* __restrict__ byte_area) {
  extern __shared__ __align__(128) unsigned char smem[];
  const SegDesc sd = q->d;
  const uint32_t t0 = item * QUEUE_PRE_TILES, t1 = min(t0 + QUEUE_PRE_TILES, sd.num_tiles);
  using C = QueueCfg<LOGB, false>;
  using P = DescPolicy<KIND, LOGB>;
  using Counter = KeyCounter<LOGB, typename P::Id>;
  constexpr bool BYTES = KIND != KIND_DELTA;
  constexpr uint32_t G = QUEUE_PRE_TILES;
  uint32_t* s_hist = reinterpret_cast<uint32_t*>(smem);
  uint32_t* s_cnt = s_hist + Counter::smem_words(C::WARPS);
  uint32_t* s_split = s_cnt + C::B * G;
  const uint32_t tid = threadIdx.x;
  P::prepare(s_split, sd.bp);
  Counter counter(P::make(sd.bp, s_split), s_hist);
  counter.clear_shared();
  __syncthreads();
  auto done = [&](uint32_t tile) {
    const uint32_t total = counter.block_total();
    if (tid < C::B) s_cnt[tid * G + (tile - t0)] = total;
  };
  uint8_t* bytes = BYTES ? byte_area + sd.bytes_off : nullptr;
  // One tile's keys in registers at a time (the other resident blocks keep
  // loads in flight); full tiles as 16-byte vectors.
  const bool vec = (reinterpret_cast<uintptr_t>(sd.kin) & 15u) == 0;
  for (uint32_t tile = t0; tile < t1; ++tile) {
    const uint32_t base = tile * C::TILE;
    const uint32_t cnt = min(C::TILE, sd.n - base);
    if (vec && cnt == C::TILE) {
      uint4 v[C::IPT / 4];
      load_tile_v4<C::THREADS, C::IPT>(sd.kin, base, v);
      count_v4<C::THREADS, C::IPT, BYTES>(v, counter, BYTES ? bytes + base : nullptr);
    } else {
#pragma unroll 4
      for (int k = 0; k < C::IPT; ++k) {
        const uint32_t i = uint32_t(k) * C::THREADS + tid;
        const bool valid = i < cnt;
        const uint32_t b = counter.ident(valid ? sd.kin[base + i] : 0u);
        counter.add_bucket(b, valid);
        if constexpr (BYTES) {
          if (valid) bytes[base + i] = uint8_t(b);
        }
      }
    }
    done(tile);
  }
  __syncthreads();
  const uint32_t k = t1 - t0;
  for (uint32_t i = tid; i < C::B * G; i += C::THREADS) {
    const uint32_t b = i / G, j = i % G;
    if (j < k) matrix[sd.matrix_off + b * sd.num_tiles + t0 + j] = s_cnt[i];
  }
}

template <int KIND>
__device__ __forceinline__ void queue_pre_kind(int logb, const QSeg* q, uint32_t item, uint32_t* matrix,
                                               uint8_t* byte_area) {
  switch (logb) {
    case 1: queue_pre<KIND, 1>(q, item, matrix, byte_area); break;
    case 2: queue_pre<KIND, 2>(q, item, matrix, byte_area); break;
    case 3: queue_pre<KIND, 3>(q, item, matrix, byte_area); break;
    case 4: queue_pre<KIND, 4>(q, item, matrix, byte_area); break;
    case 5: queue_pre<KIND, 5>(q, item, matrix, byte_area); break;
    case 6: queue_pre<KIND, 6>(q, item, matrix, byte_area); break;
    case 7: queue_pre<KIND, 7>(q, item, matrix, byte_area); break;
    default: queue_pre<KIND, 8>(q, item, matrix, byte_area); break;
  }
}

// Offsets of a POST tile: its column of the segment's scanned count matrix,
// read through L2 (SCAN items of other blocks wrote it during this launch).
// With `done` set, the block first waits for the segment's scan: the tile's
// bulk copy of keys and values is then already in flight.
struct QueueOffsets {
  const uint32_t* done;  // scan chunks finished (null: the caller waited)
  uint32_t chunks;
  ScratchHeader* hdr;
  template <class Job>
  __device__ __forceinline__ GivenOffset operator()(const Job& job, uint32_t tid, uint32_t num_buckets) const {
    if (done != nullptr) queue_wait(done, chunks, hdr);
    return GivenOffset{tid < num_buckets ? __ldcg(job.offsets + tid * job.num_tiles + job.tile) : 0u};
  }
};

// POST: one tile.  Delta segments evaluate their identifier; every other kind
// reads the bucket bytes its PRE items stored (the layout of any costly kind
// serves, since the identifier is never evaluated).  Those bytes are staged by
// the same bulk copy as the keys, so such a tile waits for its segment's scan
// (hence for its PRE items) before the copy; a delta tile waits while its
// copy is in flight.
template <int LOGB, bool KV, bool GIVEN>
__device__ __forceinline__ void queue_post_t(const QSeg* q, uint32_t tile, const uint32_t* matrix,
                                             const uint8_t* byte_area, const uint32_t* scan_done,
                                             ScratchHeader* hdr) {
  extern __shared__ __align__(128) unsigned char smem[];
  if constexpr (GIVEN) queue_wait(scan_done, q->chunks, hdr);
  const SegDesc sd = q->d;
  using C = QueueCfg<LOGB, KV>;
  using P = DescPolicy<GIVEN ? KIND_RANGE : KIND_DELTA, LOGB>;
  using L = PostLayout<C, P, GIVEN>;
  const TileJob<BucketParams> job{sd.kin, sd.vin, sd.kout, sd.vout, sd.n, sd.num_tiles, tile,
                                  matrix + sd.matrix_off, 0u, ~0u, sd.bp, 0u,
                                  GIVEN ? byte_area + sd.bytes_off : nullptr};
  bool bar_live = false;
  const QueueOffsets offs{GIVEN ? nullptr : scan_done, q->chunks, hdr};
  postscan_job<C, P, true, GIVEN, QueueOffsets, true>(job, hdr, smem, &bar_live, offs);
  __syncthreads();
  if (bar_live && threadIdx.x == 0) mbar_inval(reinterpret_cast<uint64_t*>(smem + L::OFF_BAR));
}

template <int LOGB>
__device__ __forceinline__ void queue_post_l(bool kv, bool given, const QSeg* q, uint32_t tile,
                                             const uint32_t* matrix, const uint8_t* byte_area,
                                             const uint32_t* scan_done, ScratchHeader* hdr) {
  if (kv) {
    if (given) queue_post_t<LOGB, true, true>(q, tile, matrix, byte_area, scan_done, hdr);
    else queue_post_t<LOGB, true, false>(q, tile, matrix, byte_area, scan_done, hdr);
  } else {
    if (given) queue_post_t<LOGB, false, true>(q, tile, matrix, byte_area, scan_done, hdr);
    else queue_post_t<LOGB, false, false>(q, tile, matrix, byte_area, scan_done, hdr);
  }
}

// Dynamic shared memory of the queue kernel: the largest postscan layout (the
// PRE items' histograms, tile counts and identifier areas are smaller).
template <int LOGB>
constexpr size_t queue_smem_l() {
  using PG = DescPolicy<KIND_RANGE, LOGB>;
  using PD = DescPolicy<KIND_DELTA, LOGB>;
  size_t m = PostLayout<QueueCfg<LOGB, true>, PG, true>::BYTES;
  m = m > PostLayout<QueueCfg<LOGB, false>, PG, true>::BYTES ? m : PostLayout<QueueCfg<LOGB, false>, PG, true>::BYTES;
  m = m > PostLayout<QueueCfg<LOGB, true>, PD, false>::BYTES ? m : PostLayout<QueueCfg<LOGB, true>, PD, false>::BYTES;
  m = m > PostLayout<QueueCfg<LOGB, false>, PD, false>::BYTES ? m : PostLayout<QueueCfg<LOGB, false>, PD, false>::BYTES;
  constexpr size_t pre = 4u * (KeyCounter<LOGB, Identifier<KIND_RANGE, LOGB>>::smem_words(QUEUE_WARPS) +
                               (1u << LOGB) * QUEUE_PRE_TILES + identifier_smem_words<KIND_RANGE, LOGB>());
  return m > pre ? m : pre;
}

constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t kQueueSmemBytes =
    cmax(cmax(cmax(queue_smem_l<1>(), queue_smem_l<2>()), cmax(queue_smem_l<3>(), queue_smem_l<4>())),
         cmax(cmax(queue_smem_l<5>(), queue_smem_l<6>()), cmax(queue_smem_l<7>(), queue_smem_l<8>())));

__global__ void __launch_bounds__(QUEUE_WARPS * 32, QUEUE_MIN_BLOCKS)
    batch_queue_kernel(const QSeg* __restrict__ segs, const uint2* __restrict__ items, uint32_t num_items,
                       uint32_t* matrix, uint8_t* byte_area, QueueState st, ScratchHeader* hdr) {
  __shared__ uint32_t s_item, s_next;
  __shared__ uint2 s_it, s_next_it;
  const uint32_t tid = threadIdx.x;
  if (tid == 0) {
    const uint32_t t = atomicAdd(st.ticket, 1u);
    s_item = t;
    s_it = t < num_items ? __ldg(items + t) : make_uint2(0u, 0u);
  }
  __syncthreads();
  while (true) {
    const uint32_t i = s_item;
    if (i >= num_items) break;  // block-uniform
    const uint2 it = s_it;
    // Warp 1 claims the next item while this one runs, so the ticket's and
    // the item's round trips overlap this item's work.
    if (tid == 32) {
      const uint32_t t = atomicAdd(st.ticket, 1u);
      const uint2 nx = t < num_items ? __ldg(items + t) : make_uint2(0u, 0u);
      s_next = t;
      s_next_it = nx;
      // A POST item next: pull its tile's keys and values toward L2 now, so
      // its bulk copy finds them there.
      if (t < num_items && (nx.y >> QITEM_SHIFT) == QITEM_POST) {
        const SegDesc& nd = segs[nx.x].d;
        const uint32_t tile = nx.y & ((1u << QITEM_SHIFT) - 1u);
        if (tile + 1 < nd.num_tiles && ((reinterpret_cast<uintptr_t>(nd.kin) | reinterpret_cast<uintptr_t>(nd.vin)) & 15u) == 0) {
          bulk_prefetch_l2(nd.kin + size_t(tile) * QUEUE_TILE, QUEUE_TILE * 4u);
          if (nd.vin != nullptr) bulk_prefetch_l2(nd.vin + size_t(tile) * QUEUE_TILE, QUEUE_TILE * 4u);
        }
      }
    }
    const uint32_t seg = it.x;
    const uint32_t type = it.y >> QITEM_SHIFT;
    const uint32_t idx = it.y & ((1u << QITEM_SHIFT) - 1u);
    const QSeg* q = segs + seg;
    const uint32_t meta = q->meta;
    const int kind = int(meta & 0xFFu), logb = int((meta >> 8) & 0xFFu);
    if (type == QITEM_PRE) {
      switch (kind) {
        case KIND_DELTA: queue_pre_kind<KIND_DELTA>(logb, q, idx, matrix, byte_area); break;
        case KIND_DIV: queue_pre_kind<KIND_DIV>(logb, q, idx, matrix, byte_area); break;
        case KIND_BITS: queue_pre_kind<KIND_BITS>(logb, q, idx, matrix, byte_area); break;
        case KIND_RANGE: queue_pre_kind<KIND_RANGE>(logb, q, idx, matrix, byte_area); break;
        case KIND_MASK: queue_pre_kind<KIND_MASK>(logb, q, idx, matrix, byte_area); break;
        default: queue_pre_kind<KIND_EVEN_FLOAT>(logb, q, idx, matrix, byte_area); break;
      }
      const uint32_t t0 = idx * QUEUE_PRE_TILES, nt = q->d.num_tiles;
      queue_publish(st.pre_done + seg, min(QUEUE_PRE_TILES, nt - t0));
    } else if (type == QITEM_SCAN) {
      const uint32_t num_tiles = q->d.num_tiles, off = q->d.matrix_off, status_off = q->status_off;
      queue_wait(st.pre_done + seg, num_tiles, hdr);
      scan_chunk(matrix + off, num_tiles << logb, idx, st.status + status_off, hdr);
      queue_publish(st.scan_done + seg, 1u);
    } else {
      const bool kv = (meta >> 16) & 1u, given = kind != KIND_DELTA;
      const uint32_t* done = st.scan_done + seg;
      switch (logb) {
        case 1: queue_post_l<1>(kv, given, q, idx, matrix, byte_area, done, hdr); break;
        case 2: queue_post_l<2>(kv, given, q, idx, matrix, byte_area, done, hdr); break;
        case 3: queue_post_l<3>(kv, given, q, idx, matrix, byte_area, done, hdr); break;
        case 4: queue_post_l<4>(kv, given, q, idx, matrix, byte_area, done, hdr); break;
        case 5: queue_post_l<5>(kv, given, q, idx, matrix, byte_area, done, hdr); break;
        case 6: queue_post_l<6>(kv, given, q, idx, matrix, byte_area, done, hdr); break;
        case 7: queue_post_l<7>(kv, given, q, idx, matrix, byte_area, done, hdr); break;
        default: queue_post_l<8>(kv, given, q, idx, matrix, byte_area, done, hdr); break;
      }
    }
    __syncthreads();  // shared memory is reused by the next item; s_next is written
    if (tid == 0) {
      s_item = s_next;
      s_it = s_next_it;
    }
    __syncthreads();
  }
}

}  // namespace gms
