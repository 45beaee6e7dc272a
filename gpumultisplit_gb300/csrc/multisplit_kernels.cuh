// Stable multisplit kernels for sm_103a: prescan (per-tile bucket counts) and
// postscan (stable in-tile rank, shared-memory reorder, coalesced scatter).
//
// Semantics follow the reference's block-wide multisplit
// (src/kernels/bms/bms_prescan.cuh, bms_postscan.cuh, bms_postscan_pairs.cuh):
//   * tile t covers keys [t*TILE, (t+1)*TILE) in input order;
//   * the count matrix is bucket-major, counts[b * num_tiles + t]
//     (bms_prescan.cuh:114);
//   * after an exclusive scan of that matrix, the element of bucket b that is
//     the j-th of its bucket inside tile t goes to counts[b*num_tiles+t] + j,
//     which is exactly the order of cpu_multisplit_general
//     (src/cpu_functions.h:155-220).
// The reference pads the last tile into bucket B-1 (bms_prescan.cuh:62-63);
// here the tail is simply not counted, which leaves every global offset the
// same because the padding only ever sits after all real keys.
#pragma once

#include <type_traits>

#include "gms_device.cuh"

// How a warp finds, for B > 32, the lanes holding the same bucket as each lane
// (its peer mask) in one 32-key slot:
//   0  log2(B) bit-plane ballots (logic pipe);
//   1  match.any (one instruction on its own pipe, but about 1.6x slower here);
//   2  a shared-memory atomicOr of each lane's bit into a per-warp bitmap
//      indexed by bucket, then one load (OR is order-independent, so the mask
//      is deterministic); it trades logic work for shared-memory traffic and
//      measured about 7% slower.
#ifndef GMS_PEERS_MODE
#define GMS_PEERS_MODE 0
#endif

// Threads per SM the key-only postscan's register budget is sized for: six
// 256-thread blocks (40 registers) measured 3-5% faster than four (64) at
// B <= 32 and equal above.
#ifndef GMS_KEYS_RESIDENT_THREADS
#define GMS_KEYS_RESIDENT_THREADS 1536
#endif
// The same for the key-value postscan: four blocks of 64 registers (five
// blocks gained 2% at B = 64 and lost 2% at B = 256; six spilled and lost more).
#ifndef GMS_PAIRS_RESIDENT_THREADS
#define GMS_PAIRS_RESIDENT_THREADS 1024
#endif
// Independent rank chains per warp at 65-128 buckets (1 or 2).  Two measured
// 1.7 % faster there (1.178 against 1.198 ms for 2^28 pairs, and the 7-bit
// sorts' passes 1.2 % faster); at 256 buckets the doubled count table and
// tile scan made them 2.7 % slower, and at 64 they were equal.
#ifndef GMS_RANK_CHAINS
#define GMS_RANK_CHAINS 2
#endif

namespace gms {

// Tile geometry of one (B, key/value, element widths) instance.  KW and VW
// are the 32-bit words of a key and of a value (1 or 2): 64-bit elements.
template <int LOGB_, int WARPS_, int IPT_, bool KV_, int KW_ = 1, int VW_ = 1>
struct TileCfg {
  static constexpr int LOGB = LOGB_;
  static constexpr uint32_t B = 1u << LOGB_;
  static constexpr int WARPS = WARPS_;
  static constexpr int THREADS = WARPS_ * 32;
  static constexpr int IPT = IPT_;  // keys per thread
  static constexpr uint32_t TILE = THREADS * IPT_;
  static constexpr bool KV = KV_;
  static constexpr int KW = KW_;
  static constexpr int VW = VW_;
  static constexpr bool WIDE = KW_ == 2 || (KV_ && VW_ == 2);  // any 64-bit element
  using KT = std::conditional_t<KW_ == 2, uint64_t, uint32_t>;
  using VT = std::conditional_t<VW_ == 2, uint64_t, uint32_t>;
  static_assert((KW_ == 1 || KW_ == 2) && (VW_ == 1 || VW_ == 2), "elements are 32 or 64 bits");
  static constexpr uint32_t WB = B < 32 ? 32 : B;  // row width of the per-warp count table
  // Words per count-table entry: {peer bitmap, count} pairs when the bitmap
  // peer search is used (B > 32), else the count alone.
  static constexpr uint32_t WS = (LOGB_ > 5 && GMS_PEERS_MODE == 2) ? 2 : 1;

  static_assert(IPT % 4 == 0, "IPT must be a multiple of 4 (16-byte vector loads)");
  static_assert(TILE <= 65536, "in-tile positions are packed into 16 bits");
  static_assert(THREADS >= static_cast<int>(B), "one thread per bucket in the tile scan");

};

// ------------------------------------------------------------- counting
// Counting keys per bucket.  For the smallest bucket counts every lane keeps
// the count of bucket `lane` in registers, fed by log2(B) ballots per 32 keys;
// otherwise keys are counted with shared-memory atomics into R replicas of a
// B-entry histogram (R = 32/B below 32 buckets, lane l using replica l % R), so
// few lanes of a warp ever hit the same word.
#ifndef GMS_COUNT_BALLOT_MAX_LOGB
#define GMS_COUNT_BALLOT_MAX_LOGB 0
#endif

template <int LOGB, class Id>
struct KeyCounter {
  static constexpr uint32_t B = 1u << LOGB;
  static constexpr bool kBallot = LOGB <= GMS_COUNT_BALLOT_MAX_LOGB;
  static constexpr uint32_t R = B >= 32 ? 1u : 32u / B;  // histogram replicas (atomic path)
  static constexpr uint32_t HIST_WORDS = B * R;         // >= 32
  Id ident;
  uint32_t* s_hist;                      // 2 x HIST_WORDS (atomic path) or WARPS*32 (ballot path)
  uint32_t acc[4] = {0u, 0u, 0u, 0u};    // ballot path: independent accumulators keep the chains parallel
  uint32_t xm[kBallot ? LOGB : 1];
  uint32_t slot;                          // atomic path: this lane's replica offset
  uint32_t buf = 0;                       // atomic path: histogram being filled (0 or HIST_WORDS)

  __device__ __forceinline__ KeyCounter(const Id& id, uint32_t* hist) : ident(id), s_hist(hist) {
    const uint32_t lane = lane_id();
    if constexpr (kBallot) {
#pragma unroll
      for (int i = 0; i < LOGB; ++i) xm[i] = ((lane >> i) & 1u) ? 0u : ~0u;
    }
    slot = lane & (R - 1);
  }

  // Called by all 32 lanes of the warp together; A selects an accumulator.
  template <int A = 0>
  __device__ __forceinline__ void add(uint32_t key, bool valid) {
    add_bucket<A>(ident(key), valid);
  }

  template <int A = 0>
  __device__ __forceinline__ void add_bucket(uint32_t b, bool valid) {
    if constexpr (kBallot) {
      uint32_t m = __ballot_sync(~0u, valid);
#pragma unroll
      for (int i = 0; i < LOGB; ++i) m &= __ballot_sync(~0u, (b >> i) & 1u) ^ xm[i];
      acc[A] += __popc(m);
    } else {
      if (valid) atomicAdd(&s_hist[buf + b * R + slot], 1u);
    }
  }

  // Shared words the counter needs for a block of `warps` warps.  The atomic
  // path keeps two histograms: one tile is read out and cleared while the
  // next one is counted into the other, so a tile needs one barrier.
  __host__ __device__ static constexpr uint32_t smem_words(int warps) {
    return kBallot ? uint32_t(warps) * 32u : 2u * HIST_WORDS;
  }

  // Zero the shared histograms (atomic path); all threads call, a barrier must follow.
  __device__ __forceinline__ void clear_shared() {
    if constexpr (!kBallot) {
      for (uint32_t i = threadIdx.x; i < 2u * HIST_WORDS; i += blockDim.x) s_hist[i] = 0u;
    }
  }

  // Block totals: after the call (which contains a barrier), thread b < B
  // returns the block's count of bucket b, and the counter is ready for the
  // next tile.
  __device__ __forceinline__ uint32_t block_total() {
    const uint32_t tid = threadIdx.x;
    uint32_t total = 0;
    if constexpr (kBallot) {
      const uint32_t lane = tid & 31u, warp = tid >> 5;
      if (lane < B) s_hist[warp * 32 + lane] = acc[0] + acc[1] + acc[2] + acc[3];
      acc[0] = acc[1] = acc[2] = acc[3] = 0u;
      __syncthreads();
      if (tid < B) {
        for (uint32_t w = 0; w < blockDim.x / 32; ++w) total += s_hist[w * 32 + tid];
      }
      __syncthreads();
    } else {
      // The barrier ends this tile's counting; the histogram is cleared here
      // and filled again two tiles later, after the next tile's barrier.
      __syncthreads();
      if (tid < B) {
#pragma unroll
        for (uint32_t r = 0; r < R; ++r) {
          total += s_hist[buf + tid * R + r];
          s_hist[buf + tid * R + r] = 0u;
        }
      }
      buf ^= HIST_WORDS;
    }
    return total;
  }
};

template <int THREADS, int IPT>
__device__ __forceinline__ void load_tile_v4(const uint32_t* __restrict__ keys, uint32_t base, uint4 (&v)[IPT / 4]) {
#pragma unroll
  for (int k = 0; k < IPT / 4; ++k) v[k] = ld_nc_v4(keys + base + (uint32_t(k) * THREADS + threadIdx.x) * 4u);
}

// Counts one tile held as 16-byte vectors (thread t holds keys
// (k*THREADS + t)*4 .. +3 of vector k).  WRITE_BYTES: also stores every key's
// bucket as one byte at bytes_out[(k*THREADS + t)*4 ..] (four per store).
template <int THREADS, int IPT, bool WRITE_BYTES = false, class Counter>
__device__ __forceinline__ void count_v4(const uint4 (&v)[IPT / 4], Counter& c, uint8_t* bytes_out = nullptr) {
#pragma unroll
  for (int k = 0; k < IPT / 4; ++k) {
    const uint32_t b0 = c.ident(v[k].x), b1 = c.ident(v[k].y), b2 = c.ident(v[k].z), b3 = c.ident(v[k].w);
    c.template add_bucket<0>(b0, true);
    c.template add_bucket<1>(b1, true);
    c.template add_bucket<2>(b2, true);
    c.template add_bucket<3>(b3, true);
    if constexpr (WRITE_BYTES)
      reinterpret_cast<uint32_t*>(bytes_out)[uint32_t(k) * THREADS + threadIdx.x] =
          b0 | (b1 << 8) | (b2 << 16) | (b3 << 24);
  }
}

// Counts tiles first, first+stride, ... (tiles of THREADS*IPT keys) and calls
// done(tile) after each one.  The next tile's keys are loaded into registers
// while the current tile is counted, so loads stay in flight.  WRITE_BYTES:
// every key's bucket is also stored as one byte at bytes_out[key index].
template <int THREADS, int IPT, bool WRITE_BYTES = false, class Counter, class Done>
__device__ __forceinline__ void count_tiles(const uint32_t* __restrict__ keys, uint32_t n, uint32_t first,
                                            uint32_t stride, Counter& c, Done done, uint8_t* bytes_out = nullptr,
                                            uint32_t last = ~0u) {
  constexpr uint32_t TILE = uint32_t(THREADS) * IPT;
  const uint32_t num_tiles = min(uint32_t((uint64_t(n) + TILE - 1) / TILE), last);
  const bool vec_ok = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0;
  const uint32_t full_tiles = vec_ok ? min(n / TILE, num_tiles) : 0u;  // tiles read with vector loads
  uint4 cur[IPT / 4];
  if (first < full_tiles) load_tile_v4<THREADS, IPT>(keys, first * TILE, cur);
  for (uint32_t tile = first; tile < num_tiles; tile += stride) {
    const uint32_t next = tile + stride;
    uint4 nxt[IPT / 4];
    if (next < full_tiles) load_tile_v4<THREADS, IPT>(keys, next * TILE, nxt);
    if (tile < full_tiles) {
      count_v4<THREADS, IPT, WRITE_BYTES>(cur, c, WRITE_BYTES ? bytes_out + size_t(tile) * TILE : nullptr);
    } else {
      const uint32_t base = tile * TILE;
      const uint32_t cnt = min(TILE, n - base);
#pragma unroll 4
      for (int k = 0; k < IPT; ++k) {
        const uint32_t i = uint32_t(k) * THREADS + threadIdx.x;
        const bool valid = i < cnt;
        const uint32_t b = c.ident(valid ? keys[base + i] : 0u);
        c.add_bucket(b, valid);
        if constexpr (WRITE_BYTES) {
          if (valid) bytes_out[base + i] = uint8_t(b);
        }
      }
    }
    done(tile);
#pragma unroll
    for (int k = 0; k < IPT / 4; ++k) cur[k] = nxt[k];
  }
}

// --------------------------------------------------------------- prescan
// Persistent grid over the tiles.  Writes counts[b * num_tiles + tile] for
// every tile and resets the scan state (ticket, chunk status words, error
// word) for the scan that follows.
//
// bucket_bytes (identifiers costly to evaluate; may be null): every key's
// bucket is also stored there as one byte, so the postscan need not evaluate
// the identifier again.
//
// Each block counts a contiguous run of tiles and keeps the counts of
// PRESCAN_GROUP consecutive tiles in shared memory, then writes them bucket by
// bucket: a warp stores whole runs of consecutive matrix words (the matrix is
// bucket-major) instead of one scattered word per bucket and tile.
constexpr uint32_t PRESCAN_GROUP = 8;

template <class C, class P>
__global__ void __launch_bounds__(C::THREADS) prescan_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                             uint32_t num_tiles, uint32_t* __restrict__ counts,
                                                             typename P::Params bp, ScratchHeader* hdr,
                                                             uint64_t* __restrict__ status, uint32_t num_chunks,
                                                             uint8_t* __restrict__ bucket_bytes) {
  griddep_launch_dependents();  // the scan may be scheduled now; it waits for this grid
  using Counter = KeyCounter<C::LOGB, typename P::Id>;
  constexpr uint32_t G = PRESCAN_GROUP;
  __shared__ uint32_t s_hist[Counter::smem_words(C::WARPS)];
  __shared__ uint32_t s_split[P::SMEM_WORDS];  // identifier state (RANGE splitters + table)
  __shared__ uint32_t s_cnt[C::B * G];         // counts of the current group of tiles, bucket-major

  const uint32_t tid = threadIdx.x;

  // Reset the scan state for this call.
  for (uint32_t i = blockIdx.x * C::THREADS + tid; i < num_chunks; i += gridDim.x * C::THREADS) status[i] = 0ull;
  if (blockIdx.x == 0 && tid == 0) {
    hdr->error = 0u;
    hdr->error_info = 0u;
    hdr->ticket = 0u;
    hdr->wait_limit_us = 0u;
  }

  P::prepare(s_split, bp);
  Counter counter(P::make(bp, s_split), s_hist);
  counter.clear_shared();
  __syncthreads();
  // This block's tiles: [first, last), a whole number of groups.
  const uint32_t per = ((num_tiles + gridDim.x - 1) / gridDim.x + G - 1) / G * G;
  const uint32_t first = min(blockIdx.x * per, num_tiles);
  const uint32_t last = min(first + per, num_tiles);
  auto flush = [&](uint32_t group_first) {
    __syncthreads();
    for (uint32_t i = tid; i < C::B * G; i += C::THREADS) {
      const uint32_t t = group_first + i % G;
      if (t < last) counts[(i / G) * num_tiles + t] = s_cnt[i];
    }
    __syncthreads();
  };
  auto done = [&](uint32_t tile) {
    const uint32_t total = counter.block_total();
    const uint32_t g = (tile - first) % G;
    if (tid < C::B) s_cnt[tid * G + g] = total;
    if (g == G - 1 || tile + 1 == last) flush(tile - g);
  };
  if constexpr (!P::CHEAP) {
    if (bucket_bytes != nullptr) {
      count_tiles<C::THREADS, C::IPT, true>(keys, n, first, 1u, counter, done, bucket_bytes, last);
      return;
    }
  }
  count_tiles<C::THREADS, C::IPT>(keys, n, first, 1u, counter, done, nullptr, last);
}

// ------------------------------------------------ prescan, 64-bit keys
// The prescan for 64-bit keys: the same tiles, counts, group flush and scan
// reset as prescan_kernel, and every key's bucket is always stored as one
// byte (the 64-bit postscan reads them instead of the keys' identifier).
// In a full tile, thread t loads keys 2(k*THREADS + t) and the next one as one
// 16-byte vector, for k < IPT/2; the next tile's vectors are in flight while
// the current tile is counted.
template <int THREADS, int IPT>
__device__ __forceinline__ void load_tile64(const uint64_t* __restrict__ keys, uint32_t base,
                                            uint4 (&v)[IPT / 2]) {
#pragma unroll
  for (int k = 0; k < IPT / 2; ++k)
    v[k] = ld_nc_v4(reinterpret_cast<const uint32_t*>(keys + base + (uint32_t(k) * THREADS + threadIdx.x) * 2u));
}

template <class C, class P>
__global__ void __launch_bounds__(C::THREADS) prescan64_kernel(const uint64_t* __restrict__ keys, uint32_t n,
                                                               uint32_t num_tiles, uint32_t* __restrict__ counts,
                                                               typename P::Params bp, ScratchHeader* hdr,
                                                               uint64_t* __restrict__ status, uint32_t num_chunks,
                                                               uint8_t* __restrict__ bucket_bytes) {
  griddep_launch_dependents();  // the scan may be scheduled now; it waits for this grid
  using Counter = KeyCounter<C::LOGB, typename P::Id>;
  constexpr uint32_t G = PRESCAN_GROUP;
  constexpr uint32_t TILE = C::TILE;
  constexpr int NV = C::IPT / 2;
  __shared__ uint32_t s_hist[Counter::smem_words(C::WARPS)];
  __shared__ __align__(16) uint32_t s_split[P::SMEM_WORDS];  // RANGE: 64-bit splitters + table
  __shared__ uint32_t s_cnt[C::B * G];

  const uint32_t tid = threadIdx.x;
  for (uint32_t i = blockIdx.x * C::THREADS + tid; i < num_chunks; i += gridDim.x * C::THREADS) status[i] = 0ull;
  if (blockIdx.x == 0 && tid == 0) {
    hdr->error = 0u;
    hdr->error_info = 0u;
    hdr->ticket = 0u;
    hdr->wait_limit_us = 0u;
  }

  P::prepare(s_split, bp);
  Counter counter(P::make(bp, s_split), s_hist);
  counter.clear_shared();
  __syncthreads();
  const uint32_t per = ((num_tiles + gridDim.x - 1) / gridDim.x + G - 1) / G * G;
  const uint32_t first = min(blockIdx.x * per, num_tiles);
  const uint32_t last = min(first + per, num_tiles);
  auto flush = [&](uint32_t group_first) {
    __syncthreads();
    for (uint32_t i = tid; i < C::B * G; i += C::THREADS) {
      const uint32_t t = group_first + i % G;
      if (t < last) counts[(i / G) * num_tiles + t] = s_cnt[i];
    }
    __syncthreads();
  };

  const bool vec_ok = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0;
  const uint32_t full_tiles = vec_ok ? min(n / TILE, last) : 0u;
  uint4 cur[NV];
  if (first < full_tiles) load_tile64<C::THREADS, C::IPT>(keys, first * TILE, cur);
  for (uint32_t tile = first; tile < last; ++tile) {
    uint4 nxt[NV];
    if (tile + 1 < full_tiles) load_tile64<C::THREADS, C::IPT>(keys, (tile + 1) * TILE, nxt);
    const uint32_t base = tile * TILE;
    if (tile < full_tiles) {
      uint16_t* out = reinterpret_cast<uint16_t*>(bucket_bytes + base);
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        const uint32_t b0 = counter.ident(uint64_t(cur[k].x) | (uint64_t(cur[k].y) << 32));
        const uint32_t b1 = counter.ident(uint64_t(cur[k].z) | (uint64_t(cur[k].w) << 32));
        counter.template add_bucket<0>(b0, true);
        counter.template add_bucket<1>(b1, true);
        out[uint32_t(k) * C::THREADS + tid] = uint16_t(b0 | (b1 << 8));
      }
    } else {
      const uint32_t cnt = min(TILE, n - base);
#pragma unroll 4
      for (int k = 0; k < C::IPT; ++k) {
        const uint32_t i = uint32_t(k) * C::THREADS + tid;
        const bool valid = i < cnt;
        const uint32_t b = counter.ident(valid ? keys[base + i] : 0ull);
        counter.add_bucket(b, valid);
        if (valid) bucket_bytes[base + i] = uint8_t(b);
      }
    }
    const uint32_t total = counter.block_total();
    const uint32_t g = (tile - first) % G;
    if (tid < C::B) s_cnt[tid * G + g] = total;
    if (g == G - 1 || tile + 1 == last) flush(tile - g);
#pragma unroll
    for (int k = 0; k < NV; ++k) cur[k] = nxt[k];
  }
}

// Shared-memory layout of the postscan for identifier policy P (bytes), and
// what phase 3 writes at each key's bucket-sorted position:
//   R_KEYS       the key (key-only, identifier cheap to recompute): phase 4
//                reads keys conflict-free and recomputes their buckets;
//   R_INDEX16    the key's 16-bit in-tile index (key-value, cheap identifier):
//                a small buffer keeps four tiles resident per SM;
//   R_KEYS_B,    the same plus the key's bucket as one byte, for identifiers
//   R_INDEX16_B  that are costly to recompute (RANGE, DIV, EVEN_FLOAT, user
//                functors).
// The per-warp count table holds 16-bit entries (a warp counts at most
// 32 * IPT keys and a tile holds at most 2^16), except in the bitmap peer mode.
enum ReorderMode { R_KEYS = 0, R_INDEX16 = 1, R_KEYS_B = 2, R_INDEX16_B = 3 };

template <class C, class P, bool GIVEN = false>
struct PostLayout {
  static constexpr bool CHEAP = P::CHEAP;
  static_assert(!GIVEN || !P::CHEAP, "given bucket bytes are only used for costly identifiers");
  static_assert(C::KW == 1 || GIVEN, "64-bit keys take their buckets from the prescan's bytes");
  // Keys are reordered through a 16-bit index whenever values come along or
  // keys are 64 bits wide (a sorted copy of the keys would take more room).
  static constexpr int MODE =
      (C::KV || C::KW == 2) ? (CHEAP ? R_INDEX16 : R_INDEX16_B) : (CHEAP ? R_KEYS : R_KEYS_B);
  static constexpr bool INDEXED = MODE == R_INDEX16 || MODE == R_INDEX16_B;
  static constexpr bool BUCKET_BYTES = MODE == R_KEYS_B || MODE == R_INDEX16_B;
  using WhT = std::conditional_t<C::WS == 2, uint32_t, uint16_t>;
  static constexpr size_t OFF_K = 0;
  static constexpr size_t OFF_V = OFF_K + size_t(C::TILE) * sizeof(typename C::KT);
  static constexpr size_t OFF_R = OFF_V + (C::KV ? size_t(C::TILE) * sizeof(typename C::VT) : 0);
  static constexpr size_t R_BYTES = size_t(C::TILE) * (INDEXED ? 2 : 4);
  static constexpr size_t OFF_RB = OFF_R + R_BYTES;  // bucket bytes
  static constexpr size_t OFF_WH = (OFF_RB + (BUCKET_BYTES ? C::TILE : 0) + 15) & ~size_t(15);
  // At 65-128 buckets a warp ranks its slots in CHAINS independent runs
  // (slots [c*IPT/CHAINS, (c+1)*IPT/CHAINS) against count table c), so the
  // table's read-modify-write chains of the runs interleave.  Sub-warp
  // w*CHAINS + c holds the keys of run c of warp w, in input order.
  static constexpr int CHAINS =
      (C::LOGB == 7 && C::WS == 1 && GMS_PEERS_MODE == 0 && C::IPT % GMS_RANK_CHAINS == 0) ? GMS_RANK_CHAINS : 1;
  static constexpr int SUBWARPS = C::WARPS * CHAINS;
  static constexpr size_t OFF_DELTA = (OFF_WH + size_t(SUBWARPS) * C::WB * C::WS * sizeof(WhT) + 15) & ~size_t(15);
  static constexpr size_t OFF_SPLIT = OFF_DELTA + C::B * 4;
  // With bucket bytes from the prescan the identifier is never evaluated, so
  // it needs no shared area.
  static constexpr size_t OFF_SCAN = OFF_SPLIT + (GIVEN ? 0 : P::SMEM_WORDS * 4);
  static constexpr size_t OFF_FLAG = OFF_SCAN + 32 * 4;  // warp totals of the tile scan
  static constexpr size_t OFF_BAR = (OFF_FLAG + 4 + 15) & ~size_t(15);
  static constexpr size_t BYTES = OFF_BAR + 16;
  // Blocks per SM the register budget is sized for (64 registers at 16 keys per thread).
  static constexpr int RESIDENT_THREADS = C::IPT <= 8 ? 1536 : (C::KV ? GMS_PAIRS_RESIDENT_THREADS : GMS_KEYS_RESIDENT_THREADS);
  static constexpr int THREAD_BLOCKS = RESIDENT_THREADS / C::THREADS > 0 ? RESIDENT_THREADS / C::THREADS : 1;
  // With 64-bit elements shared memory bounds the blocks per SM first
  // (228 KB per SM, 1 KB of it reserved per block).
  static constexpr int SMEM_BLOCKS = int((228u * 1024u) / (BYTES + 1024u));
  static constexpr int MIN_BLOCKS =
      C::WIDE ? (SMEM_BLOCKS < THREAD_BLOCKS ? (SMEM_BLOCKS > 0 ? SMEM_BLOCKS : 1) : THREAD_BLOCKS) : THREAD_BLOCKS;
};

// Peer mask (lanes of this warp whose key in this slot has bucket b) from
// log2(B) bit-plane ballots: lanes agree on bit i iff ballot_i ^ own_i is set,
// with own_i = 0 or ~0 by this lane's bit i.
template <int LOGB>
__device__ __forceinline__ uint32_t peers_by_ballot(uint32_t b) {
  uint32_t peers = ~0u;
#pragma unroll
  for (int i = 0; i < LOGB; ++i) {
    const uint32_t bal = __ballot_sync(~0u, (b >> i) & 1u);
    const uint32_t own = ((b >> i) & 1u) - 1u;  // bit set -> 0, clear -> ~0
    peers &= bal ^ own;
  }
  return peers;
}

// Where a tile's global bucket offsets come from.  Thread b < B holds the
// source for bucket b: aggregate() is called once the tile's count of bucket b
// is known (phase 2); offset() returns the bucket's global offset for this
// tile, in phase 2 when KNOWN_EARLY, else after the tile is sorted in shared
// memory (phase 3), just before the global stores.  GivenOffset is an entry of
// the scanned count matrix, loaded when the tile starts.
struct GivenOffset {
  static constexpr bool KNOWN_EARLY = true;  // resolved in phase 2, before the reorder
  uint32_t goff;
  __device__ __forceinline__ void aggregate(uint32_t, uint32_t) {}
  __device__ __forceinline__ uint32_t offset(uint32_t, uint32_t) { return goff; }
};

// The default source of a job's offsets: its entries of the scanned count
// matrix (minus the job's bias in a shared scan).
struct MatrixOffsets {
  template <class Job>
  __device__ __forceinline__ GivenOffset operator()(const Job& job, uint32_t tid, uint32_t num_buckets) const {
    return GivenOffset{tid < num_buckets ? job.offsets[tid * job.num_tiles + job.tile] - job.bias : 0u};
  }
};

// Phases 1-4 of the postscan for one staged tile.  FULL: the tile holds
// exactly TILE keys, so no per-key validity test is needed.
//
// GIVEN: the tile's buckets were staged as bytes at the bucket-byte area (in
// input order) by the caller, so the identifier is not evaluated; phase 3
// overwrites that area with the buckets in sorted order.
//
// STREAM_HINTS: the output stores mark their L2 lines evict-first (the batch
// queue keeps keys that are read twice in L2 meanwhile; 32-bit elements).
template <class C, class P, bool FULL, bool GIVEN = false, class Offsets = GivenOffset, bool STREAM_HINTS = false>
__device__ __forceinline__ bool postscan_tile(typename C::KT* __restrict__ kout, typename C::VT* __restrict__ vout,
                                              uint32_t n, uint32_t cnt, Offsets& offs, const typename P::Params& bp,
                                              ScratchHeader* hdr, unsigned char* smem) {
  using L = PostLayout<C, P, GIVEN>;
  using WhT = typename L::WhT;
  using KT = typename C::KT;
  using VT = typename C::VT;
  constexpr uint32_t B = C::B;
  constexpr int LOGB = C::LOGB;
  constexpr int IPT = C::IPT;
  constexpr uint32_t WB = C::WB;
  constexpr uint32_t WS = C::WS;
  KT* s_k = reinterpret_cast<KT*>(smem + L::OFF_K);
  VT* s_v = reinterpret_cast<VT*>(smem + L::OFF_V);
  uint32_t* s_r = reinterpret_cast<uint32_t*>(smem + L::OFF_R);
  uint8_t* s_rb = reinterpret_cast<uint8_t*>(smem + L::OFF_RB);
  WhT* s_wh = reinterpret_cast<WhT*>(smem + L::OFF_WH);
  uint32_t* s_delta = reinterpret_cast<uint32_t*>(smem + L::OFF_DELTA);
  const uint32_t* s_split = reinterpret_cast<const uint32_t*>(smem + L::OFF_SPLIT);
  uint32_t* s_scan = reinterpret_cast<uint32_t*>(smem + L::OFF_SCAN);
  uint32_t* s_flag = reinterpret_cast<uint32_t*>(smem + L::OFF_FLAG);
  const uint32_t tid = threadIdx.x;
  const uint32_t lane = tid & 31u;
  const uint32_t warp = tid >> 5;

  // ---- 1. stable in-warp ranks
  const typename P::Id ident = P::make(bp, s_split);
  // Bucket of the staged key at in-tile position pos.
  auto bucket_at = [&](uint32_t pos) -> uint32_t {
    if constexpr (GIVEN)
      return uint32_t(s_rb[pos]) & (B - 1);
    else
      return ident(s_k[pos]);
  };
  uint32_t packed[IPT];  // (bucket << 16) | rank among same-bucket keys of this warp
  const uint32_t wbase = warp * (IPT * 32u);
  const uint32_t lt = lanemask_lt();
  if constexpr (LOGB <= 5) {
    // Lane l counts bucket l: its mask of lanes holding bucket l comes straight
    // from the ballots, and a key's peers and earlier count are read from the
    // lane that owns its bucket.
    uint32_t xm[LOGB];
#pragma unroll
    for (int i = 0; i < LOGB; ++i) xm[i] = ((lane >> i) & 1u) ? 0u : ~0u;
    uint32_t my_cnt = 0;
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      const uint32_t pos = wbase + uint32_t(j) * 32u + lane;
      const uint32_t b = bucket_at(pos);
      uint32_t m = FULL ? ~0u : __ballot_sync(~0u, pos < cnt);
#pragma unroll
      for (int i = 0; i < LOGB; ++i) m &= __ballot_sync(~0u, (b >> i) & 1u) ^ xm[i];
      const uint32_t peers = __shfl_sync(~0u, m, b);
      const uint32_t before = __shfl_sync(~0u, my_cnt, b);
      packed[j] = (b << 16) | (before + __popc(peers & lt));
      my_cnt += __popc(m);
    }
    if (lane < B) s_wh[warp * WB + lane] = WhT(my_cnt);
  } else {
    WhT* wh = s_wh + warp * WB * WS;  // entry b: count at [b*WS + WS-1], bitmap at [b*WS] when WS == 2
    if constexpr (GMS_PEERS_MODE == 2) {
#pragma unroll
      for (int j = 0; j < IPT; ++j) {
        const uint32_t pos = wbase + uint32_t(j) * 32u + lane;
        const bool valid = FULL || pos < cnt;
        const uint32_t b = bucket_at(pos);
        uint32_t* e = reinterpret_cast<uint32_t*>(&wh[b * WS]);
        if (valid) atomicOr(e, 1u << lane);
        __syncwarp();
        const uint2 v = *reinterpret_cast<const uint2*>(e);
        const uint32_t rank = __popc(v.x & lt);
        __syncwarp();
        if (valid && rank == 0) *reinterpret_cast<uint2*>(e) = make_uint2(0u, v.y + __popc(v.x));
        __syncwarp();
        packed[j] = (b << 16) | (v.y + rank);
      }
    } else if constexpr (L::CHAINS == 2) {
      // Slots j and j + IPT/2 step together, each against its own table.
      constexpr int HALF = IPT / 2;
      WhT* wa = s_wh + (warp * 2) * WB;
      WhT* wb = wa + WB;
#pragma unroll
      for (int j = 0; j < HALF; ++j) {
        const uint32_t pa = wbase + uint32_t(j) * 32u + lane, pb = pa + uint32_t(HALF) * 32u;
        const bool va = FULL || pa < cnt, vb = FULL || pb < cnt;
        const uint32_t ba = bucket_at(pa), bb = bucket_at(pb);
        uint32_t qa = peers_by_ballot<LOGB>(ba), qb = peers_by_ballot<LOGB>(bb);
        if (!FULL) {
          qa &= __ballot_sync(~0u, va);
          qb &= __ballot_sync(~0u, vb);
        }
        const uint32_t ra = __popc(qa & lt), rb = __popc(qb & lt);
        const uint32_t xa = wa[ba], xb = wb[bb];
        __syncwarp();
        if (va && ra == 0) wa[ba] = WhT(xa + __popc(qa));
        if (vb && rb == 0) wb[bb] = WhT(xb + __popc(qb));
        __syncwarp();
        packed[j] = (ba << 16) | (xa + ra);
        packed[j + HALF] = (bb << 16) | (xb + rb);
      }
    } else {
#pragma unroll
      for (int j = 0; j < IPT; ++j) {
        const uint32_t pos = wbase + uint32_t(j) * 32u + lane;
        const bool valid = FULL || pos < cnt;
        const uint32_t b = bucket_at(pos);
#if GMS_PEERS_MODE == 1
        uint32_t peers = __match_any_sync(~0u, b);
#else
        uint32_t peers = peers_by_ballot<LOGB>(b);
#endif
        if (!FULL) peers &= __ballot_sync(~0u, valid);
        const uint32_t rank = __popc(peers & lt);
        WhT* e = &wh[b * WS + (WS - 1)];
        const uint32_t before = *e;
        __syncwarp();
        if (valid && rank == 0) *e = WhT(before + __popc(peers));
        __syncwarp();
        packed[j] = (b << 16) | (before + rank);
      }
    }
  }
  __syncthreads();

  // ---- 2. tile scan: per-warp offsets and bucket starts.  Thread b owns
  // bucket b; the bucket starts come from a block-wide exclusive scan (warp
  // scans + warp totals).
  uint32_t my_total = 0, my_start = 0;
  {
    // Key-value tiles keep the per-warp prefixes in registers across the block
    // scan and write each count-table entry once; key-only tiles, budgeted at
    // 40 registers, write the prefixes and add the start in a second pass.
    constexpr bool PREFIX_IN_REGS = C::KV;
    constexpr int SW = LOGB > 5 ? L::SUBWARPS : C::WARPS;  // count-table rows
    uint32_t pre[PREFIX_IN_REGS ? SW : 1];
    uint32_t total = 0;
    if (tid < B) {
#pragma unroll
      for (int w = 0; w < SW; ++w) {
        WhT* c_ptr = &s_wh[(w * WB + tid) * WS + (WS - 1)];
        const uint32_t c = *c_ptr;
        if constexpr (PREFIX_IN_REGS)
          pre[w] = total;
        else
          *c_ptr = WhT(total);
        total += c;
      }
      offs.aggregate(tid, total);
      if constexpr (Offsets::KNOWN_EARLY) {
        if (uint64_t(offs.offset(tid, total)) + total > n) atomicOr(s_flag, 1u);
      }
    }
    uint32_t incl = total;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(~0u, incl, d);
      if (lane >= uint32_t(d)) incl += t;
    }
    constexpr uint32_t SCAN_WARPS = (B + 31) / 32;
    if (SCAN_WARPS > 1 && lane == 31 && warp < SCAN_WARPS) s_scan[warp] = incl;
    __syncthreads();
    if (tid < B) {
      uint32_t start = incl - total;
      if constexpr (SCAN_WARPS > 1) {
#pragma unroll
        for (uint32_t w = 0; w < SCAN_WARPS; ++w) start += (w < warp) ? s_scan[w] : 0u;
      }
      if constexpr (Offsets::KNOWN_EARLY) {
        s_delta[tid] = offs.offset(tid, total) - start;
      } else {
        my_total = total;
        my_start = start;
      }
#pragma unroll
      for (int w = 0; w < SW; ++w) {
        WhT* c_ptr = &s_wh[(w * WB + tid) * WS + (WS - 1)];
        if constexpr (PREFIX_IN_REGS)
          *c_ptr = WhT(pre[w] + start);
        else
          *c_ptr = WhT(*c_ptr + start);
      }
    }
  }
  __syncthreads();
  if constexpr (Offsets::KNOWN_EARLY) {
    if (*s_flag != 0u) {  // block-uniform
      if (tid == 0) record_error(hdr, DEV_ERR_BAD_OFFSET);
      return false;
    }
  }

  // ---- 3. bucket-sorted in-tile order (positions are a permutation of [0, cnt))
  {
    constexpr int CH = LOGB > 5 ? L::CHAINS : 1;
    const WhT* wh = s_wh + warp * CH * WB * WS + (WS - 1);
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      const uint32_t pos = wbase + uint32_t(j) * 32u + lane;
      if (FULL || pos < cnt) {
        const uint32_t b = packed[j] >> 16;
        const WhT* row = wh + (j / (IPT / CH)) * WB * WS;  // the slot's chain
        const uint32_t d = uint32_t(row[b * WS]) + (packed[j] & 0xFFFFu);
        if constexpr (L::INDEXED)
          reinterpret_cast<uint16_t*>(s_r)[d] = uint16_t(pos);
        else
          s_r[d] = s_k[pos];
        if constexpr (L::BUCKET_BYTES) s_rb[d] = uint8_t(b);
      }
    }
  }
  // Offsets resolved only now: the buckets' global offsets, the per-bucket
  // shift delta = global offset - tile start, and a range check of every
  // bucket's output run against n (a corrupt offset can then never cause a
  // store outside the output).
  if constexpr (!Offsets::KNOWN_EARLY) {
    if (tid < B) {
      const uint32_t g = offs.offset(tid, my_total);
      if (uint64_t(g) + my_total > n) atomicOr(s_flag, 1u);
      s_delta[tid] = g - my_start;
    }
  }
  __syncthreads();
  if constexpr (!Offsets::KNOWN_EARLY) {
    if (*s_flag != 0u) {  // block-uniform
      if (tid == 0) record_error(hdr, DEV_ERR_BAD_OFFSET);
      return false;
    }
  }

  // ---- 4. scatter in bucket-sorted order: each bucket's run is one coalesced store
  static_assert(!STREAM_HINTS || (C::KW == 1 && C::VW == 1), "store hints are for 32-bit elements");
  uint64_t policy = 0;
  if constexpr (STREAM_HINTS) policy = l2_evict_first_policy();
#pragma unroll
  for (int j = 0; j < IPT; ++j) {
    const uint32_t p = uint32_t(j) * C::THREADS + tid;
    if (FULL || p < cnt) {
      if constexpr (L::MODE == R_KEYS) {
        const uint32_t key = s_r[p];
        kout[s_delta[ident(key)] + p] = key;
      } else if constexpr (L::MODE == R_KEYS_B) {
        kout[s_delta[s_rb[p]] + p] = s_r[p];
      } else {
        const uint32_t src = reinterpret_cast<const uint16_t*>(s_r)[p];
        const KT key = s_k[src];
        uint32_t b;
        if constexpr (L::BUCKET_BYTES)
          b = s_rb[p];
        else
          b = ident(key);
        const uint32_t g = s_delta[b] + p;
        if constexpr (STREAM_HINTS) {
          st_global_hint(kout + g, key, policy);
          if constexpr (C::KV) st_global_hint(vout + g, s_v[src], policy);
        } else {
          kout[g] = key;
          if constexpr (C::KV) vout[g] = s_v[src];
        }
      }
    }
  }
  return true;
}

// -------------------------------------------------------------- postscan
// One tile of one multisplit, as the postscan sees it.
template <class Params, class KT = uint32_t, class VT = uint32_t>
struct TileJob {
  const KT* kin;
  const VT* vin;
  KT* kout;
  VT* vout;
  uint32_t n;                // keys of this multisplit
  uint32_t num_tiles;        // its tiles
  uint32_t tile;             // this tile
  const uint32_t* offsets;   // its scanned count matrix, bucket-major
  uint32_t bias;             // subtracted from the scanned offsets (start of this multisplit in a shared scan)
  uint32_t prefetch_tile;    // a later tile of the same arrays to pull into L2 (>= num_tiles: none)
  Params bp;
  uint32_t owner;            // which multisplit of a batch (tiles with one owner share bp)
  const uint8_t* bucket_bytes;  // every key's bucket, from the prescan (GIVEN postscans only)
};

// Postscan of one tile, run by a whole block:
//  0. bulk-copy the tile's keys (and values) into shared memory, prefetch the
//     tile's B global offsets;
//  1. per warp, stable rank of every key among same-bucket keys earlier in the
//     warp's range (warp-striped slots keep input order: slot j, lane l is
//     key w*IPT*32 + j*32 + l);
//  2. tile scan: per-warp bucket offsets and the per-bucket shift
//     delta[b] = global_offset(b, tile) - tile_start(b);
//  3. write, at each key's bucket-sorted in-tile position, its key or source index;
//  4. walk the bucket-sorted order: out[delta[b] + p] = key (value), so every
//     bucket's run is a contiguous, coalesced store.
//
// PREPARE: fill the identifier's shared area first (false when the caller
// prepared it for several tiles).  Returns false when the block must stop (a
// bulk copy timed out or an offset was out of range; the error is recorded).
// With `*bar_live` the caller learns whether the tile's mbarrier was
// initialised (it must be invalidated before the next tile initialises it).
//
// GIVEN: the prescan stored every key's bucket as a byte (job.bucket_bytes);
// the tile's bytes are staged with its keys and the identifier is never
// evaluated (nor prepared).
//
// make_offsets(job, tid, B) gives thread tid the source of bucket tid's global
// offset (see GivenOffset); it is called while the tile's bulk copy is in flight.
//
// STREAM_HINTS: the tile's keys, values and bucket bytes are read, and its
// outputs written, as evict-first L2 lines (their last use).
template <class C, class P, bool PREPARE = true, bool GIVEN = false, class MakeOffsets = MatrixOffsets,
          bool STREAM_HINTS = false>
__device__ __forceinline__ bool postscan_job(const TileJob<typename P::Params, typename C::KT, typename C::VT>& job,
                                             ScratchHeader* hdr, unsigned char* smem, bool* bar_live = nullptr,
                                             MakeOffsets make_offsets = MakeOffsets()) {
  using L = PostLayout<C, P, GIVEN>;
  using KT = typename C::KT;
  using VT = typename C::VT;
  constexpr uint32_t B = C::B;
  constexpr int LOGB = C::LOGB;
  constexpr uint32_t WB = C::WB;
  KT* s_k = reinterpret_cast<KT*>(smem + L::OFF_K);
  VT* s_v = reinterpret_cast<VT*>(smem + L::OFF_V);
  uint32_t* s_wh = reinterpret_cast<uint32_t*>(smem + L::OFF_WH);
  uint32_t* s_split = reinterpret_cast<uint32_t*>(smem + L::OFF_SPLIT);
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(smem + L::OFF_BAR);

  const uint32_t tid = threadIdx.x;
  const uint32_t base = job.tile * C::TILE;
  const uint32_t cnt = min(C::TILE, job.n - base);
  const KT* kin = job.kin;
  const VT* vin = job.vin;

  // ---- 0. stage the tile
  uintptr_t addr_bits = reinterpret_cast<uintptr_t>(kin);
  if constexpr (C::KV) addr_bits |= reinterpret_cast<uintptr_t>(vin);
  // Elements moved by the bulk copy: a multiple of 4, so every array's part
  // is a whole number of 16-byte pieces.
  const uint32_t bulk = ((addr_bits & 15u) == 0) ? (cnt & ~3u) : 0u;
  if (tid == 0) *reinterpret_cast<uint32_t*>(smem + L::OFF_FLAG) = 0u;
  // Given bucket bytes: whole 16-byte pieces by the bulk copy, the rest below.
  const uint32_t bulk_b = (GIVEN && bulk != 0) ? (cnt & ~15u) : 0u;
  uint8_t* s_rb = reinterpret_cast<uint8_t*>(smem + L::OFF_RB);
  if (tid == 0 && bulk != 0) {
    mbar_init(s_bar, 1);
    fence_mbar_init();
    mbar_arrive_expect_tx(s_bar, bulk * uint32_t(sizeof(KT) + (C::KV ? sizeof(VT) : 0)) + bulk_b);
    if constexpr (STREAM_HINTS) {
      const uint64_t policy = l2_evict_first_policy();
      bulk_copy_g2s_hint(s_k, kin + base, bulk * uint32_t(sizeof(KT)), s_bar, policy);
      if constexpr (C::KV) bulk_copy_g2s_hint(s_v, vin + base, bulk * uint32_t(sizeof(VT)), s_bar, policy);
      if constexpr (GIVEN) {
        if (bulk_b != 0) bulk_copy_g2s_hint(s_rb, job.bucket_bytes + base, bulk_b, s_bar, policy);
      }
    } else {
      bulk_copy_g2s(s_k, kin + base, bulk * uint32_t(sizeof(KT)), s_bar);
      if constexpr (C::KV) bulk_copy_g2s(s_v, vin + base, bulk * uint32_t(sizeof(VT)), s_bar);
      if constexpr (GIVEN) {
        if (bulk_b != 0) bulk_copy_g2s(s_rb, job.bucket_bytes + base, bulk_b, s_bar);
      }
    }
    // Pull a tile that starts about one wave of blocks later into L2, so its
    // bulk copy does not wait on DRAM (only full tiles: never past the arrays).
    if (job.prefetch_tile < job.num_tiles - 1u) {
      bulk_prefetch_l2(kin + size_t(job.prefetch_tile) * C::TILE, C::TILE * uint32_t(sizeof(KT)));
      if constexpr (C::KV)
        bulk_prefetch_l2(vin + size_t(job.prefetch_tile) * C::TILE, C::TILE * uint32_t(sizeof(VT)));
    }
  }
  for (uint32_t i = bulk + tid; i < cnt; i += C::THREADS) {
    s_k[i] = kin[base + i];
    if constexpr (C::KV) s_v[i] = vin[base + i];
  }
  if constexpr (GIVEN) {
    // Through L2: in the batch queue other blocks of the same launch wrote them.
    for (uint32_t i = bulk_b + tid; i < cnt; i += C::THREADS) s_rb[i] = __ldcg(job.bucket_bytes + base + i);
  }
  if (bar_live) *bar_live = bulk != 0;
  auto offs = make_offsets(job, tid, B);
  if constexpr (PREPARE && !GIVEN) P::prepare(s_split, job.bp);
  if constexpr (LOGB > 5) {
    // the count table as 32-bit words (its byte size is a multiple of 4)
    constexpr uint32_t WORDS = L::SUBWARPS * WB * C::WS * sizeof(typename L::WhT) / 4;
    for (uint32_t i = tid; i < WORDS; i += C::THREADS) s_wh[i] = 0u;
  }
  __syncthreads();
  if (bulk != 0) {
    const bool ok = error_recorded(hdr) ? mbar_try_wait(s_bar, 0) : mbar_wait_bounded(s_bar, 0, hdr);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        record_error(hdr, DEV_ERR_BULK_COPY_TIMEOUT);
        mbar_wait_bounded(s_bar, 0, hdr);  // let a late copy land before the block moves on
      }
      return false;
    }
  }

  if (cnt == C::TILE)
    return postscan_tile<C, P, true, GIVEN, decltype(offs), STREAM_HINTS>(job.kout, job.vout, job.n, cnt, offs,
                                                                           job.bp, hdr, smem);
  return postscan_tile<C, P, false, GIVEN, decltype(offs), STREAM_HINTS>(job.kout, job.vout, job.n, cnt, offs,
                                                                          job.bp, hdr, smem);
}

// Persistent postscan over tiles first, first + stride, ... below last, for
// identifiers with a shared area (RANGE): the area is prepared again only when
// the tile's owner (multisplit of a batch) changes, and each tile pulls the
// block's next tile into L2.
template <class C, class P, class JobAt>
__device__ __forceinline__ void postscan_run(uint32_t first, uint32_t last, uint32_t stride, JobAt job_at,
                                             ScratchHeader* hdr, unsigned char* smem) {
  using L = PostLayout<C, P>;
  uint32_t* s_split = reinterpret_cast<uint32_t*>(smem + L::OFF_SPLIT);
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(smem + L::OFF_BAR);
  uint32_t prepared_for = ~0u;  // owner whose parameters the shared area holds
  for (uint32_t t = first; t < last; t += stride) {
    const TileJob<typename P::Params, typename C::KT, typename C::VT> job =
        job_at(t, last - t > stride ? t + stride : ~0u);
    if (job.owner != prepared_for) {  // block-uniform: every thread reads the same job
      P::prepare(s_split, job.bp);
      prepared_for = job.owner;
    }
    bool bar_live = false;
    const bool ok = postscan_job<C, P, false>(job, hdr, smem, &bar_live);
    __syncthreads();  // shared buffers are reused by the next tile
    if (!ok) return;
    if (bar_live && threadIdx.x == 0) mbar_inval(s_bar);
  }
}

// Plain postscan: one block per tile of one multisplit.  GIVEN: the buckets
// come from bucket_bytes (written by the prescan).
template <class C, class P, bool GIVEN = false>
__global__ void __launch_bounds__(C::THREADS, (PostLayout<C, P, GIVEN>::MIN_BLOCKS)) postscan_kernel(
    const typename C::KT* __restrict__ kin, const typename C::VT* __restrict__ vin, typename C::KT* __restrict__ kout,
    typename C::VT* __restrict__ vout, uint32_t n, uint32_t num_tiles, const uint32_t* __restrict__ offsets,
    typename P::Params bp, ScratchHeader* hdr, uint32_t prefetch_dist, const uint8_t* __restrict__ bucket_bytes) {
  extern __shared__ __align__(128) unsigned char smem[];
  griddep_wait();  // launched while the scan finishes: its offsets are complete past this point
  const TileJob<typename P::Params, typename C::KT, typename C::VT> job{kin,        vin,     kout, vout,
                                        n,          num_tiles, blockIdx.x, offsets,
                                        0u,         prefetch_dist != 0 ? blockIdx.x + prefetch_dist : ~0u,
                                        bp,         0u,      bucket_bytes};
  postscan_job<C, P, true, GIVEN>(job, hdr, smem);
}

// Persistent plain postscan (identifiers with a shared area): block b runs
// tiles b, b + grid, ...  Blocks that run at the same time then work on
// neighbouring tiles, whose runs of one bucket are neighbours in the output,
// so partly written sectors merge in L2 before they reach DRAM.
template <class C, class P>
__global__ void __launch_bounds__(C::THREADS, (PostLayout<C, P>::MIN_BLOCKS)) postscan_persistent_kernel(
    const typename C::KT* __restrict__ kin, const typename C::VT* __restrict__ vin, typename C::KT* __restrict__ kout,
    typename C::VT* __restrict__ vout, uint32_t n, uint32_t num_tiles, const uint32_t* __restrict__ offsets,
    typename P::Params bp, ScratchHeader* hdr) {
  extern __shared__ __align__(128) unsigned char smem[];
  griddep_wait();  // launched while the scan finishes: its offsets are complete past this point
  postscan_run<C, P>(
      blockIdx.x, num_tiles, gridDim.x,
      [&](uint32_t t, uint32_t prefetch) {
        return TileJob<typename P::Params, typename C::KT, typename C::VT>{
            kin, vin, kout, vout, n, num_tiles, t, offsets, 0u, prefetch, bp, 0u};
      },
      hdr, smem);
}

}  // namespace gms
