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

#include "gms_device.cuh"

namespace gms {

// Tile geometry of one (B, key/value) instance.
template <int LOGB_, int WARPS_, int IPT_, bool KV_>
struct TileCfg {
  static constexpr int LOGB = LOGB_;
  static constexpr uint32_t B = 1u << LOGB_;
  static constexpr int WARPS = WARPS_;
  static constexpr int THREADS = WARPS_ * 32;
  static constexpr int IPT = IPT_;  // keys per thread
  static constexpr uint32_t TILE = THREADS * IPT_;
  static constexpr bool KV = KV_;
  static constexpr uint32_t WB = B < 32 ? 32 : B;  // row width of the per-warp count table

  static_assert(IPT % 4 == 0, "IPT must be a multiple of 4 (16-byte vector loads)");
  static_assert(TILE <= 65536, "in-tile positions are packed into 16 bits");
  static_assert(THREADS >= static_cast<int>(B), "one thread per bucket in the tile scan");

  // Postscan shared-memory layout (bytes).
  static constexpr size_t OFF_K = 0;
  static constexpr size_t OFF_V = OFF_K + TILE * 4;
  static constexpr size_t OFF_R = OFF_V + (KV ? TILE * 4 : 0);
  static constexpr size_t OFF_WH = OFF_R + TILE * 4;
  static constexpr size_t OFF_DELTA = OFF_WH + size_t(WARPS) * WB * 4;
  static constexpr size_t OFF_SPLIT = OFF_DELTA + B * 4;
  static constexpr size_t OFF_SCAN = OFF_SPLIT + B * 4;
  static constexpr size_t OFF_BAR = (OFF_SCAN + B * 4 + 15) & ~size_t(15);
  static constexpr size_t POST_SMEM = OFF_BAR + 16;
};

// ------------------------------------------------------------- counting
// Counts keys into per-lane registers (B <= 32: lane l counts bucket l, from
// log2(B) ballots per 32 keys) or into a shared histogram (B > 32).
template <int LOGB, int KIND>
struct KeyCounter {
  static constexpr uint32_t B = 1u << LOGB;
  static constexpr bool kBallot = LOGB <= 5;
  Identifier<KIND, LOGB> ident;
  uint32_t* s_hist;  // B > 32
  uint32_t lane_cnt = 0;
  uint32_t xm[LOGB <= 5 ? LOGB : 1];

  __device__ __forceinline__ KeyCounter(const Identifier<KIND, LOGB>& id, uint32_t* hist) : ident(id), s_hist(hist) {
    if constexpr (kBallot) {
      const uint32_t lane = lane_id();
#pragma unroll
      for (int i = 0; i < LOGB; ++i) xm[i] = ((lane >> i) & 1u) ? 0u : ~0u;
    }
  }

  // Called by all 32 lanes of the warp together.
  __device__ __forceinline__ void add(uint32_t key, bool valid) {
    const uint32_t b = ident(key);
    if constexpr (kBallot) {
      uint32_t m = __ballot_sync(~0u, valid);
#pragma unroll
      for (int i = 0; i < LOGB; ++i) m &= __ballot_sync(~0u, (b >> i) & 1u) ^ xm[i];
      lane_cnt += __popc(m);
    } else {
      if (valid) atomicAdd(&s_hist[b], 1u);
    }
  }
};

// Count the keys keys[base .. base+cnt) of one tile of THREADS*IPT keys.
template <int THREADS, int IPT, class Counter>
__device__ __forceinline__ void count_tile(const uint32_t* __restrict__ keys, uint32_t base, uint32_t cnt,
                                           bool vec_ok, Counter& c) {
  const uint32_t tid = threadIdx.x;
  if (vec_ok && cnt == uint32_t(THREADS * IPT)) {
    uint4 v[IPT / 4];
#pragma unroll
    for (int k = 0; k < IPT / 4; ++k) v[k] = ld_nc_v4(keys + base + (uint32_t(k) * THREADS + tid) * 4u);
#pragma unroll
    for (int k = 0; k < IPT / 4; ++k) {
      c.add(v[k].x, true);
      c.add(v[k].y, true);
      c.add(v[k].z, true);
      c.add(v[k].w, true);
    }
  } else {
#pragma unroll 4
    for (int k = 0; k < IPT; ++k) {
      const uint32_t i = uint32_t(k) * THREADS + tid;
      const bool valid = i < cnt;
      const uint32_t key = valid ? keys[base + i] : 0u;
      c.add(key, valid);
    }
  }
}

// --------------------------------------------------------------- prescan
// One CTA per tile.  Writes counts[b * num_tiles + tile] and resets the scan
// state (ticket, chunk status words, error word) for the scan that follows.
template <class C, int KIND>
__global__ void __launch_bounds__(C::THREADS) prescan_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                             uint32_t num_tiles, uint32_t* __restrict__ counts,
                                                             BucketParams bp, ScratchHeader* hdr,
                                                             uint64_t* __restrict__ status, uint32_t num_chunks) {
  constexpr uint32_t B = C::B;
  __shared__ uint32_t s_hist[C::LOGB <= 5 ? C::WARPS * 32 : B];
  __shared__ uint32_t s_split[C::LOGB <= 5 ? 32 : B];  // RANGE splitters

  const uint32_t tid = threadIdx.x;
  const uint32_t tile = blockIdx.x;

  // Reset the scan state for this call.
  for (uint32_t i = tile * C::THREADS + tid; i < num_chunks; i += gridDim.x * C::THREADS) status[i] = 0ull;
  if (tile == 0 && tid == 0) {
    hdr->error = 0u;
    hdr->error_info = 0u;
    hdr->ticket = 0u;
  }

  load_splitters<KIND, C::LOGB>(s_split, bp);
  if constexpr (C::LOGB > 5) {
    for (uint32_t b = tid; b < B; b += C::THREADS) s_hist[b] = 0u;
  }
  __syncthreads();

  const uint32_t base = tile * C::TILE;
  const uint32_t cnt = min(C::TILE, n - base);
  const bool vec_ok = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0;
  Identifier<KIND, C::LOGB> ident{bp, s_split};
  KeyCounter<C::LOGB, KIND> counter(ident, s_hist);
  count_tile<C::THREADS, C::IPT>(keys, base, cnt, vec_ok, counter);

  if constexpr (C::LOGB <= 5) {
    const uint32_t lane = tid & 31u, warp = tid >> 5;
    if (lane < B) s_hist[warp * 32 + lane] = counter.lane_cnt;
    __syncthreads();
    if (tid < B) {
      uint32_t total = 0;
#pragma unroll
      for (int w = 0; w < C::WARPS; ++w) total += s_hist[w * 32 + tid];
      counts[tid * num_tiles + tile] = total;
    }
  } else {
    __syncthreads();
    for (uint32_t b = tid; b < B; b += C::THREADS) counts[b * num_tiles + tile] = s_hist[b];
  }
}

// -------------------------------------------------------------- postscan
// One CTA per tile.
//  0. bulk-copy the tile's keys (and values) into shared memory, prefetch the
//     tile's B global offsets;
//  1. per warp, stable rank of every key among same-bucket keys earlier in the
//     warp's range (warp-striped slots keep input order: slot j, lane l is
//     key w*IPT*32 + j*32 + l);
//  2. tile scan: per-warp bucket offsets and the per-bucket shift
//     delta[b] = global_offset(b, tile) - tile_start(b);
//  3. write, at each key's bucket-sorted in-tile position, its source index;
//  4. walk the bucket-sorted order: out[delta[b] + p] = key (value), so every
//     bucket's run is a contiguous, coalesced store.
template <class C, int KIND>
__global__ void __launch_bounds__(C::THREADS) postscan_kernel(
    const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
    uint32_t* __restrict__ vout, uint32_t n, uint32_t num_tiles, const uint32_t* __restrict__ offsets,
    BucketParams bp, ScratchHeader* hdr) {
  constexpr uint32_t B = C::B;
  constexpr int LOGB = C::LOGB;
  constexpr int IPT = C::IPT;
  constexpr uint32_t WB = C::WB;

  extern __shared__ __align__(128) unsigned char smem[];
  uint32_t* s_k = reinterpret_cast<uint32_t*>(smem + C::OFF_K);
  uint32_t* s_v = reinterpret_cast<uint32_t*>(smem + C::OFF_V);
  uint32_t* s_r = reinterpret_cast<uint32_t*>(smem + C::OFF_R);
  uint32_t* s_wh = reinterpret_cast<uint32_t*>(smem + C::OFF_WH);
  uint32_t* s_delta = reinterpret_cast<uint32_t*>(smem + C::OFF_DELTA);
  uint32_t* s_split = reinterpret_cast<uint32_t*>(smem + C::OFF_SPLIT);
  uint32_t* s_scan = reinterpret_cast<uint32_t*>(smem + C::OFF_SCAN);
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);

  const uint32_t tid = threadIdx.x;
  const uint32_t lane = tid & 31u;
  const uint32_t warp = tid >> 5;
  const uint32_t tile = blockIdx.x;
  const uint32_t base = tile * C::TILE;
  const uint32_t cnt = min(C::TILE, n - base);

  // ---- 0. stage the tile
  uintptr_t addr_bits = reinterpret_cast<uintptr_t>(kin);
  if constexpr (C::KV) addr_bits |= reinterpret_cast<uintptr_t>(vin);
  const uint32_t bulk = ((addr_bits & 15u) == 0) ? (cnt & ~3u) : 0u;  // elements moved by the bulk copy
  if (tid == 0 && bulk != 0) {
    mbar_init(s_bar, 1);
    fence_mbar_init();
    mbar_arrive_expect_tx(s_bar, (C::KV ? 2u : 1u) * bulk * 4u);
    bulk_copy_g2s(s_k, kin + base, bulk * 4u, s_bar);
    if constexpr (C::KV) bulk_copy_g2s(s_v, vin + base, bulk * 4u, s_bar);
  }
  for (uint32_t i = bulk + tid; i < cnt; i += C::THREADS) {
    s_k[i] = kin[base + i];
    if constexpr (C::KV) s_v[i] = vin[base + i];
  }
  const uint32_t goff = (tid < B) ? offsets[tid * num_tiles + tile] : 0u;
  load_splitters<KIND, LOGB>(s_split, bp);
  if constexpr (LOGB > 5) {
    for (uint32_t i = tid; i < C::WARPS * WB; i += C::THREADS) s_wh[i] = 0u;
  }
  __syncthreads();
  if (bulk != 0) {
    const bool ok = error_recorded(hdr) ? mbar_try_wait(s_bar, 0) : mbar_wait_bounded(s_bar, 0);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        record_error(hdr, DEV_ERR_BULK_COPY_TIMEOUT);
        mbar_wait_bounded(s_bar, 0);  // let a late copy land before the CTA exits
      }
      return;
    }
  }

  // ---- 1. stable in-warp ranks
  const Identifier<KIND, LOGB> ident{bp, s_split};
  uint32_t packed[IPT];  // (bucket << 16) | rank among same-bucket keys of this warp
  const uint32_t wbase = warp * (IPT * 32u);
  const uint32_t lt = lanemask_lt();
  if constexpr (LOGB <= 5) {
    uint32_t xm[LOGB];
#pragma unroll
    for (int i = 0; i < LOGB; ++i) xm[i] = ((lane >> i) & 1u) ? 0u : ~0u;
    uint32_t my_cnt = 0;  // keys of bucket `lane` seen so far by this warp
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      const uint32_t pos = wbase + uint32_t(j) * 32u + lane;
      const bool valid = pos < cnt;
      const uint32_t b = ident(s_k[pos]);
      uint32_t m = __ballot_sync(~0u, valid);  // -> lanes holding bucket `lane`
#pragma unroll
      for (int i = 0; i < LOGB; ++i) m &= __ballot_sync(~0u, (b >> i) & 1u) ^ xm[i];
      const uint32_t peers = __shfl_sync(~0u, m, b);
      const uint32_t before = __shfl_sync(~0u, my_cnt, b);
      packed[j] = (b << 16) | (before + __popc(peers & lt));
      my_cnt += __popc(m);
    }
    if (lane < B) s_wh[warp * WB + lane] = my_cnt;
  } else {
    uint32_t* wh = s_wh + warp * WB;
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      const uint32_t pos = wbase + uint32_t(j) * 32u + lane;
      const bool valid = pos < cnt;
      const uint32_t b = ident(s_k[pos]);
      uint32_t peers = __ballot_sync(~0u, valid);
#pragma unroll
      for (int i = 0; i < LOGB; ++i) {
        const uint32_t bal = __ballot_sync(~0u, (b >> i) & 1u);
        peers &= ((b >> i) & 1u) ? bal : ~bal;
      }
      const uint32_t rank = __popc(peers & lt);
      const uint32_t before = wh[b];
      __syncwarp();
      if (valid && rank == 0) wh[b] = before + __popc(peers);
      __syncwarp();
      packed[j] = (b << 16) | (before + rank);
    }
  }
  __syncthreads();

  // ---- 2. tile scan
  if (tid < B) {
    uint32_t running = 0;
#pragma unroll
    for (int w = 0; w < C::WARPS; ++w) {
      const uint32_t c = s_wh[w * WB + tid];
      s_wh[w * WB + tid] = running;
      running += c;
    }
    s_scan[tid] = running;
  }
  __syncthreads();
  if (warp == 0) {
    constexpr uint32_t PER = (B + 31) / 32;
    uint32_t v[PER];
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < PER; ++k) {
      const uint32_t idx = lane * PER + k;
      v[k] = idx < B ? s_scan[idx] : 0u;
      sum += v[k];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(~0u, incl, d);
      if (lane >= uint32_t(d)) incl += t;
    }
    uint32_t excl = incl - sum;
#pragma unroll
    for (uint32_t k = 0; k < PER; ++k) {
      const uint32_t idx = lane * PER + k;
      if (idx < B) s_scan[idx] = excl;
      excl += v[k];
    }
  }
  __syncthreads();
  if (tid < B) {
    const uint32_t start = s_scan[tid];
    s_delta[tid] = goff - start;
#pragma unroll
    for (int w = 0; w < C::WARPS; ++w) s_wh[w * WB + tid] += start;
  }
  __syncthreads();

  // ---- 3. bucket-sorted in-tile order
  bool bad = false;
  {
    const uint32_t* wh = s_wh + warp * WB;
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      const uint32_t pos = wbase + uint32_t(j) * 32u + lane;
      if (pos < cnt) {
        const uint32_t b = packed[j] >> 16;
        const uint32_t d = wh[b] + (packed[j] & 0xFFFFu);
        if (d < cnt)
          s_r[d] = (b << 16) | pos;
        else
          bad = true;
      }
    }
  }
  __syncthreads();

  // ---- 4. scatter (positions are checked: a corrupt offset is reported, never written)
#pragma unroll
  for (int j = 0; j < IPT; ++j) {
    const uint32_t p = uint32_t(j) * C::THREADS + tid;
    if (p < cnt) {
      const uint32_t e = s_r[p];
      const uint32_t src = e & 0xFFFFu;
      const uint32_t g = s_delta[(e >> 16) & (B - 1)] + p;
      if (g < n && src < cnt) {
        kout[g] = s_k[src];
        if constexpr (C::KV) vout[g] = s_v[src];
      } else {
        bad = true;
      }
    }
  }
  if (bad) record_error(hdr, DEV_ERR_BAD_OFFSET);
}

}  // namespace gms
