// Device-side building blocks shared by every kernel of the library:
// PTX wrappers (mbarrier, bulk async copy, relaxed global accesses), bounded
// waits that record an error instead of hanging, the scratch header, and the
// bucket identifiers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

// Counts per thread of the look-back scan (a chunk is 256 threads x this).
#ifndef GMS_SCAN_IPT
#define GMS_SCAN_IPT 16
#endif

namespace gms {

// ----------------------------------------------------------------- errors
enum DeviceError : uint32_t {
  DEV_OK = 0,
  DEV_ERR_BULK_COPY_TIMEOUT = 1,  // a bulk copy into shared memory did not complete in time
  DEV_ERR_LOOKBACK_TIMEOUT = 2,   // a scan look-back waited too long for a predecessor
  DEV_ERR_BAD_OFFSET = 3,         // a computed position fell outside the tile or the output (not written)
};

// First 256 bytes of every scratch buffer.
struct ScratchHeader {
  uint32_t error;          // first DeviceError recorded in the current call
  uint32_t error_info;     // block that recorded it
  uint32_t ticket;         // scan chunk ticket counter
  uint32_t wait_limit_us;  // bound of every wait of the current call in microseconds (0: kWaitLimitNs)
  uint32_t reserved[60];
};
static_assert(sizeof(ScratchHeader) == 256, "header is 256 bytes");

// Default wall-clock bound for every spin in the library (nanoseconds).  A
// call's prescan resets the header's wait_limit_us to 0, which selects it; a
// shorter bound written between the stages of one call applies to that call's
// scan and postscan.
constexpr uint64_t kWaitLimitNs = 1000000000ull;  // 1 s

__device__ __forceinline__ uint64_t wait_limit_ns(const ScratchHeader* h) {
  const uint32_t us = *reinterpret_cast<const volatile uint32_t*>(&h->wait_limit_us);
  return us != 0u ? uint64_t(us) * 1000ull : kWaitLimitNs;
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void record_error(ScratchHeader* h, uint32_t code) {
  if (atomicCAS(&h->error, 0u, code) == 0u) h->error_info = blockIdx.x;
}

// True once any block of the current call has recorded an error; later blocks
// then skip their waits so a failing call ends quickly.
__device__ __forceinline__ bool error_recorded(const ScratchHeader* h) {
  return *reinterpret_cast<const volatile uint32_t*>(&h->error) != 0u;
}

// ------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Invalidate an mbarrier whose phases are all complete, before its memory is
// initialised again.
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Make an initialised mbarrier visible to the async (bulk copy) proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Wait for phase `parity` of an mbarrier, giving up after the call's wait
// limit (the header's, read only when the first try fails).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, const ScratchHeader* h) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t limit = wait_limit_ns(h);
  const uint64_t t0 = global_timer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_timer_ns() - t0 > limit) return false;
  }
}

// One-dimensional bulk copy global -> shared (the TMA engine's non-tensor path).
// dst and src 16-byte aligned, bytes a multiple of 16; completion is signalled
// on `bar` as transaction bytes.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// An L2 policy that marks the lines an access touches evict-first: data read
// or written once, which should not push reusable lines out of L2.
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// bulk_copy_g2s with an L2 cache policy for the source lines.
__device__ __forceinline__ void bulk_copy_g2s_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                                   uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

__device__ __forceinline__ void st_global_hint(uint32_t* p, uint32_t v, uint64_t policy) {
  asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(policy) : "memory");
}

// Prefetch [src, src + bytes) into L2 (no completion tracking); src 16-byte
// aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void st_relaxed_u64(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization may start while the previous kernel on its stream runs;
// griddep_wait() then blocks until that kernel has completed and its writes are
// visible (a no-op for a kernel launched the ordinary way).
// griddep_launch_dependents() lets the next such kernel start once every block
// of this one has called it or exited.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;"); }

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add_u32(uint32_t* p, uint32_t v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Orders this thread's generic-proxy global accesses with its later (or
// earlier) async-proxy ones: bulk copies that read data other blocks wrote.
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

__device__ __forceinline__ uint4 ld_nc_v4(const uint32_t* p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// ----------------------------------------------------- bucket identifiers
// Kinds mirror gms_bucket_kind in include/gpumultisplit.h.
enum BucketKind : int {
  KIND_DELTA = 0,
  KIND_DIV = 1,
  KIND_BITS = 2,
  KIND_RANGE = 3,
  KIND_MASK = 4,
  KIND_EVEN_FLOAT = 5,
  NUM_KINDS = 6
};

// B = num_buckets may be any count in [2, 256]; the kernels run with
// 2^LOGB >= B buckets, the ones from B up staying empty.
struct BucketParams {
  uint32_t shift;
  uint32_t param;
  uint32_t lower;
  float inverse_delta;
  const uint32_t* splitters;  // RANGE only (device memory, B entries)
  uint32_t num_buckets;       // B
};

// v modulo b (b >= 2): a mask for powers of two, a division otherwise.
__device__ __forceinline__ uint32_t reduce_mod(uint32_t v, uint32_t b) {
  return (b & (b - 1)) == 0 ? (v & (b - 1)) : (v % b);
}

// RANGE identifiers narrow each search with a table over the key's top
// RANGE_LUT_BITS bits.  Entry t packs lo(t) | lo(t+1) << 16, where lo(t) is the
// number of splitters below t << (32 - bits) (lo(CELLS) = B): a key in cell t
// has between lo(t) and lo(t+1) splitters <= it.  With 1024 cells a cell holds
// a splitter for at most B/1024 of the keys, so most keys need one table load
// and no search.
constexpr int RANGE_LUT_BITS = 10;
constexpr uint32_t RANGE_LUT_CELLS = 1u << RANGE_LUT_BITS;
// Up to this many buckets the splitters are compared one by one (no table).
constexpr uint32_t RANGE_SCAN_MAX_B = 8;

// Shared words an identifier needs (splitters + lookup table for RANGE).
template <int KIND, int LOGB>
__host__ __device__ constexpr uint32_t identifier_smem_words() {
  return KIND != KIND_RANGE ? 1u : ((1u << LOGB) <= RANGE_SCAN_MAX_B ? (1u << LOGB) : (1u << LOGB) + RANGE_LUT_CELLS);
}

// A bucket identifier for B = 2^LOGB buckets.  `s_split` is the shared-memory
// area filled by prepare_identifier() (RANGE only).
template <int KIND, int LOGB>
struct Identifier {
  static constexpr uint32_t B = 1u << LOGB;
  BucketParams p;
  const uint32_t* s_split;

  __device__ __forceinline__ uint32_t operator()(uint32_t key) const {
    if constexpr (KIND == KIND_DELTA) {
      // key * B >> 32: the high word of the 64-bit product (the top LOGB bits
      // of the key when B = 2^LOGB).
      return __umulhi(key, p.num_buckets);
    } else if constexpr (KIND == KIND_DIV) {
      return reduce_mod(key / p.param, p.num_buckets);
    } else if constexpr (KIND == KIND_BITS) {
      return (key >> p.shift) & (B - 1);
    } else if constexpr (KIND == KIND_RANGE) {
      // c = number of splitters <= key (upper_bound); bucket = c - 1, which
      // wraps to B-1 when key < s[0].
      // With B below 2^LOGB the splitter area is padded with 0xFFFFFFFF, so
      // c is clamped to B.
      if constexpr (B <= RANGE_SCAN_MAX_B) {
        // Few splitters: compare against all of them (same address for every
        // lane, so each load is a broadcast).
        uint32_t c = 0;
#pragma unroll
        for (uint32_t i = 0; i < B; ++i) c += s_split[i] <= key ? 1u : 0u;
        c = min(c, p.num_buckets);
        return c == 0u ? p.num_buckets - 1u : c - 1u;
      } else {
        // The table bounds c to [lo(t), lo(t+1)].  Only keys whose cell holds
        // a splitter load it (a predicated load: lanes in empty cells add no
        // shared-memory traffic); only cells with two or more splitters need a
        // search over the rest.
        const uint32_t e = s_split[B + (key >> (32 - RANGE_LUT_BITS))];
        uint32_t c = e & 0xFFFFu, hi = e >> 16;
        uint32_t s0 = 0;
        if (c < hi) s0 = s_split[c];
        const bool past_first = c < hi && s0 <= key;
        c += past_first ? 1u : 0u;
        if (past_first && c < hi) {
          while (c < hi) {
            const uint32_t mid = (c + hi + 1) >> 1;
            if (s_split[mid - 1] <= key)
              c = mid;
            else
              hi = mid - 1;
          }
        }
        c = min(c, p.num_buckets);
        return c == 0u ? p.num_buckets - 1u : c - 1u;
      }
    } else if constexpr (KIND == KIND_MASK) {
      return (key & p.param) ? 1u : 0u;
    } else {  // KIND_EVEN_FLOAT
      const float x = __fmul_rn(__uint2float_rn(key - p.lower), p.inverse_delta);
      return reduce_mod(__float2uint_rz(x), p.num_buckets);
    }
  }
};

// Fill the identifier's shared area (RANGE: splitters, then the lookup table).
// No-op for other kinds.  All threads of the block must call it; a barrier
// must follow before the identifier is used.
template <int KIND, int LOGB>
__device__ __forceinline__ void prepare_identifier(uint32_t* s_split, const BucketParams& p) {
  if constexpr (KIND == KIND_RANGE) {
    constexpr uint32_t B = 1u << LOGB;
    constexpr uint32_t SHIFT = 32 - RANGE_LUT_BITS;
    for (uint32_t i = threadIdx.x; i < B; i += blockDim.x) s_split[i] = i < p.num_buckets ? p.splitters[i] : ~0u;
    __syncthreads();
    if constexpr (B <= RANGE_SCAN_MAX_B) return;
    uint32_t* lut = s_split + B;
    // Each thread fills a run of consecutive cells: one binary search for the
    // run's first cell, then a walk over the (sorted) splitters of the run.
    const uint32_t per = (RANGE_LUT_CELLS + blockDim.x - 1) / blockDim.x;
    const uint32_t t0 = threadIdx.x * per;
    if (t0 < RANGE_LUT_CELLS) {
      const uint32_t v = t0 << SHIFT;
      uint32_t lo = 0, hi = B;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s_split[mid] < v)
          lo = mid + 1;
        else
          hi = mid;
      }
      const uint32_t t1 = min(t0 + per, RANGE_LUT_CELLS);
      for (uint32_t t = t0; t < t1; ++t) {
        uint32_t next = lo;
        if (t + 1 == RANGE_LUT_CELLS) {
          next = B;
        } else {
          const uint32_t end = (t + 1) << SHIFT;
          while (next < B && s_split[next] < end) ++next;
        }
        lut[t] = lo | (next << 16);
        lo = next;
      }
    }
  }
}

// Identifier policies: what the kernels need to know about a bucket
// identifier.  DescPolicy covers the precompiled descriptor kinds; the drop-in
// C++ headers use FunctorPolicy to instantiate the same kernels with any
// device-callable functor, compiled in the caller's translation unit.
template <int KIND, int LOGB>
struct DescPolicy {
  using Params = BucketParams;
  using Id = Identifier<KIND, LOGB>;
  static constexpr bool CHEAP = KIND == KIND_DELTA || KIND == KIND_BITS || KIND == KIND_MASK;
  static constexpr bool USES_SMEM = KIND == KIND_RANGE;
  static constexpr uint32_t SMEM_WORDS = identifier_smem_words<KIND, LOGB>();
  __device__ __forceinline__ static void prepare(uint32_t* s, const Params& p) { prepare_identifier<KIND, LOGB>(s, p); }
  __device__ __forceinline__ static Id make(const Params& p, const uint32_t* s) { return Id{p, s}; }
};

// ------------------------------------------------ 64-bit key identifiers
// The same six kinds over 64-bit keys.  They run in the prescan only: the
// postscan of 64-bit keys always reads the bucket bytes the prescan stored.
struct BucketParams64 {
  uint64_t param;               // DIV: divisor; MASK: mask
  uint64_t lower;               // EVEN_FLOAT: lower level
  const uint64_t* splitters;    // RANGE: B sorted splitters (device memory)
  float inverse_delta;          // EVEN_FLOAT
  uint32_t shift;               // BITS: 0..63
  uint32_t num_buckets;         // B
};

// Shared words of a 64-bit identifier: RANGE keeps 2^LOGB splitters (two
// words each) and, above RANGE_SCAN_MAX_B, a table over the key's top
// RANGE_LUT_BITS bits, entry t = lo(t) | lo(t+1) << 16 as for 32-bit keys.
template <int KIND, int LOGB>
__host__ __device__ constexpr uint32_t identifier64_smem_words() {
  return KIND != KIND_RANGE ? 1u
                            : ((1u << LOGB) <= RANGE_SCAN_MAX_B ? 2u * (1u << LOGB)
                                                                 : 2u * (1u << LOGB) + RANGE_LUT_CELLS);
}

template <int KIND, int LOGB>
struct Identifier64 {
  static constexpr uint32_t B = 1u << LOGB;
  BucketParams64 p;
  const uint32_t* s_split;

  __device__ __forceinline__ uint32_t operator()(uint64_t key) const {
    if constexpr (KIND == KIND_DELTA) {
      // key * B >> 64: the high word of the 128-bit product.
      return uint32_t(__umul64hi(key, uint64_t(p.num_buckets)));
    } else if constexpr (KIND == KIND_DIV) {
      const uint64_t q = key / p.param;
      return (p.num_buckets & (p.num_buckets - 1)) == 0 ? uint32_t(q) & (p.num_buckets - 1)
                                                        : uint32_t(q % p.num_buckets);
    } else if constexpr (KIND == KIND_BITS) {
      return uint32_t(key >> p.shift) & (B - 1);
    } else if constexpr (KIND == KIND_RANGE) {
      const uint64_t* s = reinterpret_cast<const uint64_t*>(s_split);
      uint32_t c = 0, hi = B;
      if constexpr (B > RANGE_SCAN_MAX_B) {
        const uint32_t e = s_split[2 * B + uint32_t(key >> (64 - RANGE_LUT_BITS))];
        c = e & 0xFFFFu;
        hi = e >> 16;
      }
      // upper_bound over s[c, hi): the first splitter above the key.
      while (c < hi) {
        const uint32_t mid = (c + hi) >> 1;
        if (s[mid] <= key)
          c = mid + 1;
        else
          hi = mid;
      }
      c = min(c, p.num_buckets);
      return c == 0u ? p.num_buckets - 1u : c - 1u;
    } else if constexpr (KIND == KIND_MASK) {
      return (key & p.param) ? 1u : 0u;
    } else {  // KIND_EVEN_FLOAT
      const float x = __fmul_rn(__ull2float_rn(key - p.lower), p.inverse_delta);
      return reduce_mod(__float2uint_rz(x), p.num_buckets);
    }
  }
};

// Fill a 64-bit identifier's shared area (RANGE only; padded to 2^LOGB
// splitters with the largest key).  All threads call; a barrier must follow.
template <int KIND, int LOGB>
__device__ __forceinline__ void prepare_identifier64(uint32_t* s_split, const BucketParams64& p) {
  if constexpr (KIND == KIND_RANGE) {
    constexpr uint32_t B = 1u << LOGB;
    uint64_t* s = reinterpret_cast<uint64_t*>(s_split);
    for (uint32_t i = threadIdx.x; i < B; i += blockDim.x) s[i] = i < p.num_buckets ? p.splitters[i] : ~0ull;
    __syncthreads();
    if constexpr (B <= RANGE_SCAN_MAX_B) return;
    uint32_t* lut = s_split + 2 * B;
    for (uint32_t t = threadIdx.x; t < RANGE_LUT_CELLS; t += blockDim.x) {
      // lo(v) = number of splitters below v, for the first keys of cells t and t + 1.
      auto below = [&](uint64_t v) {
        uint32_t lo = 0, hi = B;
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (s[mid] < v)
            lo = mid + 1;
          else
            hi = mid;
        }
        return lo;
      };
      const uint32_t a = below(uint64_t(t) << (64 - RANGE_LUT_BITS));
      const uint32_t b = t + 1 == RANGE_LUT_CELLS ? B : below(uint64_t(t + 1) << (64 - RANGE_LUT_BITS));
      lut[t] = a | (b << 16);
    }
  }
}

template <int KIND, int LOGB>
struct DescPolicy64 {
  using Params = BucketParams64;
  using Id = Identifier64<KIND, LOGB>;
  static constexpr bool CHEAP = false;  // 64-bit keys always keep their buckets as bytes
  static constexpr bool USES_SMEM = KIND == KIND_RANGE;
  static constexpr uint32_t SMEM_WORDS = identifier64_smem_words<KIND, LOGB>();
  __device__ __forceinline__ static void prepare(uint32_t* s, const Params& p) {
    prepare_identifier64<KIND, LOGB>(s, p);
  }
  __device__ __forceinline__ static Id make(const Params& p, const uint32_t* s) { return Id{p, s}; }
};

// ------------------------------------------- more than 256 buckets
// B from 257 to 65536 (RANGE: to GMS_RANGE_BIG_MAX splitters) runs as two
// stable multisplits on the digits of the bucket id, least significant first:
// the low half of its bits, then the rest.  Stable passes make the result the
// multisplit by the whole id.  DigitId returns digit (id >> shift) of the id,
// 2^LOGB values wide.
#ifndef GMS_RANGE_BIG_MAX
#define GMS_RANGE_BIG_MAX 8192
#endif
constexpr uint32_t BIG_MAX_BUCKETS = 65536;

struct BucketParamsBig {
  BucketParams base;     // base.num_buckets = B, the whole bucket count
  uint32_t digit_shift;  // 0 for the low digit, its width for the high one
};

// Shared words of the full identifier: RANGE keeps up to GMS_RANGE_BIG_MAX
// splitters, then a table over the key's top RANGE_LUT_BITS bits (entry t =
// lo(t) | lo(t+1) << 16, lo(t) the splitters below the cell's first key).
template <int KIND>
__host__ __device__ constexpr uint32_t big_identifier_smem_words() {
  return KIND == KIND_RANGE ? GMS_RANGE_BIG_MAX + RANGE_LUT_CELLS : 1u;
}

// The whole bucket id of a key, in [0, B).
template <int KIND>
__device__ __forceinline__ uint32_t big_bucket_id(uint32_t key, const BucketParams& p, const uint32_t* s_split) {
  const uint32_t B = p.num_buckets;
  if constexpr (KIND == KIND_DELTA) {
    return __umulhi(key, B);
  } else if constexpr (KIND == KIND_DIV) {
    return reduce_mod(key / p.param, B);
  } else if constexpr (KIND == KIND_BITS) {
    return (key >> p.shift) & (B - 1);
  } else if constexpr (KIND == KIND_RANGE) {
    const uint32_t e = s_split[GMS_RANGE_BIG_MAX + (key >> (32 - RANGE_LUT_BITS))];
    uint32_t c = e & 0xFFFFu, hi = e >> 16;
    while (c < hi) {  // upper_bound over the cell's splitters
      const uint32_t mid = (c + hi) >> 1;
      if (s_split[mid] <= key)
        c = mid + 1;
      else
        hi = mid;
    }
    return c == 0u ? B - 1u : c - 1u;
  } else if constexpr (KIND == KIND_MASK) {
    return (key & p.param) ? 1u : 0u;
  } else {  // KIND_EVEN_FLOAT
    const float x = __fmul_rn(__uint2float_rn(key - p.lower), p.inverse_delta);
    return reduce_mod(__float2uint_rz(x), B);
  }
}

// Fill the full identifier's shared area (RANGE: B splitters and the table).
// All threads call; a barrier must follow.
template <int KIND>
__device__ __forceinline__ void prepare_big_identifier(uint32_t* s_split, const BucketParams& p) {
  if constexpr (KIND == KIND_RANGE) {
    const uint32_t B = p.num_buckets;
    for (uint32_t i = threadIdx.x; i < B; i += blockDim.x) s_split[i] = p.splitters[i];
    __syncthreads();
    uint32_t* lut = s_split + GMS_RANGE_BIG_MAX;
    for (uint32_t t = threadIdx.x; t < RANGE_LUT_CELLS; t += blockDim.x) {
      auto below = [&](uint32_t v) {  // splitters < v
        uint32_t lo = 0, hi = B;
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (s_split[mid] < v)
            lo = mid + 1;
          else
            hi = mid;
        }
        return lo;
      };
      const uint32_t a = below(t << (32 - RANGE_LUT_BITS));
      const uint32_t b = t + 1 == RANGE_LUT_CELLS ? B : below((t + 1) << (32 - RANGE_LUT_BITS));
      lut[t] = a | (b << 16);
    }
  }
}

template <int KIND, int LOGB>
struct DigitId {
  BucketParams p;
  uint32_t shift;
  const uint32_t* s_split;
  __device__ __forceinline__ uint32_t operator()(uint32_t key) const {
    return (big_bucket_id<KIND>(key, p, s_split) >> shift) & ((1u << LOGB) - 1u);
  }
};

// Policy of one digit pass: the digit is computed once, in the prescan, and
// kept as a byte for the postscan.
template <int KIND, int LOGB>
struct DigitPolicy {
  using Params = BucketParamsBig;
  using Id = DigitId<KIND, LOGB>;
  static constexpr bool CHEAP = false;
  static constexpr bool USES_SMEM = KIND == KIND_RANGE;
  static constexpr uint32_t SMEM_WORDS = big_identifier_smem_words<KIND>();
  __device__ __forceinline__ static void prepare(uint32_t* s, const Params& p) {
    prepare_big_identifier<KIND>(s, p.base);
  }
  __device__ __forceinline__ static Id make(const Params& p, const uint32_t* s) { return Id{p.base, p.digit_shift, s}; }
};

// The postscan of a digit pass reads the prescan's bytes only; one policy
// serves every identifier kind.
struct GivenBytesId {
  __device__ __forceinline__ uint32_t operator()(uint32_t) const { return 0u; }
};
struct GivenBytesPolicy {
  using Params = BucketParamsBig;
  using Id = GivenBytesId;
  static constexpr bool CHEAP = false;
  static constexpr bool USES_SMEM = false;
  static constexpr uint32_t SMEM_WORDS = 1;
  __device__ __forceinline__ static void prepare(uint32_t*, const Params&) {}
  __device__ __forceinline__ static Id make(const Params&, const uint32_t*) { return Id{}; }
};

// A user functor (operator() on a 32-bit key, returning the bucket); its
// value is reduced modulo B like every other identifier.
template <class F, int LOGB>
struct FunctorId {
  F f;
  __device__ __forceinline__ uint32_t operator()(uint32_t key) const {
    return uint32_t(f(key)) & ((1u << LOGB) - 1u);
  }
};

template <class F, int LOGB>
struct FunctorPolicy {
  using Params = F;
  using Id = FunctorId<F, LOGB>;
  static constexpr bool CHEAP = false;  // cost unknown: buckets are computed once per key and kept
  static constexpr bool USES_SMEM = false;
  static constexpr uint32_t SMEM_WORDS = 1;
  __device__ __forceinline__ static void prepare(uint32_t*, const Params&) {}
  __device__ __forceinline__ static Id make(const Params& f, const uint32_t*) { return Id{f}; }
};

}  // namespace gms
