// Bucket identifiers for the drop-in C++ API, and how a functor reaches the
// library.
//
// The reference passes any functor `uint32_t operator()(KeyT) const` to its
// kernel templates (src/api/multisplit.cuh:81-88).  Here:
//   * the functor types below (and the reference's ms_bucket_sort_*bit,
//     delta_func) map onto a gms_bucket_desc and run the precompiled kernels
//     of libgpumultisplit.so through the C ABI;
//   * any other functor type instantiates the same kernels in the caller's
//     translation unit (compile it with nvcc and -I <repo>/gpumultisplit_gb300/csrc).
// Either way the bucket id is reduced modulo B.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>

#include "gpumultisplit.h"

// ------------------------------------------------------------------ functors
// delta_func of the reference's README and drivers (README.md:85-91): a / delta.
struct delta_func {
  delta_func(uint32_t delta) : delta_(delta) {}
  uint32_t delta_;
  __forceinline__ __device__ __host__ uint32_t operator()(uint32_t a) const { return a / delta_; }
};

// Digit functors of the multisplit sort (src/api/multisplit_sort.cuh:63-98).
#define GMS_DEFINE_SORT_FUNCTOR(NAME, MASK)                                                   \
  template <uint32_t x, typename key_type>                                                    \
  struct NAME {                                                                               \
    __forceinline__ __device__ __host__ uint32_t operator()(key_type a) const {             \
      return uint32_t((a >> x) & MASK);                                                       \
    }                                                                                         \
  };
GMS_DEFINE_SORT_FUNCTOR(ms_bucket_sort_2bit, 0x03)
GMS_DEFINE_SORT_FUNCTOR(ms_bucket_sort_4bit, 0x0F)
GMS_DEFINE_SORT_FUNCTOR(ms_bucket_sort_5bit, 0x1F)
GMS_DEFINE_SORT_FUNCTOR(ms_bucket_sort_6bit, 0x3F)
GMS_DEFINE_SORT_FUNCTOR(ms_bucket_sort_7bit, 0x7F)
GMS_DEFINE_SORT_FUNCTOR(ms_bucket_sort_8bit, 0xFF)
#undef GMS_DEFINE_SORT_FUNCTOR

namespace gms {

// key * B >> 32 (B equal-width ranges of the key space).
struct delta_bucket {
  uint32_t num_buckets;
  __forceinline__ __device__ __host__ uint32_t operator()(uint32_t a) const {
    return uint32_t((uint64_t(a) * num_buckets) >> 32);
  }
};

// key >> shift (the library reduces it modulo B).
struct bits_bucket {
  uint32_t shift;
  __forceinline__ __device__ __host__ uint32_t operator()(uint32_t a) const { return shift >= 32 ? 0u : a >> shift; }
};

// (key & mask) != 0.
struct mask_bucket {
  uint32_t mask;
  __forceinline__ __device__ __host__ uint32_t operator()(uint32_t a) const { return (a & mask) ? 1u : 0u; }
};

// upper_bound(splitters[0..B), key) - 1, splitters in device memory (no host-side operator).
struct range_bucket {
  const uint32_t* d_splitters;
};

// (uint32)((float)(key - lower) * inverse_delta), truncating and saturating.
struct even_float_bucket {
  uint32_t lower;
  float inverse_delta;
  __forceinline__ __device__ __host__ uint32_t operator()(uint32_t a) const {
    const float x = float(a - lower) * inverse_delta;
    return !(x > 0.0f) ? 0u : (x >= 4294967296.0f ? 0xFFFFFFFFu : uint32_t(x));
  }
};

// Maps a functor to a descriptor: get() returns false for functor types (or
// bucket counts) the library has no descriptor for; those take the
// in-translation-unit path.
template <class F>
struct bucket_desc_of {
  static bool get(const F&, uint32_t, gms_bucket_desc*) { return false; }
};

inline gms_bucket_desc make_desc(int32_t kind, uint32_t b) {
  gms_bucket_desc d{};
  d.kind = kind;
  d.num_buckets = b;
  return d;
}

template <>
struct bucket_desc_of<delta_func> {
  static bool get(const delta_func& f, uint32_t b, gms_bucket_desc* d) {
    *d = make_desc(GMS_BUCKET_DIV, b);
    d->param = f.delta_;
    return f.delta_ != 0;
  }
};

template <>
struct bucket_desc_of<delta_bucket> {
  static bool get(const delta_bucket& f, uint32_t b, gms_bucket_desc* d) {
    // The DELTA kind uses the call's B; a functor built for another B is a different identifier.
    *d = make_desc(GMS_BUCKET_DELTA, b);
    return f.num_buckets == b;
  }
};

template <>
struct bucket_desc_of<bits_bucket> {
  static bool get(const bits_bucket& f, uint32_t b, gms_bucket_desc* d) {
    *d = make_desc(GMS_BUCKET_BITS, b);
    d->shift = f.shift;
    return true;
  }
};

template <>
struct bucket_desc_of<mask_bucket> {
  static bool get(const mask_bucket& f, uint32_t b, gms_bucket_desc* d) {
    *d = make_desc(GMS_BUCKET_MASK, b);
    d->param = f.mask;
    return true;
  }
};

template <>
struct bucket_desc_of<range_bucket> {
  static bool get(const range_bucket& f, uint32_t b, gms_bucket_desc* d) {
    *d = make_desc(GMS_BUCKET_RANGE, b);
    d->d_splitters = f.d_splitters;
    return true;
  }
};

template <>
struct bucket_desc_of<even_float_bucket> {
  static bool get(const even_float_bucket& f, uint32_t b, gms_bucket_desc* d) {
    *d = make_desc(GMS_BUCKET_EVEN_FLOAT, b);
    d->lower = f.lower;
    d->inverse_delta = f.inverse_delta;
    return true;
  }
};

// A sort digit (x, mask) is a BITS descriptor when B covers the mask exactly.
#define GMS_SORT_FUNCTOR_DESC(NAME, MASK)                                       \
  template <uint32_t x, typename key_type>                                      \
  struct bucket_desc_of<NAME<x, key_type>> {                                    \
    static bool get(const NAME<x, key_type>&, uint32_t b, gms_bucket_desc* d) { \
      *d = make_desc(GMS_BUCKET_BITS, b);                                       \
      d->shift = x;                                                             \
      return b == uint32_t(MASK) + 1u;                                          \
    }                                                                           \
  };
GMS_SORT_FUNCTOR_DESC(ms_bucket_sort_2bit, 0x03)
GMS_SORT_FUNCTOR_DESC(ms_bucket_sort_4bit, 0x0F)
GMS_SORT_FUNCTOR_DESC(ms_bucket_sort_5bit, 0x1F)
GMS_SORT_FUNCTOR_DESC(ms_bucket_sort_6bit, 0x3F)
GMS_SORT_FUNCTOR_DESC(ms_bucket_sort_7bit, 0x7F)
GMS_SORT_FUNCTOR_DESC(ms_bucket_sort_8bit, 0xFF)
#undef GMS_SORT_FUNCTOR_DESC

// Status of the last drop-in call on this thread (the reference's functions return void).
inline gms_status& last_status() {
  static thread_local gms_status s = GMS_SUCCESS;
  return s;
}

}  // namespace gms

inline gms_status multisplit_last_error() { return gms::last_status(); }
