// Drop-in replacement for the reference's api/multisplit_sort.cuh and
// api/multisplit_sort_pairs.cuh (7-bit multisplit radix sort):
// ms_sort_context, multisplit_sort_7bit_allocate[_pairs], multisplit_sort_7bit,
// multisplit_sort_7bit_pairs (argument order kin, kout, vin, vout),
// multisplit_sort_release_memory (src/api/multisplit_sort.cuh:100-364,
// src/api/multisplit_sort_pairs.cuh:21-65).  The ms_bucket_sort_*bit digit
// functors come from functors.cuh.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gpumultisplit/functors.cuh"

class ms_sort_context {
 public:
  void* d_temp_storage;
  size_t temp_storage_bytes;
  uint32_t* d_histogram;
  uint32_t* d_key_temp_ms;
  uint32_t* d_value_temp_ms;
  ms_sort_context()
      : d_temp_storage(NULL), temp_storage_bytes(0), d_histogram(NULL), d_key_temp_ms(NULL), d_value_temp_ms(NULL) {}
  ~ms_sort_context() {}
};

namespace gms {
namespace dropin {
inline void sort_allocate(uint32_t n, ms_sort_context& c, int key_value, int digit_bits = 7) {
  size_t bytes = 0;
  gms_status st = gms_sort_scratch_bytes(n, digit_bits, key_value, &bytes);
  if (st == GMS_SUCCESS && cudaMalloc(&c.d_temp_storage, bytes) != cudaSuccess) st = GMS_ERROR_CUDA;
  last_status() = st;
  if (st != GMS_SUCCESS) return;
  c.temp_storage_bytes = bytes;
  c.d_histogram = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(c.d_temp_storage) + 256);
}
}  // namespace dropin
}  // namespace gms

inline void multisplit_sort_7bit_allocate(uint32_t n_elements, ms_sort_context& context) {
  gms::dropin::sort_allocate(n_elements, context, 0);
}

inline void multisplit_sort_7bit_allocate_pairs(uint32_t n_elements, ms_sort_context& context) {
  gms::dropin::sort_allocate(n_elements, context, 1);
}

inline void multisplit_sort_release_memory(ms_sort_context& context) {
  if (context.d_temp_storage) cudaFree(context.d_temp_storage);
  context.d_temp_storage = NULL;
  context.d_histogram = NULL;
}

inline void multisplit_sort_7bit(uint32_t* d_key_in, uint32_t* d_key_out_ms, uint32_t n_elements,
                                 ms_sort_context& context) {
  gms::last_status() = gms_sort_7bit_key_only(d_key_in, d_key_out_ms, n_elements, context.d_temp_storage,
                                              context.temp_storage_bytes, 0);
}

inline void multisplit_sort_7bit_pairs(uint32_t* d_key_in, uint32_t* d_key_out_ms, uint32_t* d_value_in,
                                       uint32_t* d_value_out_ms, uint32_t n_elements, ms_sort_context& context) {
  gms::last_status() = gms_sort_7bit_key_value(d_key_in, d_key_out_ms, d_value_in, d_value_out_ms, n_elements,
                                               context.d_temp_storage, context.temp_storage_bytes, 0);
}

// The other digit widths (src/api/multisplit_sort.cuh:118-559, src/api/multisplit_sort_pairs.cuh:67-260).
#define GMS_DROPIN_SORT(BITS)                                                                                     \
  inline void multisplit_sort_##BITS##bit_allocate(uint32_t n_elements, ms_sort_context& context) {               \
    gms::dropin::sort_allocate(n_elements, context, 0, BITS);                                                     \
  }                                                                                                               \
  inline void multisplit_sort_##BITS##bit_allocate_pairs(uint32_t n_elements, ms_sort_context& context) {         \
    gms::dropin::sort_allocate(n_elements, context, 1, BITS);                                                     \
  }                                                                                                               \
  inline void multisplit_sort_##BITS##bit(uint32_t* d_key_in, uint32_t* d_key_out_ms, uint32_t n_elements,        \
                                          ms_sort_context& context) {                                             \
    gms::last_status() = gms_sort_key_only(d_key_in, d_key_out_ms, n_elements, BITS, context.d_temp_storage,      \
                                           context.temp_storage_bytes, 0);                                        \
  }                                                                                                               \
  inline void multisplit_sort_##BITS##bit_pairs(uint32_t* d_key_in, uint32_t* d_key_out_ms, uint32_t* d_value_in, \
                                                uint32_t* d_value_out_ms, uint32_t n_elements,                    \
                                                ms_sort_context& context) {                                       \
    gms::last_status() = gms_sort_key_value(d_key_in, d_key_out_ms, d_value_in, d_value_out_ms, n_elements, BITS, \
                                            context.d_temp_storage, context.temp_storage_bytes, 0);               \
  }
GMS_DROPIN_SORT(4)
GMS_DROPIN_SORT(5)
GMS_DROPIN_SORT(6)
GMS_DROPIN_SORT(8)
#undef GMS_DROPIN_SORT

// Stable sort by key bits [begin_bit, end_bit) with digit_bits-wide digits (an
// extension: the reference reaches partial-key sorts only through CUB,
// src/main/main_bms.cu:199).
inline void multisplit_sort_bits_allocate(uint32_t n_elements, ms_sort_context& context, int begin_bit, int end_bit,
                                          int digit_bits, bool pairs) {
  size_t bytes = 0;
  gms_status st = gms_sort_bits_scratch_bytes(n_elements, begin_bit, end_bit, digit_bits, pairs ? 1 : 0, &bytes);
  if (bytes < 256) bytes = 256;
  if (st == GMS_SUCCESS && cudaMalloc(&context.d_temp_storage, bytes) != cudaSuccess) st = GMS_ERROR_CUDA;
  gms::last_status() = st;
  if (st != GMS_SUCCESS) return;
  context.temp_storage_bytes = bytes;
  context.d_histogram = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(context.d_temp_storage) + 256);
}

inline void multisplit_sort_bits(uint32_t* d_key_in, uint32_t* d_key_out_ms, uint32_t n_elements,
                                 ms_sort_context& context, int begin_bit, int end_bit, int digit_bits) {
  gms::last_status() = gms_sort_bits_key_only(d_key_in, d_key_out_ms, n_elements, begin_bit, end_bit, digit_bits,
                                              context.d_temp_storage, context.temp_storage_bytes, 0);
}

inline void multisplit_sort_bits_pairs(uint32_t* d_key_in, uint32_t* d_key_out_ms, uint32_t* d_value_in,
                                       uint32_t* d_value_out_ms, uint32_t n_elements, ms_sort_context& context,
                                       int begin_bit, int end_bit, int digit_bits) {
  gms::last_status() =
      gms_sort_bits_key_value(d_key_in, d_key_out_ms, d_value_in, d_value_out_ms, n_elements, begin_bit, end_bit,
                              digit_bits, context.d_temp_storage, context.temp_storage_bytes, 0);
}
