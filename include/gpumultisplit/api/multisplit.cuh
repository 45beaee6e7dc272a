// Drop-in replacement for the reference's api/multisplit.cuh
// (src/api/multisplit.cuh:29-313): same class, function names, argument order
// and meaning, on libgpumultisplit.so.
//
//   #include "api/multisplit.cuh"      // with -I <repo>/include/gpumultisplit -I <repo>/include
//   multisplit_context ctx(num_buckets);
//   multisplit_allocate_key_value(n, ctx);
//   multisplit_key_value(d_kin, d_vin, d_kout, d_vout, n, ctx, bucket_identifier);
//   multisplit_release_memory(ctx);
//
// Functors the library knows (delta_func, ms_bucket_sort_*bit, gms::*_bucket)
// run the precompiled kernels; any other functor instantiates them here (this
// translation unit must then be compiled by nvcc with
// -I <repo>/gpumultisplit_gb300/csrc).  Calls run on the legacy default stream,
// as in the reference, and return void; multisplit_last_error() reports the
// status of the last call.  Unlike the reference the definitions are inline,
// so the header can be included by several translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "gpumultisplit/functors.cuh"
#include "gpumultisplit/generic.cuh"

class multisplit_context {
 public:
  uint32_t size_sub_prob;
  uint32_t num_sub_prob;
  uint32_t num_blocks;
  uint32_t num_buckets;
  void* d_temp_storage;
  size_t temp_storage_bytes;
  uint32_t* d_histogram;  // bucket-major count matrix inside d_temp_storage (global offsets after a call)

  multisplit_context(uint32_t n_buckets)
      : size_sub_prob(0), num_sub_prob(0), num_blocks(0), num_buckets(n_buckets), d_temp_storage(NULL),
        temp_storage_bytes(0), d_histogram(NULL) {}
  ~multisplit_context() {}
};

namespace gms {
namespace dropin {

inline void allocate(uint32_t n, multisplit_context& c, int key_value) {
  size_t bytes = 0, matrix_off = 0;
  uint32_t tile = 0, tiles = 0;
  // The reference takes powers of two from 2 to 256 only (src/api/multisplit.cuh:91-137);
  // the C ABI also takes other counts, these headers keep the reference's rule.
  const uint32_t b = c.num_buckets;
  gms_status st = (b < 2 || b > 256 || (b & (b - 1)) != 0) ? GMS_ERROR_UNSUPPORTED_BUCKETS : GMS_SUCCESS;
  if (st == GMS_SUCCESS) st = gms_multisplit_scratch_bytes(n, c.num_buckets, key_value, &bytes);
  if (st == GMS_SUCCESS) st = gms_multisplit_geometry(n, c.num_buckets, key_value, &tile, &tiles, &matrix_off);
  last_status() = st;
  if (st != GMS_SUCCESS) {
    printf("Error: not a correct number of buckets.\n");
    return;
  }
  c.size_sub_prob = tile;
  c.num_sub_prob = tiles;
  c.num_blocks = tiles;
  c.temp_storage_bytes = bytes;
  if (cudaMalloc(&c.d_temp_storage, bytes) != cudaSuccess || cudaMemset(c.d_temp_storage, 0, 256) != cudaSuccess) {
    last_status() = GMS_ERROR_CUDA;
    c.d_temp_storage = NULL;
    return;
  }
  c.d_histogram = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(c.d_temp_storage) + matrix_off);
}

template <typename KeyT, typename ValueT, typename bucket_t>
void run(const KeyT* kin, const ValueT* vin, KeyT* kout, ValueT* vout, uint32_t n, multisplit_context& c,
         const bucket_t& f, uint32_t* offsets) {
  static_assert(sizeof(KeyT) == 4, "keys are 32-bit");
  const uint32_t* k_in = reinterpret_cast<const uint32_t*>(kin);
  const uint32_t* v_in = reinterpret_cast<const uint32_t*>(vin);
  uint32_t* k_out = reinterpret_cast<uint32_t*>(kout);
  uint32_t* v_out = reinterpret_cast<uint32_t*>(vout);
  gms_bucket_desc d;
  gms_status st;
  if (bucket_desc_of<bucket_t>::get(f, c.num_buckets, &d)) {
    st = v_in ? gms_multisplit_key_value(k_in, v_in, k_out, v_out, n, &d, c.d_temp_storage, c.temp_storage_bytes,
                                         offsets, 0)
              : gms_multisplit_key_only(k_in, k_out, n, &d, c.d_temp_storage, c.temp_storage_bytes, offsets, 0);
  } else {
    st = generic_multisplit(k_in, v_in, k_out, v_out, n, c.num_buckets, f, c.d_temp_storage, c.temp_storage_bytes,
                            offsets, cudaStream_t(0));
  }
  last_status() = st;
  if (st == GMS_ERROR_UNSUPPORTED_BUCKETS) printf("Error: not a correct number of buckets.\n");
}

}  // namespace dropin
}  // namespace gms

// ==== Memory allocations for multisplit (key-only or key-value): src/api/multisplit.cuh:50-74
inline void multisplit_allocate_key_only(uint32_t num_elements, multisplit_context& context) {
  gms::dropin::allocate(num_elements, context, 0);
}

inline void multisplit_allocate_key_value(uint32_t num_elements, multisplit_context& context) {
  gms::dropin::allocate(num_elements, context, 1);
}

inline void multisplit_release_memory(multisplit_context& context) {
  if (context.d_temp_storage) cudaFree(context.d_temp_storage);
  context.d_temp_storage = NULL;
  context.d_histogram = NULL;
}

// src/api/multisplit.cuh:81-197
template <typename KeyT, typename bucket_t>
void multisplit_key_only(KeyT* d_key_in, KeyT* d_key_out, uint32_t num_elements, multisplit_context& context,
                         bucket_t bucket_identifier, uint32_t* multisplit_offset = NULL) {
  gms::dropin::run<KeyT, KeyT, bucket_t>(d_key_in, (const KeyT*)NULL, d_key_out, (KeyT*)NULL, num_elements, context,
                                        bucket_identifier, multisplit_offset);
}

// src/api/multisplit.cuh:199-313
template <typename KeyT, typename ValueT, typename bucket_t>
void multisplit_key_value(KeyT* d_key_in, ValueT* d_value_in, KeyT* d_key_out, ValueT* d_value_out,
                          uint32_t num_elements, multisplit_context& context, bucket_t bucket_identifier,
                          uint32_t* multisplit_offset = NULL) {
  static_assert(sizeof(ValueT) == 4, "values are 32-bit");
  gms::dropin::run<KeyT, ValueT, bucket_t>(d_key_in, d_value_in, d_key_out, d_value_out, num_elements, context,
                                          bucket_identifier, multisplit_offset);
}
