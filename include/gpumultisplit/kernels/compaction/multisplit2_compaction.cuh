// Drop-in replacement for the reference's
// kernels/compaction/multisplit2_compaction.cuh host API
// (src/kernels/compaction/multisplit2_compaction.cuh:477-573): a stable
// two-bucket multisplit, bucket 0 first, returning the number of bucket-0 keys
// (synchronously, like the reference).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gpumultisplit/functors.cuh"
#include "gpumultisplit/generic.cuh"

class compaction_context {
 public:
  void* d_temp_storage;
  size_t temp_storage_bytes;
  uint32_t* d_histogram;
  compaction_context() : d_temp_storage(NULL), temp_storage_bytes(0), d_histogram(NULL) {}
  ~compaction_context() {}
};

namespace gms {
namespace dropin {
inline void compaction_allocate(uint32_t n, compaction_context& c, int key_value) {
  size_t bytes = 0;
  gms_status st = gms_compaction_scratch_bytes(n, key_value, &bytes);
  if (st == GMS_SUCCESS && cudaMalloc(&c.d_temp_storage, bytes) != cudaSuccess) st = GMS_ERROR_CUDA;
  last_status() = st;
  if (st != GMS_SUCCESS) return;
  c.temp_storage_bytes = bytes;
  c.d_histogram = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(c.d_temp_storage) + 256);
}

template <typename KeyT, typename ValueT, typename bucket_t>
unsigned int compaction_run(const KeyT* kin, const ValueT* vin, KeyT* kout, ValueT* vout, uint32_t n,
                            compaction_context& c, const bucket_t& f) {
  static_assert(sizeof(KeyT) == 4 && sizeof(ValueT) == 4, "32-bit keys and values");
  const uint32_t* k_in = reinterpret_cast<const uint32_t*>(kin);
  const uint32_t* v_in = reinterpret_cast<const uint32_t*>(vin);
  uint32_t* k_out = reinterpret_cast<uint32_t*>(kout);
  uint32_t* v_out = reinterpret_cast<uint32_t*>(vout);
  uint32_t n0 = 0;
  gms_bucket_desc d;
  gms_status st;
  if (bucket_desc_of<bucket_t>::get(f, 2, &d)) {
    st = v_in ? gms_compaction_key_value(k_in, v_in, k_out, v_out, n, &d, c.d_temp_storage, c.temp_storage_bytes,
                                         &n0, 0)
              : gms_compaction_key_only(k_in, k_out, n, &d, c.d_temp_storage, c.temp_storage_bytes, &n0, 0);
  } else {
    uint32_t offsets[2] = {0, 0};
    st = generic_multisplit(k_in, v_in, k_out, v_out, n, 2, f, c.d_temp_storage, c.temp_storage_bytes, offsets,
                            cudaStream_t(0));
    n0 = n == 0 ? 0 : offsets[1];
  }
  last_status() = st;
  return st == GMS_SUCCESS ? n0 : 0;
}
}  // namespace dropin
}  // namespace gms

inline void compaction_allocate_key_only(uint32_t numElements, compaction_context& context) {
  gms::dropin::compaction_allocate(numElements, context, 0);
}

inline void compaction_allocate_key_value(uint32_t numElements, compaction_context& context) {
  gms::dropin::compaction_allocate(numElements, context, 1);
}

inline void compaction_release_memory(compaction_context& context) {
  if (context.d_temp_storage) cudaFree(context.d_temp_storage);
  context.d_temp_storage = NULL;
  context.d_histogram = NULL;
}

template <typename key_t, typename bucket_t>
unsigned int compaction_key_only(key_t* d_key_in, key_t* d_key_out, uint32_t numElements, compaction_context& context,
                                 bucket_t bucket_identifier) {
  return gms::dropin::compaction_run<key_t, key_t, bucket_t>(d_key_in, (const key_t*)NULL, d_key_out, (key_t*)NULL,
                                                             numElements, context, bucket_identifier);
}

template <typename key_t, typename value_t, typename bucket_t>
unsigned int compaction_key_value(key_t* d_key_in, value_t* d_value_in, key_t* d_key_out, value_t* d_value_out,
                                  uint32_t numElements, compaction_context& context, bucket_t bucket_identifier) {
  return gms::dropin::compaction_run<key_t, value_t, bucket_t>(d_key_in, d_value_in, d_key_out, d_value_out,
                                                               numElements, context, bucket_identifier);
}
