// Host entry points for the histogram.  The reference exposes only kernel
// templates that callers launch themselves (multisplit2_histogram_even_* /
// _range_*, src/kernels/histogram/multisplit2_histograms.cuh:36-699, launched
// as in src/main/main_histogram.cu:163-179, 272-279); these wrap the same
// binning with any n and any bucket identifier, adding into the caller-zeroed
// int histogram on the legacy default stream.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gpumultisplit/functors.cuh"
#include "gpumultisplit/generic.cuh"

// bin = (uint32)((key - lower_level) * inverse_delta), uint32 keys, num_bins <= 256.
inline void multisplit_histogram_even(const uint32_t* d_key_in, uint32_t num_elements, int* d_histogram,
                                      uint32_t num_bins, uint32_t lower_level, uint32_t upper_level,
                                      float inverse_delta) {
  gms::last_status() = gms_histogram_even(d_key_in, num_elements, d_histogram, num_bins, lower_level, upper_level,
                                          inverse_delta, 0);
}

// bin = upper_bound(d_levels[0..num_bins), key) - 1.
inline void multisplit_histogram_range(const uint32_t* d_key_in, uint32_t num_elements, int* d_histogram,
                                       uint32_t num_bins, const uint32_t* d_levels) {
  gms::last_status() = gms_histogram_range(d_key_in, num_elements, d_histogram, num_bins, d_levels, 0);
}

// Counts per bucket of any identifier (the integer definition: the same
// buckets the multisplit would form).
template <typename KeyT, typename bucket_t>
void multisplit_histogram(const KeyT* d_key_in, uint32_t num_elements, int* d_histogram, uint32_t num_buckets,
                          bucket_t bucket_identifier) {
  static_assert(sizeof(KeyT) == 4, "32-bit keys");
  const uint32_t* keys = reinterpret_cast<const uint32_t*>(d_key_in);
  gms_bucket_desc d;
  if (gms::bucket_desc_of<bucket_t>::get(bucket_identifier, num_buckets, &d))
    gms::last_status() = gms_histogram(keys, num_elements, &d, d_histogram, 0);
  else
    gms::last_status() =
        gms::dropin::generic_histogram(keys, num_elements, num_buckets, bucket_identifier, d_histogram, 0);
}
