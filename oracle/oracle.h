/* CPU oracle for the multisplit hot path -- test infrastructure only (see oracle.c). */
#ifndef GMS_ORACLE_H_
#define GMS_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORACLE_DELTA = 0,
  ORACLE_DIV = 1,
  ORACLE_BITS = 2,
  ORACLE_RANGE = 3,
  ORACLE_MASK = 4,
  ORACLE_EVEN_FLOAT = 5
};

/* Same field order as gms_bucket_desc (splitters are host memory here). */
typedef struct oracle_desc {
  int32_t kind;
  uint32_t num_buckets;
  uint32_t shift;
  uint32_t param;
  uint32_t lower;
  float inverse_delta;
  const uint32_t* splitters;
} oracle_desc;

uint32_t oracle_bucket(const oracle_desc* d, uint32_t key);
void oracle_multisplit_keys(const uint32_t* kin, uint32_t* kout, uint32_t n, const oracle_desc* d,
                            uint32_t* offsets);
void oracle_multisplit_pairs(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                             const oracle_desc* d, uint32_t* offsets);
void oracle_tile_counts(const uint32_t* kin, uint32_t n, const oracle_desc* d, uint32_t tile, uint32_t* counts);
void oracle_histogram(const uint32_t* kin, uint32_t n, const oracle_desc* d, int32_t* hist);
int oracle_sort(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                uint32_t* tmp_k, uint32_t* tmp_v, int digit_bits);
int oracle_sort_bits(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                     uint32_t* tmp_k, uint32_t* tmp_v, int begin_bit, int end_bit, int digit_bits);
void oracle_sort_7bit(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                      uint32_t* tmp_k, uint32_t* tmp_v);
uint32_t oracle_compaction(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                           const oracle_desc* d);
void oracle_multisplit_mt(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                          const oracle_desc* d, int threads);
void oracle_uniform_u32(uint32_t* out, uint64_t n, uint64_t seed);

/* 64-bit keys; same field order as gms_bucket_desc64 (splitters on the host). */
typedef struct oracle_desc64 {
  int32_t kind;
  uint32_t num_buckets;
  uint32_t shift;
  float inverse_delta;
  uint64_t param;
  uint64_t lower;
  const uint64_t* splitters;
} oracle_desc64;

uint32_t oracle_bucket64(const oracle_desc64* d, uint64_t key);
void oracle_multisplit64(const uint64_t* kin, uint64_t* kout, const void* vin, void* vout, int value_bytes,
                         uint32_t n, const oracle_desc64* d, uint32_t* offsets);
void oracle_histogram64(const uint64_t* kin, uint32_t n, const oracle_desc64* d, int32_t* hist);
int oracle_sort_bits64(const uint64_t* kin, uint64_t* kout, const void* vin, void* vout, int value_bytes, uint32_t n,
                       uint64_t* tmp_k, void* tmp_v, int begin_bit, int end_bit, int digit_bits);

#ifdef __cplusplus
}
#endif

#endif
