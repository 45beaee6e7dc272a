/*
 * CPU oracle for the multisplit hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU algorithms, used by the tests,
 * by the smoke check and as the timed CPU baseline.  The library never calls
 * it.  Each function cites the reference code it restates (paths inside the
 * owensgroup/GpuMultisplit tree).  It is pinned against the reference's own
 * CPU multisplit compiled from its sources (oracle/ref_shim.cpp) through the
 * committed golden vectors in tests/golden/.
 */
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* Bucket identifier for B buckets (any B in [2, 256]).  Every kind is reduced
 * modulo B: the reference's GPU kernels decode the bucket from its low log2(B)
 * bits with ballots (src/kernels/bms/bms_prescan.cuh:480-517), which is the
 * same reduction for the powers of two the reference takes.
 *   DELTA       key * B >> 32                     (equal-width ranges; < B)
 *   DIV         key / param                       (delta_func, src/main/main_multisplit.cu:41-47)
 *   BITS        (key >> shift)                    (ms_bucket_sort_*bit, src/api/multisplit_sort.cuh:63-98)
 *   RANGE       upper_bound(splitters, B, key) - 1, with -1 read as B-1
 *                                               (src/kernels/histogram/multisplit2_histograms.cuh:434)
 *   MASK        (key & param) != 0
 *   EVEN_FLOAT  (uint32)((float)(key - lower) * inverse_delta)
 *                                               (src/kernels/histogram/multisplit2_histograms.cuh:60)
 */
uint32_t oracle_bucket(const oracle_desc* d, uint32_t key) {
  const uint32_t B = d->num_buckets;
  switch (d->kind) {
    case ORACLE_DELTA:
      return (uint32_t)(((uint64_t)key * B) >> 32);
    case ORACLE_DIV:
      return (key / d->param) % B;
    case ORACLE_BITS:
      return (d->shift >= 32u ? 0u : (key >> d->shift)) % B;
    case ORACLE_RANGE: {
      /* upper_bound: first index whose splitter is > key. */
      uint32_t lo = 0, hi = B;
      while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2u;
        if (d->splitters[mid] <= key)
          lo = mid + 1u;
        else
          hi = mid;
      }
      return lo == 0u ? B - 1u : lo - 1u;
    }
    case ORACLE_MASK:
      return (key & d->param) ? 1u : 0u;
    case ORACLE_EVEN_FLOAT: {
      /* uint32 -> float and float * float in round-to-nearest-even (the host
       * default and CUDA's __uint2float_rn / __fmul_rn), then a truncating
       * conversion that saturates like the GPU's cvt.rzi.u32.f32. */
      const float x = (float)(uint32_t)(key - d->lower) * d->inverse_delta;
      uint32_t b;
      if (!(x > 0.0f))
        b = 0u; /* negative, zero or NaN */
      else if (x >= 4294967296.0f)
        b = 0xFFFFFFFFu;
      else
        b = (uint32_t)x;
      return b % B;
    }
    default:
      return 0u;
  }
}

/* Histogram -> exclusive scan -> stable placement: cpu_multisplit_general and
 * cpu_multisplit_pairs_general (src/cpu_functions.h:155-288).  vin/vout may be
 * NULL (key-only).  offsets (B entries) receives the bucket starts if non-NULL. */
static void multisplit(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                       const oracle_desc* d, uint32_t* offsets) {
  const uint32_t B = d->num_buckets;
  uint32_t* bins = (uint32_t*)calloc(B, sizeof(uint32_t));
  uint32_t* next = (uint32_t*)calloc(B, sizeof(uint32_t));
  for (uint32_t i = 0; i < n; ++i) bins[oracle_bucket(d, kin[i])]++;
  uint32_t run = 0;
  for (uint32_t b = 0; b < B; ++b) {
    next[b] = run;
    run += bins[b];
  }
  if (offsets) memcpy(offsets, next, B * sizeof(uint32_t));
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t b = oracle_bucket(d, kin[i]);
    const uint32_t dst = next[b]++;
    kout[dst] = kin[i];
    if (vin) vout[dst] = vin[i];
  }
  free(bins);
  free(next);
}

void oracle_multisplit_keys(const uint32_t* kin, uint32_t* kout, uint32_t n, const oracle_desc* d,
                            uint32_t* offsets) {
  multisplit(kin, kout, NULL, NULL, n, d, offsets);
}

void oracle_multisplit_pairs(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                             const oracle_desc* d, uint32_t* offsets) {
  multisplit(kin, kout, vin, vout, n, d, offsets);
}

/* Per-tile bucket counts, bucket-major: counts[b * num_tiles + t] -- the layout
 * checked by cpu_prescan_test (src/cpu_functions.h:55-103) and written by the
 * prescan kernels (src/kernels/bms/bms_prescan.cuh:114).  Keys past n are not
 * counted. */
void oracle_tile_counts(const uint32_t* kin, uint32_t n, const oracle_desc* d, uint32_t tile, uint32_t* counts) {
  const uint32_t num_tiles = (uint32_t)(((uint64_t)n + tile - 1) / tile);
  memset(counts, 0, sizeof(uint32_t) * (size_t)num_tiles * d->num_buckets);
  for (uint32_t i = 0; i < n; ++i) counts[(size_t)oracle_bucket(d, kin[i]) * num_tiles + i / tile]++;
}

/* Adds per-bucket counts into hist (the reference's histogram kernels add into
 * a caller-zeroed int array with atomics, multisplit2_histograms.cuh:88,389). */
void oracle_histogram(const uint32_t* kin, uint32_t n, const oracle_desc* d, int32_t* hist) {
  for (uint32_t i = 0; i < n; ++i) hist[oracle_bucket(d, kin[i])]++;
}

/* Multisplit radix sorts: stable multisplits on successive bit fields, least
 * significant first, with the reference's digit schedules
 * (src/api/multisplit_sort.cuh:320-559, src/api/multisplit_sort_pairs.cuh:21-260):
 *   4: eight 4-bit digits; 5: six 5-bit digits then bits [30,32);
 *   6: 4, 4, then four 6-bit digits; 7: 4 then four 7-bit digits; 8: four 8-bit.
 * tmp_k/tmp_v hold n entries; returns 0, or -1 for an unknown width. */
int oracle_sort(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                uint32_t* tmp_k, uint32_t* tmp_v, int digit_bits) {
  static const uint32_t shifts[9][8] = {{0}, {0}, {0}, {0}, {0, 4, 8, 12, 16, 20, 24, 28},
                                        {0, 5, 10, 15, 20, 25, 30}, {0, 4, 8, 14, 20, 26},
                                        {0, 4, 11, 18, 25}, {0, 8, 16, 24}};
  static const uint32_t buckets[9][8] = {{0}, {0}, {0}, {0}, {16, 16, 16, 16, 16, 16, 16, 16},
                                         {32, 32, 32, 32, 32, 32, 4}, {16, 16, 64, 64, 64, 64},
                                         {16, 128, 128, 128, 128}, {256, 256, 256, 256}};
  static const int passes[9] = {0, 0, 0, 0, 8, 7, 6, 5, 4};
  if (digit_bits < 4 || digit_bits > 8) return -1;
  const uint32_t* src_k = kin;
  const uint32_t* src_v = vin;
  const int P = passes[digit_bits];
  for (int p = 0; p < P; ++p) {
    /* the last pass writes the output buffer, earlier ones alternate */
    const int to_out = ((P - 1 - p) % 2) == 0;
    uint32_t* dk = to_out ? kout : tmp_k;
    uint32_t* dv = to_out ? vout : tmp_v;
    oracle_desc d;
    memset(&d, 0, sizeof(d));
    d.kind = ORACLE_BITS;
    d.num_buckets = buckets[digit_bits][p];
    d.shift = shifts[digit_bits][p];
    multisplit(src_k, dk, vin ? src_v : NULL, vin ? dv : NULL, n, &d, NULL);
    src_k = dk;
    src_v = dv;
  }
  return 0;
}

/* Stable sort by key bits [begin_bit, end_bit): multisplits on digits of
 * digit_bits bits from begin_bit, the last one narrower (the partial-key form
 * of the CUB radix sorts the reference's drivers use, src/main/main_bms.cu:199).
 * begin_bit == end_bit copies.  Returns 0, or -1 for an invalid range. */
int oracle_sort_bits(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                     uint32_t* tmp_k, uint32_t* tmp_v, int begin_bit, int end_bit, int digit_bits) {
  if (digit_bits < 4 || digit_bits > 8 || begin_bit < 0 || end_bit > 32 || begin_bit > end_bit) return -1;
  const int P = (end_bit - begin_bit + digit_bits - 1) / digit_bits;
  if (P == 0) {
    memcpy(kout, kin, sizeof(uint32_t) * n);
    if (vin) memcpy(vout, vin, sizeof(uint32_t) * n);
    return 0;
  }
  const uint32_t* src_k = kin;
  const uint32_t* src_v = vin;
  for (int p = 0; p < P; ++p) {
    const int shift = begin_bit + p * digit_bits;
    const int w = end_bit - shift < digit_bits ? end_bit - shift : digit_bits;
    const int to_out = ((P - 1 - p) % 2) == 0;
    uint32_t* dk = to_out ? kout : tmp_k;
    uint32_t* dv = to_out ? vout : tmp_v;
    oracle_desc d;
    memset(&d, 0, sizeof(d));
    d.kind = ORACLE_BITS;
    d.num_buckets = 1u << w;
    d.shift = (uint32_t)shift;
    multisplit(src_k, dk, vin ? src_v : NULL, vin ? dv : NULL, n, &d, NULL);
    src_k = dk;
    src_v = dv;
  }
  return 0;
}

void oracle_sort_7bit(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                      uint32_t* tmp_k, uint32_t* tmp_v) {
  oracle_sort(kin, kout, vin, vout, n, tmp_k, tmp_v, 7);
}

/* Two-bucket stable multisplit; returns the bucket-0 count
 * (src/kernels/compaction/multisplit2_compaction.cuh:525-573). */
uint32_t oracle_compaction(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                           const oracle_desc* d) {
  uint32_t offsets[2];
  multisplit(kin, kout, vin, vout, n, d, offsets);
  return n == 0 ? 0u : offsets[1];
}

/* ---------------------------------------------------------------------
 * Multi-threaded restatement (CPU baseline): the same stable result from P
 * contiguous chunks -- per-chunk histograms, an exclusive scan in
 * (bucket, chunk) order, then each chunk scatters its own keys in order.
 */
typedef struct {
  const uint32_t* kin;
  uint32_t* kout;
  const uint32_t* vin;
  uint32_t* vout;
  const oracle_desc* d;
  uint32_t begin, end;
  uint32_t* counts; /* B entries for this chunk: counts, then write cursors */
  int phase;
} mt_job;

static void* mt_worker(void* arg) {
  mt_job* j = (mt_job*)arg;
  if (j->phase == 0) {
    memset(j->counts, 0, sizeof(uint32_t) * j->d->num_buckets);
    for (uint32_t i = j->begin; i < j->end; ++i) j->counts[oracle_bucket(j->d, j->kin[i])]++;
  } else {
    for (uint32_t i = j->begin; i < j->end; ++i) {
      const uint32_t dst = j->counts[oracle_bucket(j->d, j->kin[i])]++;
      j->kout[dst] = j->kin[i];
      if (j->vin) j->vout[dst] = j->vin[i];
    }
  }
  return NULL;
}

void oracle_multisplit_mt(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                          const oracle_desc* d, int threads) {
  if (threads < 1) threads = 1;
  if ((uint32_t)threads > n / 4096u + 1u) threads = (int)(n / 4096u + 1u);
  const uint32_t B = d->num_buckets;
  mt_job* jobs = (mt_job*)calloc((size_t)threads, sizeof(mt_job));
  pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
  uint32_t* counts = (uint32_t*)calloc((size_t)threads * B, sizeof(uint32_t));
  const uint64_t per = ((uint64_t)n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    uint64_t b = per * t, e = b + per;
    if (b > n) b = n;
    if (e > n) e = n;
    jobs[t] = (mt_job){kin, kout, vin, vout, d, (uint32_t)b, (uint32_t)e, counts + (size_t)t * B, 0};
  }
  for (int phase = 0; phase < 2; ++phase) {
    if (phase == 1) {
      uint32_t run = 0;
      for (uint32_t b = 0; b < B; ++b)
        for (int t = 0; t < threads; ++t) {
          const uint32_t c = counts[(size_t)t * B + b];
          counts[(size_t)t * B + b] = run;
          run += c;
        }
    }
    for (int t = 0; t < threads; ++t) {
      jobs[t].phase = phase;
      if (t == 0) continue;
      pthread_create(&tid[t], NULL, mt_worker, &jobs[t]);
    }
    mt_worker(&jobs[0]);
    for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
  }
  free(counts);
  free(tid);
  free(jobs);
}

/* splitmix64 keys (seed, i) -> uint32, the generator of gpumultisplit_gb300/datagen.py,
 * so the oracle can build large inputs without Python. */
void oracle_uniform_u32(uint32_t* out, uint64_t n, uint64_t seed) {
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    out[i] = (uint32_t)(z >> 32);
  }
}

/* ---------------------------------------------------------------------
 * 64-bit keys.  The reference's multisplit holds 32-bit keys only
 * (src/kernels/bms/bms_postscan.cuh:38); this restates its CPU algorithm
 * (histogram -> exclusive scan -> stable placement, src/cpu_functions.h:155-288)
 * for 64-bit keys, with every identifier kind on the key's full width.
 * Values are moved as opaque elements of value_bytes (0 = key-only, 4 or 8).
 */
uint32_t oracle_bucket64(const oracle_desc64* d, uint64_t key) {
  const uint32_t B = d->num_buckets;
  switch (d->kind) {
    case ORACLE_DELTA: {
      /* key * B >> 64: the high word of the 128-bit product, from 32-bit halves. */
      const uint64_t lo = (key & 0xFFFFFFFFull) * B, hi = (key >> 32) * B;
      return (uint32_t)((hi + (lo >> 32)) >> 32);
    }
    case ORACLE_DIV:
      return (uint32_t)((key / d->param) % B);
    case ORACLE_BITS:
      return (uint32_t)((d->shift >= 64u ? 0u : (key >> d->shift)) % B);
    case ORACLE_RANGE: {
      uint32_t lo = 0, hi = B;
      while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2u;
        if (d->splitters[mid] <= key)
          lo = mid + 1u;
        else
          hi = mid;
      }
      return lo == 0u ? B - 1u : lo - 1u;
    }
    case ORACLE_MASK:
      return (key & d->param) ? 1u : 0u;
    case ORACLE_EVEN_FLOAT: {
      /* uint64 -> float (round to nearest even, as __ull2float_rn), float
       * multiply, saturating truncation: as for 32-bit keys. */
      const float x = (float)(uint64_t)(key - d->lower) * d->inverse_delta;
      uint32_t b;
      if (!(x > 0.0f))
        b = 0u;
      else if (x >= 4294967296.0f)
        b = 0xFFFFFFFFu;
      else
        b = (uint32_t)x;
      return b % B;
    }
    default:
      return 0u;
  }
}

void oracle_multisplit64(const uint64_t* kin, uint64_t* kout, const void* vin, void* vout, int value_bytes,
                         uint32_t n, const oracle_desc64* d, uint32_t* offsets) {
  const uint32_t B = d->num_buckets;
  uint32_t* bins = (uint32_t*)calloc(B, sizeof(uint32_t));
  uint32_t* next = (uint32_t*)calloc(B, sizeof(uint32_t));
  for (uint32_t i = 0; i < n; ++i) bins[oracle_bucket64(d, kin[i])]++;
  uint32_t run = 0;
  for (uint32_t b = 0; b < B; ++b) {
    next[b] = run;
    run += bins[b];
  }
  if (offsets) memcpy(offsets, next, B * sizeof(uint32_t));
  const size_t vb = (size_t)value_bytes;
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t dst = next[oracle_bucket64(d, kin[i])]++;
    kout[dst] = kin[i];
    if (vb) memcpy((char*)vout + (size_t)dst * vb, (const char*)vin + (size_t)i * vb, vb);
  }
  free(bins);
  free(next);
}

/* Stable sort of 64-bit keys by bits [begin_bit, end_bit), end_bit <= 64, in
 * digits of digit_bits bits, least significant first (the last one narrower).
 * tmp_k / tmp_v hold n elements.  Returns 0, or -1 for an invalid range. */
int oracle_sort_bits64(const uint64_t* kin, uint64_t* kout, const void* vin, void* vout, int value_bytes, uint32_t n,
                       uint64_t* tmp_k, void* tmp_v, int begin_bit, int end_bit, int digit_bits) {
  if (digit_bits < 4 || digit_bits > 8 || begin_bit < 0 || end_bit > 64 || begin_bit > end_bit) return -1;
  const int P = (end_bit - begin_bit + digit_bits - 1) / digit_bits;
  if (P == 0) {
    memcpy(kout, kin, sizeof(uint64_t) * n);
    if (value_bytes) memcpy(vout, vin, (size_t)value_bytes * n);
    return 0;
  }
  const uint64_t* src_k = kin;
  const void* src_v = vin;
  for (int p = 0; p < P; ++p) {
    const int shift = begin_bit + p * digit_bits;
    const int w = end_bit - shift < digit_bits ? end_bit - shift : digit_bits;
    const int to_out = ((P - 1 - p) % 2) == 0;
    uint64_t* dk = to_out ? kout : tmp_k;
    void* dv = to_out ? vout : tmp_v;
    oracle_desc64 d;
    memset(&d, 0, sizeof(d));
    d.kind = ORACLE_BITS;
    d.num_buckets = 1u << w;
    d.shift = (uint32_t)shift;
    oracle_multisplit64(src_k, dk, src_v, dv, value_bytes, n, &d, NULL);
    src_k = dk;
    src_v = dv;
  }
  return 0;
}

/* Adds the per-bucket counts of 64-bit keys into hist (as oracle_histogram). */
void oracle_histogram64(const uint64_t* kin, uint32_t n, const oracle_desc64* d, int32_t* hist) {
  for (uint32_t i = 0; i < n; ++i) hist[oracle_bucket64(d, kin[i])]++;
}
