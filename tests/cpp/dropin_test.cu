// Parity driver for the drop-in C++ API, in the style of the reference's
// src/main/main_multisplit.cu / main_sort.cu / main_compaction.cu: random
// inputs, one library call, a CPU stable multisplit as the check.  Exercises
// both the precompiled path (functors with a descriptor) and the
// in-translation-unit path (user functors).  Prints "ALL PASSED" on success.
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "api/multisplit.cuh"
#include "api/multisplit_histogram.cuh"
#include "api/multisplit_sort.cuh"
#include "kernels/compaction/multisplit2_compaction.cuh"

// User functors the library has no descriptor for.
struct hash_bucket {  // multiplicative hash, top 8 bits
  __host__ __device__ uint32_t operator()(uint32_t a) const { return (a * 2654435761u) >> 24; }
};
template <uint32_t flag, typename key_type>
struct test_bucket {  // src/main/main_compaction.cu:26-31
  __host__ __device__ uint32_t operator()(key_type a) const { return a & ((1u << flag) - 1u); }
};
struct mod_bucket {  // key % 5 into 8 buckets (3 left empty)
  uint32_t m;
  __host__ __device__ uint32_t operator()(uint32_t a) const { return a % m; }
};

static uint64_t rng_state = 0x1234567ull;
static uint32_t next_u32() {  // splitmix64
  uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return uint32_t((z ^ (z >> 31)) >> 32);
}

// The CPU stable multisplit every check compares against.
template <class F>
static void cpu_multisplit(const std::vector<uint32_t>& k, const std::vector<uint32_t>& v, std::vector<uint32_t>& ko,
                           std::vector<uint32_t>& vo, uint32_t B, F f, std::vector<uint32_t>* offsets = nullptr) {
  std::vector<uint32_t> cnt(B, 0), pos(B, 0);
  for (uint32_t x : k) cnt[f(x) & (B - 1)]++;
  for (uint32_t b = 1; b < B; ++b) pos[b] = pos[b - 1] + cnt[b - 1];
  if (offsets) *offsets = pos;
  ko.assign(k.size(), 0);
  vo.assign(v.size(), 0);
  for (size_t i = 0; i < k.size(); ++i) {
    const uint32_t d = pos[f(k[i]) & (B - 1)]++;
    ko[d] = k[i];
    if (!v.empty()) vo[d] = v[i];
  }
}

static int failures = 0;
#define CHECK(cond, what)                           \
  do {                                              \
    if (!(cond)) {                                  \
      printf("FAILED: %s (line %d)\n", what, __LINE__); \
      ++failures;                                   \
    }                                               \
  } while (0)

struct DeviceArrays {
  uint32_t *k, *v, *ko, *vo;
  explicit DeviceArrays(size_t n) {
    cudaMalloc(&k, 4 * std::max<size_t>(n, 1));
    cudaMalloc(&v, 4 * std::max<size_t>(n, 1));
    cudaMalloc(&ko, 4 * std::max<size_t>(n, 1));
    cudaMalloc(&vo, 4 * std::max<size_t>(n, 1));
  }
  ~DeviceArrays() {
    cudaFree(k);
    cudaFree(v);
    cudaFree(ko);
    cudaFree(vo);
  }
};

static std::vector<uint32_t> download(const uint32_t* d, size_t n) {
  std::vector<uint32_t> h(n);
  if (n) cudaMemcpy(h.data(), d, 4 * n, cudaMemcpyDeviceToHost);
  return h;
}

template <class F>
static void test_multisplit(const char* name, uint32_t n, uint32_t B, F f) {
  std::vector<uint32_t> k(n), v(n);
  for (uint32_t i = 0; i < n; ++i) {
    k[i] = next_u32();
    v[i] = i;  // values = original index pins value stability
  }
  DeviceArrays d(n);
  cudaMemcpy(d.k, k.data(), 4 * n, cudaMemcpyHostToDevice);
  cudaMemcpy(d.v, v.data(), 4 * n, cudaMemcpyHostToDevice);
  std::vector<uint32_t> rk, rv, roffs;
  cpu_multisplit(k, v, rk, rv, B, f, &roffs);

  multisplit_context ctx(B);
  multisplit_allocate_key_value(n, ctx);
  std::vector<uint32_t> offs(B, 0);
  multisplit_key_value(d.k, d.v, d.ko, d.vo, n, ctx, f, offs.data());
  cudaDeviceSynchronize();
  CHECK(multisplit_last_error() == GMS_SUCCESS, name);
  CHECK(download(d.ko, n) == rk, name);
  CHECK(download(d.vo, n) == rv, name);
  CHECK(offs == roffs, name);
  multisplit_release_memory(ctx);

  multisplit_context ctx2(B);
  multisplit_allocate_key_only(n, ctx2);
  multisplit_key_only(d.k, d.ko, n, ctx2, f);
  cudaDeviceSynchronize();
  CHECK(multisplit_last_error() == GMS_SUCCESS, name);
  CHECK(download(d.ko, n) == rk, name);
  multisplit_release_memory(ctx2);
  printf("multisplit %-28s n=%u B=%u\n", name, n, B);
}

struct SortFns {
  int bits;
  void (*allocate)(uint32_t, ms_sort_context&);
  void (*allocate_pairs)(uint32_t, ms_sort_context&);
  void (*keys)(uint32_t*, uint32_t*, uint32_t, ms_sort_context&);
  void (*pairs)(uint32_t*, uint32_t*, uint32_t*, uint32_t*, uint32_t, ms_sort_context&);
};
#define SORT_FNS(B) \
  SortFns { B, multisplit_sort_##B##bit_allocate, multisplit_sort_##B##bit_allocate_pairs, multisplit_sort_##B##bit, \
            multisplit_sort_##B##bit_pairs }

static void test_sort(uint32_t n, bool and4, SortFns fns = SORT_FNS(7)) {
  std::vector<uint32_t> k(n), v(n);
  for (uint32_t i = 0; i < n; ++i) {
    k[i] = and4 ? (next_u32() & next_u32() & next_u32() & next_u32()) : next_u32();
    v[i] = i;
  }
  std::vector<uint32_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0u);
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return k[a] < k[b]; });
  std::vector<uint32_t> rk(n);
  for (uint32_t i = 0; i < n; ++i) rk[i] = k[idx[i]];
  DeviceArrays d(n);
  cudaMemcpy(d.k, k.data(), 4 * n, cudaMemcpyHostToDevice);
  cudaMemcpy(d.v, v.data(), 4 * n, cudaMemcpyHostToDevice);
  ms_sort_context ctx;
  fns.allocate_pairs(n, ctx);
  fns.pairs(d.k, d.ko, d.v, d.vo, n, ctx);  // reference order: kin, kout, vin, vout
  cudaDeviceSynchronize();
  CHECK(multisplit_last_error() == GMS_SUCCESS, "sort pairs");
  CHECK(download(d.ko, n) == rk, "sort pairs keys");
  CHECK(download(d.vo, n) == idx, "sort pairs values (stable)");
  multisplit_sort_release_memory(ctx);
  ms_sort_context ctx2;
  fns.allocate(n, ctx2);
  fns.keys(d.k, d.ko, n, ctx2);
  cudaDeviceSynchronize();
  CHECK(download(d.ko, n) == rk, "sort keys");
  CHECK(download(d.k, n) == k, "sort leaves its input untouched");
  multisplit_sort_release_memory(ctx2);
  printf("sort %d-bit n=%u %s\n", fns.bits, n, and4 ? "and4" : "uniform");
}

static void test_sort_bits(uint32_t n, int begin, int end, int digit) {
  std::vector<uint32_t> k(n), v(n);
  for (uint32_t i = 0; i < n; ++i) {
    k[i] = next_u32();
    v[i] = i;
  }
  const uint32_t mask = end - begin >= 32 ? 0xFFFFFFFFu : ((1u << (end - begin)) - 1u);
  std::vector<uint32_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0u);
  std::stable_sort(idx.begin(), idx.end(),
                   [&](uint32_t a, uint32_t b) { return ((k[a] >> begin) & mask) < ((k[b] >> begin) & mask); });
  std::vector<uint32_t> rk(n);
  for (uint32_t i = 0; i < n; ++i) rk[i] = k[idx[i]];
  DeviceArrays d(n);
  cudaMemcpy(d.k, k.data(), 4 * n, cudaMemcpyHostToDevice);
  cudaMemcpy(d.v, v.data(), 4 * n, cudaMemcpyHostToDevice);
  ms_sort_context ctx;
  multisplit_sort_bits_allocate(n, ctx, begin, end, digit, true);
  multisplit_sort_bits_pairs(d.k, d.ko, d.v, d.vo, n, ctx, begin, end, digit);
  cudaDeviceSynchronize();
  CHECK(multisplit_last_error() == GMS_SUCCESS, "partial-key sort");
  CHECK(download(d.ko, n) == rk, "partial-key sort keys");
  CHECK(download(d.vo, n) == idx, "partial-key sort values (stable)");
  multisplit_sort_release_memory(ctx);
  printf("sort bits [%d,%d) by %d-bit digits n=%u\n", begin, end, digit, n);
}

template <class F>
static void test_compaction(const char* name, uint32_t n, F f) {
  std::vector<uint32_t> k(n), v(n);
  for (uint32_t i = 0; i < n; ++i) {
    k[i] = next_u32();
    v[i] = i;
  }
  std::vector<uint32_t> rk, rv, roffs;
  cpu_multisplit(k, v, rk, rv, 2, f, &roffs);
  const uint32_t r0 = n ? roffs[1] : 0;
  DeviceArrays d(n);
  cudaMemcpy(d.k, k.data(), 4 * n, cudaMemcpyHostToDevice);
  cudaMemcpy(d.v, v.data(), 4 * n, cudaMemcpyHostToDevice);
  compaction_context ctx;
  compaction_allocate_key_value(n, ctx);
  const unsigned int n0 = compaction_key_value(d.k, d.v, d.ko, d.vo, n, ctx, f);
  CHECK(n0 == r0, name);
  CHECK(download(d.ko, n) == rk && download(d.vo, n) == rv, name);
  compaction_release_memory(ctx);
  compaction_context ctx2;
  compaction_allocate_key_only(n, ctx2);
  CHECK(compaction_key_only(d.k, d.ko, n, ctx2, f) == r0, name);
  CHECK(download(d.ko, n) == rk, name);
  compaction_release_memory(ctx2);
  printf("compaction %-28s n=%u bucket0=%u\n", name, n, n0);
}

template <class F>
static void test_histogram(const char* name, uint32_t n, uint32_t B, F f) {
  std::vector<uint32_t> k(n);
  for (auto& x : k) x = next_u32();
  std::vector<int> ref(B, 0);
  for (uint32_t x : k) ref[f(x) & (B - 1)]++;
  DeviceArrays d(n);
  cudaMemcpy(d.k, k.data(), 4 * n, cudaMemcpyHostToDevice);
  int* hist;
  cudaMalloc(&hist, 4 * B);
  cudaMemset(hist, 0, 4 * B);
  multisplit_histogram(d.k, n, hist, B, f);
  std::vector<int> got(B);
  cudaMemcpy(got.data(), hist, 4 * B, cudaMemcpyDeviceToHost);
  CHECK(multisplit_last_error() == GMS_SUCCESS && got == ref, name);
  cudaFree(hist);
  printf("histogram %-28s n=%u B=%u\n", name, n, B);
}

int main() {
  // precompiled path
  test_multisplit("delta_func (a/delta)", 100003, 32, delta_func((0xFFFFFFFFu / 32) + 1));
  test_multisplit("ms_bucket_sort_7bit<11>", 65537, 128, ms_bucket_sort_7bit<11, uint32_t>());
  test_multisplit("gms::delta_bucket", 1 << 20, 256, gms::delta_bucket{256});
  // in-translation-unit path
  test_multisplit("user hash_bucket", 300007, 256, hash_bucket());
  test_multisplit("user mod_bucket (m=5)", 4097, 8, mod_bucket{5});
  test_multisplit("ms_bucket_sort_7bit<4>, B=256", 20000, 256, ms_bucket_sort_7bit<4, uint32_t>());
  test_multisplit("user hash_bucket, n=1", 1, 64, hash_bucket());
  test_sort(100003, false);
  test_sort(65536, true);
  test_sort(50001, false, SORT_FNS(4));
  test_sort(50002, true, SORT_FNS(5));
  test_sort(50003, false, SORT_FNS(6));
  test_sort(50004, false, SORT_FNS(8));
  test_sort_bits(70001, 3, 17, 5);
  test_sort_bits(4096, 0, 32, 8);
  test_compaction("test_bucket<1> (key & 1)", 100001, test_bucket<1, uint32_t>());
  test_compaction("gms::mask_bucket{1}", 4096, gms::mask_bucket{1});
  test_histogram("gms::delta_bucket", 1 << 20, 256, gms::delta_bucket{256});
  test_histogram("user hash_bucket", 99999, 64, hash_bucket());

  // the reference's error behaviour: an unsupported bucket count prints and does nothing
  multisplit_context bad(3);
  multisplit_allocate_key_only(100, bad);
  CHECK(multisplit_last_error() == GMS_ERROR_UNSUPPORTED_BUCKETS, "unsupported bucket count");

  if (failures == 0) printf("ALL PASSED\n");
  return failures == 0 ? 0 : 1;
}
