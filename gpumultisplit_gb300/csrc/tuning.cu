// Tuning table of the batched form and its autotuner.
//
// The batched form runs each segment with one of the tile variants of
// kTileVariants (warps per block x keys per thread).  The table maps
// (log2 B, key/value, segment size class) to a variant.  Its built-in entries
// use the plain path's 4096-key tile for every class: on GB300, 4096 segments
// of 1 Ki to 64 Ki pairs ran faster with it (0.374 ms) than with tiles that
// just hold segments of up to 2048 keys (0.402 ms) or with the autotuned table
// (0.410 ms).  gms_autotune, which is opt-in, replaces an entry with the
// variant that measured fastest on this device on segments of that class
// alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/gpumultisplit.h"
#include "ms_host.h"

namespace gms {
namespace {

constexpr int kMaxLogB = 8;

// Built-in choice for every size class: the plain path's 4096-key tile.
int builtin_variant(int) { return 0; }

// Relative gain another variant needs over the built-in one to replace it.
constexpr float kTuneMargin = 0.03f;

struct Table {
  std::mutex mu;
  int v[kMaxLogB][2][kNumSizeClasses];
  Table() { reset(); }
  void reset() {
    for (int l = 0; l < kMaxLogB; ++l)
      for (int kv = 0; kv < 2; ++kv)
        for (int c = 0; c < kNumSizeClasses; ++c) v[l][kv][c] = builtin_variant(c);
  }
};

Table& table() {
  static Table t;
  return t;
}

bool logb_of(uint32_t b, int* logb) {
  if (b < 2 || b > 256 || (b & (b - 1)) != 0) return false;
  int l = 0;
  while ((1u << l) < b) ++l;
  *logb = l;
  return true;
}

// Trial keys: splitmix64 of the index (Steele, Lea and Flood, 2014), upper 32
// bits; values = index.
__global__ void fill_trial_kernel(uint32_t* __restrict__ keys, uint32_t* __restrict__ values, uint32_t n,
                                  uint64_t seed) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint64_t z = seed + (uint64_t(i) + 1u) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    keys[i] = uint32_t(z >> 32);
    if (values) values[i] = i;
  }
}

gms_status to_status(cudaError_t e) {
  if (e == cudaSuccess) return GMS_SUCCESS;
  note_cuda_error(e);
  return GMS_ERROR_CUDA;
}

// Device buffers of one autotuning call, released on every exit path.
struct TrialBuffers {
  uint32_t* kin = nullptr;
  uint32_t* vin = nullptr;
  uint32_t* kout = nullptr;
  uint32_t* vout = nullptr;
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~TrialBuffers() {
    cudaFree(kin);
    cudaFree(vin);
    cudaFree(kout);
    cudaFree(vout);
    cudaFree(scratch);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
};

// Best-of-reps milliseconds of one batch replayed as a graph, or < 0 on error.
gms_status time_plan(TrialBuffers& tb, const std::vector<gms_segment>& segs, int variant, int reps,
                     cudaStream_t stream, float* best) {
  gms_batch_t plan = nullptr;
  gms_status st = batch_create(segs.data(), uint32_t(segs.size()), variant, &plan);
  if (st != GMS_SUCCESS) return st;
  size_t need = 0;
  gms_batch_scratch_bytes(plan, &need);
  if (need > tb.scratch_bytes) {
    cudaFree(tb.scratch);
    tb.scratch = nullptr;
    tb.scratch_bytes = 0;
    cudaError_t e = cudaMalloc(&tb.scratch, need);
    if (e != cudaSuccess) {
      gms_batch_destroy(plan);
      return to_status(e);
    }
    tb.scratch_bytes = need;
  }
  st = gms_batch_run(plan, tb.scratch, tb.scratch_bytes, 1, stream);  // binds the tables, captures the graph
  float ms_best = -1.0f;
  for (int r = 0; st == GMS_SUCCESS && r < reps; ++r) {
    cudaError_t e = cudaEventRecord(tb.ev[0], stream);
    if (e == cudaSuccess) st = gms_batch_run(plan, tb.scratch, tb.scratch_bytes, 1, stream);
    if (e == cudaSuccess && st == GMS_SUCCESS) e = cudaEventRecord(tb.ev[1], stream);
    if (e == cudaSuccess && st == GMS_SUCCESS) e = cudaEventSynchronize(tb.ev[1]);
    float ms = 0.0f;
    if (e == cudaSuccess && st == GMS_SUCCESS) e = cudaEventElapsedTime(&ms, tb.ev[0], tb.ev[1]);
    if (e != cudaSuccess) st = to_status(e);
    if (st == GMS_SUCCESS && (ms_best < 0.0f || ms < ms_best)) ms_best = ms;
  }
  gms_batch_destroy(plan);
  *best = ms_best;
  return st;
}

}  // namespace

int tuned_variant(int logb, bool kv, uint32_t n) {
  Table& t = table();
  std::lock_guard<std::mutex> lock(t.mu);
  const int v = t.v[logb - 1][kv ? 1 : 0][size_class(n)];
  return variant_valid(v, logb) ? v : 0;
}

}  // namespace gms

using namespace gms;

extern "C" {

gms_status gms_tile_variant_shape(int variant, uint32_t* warps, uint32_t* keys_per_thread, uint32_t* tile_keys) {
  if (variant < 0 || variant >= kNumTileVariants) return GMS_ERROR_INVALID_VALUE;
  if (warps) *warps = uint32_t(kTileVariants[variant].warps);
  if (keys_per_thread) *keys_per_thread = uint32_t(kTileVariants[variant].ipt);
  if (tile_keys) *tile_keys = variant_tile_keys(variant);
  return GMS_SUCCESS;
}

gms_status gms_tuning_get(uint32_t num_buckets, int key_value, int size_class_index, int* variant) {
  int logb = 0;
  if (variant == nullptr || size_class_index < 0 || size_class_index >= kNumSizeClasses)
    return GMS_ERROR_INVALID_VALUE;
  if (!logb_of(num_buckets, &logb)) return GMS_ERROR_UNSUPPORTED_BUCKETS;
  Table& t = table();
  std::lock_guard<std::mutex> lock(t.mu);
  *variant = t.v[logb - 1][key_value ? 1 : 0][size_class_index];
  return GMS_SUCCESS;
}

gms_status gms_tuning_set(uint32_t num_buckets, int key_value, int size_class_index, int variant) {
  int logb = 0;
  if (size_class_index < 0 || size_class_index >= kNumSizeClasses) return GMS_ERROR_INVALID_VALUE;
  if (!logb_of(num_buckets, &logb)) return GMS_ERROR_UNSUPPORTED_BUCKETS;
  if (!variant_valid(variant, logb)) return GMS_ERROR_INVALID_VALUE;
  Table& t = table();
  std::lock_guard<std::mutex> lock(t.mu);
  t.v[logb - 1][key_value ? 1 : 0][size_class_index] = variant;
  return GMS_SUCCESS;
}

gms_status gms_tuning_reset(void) {
  Table& t = table();
  std::lock_guard<std::mutex> lock(t.mu);
  t.reset();
  return GMS_SUCCESS;
}

gms_status gms_autotune(uint32_t bucket_mask, uint32_t key_value_mask, uint32_t keys_per_trial, int reps,
                        float* h_ms_out, gms_stream_t stream_in) {
  if ((bucket_mask & ~0x1FEu) != 0 || bucket_mask == 0 || (key_value_mask & ~3u) != 0 || key_value_mask == 0 ||
      keys_per_trial < (1u << 16) || keys_per_trial > (1u << 28) || reps < 1)
    return GMS_ERROR_INVALID_VALUE;
  auto stream = static_cast<cudaStream_t>(stream_in);
  if (h_ms_out)
    std::fill(h_ms_out, h_ms_out + kMaxLogB * 2 * kNumSizeClasses, -1.0f);
  TrialBuffers tb;
  const bool any_kv = (key_value_mask & 2u) != 0;
  const size_t bytes = size_t(keys_per_trial) * 4;
  cudaError_t e = cudaMalloc(&tb.kin, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&tb.kout, bytes);
  if (e == cudaSuccess && any_kv) e = cudaMalloc(&tb.vin, bytes);
  if (e == cudaSuccess && any_kv) e = cudaMalloc(&tb.vout, bytes);
  if (e == cudaSuccess) e = cudaEventCreate(&tb.ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&tb.ev[1]);
  if (e != cudaSuccess) return to_status(e);
  fill_trial_kernel<<<device_sm_count() * 4, 256, 0, stream>>>(tb.kin, tb.vin, keys_per_trial, 0x5EEDull);
  e = cudaGetLastError();
  if (e != cudaSuccess) return to_status(e);

  int best_v[kMaxLogB][2][kNumSizeClasses];
  for (int c = 0; c < kNumSizeClasses; ++c) {
    // Segments sized inside the class: 3/4 of its upper bound, 2^20 for the last one.
    const uint32_t seg_n = c < kNumSizeClasses - 1 ? (3u << (8 + c)) : (1u << 20);
    const uint32_t count = std::max(1u, keys_per_trial / seg_n);
    for (int logb = 1; logb <= kMaxLogB; ++logb) {
      if (!(bucket_mask & (1u << logb))) continue;
      for (int kv = 0; kv < 2; ++kv) {
        best_v[logb - 1][kv][c] = -1;
        if (!(key_value_mask & (1u << kv))) continue;
        std::vector<gms_segment> segs(count);
        for (uint32_t i = 0; i < count; ++i) {
          gms_segment& sg = segs[i];
          const size_t off = size_t(i) * seg_n;
          sg.d_key_in = tb.kin + off;
          sg.d_key_out = tb.kout + off;
          sg.d_value_in = kv ? tb.vin + off : nullptr;
          sg.d_value_out = kv ? tb.vout + off : nullptr;
          sg.n = seg_n;
          sg.desc = gms_bucket_desc{GMS_BUCKET_DELTA, 1u << logb, 0u, 0u, 0u, 0.0f, nullptr};
        }
        // The built-in entry keeps its place unless another variant is faster
        // by more than kTuneMargin (timing noise must not flip the table).
        const int builtin = builtin_variant(c);
        float builtin_ms = -1.0f, other_ms = -1.0f;
        int other = -1;
        for (int v = 0; v < kNumTileVariants; ++v) {
          if (!variant_valid(v, logb)) continue;
          float ms = -1.0f;
          const gms_status st = time_plan(tb, segs, v, reps, stream, &ms);
          if (st != GMS_SUCCESS) return st;
          if (ms < 0.0f) continue;
          if (v == builtin) {
            builtin_ms = ms;
          } else if (other_ms < 0.0f || ms < other_ms) {
            other_ms = ms;
            other = v;
          }
        }
        const bool take_other = other >= 0 && (builtin_ms < 0.0f || other_ms < builtin_ms * (1.0f - kTuneMargin));
        best_v[logb - 1][kv][c] = take_other ? other : builtin;
        const float best = take_other ? other_ms : builtin_ms;
        if (h_ms_out) h_ms_out[((logb - 1) * 2 + kv) * kNumSizeClasses + c] = best;
      }
    }
  }
  // Publish the whole result at once.
  Table& t = table();
  std::lock_guard<std::mutex> lock(t.mu);
  for (int l = 0; l < kMaxLogB; ++l)
    for (int kv = 0; kv < 2; ++kv)
      for (int c = 0; c < kNumSizeClasses; ++c)
        if (best_v[l][kv][c] >= 0 && (bucket_mask & (2u << l)) && (key_value_mask & (1u << kv)))
          t.v[l][kv][c] = best_v[l][kv][c];
  return GMS_SUCCESS;
}

}  // extern "C"
