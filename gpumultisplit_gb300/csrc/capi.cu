// The library's C ABI (include/gpumultisplit.h): argument checks, scratch
// layout, stage orchestration, and the multi-pass operations built on the
// multisplit (7-bit radix sort, two-bucket compaction).
#include <atomic>
#include <cstring>

#include "../../include/gpumultisplit.h"
#include "ms_host.h"
#include "scan_kernels.cuh"

namespace gms {

namespace {
thread_local int g_last_cuda_error = 0;

gms_status cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return GMS_SUCCESS;
  g_last_cuda_error = int(e);
  return GMS_ERROR_CUDA;
}

// Any bucket count in [2, 256]; *logb = ceil(log2(b)).
bool valid_buckets(uint32_t b, int* logb) {
  if (b < 2 || b > 256) return false;
  int l = 0;
  while ((1u << l) < b) ++l;
  *logb = l;
  return true;
}

template <int LOGB, bool KV>
constexpr uint32_t tile_of() {
  return uint32_t(TileShape<LOGB, KV>::WARPS) * 32u * uint32_t(TileShape<LOGB, KV>::IPT);
}

gms_status check_desc(const gms_bucket_desc* d, int* logb) {
  if (d == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (!valid_buckets(d->num_buckets, logb)) return GMS_ERROR_UNSUPPORTED_BUCKETS;
  switch (d->kind) {
    case GMS_BUCKET_BITS:  // a bit field: the bucket count is a power of two
      return (d->num_buckets & (d->num_buckets - 1)) == 0 ? GMS_SUCCESS : GMS_ERROR_UNSUPPORTED_BUCKETS;
    case GMS_BUCKET_DELTA:
    case GMS_BUCKET_MASK:
    case GMS_BUCKET_EVEN_FLOAT:
      return GMS_SUCCESS;
    case GMS_BUCKET_DIV:
      return d->param != 0 ? GMS_SUCCESS : GMS_ERROR_INVALID_VALUE;
    case GMS_BUCKET_RANGE:
      return d->d_splitters != nullptr ? GMS_SUCCESS : GMS_ERROR_INVALID_VALUE;
    default:
      return GMS_ERROR_INVALID_VALUE;
  }
}

BucketParams to_params(const gms_bucket_desc* d) {
  BucketParams p;
  p.shift = d->shift;
  p.param = d->param;
  p.lower = d->lower;
  p.inverse_delta = d->inverse_delta;
  p.splitters = d->d_splitters;
  p.num_buckets = d->num_buckets;
  return p;
}

cudaError_t dispatch(int kind, const MsCall& c, int stages) {
  switch (kind) {
    case KIND_DELTA: return run_multisplit<KIND_DELTA>(c, stages);
    case KIND_DIV: return run_multisplit<KIND_DIV>(c, stages);
    case KIND_BITS: return run_multisplit<KIND_BITS>(c, stages);
    case KIND_RANGE: return run_multisplit<KIND_RANGE>(c, stages);
    case KIND_MASK: return run_multisplit<KIND_MASK>(c, stages);
    case KIND_EVEN_FLOAT: return run_multisplit<KIND_EVEN_FLOAT>(c, stages);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t dispatch_hist(int kind, const uint32_t* keys, uint32_t n, int logb, const BucketParams& bp,
                          int32_t* hist, cudaStream_t s) {
  switch (kind) {
    case KIND_DELTA: return run_histogram<KIND_DELTA>(keys, n, logb, bp, hist, s);
    case KIND_DIV: return run_histogram<KIND_DIV>(keys, n, logb, bp, hist, s);
    case KIND_BITS: return run_histogram<KIND_BITS>(keys, n, logb, bp, hist, s);
    case KIND_RANGE: return run_histogram<KIND_RANGE>(keys, n, logb, bp, hist, s);
    case KIND_MASK: return run_histogram<KIND_MASK>(keys, n, logb, bp, hist, s);
    case KIND_EVEN_FLOAT: return run_histogram<KIND_EVEN_FLOAT>(keys, n, logb, bp, hist, s);
    default: return cudaErrorInvalidValue;
  }
}

// Whether [a, a + n*elem_a) and [b, b + n*elem_b) share a byte.
bool overlaps(const void* a, const void* b, uint32_t n, size_t elem_a = 4, size_t elem_b = 4) {
  if (a == nullptr || b == nullptr || n == 0) return false;
  const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
  return x < y + uintptr_t(n) * elem_b && y < x + uintptr_t(n) * elem_a;
}

// Shared body of the multisplit entry points (stage mask selects the kernels).
gms_status multisplit_impl(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                           const gms_bucket_desc* desc, bool kv, void* scratch, size_t scratch_bytes,
                           int stages, cudaStream_t stream) {
  int logb = 0;
  gms_status st = check_desc(desc, &logb);
  if (st != GMS_SUCCESS) return st;
  if (n == 0) return GMS_SUCCESS;
  if (scratch == nullptr || (reinterpret_cast<uintptr_t>(scratch) & 255u) != 0) return GMS_ERROR_INVALID_VALUE;
  if ((stages & (STAGE_PRESCAN | STAGE_POSTSCAN)) && kin == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (stages & STAGE_POSTSCAN) {
    if (kout == nullptr || overlaps(kin, kout, n)) return GMS_ERROR_INVALID_VALUE;
    if (kv && (vin == nullptr || vout == nullptr || overlaps(vin, vout, n) || overlaps(kout, vout, n)))
      return GMS_ERROR_INVALID_VALUE;
  }
  const Geometry g = make_geometry(n, logb, kv);
  if (scratch_bytes < g.bytes) return GMS_ERROR_SCRATCH_TOO_SMALL;
  MsCall c;
  c.kin = kin;
  c.vin = vin;
  c.kout = kout;
  c.vout = vout;
  c.n = n;
  c.logb = logb;
  c.kv = kv;
  c.bp = to_params(desc);
  c.scratch = static_cast<unsigned char*>(scratch);
  c.stream = stream;
  // Costly identifiers are evaluated once when the scratch has room for a
  // bucket byte per key (the prescan stores them, the postscan reads them).
  if (kind_keeps_bucket_bytes(desc->kind) && scratch_bytes >= g.bytes_full) c.bucket_bytes = c.scratch + g.off_buckets;
  return cuda_status(dispatch(desc->kind, c, stages));
}

// Bucket start offsets: matrix[b * num_tiles] for b < B (src/api/multisplit.cuh:143-149).
gms_status copy_offsets(const void* scratch, uint32_t n, int logb, uint32_t B, bool kv, uint32_t* h_offsets,
                        cudaStream_t stream, int kw = 1, int vw = 1) {
  if (n == 0) {
    for (uint32_t b = 0; b < B; ++b) h_offsets[b] = 0;
    return GMS_SUCCESS;
  }
  const Geometry g = make_geometry(n, logb, kv, kw, vw);
  const auto* matrix = static_cast<const unsigned char*>(scratch) + g.off_matrix;
  cudaError_t e = cudaMemcpy2DAsync(h_offsets, sizeof(uint32_t), matrix, size_t(g.num_tiles) * 4, sizeof(uint32_t),
                                    B, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  return cuda_status(e);
}

// Digit schedules of the reference's multisplit sorts
// (src/api/multisplit_sort.cuh:320-559, src/api/multisplit_sort_pairs.cuh:21-260):
// (shift, buckets) per pass, least significant digit first.
struct SortSchedule {
  int passes;
  uint32_t shift[16];
  uint32_t buckets[16];
};

bool sort_schedule(int digit_bits, SortSchedule* s) {
  switch (digit_bits) {
    case 4: *s = {8, {0, 4, 8, 12, 16, 20, 24, 28}, {16, 16, 16, 16, 16, 16, 16, 16}}; return true;
    case 5: *s = {7, {0, 5, 10, 15, 20, 25, 30}, {32, 32, 32, 32, 32, 32, 4}}; return true;
    case 6: *s = {6, {0, 4, 8, 14, 20, 26}, {16, 16, 64, 64, 64, 64}}; return true;
    case 7: *s = {5, {0, 4, 11, 18, 25}, {16, 128, 128, 128, 128}}; return true;
    case 8: *s = {4, {0, 8, 16, 24}, {256, 256, 256, 256}}; return true;
    default: return false;
  }
}

// Partial-key schedule: digits of digit_bits bits from begin_bit up to end_bit
// (at most key_bits), the last one narrower when the range is not a whole
// number of digits.
bool bit_schedule(int begin_bit, int end_bit, int digit_bits, SortSchedule* s, int key_bits = 32) {
  if (digit_bits < 4 || digit_bits > 8 || begin_bit < 0 || end_bit > key_bits || begin_bit > end_bit) return false;
  s->passes = 0;
  for (int sh = begin_bit; sh < end_bit; sh += digit_bits) {
    const int w = end_bit - sh < digit_bits ? end_bit - sh : digit_bits;
    s->shift[s->passes] = uint32_t(sh);
    s->buckets[s->passes] = w == 1 ? 2u : (1u << w);
    ++s->passes;
  }
  return true;
}

struct SortLayout {
  size_t ms_bytes;   // multisplit scratch (largest over the schedule's digit widths)
  size_t off_keys;   // ping-pong keys
  size_t off_vals;   // ping-pong values
  size_t bytes;
};

SortLayout sort_layout(uint32_t n, bool kv, const SortSchedule& sch) {
  SortLayout L;
  L.ms_bytes = 0;
  if (sch.passes == 0) {  // nothing to sort: the input is copied
    L.off_keys = L.off_vals = L.bytes = 0;
    return L;
  }
  for (int p = 0; p < sch.passes; ++p) {
    int logb = 0;
    valid_buckets(sch.buckets[p], &logb);
    const size_t b = make_geometry(n, logb, kv).bytes;
    L.ms_bytes = b > L.ms_bytes ? b : L.ms_bytes;
  }
  // room for the one-sweep passes too, so either method can run on it
  if (sch.passes <= kOnesweepMaxPasses) {
    uint32_t logb[kOnesweepMaxPasses];
    for (int p = 0; p < sch.passes; ++p) valid_buckets(sch.buckets[p], reinterpret_cast<int*>(&logb[p]));
    const size_t b = onesweep_scratch_bytes(n, sch.passes, logb);
    L.ms_bytes = b > L.ms_bytes ? b : L.ms_bytes;
  }
  L.off_keys = align_up(L.ms_bytes, 256);
  L.off_vals = align_up(L.off_keys + size_t(n) * 4, 256);
  L.bytes = kv ? align_up(L.off_vals + size_t(n) * 4, 256) : L.off_vals;
  return L;
}

// Which way the 32-bit sorts run their digits (gms_sort_set_method).
std::atomic<int> g_sort_method{GMS_SORT_AUTO};

bool use_onesweep(uint32_t n, int passes) {
  const int m = g_sort_method.load(std::memory_order_relaxed);
  if (passes > kOnesweepMaxPasses || m == GMS_SORT_MULTISPLIT) return false;
  return m == GMS_SORT_ONESWEEP || (n >= kOnesweepMinKeys && kOnesweepMinKeys != 0xFFFFFFFFu);
}

// LSD radix sort by stable multisplits on successive digits.  The buffers
// ping-pong between the output and the scratch copy so the last pass lands in
// the output (an odd number of passes starts in the output, an even one in the
// copy), and the input is never written.  From kOnesweepMinKeys keys up (or
// as gms_sort_set_method says) the digits run as one-sweep passes
// (onesweep.cu), with the same ping-pong and the same output.
gms_status sort_run(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                    bool kv, const SortSchedule& sch, void* scratch, size_t scratch_bytes, cudaStream_t stream) {
  if (n == 0) return GMS_SUCCESS;
  if (kin == nullptr || kout == nullptr || (scratch == nullptr && sch.passes > 0)) return GMS_ERROR_INVALID_VALUE;
  if (kv && (vin == nullptr || vout == nullptr)) return GMS_ERROR_INVALID_VALUE;
  const SortLayout L = sort_layout(n, kv, sch);
  if (scratch_bytes < L.bytes) return GMS_ERROR_SCRATCH_TOO_SMALL;
  if (sch.passes == 0) {
    if (overlaps(kin, kout, n) || (kv && overlaps(vin, vout, n))) return GMS_ERROR_INVALID_VALUE;
    cudaError_t e = cudaMemcpyAsync(kout, kin, size_t(n) * 4, cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess && kv) e = cudaMemcpyAsync(vout, vin, size_t(n) * 4, cudaMemcpyDeviceToDevice, stream);
    return cuda_status(e);
  }
  auto* base = static_cast<unsigned char*>(scratch);
  uint32_t* tk = reinterpret_cast<uint32_t*>(base + L.off_keys);
  uint32_t* tv = kv ? reinterpret_cast<uint32_t*>(base + L.off_vals) : nullptr;
  if (use_onesweep(n, sch.passes)) {
    // the same buffer checks as the multisplit passes make, pass by pass
    const uint32_t* ki = kin;
    const uint32_t* vi = vin;
    for (int p = 0; p < sch.passes; ++p) {
      const bool to_out = ((sch.passes - 1 - p) % 2) == 0;
      uint32_t* ko = to_out ? kout : tk;
      uint32_t* vo = to_out ? vout : tv;
      if (overlaps(ki, ko, n) || (kv && (overlaps(vi, vo, n) || overlaps(ko, vo, n)))) return GMS_ERROR_INVALID_VALUE;
      ki = ko;
      vi = vo;
    }
    uint32_t logb[kOnesweepMaxPasses];
    for (int p = 0; p < sch.passes; ++p) valid_buckets(sch.buckets[p], reinterpret_cast<int*>(&logb[p]));
    return cuda_status(run_onesweep_sort(kin, kout, kv ? vin : nullptr, kv ? vout : nullptr, n, kv, sch.passes,
                                         sch.shift, logb, base, tk, tv, stream));
  }
  const uint32_t* ki = kin;
  const uint32_t* vi = vin;
  for (int p = 0; p < sch.passes; ++p) {
    const bool to_out = ((sch.passes - 1 - p) % 2) == 0;
    uint32_t* ko = to_out ? kout : tk;
    uint32_t* vo = to_out ? vout : tv;
    gms_bucket_desc d{};
    d.kind = GMS_BUCKET_BITS;
    d.num_buckets = sch.buckets[p];
    d.shift = sch.shift[p];
    gms_status st = multisplit_impl(ki, kv ? vi : nullptr, ko, kv ? vo : nullptr, n, &d, kv, scratch, L.ms_bytes,
                                    STAGE_ALL, stream);
    if (st != GMS_SUCCESS) return st;
    ki = ko;
    vi = vo;
  }
  return GMS_SUCCESS;
}

gms_status sort_impl(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                     bool kv, int digit_bits, void* scratch, size_t scratch_bytes, cudaStream_t stream) {
  SortSchedule sch;
  if (!sort_schedule(digit_bits, &sch)) return GMS_ERROR_INVALID_VALUE;
  return sort_run(kin, kout, vin, vout, n, kv, sch, scratch, scratch_bytes, stream);
}

gms_status compaction_impl(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                           const gms_bucket_desc* desc, bool kv, void* scratch, size_t scratch_bytes,
                           uint32_t* h_num0, cudaStream_t stream) {
  if (desc == nullptr || desc->num_buckets != 2) return GMS_ERROR_INVALID_VALUE;
  gms_status st = multisplit_impl(kin, vin, kout, vout, n, desc, kv, scratch, scratch_bytes, STAGE_ALL, stream);
  if (st != GMS_SUCCESS || h_num0 == nullptr) return st;
  if (n == 0) {
    *h_num0 = 0;
    return GMS_SUCCESS;
  }
  // Start of bucket 1 = number of bucket-0 keys (multisplit2_compaction.cuh:541-542).
  const Geometry g = make_geometry(n, 1, kv);
  const auto* matrix = static_cast<const unsigned char*>(scratch) + g.off_matrix;
  cudaError_t e = cudaMemcpyAsync(h_num0, matrix + size_t(g.num_tiles) * 4, sizeof(uint32_t),
                                  cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  return cuda_status(e);
}

// ------------------------------------------------ more than 256 buckets
// B in (256, 65536] (RANGE: to GMS_RANGE_BIG_MAX splitters), 32-bit keys and
// values, through the one-call entry points: two stable multisplits on the
// digits of the bucket id, the low half of its bits into the scratch's
// ping-pong buffers, then the high half into the output.  Halving the bits
// keeps both passes at a small bucket count (B = 1000: 32 x 32 buckets), which
// is cheaper than a 256-bucket pass and a small one.  Offsets are read off the
// output, which is sorted by the whole id.
struct BigLayout {
  int logb_lo, logb_hi;  // bits of the low and the high digit
  size_t ms_bytes;       // scratch of either pass (with its bucket bytes)
  size_t off_keys, off_vals, off_hist, bytes;  // off_hist: B words for the bucket starts
};

BigLayout big_layout(uint32_t n, uint32_t B, bool kv) {
  BigLayout L;
  int bits = 0;
  while ((1u << bits) < B) ++bits;  // 9..16
  L.logb_lo = (bits + 1) / 2;
  L.logb_hi = bits - L.logb_lo;
  const size_t a = make_geometry(n, L.logb_lo, kv).bytes_full, b = make_geometry(n, L.logb_hi, kv).bytes_full;
  L.ms_bytes = a > b ? a : b;
  L.off_keys = align_up(L.ms_bytes, 256);
  L.off_vals = align_up(L.off_keys + size_t(n) * 4, 256);
  L.off_hist = kv ? align_up(L.off_vals + size_t(n) * 4, 256) : L.off_vals;
  L.bytes = align_up(L.off_hist + size_t(B) * 4, 256);
  return L;
}

bool is_big(const gms_bucket_desc* d) { return d != nullptr && d->num_buckets > 256; }

gms_status check_big_desc(const gms_bucket_desc* d) {
  if (d == nullptr) return GMS_ERROR_INVALID_VALUE;
  const uint32_t B = d->num_buckets;
  if (B <= 256 || B > BIG_MAX_BUCKETS) return GMS_ERROR_UNSUPPORTED_BUCKETS;
  switch (d->kind) {
    case GMS_BUCKET_BITS:
      return (B & (B - 1)) == 0 ? GMS_SUCCESS : GMS_ERROR_UNSUPPORTED_BUCKETS;
    case GMS_BUCKET_DELTA:
    case GMS_BUCKET_MASK:
    case GMS_BUCKET_EVEN_FLOAT:
      return GMS_SUCCESS;
    case GMS_BUCKET_DIV:
      return d->param != 0 ? GMS_SUCCESS : GMS_ERROR_INVALID_VALUE;
    case GMS_BUCKET_RANGE:
      if (B > GMS_RANGE_BIG_MAX) return GMS_ERROR_UNSUPPORTED_BUCKETS;
      return d->d_splitters != nullptr ? GMS_SUCCESS : GMS_ERROR_INVALID_VALUE;
    default:
      return GMS_ERROR_INVALID_VALUE;
  }
}

cudaError_t dispatch_digit_prescan(int kind, const DigitPass& c) {
  switch (kind) {
    case KIND_DELTA: return run_digit_prescan_scan<KIND_DELTA>(c);
    case KIND_DIV: return run_digit_prescan_scan<KIND_DIV>(c);
    case KIND_BITS: return run_digit_prescan_scan<KIND_BITS>(c);
    case KIND_RANGE: return run_digit_prescan_scan<KIND_RANGE>(c);
    case KIND_MASK: return run_digit_prescan_scan<KIND_MASK>(c);
    case KIND_EVEN_FLOAT: return run_digit_prescan_scan<KIND_EVEN_FLOAT>(c);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t dispatch_big_offsets(int kind, const uint32_t* sorted_keys, uint32_t n, const BucketParams& p,
                                 uint32_t* starts, cudaStream_t s) {
  switch (kind) {
    case KIND_DELTA: return run_big_offsets<KIND_DELTA>(sorted_keys, n, p, starts, s);
    case KIND_DIV: return run_big_offsets<KIND_DIV>(sorted_keys, n, p, starts, s);
    case KIND_BITS: return run_big_offsets<KIND_BITS>(sorted_keys, n, p, starts, s);
    case KIND_RANGE: return run_big_offsets<KIND_RANGE>(sorted_keys, n, p, starts, s);
    case KIND_MASK: return run_big_offsets<KIND_MASK>(sorted_keys, n, p, starts, s);
    case KIND_EVEN_FLOAT: return run_big_offsets<KIND_EVEN_FLOAT>(sorted_keys, n, p, starts, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t dispatch_big_histogram(int kind, const uint32_t* keys, uint32_t n, const BucketParams& p, uint32_t* hist,
                                   cudaStream_t s) {
  switch (kind) {
    case KIND_DELTA: return run_big_histogram<KIND_DELTA>(keys, n, p, hist, s);
    case KIND_DIV: return run_big_histogram<KIND_DIV>(keys, n, p, hist, s);
    case KIND_BITS: return run_big_histogram<KIND_BITS>(keys, n, p, hist, s);
    case KIND_RANGE: return run_big_histogram<KIND_RANGE>(keys, n, p, hist, s);
    case KIND_MASK: return run_big_histogram<KIND_MASK>(keys, n, p, hist, s);
    case KIND_EVEN_FLOAT: return run_big_histogram<KIND_EVEN_FLOAT>(keys, n, p, hist, s);
    default: return cudaErrorInvalidValue;
  }
}

gms_status multisplit_big_impl(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                               const gms_bucket_desc* desc, bool kv, void* scratch, size_t scratch_bytes,
                               uint32_t* h_offsets, cudaStream_t stream) {
  gms_status st = check_big_desc(desc);
  if (st != GMS_SUCCESS) return st;
  const uint32_t B = desc->num_buckets;
  if (n == 0) {
    if (h_offsets)
      for (uint32_t b = 0; b < B; ++b) h_offsets[b] = 0;
    return GMS_SUCCESS;
  }
  if (scratch == nullptr || (reinterpret_cast<uintptr_t>(scratch) & 255u) != 0) return GMS_ERROR_INVALID_VALUE;
  if (kin == nullptr || kout == nullptr || overlaps(kin, kout, n)) return GMS_ERROR_INVALID_VALUE;
  if (kv && (vin == nullptr || vout == nullptr || overlaps(vin, vout, n) || overlaps(kout, vout, n)))
    return GMS_ERROR_INVALID_VALUE;
  const BigLayout L = big_layout(n, B, kv);
  if (scratch_bytes < L.bytes) return GMS_ERROR_SCRATCH_TOO_SMALL;
  auto* base = static_cast<unsigned char*>(scratch);
  auto* tk = reinterpret_cast<uint32_t*>(base + L.off_keys);
  auto* tv = kv ? reinterpret_cast<uint32_t*>(base + L.off_vals) : nullptr;
  const BucketParams bp = to_params(desc);
  for (int pass = 0; pass < 2; ++pass) {
    DigitPass c;
    c.kin = pass == 0 ? kin : tk;
    c.vin = kv ? (pass == 0 ? vin : tv) : nullptr;
    c.kout = pass == 0 ? tk : kout;
    c.vout = kv ? (pass == 0 ? tv : vout) : nullptr;
    c.n = n;
    c.logb = pass == 0 ? L.logb_lo : L.logb_hi;
    c.kv = kv;
    c.bp.base = bp;
    c.bp.digit_shift = pass == 0 ? 0u : uint32_t(L.logb_lo);
    c.scratch = base;
    c.bucket_bytes = base + make_geometry(n, c.logb, kv).off_buckets;
    c.stream = stream;
    cudaError_t e = dispatch_digit_prescan(desc->kind, c);
    if (e == cudaSuccess) e = run_digit_postscan(c);
    if (e != cudaSuccess) return cuda_status(e);
  }
  if (h_offsets == nullptr) return GMS_SUCCESS;
  // The output is sorted by the whole id: every bucket start is read off it.
  auto* starts = reinterpret_cast<uint32_t*>(base + L.off_hist);
  cudaError_t e = dispatch_big_offsets(desc->kind, kout, n, bp, starts, stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_offsets, starts, size_t(B) * 4, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  return cuda_status(e);
}

// ------------------------------------------------ 64-bit keys and values
// key_bytes 4 or 8; value_bytes 0 (key-only), 4 or 8.
bool valid_widths(int key_bytes, int value_bytes) {
  return (key_bytes == 4 || key_bytes == 8) && (value_bytes == 0 || value_bytes == 4 || value_bytes == 8);
}

// The 32-bit descriptor of a 64-bit one, for 32-bit keys (whose parameters
// must fit in 32 bits; the splitters are 32-bit keys).
gms_status narrow_desc(const gms_bucket_desc64* d, gms_bucket_desc* out) {
  if (d == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (d->param > 0xFFFFFFFFull || d->lower > 0xFFFFFFFFull) return GMS_ERROR_INVALID_VALUE;
  *out = gms_bucket_desc{};
  out->kind = d->kind;
  out->num_buckets = d->num_buckets;
  out->shift = d->shift;
  out->param = uint32_t(d->param);
  out->lower = uint32_t(d->lower);
  out->inverse_delta = d->inverse_delta;
  out->d_splitters = static_cast<const uint32_t*>(d->d_splitters);
  return GMS_SUCCESS;
}

gms_status check_desc64(const gms_bucket_desc64* d, int* logb) {
  if (d == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (!valid_buckets(d->num_buckets, logb)) return GMS_ERROR_UNSUPPORTED_BUCKETS;
  switch (d->kind) {
    case GMS_BUCKET_BITS:
      if ((d->num_buckets & (d->num_buckets - 1)) != 0) return GMS_ERROR_UNSUPPORTED_BUCKETS;
      return d->shift < 64 ? GMS_SUCCESS : GMS_ERROR_INVALID_VALUE;
    case GMS_BUCKET_DELTA:
    case GMS_BUCKET_MASK:
    case GMS_BUCKET_EVEN_FLOAT:
      return GMS_SUCCESS;
    case GMS_BUCKET_DIV:
      return d->param != 0 ? GMS_SUCCESS : GMS_ERROR_INVALID_VALUE;
    case GMS_BUCKET_RANGE:
      return d->d_splitters != nullptr ? GMS_SUCCESS : GMS_ERROR_INVALID_VALUE;
    default:
      return GMS_ERROR_INVALID_VALUE;
  }
}

BucketParams64 to_params64(const gms_bucket_desc64* d) {
  BucketParams64 p{};
  p.param = d->param;
  p.lower = d->lower;
  p.splitters = static_cast<const uint64_t*>(d->d_splitters);
  p.inverse_delta = d->inverse_delta;
  p.shift = d->shift;
  p.num_buckets = d->num_buckets;
  return p;
}

cudaError_t dispatch_wide(int kind, const MsCallWide& c, int stages) {
  switch (kind) {
    case KIND_DELTA: return run_multisplit_wide<KIND_DELTA>(c, stages);
    case KIND_DIV: return run_multisplit_wide<KIND_DIV>(c, stages);
    case KIND_BITS: return run_multisplit_wide<KIND_BITS>(c, stages);
    case KIND_RANGE: return run_multisplit_wide<KIND_RANGE>(c, stages);
    case KIND_MASK: return run_multisplit_wide<KIND_MASK>(c, stages);
    case KIND_EVEN_FLOAT: return run_multisplit_wide<KIND_EVEN_FLOAT>(c, stages);
    default: return cudaErrorInvalidValue;
  }
}

// Scratch bytes a wide multisplit needs: 64-bit keys always keep their
// bucket bytes, 32-bit keys as for gms_multisplit_scratch_bytes.
size_t wide_required_bytes(const Geometry& g, int key_bytes) { return key_bytes == 8 ? g.bytes_full : g.bytes; }

// Any element widths.  32-bit keys with 32-bit (or no) values take the
// 32-bit path; everything else the 64-bit instances.
gms_status multisplit_wide_impl(const void* kin, const void* vin, void* kout, void* vout, uint32_t n, int key_bytes,
                                int value_bytes, const gms_bucket_desc64* desc, void* scratch, size_t scratch_bytes,
                                cudaStream_t stream) {
  if (!valid_widths(key_bytes, value_bytes)) return GMS_ERROR_INVALID_VALUE;
  const bool kv = value_bytes != 0;
  if (key_bytes == 4 && value_bytes != 8) {
    gms_bucket_desc d32;
    gms_status st = narrow_desc(desc, &d32);
    if (st != GMS_SUCCESS) return st;
    return multisplit_impl(static_cast<const uint32_t*>(kin), static_cast<const uint32_t*>(vin),
                           static_cast<uint32_t*>(kout), static_cast<uint32_t*>(vout), n, &d32, kv, scratch,
                           scratch_bytes, STAGE_ALL, stream);
  }
  int logb = 0;
  gms_status st = key_bytes == 8 ? check_desc64(desc, &logb) : GMS_SUCCESS;
  gms_bucket_desc d32{};
  if (key_bytes == 4) {
    st = narrow_desc(desc, &d32);
    if (st == GMS_SUCCESS) st = check_desc(&d32, &logb);
  }
  if (st != GMS_SUCCESS) return st;
  if (n == 0) return GMS_SUCCESS;
  if (scratch == nullptr || (reinterpret_cast<uintptr_t>(scratch) & 255u) != 0) return GMS_ERROR_INVALID_VALUE;
  const size_t kb = size_t(key_bytes), vb = size_t(value_bytes);
  auto misaligned = [](const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) != 0; };
  if (kin == nullptr || kout == nullptr || misaligned(kin, kb) || misaligned(kout, kb) ||
      overlaps(kin, kout, n, kb, kb))
    return GMS_ERROR_INVALID_VALUE;
  if (kv && (vin == nullptr || vout == nullptr || misaligned(vin, vb) || misaligned(vout, vb) ||
             overlaps(vin, vout, n, vb, vb) || overlaps(kout, vout, n, kb, vb)))
    return GMS_ERROR_INVALID_VALUE;
  const int kw = key_bytes / 4, vw = kv ? value_bytes / 4 : 1;
  const Geometry g = make_geometry(n, logb, kv, kw, vw);
  if (scratch_bytes < wide_required_bytes(g, key_bytes)) return GMS_ERROR_SCRATCH_TOO_SMALL;
  MsCallWide c;
  c.kin = kin;
  c.vin = kv ? vin : nullptr;
  c.kout = kout;
  c.vout = kv ? vout : nullptr;
  c.n = n;
  c.logb = logb;
  c.kv = kv;
  c.kw = kw;
  c.vw = vw;
  c.scratch = static_cast<unsigned char*>(scratch);
  c.stream = stream;
  if (key_bytes == 8) {
    c.bp64 = to_params64(desc);
    c.bucket_bytes = c.scratch + g.off_buckets;
  } else {
    c.bp = to_params(&d32);
    if (kind_keeps_bucket_bytes(desc->kind) && scratch_bytes >= g.bytes_full) c.bucket_bytes = c.scratch + g.off_buckets;
  }
  return cuda_status(dispatch_wide(desc->kind, c, STAGE_ALL));
}

// Layout of a wide sort's scratch: the multisplit's scratch (largest over the
// passes), then ping-pong keys and values.
SortLayout sort_layout_wide(uint32_t n, int key_bytes, int value_bytes, const SortSchedule& sch) {
  SortLayout L;
  L.ms_bytes = 0;
  if (sch.passes == 0) {
    L.off_keys = L.off_vals = L.bytes = 0;
    return L;
  }
  const bool kv = value_bytes != 0;
  for (int p = 0; p < sch.passes; ++p) {
    int logb = 0;
    valid_buckets(sch.buckets[p], &logb);
    const Geometry g = make_geometry(n, logb, kv, key_bytes / 4, kv ? value_bytes / 4 : 1);
    const size_t b = wide_required_bytes(g, key_bytes);
    L.ms_bytes = b > L.ms_bytes ? b : L.ms_bytes;
  }
  L.off_keys = align_up(L.ms_bytes, 256);
  L.off_vals = align_up(L.off_keys + size_t(n) * key_bytes, 256);
  L.bytes = kv ? align_up(L.off_vals + size_t(n) * value_bytes, 256) : L.off_vals;
  return L;
}

// Stable LSD sort by key bits [begin_bit, end_bit) through wide multisplits,
// ping-ponging like sort_run so the last pass lands in the output.
gms_status sort_wide_run(const void* kin, void* kout, const void* vin, void* vout, uint32_t n, int key_bytes,
                         int value_bytes, const SortSchedule& sch, void* scratch, size_t scratch_bytes,
                         cudaStream_t stream) {
  const bool kv = value_bytes != 0;
  if (n == 0) return GMS_SUCCESS;
  if (kin == nullptr || kout == nullptr || (scratch == nullptr && sch.passes > 0)) return GMS_ERROR_INVALID_VALUE;
  if (kv && (vin == nullptr || vout == nullptr)) return GMS_ERROR_INVALID_VALUE;
  const SortLayout L = sort_layout_wide(n, key_bytes, value_bytes, sch);
  if (scratch_bytes < L.bytes) return GMS_ERROR_SCRATCH_TOO_SMALL;
  const size_t kb = size_t(n) * key_bytes, vb = size_t(n) * value_bytes;
  if (sch.passes == 0) {
    if (overlaps(kin, kout, n, key_bytes, key_bytes) || (kv && overlaps(vin, vout, n, value_bytes, value_bytes)))
      return GMS_ERROR_INVALID_VALUE;
    cudaError_t e = cudaMemcpyAsync(kout, kin, kb, cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess && kv) e = cudaMemcpyAsync(vout, vin, vb, cudaMemcpyDeviceToDevice, stream);
    return cuda_status(e);
  }
  auto* base = static_cast<unsigned char*>(scratch);
  void* tk = base + L.off_keys;
  void* tv = kv ? base + L.off_vals : nullptr;
  const void* ki = kin;
  const void* vi = vin;
  for (int p = 0; p < sch.passes; ++p) {
    const bool to_out = ((sch.passes - 1 - p) % 2) == 0;
    void* ko = to_out ? kout : tk;
    void* vo = to_out ? vout : tv;
    gms_bucket_desc64 d{};
    d.kind = GMS_BUCKET_BITS;
    d.num_buckets = sch.buckets[p];
    d.shift = sch.shift[p];
    gms_status st = multisplit_wide_impl(ki, kv ? vi : nullptr, ko, kv ? vo : nullptr, n, key_bytes, value_bytes,
                                         &d, scratch, L.ms_bytes, stream);
    if (st != GMS_SUCCESS) return st;
    ki = ko;
    vi = vo;
  }
  return GMS_SUCCESS;
}

}  // namespace

uint32_t tile_keys(int logb, bool kv) {
#define GMS_TILE_CASE(L) \
  case L: return kv ? tile_of<L, true>() : tile_of<L, false>();
  switch (logb) {
    GMS_TILE_CASE(1)
    GMS_TILE_CASE(2)
    GMS_TILE_CASE(3)
    GMS_TILE_CASE(4)
    GMS_TILE_CASE(5)
    GMS_TILE_CASE(6)
    GMS_TILE_CASE(7)
    GMS_TILE_CASE(8)
    default: return 0;
  }
#undef GMS_TILE_CASE
}

cudaError_t run_scan(uint32_t* data, uint32_t m, uint64_t* status, ScratchHeader* hdr, cudaStream_t stream) {
  if (m == 0) return cudaSuccess;
  const uint32_t chunks = (m + SCAN_CHUNK - 1) / SCAN_CHUNK;
  return launch_after_previous(scan_kernel, dim3(chunks), dim3(SCAN_THREADS), 0, stream, data, m, status, hdr);
}

void note_cuda_error(cudaError_t e) { g_last_cuda_error = int(e); }

int device_sm_count() {
  static std::atomic<int> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 132;
  int v = cached[dev & 63].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 132;
  cached[dev & 63].store(v, std::memory_order_relaxed);
  return v;
}

}  // namespace gms

using namespace gms;

extern "C" {

int gms_version(void) { return 100; }

const char* gms_status_string(gms_status s) {
  switch (s) {
    case GMS_SUCCESS: return "success";
    case GMS_ERROR_INVALID_VALUE: return "invalid value";
    case GMS_ERROR_UNSUPPORTED_BUCKETS:
      return "unsupported number of buckets: 2..256, up to 65536 for the one-call multisplit and the histogram "
             "(8192 range splitters), a power of two for bit-field buckets";
    case GMS_ERROR_SCRATCH_TOO_SMALL: return "scratch buffer too small";
    case GMS_ERROR_CUDA: return "CUDA runtime error";
    case GMS_ERROR_DEVICE_TIMEOUT: return "device-side wait timed out";
    case GMS_ERROR_NOT_SUPPORTED: return "not supported";
  }
  return "unknown status";
}

int gms_last_cuda_error(void) { return g_last_cuda_error; }

gms_status gms_read_device_error(const void* d_scratch, uint32_t* h_code, gms_stream_t stream) {
  if (d_scratch == nullptr || h_code == nullptr) return GMS_ERROR_INVALID_VALUE;
  cudaError_t e = cudaMemcpyAsync(h_code, d_scratch, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_status(e);
  return *h_code == 0 ? GMS_SUCCESS : GMS_ERROR_DEVICE_TIMEOUT;
}

gms_status gms_multisplit_scratch_bytes(uint32_t max_elements, uint32_t num_buckets, int key_value,
                                        size_t* bytes) {
  int logb = 0;
  if (bytes == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (num_buckets > 256 && num_buckets <= BIG_MAX_BUCKETS) {
    *bytes = big_layout(max_elements, num_buckets, key_value != 0).bytes;
    return GMS_SUCCESS;
  }
  if (!valid_buckets(num_buckets, &logb)) return GMS_ERROR_UNSUPPORTED_BUCKETS;
  *bytes = make_geometry(max_elements, logb, key_value != 0).bytes_full;
  return GMS_SUCCESS;
}

gms_status gms_multisplit_geometry(uint32_t n, uint32_t num_buckets, int key_value, uint32_t* tile_keys_out,
                                   uint32_t* num_tiles, size_t* matrix_offset_bytes) {
  int logb = 0;
  if (!valid_buckets(num_buckets, &logb)) return GMS_ERROR_UNSUPPORTED_BUCKETS;
  const Geometry g = make_geometry(n, logb, key_value != 0);
  if (tile_keys_out) *tile_keys_out = g.tile;
  if (num_tiles) *num_tiles = g.num_tiles;
  if (matrix_offset_bytes) *matrix_offset_bytes = g.off_matrix;
  return GMS_SUCCESS;
}

gms_status gms_multisplit_key_only(const uint32_t* d_key_in, uint32_t* d_key_out, uint32_t n,
                                   const gms_bucket_desc* desc, void* d_scratch, size_t scratch_bytes,
                                   uint32_t* h_offsets, gms_stream_t stream) {
  if (is_big(desc))
    return multisplit_big_impl(d_key_in, nullptr, d_key_out, nullptr, n, desc, false, d_scratch, scratch_bytes,
                               h_offsets, stream);
  gms_status st = multisplit_impl(d_key_in, nullptr, d_key_out, nullptr, n, desc, false, d_scratch, scratch_bytes,
                                  STAGE_ALL, stream);
  if (st != GMS_SUCCESS || h_offsets == nullptr) return st;
  int logb = 0;
  valid_buckets(desc->num_buckets, &logb);
  return copy_offsets(d_scratch, n, logb, desc->num_buckets, false, h_offsets, stream);
}

gms_status gms_multisplit_key_value(const uint32_t* d_key_in, const uint32_t* d_value_in, uint32_t* d_key_out,
                                    uint32_t* d_value_out, uint32_t n, const gms_bucket_desc* desc,
                                    void* d_scratch, size_t scratch_bytes, uint32_t* h_offsets,
                                    gms_stream_t stream) {
  if (is_big(desc))
    return multisplit_big_impl(d_key_in, d_value_in, d_key_out, d_value_out, n, desc, true, d_scratch,
                               scratch_bytes, h_offsets, stream);
  gms_status st = multisplit_impl(d_key_in, d_value_in, d_key_out, d_value_out, n, desc, true, d_scratch,
                                  scratch_bytes, STAGE_ALL, stream);
  if (st != GMS_SUCCESS || h_offsets == nullptr) return st;
  int logb = 0;
  valid_buckets(desc->num_buckets, &logb);
  return copy_offsets(d_scratch, n, logb, desc->num_buckets, true, h_offsets, stream);
}

gms_status gms_multisplit_prescan(const uint32_t* d_key_in, uint32_t n, const gms_bucket_desc* desc, int key_value,
                                  void* d_scratch, size_t scratch_bytes, gms_stream_t stream) {
  return multisplit_impl(d_key_in, nullptr, nullptr, nullptr, n, desc, key_value != 0, d_scratch, scratch_bytes,
                         STAGE_PRESCAN, stream);
}

gms_status gms_multisplit_scan(uint32_t n, const gms_bucket_desc* desc, int key_value, void* d_scratch,
                               size_t scratch_bytes, gms_stream_t stream) {
  return multisplit_impl(nullptr, nullptr, nullptr, nullptr, n, desc, key_value != 0, d_scratch, scratch_bytes,
                         STAGE_SCAN, stream);
}

gms_status gms_multisplit_postscan(const uint32_t* d_key_in, const uint32_t* d_value_in, uint32_t* d_key_out,
                                   uint32_t* d_value_out, uint32_t n, const gms_bucket_desc* desc,
                                   void* d_scratch, size_t scratch_bytes, gms_stream_t stream) {
  return multisplit_impl(d_key_in, d_value_in, d_key_out, d_value_out, n, desc, d_value_in != nullptr, d_scratch,
                         scratch_bytes, STAGE_POSTSCAN, stream);
}

gms_status gms_sort_set_method(int method) {
  if (method != GMS_SORT_AUTO && method != GMS_SORT_MULTISPLIT && method != GMS_SORT_ONESWEEP)
    return GMS_ERROR_INVALID_VALUE;
  g_sort_method.store(method, std::memory_order_relaxed);
  return GMS_SUCCESS;
}

gms_status gms_sort_get_method(int* method) {
  if (method == nullptr) return GMS_ERROR_INVALID_VALUE;
  *method = g_sort_method.load(std::memory_order_relaxed);
  return GMS_SUCCESS;
}

gms_status gms_sort_scratch_bytes(uint32_t max_elements, int digit_bits, int key_value, size_t* bytes) {
  SortSchedule sch;
  if (bytes == nullptr || !sort_schedule(digit_bits, &sch)) return GMS_ERROR_INVALID_VALUE;
  *bytes = sort_layout(max_elements, key_value != 0, sch).bytes;
  return GMS_SUCCESS;
}

gms_status gms_sort_key_only(const uint32_t* d_key_in, uint32_t* d_key_out, uint32_t n, int digit_bits,
                             void* d_scratch, size_t scratch_bytes, gms_stream_t stream) {
  return sort_impl(d_key_in, d_key_out, nullptr, nullptr, n, false, digit_bits, d_scratch, scratch_bytes, stream);
}

gms_status gms_sort_key_value(const uint32_t* d_key_in, uint32_t* d_key_out, const uint32_t* d_value_in,
                              uint32_t* d_value_out, uint32_t n, int digit_bits, void* d_scratch,
                              size_t scratch_bytes, gms_stream_t stream) {
  return sort_impl(d_key_in, d_key_out, d_value_in, d_value_out, n, true, digit_bits, d_scratch, scratch_bytes,
                   stream);
}

gms_status gms_sort_bits_scratch_bytes(uint32_t max_elements, int begin_bit, int end_bit, int digit_bits,
                                      int key_value, size_t* bytes) {
  SortSchedule sch;
  if (bytes == nullptr || !bit_schedule(begin_bit, end_bit, digit_bits, &sch)) return GMS_ERROR_INVALID_VALUE;
  *bytes = sort_layout(max_elements, key_value != 0, sch).bytes;
  return GMS_SUCCESS;
}

gms_status gms_sort_bits_key_only(const uint32_t* d_key_in, uint32_t* d_key_out, uint32_t n, int begin_bit,
                                  int end_bit, int digit_bits, void* d_scratch, size_t scratch_bytes,
                                  gms_stream_t stream) {
  SortSchedule sch;
  if (!bit_schedule(begin_bit, end_bit, digit_bits, &sch)) return GMS_ERROR_INVALID_VALUE;
  return sort_run(d_key_in, d_key_out, nullptr, nullptr, n, false, sch, d_scratch, scratch_bytes, stream);
}

gms_status gms_sort_bits_key_value(const uint32_t* d_key_in, uint32_t* d_key_out, const uint32_t* d_value_in,
                                   uint32_t* d_value_out, uint32_t n, int begin_bit, int end_bit, int digit_bits,
                                   void* d_scratch, size_t scratch_bytes, gms_stream_t stream) {
  SortSchedule sch;
  if (!bit_schedule(begin_bit, end_bit, digit_bits, &sch)) return GMS_ERROR_INVALID_VALUE;
  return sort_run(d_key_in, d_key_out, d_value_in, d_value_out, n, true, sch, d_scratch, scratch_bytes, stream);
}

gms_status gms_sort_7bit_scratch_bytes(uint32_t max_elements, int key_value, size_t* bytes) {
  return gms_sort_scratch_bytes(max_elements, 7, key_value, bytes);
}

gms_status gms_sort_7bit_key_only(const uint32_t* d_key_in, uint32_t* d_key_out, uint32_t n, void* d_scratch,
                                  size_t scratch_bytes, gms_stream_t stream) {
  return gms_sort_key_only(d_key_in, d_key_out, n, 7, d_scratch, scratch_bytes, stream);
}

gms_status gms_sort_7bit_key_value(const uint32_t* d_key_in, uint32_t* d_key_out, const uint32_t* d_value_in,
                                   uint32_t* d_value_out, uint32_t n, void* d_scratch, size_t scratch_bytes,
                                   gms_stream_t stream) {
  return gms_sort_key_value(d_key_in, d_key_out, d_value_in, d_value_out, n, 7, d_scratch, scratch_bytes, stream);
}

gms_status gms_compaction_scratch_bytes(uint32_t max_elements, int key_value, size_t* bytes) {
  return gms_multisplit_scratch_bytes(max_elements, 2, key_value, bytes);
}

gms_status gms_compaction_key_only(const uint32_t* d_key_in, uint32_t* d_key_out, uint32_t n,
                                   const gms_bucket_desc* desc, void* d_scratch, size_t scratch_bytes,
                                   uint32_t* h_num_bucket0, gms_stream_t stream) {
  return compaction_impl(d_key_in, nullptr, d_key_out, nullptr, n, desc, false, d_scratch, scratch_bytes,
                         h_num_bucket0, stream);
}

gms_status gms_compaction_key_value(const uint32_t* d_key_in, const uint32_t* d_value_in, uint32_t* d_key_out,
                                    uint32_t* d_value_out, uint32_t n, const gms_bucket_desc* desc,
                                    void* d_scratch, size_t scratch_bytes, uint32_t* h_num_bucket0,
                                    gms_stream_t stream) {
  return compaction_impl(d_key_in, d_value_in, d_key_out, d_value_out, n, desc, true, d_scratch, scratch_bytes,
                         h_num_bucket0, stream);
}

gms_status gms_histogram(const uint32_t* d_key_in, uint32_t n, const gms_bucket_desc* desc, int32_t* d_hist,
                         gms_stream_t stream) {
  if (is_big(desc)) {
    gms_status st = check_big_desc(desc);
    if (st != GMS_SUCCESS) return st;
    if (d_hist == nullptr) return GMS_ERROR_INVALID_VALUE;
    if (n == 0) return GMS_SUCCESS;
    if (d_key_in == nullptr) return GMS_ERROR_INVALID_VALUE;
    return cuda_status(dispatch_big_histogram(desc->kind, d_key_in, n, to_params(desc),
                                              reinterpret_cast<uint32_t*>(d_hist), stream));
  }
  int logb = 0;
  gms_status st = check_desc(desc, &logb);
  if (st != GMS_SUCCESS) return st;
  if (d_hist == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (n == 0) return GMS_SUCCESS;
  if (d_key_in == nullptr) return GMS_ERROR_INVALID_VALUE;
  return cuda_status(dispatch_hist(desc->kind, d_key_in, n, logb, to_params(desc), d_hist, stream));
}

gms_status gms_histogram_even(const uint32_t* d_key_in, uint32_t n, int32_t* d_hist, uint32_t num_bins,
                              uint32_t lower, uint32_t upper, float inverse_delta, gms_stream_t stream) {
  (void)upper;  // the reference kernels take it but bin with lower and inverse_delta only
  gms_bucket_desc d{};
  d.kind = GMS_BUCKET_EVEN_FLOAT;
  d.num_buckets = num_bins;
  d.lower = lower;
  d.inverse_delta = inverse_delta;
  return gms_histogram(d_key_in, n, &d, d_hist, stream);
}

gms_status gms_histogram_range(const uint32_t* d_key_in, uint32_t n, int32_t* d_hist, uint32_t num_bins,
                               const uint32_t* d_levels, gms_stream_t stream) {
  gms_bucket_desc d{};
  d.kind = GMS_BUCKET_RANGE;
  d.num_buckets = num_bins;
  d.d_splitters = d_levels;
  return gms_histogram(d_key_in, n, &d, d_hist, stream);
}

gms_status gms_multisplit_wide_scratch_bytes(uint32_t max_elements, uint32_t num_buckets, int key_bytes,
                                             int value_bytes, size_t* bytes) {
  int logb = 0;
  if (bytes == nullptr || !valid_widths(key_bytes, value_bytes)) return GMS_ERROR_INVALID_VALUE;
  if (!valid_buckets(num_buckets, &logb)) return GMS_ERROR_UNSUPPORTED_BUCKETS;
  const bool kv = value_bytes != 0;
  *bytes = make_geometry(max_elements, logb, kv, key_bytes / 4, kv ? value_bytes / 4 : 1).bytes_full;
  return GMS_SUCCESS;
}

gms_status gms_multisplit_wide(const void* d_key_in, const void* d_value_in, void* d_key_out, void* d_value_out,
                               uint32_t n, int key_bytes, int value_bytes, const gms_bucket_desc64* desc,
                               void* d_scratch, size_t scratch_bytes, uint32_t* h_offsets, gms_stream_t stream) {
  gms_status st = multisplit_wide_impl(d_key_in, d_value_in, d_key_out, d_value_out, n, key_bytes, value_bytes, desc,
                                       d_scratch, scratch_bytes, stream);
  if (st != GMS_SUCCESS || h_offsets == nullptr) return st;
  int logb = 0;
  valid_buckets(desc->num_buckets, &logb);
  const bool kv = value_bytes != 0;
  return copy_offsets(d_scratch, n, logb, desc->num_buckets, kv, h_offsets, stream, key_bytes / 4,
                      kv ? value_bytes / 4 : 1);
}

gms_status gms_histogram_wide(const void* d_key_in, uint32_t n, int key_bytes, const gms_bucket_desc64* desc,
                              int32_t* d_hist, gms_stream_t stream) {
  if (key_bytes == 4) {
    gms_bucket_desc d32;
    gms_status st = narrow_desc(desc, &d32);
    if (st != GMS_SUCCESS) return st;
    return gms_histogram(static_cast<const uint32_t*>(d_key_in), n, &d32, d_hist, stream);
  }
  if (key_bytes != 8) return GMS_ERROR_INVALID_VALUE;
  int logb = 0;
  gms_status st = check_desc64(desc, &logb);
  if (st != GMS_SUCCESS) return st;
  if (d_hist == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (n == 0) return GMS_SUCCESS;
  if (d_key_in == nullptr || (reinterpret_cast<uintptr_t>(d_key_in) & 7u) != 0) return GMS_ERROR_INVALID_VALUE;
  const auto* keys = static_cast<const uint64_t*>(d_key_in);
  const BucketParams64 bp = to_params64(desc);
  cudaError_t e = cudaErrorInvalidValue;
  switch (desc->kind) {
    case KIND_DELTA: e = run_histogram64<KIND_DELTA>(keys, n, logb, bp, d_hist, stream); break;
    case KIND_DIV: e = run_histogram64<KIND_DIV>(keys, n, logb, bp, d_hist, stream); break;
    case KIND_BITS: e = run_histogram64<KIND_BITS>(keys, n, logb, bp, d_hist, stream); break;
    case KIND_RANGE: e = run_histogram64<KIND_RANGE>(keys, n, logb, bp, d_hist, stream); break;
    case KIND_MASK: e = run_histogram64<KIND_MASK>(keys, n, logb, bp, d_hist, stream); break;
    case KIND_EVEN_FLOAT: e = run_histogram64<KIND_EVEN_FLOAT>(keys, n, logb, bp, d_hist, stream); break;
    default: break;
  }
  return cuda_status(e);
}

gms_status gms_sort_wide_scratch_bytes(uint32_t max_elements, int key_bytes, int value_bytes, int begin_bit,
                                       int end_bit, int digit_bits, size_t* bytes) {
  SortSchedule sch;
  if (bytes == nullptr || !valid_widths(key_bytes, value_bytes) ||
      !bit_schedule(begin_bit, end_bit, digit_bits, &sch, 8 * key_bytes))
    return GMS_ERROR_INVALID_VALUE;
  *bytes = sort_layout_wide(max_elements, key_bytes, value_bytes, sch).bytes;
  return GMS_SUCCESS;
}

gms_status gms_sort_wide(const void* d_key_in, void* d_key_out, const void* d_value_in, void* d_value_out, uint32_t n,
                         int key_bytes, int value_bytes, int begin_bit, int end_bit, int digit_bits, void* d_scratch,
                         size_t scratch_bytes, gms_stream_t stream) {
  SortSchedule sch;
  if (!valid_widths(key_bytes, value_bytes) || !bit_schedule(begin_bit, end_bit, digit_bits, &sch, 8 * key_bytes))
    return GMS_ERROR_INVALID_VALUE;
  return sort_wide_run(d_key_in, d_key_out, d_value_in, d_value_out, n, key_bytes, value_bytes, sch, d_scratch,
                       scratch_bytes, stream);
}

}  // extern "C"
