// Host-side internals shared by the C ABI (capi.cu) and the per-identifier
// instantiation units (inst_*.cu): tile geometry, scratch layout, launchers.
#pragma once

#include <utility>

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/gpumultisplit.h"
#include "gms_device.cuh"

namespace gms {

// Tile shape per (log2 B, key/value).  Keys per tile = WARPS * 32 * IPT.
// 4096-key tiles of 8 warps x 16 keys per thread measured best on GB300 for
// every B (16 x 8 and 16 x 16 shapes, and 8 x 8, were slower); at B = 256 the
// count matrix is then 1 byte per key.
//
// With 64-bit keys or values (KW / VW = 32-bit words per key / value) the
// keys per thread (a multiple of 4) depend on the bytes a key brings, e:
//   e = 8, 64-bit keys alone  GMS_WIDE8_IPT (16)
//   e = 12                    GMS_WIDE12_IPT (16)
//   e = 16                    GMS_WIDE16_IPT (12: 3072-key tiles of 62 KB staged,
//                             three blocks per SM)
// Measured at 2^28 keys, B = 256: 64-bit keys with 64-bit values ran at 104 /
// 122 / 116 Gkeys/s with 8 / 12 / 16 keys per thread, the 12-byte pairs at
// 110-123 / 131-153 / 142-167.
#ifndef GMS_WIDE8_IPT
#define GMS_WIDE8_IPT 16
#endif
#ifndef GMS_WIDE12_IPT
#define GMS_WIDE12_IPT 16
#endif
#ifndef GMS_WIDE16_IPT
#define GMS_WIDE16_IPT 12
#endif
constexpr int tile_ipt(bool kv, int kw, int vw) {
  return kw == 1 && (!kv || vw == 1) ? 16
         : 4 * kw + (kv ? 4 * vw : 0) <= 8 ? GMS_WIDE8_IPT
         : 4 * kw + (kv ? 4 * vw : 0) <= 12 ? GMS_WIDE12_IPT
                                            : GMS_WIDE16_IPT;
}

template <int LOGB, bool KV, int KW = 1, int VW = 1>
struct TileShape {
  static constexpr int WARPS = 8;
  static constexpr int IPT = tile_ipt(KV, KW, VW);
};

uint32_t tile_keys(int logb, bool kv);

// Tile shapes the batched form can run, chosen per (bucket count, key/value,
// segment size class) by the tuning table (tuning.cu).  Variant 0 is the plain
// path's shape.  A shape needs at least one thread per bucket (tile scan).
struct TileVariantShape {
  int warps;
  int ipt;  // keys per thread
};
constexpr int kNumTileVariants = 4;
constexpr TileVariantShape kTileVariants[kNumTileVariants] = {{8, 16}, {8, 8}, {8, 4}, {4, 16}};
inline bool variant_valid(int v, int logb) {
  return v >= 0 && v < kNumTileVariants && kTileVariants[v].warps * 32 >= (1 << logb);
}
inline uint32_t variant_tile_keys(int v) { return uint32_t(kTileVariants[v].warps) * 32u * kTileVariants[v].ipt; }

// Segment size classes of the tuning table: 0 for n <= 2^10, c for
// 2^(9+c) < n <= 2^(10+c), up to kNumSizeClasses - 1 for n > 2^16.
constexpr int kNumSizeClasses = 8;
inline int size_class(uint32_t n) {
  int c = 0;
  while (c < kNumSizeClasses - 1 && n > (1u << (10 + c))) ++c;
  return c;
}

// Variant the batched form uses for a segment (the tuning table's entry).
int tuned_variant(int logb, bool kv, uint32_t n);

constexpr uint32_t kScanChunk = 256u * GMS_SCAN_IPT;  // SCAN_CHUNK in scan_kernels.cuh

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Scratch layout of one multisplit: [header 256 B][count matrix u32 x B*tiles][scan status u64 x chunks].
// The matrix always starts at byte 256, whatever n is.
struct Geometry {
  uint32_t tile = 0;
  uint32_t num_tiles = 0;
  uint32_t m = 0;           // B * num_tiles
  uint32_t num_chunks = 0;  // scan chunks
  size_t off_status = 0;
  size_t off_matrix = 0;
  size_t bytes = 0;         // what every identifier needs
  size_t off_buckets = 0;   // one byte per key, used by costly identifiers when the scratch has room
  size_t bytes_full = 0;    // bytes plus the bucket bytes (what gms_multisplit_scratch_bytes reports)
};

// kw / vw: 32-bit words per key / value (2 for 64-bit elements).
inline Geometry make_geometry(uint32_t n, int logb, bool kv, int kw = 1, int vw = 1) {
  Geometry g;
  g.tile = (kw == 1 && (vw == 1 || !kv)) ? tile_keys(logb, kv) : 8u * 32u * uint32_t(tile_ipt(kv, kw, vw));
  g.num_tiles = uint32_t((uint64_t(n) + g.tile - 1) / g.tile);
  g.m = (1u << logb) * g.num_tiles;
  g.num_chunks = (g.m + kScanChunk - 1) / kScanChunk;
  g.off_matrix = sizeof(ScratchHeader);
  g.off_status = align_up(g.off_matrix + size_t(g.m) * 4, 256);
  g.bytes = align_up(g.off_status + size_t(g.num_chunks) * 8, 256);
  g.off_buckets = g.bytes;
  g.bytes_full = align_up(g.off_buckets + size_t(n), 256);
  return g;
}

// Identifier kinds costly enough to evaluate once (in the prescan) and keep
// as one byte per key for the postscan.
inline bool kind_keeps_bucket_bytes(int kind) {
  return kind == KIND_RANGE || kind == KIND_DIV || kind == KIND_EVEN_FLOAT;
}

enum Stage : int { STAGE_PRESCAN = 1, STAGE_SCAN = 2, STAGE_POSTSCAN = 4, STAGE_ALL = 7 };

struct MsCall {
  const uint32_t* kin = nullptr;
  const uint32_t* vin = nullptr;
  uint32_t* kout = nullptr;
  uint32_t* vout = nullptr;
  uint32_t n = 0;
  int logb = 1;
  bool kv = false;
  BucketParams bp{};
  unsigned char* scratch = nullptr;  // laid out as make_geometry(n, logb, kv)
  cudaStream_t stream = nullptr;
  uint8_t* bucket_bytes = nullptr;   // in scratch, or null (see launch_multisplit)
};

// Runs the requested stages (a mask of Stage) of one multisplit.  Defined per
// identifier kind in inst_*.cu.
template <int KIND>
cudaError_t run_multisplit(const MsCall& c, int stages);

// A multisplit with 64-bit keys (kw = 2) or 64-bit values (vw = 2).  32-bit
// keys are identified with bp, 64-bit keys with bp64; 64-bit keys need
// bucket_bytes (n bytes in the scratch).
struct MsCallWide {
  const void* kin = nullptr;
  const void* vin = nullptr;
  void* kout = nullptr;
  void* vout = nullptr;
  uint32_t n = 0;
  int logb = 1;
  bool kv = false;
  int kw = 1;
  int vw = 1;
  BucketParams bp{};
  BucketParams64 bp64{};
  unsigned char* scratch = nullptr;  // laid out as make_geometry(n, logb, kv, kw, vw)
  cudaStream_t stream = nullptr;
  uint8_t* bucket_bytes = nullptr;
};

// Defined per identifier kind in inst_wide.cu (compiled once per kind).
template <int KIND>
cudaError_t run_multisplit_wide(const MsCallWide& c, int stages);
// Histogram of 64-bit keys into hist[0..B) (inst_wide.cu).
template <int KIND>
cudaError_t run_histogram64(const uint64_t* keys, uint32_t n, int logb, const BucketParams64& bp, int32_t* hist,
                            cudaStream_t stream);

// One digit pass of a multisplit with more than 256 buckets (32-bit keys and
// values): 2^logb buckets of digit (id >> bp.digit_shift); the scratch is laid
// out as make_geometry(n, logb, kv) and bucket_bytes holds n bytes.
struct DigitPass {
  const uint32_t* kin = nullptr;
  const uint32_t* vin = nullptr;
  uint32_t* kout = nullptr;
  uint32_t* vout = nullptr;
  uint32_t n = 0;
  int logb = 8;
  bool kv = false;
  BucketParamsBig bp{};
  unsigned char* scratch = nullptr;
  uint8_t* bucket_bytes = nullptr;
  cudaStream_t stream = nullptr;
};

// Prescan (identifier evaluated, digit kept as a byte) and scan of a digit
// pass; defined per kind in inst_big.cu.
template <int KIND>
cudaError_t run_digit_prescan_scan(const DigitPass& c);
// Postscan of a digit pass from the bytes (inst_big_post.cu).
cudaError_t run_digit_postscan(const DigitPass& c);
// Adds the count of every whole bucket id in [0, p.num_buckets) into hist
// (inst_big.cu).
template <int KIND>
cudaError_t run_big_histogram(const uint32_t* keys, uint32_t n, const BucketParams& p, uint32_t* hist,
                              cudaStream_t stream);
// Bucket starts of a multisplit by the whole id, from its sorted output
// (inst_big.cu): starts[0..p.num_buckets).
template <int KIND>
cudaError_t run_big_offsets(const uint32_t* sorted_keys, uint32_t n, const BucketParams& p, uint32_t* starts,
                            cudaStream_t stream);

// Histogram of keys[0..n) into hist[0..2^logb), accumulated with atomics.
template <int KIND>
cudaError_t run_histogram(const uint32_t* keys, uint32_t n, int logb, const BucketParams& bp, int32_t* hist,
                          cudaStream_t stream);

// Launches `kern` on `stream` with programmatic stream serialization: its
// blocks may be scheduled while the previous kernel on the stream finishes,
// and they wait for it (griddep_wait) before they touch its results.  The
// scan and the postscan of a multisplit are launched this way.
template <class... KArgs, class... Args>
cudaError_t launch_after_previous(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                                  Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

cudaError_t run_scan(uint32_t* data, uint32_t m, uint64_t* status, ScratchHeader* hdr, cudaStream_t stream);

struct SegDesc;

// One class of a batched multisplit (same kind, log2 B and key/value shape).
struct BatchClassLaunch {
  int logb = 1;
  bool kv = false;
  int variant = 0;                  // tile shape (kTileVariants)
  const SegDesc* segs = nullptr;    // device
  const uint2* tile_map = nullptr;  // device, class_tiles entries of (segment, tile)
  uint32_t class_tiles = 0;
  uint32_t* matrix = nullptr;       // device, the batch count matrix
  uint8_t* byte_area = nullptr;     // device, bucket bytes of segments with costly identifiers
  const uint32_t* seg_ids = nullptr;  // device, segments of a one-warp-per-segment class
  ScratchHeader* hdr = nullptr;
  cudaStream_t stream = nullptr;
};

// Launches the prescan (STAGE_PRESCAN) or postscan (STAGE_POSTSCAN) of one
// batch class with tile variant V.  Instantiated per (kind, variant) from
// inst_batch.cu.
template <int KIND, int V>
cudaError_t run_batch_class_v(const BatchClassLaunch& c, int stage);

// Segments of at most this many keys are multisplit one warp each (tuned plans).
constexpr uint32_t kWarpSegMax = 512;

// Launches the one-warp-per-segment kernel of a class of small segments:
// c.seg_ids lists c.class_tiles segments (inst_batch.cu, variant 0 units).
template <int KIND>
cudaError_t run_batch_warp(const BatchClassLaunch& c);

// Dispatch on the class's kind and variant (batch.cu).
cudaError_t run_batch_class(int kind, const BatchClassLaunch& c, int stage);

struct QSeg;

// The one-launch schedule of a batch (inst_queue.cu): its segment records and
// work list, the count matrix and bucket bytes in the queue's layout, and the
// run state (ticket, then per segment the PRE tiles and SCAN chunks done,
// zeroed before each launch) with the chunks' look-back words.
struct BatchQueueLaunch {
  const QSeg* qsegs = nullptr;   // device
  const uint2* items = nullptr;  // device
  uint32_t num_items = 0;
  uint32_t num_segs = 0;
  uint32_t* matrix = nullptr;
  uint8_t* byte_area = nullptr;
  uint32_t* state = nullptr;     // 1 + 2 * num_segs words
  uint64_t* status = nullptr;
  ScratchHeader* hdr = nullptr;
  cudaStream_t stream = nullptr;
};
cudaError_t run_batch_queue(const BatchQueueLaunch& c);

// Creates a batch plan whose every class uses `variant` (>= 0), or the tuning
// table's choice per segment (variant < 0).
gms_status batch_create(const gms_segment* segments, uint32_t count, int variant, gms_batch_t* batch);

int device_sm_count();

// One-sweep LSD sort of 32-bit keys (onesweep.cu): digit p is
// (key >> shift[p]) & (2^logb[p] - 1), passes <= 8, each logb in [1, 8].
// onesweep_scratch_bytes is what it needs in front of the ping-pong buffers;
// run_onesweep_sort sorts kin (vin) into kout (vout) through tk (tv), the
// ping-pong buffers, exactly as the multisplit passes would.
constexpr int kOnesweepMaxPasses = 8;
// Sorts of at least this many keys take the one-sweep passes by default
// (none: on GB300 they measured slower than the multisplit passes, 7.4 against
// 5.6 ms for 2^28 pairs with 7-bit digits).
constexpr uint32_t kOnesweepMinKeys = 0xFFFFFFFFu;
size_t onesweep_scratch_bytes(uint32_t n, int passes, const uint32_t* logb);
cudaError_t run_onesweep_sort(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                              bool kv, int passes, const uint32_t* shift, const uint32_t* logb,
                              unsigned char* scratch, uint32_t* tk, uint32_t* tv, cudaStream_t stream);

// Batch internals used by the serving runtime: bytes of the plan's tables, and
// a run that stages the tables through caller-owned pinned memory (at least
// batch_table_bytes) with one asynchronous copy instead of a synchronous bind.
size_t batch_table_bytes(gms_batch_t b);
gms_status batch_run_async(gms_batch_t b, void* d_scratch, size_t scratch_bytes, void* h_pinned,
                           size_t pinned_bytes, cudaStream_t stream);
// Index (in uint32 words from the start of the batch scratch) of the scanned
// offset of (segment, bucket, tile); *base receives the segment's scan base.
uint32_t batch_matrix_value_offset(gms_batch_t b, uint32_t segment, uint32_t bucket, uint32_t tile, uint32_t* base);

// Records a CUDA error for gms_last_cuda_error() (calling thread).
void note_cuda_error(cudaError_t e);

}  // namespace gms
