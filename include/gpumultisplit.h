/*
 * gpumultisplit.h -- C ABI of the GB300 (sm_103a) multisplit library.
 *
 * Plain pointers and sizes only: every pointer named d_* is a device pointer,
 * every h_* pointer is host memory.  All calls are asynchronous on `stream`
 * unless they say otherwise; a null stream is the legacy default stream, the
 * stream every reference entry point runs on.
 *
 * Each entry point cites the reference interface it replaces (paths inside the
 * owensgroup/GpuMultisplit tree).  The reference instantiates its kernels on a
 * user functor type; a precompiled ABI cannot, so the bucket identifier is a
 * POD descriptor (gms_bucket_desc) that covers the functors the reference and
 * its drivers use.  The drop-in C++ headers in include/gpumultisplit/ map
 * functor types onto descriptors.
 *
 * Scratch: the reference's contexts cudaMalloc a bucket-count matrix plus CUB
 * scan storage (src/api/multisplit.cuh:50-74).  Here the caller owns one
 * scratch buffer whose size *_scratch_bytes() reports; the library never
 * allocates.  A scratch buffer serves one call at a time (calls that overlap
 * on the GPU and share a buffer race).
 */
#ifndef GPUMULTISPLIT_H_
#define GPUMULTISPLIT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same object as cudaStream_t; declared here so the header needs no CUDA headers. */
typedef struct CUstream_st* gms_stream_t;

typedef enum gms_status {
  GMS_SUCCESS = 0,
  GMS_ERROR_INVALID_VALUE = 1,       /* null pointer, bad kind, n over capacity ... */
  GMS_ERROR_UNSUPPORTED_BUCKETS = 2, /* num_buckets outside what the call takes, or not a power of two for BITS */
  GMS_ERROR_SCRATCH_TOO_SMALL = 3,
  GMS_ERROR_CUDA = 4,                /* a CUDA runtime call failed; see gms_last_cuda_error() */
  GMS_ERROR_DEVICE_TIMEOUT = 5,      /* a bounded device-side wait gave up (read by gms_read_device_error) */
  GMS_ERROR_NOT_SUPPORTED = 6
} gms_status;

/*
 * Bucket identifier kinds.  Every kind yields a value that is reduced modulo
 * num_buckets (the reference's GPU kernels decode a bucket id from its low
 * log2(B) bits with ballots, src/kernels/bms/bms_prescan.cuh:480-517, so an
 * out-of-range id wraps the same way there).
 *
 * B may be any count in [2, 256] (the reference takes powers of two only;
 * for those every kind gives the same buckets as below).  The kernels then
 * run with the next power of two and leave the buckets from B up empty.
 * BITS needs a power of two.  Offsets and histograms hold B entries.
 *
 * gms_multisplit_key_only / _key_value, gms_multisplit_scratch_bytes and
 * gms_histogram also take B from 257 to 65536 (RANGE: up to 8192 splitters).
 * The multisplit then runs as two stable multisplits on the digits of the
 * bucket id (the low half of its bits, then the high half), through buffers
 * in the scratch; the result is the same stable order.  The stage entry points, the batched and
 * serving forms and the 64-bit entry points take B <= 256.
 *
 *  GMS_BUCKET_DELTA       key * B >> 32 (64-bit product): B equal-width key ranges.
 *  GMS_BUCKET_DIV         (key / param) mod B (delta_func, README.md:85-91, src/main/main_multisplit.cu:41-47).
 *  GMS_BUCKET_BITS        (key >> shift) & (B-1)  (ms_bucket_sort_*bit<shift>, src/api/multisplit_sort.cuh:63-98;
 *                          compaction's test_bucket<1> = key & 1, src/main/main_compaction.cu:26-31).
 *  GMS_BUCKET_RANGE       upper_bound(d_splitters[0..B), key) - 1 (cub::UpperBound on the level array,
 *                          src/kernels/histogram/multisplit2_histograms.cuh:434); keys below
 *                          d_splitters[0] give -1, i.e. bucket B-1 after the wrap.
 *                          Splitters need not be distinct.
 *  GMS_BUCKET_MASK        (key & param) != 0 (a two-bucket predicate).
 *  GMS_BUCKET_EVEN_FLOAT  (uint32)((float)(key - lower) * inverse_delta) mod B, float round-to-nearest
 *                          convert and multiply, truncating saturating convert back
 *                          (src/kernels/histogram/multisplit2_histograms.cuh:60).
 */
typedef enum gms_bucket_kind {
  GMS_BUCKET_DELTA = 0,
  GMS_BUCKET_DIV = 1,
  GMS_BUCKET_BITS = 2,
  GMS_BUCKET_RANGE = 3,
  GMS_BUCKET_MASK = 4,
  GMS_BUCKET_EVEN_FLOAT = 5
} gms_bucket_kind;

typedef struct gms_bucket_desc {
  int32_t kind;                /* gms_bucket_kind */
  uint32_t num_buckets;        /* B: 2..256, to 65536 where noted (a power of two for BITS) */
  uint32_t shift;              /* BITS */
  uint32_t param;              /* DIV: divisor (non-zero); MASK: mask */
  uint32_t lower;              /* EVEN_FLOAT: lower level */
  float inverse_delta;         /* EVEN_FLOAT: 1 / bin width */
  const uint32_t* d_splitters; /* RANGE: B sorted splitters, device memory */
} gms_bucket_desc;

/* ---------------------------------------------------------------- info */
int gms_version(void);
const char* gms_status_string(gms_status s);
/* Last CUDA error code seen by a call that returned GMS_ERROR_CUDA (per thread). */
int gms_last_cuda_error(void);

/* Device-side error word of a scratch buffer: 0 if the last call that used it
 * finished every bounded wait, else a non-zero code.  Synchronises `stream`. */
gms_status gms_read_device_error(const void* d_scratch, uint32_t* h_code, gms_stream_t stream);

/* ------------------------------------------------------------ multisplit */
/* Replaces multisplit_allocate_key_only / _key_value (src/api/multisplit.cuh:50-74):
 * scratch bytes for calls with n <= max_elements.  The size includes one byte
 * per key that identifiers costly to evaluate (range, div, even-float) use to
 * evaluate the identifier once instead of twice; a scratch without that room
 * (max_elements bytes less, rounded up to 256) still works, more slowly for
 * those identifiers. */
gms_status gms_multisplit_scratch_bytes(uint32_t max_elements, uint32_t num_buckets, int key_value,
                                        size_t* bytes);

/* Replaces multisplit_key_only (src/api/multisplit.cuh:81-197).  Stable: buckets
 * ascending, input order kept inside a bucket.  If h_offsets is non-null the
 * call synchronises and writes the B bucket start offsets there (:143-149). */
gms_status gms_multisplit_key_only(const uint32_t* d_key_in, uint32_t* d_key_out, uint32_t n,
                                   const gms_bucket_desc* desc, void* d_scratch, size_t scratch_bytes,
                                   uint32_t* h_offsets, gms_stream_t stream);

/* Replaces multisplit_key_value (src/api/multisplit.cuh:199-313); values move with their keys. */
gms_status gms_multisplit_key_value(const uint32_t* d_key_in, const uint32_t* d_value_in,
                                    uint32_t* d_key_out, uint32_t* d_value_out, uint32_t n,
                                    const gms_bucket_desc* desc, void* d_scratch, size_t scratch_bytes,
                                    uint32_t* h_offsets, gms_stream_t stream);

/* The three stages of one multisplit, callable one by one (the reference runs
 * them as prescan kernel, cub::DeviceScan::ExclusiveSum, postscan kernel:
 * src/api/multisplit.cuh:212-272).  Scratch sized by gms_multisplit_scratch_bytes
 * for the same n, B and key_value, and the same scratch_bytes passed to all
 * three (it decides whether the prescan leaves bucket bytes for the postscan).
 * After gms_multisplit_scan the count matrix in scratch holds global offsets,
 * bucket-major: offset(b, tile) at b*num_tiles+tile. */
gms_status gms_multisplit_prescan(const uint32_t* d_key_in, uint32_t n, const gms_bucket_desc* desc,
                                  int key_value, void* d_scratch, size_t scratch_bytes, gms_stream_t stream);
gms_status gms_multisplit_scan(uint32_t n, const gms_bucket_desc* desc, int key_value, void* d_scratch,
                               size_t scratch_bytes, gms_stream_t stream);
gms_status gms_multisplit_postscan(const uint32_t* d_key_in, const uint32_t* d_value_in, uint32_t* d_key_out,
                                   uint32_t* d_value_out, uint32_t n, const gms_bucket_desc* desc,
                                   void* d_scratch, size_t scratch_bytes, gms_stream_t stream);

/* Tile geometry the library uses for (n, B, key_value): keys per tile and number
 * of tiles (the reference's size_sub_prob / num_sub_prob, src/api/multisplit.cuh:29-47),
 * and the byte offset of the count matrix inside scratch. */
gms_status gms_multisplit_geometry(uint32_t n, uint32_t num_buckets, int key_value, uint32_t* tile_keys,
                                   uint32_t* num_tiles, size_t* matrix_offset_bytes);

/* Key-value multisplit that allocates nothing.  No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc where they need a multisplit
 * (allocator internals, plugin hosts that hand over only input and output
 * buffers, paths that must not allocate after start-up).  Its scratch is a fixed
 * GMS_NOALLOC_SCRATCH_BYTES array in device memory owned by the library (held on
 * every GPU that loads the library until the process exits).  A call is accepted
 * when the multisplit's minimum scratch (count matrix and scan state, without
 * the optional byte per key) fits: up to 16,764,928 pairs at 256 buckets, more
 * at fewer buckets, about 460 thousand at 1000 buckets (whose two digit passes
 * also keep ping-pong keys and values there).  Larger calls return
 * GMS_ERROR_SCRATCH_TOO_SMALL.  Range, div and even-float identifiers keep their
 * byte per key in the array only when it fits too; the output is the same.  The
 * first call on a device looks up the array's address with that device
 * current; make it before any stream capture.  All calls on a device share the
 * array, so calls that overlap on the GPU race; each call resets what it reads.
 * Output is identical to gms_multisplit_key_value (no bucket offsets). */
#define GMS_NOALLOC_SCRATCH_BYTES (4u << 20)
gms_status gms_multisplit_key_value_noalloc(const uint32_t* d_key_in, const uint32_t* d_value_in,
                                            uint32_t* d_key_out, uint32_t* d_value_out, uint32_t n,
                                            const gms_bucket_desc* desc, gms_stream_t stream);

/* ----------------------------------------------------------------- sort */
/* Replaces multisplit_sort_7bit_allocate / _allocate_pairs (src/api/multisplit_sort.cuh:151-191).
 * Includes the ping-pong key (and value) buffer the reference keeps in d_key_temp_ms. */
gms_status gms_sort_7bit_scratch_bytes(uint32_t max_elements, int key_value, size_t* bytes);

/* Replaces multisplit_sort_7bit (src/api/multisplit_sort.cuh:320-364): LSD radix
 * sort, digits [0,4) then [4,11) [11,18) [18,25) [25,32).  d_key_in is not modified. */
gms_status gms_sort_7bit_key_only(const uint32_t* d_key_in, uint32_t* d_key_out, uint32_t n, void* d_scratch,
                                  size_t scratch_bytes, gms_stream_t stream);

/* Replaces multisplit_sort_7bit_pairs (src/api/multisplit_sort_pairs.cuh:21-65).
 * Argument order follows the reference: (key_in, key_out, value_in, value_out). */
gms_status gms_sort_7bit_key_value(const uint32_t* d_key_in, uint32_t* d_key_out, const uint32_t* d_value_in,
                                   uint32_t* d_value_out, uint32_t n, void* d_scratch, size_t scratch_bytes,
                                   gms_stream_t stream);

/* The other digit widths of the reference's multisplit sorts
 * (multisplit_sort_{4,5,6,8}bit[_pairs], src/api/multisplit_sort.cuh:366-559,
 * src/api/multisplit_sort_pairs.cuh:67-260), same schedules:
 *   4: eight 4-bit passes;  5: six 5-bit passes then bits [30,32);
 *   6: 4-bit, 4-bit, then four 6-bit passes;  7: as above;  8: four 8-bit passes.
 * digit_bits outside 4..8 is GMS_ERROR_INVALID_VALUE. */
gms_status gms_sort_scratch_bytes(uint32_t max_elements, int digit_bits, int key_value, size_t* bytes);
gms_status gms_sort_key_only(const uint32_t* d_key_in, uint32_t* d_key_out, uint32_t n, int digit_bits,
                             void* d_scratch, size_t scratch_bytes, gms_stream_t stream);
gms_status gms_sort_key_value(const uint32_t* d_key_in, uint32_t* d_key_out, const uint32_t* d_value_in,
                              uint32_t* d_value_out, uint32_t n, int digit_bits, void* d_scratch,
                              size_t scratch_bytes, gms_stream_t stream);

/* How the 32-bit radix sorts above and below run their digits (process-wide,
 * default GMS_SORT_AUTO).  No counterpart in the reference, whose sorts run one
 * multisplit per digit:
 *   GMS_SORT_MULTISPLIT  prescan, scan and postscan per digit (the reference's way);
 *   GMS_SORT_ONESWEEP    one histogram pass for every digit, then one pass per
 *                        digit whose tiles find their offsets by decoupled
 *                        look-back (no count matrix, no scan);
 *   GMS_SORT_AUTO        the library's choice (at present the multisplit
 *                        passes, which measured faster on GB300).
 * Both give bit-identical output and fit the same scratch size. */
enum { GMS_SORT_AUTO = 0, GMS_SORT_MULTISPLIT = 1, GMS_SORT_ONESWEEP = 2 };
gms_status gms_sort_set_method(int method);
gms_status gms_sort_get_method(int* method);

/* Partial-key sorts: a stable sort by key bits [begin_bit, end_bit), as the
 * begin_bit / end_bit arguments of the CUB radix sorts the reference's drivers
 * compare against (src/main/main_bms.cu:199).  Digits of digit_bits (4..8)
 * bits from begin_bit, the last one narrower when the range is not a whole
 * number of digits; begin_bit == end_bit copies the input. */
gms_status gms_sort_bits_scratch_bytes(uint32_t max_elements, int begin_bit, int end_bit, int digit_bits,
                                      int key_value, size_t* bytes);
gms_status gms_sort_bits_key_only(const uint32_t* d_key_in, uint32_t* d_key_out, uint32_t n, int begin_bit,
                                  int end_bit, int digit_bits, void* d_scratch, size_t scratch_bytes,
                                  gms_stream_t stream);
gms_status gms_sort_bits_key_value(const uint32_t* d_key_in, uint32_t* d_key_out, const uint32_t* d_value_in,
                                   uint32_t* d_value_out, uint32_t n, int begin_bit, int end_bit, int digit_bits,
                                   void* d_scratch, size_t scratch_bytes, gms_stream_t stream);

/* ------------------------------------------- 64-bit keys and values */
/* No counterpart in the reference, whose kernels hold 32-bit keys and values
 * (src/kernels/bms/bms_postscan.cuh:38).  Keys are 4 or 8 bytes (key_bytes),
 * values 0 (key-only), 4 or 8 bytes (value_bytes); each array is aligned to
 * its element size.  The identifier kinds are those of gms_bucket_desc, on
 * the key's full width:
 *   DELTA       key * B >> 64 for 8-byte keys (>> 32 for 4-byte keys)
 *   DIV         (key / param) mod B
 *   BITS        (key >> shift) & (B-1), shift < 64
 *   RANGE       upper_bound(d_splitters[0..B), key) - 1, -1 read as B-1; the
 *               splitters are keys of key_bytes each
 *   MASK        (key & param) != 0
 *   EVEN_FLOAT  (uint32)((float)(key - lower) * inverse_delta) mod B, with the
 *               same round-to-nearest conversions and truncation as for 4-byte keys
 * With 4-byte keys param and lower must fit in 32 bits.  Output order, offsets
 * and stability are those of gms_multisplit_key_value.  8-byte keys are
 * identified once, in the first pass, and keep their buckets as one byte per
 * key in the scratch, so their scratch is always the size
 * gms_multisplit_wide_scratch_bytes reports. */
typedef struct gms_bucket_desc64 {
  int32_t kind;                /* gms_bucket_kind */
  uint32_t num_buckets;        /* B: 2..256 (a power of two for BITS) */
  uint32_t shift;              /* BITS */
  float inverse_delta;         /* EVEN_FLOAT: 1 / bin width */
  uint64_t param;              /* DIV: divisor (non-zero); MASK: mask */
  uint64_t lower;              /* EVEN_FLOAT: lower level */
  const void* d_splitters;     /* RANGE: B sorted splitters of key_bytes each, device memory */
} gms_bucket_desc64;

gms_status gms_multisplit_wide_scratch_bytes(uint32_t max_elements, uint32_t num_buckets, int key_bytes,
                                             int value_bytes, size_t* bytes);
gms_status gms_multisplit_wide(const void* d_key_in, const void* d_value_in, void* d_key_out, void* d_value_out,
                               uint32_t n, int key_bytes, int value_bytes, const gms_bucket_desc64* desc,
                               void* d_scratch, size_t scratch_bytes, uint32_t* h_offsets, gms_stream_t stream);
/* Adds the count of every bucket into the caller-zeroed d_hist[0..B), B <= 256
 * (as gms_histogram; 4-byte keys take gms_histogram itself). */
gms_status gms_histogram_wide(const void* d_key_in, uint32_t n, int key_bytes, const gms_bucket_desc64* desc,
                              int32_t* d_hist, gms_stream_t stream);
/* Stable sort by key bits [begin_bit, end_bit), end_bit <= 8 * key_bytes, in
 * digits of digit_bits (4..8) bits, least significant first. */
gms_status gms_sort_wide_scratch_bytes(uint32_t max_elements, int key_bytes, int value_bytes, int begin_bit,
                                       int end_bit, int digit_bits, size_t* bytes);
gms_status gms_sort_wide(const void* d_key_in, void* d_key_out, const void* d_value_in, void* d_value_out, uint32_t n,
                         int key_bytes, int value_bytes, int begin_bit, int end_bit, int digit_bits, void* d_scratch,
                         size_t scratch_bytes, gms_stream_t stream);

/* ----------------------------------------------------------- compaction */
/* Replaces compaction_allocate_key_only / _key_value
 * (src/kernels/compaction/multisplit2_compaction.cuh:491-517). */
gms_status gms_compaction_scratch_bytes(uint32_t max_elements, int key_value, size_t* bytes);

/* Replaces compaction_key_only / compaction_key_value
 * (src/kernels/compaction/multisplit2_compaction.cuh:525-573): a stable two-bucket
 * multisplit, bucket 0 first.  desc->num_buckets must be 2.  Like the reference
 * it synchronises and returns the bucket-0 count in *h_num_bucket0 (:541-547). */
gms_status gms_compaction_key_only(const uint32_t* d_key_in, uint32_t* d_key_out, uint32_t n,
                                   const gms_bucket_desc* desc, void* d_scratch, size_t scratch_bytes,
                                   uint32_t* h_num_bucket0, gms_stream_t stream);
gms_status gms_compaction_key_value(const uint32_t* d_key_in, const uint32_t* d_value_in, uint32_t* d_key_out,
                                    uint32_t* d_value_out, uint32_t n, const gms_bucket_desc* desc,
                                    void* d_scratch, size_t scratch_bytes, uint32_t* h_num_bucket0,
                                    gms_stream_t stream);

/* -------------------------------------------------------------- batched */
/* Many independent multisplits of uneven sizes and bucket counts ("segments")
 * run as one plan: per stage one launch per segment class (identifier kind,
 * bucket count, key/value shape) over a device-side tile map, and one scan over
 * all segments' count matrices laid end to end; optionally captured once into a
 * CUDA graph and replayed.  No reference counterpart (the reference runs one
 * multisplit per call, src/api/multisplit.cuh:81-313); each segment's output
 * equals gms_multisplit_key_value / _key_only on that segment alone. */
typedef struct gms_segment {
  const uint32_t* d_key_in;
  const uint32_t* d_value_in; /* null: key-only segment */
  uint32_t* d_key_out;
  uint32_t* d_value_out;      /* null iff d_value_in is null */
  uint32_t n;
  gms_bucket_desc desc;
} gms_segment;

typedef struct gms_batch_s* gms_batch_t;

/* Builds a plan for `count` segments (host work only; the segment array is copied). */
gms_status gms_batch_create(const gms_segment* segments, uint32_t count, gms_batch_t* batch);
/* Scratch the plan needs: tables, count matrix, scan state. */
gms_status gms_batch_scratch_bytes(gms_batch_t batch, size_t* bytes);
/* Runs every segment's multisplit on `stream`.  The first run with a given
 * scratch buffer uploads the plan's tables there (and synchronises); with
 * use_graph != 0 the launch sequence is captured once into a CUDA graph (per
 * scratch buffer) and replayed with one graph launch per call. */
gms_status gms_batch_run(gms_batch_t batch, void* d_scratch, size_t scratch_bytes, int use_graph,
                         gms_stream_t stream);
/* Number of kernel launches one run issues (inside the graph when use_graph != 0). */
gms_status gms_batch_launch_count(gms_batch_t batch, uint32_t* launches);
gms_status gms_batch_destroy(gms_batch_t batch);
/* Builds a plan whose every segment runs tile variant `variant` instead of
 * the tuning table's choice (for measurements and tests). */
gms_status gms_batch_create_with_variant(const gms_segment* segments, uint32_t count, int variant,
                                         gms_batch_t* batch);

/* How a run issues its work.
 *   GMS_BATCH_SCHEDULE_CLASSES  one prescan and one postscan launch per class
 *     of segments (same identifier kind, bucket count, key/value shape and
 *     tile variant) and one scan per group of segments, the classes of a
 *     stage on four side streams;
 *   GMS_BATCH_SCHEDULE_QUEUE  one persistent launch whose blocks take work
 *     items from a list in device memory: per segment, counting items for
 *     groups of 4096-key tiles, scan items for its count matrix, and one
 *     reorder item per tile.  A segment's reorder items follow its counting
 *     items closely, so its keys are usually re-read from L2; every segment
 *     uses 4096-key tiles (the tuning table is not consulted).
 * Both give identical outputs.  A plan starts with GMS_BATCH_SCHEDULE_CLASSES;
 * changing the schedule drops the plan's captured graph.  The queue needs
 * every segment's count matrix to fit 32-bit offsets; otherwise setting it
 * returns GMS_ERROR_NOT_SUPPORTED. */
enum { GMS_BATCH_SCHEDULE_CLASSES = 0, GMS_BATCH_SCHEDULE_QUEUE = 1 };
gms_status gms_batch_set_schedule(gms_batch_t batch, int schedule);
gms_status gms_batch_get_schedule(gms_batch_t batch, int* schedule);

/* -------------------------------------------------------------- tuning */
/* The batched form runs each segment with one of GMS_NUM_TILE_VARIANTS tile
 * shapes (warps per block x keys per thread), picked from a process-wide
 * table indexed by (log2 B, key/value, segment size class).  Size class c
 * covers n <= 2^10 for c = 0, 2^(9+c) < n <= 2^(10+c) for 0 < c < 7, and
 * n > 2^16 for c = 7.  A shape is valid for B only when it has at least B
 * threads.  gms_batch_create reads the table, so a change applies to plans
 * created afterwards.  The tuning calls take powers of two; a segment whose
 * B is not one uses the row of the next power of two. */
#define GMS_NUM_TILE_VARIANTS 4
#define GMS_NUM_SIZE_CLASSES 8
gms_status gms_tile_variant_shape(int variant, uint32_t* warps, uint32_t* keys_per_thread, uint32_t* tile_keys);
gms_status gms_tuning_get(uint32_t num_buckets, int key_value, int size_class, int* variant);
gms_status gms_tuning_set(uint32_t num_buckets, int key_value, int size_class, int variant);
/* Restores the built-in table (before any autotuning). */
gms_status gms_tuning_reset(void);
/* Autotuner: for every bucket count whose bit is set in bucket_mask (bit k =
 * 2^k buckets, k = 1..8), every shape in key_value_mask (bit 0 key-only, bit 1
 * key-value) and every size class, builds a batch of segments of the class's
 * size (delta identifier, about keys_per_trial keys in all), times each valid
 * variant as a graph replay on `stream` (best of `reps`) and stores the fastest
 * (the built-in entry stays unless another variant is more than 3% faster)
 * in the table.  It allocates its own device buffers (about 16 bytes per
 * trial key) and frees them before returning; it synchronises `stream`.
 * h_ms_out (optional) receives the best time per entry, indexed
 * [(k-1) * 2 + key_value] * GMS_NUM_SIZE_CLASSES + size_class (16 * 8 floats). */
gms_status gms_autotune(uint32_t bucket_mask, uint32_t key_value_mask, uint32_t keys_per_trial, int reps,
                        float* h_ms_out, gms_stream_t stream);

/* -------------------------------------------------------------- serving */
/* A request loop with continuous batching.  No reference counterpart.  A
 * scheduler thread admits submitted requests in arrival order while their
 * memory fits in a caller-provided device arena (the HBM budget), and keeps
 * launching rounds: each round takes the next step of every admitted request
 * that is not already on the GPU (a multisplit or compaction is one step, a
 * 7-bit sort five, one per digit pass) and runs them as one batched multisplit
 * (plus histogram launches).  Rounds alternate between two streams so the next
 * round is launched while the previous one is still running; requests that
 * arrive meanwhile join the next round.  Results live in the arena until
 * released.  Each result equals the plain call on that request alone. */
typedef enum gms_op {
  GMS_OP_MULTISPLIT = 0,  /* stable multisplit, desc as given */
  GMS_OP_SORT_7BIT = 1,   /* multisplit_sort_7bit[_pairs]; desc ignored */
  GMS_OP_HISTOGRAM = 2,   /* gms_histogram with desc; values ignored */
  GMS_OP_COMPACTION = 3   /* compaction with desc (2 buckets); num_bucket0 returned */
} gms_op;

typedef struct gms_request {
  int32_t op;                 /* gms_op */
  const uint32_t* d_key_in;   /* device input, valid until the request is done */
  const uint32_t* d_value_in; /* null: key-only */
  uint32_t n;
  gms_bucket_desc desc;
} gms_request;

typedef struct gms_result {
  int32_t done;            /* 1 once finished (then status is final) */
  int32_t status;          /* gms_status of the request */
  uint32_t* d_key_out;     /* in the arena: MULTISPLIT, SORT_7BIT, COMPACTION */
  uint32_t* d_value_out;   /* in the arena, when the request has values */
  int32_t* d_histogram;    /* in the arena: HISTOGRAM (desc.num_buckets counts) */
  uint32_t num_bucket0;    /* COMPACTION */
  uint32_t rounds;         /* rounds the request took part in */
  double submit_s;         /* server clock, seconds */
  double admit_s;
  double done_s;
} gms_result;

typedef struct gms_server_stats {
  uint64_t submitted;
  uint64_t completed;
  uint64_t rounds;
  uint64_t launches;       /* kernel launches issued by all rounds */
  uint64_t keys;           /* keys of completed requests */
  uint64_t arena_peak_bytes;
  uint32_t max_requests_in_round;
} gms_server_stats;

typedef struct gms_server_s* gms_server_t;

/* d_arena: device memory the server may use for outputs and round scratch
 * (64 GB in the reference serving workload).  The server also creates two
 * streams, pinned staging buffers and one scheduler thread. */
gms_status gms_server_create(void* d_arena, size_t arena_bytes, gms_server_t* server);
/* Queues a request (never blocks on the GPU).  A request larger than the
 * arena can ever hold is rejected with GMS_ERROR_SCRATCH_TOO_SMALL. */
gms_status gms_server_submit(gms_server_t server, const gms_request* request, uint64_t* id);
/* Current state of a request (result->done == 0 while pending). */
gms_status gms_server_poll(gms_server_t server, uint64_t id, gms_result* result);
/* Blocks until the request is done.  Returns GMS_ERROR_SCRATCH_TOO_SMALL
 * instead of waiting forever when the request is queued behind arena memory that
 * only the caller can free: nothing is running and the finished results the
 * caller has not released fill the arena.  Release results and wait again. */
gms_status gms_server_wait(gms_server_t server, uint64_t id, gms_result* result);
/* Ids of requests finished since the previous call (up to max). */
gms_status gms_server_take_completed(gms_server_t server, uint64_t* ids, uint32_t max, uint32_t* count);
/* Frees a finished request's arena memory and forgets it. */
gms_status gms_server_release(gms_server_t server, uint64_t id);
/* Blocks until every submitted request is done, or returns
 * GMS_ERROR_SCRATCH_TOO_SMALL when the rest wait for arena memory held by
 * finished results the caller has not released (see gms_server_wait). */
gms_status gms_server_drain(gms_server_t server);
gms_status gms_server_get_stats(gms_server_t server, gms_server_stats* stats);
/* Seconds since the server was created (the clock of gms_result times). */
double gms_server_clock(gms_server_t server);
/* Stops the scheduler (after draining) and frees host resources; the arena stays the caller's. */
gms_status gms_server_destroy(gms_server_t server);

/* ------------------------------------------------------------ histogram */
/* Adds the per-bucket counts of d_key_in[0..n) into d_hist[0..B) (the caller
 * zeroes it first, as with the reference's atomicAdd kernels).  Generalises
 * multisplit2_histogram_even_* / _range_* (src/kernels/histogram/multisplit2_histograms.cuh:36-699)
 * to every identifier kind and to any n (the reference needs n to be a whole
 * number of tiles, src/main/main_histogram.cu:76).  The bins are int counters
 * like the reference's; a bin whose count exceeds 2^31 - 1 holds it modulo 2^32. */
gms_status gms_histogram(const uint32_t* d_key_in, uint32_t n, const gms_bucket_desc* desc, int32_t* d_hist,
                         gms_stream_t stream);

/* multisplit2_histogram_even_* launch (src/main/main_histogram.cu:163-179) with
 * uint32 samples: bin = (uint32)((key - lower) * inverse_delta), wrapped modulo num_bins. */
gms_status gms_histogram_even(const uint32_t* d_key_in, uint32_t n, int32_t* d_hist, uint32_t num_bins,
                              uint32_t lower, uint32_t upper, float inverse_delta, gms_stream_t stream);

/* multisplit2_histogram_range_* launch (src/main/main_histogram.cu:272-279):
 * bin = upper_bound(d_levels[0..num_bins), key) - 1, wrapped modulo num_bins. */
gms_status gms_histogram_range(const uint32_t* d_key_in, uint32_t n, int32_t* d_hist, uint32_t num_bins,
                               const uint32_t* d_levels, gms_stream_t stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* GPUMULTISPLIT_H_ */
