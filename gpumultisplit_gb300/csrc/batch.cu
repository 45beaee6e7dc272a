// Host side of the batched multisplit: plan construction (segment classes,
// tile maps, count-matrix layout, scan groups), table upload, the launch
// sequence and its capture into a CUDA graph.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/gpumultisplit.h"
#include "batch_kernels.cuh"
#include "ms_host.h"

namespace gms {
namespace {

struct BatchClass {
  int kind = 0;
  int logb = 1;
  bool kv = false;
  int variant = 0;                 // tile shape (kTileVariants)
  bool warp = false;               // segments of at most kWarpSegMax keys, one warp each
  std::vector<uint2> tiles;        // (segment, tile)
  std::vector<uint32_t> seg_ids;   // warp classes: their segments
  size_t map_off = 0;              // byte offset of this class's map (or segment list) in scratch
  size_t work() const { return warp ? seg_ids.size() / 8 + 1 : tiles.size(); }  // for the launch order
  const void* map_data() const { return warp ? static_cast<const void*>(seg_ids.data()) : tiles.data(); }
  size_t map_bytes() const { return warp ? seg_ids.size() * sizeof(uint32_t) : tiles.size() * sizeof(uint2); }
};

// A run of consecutive segments whose n sum stays below 2^32, scanned on its own.
struct ScanGroup {
  uint32_t matrix_first = 0;  // first matrix entry
  uint32_t m = 0;             // entries
};

}  // namespace
}  // namespace gms

struct gms_batch_s {
  std::vector<gms::SegDesc> segs;
  std::vector<gms::BatchClass> classes;
  std::vector<gms::ScanGroup> groups;
  size_t off_segs = 0, off_maps = 0, off_matrix = 0, off_status = 0, off_bytes = 0, bytes = 0;
  uint32_t max_chunks = 0;
  // Bound scratch (tables uploaded) and the captured graph for it.
  std::mutex mu;
  void* bound = nullptr;
  cudaStream_t capture_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void* graph_scratch = nullptr;
  // Side streams and events of gms_batch_run: the classes of one stage run on
  // several streams so small classes overlap large ones (created on first use).
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> events;
  // The one-launch schedule (batch_queue.cuh): segment records and work list
  // (tables, uploaded with the class tables), then its run-time regions,
  // which overlay the class schedule's (a run uses one schedule).
  int schedule = GMS_BATCH_SCHEDULE_CLASSES;
  bool queue_ok = false;  // the queue's count matrix fits 32-bit offsets
  std::vector<gms::QSeg> qsegs;     // built with the plan (one record per segment)
  std::vector<uint2> qitems;        // built when the queue schedule is first selected
  size_t q_items = 0;               // the list's length, known with the plan
  void* queue_uploaded = nullptr;   // scratch that holds the queue's records and list
  size_t off_qsegs = 0, off_qitems = 0;
  size_t off_qmatrix = 0, off_qstate = 0, off_qstatus = 0, off_qbytes = 0, q_state_bytes = 0;
};

namespace gms {
namespace {

gms_status to_status(cudaError_t e) {
  if (e == cudaSuccess) return GMS_SUCCESS;
  note_cuda_error(e);
  return GMS_ERROR_CUDA;
}

// Any bucket count in [2, 256]; *logb = ceil(log2(b)).
bool log2_buckets(uint32_t b, int* logb) {
  if (b < 2 || b > 256) return false;
  int l = 0;
  while ((1u << l) < b) ++l;
  *logb = l;
  return true;
}

template <int KIND>
cudaError_t dispatch_variant(const BatchClassLaunch& c, int stage) {
  switch (c.variant) {
    case 0: return run_batch_class_v<KIND, 0>(c, stage);
    case 1: return run_batch_class_v<KIND, 1>(c, stage);
    case 2: return run_batch_class_v<KIND, 2>(c, stage);
    case 3: return run_batch_class_v<KIND, 3>(c, stage);
    default: return cudaErrorInvalidValue;
  }
}
static_assert(kNumTileVariants == 4, "dispatch_variant covers every tile variant");

cudaError_t run_batch_warp_kind(int kind, const BatchClassLaunch& c) {
  switch (kind) {
    case KIND_DELTA: return run_batch_warp<KIND_DELTA>(c);
    case KIND_DIV: return run_batch_warp<KIND_DIV>(c);
    case KIND_BITS: return run_batch_warp<KIND_BITS>(c);
    case KIND_RANGE: return run_batch_warp<KIND_RANGE>(c);
    case KIND_MASK: return run_batch_warp<KIND_MASK>(c);
    case KIND_EVEN_FLOAT: return run_batch_warp<KIND_EVEN_FLOAT>(c);
    default: return cudaErrorInvalidValue;
  }
}

constexpr int kSideStreams = 4;

cudaError_t ensure_side_streams(gms_batch_s* b) {
  if (!b->side.empty()) return cudaSuccess;
  for (int i = 0; i < kSideStreams; ++i) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      if (st) cudaStreamDestroy(st);
      return e;
    }
    b->side.push_back(st);
    b->events.push_back(ev);
  }
  cudaEvent_t fork = nullptr;
  cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
  if (e == cudaSuccess) b->events.push_back(fork);  // last event: the fork point
  return e;
}

// Launches one stage of every class.  With side streams the classes (largest
// first) are dealt round-robin to the side streams, which fork from and join
// back into `s`, so a stage's kernels of different classes can run at once.
cudaError_t launch_classes(gms_batch_s* b, BatchClassLaunch L, unsigned char* scratch, cudaStream_t s, int stage,
                           bool fork) {
  const size_t nc = b->classes.size();
  const int lanes = fork && nc > 1 ? int(std::min<size_t>(nc, b->side.size())) : 0;
  cudaError_t e = cudaSuccess;
  if (lanes > 0) {
    e = cudaEventRecord(b->events.back(), s);
    for (int i = 0; e == cudaSuccess && i < lanes; ++i) e = cudaStreamWaitEvent(b->side[i], b->events.back(), 0);
    if (e != cudaSuccess) return e;
  }
  std::vector<size_t> order(nc);
  for (size_t i = 0; i < nc; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t x, size_t y) { return b->classes[x].work() > b->classes[y].work(); });
  for (size_t k = 0; k < nc; ++k) {
    const BatchClass& c = b->classes[order[k]];
    L.logb = c.logb;
    L.kv = c.kv;
    L.variant = c.variant;
    L.stream = lanes > 0 ? b->side[k % size_t(lanes)] : s;
    if (c.warp) {  // one kernel does the whole multisplit: launched with the postscans
      if (stage != STAGE_POSTSCAN) continue;
      L.seg_ids = reinterpret_cast<const uint32_t*>(scratch + c.map_off);
      L.class_tiles = uint32_t(c.seg_ids.size());
      e = run_batch_warp_kind(c.kind, L);
    } else {
      L.tile_map = reinterpret_cast<const uint2*>(scratch + c.map_off);
      L.class_tiles = uint32_t(c.tiles.size());
      e = run_batch_class(c.kind, L, stage);
    }
    if (e != cudaSuccess) return e;
  }
  for (int i = 0; e == cudaSuccess && i < lanes; ++i) {
    e = cudaEventRecord(b->events[i], b->side[i]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, b->events[i], 0);
  }
  return e;
}

// The launch sequence of one run: reset the error word, prescan every class,
// scan every group (ticket and status words reset first), postscan every class.
cudaError_t launch_all(gms_batch_s* b, unsigned char* scratch, cudaStream_t s, bool fork = false) {
  auto* hdr = reinterpret_cast<ScratchHeader*>(scratch);
  auto* matrix = reinterpret_cast<uint32_t*>(scratch + b->off_matrix);
  auto* status = reinterpret_cast<uint64_t*>(scratch + b->off_status);
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(ScratchHeader), s);
  if (e != cudaSuccess) return e;
  BatchClassLaunch L;
  L.segs = reinterpret_cast<const SegDesc*>(scratch + b->off_segs);
  L.matrix = matrix;
  L.byte_area = scratch + b->off_bytes;
  L.hdr = hdr;
  L.stream = s;
  for (int stage : {int(STAGE_PRESCAN), int(STAGE_POSTSCAN)}) {
    if (stage == STAGE_POSTSCAN) {
      for (const ScanGroup& g : b->groups) {
        e = cudaMemsetAsync(&hdr->ticket, 0, sizeof(uint32_t), s);
        if (e == cudaSuccess)
          e = cudaMemsetAsync(status, 0, size_t((g.m + kScanChunk - 1) / kScanChunk) * sizeof(uint64_t), s);
        if (e == cudaSuccess) e = run_scan(matrix + g.matrix_first, g.m, status, hdr, s);
        if (e != cudaSuccess) return e;
      }
    }
    e = launch_classes(b, L, scratch, s, stage, fork);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Order of the queue's work list.  Counting (PRE) tiles run this many tiles
// ahead of reordering (POST) tiles, so a segment's keys are read again about
// 4 MiB of other keys after they were counted, usually still from L2.
#ifndef GMS_QUEUE_LEAD_TILES
#define GMS_QUEUE_LEAD_TILES 256
#endif
// A segment's first POST item comes at least this many resident blocks' worth
// of items (two waves) after its last SCAN item, so its scan has finished by
// the time its POST items are claimed and they rarely wait.
constexpr uint32_t kQueueScanGapWaves = 2;

// The queue's segment records (the class plan's descriptors give pointers, n
// and identifier parameters) and the sizes of its regions and work list.
// Returns false when a count matrix would need offsets of 2^32 or more.
bool queue_records(gms_batch_s* b, const gms_segment* segments, uint32_t count, uint64_t* matrix_words,
                   uint64_t* chunks_total, uint64_t* byte_total) {
  b->qsegs.assign(count, QSeg{});
  b->qitems.clear();
  b->q_items = 0;
  uint64_t m_total = 0, c_total = 0, bytes = 0;
  for (uint32_t i = 0; i < count; ++i) {
    const gms_segment& sg = segments[i];
    int logb = 0;
    log2_buckets(sg.desc.num_buckets, &logb);
    QSeg& q = b->qsegs[i];
    q.d = b->segs[i];
    q.d.num_tiles = uint32_t((uint64_t(sg.n) + QUEUE_TILE - 1) / QUEUE_TILE);
    q.d.base = 0;
    q.d.matrix_off = uint32_t(m_total);
    const uint64_t m = uint64_t(q.d.num_tiles) << logb;
    m_total = (m_total + m + 3) & ~uint64_t(3);  // every segment's counts start on 16 bytes
    if (m_total > 0xFFFFFFFFull) return false;
    q.d.bytes_off = 0;
    if (sg.desc.kind != KIND_DELTA && sg.n > 0) {
      q.d.bytes_off = bytes;
      bytes += (uint64_t(sg.n) + 15) & ~uint64_t(15);
    }
    q.chunks = uint32_t((m + kScanChunk - 1) / kScanChunk);
    q.status_off = uint32_t(c_total);
    c_total += q.chunks;
    q.meta = uint32_t(sg.desc.kind) | (uint32_t(logb) << 8) | (sg.d_value_in != nullptr ? 1u << 16 : 0u);
    b->q_items += (q.d.num_tiles + QUEUE_PRE_TILES - 1) / QUEUE_PRE_TILES + q.chunks + q.d.num_tiles;
  }
  *matrix_words = m_total;
  *chunks_total = c_total;
  *byte_total = bytes;
  return true;
}

// The queue's work list over the records.  Segments are taken class by class,
// largest first.  PRE items of a segment are followed by its SCAN items; the
// list then takes the next POST tile (in segment order) whenever that
// segment's last SCAN item is far enough back and the PRE frontier leads the
// POST frontier by GMS_QUEUE_LEAD_TILES tiles, else the next PRE or SCAN item.
// Returns false (and leaves no list) if the finished list would make an item
// wait on a later one.
bool build_queue_list(gms_batch_s* b) {
  const uint32_t count = uint32_t(b->qsegs.size());
  b->qitems.clear();
  b->qitems.reserve(b->q_items);
  std::vector<uint32_t> order;
  for (uint32_t i = 0; i < count; ++i)
    if (b->qsegs[i].d.n > 0) order.push_back(i);
  // Segments of one class (identifier kind, bucket count, key/value) run
  // together, largest first, so the blocks running at once mostly execute
  // the same code; the classes with the most keys come first.
  std::map<uint32_t, uint64_t> class_keys;
  for (uint32_t i : order) class_keys[b->qsegs[i].meta] += b->qsegs[i].d.n;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
    const uint32_t cx = b->qsegs[x].meta, cy = b->qsegs[y].meta;
    if (cx != cy) return class_keys[cx] != class_keys[cy] ? class_keys[cx] > class_keys[cy] : cx < cy;
    return b->qsegs[x].d.n > b->qsegs[y].d.n;
  });
  // PRE and SCAN items in order; the POST tiles are merged in below.
  std::vector<uint2> first_stage;
  for (uint32_t i : order) {
    const QSeg& q = b->qsegs[i];
    for (uint32_t g = 0; g * QUEUE_PRE_TILES < q.d.num_tiles; ++g)
      first_stage.push_back(make_uint2(i, (QITEM_PRE << QITEM_SHIFT) | g));
    for (uint32_t c = 0; c < q.chunks; ++c) first_stage.push_back(make_uint2(i, (QITEM_SCAN << QITEM_SHIFT) | c));
  }
  const uint64_t gap = uint64_t(kQueueScanGapWaves) * uint64_t(std::max(1, device_sm_count())) * QUEUE_MIN_BLOCKS;
  // List position of a segment's last SCAN item, once every one of them is listed.
  std::vector<uint64_t> last_scan(count, ~uint64_t(0));
  uint64_t pre_tiles = 0, post_tiles = 0;
  size_t fi = 0, post_seg = 0;
  uint32_t post_tile = 0;
  while (fi < first_stage.size() || post_seg < order.size()) {
    bool post = false;
    if (post_seg < order.size()) {
      const uint32_t s = order[post_seg];
      const bool scanned = last_scan[s] != ~uint64_t(0) && b->qitems.size() - last_scan[s] >= gap;
      post = fi >= first_stage.size() || (scanned && pre_tiles >= post_tiles + GMS_QUEUE_LEAD_TILES);
    }
    if (post) {
      const uint32_t s = order[post_seg];
      b->qitems.push_back(make_uint2(s, (QITEM_POST << QITEM_SHIFT) | post_tile));
      ++post_tiles;
      if (++post_tile == b->qsegs[s].d.num_tiles) {
        ++post_seg;
        post_tile = 0;
      }
    } else {
      const uint2 it = first_stage[fi++];
      const QSeg& q = b->qsegs[it.x];
      const uint32_t idx = it.y & ((1u << QITEM_SHIFT) - 1u);
      if ((it.y >> QITEM_SHIFT) == QITEM_PRE)
        pre_tiles += std::min<uint32_t>(QUEUE_PRE_TILES, q.d.num_tiles - idx * QUEUE_PRE_TILES);
      else if (idx + 1 == q.chunks)
        last_scan[it.x] = b->qitems.size();
      b->qitems.push_back(it);
    }
  }
  // Every item may wait only on items listed before it (the launch relies on
  // that to make progress): each segment's PRE items before its SCAN items,
  // all of them before its first POST item.  A list that breaks this is never
  // launched.
  std::vector<uint32_t> pre_seen(count, 0), scan_seen(count, 0);
  for (const uint2& it : b->qitems) {
    const QSeg& q = b->qsegs[it.x];
    const uint32_t type = it.y >> QITEM_SHIFT;
    if (type == QITEM_PRE) {
      if (scan_seen[it.x] != 0) {
        b->qitems.clear();
        return false;
      }
      pre_seen[it.x] += std::min<uint32_t>(QUEUE_PRE_TILES, q.d.num_tiles - (it.y & ((1u << QITEM_SHIFT) - 1u)) * QUEUE_PRE_TILES);
    } else if (type == QITEM_SCAN) {
      if (pre_seen[it.x] != q.d.num_tiles) {
        b->qitems.clear();
        return false;
      }
      ++scan_seen[it.x];
    } else if (scan_seen[it.x] != q.chunks) {
      b->qitems.clear();
      return false;
    }
  }
  if (b->qitems.size() != b->q_items) {
    b->qitems.clear();
    return false;
  }
  return true;
}

// One run of the queue schedule: reset the header and the run state, then the
// one launch.
cudaError_t launch_queue(gms_batch_s* b, unsigned char* scratch, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(ScratchHeader), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(scratch + b->off_qstate, 0, b->q_state_bytes, s);
  if (e != cudaSuccess) return e;
  BatchQueueLaunch L;
  L.qsegs = reinterpret_cast<const QSeg*>(scratch + b->off_qsegs);
  L.items = reinterpret_cast<const uint2*>(scratch + b->off_qitems);
  L.num_items = uint32_t(b->qitems.size());  // built before the schedule could be selected
  L.num_segs = uint32_t(b->qsegs.size());
  L.matrix = reinterpret_cast<uint32_t*>(scratch + b->off_qmatrix);
  L.byte_area = scratch + b->off_qbytes;
  L.state = reinterpret_cast<uint32_t*>(scratch + b->off_qstate);
  L.status = reinterpret_cast<uint64_t*>(scratch + b->off_qstatus);
  L.hdr = reinterpret_cast<ScratchHeader*>(scratch);
  L.stream = s;
  return run_batch_queue(L);
}

// The launch sequence of the batch's current schedule.
cudaError_t launch_schedule(gms_batch_s* b, unsigned char* scratch, cudaStream_t s, bool fork) {
  if (b->schedule == GMS_BATCH_SCHEDULE_QUEUE) return launch_queue(b, scratch, s);
  return launch_all(b, scratch, s, fork);
}

}  // namespace

cudaError_t run_batch_class(int kind, const BatchClassLaunch& c, int stage) {
  switch (kind) {
    case KIND_DELTA: return dispatch_variant<KIND_DELTA>(c, stage);
    case KIND_DIV: return dispatch_variant<KIND_DIV>(c, stage);
    case KIND_BITS: return dispatch_variant<KIND_BITS>(c, stage);
    case KIND_RANGE: return dispatch_variant<KIND_RANGE>(c, stage);
    case KIND_MASK: return dispatch_variant<KIND_MASK>(c, stage);
    case KIND_EVEN_FLOAT: return dispatch_variant<KIND_EVEN_FLOAT>(c, stage);
    default: return cudaErrorInvalidValue;
  }
}

gms_status batch_create(const gms_segment* segments, uint32_t count, int variant, gms_batch_t* batch) {
  if (batch == nullptr || (segments == nullptr && count > 0) || variant >= kNumTileVariants)
    return GMS_ERROR_INVALID_VALUE;
  auto* b = new gms_batch_s();
  std::map<std::tuple<int, int, bool, int>, size_t> class_index;
  std::vector<std::pair<uint32_t, int>> warp_segs;  // (segment, log2 B) on the one-warp path
  uint64_t matrix_total = 0, group_n = 0, byte_total = 0;
  ScanGroup group;
  for (uint32_t i = 0; i < count; ++i) {
    const gms_segment& sg = segments[i];
    int logb = 0;
    if (!log2_buckets(sg.desc.num_buckets, &logb)) {
      delete b;
      return GMS_ERROR_UNSUPPORTED_BUCKETS;
    }
    const bool kv = sg.d_value_in != nullptr;
    const int kind = sg.desc.kind;
    const bool bad_desc = kind < 0 || kind >= NUM_KINDS || (kind == KIND_DIV && sg.desc.param == 0) ||
                          (kind == KIND_RANGE && sg.desc.d_splitters == nullptr);
    if (kind == KIND_BITS && (sg.desc.num_buckets & (sg.desc.num_buckets - 1)) != 0) {
      delete b;
      return GMS_ERROR_UNSUPPORTED_BUCKETS;
    }
    const bool bad_ptrs = sg.n > 0 && (sg.d_key_in == nullptr || sg.d_key_out == nullptr ||
                                       (kv && sg.d_value_out == nullptr) || (!kv && sg.d_value_out != nullptr));
    if (bad_desc || bad_ptrs) {
      delete b;
      return GMS_ERROR_INVALID_VALUE;
    }
    SegDesc d{};
    d.kin = sg.d_key_in;
    d.vin = sg.d_value_in;
    d.kout = sg.d_key_out;
    d.vout = sg.d_value_out;
    d.n = sg.n;
    d.bp.shift = sg.desc.shift;
    d.bp.param = sg.desc.param;
    d.bp.lower = sg.desc.lower;
    d.bp.inverse_delta = sg.desc.inverse_delta;
    d.bp.splitters = sg.desc.d_splitters;
    d.bp.num_buckets = sg.desc.num_buckets;
    if (variant < 0 && sg.n > 0 && sg.n <= kWarpSegMax) {
      // One warp multisplits the whole segment; its bucket starts get matrix
      // entries after every scan group (assigned below).
      b->segs.push_back(d);
      warp_segs.emplace_back(i, logb);
      const auto key = std::make_tuple(kind, logb, kv, -1);
      auto it = class_index.find(key);
      if (it == class_index.end()) {
        it = class_index.emplace(key, b->classes.size()).first;
        BatchClass c;
        c.kind = kind;
        c.logb = logb;
        c.kv = kv;
        c.warp = true;
        b->classes.push_back(c);
      }
      b->classes[it->second].seg_ids.push_back(i);
      continue;
    }
    const int v = variant >= 0 ? variant : tuned_variant(logb, kv, sg.n);
    if (!variant_valid(v, logb)) {
      delete b;
      return GMS_ERROR_INVALID_VALUE;
    }
    const uint32_t tile = variant_tile_keys(v);
    d.num_tiles = uint32_t((uint64_t(sg.n) + tile - 1) / tile);
    const uint64_t entries = uint64_t(1u << logb) * d.num_tiles;
    // Start a new scan group when this segment would push the group's keys past
    // 2^32 - 1.  A group's counts start on a 16-byte boundary (the scan reads
    // them as 16-byte vectors); the entries skipped for that belong to no group.
    if (group_n + sg.n > 0xFFFFFFFFull) {
      group.m = uint32_t(matrix_total - group.matrix_first);
      b->groups.push_back(group);
      matrix_total = (matrix_total + 3) & ~uint64_t(3);
      group.matrix_first = uint32_t(matrix_total);
      group_n = 0;
    }
    d.base = uint32_t(group_n);
    d.matrix_off = uint32_t(matrix_total);
    d.bytes_off = 0;
    if (kind_keeps_bucket_bytes(kind)) {  // one bucket byte per key, 16-byte aligned per segment
      d.bytes_off = byte_total;
      byte_total += (uint64_t(sg.n) + 15) & ~uint64_t(15);
    }
    group_n += sg.n;
    matrix_total += entries;
    if (matrix_total > 0xFFFFFFFFull) {
      delete b;
      return GMS_ERROR_NOT_SUPPORTED;
    }
    b->segs.push_back(d);
    if (d.num_tiles == 0) continue;
    const auto key = std::make_tuple(kind, logb, kv, v);
    auto it = class_index.find(key);
    if (it == class_index.end()) {
      it = class_index.emplace(key, b->classes.size()).first;
      BatchClass c;
      c.kind = kind;
      c.logb = logb;
      c.kv = kv;
      c.variant = v;
      b->classes.push_back(c);
    }
    auto& tiles = b->classes[it->second].tiles;
    for (uint32_t t = 0; t < d.num_tiles; ++t) tiles.push_back(make_uint2(i, t));
  }
  group.m = uint32_t(matrix_total - group.matrix_first);
  if (group.m > 0) b->groups.push_back(group);
  // Bucket starts of the one-warp segments: one tile's entries each, past every group.
  for (const auto& [i, logb] : warp_segs) {
    SegDesc& d = b->segs[i];
    d.num_tiles = 1;
    d.base = 0;
    d.matrix_off = uint32_t(matrix_total);
    matrix_total += uint64_t(1u) << logb;
    if (matrix_total > 0xFFFFFFFFull) {
      delete b;
      return GMS_ERROR_NOT_SUPPORTED;
    }
  }
  for (const ScanGroup& g : b->groups)
    b->max_chunks = std::max(b->max_chunks, (g.m + kScanChunk - 1) / kScanChunk);

  size_t off = sizeof(ScratchHeader);
  b->off_segs = off;
  off = align_up(off + b->segs.size() * sizeof(SegDesc), 256);
  b->off_maps = off;
  for (BatchClass& c : b->classes) {
    c.map_off = off;
    off = align_up(off + c.map_bytes(), 256);
  }
  uint64_t q_matrix = 0, q_chunks = 0, q_bytes = 0;
  b->queue_ok = queue_records(b, segments, count, &q_matrix, &q_chunks, &q_bytes);
  if (b->queue_ok) {
    b->off_qsegs = off;
    off = align_up(off + b->qsegs.size() * sizeof(QSeg), 256);
    b->off_qitems = off;
    off = align_up(off + b->q_items * sizeof(uint2), 256);
  } else {
    b->qsegs.clear();
    b->q_items = 0;
    b->off_qsegs = b->off_qitems = off;
  }
  const size_t run_start = off;  // run-time regions of either schedule start here
  b->off_matrix = off;
  off = align_up(off + size_t(matrix_total) * 4, 256);
  b->off_status = off;
  b->off_bytes = align_up(off + size_t(b->max_chunks) * 8, 256);
  b->bytes = align_up(b->off_bytes + size_t(byte_total), 256);
  if (b->queue_ok) {
    size_t q = run_start;
    b->off_qmatrix = q;
    q = align_up(q + size_t(q_matrix) * 4, 256);
    b->off_qstate = q;  // ticket, PRE tiles done and SCAN chunks done per segment, then the look-back words
    b->off_qstatus = align_up(q + (1 + 2 * size_t(count)) * 4, 16);
    b->q_state_bytes = b->off_qstatus + size_t(q_chunks) * 8 - b->off_qstate;
    b->off_qbytes = align_up(b->off_qstatus + size_t(q_chunks) * 8, 256);
    b->bytes = std::max(b->bytes, align_up(b->off_qbytes + size_t(q_bytes), 256));
  }
  *batch = b;
  return GMS_SUCCESS;
}

}  // namespace gms

using namespace gms;

extern "C" {

gms_status gms_batch_create(const gms_segment* segments, uint32_t count, gms_batch_t* batch) {
  return batch_create(segments, count, -1, batch);
}

gms_status gms_batch_create_with_variant(const gms_segment* segments, uint32_t count, int variant,
                                         gms_batch_t* batch) {
  if (variant < 0) return GMS_ERROR_INVALID_VALUE;
  return batch_create(segments, count, variant, batch);
}

gms_status gms_batch_scratch_bytes(gms_batch_t batch, size_t* bytes) {
  if (batch == nullptr || bytes == nullptr) return GMS_ERROR_INVALID_VALUE;
  *bytes = batch->bytes;
  return GMS_SUCCESS;
}

gms_status gms_batch_launch_count(gms_batch_t batch, uint32_t* launches) {
  if (batch == nullptr || launches == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (batch->schedule == GMS_BATCH_SCHEDULE_QUEUE) {
    *launches = batch->q_items == 0 ? 0u : 1u;
    return GMS_SUCCESS;
  }
  uint32_t n = 0;
  for (const BatchClass& c : batch->classes) n += c.warp ? 1u : (c.tiles.empty() ? 0u : 2u);
  for (const ScanGroup& g : batch->groups) n += g.m > 0 ? 1u : 0u;
  *launches = n;
  return GMS_SUCCESS;
}

gms_status gms_batch_set_schedule(gms_batch_t batch, int schedule) {
  if (batch == nullptr || (schedule != GMS_BATCH_SCHEDULE_CLASSES && schedule != GMS_BATCH_SCHEDULE_QUEUE))
    return GMS_ERROR_INVALID_VALUE;
  if (schedule == GMS_BATCH_SCHEDULE_QUEUE && !batch->queue_ok) return GMS_ERROR_NOT_SUPPORTED;
  std::lock_guard<std::mutex> lock(batch->mu);
  if (schedule == GMS_BATCH_SCHEDULE_QUEUE && batch->qitems.size() != batch->q_items) {
    if (!build_queue_list(batch)) return GMS_ERROR_NOT_SUPPORTED;
    batch->queue_uploaded = nullptr;
  }
  if (batch->schedule != schedule) {
    // The captured graph holds the other schedule's launches.
    if (batch->exec) cudaGraphExecDestroy(batch->exec);
    if (batch->graph) cudaGraphDestroy(batch->graph);
    batch->exec = nullptr;
    batch->graph = nullptr;
    batch->graph_scratch = nullptr;
    batch->schedule = schedule;
  }
  return GMS_SUCCESS;
}

gms_status gms_batch_get_schedule(gms_batch_t batch, int* schedule) {
  if (batch == nullptr || schedule == nullptr) return GMS_ERROR_INVALID_VALUE;
  *schedule = batch->schedule;
  return GMS_SUCCESS;
}

gms_status gms_batch_run(gms_batch_t b, void* d_scratch, size_t scratch_bytes, int use_graph,
                         gms_stream_t stream) {
  if (b == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (b->classes.empty()) return GMS_SUCCESS;
  if (d_scratch == nullptr || (reinterpret_cast<uintptr_t>(d_scratch) & 255u) != 0)
    return GMS_ERROR_INVALID_VALUE;
  if (scratch_bytes < b->bytes) return GMS_ERROR_SCRATCH_TOO_SMALL;
  std::lock_guard<std::mutex> lock(b->mu);
  auto* scratch = static_cast<unsigned char*>(d_scratch);
  cudaError_t e = cudaSuccess;
  if (b->bound != d_scratch) {
    e = cudaMemcpyAsync(scratch + b->off_segs, b->segs.data(), b->segs.size() * sizeof(SegDesc),
                        cudaMemcpyHostToDevice, stream);
    for (size_t i = 0; e == cudaSuccess && i < b->classes.size(); ++i) {
      const BatchClass& c = b->classes[i];
      e = cudaMemcpyAsync(scratch + c.map_off, c.map_data(), c.map_bytes(), cudaMemcpyHostToDevice, stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return to_status(e);
    b->bound = d_scratch;
  }
  if (b->schedule == GMS_BATCH_SCHEDULE_QUEUE && b->queue_uploaded != d_scratch) {
    e = cudaMemcpyAsync(scratch + b->off_qsegs, b->qsegs.data(), b->qsegs.size() * sizeof(QSeg),
                        cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess && !b->qitems.empty())
      e = cudaMemcpyAsync(scratch + b->off_qitems, b->qitems.data(), b->qitems.size() * sizeof(uint2),
                          cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return to_status(e);
    b->queue_uploaded = d_scratch;
  }
  e = ensure_side_streams(b);
  if (e != cudaSuccess) return to_status(e);
  if (!use_graph) return to_status(launch_schedule(b, scratch, stream, true));

  if (b->exec == nullptr || b->graph_scratch != d_scratch) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    if (b->capture_stream == nullptr) {
      e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
      if (e != cudaSuccess) return to_status(e);
    }
    e = cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return to_status(e);
    const cudaError_t le = launch_schedule(b, scratch, b->capture_stream, true);
    e = cudaStreamEndCapture(b->capture_stream, &b->graph);
    if (le != cudaSuccess) return to_status(le);
    if (e != cudaSuccess) return to_status(e);
    e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) return to_status(e);
    b->graph_scratch = d_scratch;
  }
  return to_status(cudaGraphLaunch(b->exec, stream));
}

}  // extern "C"

namespace gms {

size_t batch_table_bytes(gms_batch_t b) { return b->off_matrix - b->off_segs; }

gms_status batch_run_async(gms_batch_t b, void* d_scratch, size_t scratch_bytes, void* h_pinned,
                           size_t pinned_bytes, cudaStream_t stream) {
  if (b == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (b->classes.empty()) return GMS_SUCCESS;
  const bool queue = b->schedule == GMS_BATCH_SCHEDULE_QUEUE;
  // The class schedule's tables end where the queue's begin.
  const size_t table = queue ? batch_table_bytes(b) : b->off_qsegs - b->off_segs;
  if (d_scratch == nullptr || scratch_bytes < b->bytes || h_pinned == nullptr || pinned_bytes < table)
    return GMS_ERROR_INVALID_VALUE;
  // Stage the segment table and tile maps in pinned memory at their scratch offsets, then one copy.
  auto* staging = static_cast<unsigned char*>(h_pinned);
  std::memcpy(staging, b->segs.data(), b->segs.size() * sizeof(SegDesc));
  for (const BatchClass& c : b->classes)
    std::memcpy(staging + (c.map_off - b->off_segs), c.map_data(), c.map_bytes());
  if (queue) {
    std::memcpy(staging + (b->off_qsegs - b->off_segs), b->qsegs.data(), b->qsegs.size() * sizeof(QSeg));
    std::memcpy(staging + (b->off_qitems - b->off_segs), b->qitems.data(), b->qitems.size() * sizeof(uint2));
  }
  auto* scratch = static_cast<unsigned char*>(d_scratch);
  cudaError_t e = cudaMemcpyAsync(scratch + b->off_segs, staging, table, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = launch_schedule(b, scratch, stream, false);
  return to_status(e);
}

uint32_t batch_matrix_value_offset(gms_batch_t b, uint32_t segment, uint32_t bucket, uint32_t tile,
                                   uint32_t* base) {
  const SegDesc& d = b->segs[segment];
  *base = d.base;
  return uint32_t(b->off_matrix / 4) + d.matrix_off + bucket * d.num_tiles + tile;
}

}  // namespace gms

extern "C" {

gms_status gms_batch_destroy(gms_batch_t b) {
  if (b == nullptr) return GMS_SUCCESS;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
  for (cudaStream_t st : b->side) cudaStreamDestroy(st);
  for (cudaEvent_t ev : b->events) cudaEventDestroy(ev);
  delete b;
  return GMS_SUCCESS;
}

}  // extern "C"
