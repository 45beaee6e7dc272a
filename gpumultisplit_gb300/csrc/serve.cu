// Serving runtime: request queue, admission against a device arena, continuous
// batching of every admitted request's next step into rounds of one batched
// multisplit each, two alternating streams, completion tracking.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/gpumultisplit.h"
#include "ms_host.h"

namespace gms {
namespace {

constexpr size_t kAlign = 256;
constexpr int kSlots = 2;  // streams, and rounds in flight at most
constexpr size_t kInitialStaging = size_t(8) << 20;  // pinned bytes per slot for round tables
constexpr size_t kInitialReadback = size_t(64) << 10;  // pinned bytes per slot for read-back words

// First-fit allocator over [0, size) with coalescing free blocks.
class Arena {
 public:
  explicit Arena(size_t size) : size_(size) {
    if (size > 0) free_[0] = size;
  }
  // Returns the offset or SIZE_MAX.
  size_t alloc(size_t bytes) {
    bytes = align_up(std::max<size_t>(bytes, 1), kAlign);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      const size_t off = it->first, rest = it->second - bytes;
      free_.erase(it);
      if (rest) free_[off + bytes] = rest;
      used_ += bytes;
      peak_ = std::max(peak_, used_);
      sizes_[off] = bytes;
      return off;
    }
    return SIZE_MAX;
  }
  void release(size_t off) {
    auto s = sizes_.find(off);
    if (s == sizes_.end()) return;
    size_t bytes = s->second;
    sizes_.erase(s);
    used_ -= bytes;
    auto next = free_.lower_bound(off);
    if (next != free_.end() && off + bytes == next->first) {
      bytes += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += bytes;
        return;
      }
    }
    free_[off] = bytes;
  }
  size_t size() const { return size_; }
  size_t peak() const { return peak_; }

 private:
  size_t size_, used_ = 0, peak_ = 0;
  std::map<size_t, size_t> free_;
  std::unordered_map<size_t, size_t> sizes_;
};

enum ReqState { QUEUED, ACTIVE, DONE };

struct Request {
  uint64_t id = 0;
  gms_request r{};
  ReqState state = QUEUED;
  bool in_flight = false;
  int pass = 0;            // sort: next digit pass
  size_t mem_off = SIZE_MAX, mem_bytes = 0;
  uint32_t *keys = nullptr, *vals = nullptr, *tmpk = nullptr, *tmpv = nullptr;
  int32_t* hist = nullptr;
  gms_result res{};
};

struct Round {
  int slot = 0;
  gms_batch_t plan = nullptr;
  size_t scratch_off = SIZE_MAX;
  cudaEvent_t done = nullptr;
  std::vector<uint64_t> reqs;
  std::vector<std::pair<uint64_t, uint32_t>> compactions;  // (request, readback index)
  std::vector<uint32_t> compaction_base;
};

// Digit schedule of the 7-bit sort (src/api/multisplit_sort.cuh:333-363).
constexpr uint32_t kSortShift[5] = {0, 4, 11, 18, 25};
constexpr uint32_t kSortBuckets[5] = {16, 128, 128, 128, 128};

}  // namespace
}  // namespace gms

struct gms_server_s {
  unsigned char* arena_base = nullptr;
  gms::Arena requests_arena{0};  // outputs of admitted requests
  gms::Arena rounds_arena{0};    // scratch of rounds in flight
  size_t rounds_off = 0;         // start of the round region in the arena
  cudaStream_t streams[gms::kSlots] = {};
  void* pinned[gms::kSlots] = {};  // table staging
  size_t pinned_cap[gms::kSlots] = {};
  uint32_t* readback[gms::kSlots] = {};  // [0] error word, [1..] compaction counts
  size_t readback_cap[gms::kSlots] = {};
  int next_slot = 0;
  std::chrono::steady_clock::time_point t0;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  // Nothing on the GPU or admitted, and the oldest queued request does not fit
  // the arena: only the caller's releases of finished results can free room.
  bool blocked_on_release = false;
  std::thread worker;
  uint64_t next_id = 1;
  std::unordered_map<uint64_t, std::unique_ptr<gms::Request>> reqs;
  std::deque<uint64_t> queue;    // QUEUED, arrival order
  std::vector<uint64_t> active;  // ACTIVE, admission order
  std::deque<gms::Round> rounds; // in flight, launch order
  std::vector<uint64_t> completed;
  gms_server_stats stats{};

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace gms {
namespace {

size_t request_bytes(const gms_request& r) {
  const size_t words = size_t(r.n) * 4;
  const bool kv = r.d_value_in != nullptr;
  switch (r.op) {
    case GMS_OP_MULTISPLIT:
    case GMS_OP_COMPACTION:
      return align_up(words, kAlign) * (kv ? 2 : 1);
    case GMS_OP_SORT_7BIT:
      return align_up(words, kAlign) * (kv ? 4 : 2);
    case GMS_OP_HISTOGRAM:
      return size_t(r.desc.num_buckets) * 4;
    default:
      return 0;
  }
}

void carve(gms_server_s* s, Request& q) {
  unsigned char* p = s->arena_base + q.mem_off;
  const size_t words = align_up(size_t(q.r.n) * 4, kAlign);
  const bool kv = q.r.d_value_in != nullptr;
  if (q.r.op == GMS_OP_HISTOGRAM) {
    q.hist = reinterpret_cast<int32_t*>(p);
    return;
  }
  q.keys = reinterpret_cast<uint32_t*>(p);
  p += words;
  if (kv) {
    q.vals = reinterpret_cast<uint32_t*>(p);
    p += words;
  }
  if (q.r.op == GMS_OP_SORT_7BIT) {
    q.tmpk = reinterpret_cast<uint32_t*>(p);
    p += words;
    if (kv) q.tmpv = reinterpret_cast<uint32_t*>(p);
  }
}

void finish(gms_server_s* s, Request& q, int status) {
  q.state = DONE;
  q.in_flight = false;
  q.res.done = 1;
  q.res.status = status;
  q.res.done_s = s->now();
  q.res.d_key_out = q.keys;
  q.res.d_value_out = q.vals;
  q.res.d_histogram = q.hist;
  s->stats.completed++;
  s->stats.keys += q.r.n;
  s->completed.push_back(q.id);
  s->active.erase(std::find(s->active.begin(), s->active.end(), q.id));
}

bool ensure_pinned(void** buf, size_t* cap, size_t need) {
  if (*cap >= need) return true;
  const size_t bytes = std::max(need, *cap * 2);
  if (*buf) cudaFreeHost(*buf);
  *buf = nullptr;
  *cap = 0;
  if (cudaHostAlloc(buf, bytes, cudaHostAllocDefault) != cudaSuccess) return false;
  *cap = bytes;
  return true;
}

// Collects finished rounds (in launch order).  Called with the lock held.
bool collect(gms_server_s* s) {
  bool progress = false;
  while (!s->rounds.empty()) {
    Round& rd = s->rounds.front();
    const cudaError_t q = cudaEventQuery(rd.done);
    if (q == cudaErrorNotReady) break;
    const uint32_t* rb = s->readback[rd.slot];
    int status = GMS_SUCCESS;
    if (q != cudaSuccess) {
      note_cuda_error(q);
      status = GMS_ERROR_CUDA;
    } else if (rb[0] != 0) {
      status = GMS_ERROR_DEVICE_TIMEOUT;
    }
    for (size_t i = 0; i < rd.compactions.size(); ++i) {
      auto it = s->reqs.find(rd.compactions[i].first);
      if (it != s->reqs.end()) it->second->res.num_bucket0 = rb[1 + rd.compactions[i].second] - rd.compaction_base[i];
    }
    for (uint64_t id : rd.reqs) {
      auto it = s->reqs.find(id);
      if (it == s->reqs.end()) continue;
      Request& qq = *it->second;
      qq.in_flight = false;
      qq.res.rounds++;
      if (status != GMS_SUCCESS) {
        finish(s, qq, status);
      } else if (qq.r.op == GMS_OP_SORT_7BIT && ++qq.pass < 5) {
        // more digit passes to go
      } else {
        finish(s, qq, GMS_SUCCESS);
      }
    }
    if (rd.scratch_off != SIZE_MAX) s->rounds_arena.release(rd.scratch_off);
    if (rd.plan) gms_batch_destroy(rd.plan);
    cudaEventDestroy(rd.done);
    s->rounds.pop_front();
    progress = true;
  }
  if (progress) s->cv_done.notify_all();
  return progress;
}

// Admits queued requests in arrival order while they fit.
bool admit(gms_server_s* s) {
  bool progress = false;
  while (!s->queue.empty()) {
    Request& q = *s->reqs[s->queue.front()];
    q.mem_bytes = request_bytes(q.r);
    const size_t off = q.mem_bytes ? s->requests_arena.alloc(q.mem_bytes) : 0;
    if (off == SIZE_MAX) break;
    q.mem_off = q.mem_bytes ? off : SIZE_MAX;
    if (q.mem_bytes) carve(s, q);
    q.state = ACTIVE;
    q.res.admit_s = s->now();
    s->active.push_back(q.id);
    s->queue.pop_front();
    progress = true;
    if (q.r.n == 0 && q.r.op != GMS_OP_HISTOGRAM) finish(s, q, GMS_SUCCESS);  // a histogram still needs zeroing
  }
  return progress;
}

void host_notify(void* p) {
  auto* s = static_cast<gms_server_s*>(p);
  s->cv_work.notify_one();
}

// Builds and launches one round from every admitted request not on the GPU.
bool launch_round(gms_server_s* s) {
  if (int(s->rounds.size()) >= kSlots) return false;
  std::vector<gms_segment> segs;
  std::vector<uint64_t> seg_req, hist_req, ids;
  for (uint64_t id : s->active) {
    Request& q = *s->reqs[id];
    if (q.in_flight || q.state != ACTIVE) continue;
    const bool kv = q.r.d_value_in != nullptr;
    if (q.r.op == GMS_OP_HISTOGRAM) {
      hist_req.push_back(id);
      continue;
    }
    gms_segment g{};
    g.n = q.r.n;
    g.desc = q.r.desc;
    if (q.r.op == GMS_OP_SORT_7BIT) {
      // ping-pong of src/api/multisplit_sort.cuh:340-363: in -> out -> tmp -> out -> tmp -> out
      const int p = q.pass;
      g.d_key_in = p == 0 ? q.r.d_key_in : (p % 2 ? q.keys : q.tmpk);
      g.d_key_out = p % 2 ? q.tmpk : q.keys;
      if (kv) {
        g.d_value_in = p == 0 ? q.r.d_value_in : (p % 2 ? q.vals : q.tmpv);
        g.d_value_out = p % 2 ? q.tmpv : q.vals;
      }
      g.desc = gms_bucket_desc{};
      g.desc.kind = GMS_BUCKET_BITS;
      g.desc.num_buckets = kSortBuckets[p];
      g.desc.shift = kSortShift[p];
    } else {
      g.d_key_in = q.r.d_key_in;
      g.d_key_out = q.keys;
      g.d_value_in = q.r.d_value_in;
      g.d_value_out = kv ? q.vals : nullptr;
    }
    segs.push_back(g);
    seg_req.push_back(id);
  }
  if (segs.empty() && hist_req.empty()) return false;
  // A round whose scratch does not fit while nothing else is in flight is cut
  // in half until it does (its other requests join later rounds).  The plan
  // that fits is the round's plan (a plan is built once per round).
  size_t keep = segs.size();
  gms_batch_t plan = nullptr;
  while (keep > 0) {
    size_t need = 0;
    if (gms_batch_create(segs.data(), uint32_t(keep), &plan) != GMS_SUCCESS) {
      plan = nullptr;
      break;
    }
    gms_batch_scratch_bytes(plan, &need);
    if (align_up(need, kAlign) <= s->rounds_arena.size() || keep == 1) break;
    gms_batch_destroy(plan);
    plan = nullptr;
    keep /= 2;
  }
  if (keep < segs.size()) {
    segs.resize(keep);
    seg_req.resize(keep);
  }

  Round rd;
  rd.slot = s->next_slot;
  cudaStream_t st = s->streams[rd.slot];
  if (!segs.empty() && plan == nullptr) {
    for (uint64_t id : seg_req) finish(s, *s->reqs[id], GMS_ERROR_INVALID_VALUE);
    return true;
  }
  size_t scratch_bytes = 0;
  if (plan) gms_batch_scratch_bytes(plan, &scratch_bytes);
  if (plan) {
    rd.scratch_off = s->rounds_arena.alloc(scratch_bytes);
    if (rd.scratch_off == SIZE_MAX) {  // wait for a round to finish
      gms_batch_destroy(plan);
      return false;
    }
  }
  size_t comp = 0;
  for (uint64_t id : seg_req) comp += s->reqs[id]->r.op == GMS_OP_COMPACTION;
  const size_t table = plan ? batch_table_bytes(plan) : 0;
  if (!ensure_pinned(&s->pinned[rd.slot], &s->pinned_cap[rd.slot], std::max<size_t>(table, 256)) ||
      !ensure_pinned(reinterpret_cast<void**>(&s->readback[rd.slot]), &s->readback_cap[rd.slot], 4 * (comp + 1))) {
    if (plan) {
      s->rounds_arena.release(rd.scratch_off);
      gms_batch_destroy(plan);
    }
    return false;
  }
  unsigned char* scratch = plan ? s->arena_base + s->rounds_off + rd.scratch_off : nullptr;
  cudaError_t e = cudaSuccess;
  gms_status gst = GMS_SUCCESS;
  uint32_t launches = 0;
  if (plan) {
    gst = batch_run_async(plan, scratch, scratch_bytes, s->pinned[rd.slot], s->pinned_cap[rd.slot], st);
    gms_batch_launch_count(plan, &launches);
  }
  for (uint64_t id : hist_req) {
    if (gst != GMS_SUCCESS) break;
    Request& q = *s->reqs[id];
    e = cudaMemsetAsync(q.hist, 0, size_t(q.r.desc.num_buckets) * 4, st);
    if (e == cudaSuccess) gst = gms_histogram(q.r.d_key_in, q.r.n, &q.r.desc, q.hist, st);
    launches += 1;
  }
  // Read back the error word and each compaction's bucket-0 count (start of bucket 1 in tile 0).
  uint32_t* rb = s->readback[rd.slot];
  if (gst == GMS_SUCCESS && plan) e = cudaMemcpyAsync(rb, scratch, 4, cudaMemcpyDeviceToHost, st);
  else if (gst == GMS_SUCCESS) rb[0] = 0;
  uint32_t k = 0;
  for (size_t i = 0; gst == GMS_SUCCESS && e == cudaSuccess && i < seg_req.size(); ++i) {
    if (s->reqs[seg_req[i]]->r.op != GMS_OP_COMPACTION || segs[i].n == 0) continue;
    uint32_t base = 0;
    const uint32_t word = batch_matrix_value_offset(plan, uint32_t(i), 1, 0, &base);
    e = cudaMemcpyAsync(rb + 1 + k, scratch + size_t(word) * 4, 4, cudaMemcpyDeviceToHost, st);
    rd.compactions.emplace_back(seg_req[i], k);
    rd.compaction_base.push_back(base);
    ++k;
  }
  if (e == cudaSuccess && gst == GMS_SUCCESS) e = cudaEventCreateWithFlags(&rd.done, cudaEventDisableTiming);
  if (e == cudaSuccess && gst == GMS_SUCCESS) e = cudaEventRecord(rd.done, st);
  if (e == cudaSuccess && gst == GMS_SUCCESS) e = cudaLaunchHostFunc(st, host_notify, s);
  if (e != cudaSuccess || gst != GMS_SUCCESS) {
    if (e != cudaSuccess) note_cuda_error(e);
    const int status = gst != GMS_SUCCESS ? gst : GMS_ERROR_CUDA;
    cudaStreamSynchronize(st);
    if (rd.done) cudaEventDestroy(rd.done);
    if (plan) {
      s->rounds_arena.release(rd.scratch_off);
      gms_batch_destroy(plan);
    }
    for (uint64_t id : seg_req) finish(s, *s->reqs[id], status);
    for (uint64_t id : hist_req) finish(s, *s->reqs[id], status);
    return true;
  }
  rd.plan = plan;
  rd.reqs = seg_req;
  rd.reqs.insert(rd.reqs.end(), hist_req.begin(), hist_req.end());
  for (uint64_t id : rd.reqs) s->reqs[id]->in_flight = true;
  s->stats.rounds++;
  s->stats.launches += launches;
  s->stats.max_requests_in_round = std::max<uint32_t>(s->stats.max_requests_in_round, uint32_t(rd.reqs.size()));
  s->rounds.push_back(std::move(rd));
  s->next_slot = (s->next_slot + 1) % kSlots;
  return true;
}

void scheduler(gms_server_s* s) {
  std::unique_lock<std::mutex> lock(s->mu);
  while (true) {
    bool progress = collect(s);
    progress |= admit(s);
    progress |= launch_round(s);
    s->stats.arena_peak_bytes = s->requests_arena.peak() + s->rounds_arena.peak();
    const bool blocked = !s->queue.empty() && s->active.empty() && s->rounds.empty();
    if (blocked != s->blocked_on_release) {
      s->blocked_on_release = blocked;
      if (blocked) s->cv_done.notify_all();  // drain and wait return instead of waiting forever
    }
    if (s->stop && s->queue.empty() && s->active.empty() && s->rounds.empty()) break;
    if (progress) continue;
    if (!s->rounds.empty()) {
      // A round is on the GPU: poll its event (only this thread touches the
      // round queue) rather than wait for the host callback, which answers
      // tens of microseconds later; new submissions are picked up between polls.
      const cudaEvent_t done = s->rounds.front().done;
      lock.unlock();
      for (int i = 0; i < 256 && cudaEventQuery(done) == cudaErrorNotReady; ++i) std::this_thread::yield();
      lock.lock();
    } else {
      s->cv_work.wait_for(lock, std::chrono::microseconds(200));
    }
  }
}

}  // namespace
}  // namespace gms

using namespace gms;

extern "C" {

gms_status gms_server_create(void* d_arena, size_t arena_bytes, gms_server_t* server) {
  if (server == nullptr || d_arena == nullptr || (reinterpret_cast<uintptr_t>(d_arena) & (kAlign - 1)) != 0 ||
      arena_bytes < (size_t(1) << 20))
    return GMS_ERROR_INVALID_VALUE;
  auto* s = new gms_server_s();
  s->arena_base = static_cast<unsigned char*>(d_arena);
  // An eighth of the arena (at most 4 GiB) is kept for round scratch, so
  // admitted requests can never starve the rounds that finish them.
  const size_t reserve = align_up(std::min(arena_bytes / 8, size_t(4) << 30), kAlign);
  const size_t req_bytes = (arena_bytes - reserve) / kAlign * kAlign;
  s->requests_arena = Arena(req_bytes);
  s->rounds_off = req_bytes;
  s->rounds_arena = Arena(arena_bytes - req_bytes);
  s->t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < kSlots; ++i) {
    if (cudaStreamCreateWithFlags(&s->streams[i], cudaStreamNonBlocking) != cudaSuccess) {
      for (int j = 0; j < i; ++j) cudaStreamDestroy(s->streams[j]);
      delete s;
      return GMS_ERROR_CUDA;
    }
  }
  // Pinned staging for the round tables and the read-back words, allocated
  // up front: growing them later frees pinned memory, which waits for the
  // whole device and stalls the round in flight on the other stream.  A
  // failure here only leaves the growth to the first rounds.
  for (int i = 0; i < kSlots; ++i) {
    ensure_pinned(&s->pinned[i], &s->pinned_cap[i], kInitialStaging);
    ensure_pinned(reinterpret_cast<void**>(&s->readback[i]), &s->readback_cap[i], kInitialReadback);
  }
  s->worker = std::thread(scheduler, s);
  *server = s;
  return GMS_SUCCESS;
}

gms_status gms_server_submit(gms_server_t s, const gms_request* r, uint64_t* id) {
  if (s == nullptr || r == nullptr || id == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (r->op < GMS_OP_MULTISPLIT || r->op > GMS_OP_COMPACTION) return GMS_ERROR_INVALID_VALUE;
  if (r->n > 0 && r->d_key_in == nullptr) return GMS_ERROR_INVALID_VALUE;
  if (r->op != GMS_OP_SORT_7BIT) {
    uint32_t b = r->desc.num_buckets;
    if (b < 2 || b > 256) return GMS_ERROR_UNSUPPORTED_BUCKETS;
    if (r->desc.kind == GMS_BUCKET_BITS && (b & (b - 1)) != 0) return GMS_ERROR_UNSUPPORTED_BUCKETS;
    if (r->op == GMS_OP_COMPACTION && b != 2) return GMS_ERROR_INVALID_VALUE;
  }
  if (request_bytes(*r) > s->requests_arena.size()) return GMS_ERROR_SCRATCH_TOO_SMALL;
  std::lock_guard<std::mutex> lock(s->mu);
  auto q = std::make_unique<Request>();
  q->id = s->next_id++;
  q->r = *r;
  q->res.submit_s = s->now();
  *id = q->id;
  s->queue.push_back(q->id);
  s->reqs.emplace(q->id, std::move(q));
  s->stats.submitted++;
  s->cv_work.notify_one();
  return GMS_SUCCESS;
}

gms_status gms_server_poll(gms_server_t s, uint64_t id, gms_result* out) {
  if (s == nullptr || out == nullptr) return GMS_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return GMS_ERROR_INVALID_VALUE;
  *out = it->second->res;
  return GMS_SUCCESS;
}

gms_status gms_server_wait(gms_server_t s, uint64_t id, gms_result* out) {
  if (s == nullptr) return GMS_ERROR_INVALID_VALUE;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return GMS_ERROR_INVALID_VALUE;
  Request* q = it->second.get();
  s->cv_done.wait(lock, [&] { return q->state == DONE || s->blocked_on_release; });
  if (q->state != DONE) return GMS_ERROR_SCRATCH_TOO_SMALL;
  if (out) *out = q->res;
  return GMS_SUCCESS;
}

gms_status gms_server_take_completed(gms_server_t s, uint64_t* ids, uint32_t max, uint32_t* count) {
  if (s == nullptr || count == nullptr || (ids == nullptr && max > 0)) return GMS_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> lock(s->mu);
  const uint32_t k = uint32_t(std::min<size_t>(max, s->completed.size()));
  std::copy(s->completed.begin(), s->completed.begin() + k, ids);
  s->completed.erase(s->completed.begin(), s->completed.begin() + k);
  *count = k;
  return GMS_SUCCESS;
}

gms_status gms_server_release(gms_server_t s, uint64_t id) {
  if (s == nullptr) return GMS_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end() || it->second->state != DONE) return GMS_ERROR_INVALID_VALUE;
  if (it->second->mem_off != SIZE_MAX) s->requests_arena.release(it->second->mem_off);
  s->reqs.erase(it);
  s->cv_work.notify_one();
  return GMS_SUCCESS;
}

gms_status gms_server_drain(gms_server_t s) {
  if (s == nullptr) return GMS_ERROR_INVALID_VALUE;
  std::unique_lock<std::mutex> lock(s->mu);
  s->cv_done.wait(lock, [&] {
    return (s->queue.empty() && s->active.empty() && s->rounds.empty()) || s->blocked_on_release;
  });
  return s->queue.empty() && s->active.empty() && s->rounds.empty() ? GMS_SUCCESS : GMS_ERROR_SCRATCH_TOO_SMALL;
}

gms_status gms_server_get_stats(gms_server_t s, gms_server_stats* out) {
  if (s == nullptr || out == nullptr) return GMS_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> lock(s->mu);
  *out = s->stats;
  return GMS_SUCCESS;
}

double gms_server_clock(gms_server_t s) { return s ? s->now() : 0.0; }

gms_status gms_server_destroy(gms_server_t s) {
  if (s == nullptr) return GMS_SUCCESS;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
    s->cv_work.notify_one();
  }
  s->worker.join();
  for (int i = 0; i < kSlots; ++i) {
    cudaStreamSynchronize(s->streams[i]);
    cudaStreamDestroy(s->streams[i]);
    if (s->pinned[i]) cudaFreeHost(s->pinned[i]);
    if (s->readback[i]) cudaFreeHost(s->readback[i]);
  }
  delete s;
  return GMS_SUCCESS;
}

}  // extern "C"
