// Host side of the one-sweep sort (onesweep.cuh): scratch layout, the digit
// histogram, and one ticketed pass kernel per digit.
#include "ms_dispatch.cuh"
#include "onesweep.cuh"

namespace gms {
namespace {

// [header 256 B][bucket starts, OS_MAX_PASSES x 256 words][tickets, one word
// per pass, padded to 256 B][status words of one digit, tiles x 2^max_logb x 8 B]
struct OnesweepLayout {
  size_t off_hist, off_tickets, off_status, bytes;
  uint32_t num_tiles;
};

OnesweepLayout onesweep_layout(uint32_t n, int passes, const uint32_t* logb) {
  OnesweepLayout L;
  uint32_t max_logb = 1;
  for (int p = 0; p < passes; ++p) max_logb = logb[p] > max_logb ? logb[p] : max_logb;
  L.num_tiles = uint32_t((uint64_t(n) + 4095u) / 4096u);  // 8 warps x 16 keys per tile, key-only or key-value
  L.off_hist = sizeof(ScratchHeader);
  L.off_tickets = L.off_hist + size_t(OS_MAX_PASSES) * OS_HIST_STRIDE * 4;
  L.off_status = align_up(L.off_tickets + size_t(OS_MAX_PASSES) * 4, 256);
  L.bytes = align_up(L.off_status + size_t(L.num_tiles) * (size_t(1) << max_logb) * 8, 256);
  return L;
}

template <int LOGB, bool KV>
cudaError_t onesweep_pass(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                          uint32_t num_tiles, uint32_t shift, ScratchHeader* hdr, uint32_t* ticket,
                          uint64_t* status, const uint32_t* bases, cudaStream_t stream) {
  using S = TileShape<LOGB, KV>;
  using C = TileCfg<LOGB, S::WARPS, S::IPT, KV>;
  using P = DescPolicy<KIND_BITS, LOGB>;
  static_assert(C::TILE == 4096, "the layout assumes 4096-key tiles");
  static std::atomic<uint64_t> smem_done{0};
  static std::atomic<int> per_sm{0};
  auto kern = onesweep_pass_kernel<C, P>;
  constexpr size_t smem = PostLayout<C, P>::BYTES;
  cudaError_t e = ensure_smem_limit(kern, smem, smem_done, sizeof(uint32_t));
  if (e != cudaSuccess) return e;
  BucketParams bp{};
  bp.shift = shift;
  bp.num_buckets = 1u << LOGB;
  const uint32_t wave = persistent_grid(kern, C::THREADS, num_tiles, per_sm, smem);
  const uint32_t dist = (GMS_PREFETCH_WAVES * wave) / 4u;
  kern<<<num_tiles, C::THREADS, smem, stream>>>(kin, vin, kout, vout, n, num_tiles, bp, hdr, ticket, status, bases,
                                                  dist);
  return cudaGetLastError();
}

template <bool KV>
cudaError_t onesweep_pass_l(int logb, const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout,
                            uint32_t n, uint32_t num_tiles, uint32_t shift, ScratchHeader* hdr, uint32_t* ticket,
                            uint64_t* status, const uint32_t* bases, cudaStream_t s) {
  switch (logb) {
#define GMS_OS_CASE(L) \
  case L: return onesweep_pass<L, KV>(kin, vin, kout, vout, n, num_tiles, shift, hdr, ticket, status, bases, s);
    GMS_OS_CASE(1)
    GMS_OS_CASE(2)
    GMS_OS_CASE(3)
    GMS_OS_CASE(4)
    GMS_OS_CASE(5)
    GMS_OS_CASE(6)
    GMS_OS_CASE(7)
    GMS_OS_CASE(8)
#undef GMS_OS_CASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

size_t onesweep_scratch_bytes(uint32_t n, int passes, const uint32_t* logb) {
  return onesweep_layout(n, passes, logb).bytes;
}

cudaError_t run_onesweep_sort(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                              bool kv, int passes, const uint32_t* shift, const uint32_t* logb,
                              unsigned char* scratch, uint32_t* tk, uint32_t* tv, cudaStream_t stream) {
  if (passes < 1 || passes > OS_MAX_PASSES || n == 0) return cudaErrorInvalidValue;
  OnesweepDigits d{};
  d.passes = passes;
  for (int p = 0; p < passes; ++p) {
    if (logb[p] < 1 || logb[p] > 8) return cudaErrorInvalidValue;
    d.shift[p] = shift[p];
    d.logb[p] = logb[p];
  }
  const OnesweepLayout L = onesweep_layout(n, passes, logb);
  auto* hdr = reinterpret_cast<ScratchHeader*>(scratch);
  auto* hist = reinterpret_cast<uint32_t*>(scratch + L.off_hist);
  auto* tickets = reinterpret_cast<uint32_t*>(scratch + L.off_tickets);
  auto* status = reinterpret_cast<uint64_t*>(scratch + L.off_status);
  // header (error word, wait limit), histograms and tickets start at zero
  cudaError_t e = cudaMemsetAsync(scratch, 0, L.off_status, stream);
  if (e != cudaSuccess) return e;
  static std::atomic<int> hist_per_sm{0};
  const uint32_t hist_grid =
      persistent_grid(onesweep_hist_kernel, 256, uint32_t((uint64_t(n) + 4095u) / 4096u), hist_per_sm);
  onesweep_hist_kernel<<<hist_grid, 256, 0, stream>>>(kin, n, d, hist);
  onesweep_bases_kernel<<<passes, 256, 0, stream>>>(hist, d);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const uint32_t* ki = kin;
  const uint32_t* vi = vin;
  for (int p = 0; p < passes; ++p) {
    const bool to_out = ((passes - 1 - p) % 2) == 0;
    uint32_t* ko = to_out ? kout : tk;
    uint32_t* vo = kv ? (to_out ? vout : tv) : nullptr;
    e = cudaMemsetAsync(status, 0, size_t(L.num_tiles) * (size_t(1) << logb[p]) * 8, stream);
    if (e != cudaSuccess) return e;
    e = kv ? onesweep_pass_l<true>(int(logb[p]), ki, vi, ko, vo, n, L.num_tiles, shift[p], hdr, tickets + p, status,
                                   hist + size_t(p) * OS_HIST_STRIDE, stream)
           : onesweep_pass_l<false>(int(logb[p]), ki, nullptr, ko, nullptr, n, L.num_tiles, shift[p], hdr,
                                    tickets + p, status, hist + size_t(p) * OS_HIST_STRIDE, stream);
    if (e != cudaSuccess) return e;
    ki = ko;
    vi = vo;
  }
  return cudaSuccess;
}

}  // namespace gms
