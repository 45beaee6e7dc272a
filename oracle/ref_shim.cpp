// Exposes the REFERENCE's own CPU multisplit (cpu_multisplit_general and
// cpu_multisplit_pairs_general, src/cpu_functions.h:155-288) through a C ABI,
// for pinning the oracle and generating golden vectors.  Test infrastructure
// only.  It includes the reference header from the reference tree at build
// time (oracle/Makefile, target `ref`); no reference source is copied here.
//
// The bucket identifiers below are functors in the reference's style
// (operator() on a uint32 key), one per descriptor kind of oracle.h.
#include <stdint.h>
#include <stdio.h>
#include <unistd.h>

#include <algorithm>
#include <functional>
#include <iostream>
#include <string>
#include <vector>

// The reference header names cudaMemcpy in a debug printer that is never
// instantiated here; the CUDA runtime header only provides the declarations.
#include <cuda_runtime.h>

#include "cpu_functions.h"
#include "oracle.h"

namespace {

struct DescFunctor {
  oracle_desc d;
  uint32_t operator()(uint32_t key) const { return oracle_bucket(&d, key); }
};

// Plain functors matching the reference's own identifiers.
struct DeltaFunc {  // delta_func (src/main/main_multisplit.cu:41-47): a / delta
  uint32_t delta;
  uint32_t operator()(uint32_t a) const { return a / delta; }
};
struct TopBits {  // key * B >> 32 for B = 2^logb
  uint32_t logb;
  uint32_t operator()(uint32_t a) const { return a >> (32 - logb); }
};
struct BitField {  // ms_bucket_sort_*bit<x> (src/api/multisplit_sort.cuh:63-98)
  uint32_t shift, mask;
  uint32_t operator()(uint32_t a) const { return (a >> shift) & mask; }
};

// cpu_multisplit_* print a newline (and more when print_mode is set) on stdout;
// keep stdout clean for callers that parse it.
struct QuietStdout {
  int saved;
  QuietStdout() {
    fflush(stdout);
    saved = dup(1);
    FILE* null = fopen("/dev/null", "w");
    if (null) {
      dup2(fileno(null), 1);
      fclose(null);
    }
  }
  ~QuietStdout() {
    fflush(stdout);
    if (saved >= 0) {
      dup2(saved, 1);
      close(saved);
    }
  }
};

template <class F>
void run(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n, F f, uint32_t B) {
  QuietStdout q;
  // The reference functions take non-const pointers but only read the inputs.
  if (vin)
    cpu_multisplit_pairs_general(const_cast<uint32_t*>(kin), kout, const_cast<uint32_t*>(vin), vout, n, f, 0, B);
  else
    cpu_multisplit_general(const_cast<uint32_t*>(kin), kout, n, f, 0, B);
}

}  // namespace

extern "C" {

// Multisplit with any oracle descriptor (bucket ids come from oracle_bucket).
void ref_multisplit(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                    const oracle_desc* d) {
  run(kin, kout, vin, vout, n, DescFunctor{*d}, d->num_buckets);
}

// Multisplit with the reference-style functors (independent of oracle_bucket):
// kind 0: key >> (32 - log2 B); 1: key / param; 2: (key >> shift) & (B-1).
void ref_multisplit_functor(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n,
                            int kind, uint32_t B, uint32_t param) {
  if (kind == 0) {
    uint32_t logb = 0;
    while ((1u << logb) < B) ++logb;
    run(kin, kout, vin, vout, n, TopBits{logb}, B);
  } else if (kind == 1) {
    run(kin, kout, vin, vout, n, DeltaFunc{param}, B);
  } else {
    run(kin, kout, vin, vout, n, BitField{param, B - 1}, B);
  }
}

// The reference's sort digit schedules (src/api/multisplit_sort.cuh:320-559)
// driven by the reference's CPU multisplit; the last pass lands in kout.
void ref_sort(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t n, uint32_t* tmp_k,
              uint32_t* tmp_v, int digit_bits) {
  struct Pass {
    uint32_t shift, mask;
  };
  std::vector<Pass> s;
  switch (digit_bits) {
    case 4: for (uint32_t x = 0; x < 32; x += 4) s.push_back({x, 0x0F}); break;
    case 5: for (uint32_t x = 0; x < 30; x += 5) s.push_back({x, 0x1F}); s.push_back({30, 0x03}); break;
    case 6: s = {{0, 0x0F}, {4, 0x0F}, {8, 0x3F}, {14, 0x3F}, {20, 0x3F}, {26, 0x3F}}; break;
    case 7: s = {{0, 0x0F}, {4, 0x7F}, {11, 0x7F}, {18, 0x7F}, {25, 0x7F}}; break;
    case 8: s = {{0, 0xFF}, {8, 0xFF}, {16, 0xFF}, {24, 0xFF}}; break;
    default: return;
  }
  const uint32_t* sk = kin;
  const uint32_t* sv = vin;
  const int P = int(s.size());
  for (int p = 0; p < P; ++p) {
    const bool to_out = ((P - 1 - p) % 2) == 0;
    uint32_t* dk = to_out ? kout : tmp_k;
    uint32_t* dv = to_out ? vout : tmp_v;
    run(sk, dk, vin ? sv : nullptr, dv, n, BitField{s[p].shift, s[p].mask}, s[p].mask + 1);
    sk = dk;
    sv = dv;
  }
}

}  // extern "C"
