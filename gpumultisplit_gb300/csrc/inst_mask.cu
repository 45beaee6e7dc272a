// Kernel instances for the MASK bucket identifier (one translation unit per
// identifier kind so the library compiles in parallel).
#include "ms_dispatch.cuh"

GMS_INSTANTIATE_KIND(gms::KIND_MASK)
