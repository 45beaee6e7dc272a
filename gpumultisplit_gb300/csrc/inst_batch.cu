// Batched-form kernel instances for one (identifier kind, tile variant).  The
// build compiles this file once per pair with -DGMS_INST_KIND=<kind>
// -DGMS_INST_VARIANT=<variant>, so the instances compile in parallel.
#include "ms_dispatch.cuh"

#if !defined(GMS_INST_KIND) || !defined(GMS_INST_VARIANT)
#error "inst_batch.cu is compiled once per (kind, variant) with GMS_INST_KIND and GMS_INST_VARIANT defined"
#endif

GMS_INSTANTIATE_BATCH(GMS_INST_KIND, GMS_INST_VARIANT)

#if GMS_INST_VARIANT == 0
GMS_INSTANTIATE_BATCH_WARP(GMS_INST_KIND)  // the one-warp-per-segment kernels, once per kind
#endif
