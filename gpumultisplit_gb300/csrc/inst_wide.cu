// Kernel instances with 64-bit keys or values for one identifier kind.  The
// build compiles this file once per kind with -DGMS_INST_KIND=<kind>, so the
// instances compile in parallel.
#include "ms_dispatch.cuh"

#if !defined(GMS_INST_KIND)
#error "inst_wide.cu is compiled once per identifier kind with GMS_INST_KIND defined"
#endif

GMS_INSTANTIATE_WIDE(GMS_INST_KIND)
