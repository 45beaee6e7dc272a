// Kernel instances of the digit passes (more than 256 buckets) for one
// identifier kind: the prescans, the whole-id histogram and the bucket starts
// read off the sorted output.  The build compiles
// this file once per kind with -DGMS_INST_KIND=<kind>.
#include "ms_dispatch.cuh"

#if !defined(GMS_INST_KIND)
#error "inst_big.cu is compiled once per identifier kind with GMS_INST_KIND defined"
#endif

GMS_INSTANTIATE_BIG(GMS_INST_KIND)
