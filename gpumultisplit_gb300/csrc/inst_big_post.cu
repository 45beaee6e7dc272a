// Postscans of the digit passes (more than 256 buckets).  They read the bytes
// the prescan kept, so one set of instances serves every identifier kind.
#include "ms_dispatch.cuh"

namespace gms {

cudaError_t run_digit_postscan(const DigitPass& c) { GMS_DIGIT_SWITCH(digit_postscan_t, ) }

}  // namespace gms
