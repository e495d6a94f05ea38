// The wavefront kernel's split-phase instantiations, compiled with multiply-add
// contraction and the approximate single-precision divide and square root (within 2
// ulp): the split form is the accuracy-first one (FP64 path length and phase), bounded
// against the FP64 oracle rather than reproducing the reference's FP32 rounding, and
// its error is set by the FP32 geometry (~1e-7 relative), which these leave unchanged.
#include "hsr_wave.cuh"

namespace hsr {

void launch_wave_split(const TraceParams &p, int grid, cudaStream_t st) {
    wave_dispatch<HSR_PHASE_SPLIT_FP64>(p, grid, st);
}

}  // namespace hsr
