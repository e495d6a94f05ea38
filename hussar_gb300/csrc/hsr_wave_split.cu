// The wavefront kernel's split-phase instantiations, compiled with multiply-add
// contraction: the split form is the accuracy-first one (FP64 path length and phase),
// bounded against the FP64 oracle rather than reproducing the reference's FP32
// rounding, and the fused forms are both faster and at least as accurate.
#include "hsr_wave.cuh"

namespace hsr {

void launch_wave_split(const TraceParams &p, bool mixed, int grid, size_t smem, cudaStream_t st) {
    if (mixed)
        wave_instance<HSR_PHASE_SPLIT_FP64, true>(p, grid, smem, st);
    else
        wave_instance<HSR_PHASE_SPLIT_FP64, false>(p, grid, smem, st);
}

}  // namespace hsr
