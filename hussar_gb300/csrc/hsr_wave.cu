// The wavefront kernel's FP32 reference-phase instantiations (compiled without
// multiply-add contraction) and its host entry points; the kernel is in hsr_wave.cuh.
#include "hsr_wave.cuh"

namespace hsr {

size_t wave_smem_bytes(int samples, bool guided) {
    // guided: the CTA's training sums and the guiding part of the stacked paths
    return sizeof(WaveShared) + 2 * size_t(samples) * sizeof(float) +
           (guided ? (kGuideMaxNodes + kGuideStackFields * kStack) * sizeof(float) : 0);
}

int wave_blocks_per_sm(int samples, bool mixed) {
    int nb = 0;
    const size_t smem = wave_smem_bytes(samples, false);
    if (mixed) {
        cudaFuncSetAttribute(k_wave<HSR_PHASE_REFERENCE_FP32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_wave<HSR_PHASE_REFERENCE_FP32, true>, kThreads, smem);
    } else {
        cudaFuncSetAttribute(k_wave<HSR_PHASE_REFERENCE_FP32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_wave<HSR_PHASE_REFERENCE_FP32, false>, kThreads, smem);
    }
    return nb > 0 ? nb : 1;
}

int launch_wave(const TraceParams &p, int phase_mode, int grid, cudaStream_t st, std::string &err) {
    const size_t smem = wave_smem_bytes(p.samples, p.do_guide != 0);
    const bool split = phase_mode == HSR_PHASE_SPLIT_FP64;
    if (p.jobs) {
        if (split)
            launch_wave_split(p, true, grid, smem, st);
        else
            wave_instance<HSR_PHASE_REFERENCE_FP32, true>(p, grid, smem, st);
    } else {
        if (split)
            launch_wave_split(p, false, grid, smem, st);
        else
            wave_instance<HSR_PHASE_REFERENCE_FP32, false>(p, grid, smem, st);
    }
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("wave launch: ") + cudaGetErrorString(e);
        return 2;
    }
    return 0;
}

}  // namespace hsr
