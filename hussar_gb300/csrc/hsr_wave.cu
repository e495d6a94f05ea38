// The wavefront kernel's FP32 reference-phase instantiations (compiled without
// multiply-add contraction) and its host entry points; the kernel is in hsr_wave.cuh.
#include "hsr_wave.cuh"

namespace hsr {

size_t wave_smem_bytes(int samples, bool guided) { return wave_smem_for<kWaveDefaultQueue>(samples, guided); }

int wave_blocks_per_sm(int samples, bool mixed, bool guided) {
    int nb = 0;
    if (mixed) {
        const size_t smem = wave_smem_for<kWaveSmallQueue>(samples, guided);
        auto *k = k_wave<HSR_PHASE_REFERENCE_FP32, true, kWaveSmallQueue>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kThreads, smem);
    } else {
        const size_t smem = wave_smem_bytes(samples, guided);
        auto *k = k_wave<HSR_PHASE_REFERENCE_FP32, false, kWaveDefaultQueue>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kThreads, smem);
    }
    return nb > 0 ? nb : 1;
}

int launch_wave(const TraceParams &p, int phase_mode, int grid, cudaStream_t st, std::string &err) {
    if (phase_mode == HSR_PHASE_SPLIT_FP64)
        launch_wave_split(p, grid, st);
    else
        wave_dispatch<HSR_PHASE_REFERENCE_FP32>(p, grid, st);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("wave launch: ") + cudaGetErrorString(e);
        return 2;
    }
    return 0;
}

}  // namespace hsr
