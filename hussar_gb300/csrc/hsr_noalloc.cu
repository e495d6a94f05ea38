// Allocation-free batch simulation: hsr_simulate_batch_device_noalloc.
//
// Some callers cannot allocate device memory while they simulate: code that runs inside
// a region where cudaMalloc is not allowed or would stall the device (for instance a
// real-time loop or work being recorded into a larger asynchronous pipeline), or a host
// framework whose own memory pool must own every device allocation. For them this entry
// point runs the plain (unguided) batched simulation of hsr_simulate_batch_device with
// every scratch buffer it needs (status word, work counter, tile prefix, FP64 range
// accumulators) in one file-scope device array of fixed size, so the call itself
// allocates nothing: no cudaMalloc, no cudaFree, no allocating library routine.
//
// Limits: at most kNoAllocMaxPoses poses and kNoAllocMaxBins range bins per call
// (1 MiB of accumulators), guiding off, the reference's 33-bin frame splat.
//
// The array is one per device and shared by every call on that device; each call clears
// the parts that must start at zero, and the last call's contents stay behind. Calls that
// overlap on the GPU (concurrent streams, or host threads issuing on the same device) use
// the same array and race: serialise them. The first call on a device looks up the
// array's device address (cudaGetSymbolAddress) with that device current; make that first
// call before any stream capture.
//
// The call runs the launch shape the scene was tuned to (hsr_autotune_batch /
// hsr_set_launch_config) and the kernel hsr_set_path_kernel selects, as
// hsr_simulate_batch_device does. Device-side conditions (traversal stack overflow, a bin
// out of range, a bad work item) set bits in the array's status word; the call returns
// before the GPU has run, so the caller reads them with hsr_noalloc_status once the work
// is done (it synchronises the stream; the word is cleared by the next call).
#include <mutex>

#include "hsr_common.cuh"
#include "hsr_internal.h"

namespace hsr {

namespace {

constexpr int kNoAllocMaxPoses = 64;
constexpr int kNoAllocMaxBins = 1024;
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocScratch {
    unsigned counters[64];                         // [0] status word, [2..3] 64-bit work counter
    long long tile_start[kNoAllocMaxPoses + 8];    // tile prefix (pose_count + 1 entries)
    double acc[2 * kNoAllocMaxPoses * kNoAllocMaxBins];
};

// The scratch array itself (device memory for the lifetime of the program on every
// device that loads this library). Host code must not pass its host-side name to a
// kernel; it uses the address looked up per device below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once per device).
hsr_status noalloc_scratch(NoAllocScratch **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
        cudaGetLastError();
        set_last_error("no usable current device for the allocation-free entry point");
        return HSR_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            set_last_error(std::string("cudaGetSymbolAddress of the static scratch failed: ") + cudaGetErrorString(e));
            return HSR_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<NoAllocScratch *>(g_noalloc_ptr[dev]);
    return HSR_OK;
}

}  // namespace

}  // namespace hsr

using namespace hsr;

extern "C" hsr_status hsr_simulate_batch_device_noalloc(hsr_scene *scene, const hsr_rf_config *rf,
                                                        int32_t samples_per_chirp, const hsr_tracer_flags *flags,
                                                        int32_t pose_count, const hsr_antenna *d_tx,
                                                        const hsr_antenna *d_rx, const int64_t *d_budget,
                                                        const int64_t *d_index_offset, int32_t phase_mode,
                                                        float *d_out_rows, void *stream) {
    const SceneDev *sc = scene_device_state(scene);
    if (!sc || !rf || !flags || !d_tx || !d_rx || !d_budget || !d_index_offset || !d_out_rows) {
        set_last_error("null argument");
        return HSR_ERR_INVALID_ARGUMENT;
    }
    // the scene's BVH lives on the device it was built on: the call must be issued there
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != sc->device) {
        cudaGetLastError();
        set_last_error("the current device is not the device the scene was built on");
        return HSR_ERR_INVALID_ARGUMENT;
    }
    const int32_t N = samples_per_chirp, P = pose_count;
    if (P <= 0 || P > kNoAllocMaxPoses) {
        set_last_error("pose_count must be in [1, " + std::to_string(kNoAllocMaxPoses) +
                       "] for the allocation-free entry point (its scratch has a fixed size)");
        return HSR_ERR_INVALID_ARGUMENT;
    }
    if (N <= 0 || N > kNoAllocMaxBins) {
        set_last_error("samples_per_chirp must be in [1, " + std::to_string(kNoAllocMaxBins) +
                       "] for the allocation-free entry point (its scratch has a fixed size)");
        return HSR_ERR_INVALID_ARGUMENT;
    }
    if (flags->maxDepth < 0) {
        set_last_error("maxDepth must be >= 0");
        return HSR_ERR_INVALID_ARGUMENT;
    }
    if (flags->doGuiding) {
        set_last_error("the allocation-free entry point runs the plain method only (doGuiding must be 0)");
        return HSR_ERR_NOT_SUPPORTED;
    }
    if (phase_mode != HSR_PHASE_REFERENCE_FP32 && phase_mode != HSR_PHASE_SPLIT_FP64) {
        set_last_error("unknown phase mode");
        return HSR_ERR_INVALID_ARGUMENT;
    }
    NoAllocScratch *s = nullptr;
    hsr_status st = noalloc_scratch(&s);
    if (st != HSR_OK) return st;
    // serialised with the scene's other calls (its tuned shape is read below); the scene
    // must not be destroyed while this call's work is in flight
    std::lock_guard<std::mutex> lk(*scene_mutex(scene));
    cudaStream_t strm = static_cast<cudaStream_t>(stream);
    // what must start at zero: status word, work counter, this call's accumulators
    cudaError_t e = cudaMemsetAsync(s->counters, 0, sizeof(s->counters), strm);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->acc, 0, sizeof(double) * 2 * size_t(P) * N, strm);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error(std::string("clearing the static scratch: ") + cudaGetErrorString(e));
        return HSR_ERR_CUDA;
    }
    // the scene's tuned work-item size where it has one, else 4096 samples (the prefix
    // holds pose_count + 1 entries whatever the tile)
    const int32_t tile = sc->tuned.tile > 0 ? sc->tuned.tile : 4096;
    int64_t *tile_start = reinterpret_cast<int64_t *>(s->tile_start);
    if (launch_tile_prefix(d_budget, P, tile, tile_start, strm) != 0) {
        set_last_error("tile prefix launch failed");
        return HSR_ERR_CUDA;
    }
    TraceParams p{};
    p.nodes = sc->nodes;
    p.tris = sc->tris;
    p.rf = *rf;
    p.flags = *flags;
    p.samples = N;
    p.pose_count = P;
    p.tx = d_tx;
    p.rx = d_rx;
    p.budget = d_budget;
    p.offset = d_index_offset;
    p.tile_start = tile_start;
    p.sample_weight = 1.f;
    p.tile = tile;
    p.acc = s->acc;
    p.status = s->counters;
    p.work_counter = s->counters + 2;
    std::string err;
    const bool wave = g_path_kernel == 0 && flags->useGeometricalOptics != 0;
    int per_sm = wave ? wave_blocks_per_sm(N, false) : trace_blocks_per_sm(N, HSR_SPLAT_DIRICHLET16, 0);
    if (wave) {
        if (sc->tuned.ctas_per_sm > 0) per_sm = std::min(per_sm, sc->tuned.ctas_per_sm);
        p.queue_threshold = sc->tuned.queue_threshold;
        p.field_on_hit = sc->tuned.field_on_hit;
        p.coherent_order = sc->tuned.coherent_order;
    }
    const int grid = sc->sm_count * per_sm;
    const int rc = wave ? launch_wave(p, phase_mode, grid, strm, err)
                        : launch_trace(p, phase_mode, HSR_SPLAT_DIRICHLET16, grid, strm, err);
    if (rc != 0) {
        set_last_error(err);
        return HSR_ERR_CUDA;
    }
    if (launch_finalize(s->acc, P, N, d_budget, 1.f, nullptr, 1, d_out_rows, strm) != 0) {
        set_last_error("finalize launch failed");
        return HSR_ERR_CUDA;
    }
    return HSR_OK;
}

extern "C" hsr_status hsr_noalloc_status(void *stream, uint32_t *out_bits) {
    if (out_bits) *out_bits = 0;
    NoAllocScratch *s = nullptr;
    hsr_status st = noalloc_scratch(&s);
    if (st != HSR_OK) return st;
    cudaStream_t strm = static_cast<cudaStream_t>(stream);
    unsigned bits = 0;
    cudaError_t e = cudaStreamSynchronize(strm);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, s->counters, sizeof(unsigned), cudaMemcpyDeviceToHost, strm);
    if (e == cudaSuccess) e = cudaStreamSynchronize(strm);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error(std::string("reading the static scratch's status word: ") + cudaGetErrorString(e));
        return HSR_ERR_CUDA;
    }
    if (out_bits) *out_bits = bits;
    if (bits) {
        set_last_error(status_text(bits));
        return HSR_ERR_DEVICE;
    }
    return HSR_OK;
}
