// Host-side internals shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hsr_gb300.h"

namespace hsr {

struct DTri;
struct DNode;

// Fine range histogram: 8 sub-bins per range bin and moments 0..3 of the sub-bin offset.
constexpr int kFineOS = 8;
constexpr int kFineMoments = 4;
constexpr int kFineRowPerBin = 2 * kFineMoments * kFineOS;  // floats per range bin per pose

// Twiddle operand of the fine-histogram synthesis for N range bins (hsr_synth.cu).
struct SynthOperand {
    int N = 0, K = 0, KK = 0, KKpad = 0, NCpad = 0;
    float *bt = nullptr;  // FP32 B^T [NCpad x KKpad]
    void *b1 = nullptr, *b2 = nullptr, *b3 = nullptr;  // its three BF16 terms
};

// Launch shape of the plain wavefront pass chosen by the autotuner (0 fields: default).
struct LaunchConfig {
    int32_t tile = 0;             // samples per work item
    int32_t ctas_per_sm = 0;      // persistent grid: SMs x this (<= the occupancy limit)
    int32_t queue_threshold = 0;  // see TraceParams::queue_threshold
    int32_t field_on_hit = 0;     // see TraceParams::field_on_hit
    int32_t coherent_order = 0;   // see TraceParams::coherent_order
};
// wavefront path stacks: 256 + the GENERATE threshold entries; three capacities
constexpr int kWaveMaxQueueThreshold = 256;  // thresholds above 128: the 512-entry stack
constexpr int kWaveDefaultQueue = 128;       // threshold 0 (the default) and up to 128: 384 entries
constexpr int kWaveSmallQueue = 64;          // thresholds up to this run with a 320-entry stack

// A resident scene: triangles + BVH on the device, plus per-scene scratch reused by
// every simulate call on this scene (calls on one scene must not overlap).
struct SceneDev {
    int device = 0;
    int64_t tri_count = 0;
    int64_t node_count = 0;
    int64_t leaf_count = 0;
    int max_depth = 0;
    DTri *tris = nullptr;
    DNode *nodes = nullptr;
    // the mesh's triangle vertex indices (kept for refits) and vertex count
    int32_t *indices = nullptr;
    int64_t vertex_count = 0;
    // refit order: the BVH's reachable internal nodes level by level from the root
    // (built at the first refit), and where each level starts
    int32_t *refit_order = nullptr;
    std::vector<int64_t> refit_levels;
    // scratch
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    unsigned *status = nullptr;  // device status word + work counter
    void *guide = nullptr;       // guiding trees + step scratch, sized for guide_cap poses
    int guide_cap = 0;
    SynthOperand synth;          // cached twiddle operand (fine-histogram synthesis)
    void *synth_scratch = nullptr;
    size_t synth_scratch_bytes = 0;
    void *frame_buf = nullptr;  // MIMO radar cube (hsr_simulate_frame), grown as needed
    size_t frame_bytes = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    LaunchConfig tuned;  // set by hsr_autotune_batch / hsr_set_launch_config
    float last_kernel_ms = 0.f;
    bool timing_valid = false;
    int sm_count = 0;
};

// Counts every device allocation the library makes (hsr_debug_alloc_count).
void note_alloc();

template <typename T> inline bool dev_alloc(T **p, size_t bytes, std::string &err) {
    note_alloc();
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), bytes ? bytes : 16);
    if (e != cudaSuccess) {
        err = std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e);
        *p = nullptr;
        cudaGetLastError();
        return false;
    }
    return true;
}

void note_launches(int64_t n);
const SceneDev *scene_device_state(const hsr_scene *s);
// Guiding trees for P poses.
// PathTracer::run's schedule (path.h:171-224) for one pose: per iteration the
// backend-run budget, Halton offset, sample weight, whether the frame is cleared
// before it, and whether it trains the guiding tree (not in the final iteration).
struct Iter {
    int64_t budget, offset;
    float weight;
    bool clear, train;
};
std::vector<Iter> schedule(int64_t samples, bool clearBeforeIteration);

// The device status word's bits as a message ("device status: ...").
std::string status_text(unsigned bits);
// The scene's call lock (calls on one scene are serialised).
std::mutex *scene_mutex(hsr_scene *s);
void set_last_error(const std::string &msg);

int bvh_build(SceneDev &s, const float *d_v, int64_t nv, const int32_t *d_idx, int64_t nt, cudaStream_t st,
              std::string &err);
// New vertex positions for the scene's mesh (same triangles): triangle records rewritten
// and every node box refitted bottom-up over the existing topology. Returns 0, 2 or 3.
int bvh_refit(SceneDev &s, const float *d_v, cudaStream_t st, std::string &err);

// Per-pose scene, chirp and accumulator row of a mixed batch (the serving loop): poses
// of one launch may trace different resident scenes with different RF configurations
// and range-bin counts. The tracer flags and the phase mode stay uniform.
struct PoseJob {
    const DNode *nodes;
    const DTri *tris;
    hsr_rf_config rf;
    int32_t samples;     // N of this pose (<= TraceParams::samples, which sizes the CTA row)
    int32_t reserved;
    int64_t acc_offset;  // first double of the pose's 2N accumulators in TraceParams::acc
};

// Launch parameters of the trace kernels (POD, passed by value).
struct TraceParams {
    const DNode *nodes;
    const DTri *tris;
    hsr_rf_config rf;
    hsr_tracer_flags flags;
    int32_t samples;        // samplesPerChirp (N)
    int32_t pose_count;
    const hsr_antenna *tx;  // [pose_count]
    const hsr_antenna *rx;  // [pose_count]
    const int64_t *budget;  // [pose_count]
    const int64_t *offset;  // [pose_count] Halton index offset
    const int64_t *tile_start;  // [pose_count + 1] prefix sum of tiles per pose
    float sample_weight;
    int32_t tile;           // samples per work item
    double *acc;            // [pose_count][N] complex (re, im) accumulators
    unsigned *status;       // status word
    unsigned *work_counter; // dynamic work item counter
    void *records;          // optional PathRecord[budget][max_rec] (tests)
    int32_t max_rec;
    unsigned long long *counters;  // optional [nodes, tris, rays] (counting instantiation)
    // per-pose sample weight (PathTracer::currentSampleWeight); nullptr: sample_weight for all
    const float *weights;
    // path guiding (doGuiding): trees [pose][kGuideMaxNodes]; train[pose] = 1 splats into
    // the training tree (every iteration but the final one, path.h:448)
    int32_t do_guide;
    const int *train;
    const int *g_samp_child;
    const float *g_samp_p;
    const int *g_train_child;
    float *g_train_acc;
    // fine-histogram mode (HSR_SPLAT_FINE_SYNTH): per pose a row of 8K FP64 sums,
    // [Re h0 .. Re h3 | Im h0 .. Im h3], K = 8 N; nullptr: Dirichlet splat
    int32_t fine_bins;      // K
    double *fine;
    // mixed batch: per-pose scene/chirp/row (nodes, tris, rf and acc rows above are then
    // unused; samples is the largest N); nullptr: uniform batch. Wavefront kernel only.
    const PoseJob *jobs;
    // wavefront kernel: GENERATE runs while a CTA holds at most this many live paths
    // (<= kWaveStack - 256; 0: that maximum)
    int32_t queue_threshold;
    // wavefront kernel, indirect-only paths: form a primary ray's antenna field only once
    // it has hit something
    int32_t field_on_hit;
    // wavefront kernel: hand each stage's samples / popped paths to threads grouped by
    // primary sample cell / reflected-direction octant
    int32_t coherent_order;
    // far-field runs (hsr_simulate_batch_ff): each pose's TX and RX;
    // nullptr: the near-field antennas tx/rx above
    const hsr_ff_antenna *ff_tx;
    const hsr_ff_antenna *ff_rx;
    // uniform batch, wavefront kernel: the first double of each pose's 2N accumulators in
    // acc (a serving tick whose requests share scene, chirp and N); nullptr: pose-major rows
    const int64_t *acc_row;
    // guided launches: the guiding-tree slot of each pose in the g_* arrays (a serving
    // tick's requests own trees of the server's pool); nullptr: the pose index
    const int32_t *guide_slot;
};


size_t guide_bytes_per_pose();
int launch_guide_reset(int P, int *samp_child, float *samp_p, int *train_child, float *train_acc, int *train_count,
                       cudaStream_t st);
int launch_guide_step(int P, const int *active, int *samp_child, float *samp_p, int *train_child, float *train_acc,
                      int *train_count, cudaStream_t st);
// longest guided schedule (PathTracer::run iterations) a call may have
constexpr int kGuideMaxIters = 50;
// guiding tree nodes per pose (hsr_guide.cuh)
constexpr int kGuideMaxNodes = 2048;

// Guiding trees for P poses, carved from one allocation.
struct GuideMem {
    int *samp_child;
    float *samp_p;
    int *train_child;
    float *train_acc;
    int *train_count;
    // the whole schedule of a guided call, iteration-major: per iteration budget and
    // Halton offset (int64), sample weight (float), train, clear and active flags (int)
    unsigned char *sched;
};

inline GuideMem carve_guide(void *base, int P) {
    GuideMem g;
    char *p = static_cast<char *>(base);
    size_t off = 0;
    const size_t M = size_t(P) * kGuideMaxNodes;
    auto take = [&](size_t bytes) {
        char *r = p + off;
        off += (bytes + 255) & ~size_t(255);
        return r;
    };
    g.samp_child = reinterpret_cast<int *>(take(4 * M));
    g.samp_p = reinterpret_cast<float *>(take(4 * M));
    g.train_child = reinterpret_cast<int *>(take(4 * M));
    g.train_acc = reinterpret_cast<float *>(take(12 * M));
    g.train_count = reinterpret_cast<int *>(take(4 * size_t(P)));
    g.sched = reinterpret_cast<unsigned char *>(take(size_t(kGuideMaxIters) * 32 * size_t(P)));
    return g;
}


int synth_build_operand(SynthOperand &op, int N, cudaStream_t st, std::string &err);
void synth_free_operand(SynthOperand &op);
size_t synth_scratch_bytes(const SynthOperand &op, int P);
int synth_run(const SynthOperand &op, const double *fine, int P, void *scratch, int engine, const int64_t *budget,
              float sample_weight, const double *tw, int normalise, float *out_rows, unsigned *status, cudaStream_t st,
              std::string &err);
int launch_clear_rows_f(double *rows, int32_t pose_count, int32_t len, const int *clear, cudaStream_t st);
// 0: tensor cores (tcgen05, split BF16); 1: CUDA cores (FP32)
extern int g_synth_engine;

// Launches (all asynchronous on `st`).
int launch_trace(const TraceParams &p, int phase_mode, int splat_mode, int grid, cudaStream_t st, std::string &err);
int launch_tile_prefix(const int64_t *budget, int32_t pose_count, int32_t tile, int64_t *tile_start, cudaStream_t st);
int launch_finalize(const double *acc, int32_t pose_count, int32_t samples, const int64_t *budget, float sample_weight,
                    const double *total_weight, int normalise, float *out_rows, cudaStream_t st);
int launch_clear_rows(double *acc, int32_t pose_count, int32_t samples, const int *clear, cudaStream_t st);
// A MIMO radar cube [chirp][sample][channel] from per-channel rows (hsr_simulate_frame).
int launch_assemble_frame(const float *rows, int32_t chirps, int32_t samples, int32_t channels, float *frame,
                          cudaStream_t st);
// The device Halton sampler at host-chosen indices (hsr_debug_halton).
int launch_debug_halton(const uint64_t *d_index, int64_t count, int dim, float *d_out);
int launch_debug_sincos_sweep(unsigned lo_bits, unsigned hi_bits, unsigned long long *d_counts);
int launch_ray_queries(const DNode *nodes, const DTri *tris, int64_t count, const float *o, const float *d,
                       const float *tfar, float *t, float *p, float *n, int32_t *prim, int32_t *vis, unsigned *status,
                       cudaStream_t st);
int trace_smem_bytes(int samples, int splat_mode, int fine_bins);
size_t wave_smem_bytes(int samples, bool guided);
// The split-phase instantiations of the wavefront kernel (hsr_wave_split.cu).
void launch_wave_split(const TraceParams &p, int grid, cudaStream_t st);
int wave_blocks_per_sm(int samples, bool mixed, bool guided = false);
int launch_wave(const TraceParams &p, int phase_mode, int grid, cudaStream_t st, std::string &err);
// 0: wavefront kernel whenever the flags allow it; 1: always the one-thread-per-sample kernel
extern int g_path_kernel;
// BVH topology of new scenes: 0 = PLOC (default), 1 = LBVH (Karras radix tree)
extern int g_bvh_builder;
extern int g_bvh_leaf_max;
extern int g_bvh_optimize;
int trace_blocks_per_sm(int samples, int splat_mode, int fine_bins);

}  // namespace hsr
