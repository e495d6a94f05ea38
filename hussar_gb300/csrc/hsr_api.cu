// The C ABI (include/hsr_gb300.h): scene residency, ray queries, backend runs, batched
// and guided simulations. Every entry point returns an hsr_status; the message of the
// last failure on the calling thread is available from hsr_last_error(). No exception
// crosses the ABI.
#include <atomic>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "hsr_common.cuh"
#include "hsr_guide.cuh"
#include "hsr_internal.h"

namespace hsr {

static thread_local std::string g_err;
int g_path_kernel = 0;
int g_synth_engine = 0;
static std::atomic<int64_t> g_launches{0};

void note_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
static std::atomic<int64_t> g_allocs{0};
void note_alloc() { g_allocs.fetch_add(1, std::memory_order_relaxed); }

static hsr_status fail(hsr_status s, const std::string &msg) {
    g_err = msg;
    return s;
}

static hsr_status cuda_fail(cudaError_t e, const char *what) {
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) return fail(HSR_ERR_OUT_OF_MEMORY, std::string(what) + ": out of memory");
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return fail(HSR_ERR_NO_DEVICE, std::string(what) + ": " + cudaGetErrorString(e));
    return fail(HSR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

static hsr_status check_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(HSR_ERR_NO_DEVICE, "no CUDA device is visible (this backend has no CPU fallback)");
    }
    return HSR_OK;
}

static hsr_status validate_common(const hsr_rf_config *rf, int32_t samples, const hsr_tracer_flags *fl) {
    if (!rf || !fl) return fail(HSR_ERR_INVALID_ARGUMENT, "null rf or flags");
    if (samples <= 0 || samples > 4096)
        return fail(HSR_ERR_INVALID_ARGUMENT, "samplesPerChirp must be in [1, 4096]");
    if (fl->maxDepth < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "maxDepth must be >= 0");
    return HSR_OK;
}

static hsr_status validate_phase(int32_t phase_mode, int32_t splat_mode) {
    if (phase_mode != HSR_PHASE_REFERENCE_FP32 && phase_mode != HSR_PHASE_SPLIT_FP64)
        return fail(HSR_ERR_INVALID_ARGUMENT, "unknown phase mode");
    if (splat_mode != HSR_SPLAT_DIRICHLET16 && splat_mode != HSR_SPLAT_FINE_SYNTH)
        return fail(HSR_ERR_INVALID_ARGUMENT, "unknown splat mode");
    return HSR_OK;
}

// Per-batch scratch for P poses with N bins, carved from one allocation owned by the scene.
struct Scratch {
    hsr_antenna *tx, *rx;
    hsr_ff_antenna *ff_tx, *ff_rx;  // far-field poses (hsr_simulate_batch_ff)
    bool far_field = false;         // the pass traces ff_tx/ff_rx instead of tx/rx
    int64_t *budget, *offset, *tile_start;
    float *weights;
    int *train, *active, *clear;
    double *tw;
    double *acc;
    double *fine;  // fine-histogram rows (HSR_SPLAT_FINE_SYNTH), P x kFineRowPerBin N FP64 sums
    float *rows;
    unsigned *counters;  // [0] status word, [2..3] 64-bit work counter
    size_t bytes;
};

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static Scratch carve(void *base, int32_t P, int32_t N, bool fine) {
    Scratch s;
    char *p = static_cast<char *>(base);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *r = p ? p + off : nullptr;
        off += align256(bytes);
        return r;
    };
    s.counters = reinterpret_cast<unsigned *>(take(64));
    s.tx = reinterpret_cast<hsr_antenna *>(take(sizeof(hsr_antenna) * P));
    s.rx = reinterpret_cast<hsr_antenna *>(take(sizeof(hsr_antenna) * P));
    s.ff_tx = reinterpret_cast<hsr_ff_antenna *>(take(sizeof(hsr_ff_antenna) * P));
    s.ff_rx = reinterpret_cast<hsr_ff_antenna *>(take(sizeof(hsr_ff_antenna) * P));
    s.budget = reinterpret_cast<int64_t *>(take(sizeof(int64_t) * P));
    s.offset = reinterpret_cast<int64_t *>(take(sizeof(int64_t) * P));
    s.tile_start = reinterpret_cast<int64_t *>(take(sizeof(int64_t) * (P + 1)));
    s.weights = reinterpret_cast<float *>(take(sizeof(float) * P));
    s.train = reinterpret_cast<int *>(take(sizeof(int) * P));
    s.active = reinterpret_cast<int *>(take(sizeof(int) * P));
    s.clear = reinterpret_cast<int *>(take(sizeof(int) * P));
    s.tw = reinterpret_cast<double *>(take(sizeof(double) * P));
    s.acc = reinterpret_cast<double *>(take(sizeof(double) * 2 * size_t(P) * N));
    s.fine = fine ? reinterpret_cast<double *>(take(sizeof(double) * kFineRowPerBin * size_t(P) * N)) : nullptr;
    s.rows = reinterpret_cast<float *>(take(sizeof(float) * 2 * size_t(P) * N));
    s.bytes = off;
    return s;
}

// Carves the scene's scratch for P poses with N bins (growing it when needed) and clears
// the status word on `st`: every call reports the device status of its own work only.
static hsr_status ensure_scratch(SceneDev &sc, int32_t P, int32_t N, Scratch &out, cudaStream_t st,
                                 bool fine = false) {
    Scratch need = carve(nullptr, P, N, fine);
    if (need.bytes > sc.scratch_bytes) {
        if (sc.scratch) {
            cudaDeviceSynchronize();
            cudaFree(sc.scratch);
        }
        sc.scratch = nullptr;
        sc.scratch_bytes = 0;
        std::string err;
        if (!dev_alloc(&sc.scratch, need.bytes, err)) return fail(HSR_ERR_OUT_OF_MEMORY, "scratch allocation: " + err);
        // the status word must start clear; the rest is initialised per call
        cudaError_t e = cudaMemset(sc.scratch, 0, 256);
        if (e != cudaSuccess) return cuda_fail(e, "scratch clear");
        sc.scratch_bytes = need.bytes;
    }
    out = carve(sc.scratch, P, N, fine);
    cudaError_t e = cudaMemsetAsync(out.counters, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return cuda_fail(e, "status clear");
    return HSR_OK;
}

// Twiddle operand for N bins (cached per scene) and the synthesis scratch for P poses.
static hsr_status ensure_synth(SceneDev &sc, int32_t N, int32_t P, cudaStream_t st) {
    if (sc.synth.N != N) {
        cudaDeviceSynchronize();
        synth_free_operand(sc.synth);
        std::string err;
        const int rc = synth_build_operand(sc.synth, N, st, err);
        if (rc != 0) {
            synth_free_operand(sc.synth);
            return fail(rc == 3 ? HSR_ERR_OUT_OF_MEMORY : HSR_ERR_CUDA, err);
        }
    }
    const size_t need = synth_scratch_bytes(sc.synth, P);
    if (need > sc.synth_scratch_bytes) {
        cudaDeviceSynchronize();
        cudaFree(sc.synth_scratch);
        sc.synth_scratch = nullptr;
        sc.synth_scratch_bytes = 0;
        std::string err;
        if (!dev_alloc(&sc.synth_scratch, need, err)) return fail(HSR_ERR_OUT_OF_MEMORY, "synthesis scratch: " + err);
        sc.synth_scratch_bytes = need;
    }
    return HSR_OK;
}

static hsr_status synthesise(SceneDev &sc, const Scratch &s, int32_t P, float sample_weight, const double *tw,
                             int normalise, float *d_out_rows, cudaStream_t st) {
    std::string err;
    if (synth_run(sc.synth, s.fine, P, sc.synth_scratch, g_synth_engine, s.budget, sample_weight, tw, normalise,
                  d_out_rows, s.counters, st, err) != 0)
        return fail(HSR_ERR_CUDA, err);
    return HSR_OK;
}

static hsr_status ensure_guide(SceneDev &sc, int P, GuideMem &out) {
    if (P > sc.guide_cap) {
        if (sc.guide) {
            cudaDeviceSynchronize();
            cudaFree(sc.guide);
        }
        sc.guide = nullptr;
        sc.guide_cap = 0;
        const size_t bytes = guide_bytes_per_pose() * size_t(P) + 8 * 256;
        std::string err;
        if (!dev_alloc(&sc.guide, bytes, err)) return fail(HSR_ERR_OUT_OF_MEMORY, "guiding allocation: " + err);
        sc.guide_cap = P;
    }
    out = carve_guide(sc.guide, P);
    return HSR_OK;
}

static constexpr int32_t kTile = 4096;  // samples per work item

// One trace launch over the poses' current budgets/offsets/weights in scratch.
// `tile` is the samples per work item: 0 takes the scene's autotuned tile (or kTile);
// the guided iterations pass their own (smaller tiles keep the SMs busy when a pass has
// few samples). The autotuned CTAs per SM and queue threshold apply to plain passes.
static hsr_status enqueue_pass(SceneDev &sc, const Scratch &s, const hsr_rf_config *rf, int32_t N,
                               const hsr_tracer_flags *fl, int32_t P, float sample_weight, bool per_pose_weights,
                               int32_t phase_mode, int32_t splat_mode, cudaStream_t st, const GuideMem *g,
                               void *records = nullptr, int max_rec = 0, unsigned long long *counters = nullptr,
                               int32_t tile = 0) {
    const bool tuned = tile == 0 && !fl->doGuiding;
    if (tile == 0) tile = (tuned && sc.tuned.tile > 0) ? sc.tuned.tile : kTile;
    cudaError_t e;
    if ((e = cudaMemsetAsync(s.counters + 2, 0, 8, st)) != cudaSuccess) return cuda_fail(e, "memset counter");
    if (launch_tile_prefix(s.budget, P, tile, s.tile_start, st) != 0)
        return cuda_fail(cudaGetLastError(), "tile prefix launch");
    TraceParams p{};
    p.nodes = sc.nodes;
    p.tris = sc.tris;
    p.rf = *rf;
    p.flags = *fl;
    p.samples = N;
    p.pose_count = P;
    p.tx = s.tx;
    p.rx = s.rx;
    p.budget = s.budget;
    p.offset = s.offset;
    p.tile_start = s.tile_start;
    p.sample_weight = sample_weight;
    p.tile = tile;
    p.acc = s.acc;
    p.status = s.counters;
    p.work_counter = s.counters + 2;
    p.records = records;
    p.max_rec = max_rec;
    p.counters = counters;
    p.weights = per_pose_weights ? s.weights : nullptr;
    p.fine = splat_mode == HSR_SPLAT_FINE_SYNTH ? s.fine : nullptr;
    p.fine_bins = kFineOS * N;
    if (s.far_field) {
        p.ff_tx = s.ff_tx;
        p.ff_rx = s.ff_rx;
    }
    p.do_guide = (fl->doGuiding && g) ? 1 : 0;
    if (p.do_guide) {
        p.train = s.train;
        p.g_samp_child = g->samp_child;
        p.g_samp_p = g->samp_p;
        p.g_train_child = g->train_child;
        p.g_train_acc = g->train_acc;
    } else {
        p.flags.doGuiding = 0;
    }
    const bool wave = g_path_kernel == 0 && fl->useGeometricalOptics && !records && !counters;
    int per_sm = wave ? wave_blocks_per_sm(N, false, p.do_guide != 0) : trace_blocks_per_sm(N, splat_mode, 0);
    if (wave && tuned) {
        if (sc.tuned.ctas_per_sm > 0) per_sm = std::min(per_sm, sc.tuned.ctas_per_sm);
        p.queue_threshold = sc.tuned.queue_threshold;
        p.field_on_hit = sc.tuned.field_on_hit;
        p.coherent_order = sc.tuned.coherent_order;
    }
    int grid = sc.sm_count * per_sm;
    // timing events only outside stream capture (a captured graph must not record the
    // scene's events: it may outlive them)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cap);
    const bool timing = cap == cudaStreamCaptureStatusNone;
    if (timing) cudaEventRecord(sc.ev0, st);
    std::string err;
    if (wave) {
        if (launch_wave(p, phase_mode, grid, st, err) != 0) return fail(HSR_ERR_CUDA, err);
    } else if (launch_trace(p, phase_mode, splat_mode, grid, st, err) != 0) {
        return fail(HSR_ERR_CUDA, err);
    }
    if (timing) {
        cudaEventRecord(sc.ev1, st);
        sc.timing_valid = true;
    }
    return HSR_OK;
}

// Plain run of every pose over its whole budget (doGuiding = 0), then fetchFrame rows.
static hsr_status run_plain(SceneDev &sc, const Scratch &s, const hsr_rf_config *rf, int32_t N,
                            const hsr_tracer_flags *fl, int32_t P, float sample_weight, int32_t phase_mode,
                            int32_t splat_mode, int normalise, float *d_out_rows, cudaStream_t st,
                            void *records = nullptr, int max_rec = 0, unsigned long long *counters = nullptr) {
    cudaError_t e;
    const bool fine = splat_mode == HSR_SPLAT_FINE_SYNTH;
    if (fine) {
        hsr_status r = ensure_synth(sc, N, P, st);
        if (r != HSR_OK) return r;
        if ((e = cudaMemsetAsync(s.fine, 0, sizeof(double) * kFineRowPerBin * size_t(P) * N, st)) != cudaSuccess)
            return cuda_fail(e, "memset fine histogram");
    } else if ((e = cudaMemsetAsync(s.acc, 0, sizeof(double) * 2 * size_t(P) * N, st)) != cudaSuccess) {
        return cuda_fail(e, "memset accumulators");
    }
    hsr_tracer_flags plain = *fl;
    plain.doGuiding = 0;
    hsr_status r = enqueue_pass(sc, s, rf, N, &plain, P, sample_weight, false, phase_mode, splat_mode, st, nullptr,
                                records, max_rec, counters);
    if (r != HSR_OK) return r;
    if (fine) return synthesise(sc, s, P, sample_weight, nullptr, normalise, d_out_rows, st);
    if (launch_finalize(s.acc, P, N, s.budget, sample_weight, nullptr, normalise, d_out_rows, st) != 0)
        return cuda_fail(cudaGetLastError(), "finalize launch");
    return HSR_OK;
}

std::vector<Iter> schedule(int64_t samples, bool clearBeforeIteration) {
    std::vector<Iter> it;
    int64_t milestone = 16384, remaining = samples, offset = 0;
    float weight = 1.f;
    bool final_iter = false, clear = true;
    while (true) {
        milestone = std::min(milestone, remaining);
        it.push_back(Iter{milestone, offset, weight, clear, !final_iter});
        offset += milestone;
        remaining -= milestone;
        if (remaining == 0) break;
        milestone *= 2;
        if (remaining < milestone * 2) {
            final_iter = true;
            milestone = remaining;
        }
        if (clearBeforeIteration) {
            clear = true;
            offset = 0;
        } else {
            clear = false;
            weight = 10.f * weight;
        }
    }
    return it;
}

// The guided schedule for every pose (host budgets); writes fetchFrame rows (normalise)
// or raw sums, and the total weights (h_total_weight, optional).
static hsr_status run_guided(SceneDev &sc, const Scratch &s, const hsr_rf_config *rf, int32_t N,
                             const hsr_tracer_flags *fl, int32_t P, const std::vector<int64_t> &budgets,
                             const std::vector<int64_t> &offsets, int32_t phase_mode, int32_t splat_mode,
                             int normalise, float *d_out_rows, cudaStream_t st, double *h_total_weight,
                             const volatile int32_t *interrupt_flag) {
    GuideMem g;
    hsr_status r = ensure_guide(sc, P, g);
    if (r != HSR_OK) return r;
    std::vector<std::vector<Iter>> sched(P);
    size_t K = 0;
    for (int p = 0; p < P; ++p) {
        sched[p] = schedule(budgets[p], fl->clearBeforeIteration != 0);
        K = std::max(K, sched[p].size());
    }
    cudaError_t e;
    const bool fine = splat_mode == HSR_SPLAT_FINE_SYNTH;
    if (fine) {
        r = ensure_synth(sc, N, P, st);
        if (r != HSR_OK) return r;
        if ((e = cudaMemsetAsync(s.fine, 0, sizeof(double) * kFineRowPerBin * size_t(P) * N, st)) != cudaSuccess)
            return cuda_fail(e, "memset fine histogram");
    } else if ((e = cudaMemsetAsync(s.acc, 0, sizeof(double) * 2 * size_t(P) * N, st)) != cudaSuccess) {
        return cuda_fail(e, "memset accumulators");
    }
    if (launch_guide_reset(P, g.samp_child, g.samp_p, g.train_child, g.train_acc, g.train_count, st) != 0)
        return cuda_fail(cudaGetLastError(), "guide reset");
    if (K > size_t(kGuideMaxIters)) return fail(HSR_ERR_INVALID_ARGUMENT, "guided budget needs too many iterations");
    // every iteration's schedule, uploaded once: the iterations then run back to back
    const size_t it_bytes = 32 * size_t(P);
    std::vector<unsigned char> blk(K * it_bytes);
    std::vector<double> tw(P, 0.0);
    std::vector<char> any_clear(K, 0), any_active(K, 0);
    std::vector<int64_t> iter_samples(K, 0);
    for (size_t k = 0; k < K; ++k) {
        unsigned char *h = blk.data() + k * it_bytes;
        int64_t *b = reinterpret_cast<int64_t *>(h);
        int64_t *o = b + P;
        float *w = reinterpret_cast<float *>(o + P);
        int *train = reinterpret_cast<int *>(w + P);
        int *clear = train + P;
        int *active = clear + P;
        for (int p = 0; p < P; ++p) {
            if (k < sched[p].size()) {
                const Iter &it = sched[p][k];
                b[p] = it.budget;
                // the caller's index offset shifts every iteration's Halton range
                o[p] = it.offset + offsets[p];
                w[p] = it.weight;
                train[p] = it.train ? 1 : 0;
                clear[p] = (k > 0 && it.clear) ? 1 : 0;
                if (it.clear) tw[p] = 0.0;
                tw[p] += double(it.budget) * double(it.weight);  // path.h:445, 466-475
                active[p] = k + 1 < sched[p].size() ? 1 : 0;
                iter_samples[k] += it.budget;
            } else {
                b[p] = 0;
                o[p] = 0;
                w[p] = 0.f;
                train[p] = clear[p] = active[p] = 0;
            }
            any_clear[k] |= clear[p] != 0;
            any_active[k] |= active[p] != 0;
        }
    }
    if ((e = cudaMemcpyAsync(g.sched, blk.data(), blk.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(e, "schedule upload");
    for (size_t k = 0; k < K; ++k) {
        if (interrupt_flag) {
            // honour the flag between iterations (PathTracer::run, path.h:188-189): let the
            // previous iteration finish before looking at it
            if (k > 0 && (e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "guided iteration");
            if (*interrupt_flag) return fail(HSR_ERR_INTERRUPTED, "interrupted between iterations");
        }
        Scratch si = s;
        unsigned char *d = g.sched + k * it_bytes;
        si.budget = reinterpret_cast<int64_t *>(d);
        si.offset = si.budget + P;
        si.weights = reinterpret_cast<float *>(si.offset + P);
        si.train = reinterpret_cast<int *>(si.weights + P);
        si.clear = si.train + P;
        si.active = si.clear + P;
        if (any_clear[k]) {
            const int rc = fine ? launch_clear_rows_f(s.fine, P, kFineRowPerBin * N, si.clear, st)
                                : launch_clear_rows(s.acc, P, N, si.clear, st);
            if (rc != 0) return cuda_fail(cudaGetLastError(), "clear rows");
        }
        // about four work items per resident CTA in this iteration
        const int64_t per_item = (iter_samples[k] + 8 * int64_t(sc.sm_count) - 1) / (8 * int64_t(sc.sm_count));
        int32_t tile = 256;
        while (tile < kTile && tile < per_item) tile *= 2;
        r = enqueue_pass(sc, si, rf, N, fl, P, 1.f, true, phase_mode, splat_mode, st, &g, nullptr, 0, nullptr, tile);
        if (r != HSR_OK) return r;
        if (any_active[k] &&
            launch_guide_step(P, si.active, g.samp_child, g.samp_p, g.train_child, g.train_acc, g.train_count, st) != 0)
            return cuda_fail(cudaGetLastError(), "guide step");
    }
    if ((e = cudaMemcpyAsync(s.tw, tw.data(), 8 * P, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(e, "weight upload");
    if (fine) {
        r = synthesise(sc, s, P, 1.f, s.tw, normalise, d_out_rows, st);
        if (r != HSR_OK) return r;
    } else if (launch_finalize(s.acc, P, N, s.budget, 1.f, s.tw, normalise, d_out_rows, st) != 0) {
        return cuda_fail(cudaGetLastError(), "finalize launch");
    }
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "guided finalize");
    if (h_total_weight)
        for (int p = 0; p < P; ++p) h_total_weight[p] = tw[p];
    return HSR_OK;
}

// The status word's bits as text (kStatus* in hsr_common.cuh; bit 3 from hsr_synth.cu).
std::string status_text(unsigned bits) {
    std::string m = "device status:";
    if (bits & kStatusStackOverflow) m += " traversal-stack-overflow";
    if (bits & kStatusBadBin) m += " bin-out-of-range";
    if (bits & kStatusBadWorkItem) m += " bad-work-item";
    if (bits & (1u << 3)) m += " synthesis-wait-timeout";
    return m;
}

static hsr_status read_status(const Scratch &s, cudaStream_t st) {
    unsigned bits = 0;
    cudaError_t e = cudaMemcpyAsync(&bits, s.counters, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "status read");
    if (bits) {
        cudaMemsetAsync(s.counters, 0, sizeof(unsigned), st);
        cudaStreamSynchronize(st);
        return fail(HSR_ERR_DEVICE, status_text(bits));
    }
    return HSR_OK;
}

static hsr_status upload_poses(const Scratch &s, int32_t P, const hsr_antenna *tx, const hsr_antenna *rx,
                               const int64_t *budget, const int64_t *offset, cudaMemcpyKind kind, cudaStream_t st) {
    cudaError_t e;
    if ((e = cudaMemcpyAsync(s.tx, tx, sizeof(hsr_antenna) * P, kind, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s.rx, rx, sizeof(hsr_antenna) * P, kind, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s.budget, budget, sizeof(int64_t) * P, kind, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s.offset, offset, sizeof(int64_t) * P, kind, st)) != cudaSuccess)
        return cuda_fail(e, "pose upload");
    return HSR_OK;
}

}  // namespace hsr

using namespace hsr;

struct hsr_scene {
    SceneDev dev;
    std::mutex mu;
    std::atomic<int> graphs{0};  // live captured graphs (they hold the BVH's pointers)
};

namespace hsr {
// Read access to a scene's device state, and the calling thread's error message, for
// entry points defined in other translation units.
const SceneDev *scene_device_state(const hsr_scene *s) { return s ? &s->dev : nullptr; }
std::mutex *scene_mutex(hsr_scene *s) { return s ? &s->mu : nullptr; }
void set_last_error(const std::string &msg) { g_err = msg; }
}  // namespace hsr

extern "C" {

int32_t hsr_abi_version(void) { return HSR_ABI_VERSION; }

const char *hsr_last_error(void) { return g_err.c_str(); }

int64_t hsr_launch_count(void) { return g_launches.load(); }

int64_t hsr_debug_alloc_count(void) { return g_allocs.load(); }

hsr_status hsr_scene_status(hsr_scene *s, void *stream, uint32_t *out_bits) {
    if (out_bits) *out_bits = 0;
    if (!s) return fail(HSR_ERR_INVALID_ARGUMENT, "null scene");
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->dev.scratch) return HSR_OK;  // no call has run on this scene yet
    cudaStream_t strm = static_cast<cudaStream_t>(stream);
    unsigned bits = 0;
    cudaError_t e = cudaStreamSynchronize(strm);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, s->dev.scratch, sizeof(unsigned), cudaMemcpyDeviceToHost, strm);
    if (e == cudaSuccess) e = cudaStreamSynchronize(strm);
    if (e != cudaSuccess) return cuda_fail(e, "status read");
    if (out_bits) *out_bits = bits;
    return bits ? fail(HSR_ERR_DEVICE, status_text(bits)) : HSR_OK;
}

void hsr_default_flags(hsr_tracer_flags *f) {
    if (!f) return;
    f->onlyIndirect = 1;
    f->maxDepth = 10;
    f->useGeometricalOptics = 1;
    f->poDiffraction = 0;
    f->doGuiding = 1;
    f->clearBeforeIteration = 1;
    f->correctPhase = 0;
    f->filterGuiding = 1;
    f->doFiltering = 1;
    f->filteringSphere = 1;
    f->produceDebugImage = 0;
    f->filteringMin = 600.f;
    f->filteringMax = 900.f;
    f->filteringRadius = 160.f;
}

hsr_status hsr_scene_create(const float *vertices, int64_t vertex_count, const int32_t *indices,
                            int64_t triangle_count, hsr_scene **out_scene) {
    if (!out_scene) return fail(HSR_ERR_INVALID_ARGUMENT, "out_scene is null");
    *out_scene = nullptr;
    if (vertex_count < 0 || triangle_count < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "negative count");
    if ((vertex_count > 0 && !vertices) || (triangle_count > 0 && !indices))
        return fail(HSR_ERR_INVALID_ARGUMENT, "null vertex or index array");
    if (triangle_count > (int64_t(1) << 30)) return fail(HSR_ERR_INVALID_ARGUMENT, "more than 2^30 triangles");
    for (int64_t i = 0; i < 3 * triangle_count; ++i)
        if (indices[i] < 0 || indices[i] >= vertex_count)
            return fail(HSR_ERR_INVALID_ARGUMENT,
                        "triangle " + std::to_string(i / 3) + " references vertex " + std::to_string(indices[i]) +
                            " outside [0, " + std::to_string(vertex_count) + ")");
    hsr_status st = check_device();
    if (st != HSR_OK) return st;
    hsr_scene *s = new hsr_scene;
    SceneDev &d = s->dev;
    cudaGetDevice(&d.device);
    cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, d.device);
    float *dv = nullptr;
    int32_t *di = nullptr;
    std::string err;
    cudaError_t e;
    if (!dev_alloc(&dv, sizeof(float) * 3 * std::max<int64_t>(vertex_count, 1), err) ||
        !dev_alloc(&di, sizeof(int32_t) * 3 * std::max<int64_t>(triangle_count, 1), err)) {
        cudaFree(dv);
        delete s;
        return fail(HSR_ERR_OUT_OF_MEMORY, err);
    }
    if (vertex_count) {
        e = cudaMemcpy(dv, vertices, sizeof(float) * 3 * vertex_count, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(dv);
            cudaFree(di);
            delete s;
            return cuda_fail(e, "vertex upload");
        }
    }
    if (triangle_count) {
        e = cudaMemcpy(di, indices, sizeof(int32_t) * 3 * triangle_count, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(dv);
            cudaFree(di);
            delete s;
            return cuda_fail(e, "index upload");
        }
    }
    int rc = bvh_build(d, dv, vertex_count, di, triangle_count, 0, err);
    cudaFree(dv);
    d.indices = di;  // kept for refits
    d.vertex_count = vertex_count;
    if (rc != 0) {
        cudaFree(d.tris);
        cudaFree(d.nodes);
        cudaFree(d.indices);
        delete s;
        return fail(rc == 3 ? HSR_ERR_OUT_OF_MEMORY : rc == 4 ? HSR_ERR_INVALID_ARGUMENT : HSR_ERR_CUDA, err);
    }
    cudaEventCreate(&d.ev0);
    cudaEventCreate(&d.ev1);
    *out_scene = s;
    return HSR_OK;
}

hsr_status hsr_scene_destroy(hsr_scene *s) {
    if (!s) return HSR_OK;
    cudaDeviceSynchronize();
    cudaFree(s->dev.tris);
    cudaFree(s->dev.nodes);
    cudaFree(s->dev.indices);
    cudaFree(s->dev.refit_order);
    cudaFree(s->dev.scratch);
    cudaFree(s->dev.guide);
    synth_free_operand(s->dev.synth);
    cudaFree(s->dev.synth_scratch);
    cudaFree(s->dev.frame_buf);
    if (s->dev.ev0) cudaEventDestroy(s->dev.ev0);
    if (s->dev.ev1) cudaEventDestroy(s->dev.ev1);
    delete s;
    return HSR_OK;
}

hsr_status hsr_scene_refit(hsr_scene *s, const float *vertices, int64_t vertex_count) {
    if (!s || (vertex_count > 0 && !vertices)) return fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    if (vertex_count != s->dev.vertex_count)
        return fail(HSR_ERR_INVALID_ARGUMENT, "refit needs the scene's " + std::to_string(s->dev.vertex_count) +
                                                  " vertices, got " + std::to_string(vertex_count));
    for (int64_t i = 0; i < 3 * vertex_count; ++i)
        if (!std::isfinite(vertices[i]))
            return fail(HSR_ERR_INVALID_ARGUMENT, "vertex " + std::to_string(i / 3) + " is not finite");
    hsr_status st = check_device();
    if (st != HSR_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != s->dev.device) return fail(HSR_ERR_INVALID_ARGUMENT, "the scene lives on another device");
    float *dv = nullptr;
    std::string err;
    if (!dev_alloc(&dv, sizeof(float) * 3 * std::max<int64_t>(vertex_count, 1), err))
        return fail(HSR_ERR_OUT_OF_MEMORY, err);
    cudaError_t e = cudaDeviceSynchronize();  // no call on the scene is still reading its BVH
    if (e == cudaSuccess && vertex_count)
        e = cudaMemcpy(dv, vertices, sizeof(float) * 3 * vertex_count, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(dv);
        return cuda_fail(e, "vertex upload");
    }
    const int rc = bvh_refit(s->dev, dv, 0, err);
    cudaFree(dv);
    if (rc != 0) return fail(rc == 3 ? HSR_ERR_OUT_OF_MEMORY : HSR_ERR_CUDA, err);
    return HSR_OK;
}

hsr_status hsr_scene_rebuild(hsr_scene *s, const float *vertices, int64_t vertex_count, const int32_t *indices,
                             int64_t triangle_count) {
    if (!s) return fail(HSR_ERR_INVALID_ARGUMENT, "null scene");
    if (s->graphs.load() > 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "the scene has captured graphs (they hold its BVH): destroy them first");
    // a new scene with the same handle: built aside, then swapped in under the scene lock
    hsr_scene *fresh = nullptr;
    hsr_status st = hsr_scene_create(vertices, vertex_count, indices, triangle_count, &fresh);
    if (st != HSR_OK) return st;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (fresh->dev.device != s->dev.device) {
            hsr_scene_destroy(fresh);
            return fail(HSR_ERR_INVALID_ARGUMENT, "the scene lives on another device");
        }
        cudaDeviceSynchronize();  // no call on the scene is still reading its BVH
        SceneDev &a = s->dev, &b = fresh->dev;
        std::swap(a.tri_count, b.tri_count);
        std::swap(a.node_count, b.node_count);
        std::swap(a.leaf_count, b.leaf_count);
        std::swap(a.max_depth, b.max_depth);
        std::swap(a.tris, b.tris);
        std::swap(a.nodes, b.nodes);
        std::swap(a.indices, b.indices);
        std::swap(a.vertex_count, b.vertex_count);
        std::swap(a.refit_order, b.refit_order);
        std::swap(a.refit_levels, b.refit_levels);
    }
    return hsr_scene_destroy(fresh);  // frees the old BVH, now held by `fresh`
}

hsr_status hsr_scene_footprint(const hsr_scene *s, int64_t *out_bytes) {
    if (!s || !out_bytes) return fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    *out_bytes = int64_t(sizeof(DTri) + 3 * sizeof(int32_t)) * std::max<int64_t>(s->dev.tri_count, 1) +
                 int64_t(sizeof(DNode)) * s->dev.node_count + int64_t(s->dev.scratch_bytes) +
                 int64_t(guide_bytes_per_pose()) * s->dev.guide_cap;
    return HSR_OK;
}

hsr_status hsr_debug_bvh(const hsr_scene *s, void *out_nodes, int64_t node_capacity, void *out_tris,
                         int64_t tri_capacity) {
    if (!s) return fail(HSR_ERR_INVALID_ARGUMENT, "null scene");
    if ((out_nodes && node_capacity < s->dev.node_count) || (out_tris && tri_capacity < s->dev.tri_count))
        return fail(HSR_ERR_INVALID_ARGUMENT, "output capacity below the scene's node or triangle count");
    cudaError_t e = cudaSuccess;
    if (out_nodes)
        e = cudaMemcpy(out_nodes, s->dev.nodes, sizeof(DNode) * size_t(s->dev.node_count), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && out_tris && s->dev.tri_count)
        e = cudaMemcpy(out_tris, s->dev.tris, sizeof(DTri) * size_t(s->dev.tri_count), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? HSR_OK : cuda_fail(e, "BVH copy");
}

hsr_status hsr_debug_halton(const uint64_t *index, int64_t count, int32_t dim, float *out) {
    if (count < 0 || dim < 0 || (count > 0 && (!index || !out))) return fail(HSR_ERR_INVALID_ARGUMENT, "bad arguments");
    hsr_status r = check_device();
    if (r != HSR_OK || count == 0) return r;
    uint64_t *d_index = nullptr;
    std::string err;
    if (!dev_alloc(&d_index, (sizeof(uint64_t) + sizeof(float)) * size_t(count), err))
        return fail(HSR_ERR_OUT_OF_MEMORY, err);
    float *d_out = reinterpret_cast<float *>(d_index + count);
    cudaError_t e = cudaMemcpy(d_index, index, sizeof(uint64_t) * size_t(count), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && launch_debug_halton(d_index, count, dim, d_out) != 0) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, sizeof(float) * size_t(count), cudaMemcpyDeviceToHost);
    cudaFree(d_index);
    return e == cudaSuccess ? HSR_OK : cuda_fail(e, "halton");
}

hsr_status hsr_debug_sincos_sweep(float lo, float hi, int64_t *out_checked, int64_t *out_mismatches,
                                  int64_t *out_slow) {
    if (!(lo >= 0.f) || !(hi >= lo) || !(hi <= 3.0e38f) || !out_checked || !out_mismatches || !out_slow)
        return fail(HSR_ERR_INVALID_ARGUMENT, "bad arguments");
    hsr_status r = check_device();
    if (r != HSR_OK) return r;
    unsigned long long *d_counts = nullptr;
    std::string err;
    if (!dev_alloc(&d_counts, 3 * sizeof(unsigned long long), err)) return fail(HSR_ERR_OUT_OF_MEMORY, err);
    unsigned lo_bits, hi_bits;
    memcpy(&lo_bits, &lo, 4);
    memcpy(&hi_bits, &hi, 4);
    unsigned long long h[3] = {0, 0, 0};
    cudaError_t e = cudaMemset(d_counts, 0, sizeof(h));
    if (e == cudaSuccess && launch_debug_sincos_sweep(lo_bits, hi_bits, d_counts) != 0) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(h, d_counts, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d_counts);
    if (e != cudaSuccess) return cuda_fail(e, "sincos sweep");
    *out_checked = int64_t(h[0]);
    *out_mismatches = int64_t(h[1]);
    *out_slow = int64_t(h[2]);
    return HSR_OK;
}

hsr_status hsr_scene_bvh_stats(const hsr_scene *s, int64_t *out_nodes, int32_t *out_max_depth, int64_t *out_leaves) {
    if (!s) return fail(HSR_ERR_INVALID_ARGUMENT, "null scene");
    if (out_nodes) *out_nodes = s->dev.node_count;
    if (out_max_depth) *out_max_depth = s->dev.max_depth;
    if (out_leaves) *out_leaves = s->dev.leaf_count;
    return HSR_OK;
}

static hsr_status ray_queries(const hsr_scene *s, int64_t count, const float *o, const float *d, const float *tfar,
                              float *t, float *p, float *n, int32_t *prim, int32_t *vis) {
    if (!s || count < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "bad scene or count");
    if (count == 0) return HSR_OK;
    if (!o || !d || !tfar) return fail(HSR_ERR_INVALID_ARGUMENT, "null ray arrays");
    // layout (floats per ray): origin 3, direction 3, tfar 1, t 1, hit point 3, normal 3, prim/visible 1
    float *buf = nullptr;
    size_t fl = size_t(count) * 15;
    std::string err;
    if (!dev_alloc(&buf, sizeof(float) * fl + sizeof(unsigned) * 4, err)) return fail(HSR_ERR_OUT_OF_MEMORY, err);
    float *d_o = buf, *d_d = buf + 3 * count, *d_tf = buf + 6 * count, *d_t = buf + 7 * count;
    float *d_p = buf + 8 * count, *d_n = buf + 11 * count;
    int32_t *d_pr = reinterpret_cast<int32_t *>(buf + 14 * count);
    unsigned *d_status = reinterpret_cast<unsigned *>(buf + fl);
    cudaMemset(d_status, 0, sizeof(unsigned));
    cudaMemcpy(d_o, o, sizeof(float) * 3 * count, cudaMemcpyHostToDevice);
    cudaMemcpy(d_d, d, sizeof(float) * 3 * count, cudaMemcpyHostToDevice);
    cudaMemcpy(d_tf, tfar, sizeof(float) * count, cudaMemcpyHostToDevice);
    int rc = launch_ray_queries(s->dev.nodes, s->dev.tris, count, d_o, d_d, d_tf, d_t, d_p, d_n, d_pr,
                                vis ? d_pr : nullptr, d_status, 0);
    cudaError_t e = cudaDeviceSynchronize();
    if (rc != 0 || e != cudaSuccess) {
        cudaFree(buf);
        return cuda_fail(e != cudaSuccess ? e : cudaGetLastError(), "ray query");
    }
    if (vis) {
        cudaMemcpy(vis, d_pr, sizeof(int32_t) * count, cudaMemcpyDeviceToHost);
    } else {
        if (t) cudaMemcpy(t, d_t, sizeof(float) * count, cudaMemcpyDeviceToHost);
        if (p) cudaMemcpy(p, d_p, sizeof(float) * 3 * count, cudaMemcpyDeviceToHost);
        if (n) cudaMemcpy(n, d_n, sizeof(float) * 3 * count, cudaMemcpyDeviceToHost);
        if (prim) cudaMemcpy(prim, d_pr, sizeof(int32_t) * count, cudaMemcpyDeviceToHost);
    }
    unsigned bits = 0;
    cudaMemcpy(&bits, d_status, sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (bits) return fail(HSR_ERR_DEVICE, "device status: traversal-stack-overflow");
    return HSR_OK;
}

hsr_status hsr_intersect(const hsr_scene *s, int64_t count, const float *o, const float *d, const float *tfar,
                         float *t, float *p, float *n, int32_t *prim) {
    return ray_queries(s, count, o, d, tfar, t, p, n, prim, nullptr);
}

hsr_status hsr_visible(const hsr_scene *s, int64_t count, const float *o, const float *d, const float *tfar,
                       int32_t *vis) {
    if (!vis) return fail(HSR_ERR_INVALID_ARGUMENT, "null output");
    return ray_queries(s, count, o, d, tfar, nullptr, nullptr, nullptr, nullptr, vis);
}

hsr_status hsr_debug_records(hsr_scene *s, const hsr_rf_config *rf, int32_t samples, const hsr_tracer_flags *fl,
                             const hsr_antenna *tx, const hsr_antenna *rx, int64_t budget, int64_t index_offset,
                             int32_t max_rec, void *records) {
    hsr_status st = validate_common(rf, samples, fl);
    if (st != HSR_OK) return st;
    if (!s || !tx || !rx || !records || budget <= 0 || max_rec <= 0 || budget > (int64_t(1) << 22))
        return fail(HSR_ERR_INVALID_ARGUMENT, "bad record request");
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    if ((st = ensure_scratch(s->dev, 1, samples, sc, 0)) != HSR_OK) return st;
    const size_t rec_bytes = size_t(budget) * max_rec * 36;
    void *d_rec = nullptr;
    std::string err;
    if (!dev_alloc(&d_rec, rec_bytes, err)) return fail(HSR_ERR_OUT_OF_MEMORY, err);
    std::vector<int32_t> init(rec_bytes / 4, 0);  // unused slots: depth = -1
    for (size_t i = 0; i < init.size(); i += 9) init[i] = -1;
    cudaMemcpy(d_rec, init.data(), rec_bytes, cudaMemcpyHostToDevice);
    if ((st = upload_poses(sc, 1, tx, rx, &budget, &index_offset, cudaMemcpyHostToDevice, 0)) != HSR_OK) {
        cudaFree(d_rec);
        return st;
    }
    st = run_plain(s->dev, sc, rf, samples, fl, 1, 1.f, HSR_PHASE_REFERENCE_FP32, HSR_SPLAT_DIRICHLET16, 0, sc.rows,
                   0, d_rec, max_rec);
    if (st == HSR_OK) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) st = cuda_fail(e, "record run");
    }
    if (st == HSR_OK) cudaMemcpy(records, d_rec, rec_bytes, cudaMemcpyDeviceToHost);
    cudaFree(d_rec);
    if (st == HSR_OK) st = read_status(sc, 0);
    return st;
}

hsr_status hsr_backend_run(const hsr_scene *cs, const hsr_rf_config *rf, const hsr_frame_config *frame,
                           const hsr_antenna *tx, const hsr_antenna *rx, const hsr_tracer_flags *fl, int64_t budget,
                           int64_t index_offset, float sample_weight, int32_t phase_mode, float *frame_inout,
                           double *total_weight_inout, const volatile int32_t *interrupt_flag) {
    hsr_scene *s = const_cast<hsr_scene *>(cs);
    if (!s || !frame || !tx || !rx || !frame_inout || !total_weight_inout)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    if (frame->chirpCount <= 0 || frame->samplesPerChirp <= 0 || frame->channelCount <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "frame dimensions must be positive");
    hsr_status st = validate_common(rf, frame->samplesPerChirp, fl);
    if (st != HSR_OK) return st;
    if (fl->doGuiding)
        return fail(HSR_ERR_NOT_SUPPORTED,
                    "a guided backend run needs the sampling tree of the schedule: use hsr_path_tracer_run");
    if (budget < 0 || index_offset < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "negative budget or offset");
    if ((st = validate_phase(phase_mode, HSR_SPLAT_DIRICHLET16)) != HSR_OK) return st;
    if (interrupt_flag && *interrupt_flag) return fail(HSR_ERR_INTERRUPTED, "interrupted before start");
    if (budget == 0) return HSR_OK;
    const int32_t N = frame->samplesPerChirp;
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    cudaStream_t strm = 0;
    if ((st = ensure_scratch(s->dev, 1, N, sc, strm)) != HSR_OK) return st;
    if ((st = upload_poses(sc, 1, tx, rx, &budget, &index_offset, cudaMemcpyHostToDevice, strm)) != HSR_OK) return st;
    st = run_plain(s->dev, sc, rf, N, fl, 1, sample_weight, phase_mode, HSR_SPLAT_DIRICHLET16, 0, sc.rows, strm);
    if (st != HSR_OK) return st;
    std::vector<float> row(2 * size_t(N));
    cudaError_t e;
    if ((e = cudaMemcpyAsync(row.data(), sc.rows, sizeof(float) * 2 * N, cudaMemcpyDeviceToHost, strm)) !=
        cudaSuccess)
        return cuda_fail(e, "row download");
    if ((e = cudaStreamSynchronize(strm)) != cudaSuccess) return cuda_fail(e, "backend run");
    if ((st = read_status(sc, strm)) != HSR_OK) return st;
    // the reference writes only chirp 0 / channel 0 (path.h:130, 291-292)
    const int C = frame->channelCount;
    for (int32_t k = 0; k < N; ++k) {
        size_t id = size_t(k) * C;
        frame_inout[2 * id] += row[2 * k];
        frame_inout[2 * id + 1] += row[2 * k + 1];
    }
    double w = 0;
    for (int64_t i = 0; i < budget; ++i) w += double(sample_weight);
    *total_weight_inout += w;
    return HSR_OK;
}

// ---- the guiding tree of one pose, for guided backend runs -------------------------
struct hsr_guide {
    hsr_scene *scene = nullptr;
    void *mem = nullptr;
    GuideMem g;
    int *active = nullptr;  // device int 1: the step's "this pose continues" flag
};

hsr_status hsr_guide_create(hsr_scene *s, hsr_guide **out) {
    if (!out) return fail(HSR_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    if (!s) return fail(HSR_ERR_INVALID_ARGUMENT, "null scene");
    hsr_status st = check_device();
    if (st != HSR_OK) return st;
    std::unique_ptr<hsr_guide> g(new hsr_guide());
    g->scene = s;
    std::string err;
    if (!dev_alloc(&g->mem, guide_bytes_per_pose() + 8 * 256, err) || !dev_alloc(&g->active, 256, err)) {
        cudaFree(g->mem);
        return fail(HSR_ERR_OUT_OF_MEMORY, "guiding tree: " + err);
    }
    g->g = carve_guide(g->mem, 1);
    const int one = 1;
    cudaError_t e = cudaMemcpy(g->active, &one, sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess &&
        launch_guide_reset(1, g->g.samp_child, g->g.samp_p, g->g.train_child, g->g.train_acc, g->g.train_count, 0) != 0)
        e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        cudaFree(g->mem);
        cudaFree(g->active);
        return cuda_fail(e, "guiding tree reset");
    }
    *out = g.release();
    return HSR_OK;
}

hsr_status hsr_guide_reset(hsr_guide *g) {
    if (!g) return fail(HSR_ERR_INVALID_ARGUMENT, "null guide");
    if (launch_guide_reset(1, g->g.samp_child, g->g.samp_p, g->g.train_child, g->g.train_acc, g->g.train_count, 0) !=
        0)
        return cuda_fail(cudaGetLastError(), "guide reset");
    cudaError_t e = cudaStreamSynchronize(0);
    return e == cudaSuccess ? HSR_OK : cuda_fail(e, "guide reset");
}

hsr_status hsr_guide_step(hsr_guide *g) {
    if (!g) return fail(HSR_ERR_INVALID_ARGUMENT, "null guide");
    if (launch_guide_step(1, g->active, g->g.samp_child, g->g.samp_p, g->g.train_child, g->g.train_acc,
                          g->g.train_count, 0) != 0)
        return cuda_fail(cudaGetLastError(), "guide step");
    cudaError_t e = cudaStreamSynchronize(0);
    return e == cudaSuccess ? HSR_OK : cuda_fail(e, "guide step");
}

hsr_status hsr_guide_read(hsr_guide *g, int32_t *out_count, int32_t *samp_child, float *samp_p,
                          int32_t *train_child, float *train_acc2) {
    if (!g || !out_count || !samp_child || !samp_p || !train_child || !train_acc2)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<float> acc(3 * size_t(kGuideMaxNodes));
    int count = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(samp_child, g->g.samp_child, 4 * size_t(kGuideMaxNodes), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(samp_p, g->g.samp_p, 4 * size_t(kGuideMaxNodes), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(train_child, g->g.train_child, 4 * size_t(kGuideMaxNodes), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(acc.data(), g->g.train_acc, 4 * acc.size(), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&count, g->g.train_count, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "guide read");
    for (int i = 0; i < kGuideMaxNodes; ++i) train_acc2[i] = acc[3 * size_t(i) + 2];
    *out_count = count;
    return HSR_OK;
}

hsr_status hsr_guide_write(hsr_guide *g, int32_t count, const int32_t *samp_child, const float *samp_p,
                           const int32_t *train_child, const float *train_acc2) {
    if (!g || !samp_child || !samp_p || !train_child || !train_acc2)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    if (count < 1 || count > kGuideMaxNodes)
        return fail(HSR_ERR_INVALID_ARGUMENT, "node count outside 1.." + std::to_string(kGuideMaxNodes));
    // every link must name a child pair inside the array: the device descents and the
    // step index through them
    for (int i = 0; i < kGuideMaxNodes; ++i)
        if (samp_child[i] < -1 || samp_child[i] + 1 >= kGuideMaxNodes || (samp_child[i] >= 0 && samp_child[i] <= i) ||
            train_child[i] < -1 || train_child[i] + 1 >= kGuideMaxNodes ||
            (train_child[i] >= 0 && train_child[i] <= i))
            return fail(HSR_ERR_INVALID_ARGUMENT, "node " + std::to_string(i) + ": child link out of range");
    std::vector<float> acc(3 * size_t(kGuideMaxNodes), 0.f);
    for (int i = 0; i < kGuideMaxNodes; ++i) acc[3 * size_t(i) + 2] = train_acc2[i];
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(g->g.samp_child, samp_child, 4 * size_t(kGuideMaxNodes), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(g->g.samp_p, samp_p, 4 * size_t(kGuideMaxNodes), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(g->g.train_child, train_child, 4 * size_t(kGuideMaxNodes), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(g->g.train_acc, acc.data(), 4 * acc.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(g->g.train_count, &count, sizeof(int), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? HSR_OK : cuda_fail(e, "guide write");
}

hsr_status hsr_guide_destroy(hsr_guide *g) {
    if (!g) return HSR_OK;
    cudaDeviceSynchronize();
    cudaFree(g->mem);
    cudaFree(g->active);
    delete g;
    return HSR_OK;
}

hsr_status hsr_backend_run_guided(hsr_scene *s, const hsr_rf_config *rf, const hsr_frame_config *frame,
                                  const hsr_antenna *tx, const hsr_antenna *rx, const hsr_tracer_flags *fl,
                                  int64_t budget, int64_t index_offset, float sample_weight, int32_t train,
                                  hsr_guide *guide, int32_t phase_mode, float *frame_inout,
                                  double *total_weight_inout, const volatile int32_t *interrupt_flag) {
    if (!s || !frame || !tx || !rx || !guide || !frame_inout || !total_weight_inout)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    if (guide->scene != s) return fail(HSR_ERR_INVALID_ARGUMENT, "the guide belongs to another scene");
    if (frame->chirpCount <= 0 || frame->samplesPerChirp <= 0 || frame->channelCount <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "frame dimensions must be positive");
    hsr_status st = validate_common(rf, frame->samplesPerChirp, fl);
    if (st != HSR_OK) return st;
    if (budget < 0 || index_offset < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "negative budget or offset");
    if ((st = validate_phase(phase_mode, HSR_SPLAT_DIRICHLET16)) != HSR_OK) return st;
    if (interrupt_flag && *interrupt_flag) return fail(HSR_ERR_INTERRUPTED, "interrupted before start");
    if (budget == 0) return HSR_OK;
    const int32_t N = frame->samplesPerChirp;
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    cudaStream_t strm = 0;
    if ((st = ensure_scratch(s->dev, 1, N, sc, strm)) != HSR_OK) return st;
    if ((st = upload_poses(sc, 1, tx, rx, &budget, &index_offset, cudaMemcpyHostToDevice, strm)) != HSR_OK) return st;
    cudaError_t e;
    const int tr = train ? 1 : 0;
    if ((e = cudaMemcpyAsync(sc.train, &tr, sizeof(int), cudaMemcpyHostToDevice, strm)) != cudaSuccess ||
        (e = cudaMemsetAsync(sc.acc, 0, sizeof(double) * 2 * size_t(N), strm)) != cudaSuccess)
        return cuda_fail(e, "guided run set-up");
    hsr_tracer_flags g = *fl;
    g.doGuiding = 1;
    // about four work items per resident CTA, as the guided schedule's iterations use
    const int64_t per_item = (budget + 8 * int64_t(s->dev.sm_count) - 1) / (8 * int64_t(s->dev.sm_count));
    int32_t tile = 256;
    while (tile < kTile && tile < per_item) tile *= 2;
    if ((st = enqueue_pass(s->dev, sc, rf, N, &g, 1, sample_weight, false, phase_mode, HSR_SPLAT_DIRICHLET16, strm,
                           &guide->g, nullptr, 0, nullptr, tile)) != HSR_OK)
        return st;
    if (launch_finalize(sc.acc, 1, N, sc.budget, sample_weight, nullptr, 0, sc.rows, strm) != 0)
        return cuda_fail(cudaGetLastError(), "finalize launch");
    std::vector<float> row(2 * size_t(N));
    if ((e = cudaMemcpyAsync(row.data(), sc.rows, sizeof(float) * 2 * N, cudaMemcpyDeviceToHost, strm)) !=
        cudaSuccess)
        return cuda_fail(e, "row download");
    if ((e = cudaStreamSynchronize(strm)) != cudaSuccess) return cuda_fail(e, "guided backend run");
    if ((st = read_status(sc, strm)) != HSR_OK) return st;
    const int C = frame->channelCount;
    for (int32_t k = 0; k < N; ++k) {
        size_t id = size_t(k) * C;
        frame_inout[2 * id] += row[2 * k];
        frame_inout[2 * id + 1] += row[2 * k + 1];
    }
    double w = 0;
    for (int64_t i = 0; i < budget; ++i) w += double(sample_weight);
    *total_weight_inout += w;
    return HSR_OK;
}

hsr_status hsr_path_tracer_run(hsr_scene *s, const hsr_rf_config *rf, const hsr_frame_config *frame,
                               const hsr_antenna *tx, const hsr_antenna *rx, const hsr_tracer_flags *fl,
                               int64_t samples, int32_t phase_mode, float *frame_out, double *total_weight_out,
                               const volatile int32_t *interrupt_flag) {
    if (!s || !frame || !tx || !rx || !frame_out || !total_weight_out)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    if (frame->chirpCount <= 0 || frame->samplesPerChirp <= 0 || frame->channelCount <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "frame dimensions must be positive");
    hsr_status st = validate_common(rf, frame->samplesPerChirp, fl);
    if (st != HSR_OK) return st;
    if (samples < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "negative sample count");
    if ((st = validate_phase(phase_mode, HSR_SPLAT_DIRICHLET16)) != HSR_OK) return st;
    const size_t n = size_t(frame->chirpCount) * frame->samplesPerChirp * frame->channelCount;
    std::memset(frame_out, 0, sizeof(float) * 2 * n);  // clearFrame (path.h:174)
    *total_weight_out = 0.0;
    if (interrupt_flag && *interrupt_flag) return fail(HSR_ERR_INTERRUPTED, "interrupted before start");
    if (!fl->doGuiding) {
        return hsr_backend_run(s, rf, frame, tx, rx, fl, samples, 0, 1.f, phase_mode, frame_out, total_weight_out,
                               interrupt_flag);
    }
    const int32_t N = frame->samplesPerChirp;
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    cudaStream_t strm = 0;
    if ((st = ensure_scratch(s->dev, 1, N, sc, strm)) != HSR_OK) return st;
    int64_t zero = 0;
    if ((st = upload_poses(sc, 1, tx, rx, &samples, &zero, cudaMemcpyHostToDevice, strm)) != HSR_OK) return st;
    double tw = 0.0;
    st = run_guided(s->dev, sc, rf, N, fl, 1, std::vector<int64_t>{samples}, std::vector<int64_t>{0}, phase_mode,
                    HSR_SPLAT_DIRICHLET16, 0, sc.rows, strm, &tw, interrupt_flag);
    if (st != HSR_OK) return st;
    std::vector<float> row(2 * size_t(N));
    cudaError_t e;
    if ((e = cudaMemcpyAsync(row.data(), sc.rows, sizeof(float) * 2 * N, cudaMemcpyDeviceToHost, strm)) !=
        cudaSuccess)
        return cuda_fail(e, "row download");
    if ((e = cudaStreamSynchronize(strm)) != cudaSuccess) return cuda_fail(e, "guided run");
    if ((st = read_status(sc, strm)) != HSR_OK) return st;
    const int C = frame->channelCount;
    for (int32_t k = 0; k < N; ++k) {
        size_t id = size_t(k) * C;
        frame_out[2 * id] = row[2 * k];
        frame_out[2 * id + 1] = row[2 * k + 1];
    }
    *total_weight_out = tw;
    return HSR_OK;
}

hsr_status hsr_simulate_batch_device(hsr_scene *s, const hsr_rf_config *rf, int32_t N, const hsr_tracer_flags *fl,
                                     int32_t P, const hsr_antenna *d_tx, const hsr_antenna *d_rx,
                                     const int64_t *d_budget, const int64_t *d_offset, int32_t phase_mode,
                                     int32_t splat_mode, float *d_out_rows, void *stream) {
    if (!s || !d_tx || !d_rx || !d_budget || !d_offset || !d_out_rows || P <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument or no poses");
    hsr_status st = validate_common(rf, N, fl);
    if (st != HSR_OK) return st;
    if ((st = validate_phase(phase_mode, splat_mode)) != HSR_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    cudaStream_t strm = static_cast<cudaStream_t>(stream);
    if ((st = ensure_scratch(s->dev, P, N, sc, strm, splat_mode == HSR_SPLAT_FINE_SYNTH)) != HSR_OK) return st;
    if ((st = upload_poses(sc, P, d_tx, d_rx, d_budget, d_offset, cudaMemcpyDeviceToDevice, strm)) != HSR_OK)
        return st;
    if (!fl->doGuiding)
        return run_plain(s->dev, sc, rf, N, fl, P, 1.f, phase_mode, splat_mode, 1, d_out_rows, strm);
    // the guided schedule is planned on the host: it reads the budgets back (synchronising)
    std::vector<int64_t> b(P), o(P);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(b.data(), d_budget, 8 * P, cudaMemcpyDeviceToHost, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(o.data(), d_offset, 8 * P, cudaMemcpyDeviceToHost, strm)) != cudaSuccess ||
        (e = cudaStreamSynchronize(strm)) != cudaSuccess)
        return cuda_fail(e, "budget read-back");
    return run_guided(s->dev, sc, rf, N, fl, P, b, o, phase_mode, splat_mode, 1, d_out_rows, strm, nullptr, nullptr);
}

hsr_status hsr_simulate_batch(hsr_scene *s, const hsr_rf_config *rf, int32_t N, const hsr_tracer_flags *fl, int32_t P,
                              const hsr_antenna *tx, const hsr_antenna *rx, const int64_t *budget,
                              const int64_t *offset, int32_t phase_mode, int32_t splat_mode, float *out_rows,
                              void *stream) {
    if (!s || !tx || !rx || !budget || !offset || !out_rows || P <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument or no poses");
    hsr_status st = validate_common(rf, N, fl);
    if (st != HSR_OK) return st;
    for (int32_t i = 0; i < P; ++i)
        if (budget[i] < 0 || offset[i] < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "negative budget or offset");
    if ((st = validate_phase(phase_mode, splat_mode)) != HSR_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    cudaStream_t strm = static_cast<cudaStream_t>(stream);
    if ((st = ensure_scratch(s->dev, P, N, sc, strm, splat_mode == HSR_SPLAT_FINE_SYNTH)) != HSR_OK) return st;
    if ((st = upload_poses(sc, P, tx, rx, budget, offset, cudaMemcpyHostToDevice, strm)) != HSR_OK) return st;
    if (!fl->doGuiding) {
        st = run_plain(s->dev, sc, rf, N, fl, P, 1.f, phase_mode, splat_mode, 1, sc.rows, strm);
    } else {
        st = run_guided(s->dev, sc, rf, N, fl, P, std::vector<int64_t>(budget, budget + P),
                        std::vector<int64_t>(offset, offset + P), phase_mode, splat_mode, 1, sc.rows, strm, nullptr,
                        nullptr);
    }
    if (st != HSR_OK) return st;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(out_rows, sc.rows, sizeof(float) * 2 * size_t(P) * N, cudaMemcpyDeviceToHost, strm)) !=
        cudaSuccess)
        return cuda_fail(e, "row download");
    if ((e = cudaStreamSynchronize(strm)) != cudaSuccess) return cuda_fail(e, "batch run");
    return read_status(sc, strm);
}

hsr_status hsr_simulate_frame(hsr_scene *s, const hsr_rf_config *rf, const hsr_frame_config *frame,
                              const hsr_tracer_flags *fl, int32_t tx_count, const hsr_antenna *tx, int32_t rx_count,
                              const hsr_antenna *rx, int64_t budget, int64_t index_offset, int32_t phase_mode,
                              int32_t splat_mode, float *frame_out, void *stream) {
    if (!s || !frame || !tx || !rx || !frame_out || tx_count <= 0 || rx_count <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument or no antennas");
    if (frame->chirpCount <= 0 || frame->samplesPerChirp <= 0 || frame->channelCount != tx_count * rx_count)
        return fail(HSR_ERR_INVALID_ARGUMENT, "the frame needs chirps > 0 and tx_count x rx_count channels");
    if (budget < 0 || index_offset < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "negative budget or offset");
    const int32_t N = frame->samplesPerChirp, C = frame->channelCount;
    hsr_status st = validate_common(rf, N, fl);
    if (st != HSR_OK) return st;
    if ((st = validate_phase(phase_mode, splat_mode)) != HSR_OK) return st;
    // channel c = (TX c / rx_count, RX c % rx_count): every virtual channel a pose of one batch
    std::vector<hsr_antenna> ctx(C), crx(C);
    for (int32_t c = 0; c < C; ++c) {
        ctx[c] = tx[c / rx_count];
        crx[c] = rx[c % rx_count];
    }
    std::vector<int64_t> b(C, budget), o(C, index_offset);
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    cudaStream_t strm = static_cast<cudaStream_t>(stream);
    if ((st = ensure_scratch(s->dev, C, N, sc, strm, splat_mode == HSR_SPLAT_FINE_SYNTH)) != HSR_OK) return st;
    const size_t bytes = sizeof(float) * 2 * size_t(frame->chirpCount) * N * C;
    if (bytes > s->dev.frame_bytes) {
        cudaStreamSynchronize(strm);
        cudaFree(s->dev.frame_buf);
        s->dev.frame_buf = nullptr;
        s->dev.frame_bytes = 0;
        std::string err;
        if (!dev_alloc(&s->dev.frame_buf, bytes, err)) return fail(HSR_ERR_OUT_OF_MEMORY, "frame buffer: " + err);
        s->dev.frame_bytes = bytes;
    }
    if ((st = upload_poses(sc, C, ctx.data(), crx.data(), b.data(), o.data(), cudaMemcpyHostToDevice, strm)) !=
        HSR_OK)
        return st;
    st = fl->doGuiding ? run_guided(s->dev, sc, rf, N, fl, C, b, o, phase_mode, splat_mode, 1, sc.rows, strm,
                                    nullptr, nullptr)
                       : run_plain(s->dev, sc, rf, N, fl, C, 1.f, phase_mode, splat_mode, 1, sc.rows, strm);
    if (st != HSR_OK) return st;
    float *d_frame = static_cast<float *>(s->dev.frame_buf);
    if (launch_assemble_frame(sc.rows, frame->chirpCount, N, C, d_frame, strm) != 0)
        return cuda_fail(cudaGetLastError(), "frame assembly");
    cudaError_t e;
    if ((e = cudaMemcpyAsync(frame_out, d_frame, bytes, cudaMemcpyDeviceToHost, strm)) != cudaSuccess)
        return cuda_fail(e, "frame download");
    if ((e = cudaStreamSynchronize(strm)) != cudaSuccess) return cuda_fail(e, "frame simulation");
    return read_status(sc, strm);
}

hsr_status hsr_simulate_batch_ff(hsr_scene *s, const hsr_rf_config *rf, int32_t N, const hsr_tracer_flags *fl,
                                 int32_t P, const hsr_ff_antenna *tx, const hsr_ff_antenna *rx, const int64_t *budget,
                                 const int64_t *offset, int32_t phase_mode, float *out_rows) {
    if (!s || !tx || !rx || !budget || !offset || !out_rows || P <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument or no poses");
    hsr_status st = validate_common(rf, N, fl);
    if (st != HSR_OK) return st;
    if (fl->doGuiding) return fail(HSR_ERR_NOT_SUPPORTED, "far-field runs are plain (doGuiding = 0)");
    if ((st = validate_phase(phase_mode, HSR_SPLAT_DIRICHLET16)) != HSR_OK) return st;
    for (int32_t i = 0; i < P; ++i) {
        if (budget[i] < 0 || offset[i] < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "negative budget or offset");
        for (const hsr_ff_antenna *a : {tx + i, rx + i})
            if (!(a->radius > 0.f)) return fail(HSR_ERR_INVALID_ARGUMENT, "far-field antenna radius must be positive");
    }
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    cudaStream_t strm = nullptr;
    if ((st = ensure_scratch(s->dev, P, N, sc, strm)) != HSR_OK) return st;
    sc.far_field = true;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(sc.ff_tx, tx, sizeof(hsr_ff_antenna) * P, cudaMemcpyHostToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.ff_rx, rx, sizeof(hsr_ff_antenna) * P, cudaMemcpyHostToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.budget, budget, sizeof(int64_t) * P, cudaMemcpyHostToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.offset, offset, sizeof(int64_t) * P, cudaMemcpyHostToDevice, strm)) != cudaSuccess)
        return cuda_fail(e, "far-field pose upload");
    st = run_plain(s->dev, sc, rf, N, fl, P, 1.f, phase_mode, HSR_SPLAT_DIRICHLET16, 1, sc.rows, strm);
    if (st != HSR_OK) return st;
    if ((e = cudaMemcpyAsync(out_rows, sc.rows, sizeof(float) * 2 * size_t(P) * N, cudaMemcpyDeviceToHost, strm)) !=
        cudaSuccess)
        return cuda_fail(e, "row download");
    if ((e = cudaStreamSynchronize(strm)) != cudaSuccess) return cuda_fail(e, "far-field batch run");
    return read_status(sc, strm);
}

// ---- autotuning of the plain wavefront launch --------------------------------------
// Times the trace kernel (CUDA events) of the caller's batch under each candidate
// launch shape and keeps the fastest on the scene. Coordinate search: the work-item tile,
// then CTAs per SM, then the queue threshold; every trial runs twice, the faster counts.
// The candidates change only the grouping of sums, not the samples: rows agree with the
// default shape up to FP32/FP64 summation order.
hsr_status hsr_autotune_batch(hsr_scene *s, const hsr_rf_config *rf, int32_t N, const hsr_tracer_flags *fl, int32_t P,
                              const hsr_antenna *tx, const hsr_antenna *rx, const int64_t *budget,
                              const int64_t *offset, int32_t phase_mode, int32_t splat_mode,
                              hsr_launch_config *out_best) {
    if (!s || !tx || !rx || !budget || !offset || !out_best || P <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument or no poses");
    hsr_status st = validate_common(rf, N, fl);
    if (st != HSR_OK) return st;
    if ((st = validate_phase(phase_mode, splat_mode)) != HSR_OK) return st;
    if (fl->doGuiding || !fl->useGeometricalOptics)
        return fail(HSR_ERR_NOT_SUPPORTED, "the autotuner tunes the plain wavefront launch (GO mode, no guiding)");
    for (int32_t i = 0; i < P; ++i)
        if (budget[i] < 0 || offset[i] < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "negative budget or offset");
    std::lock_guard<std::mutex> lk(s->mu);
    SceneDev &d = s->dev;
    Scratch sc;
    if ((st = ensure_scratch(d, P, N, sc, nullptr, splat_mode == HSR_SPLAT_FINE_SYNTH)) != HSR_OK) return st;
    if ((st = upload_poses(sc, P, tx, rx, budget, offset, cudaMemcpyHostToDevice, nullptr)) != HSR_OK) return st;
    const LaunchConfig saved = d.tuned;
    auto trial = [&](const LaunchConfig &c, float &ms) -> hsr_status {
        d.tuned = c;
        ms = 1e30f;
        for (int r = 0; r < 2; ++r) {
            hsr_status rs = run_plain(d, sc, rf, N, fl, P, 1.f, phase_mode, splat_mode, 1, sc.rows, nullptr);
            if (rs != HSR_OK) return rs;
            cudaError_t e = cudaEventSynchronize(d.ev1);
            if (e != cudaSuccess) return cuda_fail(e, "autotune trial");
            float t = 0.f;
            cudaEventElapsedTime(&t, d.ev0, d.ev1);
            ms = std::min(ms, t);
        }
        return read_status(sc, nullptr);
    };
    LaunchConfig best;  // the default shape
    float best_ms = 0.f, ms = 0.f;
    if ((st = trial(best, best_ms)) != HSR_OK) {
        d.tuned = saved;
        return st;
    }
    const float default_ms = best_ms;
    const int32_t tiles[] = {1024, 2048, 4096, 8192, 16384};
    const int32_t ctas[] = {2, 3, 4};
    const int32_t thresholds[] = {32, 64, kWaveDefaultQueue, kWaveMaxQueueThreshold};
    for (int32_t t : tiles) {
        LaunchConfig c = best;
        c.tile = t;
        if ((st = trial(c, ms)) != HSR_OK) break;
        if (ms < best_ms) best_ms = ms, best = c;
    }
    for (int32_t k = 0; st == HSR_OK && k < 3; ++k) {
        LaunchConfig c = best;
        c.ctas_per_sm = ctas[k];
        if ((st = trial(c, ms)) != HSR_OK) break;
        if (ms < best_ms) best_ms = ms, best = c;
    }
    for (int32_t k = 0; st == HSR_OK && k < 4; ++k) {
        LaunchConfig c = best;
        c.queue_threshold = thresholds[k];
        if ((st = trial(c, ms)) != HSR_OK) break;
        if (ms < best_ms) best_ms = ms, best = c;
    }
    if (st == HSR_OK) {  // the primary field formed on a hit (pays where most primaries miss)
        LaunchConfig c = best;
        c.field_on_hit = 1;
        if ((st = trial(c, ms)) == HSR_OK && ms < best_ms) best_ms = ms, best = c;
    }
    if (st == HSR_OK) {  // coherent stage order (pays where traversal dominates)
        LaunchConfig c = best;
        c.coherent_order = 1;
        if ((st = trial(c, ms)) == HSR_OK && ms < best_ms) best_ms = ms, best = c;
    }
    if (st != HSR_OK) {
        d.tuned = saved;
        return st;
    }
    // store the shape explicitly: a threshold of 0 means "the default" to the kernel, but
    // the serving ticks read the scene's tuned threshold to pick their path stack
    if (best.queue_threshold <= 0) best.queue_threshold = kWaveDefaultQueue;
    d.tuned = best;
    out_best->tile = best.tile > 0 ? best.tile : kTile;
    out_best->ctas_per_sm = best.ctas_per_sm;
    out_best->queue_threshold = best.queue_threshold > 0 ? best.queue_threshold : kWaveDefaultQueue;
    out_best->field_on_hit = best.field_on_hit;
    out_best->coherent_order = best.coherent_order;
    out_best->trace_ms = best_ms;
    out_best->default_trace_ms = default_ms;
    return HSR_OK;
}

hsr_status hsr_set_launch_config(hsr_scene *s, const hsr_launch_config *c) {
    if (!s) return fail(HSR_ERR_INVALID_ARGUMENT, "null scene");
    LaunchConfig l;
    if (c) {
        if (c->tile < 0 || (c->tile > 0 && (c->tile < 32 || c->tile > (1 << 20))) || c->ctas_per_sm < 0 ||
            c->ctas_per_sm > 32 || c->queue_threshold < 0 || c->queue_threshold > kWaveMaxQueueThreshold ||
            (c->field_on_hit != 0 && c->field_on_hit != 1) || (c->coherent_order != 0 && c->coherent_order != 1))
            return fail(HSR_ERR_INVALID_ARGUMENT, "launch config out of range");
        l.tile = c->tile;
        l.ctas_per_sm = c->ctas_per_sm;
        l.queue_threshold = c->queue_threshold;
        l.field_on_hit = c->field_on_hit;
        l.coherent_order = c->coherent_order;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->dev.tuned = l;  // null: back to the default shape
    return HSR_OK;
}

hsr_status hsr_get_launch_config(const hsr_scene *s, hsr_launch_config *out) {
    if (!s || !out) return fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    out->tile = s->dev.tuned.tile;
    out->ctas_per_sm = s->dev.tuned.ctas_per_sm;
    out->queue_threshold = s->dev.tuned.queue_threshold;
    out->field_on_hit = s->dev.tuned.field_on_hit;
    out->coherent_order = s->dev.tuned.coherent_order;
    out->trace_ms = 0.f;
    out->default_trace_ms = 0.f;
    return HSR_OK;
}

hsr_status hsr_debug_traversal_counts(hsr_scene *s, const hsr_rf_config *rf, int32_t N, const hsr_tracer_flags *fl,
                                      int32_t P, const hsr_antenna *tx, const hsr_antenna *rx, const int64_t *budget,
                                      const int64_t *offset, int64_t *out_counts) {
    if (!s || !tx || !rx || !budget || !offset || !out_counts || P <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument or no poses");
    hsr_status st = validate_common(rf, N, fl);
    if (st != HSR_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    if ((st = ensure_scratch(s->dev, P, N, sc, nullptr)) != HSR_OK) return st;
    unsigned long long *d_cnt = nullptr;
    std::string err;
    if (!dev_alloc(&d_cnt, 4 * sizeof(unsigned long long), err)) return fail(HSR_ERR_OUT_OF_MEMORY, err);
    cudaMemset(d_cnt, 0, 4 * sizeof(unsigned long long));
    if ((st = upload_poses(sc, P, tx, rx, budget, offset, cudaMemcpyHostToDevice, 0)) != HSR_OK) {
        cudaFree(d_cnt);
        return st;
    }
    st = run_plain(s->dev, sc, rf, N, fl, P, 1.f, HSR_PHASE_REFERENCE_FP32, HSR_SPLAT_DIRICHLET16, 1, sc.rows, 0,
                   nullptr, 0, d_cnt);
    unsigned long long h[4] = {0, 0, 0, 0};
    if (st == HSR_OK) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) st = cuda_fail(e, "counting run");
    }
    if (st == HSR_OK) cudaMemcpy(h, d_cnt, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d_cnt);
    for (int i = 0; i < 3; ++i) out_counts[i] = int64_t(h[i]);
    if (st == HSR_OK) st = read_status(sc, 0);
    return st;
}

hsr_status hsr_set_path_kernel(int32_t kind) {
    if (kind != 0 && kind != 1) return fail(HSR_ERR_INVALID_ARGUMENT, "kind must be 0 or 1");
    g_path_kernel = kind;
    return HSR_OK;
}

hsr_status hsr_set_bvh_builder(int32_t builder) {
    if (builder != 0 && builder != 1) return fail(HSR_ERR_INVALID_ARGUMENT, "builder must be 0 or 1");
    g_bvh_builder = builder;
    return HSR_OK;
}

hsr_status hsr_set_bvh_leaf_size(int32_t triangles) {
    if (triangles < 1 || triangles > 8) return fail(HSR_ERR_INVALID_ARGUMENT, "leaf size must be 1..8");
    g_bvh_leaf_max = triangles;
    return HSR_OK;
}

hsr_status hsr_set_bvh_optimize(int32_t passes) {
    if (passes < 0 || passes > 64) return fail(HSR_ERR_INVALID_ARGUMENT, "passes must be 0..64");
    g_bvh_optimize = passes;
    return HSR_OK;
}

hsr_status hsr_set_synth_engine(int32_t engine) {
    if (engine != 0 && engine != 1) return fail(HSR_ERR_INVALID_ARGUMENT, "engine must be 0 or 1");
    g_synth_engine = engine;
    return HSR_OK;
}

hsr_status hsr_last_kernel_ms(const hsr_scene *s, float *out_ms) {
    if (!s || !out_ms) return fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    if (!s->dev.timing_valid) return fail(HSR_ERR_INVALID_ARGUMENT, "no launch recorded yet");
    cudaError_t e = cudaEventSynchronize(s->dev.ev1);
    if (e != cudaSuccess) return cuda_fail(e, "event sync");
    e = cudaEventElapsedTime(out_ms, s->dev.ev0, s->dev.ev1);
    if (e != cudaSuccess) return cuda_fail(e, "event elapsed");
    return HSR_OK;
}

// ---- measurement support: L2 read bandwidth ----------------------------------------
namespace {
// Every thread sweeps its share of an L2-resident buffer `sweeps` times with L2-cached
// (not L1) loads; the checksum keeps the loads.
__global__ void k_l2_read(const float4 *__restrict__ buf, int64_t n4, int sweeps, float *sink) {
    float acc = 0.f;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int s = 0; s < sweeps; ++s)
        for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n4; i += stride) {
            const float4 v = __ldcg(buf + i);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    if (acc == 1234567.f) sink[0] = acc;
}
}  // namespace

hsr_status hsr_measure_l2_read(int64_t bytes, int32_t sweeps, double *out_gbs) {
    if (!out_gbs || bytes < (1 << 20) || sweeps < 1) return fail(HSR_ERR_INVALID_ARGUMENT, "bad L2 measurement size");
    hsr_status st = check_device();
    if (st != HSR_OK) return st;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t n4 = bytes / 16;
    float4 *buf = nullptr;
    float *sink = nullptr;
    std::string err;
    if (!dev_alloc(&buf, size_t(n4) * 16, err) || !dev_alloc(&sink, 16, err)) {
        cudaFree(buf);
        return fail(HSR_ERR_OUT_OF_MEMORY, err);
    }
    cudaMemset(buf, 0, size_t(n4) * 16);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 0.f;
    for (int r = 0; r < 6; ++r) {  // the first run warms L2 and is not counted
        cudaEventRecord(e0);
        k_l2_read<<<sms * 8, 256>>>(buf, n4, sweeps, sink);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && (best == 0.f || ms < best)) best = ms;
    }
    note_launches(6);
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) return cuda_fail(e, "L2 read kernel");
    *out_gbs = double(n4) * 16.0 * sweeps / (double(best) / 1000.0) / 1e9;
    return HSR_OK;
}

// ---- a plain batch captured into a CUDA graph ------------------------------------
struct hsr_batch_graph {
    hsr_scene *scene = nullptr;
    void *scratch = nullptr;
    unsigned *status = nullptr;
    // fine-histogram synthesis: the graph's own twiddle operand and synthesis scratch
    // (the scene's are rebuilt when another call uses another N)
    SynthOperand synth;
    void *synth_scratch = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t kernel_nodes = 0;  // kernels one replay launches (hsr_launch_count)
};

hsr_status hsr_batch_graph_create(hsr_scene *s, const hsr_rf_config *rf, int32_t N, const hsr_tracer_flags *fl,
                                  int32_t P, const hsr_antenna *d_tx, const hsr_antenna *d_rx,
                                  const int64_t *d_budget, const int64_t *d_offset, int32_t phase_mode,
                                  int32_t splat_mode, float *d_out_rows, hsr_batch_graph **out) {
    if (!out) return fail(HSR_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    if (!s || !d_tx || !d_rx || !d_budget || !d_offset || !d_out_rows || P <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument or no poses");
    hsr_status st = validate_common(rf, N, fl);
    if (st != HSR_OK) return st;
    if ((st = validate_phase(phase_mode, splat_mode)) != HSR_OK) return st;
    if (fl->doGuiding)
        return fail(HSR_ERR_NOT_SUPPORTED, "a batch graph runs the plain method (doGuiding must be 0)");
    std::lock_guard<std::mutex> lk(s->mu);
    std::unique_ptr<hsr_batch_graph> g(new hsr_batch_graph());
    g->scene = s;
    const bool fine = splat_mode == HSR_SPLAT_FINE_SYNTH;
    const Scratch need = carve(nullptr, P, N, fine);
    std::string aerr;
    if (!dev_alloc(&g->scratch, need.bytes, aerr)) return fail(HSR_ERR_OUT_OF_MEMORY, "graph scratch: " + aerr);
    cudaError_t e;
    // the scene's state as the capture sees it, with the graph's own synthesis operand and
    // scratch (allocated here, before the capture; run_plain's ensure_synth then finds
    // them in place)
    SceneDev gdev = s->dev;
    gdev.synth = SynthOperand{};
    gdev.synth_scratch = nullptr;
    gdev.synth_scratch_bytes = 0;
    auto cleanup = [&]() {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        if (g->graph) cudaGraphDestroy(g->graph);
        cudaFree(g->scratch);
        synth_free_operand(gdev.synth);
        cudaFree(gdev.synth_scratch);
    };
    if ((e = cudaMemset(g->scratch, 0, 256)) != cudaSuccess) {
        cleanup();
        return cuda_fail(e, "graph scratch clear");
    }
    if (fine) {
        if ((st = ensure_synth(gdev, N, P, nullptr)) != HSR_OK || (e = cudaDeviceSynchronize()) != cudaSuccess) {
            cleanup();
            return st != HSR_OK ? st : cuda_fail(e, "graph synthesis operand");
        }
    }
    const Scratch sc = carve(g->scratch, P, N, fine);
    g->status = sc.counters;
    cudaStream_t cs = nullptr;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) {
        cleanup();
        return cuda_fail(e, "capture stream");
    }
    hsr_status rst = HSR_OK;
    if ((e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
        rst = cuda_fail(e, "begin capture");
    } else {
        rst = upload_poses(sc, P, d_tx, d_rx, d_budget, d_offset, cudaMemcpyDeviceToDevice, cs);
        if (rst == HSR_OK) rst = run_plain(gdev, sc, rf, N, fl, P, 1.f, phase_mode, splat_mode, 1, d_out_rows, cs);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(cs, &graph);
        g->graph = graph;
        if (rst == HSR_OK && e != cudaSuccess) rst = cuda_fail(e, "end capture");
        if (rst == HSR_OK && (e = cudaGraphInstantiate(&g->exec, g->graph, 0)) != cudaSuccess)
            rst = cuda_fail(e, "graph instantiation");
    }
    cudaStreamDestroy(cs);
    if (rst != HSR_OK) {
        cudaGetLastError();
        cleanup();
        return rst;
    }
    g->synth = gdev.synth;
    g->synth_scratch = gdev.synth_scratch;
    size_t n_nodes = 0;
    if (cudaGraphGetNodes(g->graph, nullptr, &n_nodes) == cudaSuccess && n_nodes > 0) {
        std::vector<cudaGraphNode_t> nodes(n_nodes);
        if (cudaGraphGetNodes(g->graph, nodes.data(), &n_nodes) == cudaSuccess)
            for (size_t i = 0; i < n_nodes; ++i) {
                cudaGraphNodeType ty;
                if (cudaGraphNodeGetType(nodes[i], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel)
                    ++g->kernel_nodes;
            }
    }
    cudaGetLastError();
    s->graphs.fetch_add(1);
    *out = g.release();
    return HSR_OK;
}

hsr_status hsr_batch_graph_launch(hsr_batch_graph *g, void *stream) {
    if (!g || !g->exec) return fail(HSR_ERR_INVALID_ARGUMENT, "null graph");
    cudaError_t e = cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "graph launch");
    note_launches(std::max<int64_t>(g->kernel_nodes, 1));
    return HSR_OK;
}

hsr_status hsr_batch_graph_status(hsr_batch_graph *g) {
    if (!g) return fail(HSR_ERR_INVALID_ARGUMENT, "null graph");
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "graph synchronisation");
    unsigned bits = 0;
    if ((e = cudaMemcpy(&bits, g->status, sizeof(bits), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail(e, "graph status read");
    if (bits) return fail(HSR_ERR_DEVICE, "a graph launch reported device status " + std::to_string(bits));
    return HSR_OK;
}

hsr_status hsr_batch_graph_destroy(hsr_batch_graph *g) {
    if (!g) return HSR_OK;
    cudaDeviceSynchronize();
    if (g->scene) g->scene->graphs.fetch_sub(1);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    cudaFree(g->scratch);
    synth_free_operand(g->synth);
    cudaFree(g->synth_scratch);
    delete g;
    return HSR_OK;
}

}  // extern "C"
