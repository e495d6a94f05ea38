// The C ABI (include/hsr_gb300.h): scene residency, ray queries and simulate calls.
// Every entry point returns an hsr_status; the message of the last failure on the
// calling thread is available from hsr_last_error(). No exception crosses the ABI.
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "hsr_common.cuh"
#include "hsr_internal.h"

namespace hsr {

static thread_local std::string g_err;
int g_path_kernel = 0;
static std::atomic<int64_t> g_launches{0};

void note_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

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
    if (fl->doGuiding)
        return fail(HSR_ERR_NOT_SUPPORTED, "doGuiding=1 runs through the guided schedule, not a plain backend run");
    return HSR_OK;
}

// Scratch layout for a batch of P poses with N bins, carved from one allocation.
struct Scratch {
    hsr_antenna *tx, *rx;
    int64_t *budget, *offset, *tile_start;
    double *acc;
    float *rows;
    unsigned *counters;  // [0] status, [2..3] 64-bit work counter
    size_t bytes;
};

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static Scratch carve(void *base, int32_t P, int32_t N) {
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
    s.budget = reinterpret_cast<int64_t *>(take(sizeof(int64_t) * P));
    s.offset = reinterpret_cast<int64_t *>(take(sizeof(int64_t) * P));
    s.tile_start = reinterpret_cast<int64_t *>(take(sizeof(int64_t) * (P + 1)));
    s.acc = reinterpret_cast<double *>(take(sizeof(double) * 2 * size_t(P) * N));
    s.rows = reinterpret_cast<float *>(take(sizeof(float) * 2 * size_t(P) * N));
    s.bytes = off;
    return s;
}

static hsr_status ensure_scratch(SceneDev &sc, int32_t P, int32_t N, Scratch &out) {
    Scratch need = carve(nullptr, P, N);
    if (need.bytes > sc.scratch_bytes) {
        if (sc.scratch) cudaFree(sc.scratch);
        sc.scratch = nullptr;
        sc.scratch_bytes = 0;
        cudaError_t e = cudaMalloc(&sc.scratch, need.bytes);
        if (e != cudaSuccess) return cuda_fail(e, "scratch allocation");
        // the status word must start clear; the rest is initialised per call
        e = cudaMemset(sc.scratch, 0, 256);
        if (e != cudaSuccess) return cuda_fail(e, "scratch clear");
        sc.scratch_bytes = need.bytes;
    }
    out = carve(sc.scratch, P, N);
    return HSR_OK;
}

static constexpr int32_t kTile = 4096;  // samples per work item (16 per thread at 256 threads)

// Enqueues one batch: poses/budgets already in scratch (device), accumulators zeroed here.
static hsr_status enqueue_batch(SceneDev &sc, const Scratch &s, const hsr_rf_config *rf, int32_t N,
                                const hsr_tracer_flags *fl, int32_t P, float sample_weight, int32_t phase_mode,
                                int32_t splat_mode, int normalise, float *d_out_rows, cudaStream_t st,
                                void *records, int max_rec, unsigned long long *counters = nullptr) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(s.acc, 0, sizeof(double) * 2 * size_t(P) * N, st)) != cudaSuccess)
        return cuda_fail(e, "memset accumulators");
    if ((e = cudaMemsetAsync(s.counters + 2, 0, 8, st)) != cudaSuccess) return cuda_fail(e, "memset counter");
    if (launch_tile_prefix(s.budget, P, kTile, s.tile_start, st) != 0)
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
    p.tile = kTile;
    p.acc = s.acc;
    p.status = s.counters;
    p.work_counter = s.counters + 2;
    p.records = records;
    p.max_rec = max_rec;
    p.counters = counters;
    const bool wave = g_path_kernel == 0 && fl->useGeometricalOptics && !records && !counters;
    int grid = sc.sm_count * (wave ? wave_blocks_per_sm(N) : trace_blocks_per_sm(N, splat_mode, 0));
    cudaEventRecord(sc.ev0, st);
    std::string err;
    if (wave) {
        if (launch_wave(p, phase_mode, grid, st, err) != 0) return fail(HSR_ERR_CUDA, err);
    } else if (launch_trace(p, phase_mode, splat_mode, grid, st, err) != 0) {
        return fail(HSR_ERR_CUDA, err);
    }
    cudaEventRecord(sc.ev1, st);
    sc.timing_valid = true;
    if (launch_finalize(s.acc, P, N, s.budget, sample_weight, normalise, d_out_rows, st) != 0)
        return cuda_fail(cudaGetLastError(), "finalize launch");
    return HSR_OK;
}

static hsr_status read_status(SceneDev &sc, const Scratch &s, cudaStream_t st) {
    unsigned bits = 0;
    cudaError_t e = cudaMemcpyAsync(&bits, s.counters, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "status read");
    if (bits) {
        cudaMemsetAsync(s.counters, 0, sizeof(unsigned), st);
        cudaStreamSynchronize(st);
        std::string m = "device status:";
        if (bits & kStatusStackOverflow) m += " traversal-stack-overflow";
        if (bits & kStatusBadBin) m += " bin-out-of-range";
        if (bits & kStatusBadWorkItem) m += " bad-work-item";
        return fail(HSR_ERR_DEVICE, m);
    }
    (void)sc;
    return HSR_OK;
}

}  // namespace hsr

using namespace hsr;

struct hsr_scene {
    SceneDev dev;
    std::mutex mu;
};

extern "C" {

int32_t hsr_abi_version(void) { return HSR_ABI_VERSION; }

const char *hsr_last_error(void) { return g_err.c_str(); }

int64_t hsr_launch_count(void) { return g_launches.load(); }

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
    cudaFree(di);
    if (rc != 0) {
        cudaFree(d.tris);
        cudaFree(d.nodes);
        delete s;
        return fail(rc == 3 ? HSR_ERR_OUT_OF_MEMORY : HSR_ERR_CUDA, err);
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
    cudaFree(s->dev.scratch);
    if (s->dev.ev0) cudaEventDestroy(s->dev.ev0);
    if (s->dev.ev1) cudaEventDestroy(s->dev.ev1);
    delete s;
    return HSR_OK;
}

hsr_status hsr_scene_footprint(const hsr_scene *s, int64_t *out_bytes) {
    if (!s || !out_bytes) return fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    *out_bytes = int64_t(sizeof(DTri)) * std::max<int64_t>(s->dev.tri_count, 1) +
                 int64_t(sizeof(DNode)) * s->dev.node_count + int64_t(s->dev.scratch_bytes);
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

// Records of individual next-event estimates (tests): records is a HOST array of
// budget * max_rec PathRecord-sized entries (9 x 4 bytes each).
hsr_status hsr_debug_records(hsr_scene *s, const hsr_rf_config *rf, int32_t samples, const hsr_tracer_flags *fl,
                             const hsr_antenna *tx, const hsr_antenna *rx, int64_t budget, int64_t index_offset,
                             int32_t max_rec, void *records) {
    hsr_status st = validate_common(rf, samples, fl);
    if (st != HSR_OK) return st;
    if (!s || !tx || !rx || !records || budget <= 0 || max_rec <= 0 || budget > (int64_t(1) << 22))
        return fail(HSR_ERR_INVALID_ARGUMENT, "bad record request");
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    if ((st = ensure_scratch(s->dev, 1, samples, sc)) != HSR_OK) return st;
    const size_t rec_bytes = size_t(budget) * max_rec * 36;
    void *d_rec = nullptr;
    std::string err;
    if (!dev_alloc(&d_rec, rec_bytes, err)) return fail(HSR_ERR_OUT_OF_MEMORY, err);
    // unused slots: depth = -1
    std::vector<int32_t> init(rec_bytes / 4, 0);
    for (size_t i = 0; i < init.size(); i += 9) init[i] = -1;
    cudaMemcpy(d_rec, init.data(), rec_bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(sc.tx, tx, sizeof(hsr_antenna), cudaMemcpyHostToDevice);
    cudaMemcpy(sc.rx, rx, sizeof(hsr_antenna), cudaMemcpyHostToDevice);
    cudaMemcpy(sc.budget, &budget, sizeof(int64_t), cudaMemcpyHostToDevice);
    cudaMemcpy(sc.offset, &index_offset, sizeof(int64_t), cudaMemcpyHostToDevice);
    st = enqueue_batch(s->dev, sc, rf, samples, fl, 1, 1.f, HSR_PHASE_REFERENCE_FP32, HSR_SPLAT_DIRICHLET16, 0,
                       sc.rows, 0, d_rec, max_rec);
    if (st == HSR_OK) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) st = cuda_fail(e, "record run");
    }
    if (st == HSR_OK) cudaMemcpy(records, d_rec, rec_bytes, cudaMemcpyDeviceToHost);
    cudaFree(d_rec);
    if (st == HSR_OK) st = read_status(s->dev, sc, 0);
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
    if (budget < 0 || index_offset < 0) return fail(HSR_ERR_INVALID_ARGUMENT, "negative budget or offset");
    if (phase_mode != HSR_PHASE_REFERENCE_FP32 && phase_mode != HSR_PHASE_SPLIT_FP64)
        return fail(HSR_ERR_INVALID_ARGUMENT, "unknown phase mode");
    if (interrupt_flag && *interrupt_flag) return fail(HSR_ERR_INTERRUPTED, "interrupted before start");
    if (budget == 0) return HSR_OK;
    const int32_t N = frame->samplesPerChirp;
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    if ((st = ensure_scratch(s->dev, 1, N, sc)) != HSR_OK) return st;
    cudaStream_t strm = 0;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(sc.tx, tx, sizeof(hsr_antenna), cudaMemcpyHostToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.rx, rx, sizeof(hsr_antenna), cudaMemcpyHostToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.budget, &budget, sizeof(int64_t), cudaMemcpyHostToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.offset, &index_offset, sizeof(int64_t), cudaMemcpyHostToDevice, strm)) !=
            cudaSuccess)
        return cuda_fail(e, "pose upload");
    st = enqueue_batch(s->dev, sc, rf, N, fl, 1, sample_weight, phase_mode, HSR_SPLAT_DIRICHLET16, 0, sc.rows, strm,
                       nullptr, 0);
    if (st != HSR_OK) return st;
    std::vector<float> row(2 * size_t(N));
    if ((e = cudaMemcpyAsync(row.data(), sc.rows, sizeof(float) * 2 * N, cudaMemcpyDeviceToHost, strm)) !=
        cudaSuccess)
        return cuda_fail(e, "row download");
    if ((e = cudaStreamSynchronize(strm)) != cudaSuccess) return cuda_fail(e, "backend run");
    if ((st = read_status(s->dev, sc, strm)) != HSR_OK) return st;
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

hsr_status hsr_simulate_batch_device(hsr_scene *s, const hsr_rf_config *rf, int32_t N, const hsr_tracer_flags *fl,
                                     int32_t P, const hsr_antenna *d_tx, const hsr_antenna *d_rx,
                                     const int64_t *d_budget, const int64_t *d_offset, int32_t phase_mode,
                                     int32_t splat_mode, float *d_out_rows, void *stream) {
    if (!s || !d_tx || !d_rx || !d_budget || !d_offset || !d_out_rows || P <= 0)
        return fail(HSR_ERR_INVALID_ARGUMENT, "null argument or no poses");
    hsr_status st = validate_common(rf, N, fl);
    if (st != HSR_OK) return st;
    if (phase_mode != HSR_PHASE_REFERENCE_FP32 && phase_mode != HSR_PHASE_SPLIT_FP64)
        return fail(HSR_ERR_INVALID_ARGUMENT, "unknown phase mode");
    if (splat_mode != HSR_SPLAT_DIRICHLET16)
        return fail(HSR_ERR_NOT_SUPPORTED, "splat mode not available in this build");
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    if ((st = ensure_scratch(s->dev, P, N, sc)) != HSR_OK) return st;
    cudaStream_t strm = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(sc.tx, d_tx, sizeof(hsr_antenna) * P, cudaMemcpyDeviceToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.rx, d_rx, sizeof(hsr_antenna) * P, cudaMemcpyDeviceToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.budget, d_budget, sizeof(int64_t) * P, cudaMemcpyDeviceToDevice, strm)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(sc.offset, d_offset, sizeof(int64_t) * P, cudaMemcpyDeviceToDevice, strm)) != cudaSuccess)
        return cuda_fail(e, "pose staging");
    return enqueue_batch(s->dev, sc, rf, N, fl, P, 1.f, phase_mode, splat_mode, 1, d_out_rows, strm, nullptr, 0);
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
    if (phase_mode != HSR_PHASE_REFERENCE_FP32 && phase_mode != HSR_PHASE_SPLIT_FP64)
        return fail(HSR_ERR_INVALID_ARGUMENT, "unknown phase mode");
    if (splat_mode != HSR_SPLAT_DIRICHLET16)
        return fail(HSR_ERR_NOT_SUPPORTED, "splat mode not available in this build");
    std::lock_guard<std::mutex> lk(s->mu);
    Scratch sc;
    if ((st = ensure_scratch(s->dev, P, N, sc)) != HSR_OK) return st;
    cudaStream_t strm = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(sc.tx, tx, sizeof(hsr_antenna) * P, cudaMemcpyHostToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.rx, rx, sizeof(hsr_antenna) * P, cudaMemcpyHostToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.budget, budget, sizeof(int64_t) * P, cudaMemcpyHostToDevice, strm)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sc.offset, offset, sizeof(int64_t) * P, cudaMemcpyHostToDevice, strm)) != cudaSuccess)
        return cuda_fail(e, "pose upload");
    st = enqueue_batch(s->dev, sc, rf, N, fl, P, 1.f, phase_mode, splat_mode, 1, sc.rows, strm, nullptr, 0);
    if (st != HSR_OK) return st;
    if ((e = cudaMemcpyAsync(out_rows, sc.rows, sizeof(float) * 2 * size_t(P) * N, cudaMemcpyDeviceToHost, strm)) !=
        cudaSuccess)
        return cuda_fail(e, "row download");
    if ((e = cudaStreamSynchronize(strm)) != cudaSuccess) return cuda_fail(e, "batch run");
    return read_status(s->dev, sc, strm);
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
    if ((st = ensure_scratch(s->dev, P, N, sc)) != HSR_OK) return st;
    unsigned long long *d_cnt = nullptr;
    std::string err;
    if (!dev_alloc(&d_cnt, 4 * sizeof(unsigned long long), err)) return fail(HSR_ERR_OUT_OF_MEMORY, err);
    cudaMemset(d_cnt, 0, 4 * sizeof(unsigned long long));
    cudaMemcpy(sc.tx, tx, sizeof(hsr_antenna) * P, cudaMemcpyHostToDevice);
    cudaMemcpy(sc.rx, rx, sizeof(hsr_antenna) * P, cudaMemcpyHostToDevice);
    cudaMemcpy(sc.budget, budget, sizeof(int64_t) * P, cudaMemcpyHostToDevice);
    cudaMemcpy(sc.offset, offset, sizeof(int64_t) * P, cudaMemcpyHostToDevice);
    st = enqueue_batch(s->dev, sc, rf, N, fl, P, 1.f, HSR_PHASE_REFERENCE_FP32, HSR_SPLAT_DIRICHLET16, 1, sc.rows, 0,
                       nullptr, 0, d_cnt);
    unsigned long long h[4] = {0, 0, 0, 0};
    if (st == HSR_OK) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) st = cuda_fail(e, "counting run");
    }
    if (st == HSR_OK) cudaMemcpy(h, d_cnt, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d_cnt);
    for (int i = 0; i < 3; ++i) out_counts[i] = int64_t(h[i]);
    if (st == HSR_OK) st = read_status(s->dev, sc, 0);
    return st;
}

hsr_status hsr_set_path_kernel(int32_t kind) {
    if (kind != 0 && kind != 1) return fail(HSR_ERR_INVALID_ARGUMENT, "kind must be 0 or 1");
    g_path_kernel = kind;
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

}  // extern "C"
