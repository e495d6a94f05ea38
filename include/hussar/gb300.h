/*
 * hussar/gb300.h — C++ drop-in backend over the C ABI (hsr_gb300.h).
 *
 * hussar::gb300::Backend has the constructor and run() of the reference backends:
 *   Backend(const TriangleMesh &mesh, Integrator &integrator)   (arch/cpu.h:18-20, arch/gpu.h:18-20)
 *   void run(const Scene &scene, long budget, bool *interruptFlag = nullptr)
 *                                                               (arch/cpu.h:44-46, arch/gpu.h:26-32)
 * and is used the same way: PathTracer::run<Backend>(backend, scene, samples) calls
 * backend.run(scene, budget, flag) once per schedule step (integrators/path.h:171-224).
 *
 * It is duck-typed like the reference's backends, so it works with
 *  - libhussar's own types (Eigen vectors, radar::Frame, hussar::PathTracer) once
 *    PathTracer befriends hussar::gb300::BackendAccess (one friend declaration in
 *    path.h), and
 *  - the self-contained mirror types in hussar/gb300_types.h.
 * Requirements on the types:
 *   mesh.vertexBuffer[i].x()/.y()/.z(), mesh.indexBuffer[i].v0/.v1/.v2
 *   scene.rfConfig.{startFreq,freqSlope,adcRate,idleTime,rampTime,antennaDelay}
 *   scene.tx/rx.position().x().., scene.tx/rx.rotation()(row, col)
 *   integrator: the public flags of path.h:153-169, produceDebugImage, and (through
 *   BackendAccess) frame, totalWeight, sampleIndexOffset, currentSampleWeight and
 *   isFinalIteration.
 * Guiding (doGuiding = true, the reference's default, path.h:158): PathTracer::run calls
 * run() once per iteration of its doubling schedule (path.h:186-224) and steps its own
 * guiding tree in between. The backend keeps the device tree of the schedule
 * (hsr_guide_*) and follows the same steps: a run that is not a final iteration and
 * traces at most the first milestone (16384 samples, path.h:185) starts a schedule
 * (reset), every later one steps the tree first (the reference steps after every
 * non-final iteration), and only non-final iterations train it. The integrator's own
 * tree (libguiding) is not used.
 * Errors: a non-OK hsr_status becomes std::runtime_error (the reference's
 * sutil::Exception derives from std::runtime_error, Exception.h:243); an interrupted
 * run returns silently like cpu::Backend (arch/cpu.h:25).
 */
#ifndef HUSSAR_GB300_H
#define HUSSAR_GB300_H

#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "../hsr_gb300.h"

namespace hussar {
namespace gb300 {

inline void check(hsr_status s) {
    if (s != HSR_OK && s != HSR_ERR_INTERRUPTED) throw std::runtime_error(std::string("gb300: ") + hsr_last_error());
}

/* Access to the integrator state the reference keeps protected/private
 * (path.h:140, 457-464; integrator.h:170). Specialise or befriend as needed. */
template <typename Integrator> struct BackendAccess {
    static auto &frame(Integrator &it) { return it.frame; }
    static double totalWeight(Integrator &it) { return double(it.totalWeight); }
    static void setTotalWeight(Integrator &it, double w) { it.totalWeight = w; }
    static long sampleIndexOffset(Integrator &it) { return long(it.sampleIndexOffset); }
    static float currentSampleWeight(Integrator &it) { return float(it.currentSampleWeight); }
    static bool isFinalIteration(Integrator &it) { return bool(it.isFinalIteration); }
};

template <typename Vec> inline void put3(float *out, const Vec &v) {
    out[0] = float(v.x());
    out[1] = float(v.y());
    out[2] = float(v.z());
}

template <typename Antenna> inline hsr_antenna to_hsr(const Antenna &a) {
    hsr_antenna r;
    put3(r.position, a.position());
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.rotation[3 * i + j] = float(a.rotation()(i, j));
    return r;
}

template <typename Rf> inline hsr_rf_config to_hsr_rf(const Rf &rf) {
    return hsr_rf_config{float(rf.startFreq), float(rf.freqSlope), float(rf.adcRate),
                         float(rf.idleTime),  float(rf.rampTime),  float(rf.antennaDelay)};
}

template <typename Integrator> inline hsr_tracer_flags to_hsr_flags(const Integrator &it) {
    hsr_tracer_flags f;
    f.onlyIndirect = it.onlyIndirect;
    f.maxDepth = it.maxDepth;
    f.useGeometricalOptics = it.useGeometricalOptics;
    f.poDiffraction = it.poDiffraction;
    f.doGuiding = it.doGuiding;  // the schedule is the integrator's; each run is one iteration
    f.clearBeforeIteration = it.clearBeforeIteration;
    f.correctPhase = it.correctPhase;
    f.filterGuiding = it.filterGuiding;
    f.doFiltering = it.doFiltering;
    f.filteringSphere = it.filteringSphere;
    f.produceDebugImage = it.produceDebugImage;
    f.filteringMin = float(it.filteringMin);
    f.filteringMax = float(it.filteringMax);
    f.filteringRadius = float(it.filteringRadius);
    return f;
}

/* The scene as the C ABI sees it. */
struct SceneView {
    hsr_rf_config rf;
    hsr_antenna tx, rx;
};

struct Backend {
    template <typename Mesh, typename Integrator>
    Backend(const Mesh &mesh, Integrator &integrator) {
        std::vector<float> v(3 * mesh.vertexBuffer.size());
        for (size_t i = 0; i < mesh.vertexBuffer.size(); ++i) put3(&v[3 * i], mesh.vertexBuffer[i]);
        std::vector<int32_t> idx(3 * mesh.indexBuffer.size());
        for (size_t i = 0; i < mesh.indexBuffer.size(); ++i) {
            idx[3 * i] = mesh.indexBuffer[i].v0;
            idx[3 * i + 1] = mesh.indexBuffer[i].v1;
            idx[3 * i + 2] = mesh.indexBuffer[i].v2;
        }
        check(hsr_scene_create(v.data(), int64_t(mesh.vertexBuffer.size()), idx.data(),
                               int64_t(mesh.indexBuffer.size()), &m_scene));
        // the integrator is held by reference and must outlive the backend (arch/cpu.h:21)
        m_run = [this, &integrator](const SceneView &sv, long budget, bool *interruptFlag) {
            using A = BackendAccess<Integrator>;
            auto &frame = A::frame(integrator);
            auto fc = frame.config();
            hsr_frame_config f{fc.chirpCount, fc.samplesPerChirp, fc.channelCount};
            const size_t n = size_t(fc.chirpCount) * fc.samplesPerChirp * fc.channelCount;
            std::vector<float> buf(2 * n);
            for (size_t i = 0; i < n; ++i) {
                buf[2 * i] = frame(i).real();
                buf[2 * i + 1] = frame(i).imag();
            }
            hsr_tracer_flags fl = to_hsr_flags(integrator);
            double w = A::totalWeight(integrator);
            int32_t flag = (interruptFlag && *interruptFlag) ? 1 : 0;
            hsr_status s;
            if (fl.doGuiding) {
                const bool final_iteration = A::isFinalIteration(integrator);
                if (!m_guide) check(hsr_guide_create(m_scene, &m_guide));
                if (!final_iteration && budget <= 16384)
                    check(hsr_guide_reset(m_guide));  // a new PathTracer::run (path.h:180-185)
                else
                    check(hsr_guide_step(m_guide));  // stepGuiding() after the previous iteration
                s = hsr_backend_run_guided(m_scene, &sv.rf, &f, &sv.tx, &sv.rx, &fl, budget,
                                           A::sampleIndexOffset(integrator), A::currentSampleWeight(integrator),
                                           final_iteration ? 0 : 1, m_guide, HSR_PHASE_REFERENCE_FP32, buf.data(),
                                           &w, &flag);
            } else {
                s = hsr_backend_run(m_scene, &sv.rf, &f, &sv.tx, &sv.rx, &fl, budget,
                                    A::sampleIndexOffset(integrator), A::currentSampleWeight(integrator),
                                    HSR_PHASE_REFERENCE_FP32, buf.data(), &w, &flag);
            }
            check(s);
            if (s == HSR_ERR_INTERRUPTED) return;
            for (size_t i = 0; i < n; ++i) {
                frame(i).real() = buf[2 * i];
                frame(i).imag() = buf[2 * i + 1];
            }
            A::setTotalWeight(integrator, w);
        };
    }

    Backend(const Backend &) = delete;
    Backend &operator=(const Backend &) = delete;

    ~Backend() {
        hsr_guide_destroy(m_guide);
        hsr_scene_destroy(m_scene);
    }

    template <typename Scene> void run(const Scene &scene, long budget, bool *interruptFlag = nullptr) {
        SceneView sv{to_hsr_rf(scene.rfConfig), to_hsr(scene.tx), to_hsr(scene.rx)};
        m_run(sv, budget, interruptFlag);
    }

    hsr_scene *handle() const { return m_scene; }

private:
    hsr_scene *m_scene = nullptr;
    hsr_guide *m_guide = nullptr;  // the guided schedule's device tree (created on first use)
    std::function<void(const SceneView &, long, bool *)> m_run;
};

/* A serving loop over resident scenes (hsr_server_*): requests from any thread, traced
 * in shared batching ticks. No counterpart in the reference, whose backends trace one
 * pose per synchronous run() (src/arch/gpu.cpp:499-532). The tracer flags come from an
 * integrator (its public flags of path.h:153-169; with doGuiding every request runs the
 * guided schedule). A request's row is the fetchFrame() row of a run of `budget`
 * samples at index offset `offset`. */
class Server {
public:
    explicit Server(const hsr_server_config &config) { check(hsr_server_create(&config, &m_server)); }

    template <typename Integrator>
    explicit Server(const Integrator &integrator, int32_t phase_mode = HSR_PHASE_REFERENCE_FP32,
                    int32_t max_slots = 0, int64_t memory_bytes = 0) {
        hsr_server_config c;
        hsr_default_server_config(&c);
        c.flags = to_hsr_flags(integrator);
        c.phase_mode = phase_mode;
        if (max_slots > 0) c.max_slots = max_slots;
        if (memory_bytes > 0) c.memory_bytes = memory_bytes;
        check(hsr_server_create(&c, &m_server));
    }

    Server(const Server &) = delete;
    Server &operator=(const Server &) = delete;
    /* Finishes the device work; requests still queued fail with HSR_ERR_INTERRUPTED. */
    ~Server() { hsr_server_destroy(m_server); }

    /* The backend's scene stays resident; it must outlive the server. */
    int32_t addScene(const Backend &backend) {
        int32_t id = -1;
        check(hsr_server_add_scene(m_server, backend.handle(), &id));
        return id;
    }

    /* Queues one pose; `out_row` (complex64[samples_per_chirp], as float re/im pairs) must
     * stay valid until wait() reports the ticket finished. */
    template <typename Scene>
    uint64_t submit(int32_t scene_id, const Scene &scene, int32_t samples_per_chirp, long budget, float *out_row,
                    long index_offset = 0) {
        hsr_request r;
        r.scene = scene_id;
        r.samples_per_chirp = samples_per_chirp;
        r.rf = to_hsr_rf(scene.rfConfig);
        r.tx = to_hsr(scene.tx);
        r.rx = to_hsr(scene.rx);
        r.budget = int64_t(budget);
        r.index_offset = int64_t(index_offset);
        r.out_row = out_row;
        uint64_t ticket = 0;
        check(hsr_server_submit(m_server, &r, &ticket));
        return ticket;
    }

    /* Blocks until the request finishes (timeout_ms < 0) or the timeout passes; returns
     * false on a timeout. A request that failed throws. */
    bool wait(uint64_t ticket, hsr_request_result *result = nullptr, int32_t timeout_ms = -1) {
        hsr_request_result r;
        hsr_status s = hsr_server_wait(m_server, ticket, timeout_ms, &r);
        if (s == HSR_ERR_TIMEOUT) return false;
        check(s);
        if (r.status != HSR_OK)
            throw std::runtime_error("gb300: request failed with status " + std::to_string(r.status));
        if (result) *result = r;
        return true;
    }

    hsr_server_stats stats() const {
        hsr_server_stats s;
        check(hsr_server_get_stats(m_server, &s));
        return s;
    }

    void resetStats() { check(hsr_server_reset_stats(m_server)); }

    hsr_server *handle() const { return m_server; }

private:
    hsr_server *m_server = nullptr;
};

}  // namespace gb300
}  // namespace hussar

#endif
