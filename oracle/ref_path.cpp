/*
 * ORACLE — TEST INFRASTRUCTURE ONLY.
 *
 * Runs the reference's own integrator on the CPU: PathTracer::run and PathTracer::sample
 * (libhussar/include/hussar/integrators/path.h:171-451) with the reference's emitters,
 * geometry, intersection, integrator splat and radar frame
 * (core/emitter.h, core/geometry.h, core/intersection.h, core/integrator.h,
 * samplers/halton.h, libradar/include/radar/radar.h), compiled from the reference tree
 * in place by oracle/Makefile.ref into oracle/_ref/libhsr_refpath.so. What the reference
 * takes from absent third-party code is supplied here or by oracle/ref_shim/:
 *   - Eigen: a stand-in for the fixed-size dense subset the path uses (ref_shim/Eigen);
 *   - libguiding: a uniform stub, so only doGuiding = false is run;
 *   - Embree: the backend's RT (src/arch/cpu.cpp:9-87) below, with the oracle's BVH for
 *     the closest-hit and occlusion queries (tnear = Epsilon, tfar = isect.tMax) and the
 *     hit's normal formed as cpu.cpp does (geometric normal, normalized, faceforwarded);
 *     the geometric normal is (v1 - v0) x (v2 - v0);
 *   - the debug-image EXR/tev writers: no-op stand-ins (off the hot path).
 * The backend traces the samples of cpu::Backend::run (arch/cpu.h:18-46) on one thread,
 * in index order, so float frame sums are added in a fixed order.
 *
 * The outputs pin the restatement in hsr_oracle.cpp (tests/golden/make_golden.py records
 * them; tests/test_oracle_golden.py compares).
 */
#include <cstdint>
#include <cstring>
#include <memory>

#include <hussar/integrators/path.h>

#include "hsr_oracle.h"

namespace {

struct OracleRT {
    void *scene;
    const float *v;
    const int32_t *f;

    // Backend::RT::visible (src/arch/cpu.cpp:53-61): occlusion on (Epsilon, tMax)
    bool visible(hussar::Intersection &isect) const {
        const float o[3] = {isect.ray.o.x(), isect.ray.o.y(), isect.ray.o.z()};
        const float d[3] = {isect.ray.d.x(), isect.ray.d.y(), isect.ray.d.z()};
        const float tfar = isect.tMax;
        int32_t vis = 0;
        oracle_visible(scene, 1, o, d, &tfar, &vis);
        return vis != 0;
    }

    // Backend::RT::intersect (src/arch/cpu.cpp:63-87)
    void intersect(hussar::Intersection &isect) const {
        const float o[3] = {isect.ray.o.x(), isect.ray.o.y(), isect.ray.o.z()};
        const float d[3] = {isect.ray.d.x(), isect.ray.d.y(), isect.ray.d.z()};
        const float tfar = isect.tMax;
        float t = 0.f, p[3], n[3];
        int32_t prim = -1;
        oracle_intersect(scene, 1, o, d, &tfar, &t, p, n, &prim);
        if (prim >= 0) {
            const float *a = v + 3 * f[3 * prim], *b = v + 3 * f[3 * prim + 1], *c = v + 3 * f[3 * prim + 2];
            const hussar::Vector3f v0(a[0], a[1], a[2]), v1(b[0], b[1], b[2]), v2(c[0], c[1], c[2]);
            const hussar::Vector3f ng = (v1 - v0).cross(v2 - v0);
            isect.t = t;
            isect.p = isect.ray(isect.t);
            isect.n = hussar::Vector3f(ng.x(), ng.y(), ng.z()).normalized();
            if (isect.n.dot(isect.ray.d) > 0) {
                // faceforward
                isect.n = -isect.n;
            }
        }
    }
};

// cpu::Backend's sample loop on one thread (arch/cpu.h:21-41 with a single worker)
struct OneThreadBackend {
    hussar::PathTracer &integrator;
    OracleRT rt;
    void run(const hussar::Scene &scene, long budget, bool *interruptFlag = nullptr) {
        for (long i = 0; i < budget && !(interruptFlag && *interruptFlag); ++i) integrator.sample(scene, rt, i);
    }
};

// The tracer with read access to the raw frame sums and the total weight (protected in
// Integrator / PathTracer, path.h:457-464, integrator.h:170).
struct Probe : hussar::PathTracer {
    const hussar::RadarFrame &raw() const { return frame; }
    double weight() const { return totalWeight; }
};

hussar::NFAntenna antenna(const hsr_antenna_o &a) {
    hussar::Matrix33f rot;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) rot(i, j) = a.rotation[3 * i + j];
    return hussar::NFAntenna(hussar::Vector3f(a.position[0], a.position[1], a.position[2]), rot,
                             hussar::AWRAngularDistribution());
}

}  // namespace

extern "C" {

/* PathTracer::run(backend, scene, budget) with doGuiding = false (path.h:171-182) on the
 * mesh, then the frame's raw sums (complex64 [chirp][sample][channel], interleaved) and
 * totalWeight. libm_trig: the oracle's trig mode for its own ray queries is irrelevant
 * here (the reference's UniformSampleSphere uses the platform's sinf/cosf). */
int ref_path_frame(const float *vertices, int64_t nv, const int32_t *indices, int64_t nt, const hsr_rf_config_o *rf,
                   const hsr_frame_config_o *fc, const hsr_antenna_o *tx, const hsr_antenna_o *rx,
                   const hsr_tracer_flags_o *fl, int64_t budget, float *frame_out, double *weight_out) {
    if (fl->doGuiding) return 2;  // libguiding is absent: the plain method only
    void *sc = oracle_scene_create(vertices, nv, indices, nt);
    if (!sc) return 1;
    {
        std::unique_ptr<Probe> pt(new Probe());
        pt->onlyIndirect = fl->onlyIndirect != 0;
        pt->maxDepth = fl->maxDepth;
        pt->useGeometricalOptics = fl->useGeometricalOptics != 0;
        pt->poDiffraction = fl->poDiffraction != 0;
        pt->doGuiding = false;
        pt->clearBeforeIteration = fl->clearBeforeIteration != 0;
        pt->correctPhase = fl->correctPhase != 0;
        pt->filterGuiding = fl->filterGuiding != 0;
        pt->doFiltering = fl->doFiltering != 0;
        pt->filteringSphere = fl->filteringSphere != 0;
        pt->filteringMin = fl->filteringMin;
        pt->filteringMax = fl->filteringMax;
        pt->filteringRadius = fl->filteringRadius;
        pt->produceDebugImage = fl->produceDebugImage != 0;
        radar::FrameConfig cfg;
        cfg.chirpCount = fc->chirpCount;
        cfg.samplesPerChirp = fc->samplesPerChirp;
        cfg.channelCount = fc->channelCount;
        pt->configureFrame(cfg);
        hussar::Scene scene;
        scene.rfConfig.startFreq = rf->startFreq;
        scene.rfConfig.freqSlope = rf->freqSlope;
        scene.rfConfig.adcRate = rf->adcRate;
        scene.rfConfig.idleTime = rf->idleTime;
        scene.rfConfig.rampTime = rf->rampTime;
        scene.rfConfig.antennaDelay = rf->antennaDelay;
        scene.tx = antenna(*tx);
        scene.rx = antenna(*rx);
        OneThreadBackend be{*pt, OracleRT{sc, vertices, indices}};
        pt->run(be, scene, long(budget));
        const size_t n = cfg.sampleCount();
        for (size_t i = 0; i < n; ++i) {
            const radar::Complex c = const_cast<hussar::RadarFrame &>(pt->raw())(i);
            frame_out[2 * i] = c.real();
            frame_out[2 * i + 1] = c.imag();
        }
        *weight_out = pt->weight();
    }
    oracle_scene_destroy(sc);
    return 0;
}

/* Integrator::measureRay (integrator.h:107-110) as the reference compiles it. */
void ref_measure_ray(float delta_t, float startFreq, float freqSlope, float *out2) {
    struct M : hussar::PathTracer {
        radar::Complex at(float dt, const radar::RFConfig &rf) const { return measureRay(dt, rf); }
    } m;
    radar::RFConfig rf{};
    rf.startFreq = startFreq;
    rf.freqSlope = freqSlope;
    const radar::Complex c = m.at(delta_t, rf);
    out2[0] = c.real();
    out2[1] = c.imag();
}

/* UniformSampleSphere (core/sampling.h:38-43) as the reference compiles it. */
void ref_uniform_sample_sphere(float u0, float u1, float *d) {
    const hussar::Vector3f v = hussar::UniformSampleSphere(hussar::Vector2f(u0, u1));
    d[0] = v.x();
    d[1] = v.y();
    d[2] = v.z();
}

/* HaltonSampler::get2D (samplers/halton.h:23-26) after `dims` get1D calls, as the compiler
 * of this library ordered the two get1D calls of its Vector2f(get1D(), get1D()). */
void ref_halton_get2d(uint64_t index, int dims, float *out2) {
    hussar::HaltonSampler s;
    s.setSampleIndex(long(index));
    for (int i = 0; i < dims; ++i) s.get1D();
    const hussar::Vector2f v = s.get2D();
    out2[0] = v.x();
    out2[1] = v.y();
}

}  // extern "C"
