/*
 * hussar/gb300_types.h — self-contained mirror of the libhussar / libradar types a
 * program needs to drive the GB300 backend without libhussar, Eigen or libguiding:
 *
 *   radar::RFConfig, radar::FrameConfig, radar::Frame   libradar/include/radar/radar.h:113-701
 *   hussar::Vector3f, hussar::Matrix33f                 (the Eigen types of core/geometry.h:12-33)
 *   hussar::TriangleMesh (addQuad, addBox)              libhussar/include/hussar/core/mesh.h:14-55
 *   hussar::WavefrontFile (OBJ input)                   libhussar/include/hussar/io/wavefront.h:12-67
 *   hussar::AWRAngularDistribution, hussar::NFAntenna   libhussar/include/hussar/core/emitter.h:109-214
 *   hussar::Scene                                       libhussar/include/hussar/core/scene.h:9-14
 *   hussar::PathTracer (flags, run, fetchFrame)         libhussar/include/hussar/integrators/path.h:133-476
 *
 * Same names, members and meaning as the reference, so example programs such as
 * examples/src/1_dihedral.cpp read the same. PathTracer::run follows path.h's schedule:
 * one backend run, or with doGuiding = true (the default) the doubling iterations, the
 * guiding tree living in the backend.
 */
#ifndef HUSSAR_GB300_TYPES_H
#define HUSSAR_GB300_TYPES_H

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../hsr_gb300.h"

namespace radar {

using Float = float;
constexpr float SPEED_OF_LIGHT = 299792458;

struct RFConfig {
    Float startFreq = 0, freqSlope = 0, adcRate = 0, idleTime = 0, rampTime = 0, antennaDelay = 0;
    Float bandwidth() const { return freqSlope * rampTime; }
    Float chirpFrequency() const { return 1.f / (idleTime + rampTime); }
};

struct FrameConfig {
    int chirpCount = 1, samplesPerChirp = 1, channelCount = 1;
    size_t sampleCount() const { return size_t(chirpCount) * samplesPerChirp * channelCount; }
};

/* A complex64 radar cube [chirp][sample][channel]. */
struct Frame {
    struct Complex {
        float re = 0, im = 0;
        float &real() { return re; }
        float &imag() { return im; }
        float real() const { return re; }
        float imag() const { return im; }
    };

    void configure(const FrameConfig &c) {
        m_config = c;
        m_data.assign(c.sampleCount(), Complex{});
    }
    void clear() {
        for (auto &c : m_data) c = Complex{};
    }
    FrameConfig config() const { return m_config; }
    size_t sampleCount() const { return m_config.sampleCount(); }
    Complex &operator()(size_t i) { return m_data[i]; }
    const Complex &operator()(size_t i) const { return m_data[i]; }
    Frame operator/(Float f) const {
        Frame r = *this;
        float s = 1.f / f;
        for (auto &c : r.m_data) {
            c.re *= s;
            c.im *= s;
        }
        return r;
    }

private:
    FrameConfig m_config;
    std::vector<Complex> m_data;
};

}  // namespace radar

namespace hussar {

using Float = float;
constexpr Float Pi = 3.14159265358979323846f;

struct Vector3f {
    float v[3] = {0, 0, 0};
    Vector3f() = default;
    Vector3f(float x, float y, float z) : v{x, y, z} {}
    float x() const { return v[0]; }
    float y() const { return v[1]; }
    float z() const { return v[2]; }
    float operator[](int i) const { return v[i]; }
    Vector3f operator+(const Vector3f &o) const { return {v[0] + o.v[0], v[1] + o.v[1], v[2] + o.v[2]}; }
    Vector3f operator-(const Vector3f &o) const { return {v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]}; }
};

struct Matrix33f {
    float m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    float operator()(int r, int c) const { return m[3 * r + c]; }
    float &operator()(int r, int c) { return m[3 * r + c]; }
    Matrix33f operator*(const Matrix33f &o) const {
        Matrix33f r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r(i, j) = (*this)(i, 0) * o(0, j) + ((*this)(i, 1) * o(1, j) + (*this)(i, 2) * o(2, j));
        return r;
    }
    Vector3f operator*(const Vector3f &v) const {
        return {m[0] * v.x() + (m[1] * v.y() + m[2] * v.z()), m[3] * v.x() + (m[4] * v.y() + m[5] * v.z()),
                m[6] * v.x() + (m[7] * v.y() + m[8] * v.z())};
    }
    /* Eigen::AngleAxisf(angle, UnitY).toRotationMatrix() */
    static Matrix33f rotationY(float angle) {
        Matrix33f r;
        float c = std::cos(angle), s = std::sin(angle);
        r.m[0] = c, r.m[1] = 0, r.m[2] = s;
        r.m[3] = 0, r.m[4] = 1, r.m[5] = 0;
        r.m[6] = -s, r.m[7] = 0, r.m[8] = c;
        return r;
    }
};

struct TriangleMesh {
    struct IndexTriplet {
        int v0, v1, v2;
    };
    std::vector<Vector3f> vertexBuffer;
    std::vector<IndexTriplet> indexBuffer;

    void addQuad(const Vector3f &a, const Vector3f &b, const Vector3f &c) {
        int i = int(vertexBuffer.size());
        vertexBuffer.push_back(a);
        vertexBuffer.push_back(a + b);
        vertexBuffer.push_back(a + b + c);
        vertexBuffer.push_back(a + c);
        indexBuffer.push_back({i + 0, i + 1, i + 2});
        indexBuffer.push_back({i + 0, i + 2, i + 3});
    }

    void addBox(const Vector3f &mn, const Vector3f &mx) {
        Vector3f d = mx - mn;
        addQuad(mn, Vector3f(0.f, d.y(), 0.f), Vector3f(0.f, 0.f, d.z()));
        addQuad(mn, Vector3f(0.f, 0.f, d.z()), Vector3f(d.x(), 0.f, 0.f));
        addQuad(mn, Vector3f(d.x(), 0.f, 0.f), Vector3f(0.f, d.y(), 0.f));
        d = mn - mx;
        addQuad(mx, Vector3f(0.f, d.y(), 0.f), Vector3f(d.x(), 0.f, 0.f));
        addQuad(mx, Vector3f(0.f, 0.f, d.z()), Vector3f(0.f, d.y(), 0.f));
        addQuad(mx, Vector3f(d.x(), 0.f, 0.f), Vector3f(0.f, 0.f, d.z()));
    }
};

/* hussar::WavefrontFile (io/wavefront.h:12-67): read(mesh) appends an OBJ file's vertices
 * and triangles to the mesh, indices shifted by the vertices it already holds; parsed by
 * the library (hsr_read_obj). The reference logs an error and exits on a bad file; this
 * throws std::runtime_error. */
class WavefrontFile {
public:
    explicit WavefrontFile(const std::string &path) : m_path(path) {}

    void read(TriangleMesh &mesh) {
        int64_t nv = 0, nt = 0;
        const int64_t offset = int64_t(mesh.vertexBuffer.size());
        if (hsr_read_obj(m_path.c_str(), offset, nullptr, 0, nullptr, 0, &nv, &nt, nullptr) != HSR_OK)
            throw std::runtime_error(std::string("WavefrontFile: ") + hsr_last_error());
        std::vector<float> v(3 * size_t(nv));
        std::vector<int32_t> f(3 * size_t(nt));
        if (hsr_read_obj(m_path.c_str(), offset, v.data(), nv, f.data(), nt, &nv, &nt, nullptr) != HSR_OK)
            throw std::runtime_error(std::string("WavefrontFile: ") + hsr_last_error());
        for (int64_t i = 0; i < nv; ++i) mesh.vertexBuffer.push_back(Vector3f(v[3 * i], v[3 * i + 1], v[3 * i + 2]));
        for (int64_t i = 0; i < nt; ++i) mesh.indexBuffer.push_back({f[3 * i], f[3 * i + 1], f[3 * i + 2]});
    }

private:
    std::string m_path;
};

struct AWRAngularDistribution {};

class NFAntenna {
public:
    NFAntenna() = default;
    NFAntenna(const Vector3f &position, const Matrix33f &rotation, const AWRAngularDistribution & = {})
        : m_position(position), m_rotation(rotation) {
        const Matrix33f &r = m_rotation;
        double det = double(r(0, 0)) * (double(r(1, 1)) * r(2, 2) - double(r(1, 2)) * r(2, 1)) -
                     double(r(0, 1)) * (double(r(1, 0)) * r(2, 2) - double(r(1, 2)) * r(2, 0)) +
                     double(r(0, 2)) * (double(r(1, 0)) * r(2, 1) - double(r(1, 1)) * r(2, 0));
        if (std::abs(std::abs(det) - 1) >= 1e-2)  // emitter.h:166-169
            throw std::invalid_argument("supplied rotation matrix is - in fact - not a rotation matrix!");
    }
    const Vector3f &position() const { return m_position; }
    const Matrix33f &rotation() const { return m_rotation; }

private:
    Vector3f m_position;
    Matrix33f m_rotation;
};

struct Scene {
    radar::RFConfig rfConfig;
    NFAntenna rx;
    NFAntenna tx;
};

namespace gb300 {
template <typename Integrator> struct BackendAccess;
}

class PathTracer {
public:
    bool onlyIndirect = true;
    int maxDepth = 10;
    bool useGeometricalOptics = true;
    bool poDiffraction = false;
    bool doGuiding = true;
    bool clearBeforeIteration = true;
    bool correctPhase = false;
    bool filterGuiding = true;
    bool doFiltering = true;
    bool filteringSphere = true;
    Float filteringMin = 600;
    Float filteringMax = 900;
    Float filteringRadius = 160;
    bool produceDebugImage = false;

    void configureFrame(const radar::FrameConfig &c) { frame.configure(c); }

    // PathTracer::run (path.h:171-224): one backend run, or with guiding the doubling
    // schedule from 16384 samples whose last iteration takes the remainder; the backend
    // keeps the guiding tree and steps it between iterations
    template <typename Backend> void run(Backend &backend, const Scene &scene, long samples,
                                         bool *interruptFlag = nullptr) {
        frame.clear();
        totalWeight = 0;
        sampleIndexOffset = 0;
        currentSampleWeight = 1.f;
        if (!doGuiding) {
            backend.run(scene, samples, interruptFlag);
            return;
        }
        isFinalIteration = false;
        long milestone = 16384;
        long remainingSamples = samples;
        while (true) {
            milestone = std::min(milestone, remainingSamples);
            backend.run(scene, milestone, interruptFlag);
            if (interruptFlag && *interruptFlag) return;
            sampleIndexOffset += milestone;
            remainingSamples -= milestone;
            if (remainingSamples == 0) break;
            milestone *= 2;
            if (remainingSamples < milestone * 2) {
                isFinalIteration = true;
                milestone = remainingSamples;
            }
            if (clearBeforeIteration) {
                frame.clear();
                totalWeight = 0;
                sampleIndexOffset = 0;
            } else {
                currentSampleWeight = 10 * currentSampleWeight;
            }
        }
    }

    radar::Frame fetchFrame() const { return frame / Float(totalWeight); }

protected:
    template <typename> friend struct gb300::BackendAccess;
    radar::Frame frame;
    double totalWeight = 0;
    long sampleIndexOffset = 0;
    Float currentSampleWeight = 1.f;
    bool isFinalIteration = false;
};

}  // namespace hussar

#endif
