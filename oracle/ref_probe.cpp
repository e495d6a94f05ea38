/*
 * ORACLE — TEST INFRASTRUCTURE ONLY.
 * Exposes pieces of the reference that compile without Eigen/Embree/OptiX, built
 * straight from the reference's own headers by oracle/Makefile.ref:
 *   - hussar::radicalInverse (libhussar/include/hussar/samplers/halton.h:38-67)
 *   - radar::Frame::PIndex::setTime (libradar/include/radar/radar.h:232-241)
 *   - radar::Frame::splat<16> (libradar/include/radar/radar.h:564-626)
 *   - radar's std::exp(complex) -> polar (libradar/include/radar/complex.h:184-187, 249-251)
 * The outputs pin the oracle's restatement (tests/golden/make_golden.py).
 */
#include <cstdint>
#include <memory>
#include <hussar/hussar.h>
#include <hussar/core/logging.h>
#define HUSSAR_CORE_SAMPLER_H  // sampler.h needs Eigen; halton.h only needs Vector2f from it
namespace hussar {
struct Vector2f {
    float a, b;
    Vector2f(float x, float y) : a(x), b(y) {}
};
}  // namespace hussar
#include <hussar/samplers/halton.h>
#include <radar/radar.h>

using RefFrame = radar::Frame<std::allocator<radar::Complex>>;

extern "C" {

float ref_radical_inverse(uint64_t index, int dim) { return hussar::radicalInverse(index, uint16_t(dim)); }

float ref_halton_sample(uint64_t index, int dims, float *out) {
    hussar::HaltonSampler s;
    s.setSampleIndex(long(index));
    for (int i = 0; i < dims; ++i) out[i] = s.get1D();
    return dims > 0 ? out[0] : 0.f;
}

float ref_set_time(float delta_t, float startFreq, float freqSlope, float adcRate, int samplesPerChirp) {
    radar::RFConfig rf{};
    rf.startFreq = startFreq;
    rf.freqSlope = freqSlope;
    rf.adcRate = adcRate;
    radar::FrameConfig fc{};
    fc.chirpCount = 1;
    fc.samplesPerChirp = samplesPerChirp;
    fc.channelCount = 1;
    RefFrame::PIndex idx;
    idx.setTime(delta_t, rf, fc);
    return idx.sample;
}

/* frame: chirps*samples*channels complex64 (interleaved), ADDED to */
void ref_frame_splat(int chirps, int samples, int channels, float ic, float is, float ich, float re, float im,
                     float *frame) {
    radar::FrameConfig fc{};
    fc.chirpCount = chirps;
    fc.samplesPerChirp = samples;
    fc.channelCount = channels;
    RefFrame f;
    f.configure(fc);
    f.clear();
    RefFrame::PIndex idx;
    idx.chirp = ic;
    idx.sample = is;
    idx.channel = ich;
    f.splat(idx, radar::Complex(re, im));
    for (size_t i = 0; i < f.sampleCount(); ++i) {
        frame[2 * i] += f(i).real();
        frame[2 * i + 1] += f(i).imag();
    }
}

void ref_cexp(float angle, float *out2) {
    radar::Complex c = std::exp(radar::Complex(0, angle));
    out2[0] = c.real();
    out2[1] = c.imag();
}
}
