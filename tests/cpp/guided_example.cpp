// The reference's default integrator (doGuiding = true, path.h:158) through the C++
// drop-in: PathTracer::run's doubling schedule (path.h:171-224) calls gb300::Backend::run
// once per iteration; the backend keeps the device guiding tree and steps it between
// iterations. Writes each pose's fetchFrame() as raw complex64 and its total weight.
//
// usage: guided_example <out.SIM> <poses> <samples>
#include <hussar/gb300.h>
#include <hussar/gb300_types.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>

using namespace hussar;

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s out.SIM poses samples\n", argv[0]);
        return 2;
    }
    const int poses = std::atoi(argv[2]);
    const long samples = std::atol(argv[3]);
    radar::RFConfig rf;
    rf.antennaDelay = 0.43e-9f;
    rf.startFreq = 77e9f;
    rf.freqSlope = 4e9f / 51.2e-6f;
    rf.adcRate = 5e6f;
    rf.idleTime = 100e-6f;
    rf.rampTime = 51.2e-6f;
    radar::FrameConfig frameConfig;
    frameConfig.chirpCount = 1;
    frameConfig.samplesPerChirp = 256;
    frameConfig.channelCount = 1;
    TriangleMesh mesh;
    const float size = 0.1f;
    mesh.addQuad(Vector3f(0, 0, 0), Vector3f(0, size, 0), Vector3f(0, 0, size));
    mesh.addQuad(Vector3f(0, 0, 0), Vector3f(size, 0, 0), Vector3f(0, size, 0));
    Scene scene;
    scene.rfConfig = rf;
    PathTracer integrator;  // doGuiding = true: the reference's default
    integrator.maxDepth = 2;
    integrator.configureFrame(frameConfig);
    try {
        gb300::Backend backend{mesh, integrator};
        std::ofstream file(argv[1], std::ios::binary);
        Matrix33f facing;
        facing(0, 0) = 0, facing(0, 1) = 0, facing(0, 2) = -1;
        facing(1, 0) = 0, facing(1, 1) = -1, facing(1, 2) = 0;
        facing(2, 0) = -1, facing(2, 1) = 0, facing(2, 2) = 0;
        for (int k = 0; k < poses; ++k) {
            float th = (90.f * k / float(poses > 1 ? poses - 1 : 1)) / 180.f * Pi;
            Matrix33f rotation = Matrix33f::rotationY(-th);
            Vector3f position(std::cos(th), size / 2, std::sin(th));
            scene.tx = NFAntenna{position, rotation * facing, AWRAngularDistribution()};
            scene.rx = scene.tx;
            integrator.run(backend, scene, samples);
            radar::Frame frame = integrator.fetchFrame();
            for (size_t i = 0; i < frame.sampleCount(); ++i) {
                float v[2] = {frame(i).real(), frame(i).imag()};
                file.write(reinterpret_cast<const char *>(v), sizeof(v));
            }
        }
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
