// A scene read from an OBJ file (hussar::WavefrontFile, io/wavefront.h:12-67) and traced
// through the C++ drop-in: the reference's flow of examples/src/2_large_scene.cpp:135-160
// (read the mesh, build the backend once, run the integrator per pose).
//
// usage: obj_example <scene.obj> <out.SIM> <samples> <max_depth> <N> <adc_rate> <12 floats: position, row-major rotation>
#include <hussar/gb300.h>
#include <hussar/gb300_types.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>

using namespace hussar;

int main(int argc, char **argv) {
    if (argc < 19) {
        std::fprintf(stderr, "usage: %s scene.obj out.SIM samples max_depth N adc_rate x y z r00..r22\n", argv[0]);
        return 2;
    }
    const long samples = std::atol(argv[3]);
    radar::RFConfig rf;
    rf.antennaDelay = 0.43e-9f;
    rf.startFreq = 77e9f;
    rf.freqSlope = 4e9f / 51.2e-6f;
    rf.adcRate = float(std::atof(argv[6]));
    rf.idleTime = 100e-6f;
    rf.rampTime = 51.2e-6f;
    radar::FrameConfig frameConfig;
    frameConfig.chirpCount = 1;
    frameConfig.samplesPerChirp = std::atoi(argv[5]);
    frameConfig.channelCount = 1;
    try {
        TriangleMesh mesh;
        WavefrontFile(argv[1]).read(mesh);
        Scene scene;
        scene.rfConfig = rf;
        Matrix33f rot;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) rot(i, j) = float(std::atof(argv[10 + 3 * i + j]));
        scene.tx = NFAntenna{Vector3f(float(std::atof(argv[7])), float(std::atof(argv[8])), float(std::atof(argv[9]))),
                             rot, AWRAngularDistribution()};
        scene.rx = scene.tx;
        PathTracer integrator;
        integrator.doGuiding = false;
        integrator.maxDepth = std::atoi(argv[4]);
        integrator.configureFrame(frameConfig);
        gb300::Backend backend{mesh, integrator};
        integrator.run(backend, scene, samples);
        radar::Frame frame = integrator.fetchFrame();
        std::ofstream file(argv[2], std::ios::binary);
        for (size_t i = 0; i < frame.sampleCount(); ++i) {
            float v[2] = {frame(i).real(), frame(i).imag()};
            file.write(reinterpret_cast<const char *>(v), sizeof(v));
        }
        std::printf("%zu vertices, %zu triangles\n", mesh.vertexBuffer.size(), mesh.indexBuffer.size());
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
