// Serving through the C++ wrapper (hussar::gb300::Server in include/hussar/gb300.h):
// the dihedral of examples/src/1_dihedral.cpp:23-127 kept resident, its poses submitted
// from several client threads at once, each request waited on by the thread that made
// it. Writes every pose's row as raw complex64 in pose order, like the example's .SIM.
//
// usage: serve_example <out.SIM> <poses> <samples> <threads>
// Also writes <out.SIM>.poses: per pose 12 floats (position, row-major rotation).
#include <hussar/gb300.h>
#include <hussar/gb300_types.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <thread>
#include <vector>

using namespace hussar;

int main(int argc, char **argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s out.SIM poses samples threads\n", argv[0]);
        return 2;
    }
    const int poses = std::atoi(argv[2]);
    const long samples = std::atol(argv[3]);
    const int threads = std::atoi(argv[4]);
    const int N = 256;

    Scene scene;
    scene.rfConfig.antennaDelay = 0.43e-9f;
    scene.rfConfig.startFreq = 77e9f;
    scene.rfConfig.freqSlope = 4e9f / 51.2e-6f;
    scene.rfConfig.adcRate = 5e6f;
    scene.rfConfig.idleTime = 100e-6f;
    scene.rfConfig.rampTime = 51.2e-6f;

    TriangleMesh mesh;
    const float size = 0.1f;
    mesh.addQuad(Vector3f(0, 0, 0), Vector3f(0, size, 0), Vector3f(0, 0, size));
    mesh.addQuad(Vector3f(0, 0, 0), Vector3f(size, 0, 0), Vector3f(0, size, 0));

    PathTracer integrator;
    integrator.doGuiding = false;
    integrator.maxDepth = 2;

    Matrix33f facing;
    facing(0, 0) = 0, facing(0, 1) = 0, facing(0, 2) = -1;
    facing(1, 0) = 0, facing(1, 1) = -1, facing(1, 2) = 0;
    facing(2, 0) = -1, facing(2, 1) = 0, facing(2, 2) = 0;
    std::vector<Scene> pose(poses, scene);
    for (int k = 0; k < poses; ++k) {
        float th = (90.f * k / float(poses > 1 ? poses - 1 : 1)) / 180.f * Pi;
        Vector3f position(std::cos(th), size / 2, std::sin(th));
        pose[k].tx = NFAntenna{position, Matrix33f::rotationY(-th) * facing, AWRAngularDistribution()};
        pose[k].rx = pose[k].tx;
    }

    std::vector<float> rows(size_t(poses) * 2 * N, 0.f);
    try {
        gb300::Backend backend{mesh, integrator};
        gb300::Server server{integrator, HSR_PHASE_REFERENCE_FP32, 64};
        const int id = server.addScene(backend);
        std::vector<std::thread> clients;
        std::vector<std::string> errors(threads);
        for (int t = 0; t < threads; ++t) {
            clients.emplace_back([&, t] {
                try {
                    // each client owns the poses k = t mod threads and keeps two in flight
                    std::vector<uint64_t> inflight;
                    for (int k = t; k < poses; k += threads) {
                        inflight.push_back(server.submit(id, pose[k], N, samples, &rows[size_t(k) * 2 * N]));
                        if (inflight.size() == 2) {
                            server.wait(inflight.front());
                            inflight.erase(inflight.begin());
                        }
                    }
                    for (uint64_t tk : inflight) server.wait(tk);
                } catch (const std::exception &e) {
                    errors[t] = e.what();
                }
            });
        }
        for (auto &c : clients) c.join();
        for (auto &e : errors)
            if (!e.empty()) throw std::runtime_error(e);
        hsr_server_stats st = server.stats();
        std::printf("completed %lld failed %lld ticks %lld max_batch %d p50 %.3f ms p99 %.3f ms\n",
                    (long long)st.completed, (long long)st.failed, (long long)st.ticks, st.max_batch, st.p50_ms,
                    st.p99_ms);
        if (st.completed != poses || st.failed != 0) throw std::runtime_error("request count mismatch");
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    std::ofstream file(argv[1], std::ios::binary);
    file.write(reinterpret_cast<const char *>(rows.data()), rows.size() * sizeof(float));
    std::ofstream posefile(std::string(argv[1]) + ".poses", std::ios::binary);
    for (int k = 0; k < poses; ++k) {
        posefile.write(reinterpret_cast<const char *>(pose[k].tx.position().v), 3 * sizeof(float));
        posefile.write(reinterpret_cast<const char *>(pose[k].tx.rotation().m), 9 * sizeof(float));
    }
    return 0;
}
