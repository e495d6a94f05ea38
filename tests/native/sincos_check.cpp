// CPU check of the primary direction's sine and cosine (hussar_gb300/csrc/hsr_common.cuh,
// compiled from the product's header): for every stride-th float x in [-8, 8],
// sincos_cr must give sincos_rounded's bits, and the double-float evaluation sincos_df
// must stay within its stated relative error of sin and cos in long double.
// Output: one line "checked N mismatches M max_log2_rel_err E slow S".
#include "hsr_common.cuh"

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

using namespace hsr;

int main(int argc, char **argv) {
    const unsigned stride = argc > 1 ? unsigned(std::atoi(argv[1])) : 1u;
    const int threads = argc > 2 ? std::atoi(argv[2]) : 4;
    if (stride < 1 || threads < 1) return 2;
    const unsigned hi = f32_bits(8.f);
    std::vector<long> checked(threads), bad(threads), slow(threads);
    std::vector<long double> err(threads);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&, t] {
            for (unsigned u = unsigned(t) * stride; u <= hi; u += unsigned(threads) * stride) {
                for (unsigned sign = 0; sign < 2; ++sign) {
                    const float x = f32_from_bits(u | (sign << 31));
                    float s0, c0, s1, c1;
                    sincos_rounded(x, &s0, &c0);
                    sincos_cr(x, &s1, &c1);
                    if (f32_bits(s0) != f32_bits(s1) || f32_bits(c0) != f32_bits(c1)) ++bad[t];
                    ++checked[t];
                    const float ax = std::fabs(x);
                    if (ax < 0x1p-14f) {
                        ++slow[t];
                        continue;
                    }
                    dfloat sv, cv;
                    sincos_df(x, sv, cv);
                    if (!rounds_to_high(sv) || !rounds_to_high(cv)) ++slow[t];
                    const long double S = sinl((long double)x), C = cosl((long double)x);
                    const long double es = fabsl(((long double)sv.h + sv.l) - S) / fabsl(S);
                    const long double ec = fabsl(((long double)cv.h + cv.l) - C) / fabsl(C);
                    if (es > err[t]) err[t] = es;
                    if (ec > err[t]) err[t] = ec;
                }
            }
        });
    for (auto &p : pool) p.join();
    long n = 0, b = 0, sl = 0;
    long double e = 0;
    for (int t = 0; t < threads; ++t) {
        n += checked[t];
        b += bad[t];
        sl += slow[t];
        if (err[t] > e) e = err[t];
    }
    std::printf("checked %ld mismatches %ld max_log2_rel_err %.3f slow %ld\n", n, b, double(log2l(e)), sl);
    return 0;
}
