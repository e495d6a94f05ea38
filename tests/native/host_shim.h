// Host definitions of the CUDA device intrinsics the traversal header uses, so that the
// product's own device code (hussar_gb300/csrc/hsr_traverse.cuh) compiles and runs on the
// CPU in the tests. Semantics as in CUDA: __fmaf_rn
// is a single-rounding fused multiply-add, the bit casts are exact, atomics are plain
// read-modify-writes (the tests run one thread).
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
inline float __uint_as_float(unsigned u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline unsigned __float_as_uint(float f) {
    unsigned u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float __int_as_float(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}
inline int __float_as_int(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i;
}
template <class T> inline T __ldg(const T *p) { return *p; }
inline int __ffs(int x) { return __builtin_ffs(x); }
inline unsigned umin(unsigned a, unsigned b) { return a < b ? a : b; }
inline unsigned umax(unsigned a, unsigned b) { return a < b ? b : a; }
inline unsigned atomicOr(unsigned *p, unsigned v) {
    const unsigned o = *p;
    *p |= v;
    return o;
}
