// Device math shared by the GB300 kernels: constants, vectors, complex numbers and
// the error/status word. Operation orders follow the reference's scalar code
// (libhussar/include/hussar/core/geometry.h:69-143, libradar/include/radar/complex.h)
// because the trace kernels are compiled with -fmad=false: every + - * / here rounds
// exactly like the CPU restatement, so hit/miss decisions agree bit-for-bit.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

namespace hsr {

// hussar.h:37-52, radar.h:107
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInv4Pi = 0.07957747154594766788f;
constexpr float kSpeedOfLight = 299792458.f;
constexpr float kEpsilon = 5e-5f;

// Device status word bits (checked by the host after each synchronising call).
enum StatusBits : unsigned {
    kStatusStackOverflow = 1u << 0,   // traversal stack would have overflowed; ray treated as miss
    kStatusBadBin = 1u << 1,          // a splat bin was outside the frame (guarded, skipped)
    kStatusBadWorkItem = 1u << 2,     // work item index out of range (guarded)
    // bit 3: a synthesis GEMM wait gave up (hsr_synth.cu)
};

// sin and cos of a float angle, each rounded once to float (for |x| up to a few 2pi).
// x - k pi/2 (k = nearest integer to x 2/pi) in double by a two-part pi/2 with fused
// multiply-adds, then the Taylor series of sin (to degree 15) and cos (to degree 16) on
// the remainder (|r| <= pi/4: truncation below 7e-17 relative) by Horner's rule in
// double, rounded to float. Every operation is an IEEE double operation with a single
// rounding (fma, *, +, rint, the final conversion), so the host and the device compute
// the same bits for the same x; the float results are the correctly rounded ones except
// where the exact value lies within ~2^-50 of a float rounding midpoint. Coefficients are
// 1/n! rounded to double (hex literals).
__host__ __device__ inline void sincos_rounded(float x, float *s, float *c) {
    const double xd = double(x);
    const double k = rint(xd * 0x1.45f306dc9c883p-1);                 // x 2/pi
    double r = fma(-k, 0x1.921fb54442d18p+0, xd);                       // pi/2, high part
    r = fma(-k, 0x1.1a62633145c07p-54, r);                              // pi/2, low part
    const double z = r * r;
    double ps = -0x1.ae7f3e733b81fp-41;                                 // -1/15!
    ps = fma(ps, z, 0x1.6124613a86d09p-33);                             //  1/13!
    ps = fma(ps, z, -0x1.ae64567f544e4p-26);                            // -1/11!
    ps = fma(ps, z, 0x1.71de3a556c734p-19);                             //  1/9!
    ps = fma(ps, z, -0x1.a01a01a01a01ap-13);                            // -1/7!
    ps = fma(ps, z, 0x1.1111111111111p-7);                              //  1/5!
    ps = fma(ps, z, -0x1.5555555555555p-3);                             // -1/3!
    const double sr = fma(r * z, ps, r);
    double pc = 0x1.ae7f3e733b81fp-45;                                  //  1/16!
    pc = fma(pc, z, -0x1.93974a8c07c9dp-37);                            // -1/14!
    pc = fma(pc, z, 0x1.1eed8eff8d898p-29);                             //  1/12!
    pc = fma(pc, z, -0x1.27e4fb7789f5cp-22);                            // -1/10!
    pc = fma(pc, z, 0x1.a01a01a01a01ap-16);                             //  1/8!
    pc = fma(pc, z, -0x1.6c16c16c16c17p-10);                            // -1/6!
    pc = fma(pc, z, 0x1.5555555555555p-5);                              //  1/4!
    pc = fma(pc, z, -0.5);                                              // -1/2!
    const double cr = fma(z, pc, 1.0);
    const int q = int(k) & 3;
    const double sv = q == 0 ? sr : q == 1 ? cr : q == 2 ? -sr : -cr;
    const double cv = q == 0 ? cr : q == 1 ? -sr : q == 2 ? -cr : sr;
    *s = static_cast<float>(sv);
    *c = static_cast<float>(cv);
}

// Single-precision operations with one rounding each and no contraction, the same on
// the device (the _rn intrinsics) and on the host (host code compiles with
// -ffp-contract=off).
__host__ __device__ __forceinline__ float rn_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ __forceinline__ float rn_mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ __forceinline__ float rn_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
__host__ __device__ __forceinline__ unsigned f32_bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    unsigned u;
    memcpy(&u, &x, 4);
    return u;
#endif
}
__host__ __device__ __forceinline__ float f32_from_bits(unsigned u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}

// Double-float values h + l (|l| <= ulp(h) / 2 after a normalising sum) and the
// error-free transformations they are built from (Knuth's TwoSum, Dekker's Fast2Sum,
// the FMA form of Dekker's TwoProduct).
struct dfloat {
    float h, l;
};
__host__ __device__ __forceinline__ dfloat two_sum(float a, float b) {
    const float s = rn_add(a, b);
    const float bb = rn_add(s, -a);
    return dfloat{s, rn_add(rn_add(a, -rn_add(s, -bb)), rn_add(b, -bb))};
}
__host__ __device__ __forceinline__ dfloat fast_two_sum(float a, float b) {  // |a| >= |b|, or a == 0
    const float s = rn_add(a, b);
    return dfloat{s, rn_add(b, -rn_add(s, -a))};
}
__host__ __device__ __forceinline__ dfloat two_prod(float a, float b) {
    const float p = rn_mul(a, b);
    return dfloat{p, rn_fma(a, b, -p)};
}
// (a.h + a.l)(b.h + b.l) without the a.l b.l term
__host__ __device__ __forceinline__ dfloat mul_df(dfloat a, dfloat b) {
    dfloat p = two_prod(a.h, b.h);
    p.l = rn_add(p.l, rn_fma(a.h, b.l, rn_mul(a.l, b.h)));
    return p;
}

// Ziv's rounding test for a normalised double-float v whose exact value lies within
// |v.h| 2^-37 of v.h + v.l: true when every such value rounds to v.h (nearest, ties to
// even), i.e. v.h is the correctly rounded float of the exact value. Values whose
// magnitude is below 2^-100 are never certified.
__host__ __device__ __forceinline__ bool rounds_to_high(dfloat v) {
    const unsigned bits = f32_bits(v.h) & 0x7fffffffu;
    const int e = int(bits >> 23);
    if (e < 27 || e > 253) return false;
    const float a = f32_from_bits(bits);
    const float ulp = f32_from_bits(unsigned(e - 23) << 23);
    const float err = rn_mul(a, 0x1p-37f);
    const float l = v.h < 0.f ? -v.l : v.l;  // > 0: away from zero
    // the half-gaps to the neighbouring floats, shortened by 1e-5 ulp to cover the
    // rounding of l + err; below a power of two the gap is half as wide
    const float up = rn_mul(ulp, 0.49999f);
    const float down = (bits & 0x7fffffu) == 0u ? rn_mul(ulp, 0.249995f) : up;
    return l >= 0.f ? rn_add(l, err) < up : rn_add(-l, err) < down;
}

// sin x and cos x as double-floats for 2^-14 <= |x| <= 8 (sincos_cr's fast path; no
// intermediate value is subnormal there).
// Method: Cody-Waite reduction x = k pi/2 + r with pi/2 = C1 + C2 + C3 (C1 has 21
// significant bits, so k C1 and x - k C1 are exact for |k| <= 5), r as a double-float;
// the Taylor series sin r = r (1 - z/3! + z^2/5! - ...) and cos r = 1 - z/2! + z^2/4! -
// ... in z = r^2 (|r| <= pi/4 + 1e-7), the terms up to z^3 in double-float arithmetic and
// the rest, below 4e-6, in float (where its rounding, a few float ulps of the rest, sets
// the error). Relative error below 2^-38.8; the largest over every float in [2^-14, 8],
// against long double: 2^-40.2.
__host__ __device__ __forceinline__ void sincos_df(float x, dfloat &sv, dfloat &cv) {
    const float k = rintf(rn_mul(x, 0x1.45f306p-1f));                 // x 2/pi
    const float r1 = rn_fma(-k, 0x1.921fb0p+0f, x);                    // exact
    const dfloat kc2 = two_prod(k, 0x1.5110b4p-22f);
    const dfloat s1 = two_sum(r1, -kc2.h);
    const dfloat r = fast_two_sum(s1.h, rn_add(rn_add(s1.l, -kc2.l), -rn_mul(k, 0x1.84698ap-48f)));
    dfloat z = two_prod(r.h, r.h);
    z.l = rn_fma(rn_add(r.h, r.h), r.l, z.l);
    const dfloat z2 = mul_df(z, z);
    const dfloat z3 = mul_df(z2, z);
    const float z4 = rn_fma(z2.h, z2.h, rn_mul(rn_add(z2.h, z2.h), z2.l));
    // sin r / r = 1 - z/3! + z^2/5! - z^3/7! + z^4 (1/9! - z/11! + z^2/13!)
    const dfloat a1 = mul_df(z, dfloat{-0x1.555556p-3f, 0x1.555556p-28f});
    const dfloat a2 = mul_df(z2, dfloat{0x1.111112p-7f, -0x1.dddddep-32f});
    const dfloat a3 = mul_df(z3, dfloat{-0x1.a01a02p-13f, 0x1.7f97fap-39f});
    float ts = rn_fma(z.h, 0x1.612462p-33f, -0x1.ae6456p-26f);
    ts = rn_fma(ts, z.h, 0x1.71de3ap-19f);
    dfloat sr = fast_two_sum(1.f, a1.h);
    float sl = sr.l;
    sr = fast_two_sum(sr.h, a2.h);
    sl = rn_add(sl, sr.l);
    sr = fast_two_sum(sr.h, a3.h);
    sl = rn_add(rn_add(rn_add(sl, sr.l), rn_add(rn_add(a1.l, a2.l), a3.l)), rn_mul(z4, ts));
    sr = mul_df(r, dfloat{sr.h, sl});
    sr = fast_two_sum(sr.h, sr.l);
    // cos r = 1 - z/2! + z^2/4! - z^3/6! + z^4 (1/8! - z/10! + z^2/12! - z^3/14!)
    const dfloat b2 = mul_df(z2, dfloat{0x1.555556p-5f, -0x1.555556p-30f});
    const dfloat b3 = mul_df(z3, dfloat{-0x1.6c16c2p-10f, 0x1.27d27ep-35f});
    float tc = rn_fma(z.h, -0x1.93974ap-37f, 0x1.1eed8ep-29f);
    tc = rn_fma(tc, z.h, -0x1.27e4fcp-22f);
    tc = rn_fma(tc, z.h, 0x1.a01a02p-16f);
    dfloat cr = fast_two_sum(1.f, rn_mul(z.h, -0.5f));
    float cl = rn_add(cr.l, rn_mul(z.l, -0.5f));
    cr = fast_two_sum(cr.h, b2.h);
    cl = rn_add(cl, cr.l);
    cr = fast_two_sum(cr.h, b3.h);
    cl = rn_add(rn_add(rn_add(cl, cr.l), rn_add(b2.l, b3.l)), rn_mul(z4, tc));
    cr = fast_two_sum(cr.h, cl);
    // quadrant
    const int q = int(k) & 3;
    const dfloat ns = dfloat{-sr.h, -sr.l}, nc = dfloat{-cr.h, -cr.l};
    sv = q == 0 ? sr : q == 1 ? cr : q == 2 ? ns : nc;
    cv = q == 0 ? cr : q == 1 ? ns : q == 2 ? nc : sr;
}

// sincos_rounded's results (the same bits for every float x) at a fraction of its
// double-precision operations: for 2^-14 <= |x| <= 8 the double-floats of sincos_df are
// returned when the rounding test certifies both, which holds for all but about 0.05 %
// of arguments (1.4 % of warps of uniformly distributed angles); those, and every x outside that range, take sincos_rounded. Checked
// against sincos_rounded for every float in [-8, 8] (the rounding test is what makes the
// two agree: sincos_rounded is correctly rounded except within 2^-50 of a midpoint, and
// a certified value is further than 2^-37 from one).
__host__ __device__ __forceinline__ void sincos_cr(float x, float *s, float *c) {
    const float ax = fabsf(x);
    if (ax >= 0x1p-14f && ax <= 8.f) {
        dfloat sv, cv;
        sincos_df(x, sv, cv);
        if (rounds_to_high(sv) && rounds_to_high(cv)) {
            *s = sv.h;
            *c = cv.h;
            return;
        }
    }
    sincos_rounded(x, s, c);
}

struct f3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 scl3(float s, f3 a) { return f3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ f3 neg3(f3 a) { return f3{-a.x, -a.y, -a.z}; }
// 3-term reductions in the order x0 + (x1 + x2)
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__device__ __forceinline__ float sqn3(f3 a) { return a.x * a.x + (a.y * a.y + a.z * a.z); }
__device__ __forceinline__ float nrm3(f3 a) { return sqrtf(sqn3(a)); }
__device__ __forceinline__ f3 crs3(f3 a, f3 b) {
    return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ f3 div3(f3 a, float s) { return f3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ f3 nrmz3(f3 a) {
    float n = sqn3(a);
    if (n > 0.f) {
        float s = sqrtf(n);
        return f3{a.x / s, a.y / s, a.z / s};
    }
    return a;
}

struct cf {
    float re, im;
};
__device__ __forceinline__ cf cadd(cf a, cf b) { return cf{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cf csub(cf a, cf b) { return cf{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cf cmul(cf a, cf b) {
    float r = a.re * b.re - a.im * b.im;
    float i = a.re * b.im + a.im * b.re;
    return cf{r, i};
}
__device__ __forceinline__ cf cscl(cf a, float s) { return cf{a.re * s, a.im * s}; }
__device__ __forceinline__ cf cdiv(cf a, float s) { return cf{a.re / s, a.im / s}; }
__device__ __forceinline__ cf cconj(cf a) { return cf{a.re, -a.im}; }

// complex 3-vector (the ray's H field)
struct c3 {
    cf v[3];
};
__device__ __forceinline__ c3 c3_real(f3 a) {
    c3 r;
    r.v[0] = cf{a.x, 0.f};
    r.v[1] = cf{a.y, 0.f};
    r.v[2] = cf{a.z, 0.f};
    return r;
}
__device__ __forceinline__ c3 c3_scl(c3 a, float s) {
#pragma unroll
    for (int i = 0; i < 3; ++i) a.v[i] = cscl(a.v[i], s);
    return a;
}
__device__ __forceinline__ c3 c3_div(c3 a, float s) {
#pragma unroll
    for (int i = 0; i < 3; ++i) a.v[i] = cdiv(a.v[i], s);
    return a;
}
__device__ __forceinline__ c3 c3_cmul(c3 a, cf s) {
#pragma unroll
    for (int i = 0; i < 3; ++i) a.v[i] = cmul(a.v[i], s);
    return a;
}
__device__ __forceinline__ c3 c3_sub(c3 a, c3 b) {
#pragma unroll
    for (int i = 0; i < 3; ++i) a.v[i] = csub(a.v[i], b.v[i]);
    return a;
}
// real x complex cross product with the conjugated result (Eigen MatrixBase::cross)
__device__ __forceinline__ c3 crs_rc(f3 a, const c3 &b) {
    c3 r;
    r.v[0] = cconj(csub(cscl(b.v[2], a.y), cscl(b.v[1], a.z)));
    r.v[1] = cconj(csub(cscl(b.v[0], a.z), cscl(b.v[2], a.x)));
    r.v[2] = cconj(csub(cscl(b.v[1], a.x), cscl(b.v[0], a.y)));
    return r;
}
// sum_i a_i b_i for real a
__device__ __forceinline__ cf dot_rc(f3 a, const c3 &b) {
    return cadd(cscl(b.v[0], a.x), cadd(cscl(b.v[1], a.y), cscl(b.v[2], a.z)));
}
// Hermitian sum_i conj(a_i) b_i (geometry.h:138)
__device__ __forceinline__ cf dot_cc(const c3 &a, const c3 &b) {
    return cadd(cmul(cconj(a.v[0]), b.v[0]), cadd(cmul(cconj(a.v[1]), b.v[1]), cmul(cconj(a.v[2]), b.v[2])));
}
// Eigen isZero(1e-20): every |h_i|^2 <= 1e-20f * 1e-20f (a float denormal; no FTZ here)
__device__ __forceinline__ bool c3_is_zero(const c3 &a) {
    const float prec = 1e-20f;
    const float lim = prec * prec;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float a2 = a.v[i].re * a.v[i].re + a.v[i].im * a.v[i].im;
        if (!(a2 <= lim)) return false;
    }
    return true;
}

// Row-major 3x3
struct m33 {
    float m[9];
};
__device__ __forceinline__ f3 mulv(const m33 &M, f3 v) {
    return f3{M.m[0] * v.x + (M.m[1] * v.y + M.m[2] * v.z), M.m[3] * v.x + (M.m[4] * v.y + M.m[5] * v.z),
              M.m[6] * v.x + (M.m[7] * v.y + M.m[8] * v.z)};
}
__device__ __forceinline__ f3 mulTv(const m33 &M, f3 v) {
    return f3{M.m[0] * v.x + (M.m[3] * v.y + M.m[6] * v.z), M.m[1] * v.x + (M.m[4] * v.y + M.m[7] * v.z),
              M.m[2] * v.x + (M.m[5] * v.y + M.m[8] * v.z)};
}
__device__ __forceinline__ c3 mulcv(const m33 &M, const c3 &h) {
    c3 r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
        r.v[i] = cadd(cscl(h.v[0], M.m[3 * i]), cadd(cscl(h.v[1], M.m[3 * i + 1]), cscl(h.v[2], M.m[3 * i + 2])));
    return r;
}

// Scene storage on the device -------------------------------------------------------
// Triangle record: v0, e1 = v1 - v0, e2 = v2 - v0 (exactly the float differences the
// CPU restatement forms), original primitive id in v0.w. 48 bytes, three 16-byte loads.
struct __align__(16) DTri {
    float4 v0;
    float4 e1;
    float4 e2;
};

// Binary BVH node holding both child boxes (64 bytes, four 16-byte loads).
// child >= 0: internal node index; child < 0: a leaf of ((~child) & 7) + 1 triangles in
// consecutive slots from (~child) >> 3.
struct __align__(16) DNode {
    float4 a;  // c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y
    float4 b;  // c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y
    float4 c;  // c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z
    int4 d;    // child0, child1, unused, unused
};

}  // namespace hsr
