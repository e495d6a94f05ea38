/*
 * ORACLE — TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement of libhussar's radar path tracer, used only by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker
 * and the timed CPU reference. The product (hussar_gb300/, libhsr_gb300.so) never
 * links, loads or calls anything in this directory.
 *
 * What it restates (file:line within the reference project):
 *   - HaltonSampler / radicalInverse<base>   libhussar/include/hussar/samplers/halton.h:11-67
 *   - UniformSampleSphere, UniformSpherePdf  libhussar/include/hussar/core/sampling.h:38-47
 *   - AWRAngularDistribution, NFAntenna      libhussar/include/hussar/core/emitter.h:109-214
 *   - SurfaceEmitter                         libhussar/include/hussar/core/emitter.h:53-82
 *   - Ray, Intersection                      libhussar/include/hussar/core/geometry.h:69-143,
 *                                            libhussar/include/hussar/core/intersection.h:16-57
 *   - PathTracer::sample                     libhussar/include/hussar/integrators/path.h:235-451
 *   - PathTracer::run (guided schedule)      libhussar/include/hussar/integrators/path.h:171-224
 *   - GuidingWrapper sample/splat/step       libhussar/include/hussar/integrators/path.h:17-131
 *     over the product's own 2-D tree (libguiding's BTree is not in the reference sources)
 *   - Integrator::measureRay/splat/reflect   libhussar/include/hussar/core/integrator.h:107-168
 *   - Frame::PIndex::setTime/setVelocity     libradar/include/radar/radar.h:232-251
 *   - Frame::splat<16>                       libradar/include/radar/radar.h:564-626
 *   - host atomicAdd(float*) (CAS loop)      libradar/include/radar/radar.h:63-83
 *   - cpu::Backend::run batch scheduler      libhussar/include/hussar/arch/cpu.h:18-46
 *   - Embree hit semantics (tnear=Epsilon, faceforwarded normalised Ng)
 *                                            libhussar/src/arch/cpu.cpp:9-87
 *
 * Precision: templated on Real. Real=float follows the reference's single-precision
 * expression order (including the places where the reference widens to double:
 * std::pow in the AWR pattern, cos/sin in radar::polar, M_PI in Frame::splat).
 * Real=double is the FP64 oracle: the same estimator, every operation in double.
 *
 * Eigen (absent from this container) fixes some operation orders in the reference;
 * they are restated here as Eigen documents/implements them:
 *   - a.dot(b) for complex a is sum(conj(a_i) * b_i)          (geometry.h:138)
 *   - 3-term reductions (dot, squaredNorm, 3x3 mat-vec rows) are x0 + (x1 + x2)
 *   - v.normalized() is v / sqrt(squaredNorm)
 *   - cross() of complex vectors conjugates the result
 * Embree (absent) is replaced by a BVH of its own (PLOC clustering, leaves of up to 4
 * triangles; a binned-SAH build as the fallback) with a Moller-Trumbore triangle
 * test; hits are accepted for tnear < t <= tfar, equal-t ties go to the lower
 * primitive id, so the answers do not depend on the tree. Parity with Embree/OptiX/Eigen themselves is unpinned.
 *
 * Build: oracle/Makefile (g++ -O3 -ffp-contract=off, no -march: the same bits on
 * x86-64 and aarch64).
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <mutex>
#include <thread>
#include <vector>

#include "hsr_oracle.h"

namespace oracle {

// ----------------------------------------------------------------------------------
// Constants (hussar.h:37-52, radar.h:107)
// ----------------------------------------------------------------------------------
template <typename R> struct Consts;
template <> struct Consts<float> {
    static constexpr float Pi = 3.14159265358979323846f;
    static constexpr float Inv4Pi = 0.07957747154594766788f;
    static constexpr float SpeedOfLight = 299792458.f;  // radar.h:107 (float)
    static constexpr float Epsilon = 5e-5f;             // hussar.h:52
};
template <> struct Consts<double> {
    static constexpr double Pi = 3.14159265358979323846;
    static constexpr double Inv4Pi = 0.07957747154594766788;
    static constexpr double SpeedOfLight = 299792458.0;
    static constexpr double Epsilon = 5e-5;
};

template <typename R> struct V3 {
    R x, y, z;
};
template <typename R> struct Cx {
    R re, im;
};
template <typename R> struct CV3 {
    Cx<R> c[3];
};

template <typename R> static inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <typename R> static inline V3<R> add(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename R> static inline V3<R> sub(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename R> static inline V3<R> scale(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename R> static inline V3<R> neg(V3<R> a) { return {-a.x, -a.y, -a.z}; }
// Eigen redux order for 3 terms: x0 + (x1 + x2)
template <typename R> static inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
template <typename R> static inline R sqnorm(V3<R> a) { return a.x * a.x + (a.y * a.y + a.z * a.z); }
template <typename R> static inline R norm(V3<R> a) { return std::sqrt(sqnorm(a)); }
template <typename R> static inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename R> static inline V3<R> normalized(V3<R> a) {
    R n = sqnorm(a);
    if (n > R(0)) {
        R s = std::sqrt(n);
        return {a.x / s, a.y / s, a.z / s};
    }
    return a;
}
template <typename R> static inline V3<R> divs(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }

// complex (libradar/include/radar/complex.h)
template <typename R> static inline Cx<R> cadd(Cx<R> a, Cx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <typename R> static inline Cx<R> csub(Cx<R> a, Cx<R> b) { return {a.re - b.re, a.im - b.im}; }
template <typename R> static inline Cx<R> cmul(Cx<R> a, Cx<R> b) {  // complex.h:56-61
    R r = a.re * b.re - a.im * b.im;
    R i = a.re * b.im + a.im * b.re;
    return {r, i};
}
template <typename R> static inline Cx<R> cscale(Cx<R> a, R s) { return {a.re * s, a.im * s}; }  // complex.h:48-52
template <typename R> static inline Cx<R> cdivs(Cx<R> a, R s) { return {a.re / s, a.im / s}; }   // complex.h:69-73
template <typename R> static inline Cx<R> cconj(Cx<R> a) { return {a.re, -a.im}; }
// radar::polar(1, angle) with the reference's unqualified cos/sin (complex.h:184-187),
// which resolve to ::cos(double)/::sin(double) for a float angle.
template <typename R> static inline Cx<R> cexpj(R angle) {
    double a = double(angle);
    return {R(std::cos(a)), R(std::sin(a))};
}
// std::abs(radar::complex) (complex.h:225-237)
template <typename R> static inline R cabs(Cx<R> z) {
    R x = std::abs(z.re), y = std::abs(z.im);
    R s = x < y ? y : x;
    if (s == R(0)) return s;
    x /= s;
    y /= s;
    return s * std::sqrt(x * x + y * y);
}

template <typename R> static inline CV3<R> cv3_real(V3<R> v) {
    CV3<R> r;
    r.c[0] = {v.x, R(0)};
    r.c[1] = {v.y, R(0)};
    r.c[2] = {v.z, R(0)};
    return r;
}
template <typename R> static inline CV3<R> cv3_scale(CV3<R> a, R s) {
    for (int i = 0; i < 3; ++i) a.c[i] = cscale(a.c[i], s);
    return a;
}
template <typename R> static inline CV3<R> cv3_divs(CV3<R> a, R s) {
    for (int i = 0; i < 3; ++i) a.c[i] = cdivs(a.c[i], s);
    return a;
}
template <typename R> static inline CV3<R> cv3_cmul(CV3<R> a, Cx<R> s) {
    for (int i = 0; i < 3; ++i) a.c[i] = cmul(a.c[i], s);
    return a;
}
template <typename R> static inline CV3<R> cv3_sub(CV3<R> a, CV3<R> b) {
    for (int i = 0; i < 3; ++i) a.c[i] = csub(a.c[i], b.c[i]);
    return a;
}
// real x complex cross product, conjugated like Eigen's MatrixBase::cross
template <typename R> static inline CV3<R> cross_rc(V3<R> a, const CV3<R> &b) {
    auto m = [](R s, Cx<R> z) { return Cx<R>{z.re * s, z.im * s}; };  // float*complex, complex.h:128-132
    CV3<R> r;
    r.c[0] = cconj(csub(m(a.y, b.c[2]), m(a.z, b.c[1])));
    r.c[1] = cconj(csub(m(a.z, b.c[0]), m(a.x, b.c[2])));
    r.c[2] = cconj(csub(m(a.x, b.c[1]), m(a.y, b.c[0])));
    return r;
}
// real . complex: sum(conj(a_i) b_i) with a real -> sum(a_i b_i), Eigen order
template <typename R> static inline Cx<R> dot_rc(V3<R> a, const CV3<R> &b) {
    Cx<R> t0 = cscale(b.c[0], a.x), t1 = cscale(b.c[1], a.y), t2 = cscale(b.c[2], a.z);
    return cadd(t0, cadd(t1, t2));
}
// complex . complex (Hermitian): sum(conj(a_i) b_i) (geometry.h:138)
template <typename R> static inline Cx<R> dot_cc(const CV3<R> &a, const CV3<R> &b) {
    Cx<R> t0 = cmul(cconj(a.c[0]), b.c[0]), t1 = cmul(cconj(a.c[1]), b.c[1]),
          t2 = cmul(cconj(a.c[2]), b.c[2]);
    return cadd(t0, cadd(t1, t2));
}
// Eigen isZero(1e-20): every |coeff|^2 <= prec^2
template <typename R> static inline bool cv3_is_zero(const CV3<R> &a) {
    const R prec = R(1e-20);
    const R lim = prec * prec;
    for (int i = 0; i < 3; ++i) {
        R a2 = a.c[i].re * a.c[i].re + a.c[i].im * a.c[i].im;
        if (!(a2 <= lim)) return false;
    }
    return true;
}

// 3x3 row-major matrix
template <typename R> struct M33 {
    R m[9];
};
template <typename R> static inline V3<R> mulv(const M33<R> &M, V3<R> v) {
    return {M.m[0] * v.x + (M.m[1] * v.y + M.m[2] * v.z), M.m[3] * v.x + (M.m[4] * v.y + M.m[5] * v.z),
            M.m[6] * v.x + (M.m[7] * v.y + M.m[8] * v.z)};
}
template <typename R> static inline V3<R> mulTv(const M33<R> &M, V3<R> v) {
    return {M.m[0] * v.x + (M.m[3] * v.y + M.m[6] * v.z), M.m[1] * v.x + (M.m[4] * v.y + M.m[7] * v.z),
            M.m[2] * v.x + (M.m[5] * v.y + M.m[8] * v.z)};
}
template <typename R> static inline CV3<R> mulcv(const M33<R> &M, const CV3<R> &h) {
    CV3<R> r;
    for (int i = 0; i < 3; ++i) {
        Cx<R> t0 = cscale(h.c[0], M.m[3 * i + 0]);
        Cx<R> t1 = cscale(h.c[1], M.m[3 * i + 1]);
        Cx<R> t2 = cscale(h.c[2], M.m[3 * i + 2]);
        r.c[i] = cadd(t0, cadd(t1, t2));
    }
    return r;
}

// ----------------------------------------------------------------------------------
// Halton sampler (halton.h:11-67)
// ----------------------------------------------------------------------------------
template <typename R, int base> static inline R radical_inverse_b(uint64_t v) {
    const R invBase = R(1) / R(base);
    uint64_t reversed = 0;
    R invBaseN = 1;
    while (v) {
        uint64_t next = v / base;
        uint64_t digit = v - next * base;
        reversed = reversed * base + digit;
        invBaseN *= invBase;
        v = next;
    }
    const R ome = std::nextafter(R(1), R(0));
    return std::min(R(reversed) * invBaseN, ome);
}

template <typename R> static inline R radical_inverse(uint64_t v, unsigned dim) {
    switch (dim) {
        case 0: return radical_inverse_b<R, 2>(v);
        case 1: return radical_inverse_b<R, 3>(v);
        case 2: return radical_inverse_b<R, 5>(v);
        case 3: return radical_inverse_b<R, 7>(v);
        case 4: return radical_inverse_b<R, 11>(v);
        case 5: return radical_inverse_b<R, 13>(v);
        case 6: return radical_inverse_b<R, 17>(v);
        case 7: return radical_inverse_b<R, 19>(v);
        case 8: return radical_inverse_b<R, 23>(v);
        case 9: return radical_inverse_b<R, 29>(v);
        default: return R(0);  // halton.h:1082-1084: Assert (no-op in release), return 0
    }
}

template <typename R> struct Halton {
    uint64_t index = 0;
    uint16_t dim = 0;
    bool float_samples = false;  // FP64 run of exactly the FP32 run's (float) sample values
    R get1D() {
        R u = radical_inverse<R>(index, dim++);
        return float_samples ? R(float(radical_inverse<float>(index, unsigned(dim - 1)))) : u;
    }
    // HaltonSampler::get2D (halton.h:23-26) returns Vector2f(get1D(), get1D()); C++ leaves
    // the order of the two calls unspecified, and GCC evaluates the second argument first,
    // so a GCC build of the reference gets (next dimension + 1, next dimension).
    void get2D(R &u0, R &u1) {
        u1 = get1D();
        u0 = get1D();
    }
};

// ----------------------------------------------------------------------------------
// Sampling, antenna pattern, antennas (sampling.h:38-47, emitter.h:109-214)
// ----------------------------------------------------------------------------------
// The reference's std::sin/std::cos of a float angle resolve to the platform's sinf/cosf,
// which are not correctly rounded everywhere (glibc 2.39: one ulp off on 1.3 % of
// uniformly distributed angles), so the reference's primary directions depend on the libm
// it was built against. The FP32 restatement therefore offers both: the libm's sinf/cosf
// (g_libm_trig = 1, what a glibc build of the reference computes; used to pin against the
// reference's own code) and, by default, sin and cos rounded once to float from a double
// evaluation whose every step is a single IEEE rounding (x - k pi/2 by a two-part pi/2 with
// fma, Taylor series to degree 15/16 by Horner's rule with fma), which any IEEE machine,
// the GPU included, evaluates to the same bits.
static int g_libm_trig = 0;

static inline void sincos_once_rounded(float x, float &s, float &c) {
    const double xd = double(x);
    const double k = std::rint(xd * 0x1.45f306dc9c883p-1);
    double r = std::fma(-k, 0x1.921fb54442d18p+0, xd);
    r = std::fma(-k, 0x1.1a62633145c07p-54, r);
    const double z = r * r;
    // sin(r) = r + r z (-1/3! + z (1/5! - z (1/7! - ...))), cos(r) = 1 + z (-1/2! + z (1/4! - ...))
    static const double S[7] = {-0x1.ae7f3e733b81fp-41, 0x1.6124613a86d09p-33, -0x1.ae64567f544e4p-26,
                                0x1.71de3a556c734p-19, -0x1.a01a01a01a01ap-13, 0x1.1111111111111p-7,
                                -0x1.5555555555555p-3};
    static const double C[8] = {0x1.ae7f3e733b81fp-45, -0x1.93974a8c07c9dp-37, 0x1.1eed8eff8d898p-29,
                                -0x1.27e4fb7789f5cp-22, 0x1.a01a01a01a01ap-16, -0x1.6c16c16c16c17p-10,
                                0x1.5555555555555p-5, -0.5};
    double ps = S[0];
    for (int i = 1; i < 7; ++i) ps = std::fma(ps, z, S[i]);
    double pc = C[0];
    for (int i = 1; i < 8; ++i) pc = std::fma(pc, z, C[i]);
    const double sr = std::fma(r * z, ps, r), cr = std::fma(z, pc, 1.0);
    switch (int(k) & 3) {
        case 0: s = float(sr); c = float(cr); break;
        case 1: s = float(cr); c = float(-sr); break;
        case 2: s = float(-sr); c = float(-cr); break;
        default: s = float(-cr); c = float(sr); break;
    }
}

template <typename R> static inline V3<R> uniform_sample_sphere(R u0, R u1) {
    R phi = R(2) * Consts<R>::Pi * u0;
    R y = R(2) * u1 - R(1);
    R r = std::sqrt(std::max(R(0), R(1) - y * y));
    R sp = std::sin(phi), cp = std::cos(phi);
    if (sizeof(R) == 4 && !g_libm_trig) {
        float fs, fc;
        sincos_once_rounded(float(phi), fs, fc);
        sp = R(fs);
        cp = R(fc);
    }
    return {-r * sp, y, -r * cp};
}

// AWRAngularDistribution::evaluate (emitter.h:126-136)
template <typename R> static inline CV3<R> awr_evaluate(V3<R> d) {
    // Vector3c(0,1,0).cross(d): real-valued (d.z, 0, -d.x) (zeros as the conjugated cross gives them)
    CV3<R> H;
    H.c[0] = {R(1) * d.z - R(0) * d.y, -(R(0) * d.z - R(0) * d.y)};
    H.c[1] = {R(0) * d.x - R(0) * d.z, -(R(0) * d.x - R(0) * d.z)};
    H.c[2] = {R(0) * d.y - R(1) * d.x, -(R(0) * d.y - R(0) * d.x)};
    // clamped at zero where 1 - d.x^2 rounds negative (the reference's sqrt would give NaN
    // and a NaN frame): a deliberate deviation, on directions within ~1e-4 rad of an axis
    R cos_h = std::sqrt(std::max(R(1) - d.x * d.x, R(0)));
    R cos_e = std::sqrt(std::max(R(1) - d.y * d.y, R(0)));
    // 2.622 / pow(double, 6) is evaluated in double and converted to the scalar type
    R s1 = R(2.622 / std::pow(double(cos_h) - 1.8, 6));
    R s2 = R(0.625 / std::pow(double(cos_e) - 1.5, 4));
    H = cv3_scale(H, s1);
    H = cv3_scale(H, s2);
    return H;
}

template <typename R> struct Antenna {
    V3<R> pos;
    M33<R> rot;
};

template <typename R> struct Ray {
    V3<R> o{}, d{};
    R time = 0;
    R frequency = 0;
    int depth = 0;
    CV3<R> H{};
    R k0() const { return R(2) * Consts<R>::Pi * frequency / Consts<R>::SpeedOfLight; }
    R wavelength() const { return Consts<R>::SpeedOfLight / frequency; }
    void addDistance(R dist) { time += dist / Consts<R>::SpeedOfLight; }
    V3<R> at(R t) const { return add(o, scale(t, d)); }
};

template <typename R> struct Isect {
    R t = std::numeric_limits<R>::infinity();
    R tMax = std::numeric_limits<R>::infinity();
    V3<R> p{}, n{};
    Ray<R> ray;
    void reset() {
        t = std::numeric_limits<R>::infinity();
        tMax = std::numeric_limits<R>::infinity();
    }
    bool valid() const { return t < tMax; }
    V3<R> wi() const { return neg(ray.d); }
    V3<R> R_() const { return sub(scale(R(2) * dot(n, wi()), n), wi()); }
    R cosTheta() const { return std::abs(dot(n, wi())); }
};

// NFAntenna::sample (emitter.h:174-180)
template <typename R> static inline void antenna_sample(const Antenna<R> &a, R u0, R u1, Ray<R> &ray) {
    ray.o = a.pos;
    V3<R> d = uniform_sample_sphere(u0, u1);
    CV3<R> H = cv3_divs(awr_evaluate(d), Consts<R>::Inv4Pi);
    ray.d = mulv(a.rot, d);
    ray.H = mulcv(a.rot, H);
}
// NFAntenna::evaluate (emitter.h:182-186)
template <typename R> static inline void antenna_evaluate(const Antenna<R> &a, Ray<R> &ray) {
    ray.o = a.pos;
    CV3<R> H = awr_evaluate(mulTv(a.rot, ray.d));
    ray.H = mulcv(a.rot, H);
}
// NFAntenna::connect (emitter.h:188-193)
template <typename R> static inline void antenna_connect(Isect<R> &nee) {
    R r = nee.t;
    nee.ray.addDistance(r);
    nee.ray.H = cv3_scale(nee.ray.H, R(1) / (R(4) * Consts<R>::Pi * r));
}
// NFAntenna::nee (emitter.h:195-203)
template <typename R> static inline CV3<R> antenna_nee(const Antenna<R> &a, Isect<R> &nee) {
    nee.ray.d = sub(a.pos, nee.ray.o);
    R r = norm(nee.ray.d);
    nee.ray.d = divs(nee.ray.d, r);
    nee.tMax = r;
    CV3<R> H = awr_evaluate(mulTv(a.rot, neg(nee.ray.d)));
    return mulcv(a.rot, H);
}

// FFAntenna (emitter.h:226-291): a far-field antenna, a disk of `radius` at
// sceneCenter + dir * radius facing the scene; the frame is buildFrame(-dir)
// (geometry.h:45-53) and the sample pdf 1 / (4 radius^2) (double, then rounded).
template <typename R> struct FfAntenna {
    V3<R> dir, center, e0, e1;
    CV3<R> pol;
    R radius, pdf;
};
template <typename R> static FfAntenna<R> to_ff(const hsr_ff_antenna_o &a) {
    FfAntenna<R> f;
    f.dir = {R(a.direction[0]), R(a.direction[1]), R(a.direction[2])};
    for (int i = 0; i < 3; ++i) f.pol.c[i] = {R(a.polarization[2 * i]), R(a.polarization[2 * i + 1])};
    f.radius = R(a.radius);
    V3<R> c = {R(a.scene_center[0]), R(a.scene_center[1]), R(a.scene_center[2])};
    f.center = add(c, scale(f.radius, f.dir));  // emitter.h:238
    V3<R> d = neg(f.dir);
    if (std::abs(d.x) > std::abs(d.y))
        f.e0 = divs(v3(-d.z, R(0), d.x), R(std::sqrt(d.x * d.x + d.z * d.z)));
    else
        f.e0 = divs(v3(R(0), d.z, -d.y), R(std::sqrt(d.y * d.y + d.z * d.z)));
    f.e1 = cross(d, f.e0);
    f.pdf = R(1.0 / (4.0 * std::pow(double(a.radius), 2)));  // emitter.h:246
    return f;
}
// FFAntenna::sample (emitter.h:241-248)
template <typename R> static inline void ff_sample(const FfAntenna<R> &a, R u0, R u1, Ray<R> &ray) {
    R s0 = R(2) * u0 - R(1), s1 = R(2) * u1 - R(1);
    V3<R> q = {a.e0.x * s0 + a.e1.x * s1, a.e0.y * s0 + a.e1.y * s1, a.e0.z * s0 + a.e1.z * s1};
    ray.o = add(scale(a.radius, q), a.center);
    ray.d = neg(a.dir);
    ray.H = cv3_divs(a.pol, a.pdf);
}
// FFAntenna::nee (emitter.h:261-273); false where it returns Vector3c::Zero() (the point
// projects more than 1 from the disk centre), which contributes nothing
template <typename R> static inline bool ff_nee(const FfAntenna<R> &a, Isect<R> &nee, CV3<R> &H) {
    V3<R> local = sub(nee.ray.o, a.center);
    local = sub(local, scale(dot(local, a.dir), a.dir));
    if (norm(local) > R(1)) return false;
    nee.ray.d = a.dir;
    nee.tMax = norm(sub(add(local, a.center), nee.ray.o));
    H = cv3_scale(a.pol, R(4) * Consts<R>::Pi * nee.tMax);
    return true;
}

// SurfaceEmitter (emitter.h:53-82)
template <typename R> static inline void surface_evaluate(const Isect<R> &incoming, Ray<R> &ray) {
    CV3<R> J = cross_rc(incoming.n, incoming.ray.H);
    J = cv3_scale(J, R(2));
    ray.H = cross_rc(ray.d, J);
    if (dot(ray.d, incoming.n) < R(0)) {
        for (int i = 0; i < 3; ++i) ray.H.c[i] = {R(0), R(0)};
    }
}
template <typename R> static inline void surface_connect(const Isect<R> &incoming, Isect<R> &outgoing) {
    R r = outgoing.t;
    outgoing.ray.addDistance(r);
    Cx<R> g = {R(1) / std::max(r, R(1e-3)), incoming.ray.k0()};  // Complex(0, k0) + 1/max(r,1e-3)
    g = cdivs(g, R(4) * Consts<R>::Pi * r);
    outgoing.ray.H = cv3_cmul(outgoing.ray.H, g);
}
template <typename R> static inline void surface_sample(const Isect<R> &incoming, R u0, R u1, Ray<R> &ray) {
    ray.d = uniform_sample_sphere(u0, u1);
    ray.H = cv3_scale(ray.H, R(1) / Consts<R>::Inv4Pi);
    surface_evaluate(incoming, ray);
}

// ----------------------------------------------------------------------------------
// Mesh + BVH (replaces Embree; hit semantics of src/arch/cpu.cpp:9-87)
// ----------------------------------------------------------------------------------
struct Mesh {
    std::vector<float> v;    // 3 per vertex
    std::vector<int32_t> f;  // 3 per triangle
    int64_t nt = 0;
};

struct BNode {
    float lo[3], hi[3];
    int32_t left;   // internal: index of first child (second = left + 1); leaf: first prim slot
    int32_t count;  // 0 for internal
};

struct Bvh {
    std::vector<BNode> nodes;
    std::vector<int32_t> prims;  // triangle ids in leaf order
    std::vector<float> tv;       // the vertices (v0, v1, v2) of prims[i] at 9 i: one fetch per test
};

struct Scene {
    Mesh mesh;
    Bvh bvh;
};

static bool build_bvh_ploc(Scene &s, const std::vector<float> &lo, const std::vector<float> &hi,
                           const std::vector<float> &cen);
static void build_bvh_sah(Scene &s, const std::vector<float> &lo, const std::vector<float> &hi,
                          const std::vector<float> &cen);

static void build_bvh(Scene &s) {
    const int64_t nt = s.mesh.nt;
    std::vector<float> lo(3 * nt), hi(3 * nt), cen(3 * nt);
    for (int64_t t = 0; t < nt; ++t) {
        for (int a = 0; a < 3; ++a) {
            float mn = std::numeric_limits<float>::infinity(), mx = -mn;
            for (int k = 0; k < 3; ++k) {
                float x = s.mesh.v[3 * s.mesh.f[3 * t + k] + a];
                mn = std::min(mn, x);
                mx = std::max(mx, x);
            }
            // padding keeps the box test conservative against rounding
            float pad = (std::abs(mn) + std::abs(mx)) * 1e-6f + 1e-7f;
            lo[3 * t + a] = mn - pad;
            hi[3 * t + a] = mx + pad;
            cen[3 * t + a] = 0.5f * (mn + mx);
        }
    }
    s.bvh.prims.resize(nt);
    for (int64_t i = 0; i < nt; ++i) s.bvh.prims[i] = int32_t(i);
    s.bvh.nodes.clear();
    if (!build_bvh_ploc(s, lo, hi, cen)) {
        s.bvh.nodes.clear();
        for (int64_t i = 0; i < nt; ++i) s.bvh.prims[i] = int32_t(i);
        build_bvh_sah(s, lo, hi, cen);
    }
    s.bvh.tv.resize(size_t(9) * nt);
    for (int64_t i = 0; i < nt; ++i)
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) s.bvh.tv[9 * i + 3 * k + a] = s.mesh.v[3 * s.mesh.f[3 * s.bvh.prims[i] + k] + a];
}

// Top-down binned SAH (32 bins on the axis of largest centroid extent, the median where
// no split separates): the fallback of build_bvh_ploc.
static void build_bvh_sah(Scene &s, const std::vector<float> &lo, const std::vector<float> &hi,
                          const std::vector<float> &cen) {
    const int64_t nt = s.mesh.nt;
    s.bvh.nodes.reserve(2 * std::max<int64_t>(nt, 1));
    struct Task {
        int32_t node, first, count;
    };
    std::vector<Task> stack;
    s.bvh.nodes.push_back(BNode{});
    stack.push_back({0, 0, int32_t(nt)});
    const int kBins = 32;
    while (!stack.empty()) {
        Task tk = stack.back();
        stack.pop_back();
        BNode nd;
        for (int a = 0; a < 3; ++a) {
            nd.lo[a] = std::numeric_limits<float>::infinity();
            nd.hi[a] = -std::numeric_limits<float>::infinity();
        }
        float clo[3], chi[3];
        for (int a = 0; a < 3; ++a) {
            clo[a] = std::numeric_limits<float>::infinity();
            chi[a] = -clo[a];
        }
        for (int32_t i = tk.first; i < tk.first + tk.count; ++i) {
            int32_t p = s.bvh.prims[i];
            for (int a = 0; a < 3; ++a) {
                nd.lo[a] = std::min(nd.lo[a], lo[3 * p + a]);
                nd.hi[a] = std::max(nd.hi[a], hi[3 * p + a]);
                clo[a] = std::min(clo[a], cen[3 * p + a]);
                chi[a] = std::max(chi[a], cen[3 * p + a]);
            }
        }
        if (tk.count <= 4) {
            nd.left = tk.first;
            nd.count = tk.count;
            s.bvh.nodes[tk.node] = nd;
            continue;
        }
        // binned SAH (32 bins) over each axis with a centroid extent; the cheapest split wins
        int axis = 0;
        float ext = chi[0] - clo[0];
        for (int a = 1; a < 3; ++a)
            if (chi[a] - clo[a] > ext) {
                ext = chi[a] - clo[a];
                axis = a;
            }
        int32_t mid = tk.first + tk.count / 2;
        {
            struct Bin {
                float lo[3], hi[3];
                int n;
            };
            auto area = [](const float *l, const float *h) {
                float dx = h[0] - l[0], dy = h[1] - l[1], dz = h[2] - l[2];
                if (dx < 0) return 0.f;
                return dx * dy + dy * dz + dz * dx;
            };
            float best = std::numeric_limits<float>::infinity();
            int bestSplit = -1, bestAxis = -1;
            for (int ax = 0; ax < 3; ++ax) {
                const float ex = chi[ax] - clo[ax];
                if (!(ex > 0.f)) continue;
                Bin bins[kBins];
                for (auto &b : bins) {
                    for (int a = 0; a < 3; ++a) {
                        b.lo[a] = std::numeric_limits<float>::infinity();
                        b.hi[a] = -b.lo[a];
                    }
                    b.n = 0;
                }
                for (int32_t i = tk.first; i < tk.first + tk.count; ++i) {
                    int32_t p = s.bvh.prims[i];
                    int bi = std::min(std::max(int((cen[3 * p + ax] - clo[ax]) / ex * kBins), 0), kBins - 1);
                    Bin &b = bins[bi];
                    b.n++;
                    for (int a = 0; a < 3; ++a) {
                        b.lo[a] = std::min(b.lo[a], lo[3 * p + a]);
                        b.hi[a] = std::max(b.hi[a], hi[3 * p + a]);
                    }
                }
                // suffix sweep for the right side, prefix for the left
                float rlo[kBins][3], rhi[kBins][3];
                int rn[kBins];
                for (int b = kBins - 1; b >= 0; --b) {
                    for (int a = 0; a < 3; ++a) {
                        rlo[b][a] = b + 1 < kBins ? std::min(rlo[b + 1][a], bins[b].lo[a]) : bins[b].lo[a];
                        rhi[b][a] = b + 1 < kBins ? std::max(rhi[b + 1][a], bins[b].hi[a]) : bins[b].hi[a];
                    }
                    rn[b] = (b + 1 < kBins ? rn[b + 1] : 0) + bins[b].n;
                }
                float L[3], H[3];
                for (int a = 0; a < 3; ++a) {
                    L[a] = std::numeric_limits<float>::infinity();
                    H[a] = -L[a];
                }
                int nl = 0;
                for (int sp = 1; sp < kBins; ++sp) {
                    nl += bins[sp - 1].n;
                    for (int a = 0; a < 3; ++a) {
                        L[a] = std::min(L[a], bins[sp - 1].lo[a]);
                        H[a] = std::max(H[a], bins[sp - 1].hi[a]);
                    }
                    const int nr = rn[sp];
                    if (nl == 0 || nr == 0) continue;
                    float c = area(L, H) * nl + area(rlo[sp], rhi[sp]) * nr;
                    if (c < best) {
                        best = c;
                        bestSplit = sp;
                        bestAxis = ax;
                    }
                }
            }
            if (bestSplit > 0) {
                const int ax = bestAxis;
                const float ex = chi[ax] - clo[ax];
                auto it = std::partition(
                    s.bvh.prims.begin() + tk.first, s.bvh.prims.begin() + tk.first + tk.count, [&](int32_t p) {
                        return std::min(std::max(int((cen[3 * p + ax] - clo[ax]) / ex * kBins), 0), kBins - 1) <
                               bestSplit;
                    });
                mid = int32_t(it - s.bvh.prims.begin());
                axis = ax;
            }
        }
        if (mid <= tk.first || mid >= tk.first + tk.count) {
            std::nth_element(s.bvh.prims.begin() + tk.first, s.bvh.prims.begin() + tk.first + tk.count / 2,
                             s.bvh.prims.begin() + tk.first + tk.count,
                             [&](int32_t a, int32_t b) { return cen[3 * a + axis] < cen[3 * b + axis]; });
            mid = tk.first + tk.count / 2;
        }
        int32_t l = int32_t(s.bvh.nodes.size());
        s.bvh.nodes.push_back(BNode{});
        s.bvh.nodes.push_back(BNode{});
        nd.left = l;
        nd.count = 0;
        s.bvh.nodes[tk.node] = nd;
        stack.push_back({l, tk.first, mid - tk.first});
        stack.push_back({l + 1, mid, tk.first + tk.count - mid});
    }
}

// Parallel locally-ordered clustering (Meister and Bittner 2018) over the Morton order of
// the centroids (21 bits per axis): each cluster finds, within 64 positions, the one whose
// merged box has the smallest surface area (ties: the lower position), mutual pairs
// merge, repeat; the searches run on all host threads. Subtrees of at most 4 triangles
// then become leaves, in the node layout the traversal reads (children at left and
// left + 1). A tree deeper than 100 levels (the traversal stack holds 128 entries) or a
// pass that merges nothing returns false, and build_bvh falls back to build_bvh_sah.
static bool build_bvh_ploc(Scene &s, const std::vector<float> &lo, const std::vector<float> &hi,
                           const std::vector<float> &cen) {
    const int64_t nt = s.mesh.nt;
    if (nt < 8 || nt >= (int64_t(1) << 30)) return false;
    float cl[3], ch[3];
    for (int a = 0; a < 3; ++a) {
        cl[a] = std::numeric_limits<float>::infinity();
        ch[a] = -cl[a];
    }
    for (int64_t t = 0; t < nt; ++t)
        for (int a = 0; a < 3; ++a) {
            cl[a] = std::min(cl[a], cen[3 * t + a]);
            ch[a] = std::max(ch[a], cen[3 * t + a]);
        }
    std::vector<std::pair<uint64_t, int32_t>> key(static_cast<size_t>(nt));
    for (int64_t t = 0; t < nt; ++t) {
        uint64_t code = 0;
        for (int a = 0; a < 3; ++a) {
            const float ext = ch[a] - cl[a];
            float u = ext > 0.f ? (cen[3 * t + a] - cl[a]) / ext : 0.5f;
            u = std::min(std::max(u, 0.f), 1.f);
            const uint64_t q = uint64_t(std::min(u * 2097152.f, 2097151.f));
            for (int b = 0; b < 21; ++b) code |= ((q >> b) & 1u) << (3 * b + a);
        }
        key[size_t(t)] = {code, int32_t(t)};
    }
    std::sort(key.begin(), key.end());
    struct PNode {  // a merge: children (>= 0 merge index, < 0 ~triangle), box, triangles
        int32_t c[2];
        float lo[3], hi[3];
        int32_t count;
    };
    std::vector<PNode> pn;
    pn.reserve(size_t(nt));
    std::vector<int32_t> id(static_cast<size_t>(nt));
    std::vector<float> box(static_cast<size_t>(6 * nt));
    for (int64_t i = 0; i < nt; ++i) {
        const int32_t t = key[size_t(i)].second;
        id[size_t(i)] = ~t;
        for (int a = 0; a < 3; ++a) {
            box[6 * i + a] = lo[3 * size_t(t) + a];
            box[6 * i + 3 + a] = hi[3 * size_t(t) + a];
        }
    }
    auto merged_area = [&](const float *a, const float *b) {
        const float dx = std::max(a[3], b[3]) - std::min(a[0], b[0]);
        const float dy = std::max(a[4], b[4]) - std::min(a[1], b[1]);
        const float dz = std::max(a[5], b[5]) - std::min(a[2], b[2]);
        return dx * dy + dy * dz + dz * dx;
    };
    const int R = 64;
    const int threads = int(std::max(1u, std::thread::hardware_concurrency()));
    std::vector<int32_t> nearest;
    while (id.size() > 1) {
        const int64_t n = int64_t(id.size());
        nearest.assign(size_t(n), -1);
        std::vector<std::thread> pool;
        for (int w = 0; w < threads; ++w)
            pool.emplace_back([&, w] {
                const int64_t a = n * w / threads, b = n * (w + 1) / threads;
                for (int64_t i = a; i < b; ++i) {
                    float best = std::numeric_limits<float>::infinity();
                    int64_t bj = -1;
                    for (int64_t j = std::max<int64_t>(0, i - R); j <= std::min<int64_t>(n - 1, i + R); ++j) {
                        if (j == i) continue;
                        const float ar = merged_area(&box[6 * i], &box[6 * j]);
                        if (ar < best) {
                            best = ar;
                            bj = j;
                        }
                    }
                    nearest[size_t(i)] = int32_t(bj);
                }
            });
        for (auto &th : pool) th.join();
        std::vector<int32_t> nid;
        std::vector<float> nbox;
        nid.reserve(size_t(n));
        nbox.reserve(size_t(6) * n);
        for (int64_t i = 0; i < n; ++i) {
            const int64_t j = nearest[size_t(i)];
            const bool mutual = j >= 0 && nearest[size_t(j)] == i;
            if (mutual && i > j) continue;  // merged by j
            if (mutual) {
                PNode m;
                m.c[0] = id[size_t(i)];
                m.c[1] = id[size_t(j)];
                m.count = (m.c[0] < 0 ? 1 : pn[size_t(m.c[0])].count) + (m.c[1] < 0 ? 1 : pn[size_t(m.c[1])].count);
                for (int a = 0; a < 3; ++a) {
                    m.lo[a] = std::min(box[6 * i + a], box[6 * j + a]);
                    m.hi[a] = std::max(box[6 * i + 3 + a], box[6 * j + 3 + a]);
                }
                pn.push_back(m);
                nid.push_back(int32_t(pn.size() - 1));
                for (int a = 0; a < 3; ++a) nbox.push_back(m.lo[a]);
                for (int a = 0; a < 3; ++a) nbox.push_back(m.hi[a]);
            } else {
                nid.push_back(id[size_t(i)]);
                for (int a = 0; a < 6; ++a) nbox.push_back(box[6 * i + a]);
            }
        }
        if (int64_t(nid.size()) == n) return false;
        id.swap(nid);
        box.swap(nbox);
    }
    // the node layout: a subtree of at most 4 triangles is a leaf, its triangles gathered
    // in order; otherwise two consecutive nodes for the children
    struct Task {
        int32_t ref, node, depth;
    };
    std::vector<Task> stack{{id[0], 0, 0}};
    s.bvh.nodes.assign(1, BNode{});
    int32_t filled = 0;
    std::vector<int32_t> gather;
    while (!stack.empty()) {
        const Task tk = stack.back();
        stack.pop_back();
        if (tk.depth > 100) return false;
        BNode nd;
        const int32_t cnt = tk.ref < 0 ? 1 : pn[size_t(tk.ref)].count;
        if (tk.ref < 0) {
            const int32_t t = ~tk.ref;
            for (int a = 0; a < 3; ++a) {
                nd.lo[a] = lo[3 * size_t(t) + a];
                nd.hi[a] = hi[3 * size_t(t) + a];
            }
        } else {
            for (int a = 0; a < 3; ++a) {
                nd.lo[a] = pn[size_t(tk.ref)].lo[a];
                nd.hi[a] = pn[size_t(tk.ref)].hi[a];
            }
        }
        if (cnt <= 4) {
            gather.assign(1, tk.ref);
            nd.left = filled;
            nd.count = cnt;
            while (!gather.empty()) {
                const int32_t r = gather.back();
                gather.pop_back();
                if (r < 0) {
                    s.bvh.prims[size_t(filled++)] = ~r;
                } else {
                    gather.push_back(pn[size_t(r)].c[1]);
                    gather.push_back(pn[size_t(r)].c[0]);
                }
            }
            s.bvh.nodes[size_t(tk.node)] = nd;
            continue;
        }
        const int32_t l = int32_t(s.bvh.nodes.size());
        s.bvh.nodes.push_back(BNode{});
        s.bvh.nodes.push_back(BNode{});
        nd.left = l;
        nd.count = 0;
        s.bvh.nodes[size_t(tk.node)] = nd;
        stack.push_back({pn[size_t(tk.ref)].c[1], l + 1, tk.depth + 1});
        stack.push_back({pn[size_t(tk.ref)].c[0], l, tk.depth + 1});
    }
    return filled == nt;
}

// Moller-Trumbore in precision R. Accepts tnear < t <= tfar.
template <typename R>
static inline bool tri_hit(const float *vtx, V3<R> o, V3<R> d, R tnear, R tfar, R &t_out) {
    const float *v0f = vtx, *v1f = vtx + 3, *v2f = vtx + 6;
    V3<R> v0{R(v0f[0]), R(v0f[1]), R(v0f[2])};
    V3<R> v1{R(v1f[0]), R(v1f[1]), R(v1f[2])};
    V3<R> v2{R(v2f[0]), R(v2f[1]), R(v2f[2])};
    V3<R> e1 = sub(v1, v0), e2 = sub(v2, v0);
    V3<R> pv = cross(d, e2);
    R det = dot(e1, pv);
    if (det == R(0)) return false;
    R inv = R(1) / det;
    V3<R> tv = sub(o, v0);
    R u = dot(tv, pv) * inv;
    if (u < R(0) || u > R(1)) return false;
    V3<R> qv = cross(tv, e1);
    R v = dot(d, qv) * inv;
    if (v < R(0) || u + v > R(1)) return false;
    R t = dot(e2, qv) * inv;
    if (!(t > tnear && t <= tfar)) return false;
    t_out = t;
    return true;
}

template <typename R> static inline V3<R> tri_normal(const Mesh &m, int32_t prim) {
    const float *v0f = &m.v[3 * m.f[3 * prim + 0]];
    const float *v1f = &m.v[3 * m.f[3 * prim + 1]];
    const float *v2f = &m.v[3 * m.f[3 * prim + 2]];
    V3<R> v0{R(v0f[0]), R(v0f[1]), R(v0f[2])};
    V3<R> v1{R(v1f[0]), R(v1f[1]), R(v1f[2])};
    V3<R> v2{R(v2f[0]), R(v2f[1]), R(v2f[2])};
    return normalized(cross(sub(v1, v0), sub(v2, v0)));
}

template <typename R>
static inline bool box_hit(const BNode &n, V3<R> o, V3<R> inv, R tnear, R tfar) {
    R t0x = (R(n.lo[0]) - o.x) * inv.x, t1x = (R(n.hi[0]) - o.x) * inv.x;
    R t0y = (R(n.lo[1]) - o.y) * inv.y, t1y = (R(n.hi[1]) - o.y) * inv.y;
    R t0z = (R(n.lo[2]) - o.z) * inv.z, t1z = (R(n.hi[2]) - o.z) * inv.z;
    // fmin/fmax ignore NaN (0 * inf), which leaves that slab unbounded: conservative
    R tmin = std::fmax(std::fmax(std::fmin(t0x, t1x), std::fmin(t0y, t1y)), std::fmax(std::fmin(t0z, t1z), tnear));
    R tmax = std::fmin(std::fmin(std::fmax(t0x, t1x), std::fmax(t0y, t1y)), std::fmin(std::fmax(t0z, t1z), tfar));
    return tmin <= tmax * R(1.0000004);
}

// entry distance of a box the ray reaches (box_hit's test), +inf for one it misses
template <typename R>
static inline R box_entry(const BNode &n, V3<R> o, V3<R> inv, R tnear, R tfar) {
    R t0x = (R(n.lo[0]) - o.x) * inv.x, t1x = (R(n.hi[0]) - o.x) * inv.x;
    R t0y = (R(n.lo[1]) - o.y) * inv.y, t1y = (R(n.hi[1]) - o.y) * inv.y;
    R t0z = (R(n.lo[2]) - o.z) * inv.z, t1z = (R(n.hi[2]) - o.z) * inv.z;
    R tmin = std::fmax(std::fmax(std::fmin(t0x, t1x), std::fmin(t0y, t1y)), std::fmax(std::fmin(t0z, t1z), tnear));
    R tmax = std::fmin(std::fmin(std::fmax(t0x, t1x), std::fmax(t0y, t1y)), std::fmin(std::fmax(t0z, t1z), tfar));
    return tmin <= tmax * R(1.0000004) ? tmin : std::numeric_limits<R>::infinity();
}

// closest hit; returns prim or -1
template <typename R>
static int32_t closest_hit(const Scene &s, V3<R> o, V3<R> d, R tnear, R tfar, R &t_best) {
    V3<R> inv{R(1) / d.x, R(1) / d.y, R(1) / d.z};
    int32_t best = -1;
    t_best = tfar;
    if (s.bvh.nodes.empty() || s.mesh.nt == 0) return -1;
    int32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const BNode &n = s.bvh.nodes[stack[--sp]];
        if (!box_hit(n, o, inv, tnear, t_best)) continue;
        if (n.count) {
            for (int32_t i = n.left; i < n.left + n.count; ++i) {
                int32_t p = s.bvh.prims[i];
                R t;
                if (tri_hit(&s.bvh.tv[size_t(9) * i], o, d, tnear, tfar, t)) {
                    if (t < t_best || (t == t_best && (best < 0 || p < best))) {
                        t_best = t;
                        best = p;
                    }
                }
            }
        } else {
            // nearer child first (pops last): only the pruning order changes, every node
            // is still re-tested against the current closest hit when it is popped
            const R e0 = box_entry(s.bvh.nodes[n.left], o, inv, tnear, t_best);
            const R e1 = box_entry(s.bvh.nodes[n.left + 1], o, inv, tnear, t_best);
            if (e1 < e0) {
                stack[sp++] = n.left;
                stack[sp++] = n.left + 1;
            } else {
                stack[sp++] = n.left + 1;
                stack[sp++] = n.left;
            }
        }
    }
    return best;
}

template <typename R> static bool occluded(const Scene &s, V3<R> o, V3<R> d, R tnear, R tfar) {
    V3<R> inv{R(1) / d.x, R(1) / d.y, R(1) / d.z};
    if (s.bvh.nodes.empty() || s.mesh.nt == 0) return false;
    int32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const BNode &n = s.bvh.nodes[stack[--sp]];
        if (!box_hit(n, o, inv, tnear, tfar)) continue;
        if (n.count) {
            for (int32_t i = n.left; i < n.left + n.count; ++i) {
                R t;
                if (tri_hit(&s.bvh.tv[size_t(9) * i], o, d, tnear, tfar, t)) return true;
            }
        } else {
            stack[sp++] = n.left + 1;
            stack[sp++] = n.left;
        }
    }
    return false;
}

// RT::intersect (src/arch/cpu.cpp:63-87)
template <typename R> static inline void rt_intersect(const Scene &s, Isect<R> &is) {
    R t;
    int32_t p = closest_hit(s, is.ray.o, is.ray.d, Consts<R>::Epsilon, is.tMax, t);
    if (p >= 0) {
        is.t = t;
        is.p = is.ray.at(t);
        is.n = tri_normal<R>(s.mesh, p);
        if (dot(is.n, is.ray.d) > R(0)) is.n = neg(is.n);
    }
}
// RT::visible (src/arch/cpu.cpp:53-61)
template <typename R> static inline bool rt_visible(const Scene &s, const Isect<R> &is) {
    return !occluded(s, is.ray.o, is.ray.d, Consts<R>::Epsilon, is.tMax);
}

// ----------------------------------------------------------------------------------
// Frame (radar.h:173-701), accumulated in Real with a CAS loop like radar.h:63-83
// ----------------------------------------------------------------------------------
template <typename R> static inline void atomic_add(R *addr, R v) {
    using U = typename std::conditional<sizeof(R) == 4, uint32_t, uint64_t>::type;
    auto &bits = *reinterpret_cast<std::atomic<U> *>(addr);
    U oldBits = bits.load(), newBits;
    do {
        R f;
        std::memcpy(&f, &oldBits, sizeof(R));
        f = f + v;
        std::memcpy(&newBits, &f, sizeof(R));
    } while (!bits.compare_exchange_weak(oldBits, newBits));
}

template <typename R> struct Frame {
    int chirps = 1, samples = 1, channels = 1;
    R *data = nullptr;  // interleaved re, im
    bool exact = false; // exact finite-N Dirichlet synthesis instead of Frame::splat<16>
    size_t index(int c, int s, int ch) const { return (size_t(c) * samples + s) * channels + ch; }
};

// radar.h:91-96 safe_modulo(T a, unsigned b): `a % b` converts a negative int to
// unsigned first, so a negative a wraps as (a + 2^32) mod b. That equals the true
// modulo only when b divides 2^32 (powers of two); restated as the reference computes it.
static inline int safe_mod(int a, int b) {
    int m = int(unsigned(a) % unsigned(b));
    if (m < 0) m += b;
    return m;
}

// Frame::splat<16> (radar.h:564-626) for an index whose chirp/channel are integral
template <typename R> static void frame_splat(Frame<R> &f, R idx_chirp, R idx_sample, R idx_channel, Cx<R> value) {
    R raw[3] = {idx_chirp, idx_sample, idx_channel};
    int center[3];
    R shifts[3];
    R weight = 1;
    for (int i = 0; i < 3; ++i) {
        center[i] = int(std::round(raw[i]));
        R shift = raw[i] - R(center[i]);
        if (std::abs(shift) < R(1e-4)) {
            shifts[i] = 0;
            continue;
        }
        shifts[i] = shift;
        R shiftPi = R(M_PI * double(shift));
        value = cmul(value, cexpj(shiftPi));
        weight = R(double(weight) * (double(std::sin(shiftPi)) / M_PI));
    }
    const int dims[3] = {f.chirps, f.samples, f.channels};
    // recursive expansion over the three components (only non-zero shifts expand)
    int lo[3], hi[3];
    for (int i = 0; i < 3; ++i) {
        lo[i] = shifts[i] == R(0) ? 0 : -16;
        hi[i] = shifts[i] == R(0) ? 0 : 16;
    }
    for (int a = lo[0]; a <= hi[0]; ++a) {
        R w0 = shifts[0] == R(0) ? weight : weight / (shifts[0] - R(a));
        int c = shifts[0] == R(0) ? center[0] : safe_mod(center[0] + a, dims[0]);
        for (int b = lo[1]; b <= hi[1]; ++b) {
            R w1 = shifts[1] == R(0) ? w0 : w0 / (shifts[1] - R(b));
            int s = shifts[1] == R(0) ? center[1] : safe_mod(center[1] + b, dims[1]);
            for (int k = lo[2]; k <= hi[2]; ++k) {
                R w2 = shifts[2] == R(0) ? w1 : w1 / (shifts[2] - R(k));
                int ch = shifts[2] == R(0) ? center[2] : safe_mod(center[2] + k, dims[2]);
                // the reference indexes center directly for a delta component; a rounded
                // index equal to the dimension (e.g. sample >= N-0.5) would be out of
                // bounds there. It is wrapped here (the spectrum is periodic).
                c = safe_mod(c, dims[0]);
                s = safe_mod(s, dims[1]);
                ch = safe_mod(ch, dims[2]);
                size_t id = f.index(c, s, ch);
                atomic_add(&f.data[2 * id + 0], w2 * value.re);
                atomic_add(&f.data[2 * id + 1], w2 * value.im);
            }
        }
    }
}

// The spectrum of one sampled complex exponential, without truncation: the value the
// contribution adds to range bin m is value * D_N(b - m) / N with
// D_N(x) = sum_{n<N} exp(j 2 pi x n / N) = exp(j pi x (N-1)/N) sin(pi x) / sin(pi x / N).
// (Frame::splat<16>, radar.h:564-626, is its N -> infinity limit truncated to +-16 bins.)
// Evaluated in double; used by the FP64 oracle of the fine-histogram synthesis mode.
template <typename R> static void frame_splat_exact(Frame<R> &f, double b, Cx<R> value) {
    const int N = f.samples;
    const double pi = 3.14159265358979323846;
    for (int m = 0; m < N; ++m) {
        double x = b - double(m);
        double xr = std::fmod(x, double(N));
        if (xr < 0) xr += N;
        double re, im;
        if (std::abs(std::sin(pi * xr / N)) < 1e-12) {
            re = 1.0;  // D_N / N at multiples of N
            im = 0.0;
        } else {
            double mag = std::sin(pi * xr) / std::sin(pi * xr / N) / N;
            double ph = pi * xr * (N - 1) / N;
            re = mag * std::cos(ph);
            im = mag * std::sin(ph);
        }
        double vr = double(value.re), vi = double(value.im);
        size_t id = f.index(0, m, 0);
        atomic_add(&f.data[2 * id + 0], R(vr * re - vi * im));
        atomic_add(&f.data[2 * id + 1], R(vr * im + vi * re));
    }
}

// ----------------------------------------------------------------------------------
// Integrator + PathTracer::sample (path.h:235-451, integrator.h:107-168)
// ----------------------------------------------------------------------------------
// Integrator::measureRay (integrator.h:107-110): exp(j 2 pi (f0 - dt S / 2) dt), the
// angle in R and its cos/sin through radar::polar (cexpj)
template <typename R> static inline Cx<R> measure_ray(R dt, R startFreq, R freqSlope) {
    R angle = R(2) * Consts<R>::Pi * (startFreq - dt * freqSlope / R(2)) * dt;
    return cexpj(angle);
}

// PIndex::setTime (radar.h:232-241): the fractional range bin N frac(dt S / adcRate);
// a CW configuration (slope 0) puts everything in bin 0
template <typename R> static inline R set_time_sample(R delta_t, R freqSlope, R adcRate, int samples) {
    if (freqSlope == R(0)) return R(0);
    R delta_f = delta_t * freqSlope;
    R x = delta_f / adcRate;
    return R(samples) * (x - std::floor(x));
}

template <typename R> struct Rf {
    R startFreq, freqSlope, adcRate, idleTime, rampTime, antennaDelay;
    R bandwidth() const { return freqSlope * rampTime; }
    R chirpFrequency() const { return R(1) / (idleTime + rampTime); }
};

struct Flags {
    bool onlyIndirect, useGO, poDiffraction, doGuiding, correctPhase, filterGuiding, doFiltering,
        filteringSphere, produceDebugImage;
    int maxDepth;
    float filteringMin, filteringMax, filteringRadius;
};

// ----------------------------------------------------------------------------------
// Path guiding of the TX primary sample square: GuidingWrapper (path.h:17-131) with the
// settings of PathTracer::setup (path.h:226-233: uniform mixture 0.1, split threshold
// 0.005, second moment). The reference's distribution is libguiding's BTree (the
// 3rdparty/libguiding submodule, github.com/iRath96/libguiding, absent from the
// reference sources, so its own code and pinned commit are unknown here). Restated is
// the product's tree, which follows that interface:
//   - a 2-D binary tree over [0,1)^2; a node's region halves at its midpoint along x0 at
//     even depths and x1 at odd ones; the children of a node are stored as a pair (first
//     child c, second c + 1), -1 marks a leaf; at most 2048 nodes and depth 24;
//   - sampling tree: per node the probability of its first child;
//   - training tree: per node the sum of w d^2 (the second-moment statistic of
//     GuidingWrapper::splat(density d, weight w), path.h:96-111, 448-450);
//   - step (path.h:119-126): build leaf energies sqrt(sum w d^2 * area) and sums up the
//     tree, copy into the sampling tree, refine the training tree in pre-order: a node
//     whose energy fraction exceeds the threshold is split (an old leaf into halves of
//     half the fraction each), anything else becomes a leaf; statistics restart at 0.
// ----------------------------------------------------------------------------------
constexpr int kGuideNodes = 2048;
constexpr int kGuideDepth = 24;
constexpr float kGuideUniform = 0.1f;     // path.h:229
constexpr float kGuideSplit = 0.005f;     // path.h:230
constexpr float kBelowOne = 0x1.fffffep-1f;

struct GuideTree {
    std::vector<int32_t> samp_child = std::vector<int32_t>(kGuideNodes, -1);
    std::vector<float> samp_p = std::vector<float>(kGuideNodes, 0.5f);
    std::vector<int32_t> train_child = std::vector<int32_t>(kGuideNodes, -1);
    std::vector<float> acc2 = std::vector<float>(kGuideNodes, 0.f);
    int32_t count = 1;  // nodes of the training tree
};

// descent by position: the density of the tree at x relative to uniform (with pf), or
// the leaf holding x
static float tree_locate(const int32_t *child, const float *pf, float x0, float x1, int32_t *leaf) {
    float pdf = 1.f;
    float lo[2] = {0.f, 0.f}, half[2] = {1.f, 1.f};
    const float x[2] = {x0, x1};
    int32_t node = 0;
    for (int depth = 0; depth < kGuideDepth && child[node] >= 0; ++depth) {
        const int ax = depth & 1;
        half[ax] *= 0.5f;
        const bool first = x[ax] < lo[ax] + half[ax];
        if (pf) pdf *= 2.f * (first ? pf[node] : 1.f - pf[node]);
        if (!first) lo[ax] += half[ax];
        node = child[node] + (first ? 0 : 1);
    }
    if (leaf) *leaf = node;
    return pdf;
}

// warps x through the sampling tree (each level picks a child by its probability and
// rescales the coordinate of that level's axis); returns the tree density there
static float tree_warp(const int32_t *child, const float *pf, float &x0, float &x1) {
    float pdf = 1.f;
    float lo[2] = {0.f, 0.f}, half[2] = {1.f, 1.f};
    float x[2] = {x0, x1};
    int32_t node = 0;
    for (int depth = 0; depth < kGuideDepth && child[node] >= 0; ++depth) {
        const int ax = depth & 1;
        const float p = pf[node];
        half[ax] *= 0.5f;
        if (x[ax] < p) {
            x[ax] = p > 0.f ? x[ax] / p : 0.f;
            pdf *= 2.f * p;
            node = child[node];
        } else {
            x[ax] = p < 1.f ? (x[ax] - p) / (1.f - p) : 0.f;
            pdf *= 2.f * (1.f - p);
            lo[ax] += half[ax];
            node = child[node] + 1;
        }
        x[ax] = std::min(std::max(x[ax], 0.f), kBelowOne);
    }
    x0 = std::min(lo[0] + x[0] * half[0], kBelowOne);
    x1 = std::min(lo[1] + x[1] * half[1], kBelowOne);
    return pdf;
}

// GuidingWrapper::sample (path.h:54-82): warps (x0, x1) in place, returns the mixture pdf
static float guide_mix_sample(const GuideTree &g, float &x0, float &x1) {
    float pdf = 1.f - kGuideUniform;
    if (x0 < kGuideUniform) {
        x0 /= kGuideUniform;
        pdf *= tree_locate(g.samp_child.data(), g.samp_p.data(), x0, x1, nullptr);
    } else {
        x0 -= kGuideUniform;
        x0 /= 1.f - kGuideUniform;
        pdf *= tree_warp(g.samp_child.data(), g.samp_p.data(), x0, x1);
    }
    return pdf + kGuideUniform;
}

// GuidingWrapper::splat (path.h:96-111) as PathTracer::sample calls it (path.h:448-450):
// density |guidingWeight| * pdf, weight 1 / pdf, at the warped primary sample
static void guide_train(GuideTree &g, Cx<float> gw, float pdf, float x0, float x1) {
    if (!(pdf > 0.f)) return;
    const float density = cabs(gw) * pdf;
    if (density == 0.f) return;
    const float weight = 1.f / pdf;
    int32_t leaf = 0;
    tree_locate(g.train_child.data(), nullptr, x0, x1, &leaf);
    g.acc2[leaf] += weight * density * density;
}

// GuidingWrapper::step (path.h:119-126)
static void guide_step(GuideTree &g) {
    const int n = std::min(std::max(g.count, 1), kGuideNodes);
    const int32_t *tc = g.train_child.data();
    std::vector<int> depth(n, 0);
    std::vector<float> e(n, 0.f);
    for (int i = 0; i < n; ++i)  // children follow their parent
        if (tc[i] >= 0 && tc[i] + 1 < n) depth[tc[i]] = depth[tc[i] + 1] = depth[i] + 1;
    for (int i = n - 1; i >= 0; --i)
        e[i] = tc[i] < 0 ? std::sqrt(std::max(g.acc2[i], 0.f) * std::ldexp(1.f, -depth[i])) : e[tc[i]] + e[tc[i] + 1];
    for (int i = 0; i < n; ++i) {
        g.samp_child[i] = tc[i];
        if (tc[i] >= 0) {
            const float s = e[tc[i]] + e[tc[i] + 1];
            g.samp_p[i] = s > 0.f ? e[tc[i]] / s : 0.5f;
        } else {
            g.samp_p[i] = 0.5f;
        }
    }
    int ncount = n;
    const float total = e[0];
    if (total > 0.f) {
        struct Pending {
            int old;    // node of the old training tree (-1: inside a split old leaf)
            float f;    // energy fraction
            int d;      // depth
            int slot;   // node of the new tree
        };
        constexpr int kMaxPending = 2 * kGuideDepth + 4;
        std::vector<int32_t> out(kGuideNodes, -1);
        Pending stack[kMaxPending];
        int top = 0;
        ncount = 1;
        stack[top++] = Pending{0, 1.f, 0, 0};
        while (top > 0) {
            const Pending it = stack[--top];
            const bool split = it.f > kGuideSplit && it.d < kGuideDepth && ncount + 2 <= kGuideNodes &&
                               top + 2 <= kMaxPending;
            if (!split) {
                out[it.slot] = -1;
                continue;
            }
            const int c = ncount;
            ncount += 2;
            out[it.slot] = c;
            if (it.old >= 0 && tc[it.old] >= 0) {
                const int oc = tc[it.old];
                const float eo = e[it.old];
                const float f0 = eo > 0.f ? it.f * (e[oc] / eo) : 0.5f * it.f;
                const float f1 = eo > 0.f ? it.f * (e[oc + 1] / eo) : 0.5f * it.f;
                stack[top++] = Pending{oc + 1, f1, it.d + 1, c + 1};
                stack[top++] = Pending{oc, f0, it.d + 1, c};
            } else {
                stack[top++] = Pending{-1, 0.5f * it.f, it.d + 1, c + 1};
                stack[top++] = Pending{-1, 0.5f * it.f, it.d + 1, c};
            }
        }
        for (int i = 0; i < ncount; ++i) g.train_child[i] = out[i];
    }
    std::fill(g.acc2.begin(), g.acc2.end(), 0.f);
    g.count = ncount;
}

template <typename R> struct Tracer {
    const Scene *scene;
    Rf<R> rf;
    Antenna<R> tx, rx;
    bool farField = false;  // TX and RX are the far-field antennas below
    FfAntenna<R> ftx, frx;
    Flags fl;
    Frame<R> frame;
    R currentSampleWeight = 1;
    int64_t sampleIndexOffset = 0;
    bool floatSamples = false;
    oracle_record *records = nullptr;  // optional per-sample event log
    int maxRecords = 0;
    GuideTree *guide = nullptr;  // doGuiding: the pose's tree (single-threaded runs)
    bool guideTrain = false;     // splat into its training tree (not the final iteration)

    Cx<R> measureRay(R dt) const { return measure_ray(dt, rf.startFreq, rf.freqSlope); }

    // Integrator::splat (integrator.h:113-148) without the debug image
    void splat(int channel, R delta_t, R dphase, Cx<R> measurement, R weight, oracle_record *rec) {
        if (!fl.produceDebugImage) {
            if (weight == R(0) || (measurement.re == R(0) || measurement.im == R(0))) return;
        }
        delta_t += rf.antennaDelay;
        R sample = set_time_sample(delta_t, rf.freqSlope, rf.adcRate, frame.samples);
        R delta_p = R(2) * rf.startFreq * R(0) / Consts<R>::SpeedOfLight;
        R y = delta_p / rf.chirpFrequency();
        R chirp = R(frame.chirps) * (y - std::floor(y));
        Cx<R> contribution = cmul(measurement, measureRay(delta_t));
        Cx<R> value = cscale(contribution, weight);
        if (rec) {
            rec->bin = double(sample);
            rec->value_re = double(value.re);
            rec->value_im = double(value.im);
            rec->splatted = 1;
        }
        if (frame.exact)
            frame_splat_exact(frame, double(sample), value);
        else
            frame_splat(frame, chirp, sample, R(channel), value);
    }

    void reflectRay(Ray<R> &ray, const Isect<R> &isect) const {  // integrator.h:164-168
        CV3<R> H = ray.H;
        ray.d = isect.R_();
        Cx<R> nh = dot_rc(isect.n, H);
        V3<R> n2 = scale(R(2), isect.n);
        CV3<R> t;
        for (int i = 0; i < 3; ++i) t.c[i] = cscale(nh, i == 0 ? n2.x : i == 1 ? n2.y : n2.z);
        ray.H = cv3_sub(t, H);
    }

    void sample(int64_t index) {
        Halton<R> sampler;
        sampler.index = uint64_t(sampleIndexOffset + index);
        sampler.dim = 0;
        sampler.float_samples = floatSamples;
        const R maxDist = rf.adcRate / rf.freqSlope * Consts<R>::SpeedOfLight;
        const R sampleWeight = currentSampleWeight;
        R primaryPdf = 1;
        Cx<R> guidingWeight{R(0), R(0)};
        float gx0 = 0.f, gx1 = 0.f;  // the primary sample after guiding (training position)
        Isect<R> isect;
        Ray<R> &ray = isect.ray;
        ray.frequency = rf.startFreq + sampler.get1D() * rf.bandwidth();
        Isect<R> incoming;  // SurfaceEmitter::incoming
        R r = 0;
        R cosTheta = 1;
        int nrec = 0;
        while (true) {
            V3<R> tmpd = ray.d;
            if (ray.depth == 0) {
                R u0, u1;
                sampler.get2D(u0, u1);
                if (guide) {  // GuidingWrapper::sample in float (path.h:265-270)
                    gx0 = float(u0);
                    gx1 = float(u1);
                    primaryPdf = R(guide_mix_sample(*guide, gx0, gx1));
                    u0 = R(gx0);
                    u1 = R(gx1);
                }
                if (farField)
                    ff_sample(ftx, u0, u1, ray);
                else
                    antenna_sample(tx, u0, u1, ray);
                ray.H = cv3_scale(ray.H, R(1) / primaryPdf);
            } else {
                if (!fl.useGO) {
                    R u0, u1;
                    sampler.get2D(u0, u1);
                    surface_sample(incoming, u0, u1, ray);
                } else {
                    reflectRay(ray, isect);
                }
            }

            // next event estimation (single RX channel, path.h:292)
            do {
                if (ray.depth == 0 && fl.onlyIndirect) break;
                Isect<R> nee = isect;
                nee.t = std::numeric_limits<R>::infinity();
                CV3<R> Hrx;
                if (farField) {
                    // the direct term: FFAntenna::evaluate zeroes the ray (emitter.h:253-255)
                    if (ray.depth == 0) break;
                    if (!ff_nee(frx, nee, Hrx)) break;
                } else {
                    Hrx = antenna_nee(rx, nee);
                }
                if (!fl.poDiffraction && !rt_visible(*scene, nee)) break;
                nee.t = nee.tMax;
                if (ray.depth == 0) {
                    antenna_evaluate(tx, nee.ray);
                    antenna_connect(nee);
                } else {
                    surface_evaluate(incoming, nee.ray);
                    surface_connect(incoming, nee);
                }
                Cx<R> v = dot_cc(nee.ray.H, Hrx);
                R dphase = 0;
                if (ray.depth > 0) {
                    if (fl.correctPhase) {
                        V3<R> rxPos = nee.ray.at(nee.t);
                        V3<R> virtualTx = sub(nee.ray.o, scale(r, ray.d));
                        R dist = norm(sub(virtualTx, rxPos));
                        nee.ray.time = dist / Consts<R>::SpeedOfLight;
                        R pw = Consts<R>::Pi * R(fl.filteringRadius) * nee.ray.wavelength();
                        v = cdivs(cscale(dot_cc(ray.H, Hrx), Consts<R>::Pi * dist), R(double(pw) * double(pw)));
                        v = cdivs(v, R(4) * Consts<R>::Pi);
                    } else if (fl.useGO) {
                        v = cscale(v, r / cosTheta);
                        v = cdivs(v, R(4) * Consts<R>::Pi);
                        if (double(cosTheta) < 1e-3) break;
                    }
                    if (fl.filteringSphere) {
                        V3<R> rxPos = nee.ray.at(nee.t);
                        R lambda = std::max<R>(R(0), dot(ray.d, sub(rxPos, ray.o)));
                        R rxDist = norm(sub(ray.at(lambda), rxPos));
                        dphase = rxDist;
                    } else {
                        R c = dot(normalized(sub(nee.ray.d, tmpd)), isect.n);
                        dphase = r * std::sqrt(R(1) - c * c) / c;
                    }
                    dphase /= nee.ray.wavelength();
                    if (fl.doFiltering) {
                        if (fl.filteringSphere) {
                            if (dphase > R(fl.filteringRadius)) {
                                if (fl.correctPhase) {
                                    if (fl.filterGuiding) {  // path.h:363-367
                                        const R q = dphase / R(fl.filteringRadius);
                                        guidingWeight = cadd(guidingWeight, cdivs(v, R(double(q) * double(q) + 1.0)));
                                    }
                                    v = {R(0), R(0)};
                                } else {
                                    R q = dphase / R(fl.filteringRadius) - R(1);
                                    R taper = std::max<R>(R(1.0 - 0.20 * double(q)), R(0));
                                    v = cscale(v, taper);
                                }
                            }
                        } else {
                            if (dphase > R(fl.filteringMax)) {
                                if (fl.filterGuiding) {  // path.h:378-382
                                    const R q = dphase / R(fl.filteringMax);
                                    guidingWeight = cadd(guidingWeight, cdivs(v, R(double(q) * double(q) + 1.0)));
                                }
                                v = {R(0), R(0)};
                            }
                            if (dphase > R(fl.filteringMin))
                                v = cscale(v, (R(fl.filteringMax) - dphase) / (R(fl.filteringMax) - R(fl.filteringMin)));
                        }
                    }
                }
                if (ray.depth > 0) guidingWeight = cadd(guidingWeight, v);  // path.h:389-391
                oracle_record *rec = nullptr;
                if (records && nrec < maxRecords) {
                    rec = &records[nrec++];
                    rec->depth = ray.depth;
                    rec->time = double(nee.ray.time);
                    rec->v_re = double(v.re);
                    rec->v_im = double(v.im);
                    rec->dphase = double(dphase);
                    rec->splatted = 0;
                }
                splat(0, nee.ray.time, dphase, v, sampleWeight, rec);
            } while (false);

            if (ray.depth >= fl.maxDepth || r >= maxDist) break;
            if (cv3_is_zero(ray.H)) break;
            isect.reset();
            rt_intersect(*scene, isect);
            if (!isect.valid()) break;
            cosTheta = isect.cosTheta();
            if (double(cosTheta) < 1e-3) break;
            r += isect.t;
            if (!fl.useGO) {
                if (ray.depth == 0) {
                    if (!farField) antenna_connect(isect);  // FFAntenna::connect does nothing
                } else {
                    surface_connect(incoming, isect);
                }
                ray.H = cv3_scale(ray.H, isect.t * isect.t / cosTheta);
            } else {
                ray.addDistance(isect.t);
            }
            if (cv3_is_zero(ray.H)) break;
            incoming = isect;
            ray.o = isect.p;
            ray.depth++;
        }
        // path.h:448-450 (the splat's float arguments)
        if (guide && guideTrain && primaryPdf > R(0))
            guide_train(*guide, Cx<float>{float(guidingWeight.re), float(guidingWeight.im)}, float(primaryPdf), gx0,
                        gx1);
    }
};

template <typename R> static Antenna<R> to_antenna(const hsr_antenna_o &a) {
    Antenna<R> r;
    r.pos = {R(a.position[0]), R(a.position[1]), R(a.position[2])};
    for (int i = 0; i < 9; ++i) r.rot.m[i] = R(a.rotation[i]);
    return r;
}

static Flags to_flags(const hsr_tracer_flags_o &f) {
    Flags r;
    r.onlyIndirect = f.onlyIndirect != 0;
    r.maxDepth = f.maxDepth;
    r.useGO = f.useGeometricalOptics != 0;
    r.poDiffraction = f.poDiffraction != 0;
    r.doGuiding = f.doGuiding != 0;
    r.correctPhase = f.correctPhase != 0;
    r.filterGuiding = f.filterGuiding != 0;
    r.doFiltering = f.doFiltering != 0;
    r.filteringSphere = f.filteringSphere != 0;
    r.produceDebugImage = f.produceDebugImage != 0;
    r.filteringMin = f.filteringMin;
    r.filteringMax = f.filteringMax;
    r.filteringRadius = f.filteringRadius;
    return r;
}

template <typename R>
static void setup_tracer(Tracer<R> &tr, const Scene *s, const hsr_rf_config_o *rf, const hsr_antenna_o *tx,
                         const hsr_antenna_o *rx, const hsr_tracer_flags_o *fl) {
    tr.scene = s;
    tr.rf = Rf<R>{R(rf->startFreq), R(rf->freqSlope), R(rf->adcRate), R(rf->idleTime), R(rf->rampTime),
                  R(rf->antennaDelay)};
    tr.tx = to_antenna<R>(*tx);
    tr.rx = to_antenna<R>(*rx);
    tr.fl = to_flags(*fl);
}

// cpu::Backend::run (arch/cpu.h:21-41): batches of 256 from a mutex-protected counter
template <typename F> static void run_batches(int64_t budget, int threads, F &&work) {
    if (threads <= 0) threads = int(std::max(1u, std::thread::hardware_concurrency()));
    int64_t counter = 0;
    std::mutex mu;
    auto worker = [&]() {
        while (true) {
            int64_t batch, index;
            {
                std::unique_lock<std::mutex> lock(mu);
                batch = std::min<int64_t>(budget - counter, 256);
                if (batch <= 0) break;
                index = counter;
                counter += batch;
            }
            for (int64_t j = 0; j < batch; ++j) work(index + j);
        }
    };
    std::vector<std::thread> pool;
    for (int i = 1; i < threads; ++i) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
}

template <typename R>
static int simulate(const Scene *s, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc,
                    const hsr_antenna_o *tx, const hsr_antenna_o *rx, const hsr_tracer_flags_o *fl,
                    int64_t budget, int64_t offset, float sampleWeight, int threads, double *frame_out,
                    double *weight_out, bool floatSamples = false, bool exact = false,
                    const hsr_ff_antenna_o *ftx = nullptr, const hsr_ff_antenna_o *frx = nullptr) {
    Tracer<R> tr;
    setup_tracer(tr, s, rf, tx, rx, fl);
    if (ftx) {
        tr.farField = true;
        tr.ftx = to_ff<R>(*ftx);
        tr.frx = to_ff<R>(*frx);
    }
    tr.floatSamples = floatSamples;
    tr.frame.exact = exact;
    tr.currentSampleWeight = R(sampleWeight);
    tr.sampleIndexOffset = offset;
    tr.frame.chirps = fc->chirpCount;
    tr.frame.samples = fc->samplesPerChirp;
    tr.frame.channels = fc->channelCount;
    size_t n = size_t(fc->chirpCount) * fc->samplesPerChirp * fc->channelCount;
    std::vector<R> data(2 * n, R(0));
    tr.frame.data = data.data();
    run_batches(budget, threads, [&](int64_t i) { tr.sample(i); });
    for (size_t i = 0; i < 2 * n; ++i) frame_out[i] += double(data[i]);
    // PathTracer::incrementTotalWeight adds the float sample weight in double per sample
    double w = 0;
    for (int64_t i = 0; i < budget; ++i) w += double(float(sampleWeight));
    *weight_out += w;
    return 0;
}

}  // namespace oracle

using namespace oracle;

extern "C" {

int oracle_abi_version(void) { return 1; }

float oracle_radical_inverse_f(uint64_t index, int dim) { return radical_inverse<float>(index, unsigned(dim)); }
double oracle_radical_inverse_d(uint64_t index, int dim) { return radical_inverse<double>(index, unsigned(dim)); }

void *oracle_scene_create(const float *vertices, int64_t nv, const int32_t *indices, int64_t nt) {
    if ((nv > 0 && !vertices) || (nt > 0 && !indices) || nv < 0 || nt < 0) return nullptr;
    for (int64_t i = 0; i < 3 * nt; ++i)
        if (indices[i] < 0 || indices[i] >= nv) return nullptr;
    Scene *s = new Scene;
    s->mesh.v.assign(vertices, vertices + 3 * nv);
    s->mesh.f.assign(indices, indices + 3 * nt);
    s->mesh.nt = nt;
    build_bvh(*s);
    return s;
}

void oracle_scene_destroy(void *s) { delete static_cast<Scene *>(s); }

int oracle_intersect(void *sp, int64_t count, const float *o, const float *d, const float *tfar, float *t_out,
                     float *p_out, float *n_out, int32_t *prim_out) {
    const Scene &s = *static_cast<Scene *>(sp);
    for (int64_t i = 0; i < count; ++i) {
        Isect<float> is;
        is.ray.o = {o[3 * i], o[3 * i + 1], o[3 * i + 2]};
        is.ray.d = {d[3 * i], d[3 * i + 1], d[3 * i + 2]};
        is.tMax = tfar[i];
        float t;
        int32_t p = closest_hit(s, is.ray.o, is.ray.d, Consts<float>::Epsilon, is.tMax, t);
        prim_out[i] = p;
        if (p >= 0) {
            rt_intersect(s, is);
            t_out[i] = is.t;
            p_out[3 * i] = is.p.x;
            p_out[3 * i + 1] = is.p.y;
            p_out[3 * i + 2] = is.p.z;
            n_out[3 * i] = is.n.x;
            n_out[3 * i + 1] = is.n.y;
            n_out[3 * i + 2] = is.n.z;
        } else {
            t_out[i] = std::numeric_limits<float>::infinity();
            for (int k = 0; k < 3; ++k) p_out[3 * i + k] = n_out[3 * i + k] = 0.f;
        }
    }
    return 0;
}

int oracle_visible(void *sp, int64_t count, const float *o, const float *d, const float *tfar, int32_t *vis) {
    const Scene &s = *static_cast<Scene *>(sp);
    for (int64_t i = 0; i < count; ++i) {
        V3<float> oo{o[3 * i], o[3 * i + 1], o[3 * i + 2]}, dd{d[3 * i], d[3 * i + 1], d[3 * i + 2]};
        vis[i] = occluded(s, oo, dd, Consts<float>::Epsilon, tfar[i]) ? 0 : 1;
    }
    return 0;
}

int oracle_simulate(void *sp, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc, const hsr_antenna_o *tx,
                    const hsr_antenna_o *rx, const hsr_tracer_flags_o *fl, int64_t budget, int64_t offset,
                    float sample_weight, int precision, int threads, double *frame_out, double *weight_out) {
    if (!sp || !rf || !fc || !tx || !rx || !fl || !frame_out || !weight_out || budget < 0) return 1;
    if (fc->chirpCount <= 0 || fc->samplesPerChirp <= 0 || fc->channelCount <= 0) return 1;
    if (fl->doGuiding) return 2;  // guided runs are not restated here
    const Scene *s = static_cast<Scene *>(sp);
    const bool exact = (precision & 0x100) != 0;  // exact finite-N synthesis instead of splat<16>
    precision &= 0xff;
    if (precision == 64 || precision == 65)
        return simulate<double>(s, rf, fc, tx, rx, fl, budget, offset, sample_weight, threads, frame_out, weight_out,
                                precision == 65, exact);
    if (exact)
        return simulate<float>(s, rf, fc, tx, rx, fl, budget, offset, sample_weight, threads, frame_out, weight_out,
                               false, true);
    return simulate<float>(s, rf, fc, tx, rx, fl, budget, offset, sample_weight, threads, frame_out, weight_out);
}

int oracle_simulate_ff(void *sp, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc, const hsr_ff_antenna_o *tx,
                       const hsr_ff_antenna_o *rx, const hsr_tracer_flags_o *fl, int64_t budget, int64_t offset,
                       float sample_weight, int precision, int threads, double *frame_out, double *weight_out) {
    if (!sp || !rf || !fc || !tx || !rx || !fl || !frame_out || !weight_out || budget < 0) return 1;
    if (fc->chirpCount <= 0 || fc->samplesPerChirp <= 0 || fc->channelCount <= 0) return 1;
    if (fl->doGuiding) return 2;
    const Scene *s = static_cast<Scene *>(sp);
    hsr_antenna_o unused{};  // the near-field antennas are not read in far-field runs
    if (precision == 64 || precision == 65)
        return simulate<double>(s, rf, fc, &unused, &unused, fl, budget, offset, sample_weight, threads, frame_out,
                                weight_out, precision == 65, false, tx, rx);
    return simulate<float>(s, rf, fc, &unused, &unused, fl, budget, offset, sample_weight, threads, frame_out,
                           weight_out, false, false, tx, rx);
}

int oracle_records(void *sp, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc, const hsr_antenna_o *tx,
                   const hsr_antenna_o *rx, const hsr_tracer_flags_o *fl, int64_t first, int64_t count,
                   int64_t offset, int max_records, oracle_record *out) {
    if (!sp || !out || max_records <= 0) return 1;
    const Scene *s = static_cast<Scene *>(sp);
    Tracer<float> tr;
    setup_tracer(tr, s, rf, tx, rx, fl);
    tr.sampleIndexOffset = offset;
    tr.frame.chirps = fc->chirpCount;
    tr.frame.samples = fc->samplesPerChirp;
    tr.frame.channels = fc->channelCount;
    size_t n = size_t(fc->chirpCount) * fc->samplesPerChirp * fc->channelCount;
    std::vector<float> data(2 * n, 0.f);
    tr.frame.data = data.data();
    tr.maxRecords = max_records;
    for (int64_t i = 0; i < count; ++i) {
        oracle_record *rec = out + i * max_records;
        for (int k = 0; k < max_records; ++k) {
            rec[k] = oracle_record{};
            rec[k].depth = -1;
        }
        tr.records = rec;
        tr.sample(first + i);
    }
    return 0;
}

void oracle_frame_splat(int chirps, int samples, int channels, float ic, float is, float ich, float re, float im,
                        float *frame) {
    Frame<float> f;
    f.chirps = chirps;
    f.samples = samples;
    f.channels = channels;
    f.data = frame;
    frame_splat(f, ic, is, ich, Cx<float>{re, im});
}

void oracle_awr_evaluate(const float *d, float *H6) {
    CV3<float> H = awr_evaluate(V3<float>{d[0], d[1], d[2]});
    for (int i = 0; i < 3; ++i) {
        H6[2 * i] = H.c[i].re;
        H6[2 * i + 1] = H.c[i].im;
    }
}

void oracle_uniform_sample_sphere(float u0, float u1, float *d) {
    V3<float> v = uniform_sample_sphere(u0, u1);
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
}

void oracle_measure_ray(float dt, float startFreq, float freqSlope, float *out2) {
    Cx<float> c = measure_ray(dt, startFreq, freqSlope);
    out2[0] = c.re;
    out2[1] = c.im;
}

float oracle_set_time(float delta_t, float freqSlope, float adcRate, int samples) {
    return set_time_sample(delta_t, freqSlope, adcRate, samples);
}

void oracle_cexp(float angle, float *out2) {
    Cx<float> c = cexpj(angle);
    out2[0] = c.re;
    out2[1] = c.im;
}

void oracle_set_libm_trig(int on) { g_libm_trig = on ? 1 : 0; }

void oracle_sincos_rounded(float x, float *s, float *c) { sincos_once_rounded(x, *s, *c); }

int64_t oracle_bvh_nodes(void *sp) { return int64_t(static_cast<Scene *>(sp)->bvh.nodes.size()); }

// ---- path guiding (GuidingWrapper, path.h:17-131; PathTracer::run, path.h:171-224) ----

void *oracle_guide_create(void) { return new GuideTree(); }

void oracle_guide_destroy(void *g) { delete static_cast<GuideTree *>(g); }

// GuidingWrapper::reset (path.h:47-50)
void oracle_guide_reset(void *g) { *static_cast<GuideTree *>(g) = GuideTree(); }

void oracle_guide_step(void *g) { guide_step(*static_cast<GuideTree *>(g)); }

// the whole state: 2048 entries per array; returns the training tree's node count
int32_t oracle_guide_get(void *gp, int32_t *samp_child, float *samp_p, int32_t *train_child, float *acc2) {
    const GuideTree &g = *static_cast<GuideTree *>(gp);
    std::copy(g.samp_child.begin(), g.samp_child.end(), samp_child);
    std::copy(g.samp_p.begin(), g.samp_p.end(), samp_p);
    std::copy(g.train_child.begin(), g.train_child.end(), train_child);
    std::copy(g.acc2.begin(), g.acc2.end(), acc2);
    return g.count;
}

int oracle_guide_set(void *gp, int32_t count, const int32_t *samp_child, const float *samp_p,
                     const int32_t *train_child, const float *acc2) {
    if (count < 1 || count > kGuideNodes) return 1;
    GuideTree &g = *static_cast<GuideTree *>(gp);
    g.samp_child.assign(samp_child, samp_child + kGuideNodes);
    g.samp_p.assign(samp_p, samp_p + kGuideNodes);
    g.train_child.assign(train_child, train_child + kGuideNodes);
    g.acc2.assign(acc2, acc2 + kGuideNodes);
    g.count = count;
    return 0;
}

// GuidingWrapper::sample on (x0, x1): the warped point and the mixture pdf
float oracle_guide_sample(void *gp, float x0, float x1, float *y) {
    const float pdf = guide_mix_sample(*static_cast<GuideTree *>(gp), x0, x1);
    y[0] = x0;
    y[1] = x1;
    return pdf;
}

// One guided iteration (the backend run of one PathTracer::run iteration) on one thread,
// in FP32: Halton indices offset .. offset + budget - 1, sample weight, training into
// the tree when `train`. Adds the frame's sums to frame_out and the weight to weight_out.
int oracle_guided_pass(void *sp, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc, const hsr_antenna_o *tx,
                       const hsr_antenna_o *rx, const hsr_tracer_flags_o *fl, int64_t budget, int64_t offset,
                       float sample_weight, int train, void *gp, double *frame_out, double *weight_out) {
    if (!sp || !rf || !fc || !tx || !rx || !fl || !gp || !frame_out || !weight_out || budget < 0) return 1;
    if (fc->chirpCount <= 0 || fc->samplesPerChirp <= 0 || fc->channelCount <= 0) return 1;
    Tracer<float> tr;
    setup_tracer(tr, static_cast<Scene *>(sp), rf, tx, rx, fl);
    tr.guide = static_cast<GuideTree *>(gp);
    tr.guideTrain = train != 0;
    tr.currentSampleWeight = sample_weight;
    tr.sampleIndexOffset = offset;
    tr.frame.chirps = fc->chirpCount;
    tr.frame.samples = fc->samplesPerChirp;
    tr.frame.channels = fc->channelCount;
    const size_t n = size_t(fc->chirpCount) * fc->samplesPerChirp * fc->channelCount;
    std::vector<float> data(2 * n, 0.f);
    tr.frame.data = data.data();
    for (int64_t i = 0; i < budget; ++i) tr.sample(i);
    for (size_t i = 0; i < 2 * n; ++i) frame_out[i] += double(data[i]);
    double w = 0;
    for (int64_t i = 0; i < budget; ++i) w += double(sample_weight);
    *weight_out += w;
    return 0;
}

// PathTracer::run (path.h:171-224) with doGuiding: the doubling schedule from 16384
// samples, training on every iteration but the final one, the frame cleared between
// iterations (clearBeforeIteration) or later samples weighted 10x, a step between
// iterations. Overwrites frame_out / weight_out with the frame's sums and total weight;
// the tree ends in its state after the last step.
int oracle_path_tracer_run(void *sp, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc,
                           const hsr_antenna_o *tx, const hsr_antenna_o *rx, const hsr_tracer_flags_o *fl,
                           int64_t samples, void *gp, double *frame_out, double *weight_out) {
    if (!fl || !fc || !gp || !frame_out || !weight_out || samples < 0 || !fl->doGuiding) return 1;
    const size_t n = 2 * size_t(fc->chirpCount) * fc->samplesPerChirp * fc->channelCount;
    GuideTree &g = *static_cast<GuideTree *>(gp);
    g = GuideTree();
    std::fill(frame_out, frame_out + n, 0.0);
    *weight_out = 0;
    int64_t offset = 0, milestone = 16384, remaining = samples;
    float weight = 1.f;
    bool final_iteration = false;
    while (remaining > 0) {
        milestone = std::min(milestone, remaining);
        const int rc = oracle_guided_pass(sp, rf, fc, tx, rx, fl, milestone, offset, weight, !final_iteration, gp,
                                          frame_out, weight_out);
        if (rc) return rc;
        offset += milestone;
        remaining -= milestone;
        if (remaining == 0) break;
        milestone *= 2;
        if (remaining < milestone * 2) {
            final_iteration = true;
            milestone = remaining;
        }
        if (fl->clearBeforeIteration) {
            std::fill(frame_out, frame_out + n, 0.0);
            *weight_out = 0;
            offset = 0;
        } else {
            weight = 10 * weight;
        }
        guide_step(g);
    }
    return 0;
}

}  // extern "C"
