// Per-path device math shared by the trace kernels: Halton sampling, the antenna
// model, physical-optics re-radiation, next-event estimation, phase/bin evaluation and
// the frame splat. Each function restates one piece of libhussar's PathTracer
// (file:line given per function). Both kernels call the same functions, so they
// compute identical per-path values.
#pragma once
#include <math_constants.h>

#include "hsr_common.cuh"
#include "hsr_internal.h"
#include "hsr_guide.cuh"
#include "hsr_traverse.cuh"

namespace hsr {

// Tables of the chunked radical inverse (bases 3 and 5): rev[c] is c's kDigits base-kBase
// digits in reverse order (leading zeros included); inv_pow[n] is (1/kBase)^n formed by n
// sequential float multiplications, the value the reference's loop leaves in invBaseN
// after n digits. Built at compile time.
template <int kBase, int kDigits> struct RadicalTable {
    static constexpr int size() {
        int s = 1;
        for (int i = 0; i < kDigits; ++i) s *= kBase;
        return s;
    }
    unsigned short rev[size()];
    float inv_pow[48];
    constexpr RadicalTable() : rev(), inv_pow() {
        for (int c = 0; c < size(); ++c) {
            int w = c, r = 0;
            for (int i = 0; i < kDigits; ++i) {
                r = r * kBase + w % kBase;
                w /= kBase;
            }
            rev[c] = static_cast<unsigned short>(r);
        }
        const float inv = 1.f / float(kBase);
        float x = 1.f;
        for (int n = 0; n < 48; ++n) {
            inv_pow[n] = x;
            x *= inv;
        }
    }
};
__device__ constexpr RadicalTable<3, 6> kRadical3{};
__device__ constexpr RadicalTable<5, 4> kRadical5{};

template <int kBase> __device__ __forceinline__ const auto &radical_table() {
    if constexpr (kBase == 3)
        return kRadical3;
    else
        return kRadical5;
}

// radicalInverse<base> (libhussar/include/hussar/samplers/halton.h:38-54)
template <int kBase> __device__ __forceinline__ float radical_inverse(uint64_t v) {
    if (kBase == 2) {
        // base 2: the reversed digits are the bit reversal of v's d significant bits, and
        // the reference's float(reversed) * 2^-d equals float(brev64(v)) * 2^-64 exactly
        // (brev64(v) = reversed * 2^(64-d); rounding commutes with the power-of-two scale)
        return fminf(__ull2float_rn(__brevll(v)) * 0x1p-64f, 0.99999994f);
    }
    if constexpr (kBase == 3 || kBase == 5) {
        if (v < (1ull << 26)) {
            // the reference's digit loop, several digits per step: while a whole chunk of
            // kDigits digits remains, reversed = reversed * B^kDigits + rev[chunk] (the
            // integer the digit-by-digit loop forms), then the last digits one by one
            const auto &T = radical_table<kBase>();
            constexpr unsigned kChunk = sizeof(T.rev) / sizeof(T.rev[0]);
            constexpr int kDigits = kBase == 3 ? 6 : 4;
            unsigned w = unsigned(v), rev = 0;
            int n = 0;
            while (w >= kChunk) {
                const unsigned next = w / kChunk;
                rev = rev * kChunk + __ldg(&T.rev[w - next * kChunk]);
                n += kDigits;
                w = next;
            }
            while (w) {
                const unsigned next = w / kBase;
                rev = rev * kBase + (w - next * kBase);
                ++n;
                w = next;
            }
            return fminf(__uint2float_rn(rev) * __ldg(&T.inv_pow[n]), 0.99999994f);
        }
    }
    const float invBase = 1.f / float(kBase);
    float invBaseN = 1.f;
    uint64_t reversed;
    if (v < (1ull << 26)) {
        // below 2^26 the reversed digits of every base <= 29 stay below 29 * 2^26 < 2^32:
        // the same integer in 32-bit arithmetic (cheaper constant divisions)
        unsigned w = unsigned(v), rev = 0;
        while (w) {
            unsigned next = w / kBase;
            unsigned digit = w - next * kBase;
            rev = rev * kBase + digit;
            invBaseN *= invBase;
            w = next;
        }
        reversed = rev;
    } else {
        reversed = 0;
        while (v) {
            uint64_t next = v / kBase;
            uint64_t digit = v - next * kBase;
            reversed = reversed * kBase + digit;
            invBaseN *= invBase;
            v = next;
        }
    }
    const float ome = 0.99999994f;  // nextafter(1.f, 0.f)
    return fminf(__ull2float_rn(reversed) * invBaseN, ome);
}

// HaltonSampler::get2D (halton.h:23-26) is Vector2f(get1D(), get1D()): C++ leaves the order
// of the two calls unspecified and GCC evaluates the second argument first, so a GCC build
// of the reference draws (dimension d + 1, dimension d) for the pair that starts at d.
// The pairs here follow that build: primary = (halton(i, 2), halton(i, 1)).
constexpr int kGet2DFirst = 1;   // dimension offset of the pair's first component
constexpr int kGet2DSecond = 0;  // and of its second

// HaltonSampler::get1D dimension table (halton.h:56-67; dims >= 10 return 0, :1082-1084)
__device__ __forceinline__ float halton(uint64_t index, int dim) {
    switch (dim) {
        case 0: return radical_inverse<2>(index);
        case 1: return radical_inverse<3>(index);
        case 2: return radical_inverse<5>(index);
        case 3: return radical_inverse<7>(index);
        case 4: return radical_inverse<11>(index);
        case 5: return radical_inverse<13>(index);
        case 6: return radical_inverse<17>(index);
        case 7: return radical_inverse<19>(index);
        case 8: return radical_inverse<23>(index);
        case 9: return radical_inverse<29>(index);
        default: return 0.f;
    }
}

struct Ant {
    f3 pos;
    m33 rot;
};

__device__ __forceinline__ Ant load_ant(const hsr_antenna *a) {
    Ant r;
    r.pos = mk3(__ldg(&a->position[0]), __ldg(&a->position[1]), __ldg(&a->position[2]));
#pragma unroll
    for (int i = 0; i < 9; ++i) r.rot.m[i] = __ldg(&a->rotation[i]);
    return r;
}

// UniformSampleSphere (libhussar/include/hussar/core/sampling.h:38-43). kExact (the
// reference-phase parity instantiations): sin and cos of phi correctly rounded
// (sincos_cr: sincos_rounded's bits, mostly without its double-precision operations),
// bit for bit what the CPU restatement computes; the reference's
// std::sin/std::cos of a float resolve to the platform's sinf/cosf, which are not
// correctly rounded everywhere (glibc 2.39: one ulp off on 1.3 % of uniformly
// distributed angles), and CUDA's sincosf differs from both by up to two ulps. A one-ulp
// change of a primary direction moves the hit points of far sensors by micrometres,
// enough to change PO amplitudes measurably on large scenes. The split-phase form keeps
// the fast sincosf (it is bounded against the FP64 oracle, not matched bit for bit).
template <bool kExact = true> __device__ __forceinline__ f3 uniform_sample_sphere(float u0, float u1) {
    float phi = 2.f * kPi * u0;
    float y = 2.f * u1 - 1.f;
    float r = sqrtf(fmaxf(0.f, 1.f - y * y));
    float s, c;
    if (kExact)
        sincos_cr(phi, &s, &c);
    else
        sincosf(phi, &s, &c);
    return mk3(-r * s, y, -r * c);
}

// AWRAngularDistribution::evaluate (libhussar/include/hussar/core/emitter.h:126-136):
// H = (0,1,0) x d scaled by 2.622/(cos_h-1.8)^6 and 0.625/(cos_e-1.5)^4. The reference
// forms the two scale factors in double; here they are single precision (a few ulps).
__device__ __forceinline__ c3 awr_eval(f3 d) {
    // 1 - d.x^2 can round below zero for a direction within ~1e-4 rad of the antenna's x
    // (or y) axis (a receiver's rotation and the unit direction each carry rounding), where
    // the reference takes the square root of a negative number and its frame turns NaN;
    // the argument is clamped at zero (a deliberate deviation, only on those directions)
    float cos_h = sqrtf(fmaxf(1.f - d.x * d.x, 0.f));
    float cos_e = sqrtf(fmaxf(1.f - d.y * d.y, 0.f));
    float a = cos_h - 1.8f;
    float a2 = a * a;
    float s1 = 2.622f / (a2 * a2 * a2);
    float b = cos_e - 1.5f;
    float b2 = b * b;
    float s2 = 0.625f / (b2 * b2);
    c3 H;
    H.v[0] = cf{(d.z * s1) * s2, 0.f};
    H.v[1] = cf{0.f, 0.f};
    H.v[2] = cf{((-d.x) * s1) * s2, 0.f};
    return H;
}

// NFAntenna::sample (emitter.h:174-180): primary ray from the TX antenna
// Its field for the local direction ld (the rotated pattern over the sample density):
// the same operations, so that a caller may form it only once the primary ray hits.
__device__ __forceinline__ c3 antenna_field(const Ant &tx, f3 ld) {
    return mulcv(tx.rot, c3_div(awr_eval(ld), kInv4Pi));
}

template <bool kExact = true>
__device__ __forceinline__ void antenna_sample(const Ant &tx, float u0, float u1, f3 &d, c3 &H) {
    f3 ld = uniform_sample_sphere<kExact>(u0, u1);
    c3 lH = c3_div(awr_eval(ld), kInv4Pi);
    d = mulv(tx.rot, ld);
    H = mulcv(tx.rot, lH);
}

// SurfaceEmitter::evaluate (emitter.h:64-70): J = 2 n x H_in; H = d x J; zero behind the surface
__device__ __forceinline__ c3 surface_eval(f3 inc_n, const c3 &inc_H, f3 d) {
    c3 J = c3_scl(crs_rc(inc_n, inc_H), 2.f);
    c3 H = crs_rc(d, J);
    if (dot3(d, inc_n) < 0.f) {
#pragma unroll
        for (int i = 0; i < 3; ++i) H.v[i] = cf{0.f, 0.f};
    }
    return H;
}

// SurfaceEmitter::connect green's function (emitter.h:72-81)
__device__ __forceinline__ cf green(float k0, float r) {
    cf g = cf{1.f / fmaxf(r, 1e-3f), k0};
    return cdiv(g, 4.f * kPi * r);
}

// Integrator::reflectRay (integrator.h:164-168): d' = R(), H' = 2 n (n.H) - H
__device__ __forceinline__ void reflect(f3 n, f3 &d, c3 &H) {
    f3 wi = neg3(d);
    d = sub3(scl3(2.f * dot3(n, wi), n), wi);
    cf nh = dot_rc(n, H);
    f3 n2 = scl3(2.f, n);
    c3 t;
    t.v[0] = cscl(nh, n2.x);
    t.v[1] = cscl(nh, n2.y);
    t.v[2] = cscl(nh, n2.z);
    H = c3_sub(t, H);
}

// safe_modulo(int, unsigned) of radar.h:91-96, including its unsigned wrap of negative values
__device__ __forceinline__ int ref_mod(int a, int n) {
    if (a >= 0) return a < n ? a : a % n;
    return int(unsigned(a) % unsigned(n));
}

// One next-event estimate (path.h:292-397 with Integrator::splat's index/phase,
// integrator.h:113-135): the value the sample adds to the frame and where.
struct NeeOut {
    float time;    // nee.ray.time (before antennaDelay)
    cf v;          // measurement after scaling and filtering
    float dphase;
    float sample;  // fractional range bin
    cf value;      // weight * v * measureRay(dt)
    cf gw_add;     // what this estimate adds to guidingWeight (path.h:363-394)
    bool splat;    // passed the splat early-out
};

// FFAntenna (libhussar/include/hussar/core/emitter.h:226-291) of one pose, with what its
// constructor and sample() derive: the disk centre (sceneCenter + dir * radius), the
// disk frame buildFrame(-dir) (core/geometry.h:45-53) and the pdf 1 / (4 radius^2),
// formed in double and rounded once, as the reference's
// `Float pdf = 1 / (4 * std::pow(m_radius, 2))` is.
struct FfAnt {
    f3 dir, center, e0, e1;
    c3 pol;
    float radius, pdf;
};

__device__ __forceinline__ FfAnt load_ff(const hsr_ff_antenna *a) {
    FfAnt r;
    r.dir = mk3(__ldg(&a->direction[0]), __ldg(&a->direction[1]), __ldg(&a->direction[2]));
#pragma unroll
    for (int i = 0; i < 3; ++i) r.pol.v[i] = cf{__ldg(&a->polarization[2 * i]), __ldg(&a->polarization[2 * i + 1])};
    r.radius = __ldg(&a->radius);
    const f3 c = mk3(__ldg(&a->scene_center[0]), __ldg(&a->scene_center[1]), __ldg(&a->scene_center[2]));
    r.center = add3(c, scl3(r.radius, r.dir));
    const f3 d = neg3(r.dir);
    if (fabsf(d.x) > fabsf(d.y))
        r.e0 = div3(mk3(-d.z, 0.f, d.x), sqrtf(d.x * d.x + d.z * d.z));
    else
        r.e0 = div3(mk3(0.f, d.z, -d.y), sqrtf(d.y * d.y + d.z * d.z));
    r.e1 = crs3(d, r.e0);
    r.pdf = __double2float_rn(1.0 / (4.0 * (double(r.radius) * double(r.radius))));
    return r;
}

// FFAntenna::sample (emitter.h:241-248): a point of the disk's square (2u - 1, 2v - 1)
// in the disk frame, scaled by the radius; the ray travels along -dir; H = pol / pdf.
__device__ __forceinline__ void ff_sample(const FfAnt &a, float u0, float u1, f3 &o, f3 &d, c3 &H) {
    const float s0 = 2.f * u0 - 1.f, s1 = 2.f * u1 - 1.f;
    const f3 q = mk3(a.e0.x * s0 + a.e1.x * s1, a.e0.y * s0 + a.e1.y * s1, a.e0.z * s0 + a.e1.z * s1);
    o = add3(scl3(a.radius, q), a.center);
    d = neg3(a.dir);
    H = c3_div(a.pol, a.pdf);
}

// Returns false when the estimate is occluded or skipped (no record, no splat).
// depth == 0: direct TX->RX connection (only with onlyIndirect = false).
// `nodes`/`tris` are the scene the pose traces, `rf`/`samples` its chirp and range bins
// (uniform over a launch, or the pose's PoseJob in a mixed batch). kFF: far-field TX and
// RX (`ff_rx` the receiver): FFAntenna::nee replaces NFAntenna::nee, and the direct term
// is zero (FFAntenna::evaluate zeroes the ray, emitter.h:253-255).
template <int kPhase, bool kCount, bool kFF = false>
__device__ __forceinline__ bool nee_eval(const TraceParams &p, const DNode *nodes, const DTri *tris,
                                         const hsr_rf_config &rf, int samples, const Ant &tx, const Ant &rx, int depth,
                                         f3 o, f3 d, f3 tmpd, f3 hit_n, const c3 &inc_H, const c3 &H, float time,
                                         double plen, float r, float cosTheta, float freq, float sampleWeight,
                                         NeeOut &out, TraversalCounters *cnt, unsigned *rays,
                                         const FfAnt *ff_rx = nullptr) {
    const hsr_tracer_flags &fl = p.flags;
    f3 nd;
    float rr;
    c3 Hrx;
    if (kFF) {
        if (depth == 0) return false;
        // FFAntenna::nee (emitter.h:261-273): along +dir to the disk's plane, while the
        // point projects within 1 of the disk centre (else H = 0: nothing to splat)
        f3 local = sub3(o, ff_rx->center);
        local = sub3(local, scl3(dot3(local, ff_rx->dir), ff_rx->dir));
        if (nrm3(local) > 1.f) return false;
        nd = ff_rx->dir;
        rr = nrm3(sub3(add3(local, ff_rx->center), o));
        Hrx = c3_scl(ff_rx->pol, 4.f * kPi * rr);
    } else {
        // NFAntenna::nee (emitter.h:195-203)
        nd = sub3(rx.pos, o);
        rr = nrm3(nd);
        nd = div3(nd, rr);
        Hrx = mulcv(rx.rot, awr_eval(mulTv(rx.rot, neg3(nd))));
    }
    const float tMax = rr;
    if (!fl.poDiffraction) {
        if (kCount) (*rays)++;
        if (any_hit<kCount>(nodes, tris, o, nd, kEpsilon, tMax, p.status, cnt)) return false;
    }
    const float nt = tMax;
    f3 no = o;
    float ntime = time;
    double nlen = plen;
    c3 nH;
    if (depth == 0) {
        // NFAntenna::evaluate + connect (emitter.h:182-193)
        no = tx.pos;
        nH = mulcv(tx.rot, awr_eval(mulTv(tx.rot, nd)));
        ntime += nt / kSpeedOfLight;
        nlen += double(nt);
        nH = c3_scl(nH, 1.f / (4.f * kPi * nt));
    } else {
        nH = surface_eval(hit_n, inc_H, nd);
        ntime += nt / kSpeedOfLight;
        nlen += double(nt);
        nH = c3_cmul(nH, green(2.f * kPi * freq / kSpeedOfLight, nt));
    }
    cf v = dot_cc(nH, Hrx);
    const float wavelength = kSpeedOfLight / freq;
    float dphase = 0.f;
    cf gw = cf{0.f, 0.f};
    if (depth > 0) {
        if (fl.correctPhase) {
            f3 rxPos = add3(no, scl3(nt, nd));
            f3 virtualTx = sub3(no, scl3(r, d));
            float dist = nrm3(sub3(virtualTx, rxPos));
            ntime = dist / kSpeedOfLight;
            nlen = double(dist);
            float pw = kPi * fl.filteringRadius * wavelength;
            v = cdiv(cscl(dot_cc(H, Hrx), kPi * dist), pw * pw);
            v = cdiv(v, 4.f * kPi);
        } else if (fl.useGeometricalOptics) {
            v = cscl(v, r / cosTheta);
            v = cdiv(v, 4.f * kPi);
            if (cosTheta < 0.001f) return false;  // (double)cosTheta < 1e-3
        }
        if (fl.filteringSphere) {
            f3 rxPos = add3(no, scl3(nt, nd));
            float lam = fmaxf(0.f, dot3(d, sub3(rxPos, o)));
            dphase = nrm3(sub3(add3(o, scl3(lam, d)), rxPos));
        } else {
            float c = dot3(nrmz3(sub3(nd, tmpd)), hit_n);
            dphase = r * sqrtf(1.f - c * c) / c;
        }
        dphase /= wavelength;
        if (fl.doFiltering) {
            if (fl.filteringSphere) {
                if (dphase > fl.filteringRadius) {
                    if (fl.correctPhase) {
                        if (fl.filterGuiding) {
                            const float q = dphase / fl.filteringRadius;
                            gw = cadd(gw, cdiv(v, float(double(q) * double(q) + 1.0)));
                        }
                        v = cf{0.f, 0.f};
                    } else {
                        float q = dphase / fl.filteringRadius - 1.f;
                        float taper = fmaxf(float(1.0 - 0.20 * double(q)), 0.f);
                        v = cscl(v, taper);
                    }
                }
            } else {
                if (dphase > fl.filteringMax) {
                    if (fl.filterGuiding) {
                        const float q = dphase / fl.filteringMax;
                        gw = cadd(gw, cdiv(v, float(double(q) * double(q) + 1.0)));
                    }
                    v = cf{0.f, 0.f};
                }
                if (dphase > fl.filteringMin)
                    v = cscl(v, (fl.filteringMax - dphase) / (fl.filteringMax - fl.filteringMin));
            }
        }
    }
    if (depth > 0) gw = cadd(gw, v);
    out.time = ntime;
    out.v = v;
    out.dphase = dphase;
    out.gw_add = gw;
    out.splat = false;
    out.sample = 0.f;
    out.value = cf{0.f, 0.f};
    // Integrator::splat (integrator.h:113-135)
    if (!fl.produceDebugImage) {
        if (sampleWeight == 0.f || v.re == 0.f || v.im == 0.f) return true;
    }
    float sample;
    cf ph;
    if (kPhase == HSR_PHASE_REFERENCE_FP32) {
        float dt = ntime + rf.antennaDelay;
        if (rf.freqSlope == 0.f) {
            sample = 0.f;
        } else {
            float x = dt * rf.freqSlope / rf.adcRate;  // PIndex::setTime (radar.h:232-241)
            sample = float(samples) * (x - floorf(x));
        }
        // Integrator::measureRay (integrator.h:107-110)
        float angle = 2.f * kPi * (rf.startFreq - dt * rf.freqSlope / 2.f) * dt;
        float s, c;
        sincosf(angle, &s, &c);
        ph = cf{c, s};
    } else {
        // path length reduced to phase in FP64: cycles = f0 dt - S dt^2 / 2 (mod 1)
        // FP64 divides are long sequences on this part: multiply by reciprocals (<= 1 ulp)
        double dt = nlen * (1.0 / 299792458.0) + double(rf.antennaDelay);
        if (rf.freqSlope == 0.f) {
            sample = 0.f;
        } else {
            double x = dt * (double(rf.freqSlope) / double(rf.adcRate));
            sample = float(double(samples) * (x - floor(x)));
        }
        double cyc = (double(rf.startFreq) - dt * double(rf.freqSlope) * 0.5) * dt;
        float frac = float(cyc - floor(cyc));
        float s, c;
        sincospif(2.f * frac, &s, &c);
        ph = cf{c, s};
    }
    out.sample = sample;
    out.value = cscl(cmul(v, ph), sampleWeight);
    out.splat = true;
    return true;
}

// Frame::splat<16> (libradar/include/radar/radar.h:564-626) restricted to the row the
// reference writes (chirp and channel indices are exactly 0: delta components).
// Prepared form: center bin, fractional shift, phase-rotated value and sinc weight.
struct SplatItem {
    int center;
    float shift;  // 0 => delta peak
    cf value;
    float w;
};

__device__ __forceinline__ SplatItem splat_prepare(float sample, cf value) {
    SplatItem it;
    it.center = int(roundf(sample));
    float shift = sample - float(it.center);
    if (fabsf(shift) < 1e-4f) {
        it.shift = 0.f;
        it.value = value;
        it.w = 1.f;
        return it;
    }
    float shiftPi = float(CUDART_PI * double(shift));
    float sn, cs;
    sincosf(shiftPi, &sn, &cs);
    it.shift = shift;
    it.value = cmul(value, cf{cs, sn});
    it.w = sinf(shiftPi) / kPi;
    return it;
}

// One thread adds a whole item (33 bins, or 1 for a delta peak).
__device__ __forceinline__ void splat_serial(float *s_re, float *s_im, int n, const SplatItem &it) {
    if (it.shift == 0.f) {
        // the reference indexes `center` unwrapped here; center == N (sample >= N-0.5)
        // would be out of bounds. Wrapped instead (the spectrum is periodic).
        int bin = ref_mod(it.center, n);
        atomicAdd(&s_re[bin], it.value.re);
        atomicAdd(&s_im[bin], it.value.im);
        return;
    }
    const bool inside = (it.center - 16 >= 0) && (it.center + 16 < n);
#pragma unroll 11
    for (int s = -16; s <= 16; ++s) {
        int bin = inside ? it.center + s : ref_mod(it.center + s, n);
        float ws = it.w / (it.shift - float(s));
        atomicAdd(&s_re[bin], ws * it.value.re);
        atomicAdd(&s_im[bin], ws * it.value.im);
    }
}

// 1 / x by the hardware approximation (rcp.approx.ftz.f32, within 1 ulp for normal x).
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// An item of a warp's cooperative splat: the fractional shift (0 => delta peak), the
// value times the sinc weight (weight 1 for a delta peak), and the center bin. The
// owning lane forms it once; every lane then needs only its own bin's 1 / (shift - s).
__device__ __forceinline__ float4 splat_item(float sample, cf value) {
    const SplatItem it = splat_prepare(sample, value);
    return make_float4(it.shift, it.w * it.value.re, it.w * it.value.im, __int_as_float(it.center));
}

// A full warp adds the items of the lanes with `has` set cooperatively: lane l owns
// window offset l - 16 (lane 0 also owns +16), so one item's 33 bins are distinct
// addresses updated by distinct lanes. Items are broadcast by shuffles in lane order;
// each lane sums its bin over a run of items with the same center in registers and adds
// the sum once when the center changes (coherent returns put most of a warp's items on
// one center, and the shared-memory atomics on those few bins are what limits the
// splat). The per-bin factor 1 / (shift - s) is the hardware reciprocal (within 1 ulp;
// the reference divides, radar.h:612-618; |shift - s| >= 1e-4, so it is never
// subnormal). Must be called by all 32 lanes.
__device__ __forceinline__ void splat_warp(float *s_re, float *s_im, int n, bool has, float4 mine) {
    unsigned mask = __ballot_sync(0xffffffffu, has);
    if (mask == 0u) return;
    const int lane = threadIdx.x & 31;
    const int s = lane - 16;
    const float fs = float(s);
    int center = INT_MIN;  // no run open
    float ar = 0.f, ai = 0.f, er = 0.f, ei = 0.f;  // this lane's bin, and lane 0's bin +16
    auto flush = [&]() {
        const bool inside = (center - 16 >= 0) && (center + 16 < n);
        if (ar != 0.f || ai != 0.f) {
            const int bin = inside ? center + s : ref_mod(center + s, n);
            atomicAdd(&s_re[bin], ar);
            atomicAdd(&s_im[bin], ai);
        }
        if (lane == 0 && (er != 0.f || ei != 0.f)) {
            const int bin = inside ? center + 16 : ref_mod(center + 16, n);
            atomicAdd(&s_re[bin], er);
            atomicAdd(&s_im[bin], ei);
        }
        ar = ai = er = ei = 0.f;
    };
    while (mask) {
        const int j = __ffs(mask) - 1;
        mask &= mask - 1;
        const float shift = __shfl_sync(0xffffffffu, mine.x, j);
        const float wr = __shfl_sync(0xffffffffu, mine.y, j);
        const float wi = __shfl_sync(0xffffffffu, mine.z, j);
        const int c = __shfl_sync(0xffffffffu, __float_as_int(mine.w), j);
        if (c != center) {
            if (center != INT_MIN) flush();
            center = c;
        }
        if (shift == 0.f) {
            if (s == 0) {
                ar += wr;
                ai += wi;
            }
            continue;
        }
        const float rcp = rcp_approx(shift - fs);
        ar = __fmaf_rn(wr, rcp, ar);
        ai = __fmaf_rn(wi, rcp, ai);
        if (lane == 0) {
            const float r16 = rcp_approx(shift - 16.f);
            er = __fmaf_rn(wr, r16, er);
            ei = __fmaf_rn(wi, r16, ei);
        }
    }
    flush();
}

// Fine range histogram (HSR_SPLAT_FINE_SYNTH): 8 sub-bins per range bin with moments
// h_d += c eps^d / d! (d = 0..3) of the sub-bin offset eps (in bins); the spectrum is
// synthesised from it afterwards (hsr_synth.cu). `row` is the pose's
// [Re h0..h3 | Im h0..h3] row, K = 8 N. The terms are FP32; the sums are FP64, since a
// coherent return adds millions of nearly equal terms to one sub-bin.
__device__ __forceinline__ void splat_fine(double *row, int K, float sample, cf value) {
    const float bs = sample * float(kFineOS);
    const float kk = rintf(bs);
    const float eps = (bs - kk) * (1.f / float(kFineOS));
    int k = int(kk);
    if (k >= K) k -= K;
    if (k < 0) k += K;
    if (k < 0 || k >= K) k = 0;  // NaN/inf samples land in bin 0 rather than out of bounds
    float m = 1.f;
#pragma unroll
    for (int d = 0; d < kFineMoments; ++d) {
        atomicAdd(row + d * K + k, double(value.re * m));
        atomicAdd(row + (kFineMoments + d) * K + k, double(value.im * m));
        m = m * eps / float(d + 1);
    }
}

__device__ __forceinline__ int find_pose(const int64_t *__restrict__ tile_start, int pose_count, int64_t item) {
    int lo = 0, hi = pose_count;  // tile_start[lo] <= item < tile_start[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (__ldg(&tile_start[mid]) <= item)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// A CTA's shared-memory row holds FP32 partial sums of at most this many samples of one
// pose before it is flushed to the FP64 accumulators.
constexpr long long kFlushSamples = 65536;

// Flushes a CTA's shared-memory row into the pose's FP64 accumulators and clears it.
__device__ __forceinline__ void flush_row(double *acc, float *s_re, float *s_im, int n) {
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        float re = s_re[k], im = s_im[k];
        if (re != 0.f) atomicAdd(&acc[2 * k], double(re));
        if (im != 0.f) atomicAdd(&acc[2 * k + 1], double(im));
        s_re[k] = 0.f;
        s_im[k] = 0.f;
    }
}

}  // namespace hsr

namespace hsr {

// Per-pose state a CTA loads when it starts on a pose.
struct PoseCtx {
    Ant tx, rx;
    int64_t offset;
    double *fine_row;  // fine-histogram row of the pose (nullptr: Dirichlet splat)
    float weight;
    int train;
    const int *samp_child;
    const float *samp_p;
    const int *train_child;
    float *train_acc;
};

__device__ __forceinline__ PoseCtx load_pose(const TraceParams &p, int pose) {
    PoseCtx c;
    c.tx = load_ant(p.tx + pose);
    c.rx = load_ant(p.rx + pose);
    c.offset = __ldg(&p.offset[pose]);
    c.fine_row = p.fine ? p.fine + size_t(pose) * 2 * kFineMoments * p.fine_bins : nullptr;
    c.weight = p.weights ? __ldg(&p.weights[pose]) : p.sample_weight;
    c.train = (p.do_guide && p.train) ? __ldg(&p.train[pose]) : 0;
    const size_t g = size_t(p.guide_slot ? __ldg(&p.guide_slot[pose]) : pose) * kGuideMaxNodes;
    c.samp_child = p.do_guide ? p.g_samp_child + g : nullptr;
    c.samp_p = p.do_guide ? p.g_samp_p + g : nullptr;
    c.train_child = p.do_guide ? p.g_train_child + g : nullptr;
    c.train_acc = p.do_guide ? p.g_train_acc + 3 * g : nullptr;
    return c;
}

// guiding.splat(|guidingWeight| * primaryPdf, {}, 1 / primaryPdf, primary) (path.h:448-450).
// Only the second moment drives the tree, so zero-density samples add nothing. The sum
// goes to `acc2[stride * leaf]`: the pose's training accumulators in global memory
// (stride 3, slot 2), or a CTA's shared-memory copy (stride 1) flushed by flush_guide;
// `train_child` is the training topology (global, or the CTA's staged copy).
__device__ __forceinline__ void guide_train(const PoseCtx &c, const int *train_child, float *acc2, int stride, cf gw,
                                            float pdf, float x0, float x1) {
    if (!c.train || !(pdf > 0.f)) return;
    // std::abs(radar::complex) (complex.h:225-237)
    float ax = fabsf(gw.re), ay = fabsf(gw.im);
    float s = ax < ay ? ay : ax;
    float mag = 0.f;
    if (s != 0.f) {
        ax /= s;
        ay /= s;
        mag = s * sqrtf(ax * ax + ay * ay);
    }
    const float density = mag * pdf;
    if (density == 0.f) return;
    const float weight = 1.f / pdf;
    const int leaf = guide_leaf(train_child, x0, x1);
    atomicAdd(&acc2[stride * leaf], weight * density * density);
}

// Adds a CTA's shared-memory training sums to the pose's accumulators and clears them.
__device__ __forceinline__ void flush_guide(const PoseCtx &c, float *s_g) {
    for (int i = threadIdx.x; i < kGuideMaxNodes; i += blockDim.x) {
        const float v = s_g[i];
        if (v != 0.f) {
            if (c.train) atomicAdd(&c.train_acc[3 * i + 2], v);
            s_g[i] = 0.f;
        }
    }
}

}  // namespace hsr
