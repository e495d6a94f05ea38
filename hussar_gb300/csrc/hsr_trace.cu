// The radar path tracer on GB300: one thread traces one Monte Carlo sample
// (libhussar/include/hussar/integrators/path.h:235-451), CTAs pull (pose, sample-tile)
// work items from a device counter (persistent grid), and each CTA accumulates its
// pose's range row in shared memory, flushing it to FP64 accumulators when it moves
// to another pose.
//
// Compiled with -fmad=false: every expression that the CPU restatement evaluates in
// float rounds identically here (only the slab test uses explicit FMAs), so paths hit
// the same triangles and land in the same bins. The transcendental functions are
// CUDA's full-accuracy single-precision ones; the reference evaluates the AWR
// polynomial scale factors and cos/sin of the phase in double, which differs from
// these by a few float ulps (far below the 1e-4 relative-L2 parity bar).
#include <math_constants.h>

#include "hsr_common.cuh"
#include "hsr_internal.h"
#include "hsr_traverse.cuh"

namespace hsr {

namespace {

// radicalInverse<base> (libhussar/include/hussar/samplers/halton.h:38-54)
template <int kBase> __device__ __forceinline__ float radical_inverse(uint64_t v) {
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
        default: return 0.f;  // halton.h:1082-1084
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

// UniformSampleSphere (libhussar/include/hussar/core/sampling.h:38-43)
__device__ __forceinline__ f3 uniform_sample_sphere(float u0, float u1) {
    float phi = 2.f * kPi * u0;
    float y = 2.f * u1 - 1.f;
    float r = sqrtf(fmaxf(0.f, 1.f - y * y));
    float s, c;
    sincosf(phi, &s, &c);
    return mk3(-r * s, y, -r * c);
}

// AWRAngularDistribution::evaluate (libhussar/include/hussar/core/emitter.h:126-136):
// H = (0,1,0) x d scaled by 2.622/(cos_h-1.8)^6 and 0.625/(cos_e-1.5)^4
__device__ __forceinline__ c3 awr_eval(f3 d) {
    float cos_h = sqrtf(1.f - d.x * d.x);
    float cos_e = sqrtf(1.f - d.y * d.y);
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

// safe_modulo(int, unsigned) of radar.h:91-96, including its unsigned wrap of negative values
__device__ __forceinline__ int ref_mod(int a, int n) {
    if (a >= 0) return a < n ? a : a % n;
    return int(unsigned(a) % unsigned(n));
}

struct SplatCtx {
    float *s_re;
    float *s_im;
    int n;
};

// Frame::splat<16> (libradar/include/radar/radar.h:564-626) restricted to the row the
// reference writes (chirp and channel indices are exactly 0: delta components).
__device__ __forceinline__ void splat_dirichlet(const SplatCtx &sc, float sample, cf value, unsigned *status) {
    int center = int(roundf(sample));
    float shift = sample - float(center);
    if (fabsf(shift) < 1e-4f) {
        // the reference indexes `center` unwrapped here; center == N (sample >= N-0.5)
        // would be out of bounds. Wrapped instead (the spectrum is periodic).
        int bin = ref_mod(center, sc.n);
        atomicAdd(&sc.s_re[bin], value.re);
        atomicAdd(&sc.s_im[bin], value.im);
        return;
    }
    float shiftPi = float(CUDART_PI * double(shift));
    float sn, cs;
    sincosf(shiftPi, &sn, &cs);
    value = cmul(value, cf{cs, sn});
    float w = sinf(shiftPi) / kPi;
    const bool inside = (center - 16 >= 0) && (center + 16 < sc.n);
#pragma unroll 11
    for (int s = -16; s <= 16; ++s) {
        int bin = inside ? center + s : ref_mod(center + s, sc.n);
        float ws = w / (shift - float(s));
        atomicAdd(&sc.s_re[bin], ws * value.re);
        atomicAdd(&sc.s_im[bin], ws * value.im);
    }
}

struct PathRecord {  // one next-event estimate (tests only)
    int32_t depth;
    int32_t splatted;
    float time;
    float v_re, v_im;
    float dphase;
    float bin;
    float value_re, value_im;
};

template <int kPhase, bool kRecord, bool kCount>
__device__ void trace_sample(const TraceParams &p, const Ant &tx, const Ant &rx, uint64_t hindex, const SplatCtx &sc,
                             PathRecord *rec, int max_rec, TraversalCounters *cnt, unsigned *rays) {
    const hsr_rf_config &rf = p.rf;
    const hsr_tracer_flags &fl = p.flags;
    const float inf = CUDART_INF_F;
    int dim = 0;
    const float maxDist = rf.adcRate / rf.freqSlope * kSpeedOfLight;
    const float sampleWeight = p.sample_weight;
    const float primaryPdf = 1.f;
    const float bandwidth = rf.freqSlope * rf.rampTime;
    const float freq = rf.startFreq + halton(hindex, dim++) * bandwidth;
    const float k0 = 2.f * kPi * freq / kSpeedOfLight;
    const float wavelength = kSpeedOfLight / freq;

    f3 o = mk3(0.f, 0.f, 0.f), d = mk3(0.f, 0.f, 0.f);
    float time = 0.f;
    double plen = 0.0;  // path length in FP64 (split-phase mode)
    int depth = 0;
    c3 H;
    f3 hit_n = mk3(0.f, 0.f, 0.f);
    f3 inc_n = mk3(0.f, 0.f, 0.f);
    c3 inc_H;
    float r = 0.f, cosTheta = 1.f;
    int nrec = 0;

    while (true) {
        const f3 tmpd = d;
        if (depth == 0) {
            float u0 = halton(hindex, dim++);
            float u1 = halton(hindex, dim++);
            // NFAntenna::sample (emitter.h:174-180)
            o = tx.pos;
            f3 ld = uniform_sample_sphere(u0, u1);
            c3 lH = c3_div(awr_eval(ld), kInv4Pi);
            d = mulv(tx.rot, ld);
            H = mulcv(tx.rot, lH);
            H = c3_scl(H, 1.f / primaryPdf);
        } else if (!fl.useGeometricalOptics) {
            float u0 = halton(hindex, dim++);
            float u1 = halton(hindex, dim++);
            d = uniform_sample_sphere(u0, u1);
            H = surface_eval(inc_n, inc_H, d);
        } else {
            // Integrator::reflectRay (integrator.h:164-168)
            f3 wi = neg3(d);
            d = sub3(scl3(2.f * dot3(hit_n, wi), hit_n), wi);
            cf nh = dot_rc(hit_n, H);
            f3 n2 = scl3(2.f, hit_n);
            c3 t;
            t.v[0] = cscl(nh, n2.x);
            t.v[1] = cscl(nh, n2.y);
            t.v[2] = cscl(nh, n2.z);
            H = c3_sub(t, H);
        }

        // next event estimation towards the single RX antenna (path.h:292-397)
        if (!(depth == 0 && fl.onlyIndirect)) {
            do {
                // NFAntenna::nee (emitter.h:195-203)
                f3 nd = sub3(rx.pos, o);
                float rr = nrm3(nd);
                nd = div3(nd, rr);
                const float tMax = rr;
                c3 Hrx = mulcv(rx.rot, awr_eval(mulTv(rx.rot, neg3(nd))));
                if (!fl.poDiffraction) {
                    if (kCount) (*rays)++;
                    if (any_hit<kCount>(p.nodes, p.tris, o, nd, kEpsilon, tMax, p.status, cnt)) break;
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
                    nH = surface_eval(inc_n, inc_H, nd);
                    ntime += nt / kSpeedOfLight;
                    nlen += double(nt);
                    nH = c3_cmul(nH, green(k0, nt));
                }
                cf v = dot_cc(nH, Hrx);
                float dphase = 0.f;
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
                        if (cosTheta < 0.001f) break;  // (double)cosTheta < 1e-3
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
                                    v = cf{0.f, 0.f};
                                } else {
                                    float q = dphase / fl.filteringRadius - 1.f;
                                    float taper = fmaxf(float(1.0 - 0.20 * double(q)), 0.f);
                                    v = cscl(v, taper);
                                }
                            }
                        } else {
                            if (dphase > fl.filteringMax) v = cf{0.f, 0.f};
                            if (dphase > fl.filteringMin)
                                v = cscl(v, (fl.filteringMax - dphase) / (fl.filteringMax - fl.filteringMin));
                        }
                    }
                }
                PathRecord *rc = nullptr;
                if (kRecord && nrec < max_rec) {
                    rc = rec + nrec++;
                    rc->depth = depth;
                    rc->time = ntime;
                    rc->v_re = v.re;
                    rc->v_im = v.im;
                    rc->dphase = dphase;
                    rc->splatted = 0;
                }
                // Integrator::splat (integrator.h:113-135)
                if (!fl.produceDebugImage) {
                    if (sampleWeight == 0.f || v.re == 0.f || v.im == 0.f) break;
                }
                float sample;
                cf ph;
                if (kPhase == HSR_PHASE_REFERENCE_FP32) {
                    float dt = ntime + rf.antennaDelay;
                    if (rf.freqSlope == 0.f) {
                        sample = 0.f;
                    } else {
                        float x = dt * rf.freqSlope / rf.adcRate;
                        sample = float(p.samples) * (x - floorf(x));
                    }
                    // Integrator::measureRay (integrator.h:107-110)
                    float angle = 2.f * kPi * (rf.startFreq - dt * rf.freqSlope / 2.f) * dt;
                    float s, c;
                    sincosf(angle, &s, &c);
                    ph = cf{c, s};
                } else {
                    // FP64 reduction of the path length: cycles = f0 dt - S dt^2 / 2 (mod 1)
                    double dt = nlen / 299792458.0 + double(rf.antennaDelay);
                    if (rf.freqSlope == 0.f) {
                        sample = 0.f;
                    } else {
                        double x = dt * double(rf.freqSlope) / double(rf.adcRate);
                        sample = float(double(p.samples) * (x - floor(x)));
                    }
                    double cyc = (double(rf.startFreq) - dt * double(rf.freqSlope) * 0.5) * dt;
                    float frac = float(cyc - floor(cyc));
                    float s, c;
                    sincospif(2.f * frac, &s, &c);
                    ph = cf{c, s};
                }
                cf value = cscl(cmul(v, ph), sampleWeight);
                if (kRecord && rc) {
                    rc->bin = sample;
                    rc->value_re = value.re;
                    rc->value_im = value.im;
                    rc->splatted = 1;
                }
                splat_dirichlet(sc, sample, value, p.status);
            } while (false);
        }

        // random walk (path.h:399-442)
        if (depth >= fl.maxDepth || r >= maxDist) break;
        if (c3_is_zero(H)) break;
        float th;
        int primh;
        if (kCount) (*rays)++;
        int slot = closest_hit<kCount>(p.nodes, p.tris, o, d, kEpsilon, inf, th, primh, p.status, cnt);
        if (slot < 0) break;
        DTri T = load_tri(p.tris, slot);
        hit_n = hit_normal(T, d);
        f3 hp = add3(o, scl3(th, d));
        cosTheta = fabsf(dot3(hit_n, neg3(d)));
        if (cosTheta < 0.001f) break;
        r += th;
        if (!fl.useGeometricalOptics) {
            time += th / kSpeedOfLight;
            plen += double(th);
            if (depth == 0) {
                H = c3_scl(H, 1.f / (4.f * kPi * th));
            } else {
                H = c3_cmul(H, green(k0, th));
            }
            H = c3_scl(H, th * th / cosTheta);
        } else {
            time += th / kSpeedOfLight;
            plen += double(th);
        }
        if (c3_is_zero(H)) break;
        inc_n = hit_n;
        inc_H = H;
        o = hp;
        depth++;
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

template <int kPhase, bool kRecord, bool kCount>
__global__ void __launch_bounds__(256, 2) k_trace(TraceParams p) {
    TraversalCounters cnt{0u, 0u};
    unsigned rays = 0;
    PathRecord *records = static_cast<PathRecord *>(p.records);
    const int max_rec = p.max_rec;
    extern __shared__ float smem[];
    __shared__ long long s_item;
    SplatCtx sc{smem, smem + p.samples, p.samples};
    for (int k = threadIdx.x; k < 2 * p.samples; k += blockDim.x) smem[k] = 0.f;
    int cur_pose = -1;
    Ant tx, rx;
    int64_t first = 0, last = 0, offset = 0;
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = (long long)atomicAdd((unsigned long long *)p.work_counter, 1ull);
        __syncthreads();
        const int64_t item = s_item;
        if (item >= __ldg(&p.tile_start[p.pose_count])) break;
        const int pose = find_pose(p.tile_start, p.pose_count, item);
        if (pose != cur_pose) {
            if (cur_pose >= 0) {
                double *acc = p.acc + 2 * int64_t(cur_pose) * p.samples;
                for (int k = threadIdx.x; k < p.samples; k += blockDim.x) {
                    float re = smem[k], im = smem[p.samples + k];
                    if (re != 0.f) atomicAdd(&acc[2 * k], double(re));
                    if (im != 0.f) atomicAdd(&acc[2 * k + 1], double(im));
                    smem[k] = 0.f;
                    smem[p.samples + k] = 0.f;
                }
                __syncthreads();
            }
            cur_pose = pose;
            tx = load_ant(p.tx + pose);
            rx = load_ant(p.rx + pose);
            offset = __ldg(&p.offset[pose]);
        }
        const int64_t budget = __ldg(&p.budget[pose]);
        first = (item - __ldg(&p.tile_start[pose])) * p.tile;
        last = min(first + p.tile, budget);
        for (int64_t s = first + threadIdx.x; s < last; s += blockDim.x) {
            trace_sample<kPhase, kRecord, kCount>(p, tx, rx, uint64_t(offset + s), sc,
                                                  kRecord ? records + s * max_rec : nullptr, max_rec, &cnt, &rays);
        }
    }
    if (cur_pose >= 0) {
        __syncthreads();
        double *acc = p.acc + 2 * int64_t(cur_pose) * p.samples;
        for (int k = threadIdx.x; k < p.samples; k += blockDim.x) {
            float re = smem[k], im = smem[p.samples + k];
            if (re != 0.f) atomicAdd(&acc[2 * k], double(re));
            if (im != 0.f) atomicAdd(&acc[2 * k + 1], double(im));
        }
    }
    if (kCount) {
        atomicAdd(&p.counters[0], (unsigned long long)cnt.nodes);
        atomicAdd(&p.counters[1], (unsigned long long)cnt.tris);
        atomicAdd(&p.counters[2], (unsigned long long)rays);
    }
}

__global__ void k_tile_prefix(const int64_t *__restrict__ budget, int32_t pose_count, int32_t tile,
                              int64_t *__restrict__ tile_start) {
    // one CTA: serial-in-chunks prefix sum (pose counts are at most a few thousand)
    __shared__ int64_t s_base;
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    for (int32_t c0 = 0; c0 < pose_count; c0 += blockDim.x) {
        int32_t i = c0 + threadIdx.x;
        int64_t tiles = 0;
        if (i < pose_count) {
            int64_t b = budget[i];
            tiles = b > 0 ? (b + tile - 1) / tile : 0;
        }
        // inclusive scan in shared memory
        __shared__ int64_t sc[1024];
        sc[threadIdx.x] = tiles;
        __syncthreads();
        for (int off = 1; off < blockDim.x; off <<= 1) {
            int64_t v = threadIdx.x >= off ? sc[threadIdx.x - off] : 0;
            __syncthreads();
            sc[threadIdx.x] += v;
            __syncthreads();
        }
        if (i < pose_count) tile_start[i] = s_base + sc[threadIdx.x] - tiles;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_base += sc[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_start[pose_count] = s_base;
}

// fetchFrame (path.h:453-455): frame / totalWeight with totalWeight = budget * weight
__global__ void k_finalize(const double *__restrict__ acc, int32_t pose_count, int32_t samples,
                           const int64_t *__restrict__ budget, float sample_weight, int normalise,
                           float *__restrict__ out) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    int64_t n = int64_t(pose_count) * samples;
    if (i >= n) return;
    int pose = int(i / samples);
    float re = float(acc[2 * i]), im = float(acc[2 * i + 1]);
    if (normalise) {
        double tw = double(budget[pose]) * double(sample_weight);
        float inv = 1.f / float(tw);
        re *= inv;
        im *= inv;
    }
    out[2 * i] = re;
    out[2 * i + 1] = im;
}

__global__ void k_ray_queries(const DNode *__restrict__ nodes, const DTri *__restrict__ tris, int64_t count,
                              const float *__restrict__ o, const float *__restrict__ d, const float *__restrict__ tfar,
                              float *t, float *pp, float *nn, int32_t *prim, int32_t *vis, unsigned *status) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= count) return;
    f3 oo = mk3(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
    f3 dd = mk3(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
    if (vis) {
        vis[i] = any_hit<false>(nodes, tris, oo, dd, kEpsilon, tfar[i], status, nullptr) ? 0 : 1;
        return;
    }
    float th;
    int pr;
    int slot = closest_hit<false>(nodes, tris, oo, dd, kEpsilon, tfar[i], th, pr, status, nullptr);
    if (slot >= 0) {
        DTri T = load_tri(tris, slot);
        f3 n = hit_normal(T, dd);
        f3 hp = add3(oo, scl3(th, dd));
        t[i] = th;
        prim[i] = pr;
        pp[3 * i] = hp.x;
        pp[3 * i + 1] = hp.y;
        pp[3 * i + 2] = hp.z;
        nn[3 * i] = n.x;
        nn[3 * i + 1] = n.y;
        nn[3 * i + 2] = n.z;
    } else {
        t[i] = CUDART_INF_F;
        prim[i] = -1;
        for (int k = 0; k < 3; ++k) pp[3 * i + k] = nn[3 * i + k] = 0.f;
    }
}

}  // namespace

int trace_smem_bytes(int samples, int splat_mode, int fine_bins) {
    (void)splat_mode;
    (void)fine_bins;
    return 2 * samples * int(sizeof(float));
}

int trace_blocks_per_sm(int samples, int splat_mode, int fine_bins) {
    int nb = 0;
    int smem = trace_smem_bytes(samples, splat_mode, fine_bins);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_trace<HSR_PHASE_REFERENCE_FP32, false, false>, 256, smem);
    return nb > 0 ? nb : 1;
}

int launch_trace(const TraceParams &p, int phase_mode, int splat_mode, int grid, cudaStream_t st, std::string &err) {
    (void)splat_mode;
    int smem = trace_smem_bytes(p.samples, splat_mode, p.fine_bins);
    if (smem > 48 * 1024) {
        cudaFuncSetAttribute(k_trace<HSR_PHASE_REFERENCE_FP32, false, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaFuncSetAttribute(k_trace<HSR_PHASE_SPLIT_FP64, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
        cudaFuncSetAttribute(k_trace<HSR_PHASE_REFERENCE_FP32, true, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaFuncSetAttribute(k_trace<HSR_PHASE_REFERENCE_FP32, false, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    }
    if (p.records) {
        k_trace<HSR_PHASE_REFERENCE_FP32, true, false><<<grid, 256, smem, st>>>(p);
    } else if (p.counters) {
        k_trace<HSR_PHASE_REFERENCE_FP32, false, true><<<grid, 256, smem, st>>>(p);
    } else if (phase_mode == HSR_PHASE_SPLIT_FP64) {
        k_trace<HSR_PHASE_SPLIT_FP64, false, false><<<grid, 256, smem, st>>>(p);
    } else {
        k_trace<HSR_PHASE_REFERENCE_FP32, false, false><<<grid, 256, smem, st>>>(p);
    }
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("trace launch: ") + cudaGetErrorString(e);
        return 2;
    }
    return 0;
}

int launch_tile_prefix(const int64_t *budget, int32_t pose_count, int32_t tile, int64_t *tile_start, cudaStream_t st) {
    k_tile_prefix<<<1, 1024, 0, st>>>(budget, pose_count, tile, tile_start);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_finalize(const double *acc, int32_t pose_count, int32_t samples, const int64_t *budget, float sample_weight,
                    int normalise, float *out_rows, cudaStream_t st) {
    int64_t n = int64_t(pose_count) * samples;
    k_finalize<<<unsigned((n + 255) / 256), 256, 0, st>>>(acc, pose_count, samples, budget, sample_weight, normalise,
                                                           out_rows);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_ray_queries(const DNode *nodes, const DTri *tris, int64_t count, const float *o, const float *d,
                       const float *tfar, float *t, float *p, float *n, int32_t *prim, int32_t *vis, unsigned *status,
                       cudaStream_t st) {
    if (count <= 0) return 0;
    k_ray_queries<<<unsigned((count + 255) / 256), 256, 0, st>>>(nodes, tris, count, o, d, tfar, t, p, n, prim, vis,
                                                                  status);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace hsr
