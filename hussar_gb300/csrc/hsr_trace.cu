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
#include "hsr_path.cuh"

namespace hsr {

namespace {

struct PathRecord {  // one next-event estimate (tests only)
    int32_t depth;
    int32_t splatted;
    float time;
    float v_re, v_im;
    float dphase;
    float bin;
    float value_re, value_im;
};

// One sample, one thread: PathTracer::sample (path.h:235-451) for every flag combination.
// kFF: the pose's TX and RX are far-field antennas (ftx, frx; FFAntenna, emitter.h:226-291).
template <int kPhase, bool kRecord, bool kCount, bool kFF>
__device__ void trace_sample(const TraceParams &p, const PoseCtx &pc, uint64_t hindex, float *s_re, float *s_im,
                             PathRecord *rec, int max_rec, TraversalCounters *cnt, unsigned *rays, const FfAnt &ftx,
                             const FfAnt &frx) {
    const Ant &tx = pc.tx;
    const Ant &rx = pc.rx;
    const hsr_rf_config &rf = p.rf;
    const hsr_tracer_flags &fl = p.flags;
    const float inf = CUDART_INF_F;
    int dim = 0;
    const float maxDist = rf.adcRate / rf.freqSlope * kSpeedOfLight;
    float primaryPdf = 1.f;
    float px = 0.f, py = 0.f;
    cf gw = cf{0.f, 0.f};
    const float bandwidth = rf.freqSlope * rf.rampTime;
    const float freq = rf.startFreq + halton(hindex, dim++) * bandwidth;
    const float k0 = 2.f * kPi * freq / kSpeedOfLight;

    f3 o = mk3(0.f, 0.f, 0.f), d = mk3(0.f, 0.f, 0.f);
    float time = 0.f;
    double plen = 0.0;  // path length in FP64 (split-phase mode)
    int depth = 0;
    c3 H;
    f3 hit_n = mk3(0.f, 0.f, 0.f);
    c3 inc_H;
    float r = 0.f, cosTheta = 1.f;
    int nrec = 0;

    while (true) {
        const f3 tmpd = d;
        if (depth == 0) {
            px = halton(hindex, dim + kGet2DFirst);  // get2D (GCC order, hsr_path.cuh)
            py = halton(hindex, dim + kGet2DSecond);
            dim += 2;
            if (fl.doGuiding) primaryPdf = guide_sample(pc.samp_child, pc.samp_p, px, py);
            if (kFF) {
                ff_sample(ftx, px, py, o, d, H);
            } else {
                o = tx.pos;
                antenna_sample<kPhase == HSR_PHASE_REFERENCE_FP32>(tx, px, py, d, H);
            }
            H = c3_scl(H, 1.f / primaryPdf);
        } else if (!fl.useGeometricalOptics) {
            const float u0 = halton(hindex, dim + kGet2DFirst);
            const float u1 = halton(hindex, dim + kGet2DSecond);
            dim += 2;
            d = uniform_sample_sphere<kPhase == HSR_PHASE_REFERENCE_FP32>(u0, u1);
            H = surface_eval(hit_n, inc_H, d);
        } else {
            reflect(hit_n, d, H);
        }

        // next event estimation towards the single RX antenna (path.h:292-397)
        if (!(depth == 0 && fl.onlyIndirect)) {
            NeeOut ne;
            if (nee_eval<kPhase, kCount, kFF>(p, p.nodes, p.tris, p.rf, p.samples, tx, rx, depth, o, d, tmpd, hit_n,
                                              inc_H, H, time, plen, r, cosTheta, freq, pc.weight, ne, cnt, rays,
                                              &frx)) {
                gw = cadd(gw, ne.gw_add);
                if (kRecord && nrec < max_rec) {
                    PathRecord *rc = rec + nrec++;
                    rc->depth = depth;
                    rc->time = ne.time;
                    rc->v_re = ne.v.re;
                    rc->v_im = ne.v.im;
                    rc->dphase = ne.dphase;
                    rc->splatted = ne.splat ? 1 : 0;
                    rc->bin = ne.sample;
                    rc->value_re = ne.value.re;
                    rc->value_im = ne.value.im;
                }
                if (ne.splat) {
                    if (pc.fine_row)
                        splat_fine(pc.fine_row, p.fine_bins, ne.sample, ne.value);
                    else
                        splat_serial(s_re, s_im, p.samples, splat_prepare(ne.sample, ne.value));
                }
            }
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
        // non-GO primary segment of a far-field TX: FFAntenna::connect does nothing (no
        // time of flight, no 1 / (4 pi r)); every other segment adds its distance
        if (!(kFF && depth == 0 && !fl.useGeometricalOptics)) {
            time += th / kSpeedOfLight;
            plen += double(th);
        }
        if (!fl.useGeometricalOptics) {
            if (depth == 0) {
                if (!kFF) H = c3_scl(H, 1.f / (4.f * kPi * th));
            } else {
                H = c3_cmul(H, green(k0, th));
            }
            H = c3_scl(H, th * th / cosTheta);
        }
        if (c3_is_zero(H)) break;
        inc_H = H;
        o = hp;
        depth++;
    }
    if (pc.train) guide_train(pc, pc.train_child, pc.train_acc + 2, 3, gw, primaryPdf, px, py);
}

template <int kPhase, bool kRecord, bool kCount, bool kFF = false>
__global__ void __launch_bounds__(256, 2) k_trace(TraceParams p) {
    TraversalCounters cnt{0u, 0u};
    unsigned rays = 0;
    PathRecord *records = static_cast<PathRecord *>(p.records);
    const int max_rec = p.max_rec;
    extern __shared__ float smem[];
    __shared__ long long s_item;
    float *s_re = smem, *s_im = smem + p.samples;
    for (int k = threadIdx.x; k < 2 * p.samples; k += blockDim.x) smem[k] = 0.f;
    int cur_pose = -1;
    long long since_flush = 0;  // samples of cur_pose in the row since its last flush (CTA-uniform)
    PoseCtx pc;
    FfAnt ftx{}, frx{};
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = (long long)atomicAdd((unsigned long long *)p.work_counter, 1ull);
        __syncthreads();
        const int64_t item = s_item;
        if (item >= __ldg(&p.tile_start[p.pose_count])) break;
        const int pose = find_pose(p.tile_start, p.pose_count, item);
        if (pose != cur_pose) {
            if (cur_pose >= 0) {
                flush_row(p.acc + 2 * int64_t(cur_pose) * p.samples, s_re, s_im, p.samples);
                __syncthreads();
            }
            cur_pose = pose;
            pc = load_pose(p, pose);
            if (kFF) {
                ftx = load_ff(p.ff_tx + pose);
                frx = load_ff(p.ff_rx + pose);
            }
            since_flush = 0;
        }
        const int64_t budget = __ldg(&p.budget[pose]);
        const int64_t first = (item - __ldg(&p.tile_start[pose])) * p.tile;
        const int64_t last = min(first + p.tile, budget);
        for (int64_t s = first + threadIdx.x; s < last; s += blockDim.x) {
            trace_sample<kPhase, kRecord, kCount, kFF>(p, pc, uint64_t(pc.offset + s), s_re, s_im,
                                                       kRecord ? records + s * max_rec : nullptr, max_rec, &cnt, &rays,
                                                       ftx, frx);
        }
        since_flush += last - first;
        if (since_flush >= kFlushSamples) {
            // bound the FP32 partial sums: move the row to the FP64 accumulators
            __syncthreads();
            flush_row(p.acc + 2 * int64_t(cur_pose) * p.samples, s_re, s_im, p.samples);
            since_flush = 0;
        }
    }
    if (cur_pose >= 0) {
        __syncthreads();
        flush_row(p.acc + 2 * int64_t(cur_pose) * p.samples, s_re, s_im, p.samples);
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

// fetchFrame (path.h:453-455): frame / totalWeight, with totalWeight = budget * weight
// (plain runs) or the schedule's accumulated weight (total_weight, guided runs)
__global__ void k_finalize(const double *__restrict__ acc, int32_t pose_count, int32_t samples,
                           const int64_t *__restrict__ budget, float sample_weight,
                           const double *__restrict__ total_weight, int normalise, float *__restrict__ out) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    int64_t n = int64_t(pose_count) * samples;
    if (i >= n) return;
    int pose = int(i / samples);
    float re = float(acc[2 * i]), im = float(acc[2 * i + 1]);
    if (normalise) {
        double tw = total_weight ? total_weight[pose] : double(budget[pose]) * double(sample_weight);
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
    if (p.ff_tx) {
        if (smem > 48 * 1024) {
            cudaFuncSetAttribute(k_trace<HSR_PHASE_REFERENCE_FP32, false, false, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            cudaFuncSetAttribute(k_trace<HSR_PHASE_SPLIT_FP64, false, false, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        }
        if (phase_mode == HSR_PHASE_SPLIT_FP64)
            k_trace<HSR_PHASE_SPLIT_FP64, false, false, true><<<grid, 256, smem, st>>>(p);
        else
            k_trace<HSR_PHASE_REFERENCE_FP32, false, false, true><<<grid, 256, smem, st>>>(p);
    } else if (p.records) {
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

// Zeroes the accumulator rows of the poses with clear[pose] != 0 (clearFrame, path.h:147-150).
__global__ void k_clear_rows(double *acc, int32_t pose_count, int32_t samples, const int *__restrict__ clear) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= int64_t(pose_count) * samples) return;
    if (clear[i / samples]) {
        acc[2 * i] = 0.0;
        acc[2 * i + 1] = 0.0;
    }
}

// Zeroes the fine-histogram rows (len floats each) of the poses with clear[pose] != 0.
__global__ void k_clear_rows_f(double *rows, int32_t pose_count, int32_t len, const int *__restrict__ clear) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= int64_t(pose_count) * len) return;
    if (clear[i / len]) rows[i] = 0.0;
}

int launch_clear_rows_f(double *rows, int32_t pose_count, int32_t len, const int *clear, cudaStream_t st) {
    int64_t n = int64_t(pose_count) * len;
    k_clear_rows_f<<<unsigned((n + 255) / 256), 256, 0, st>>>(rows, pose_count, len, clear);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_clear_rows(double *acc, int32_t pose_count, int32_t samples, const int *clear, cudaStream_t st) {
    int64_t n = int64_t(pose_count) * samples;
    k_clear_rows<<<unsigned((n + 255) / 256), 256, 0, st>>>(acc, pose_count, samples, clear);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_tile_prefix(const int64_t *budget, int32_t pose_count, int32_t tile, int64_t *tile_start, cudaStream_t st) {
    k_tile_prefix<<<1, 1024, 0, st>>>(budget, pose_count, tile, tile_start);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_finalize(const double *acc, int32_t pose_count, int32_t samples, const int64_t *budget, float sample_weight,
                    const double *total_weight, int normalise, float *out_rows, cudaStream_t st) {
    int64_t n = int64_t(pose_count) * samples;
    k_finalize<<<unsigned((n + 255) / 256), 256, 0, st>>>(acc, pose_count, samples, budget, sample_weight,
                                                           total_weight, normalise, out_rows);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

namespace {
// The radar cube of a MIMO frame (radar.h:487-494: [chirp][sample][channel], complex64)
// from the channels' fetchFrame rows: a static scene puts everything in Doppler bin 0
// (PIndex::setVelocity(0), path.h:130), so chirp 0 holds row c at channel c and every
// other chirp is zero.
__global__ void k_assemble_frame(const float2 *__restrict__ rows, int32_t chirps, int32_t samples, int32_t channels,
                                 float2 *__restrict__ frame) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const int64_t n = int64_t(chirps) * samples * channels;
    if (i >= n) return;
    const int32_t c = int32_t(i % channels);
    const int64_t cs = i / channels;
    const int32_t k = int32_t(cs % samples), chirp = int32_t(cs / samples);
    frame[i] = chirp == 0 ? rows[int64_t(c) * samples + k] : make_float2(0.f, 0.f);
}

__global__ void k_debug_halton(const uint64_t *index, int64_t count, int dim, float *out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < count) out[i] = halton(index[i], dim);
}

// Every float x with |x| bits in [lo_bits, hi_bits], both signs: sincos_cr against
// sincos_rounded. counts: [0] arguments checked, [1] mismatches, [2] arguments where
// sincos_cr took sincos_rounded (outside the fast range or not certified).
__global__ void k_debug_sincos_sweep(unsigned lo_bits, unsigned hi_bits, unsigned long long *counts) {
    unsigned long long checked = 0, bad = 0, slow = 0;
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned u = lo_bits + blockIdx.x * blockDim.x + threadIdx.x; u <= hi_bits && u >= lo_bits; u += stride) {
        for (unsigned sign = 0; sign < 2; ++sign) {
            const float x = __uint_as_float(u | (sign << 31));
            float s0, c0, s1, c1;
            sincos_rounded(x, &s0, &c0);
            sincos_cr(x, &s1, &c1);
            bad += (__float_as_uint(s0) != __float_as_uint(s1)) || (__float_as_uint(c0) != __float_as_uint(c1));
            dfloat sv, cv;
            sincos_df(x, sv, cv);
            const float ax = fabsf(x);
            slow += !(ax >= 0x1p-14f && ax <= 8.f && rounds_to_high(sv) && rounds_to_high(cv));
            ++checked;
        }
        if (u > hi_bits - stride) break;  // the next u would wrap past 2^32
    }
    atomicAdd(&counts[0], checked);
    if (bad) atomicAdd(&counts[1], bad);
    if (slow) atomicAdd(&counts[2], slow);
}
}  // namespace

int launch_assemble_frame(const float *rows, int32_t chirps, int32_t samples, int32_t channels, float *frame,
                          cudaStream_t st) {
    const int64_t n = int64_t(chirps) * samples * channels;
    k_assemble_frame<<<unsigned((n + 255) / 256), 256, 0, st>>>(reinterpret_cast<const float2 *>(rows), chirps,
                                                                 samples, channels, reinterpret_cast<float2 *>(frame));
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_debug_halton(const uint64_t *d_index, int64_t count, int dim, float *d_out) {
    if (count <= 0) return 0;
    k_debug_halton<<<unsigned((count + 255) / 256), 256>>>(d_index, count, dim, d_out);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_debug_sincos_sweep(unsigned lo_bits, unsigned hi_bits, unsigned long long *d_counts) {
    k_debug_sincos_sweep<<<152 * 16, 256>>>(lo_bits, hi_bits, d_counts);
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
