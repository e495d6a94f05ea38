// Wavefront form of the radar path tracer (geometrical-optics mode, the reference's
// default, path.h:156): the same per-path arithmetic as the one-thread-per-sample
// kernel, reorganised so that warps stay converged.
//
// A persistent CTA of 256 threads keeps a stack of up to 384 live path states in
// shared memory (four CTAs per SM: 64 registers; ~32 KB of shared memory each plus the
// range row, so that four CTAs leave about 90 KB of the SM's L1 to the BVH) and
// alternates two stages:
//   GENERATE  (at most 128 live paths, or the autotuned queue threshold): 256 new
//             samples, one per thread: Halton point,
//             antenna ray, closest hit; paths that hit something are pushed.
//   EXTEND    (otherwise): 256 paths popped, one per thread: specular reflection,
//             next-event estimate towards RX (shadow ray, PO re-radiation, filtering,
//             phase), and the next closest hit; survivors are pushed back.
// Every next-event contribution is splatted by its warp cooperatively: lane l owns
// window offset l-16 of Frame::splat<16>, so one contribution's 33 bins are 33 distinct
// shared-memory addresses updated in one pass. The CTA's range row lives in shared
// memory and is flushed to the pose's FP64 accumulators when the CTA changes pose.
// Work items are (pose, 4096-sample tile) pairs pulled from a device counter.
//
// The kernel is a template over the phase mode; hsr_wave.cu instantiates the FP32
// reference-phase forms without multiply-add contraction (so the float expressions round
// as the CPU restatement does) and hsr_wave_split.cu the split-phase forms with it.
//
// Mixed batches (kMixed, the serving loop): each pose names its own resident scene,
// chirp, range-bin count and accumulator row (PoseJob). A CTA works on one pose at a
// time, so these are CTA-uniform: thread 0 copies the pose's job into shared memory
// when the CTA switches pose, and the arithmetic is the uniform kernel's.
#pragma once
#include "hsr_path.cuh"

namespace hsr {

namespace {

constexpr int kThreads = 256;
// GENERATE hands its samples to threads grouped by the cell of their primary sample point
// (4 x 2 cells of the unit square): a warp's primary rays leave the antenna in one part
// of the sphere, and their hits, pushed together, come back as neighbouring stack entries
constexpr int kPrimaryCells = 8;

// A CTA's live path states: a stack of kThreads + kQueue entries, where kQueue bounds the
// paths left when GENERATE runs (the queue threshold). Three capacities are built: 384
// entries (the default, thresholds up to 128), 320 (up to 64), whose 5 KB less shared
// memory per CTA leaves more of the SM's L1 to the BVH (4 % on the dense boxes scenes,
// which the autotuner runs at threshold 32 or 64), and 512 (up to 256), whose fuller
// EXTEND stages pay where the BVH stays in L1 anyway (7 % on the sphere bench).
template <int kCap> struct WaveShared {
    float ox[kCap], oy[kCap], oz[kCap];  // hit point (origin of the next segment)
    float dx[kCap], dy[kCap], dz[kCap];  // incoming direction
    float h[6][kCap];                    // incoming H field (re, im) x 3
    float nx[kCap], ny[kCap], nz[kCap];  // faceforwarded normal at the hit
    float r[kCap], cosT[kCap], freq[kCap];
    int depth[kCap];
    // the phase input: time of flight (FP32 reference phase, as float) or the FP64 path
    // length (split phase); each mode carries only its own
    double tlen[kCap];
    int count;
    int pose, pending_pose, exhausted;
    long long gen, gen_end, pending_first, pending_last;
    long long since_flush;      // samples generated since the row was last flushed
    PoseJob job;                // mixed batches: the current pose's scene, chirp and row
    int cell_count[kThreads / 32][kPrimaryCells];  // GENERATE: samples per warp and cell
    int cell_total[kPrimaryCells];
    short order[kThreads];      // GENERATE: stage sample offset of each thread
    FfAnt ff[2];                // far-field launches: the current pose's TX and RX
    float max_dist, bandwidth;  // mixed batches: derived from job.rf
};

struct Guided {  // the guiding part of a path's state
    float x0, x1, pdf;
    cf gw;
};

// Guided launches keep the guiding part of each stacked path (primary sample, pdf,
// weight) in five more [kCap] arrays after the training sums (`gst`, null otherwise).
constexpr int kGuideStackFields = 5;

template <int kPhase, int kCap>
__device__ __forceinline__ void push_path(WaveShared<kCap> &S, float *gst, f3 o, f3 d, const c3 &H, f3 n, float time,
                                          float r, float cosT, float freq, int depth, double plen, const Guided &g) {
    // one shared atomic per warp: the lanes pushing here take consecutive slots
    const unsigned active = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(active) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&S.count, __popc(active));
    base = __shfl_sync(active, base, leader);
    const int slot = base + __popc(active & ((1u << lane) - 1u));  // < kCap by construction (see k_wave)
    S.ox[slot] = o.x;
    S.oy[slot] = o.y;
    S.oz[slot] = o.z;
    S.dx[slot] = d.x;
    S.dy[slot] = d.y;
    S.dz[slot] = d.z;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        S.h[2 * i][slot] = H.v[i].re;
        S.h[2 * i + 1][slot] = H.v[i].im;
    }
    S.nx[slot] = n.x;
    S.ny[slot] = n.y;
    S.nz[slot] = n.z;
    S.r[slot] = r;
    S.cosT[slot] = cosT;
    S.freq[slot] = freq;
    S.depth[slot] = depth;
    if (kPhase == HSR_PHASE_REFERENCE_FP32)
        reinterpret_cast<float *>(S.tlen)[slot] = time;
    else
        S.tlen[slot] = plen;
    if (gst) {
        gst[slot] = g.x0;
        gst[kCap + slot] = g.x1;
        gst[2 * kCap + slot] = g.pdf;
        gst[3 * kCap + slot] = g.gw.re;
        gst[4 * kCap + slot] = g.gw.im;
    }
}

// A stable counting sort of the stage's items by key (< kPrimaryCells; the items
// [0, n) of the stage, thread t holding item t's key, threads t >= n holding
// kPrimaryCells): afterwards S.order[j] is the item thread j works on, for j < n. The
// order is the same in every run. Called by the whole CTA.
template <int kCap> __device__ __forceinline__ void order_by_key(WaveShared<kCap> &S, int key) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (lane < kPrimaryCells) S.cell_count[warp][lane] = 0;
    __syncwarp();
    if (rank == 0 && key < kPrimaryCells) S.cell_count[warp][key] = __popc(peers);
    __syncthreads();
    if (tid < kPrimaryCells) {
        int t = 0;
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) t += S.cell_count[w][tid];
        S.cell_total[tid] = t;
    }
    __syncthreads();
    if (key < kPrimaryCells) {
        int base = rank;
        for (int k = 0; k < key; ++k) base += S.cell_total[k];
        for (int w = 0; w < warp; ++w) base += S.cell_count[w][key];
        S.order[base] = short(tid);  // < n: the keyed items are the stage's
    }
    __syncthreads();
}

// Closest hit of the segment (o, d) and the bookkeeping of path.h:407-442 (GO mode).
// Returns true (and the new state) when the path continues with a stored hit. The
// reference's zero-field test (path.h:413, 439) is the caller's: in GO mode the field
// does not change across the hit, so testing it before or after is the same.
__device__ __forceinline__ bool walk(const TraceParams &p, const DNode *nodes, const DTri *tris, f3 o, f3 d,
                                     float &time, float &r, double &plen, f3 &hp, f3 &n, float &cosT) {
    float th;
    int primh;
    const int slot = closest_hit<false>(nodes, tris, o, d, kEpsilon, CUDART_INF_F, th, primh, p.status, nullptr);
    if (slot < 0) return false;
    DTri T = load_tri(tris, slot);
    n = hit_normal(T, d);
    hp = add3(o, scl3(th, d));
    cosT = fabsf(dot3(n, neg3(d)));
    if (cosT < 0.001f) return false;
    r += th;
    time += th / kSpeedOfLight;
    plen += double(th);
    return true;
}

// PathTracer::run's derived chirp quantities (path.h:240, radar.h:128-130).
__device__ __forceinline__ float max_distance(const hsr_rf_config &rf) {
    return rf.adcRate / rf.freqSlope * kSpeedOfLight;
}
__device__ __forceinline__ float chirp_bandwidth(const hsr_rf_config &rf) { return rf.freqSlope * rf.rampTime; }

// FP64 accumulator row of a pose: the pose's job row (mixed), its listed row, or
// pose-major rows of 2N.
template <bool kMixed, class Shared>
__device__ __forceinline__ double *pose_row(const TraceParams &p, const Shared &S, int pose) {
    if (kMixed) return p.acc + S.job.acc_offset;
    return p.acc + (p.acc_row ? __ldg(&p.acc_row[pose]) : 2 * int64_t(pose) * p.samples);
}

// Four CTAs per SM (64 registers): the spills cost less than the latency the extra
// warps hide (measured: 1.2x on the sphere bench, 1.13x on the serving mix over two).
// kLazy (the field_on_hit launch shape): with indirect-only paths, a primary ray's
// antenna field is formed only once the ray has hit something.
template <int kPhase, bool kMixed, int kQueue, bool kFF = false, bool kLazy = false>
__global__ void __launch_bounds__(kThreads, 4) k_wave(TraceParams p) {
    constexpr int kCap = kThreads + kQueue;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WaveShared<kCap> &S = *reinterpret_cast<WaveShared<kCap> *>(smem_raw);
    float *s_re = reinterpret_cast<float *>(smem_raw + sizeof(WaveShared<kCap>));
    float *s_im = s_re + p.samples;  // the row is sized for the largest N of the launch
    // guided launches: the CTA's training sums (second moment per training-tree node)
    float *s_g = s_re + 2 * p.samples;
    float *gst = p.do_guide ? s_g + kGuideMaxNodes : nullptr;
    const int tid = threadIdx.x;
    const hsr_tracer_flags &fl = p.flags;
    // the scene, chirp and row of the current pose: launch-uniform, or the pose's job
    const hsr_rf_config &rf = kMixed ? S.job.rf : p.rf;
    const float maxDist0 = max_distance(p.rf), bandwidth0 = chirp_bandwidth(p.rf);
#define HSR_NODES (kMixed ? S.job.nodes : p.nodes)
#define HSR_TRIS (kMixed ? S.job.tris : p.tris)
#define HSR_N (kMixed ? S.job.samples : p.samples)
#define HSR_MAXDIST (kMixed ? S.max_dist : maxDist0)
#define HSR_BANDWIDTH (kMixed ? S.bandwidth : bandwidth0)
    const long long total = __ldg(&p.tile_start[p.pose_count]);
    static_assert(kQueue <= kWaveMaxQueueThreshold, "queue threshold bound");
    const int queue_threshold = (p.queue_threshold > 0 && p.queue_threshold < kQueue) ? p.queue_threshold : kQueue;

    for (int k = tid; k < 2 * p.samples; k += kThreads) s_re[k] = 0.f;
    if (p.do_guide)
        for (int k = tid; k < kGuideMaxNodes; k += kThreads) s_g[k] = 0.f;
    if (tid == 0) {
        S.count = 0;
        S.pose = -1;
        S.pending_pose = -1;
        S.exhausted = 0;
        S.gen = S.gen_end = 0;
        S.since_flush = 0;
    }
    __syncthreads();

    PoseCtx pc;
    int cur_pose = -1;

    while (true) {
        // thread 0 pulls work items while the generation range is used up
        if (tid == 0) {
            while (S.gen >= S.gen_end && !S.exhausted && S.pending_pose < 0) {
                const long long item = (long long)atomicAdd((unsigned long long *)p.work_counter, 1ull);
                if (item >= total) {
                    S.exhausted = 1;
                    break;
                }
                const int pose = find_pose(p.tile_start, p.pose_count, item);
                const long long first = (item - __ldg(&p.tile_start[pose])) * p.tile;
                const long long last = min(first + (long long)p.tile, (long long)__ldg(&p.budget[pose]));
                if (pose == S.pose) {
                    S.gen = first;
                    S.gen_end = last;
                } else {
                    S.pending_pose = pose;
                    S.pending_first = first;
                    S.pending_last = last;
                }
            }
        }
        __syncthreads();
        const int count = S.count;
        const long long gen = S.gen, gen_end = S.gen_end;
        const int pending = S.pending_pose;
        const int exhausted = S.exhausted;
        const long long since_flush = S.since_flush;
        __syncthreads();  // every thread has read the shared control words

        if (since_flush >= kFlushSamples && cur_pose >= 0) {
            // bound the FP32 partial sums: move the row to the FP64 accumulators
            flush_row(pose_row<kMixed>(p, S, cur_pose), s_re, s_im, HSR_N);
            if (p.do_guide) flush_guide(pc, s_g);
            if (tid == 0) S.since_flush = 0;
            __syncthreads();
            continue;
        }

        if (gen < gen_end && count <= queue_threshold) {
            // ---------------- GENERATE ----------------
            if (tid == 0) {
                S.gen = min(gen + (long long)kThreads, gen_end);
                S.since_flush += S.gen - gen;
            }
            // the stage's samples gen + [0, n), ordered by primary cell: thread t traces
            // sample gen + S.order[t]
            const int n_stage = int(min((long long)kThreads, gen_end - gen));
            if (p.coherent_order) {
                int key = kPrimaryCells;
                if (tid < n_stage) {
                    const uint64_t h0 = uint64_t(pc.offset + gen + tid);
                    const float u0 = halton(h0, 1 + kGet2DFirst), u1 = halton(h0, 1 + kGet2DSecond);
                    key = min(int(u0 * 4.f), 3) * 2 + min(int(u1 * 2.f), 1);
                }
                order_by_key(S, key);
            }
            const long long s = gen + (p.coherent_order && tid < n_stage ? S.order[tid] : tid);
            bool has_item = false;
            float4 item = make_float4(0.f, 0.f, 0.f, 0.f);
            if (s < gen_end) {
                const uint64_t hindex = uint64_t(pc.offset + s);
                const float freq = rf.startFreq + halton(hindex, 0) * HSR_BANDWIDTH;
                Guided g{halton(hindex, 1 + kGet2DFirst), halton(hindex, 1 + kGet2DSecond), 1.f, cf{0.f, 0.f}};
                if (fl.doGuiding) g.pdf = guide_sample(pc.samp_child, pc.samp_p, g.x0, g.x1);
                f3 o, d;
                c3 H;
                f3 ldir = mk3(0.f, 0.f, 0.f);  // kLazy: the local direction the field is formed from
                const bool deferred = kLazy && fl.onlyIndirect;
                if (kFF) {
                    ff_sample(S.ff[0], g.x0, g.x1, o, d, H);
                    H = c3_scl(H, 1.f / g.pdf);
                } else if (kLazy) {
                    o = pc.tx.pos;
                    ldir = uniform_sample_sphere<kPhase == HSR_PHASE_REFERENCE_FP32>(g.x0, g.x1);
                    d = mulv(pc.tx.rot, ldir);
                    if (!deferred) H = c3_scl(antenna_field(pc.tx, ldir), 1.f / g.pdf);
                } else {
                    o = pc.tx.pos;
                    antenna_sample<kPhase == HSR_PHASE_REFERENCE_FP32>(pc.tx, g.x0, g.x1, d, H);
                    H = c3_scl(H, 1.f / g.pdf);
                }
                if (!fl.onlyIndirect) {
                    NeeOut ne;
                    if (nee_eval<kPhase, false, kFF>(p, HSR_NODES, HSR_TRIS, rf, HSR_N, pc.tx, pc.rx, 0, o, d,
                                                     mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 0.f), H, H, 0.f, 0.0, 0.f,
                                                     1.f, freq, pc.weight, ne, nullptr, nullptr, &S.ff[1]) &&
                        ne.splat) {
                        if (pc.fine_row) {
                            splat_fine(pc.fine_row, p.fine_bins, ne.sample, ne.value);
                        } else {
                            item = splat_item(ne.sample, ne.value);
                            has_item = true;
                        }
                    }
                }
                bool alive = false;
                if (!(0 >= fl.maxDepth || 0.f >= HSR_MAXDIST) && (deferred || !c3_is_zero(H))) {
                    float time = 0.f, r = 0.f, cosT;
                    double plen = 0.0;
                    f3 hp, n;
                    if (walk(p, HSR_NODES, HSR_TRIS, o, d, time, r, plen, hp, n, cosT)) {
                        // deferred: the field now (the same operations as antenna_sample); a
                        // zero field ends the path as the reference's test before tracing would
                        if (deferred) H = c3_scl(antenna_field(pc.tx, ldir), 1.f / g.pdf);
                        if (!deferred || !c3_is_zero(H)) {
                            push_path<kPhase, kCap>(S, gst, hp, d, H, n, time, r, cosT, freq, 1, plen, g);
                            alive = true;
                        }
                    }
                }
                if (!alive) guide_train(pc, pc.train_child, s_g, 1, g.gw, g.pdf, g.x0, g.x1);
            }
            if (!fl.onlyIndirect) splat_warp(s_re, s_im, HSR_N, has_item, item);
            __syncthreads();
            continue;
        }

        if (count > 0) {
            // ---------------- EXTEND ----------------
            const int n = min(count, kThreads);
            const bool mine = tid < n;
            f3 o, din, nrm;
            c3 Hin;
            float time = 0.f, r = 0.f, cosT = 1.f, freq = 0.f;
            int depth = 0;
            double plen = 0.0;
            Guided g{0.f, 0.f, 1.f, cf{0.f, 0.f}};
            // the popped paths, ordered by the octant of their reflected direction: thread t
            // continues stack entry count - 1 - S.order[t]
            if (p.coherent_order) {
                int key = kPrimaryCells;
                if (mine) {
                    const int e = count - 1 - tid;
                    const f3 di = mk3(S.dx[e], S.dy[e], S.dz[e]), nn = mk3(S.nx[e], S.ny[e], S.nz[e]);
                    const float dn = 2.f * dot3(di, nn);
                    key = (di.x - dn * nn.x < 0.f ? 1 : 0) | (di.y - dn * nn.y < 0.f ? 2 : 0) |
                          (di.z - dn * nn.z < 0.f ? 4 : 0);
                }
                order_by_key(S, key);
            }
            if (mine) {
                const int slot = count - 1 - (p.coherent_order ? S.order[tid] : tid);
                if (gst)
                    g = Guided{gst[slot], gst[kCap + slot], gst[2 * kCap + slot],
                               cf{gst[3 * kCap + slot], gst[4 * kCap + slot]}};
                o = mk3(S.ox[slot], S.oy[slot], S.oz[slot]);
                din = mk3(S.dx[slot], S.dy[slot], S.dz[slot]);
#pragma unroll
                for (int i = 0; i < 3; ++i) Hin.v[i] = cf{S.h[2 * i][slot], S.h[2 * i + 1][slot]};
                nrm = mk3(S.nx[slot], S.ny[slot], S.nz[slot]);
                if (kPhase == HSR_PHASE_REFERENCE_FP32)
                    time = reinterpret_cast<const float *>(S.tlen)[slot];
                else
                    plen = S.tlen[slot];
                r = S.r[slot];
                cosT = S.cosT[slot];
                freq = S.freq[slot];
                depth = S.depth[slot];
            }
            __syncthreads();  // all pops read before the stack shrinks
            if (tid == 0) S.count = count - n;
            __syncthreads();
            bool has_item = false;
            float4 item = make_float4(0.f, 0.f, 0.f, 0.f);
            if (mine) {
                f3 d = din;
                c3 H = Hin;
                reflect(nrm, d, H);
                NeeOut ne;
                if (nee_eval<kPhase, false, kFF>(p, HSR_NODES, HSR_TRIS, rf, HSR_N, pc.tx, pc.rx, depth, o, d, din,
                                                 nrm, Hin, H, time, plen, r, cosT, freq, pc.weight, ne, nullptr,
                                                 nullptr, &S.ff[1])) {
                    g.gw = cadd(g.gw, ne.gw_add);
                    if (ne.splat) {
                        if (pc.fine_row) {
                            splat_fine(pc.fine_row, p.fine_bins, ne.sample, ne.value);
                        } else {
                            item = splat_item(ne.sample, ne.value);
                            has_item = true;
                        }
                    }
                }
                bool alive = false;
                if (!(depth >= fl.maxDepth || r >= HSR_MAXDIST) && !c3_is_zero(H)) {
                    f3 hp, n2;
                    float cosT2;
                    if (walk(p, HSR_NODES, HSR_TRIS, o, d, time, r, plen, hp, n2, cosT2)) {
                        push_path<kPhase, kCap>(S, gst, hp, d, H, n2, time, r, cosT2, freq, depth + 1, plen, g);
                        alive = true;
                    }
                }
                if (!alive) guide_train(pc, pc.train_child, s_g, 1, g.gw, g.pdf, g.x0, g.x1);
            }
            splat_warp(s_re, s_im, HSR_N, has_item, item);
            __syncthreads();
            continue;
        }

        if (pending >= 0) {
            // stack drained: finish the old pose's row and switch to the new pose
            if (cur_pose >= 0) {
                flush_row(pose_row<kMixed>(p, S, cur_pose), s_re, s_im, HSR_N);
                if (p.do_guide) flush_guide(pc, s_g);
            }
            cur_pose = pending;
            pc = load_pose(p, cur_pose);
            __syncthreads();  // every thread is done with the old pose's job
            if (tid == 0) {
                if (kMixed) {
                    S.job = p.jobs[pending];
                    S.max_dist = max_distance(S.job.rf);
                    S.bandwidth = chirp_bandwidth(S.job.rf);
                }
                if (kFF) {
                    S.ff[0] = load_ff(p.ff_tx + pending);
                    S.ff[1] = load_ff(p.ff_rx + pending);
                }
                S.pose = pending;
                S.since_flush = 0;
                S.gen = S.pending_first;
                S.gen_end = S.pending_last;
                S.pending_pose = -1;
            }
            __syncthreads();
            continue;
        }
        if (exhausted) break;
    }
    if (cur_pose >= 0) {
        __syncthreads();
        flush_row(pose_row<kMixed>(p, S, cur_pose), s_re, s_im, HSR_N);
        if (p.do_guide) flush_guide(pc, s_g);
    }
#undef HSR_NODES
#undef HSR_TRIS
#undef HSR_N
#undef HSR_MAXDIST
#undef HSR_BANDWIDTH
}

// Dynamic shared memory of a launch: the stack, the range row of N bins and, guided, the
// CTA's training sums and the guiding part of the stacked paths.
template <int kQueue> size_t wave_smem_for(int samples, bool guided) {
    constexpr int kCap = kThreads + kQueue;
    return sizeof(WaveShared<kCap>) + 2 * size_t(samples) * sizeof(float) +
           (guided ? (kGuideMaxNodes + kGuideStackFields * kCap) * sizeof(float) : 0);
}

// The stack capacity (as its GENERATE threshold) a launch with threshold q runs: 64 for
// 1..64, 256 above 128, else (0 = the default, or 65..128) 128.
inline int wave_capacity(int32_t q) {
    return (q > 0 && q <= kWaveSmallQueue) ? kWaveSmallQueue : (q > kWaveDefaultQueue ? kWaveMaxQueueThreshold
                                                                                      : kWaveDefaultQueue);
}

// The launch of one instantiation.
template <int kPhase, bool kMixed, int kQueue, bool kFF = false, bool kLazy = false>
void wave_instance(const TraceParams &p, int grid, cudaStream_t st) {
    const size_t smem = wave_smem_for<kQueue>(p.samples, p.do_guide != 0);
    cudaFuncSetAttribute(k_wave<kPhase, kMixed, kQueue, kFF, kLazy>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(smem));
    k_wave<kPhase, kMixed, kQueue, kFF, kLazy><<<grid, kThreads, smem, st>>>(p);
}

// The uniform form at one capacity, with the primary field formed eagerly or on a hit.
template <int kPhase, int kQueue> void wave_uniform(const TraceParams &p, int grid, cudaStream_t st) {
    if (p.field_on_hit)
        wave_instance<kPhase, false, kQueue, false, true>(p, grid, st);
    else
        wave_instance<kPhase, false, kQueue>(p, grid, st);
}

// Every instantiation of one phase mode: the mixed form (serving ticks) and the uniform
// form, each at both stack capacities. The mixed form takes the small stack unless the
// tick asks for a threshold above 64 (its default: on the serving mix of dense boxes
// and urban scenes it gives 1.18x the capacity of the 384-entry stack).
template <int kPhase> void wave_dispatch(const TraceParams &p, int grid, cudaStream_t st) {
    const int cap = wave_capacity(p.queue_threshold);
    if (p.ff_tx) {  // far-field runs: the uniform form at the default capacity
        wave_instance<kPhase, false, kWaveDefaultQueue, true>(p, grid, st);
    } else if (p.jobs) {  // the mixed form is built at the two smaller capacities
        if (p.queue_threshold > kWaveSmallQueue)
            wave_instance<kPhase, true, kWaveDefaultQueue>(p, grid, st);
        else
            wave_instance<kPhase, true, kWaveSmallQueue>(p, grid, st);
    } else if (cap == kWaveSmallQueue) {
        wave_uniform<kPhase, kWaveSmallQueue>(p, grid, st);
    } else if (cap == kWaveMaxQueueThreshold) {
        wave_uniform<kPhase, kWaveMaxQueueThreshold>(p, grid, st);
    } else {
        wave_uniform<kPhase, kWaveDefaultQueue>(p, grid, st);
    }
}

}  // namespace

}  // namespace hsr
