// Serving: continuous batching of simulation requests over resident scenes.
//
// The reference runs one pose per synchronous backend call (src/arch/gpu.cpp:499-532;
// the examples loop poses on the host, examples/src/2_large_scene.cpp:149-166). Here a
// server owns a stream and a worker thread and runs *ticks*: one persistent wavefront
// launch (k_wave, mixed form) over a slice of every admitted request, each slice a
// (pose, Halton range) segment with its own scene, chirp and accumulator row. Requests
// that arrive while a tick is on the device are admitted for the next tick, so the
// device keeps working on a changing set of requests instead of a queue of whole jobs.
//
//   admission  FIFO, when a slot (max_slots) and device memory for the request's FP64
//              accumulator row (first-fit arena of memory_bytes) are free;
//   planning   the tick's sample target (measured samples/ms x tick_ms, at least four
//              1024-sample tiles per resident CTA so every SM has work and the tail is
//              short) is split by water-filling in order of the smallest remainder:
//              short requests finish in one tick, long ones share the rest; every chunk
//              but a request's last is a whole number of tiles, so a request's samples
//              are exactly the Halton indices of a standalone hsr_simulate_batch run;
//   one tick   one H2D copy of the tick block (segments, tile prefix, jobs, finalize
//              list, zeroed status/work counter), k_wave, k_serve_finalize for requests
//              whose last chunk ran (row = acc / budget, then the accumulators are
//              cleared so free arena memory stays zero), D2H of the status word and the
//              finished rows, and a host callback that wakes the worker;
//   pipelining two tick slots on two streams: the next tick is built while one runs,
//              and its CTAs take the SMs the running tick's tail frees. A tick's
//              finalize waits for the previous tick (requests span ticks), which also
//              keeps completions in order.
//   guiding    (server flags with doGuiding) every request runs PathTracer::run's
//              doubling schedule (path.h:171-224) over a guiding tree of the server's
//              pool (one per slot, reset at admission): a request's chunks come from its
//              current iteration (Halton offset, sample weight and training flag of that
//              iteration); the tick that places an iteration's last chunk, once the
//              previous tick is done too, clears the request's row when the next iteration
//              starts a fresh frame and steps its tree (k_guide_step: build, copy,
//              refine); the request is planned again only after that tick has finished,
//              so the next iteration samples the stepped tree. The final iteration does
//              not train, and its row is normalised by that iteration's total weight.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "hsr_common.cuh"
#include "hsr_internal.h"

namespace hsr {

namespace {

using Clock = std::chrono::steady_clock;

constexpr int32_t kServeTile = 1024;  // samples per work item
constexpr int kTickSlots = 2;
constexpr int kTilesPerCta = 4;  // minimum tick size, in tiles per resident CTA
constexpr int32_t kServeMaxTile = 16384;  // largest work item of a tick with large chunks
constexpr int kEndRing = 4;      // tick-end events kept for the busy-time union

struct FinJob {
    int64_t acc_offset;  // doubles into the arena
    int64_t out_offset;  // floats into the tick's output block
    double total_weight;  // the frame's totalWeight: budget (plain), the schedule's (guided)
    int32_t samples;
    int32_t reserved;
};

// fetchFrame of finished requests: row = acc / totalWeight (path.h:445,453-455; plain:
// budget x sample weight 1), rounded as k_finalize; then clears the accumulators. One CTA
// per request.
__global__ void k_serve_finalize(const FinJob *__restrict__ jobs, double *acc, float *out) {
    const FinJob j = jobs[blockIdx.x];
    double *a = acc + j.acc_offset;
    float *o = out + j.out_offset;
    const float inv = 1.f / float(j.total_weight);
    for (int k = threadIdx.x; k < j.samples; k += blockDim.x) {
        float re = float(a[2 * k]), im = float(a[2 * k + 1]);
        o[2 * k] = re * inv;
        o[2 * k + 1] = im * inv;
        a[2 * k] = 0.0;
        a[2 * k + 1] = 0.0;
    }
}

// clearFrame between guided iterations (path.h:212-215): zero the listed rows
__global__ void k_serve_clear(const FinJob *__restrict__ jobs, double *acc) {
    const FinJob j = jobs[blockIdx.x];
    double *a = acc + j.acc_offset;
    for (int k = threadIdx.x; k < 2 * j.samples; k += blockDim.x) a[k] = 0.0;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// First-fit allocator over [0, size) (offsets and sizes in bytes, multiples of 256).
class Arena {
  public:
    void init(int64_t size) {
        free_.clear();
        if (size > 0) free_[0] = size;
        used_ = 0;
    }
    int64_t alloc(int64_t bytes) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const int64_t off = it->first, rest = it->second - bytes;
            free_.erase(it);
            if (rest > 0) free_[off + bytes] = rest;
            used_ += bytes;
            return off;
        }
        return -1;
    }
    void release(int64_t off, int64_t bytes) {
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    int64_t used() const { return used_; }

  private:
    std::map<int64_t, int64_t> free_;
    int64_t used_ = 0;
};

struct Req {
    hsr_request r{};
    uint64_t ticket = 0;
    const SceneDev *scene = nullptr;
    Clock::time_point t_submit, t_admit, t_done;
    int64_t scheduled = 0;  // samples handed to ticks (all iterations)
    // guided requests: the schedule, the current iteration and how much of it was handed
    // out, the pool tree, and the tick whose end releases the next iteration
    std::vector<Iter> sched;
    int iter = 0;
    int64_t iter_done = 0;
    int guide_slot = -1;
    bool needs_reset = false;
    bool waiting = false;
    int64_t wait_seq = -1;
    int64_t arena_off = -1, arena_bytes = 0;
    int32_t ticks = 0;
    int32_t in_flight = 0;  // queued ticks that contain a segment of it
    bool finalize_queued = false;
    bool failed = false;
    bool done = false;
    hsr_status status = HSR_OK;
};
using ReqPtr = std::shared_ptr<Req>;

// Fixed layout of a tick's input block (host pinned and device), for `cap` segments.
struct TickLayout {
    size_t counters = 0, tile = 0, budget = 0, offset = 0, tx = 0, rx = 0, jobs = 0, acc_row = 0, fin = 0;
    size_t weight = 0, train = 0, slot = 0, active = 0, clear = 0, bytes = 0;
    void init(int cap) {
        size_t o = 0;
        counters = o;
        o += 256;
        tile = o;
        o = align256(o + sizeof(int64_t) * (cap + 1));
        budget = o;
        o = align256(o + sizeof(int64_t) * cap);
        offset = o;
        o = align256(o + sizeof(int64_t) * cap);
        tx = o;
        o = align256(o + sizeof(hsr_antenna) * cap);
        rx = o;
        o = align256(o + sizeof(hsr_antenna) * cap);
        jobs = o;
        o = align256(o + sizeof(PoseJob) * cap);
        acc_row = o;
        o = align256(o + sizeof(int64_t) * cap);
        fin = o;
        o = align256(o + sizeof(FinJob) * cap);
        // guided ticks: per segment sample weight, training flag and tree slot; per pool
        // tree the step flag; rows cleared between iterations
        weight = o;
        o = align256(o + sizeof(float) * cap);
        train = o;
        o = align256(o + sizeof(int32_t) * cap);
        slot = o;
        o = align256(o + sizeof(int32_t) * cap);
        active = o;
        o = align256(o + sizeof(int32_t) * cap);
        clear = o;
        o = align256(o + sizeof(FinJob) * cap);
        bytes = o;
    }
};

struct TickSlot {
    cudaStream_t stream = nullptr;
    int64_t seq = -1;  // tick number
    unsigned char *h_in = nullptr, *d_in = nullptr;
    float *h_out = nullptr, *d_out = nullptr;
    unsigned *h_status = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<ReqPtr> members;                         // requests with a segment in the tick
    std::vector<std::pair<ReqPtr, int64_t>> finishing;  // requests finalized by it (out offset)
    std::vector<ReqPtr> stepping;                        // guided requests ending an iteration in it
    int64_t samples = 0;
};

}  // namespace

// Water-filling split of a tick's sample target (see the file comment).
void plan_tick(int n, const int64_t *remaining, int64_t target, int32_t tile, int64_t *chunk) {
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return remaining[a] < remaining[b]; });
    int64_t left = std::max<int64_t>(target, int64_t(tile) * n);
    int k = n;
    for (int i : order) {
        int64_t fair = (left / k + tile - 1) / tile * tile;
        if (fair < tile) fair = tile;
        const int64_t c = std::min(remaining[i], fair);
        chunk[i] = c > 0 ? c : 0;
        left = std::max<int64_t>(left - chunk[i], 0);
        --k;
    }
}

}  // namespace hsr

using namespace hsr;

struct hsr_server {
    hsr_server_config cfg{};
    int device = 0, sm_count = 0;
    int64_t min_tick = 0;      // samples: kTilesPerCta tiles per resident CTA
    cudaEvent_t end_ev[kEndRing] = {};  // end of tick k at k % kEndRing
    int64_t built = 0;         // ticks queued so far
    double *d_arena = nullptr;
    Arena arena;
    // guided serving: one guiding tree per slot, and the free trees
    bool guided = false;
    void *d_guide = nullptr;
    GuideMem guide{};
    std::vector<int> free_trees;
    TickLayout layout;
    TickSlot slots[kTickSlots];
    int64_t out_floats_cap = 0;
    std::map<int, int> blocks_cache;  // N -> k_wave CTAs per SM (mixed form)

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<const SceneDev *> scenes;
    std::deque<ReqPtr> queue;
    std::vector<ReqPtr> active;
    std::unordered_map<uint64_t, ReqPtr> tickets;
    uint64_t next_ticket = 1;
    int64_t ticks_finished = 0;  // written by the host callback
    bool stop = false;
    bool admission_blocked = false;  // the queue head waits for accumulator memory
    double rate = 5.0e5;  // samples per device ms (updated from measured ticks)

    // statistics
    int64_t st_submitted = 0, st_completed = 0, st_failed = 0, st_ticks = 0, st_samples = 0, st_while_busy = 0;
    int64_t st_mem_peak = 0;
    int32_t st_max_batch = 0, st_max_resident = 0;
    double st_device_ms = 0.0;
    std::vector<double> latencies;

    std::thread worker;

    ~hsr_server();
    void run();
    bool build_tick(TickSlot &t, bool busy, int64_t &ticks_launched);
    void complete_tick(TickSlot &t);
    void finish_request(const ReqPtr &q, hsr_status st, Clock::time_point now);
};

namespace {

void CUDART_CB on_tick_done(void *arg) {
    hsr_server *s = static_cast<hsr_server *>(arg);
    // notified under the lock: once the worker has seen this tick, `s` is not touched
    std::lock_guard<std::mutex> lk(s->mu);
    ++s->ticks_finished;
    s->cv_work.notify_all();
}

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

hsr_server::~hsr_server() {
    for (TickSlot &t : slots)
        if (t.stream) cudaStreamSynchronize(t.stream);
    for (cudaEvent_t e : end_ev)
        if (e) cudaEventDestroy(e);
    for (TickSlot &t : slots) {
        if (t.stream) cudaStreamDestroy(t.stream);
        if (t.h_in) cudaFreeHost(t.h_in);
        if (t.h_out) cudaFreeHost(t.h_out);
        if (t.h_status) cudaFreeHost(t.h_status);
        if (t.d_in) cudaFree(t.d_in);
        if (t.d_out) cudaFree(t.d_out);
        if (t.ev0) cudaEventDestroy(t.ev0);
        if (t.ev1) cudaEventDestroy(t.ev1);
    }
    if (d_arena) cudaFree(d_arena);
    if (d_guide) cudaFree(d_guide);
}

// Called with `mu` held.
void hsr_server::finish_request(const ReqPtr &q, hsr_status st, Clock::time_point now) {
    q->done = true;
    q->status = st;
    q->t_done = now;
    if (q->arena_off >= 0) {
        arena.release(q->arena_off, q->arena_bytes);
        q->arena_off = -1;
        admission_blocked = false;
    }
    if (q->guide_slot >= 0) {
        free_trees.push_back(q->guide_slot);
        q->guide_slot = -1;
    }
    active.erase(std::remove(active.begin(), active.end(), q), active.end());
    if (st == HSR_OK) {
        ++st_completed;
        latencies.push_back(ms_between(q->t_submit, now));
    } else {
        ++st_failed;
    }
}

// Builds and queues one tick in slot `t`. Returns false when there is nothing to run.
bool hsr_server::build_tick(TickSlot &t, bool busy, int64_t &ticks_launched) {
    std::vector<ReqPtr> cand;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (stop) return false;
        // admission: FIFO while a slot and accumulator memory are free
        while (!queue.empty() && int(active.size()) < cfg.max_slots) {
            ReqPtr q = queue.front();
            const int64_t bytes = int64_t(align256(sizeof(double) * 2 * size_t(q->r.samples_per_chirp)));
            const int64_t off = arena.alloc(bytes);
            if (off < 0) {
                admission_blocked = true;
                break;
            }
            queue.pop_front();
            q->arena_off = off;
            q->arena_bytes = bytes;
            q->t_admit = Clock::now();
            if (guided) {
                // a free tree always exists: there are as many as slots
                q->guide_slot = free_trees.back();
                free_trees.pop_back();
                q->needs_reset = true;
                q->sched = schedule(q->r.budget, cfg.flags.clearBeforeIteration != 0);
            }
            active.push_back(q);
            if (busy) ++st_while_busy;
        }
        st_max_resident = std::max(st_max_resident, int32_t(active.size()));
        st_mem_peak = std::max(st_mem_peak, arena.used());
        for (const ReqPtr &q : active)
            if (!q->failed && !q->finalize_queued && !q->waiting) cand.push_back(q);
    }
    if (cand.empty()) return false;

    const int n = int(cand.size());
    std::vector<int64_t> remaining(n), chunk(n);
    for (int i = 0; i < n; ++i)
        remaining[i] = guided ? cand[i]->sched[cand[i]->iter].budget - cand[i]->iter_done
                              : cand[i]->r.budget - cand[i]->scheduled;
    const double target = std::min(std::max(rate * double(cfg.tick_ms), double(min_tick)), double(int64_t(1) << 32));
    plan_tick(n, remaining.data(), int64_t(target), kServeTile, chunk.data());
    // work items of this tick: kServeTile samples, or larger (up to kServeMaxTile) when the
    // tick still has kTilesPerCta items per resident CTA at the larger size. A CTA pulls
    // items spaced by the number of CTAs, pose-major, so with many requests in a tick it
    // changes pose (stack drain, row flush) nearly every item; larger items amortise that.
    int64_t tick_samples = 0;
    for (int i = 0; i < n; ++i) tick_samples += chunk[i];
    const int64_t resident_ctas = min_tick / (int64_t(kTilesPerCta) * kServeTile);
    int32_t tick_tile = kServeTile;
    while (tick_tile < kServeMaxTile && tick_samples >= 2 * int64_t(tick_tile) * kTilesPerCta * resident_ctas)
        tick_tile *= 2;

    // fill the tick block: segments in ascending remainder (shortest first)
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return remaining[a] < remaining[b]; });
    unsigned char *h = t.h_in;
    std::memset(h + layout.counters, 0, 256);
    int64_t *tile = reinterpret_cast<int64_t *>(h + layout.tile);
    int64_t *budget = reinterpret_cast<int64_t *>(h + layout.budget);
    int64_t *offset = reinterpret_cast<int64_t *>(h + layout.offset);
    hsr_antenna *tx = reinterpret_cast<hsr_antenna *>(h + layout.tx);
    hsr_antenna *rx = reinterpret_cast<hsr_antenna *>(h + layout.rx);
    PoseJob *jobs = reinterpret_cast<PoseJob *>(h + layout.jobs);
    int64_t *acc_row = reinterpret_cast<int64_t *>(h + layout.acc_row);
    FinJob *fin = reinterpret_cast<FinJob *>(h + layout.fin);
    float *weight = reinterpret_cast<float *>(h + layout.weight);
    int32_t *train = reinterpret_cast<int32_t *>(h + layout.train);
    int32_t *slot = reinterpret_cast<int32_t *>(h + layout.slot);
    int32_t *step_active = reinterpret_cast<int32_t *>(h + layout.active);
    FinJob *clear = reinterpret_cast<FinJob *>(h + layout.clear);
    if (guided) std::memset(step_active, 0, sizeof(int32_t) * size_t(cfg.max_slots));
    std::vector<int> resets;
    t.members.clear();
    t.finishing.clear();
    t.stepping.clear();
    t.samples = 0;
    int P = 0, F = 0, C = 0, maxN = 1;
    // the tick's GENERATE threshold: the smallest of its scenes' tuned thresholds, where a
    // scene never tuned (or tuned to 64 or less) counts as 64
    int32_t queue_threshold = kWaveMaxQueueThreshold;
    // the coherent stage order when every scene in the tick was tuned to it
    bool coherent = true;
    // a tick whose requests share one scene, chirp and N runs the uniform kernel
    bool uniform = true;
    const ReqPtr *first = nullptr;
    int64_t out_off = 0;
    tile[0] = 0;
    for (int i : order) {
        const ReqPtr &q = cand[i];
        if (q->needs_reset) {
            resets.push_back(q->guide_slot);
            q->needs_reset = false;
        }
        const Iter *it = guided ? &q->sched[q->iter] : nullptr;
        if (chunk[i] > 0) {
            tx[P] = q->r.tx;
            rx[P] = q->r.rx;
            budget[P] = chunk[i];
            // guided: the iteration's Halton range (each iteration restarts at the caller's
            // offset when it clears the frame, path.h:212-215) at its sample weight
            offset[P] = q->r.index_offset + (guided ? it->offset + q->iter_done : q->scheduled);
            weight[P] = guided ? it->weight : 1.f;
            train[P] = guided && it->train ? 1 : 0;
            slot[P] = guided ? q->guide_slot : 0;
            PoseJob &j = jobs[P];
            j.nodes = q->scene->nodes;
            j.tris = q->scene->tris;
            j.rf = q->r.rf;
            j.samples = q->r.samples_per_chirp;
            j.reserved = 0;
            j.acc_offset = q->arena_off / int64_t(sizeof(double));
            acc_row[P] = j.acc_offset;
            if (!first) {
                first = &q;
            } else if ((*first)->scene != q->scene || (*first)->r.samples_per_chirp != q->r.samples_per_chirp ||
                       std::memcmp(&(*first)->r.rf, &q->r.rf, sizeof(hsr_rf_config)) != 0) {
                uniform = false;
            }
            tile[P + 1] = tile[P] + (chunk[i] + tick_tile - 1) / tick_tile;
            maxN = std::max(maxN, q->r.samples_per_chirp);
            queue_threshold = std::min(queue_threshold, std::max(q->scene->tuned.queue_threshold, kWaveSmallQueue));
            if (q->scene->tuned.queue_threshold <= kWaveSmallQueue) queue_threshold = kWaveSmallQueue;
            coherent = coherent && q->scene->tuned.coherent_order != 0;
            ++P;
            q->scheduled += chunk[i];
            q->iter_done += chunk[i];
            q->ticks += 1;
            q->in_flight += 1;
            t.members.push_back(q);
            t.samples += chunk[i];
        }
        if (guided && q->iter_done == it->budget && q->iter + 1 < int(q->sched.size())) {
            // the iteration's last chunk: after this tick (and the previous one) the tree is
            // stepped and, when the next iteration starts a fresh frame, the row cleared;
            // the request waits for this tick before it is planned again
            step_active[q->guide_slot] = 1;
            if (q->sched[q->iter + 1].clear)
                clear[C++] = FinJob{q->arena_off / int64_t(sizeof(double)), 0, 0.0, q->r.samples_per_chirp, 0};
            q->waiting = true;
            q->wait_seq = built;
            t.stepping.push_back(q);
            continue;
        }
        if (guided ? q->iter_done == it->budget : q->scheduled == q->r.budget) {
            // the frame's totalWeight: the final iteration's samples at its weight when the
            // frame was cleared before it, else the weighted sum since the start
            double tw = double(q->r.budget);
            if (guided) {
                tw = 0.0;
                for (const Iter &k : q->sched) {
                    if (k.clear) tw = 0.0;
                    tw += double(k.budget) * double(k.weight);
                }
            }
            fin[F] = FinJob{q->arena_off / int64_t(sizeof(double)), out_off, tw, q->r.samples_per_chirp, 0};
            t.finishing.emplace_back(q, out_off);
            out_off += 2 * int64_t(q->r.samples_per_chirp);
            q->finalize_queued = true;
            ++F;
        }
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        st_max_batch = std::max(st_max_batch, P);
    }

    cudaStream_t stream = t.stream;
    cudaError_t e = cudaMemcpyAsync(t.d_in, t.h_in, layout.bytes, cudaMemcpyHostToDevice, stream);
    cudaEventRecord(t.ev0, stream);
    std::string err;
    // newly admitted guided requests start from a fresh tree (GuidingWrapper::reset, path.h:180)
    for (size_t k = 0; e == cudaSuccess && k < resets.size(); ++k) {
        const size_t g = size_t(resets[k]) * kGuideMaxNodes;
        if (launch_guide_reset(1, guide.samp_child + g, guide.samp_p + g, guide.train_child + g,
                               guide.train_acc + 3 * g, guide.train_count + resets[k], stream) != 0)
            e = cudaErrorLaunchFailure;
    }
    if (e == cudaSuccess && P > 0) {
        TraceParams p{};
        p.flags = cfg.flags;
        p.flags.doGuiding = guided ? 1 : 0;
        if (guided) {
            p.do_guide = 1;
            p.train = reinterpret_cast<const int *>(t.d_in + layout.train);
            p.weights = reinterpret_cast<const float *>(t.d_in + layout.weight);
            p.guide_slot = reinterpret_cast<const int32_t *>(t.d_in + layout.slot);
            p.g_samp_child = guide.samp_child;
            p.g_samp_p = guide.samp_p;
            p.g_train_child = guide.train_child;
            p.g_train_acc = guide.train_acc;
        }
        p.samples = maxN;
        p.pose_count = P;
        p.tx = reinterpret_cast<const hsr_antenna *>(t.d_in + layout.tx);
        p.rx = reinterpret_cast<const hsr_antenna *>(t.d_in + layout.rx);
        p.budget = reinterpret_cast<const int64_t *>(t.d_in + layout.budget);
        p.offset = reinterpret_cast<const int64_t *>(t.d_in + layout.offset);
        p.tile_start = reinterpret_cast<const int64_t *>(t.d_in + layout.tile);
        p.sample_weight = 1.f;
        p.tile = tick_tile;
        p.acc = d_arena;
        p.status = reinterpret_cast<unsigned *>(t.d_in + layout.counters);
        p.work_counter = p.status + 2;
        p.jobs = reinterpret_cast<const PoseJob *>(t.d_in + layout.jobs);
        // the path stack and GENERATE threshold of the tick: a larger stack only when every
        // scene in it was autotuned to a threshold above 64 (hsr_autotune_batch);
        // otherwise, and for scenes never tuned, the small stack (the faster one on dense
        // scenes, where it leaves more of the L1 to the BVH)
        p.queue_threshold = queue_threshold;
        p.coherent_order = coherent ? 1 : 0;
        if (uniform) {
            // one scene, chirp and N: the uniform kernel (no per-pose job loads, fewer
            // registers), writing each request's rows through acc_row
            const ReqPtr &q0 = *first;
            p.jobs = nullptr;
            p.nodes = q0->scene->nodes;
            p.tris = q0->scene->tris;
            p.rf = q0->r.rf;
            p.samples = q0->r.samples_per_chirp;
            p.acc_row = reinterpret_cast<const int64_t *>(t.d_in + layout.acc_row);
            p.field_on_hit = q0->scene->tuned.field_on_hit;
            p.coherent_order = q0->scene->tuned.coherent_order;
        }
        auto it = blocks_cache.find(maxN);
        if (it == blocks_cache.end()) it = blocks_cache.emplace(maxN, wave_blocks_per_sm(maxN, true, guided)).first;
        if (launch_wave(p, cfg.phase_mode, sm_count * it->second, stream, err) != 0) e = cudaErrorLaunchFailure;
    }
    // requests span ticks: everything after this point waits for the previous tick
    if (e == cudaSuccess && built > 0) e = cudaStreamWaitEvent(stream, end_ev[(built - 1) % kEndRing], 0);
    // guided iterations that ended here: clear the rows the next iteration starts afresh,
    // then step the trees (every chunk of the iteration has run: this tick and the last)
    if (e == cudaSuccess && C > 0) {
        k_serve_clear<<<C, 256, 0, stream>>>(reinterpret_cast<const FinJob *>(t.d_in + layout.clear), d_arena);
        note_launches(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && !t.stepping.empty() &&
        launch_guide_step(cfg.max_slots, reinterpret_cast<const int *>(t.d_in + layout.active), guide.samp_child,
                          guide.samp_p, guide.train_child, guide.train_acc, guide.train_count, stream) != 0)
        e = cudaErrorLaunchFailure;
    if (e == cudaSuccess && F > 0) {
        k_serve_finalize<<<F, 256, 0, stream>>>(reinterpret_cast<const FinJob *>(t.d_in + layout.fin), d_arena,
                                                t.d_out);
        note_launches(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(t.h_status, t.d_in + layout.counters, 256, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess && out_off > 0)
        e = cudaMemcpyAsync(t.h_out, t.d_out, sizeof(float) * out_off, cudaMemcpyDeviceToHost, stream);
    cudaEventRecord(t.ev1, stream);
    cudaEventRecord(end_ev[built % kEndRing], stream);
    if (e == cudaSuccess) e = cudaLaunchHostFunc(stream, on_tick_done, this);
    if (e != cudaSuccess) {
        // the tick could not be queued: fail its requests once nothing of theirs runs
        cudaGetLastError();
        for (TickSlot &o : slots) cudaStreamSynchronize(o.stream);
        std::lock_guard<std::mutex> lk(mu);
        set_last_error(err.empty() ? std::string("serving tick: ") + cudaGetErrorString(e) : err);
        const Clock::time_point now = Clock::now();
        for (const ReqPtr &q : t.members) q->in_flight -= 1;
        for (const ReqPtr &q : t.members) q->failed = true;
        for (auto &fo : t.finishing) fo.first->failed = true;  // includes zero-budget requests
        for (const ReqPtr &q : t.stepping) q->failed = true;
        std::vector<ReqPtr> gone;
        for (const ReqPtr &q : active)
            if (q->failed && q->in_flight == 0 && !q->done) gone.push_back(q);
        for (const ReqPtr &q : gone) {
            if (q->arena_off >= 0) cudaMemset(d_arena + q->arena_off / 8, 0, q->arena_bytes);
            finish_request(q, HSR_ERR_CUDA, now);
        }
        t.members.clear();
        t.finishing.clear();
        t.stepping.clear();
        cv_done.notify_all();
        return false;
    }
    t.seq = built++;
    ++ticks_launched;
    return true;
}

// After the tick's host callback ran: hand out finished rows, update statistics.
void hsr_server::complete_tick(TickSlot &t) {
    // device time this tick adds to the busy union: from the later of its start and the
    // previous tick's end
    float ms = 0.f, gap = 0.f;
    cudaEventElapsedTime(&ms, t.ev0, t.ev1);
    if (t.seq > 0 && cudaEventElapsedTime(&gap, end_ev[(t.seq - 1) % kEndRing], t.ev0) == cudaSuccess && gap < 0.f)
        ms = std::max(0.f, ms + gap);
    cudaGetLastError();
    const unsigned status = t.h_status[0];
    if (status == 0)
        for (auto &fo : t.finishing)
            std::memcpy(fo.first->r.out_row, t.h_out + fo.second,
                        sizeof(float) * 2 * size_t(fo.first->r.samples_per_chirp));
    {
        std::lock_guard<std::mutex> lk(mu);
        const Clock::time_point now = Clock::now();
        for (const ReqPtr &q : t.members) q->in_flight -= 1;
        if (status != 0) {
            set_last_error("serving tick: device status word " + std::to_string(status));
            for (const ReqPtr &q : t.members) q->failed = true;
            for (auto &fo : t.finishing) fo.first->failed = true;
        }
        for (auto &fo : t.finishing)
            if (!fo.first->done && !fo.first->failed) finish_request(fo.first, HSR_OK, now);
        // guided requests whose iteration ended in this tick: its step has run, so the next
        // iteration may be planned
        for (const ReqPtr &q : t.stepping) {
            if (status != 0) q->failed = true;
            q->iter += 1;
            q->iter_done = 0;
            q->waiting = false;
        }
        // failed requests release their accumulators once no queued tick uses them
        std::vector<ReqPtr> failed;
        for (const ReqPtr &q : active)
            if (q->failed && q->in_flight == 0 && !q->done) failed.push_back(q);
        for (const ReqPtr &q : failed) {
            if (q->arena_off >= 0) cudaMemsetAsync(d_arena + q->arena_off / 8, 0, q->arena_bytes, t.stream);
            finish_request(q, HSR_ERR_DEVICE, now);
        }
        ++st_ticks;
        st_samples += t.samples;
        st_device_ms += ms;
        if (ms > 0.05f && t.samples > 0) rate = 0.5 * rate + 0.5 * double(t.samples) / double(ms);
    }
    t.members.clear();
    t.finishing.clear();
    t.stepping.clear();
    cv_done.notify_all();
}

void hsr_server::run() {
    cudaSetDevice(device);
    std::deque<int> inflight;  // tick slots on the device, oldest first
    int next = 0;
    int64_t launched = 0, completed = 0;
    while (true) {
        // hand out ticks whose callback has run (they finish in order)
        int64_t finished;
        {
            std::lock_guard<std::mutex> lk(mu);
            finished = ticks_finished;
        }
        while (completed < finished && !inflight.empty()) {
            complete_tick(slots[inflight.front()]);
            inflight.pop_front();
            ++completed;
        }
        if (int(inflight.size()) < kTickSlots && build_tick(slots[next], !inflight.empty(), launched)) {
            inflight.push_back(next);
            next = (next + 1) % kTickSlots;
            continue;
        }
        std::unique_lock<std::mutex> lk(mu);
        if (stop && inflight.empty()) break;
        // sleep until a tick finishes, a request arrives, or the server stops
        cv_work.wait(lk, [&] {
            if (ticks_finished > completed) return true;
            if (stop) return inflight.empty();
            if (int(inflight.size()) >= kTickSlots) return false;
            if (!queue.empty() && int(active.size()) < cfg.max_slots && !admission_blocked) return true;
            for (const ReqPtr &q : active)
                if (!q->failed && !q->finalize_queued && !q->waiting) return true;
            return false;
        });
        if (stop && inflight.empty() && ticks_finished == completed) break;
    }
    // stopping: fail what did not finish
    std::lock_guard<std::mutex> lk(mu);
    const Clock::time_point now = Clock::now();
    std::vector<ReqPtr> left(active.begin(), active.end());
    for (const ReqPtr &q : left)
        if (!q->done) finish_request(q, HSR_ERR_INTERRUPTED, now);
    for (const ReqPtr &q : queue) {
        q->done = true;
        q->status = HSR_ERR_INTERRUPTED;
        q->t_done = now;
        ++st_failed;
    }
    queue.clear();
    cv_done.notify_all();
}

namespace {

hsr_status serve_fail(hsr_status s, const std::string &msg) {
    set_last_error(msg);
    return s;
}

}  // namespace

extern "C" {

void hsr_default_server_config(hsr_server_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->max_slots = 256;
    c->max_samples_per_chirp = 1024;
    c->memory_bytes = int64_t(64) << 20;
    c->tick_ms = 4.f;
    c->phase_mode = HSR_PHASE_REFERENCE_FP32;
    hsr_default_flags(&c->flags);
    c->flags.doGuiding = 0;
}

hsr_status hsr_debug_plan_tick(int32_t count, const int64_t *remaining, int64_t target, int32_t tile,
                               int64_t *out_chunk) {
    if (count < 0 || (count > 0 && (!remaining || !out_chunk)) || tile <= 0)
        return serve_fail(HSR_ERR_INVALID_ARGUMENT, "bad tick plan arguments");
    for (int i = 0; i < count; ++i)
        if (remaining[i] < 0) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "negative remainder");
    plan_tick(count, remaining, target, tile, out_chunk);
    return HSR_OK;
}

hsr_status hsr_server_create(const hsr_server_config *cfg, hsr_server **out) {
    if (!cfg || !out) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (cfg->max_slots < 1 || cfg->max_slots > 4096)
        return serve_fail(HSR_ERR_INVALID_ARGUMENT, "max_slots must be in [1, 4096]");
    if (cfg->max_samples_per_chirp < 1 || cfg->max_samples_per_chirp > 4096)
        return serve_fail(HSR_ERR_INVALID_ARGUMENT, "max_samples_per_chirp must be in [1, 4096]");
    if (cfg->memory_bytes < 256) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "memory_bytes must be >= 256");
    if (!(cfg->tick_ms > 0.f)) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "tick_ms must be > 0");
    if (cfg->phase_mode != HSR_PHASE_REFERENCE_FP32 && cfg->phase_mode != HSR_PHASE_SPLIT_FP64)
        return serve_fail(HSR_ERR_INVALID_ARGUMENT, "unknown phase mode");
    if (!cfg->flags.useGeometricalOptics)
        return serve_fail(HSR_ERR_NOT_SUPPORTED, "the server traces geometrical optics");
    if (cfg->flags.maxDepth < 0) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "maxDepth must be >= 0");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return serve_fail(HSR_ERR_NO_DEVICE, "no CUDA device is visible");
    }
    std::unique_ptr<hsr_server> s(new hsr_server());
    s->cfg = *cfg;
    s->cfg.memory_bytes = int64_t(align256(size_t(cfg->memory_bytes)));
    cudaGetDevice(&s->device);
    cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
    std::string err;
    cudaError_t e = cudaSuccess;
    for (TickSlot &t : s->slots)
        if ((e = cudaStreamCreateWithFlags(&t.stream, cudaStreamNonBlocking)) != cudaSuccess)
            return serve_fail(HSR_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e));
    for (cudaEvent_t &ev : s->end_ev)
        if (cudaEventCreate(&ev) != cudaSuccess) {
            cudaGetLastError();
            return serve_fail(HSR_ERR_CUDA, "tick end events");
        }
    s->guided = cfg->flags.doGuiding != 0;
    s->min_tick = int64_t(kTilesPerCta) * kServeTile * s->sm_count *
                  wave_blocks_per_sm(cfg->max_samples_per_chirp, true, s->guided);
    if (!dev_alloc(&s->d_arena, size_t(s->cfg.memory_bytes), err)) return serve_fail(HSR_ERR_OUT_OF_MEMORY, err);
    if (s->guided) {
        if (!dev_alloc(&s->d_guide, guide_bytes_per_pose() * size_t(cfg->max_slots) + 8 * 256, err))
            return serve_fail(HSR_ERR_OUT_OF_MEMORY, "guiding trees: " + err);
        s->guide = carve_guide(s->d_guide, cfg->max_slots);
        for (int k = cfg->max_slots - 1; k >= 0; --k) s->free_trees.push_back(k);
    }
    if ((e = cudaMemset(s->d_arena, 0, size_t(s->cfg.memory_bytes))) != cudaSuccess)
        return serve_fail(HSR_ERR_CUDA, std::string("arena clear: ") + cudaGetErrorString(e));
    s->arena.init(s->cfg.memory_bytes);
    s->layout.init(cfg->max_slots);
    s->out_floats_cap = 2 * int64_t(cfg->max_slots) * cfg->max_samples_per_chirp;
    for (TickSlot &t : s->slots) {
        if (cudaMallocHost(reinterpret_cast<void **>(&t.h_in), s->layout.bytes) != cudaSuccess ||
            cudaMallocHost(reinterpret_cast<void **>(&t.h_out), sizeof(float) * s->out_floats_cap) != cudaSuccess ||
            cudaMallocHost(reinterpret_cast<void **>(&t.h_status), 256) != cudaSuccess) {
            cudaGetLastError();
            return serve_fail(HSR_ERR_OUT_OF_MEMORY, "pinned host buffers for the tick slots");
        }
        if (!dev_alloc(&t.d_in, s->layout.bytes, err) ||
            !dev_alloc(&t.d_out, sizeof(float) * size_t(s->out_floats_cap), err))
            return serve_fail(HSR_ERR_OUT_OF_MEMORY, err);
        if (cudaEventCreate(&t.ev0) != cudaSuccess || cudaEventCreate(&t.ev1) != cudaSuccess) {
            cudaGetLastError();
            return serve_fail(HSR_ERR_CUDA, "tick events");
        }
    }
    hsr_server *raw = s.release();
    raw->worker = std::thread([raw] { raw->run(); });
    *out = raw;
    return HSR_OK;
}

hsr_status hsr_server_add_scene(hsr_server *s, hsr_scene *scene, int32_t *out_id) {
    const SceneDev *sd = scene_device_state(scene);
    if (!s || !sd || !out_id) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    if (sd->device != s->device) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "scene lives on another device");
    std::lock_guard<std::mutex> lk(s->mu);
    s->scenes.push_back(sd);
    *out_id = int32_t(s->scenes.size() - 1);
    return HSR_OK;
}

hsr_status hsr_server_submit(hsr_server *s, const hsr_request *r, uint64_t *out_ticket) {
    if (!s || !r || !out_ticket) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    if (!r->out_row) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "out_row is null");
    if (r->samples_per_chirp < 1 || r->samples_per_chirp > s->cfg.max_samples_per_chirp)
        return serve_fail(HSR_ERR_INVALID_ARGUMENT, "samples_per_chirp outside [1, max_samples_per_chirp]");
    if (r->budget < 0 || r->index_offset < 0)
        return serve_fail(HSR_ERR_INVALID_ARGUMENT, "budget and index_offset must be >= 0");
    if (!(r->rf.adcRate > 0.f) || !std::isfinite(r->rf.startFreq) || !std::isfinite(r->rf.freqSlope))
        return serve_fail(HSR_ERR_INVALID_ARGUMENT, "bad RF configuration");
    if (int64_t(align256(sizeof(double) * 2 * size_t(r->samples_per_chirp))) > s->cfg.memory_bytes)
        return serve_fail(HSR_ERR_INVALID_ARGUMENT, "the request's accumulators exceed the server's memory");
    auto q = std::make_shared<Req>();
    q->r = *r;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return serve_fail(HSR_ERR_INTERRUPTED, "server is stopping");
        if (r->scene < 0 || r->scene >= int32_t(s->scenes.size()))
            return serve_fail(HSR_ERR_INVALID_ARGUMENT, "unknown scene id");
        q->scene = s->scenes[r->scene];
        q->ticket = s->next_ticket++;
        q->t_submit = Clock::now();
        s->queue.push_back(q);
        s->tickets[q->ticket] = q;
        ++s->st_submitted;
        *out_ticket = q->ticket;
    }
    s->cv_work.notify_all();
    return HSR_OK;
}

hsr_status hsr_server_wait(hsr_server *s, uint64_t ticket, int32_t timeout_ms, hsr_request_result *out) {
    if (!s) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "unknown ticket");
    ReqPtr q = it->second;
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, [&] { return q->done; });
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return q->done; })) {
        return HSR_ERR_TIMEOUT;
    }
    if (out) {
        out->status = q->status;
        out->ticks = q->ticks;
        out->queue_ms = q->t_admit.time_since_epoch().count() ? ms_between(q->t_submit, q->t_admit) : 0.0;
        out->latency_ms = ms_between(q->t_submit, q->t_done);
    }
    s->tickets.erase(ticket);
    return HSR_OK;
}

hsr_status hsr_server_get_stats(hsr_server *s, hsr_server_stats *o) {
    if (!s || !o) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(o, 0, sizeof(*o));
    o->submitted = s->st_submitted;
    o->completed = s->st_completed;
    o->failed = s->st_failed;
    o->ticks = s->st_ticks;
    o->samples = s->st_samples;
    o->device_ms = s->st_device_ms;
    o->max_batch = s->st_max_batch;
    o->max_resident = s->st_max_resident;
    o->admitted_while_busy = s->st_while_busy;
    o->memory_bytes_peak = s->st_mem_peak;
    for (const SceneDev *sd : s->scenes)
        o->scene_bytes += sd->tri_count * int64_t(sizeof(DTri) + 3 * sizeof(int32_t)) +
                          sd->node_count * int64_t(sizeof(DNode));
    if (!s->latencies.empty()) {
        std::vector<double> v = s->latencies;
        auto pct = [&](double q) {
            const size_t k = std::min(v.size() - 1, size_t(std::ceil(q * double(v.size()))) - (q > 0 ? 1 : 0));
            std::nth_element(v.begin(), v.begin() + k, v.end());
            return v[k];
        };
        o->p50_ms = pct(0.50);
        o->p99_ms = pct(0.99);
        o->max_ms = *std::max_element(v.begin(), v.end());
    }
    return HSR_OK;
}

hsr_status hsr_server_reset_stats(hsr_server *s) {
    if (!s) return serve_fail(HSR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    s->st_submitted = s->st_completed = s->st_failed = s->st_ticks = s->st_samples = s->st_while_busy = 0;
    s->st_mem_peak = s->arena.used();
    s->st_max_batch = 0;
    s->st_max_resident = int32_t(s->active.size());
    s->st_device_ms = 0.0;
    s->latencies.clear();
    return HSR_OK;
}

hsr_status hsr_server_destroy(hsr_server *s) {
    if (!s) return HSR_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    delete s;
    return HSR_OK;
}

}  // extern "C"
