/*
 * hsr_gb300.h — C ABI of the GB300 radar path-tracing backend.
 *
 * This library replaces libhussar's two ray-tracing backends:
 *   - cpu::Backend (Embree), libhussar/include/hussar/arch/cpu.h:17-63, src/arch/cpu.cpp:32-87
 *   - gpu::Backend (OptiX),  libhussar/include/hussar/arch/gpu.h:17-47, src/arch/gpu.cpp:482-532
 * together with the integrator they run, PathTracer::sample
 * (libhussar/include/hussar/integrators/path.h:235-451), and the frame splat it feeds
 * (libradar/include/radar/radar.h:564-626).
 *
 * Everything is plain C: POD structs, pointers and sizes. No exceptions cross this
 * boundary; every call returns an hsr_status and hsr_last_error() gives the message
 * of the last failure on the calling thread. The reference reports the same failures
 * by throwing sutil::Exception (src/arch/gpu/host/sutil/Exception.h:91-191) or by
 * Log(EError) + exit(-1) (core/logging.h:43-46).
 *
 * Device: one NVIDIA GB300 (sm_103a). There is no CPU fallback: without a usable GPU
 * every entry point that computes returns HSR_ERR_NO_DEVICE.
 */
#ifndef HSR_GB300_H
#define HSR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HSR_ABI_VERSION 5

typedef enum hsr_status {
    HSR_OK = 0,
    HSR_ERR_INVALID_ARGUMENT = 1,  /* bad pointer, size or configuration */
    HSR_ERR_CUDA = 2,              /* a CUDA runtime call failed */
    HSR_ERR_OUT_OF_MEMORY = 3,     /* device allocation failed */
    HSR_ERR_INTERRUPTED = 4,       /* the caller's interrupt flag was set */
    HSR_ERR_DEVICE = 5,            /* a kernel reported an error in its device status word */
    HSR_ERR_NOT_SUPPORTED = 6,     /* a flag combination this backend does not implement */
    HSR_ERR_NO_DEVICE = 7,         /* no CUDA device is visible */
    HSR_ERR_TIMEOUT = 8            /* a served request has not finished within the wait */
} hsr_status;

/* FMCW ramp parameters; field-for-field radar::RFConfig (libradar/include/radar/radar.h:113-136).
 * Units: Hz, Hz/s, Hz, s, s, s. */
typedef struct hsr_rf_config {
    float startFreq;
    float freqSlope;
    float adcRate;
    float idleTime;
    float rampTime;
    float antennaDelay;
} hsr_rf_config;

/* Radar cube shape; radar::FrameConfig (libradar/include/radar/radar.h:141-164).
 * The cube is stored [chirp][sample][channel] (radar.h:487-494). */
typedef struct hsr_frame_config {
    int32_t chirpCount;
    int32_t samplesPerChirp;
    int32_t channelCount;
} hsr_frame_config;

/* A point antenna with the AWR1243 radiation pattern; hussar::NFAntenna
 * (libhussar/include/hussar/core/emitter.h:159-214). rotation is the 3x3 matrix
 * m_rotation in row-major order (rotation[3*row + col]); its third column is the
 * boresight direction. */
typedef struct hsr_antenna {
    float position[3];
    float rotation[9];
} hsr_antenna;

/* FFAntenna (libhussar/include/hussar/core/emitter.h:218-291): a far-field antenna, a plane
 * wave in the reference's terms. It is a disk of `radius` centred at
 * scene_center + direction * radius, facing the scene: as a transmitter it launches rays
 * along -direction from a uniformly sampled point of the disk's square (2u - 1, 2v - 1 in
 * the frame of buildFrame(-direction), geometry.h:45-53) with H = polarization / pdf,
 * pdf = 1 / (4 radius^2); as a receiver it is reached from a hit point p along
 * +direction over the distance to the disk's plane, with H = polarization * 4 pi * that
 * distance, and only while p projects within 1 (not `radius`, as the reference tests)
 * of the disk's centre. `direction` must be normalised and `polarization` orthogonal
 * to it (complex, re/im per axis). */
typedef struct hsr_ff_antenna {
    float direction[3];
    float polarization[6];
    float scene_center[3];
    float radius;
} hsr_ff_antenna;

/* PathTracer's public configuration members (libhussar/include/hussar/integrators/path.h:153-169)
 * plus Integrator::produceDebugImage (core/integrator.h:58), which in the reference also
 * turns off the zero-contribution early-out of Integrator::splat (integrator.h:121-124).
 * Booleans are 0/1. */
typedef struct hsr_tracer_flags {
    int32_t onlyIndirect;
    int32_t maxDepth;
    int32_t useGeometricalOptics;
    int32_t poDiffraction;
    int32_t doGuiding;
    int32_t clearBeforeIteration;
    int32_t correctPhase;
    int32_t filterGuiding;
    int32_t doFiltering;
    int32_t filteringSphere;
    int32_t produceDebugImage;
    float filteringMin;
    float filteringMax;
    float filteringRadius;
} hsr_tracer_flags;

/* How the path phase and range bin are evaluated.
 *  HSR_PHASE_REFERENCE_FP32: the reference's own single-precision expression
 *      2*Pi*(f0 - dt*S/2)*dt (core/integrator.h:107-110) and bin N*frac(dt*S/adcRate)
 *      (radar.h:232-241). This is the parity mode.
 *  HSR_PHASE_SPLIT_FP64: the path length is carried in FP64; phase cycles and bin are
 *      reduced modulo one in FP64, the trig is FP32. */
typedef enum hsr_phase_mode {
    HSR_PHASE_REFERENCE_FP32 = 0,
    HSR_PHASE_SPLIT_FP64 = 1
} hsr_phase_mode;

/* How each next-event contribution reaches the range bins.
 *  HSR_SPLAT_DIRICHLET16: radar::Frame::splat<16> (radar.h:564-626): 33 bins of the
 *      truncated sinc kernel per contribution. This is the parity mode.
 *  HSR_SPLAT_FINE_SYNTH: contributions go to a fine complex range histogram with
 *      moment correction; a complex histogram x twiddle GEMM on the tensor cores then
 *      synthesises the exact (untruncated) spectrum. */
typedef enum hsr_splat_mode {
    HSR_SPLAT_DIRICHLET16 = 0,
    HSR_SPLAT_FINE_SYNTH = 1
} hsr_splat_mode;

typedef struct hsr_scene hsr_scene;   /* resident triangle mesh + device BVH */

/* Library / device information. */
int32_t hsr_abi_version(void);
const char *hsr_last_error(void);
/* Number of kernel launches this library has issued in the calling process. */
int64_t hsr_launch_count(void);
/* Device allocations (cudaMalloc) the library has made so far in this process: scenes,
 * scratch, operands, graphs. No counterpart in the reference; lets a caller check that a
 * call allocated nothing. */
int64_t hsr_debug_alloc_count(void);

/* Fills default PathTracer flags exactly as the reference initialises them
 * (path.h:153-169: onlyIndirect=1, maxDepth=10, useGeometricalOptics=1,
 * poDiffraction=0, doGuiding=1, clearBeforeIteration=1, correctPhase=0,
 * filterGuiding=1, doFiltering=1, filteringSphere=1, filteringMin=600,
 * filteringMax=900, filteringRadius=160; produceDebugImage=0). */
void hsr_default_flags(hsr_tracer_flags *flags);

/* Builds a resident scene from a triangle mesh: the device BVH is built once here.
 * Replaces the Backend constructors Backend(const TriangleMesh&, Integrator&)
 * (arch/cpu.h:18-20 -> src/arch/cpu.cpp:32-47 rtcCommitScene; arch/gpu.h:18-20 ->
 * src/arch/gpu.cpp:482-493 buildMeshAccel). vertices: vertex_count x 3 floats
 * (TriangleMesh::vertexBuffer, core/mesh.h:27); indices: triangle_count x 3 int32
 * (TriangleMesh::indexBuffer, core/mesh.h:28). The caller's arrays may be freed after
 * the call returns (the reference copies them too, src/arch/cpu.cpp:36-40). */
hsr_status hsr_scene_create(const float *vertices, int64_t vertex_count,
                            const int32_t *indices, int64_t triangle_count,
                            hsr_scene **out_scene);
hsr_status hsr_scene_destroy(hsr_scene *scene);

/* Scene changes for resident scenes (the serving pool keeps scene handles): the
 * reference builds its Embree scene or OptiX acceleration structure once per Backend
 * (src/arch/cpu.cpp:32-47, src/arch/gpu.cpp:482-493) and has no update.
 * hsr_scene_refit: new positions for the scene's vertices (the same count; the triangles
 *   keep their vertex indices): the triangle records are rewritten and every BVH box is
 *   refitted bottom-up over the existing tree (ray-query answers are exact whatever the
 *   tree; a tree refitted after large motions only traverses more slowly).
 * hsr_scene_rebuild: a new mesh under the same handle (a full build, then swapped in);
 *   refused (HSR_ERR_INVALID_ARGUMENT) while batch graphs captured on the scene exist,
 *   since they hold the old BVH's device addresses.
 * Both wait for the device first, and must not overlap a call or a serving tick that
 * uses the scene. */
hsr_status hsr_scene_refit(hsr_scene *scene, const float *vertices, int64_t vertex_count);
hsr_status hsr_scene_rebuild(hsr_scene *scene, const float *vertices, int64_t vertex_count,
                             const int32_t *indices, int64_t triangle_count);
/* Device bytes held by the scene (triangle records and vertex indices, BVH nodes). */
hsr_status hsr_scene_footprint(const hsr_scene *scene, int64_t *out_bytes);
/* BVH statistics for tests: internal node count, maximum depth, triangle count. */
hsr_status hsr_scene_bvh_stats(const hsr_scene *scene, int64_t *out_nodes,
                               int32_t *out_max_depth, int64_t *out_leaves);

/* Closest-hit and occlusion queries over a batch of rays (host arrays), the two RT
 * callbacks of the reference backends: RT::intersect (src/arch/cpu.cpp:63-87,
 * src/arch/gpu/device/kernel.cu:45-63,76-98) and RT::visible (cpu.cpp:53-61,
 * kernel.cu:24-43). Rays start at tnear = 5e-5 (hussar.h:52, cpu.cpp:12).
 * origins/directions: count x 3 floats; tfar: count floats.
 * Outputs: t (inf on miss), hit point p (count x 3), faceforwarded unit normal n
 * (count x 3), primitive id (-1 on miss) / visible flags (1 = unoccluded). */
hsr_status hsr_intersect(const hsr_scene *scene, int64_t count, const float *origins,
                         const float *directions, const float *tfar, float *out_t,
                         float *out_p, float *out_n, int32_t *out_prim);
hsr_status hsr_visible(const hsr_scene *scene, int64_t count, const float *origins,
                       const float *directions, const float *tfar, int32_t *out_visible);

/* One Backend::run call (arch/cpu.h:44-46, arch/gpu.h:26-32) for the plain (unguided)
 * PathTracer: traces samples index_offset + [0, budget) of the Halton sequence
 * (path.h:237-238) and ADDS each sample's splats, scaled by sample_weight
 * (PathTracer::currentSampleWeight, path.h:242), into frame_inout, and
 * budget*sample_weight into *total_weight_inout (path.h:445, 466-475).
 * frame_inout: host array of chirpCount*samplesPerChirp*channelCount complex64
 * values, interleaved (re, im), layout [chirp][sample][channel].
 * interrupt_flag: optional; when it is non-zero at entry the call returns
 * HSR_ERR_INTERRUPTED without work (the reference polls it per 256-sample batch,
 * arch/cpu.h:25). Synchronous. doGuiding must be 0 here (use hsr_path_tracer_run). */
hsr_status hsr_backend_run(const hsr_scene *scene, const hsr_rf_config *rf,
                           const hsr_frame_config *frame, const hsr_antenna *tx,
                           const hsr_antenna *rx, const hsr_tracer_flags *flags,
                           int64_t budget, int64_t index_offset, float sample_weight,
                           int32_t phase_mode, float *frame_inout,
                           double *total_weight_inout, const volatile int32_t *interrupt_flag);

/* The guiding tree of one pose (GuidingWrapper, path.h:17-131: the 10 % uniform / 90 %
 * tree mixture over the primary sample square, split threshold 0.005, second moment,
 * path.h:229-232) on the device, for callers that run PathTracer::run's schedule
 * themselves (a C++ PathTracer calling its backend once per iteration): create it on
 * the scene, reset it at the start of a schedule (GuidingWrapper::reset, path.h:47-50),
 * run each iteration with hsr_backend_run_guided, and step it between iterations
 * (GuidingWrapper::step, path.h:116-124: build, copy to the sampling tree, refine). The
 * tree is this library's own (libguiding is not part of the reference sources). */
typedef struct hsr_guide hsr_guide;
hsr_status hsr_guide_create(hsr_scene *scene, hsr_guide **out_guide);
hsr_status hsr_guide_reset(hsr_guide *guide);
hsr_status hsr_guide_step(hsr_guide *guide);
hsr_status hsr_guide_destroy(hsr_guide *guide);

/* The guide's tree as host arrays of HSR_GUIDE_MAX_NODES entries: the sampling tree
 * (index of a node's first child, whose pair is (c, c + 1), -1 for a leaf; probability
 * of the first child) and the training tree (child links; per node the sum of w d^2 that
 * GuidingWrapper::splat adds, path.h:96-111). Read returns the training tree's node
 * count; write replaces the state (links must point past their node and stay inside the
 * arrays). For inspection, warm starts, and checks against a CPU restatement of the
 * tree. Synchronous (they wait for the device). */
#define HSR_GUIDE_MAX_NODES 2048
hsr_status hsr_guide_read(hsr_guide *guide, int32_t *out_count, int32_t *samp_child, float *samp_p,
                          int32_t *train_child, float *train_acc2);
hsr_status hsr_guide_write(hsr_guide *guide, int32_t count, const int32_t *samp_child, const float *samp_p,
                           const int32_t *train_child, const float *train_acc2);

/* One guided iteration of PathTracer::run (path.h:186-224): as hsr_backend_run, with each
 * sample's primary direction drawn from the guide's sampling tree (GuidingWrapper::sample,
 * path.h:265-270) and, when `train` is non-zero (every iteration but the final one,
 * path.h:448-450), |guidingWeight| * pdf splatted into its training tree. The flags'
 * doGuiding is ignored (this call is guided). Synchronous. */
hsr_status hsr_backend_run_guided(hsr_scene *scene, const hsr_rf_config *rf, const hsr_frame_config *frame,
                                  const hsr_antenna *tx, const hsr_antenna *rx, const hsr_tracer_flags *flags,
                                  int64_t budget, int64_t index_offset, float sample_weight, int32_t train,
                                  hsr_guide *guide, int32_t phase_mode, float *frame_inout,
                                  double *total_weight_inout, const volatile int32_t *interrupt_flag);

/* PathTracer::run (path.h:171-224) for one pose, guided or plain: clears the frame,
 * then (doGuiding = 0) one backend run over Halton indices [0, samples), or (doGuiding =
 * 1) the doubling schedule from 16384 samples with device path guiding of the primary
 * sample square (GuidingWrapper, path.h:17-131, settings path.h:229-232) trained on
 * every iteration but the final one, clearing the frame between iterations when
 * clearBeforeIteration is set (else weighting later samples 10x, path.h:212-220).
 * Outputs the frame's raw sums (host, complex64 [chirp][sample][channel], overwritten)
 * and its total weight; fetchFrame() is frame_out / *total_weight_out. The guided
 * estimator is the reference's; its tree (a 2-D adaptive binary tree with the same
 * uniform mixture, split threshold and second-moment criterion) is this library's own,
 * libguiding not being part of the reference sources. */
hsr_status hsr_path_tracer_run(hsr_scene *scene, const hsr_rf_config *rf,
                               const hsr_frame_config *frame, const hsr_antenna *tx,
                               const hsr_antenna *rx, const hsr_tracer_flags *flags,
                               int64_t samples, int32_t phase_mode, float *frame_out,
                               double *total_weight_out, const volatile int32_t *interrupt_flag);

/* Batched simulation: pose_count independent sensor poses (tx[i], rx[i]) with their
 * own sample budgets, all traced by ONE persistent launch on `stream`
 * (a cudaStream_t, or NULL for the legacy default stream).
 * Each pose p traces Halton indices index_offset[p] + [0, budget[p]).
 * Output (DEVICE pointer): out_rows[p*samplesPerChirp + k] = the normalised
 * frame row (chirp 0, channel 0) of pose p, i.e. fetchFrame() (path.h:453-455)
 * restricted to the only row the reference writes (velocity 0, path.h:130; one RX
 * channel, path.h:291-292); complex64 interleaved.
 * All pointer arguments are DEVICE pointers (inputs already resident). Asynchronous
 * on `stream`; scratch is owned by the scene and reused across calls on it, so calls
 * on one scene must not overlap. With flags->doGuiding every pose runs the guided
 * schedule of hsr_path_tracer_run (its own tree); the schedule is planned on the host,
 * so that form reads the budgets back and synchronises between iterations. */
hsr_status hsr_simulate_batch_device(hsr_scene *scene, const hsr_rf_config *rf,
                                     int32_t samples_per_chirp, const hsr_tracer_flags *flags,
                                     int32_t pose_count, const hsr_antenna *d_tx,
                                     const hsr_antenna *d_rx, const int64_t *d_budget,
                                     const int64_t *d_index_offset, int32_t phase_mode,
                                     int32_t splat_mode, float *d_out_rows, void *stream);

/* WavefrontFile::read (io/wavefront.h:12-67): the vertices and triangles of an OBJ file,
 * for hsr_scene_create. 'v x y z' lines give vertices, 'f a b c' lines triangles from the
 * first three 1-based vertex indices (an 'a/b/c' token's vertex index is the number
 * before the first '/'; the reference's `>> int` parse stops there and fails the rest of
 * the file), written as 0-based indices shifted by vertex_offset (the vertices the
 * caller's mesh already holds, wavefront.h:23, 42-48); '#' comment lines, 's' and empty
 * lines are skipped, other commands are counted in *out_unsupported (may be NULL) and
 * skipped. Call with vertices = indices = NULL for the counts, then with buffers of
 * 3 * vertex count floats and 3 * triangle count ints. Host only (no device needed). */
hsr_status hsr_read_obj(const char *path, int64_t vertex_offset, float *vertices, int64_t vertex_capacity,
                        int32_t *indices, int64_t triangle_capacity, int64_t *out_vertex_count,
                        int64_t *out_triangle_count, int64_t *out_unsupported);

/* Device status of the last call on this scene: synchronises `stream` (the stream that
 * call ran on) and reads the status word that call's kernels set, into *out_bits (may be
 * NULL): traversal stack overflow (bit 0), a bin out of range (bit 1), a bad work item
 * (bit 2), a synthesis wait that gave up (bit 3). Returns HSR_ERR_DEVICE with the bits
 * named in hsr_last_error() when any is set. The synchronous entry points report their
 * own status on return; hsr_simulate_batch_device returns before the GPU has run, so its
 * status is read here. Every call on a scene starts with a clear word, so read it before
 * the next call on the scene. The reference throws on device errors from its synchronous
 * launch (sutil::Exception, Exception.h:91-191); this is the asynchronous counterpart. */
hsr_status hsr_scene_status(hsr_scene *scene, void *stream, uint32_t *out_bits);

/* A MIMO radar frame: tx_count x rx_count virtual channels (channel c pairs TX c / rx_count
 * with RX c % rx_count), each the fetchFrame() of a run of `budget` samples from Halton
 * index `index_offset` (plain, or with flags->doGuiding PathTracer::run's guided
 * schedule), all channels traced as one batch. frame_out (HOST) receives the radar cube
 * in the reference's layout [chirp][sample][channel], complex64 interleaved
 * (radar.h:487-494): a static scene's energy sits in Doppler bin 0 (PIndex::setVelocity(0),
 * path.h:130), so chirp 0 holds the channels' rows and every other chirp is zero. The
 * reference's PathTracer writes one channel per run (path.h:291-292); this traces the
 * array's channels together. frame->channelCount must be tx_count * rx_count.
 * Synchronous on `stream`. */
hsr_status hsr_simulate_frame(hsr_scene *scene, const hsr_rf_config *rf, const hsr_frame_config *frame,
                              const hsr_tracer_flags *flags, int32_t tx_count, const hsr_antenna *tx,
                              int32_t rx_count, const hsr_antenna *rx, int64_t budget, int64_t index_offset,
                              int32_t phase_mode, int32_t splat_mode, float *frame_out, void *stream);

/* Allocation-free form of hsr_simulate_batch_device, for callers that cannot allocate
 * device memory while they simulate (a real-time loop, work recorded into a larger
 * asynchronous pipeline, a framework whose memory pool must own every allocation).
 * It has no counterpart in the reference. Same arguments and output as
 * hsr_simulate_batch_device for the plain method (doGuiding = 0, the 33-bin frame
 * splat); its scratch (status, work counter, tile prefix, FP64 accumulators) lives in a
 * fixed file-scope device array of the library (about 1 MiB per device, held for the
 * life of the program), so the call performs no allocation. Limits: at most 64 poses
 * and 1024 range bins per call; larger requests return HSR_ERR_INVALID_ARGUMENT.
 * The array is shared by all calls on a device and keeps the last call's contents:
 * calls that overlap on the GPU race and must be serialised by the caller. The first
 * call on a device looks the array's address up (make it before any stream capture).
 * The call must be issued with the scene's device current, uses the scene's tuned launch
 * shape and the kernel hsr_set_path_kernel selects, and returns before the GPU has run:
 * read its device status with hsr_noalloc_status. */
hsr_status hsr_simulate_batch_device_noalloc(hsr_scene *scene, const hsr_rf_config *rf,
                                             int32_t samples_per_chirp,
                                             const hsr_tracer_flags *flags, int32_t pose_count,
                                             const hsr_antenna *d_tx, const hsr_antenna *d_rx,
                                             const int64_t *d_budget,
                                             const int64_t *d_index_offset, int32_t phase_mode,
                                             float *d_out_rows, void *stream);

/* Device status of the last hsr_simulate_batch_device_noalloc call on the current
 * device: synchronises `stream` and reads the status word in the library's static
 * scratch (bits as hsr_scene_status; HSR_ERR_DEVICE when any is set). Allocates nothing.
 * The next allocation-free call on the device clears the word. No counterpart in the
 * reference. */
hsr_status hsr_noalloc_status(void *stream, uint32_t *out_bits);

/* Far-field runs (RCS-style): as hsr_simulate_batch for the plain method, with each
 * pose's TX and RX a far-field antenna (hsr_ff_antenna). In the reference an FFAntenna
 * derives from Antenna, while Scene holds NFAntenna by value (scene.h:9-14), so
 * PathTracer::sample (path.h:235-451) is restated here with FFAntenna's sample, nee,
 * evaluate and connect (emitter.h:241-283): the direct TX -> RX term is zero (evaluate
 * zeroes the ray), and in the non-GO mode the primary segment adds no time of flight and
 * no 1 / (4 pi r) (connect does nothing). The GO mode runs on the wavefront kernel, the
 * non-GO mode on the one-thread-per-sample one; doGuiding must be 0
 * (HSR_ERR_NOT_SUPPORTED otherwise). HOST inputs and outputs, synchronous. */
hsr_status hsr_simulate_batch_ff(hsr_scene *scene, const hsr_rf_config *rf, int32_t samples_per_chirp,
                                 const hsr_tracer_flags *flags, int32_t pose_count, const hsr_ff_antenna *tx,
                                 const hsr_ff_antenna *rx, const int64_t *budget, const int64_t *index_offset,
                                 int32_t phase_mode, float *out_rows);

/* As hsr_simulate_batch_device, with HOST inputs and outputs: copies poses and budgets
 * in, runs, copies the rows out and synchronises. */
hsr_status hsr_simulate_batch(hsr_scene *scene, const hsr_rf_config *rf,
                              int32_t samples_per_chirp, const hsr_tracer_flags *flags,
                              int32_t pose_count, const hsr_antenna *tx,
                              const hsr_antenna *rx, const int64_t *budget,
                              const int64_t *index_offset, int32_t phase_mode,
                              int32_t splat_mode, float *out_rows, void *stream);

/* Test support: traces samples index_offset + [0, budget) of one pose and writes one
 * record per next-event estimate (path.h:292-397) into the HOST array `records`
 * (budget * max_records entries of 9 x 4 bytes: int32 depth (-1 = unused), int32
 * splatted, float time, v_re, v_im, dphase, bin, value_re, value_im). */
hsr_status hsr_debug_records(hsr_scene *scene, const hsr_rf_config *rf, int32_t samples_per_chirp,
                             const hsr_tracer_flags *flags, const hsr_antenna *tx, const hsr_antenna *rx,
                             int64_t budget, int64_t index_offset, int32_t max_records, void *records);

/* Measurement support: runs the counting instantiation of the trace kernel on a batch
 * (host arrays, as hsr_simulate_batch) and returns the exact traversal work of that
 * launch: out_counts[0] BVH nodes fetched (64 B each), [1] triangles fetched (48 B each),
 * [2] rays traced (closest-hit + shadow). */
hsr_status hsr_debug_traversal_counts(hsr_scene *scene, const hsr_rf_config *rf,
                                      int32_t samples_per_chirp, const hsr_tracer_flags *flags,
                                      int32_t pose_count, const hsr_antenna *tx,
                                      const hsr_antenna *rx, const int64_t *budget,
                                      const int64_t *index_offset, int64_t *out_counts);

/* Measurement support: read bandwidth of an L2-resident buffer of `bytes` (L2-cached
 * loads, `sweeps` passes in one launch, best of five launches, CUDA events), the L2
 * denominator of the traversal roofline. Synchronous. */
hsr_status hsr_measure_l2_read(int64_t bytes, int32_t sweeps, double *out_gbs);

/* Copies the scene's device BVH to the host (tests): out_nodes receives node_count binary
 * nodes of 64 bytes each, both child boxes and child references (layout in
 * hussar_gb300/csrc/hsr_common.cuh, struct DNode; a negative reference c is a leaf of
 * ((~c) & 7) + 1 triangles in consecutive slots from (~c) >> 3; the nodes are stored depth
 * first from the root, node 0, so a node's first child, when internal, is the next node),
 * out_tris triangle_count 48-byte records
 * {v0.xyz, original id bits, v1-v0, 0, v2-v0, 0} in slot order. Either pointer may be
 * null; capacities are in records. */
hsr_status hsr_debug_bvh(const hsr_scene *scene, void *out_nodes, int64_t node_capacity, void *out_tris,
                         int64_t tri_capacity);

/* The device Halton sampler (HaltonSampler::get1D, halton.h:56-67, 1082-1084) at `count`
 * host indices in dimension `dim` (0..9; larger dimensions give 0 as in the reference),
 * into out[count] (host). For tests: the trace kernels call the same device function. */
hsr_status hsr_debug_halton(const uint64_t *index, int64_t count, int32_t dim, float *out);

/* The primary direction's sine and cosine on the device (UniformSampleSphere,
 * sampling.h:38-43, in the reference-phase kernels): for every float x with lo <= |x| <= hi
 * (0 <= lo <= hi), both signs, the fast certified evaluation the kernels call against the
 * double-precision one it stands for. out_checked: arguments; out_mismatches: arguments
 * where the two differ in any bit (0 is the requirement); out_slow: arguments the fast
 * evaluation passed to the double-precision one. For tests. Synchronous. */
hsr_status hsr_debug_sincos_sweep(float lo, float hi, int64_t *out_checked, int64_t *out_mismatches,
                                  int64_t *out_slow);

/* ---- Autotuning of the plain wavefront launch ---------------------------------------
 * No counterpart in the reference. The launch shape of a plain batch: samples per work
 * item (tile), persistent CTAs per SM, and the queue threshold (GENERATE runs while a CTA
 * holds at most this many live paths; at most 256: thresholds up to 64 run a 320-entry
 * path stack, up to 128 a 384-entry one, above 128 a 512-entry one). Zero fields mean
 * the default shape (threshold 128). field_on_hit = 1 forms a primary ray's antenna field
 * only once the ray has hit something (for indirect-only paths: the field of a ray that
 * misses is never used), which pays where most primary rays miss and costs registers
 * elsewhere. coherent_order = 1 hands each stage's samples and paths to threads grouped
 * by primary sample cell and by reflected-direction octant (a counting sort per stage),
 * which pays on traversal-heavy scenes and costs three CTA barriers per stage elsewhere.
 * The shape changes the grouping of sums and the work done, not the samples traced nor
 * their values. */
typedef struct hsr_launch_config {
    int32_t tile;
    int32_t ctas_per_sm;
    int32_t queue_threshold;
    float trace_ms;          /* hsr_autotune_batch: the chosen shape's trace-kernel time */
    float default_trace_ms;  /* and the default shape's, on the same batch */
    int32_t field_on_hit;
    int32_t coherent_order;
} hsr_launch_config;

/* Runs the given batch (host arrays, as hsr_simulate_batch; plain GO mode) under
 * candidate shapes, keeps the fastest for later plain runs on this scene and returns it. */
hsr_status hsr_autotune_batch(hsr_scene *scene, const hsr_rf_config *rf, int32_t samples_per_chirp,
                              const hsr_tracer_flags *flags, int32_t pose_count, const hsr_antenna *tx,
                              const hsr_antenna *rx, const int64_t *budget, const int64_t *index_offset,
                              int32_t phase_mode, int32_t splat_mode, hsr_launch_config *out_best);
/* Sets the scene's launch shape (NULL: the default). */
hsr_status hsr_set_launch_config(hsr_scene *scene, const hsr_launch_config *config);
hsr_status hsr_get_launch_config(const hsr_scene *scene, hsr_launch_config *out);

/* Which trace kernel the simulate calls use (process-wide): 0 (default) = the wavefront
 * kernel whenever geometrical optics is on, 1 = always the one-thread-per-sample kernel.
 * Both compute the same per-path values; tests use this to check each one. */
hsr_status hsr_set_path_kernel(int32_t kind);

/* BVH topology for scenes created afterwards (process-wide): 0 (default) = PLOC
 * clustering over the Morton order (surface-area driven), 1 = LBVH radix tree. Both
 * give bit-identical ray-query results; only the traversal cost differs. */
hsr_status hsr_set_bvh_builder(int32_t builder);

/* Largest BVH leaf (triangles, 1..8, default 4) for scenes created afterwards
 * (process-wide): subtrees of at most this many triangles become one leaf where a
 * surface-area cost estimate finds testing their triangles cheaper than visiting their
 * nodes. Ray-query results do not depend on it (equal-distance hits go to the lower
 * primitive id); only the traversal cost does. */
hsr_status hsr_set_bvh_leaf_size(int32_t triangles);

/* Insertion passes over the BVH after its build (0..64, default 32; 0 = none) for scenes
 * created afterwards (process-wide). A pass takes every subtree out and re-inserts it
 * where the tree's surface-area cost grows least, in parallel with conflicting moves
 * resolved by priority; passes stop early once they move fewer than 1 in 20,000 nodes.
 * Fewer node visits per ray (on the 1 M-triangle boxes scene about a quarter fewer); the
 * ray-query results do not depend on it. The build keeps its own tree if the result is
 * deeper than 60 levels. */
hsr_status hsr_set_bvh_optimize(int32_t passes);

/* Engine of the fine-histogram synthesis GEMM (process-wide): 0 (default) = tensor cores
 * (tcgen05.mma, operands split into three BF16 terms, FP32 accumulation), 1 = CUDA cores
 * in FP32. Both compute the same product; tests use this to check one against the other. */
hsr_status hsr_set_synth_engine(int32_t engine);

/* Timing of the most recent batch launch on this scene: device milliseconds of the
 * trace kernel alone, measured with CUDA events on the launching stream. */
hsr_status hsr_last_kernel_ms(const hsr_scene *scene, float *out_ms);

/* ---- A plain batch captured into a CUDA graph --------------------------------------
 *
 * No counterpart in the reference (its GPU backend launches one pose per call). Captures
 * hsr_simulate_batch_device's plain method (doGuiding = 0) with the given phase and splat
 * modes for fixed device buffers once; every launch replays the whole batch (pose upload,
 * work-item prefix, the persistent trace launch, then the fetchFrame rows, or with
 * HSR_SPLAT_FINE_SYNTH the tensor-core synthesis of the rows) as one graph launch and
 * reads the buffers' current contents, so poses, budgets and offsets may change between
 * launches (the pose count, N, chirp and flags may not). The graph owns its scratch (and,
 * for synthesis, its own twiddle operand); it uses the scene's BVH and launch shape, so
 * destroy it before the scene. hsr_launch_count counts a replay as the kernels it runs. */
typedef struct hsr_batch_graph hsr_batch_graph;

hsr_status hsr_batch_graph_create(hsr_scene *scene, const hsr_rf_config *rf, int32_t samples_per_chirp,
                                  const hsr_tracer_flags *flags, int32_t pose_count, const hsr_antenna *d_tx,
                                  const hsr_antenna *d_rx, const int64_t *d_budget,
                                  const int64_t *d_index_offset, int32_t phase_mode, int32_t splat_mode,
                                  float *d_out_rows, hsr_batch_graph **out_graph);
/* Asynchronous on `stream` (a cudaStream_t; NULL = legacy default stream). */
hsr_status hsr_batch_graph_launch(hsr_batch_graph *graph, void *stream);
/* Synchronises the device; HSR_ERR_DEVICE if any launch so far set the status word. */
hsr_status hsr_batch_graph_status(hsr_batch_graph *graph);
hsr_status hsr_batch_graph_destroy(hsr_batch_graph *graph);

/* ---- Serving: continuous batching over resident scenes ------------------------------
 *
 * No counterpart in the reference, whose backends run one pose per synchronous call
 * (src/arch/gpu.cpp:499-532, examples/src/2_large_scene.cpp:149-166). A server keeps
 * several scenes resident and traces requests (scene, pose, chirp, range bins, budget)
 * as they arrive: a worker thread runs batching ticks, each one persistent launch over
 * a slice of every admitted request, so requests that arrive while others run join the
 * next tick and their work shares the device. Requests are admitted when a slot and
 * device memory for their accumulators are free. A request's result is the row
 * hsr_simulate_batch gives for the same scene, pose, chirp, budget and index offset
 * (the same Halton samples; only the summation order differs). The tracer flags and the
 * phase mode are per server; geometrical optics must be on. With flags.doGuiding every
 * request runs PathTracer::run's guided schedule (path.h:171-224) across ticks over a
 * guiding tree of the server (one per slot): an iteration's chunks share ticks with
 * other requests, the tick that ends an iteration steps the request's tree, and the next
 * iteration starts in a tick after it; the row equals hsr_simulate_batch's guided row up
 * to the order of the float training sums. A tick runs
 * the larger path stack (GENERATE threshold 128) only when every scene in it was
 * autotuned (hsr_autotune_batch) to a threshold above 64, and larger work items when
 * its requests' chunks are large. */
typedef struct hsr_server hsr_server;

typedef struct hsr_server_config {
    int32_t max_slots;             /* requests admitted at once (each holds a slot) */
    int32_t max_samples_per_chirp; /* largest N a request may ask for */
    int64_t memory_bytes;          /* device memory for request state (admission by footprint) */
    float tick_ms;                 /* target device time of one batching tick */
    int32_t phase_mode;            /* hsr_phase_mode shared by every request */
    hsr_tracer_flags flags;        /* tracer flags shared by every request */
} hsr_server_config;

typedef struct hsr_request {
    int32_t scene;                 /* id returned by hsr_server_add_scene */
    int32_t samples_per_chirp;     /* N, 1 .. max_samples_per_chirp */
    hsr_rf_config rf;
    hsr_antenna tx, rx;
    int64_t budget;                /* Halton indices index_offset + [0, budget) */
    int64_t index_offset;
    float *out_row;                /* host complex64[N]: the fetchFrame row, written before completion */
} hsr_request;

typedef struct hsr_request_result {
    int32_t status;                /* hsr_status of the request */
    int32_t ticks;                 /* batching ticks the request took part in */
    double queue_ms;               /* submit -> admitted */
    double latency_ms;             /* submit -> row written */
} hsr_request_result;

typedef struct hsr_server_stats {
    int64_t submitted, completed, failed;
    int64_t ticks;
    int64_t samples;               /* paths traced by the ticks */
    double device_ms;              /* summed device time of the ticks (CUDA events) */
    double p50_ms, p99_ms, max_ms; /* latency of completed requests (submit -> row written) */
    int32_t max_batch;             /* most requests in one tick */
    int32_t max_resident;          /* most requests admitted at once */
    int64_t admitted_while_busy;   /* requests admitted while a tick was on the device */
    int64_t memory_bytes_peak;     /* most request-state bytes held at once */
    int64_t scene_bytes;           /* device bytes of the registered scenes */
} hsr_server_stats;

/* max_slots 256, N <= 1024, 64 MiB of request state, 4 ms ticks, FP32 reference phase,
 * the reference's PathTracer defaults with doGuiding = 0. */
void hsr_default_server_config(hsr_server_config *config);
hsr_status hsr_server_create(const hsr_server_config *config, hsr_server **out_server);
/* Registers a resident scene (not owned: it must outlive the server). Thread-safe. */
hsr_status hsr_server_add_scene(hsr_server *server, hsr_scene *scene, int32_t *out_id);
/* Queues a request (copied; out_row must stay valid until the request completes).
 * Thread-safe. */
hsr_status hsr_server_submit(hsr_server *server, const hsr_request *request, uint64_t *out_ticket);
/* Waits up to timeout_ms (< 0: forever) for a request. HSR_OK: finished, `out` filled
 * and the ticket released; HSR_ERR_TIMEOUT: still running (wait again). Thread-safe. */
hsr_status hsr_server_wait(hsr_server *server, uint64_t ticket, int32_t timeout_ms,
                           hsr_request_result *out);
hsr_status hsr_server_get_stats(hsr_server *server, hsr_server_stats *out);
/* Clears the counters and the latency record (e.g. after a warm-up). */
hsr_status hsr_server_reset_stats(hsr_server *server);
/* Finishes the ticks on the device, fails queued and unfinished requests with
 * HSR_ERR_INTERRUPTED, and frees the server. */
hsr_status hsr_server_destroy(hsr_server *server);

/* The tick planner (host only, no device): splits a tick's sample target over requests
 * with `remaining` samples each, by water-filling in order of the smallest remainder;
 * every chunk but a request's last is a multiple of `tile`. */
hsr_status hsr_debug_plan_tick(int32_t count, const int64_t *remaining, int64_t target, int32_t tile,
                               int64_t *out_chunk);

#ifdef __cplusplus
}
#endif

#endif /* HSR_GB300_H */
