/*
 * ORACLE — TEST INFRASTRUCTURE ONLY. C interface of the CPU restatement in
 * hsr_oracle.cpp, loaded by tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg through ctypes. The structs have the same layout as the
 * product's C ABI structs (include/hsr_gb300.h) so both can be fed the same bytes.
 */
#ifndef HSR_ORACLE_H
#define HSR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hsr_rf_config_o {
    float startFreq, freqSlope, adcRate, idleTime, rampTime, antennaDelay;
} hsr_rf_config_o;

typedef struct hsr_frame_config_o {
    int32_t chirpCount, samplesPerChirp, channelCount;
} hsr_frame_config_o;

typedef struct hsr_antenna_o {
    float position[3];
    float rotation[9];
} hsr_antenna_o;

typedef struct hsr_ff_antenna_o {
    float direction[3];
    float polarization[6];
    float scene_center[3];
    float radius;
} hsr_ff_antenna_o;

typedef struct hsr_tracer_flags_o {
    int32_t onlyIndirect, maxDepth, useGeometricalOptics, poDiffraction, doGuiding, clearBeforeIteration,
        correctPhase, filterGuiding, doFiltering, filteringSphere, produceDebugImage;
    float filteringMin, filteringMax, filteringRadius;
} hsr_tracer_flags_o;

/* One next-event estimate of one sample (path.h:292-397). */
typedef struct oracle_record {
    int32_t depth;     /* -1: unused slot */
    int32_t splatted;  /* 1 if Integrator::splat passed its early-out */
    double time;       /* nee.ray.time before antennaDelay */
    double v_re, v_im; /* measurement after scaling and filtering */
    double dphase;
    double bin;        /* fractional sample index */
    double value_re, value_im; /* weight * measurement * measureRay */
} oracle_record;

int oracle_abi_version(void);
float oracle_radical_inverse_f(uint64_t index, int dim);
double oracle_radical_inverse_d(uint64_t index, int dim);
void *oracle_scene_create(const float *vertices, int64_t nv, const int32_t *indices, int64_t nt);
void oracle_scene_destroy(void *scene);
int64_t oracle_bvh_nodes(void *scene);
int oracle_intersect(void *scene, int64_t count, const float *o, const float *d, const float *tfar,
                     float *t_out, float *p_out, float *n_out, int32_t *prim_out);
int oracle_visible(void *scene, int64_t count, const float *o, const float *d, const float *tfar,
                   int32_t *vis);
/* precision: 32 (reference single-precision semantics), 64 (FP64 oracle) or 65 (FP64
 * oracle fed the float-rounded Halton values of the FP32 run: the same sample set);
 * OR 0x100 to replace Frame::splat<16> by the exact finite-N Dirichlet synthesis (the
 * estimator of the fine-histogram mode).
 * frame_out: 2*chirps*samples*channels doubles, ADDED to. */
int oracle_simulate(void *scene, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc,
                    const hsr_antenna_o *tx, const hsr_antenna_o *rx, const hsr_tracer_flags_o *fl,
                    int64_t budget, int64_t offset, float sample_weight, int precision, int threads,
                    double *frame_out, double *weight_out);
/* Far-field TX and RX (FFAntenna, emitter.h:226-291); precision 32, 64 or 65 as above. */
int oracle_simulate_ff(void *scene, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc,
                       const hsr_ff_antenna_o *tx, const hsr_ff_antenna_o *rx, const hsr_tracer_flags_o *fl,
                       int64_t budget, int64_t offset, float sample_weight, int precision, int threads,
                       double *frame_out, double *weight_out);
int oracle_records(void *scene, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc,
                   const hsr_antenna_o *tx, const hsr_antenna_o *rx, const hsr_tracer_flags_o *fl,
                   int64_t first, int64_t count, int64_t offset, int max_records, oracle_record *out);
void oracle_frame_splat(int chirps, int samples, int channels, float ic, float is, float ich, float re,
                        float im, float *frame);
void oracle_awr_evaluate(const float *d, float *H6);
void oracle_uniform_sample_sphere(float u0, float u1, float *d);
void oracle_measure_ray(float dt, float startFreq, float freqSlope, float *out2);
/* PIndex::setTime's fractional bin for a delay that already includes antennaDelay. */
/* std::exp(Complex(0, angle)) as radar::polar forms it (cos/sin of the widened angle). */
void oracle_cexp(float angle, float *out2);
float oracle_set_time(float delta_t, float freqSlope, float adcRate, int samples);
/* 1: primary directions from the libm's sinf/cosf (a glibc build of the reference);
 * 0 (default): sin/cos rounded once to float, what the GPU computes. Not thread-safe:
 * set it before a simulation starts. */
void oracle_set_libm_trig(int on);
void oracle_sincos_rounded(float x, float *s, float *c);

/* Path guiding: the product's 2-D tree behind GuidingWrapper (path.h:17-131), restated.
 * Arrays are 2048 entries (the tree's capacity); get returns the training node count. */
void *oracle_guide_create(void);
void oracle_guide_destroy(void *guide);
void oracle_guide_reset(void *guide);
void oracle_guide_step(void *guide);
int32_t oracle_guide_get(void *guide, int32_t *samp_child, float *samp_p, int32_t *train_child, float *acc2);
int oracle_guide_set(void *guide, int32_t count, const int32_t *samp_child, const float *samp_p,
                     const int32_t *train_child, const float *acc2);
float oracle_guide_sample(void *guide, float x0, float x1, float *y2);
/* one guided iteration on one thread, FP32; adds to frame_out / weight_out */
int oracle_guided_pass(void *scene, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc,
                       const hsr_antenna_o *tx, const hsr_antenna_o *rx, const hsr_tracer_flags_o *fl,
                       int64_t budget, int64_t offset, float sample_weight, int train, void *guide,
                       double *frame_out, double *weight_out);
/* PathTracer::run's guided schedule (path.h:171-224); overwrites frame_out / weight_out */
int oracle_path_tracer_run(void *scene, const hsr_rf_config_o *rf, const hsr_frame_config_o *fc,
                           const hsr_antenna_o *tx, const hsr_antenna_o *rx, const hsr_tracer_flags_o *fl,
                           int64_t samples, void *guide, double *frame_out, double *weight_out);

#ifdef __cplusplus
}
#endif
#endif
