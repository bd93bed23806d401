/*
 * pm_oracle.h -- CPU restatement of the PatchMatch multi-view-stereo hot path of
 * yhsa678/patchMatch_cuda (TEST INFRASTRUCTURE ONLY).
 *
 * This oracle is the checker for the CUDA engine in patchmatch_cuda_gb300/. Only the
 * tests, the smoke entry point and the CPU-baseline legs of bench.py may load it. The
 * product path never calls it.
 *
 * Parity status: pinned to the reference's own code. yhsa678/patchMatch_cuda ships no tests,
 * fixtures or golden vectors, and its CUDA build cannot run here (it needs CUDA texture
 * references, which CUDA 12 removed, plus OpenCV and Boost); its device code does compile for
 * the CPU (oracle/ref_host.cpp runs the kernels extracted unchanged by ref_extract.sh). That
 * host run, with the reference's random states drawn as the stream mode below draws them,
 * writes the golden vectors under tests/golden/ (ref_*.npz) that this restatement must
 * reproduce: box sums, NCC, initial costs, messages, the tie rule, single sweeps in every
 * direction and whole runs. Known-answer tests derived from the reference code (identical
 * windows -> 0, flat window -> 1, window outside the source -> 2, tie rule, message fixed
 * points) and the ground truth of seeded synthetic scenes add to that.
 *
 * Numbers: built with real = double (the FP64 oracle) or, with -DPMO_REAL_FLOAT, with
 * real = float (the timed CPU baseline). The API always passes double arrays.
 */
#ifndef PM_ORACLE_H
#define PM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Sweep directions, in the order the reference schedules them within one iteration
 * (patchMatch.cu:344-391). LR and RL run on the transposed maps in the reference
 * (isRotated = true). */
enum { PMO_DIR_LR = 0, PMO_DIR_TB = 1, PMO_DIR_RL = 2, PMO_DIR_BT = 3 };

/* Purposes of random draws. A draw is keyed by (pixel, sweep, purpose, sub-index), so
 * every draw of the reference's per-thread curand stream maps to one Philox counter. */
enum {
    PMO_RNG_INIT = 1,      /* initial depth, array2d_wrapper.cu:15                     */
    PMO_RNG_BWD = 2,       /* cost==2 replacement in computeMessageBackward (:680-682)  */
    PMO_RNG_FWD_PRE = 3,   /* same, forward message with the old costs (:905)           */
    PMO_RNG_FWD_POST = 4,  /* same, forward message with the new costs (:874, :999)     */
    PMO_RNG_RAND_DEPTH = 5,/* random depth hypothesis (:937)                           */
    PMO_RNG_SAMPLE = 6,    /* view sample j (:942)                                      */
    PMO_RNG_REFINE = 7     /* refinement trial (the engine's; the reference never runs
                              its depthRefinement kernel, :717-773)                    */
};

typedef struct pmo_problem {
    int width, height;              /* reference image size                               */
    int n_src;                      /* number of source views                             */
    int half_window;                /* halfWindowSize, window side = 2*hw+1               */
    const float *ref;               /* height*width reference texels (u8/255 or filtered) */
    const float *const *src;        /* n_src source images, row-major texels               */
    const int *src_width;
    const int *src_height;
    const double *hh;               /* n_src*18: H1 (row-major 3x3) then H2, image.cpp:4-13 */
    double inv_k[4];                /* K^-1 (0,0), (0,2), (1,1), (1,2), patchMatch.cu:155-156 */
    double orientation[3];          /* plane normal (orientationX, 0, orientationZ)        */
    double depth_near, depth_far;
    float sp_alpha;                 /* SPMAlpha; squared in float as at patchMatch.cu:316  */
    uint64_t seed;
    uint32_t batch_id;              /* fourth Philox counter word                          */
    int quirks;                     /* nonzero: keep the reference's ref/source window
                                       misalignment at the leading edge (:546)            */
    int sampler;                    /* 0: exact bilinear weights; 1: texture-unit weights
                                       (fractions rounded half-up to 1/256, cross term
                                       alpha*beta rounded likewise) on single-precision
                                       coordinates formed as the engine forms them        */
    float perturbation;             /* 0: uniform random hypothesis (the reference). > 0: the
                                       engine's local search: half of the pixels (second
                                       Philox word >= 1/2) draw within +-perturbation x
                                       2^(-sweep/4) of their current depth                */
    int planes;                     /* 0: one plane normal for every pixel, the reference's
                                       orientation (patchMatch.cu:32, main.cpp:65-76).
                                       1: a slanted plane per pixel, n ~ (a, b, 1) in the
                                       reference camera (no counterpart in the reference) */
    const double *ee;               /* planes: n_src*3, e = K_s T_rel, the column vector of
                                       H2 = K_s T_rel n^T K_r^-1 (image.cpp:4-13)           */
    float plane_depth_step;         /* planes: relative half-width of the local search's depth
                                       perturbation at sweep 0 (scaled by 2^(-sweep/4))      */
    float plane_slope_step;         /* planes: half-width of its slope perturbation at sweep 0 */
    int rng_stream;                 /* 0: keyed draws (the engine's). 1: the reference's order
                                       of draws from per-pixel random states (array2d_psng):
                                       the initial depth of pixel i is the next draw of state i,
                                       a sweep line draws from one state -- state x for
                                       vertical sweeps over column x, state y*width for
                                       horizontal sweeps over row y (patchMatch.cu:838-843,
                                       :1034-1039) -- in the reference's order: backward
                                       messages, the first step's forward message, then per
                                       step the forward message, the random depth, the view
                                       samples and the refreshed forward message. Draw k of
                                       state s is Philox of counter (s, k, PMO_STREAM_PURPOSE
                                       << 16, 0). Not with planes or perturbation.           */
    uint32_t *rng_counts;           /* rng_stream: width*height draws made so far per state,
                                       updated in place                                     */
} pmo_problem;

#define PMO_STREAM_PURPOSE 0x5EEDu

/* Slanted-plane mode. A pixel's plane is its depth d (reference-camera z) and slopes (a, b):
 * normal n ~ (a, b, 1), so n . X = d s with the plane scale
 * s = a (ik00 (x + 1/2) + ik02) + b (ik11 (y + 1/2) + ik12) + 1 (floored at PMO_SCALE_MIN), and
 * the homography is H1 - e g^T / (d s) with g = (a ik00, b ik11, a ik02 + b ik12 + 1). */
#define PMO_SLOPE_DRAW 1.0f     /* random slopes are uniform in [-1, 1]^2                  */
#define PMO_SLOPE_MAX 2.0f      /* perturbed slopes clamp to [-2, 2]                       */
#define PMO_SCALE_MIN 0.0625f

void pmo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double pmo_uniform(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3);

void pmo_init_relative(const double k_ref[9], const double r_ref[9], const double t_ref[3],
                       const double k_src[9], const double r_src[9], const double t_src[3],
                       double orientation_x, double orientation_z,
                       double out_hh[18], double out_inv_k[4]);
/* e = K_s T_rel = K_s R_s (C_s - C_r) (image.cpp:4-13), the plane-mode translation term. */
void pmo_translation_term(const double r_ref[9], const double t_ref[3], const double k_src[9],
                          const double r_src[9], const double t_src[3], double out_e[3]);

int pmo_prefilter(const float *in, int width, int height, int mode, float sigma, float *out);
void pmo_box_moments(const float *img, int width, int height, int half_window,
                     double *sum_i, double *sum_ii);

/* Source fetch at texel coordinates (texel i at i), patchMatch.cu:543. */
void pmo_sample(const pmo_problem *p, int view, int n, const float *xs, const float *ys,
                double *out);
double pmo_ncc(const pmo_problem *p, const double *sum_i, const double *sum_ii,
               int x, int y, int view, double depth, int axis);
void pmo_ncc_batch(const pmo_problem *p, const double *sum_i, const double *sum_ii, int n,
                   const int *xs, const int *ys, const int *views, const double *depths,
                   const int *axes, double *out);

void pmo_init_depth(const pmo_problem *p, double *depth);
long long pmo_initial_costs(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                            const double *depth, double *cost);
long long pmo_sweep(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                    double *depth, double *cost, int dir, uint32_t sweep_id, int num_samples,
                    unsigned char *view_sel, int line_begin, int line_end);
/* Depth refinement as the engine's refine_kernel: per pixel, trials hypotheses d0 + sigma z
 * (z = sqrt(3) (u1 + u2 + u3 + u4 - 2) in float from one Philox counter keyed (pixel, sweep_id,
 * PMO_RNG_REFINE << 16 | trial, batch_id)), hypotheses outside [near, far] skipped, each scored
 * by the mean cost over the views in rows 0 .. num_samples-1 of view_sel (entries >= n_src:
 * none); the lowest mean below the current depth's replaces it. In place on depth; returns
 * the evaluation count. */
long long pmo_refine(const pmo_problem *p, const double *sum_i, const double *sum_ii, double *depth,
                     const unsigned char *view_sel, int num_samples, int trials, float sigma,
                     uint32_t sweep_id, int axis);
long long pmo_run(const pmo_problem *p, int iterations, int num_samples,
                  const double *sum_i, const double *sum_ii,
                  double *depth, double *cost, unsigned char *view_sel);

/* Slanted-plane mode (p->planes = 1): slopes hold (a, b) per pixel, height*width*2 floats.
 * Initial slopes are uniform in [-PMO_SLOPE_DRAW, PMO_SLOPE_DRAW]^2 from words 1 and 2 of the
 * initial-depth counter. In a sweep the three hypotheses are: the previous step's plane carried
 * to this pixel (d' = d s_prev / s_here under its slopes), the current plane, and a random one
 * from the four words of the random-depth counter: word 1 < 1/3 a uniform depth with the
 * current slopes (the reference's random depth); < 2/3 the current depth with uniform slopes;
 * else a local perturbation of both (plane_depth_step, plane_slope_step, each x 2^(-sweep/4)). */
void pmo_init_planes(const pmo_problem *p, float *slopes);
double pmo_ncc_plane(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                     int x, int y, int view, double depth, float a, float b, int axis);
void pmo_ncc_plane_batch(const pmo_problem *p, const double *sum_i, const double *sum_ii, int n,
                         const int *xs, const int *ys, const int *views, const double *depths,
                         const float *slopes, const int *axes, double *out);
long long pmo_initial_costs_planes(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                                   const double *depth, const float *slopes, double *cost);
long long pmo_sweep_planes(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                           double *depth, float *slopes, double *cost, int dir, uint32_t sweep_id,
                           int num_samples, unsigned char *view_sel, int line_begin, int line_end);
long long pmo_refine_planes(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                            double *depth, const float *slopes, const unsigned char *view_sel,
                            int num_samples, int trials, float sigma, uint32_t sweep_id, int axis);
long long pmo_run_planes(const pmo_problem *p, int iterations, int num_samples,
                         const double *sum_i, const double *sum_ii, double *depth, float *slopes,
                         double *cost, unsigned char *view_sel);

/* Message updates and the tie rule, exposed for known-answer tests. */
double pmo_msg_forward(double msg, double cost, double u_if_two, float sp_alpha);
double pmo_msg_backward(double msg, double cost, double u_if_two, float sp_alpha);
int pmo_find_min_cost(const double cost[3]);

int pmo_num_threads(void);
int pmo_real_bytes(void);

#ifdef __cplusplus
}
#endif
#endif
