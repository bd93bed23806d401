/*
 * pm_oracle.c -- CPU restatement of the PatchMatch MVS hot path of
 * yhsa678/patchMatch_cuda. TEST INFRASTRUCTURE ONLY (the checker for the CUDA engine);
 * see pm_oracle.h for the parity status ("parity unpinned" by the reference, pinned by
 * code-derived known-answer tests and synthetic ground truth).
 *
 * Every function names the reference lines it restates (paths relative to the
 * reference project root). Differences that are definitions rather than arithmetic:
 *  - Random numbers: the reference draws from per-column curand XORWOW states
 *    (array2d_psng.cu:3-17). Here every draw is one Philox4x32-10 output keyed by
 *    (pixel, sweep, purpose, sub-index); the uniform is ((x >> 8) + 1) * 2^-24 in (0, 1],
 *    the same interval curand_uniform returns.
 *  - Bilinear source sampling, texel i at coordinate i, zero border (the reference's
 *    tex2DLayered(u/z + 0.5, v/z + 0.5) fetch, patchMatch.cu:543), either with exact
 *    weights or with the texture unit's fixed-point weights (sampler 1).
 *  - Message storage: the reference keeps emissions in float and builds with
 *    --use_fast_math (cmakelists_32bit.txt:11), so an emission below FLT_MIN becomes 0 and
 *    so do messages and posteriors that fall below FLT_MIN. This restatement rounds the
 *    emission to float and flushes those values to zero as well; where every view's
 *    posterior is then zero the CDF is 0/0 and no view is sampled.
 *  - A view sample whose CDF search finds no view (only possible when the posterior
 *    CDF is NaN) is skipped; the reference then indexes layer -1 (undefined). If no
 *    sample of a pixel finds a view the current depth is kept.
 */
#include "pm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef PMO_REAL_FLOAT
typedef float real;
#define R_SQRT sqrtf
#define R_EXP expf
#define R_FLOOR floorf
#else
typedef double real;
#define R_SQRT sqrt
#define R_EXP exp
#define R_FLOOR floor
#endif

/* Constants of patchMatch.cu:9-10 and :673/:697, rounded to float as the reference
 * declares them. CHANGE_STATE_PROB is the float difference 1.0f - 0.999f. */
#define FIX_STATE_PROB ((real)0.999f)
#define CHANGE_STATE_PROB ((real)(1.0f - 0.999f))
#define UNIFORM_EMISSION_COST ((real)0.83f)

/* ------------------------------------------------------------------------------------
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2,
 * 3", SC'11): 10 rounds of the 4x32 Philox S-box with multipliers 0xD2511F53 and
 * 0xCD9E8D57 and Weyl key increments 0x9E3779B9 and 0xBB67AE85.
 * ---------------------------------------------------------------------------------- */
void pmo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

double pmo_uniform(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3)
{
    uint32_t ctr[4] = {c0, c1, c2, c3};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t out[4];
    pmo_philox4x32_10(ctr, key, out);
    return (double)((out[0] >> 8) + 1u) * (1.0 / 16777216.0);
}

static inline real draw(const pmo_problem *p, int pixel, uint32_t sweep, int purpose, int sub)
{
    return (real)pmo_uniform(p->seed, (uint32_t)pixel, sweep,
                             ((uint32_t)purpose << 16) | (uint32_t)sub, p->batch_id);
}

/* Stream mode: the next draw of random state `state` (pmo_problem.rng_stream). */
static inline real stream_draw(const pmo_problem *p, uint32_t state)
{
    const uint32_t k = p->rng_counts[state]++;
    return (real)pmo_uniform(p->seed, state, k, PMO_STREAM_PURPOSE << 16, 0u);
}

/* A depth hypothesis U * (far - near) + near as the reference forms it: in float, the span
 * rounded to float first (array2d_wrapper.cu:15, patchMatch.cu:937), one fused multiply-add
 * (an exact float product fits a double, so rounding the double sum once is the fused result). */
static inline double float_depth(double u, double near, double far)
{
    const float span = (float)((double)(float)far - (double)(float)near);
    return (double)(float)((double)(float)u * (double)span + (double)(float)near);
}

/* ------------------------------------------------------------------------------------
 * Camera setup: Image::updateCamParam (image.cpp:39-61: C = -R^T T, K^-1, R^-1 = R^T)
 * and Image::init_relative (image.cpp:4-13):
 *   R_rel = R_s R_r^T,  T_rel = R_s (C_s - C_r),
 *   H1 = K_s R_rel K_r^-1,  H2 = K_s T_rel n^T K_r^-1,  n = (orientationX, 0, orientationZ).
 * The reference does this in float (cv::Mat CV_32F); here in double.
 * ---------------------------------------------------------------------------------- */
static void mat3_mul(const double *a, const double *b, double *out)
{
    double t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            t[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
    memcpy(out, t, sizeof t);
}

static void mat3_inverse(const double *m, double *out)
{
    double c00 = m[4] * m[8] - m[5] * m[7];
    double c01 = m[5] * m[6] - m[3] * m[8];
    double c02 = m[3] * m[7] - m[4] * m[6];
    double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    double inv = 1.0 / det;
    out[0] = c00 * inv;
    out[1] = (m[2] * m[7] - m[1] * m[8]) * inv;
    out[2] = (m[1] * m[5] - m[2] * m[4]) * inv;
    out[3] = c01 * inv;
    out[4] = (m[0] * m[8] - m[2] * m[6]) * inv;
    out[5] = (m[2] * m[3] - m[0] * m[5]) * inv;
    out[6] = c02 * inv;
    out[7] = (m[1] * m[6] - m[0] * m[7]) * inv;
    out[8] = (m[0] * m[4] - m[1] * m[3]) * inv;
}

void pmo_init_relative(const double k_ref[9], const double r_ref[9], const double t_ref[3],
                       const double k_src[9], const double r_src[9], const double t_src[3],
                       double orientation_x, double orientation_z,
                       double out_hh[18], double out_inv_k[4])
{
    double c_ref[3], c_src[3], rt_ref[9], k_ref_inv[9];
    for (int i = 0; i < 3; ++i) {
        c_ref[i] = -(r_ref[i] * t_ref[0] + r_ref[3 + i] * t_ref[1] + r_ref[6 + i] * t_ref[2]);
        c_src[i] = -(r_src[i] * t_src[0] + r_src[3 + i] * t_src[1] + r_src[6 + i] * t_src[2]);
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) rt_ref[3 * i + j] = r_ref[3 * j + i];
    mat3_inverse(k_ref, k_ref_inv);

    double r_rel[9], h1[9];
    mat3_mul(r_src, rt_ref, r_rel);
    mat3_mul(k_src, r_rel, h1);
    mat3_mul(h1, k_ref_inv, h1);

    double dc[3] = {c_src[0] - c_ref[0], c_src[1] - c_ref[1], c_src[2] - c_ref[2]};
    double t_rel[3], kt[3];
    for (int i = 0; i < 3; ++i)
        t_rel[i] = r_src[3 * i] * dc[0] + r_src[3 * i + 1] * dc[1] + r_src[3 * i + 2] * dc[2];
    for (int i = 0; i < 3; ++i)
        kt[i] = k_src[3 * i] * t_rel[0] + k_src[3 * i + 1] * t_rel[1] + k_src[3 * i + 2] * t_rel[2];
    double n[3] = {orientation_x, 0.0, orientation_z};
    double nk[3]; /* n^T K_r^-1 (row vector) */
    for (int j = 0; j < 3; ++j)
        nk[j] = n[0] * k_ref_inv[j] + n[1] * k_ref_inv[3 + j] + n[2] * k_ref_inv[6 + j];
    for (int i = 0; i < 9; ++i) out_hh[i] = h1[i];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out_hh[9 + 3 * i + j] = kt[i] * nk[j];
    out_inv_k[0] = k_ref_inv[0];
    out_inv_k[1] = k_ref_inv[2];
    out_inv_k[2] = k_ref_inv[4];
    out_inv_k[3] = k_ref_inv[5];
}

void pmo_translation_term(const double r_ref[9], const double t_ref[3], const double k_src[9],
                          const double r_src[9], const double t_src[3], double out_e[3])
{
    double c_ref[3], c_src[3], t_rel[3];
    for (int i = 0; i < 3; ++i) {
        c_ref[i] = -(r_ref[i] * t_ref[0] + r_ref[3 + i] * t_ref[1] + r_ref[6 + i] * t_ref[2]);
        c_src[i] = -(r_src[i] * t_src[0] + r_src[3 + i] * t_src[1] + r_src[6 + i] * t_src[2]);
    }
    const double dc[3] = {c_src[0] - c_ref[0], c_src[1] - c_ref[1], c_src[2] - c_ref[2]};
    for (int i = 0; i < 3; ++i)
        t_rel[i] = r_src[3 * i] * dc[0] + r_src[3 * i + 1] * dc[1] + r_src[3 * i + 2] * dc[2];
    for (int i = 0; i < 3; ++i)
        out_e[i] = k_src[3 * i] * t_rel[0] + k_src[3 * i + 1] * t_rel[1] + k_src[3 * i + 2] * t_rel[2];
}

/* ------------------------------------------------------------------------------------
 * GaussianBlurCUDA (GaussianBlurCUDA.cu:73-199): separable row then column filter of a
 * float image. The class reads its input through a texture reference whose modes it never
 * sets (:22, :132-149), so the defaults hold: point filtering and clamp addressing, a tap
 * outside the image reads the nearest edge pixel. Width = (int)(5*sigma), made odd, clamped
 * to [5, 45] (:99-115). mode 1 ("box") keeps the reference class as written, which
 * overwrites the Gaussian weights with 1/width (:128-129); mode 2 uses the Gaussian weights
 * the class computes before that overwrite, normalised to sum 1 (the class's normalisation
 * is commented out, :125-126); mode 0 copies. Taps are summed in the kernels' order,
 * k = -radius .. radius with weight[radius - k] (:49, :67).
 * ---------------------------------------------------------------------------------- */
int pmo_prefilter(const float *in, int width, int height, int mode, float sigma, float *out)
{
    if (mode == 0) {
        memcpy(out, in, sizeof(float) * (size_t)width * height);
        return 0;
    }
    if (mode == 2 && !(sigma > 0.0f)) return -1;
    int kw = (int)(5.0f * sigma);
    if (kw % 2 == 0) kw += 1;
    int radius = (kw - 1) >> 1;
    if (kw > 45) { radius = 22; kw = 45; }
    else if (kw < 5) { radius = 2; kw = 5; }
    real weights[45];
    if (mode == 1) {
        for (int i = 0; i < kw; ++i) weights[i] = (real)1.0 / (real)kw;
    } else {
        real rv = (real)-0.5 / ((real)sigma * (real)sigma), ksum = 0;
        for (int i = -radius; i <= radius; ++i) {
            weights[i + radius] = R_EXP((real)(i * i) * rv);
            ksum += weights[i + radius];
        }
        for (int i = 0; i < kw; ++i) weights[i] /= ksum;
    }
    real *tmp = (real *)malloc(sizeof(real) * (size_t)width * height);
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            real s = 0;
            for (int k = -radius; k <= radius; ++k) {
                const int xx = x + k < 0 ? 0 : (x + k >= width ? width - 1 : x + k);
                const real v = (real)in[(size_t)y * width + xx];
                s += v * weights[radius - k];
            }
            tmp[(size_t)y * width + x] = s;
        }
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            real s = 0;
            for (int k = -radius; k <= radius; ++k) {
                const int yy = y + k < 0 ? 0 : (y + k >= height ? height - 1 : y + k);
                const real v = tmp[(size_t)yy * width + x];
                s += v * weights[radius - k];
            }
            out[(size_t)y * width + x] = (float)s;
        }
    free(tmp);
    return 0;
}

/* ------------------------------------------------------------------------------------
 * Reference-window moments, Array2d_refImg::filterImage (array2d_refImg.cu:11-67,
 * :100-132): box sums of I and I*I over the (2hw+1)^2 window with zero border, row pass
 * then column pass.
 * ---------------------------------------------------------------------------------- */
void pmo_box_moments(const float *img, int width, int height, int half_window,
                     double *sum_i, double *sum_ii)
{
    real *row_i = (real *)malloc(sizeof(real) * (size_t)width * height);
    real *row_ii = (real *)malloc(sizeof(real) * (size_t)width * height);
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            real a = 0, b = 0;
            for (int k = -half_window; k <= half_window; ++k) {
                int xx = x + k;
                real v = (xx >= 0 && xx < width) ? (real)img[(size_t)y * width + xx] : 0;
                a += v;
                b += v * v;
            }
            row_i[(size_t)y * width + x] = a;
            row_ii[(size_t)y * width + x] = b;
        }
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            real a = 0, b = 0;
            for (int k = -half_window; k <= half_window; ++k) {
                int yy = y + k;
                if (yy < 0 || yy >= height) continue;
                a += row_i[(size_t)yy * width + x];
                b += row_ii[(size_t)yy * width + x];
            }
            sum_i[(size_t)y * width + x] = (double)a;
            sum_ii[(size_t)y * width + x] = (double)b;
        }
    free(row_i);
    free(row_ii);
}

/* ------------------------------------------------------------------------------------
 * Source fetch: tex2DLayered(allImgsTexture, u/z + 0.5, v/z + 0.5, view) with linear
 * filtering and border addressing (patchMatch.cu:192-195, :543). In the texture's
 * convention texel i sits at coordinate i + 0.5, so the +0.5 puts texel i at u/z = i.
 * ---------------------------------------------------------------------------------- */
static inline real texel(const float *img, int w, int h, int x, int y)
{
    return (x >= 0 && x < w && y >= 0 && y < h) ? (real)img[(size_t)y * w + x] : (real)0;
}

/* Texture-unit weight: a fraction rounded half-up to a multiple of 1/256 (measured on the
 * GB300's texture units; the CUDA programming guide documents 8 fractional bits). */
static inline real q8(real f) { return R_FLOOR(f * (real)256 + (real)0.5) / (real)256; }

static inline real sample_bilinear(const float *img, int w, int h, real xs, real ys, int hw)
{
    if (!(xs > (real)-1 && xs < (real)w && ys > (real)-1 && ys < (real)h)) return 0;
    real fx = R_FLOOR(xs), fy = R_FLOOR(ys);
    int x0 = (int)fx, y0 = (int)fy;
    real ax = xs - fx, ay = ys - fy;
    real t00 = texel(img, w, h, x0, y0), t10 = texel(img, w, h, x0 + 1, y0);
    real t01 = texel(img, w, h, x0, y0 + 1), t11 = texel(img, w, h, x0 + 1, y0 + 1);
    if (hw) {
        const real a = q8(ax), b = q8(ay), ab = q8(a * b);
        return t00 * ((real)1 - a - b + ab) + t10 * (a - ab) + t01 * (b - ab) + t11 * ab;
    }
    return ((real)1 - ax) * ((real)1 - ay) * t00 + ax * ((real)1 - ay) * t10 +
           ((real)1 - ax) * ay * t01 + ax * ay * t11;
}

void pmo_sample(const pmo_problem *p, int view, int n, const float *xs, const float *ys,
                double *out)
{
    for (int i = 0; i < n; ++i)
        out[i] = (double)sample_bilinear(p->src[view], p->src_width[view], p->src_height[view],
                                         (real)xs[i], (real)ys[i], p->sampler);
}

/* ------------------------------------------------------------------------------------
 * Single-precision coordinate arithmetic of the texture-filtering sampler (sampler 1). The
 * texture unit's 1/256 weights are discontinuous in the coordinate, so FP64 coordinates would
 * round an occasional weight the other way than the engine's FP32 ones. The reference itself
 * forms these coordinates in float (patchMatch.cu:462-505, :543); sampler 1 follows the
 * engine's explicit single-precision sequence: fused multiply-adds and correctly rounded
 * reciprocals and products. An exact product of two floats fits a double, so one rounding
 * of a double sum gives the fused result (double rounding differs only in rare halfway ties).
 * ---------------------------------------------------------------------------------- */
static inline float f_fma(float a, float b, float c) { return (float)((double)a * (double)b + (double)c); }
static inline float f_mul(float a, float b) { return (float)((double)a * (double)b); }
static inline float f_add(float a, float b) { return (float)((double)a + (double)b); }
static inline float f_rcp(float a) { return (float)(1.0 / (double)a); }

static float device_scale(const pmo_problem *p, int x)
{
    return f_add(f_mul((float)p->orientation[0],
                       f_fma((float)p->inv_k[0], f_add((float)x, 0.5f), (float)p->inv_k[1])),
                 (float)p->orientation[2]);
}

/* The texture's half-texel offset folded into the first two rows of T, evaluated at the
 * window origin (ox, oy): out[0..8] = c0 (3), c1 (3), base (3). */
static void warp_tail(float t[9], float ox, float oy, float out[9])
{
    for (int i = 0; i < 3; ++i) {
        t[i] = f_fma(0.5f, t[6 + i], t[i]);
        t[3 + i] = f_fma(0.5f, t[6 + i], t[3 + i]);
    }
    out[0] = t[0]; out[1] = t[3]; out[2] = t[6];
    out[3] = t[1]; out[4] = t[4]; out[5] = t[7];
    out[6] = f_fma(t[0], ox, f_fma(t[1], oy, t[2]));
    out[7] = f_fma(t[3], ox, f_fma(t[4], oy, t[5]));
    out[8] = f_fma(t[6], ox, f_fma(t[7], oy, t[8]));
}

/* T = H1 - s H2 with s = 1/(depth scale). */
static void device_warp(const pmo_problem *p, int view, float depth, float scale, float ox,
                        float oy, float out[9])
{
    const double *hh = p->hh + 18 * (size_t)view;
    const float s = f_rcp(f_mul(depth, scale));
    float t[9];
    for (int i = 0; i < 9; ++i) t[i] = f_fma(-s, (float)hh[9 + i], (float)hh[i]);
    warp_tail(t, ox, oy, out);
}

/* Slanted-plane mode: g = (a ik00, b ik11, a ik02 + b ik12 + 1) = K_r^-T n for n = (a, b, 1),
 * and the plane scale s = g . (x + 1/2, y + 1/2, 1) floored at PMO_SCALE_MIN, in the engine's
 * single-precision steps. */
typedef struct { float g0, g1, g2, s; } plane_terms_t;

static inline plane_terms_t plane_terms(const pmo_problem *p, float a, float b, int x, int y)
{
    plane_terms_t r;
    r.g0 = f_mul(a, (float)p->inv_k[0]);
    r.g1 = f_mul(b, (float)p->inv_k[2]);
    r.g2 = f_fma(a, (float)p->inv_k[1], f_fma(b, (float)p->inv_k[3], 1.0f));
    const float s = f_fma(r.g0, f_add((float)x, 0.5f), f_fma(r.g1, f_add((float)y, 0.5f), r.g2));
    r.s = s < PMO_SCALE_MIN ? PMO_SCALE_MIN : s;
    return r;
}

/* T = H1 - e g^T / (depth s), each product e_r g_c rounded to float. */
static void device_warp_plane(const pmo_problem *p, int view, float depth, plane_terms_t G,
                              float ox, float oy, float out[9])
{
    const double *hh = p->hh + 18 * (size_t)view;
    const double *e = p->ee + 3 * (size_t)view;
    const float inv = f_rcp(f_mul(depth, G.s));
    const float g[3] = {G.g0, G.g1, G.g2};
    float t[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            t[3 * r + c] = f_fma(-inv, f_mul((float)e[r], g[c]), (float)hh[3 * r + c]);
    warp_tail(t, ox, oy, out);
}

/* Plane scale s = n^T K^-1 (x + 1/2, y + 1/2, 1): patchMatch.cu:798-800, :876-883 with
 * orientation[1] = 0 (the reference accumulates it row by row; this evaluates it). */
static inline real plane_scale(const pmo_problem *p, int x)
{
    return (real)(p->orientation[0] * (p->inv_k[0] * (x + 0.5) + p->inv_k[1]) + p->orientation[2]);
}

/* ------------------------------------------------------------------------------------
 * computeNCC<W> (patchMatch.cu:433-611): 1 - NCC over the in-bounds pixels of the
 * (2hw+1)^2 window centred on reference pixel (x, y), the source sampled through the
 * plane-induced homography T = H1 - H2 / depth / scale (:462-474).
 *   axis 0: the sweep's column axis is image x (isRotated = false, vertical sweeps);
 *   axis 1: the sweep's column axis is image y (isRotated = true, horizontal sweeps and
 *           computeAllCostGivenDepth).
 * The window's reference values advance only over in-bounds columns of the sweep's
 * column axis (refImg_I_Ind++, :546): with quirks on, leading out-of-bounds columns
 * shift the reference samples paired with the source samples (texture border 0).
 * Result: 2 if sum(I'^2) == 0; variances below 1e-5 clamp to 0 (:599-600); 1 if their
 * product is 0; else 1 - (sum(I I') - sum(I) sum(I')/n) / sqrt(c1 c2).
 * ---------------------------------------------------------------------------------- */
static real ncc_eval(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                     int x, int y, int view, real depth, int axis, real scale, const float *plane)
{
    const int hw = p->half_window, w = 2 * hw + 1, W = p->width, H = p->height;
    const double *hh = p->hh + 18 * (size_t)view;
    real t[9];
    plane_terms_t G = {0, 0, 0, 0};
    if (plane) {
        /* slanted plane (a, b) = plane[0..1]: T = H1 - e g^T / (depth s) */
        G = plane_terms(p, plane[0], plane[1], x, y);
        const double *e = p->ee + 3 * (size_t)view;
        const real g[3] = {(real)G.g0, (real)G.g1, (real)G.g2};
        const real rho = depth * (real)G.s;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) t[3 * r + c] = (real)hh[3 * r + c] - (real)e[r] * g[c] / rho;
    } else {
        for (int i = 0; i < 9; ++i) t[i] = (real)hh[i] - (real)hh[9 + i] / depth / scale;
    }
    const float *src = p->src[view];
    const int sw = p->src_width[view], sh = p->src_height[view];
    float dw[9];
    if (p->sampler == 1) {
        if (plane)
            device_warp_plane(p, view, (float)depth, G, (float)(x - hw) + 0.5f, (float)(y - hw) + 0.5f, dw);
        else
            device_warp(p, view, (float)depth, device_scale(p, x), (float)(x - hw) + 0.5f,
                        (float)(y - hw) + 0.5f, dw);
    }
    int lead = 0;
    if (p->quirks) lead = axis == 0 ? (hw - x > 0 ? hw - x : 0) : (hw - y > 0 ? hw - y : 0);

    real s_j = 0, s_jj = 0, s_ij = 0;
    int n = 0;
    for (int dy = 0; dy < w; ++dy) {
        int yy = y - hw + dy;
        if (yy < 0 || yy >= H) continue;
        real r_j = 0, r_jj = 0, r_ij = 0;
        for (int dx = 0; dx < w; ++dx) {
            int xx = x - hw + dx;
            if (xx < 0 || xx >= W) continue;
            real jv;
            if (p->sampler == 1) {
                const float fdx = (float)dx, fdy = (float)dy;
                /* the engine walks down window column dx: column base, then row dy */
                const float pu = f_fma(dw[3], fdy, f_fma(dw[0], fdx, dw[6]));
                const float pv = f_fma(dw[4], fdy, f_fma(dw[1], fdx, dw[7]));
                float pz = f_fma(dw[5], fdy, f_fma(dw[2], fdx, dw[8]));
                pz = fabsf(pz) < 1e-20f ? 1e-20f : pz;
                const float r = f_rcp(pz);
                /* texture coordinates carry the half-texel offset; texel i sits at i + 1/2 */
                jv = sample_bilinear(src, sw, sh, (real)((double)f_mul(pu, r) - 0.5),
                                     (real)((double)f_mul(pv, r) - 0.5), 1);
            } else {
                real px = (real)xx + (real)0.5, py = (real)yy + (real)0.5;
                real u = t[0] * px + t[1] * py + t[2];
                real v = t[3] * px + t[4] * py + t[5];
                real z = t[6] * px + t[7] * py + t[8];
                jv = sample_bilinear(src, sw, sh, u / z, v / z, 0);
            }
            int rx = axis == 0 ? xx - lead : xx;
            int ry = axis == 0 ? yy : yy - lead;
            real iv = texel(p->ref, W, H, rx, ry);
            r_j += jv;
            r_jj += jv * jv;
            r_ij += iv * jv;
            ++n;
        }
        s_j += r_j;
        s_jj += r_jj;
        s_ij += r_ij;
    }
    if (s_jj == 0) return 2;
    real si = (real)sum_i[(size_t)y * W + x], sii = (real)sum_ii[(size_t)y * W + x];
    real rn = (real)n;
    real c1 = sii - si * si / rn;
    real c2 = s_jj - s_j * s_j / rn;
    c1 = c1 < (real)0.00001 ? (real)0 : c1;
    c2 = c2 < (real)0.00001 ? (real)0 : c2;
    real c = R_SQRT(c1 * c2);
    if (c == 0) return 1;
    return (real)1 - (s_ij - si * s_j / rn) / c;
}

double pmo_ncc(const pmo_problem *p, const double *sum_i, const double *sum_ii,
               int x, int y, int view, double depth, int axis)
{
    return (double)ncc_eval(p, sum_i, sum_ii, x, y, view, (real)depth, axis, plane_scale(p, x), NULL);
}

double pmo_ncc_plane(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                     int x, int y, int view, double depth, float a, float b, int axis)
{
    const float ab[2] = {a, b};
    return (double)ncc_eval(p, sum_i, sum_ii, x, y, view, (real)depth, axis, 0, ab);
}

void pmo_ncc_plane_batch(const pmo_problem *p, const double *sum_i, const double *sum_ii, int n,
                         const int *xs, const int *ys, const int *views, const double *depths,
                         const float *slopes, const int *axes, double *out)
{
    #pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; ++i)
        out[i] = (double)ncc_eval(p, sum_i, sum_ii, xs[i], ys[i], views[i], (real)depths[i], axes[i], 0,
                                  slopes + 2 * (size_t)i);
}

void pmo_ncc_batch(const pmo_problem *p, const double *sum_i, const double *sum_ii, int n,
                   const int *xs, const int *ys, const int *views, const double *depths,
                   const int *axes, double *out)
{
    #pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; ++i)
        out[i] = pmo_ncc(p, sum_i, sum_ii, xs[i], ys[i], views[i], depths[i], axes[i]);
}

static long long refine_impl(const pmo_problem *p, const double *sum_i, const double *sum_ii, double *depth,
                             const float *slopes, const unsigned char *view_sel, int num_samples, int trials,
                             float sigma, uint32_t sweep_id, int axis)
{
    const int W = p->width, H = p->height, V = p->n_src;
    const int npix = W * H;
    const float d_lo = (float)p->depth_near;
    const float d_hi = f_add(d_lo, (float)((double)(float)p->depth_far - (double)d_lo));
    const float sqrt3 = (float)1.7320508075688772;
    long long evals = 0;
    #pragma omp parallel for schedule(dynamic, 64) reduction(+ : evals)
    for (int pix = 0; pix < npix; ++pix) {
        const int x = pix % W, y = pix / W;
        int views[32], nv = 0;
        for (int k = 0; k < num_samples && k < 32; ++k) {
            const int v = view_sel[(size_t)k * npix + pix];
            if (v < V) views[nv++] = v;
        }
        if (nv == 0) continue;
        const real scale = plane_scale(p, x);
        const float *pl = slopes ? slopes + 2 * (size_t)pix : NULL;
        const float d0 = (float)depth[pix];
        real best_cost = 0;
        for (int k = 0; k < nv; ++k) best_cost += ncc_eval(p, sum_i, sum_ii, x, y, views[k], (real)d0, axis, scale, pl);
        best_cost /= (real)nv;
        evals += nv;
        float best = d0;
        for (int t = 0; t < trials; ++t) {
            const uint32_t ctr[4] = {(uint32_t)pix, sweep_id, ((uint32_t)PMO_RNG_REFINE << 16) | (uint32_t)t,
                                     p->batch_id};
            const uint32_t key[2] = {(uint32_t)p->seed, (uint32_t)(p->seed >> 32)};
            uint32_t o[4];
            pmo_philox4x32_10(ctr, key, o);
            float u[4];
            for (int k = 0; k < 4; ++k) u[k] = (float)((o[k] >> 8) + 1u) * (1.0f / 16777216.0f);
            const float z = f_add(f_add(f_add(u[0], u[1]), f_add(u[2], u[3])), -2.0f);
            const float dn = f_add(d0, f_mul(f_mul(z, sqrt3), sigma));
            if (!(dn >= d_lo && dn <= d_hi)) continue;
            real c = 0;
            for (int k = 0; k < nv; ++k) c += ncc_eval(p, sum_i, sum_ii, x, y, views[k], (real)dn, axis, scale, pl);
            c /= (real)nv;
            evals += nv;
            if (c < best_cost) {
                best_cost = c;
                best = dn;
            }
        }
        depth[pix] = (double)best;
    }
    return evals;
}

long long pmo_refine(const pmo_problem *p, const double *sum_i, const double *sum_ii, double *depth,
                     const unsigned char *view_sel, int num_samples, int trials, float sigma,
                     uint32_t sweep_id, int axis)
{
    return refine_impl(p, sum_i, sum_ii, depth, NULL, view_sel, num_samples, trials, sigma, sweep_id, axis);
}

long long pmo_refine_planes(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                            double *depth, const float *slopes, const unsigned char *view_sel,
                            int num_samples, int trials, float sigma, uint32_t sweep_id, int axis)
{
    return refine_impl(p, sum_i, sum_ii, depth, slopes, view_sel, num_samples, trials, sigma, sweep_id, axis);
}

/* ------------------------------------------------------------------------------------
 * HMM view-selection messages, computeMessageBackward / computeMessageForward
 * (patchMatch.cu:669-715). A cost of exactly 2 (window outside the source) is replaced
 * by 2*U(0,1] (:680-682, :706-707). Emission e = exp(-c^2 / (2 alpha^2)) (evaluated in
 * double by the reference because of the -0.5 literal), uniform emission
 * u = exp(-0.83^2 / (2 alpha^2)), transition 0.999 / (1 - 0.999).
 * ---------------------------------------------------------------------------------- */
static inline real alpha_sq(float sp_alpha) { return (real)(sp_alpha * sp_alpha); }

static inline real uniform_emission(real a2)
{
    return R_EXP((real)-0.5 * UNIFORM_EMISSION_COST * UNIFORM_EMISSION_COST / a2);
}

/* Values below the smallest normal float flush to zero (the reference's float storage
 * under --use_fast_math). */
static inline real ftz(real x) { return (x < (real)1.17549435e-38f && x > (real)-1.17549435e-38f) ? (real)0 : x; }

static inline real emission(real c, real a2)
{
    return ftz((real)(float)R_EXP((real)-0.5 * c * c / a2));
}

static inline real msg_backward(real m, real e, real u)
{
    real zn0 = m * e * FIX_STATE_PROB + ((real)1 - m) * u * CHANGE_STATE_PROB;
    real zn1 = m * e * CHANGE_STATE_PROB + ((real)1 - m) * u * FIX_STATE_PROB;
    return ftz(zn0 / (zn0 + zn1));
}

static inline real msg_forward(real m, real e, real u)
{
    real zn0 = (m * FIX_STATE_PROB + ((real)1 - m) * CHANGE_STATE_PROB) * e;
    real zn1 = (m * CHANGE_STATE_PROB + ((real)1 - m) * FIX_STATE_PROB) * u;
    return ftz(zn0 / (zn0 + zn1));
}

double pmo_msg_forward(double msg, double cost, double u_if_two, float sp_alpha)
{
    real a2 = alpha_sq(sp_alpha);
    real c = (real)cost;
    if (c == (real)2) c = (real)u_if_two * (real)2;
    return (double)msg_forward((real)msg, emission(c, a2), uniform_emission(a2));
}

double pmo_msg_backward(double msg, double cost, double u_if_two, float sp_alpha)
{
    real a2 = alpha_sq(sp_alpha);
    real c = (real)cost;
    if (c == (real)2) c = (real)u_if_two * (real)2;
    return (double)msg_backward((real)msg, emission(c, a2), uniform_emission(a2));
}

/* findMinCost (patchMatch.cu:613-618): ties go to the later index. */
static inline int find_min_cost(const real c[3])
{
    int idx = c[0] < c[1] ? 0 : 1;
    return c[idx] < c[2] ? idx : 2;
}

int pmo_find_min_cost(const double cost[3])
{
    real c[3] = {(real)cost[0], (real)cost[1], (real)cost[2]};
    return find_min_cost(c);
}

/* ------------------------------------------------------------------------------------
 * Initial depth, generate_kernel_float (array2d_wrapper.cu:3-20):
 * depth = (1 - U(0,1]) * (far - near) + near, in float like the reference's depth map.
 * ---------------------------------------------------------------------------------- */
void pmo_init_depth(const pmo_problem *p, double *depth)
{
    const int n = p->width * p->height;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const float u = p->rng_stream ? (float)stream_draw(p, (uint32_t)i)
                                      : (float)draw(p, i, 0xFFFFFFFFu, PMO_RNG_INIT, 0);
        depth[i] = float_depth((double)(1.0f - u), p->depth_near, p->depth_far);
    }
}

/* Slanted-plane mode: initial slopes uniform in [-PMO_SLOPE_DRAW, PMO_SLOPE_DRAW]^2 from words
 * 1 and 2 of the initial-depth counter (word 0 is the depth). */
void pmo_init_planes(const pmo_problem *p, float *slopes)
{
    const int n = p->width * p->height;
    const uint32_t key[2] = {(uint32_t)p->seed, (uint32_t)(p->seed >> 32)};
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const uint32_t ctr[4] = {(uint32_t)i, 0xFFFFFFFFu, (uint32_t)PMO_RNG_INIT << 16, p->batch_id};
        uint32_t o[4];
        pmo_philox4x32_10(ctr, key, o);
        for (int k = 0; k < 2; ++k) {
            const float u = (float)((o[1 + k] >> 8) + 1u) * (1.0f / 16777216.0f);
            slopes[2 * (size_t)i + k] = f_mul(PMO_SLOPE_DRAW, f_fma(2.0f, u, -1.0f));
        }
    }
}

static long long initial_costs_impl(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                                    const double *depth, const float *slopes, double *cost)
{
    const int W = p->width, H = p->height, V = p->n_src;
    #pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            real scale = plane_scale(p, x);
            size_t pix = (size_t)y * W + x;
            const float *pl = slopes ? slopes + 2 * pix : NULL;
            for (int v = 0; v < V; ++v)
                cost[pix * V + v] = (double)ncc_eval(p, sum_i, sum_ii, x, y, v,
                                                     (real)depth[pix], 1, scale, pl);
        }
    return (long long)W * H * V;
}

long long pmo_initial_costs_planes(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                                   const double *depth, const float *slopes, double *cost)
{
    return initial_costs_impl(p, sum_i, sum_ii, depth, slopes, cost);
}

/* computeAllCostGivenDepth<W> (patchMatch.cu:775-816): every view's cost at the current
 * depth. The reference runs it on the transposed maps (isRotated = true, :338-343). */
long long pmo_initial_costs(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                            const double *depth, double *cost)
{
    return initial_costs_impl(p, sum_i, sum_ii, depth, NULL, cost);
}

/* ------------------------------------------------------------------------------------
 * One directional sweep, topToDown<W> / downToTop<W> (patchMatch.cu:818-1209).
 * A "line" is one column of the sweep (one reference thread); steps run along it in
 * processing order. Per line:
 *  1. backward messages over the whole line in reverse processing order; the message
 *     before a step's update is stored for that step (:856-869, :1050-1059);
 *  2. forward message at the first step from 0.5 (:872-874, :1063-1067);
 *  3. for every later step: forward message with the old costs (:905), posterior
 *     q = a b / (a b + (1-a)(1-b)) turned into a CDF (:909-923); random depth (:937);
 *     S view samples, the first view whose CDF value is >= u (with replacement,
 *     :940-961); average costs of the previous step's depth, the current depth and the
 *     random depth (:965-973); argmin with ties to the later index (:975); write the
 *     depth; refresh every view's cost at the chosen depth unless the current depth
 *     won (:983-994); forward message from the previous step's message with the new
 *     costs (:996-999). The final sweep of the last iteration records the sampled
 *     views (:1159-1163).
 * Returns the number of NCC evaluations the algorithm performed.
 * ---------------------------------------------------------------------------------- */
static long long sweep_impl(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                            double *depth, float *slopes, double *cost, int dir, uint32_t sweep_id,
                            int num_samples, unsigned char *view_sel, int line_begin, int line_end)
{
    const int W = p->width, H = p->height, V = p->n_src, S = num_samples;
    const int rotated = (dir == PMO_DIR_LR || dir == PMO_DIR_RL);
    const int forward = (dir == PMO_DIR_LR || dir == PMO_DIR_TB);
    const int nlines = rotated ? H : W;
    const int nsteps = rotated ? W : H;
    const int axis = rotated ? 1 : 0;
    const real a2 = alpha_sq(p->sp_alpha);
    const real u_emit = uniform_emission(a2);
    const float perturb = p->perturbation > 0.0f ? p->perturbation * exp2f(-0.25f * (float)sweep_id) : 0.0f;
    /* slanted-plane mode: the local search's widths in this sweep, the depth range in float */
    const int planar = slopes != NULL;
    const float dstep = p->plane_depth_step * exp2f(-0.25f * (float)sweep_id);
    const float sstep = p->plane_slope_step * exp2f(-0.25f * (float)sweep_id);
    const float d_lo = (float)p->depth_near;
    const float d_hi = f_add(d_lo, (float)((double)(float)p->depth_far - (double)d_lo));
    if (line_begin < 0) line_begin = 0;
    if (line_end < 0 || line_end > nlines) line_end = nlines;
    if (p->rng_stream && (planar || perturb > 0.0f || !p->rng_counts)) return -1;
    long long evals = 0;

    #pragma omp parallel reduction(+ : evals)
    {
        real *beta_all = (real *)malloc(sizeof(real) * (size_t)nsteps * V);
        real *beta = (real *)malloc(sizeof(real) * V);
        real *alpha = (real *)malloc(sizeof(real) * V);
        real *cdf = (real *)malloc(sizeof(real) * V);
        real *c_old = (real *)malloc(sizeof(real) * V);
        int *vsel = (int *)malloc(sizeof(int) * (S > 0 ? S : 1));

        #pragma omp for schedule(dynamic, 1)
        for (int line = line_begin; line < line_end; ++line) {
#define COORD(k) (forward ? (k) : (nsteps - 1 - (k)))
#define PX(k) (rotated ? COORD(k) : line)
#define PY(k) (rotated ? line : COORD(k))
            /* stream mode: the line's random state (the first pixel of its row or column) */
            const uint32_t state = rotated ? (uint32_t)line * (uint32_t)W : (uint32_t)line;
#define DRAW(pix, purpose, sub) (p->rng_stream ? stream_draw(p, state) : draw(p, pix, sweep_id, purpose, sub))
            /* 1. backward messages */
            for (int v = 0; v < V; ++v) beta[v] = (real)0.5;
            for (int k = nsteps - 1; k >= 0; --k) {
                int pix = PY(k) * W + PX(k);
                for (int v = 0; v < V; ++v) {
                    beta_all[(size_t)k * V + v] = beta[v];
                    real c = (real)cost[(size_t)pix * V + v];
                    if (c == (real)2) c = DRAW(pix, PMO_RNG_BWD, v) * (real)2;
                    beta[v] = msg_backward(beta[v], emission(c, a2), u_emit);
                }
            }
            /* 2. forward message at the first step */
            {
                int pix = PY(0) * W + PX(0);
                for (int v = 0; v < V; ++v) {
                    real c = (real)cost[(size_t)pix * V + v];
                    if (c == (real)2) c = DRAW(pix, PMO_RNG_FWD_POST, v) * (real)2;
                    alpha[v] = msg_forward((real)0.5, emission(c, a2), u_emit);
                }
            }
            real d_former = (real)depth[PY(0) * W + PX(0)];
            /* slanted-plane mode: the previous step's plane and pixel */
            float a_former = 0, b_former = 0;
            int x_former = PX(0), y_former = PY(0);
            if (planar) {
                a_former = slopes[2 * ((size_t)PY(0) * W + PX(0))];
                b_former = slopes[2 * ((size_t)PY(0) * W + PX(0)) + 1];
            }
            /* 3. propagation */
            for (int k = 1; k < nsteps; ++k) {
                const int x = PX(k), y = PY(k);
                const int pix = y * W + x;
                const real scale = plane_scale(p, x);
                double *cpix = cost + (size_t)pix * V;
                for (int v = 0; v < V; ++v) {
                    real c = (real)cpix[v];
                    c_old[v] = c;
                    if (c == (real)2) c = DRAW(pix, PMO_RNG_FWD_PRE, v) * (real)2;
                    real a = msg_forward(alpha[v], emission(c, a2), u_emit);
                    real b = beta_all[(size_t)k * V + v];
                    real zn0 = a * b;
                    real zn1 = ((real)1 - a) * ((real)1 - b);
                    cdf[v] = ftz(zn0 / (zn0 + zn1));
                }
                for (int v = 1; v < V; ++v) cdf[v] += cdf[v - 1];
                for (int v = 0; v < V; ++v) cdf[v] /= cdf[V - 1];

                const real d_cur = (real)depth[pix];
                real d_rand;
                /* plane hypotheses (slanted-plane mode): former, current, random */
                float pl_f[2] = {0, 0}, pl_c[2] = {0, 0}, pl_r[2] = {0, 0};
                real d_prop = d_former;
                {
                    const uint32_t ctr[4] = {(uint32_t)pix, sweep_id, ((uint32_t)PMO_RNG_RAND_DEPTH << 16), p->batch_id};
                    const uint32_t key[2] = {(uint32_t)p->seed, (uint32_t)(p->seed >> 32)};
                    uint32_t o[4];
                    pmo_philox4x32_10(ctr, key, o);
                    float uw[4];
                    for (int k = 0; k < 4; ++k) uw[k] = (float)((o[k] >> 8) + 1u) * (1.0f / 16777216.0f);
                    if (p->rng_stream) uw[0] = (float)stream_draw(p, state);  /* :937 */
                    const float u = uw[0], u2 = uw[1];
                    d_rand = (real)float_depth((double)u, p->depth_near, p->depth_far);
                    if (planar) {
                        /* the previous step's plane carried to this pixel: d s_prev / s_here */
                        pl_f[0] = a_former;
                        pl_f[1] = b_former;
                        const plane_terms_t gq = plane_terms(p, a_former, b_former, x_former, y_former);
                        const plane_terms_t gp = plane_terms(p, a_former, b_former, x, y);
                        float df = f_mul((float)d_former, f_mul(gq.s, f_rcp(gp.s)));
                        df = df < d_lo ? d_lo : (df > d_hi ? d_hi : df);
                        d_prop = (real)df;
                        pl_c[0] = slopes[2 * (size_t)pix];
                        pl_c[1] = slopes[2 * (size_t)pix + 1];
                        if (u2 < 0.33333334f) {
                            /* uniform depth, current slopes (the reference's random depth) */
                            pl_r[0] = pl_c[0];
                            pl_r[1] = pl_c[1];
                        } else if (u2 < 0.6666667f) {
                            /* current depth, uniform slopes */
                            d_rand = d_cur;
                            pl_r[0] = f_mul(PMO_SLOPE_DRAW, f_fma(2.0f, uw[2], -1.0f));
                            pl_r[1] = f_mul(PMO_SLOPE_DRAW, f_fma(2.0f, uw[3], -1.0f));
                        } else {
                            /* local perturbation of depth and slopes */
                            float dr = f_mul((float)d_cur, f_fma(dstep, f_fma(2.0f, u, -1.0f), 1.0f));
                            d_rand = (real)(dr < d_lo ? d_lo : (dr > d_hi ? d_hi : dr));
                            for (int k = 0; k < 2; ++k) {
                                const float sl = f_fma(sstep, f_fma(2.0f, uw[2 + k], -1.0f), pl_c[k]);
                                pl_r[k] = sl < -PMO_SLOPE_MAX ? -PMO_SLOPE_MAX : (sl > PMO_SLOPE_MAX ? PMO_SLOPE_MAX : sl);
                            }
                        }
                    } else if (perturb > 0.0f && u2 >= 0.5f) {
                        /* the engine's local search, in its single-precision arithmetic */
                        const float lo = (float)p->depth_near;
                        const float hi = f_add(lo, (float)((double)(float)p->depth_far - (double)lo));
                        float dr = f_mul((float)d_cur, f_fma(perturb, f_fma(2.0f, u, -1.0f), 1.0f));
                        dr = dr < lo ? lo : (dr > hi ? hi : dr);
                        d_rand = (real)dr;
                    }
                }
                const float *plf = planar ? pl_f : NULL, *plr = planar ? pl_r : NULL;
                real c3[3] = {0, 0, 0};
                int tested = 0;
                for (int j = 0; j < S; ++j) {
                    real u = DRAW(pix, PMO_RNG_SAMPLE, j);
                    int view = -1;
                    for (int v = 0; v < V; ++v)
                        if (u <= cdf[v]) { view = v; break; }
                    vsel[j] = view;
                    if (view < 0) continue;
                    ++tested;
                    c3[0] += ncc_eval(p, sum_i, sum_ii, x, y, view, d_prop, axis, scale, plf);
                    c3[1] += c_old[view];
                    c3[2] += ncc_eval(p, sum_i, sum_ii, x, y, view, d_rand, axis, scale, plr);
                }
                evals += 2 * tested;
                int idx = 1;
                if (tested > 0) {
                    real inv = (real)1 / (real)tested;
                    c3[0] *= inv; c3[1] *= inv; c3[2] *= inv;
                    idx = find_min_cost(c3);
                }
                const real best = idx == 0 ? d_prop : (idx == 1 ? d_cur : d_rand);
                const float *pl_best = idx == 0 ? pl_f : (idx == 1 ? pl_c : pl_r);
                depth[pix] = (double)best;
                d_former = best;
                if (planar) {
                    a_former = slopes[2 * (size_t)pix] = pl_best[0];
                    b_former = slopes[2 * (size_t)pix + 1] = pl_best[1];
                    x_former = x;
                    y_former = y;
                }
                if (idx != 1) {
                    for (int v = 0; v < V; ++v)
                        cpix[v] = (double)ncc_eval(p, sum_i, sum_ii, x, y, v, best, axis, scale,
                                                   planar ? pl_best : NULL);
                    evals += V;
                }
                for (int v = 0; v < V; ++v) {
                    real c = (real)cpix[v];
                    if (c == (real)2) c = DRAW(pix, PMO_RNG_FWD_POST, v) * (real)2;
                    alpha[v] = msg_forward(alpha[v], emission(c, a2), u_emit);
                }
                if (view_sel)
                    for (int j = 0; j < S; ++j)
                        view_sel[(size_t)j * W * H + pix] =
                            (unsigned char)(vsel[j] < 0 ? 255 : vsel[j]);
            }
#undef COORD
#undef PX
#undef PY
#undef DRAW
        }
        free(beta_all); free(beta); free(alpha); free(cdf); free(c_old); free(vsel);
    }
    return evals;
}

long long pmo_sweep(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                    double *depth, double *cost, int dir, uint32_t sweep_id, int num_samples,
                    unsigned char *view_sel, int line_begin, int line_end)
{
    return sweep_impl(p, sum_i, sum_ii, depth, NULL, cost, dir, sweep_id, num_samples, view_sel, line_begin,
                      line_end);
}

long long pmo_sweep_planes(const pmo_problem *p, const double *sum_i, const double *sum_ii,
                           double *depth, float *slopes, double *cost, int dir, uint32_t sweep_id,
                           int num_samples, unsigned char *view_sel, int line_begin, int line_end)
{
    return sweep_impl(p, sum_i, sum_ii, depth, slopes, cost, dir, sweep_id, num_samples, view_sel, line_begin,
                      line_end);
}

/* PatchMatch::run<W> (patchMatch.cu:307-394): iteration 0 samples one view and first
 * computes every cost at the initial depth; each iteration sweeps left-to-right,
 * top-to-bottom, right-to-left, bottom-to-top; the last sweep of the last iteration
 * records the sampled views. Sweep id = 4 * iteration + direction. */
long long pmo_run(const pmo_problem *p, int iterations, int num_samples,
                  const double *sum_i, const double *sum_ii,
                  double *depth, double *cost, unsigned char *view_sel)
{
    long long evals = 0;
    pmo_init_depth(p, depth);
    for (int it = 0; it < iterations; ++it) {
        int s = it == 0 ? 1 : num_samples;
        if (it == 0) evals += pmo_initial_costs(p, sum_i, sum_ii, depth, cost);
        for (int d = 0; d < 4; ++d) {
            unsigned char *vs = (it == iterations - 1 && d == PMO_DIR_BT) ? view_sel : NULL;
            evals += pmo_sweep(p, sum_i, sum_ii, depth, cost, d, (uint32_t)(4 * it + d), s, vs,
                               0, -1);
        }
    }
    return evals;
}

long long pmo_run_planes(const pmo_problem *p, int iterations, int num_samples,
                         const double *sum_i, const double *sum_ii, double *depth, float *slopes,
                         double *cost, unsigned char *view_sel)
{
    long long evals = 0;
    pmo_init_depth(p, depth);
    pmo_init_planes(p, slopes);
    for (int it = 0; it < iterations; ++it) {
        int s = it == 0 ? 1 : num_samples;
        if (it == 0) evals += initial_costs_impl(p, sum_i, sum_ii, depth, slopes, cost);
        for (int d = 0; d < 4; ++d) {
            unsigned char *vs = (it == iterations - 1 && d == PMO_DIR_BT) ? view_sel : NULL;
            evals += sweep_impl(p, sum_i, sum_ii, depth, slopes, cost, d, (uint32_t)(4 * it + d), s, vs, 0, -1);
        }
    }
    return evals;
}

int pmo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int pmo_real_bytes(void) { return (int)sizeof(real); }
