/*
 * ref_host_shim.h -- host stand-ins for the CUDA device-language features that the
 * reference's kernels use, so that those kernels (extracted line for line from the
 * reference's sources by oracle/ref_extract.sh) compile with g++ and run on the CPU.
 * TEST INFRASTRUCTURE ONLY: the reference run this way pins the oracle (pm_oracle.c).
 *
 * What each stand-in models:
 *  - __global__ / __device__ / __constant__ are empty; __shared__ is `static`: a kernel's
 *    shared arrays are shared by the threads of the block that runs (blocks run one after
 *    another; ref_host.cpp runs a block's 32 threads as 32 host threads).
 *  - threadIdx / blockIdx are per host thread; blockDim is the launch's.
 *  - texture<T, type, mode> references with CUDA's defaults for a texture reference (clamp
 *    addressing, point filtering, unnormalised coordinates): the host code sets the modes the
 *    reference's host code sets. tex2DLayered reads a layered array of texels, tex2D a 2-D one
 *    (layer 0). Border addressing reads 0 outside the array, clamp addressing the nearest edge
 *    texel. Point or linear filtering in CUDA's
 *    documented convention (texel i centred at coordinate i + 0.5; linear filtering weights
 *    the 2x2 texels around (x - 0.5, y - 0.5) by their fractions), uchar texels read as the
 *    float value / 255 (cudaReadModeNormalizedFloat). Linear weights are either exact or the
 *    texture unit's fixed-point ones (fractions and their product rounded half up to 1/256,
 *    the model the engine's hardware-sampler tests check on the GPU). The layer index is
 *    clamped to the array's layers. Point fetches outside the array's rows or with
 *    non-finite coordinates are counted (the reference reads the homography table at row -1
 *    when a view sample finds no view, patchMatch.cu:940-968).
 *  - curandState / curand_uniform (the reference's XORWOW, array2d_psng.cu): a sequential
 *    stream per state, draw k of state `id` = Philox4x32-10 of counter
 *    (id, k, PMR_STREAM_PURPOSE << 16, 0) under the problem's seed, as ((x >> 8) + 1) 2^-24
 *    in (0, 1]; the oracle's stream mode draws the same numbers.
 *
 * PMR_REAL is the precision the reference's float arithmetic runs in: float (as written) or
 * double (ref_host.cpp compiled with -DPMR_REAL=double, which also widens the extracted
 * code's `float` to double).
 */
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>


#ifndef PMR_REAL
#define PMR_REAL float
#endif
typedef PMR_REAL pmr_real;

typedef unsigned char uchar;

#define __global__
#define __device__
#define __host__
#define __constant__
#define __forceinline__ inline
#define __shared__ static

struct pmr_dim3 {
    unsigned int x, y, z;
};
extern thread_local pmr_dim3 threadIdx, blockIdx;
extern pmr_dim3 blockDim, gridDim;

enum pmr_texture_type { cudaTextureType2D = 0x02, cudaTextureType2DLayered = 0xF2 };
enum cudaTextureReadMode { cudaReadModeElementType = 0, cudaReadModeNormalizedFloat = 1 };
enum cudaTextureAddressMode { cudaAddressModeWrap, cudaAddressModeClamp, cudaAddressModeMirror, cudaAddressModeBorder };
enum cudaTextureFilterMode { cudaFilterModePoint, cudaFilterModeLinear };

/* A texture reference bound to a (layered) array of width x height texels per layer. */
template <class T, int type, cudaTextureReadMode mode>
struct texture {
    const T *data = nullptr;
    int width = 0, height = 0, layers = 0;
    cudaTextureAddressMode addressMode[3] = {cudaAddressModeClamp, cudaAddressModeClamp, cudaAddressModeClamp};
    cudaTextureFilterMode filterMode = cudaFilterModePoint;
    int normalized = 0;
    int fixed_point_weights = 0;                 /* linear filtering: 1/256 weights */
};

template <class T, int type, cudaTextureReadMode mode>
static inline pmr_real pmr_texel(const texture<T, type, mode> &t, int x, int y, int layer)
{
    if (t.addressMode[0] == cudaAddressModeClamp) x = x < 0 ? 0 : (x >= t.width ? t.width - 1 : x);
    if (t.addressMode[1] == cudaAddressModeClamp) y = y < 0 ? 0 : (y >= t.height ? t.height - 1 : y);
    if (x < 0 || y < 0 || x >= t.width || y >= t.height) return (pmr_real)0;
    const T v = t.data[((size_t)layer * t.height + y) * t.width + x];
    /* the texture unit returns a normalized texel as the float v / 255 */
    return mode == cudaReadModeNormalizedFloat ? (pmr_real)((float)v / 255.0f) : (pmr_real)v;
}

static inline pmr_real pmr_q8(pmr_real f) { return (pmr_real)floor((double)f * 256.0 + 0.5) / (pmr_real)256; }

/* Point fetches made by this host thread (only the homography table is point-filtered: 18
 * per computeNCC call, so their count / 18 is the number of NCC evaluations), and those
 * outside the table's rows. */
extern thread_local unsigned long long pmr_point_fetches, pmr_point_outside;

template <class T, int type, cudaTextureReadMode mode>
static pmr_real tex2DLayered(const texture<T, type, mode> &t, pmr_real x, pmr_real y, int layer)
{
    if (t.filterMode == cudaFilterModePoint) ++pmr_point_fetches;
    if (!isfinite((double)x) || !isfinite((double)y)) {
        if (t.filterMode == cudaFilterModePoint) ++pmr_point_outside;
        return (pmr_real)0;
    }
    layer = layer < 0 ? 0 : (layer >= t.layers ? t.layers - 1 : layer);
    if (t.filterMode == cudaFilterModePoint) {
        const double fx = floor((double)x), fy = floor((double)y);
        if (fy < 0.0 || fy >= (double)t.height) ++pmr_point_outside;
        if (t.addressMode[0] != cudaAddressModeClamp && (fx < 0.0 || fx >= (double)t.width)) return (pmr_real)0;
        if (t.addressMode[1] != cudaAddressModeClamp && (fy < 0.0 || fy >= (double)t.height)) return (pmr_real)0;
        const double cx = fx < 0.0 ? -1.0 : (fx > (double)t.width ? (double)t.width : fx);
        const double cy = fy < 0.0 ? -1.0 : (fy > (double)t.height ? (double)t.height : fy);
        return pmr_texel(t, (int)cx, (int)cy, layer);
    }
    /* linear filtering: border addressing, the reference's only linear textures */
    const pmr_real xb = x - (pmr_real)0.5, yb = y - (pmr_real)0.5;
    if (!(xb > (pmr_real)-1 && xb < (pmr_real)t.width && yb > (pmr_real)-1 && yb < (pmr_real)t.height))
        return (pmr_real)0;
    const pmr_real fx = (pmr_real)floor((double)xb), fy = (pmr_real)floor((double)yb);
    const int x0 = (int)fx, y0 = (int)fy;
    pmr_real a = xb - fx, b = yb - fy;
    const pmr_real t00 = pmr_texel(t, x0, y0, layer), t10 = pmr_texel(t, x0 + 1, y0, layer);
    const pmr_real t01 = pmr_texel(t, x0, y0 + 1, layer), t11 = pmr_texel(t, x0 + 1, y0 + 1, layer);
    if (t.fixed_point_weights) {
        a = pmr_q8(a);
        b = pmr_q8(b);
        const pmr_real ab = pmr_q8(a * b);
        return t00 * ((pmr_real)1 - a - b + ab) + t10 * (a - ab) + t01 * (b - ab) + t11 * ab;
    }
    return ((pmr_real)1 - a) * ((pmr_real)1 - b) * t00 + a * ((pmr_real)1 - b) * t10 +
           ((pmr_real)1 - a) * b * t01 + a * b * t11;
}

/* A non-layered 2-D texture reference (GaussianBlurCUDA.cu:22): layer 0 of the bound array. */
template <class T, cudaTextureReadMode mode>
static inline pmr_real tex2D(const texture<T, cudaTextureType2D, mode> &t, pmr_real x, pmr_real y)
{
    return tex2DLayered(t, x, y, 0);
}

/* __mul24: the product of the low 24 bits of a and b, each read as a signed 24-bit integer;
 * the low 32 bits of the 48-bit product. */
static inline int __mul24(int a, int b)
{
    const int64_t a24 = (int64_t)(int32_t)((uint32_t)a << 8) >> 8, b24 = (int64_t)(int32_t)((uint32_t)b << 8) >> 8;
    return (int)(uint32_t)(uint64_t)(a24 * b24);
}

/* ---- random numbers ------------------------------------------------------------------------ */
#define PMR_STREAM_PURPOSE 0x5EEDu

struct curandState {
    uint32_t id;     /* which state (the reference keeps one per pixel, array2d_psng) */
    uint32_t count;  /* draws made so far */
};

extern uint64_t pmr_seed;

static inline void pmr_philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1, n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

static inline float curand_uniform(curandState *s)
{
    uint32_t c[4] = {s->id, s->count++, PMR_STREAM_PURPOSE << 16, 0u};
    pmr_philox(c, (uint32_t)pmr_seed, (uint32_t)(pmr_seed >> 32));
    return (float)((c[0] >> 8) + 1u) * (1.0f / 16777216.0f);
}

/* The block's dynamic shared memory (topToDown / downToTop: V floats and the selected-view
 * bit words per thread). */
extern unsigned char pmr_dynamic_shared[];

/* Barrier of the running block's threads (ref_host.cpp). */
void pmr_block_barrier();
