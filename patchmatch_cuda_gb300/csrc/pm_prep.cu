// pm_prep.cu -- per-handle preparation kernels and small utilities.
//
//  u8 -> float texels (cudaReadModeNormalizedFloat of patchMatch.cu:27-28 made explicit),
//  separable prefilter (GaussianBlurCUDA.cu:39-70), reference-window box moments
//  (array2d_refImg.cu:11-67, summed in double here), FP16 texel conversion, random initial depth
//  (array2d_wrapper.cu:3-20), source sampling queries, the layered transpose
//  (cudaTranspose.h:9-46) and raw Philox output.
#include <cuda_fp16.h>

#include "pm_internal.h"

namespace pm {

namespace {

constexpr int MAX_FILTER_TAPS = 45;
struct FilterTaps {
    float w[MAX_FILTER_TAPS];
};

__global__ void u8_to_float_kernel(const uint8_t *__restrict__ in, int in_pitch,
                                   float *__restrict__ out, int w, int h)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x < w && y < h) out[(size_t)y * w + x] = (float)in[(size_t)y * in_pitch + x] / 255.0f;
}

// One 1-D pass of the separable filter; dir 0 = along x, 1 = along y. A tap outside the image
// reads the nearest edge pixel: the reference class samples a texture reference left at its
// default clamp addressing (GaussianBlurCUDA.cu:22). Taps are applied in the reference's order
// (k = -radius .. radius, weight[radius - k]).
__global__ void filter_pass_kernel(const float *__restrict__ in, float *__restrict__ out, int w,
                                   int h, int radius, int dir, const FilterTaps taps)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    float s = 0.0f;
    for (int k = -radius; k <= radius; ++k) {
        const int xx = dir == 0 ? min(max(x + k, 0), w - 1) : x;
        const int yy = dir == 0 ? y : min(max(y + k, 0), h - 1);
        s += in[(size_t)yy * w + xx] * taps.w[radius - k];
    }
    out[(size_t)y * w + x] = s;
}

// Row pass of the window box sums in double precision.
__global__ void box_rows_kernel(const float *__restrict__ img, double *__restrict__ ri,
                                double *__restrict__ rii, int w, int h, int hw)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    double a = 0.0, b = 0.0;
    for (int k = -hw; k <= hw; ++k) {
        const int xx = x + k;
        const double v = (xx >= 0 && xx < w) ? (double)img[(size_t)y * w + xx] : 0.0;
        a += v;
        b += v * v;
    }
    ri[(size_t)y * w + x] = a;
    rii[(size_t)y * w + x] = b;
}

// Column pass; also the reference variance term c1 = S_II - S_I^2 / n over the n in-bounds
// window pixels, clamped to 0 below 1e-5 like patchMatch.cu:597-599.
__global__ void box_cols_kernel(const double *__restrict__ ri, const double *__restrict__ rii,
                                float *__restrict__ si, float *__restrict__ sii,
                                float *__restrict__ c1, int w, int h, int hw)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    double a = 0.0, b = 0.0;
    for (int k = -hw; k <= hw; ++k) {
        const int yy = y + k;
        if (yy < 0 || yy >= h) continue;
        a += ri[(size_t)yy * w + x];
        b += rii[(size_t)yy * w + x];
    }
    const int nx = min(x + hw, w - 1) - max(x - hw, 0) + 1;
    const int ny = min(y + hw, h - 1) - max(y - hw, 0) + 1;
    const double v = b - a * a / (double)(nx * ny);
    si[(size_t)y * w + x] = (float)a;
    sii[(size_t)y * w + x] = (float)b;
    c1[(size_t)y * w + x] = v < 0.00001 ? 0.0f : (float)v;
}

__global__ void float_to_half_kernel(const float *__restrict__ in, __half *__restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2half_rn(in[i]);
}

__global__ void init_depth_kernel(const RefDesc *refs, int r, int npix)
{
    const RefDesc &D = refs[r];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const float4 u = draw_uniform4(D.seed, (uint32_t)i, INIT_SWEEP_ID, RNG_INIT, 0, D.batch_id);
    D.depth[i] = fmaf(1.0f - u.x, D.depth_span, D.depth_near);
    // slanted planes: slopes uniform in [-SLOPE_DRAW, SLOPE_DRAW]^2 from the same counter
    if (D.planes)
        D.slopes[i] = make_float2(__fmul_rn(SLOPE_DRAW, fmaf(2.0f, u.y, -1.0f)),
                                  __fmul_rn(SLOPE_DRAW, fmaf(2.0f, u.z, -1.0f)));
}

__global__ void sample_kernel(const RefDesc *refs, int r, int view, int n,
                              const float *__restrict__ xs, const float *__restrict__ ys,
                              float *__restrict__ out)
{
    const RefDesc &D = refs[r];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = D.hw_filter ? sample_source_hw(D.tex_layered, view, xs[i], ys[i])
                             : sample_source(D.tex[view], xs[i], ys[i], D.src_w[view], D.src_h[view]);
}

// 32x32 shared tile with one column of padding against bank conflicts; blockIdx.z = layer.
__global__ void transpose_kernel(const float *__restrict__ in, size_t in_pitch,
                                 float *__restrict__ out, size_t out_pitch, int w, int h)
{
    __shared__ float tile[32][33];
    const int layer = blockIdx.z;
    const float *lin = (const float *)((const char *)in + (size_t)layer * h * in_pitch);
    float *lout = (float *)((char *)out + (size_t)layer * w * out_pitch);
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int x = bx + threadIdx.x, y = by + j;
        if (x < w && y < h) tile[j][threadIdx.x] = *(const float *)((const char *)lin + (size_t)y * in_pitch + (size_t)x * 4);
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int ox = by + threadIdx.x, oy = bx + j;  // output column = input row
        if (ox < h && oy < w) *(float *)((char *)lout + (size_t)oy * out_pitch + (size_t)ox * 4) = tile[threadIdx.x][j];
    }
}

__global__ void philox_kernel(uint64_t seed, int n, const uint4 *__restrict__ ctr,
                              uint4 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = philox4x32_10(ctr[i], make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
}

inline dim3 grid2d(int w, int h, dim3 b) { return dim3((w + b.x - 1) / b.x, (h + b.y - 1) / b.y); }

}  // namespace

cudaError_t launch_u8_to_float(const uint8_t *in, int in_pitch, float *out, int w, int h,
                               cudaStream_t s)
{
    const dim3 b(32, 8);
    u8_to_float_kernel<<<grid2d(w, h, b), b, 0, s>>>(in, in_pitch, out, w, h);
    return cudaGetLastError();
}

cudaError_t launch_filter(const float *in, float *tmp, float *out, int w, int h, int radius,
                          const float *weights, cudaStream_t s)
{
    if (radius < 0 || 2 * radius + 1 > MAX_FILTER_TAPS) return cudaErrorInvalidValue;
    FilterTaps taps{};
    for (int i = 0; i < 2 * radius + 1; ++i) taps.w[i] = weights[i];
    const dim3 b(32, 8);
    filter_pass_kernel<<<grid2d(w, h, b), b, 0, s>>>(in, tmp, w, h, radius, 0, taps);
    filter_pass_kernel<<<grid2d(w, h, b), b, 0, s>>>(tmp, out, w, h, radius, 1, taps);
    return cudaGetLastError();
}

cudaError_t launch_box_moments(const float *img, double *row_i, double *row_ii, float *sum_i,
                               float *sum_ii, float *c1, int w, int h, int hw, cudaStream_t s)
{
    const dim3 b(32, 8);
    box_rows_kernel<<<grid2d(w, h, b), b, 0, s>>>(img, row_i, row_ii, w, h, hw);
    box_cols_kernel<<<grid2d(w, h, b), b, 0, s>>>(row_i, row_ii, sum_i, sum_ii, c1, w, h, hw);
    return cudaGetLastError();
}

cudaError_t launch_float_to_half(const float *in, void *out, int n, cudaStream_t s)
{
    float_to_half_kernel<<<(n + 255) / 256, 256, 0, s>>>(in, (__half *)out, n);
    return cudaGetLastError();
}

cudaError_t launch_init_depth(const RefDesc *refs, int r, int npix, cudaStream_t s)
{
    init_depth_kernel<<<(npix + 255) / 256, 256, 0, s>>>(refs, r, npix);
    return cudaGetLastError();
}

cudaError_t launch_sample(const RefDesc *refs, int r, int view, int n, const float *xs,
                          const float *ys, float *out, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    sample_kernel<<<(n + 255) / 256, 256, 0, s>>>(refs, r, view, n, xs, ys, out);
    return cudaGetLastError();
}

cudaError_t launch_transpose(const float *in, size_t in_pitch, float *out, size_t out_pitch,
                             int w, int h, int layers, cudaStream_t s)
{
    if (w <= 0 || h <= 0 || layers <= 0 || layers > 65535) return cudaErrorInvalidValue;
    transpose_kernel<<<dim3((w + 31) / 32, (h + 31) / 32, layers), dim3(32, 8), 0, s>>>(
        in, in_pitch, out, out_pitch, w, h);
    return cudaGetLastError();
}

cudaError_t launch_philox(uint64_t seed, int n, const uint32_t *ctr, uint32_t *out,
                          cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    philox_kernel<<<(n + 255) / 256, 256, 0, s>>>(seed, n, (const uint4 *)ctr, (uint4 *)out);
    return cudaGetLastError();
}


// Counts significands of [1, 2) and (-2, -1] (plus 2^k scalings) where rcp_nr differs from
// the correctly rounded reciprocal.
__global__ void check_rcp_kernel(int exp_shift, unsigned long long *mismatches)
{
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= (1u << 23)) return;
    unsigned bad = 0;
#pragma unroll
    for (int sign = 0; sign < 2; ++sign) {
        const float x = __uint_as_float(((uint32_t)sign << 31) | ((uint32_t)(127 + exp_shift) << 23) | m);
        bad += __float_as_uint(rcp_nr(x)) != __float_as_uint(__frcp_rn(x));
    }
    bad = __reduce_add_sync(FULL_MASK, bad);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(mismatches, (unsigned long long)bad);
}

cudaError_t launch_check_rcp(int exp_shift, unsigned long long *mismatches, cudaStream_t s)
{
    check_rcp_kernel<<<(1u << 23) / 256, 256, 0, s>>>(exp_shift, mismatches);
    return cudaGetLastError();
}


// Texture-filtering throughput of a layered u8 texture in the NCC's access pattern (half-warps
// of 16 adjacent columns, 15 rows per loop, coordinates kept inside the texture): the peak the
// sweep kernel's sample rate is compared with.
__global__ void tex_peak_kernel(cudaTextureObject_t tex, int layers, int w, int h, int iters, float *sink)
{
    const int lane = threadIdx.x & 31, half = lane >> 4, c = lane & 15;
    const unsigned gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    float acc = 0.0f;
    unsigned s = gw * 2654435761u + 12345u;
    for (int it = 0; it < iters; ++it) {
        s = s * 1664525u + 1013904223u;
        const float x0 = 20.0f + (float)((s >> 8) % (unsigned)(w - 60)) + 0.37f * half;
        const float y0 = 20.0f + (float)((s >> 4) % (unsigned)(h - 60)) + 0.21f;
        const int layer = (int)((s >> 20) % (unsigned)layers);
#pragma unroll
        for (int r = 0; r < 15; ++r)
            acc += tex2DLayered<float>(tex, x0 + 1.003f * c + 0.013f * r, y0 + 0.997f * r, layer);
    }
    if (acc == -1.0f) sink[0] = acc;  // keeps the fetches; never true for these texels
}

cudaError_t measure_texture_peak(double *samples_per_s)
{
    const int W = 1280, H = 720, L = 10, threads = 256, iters = 200;
    int sms = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    if (e != cudaSuccess) return e;
    cudaArray_t arr = nullptr;
    const cudaChannelFormatDesc cd = cudaCreateChannelDesc<uint8_t>();
    e = cudaMalloc3DArray(&arr, &cd, make_cudaExtent(W, H, L), cudaArrayLayered);
    if (e != cudaSuccess) return e;
    cudaTextureObject_t tex = 0;
    float *sink = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td{};
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeNormalizedFloat;
    e = cudaCreateTextureObject(&tex, &rd, &td, nullptr);
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(float));
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    const int blocks = sms * 16;
    if (e == cudaSuccess) {
        tex_peak_kernel<<<blocks, threads>>>(tex, L, W, H, 5, sink);
        e = cudaEventRecord(a);
    }
    if (e == cudaSuccess) {
        tex_peak_kernel<<<blocks, threads>>>(tex, L, W, H, iters, sink);
        e = cudaEventRecord(b);
    }
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e == cudaSuccess) *samples_per_s = (double)blocks * threads * iters * 15 / (ms * 1e-3);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (sink) cudaFree(sink);
    if (tex) cudaDestroyTextureObject(tex);
    cudaFreeArray(arr);
    return e;
}

}  // namespace pm
