// pm_proposal.cu -- the learned proposal's image side: quarter-resolution images, the
// plane-sweep input of the network, and the initial depth map from its output. No counterpart
// in the reference, whose initialisation is a uniform random depth (array2d_wrapper.cu:3-20);
// pixels the network is not confident about keep exactly that initialisation.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pm_internal.h"

namespace pm {
namespace {

// Mean of each 4x4 block of a u8 image, scaled to [0, 1].
__global__ void quarter_kernel(const uint8_t *__restrict__ img, int pitch, int w4, int h4, float *__restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w4 || y >= h4) return;
    int s = 0;
#pragma unroll
    for (int dy = 0; dy < 4; ++dy)
#pragma unroll
        for (int dx = 0; dx < 4; ++dx) s += img[(size_t)(4 * y + dy) * pitch + 4 * x + dx];
    out[(size_t)y * w4 + x] = (float)s * (1.0f / (16.0f * 255.0f));
}

// Bilinear sample of a quarter-resolution image at continuous texel coordinates (texel j at
// j), zero outside.
__device__ __forceinline__ float bilinear(const float *img, int w, int h, float x, float y)
{
    if (!(x > -1.0f && x < (float)w && y > -1.0f && y < (float)h)) return 0.0f;
    const float fx = floorf(x), fy = floorf(y);
    const int x0 = (int)fx, y0 = (int)fy;
    const float ax = x - fx, ay = y - fy;
    auto t = [&](int xx, int yy) { return (xx >= 0 && xx < w && yy >= 0 && yy < h) ? img[(size_t)yy * w + xx] : 0.0f; };
    const float top = t(x0, y0) + ax * (t(x0 + 1, y0) - t(x0, y0));
    const float bot = t(x0, y0 + 1) + ax * (t(x0 + 1, y0 + 1) - t(x0, y0 + 1));
    return top + ay * (bot - top);
}

// Network input [hp][wp][17]: channel 0 the reference, channels 1 + 8 j + i source j warped
// onto the fronto-parallel plane at depth i of 8 (uniform in inverse depth). Quarter pixel
// (u, v) stands for the full-resolution block centre (4u + 1.5, 4v + 1.5); the homography of
// the plane z = d is T = H1 - H2 / d (normal (0, 0, 1)). Padding pixels are zero.
__global__ void sweep_input_kernel(ProposalGeom g, const float *__restrict__ ref_q,
                                   const float *__restrict__ src0, const float *__restrict__ src1,
                                   float *__restrict__ out)
{
    const int u = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y * blockDim.y + threadIdx.y;
    if (u >= g.wp || v >= g.hp) return;
    float *o = out + ((size_t)v * g.wp + u) * PROPOSAL_IN_CH;
    if (u >= g.w4 || v >= g.h4) {
        for (int c = 0; c < PROPOSAL_IN_CH; ++c) o[c] = 0.0f;
        return;
    }
    o[0] = ref_q[(size_t)v * g.w4 + u];
    const float px = 4.0f * u + 2.0f, py = 4.0f * v + 2.0f;  // pixel-centre coordinates
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const float *hh = g.hh[j];
        const float *img = j == 0 ? src0 : src1;
        for (int i = 0; i < PROPOSAL_PLANES; ++i) {
            const float inv_d = g.inv_far + ((float)i + 0.5f) * (1.0f / PROPOSAL_PLANES) * g.inv_range;
            float t[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) t[k] = hh[k] - hh[9 + k] * inv_d;
            const float x = t[0] * px + t[1] * py + t[2];
            const float y = t[3] * px + t[4] * py + t[5];
            const float z = t[6] * px + t[7] * py + t[8];
            float val = 0.0f;
            if (z > 1e-6f) {
                // full-resolution texel coordinate x / z -> quarter texel (x / z - 1.5) / 4
                val = bilinear(img, g.sw4[j], g.sh4[j], (x / z - 1.5f) * 0.25f, (y / z - 1.5f) * 0.25f);
            }
            o[1 + 8 * j + i] = val;
        }
    }
}

// Initial depth from the network's (s, confidence) map: bilinear at the pixel's quarter
// coordinate; pixels below the confidence threshold get the random initialisation of
// init_depth_kernel (the same draw).
__global__ void proposal_init_kernel(const RefDesc *refs, int r, ProposalGeom g, const float *__restrict__ prob,
                                     float threshold)
{
    const RefDesc &D = refs[r];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int npix = D.width * D.height;
    if (i >= npix) return;
    const int x = i % D.width, y = i / D.width;
    const float qx = fminf(fmaxf((x - 1.5f) * 0.25f, 0.0f), (float)(g.w4 - 1));
    const float qy = fminf(fmaxf((y - 1.5f) * 0.25f, 0.0f), (float)(g.h4 - 1));
    const int x0 = (int)qx, y0 = (int)qy;
    const int x1 = min(x0 + 1, g.w4 - 1), y1 = min(y0 + 1, g.h4 - 1);
    const float ax = qx - x0, ay = qy - y0;
    float s = 0.0f, c = 0.0f;
    const int xs[2] = {x0, x1}, ys[2] = {y0, y1};
    const float wx[2] = {1.0f - ax, ax}, wy[2] = {1.0f - ay, ay};
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const float* q = prob + ((size_t)ys[a] * g.wp + xs[b]) * 2;
            s += wy[a] * wx[b] * q[0];
            c += wy[a] * wx[b] * q[1];
        }
    float depth;
    float2 sl = make_float2(0.0f, 0.0f);  // slanted planes: fronto-parallel where predicted
    if (c >= threshold) {
        depth = 1.0f / (g.inv_far + s * g.inv_range);
        depth = fminf(fmaxf(depth, D.depth_near), D.depth_near + D.depth_span);
    } else {
        // the random initialisation (init_depth_kernel), slopes included
        const float4 u = draw_uniform4(D.seed, (uint32_t)i, INIT_SWEEP_ID, RNG_INIT, 0, D.batch_id);
        depth = fmaf(1.0f - u.x, D.depth_span, D.depth_near);
        sl = make_float2(__fmul_rn(SLOPE_DRAW, fmaf(2.0f, u.y, -1.0f)), __fmul_rn(SLOPE_DRAW, fmaf(2.0f, u.z, -1.0f)));
    }
    D.depth[i] = depth;
    if (D.planes) D.slopes[i] = sl;
}

}  // namespace

cudaError_t launch_quarter(const uint8_t *img, int pitch, int w4, int h4, float *out, cudaStream_t s)
{
    if (w4 <= 0 || h4 <= 0) return cudaSuccess;
    const dim3 b(32, 8), gr((w4 + 31) / 32, (h4 + 7) / 8);
    quarter_kernel<<<gr, b, 0, s>>>(img, pitch, w4, h4, out);
    return cudaGetLastError();
}

cudaError_t launch_sweep_input(const ProposalGeom &g, const float *ref_q, const float *src0, const float *src1,
                               float *out, cudaStream_t s)
{
    const dim3 b(32, 8), gr((g.wp + 31) / 32, (g.hp + 7) / 8);
    sweep_input_kernel<<<gr, b, 0, s>>>(g, ref_q, src0, src1, out);
    return cudaGetLastError();
}

cudaError_t launch_proposal_init(const RefDesc *refs, int r, int npix, const ProposalGeom &g, const float *prob,
                                 float threshold, cudaStream_t s)
{
    proposal_init_kernel<<<(npix + 255) / 256, 256, 0, s>>>(refs, r, g, prob, threshold);
    return cudaGetLastError();
}

}  // namespace pm
