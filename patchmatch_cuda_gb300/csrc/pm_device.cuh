// pm_device.cuh -- device building blocks of the PatchMatch engine (sm_103a).
//
// A windowed NCC maps lanes to window columns and loops over the window's rows, so the
// projective coordinates of a lane's samples advance along one column of the homography and
// every lane reads its reference values from a shared table without bank conflicts. Windows
// up to 16 wide give each half-warp its own hypothesis (two evaluations per warp pass); wider
// windows give every lane one or two columns of both hypotheses. Moments are accumulated per
// column shifted by the column's first sample and combined across lanes exactly (a window
// mean first, then the centred second moment and covariance), which is accurate in FP32
// without keeping the samples.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pm {

constexpr unsigned FULL_MASK = 0xffffffffu;
constexpr int MAX_VIEWS = 32;

// Random-draw purposes; a draw is keyed by (pixel, sweep, purpose << 16 | sub, batch).
enum : uint32_t {
    RNG_INIT = 1, RNG_BWD = 2, RNG_FWD_PRE = 3, RNG_FWD_POST = 4, RNG_RAND_DEPTH = 5,
    RNG_SAMPLE = 6, RNG_REFINE = 7
};
constexpr uint32_t INIT_SWEEP_ID = 0xFFFFFFFFu;

// Per-view homography table entries (float4): H1 (floats 0-8), H2 (9-17) for the one plane
// normal of the reference, e = K_s T_rel (18-20) for per-pixel planes, padding (21-23).
constexpr int HH_F4 = 6;

// Slanted-plane mode (no counterpart in the reference, whose plane normal is one constant,
// patchMatch.cu:32): a pixel's plane is its depth d and slopes (a, b), normal n ~ (a, b, 1) in
// the reference camera, so n . X = d s with the plane scale s = g . (x + 1/2, y + 1/2, 1),
// g = (a ik00, b ik11, a ik02 + b ik12 + 1), floored at SCALE_MIN; the homography is
// H1 - e g^T / (d s). Random slopes are uniform in [-SLOPE_DRAW, SLOPE_DRAW]^2, perturbed
// slopes clamp to [-SLOPE_MAX, SLOPE_MAX].
constexpr float SLOPE_DRAW = 1.0f;
constexpr float SLOPE_MAX = 2.0f;
constexpr float SCALE_MIN = 0.0625f;
// The random hypothesis's kind from its counter's second word u: u < 1/3 a uniform depth with
// the current slopes, u < 2/3 the current depth with uniform slopes, else a local perturbation.
constexpr float PLANE_P_DEPTH = 0.33333334f;
constexpr float PLANE_P_SLOPE = 0.6666667f;

// Transition probabilities and the uniform-emission cost of the HMM, as float constants
// (FIX_STATE_PROB 0.999f and CHANGE_STATE_PROB = 1.0f - 0.999f).
constexpr float FIX_STATE_PROB = 0.999f;
constexpr float CHANGE_STATE_PROB = 1.0f - 0.999f;

// Everything a kernel needs about one reference image. Lives in device memory; a launch
// may cover several references (batched runs).
struct RefDesc {
    int width, height, n_src, num_samples;
    float depth_near, depth_span;   // near, far - near
    float a2;                       // SPMAlpha^2 (float product)
    float u_emit;                   // exp(-0.83^2 / (2 a2))
    float nx, nz, ik00, ik02;       // plane scale s = nx (ik00 (x+1/2) + ik02) + nz
    float ik11, ik12;               // K^-1 (1,1), (1,2): slanted-plane mode
    int planes;                     // 1: a slanted plane per pixel (slopes); 0: one normal
    float plane_dstep, plane_sstep; // slanted planes: local search half-widths at sweep 0
    int quirks;
    int hw_filter;                  // textures filter bilinearly in hardware
    int record_sweep;               // >= 0: views are recorded only in this sweep (batches,
                                    // whose launches record for all references); -1: whenever
                                    // the launch records
    uint32_t batch_id;
    uint64_t seed;
    const float *ref;               // height*width texels
    const float *sum_i;             // box sums of the window
    const float *sum_ii;
    const float *c1;                // S_II - S_I^2 / n (FP64 prep), clamped below 1e-5
    float *depth;                   // height*width
    float *cost;                    // height*width*n_src, pixel-major
    float *beta;                    // scratch: width*height*n_src backward messages
    uint8_t *view_sel;              // num_samples*height*width or null
    float2 *slopes;                 // height*width plane slopes (a, b); slanted-plane mode
    unsigned long long *evals;      // [0] algorithmic count, [1] computed count
    const float4 *hh;               // n_src * HH_F4 float4: H1 (9), H2 (9), e (3), pad (3)
    cudaTextureObject_t tex_layered;  // all sources as layers (texture-filtering sampler)
    cudaTextureObject_t tex[MAX_VIEWS];
    float src_w[MAX_VIEWS], src_h[MAX_VIEWS];
};

// ---- Philox4x32-10 (Salmon et al., SC'11) ----------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// Uniform in (0, 1], 24-bit: ((x >> 8) + 1) * 2^-24 (the interval of curand_uniform).
__device__ __forceinline__ float draw_uniform(uint64_t seed, uint32_t pixel, uint32_t sweep,
                                              uint32_t purpose, uint32_t sub, uint32_t batch)
{
    const uint4 o = philox4x32_10(make_uint4(pixel, sweep, (purpose << 16) | sub, batch),
                                  make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    return (float)((o.x >> 8) + 1u) * (1.0f / 16777216.0f);
}

// The same counter's first two words as uniforms in (0, 1]: (x, y).
__device__ __forceinline__ float2 draw_uniform2(uint64_t seed, uint32_t pixel, uint32_t sweep,
                                                uint32_t purpose, uint32_t sub, uint32_t batch)
{
    const uint4 o = philox4x32_10(make_uint4(pixel, sweep, (purpose << 16) | sub, batch),
                                  make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    return make_float2((float)((o.x >> 8) + 1u) * (1.0f / 16777216.0f),
                       (float)((o.y >> 8) + 1u) * (1.0f / 16777216.0f));
}

// All four words of the counter as uniforms in (0, 1].
__device__ __forceinline__ float4 draw_uniform4(uint64_t seed, uint32_t pixel, uint32_t sweep,
                                                uint32_t purpose, uint32_t sub, uint32_t batch)
{
    const uint4 o = philox4x32_10(make_uint4(pixel, sweep, (purpose << 16) | sub, batch),
                                  make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    constexpr float k = 1.0f / 16777216.0f;
    return make_float4((float)((o.x >> 8) + 1u) * k, (float)((o.y >> 8) + 1u) * k,
                       (float)((o.z >> 8) + 1u) * k, (float)((o.w >> 8) + 1u) * k);
}

// ---- source fetch --------------------------------------------------------------------------
// The reference samples tex2DLayered(src, u/z + 0.5, v/z + 0.5) with linear filtering and a
// zero border (patchMatch.cu:543): bilinear interpolation at (u/z, v/z) with texel i at
// coordinate i. Here the four texels come from one gather (tld4) centred on the 2x2
// footprint, and the weights are exact FP32 fractions. Gather order (x0,y1), (x1,y1),
// (x1,y0), (x0,y0).
__device__ __forceinline__ float sample_source(cudaTextureObject_t tex, float xs, float ys,
                                               float sw, float sh)
{
    if (!(xs > -1.0f && xs < sw && ys > -1.0f && ys < sh)) return 0.0f;
    const float fx = floorf(xs), fy = floorf(ys);
    const float ax = xs - fx, ay = ys - fy;
    const float4 g = tex2Dgather<float4>(tex, fx + 1.0f, fy + 1.0f, 0);
    const float top = fmaf(ax, g.z - g.w, g.w);
    const float bot = fmaf(ax, g.y - g.x, g.x);
    return fmaf(ay, bot - top, top);
}

// Texture-unit bilinear filtering at source coordinate (xs, ys) (texel i at i) of layer `view`:
// the fetch of patchMatch.cu:543 itself, with the hardware's fixed-point weights. All sources
// share one layered texture (zero-padded to the largest view), so the texture handle is the
// same for every lane.
__device__ __forceinline__ float sample_source_hw(cudaTextureObject_t tex, int view, float xs, float ys)
{
    return tex2DLayered<float>(tex, xs + 0.5f, ys + 0.5f, view);
}

// The same fetch without a branch: coordinates are clamped to a safe finite range (NaN maps to
// the low end), the gather always runs, and out-of-range results are replaced by 0 afterwards.
__device__ __forceinline__ float sample_source_nb(cudaTextureObject_t tex, float xs, float ys,
                                                  float sw, float sh)
{
    const bool in = xs > -1.0f && xs < sw && ys > -1.0f && ys < sh;
    const float xc = fminf(fmaxf(xs, -2.0f), sw + 1.0f);
    const float yc = fminf(fmaxf(ys, -2.0f), sh + 1.0f);
    const float fx = floorf(xc), fy = floorf(yc);
    const float ax = xc - fx, ay = yc - fy;
    const float4 g = tex2Dgather<float4>(tex, fx + 1.0f, fy + 1.0f, 0);
    const float top = fmaf(ax, g.z - g.w, g.w);
    const float bot = fmaf(ax, g.y - g.x, g.x);
    return in ? fmaf(ay, bot - top, top) : 0.0f;
}

// 1/x rounded to nearest for normal x whose reciprocal is normal, without a slow path: the
// hardware approximation (rcp.approx) refined by one Newton-Raphson correction
// r <- r + r (1 - x r), the residual formed exactly by a fused multiply-add (Markstein's
// correction step, IBM J. Res. Dev. 34(1), 1990). pm_check_reciprocal compares it with the
// correctly rounded reciprocal over every significand of a binade, both signs; it agrees on
// every binade from 2^-120 to 2^120.
__device__ __forceinline__ float rcp_nr(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    const float e = fmaf(-x, r, 1.0f);
    return fmaf(r, e, r);
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

// HMM messages (patchMatch.cu:669-715). e = exp(-c^2 / (2 a2)); a cost of exactly 2 is
// replaced by 2 U(0,1] by the caller. The reference stores emissions and messages in float
// and builds with --use_fast_math, so values below the smallest normal float become zero;
// ftz() keeps that behaviour whatever the compiler's denormal mode.
__device__ __forceinline__ float ftz(float x) { return fabsf(x) < 1.17549435e-38f ? 0.0f : x; }

__device__ __forceinline__ float emission(float c, float a2) { return ftz(expf(-0.5f * c * c / a2)); }

__device__ __forceinline__ float msg_backward(float m, float e, float u)
{
    const float zn0 = m * e * FIX_STATE_PROB + (1.0f - m) * u * CHANGE_STATE_PROB;
    const float zn1 = m * e * CHANGE_STATE_PROB + (1.0f - m) * u * FIX_STATE_PROB;
    return ftz(zn0 / (zn0 + zn1));
}

__device__ __forceinline__ float msg_forward(float m, float e, float u)
{
    const float zn0 = (m * FIX_STATE_PROB + (1.0f - m) * CHANGE_STATE_PROB) * e;
    const float zn1 = (m * CHANGE_STATE_PROB + (1.0f - m) * FIX_STATE_PROB) * u;
    return ftz(zn0 / (zn0 + zn1));
}

// ---- windows ---------------------------------------------------------------------------------
// A window's samples are addressed as (dx, dy), 0 <= dx, dy < W. An evaluation maps lanes to
// window columns and loops over the rows: for W <= 16 each half-warp runs its own evaluation
// (lane & 15 = column), for larger windows the warp runs both evaluations of a pair with lane
// (and lane + 32) as columns.
template <int W>
struct Window {
    static constexpr int HW = W / 2;
    static constexpr int NSAMP = W * W;
    static constexpr int TAB = ((NSAMP + 31) / 32) * 32;  // table entries, padded
    static constexpr bool HALF = W <= 16;
    static constexpr int COLS = HALF ? 1 : (W + 31) / 32;  // columns per lane
};

// Scalars of one pixel's reference window. The values b = R - mu of its samples live in a
// table tab[dy * W + dx] (zero outside the image) with the column sums col[dx] = sum_dy b;
// mu = S_I / n is the window mean over its n in-bounds pixels and R the reference value the
// reference pairs with the source sample: the sample at the same position, except at the
// leading edge where the reference's pairing is shifted over the out-of-bounds columns
// (patchMatch.cu:546; kept when quirks are on).
struct WinCtl {
    float ox, oy;        // window origin in reference pixel-centre coordinates
    float scale;         // plane scale at the pixel
    float c1;            // S_II - S_I^2 / n (FP64 preparation), clamped
    float inv_n;         // 1 / n
    float rows, inv_rows;  // in-bounds rows
    float bsum;          // sum over in-bounds samples of (R_paired - R): 0 unless shifted
    int x0, y0;          // window origin in pixels
    int full;            // the window lies inside the image
    int dy_lo, dy_hi;    // in-bounds rows
};

// The scalar part of a window (lane 0 of the loading warp): origin, plane scale, c1, 1 / n,
// the in-bounds rows [cy0, cy1], the leading-edge term bsum, and whether it lies inside the image.
__device__ __forceinline__ void window_scalars(const RefDesc &D, int x, int y, int x0, int y0, int cy0, int cy1,
                                               float n, float c1, float bsum, bool full, WinCtl &wc)
{
    wc.ox = (float)x0 + 0.5f;
    wc.oy = (float)y0 + 0.5f;
    // explicit IEEE operations: the texture-filtering sampler's coordinates are replicated bit
    // for bit by the oracle
    wc.scale = __fadd_rn(__fmul_rn(D.nx, fmaf(D.ik00, __fadd_rn((float)x, 0.5f), D.ik02)), D.nz);
    wc.c1 = c1;
    wc.inv_n = 1.0f / n;
    wc.rows = (float)(cy1 - cy0 + 1);
    wc.inv_rows = 1.0f / wc.rows;
    wc.bsum = bsum;
    wc.x0 = x0;
    wc.y0 = y0;
    wc.full = full;
    wc.dy_lo = cy0 - y0;
    wc.dy_hi = cy1 - y0;
}

// Loads pixel (x, y)'s window with one warp, lane c owning columns c and c + 32. axis selects
// which image axis is the sweep's column axis for the leading-edge shift (0: x, vertical
// sweeps; 1: y).
template <int W>
__device__ __forceinline__ void load_window(const RefDesc &D, int x, int y, int axis, int lane,
                                            float *tab, float *col, WinCtl &wc)
{
    constexpr int HW = Window<W>::HW;
    const int Wd = D.width, Hd = D.height;
    const int x0 = x - HW, y0 = y - HW;
    int lead_x = 0, lead_y = 0;
    if (D.quirks) {
        if (axis == 0) lead_x = x0 < 0 ? -x0 : 0;
        else lead_y = y0 < 0 ? -y0 : 0;
    }
    const bool shifted = (lead_x | lead_y) != 0;
    const int cx0 = max(x0, 0), cx1 = min(x + HW, Wd - 1);
    const int cy0 = max(y0, 0), cy1 = min(y + HW, Hd - 1);
    const float n = (float)((cx1 - cx0 + 1) * (cy1 - cy0 + 1));
    const size_t pix = (size_t)y * Wd + x;
    const float mu = __ldg(D.sum_i + pix) / n;
    float sh = 0.0f;
    constexpr int CHUNK = W < 16 ? W : 16;  // rows loaded before any is stored
#pragma unroll
    for (int q = 0; q < (W + 31) / 32; ++q) {
        const int c = lane + 32 * q;
        if (c >= W) continue;
        const int xx = x0 + c;
        const bool col_in = xx >= 0 && xx < Wd;
        float cs = 0.0f;
        for (int dy0 = 0; dy0 < W; dy0 += CHUNK) {
            float rp[CHUNK], ro[CHUNK];
#pragma unroll
            for (int i = 0; i < CHUNK; ++i) {
                const int yy = y0 + dy0 + i;
                const bool in = dy0 + i < W && col_in && yy >= 0 && yy < Hd;
                const int rx = xx - lead_x, ry = yy - lead_y;
                rp[i] = (in && rx >= 0 && ry >= 0) ? __ldg(D.ref + (size_t)ry * Wd + rx) : 0.0f;
                ro[i] = (in && shifted) ? __ldg(D.ref + (size_t)yy * Wd + xx) : 0.0f;
            }
#pragma unroll
            for (int i = 0; i < CHUNK; ++i) {
                const int dy = dy0 + i, yy = y0 + dy;
                if (dy >= W) break;
                const bool in = col_in && yy >= 0 && yy < Hd;
                const float b = in ? rp[i] - mu : 0.0f;
                if (in && shifted) sh += rp[i] - ro[i];
                tab[dy * W + c] = b;
                cs += b;
            }
        }
        col[c] = cs;
    }
    if (shifted) sh = warp_sum(sh);
    if (lane == 0)
        window_scalars(D, x, y, x0, y0, cy0, cy1, n, __ldg(D.c1 + pix), shifted ? sh : 0.0f,
                       x0 >= 0 && y0 >= 0 && x + HW < Wd && y + HW < Hd, wc);
}

// The sweep kernel's sliding form of load_window for windows inside the image. The raw
// reference values of the current window live in a ring `raw` of W x W floats indexed by image
// line modulo W (filled by load_window), so a step of a sweep loads only the line that enters
// the window:
//   rows (vertical sweeps):     raw[(yy % W) * W + c]  = R(x0 + c, yy)
//   columns (horizontal ones):  raw[dy * W + (xx % W)] = R(xx, y0 + dy)
// `enter` is the image row (rows) or column that entered since the previous step, or -1 to fill
// the whole ring (a step whose previous window was cut by the border). The table and
// column sums are then formed from the ring with load_window's arithmetic in its order, so both
// give the same values.
template <int W>
__device__ __forceinline__ void ring_window(const RefDesc &D, int x, int y, bool rows, int enter, int lane,
                                            float *raw, float *tab, float *col, WinCtl &wc)
{
    constexpr int HW = Window<W>::HW;
    const int Wd = D.width;
    const int x0 = x - HW, y0 = y - HW;
    // the window's box sum and c1 load together with the entering line: one round trip
    const size_t pix = (size_t)y * Wd + x;
    const float sum_i = __ldg(D.sum_i + pix);
    const float c1 = lane == 0 ? __ldg(D.c1 + pix) : 0.0f;
#pragma unroll
    for (int q = 0; q < (W + 31) / 32; ++q) {
        const int c = lane + 32 * q;  // a window column, or a window row for an entering column
        if (c >= W) continue;
        if (enter < 0) {
            // one value at a time (a fill happens once per run of inside windows)
#pragma unroll 1
            for (int dy = 0; dy < W; ++dy) {
                const float r = __ldg(D.ref + (size_t)(y0 + dy) * Wd + x0 + c);
                raw[rows ? ((y0 + dy) % W) * W + c : dy * W + (x0 + c) % W] = r;
            }
        } else if (rows) {
            raw[(enter % W) * W + c] = __ldg(D.ref + (size_t)enter * Wd + x0 + c);
        } else {
            raw[c * W + enter % W] = __ldg(D.ref + (size_t)(y0 + c) * Wd + enter);
        }
    }
    __syncwarp();
    const float n = (float)(W * W);
    const float mu = sum_i / n;
#pragma unroll
    for (int q = 0; q < (W + 31) / 32; ++q) {
        const int c = lane + 32 * q;
        if (c >= W) continue;
        const int cslot = (x0 + c) % W;
        int rslot = y0 % W;
        float cs = 0.0f;
        for (int dy = 0; dy < W; ++dy) {
            const float b = (rows ? raw[rslot * W + c] : raw[dy * W + cslot]) - mu;
            rslot = rslot + 1 == W ? 0 : rslot + 1;
            tab[dy * W + c] = b;
            cs += b;
        }
        col[c] = cs;
    }
    if (lane == 0) window_scalars(D, x, y, x0, y0, y0, y0 + W - 1, n, c1, 0.0f, true, wc);
}

// ring_window for the lines within a half-window of an image edge: windows whose extent along
// the sweep lies inside the image but which the border cuts across the line, the same cut for
// every step of the line. The ring holds load_window's values: zeros off the image and, on a
// line at the leading edge with the reference's misaligned tile (quirks), the shifted values it
// pairs with the window in `raw` and the unshifted ones in `raw_o`. The table, column sums and
// leading-edge term are formed with load_window's arithmetic in its order, so both give the
// same values.
template <int W>
__device__ __forceinline__ void ring_window_cut(const RefDesc &D, int x, int y, bool rows, int enter, int lane,
                                                float *raw, float *raw_o, float *tab, float *col, WinCtl &wc)
{
    constexpr int HW = Window<W>::HW;
    const int Wd = D.width, Hd = D.height;
    const int x0 = x - HW, y0 = y - HW;
    const int lead = !D.quirks ? 0 : rows ? (x0 < 0 ? -x0 : 0) : (y0 < 0 ? -y0 : 0);
    const bool shifted = lead != 0;
    const int a0 = rows ? x0 : y0, alen = rows ? Wd : Hd;
    const int cx0 = max(x0, 0), cx1 = min(x + HW, Wd - 1);
    const int cy0 = max(y0, 0), cy1 = min(y + HW, Hd - 1);
    const size_t pix = (size_t)y * Wd + x;
    const float sum_i = __ldg(D.sum_i + pix);
    const float c1 = lane == 0 ? __ldg(D.c1 + pix) : 0.0f;
    // the entering line, or every line of the window: lane i is the window's column (rows) or
    // row (columns) i across the sweep
    const size_t stride = rows ? 1 : (size_t)Wd;
#pragma unroll
    for (int q = 0; q < (W + 31) / 32; ++q) {
        const int i = lane + 32 * q;
        if (i >= W) continue;
        const int ai = a0 + i;                   // image column (rows) or row (columns)
        const bool in = (unsigned)ai < (unsigned)alen;
        const bool p_in = in && ai - lead >= 0;  // the shifted read stays on the image
        const int k0 = enter < 0 ? 0 : W - 1, k1 = W;
#pragma unroll 1
        for (int k = k0; k < k1; ++k) {
            const int along = enter < 0 ? (rows ? y0 : x0) + k : enter;
            const int slot = rows ? (along % W) * W + i : i * W + along % W;
            const size_t at = rows ? (size_t)along * Wd : (size_t)along;
            raw[slot] = p_in ? __ldg(D.ref + at + (size_t)(ai - lead) * stride) : 0.0f;
            if (shifted) raw_o[slot] = in ? __ldg(D.ref + at + (size_t)ai * stride) : 0.0f;
        }
    }
    __syncwarp();
    const float n = (float)((cx1 - cx0 + 1) * (cy1 - cy0 + 1));
    const float mu = sum_i / n;
    float sh = 0.0f;
#pragma unroll
    for (int q = 0; q < (W + 31) / 32; ++q) {
        const int c = lane + 32 * q;
        if (c >= W) continue;
        const bool col_in = !rows || (unsigned)(x0 + c) < (unsigned)Wd;
        const int cslot = rows ? 0 : (x0 + c) % W;
        int rslot = rows ? y0 % W : 0;
        float cs = 0.0f;
        for (int dy = 0; dy < W; ++dy) {
            const int at = rows ? rslot * W + c : dy * W + cslot;
            const bool in = col_in && (rows || (unsigned)(y0 + dy) < (unsigned)Hd);
            const float v = raw[at];
            const float b = in ? v - mu : 0.0f;
            if (in && shifted) sh += v - raw_o[at];
            rslot = rslot + 1 == W ? 0 : rslot + 1;
            tab[dy * W + c] = b;
            cs += b;
        }
        col[c] = cs;
    }
    if (shifted) sh = warp_sum(sh);
    if (lane == 0) window_scalars(D, x, y, x0, y0, cy0, cy1, n, c1, shifted ? sh : 0.0f, false, wc);
}

// A homography's first two columns and its value at the window origin (see warp_setup).
struct WarpSetup {
    float c0x, c0y, c0z, c1x, c1y, c1z, bx, by, bz;
};

// g = K_r^-T n for n = (a, b, 1) and the plane scale at pixel centre (px, py), with explicit
// single-precision steps (the oracle repeats them bit for bit).
struct PlaneG {
    float g0, g1, g2, s;
};

__device__ __forceinline__ PlaneG plane_terms(const RefDesc &D, float2 sl, float px, float py)
{
    PlaneG r;
    r.g0 = __fmul_rn(sl.x, D.ik00);
    r.g1 = __fmul_rn(sl.y, D.ik11);
    r.g2 = fmaf(sl.x, D.ik02, fmaf(sl.y, D.ik12, 1.0f));
    const float s = fmaf(r.g0, px, fmaf(r.g1, py, r.g2));
    r.s = s < SCALE_MIN ? SCALE_MIN : s;
    return r;
}

// Plane-induced homography of (view, depth): T = H1 - H2 / (depth * scale)
// (patchMatch.cu:462-474), or with per-pixel planes T = H1 - e g^T / (depth * s); its first two
// columns and T (ox, oy, 1) at the window origin.
template <bool HW, bool PL>
__device__ __forceinline__ WarpSetup warp_setup(const RefDesc &D, const float4 *hh, int view, float depth,
                                                float2 sl, float scale, float ox, float oy, float hwf)
{
    const float4 *h = hh + HH_F4 * view;
    const float4 a = h[0], b = h[1], c = h[2];
    // floats 0-8: H1 (row-major), 9-17: H2, 18-20: e
    const float h1[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x};
    float t[9];
    if (PL) {
        const float4 e4 = h[4], e5 = h[5];
        const float e[3] = {e4.z, e4.w, e5.x};
        // the pixel centre x + 1/2 = ox + half-window, exactly
        const PlaneG G = plane_terms(D, sl, ox + hwf, oy + hwf);
        const float g[3] = {G.g0, G.g1, G.g2};
        const float s = HW ? rcp_nr(__fmul_rn(depth, G.s)) : __fdividef(1.0f, depth * G.s);
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int k = 0; k < 3; ++k) t[3 * r + k] = fmaf(-s, __fmul_rn(e[r], g[k]), h1[3 * r + k]);
    } else {
        const float4 d = h[3], e = h[4];
        const float h2[9] = {c.y, c.z, c.w, d.x, d.y, d.z, d.w, e.x, e.y};
        // texture-filtering sampler: correctly rounded, so the oracle reproduces the coordinates
        const float s = HW ? rcp_nr(__fmul_rn(depth, scale)) : __fdividef(1.0f, depth * scale);
#pragma unroll
        for (int i = 0; i < 9; ++i) t[i] = fmaf(-s, h2[i], h1[i]);
    }
    if (HW) {
        // texture coordinates are (u/z + 1/2, v/z + 1/2): add z/2 to the first two rows
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            t[i] = fmaf(0.5f, t[6 + i], t[i]);
            t[3 + i] = fmaf(0.5f, t[6 + i], t[3 + i]);
        }
    }
    WarpSetup w;
    w.c0x = t[0]; w.c0y = t[3]; w.c0z = t[6];
    w.c1x = t[1]; w.c1y = t[4]; w.c1z = t[7];
    w.bx = fmaf(t[0], ox, fmaf(t[1], oy, t[2]));
    w.by = fmaf(t[3], ox, fmaf(t[4], oy, t[5]));
    w.bz = fmaf(t[6], ox, fmaf(t[7], oy, t[8]));
    return w;
}

// Source sample at homogeneous coordinates (px, py, pz).
template <bool HW>
__device__ __forceinline__ float fetch(cudaTextureObject_t tex, int layer, float sw, float sh,
                                       float px, float py, float pz)
{
    if (HW) {
        // keep the coordinate finite on the source camera's principal plane (border -> 0);
        // px, py already carry the texture's half-texel offset
        pz = fabsf(pz) < 1e-20f ? 1e-20f : pz;
        const float r = rcp_nr(pz);
        return tex2DLayered<float>(tex, __fmul_rn(px, r), __fmul_rn(py, r), layer);
    }
    const float r = __fdividef(1.0f, pz);
    return sample_source_nb(tex, px * r, py * r, sw, sh);
}

// Moments of one window column under one hypothesis, shifted by the column's first sample K
// (accurate in FP32 without holding the samples):
//   s1 = sum (J - K), s2 = sum (J - K)^2, sx = sum (J - K) b
// over the column's in-bounds samples, b = R - mu from the window table.
struct ColMoments {
    float k, s1, s2, sx;
};

template <int W, bool HW, bool FULL>
__device__ __forceinline__ void column_moments(const WarpSetup &A, cudaTextureObject_t tex, int layer,
                                               float sw, float sh, const float *tab, int c,
                                               bool col_ok, const WinCtl &wc, ColMoments &m)
{
    const int cc = c < W ? c : W - 1;  // idle lanes read a valid entry and discard it
    const float fc = (float)c;
    const float colx = fmaf(A.c0x, fc, A.bx), coly = fmaf(A.c0y, fc, A.by), colz = fmaf(A.c0z, fc, A.bz);
    m.k = m.s1 = m.s2 = m.sx = 0.0f;
    // the exact sampler's gathers hold four texels each: fewer rows in flight
    constexpr int UNROLL = HW ? W : 4;
#pragma unroll UNROLL
    for (int dy = 0; dy < W; ++dy) {
        const float fdy = (float)dy;
        float j = 0.0f;
        if (col_ok)
            j = fetch<HW>(tex, layer, sw, sh, fmaf(A.c1x, fdy, colx), fmaf(A.c1y, fdy, coly),
                          fmaf(A.c1z, fdy, colz));
        const float b = tab[dy * W + cc];
        // the shift: row 0's sample, or 0 when row 0 lies outside the reference image (a window
        // cut at the top), so that K = 0 and s2 = 0 say exactly that every in-bounds sample is 0
        if (dy == 0) m.k = (FULL || wc.dy_lo == 0) ? j : 0.0f;
        // lanes off the window's columns fetch nothing: j = K = 0 there
        const float d = (FULL || (dy >= wc.dy_lo && dy <= wc.dy_hi)) ? j - m.k : 0.0f;
        m.s1 += d;
        m.s2 = fmaf(d, d, m.s2);
        m.sx = fmaf(d, b, m.sx);
    }
}

// Per-lane terms of the second reduction stage from the column moments, the column sum bcol
// of b and the window mean mj: the column's centred second moment and its covariance with
// the reference.
__device__ __forceinline__ void column_terms(const ColMoments &m, bool col_ok, float rows,
                                             float inv_rows, float mj, float bcol, float &c2,
                                             float &x)
{
    if (!col_ok) return;
    const float mean = fmaf(m.s1, inv_rows, m.k);
    const float dm = mean - mj;
    c2 += fmaf(rows * dm, dm, fmaf(-m.s1 * inv_rows, m.s1, m.s2));
    x += fmaf(m.k - mj, bcol, m.sx);
}

// 1 - NCC (patchMatch.cu:594-610): 2 when every source sample is zero, variances below 1e-5
// clamp to 0, 1 when their product is 0. The reference forms
// 1 - (S_IJ - S_I S_J / n) / sqrt(c1 c2) from raw sums, which cancels badly in FP32 for weakly
// textured windows; here c2 = sum (J - mu_J)^2 and the covariance
// sum (J - mu_J)(R - mu) + mu_J sum (R_paired - R) are assembled from shifted column moments,
// equal to the reference's in exact arithmetic (the last term, the leading-edge shift, is
// zero for aligned windows).
__device__ __forceinline__ float ncc_finalize(bool all_zero, float c2, float x, float c1, float mu_j,
                                              float bsum)
{
    if (all_zero) return 2.0f;
    c2 = c2 < 0.00001f ? 0.0f : c2;
    const float cc = c1 * c2;
    if (cc == 0.0f) return 1.0f;
    return 1.0f - fmaf(mu_j, bsum, x) * rsqrtf(cc);
}

// Two windowed NCC evaluations of one pixel, (view va, depth da) and (vb, db); every lane
// receives both results. hh: the homography table (D.hh or a shared-memory copy). FULL: the
// window lies inside the reference image.
template <int W, bool HW, bool FULL, bool PL>
__device__ __forceinline__ void ncc_pair_core(const RefDesc &D, const float4 *hh, const WinCtl &wc,
                                              const float *tab, const float *col, int lane, int va,
                                              float da, float2 sa, int vb, float db, float2 sb, float &ra,
                                              float &rb)
{
    if (Window<W>::HALF) {
        const int half = lane >> 4, c = lane & 15;
        const int v = half ? vb : va;
        const WarpSetup A = warp_setup<HW, PL>(D, hh, v, half ? db : da, half ? sb : sa, wc.scale, wc.ox, wc.oy,
                                                   (float)Window<W>::HW);
        const cudaTextureObject_t tex = HW ? D.tex_layered : D.tex[v];
        const bool col_ok = c < W && (FULL || (unsigned)(wc.x0 + c) < (unsigned)D.width);
        ColMoments m;
        column_moments<W, HW, FULL>(A, tex, v, D.src_w[v], D.src_h[v], tab, c, col_ok, wc, m);
        // stage 1: sum of J over the half (sum = rows K + s1 per column), all-zero test
        const float rows = FULL ? (float)W : wc.rows;
        const float inv_rows = FULL ? 1.0f / (float)W : wc.inv_rows;
        float sj = col_ok ? fmaf(rows, m.k, m.s1) : 0.0f;
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) sj += __shfl_xor_sync(FULL_MASK, sj, o);
        const unsigned nz = __ballot_sync(FULL_MASK, col_ok && (m.k != 0.0f || m.s2 != 0.0f));
        const bool all_zero = ((nz >> (16 * half)) & 0xFFFFu) == 0;
        const float mj = sj * wc.inv_n;
        // stage 2: centred second moment and covariance
        float c2 = 0.0f, x = 0.0f;
        column_terms(m, col_ok, rows, inv_rows, mj, col[c < W ? c : W - 1], c2, x);
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
            c2 += __shfl_xor_sync(FULL_MASK, c2, o);
            x += __shfl_xor_sync(FULL_MASK, x, o);
        }
        const float res = ncc_finalize(all_zero, c2, x, wc.c1, mj, wc.bsum);
        ra = __shfl_sync(FULL_MASK, res, 0);
        rb = __shfl_sync(FULL_MASK, res, 16);
    } else {
        constexpr int COLS = Window<W>::COLS;
        const int vv[2] = {va, vb};
        const float dd[2] = {da, db};
        const float2 ss[2] = {sa, sb};
        const float rows = FULL ? (float)W : wc.rows;
        const float inv_rows = FULL ? 1.0f / (float)W : wc.inv_rows;
        float out[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int v = vv[e];
            const WarpSetup A = warp_setup<HW, PL>(D, hh, v, dd[e], ss[e], wc.scale, wc.ox, wc.oy, (float)Window<W>::HW);
            const cudaTextureObject_t tex = HW ? D.tex_layered : D.tex[v];
            ColMoments m[COLS];
            bool ok[COLS];
#pragma unroll
            for (int q = 0; q < COLS; ++q) {
                const int c = lane + 32 * q;
                ok[q] = c < W && (FULL || (unsigned)(wc.x0 + c) < (unsigned)D.width);
                column_moments<W, HW, FULL>(A, tex, v, D.src_w[v], D.src_h[v], tab, c, ok[q], wc, m[q]);
            }
            float sj = 0.0f;
            bool nzl = false;
#pragma unroll
            for (int q = 0; q < COLS; ++q) {
                if (ok[q]) sj += fmaf(rows, m[q].k, m[q].s1);
                nzl = nzl || (ok[q] && (m[q].k != 0.0f || m[q].s2 != 0.0f));
            }
            sj = warp_sum(sj);
            const bool all_zero = __ballot_sync(FULL_MASK, nzl) == 0;
            const float mj = sj * wc.inv_n;
            float c2 = 0.0f, x = 0.0f;
#pragma unroll
            for (int q = 0; q < COLS; ++q) {
                const int c = lane + 32 * q;
                column_terms(m[q], ok[q], rows, inv_rows, mj, col[c < W ? c : W - 1], c2, x);
            }
            c2 = warp_sum(c2);
            x = warp_sum(x);
            out[e] = ncc_finalize(all_zero, c2, x, wc.c1, mj, wc.bsum);
        }
        ra = out[0];
        rb = out[1];
    }
}

// Windows cut by the image border. Inline: the lines along the image's edges cut every window,
// and the sweep lasts as long as its slowest line (an out-of-line call measured 4 % slower).
template <int W, bool HW, bool PL>
__device__ __forceinline__ void ncc_pair_edge(const RefDesc &D, const float4 *hh, const WinCtl &wc,
                                           const float *tab, const float *col, int lane, int va,
                                           float da, float2 sa, int vb, float db, float2 sb, float &ra,
                                           float &rb)
{
    ncc_pair_core<W, HW, false, PL>(D, hh, wc, tab, col, lane, va, da, sa, vb, db, sb, ra, rb);
}

// PL: slanted-plane mode; sa, sb are then the hypotheses' plane slopes (ignored otherwise).
template <int W, bool HW, bool PL>
__device__ __forceinline__ void ncc_pair(const RefDesc &D, const float4 *hh, const WinCtl &wc,
                                         const float *tab, const float *col, int lane, int va,
                                         float da, float2 sa, int vb, float db, float2 sb, float &ra,
                                         float &rb)
{
    if (wc.full) ncc_pair_core<W, HW, true, PL>(D, hh, wc, tab, col, lane, va, da, sa, vb, db, sb, ra, rb);
    else ncc_pair_edge<W, HW, PL>(D, hh, wc, tab, col, lane, va, da, sa, vb, db, sb, ra, rb);
}

// Copies a reference's descriptor and homography table into shared memory (all threads of
// the block take part; synchronise before use). Fields read on every step then never miss in
// an L1 that texture traffic keeps busy.
__device__ __forceinline__ void stage_ref(const RefDesc &src, RefDesc &dst, float4 *hh)
{
    static_assert(sizeof(RefDesc) % 4 == 0, "RefDesc is copied in words");
    const uint32_t *s = reinterpret_cast<const uint32_t *>(&src);
    uint32_t *d = reinterpret_cast<uint32_t *>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(RefDesc) / 4); i += blockDim.x) d[i] = s[i];
    const float4 *h = src.hh;
    const int n = HH_F4 * src.n_src;
    for (int i = threadIdx.x; i < n; i += blockDim.x) hh[i] = __ldg(h + i);
}

}  // namespace pm
