// pm_device.cuh -- device building blocks of the PatchMatch engine (sm_103a).
//
// One warp owns one line of a sweep (a reference-image column for vertical sweeps, a row
// for horizontal ones). For a windowed NCC every lane owns ceil(w*w/32) "slots" of the
// window: slot i of lane l is window sample k = l + 32 i, (dx, dy) = (k % w, k / w). The
// reference values of a lane's slots are loaded once per step into registers and reused
// by every hypothesis of that step; the three source moments of an evaluation are summed
// per lane and then across the warp with a butterfly of shuffles.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pm {

constexpr unsigned FULL_MASK = 0xffffffffu;
constexpr int MAX_VIEWS = 32;

// Random-draw purposes; a draw is keyed by (pixel, sweep, purpose << 16 | sub, batch).
enum : uint32_t {
    RNG_INIT = 1, RNG_BWD = 2, RNG_FWD_PRE = 3, RNG_FWD_POST = 4, RNG_RAND_DEPTH = 5,
    RNG_SAMPLE = 6
};
constexpr uint32_t INIT_SWEEP_ID = 0xFFFFFFFFu;

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
    int quirks;
    int hw_filter;                  // textures filter bilinearly in hardware
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
    unsigned long long *evals;      // [0] algorithmic count, [1] computed count
    const float4 *hh;               // n_src * 5 float4: H1 (9), H2 (9), pad (2)
    const double *hh64;             // n_src * 18 (mixed precision window origin)
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

// ---- window slots ---------------------------------------------------------------------------
template <int W>
struct Window {
    static constexpr int HW = W / 2;
    static constexpr int NSAMP = W * W;
    static constexpr int NS = (NSAMP + 31) / 32;
};

// Per-step state of one pixel's window, held by every lane for its own slots.
//
// The reference evaluates 1 - (S_IJ - S_I S_J / n) / sqrt(c1 c2) from raw sums
// (patchMatch.cu:594-610), which cancels badly in FP32 for weakly textured windows. Here
//   c1 = S_II - S_I^2 / n          comes from the FP64 preparation pass (per pixel),
//   c2 = sum (J - mu_J)^2          is summed from source samples centred on their own mean,
//   cov = sum (J - mu_J)(R - mu) + mu_J * sum (R - mu)
// with mu = S_I / n the reference window mean and R the reference value the reference pairs
// with each source sample. In exact arithmetic this equals the reference's covariance,
// including its leading-edge misalignment (the last term is zero for aligned windows).
template <int W>
struct PixelWindow {
    static constexpr int NS = Window<W>::NS;
    float *b;            // this warp's shared table: b[32 * i + lane] = R - mu of slot i
    uint64_t inb;        // slot in bounds
    bool full;           // the whole window lies inside the reference image
    float ox, oy;        // window origin in reference pixel-centre coordinates
    float n, inv_n;      // in-bounds count
    float c1;            // reference variance term, clamped
    float bsum;          // sum over in-bounds slots of (R_paired - mu); 0 when aligned
    float scale;         // plane scale at this pixel
};

// Loads a pixel's window for lane `lane`. axis selects which image axis is the sweep's
// column axis for the reference's misalignment (0: x, vertical sweeps; 1: y).
template <int W>
__device__ __forceinline__ void load_window(const RefDesc &D, int x, int y, int axis, int lane,
                                            const float2 *slots, float *btab, PixelWindow<W> &pw)
{
    constexpr int HW = Window<W>::HW, NS = Window<W>::NS, NSAMP = Window<W>::NSAMP;
    const int Wd = D.width, Hd = D.height;
    const int x0 = x - HW, y0 = y - HW;
    int lead_x = 0, lead_y = 0;
    if (D.quirks) {
        if (axis == 0) lead_x = x0 < 0 ? -x0 : 0;
        else lead_y = y0 < 0 ? -y0 : 0;
    }
    const int cx0 = max(x0, 0), cx1 = min(x + HW, Wd - 1);
    const int cy0 = max(y0, 0), cy1 = min(y + HW, Hd - 1);
    pw.n = (float)((cx1 - cx0 + 1) * (cy1 - cy0 + 1));
    pw.full = x0 >= 0 && y0 >= 0 && x + HW < Wd && y + HW < Hd;
    pw.inv_n = 1.0f / pw.n;
    const size_t pix = (size_t)y * Wd + x;
    const float mu = __ldg(D.sum_i + pix) / pw.n;
    pw.c1 = __ldg(D.c1 + pix);
    uint64_t inb = 0;
    float bs = 0.0f;
    const bool shifted = (lead_x | lead_y) != 0;
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        const int k = lane + 32 * i;
        const float2 o = slots[32 * i + lane];
        const int xx = x0 + (int)o.x, yy = y0 + (int)o.y;
        const bool in = (k < NSAMP) && xx >= 0 && xx < Wd && yy >= 0 && yy < Hd;
        float r = 0.0f;
        if (in) {
            r = __ldg(D.ref + (size_t)yy * Wd + xx);
            if (shifted) {
                // the reference pairs this source sample with a reference value shifted
                // back over the leading out-of-bounds columns (zero outside the image)
                const int rx = xx - lead_x, ry = yy - lead_y;
                const float rm = (rx >= 0 && ry >= 0) ? __ldg(D.ref + (size_t)ry * Wd + rx) : 0.0f;
                bs += rm - r;
                r = rm;
            }
            inb |= (uint64_t)1 << i;
            r -= mu;
        }
        btab[32 * i + lane] = r;
    }
    pw.b = btab;
    pw.inb = inb;
    // sum(R_paired - mu) = sum(R_paired) - sum(R): exactly zero for aligned windows
    pw.bsum = shifted ? warp_sum(bs) : 0.0f;
    pw.ox = (float)x0 + 0.5f;
    pw.oy = (float)y0 + 0.5f;
    // explicit IEEE operations: the texture-filtering sampler's coordinates are replicated
    // bit for bit by the oracle
    pw.scale = __fadd_rn(__fmul_rn(D.nx, fmaf(D.ik00, __fadd_rn((float)x, 0.5f), D.ik02)), D.nz);
}

// 1 - NCC (patchMatch.cu:594-610): 2 when every source sample is zero, variances below 1e-5
// clamp to 0, 1 when their product is 0.
__device__ __forceinline__ float ncc_finalize(float sj, float c2, float x, float c1, float mu_j,
                                              float bsum)
{
    if (sj == 0.0f) return 2.0f;
    c2 = c2 < 0.00001f ? 0.0f : c2;
    const float cc = c1 * c2;
    if (cc == 0.0f) return 1.0f;
    return 1.0f - fmaf(mu_j, bsum, x) * rsqrtf(cc);
}

// Plane-induced homography of (view, depth) applied at the window origin:
// T = H1 - H2 / (depth * scale) (patchMatch.cu:462-474); returns T's first two columns and
// T (ox, oy, 1).
struct WarpSetup {
    float c0x, c0y, c0z, c1x, c1y, c1z, bx, by, bz;
};

template <bool HW>
__device__ __forceinline__ WarpSetup warp_setup(const RefDesc &D, int view, float depth,
                                                float scale, float ox, float oy)
{
    const float4 *h = D.hh + 5 * view;
    const float4 a = __ldg(h), b = __ldg(h + 1), c = __ldg(h + 2), d = __ldg(h + 3),
                 e = __ldg(h + 4);
    // 20 floats per view: H1 (row-major, floats 0-8), H2 (floats 9-17), 2 pad.
    const float h1[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x};
    const float h2[9] = {c.y, c.z, c.w, d.x, d.y, d.z, d.w, e.x, e.y};
    // texture-filtering sampler: correctly rounded, so the oracle reproduces the coordinates
    const float s = HW ? __frcp_rn(__fmul_rn(depth, scale)) : __fdividef(1.0f, depth * scale);
    float t[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) t[i] = fmaf(-s, h2[i], h1[i]);
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

template <bool HW>
__device__ __forceinline__ float warp_sample(const WarpSetup &A, cudaTextureObject_t tex, int layer,
                                             float sw, float sh, float dx, float dy)
{
    const float px = fmaf(A.c0x, dx, fmaf(A.c1x, dy, A.bx));
    const float py = fmaf(A.c0y, dx, fmaf(A.c1y, dy, A.by));
    float pz = fmaf(A.c0z, dx, fmaf(A.c1z, dy, A.bz));
    if (HW) {
        // keep the coordinate finite on the source camera's principal plane (border -> 0);
        // px, py already carry the texture's half-texel offset
        pz = fabsf(pz) < 1e-20f ? 1e-20f : pz;
        const float r = __frcp_rn(pz);
        return tex2DLayered<float>(tex, __fmul_rn(px, r), __fmul_rn(py, r), layer);
    }
    const float r = __fdividef(1.0f, pz);
    return sample_source_nb(tex, px * r, py * r, sw, sh);
}

// Whether lane `lane`'s slot i is a window sample: the window may not fill the last slot.
template <int W>
__device__ __forceinline__ bool slot_exists(int i, int lane)
{
    return i < Window<W>::NS - 1 || lane + 32 * i < Window<W>::NSAMP;
}

// E windowed NCC evaluations (views v[e] at depths d[e], E = 1 or 2) for one pixel; every
// lane returns the results. Source samples stay in registers for the centred second pass.
// FULL: the window lies inside the image, so only the last slot needs a test.
template <int W, int E, bool HW, bool FULL>
__device__ __forceinline__ void eval_core(const RefDesc &D, const PixelWindow<W> &pw,
                                          const float2 *slots, int lane, const int (&v)[E],
                                          const float (&d)[E], float (&out)[E])
{
    constexpr int NS = Window<W>::NS;
    constexpr int LAST_LANES = Window<W>::NSAMP - 32 * (NS - 1);  // lanes holding the last slot
    WarpSetup A[E];
    cudaTextureObject_t tex[E];
    float sw[E], sh[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        A[e] = warp_setup<HW>(D, v[e], d[e], pw.scale, pw.ox, pw.oy);
        tex[e] = HW ? D.tex_layered : D.tex[v[e]];
        sw[e] = D.src_w[v[e]];
        sh[e] = D.src_h[v[e]];
    }
    float smp[E][NS];
    float j[E];
#pragma unroll
    for (int e = 0; e < E; ++e) j[e] = 0.f;
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        const float2 o = slots[32 * i + lane];
        // Interior windows sample every full slot unconditionally (no branch between the
        // fetches, so they can all be in flight at once); the partially filled last slot and
        // windows cut by the image border keep a per-slot test.
        const bool guarded = !FULL || (i == NS - 1 && LAST_LANES < 32);
        const bool take = FULL ? (i < NS - 1 || lane < LAST_LANES) : ((pw.inb >> i) & 1) != 0;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            float sv = 0.f;
            if (guarded) {
                if (take) sv = warp_sample<HW>(A[e], tex[e], v[e], sw[e], sh[e], o.x, o.y);
            } else {
                sv = warp_sample<HW>(A[e], tex[e], v[e], sw[e], sh[e], o.x, o.y);
            }
            smp[e][i] = sv;
            j[e] += sv;
        }
    }
    float m[E], q[E], x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        j[e] = warp_sum(j[e]);
        m[e] = j[e] * pw.inv_n;
        q[e] = 0.f;
        x[e] = 0.f;
    }
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        const bool take = FULL ? (i < NS - 1 || lane < LAST_LANES) : ((pw.inb >> i) & 1) != 0;
        const float bi = pw.b[32 * i + lane];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const float de = take ? smp[e][i] - m[e] : 0.0f;
            q[e] = fmaf(de, de, q[e]);
            x[e] = fmaf(de, bi, x[e]);
        }
    }
#pragma unroll
    for (int e = 0; e < E; ++e) {
        q[e] = warp_sum(q[e]);
        x[e] = warp_sum(x[e]);
        out[e] = ncc_finalize(j[e], q[e], x[e], pw.c1, m[e], pw.bsum);
    }
}

template <int W, bool HW>
__device__ __forceinline__ float eval_one(const RefDesc &D, const PixelWindow<W> &pw,
                                          const float2 *slots, int lane, int v, float d)
{
    const int vv[1] = {v};
    const float dd[1] = {d};
    float out[1];
    if (pw.full) eval_core<W, 1, HW, true>(D, pw, slots, lane, vv, dd, out);
    else eval_core<W, 1, HW, false>(D, pw, slots, lane, vv, dd, out);
    return out[0];
}

template <int W, bool HW>
__device__ __forceinline__ void eval_pair(const RefDesc &D, const PixelWindow<W> &pw,
                                          const float2 *slots, int lane, int va, float da,
                                          int vb, float db, float &out_a, float &out_b)
{
    const int vv[2] = {va, vb};
    const float dd[2] = {da, db};
    float out[2];
    if (pw.full) eval_core<W, 2, HW, true>(D, pw, slots, lane, vv, dd, out);
    else eval_core<W, 2, HW, false>(D, pw, slots, lane, vv, dd, out);
    out_a = out[0];
    out_b = out[1];
}

// Window offsets (dx, dy) of every lane's slots: table[32 * i + lane] for slot i, filled
// cooperatively by a CTA (synchronise before use).
template <int W>
__device__ __forceinline__ void fill_slot_table(float2 *table)
{
    for (int k = threadIdx.x; k < 32 * Window<W>::NS; k += blockDim.x)
        table[k] = make_float2((float)(k % W), (float)(k / W));
}

}  // namespace pm
