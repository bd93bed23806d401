// pm_sweep.cuh -- the PatchMatch kernels templated on the window side W (odd, 3..45).
//
//  sweep_kernel<W>  one directional sweep, topToDown / downToTop (patchMatch.cu:818-1209).
//                   One CTA per line with 1-6 warps: warp 0 holds the line's sequential
//                   state, every warp evaluates NCCs, the next step's reference window is
//                   loaded one step ahead (see the kernel's comment).
//  costs_kernel<W>  every view's cost at the current depth, computeAllCostGivenDepth
//                   (patchMatch.cu:775-816); one warp per pixel, two views per pass.
//  eval_kernel<W>   windowed NCC for arbitrary (x, y, view, depth, axis) queries.
//  refine_kernel<W> depth refinement around the final depth on the last sweep's sampled views.
#pragma once

#include "pm_device.cuh"

namespace pm {

constexpr int MAX_BATCH_REFS = 256;
constexpr int MAX_WARPS_PER_LINE = 6;
// Register caps of the sweep kernel: 72 per thread with the texture-filtering sampler up to a
// 16-column window (the half-warp layout: nine 3-warp lines resident per SM), 96 for wider
// windows (the whole-warp layout's fully unrolled column holds more samples in flight: at 72
// the 19x19 kernel spilled 420 bytes, and the 8 x 3072x2048 batch took 13.4 s against 12.4 s
// at 96 and 12.9 s at 128); 96 with the exact sampler, whose gathers hold four texels.
template <int W, bool HW> struct SweepRegs { static constexpr int value = HW ? (W > 16 ? 96 : 72) : 96; };
constexpr int COST_BLOCK = 128;

struct SweepArgs {
    const RefDesc *refs;                 // device array of nrefs descriptors
    int nrefs;
    int total_lines;
    int dir;                             // pm_direction
    uint32_t sweep_id;
    int num_samples;                     // > 0 overrides the descriptors' (iteration 0: 1)
    int record_views;
    float perturb;                       // > 0: local random search of half-width perturb
    float decay;                         // 2^(-sweep/4): scales the slanted-plane search widths
    int line_mode;                       // which lines of each reference the blocks take (LineMode)
    int line_start[MAX_BATCH_REFS + 1];  // prefix sums of lines per reference
};

// The lines of a sweep a launch covers. A line within a half-window of an image edge (its
// windows cut across the line at every step) does more per step than an interior one, and the
// sweep lasts as long as its slowest line, so a sweep can run as two concurrent launches: the
// interior lines, and the edge lines with more warps per line, which the hardware places on the
// SMs the interior launch leaves room on.
enum LineMode : int {
    LINES_ALL = 0,       // lines 0 .. n-1
    LINES_INTERIOR = 1,  // lines hw .. n-hw-1
    LINES_EDGES = 2,     // lines 0 .. hw-1 and n-hw .. n-1 (every line when n < 2 hw)
};

// Lines of a reference a launch in `mode` covers, for a sweep of n lines and half-window hw.
__host__ __device__ inline int mode_lines(int mode, int n, int hw)
{
    const int interior = n > 2 * hw ? n - 2 * hw : 0;
    return mode == LINES_ALL ? n : mode == LINES_INTERIOR ? interior : n - interior;
}

__device__ __forceinline__ int find_ref(const SweepArgs &A, int gline)
{
    int lo = 0, hi = A.nrefs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (gline >= A.line_start[mid]) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Index of the t-th set bit of m (t < popc(m)).
__device__ __forceinline__ int nth_bit(unsigned m, int t)
{
    for (int i = 0; i < t; ++i) m &= m - 1;
    return __ffs(m) - 1;
}

// Per-step decisions of warp 0, published to the line's other warps (double-buffered by step
// parity: warp 0 writes step k+1's block while slower warps may still read step k's).
struct StepCtl {
    unsigned umask;          // views drawn by at least one sample
    int tested;              // samples that found a view
    float c1sum;             // sum of the drawn views' current costs, in draw order
    float d_former, d_rand, d_cur;
    int8_t sel[MAX_VIEWS];   // view of each draw, -1 when the CDF found none
};

// Slanted-plane mode: slopes of a step's three hypotheses (former, current, random), beside its
// StepCtl (only the plane-mode kernels use it).
struct PlaneCtl {
    float2 sl_f, sl_c, sl_r;
};

// The view-sample and random-depth draws of one step, made one step ahead (double-buffered).
// The cost-2 replacement draws are made by warp 0 when a cost of 2 occurs.
struct StepDraws {
    float sample[MAX_VIEWS];  // view samples (RNG_SAMPLE)
    float depth;              // random depth (RNG_RAND_DEPTH, first word)
    float mode;               // local or global random search (RNG_RAND_DEPTH, second word)
};

// One Philox counter per drawing lane (a single call site, so the lanes do not diverge). PL: the
// random-depth counter's third and fourth words go to *slopes (random slopes).
template <bool PL>
__device__ __forceinline__ void make_draws(const RefDesc &D, uint32_t pix, uint32_t sweep, int S,
                                           int lane, StepDraws &out, float2 *slopes)
{
    const uint64_t seed = D.seed;
    const uint32_t batch = D.batch_id;
    // lanes below S draw the view samples; the last lane the random depth (when S < 32)
    const bool depth_lane = lane == 31 && S < 32;
    if (lane < S || depth_lane) {
        if (PL) {
            const float4 u = draw_uniform4(seed, pix, sweep, depth_lane ? RNG_RAND_DEPTH : RNG_SAMPLE,
                                           depth_lane ? 0 : lane, batch);
            if (depth_lane) {
                out.depth = u.x;
                out.mode = u.y;
                *slopes = make_float2(u.z, u.w);
            } else {
                out.sample[lane] = u.x;
            }
        } else {
            const float2 u = draw_uniform2(seed, pix, sweep, depth_lane ? RNG_RAND_DEPTH : RNG_SAMPLE,
                                           depth_lane ? 0 : lane, batch);
            if (depth_lane) {
                out.depth = u.x;
                out.mode = u.y;
            } else {
                out.sample[lane] = u.x;
            }
        }
    }
    if (S >= 32 && lane == 0) {
        const float4 u = draw_uniform4(seed, pix, sweep, RNG_RAND_DEPTH, 0, batch);
        out.depth = u.x;
        out.mode = u.y;
        if (PL) *slopes = make_float2(u.z, u.w);
    }
}

// One directional sweep. One CTA per line of `blockDim.x / 32` warps. Warp 0 owns the line's
// sequential state (lane = source view): messages, posterior CDF, view samples, the argmin's
// current costs and the commit of each step; every warp evaluates NCCs. Per step:
//   before B1  warp 0 samples views and publishes them; warp 1 loads the next step's
//              reference window and warp 2 makes the draws two steps ahead (double and
//              triple buffers; with fewer warps the lower ones take these roles on);
//   B1 .. B2   each drawn view's NCC at the previous step's depth and at the random depth,
//              both in one pass over the window, the views spread over the warps;
//   B2 .. B3   every warp forms the same argmin; unless the current depth won, the other
//              views' NCCs at the chosen depth, two views per pass;
//   after B3   warp 0 commits the costs, the depth and the forward message.
template <int W, bool HW, bool PL>
__global__ void __maxnreg__((SweepRegs<W, HW>::value)) sweep_kernel(const __grid_constant__ SweepArgs A)
{
    constexpr int TAB = Window<W>::TAB;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    const int gline = blockIdx.x;
    const int r = find_ref(A, gline);
    __shared__ RefDesc D;
    __shared__ float4 s_hh[HH_F4 * MAX_VIEWS];
    stage_ref(A.refs[r], D, s_hh);
    __syncthreads();
    const int Wd = D.width, Hd = D.height, V = D.n_src;
    const int S = A.num_samples > 0 ? A.num_samples : D.num_samples;
    const bool rot = (A.dir == 0 || A.dir == 2);
    // the block's line: its index among the reference's lines of this launch's mode
    const int nlines = rot ? Hd : Wd, local = gline - A.line_start[r];
    const int line = A.line_mode == LINES_INTERIOR ? Window<W>::HW + local
                     : A.line_mode == LINES_EDGES && local >= min(Window<W>::HW, nlines)
                         ? nlines - mode_lines(LINES_EDGES, nlines, Window<W>::HW) + local
                         : local;
    const bool fwd = (A.dir == 0 || A.dir == 1);
    const int axis = rot ? 1 : 0;
    const int nsteps = rot ? Wd : Hd;
    const float a2 = D.a2, u_emit = D.u_emit;
    const uint32_t sweep = A.sweep_id;
    const bool vl = lane < V;
    const unsigned all_views = V >= 32 ? FULL_MASK : ((1u << V) - 1u);
    float *cost = D.cost;
    float *bline = D.beta + (size_t)line * nsteps * V;
    // before B1 of step k, warp 1 loads step k+1's window and warp 2 makes step k+2's draws
    // (with fewer warps the lower ones take these roles on)
    const int w_load = nw > 1 ? 1 : 0;
    const int w_draw = nw > 2 ? 2 : w_load;
    const int n_eval = nw;
    // evaluation tasks go to warps 1, 2, ..., nw-1, then 0
    const int task0 = (warp + n_eval - 1) % n_eval;

    __shared__ float s_tab[2][TAB];
    __shared__ float s_col[2][W];
    __shared__ WinCtl s_win[2];
    __shared__ StepDraws s_draw[3];
    __shared__ StepCtl s_ctl[2];
    __shared__ float s_res_f[MAX_VIEWS];  // NCC(view, previous step's depth)
    __shared__ float s_res_r[MAX_VIEWS];  // NCC(view, random depth)
    __shared__ float s_new[MAX_VIEWS];    // refreshed costs
    __shared__ float s_raw[W * W];        // reference values of the current window (ring)
    __shared__ float s_raw_o[W * W];      // the unshifted ones on a leading-edge line (quirks)
    __shared__ float2 s_wsl[2];           // slanted planes: the current slopes of steps k, k+1
    __shared__ float2 s_dsl[3];           // slanted planes: random-slope draws of steps k .. k+2
    __shared__ PlaneCtl s_pctl[2];        // slanted planes: the hypotheses' slopes

#define PM_PIXEL(k, x, y)                                    \
    do {                                                     \
        const int c_ = fwd ? (k) : nsteps - 1 - (k);         \
        x = rot ? c_ : line;                                 \
        y = rot ? line : c_;                                 \
    } while (0)

    // step kk's window (loader warp): when its extent along the sweep lies inside the image,
    // from the ring s_raw, sliding it by the entering line when it holds the previous step's
    // window (lines within a half-window of an edge, whose windows the border cuts across the
    // line, have a variant of their own); otherwise (a line's first and last half-window of
    // steps) loaded whole
    constexpr int HWIN = Window<W>::HW;
    const bool cut_line = line < HWIN || line + HWIN >= nlines;
    int ring_step = -1;  // the step whose window the ring holds
    auto load_step = [&](int kk, int xn, int yn) {
        if (rot ? (xn >= HWIN && xn + HWIN < Wd) : (yn >= HWIN && yn + HWIN < Hd)) {
            const int enter = ring_step != kk - 1 ? -1
                              : rot ? (fwd ? xn + HWIN : xn - HWIN) : (fwd ? yn + HWIN : yn - HWIN);
            if (cut_line)
                ring_window_cut<W>(D, xn, yn, !rot, enter, lane, s_raw, s_raw_o, s_tab[kk & 1], s_col[kk & 1],
                                   s_win[kk & 1]);
            else
                ring_window<W>(D, xn, yn, !rot, enter, lane, s_raw, s_tab[kk & 1], s_col[kk & 1], s_win[kk & 1]);
            ring_step = kk;
        } else {
            load_window<W>(D, xn, yn, axis, lane, s_tab[kk & 1], s_col[kk & 1], s_win[kk & 1]);
            ring_step = -1;
        }
        if (PL && lane == 0) s_wsl[kk & 1] = D.slopes[yn * Wd + xn];
    };

    // step k+1's window and step k+2's draws
    auto prep_step = [&](int k) {
        int xn, yn;
        if (warp == w_load && k + 1 < nsteps) {
            PM_PIXEL(k + 1, xn, yn);
            load_step(k + 1, xn, yn);
        }
        if (warp == w_draw && k + 2 < nsteps) {
            PM_PIXEL(k + 2, xn, yn);
            make_draws<PL>(D, (uint32_t)(yn * Wd + xn), sweep, S, lane, s_draw[(k + 2) % 3], &s_dsl[(k + 2) % 3]);
        }
    };

    float alpha = 0.5f, d_former = 0.0f;
    float c_next = 0.0f, b_next = 0.0f, d_next = 0.0f;
    // slanted-plane mode: the previous step's slopes and their plane scale at its own pixel
    // (x, y, s), kept in shared memory by warp 0's lane 0 so that no register holds them across
    // the NCC passes; a step's current slopes, loaded with its window (s_wsl[k & 1])
    __shared__ float4 s_former;
    unsigned long long n_alg = 0, n_done = 0;
    // backward messages in reverse processing order (patchMatch.cu:856-869, :1050-1059). Every
    // step's emissions are independent of the messages: all warps form them first (with the
    // cost-2 replacement draws) into the line's message buffer, then warp 0 runs the recurrence
    // over them, loading PB steps at a time so that their latency overlaps
    for (int i = threadIdx.x; i < nsteps * V; i += blockDim.x) {
        const int k = i / V, v = i - k * V;
        int x, y;
        PM_PIXEL(k, x, y);
        const uint32_t pix = (uint32_t)(y * Wd + x);
        float c = cost[(size_t)pix * V + v];
        if (c == 2.0f) c = 2.0f * draw_uniform(D.seed, pix, sweep, RNG_BWD, v, D.batch_id);
        bline[i] = emission(c, a2);
    }
    __syncthreads();
    if (warp == 0) {
        float beta = 0.5f;
        constexpr int PB = 16;
        for (int k0 = nsteps - 1; k0 >= 0; k0 -= PB) {
            float e[PB];
#pragma unroll
            for (int j = 0; j < PB; ++j) e[j] = vl && k0 - j >= 0 ? bline[(size_t)(k0 - j) * V + lane] : 0.0f;
#pragma unroll
            for (int j = 0; j < PB; ++j) {
                if (vl && k0 - j >= 0) {
                    bline[(size_t)(k0 - j) * V + lane] = beta;
                    beta = msg_backward(beta, e[j], u_emit);
                }
            }
        }
        // forward message at the first step (patchMatch.cu:872-874)
        int x, y;
        PM_PIXEL(0, x, y);
        const uint32_t pix = (uint32_t)(y * Wd + x);
        if (vl) {
            float c = cost[(size_t)pix * V + lane];
            if (c == 2.0f) c = 2.0f * draw_uniform(D.seed, pix, sweep, RNG_FWD_POST, lane, D.batch_id);
            alpha = msg_forward(0.5f, emission(c, a2), u_emit);
        }
        d_former = D.depth[pix];
        if (PL && lane == 0) {
            const float2 sl = D.slopes[pix];
            s_former = make_float4(sl.x, sl.y, plane_terms(D, sl, (float)x + 0.5f, (float)y + 0.5f).s, 0.0f);
        }
        if (nsteps > 1) {
            PM_PIXEL(1, x, y);
            const uint32_t p1 = (uint32_t)(y * Wd + x);
            if (vl) {
                c_next = cost[(size_t)p1 * V + lane];
                b_next = bline[(size_t)V + lane];
            }
            d_next = D.depth[p1];
        }
    }
    // step k's window in s_tab[k & 1], its draws in s_draw[k % 3]
    if (warp == w_load && nsteps > 1) {
        int x, y;
        PM_PIXEL(1, x, y);
        load_step(1, x, y);
    }
    if (warp == w_draw) {
        for (int k = 1; k < nsteps && k <= 2; ++k) {
            int x, y;
            PM_PIXEL(k, x, y);
            make_draws<PL>(D, (uint32_t)(y * Wd + x), sweep, S, lane, s_draw[k], &s_dsl[k]);
        }
    }
    __syncthreads();

    // propagation (patchMatch.cu:888-1000)
    for (int k = 1; k < nsteps; ++k) {
        const int buf = k & 1;
        int x, y;
        PM_PIXEL(k, x, y);
        const uint32_t pix = (uint32_t)(y * Wd + x);
        prep_step(k);
        float c_old = 0.0f;
        int my_sel = -1;
        if (warp == 0) {
            const StepDraws &dr = s_draw[k % 3];
            c_old = c_next;
            const float b = b_next;
            const float d_cur = d_next;
            if (k + 1 < nsteps) {  // prefetch the next step's costs, message and depth
                int xn, yn;
                PM_PIXEL(k + 1, xn, yn);
                const uint32_t pn = (uint32_t)(yn * Wd + xn);
                if (vl) {
                    c_next = cost[(size_t)pn * V + lane];
                    b_next = bline[(size_t)(k + 1) * V + lane];
                }
                d_next = D.depth[pn];
            }
            // forward message with the old costs, posterior, CDF (:905-923)
            float q = 0.0f;
            if (vl) {
                float c = c_old;
                if (c == 2.0f) c = 2.0f * draw_uniform(D.seed, pix, sweep, RNG_FWD_PRE, lane, D.batch_id);
                const float a = msg_forward(alpha, emission(c, a2), u_emit);
                const float z0 = a * b, z1 = (1.0f - a) * (1.0f - b);
                q = ftz(z0 / (z0 + z1));
            }
            float cdf = q;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float t = __shfl_up_sync(FULL_MASK, cdf, o);
                if (lane >= o) cdf += t;
            }
            cdf = cdf / __shfl_sync(FULL_MASK, cdf, V - 1);
            // random depth and view samples, first view with u <= CDF (:937-961)
            // the random hypothesis: uniform in [near, far] (patchMatch.cu:937); with a local
            // search (no counterpart in the reference) half of the pixels instead draw within
            // +-perturb (relative) of their current depth
            float d_rand = fmaf(dr.depth, D.depth_span, D.depth_near);
            float d_prop = d_former;
            if (PL) {
                // slanted planes (lane 0 publishes them): the previous step's plane carried to
                // this pixel (d s_prev / s_here), and a random hypothesis of one of three kinds
                if (lane == 0) {
                    const float lo = D.depth_near, hi = __fadd_rn(D.depth_near, D.depth_span);
                    const float4 f = s_former;
                    const float2 sl_f = make_float2(f.x, f.y), sl_cur = s_wsl[buf];
                    const PlaneG gp = plane_terms(D, sl_f, (float)x + 0.5f, (float)y + 0.5f);
                    d_prop = fminf(fmaxf(__fmul_rn(d_former, __fmul_rn(f.z, rcp_nr(gp.s))), lo), hi);
                    const float2 u = s_dsl[k % 3];
                    float2 sl_r = sl_cur;
                    if (dr.mode < PLANE_P_DEPTH) {
                        // a uniform depth with the current slopes (the reference's random depth)
                    } else if (dr.mode < PLANE_P_SLOPE) {
                        d_rand = d_cur;
                        sl_r = make_float2(__fmul_rn(SLOPE_DRAW, fmaf(2.0f, u.x, -1.0f)),
                                           __fmul_rn(SLOPE_DRAW, fmaf(2.0f, u.y, -1.0f)));
                    } else {
                        const float dstep = __fmul_rn(D.plane_dstep, A.decay);
                        const float sstep = __fmul_rn(D.plane_sstep, A.decay);
                        d_rand = fminf(fmaxf(__fmul_rn(d_cur, fmaf(dstep, fmaf(2.0f, dr.depth, -1.0f), 1.0f)), lo), hi);
                        sl_r.x = fminf(fmaxf(fmaf(sstep, fmaf(2.0f, u.x, -1.0f), sl_cur.x), -SLOPE_MAX), SLOPE_MAX);
                        sl_r.y = fminf(fmaxf(fmaf(sstep, fmaf(2.0f, u.y, -1.0f), sl_cur.y), -SLOPE_MAX), SLOPE_MAX);
                    }
                    PlaneCtl &P = s_pctl[buf];
                    P.sl_f = sl_f;
                    P.sl_c = sl_cur;
                    P.sl_r = sl_r;
                }
            } else if (A.perturb > 0.0f && dr.mode >= 0.5f) {
                d_rand = fminf(fmaxf(__fmul_rn(d_cur, fmaf(A.perturb, fmaf(2.0f, dr.depth, -1.0f), 1.0f)),
                                     D.depth_near),
                               D.depth_near + D.depth_span);
            }
            const float u_mine = lane < S ? dr.sample[lane] : 2.0f;
            StepCtl &C = s_ctl[buf];
            unsigned umask = 0;
            int tested = 0;
            float c1 = 0.0f;
            for (int j = 0; j < S; ++j) {
                const float uj = __shfl_sync(FULL_MASK, u_mine, j);
                const unsigned bal = __ballot_sync(FULL_MASK, vl && uj <= cdf);
                const int view = bal ? __ffs(bal) - 1 : -1;
                if (lane == j) my_sel = view;
                if (view >= 0) {
                    umask |= 1u << view;
                    ++tested;
                    c1 += __shfl_sync(FULL_MASK, c_old, view);
                }
            }
            if (lane < S) C.sel[lane] = (int8_t)my_sel;
            if (lane == 0) {
                C.umask = umask;
                C.tested = tested;
                C.c1sum = c1;
                C.d_former = d_prop;
                C.d_rand = d_rand;
                C.d_cur = d_cur;
            }
        }
        __syncthreads();  // B1

        const StepCtl &C = s_ctl[buf];
        const WinCtl &wc = s_win[buf];
        const float *tab = s_tab[buf];
        const float *col = s_col[buf];
        const unsigned umask = C.umask;
        const int nu = __popc(umask);
        const int tested = C.tested;
        // phase 0: each drawn view at the previous step's depth and at the random depth, in
        // one pass; phase 1 (unless the current depth won): every other view's cost at the
        // chosen depth (:983-994), two views per pass. One call site for both phases.
        int idx = 1, nn = 0;
        unsigned need = 0;
        float best = C.d_cur;
        for (int phase = 0; phase < 2; ++phase) {
            const int ntask = phase == 0 ? nu : (nn + 1) >> 1;
            for (int t = task0; t < ntask; t += n_eval) {
                int va, vb;
                float da, db;
                float2 sa, sb;
                if (phase == 0) {
                    va = vb = nth_bit(umask, t);
                    da = C.d_former;
                    db = C.d_rand;
                    sa = PL ? s_pctl[buf].sl_f : make_float2(0.0f, 0.0f);
                    sb = PL ? s_pctl[buf].sl_r : make_float2(0.0f, 0.0f);
                } else {
                    va = nth_bit(need, 2 * t);
                    vb = 2 * t + 1 < nn ? nth_bit(need, 2 * t + 1) : va;
                    da = db = best;
                    sa = sb = PL ? (idx == 0 ? s_pctl[buf].sl_f : s_pctl[buf].sl_r) : make_float2(0.0f, 0.0f);
                }
                float ra, rb;
                ncc_pair<W, HW, PL>(D, s_hh, wc, tab, col, lane, va, da, sa, vb, db, sb, ra, rb);
                if (lane == 0) {
                    if (phase == 0) {
                        s_res_f[va] = ra;
                        s_res_r[va] = rb;
                    } else {
                        s_new[va] = ra;
                        s_new[vb] = rb;
                    }
                }
            }
            __syncthreads();  // B2 after phase 0, B3 after phase 1
            if (phase == 1) break;
            // average over the samples in draw order, argmin with ties to the later index
            // (:965-979); every warp forms the same result from the same values
            if (tested > 0) {
                int sv = -1;
                float rf = 0.0f, rr = 0.0f;
                if (lane < S) {
                    sv = C.sel[lane];
                    if (sv >= 0) {
                        rf = s_res_f[sv];
                        rr = s_res_r[sv];
                    }
                }
                float c0 = 0.0f, c2 = 0.0f;
                for (int j = 0; j < S; ++j) {
                    const int view = __shfl_sync(FULL_MASK, sv, j);
                    const float f = __shfl_sync(FULL_MASK, rf, j), g = __shfl_sync(FULL_MASK, rr, j);
                    if (view < 0) continue;
                    c0 += f;
                    c2 += g;
                }
                const float inv = 1.0f / (float)tested;
                float c1 = C.c1sum;
                c0 *= inv; c1 *= inv; c2 *= inv;
                idx = c0 < c1 ? 0 : 1;
                idx = (idx == 0 ? c0 : c1) < c2 ? idx : 2;
            }
            best = idx == 0 ? C.d_former : (idx == 1 ? C.d_cur : C.d_rand);
            if (idx == 1) break;
            need = all_views & ~umask;
            nn = __popc(need);
        }

        if (warp == 0) {
            float c_new = c_old;
            if (idx != 1) {
                if (vl) {
                    c_new = (umask >> lane) & 1u ? (idx == 0 ? s_res_f[lane] : s_res_r[lane]) : s_new[lane];
                    cost[(size_t)pix * V + lane] = c_new;
                }
                if (lane == 0) {
                    n_alg += V;
                    n_done += nn;
                }
            }
            if (lane == 0) {
                D.depth[pix] = best;
                if (PL) {
                    const PlaneCtl &P = s_pctl[buf];
                    const float2 sl = idx == 0 ? P.sl_f : (idx == 1 ? P.sl_c : P.sl_r);
                    D.slopes[pix] = sl;
                    s_former = make_float4(sl.x, sl.y, plane_terms(D, sl, (float)x + 0.5f, (float)y + 0.5f).s, 0.0f);
                }
                n_alg += 2 * tested;
                n_done += 2 * nu;
            }
            if (A.record_views && lane < S && (D.record_sweep < 0 || (int)sweep == D.record_sweep))
                D.view_sel[(size_t)lane * Wd * Hd + pix] = (uint8_t)(my_sel < 0 ? 255 : my_sel);
            // forward message from the previous step's with the new costs (:996-999)
            if (vl) {
                float c = c_new;
                if (c == 2.0f) c = 2.0f * draw_uniform(D.seed, pix, sweep, RNG_FWD_POST, lane, D.batch_id);
                alpha = msg_forward(alpha, emission(c, a2), u_emit);
            }
            d_former = best;
        }
    }
#undef PM_PIXEL
    if (warp == 0 && lane == 0) {
        atomicAdd(D.evals, n_alg);
        atomicAdd(D.evals + 1, n_done);
    }
}

// All views' costs at the current depth for every pixel of one reference; one warp per pixel,
// two views per pass.
template <int W, bool HW, bool PL>
__global__ void __launch_bounds__(COST_BLOCK) costs_kernel(const RefDesc *refs, int r, int axis)
{
    constexpr int TAB = Window<W>::TAB;
    __shared__ RefDesc D;
    __shared__ float4 s_hh[HH_F4 * MAX_VIEWS];
    stage_ref(refs[r], D, s_hh);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int V = D.n_src;
    const int npix = D.width * D.height;
    __shared__ float tabs[COST_BLOCK / 32][TAB];
    __shared__ float cols[COST_BLOCK / 32][W];
    __shared__ WinCtl wcs[COST_BLOCK / 32];
    float *tab = tabs[threadIdx.x >> 5];
    float *col = cols[threadIdx.x >> 5];
    WinCtl &wc = wcs[threadIdx.x >> 5];
    const int warps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int p = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); p < npix; p += warps) {
        const int x = p % D.width, y = p / D.width;
        __syncwarp();
        load_window<W>(D, x, y, axis, lane, tab, col, wc);
        __syncwarp();
        const float d = D.depth[p];
        const float2 sl = PL ? D.slopes[p] : make_float2(0.0f, 0.0f);
        float mine = 0.0f;
        for (int v = 0; v < V; v += 2) {
            const int vb = v + 1 < V ? v + 1 : v;
            float na, nb;
            ncc_pair<W, HW, PL>(D, s_hh, wc, tab, col, lane, v, d, sl, vb, d, sl, na, nb);
            if (lane == v) mine = na;
            if (lane == vb) mine = nb;
        }
        if (lane < V) D.cost[(size_t)p * V + lane] = mine;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(D.evals, (unsigned long long)npix * V);
        atomicAdd(D.evals + 1, (unsigned long long)npix * V);
    }
}

// Windowed NCC for a list of queries, one warp per query; slopes (slanted-plane mode) may be
// null.
template <int W, bool HW, bool PL>
__global__ void __launch_bounds__(COST_BLOCK) eval_kernel(const RefDesc *refs, int r, int n,
                                                          const int4 *q, const float *depths,
                                                          const float2 *slopes, float *out)
{
    constexpr int TAB = Window<W>::TAB;
    __shared__ RefDesc D;
    __shared__ float4 s_hh[HH_F4 * MAX_VIEWS];
    stage_ref(refs[r], D, s_hh);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    __shared__ float tabs[COST_BLOCK / 32][TAB];
    __shared__ float cols[COST_BLOCK / 32][W];
    __shared__ WinCtl wcs[COST_BLOCK / 32];
    float *tab = tabs[threadIdx.x >> 5];
    float *col = cols[threadIdx.x >> 5];
    WinCtl &wc = wcs[threadIdx.x >> 5];
    const int warps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < n; i += warps) {
        const int4 t = q[i];  // x, y, view, axis
        __syncwarp();
        load_window<W>(D, t.x, t.y, t.w, lane, tab, col, wc);
        __syncwarp();
        float v, unused;
        const float2 sl = PL && slopes ? slopes[i] : make_float2(0.0f, 0.0f);
        ncc_pair<W, HW, PL>(D, s_hh, wc, tab, col, lane, t.z, depths[i], sl, t.z, depths[i], sl, v, unused);
        if (lane == 0) out[i] = v;
    }
}

// Depth refinement after the last sweep, the step the reference leaves out (patchMatch.cu:396;
// its never-launched depthRefinement kernel, :717-773): `trials` hypotheses d0 + sigma z around
// the current depth d0, z approximately standard normal (Irwin-Hall: sqrt(3) (u1 + u2 + u3 + u4
// - 2) from the four 24-bit uniforms of one Philox counter, in FP32 in this order), each scored
// by the mean cost over the views the last sweep sampled for the pixel (view_sel rows 0 ..
// samples-1, entries >= n_src meaning none); the lowest mean below the current depth's mean
// replaces it. Hypotheses outside [near, far] are skipped. Where the reference's kernel
// compares against one stored view cost and writes an uninitialised depth when no trial
// improves, this one compares against the mean at the current depth and keeps that depth.
// One warp per pixel.
constexpr float REFINE_SQRT3 = 1.7320508075688772f;

template <int W, bool HW, bool PL>
__global__ void __launch_bounds__(COST_BLOCK) refine_kernel(const RefDesc *refs, int r, int axis, int trials,
                                                            float sigma, uint32_t sweep_id, int samples)
{
    constexpr int TAB = Window<W>::TAB;
    __shared__ RefDesc D;
    __shared__ float4 s_hh[HH_F4 * MAX_VIEWS];
    stage_ref(refs[r], D, s_hh);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int npix = D.width * D.height;
    const int S = samples > 0 ? min(samples, D.num_samples) : D.num_samples;
    __shared__ float tabs[COST_BLOCK / 32][TAB];
    __shared__ float cols[COST_BLOCK / 32][W];
    __shared__ WinCtl wcs[COST_BLOCK / 32];
    float *tab = tabs[threadIdx.x >> 5];
    float *col = cols[threadIdx.x >> 5];
    WinCtl &wc = wcs[threadIdx.x >> 5];
    const float d_lo = D.depth_near, d_hi = __fadd_rn(D.depth_near, D.depth_span);
    unsigned long long evals = 0;
    const int warps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int p = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); p < npix; p += warps) {
        const int x = p % D.width, y = p / D.width;
        const int my_view = (lane < S && D.view_sel) ? (int)D.view_sel[(size_t)lane * npix + p] : 255;
        const unsigned mask = __ballot_sync(FULL_MASK, my_view < D.n_src);
        if (!mask) continue;
        const int nv = __popc(mask);
        __syncwarp();
        load_window<W>(D, x, y, axis, lane, tab, col, wc);
        __syncwarp();
        const float d0 = D.depth[p];
        const float2 sl = PL ? D.slopes[p] : make_float2(0.0f, 0.0f);
        auto score = [&](float dd) {
            float sum = 0.0f;
            for (int t = 0; t < nv; t += 2) {
                const int va = __shfl_sync(FULL_MASK, my_view, nth_bit(mask, t));
                const int vb = t + 1 < nv ? __shfl_sync(FULL_MASK, my_view, nth_bit(mask, t + 1)) : va;
                float na, nb;
                ncc_pair<W, HW, PL>(D, s_hh, wc, tab, col, lane, va, dd, sl, vb, dd, sl, na, nb);
                sum = __fadd_rn(sum, na);
                if (t + 1 < nv) sum = __fadd_rn(sum, nb);
            }
            return __fdiv_rn(sum, (float)nv);
        };
        float best = d0, best_cost = score(d0);
        evals += (unsigned long long)nv;
        for (int t = 0; t < trials; ++t) {
            const float4 u = draw_uniform4(D.seed, (uint32_t)p, sweep_id, RNG_REFINE, (uint32_t)t, D.batch_id);
            const float z = __fadd_rn(__fadd_rn(__fadd_rn(u.x, u.y), __fadd_rn(u.z, u.w)), -2.0f);
            const float dn = __fadd_rn(d0, __fmul_rn(__fmul_rn(z, REFINE_SQRT3), sigma));
            if (!(dn >= d_lo && dn <= d_hi)) continue;
            const float c = score(dn);
            evals += (unsigned long long)nv;
            if (c < best_cost) {
                best = dn;
                best_cost = c;
            }
        }
        if (lane == 0) D.depth[p] = best;
    }
    if (lane == 0 && evals) {
        atomicAdd(D.evals, evals);
        atomicAdd(D.evals + 1, evals);
    }
}

}  // namespace pm
