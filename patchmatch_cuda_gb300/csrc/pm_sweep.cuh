// pm_sweep.cuh -- the PatchMatch kernels templated on the window side W (odd, 3..45).
//
//  sweep_kernel<W>  one directional sweep, topToDown / downToTop (patchMatch.cu:818-1209).
//                   One CTA per line with 1-4 warps. Every warp keeps its own copy of the
//                   step's window and of the sequential per-step state (messages, CDF,
//                   samples, argmin: identical arithmetic, so identical values); the NCC
//                   evaluations of a step are split across the warps and exchanged through
//                   shared memory.
//  costs_kernel<W>  every view's cost at the current depth, computeAllCostGivenDepth
//                   (patchMatch.cu:775-816); one warp per pixel.
//  eval_kernel<W>   windowed NCC for arbitrary (x, y, view, depth, axis) queries.
#pragma once

#include "pm_device.cuh"

namespace pm {

constexpr int MAX_BATCH_REFS = 256;
constexpr int MAX_WARPS_PER_LINE = 4;
constexpr int COST_BLOCK = 128;

struct SweepArgs {
    const RefDesc *refs;                 // device array of nrefs descriptors
    int nrefs;
    int total_lines;
    int dir;                             // pm_direction
    uint32_t sweep_id;
    int num_samples;                     // > 0 overrides the descriptors' (iteration 0: 1)
    int record_views;
    int line_start[MAX_BATCH_REFS + 1];  // prefix sums of lines per reference
};

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

template <int W, bool HW>
__global__ void __launch_bounds__(32 * MAX_WARPS_PER_LINE, 4)
sweep_kernel(const __grid_constant__ SweepArgs A)
{
    constexpr int NS = Window<W>::NS;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int wpl = blockDim.x >> 5;
    const int gline = blockIdx.x;
    const int r = find_ref(A, gline);
    const RefDesc &D = A.refs[r];
    const int line = gline - A.line_start[r];
    const int Wd = D.width, Hd = D.height, V = D.n_src;
    const int S = A.num_samples > 0 ? A.num_samples : D.num_samples;
    const bool rot = (A.dir == 0 || A.dir == 2);
    const bool fwd = (A.dir == 0 || A.dir == 1);
    const int axis = rot ? 1 : 0;
    const int nsteps = rot ? Wd : Hd;
    const float a2 = D.a2, u_emit = D.u_emit;
    const uint64_t seed = D.seed;
    const uint32_t batch = D.batch_id, sweep = A.sweep_id;
    const bool vl = lane < V;
    const unsigned all_views = V >= 32 ? FULL_MASK : ((1u << V) - 1u);
    float *cost = D.cost;
    float *bline = D.beta + (size_t)line * nsteps * V;

    __shared__ float s_res_f[2][MAX_VIEWS];  // NCC(view, previous step's depth), by step parity
    __shared__ float s_res_r[2][MAX_VIEWS];  // NCC(view, random depth)
    __shared__ float s_new[MAX_VIEWS];       // refreshed costs

    __shared__ float2 slots[32 * NS];
    __shared__ float btabs[MAX_WARPS_PER_LINE][32 * NS];
    float *btab = btabs[warp];
    fill_slot_table<W>(slots);
    __syncthreads();

#define PM_PIXEL(k, x, y)                                    \
    do {                                                     \
        const int c_ = fwd ? (k) : nsteps - 1 - (k);         \
        x = rot ? c_ : line;                                 \
        y = rot ? line : c_;                                 \
    } while (0)

    // 1. backward messages in reverse processing order (patchMatch.cu:856-869, :1050-1059)
    if (warp == 0) {
        float beta = 0.5f;
#pragma unroll 4
        for (int k = nsteps - 1; k >= 0; --k) {
            int x, y;
            PM_PIXEL(k, x, y);
            const uint32_t pix = (uint32_t)(y * Wd + x);
            if (vl) {
                bline[(size_t)k * V + lane] = beta;
                float c = cost[(size_t)pix * V + lane];
                if (c == 2.0f) c = 2.0f * draw_uniform(seed, pix, sweep, RNG_BWD, lane, batch);
                beta = msg_backward(beta, emission(c, a2), u_emit);
            }
        }
    }
    __syncthreads();

    // 2. forward message at the first step (patchMatch.cu:872-874)
    float alpha = 0.5f, d_former;
    {
        int x, y;
        PM_PIXEL(0, x, y);
        const uint32_t pix = (uint32_t)(y * Wd + x);
        if (vl) {
            float c = cost[(size_t)pix * V + lane];
            if (c == 2.0f) c = 2.0f * draw_uniform(seed, pix, sweep, RNG_FWD_POST, lane, batch);
            alpha = msg_forward(0.5f, emission(c, a2), u_emit);
        }
        d_former = D.depth[pix];
    }

    unsigned long long n_alg = 0, n_done = 0;
    // 3. propagation (patchMatch.cu:888-1000)
    for (int k = 1; k < nsteps; ++k) {
        const int par = k & 1;
        int x, y;
        PM_PIXEL(k, x, y);
        const uint32_t pix = (uint32_t)(y * Wd + x);
        const float c_old = vl ? cost[(size_t)pix * V + lane] : 0.0f;
        const float b = vl ? bline[(size_t)k * V + lane] : 0.0f;
        const float d_cur = D.depth[pix];
        PixelWindow<W> pw;
        load_window<W>(D, x, y, axis, lane, slots, btab, pw);

        // forward message with the old costs, posterior, CDF (:905-923)
        float q = 0.0f;
        if (vl) {
            float c = c_old;
            if (c == 2.0f) c = 2.0f * draw_uniform(seed, pix, sweep, RNG_FWD_PRE, lane, batch);
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
        const float d_rand =
            fmaf(draw_uniform(seed, pix, sweep, RNG_RAND_DEPTH, 0, batch), D.depth_span, D.depth_near);
        const float u_mine = lane < S ? draw_uniform(seed, pix, sweep, RNG_SAMPLE, lane, batch) : 2.0f;
        int my_sel = -1;
        unsigned umask = 0;
        for (int j = 0; j < S; ++j) {
            const float uj = __shfl_sync(FULL_MASK, u_mine, j);
            const unsigned bal = __ballot_sync(FULL_MASK, vl && uj <= cdf);
            const int view = bal ? __ffs(bal) - 1 : -1;
            if (lane == j) my_sel = view;
            if (view >= 0) umask |= 1u << view;
        }

        // Two phases of NCC evaluations, split across the line's warps (one call site):
        //  phase 0: every sampled view at the previous step's depth and the random depth;
        //  phase 1: every view at the chosen depth unless the current depth won (:983-994),
        //           sampled views reusing phase 0's identical evaluation.
        const int nu = __popc(umask);
        int idx = 1, tested = 0, nn = 0;
        unsigned need = 0;
        float best = d_cur;
        for (int phase = 0; phase < 2; ++phase) {
            const int ntasks = phase == 0 ? 2 * nu : nn;
            for (int t = warp; t < ntasks; t += wpl) {
                int v;
                float d;
                float *dst;
                if (phase == 0) {
                    v = nth_bit(umask, t >> 1);
                    d = (t & 1) ? d_rand : d_former;
                    dst = (t & 1) ? &s_res_r[par][v] : &s_res_f[par][v];
                } else {
                    v = nth_bit(need, t);
                    d = best;
                    dst = &s_new[v];
                }
                const float res = eval_one<W, HW>(D, pw, slots, lane, v, d);
                if (lane == 0) *dst = res;
            }
            if (phase == 1 && ntasks == 0) break;
            __syncthreads();
            if (phase == 1) break;
            // average over the samples in draw order, argmin with ties to the later index
            // (:965-979)
            float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
            for (int j = 0; j < S; ++j) {
                const int view = __shfl_sync(FULL_MASK, my_sel, j);
                if (view < 0) continue;
                ++tested;
                c0 += s_res_f[par][view];
                c1 += __shfl_sync(FULL_MASK, c_old, view);
                c2 += s_res_r[par][view];
            }
            if (tested > 0) {
                const float inv = 1.0f / (float)tested;
                c0 *= inv; c1 *= inv; c2 *= inv;
                idx = c0 < c1 ? 0 : 1;
                idx = (idx == 0 ? c0 : c1) < c2 ? idx : 2;
            }
            best = idx == 0 ? d_former : (idx == 1 ? d_cur : d_rand);
            if (idx == 1) break;
            need = all_views & ~umask;
            nn = __popc(need);
        }
        d_former = best;

        float c_new = c_old;
        if (idx != 1) {
            if (vl) c_new = (umask >> lane) & 1u ? (idx == 0 ? s_res_f[par][lane] : s_res_r[par][lane])
                                                 : s_new[lane];
            if (warp == 0) {
                if (vl) cost[(size_t)pix * V + lane] = c_new;
                if (lane == 0) {
                    n_alg += V;
                    n_done += nn;
                }
            }
        }
        if (warp == 0) {
            if (lane == 0) {
                D.depth[pix] = best;
                n_alg += 2 * tested;
                n_done += 2 * nu;
            }
            if (A.record_views && lane < S)
                D.view_sel[(size_t)lane * Wd * Hd + pix] = (uint8_t)(my_sel < 0 ? 255 : my_sel);
        }

        // forward message from the previous step's with the new costs (:996-999)
        if (vl) {
            float c = c_new;
            if (c == 2.0f) c = 2.0f * draw_uniform(seed, pix, sweep, RNG_FWD_POST, lane, batch);
            alpha = msg_forward(alpha, emission(c, a2), u_emit);
        }
    }
#undef PM_PIXEL
    if (warp == 0 && lane == 0) {
        atomicAdd(D.evals, n_alg);
        atomicAdd(D.evals + 1, n_done);
    }
}

// All views' costs at the current depth for every pixel of one reference.
template <int W, bool HW>
__global__ void __launch_bounds__(COST_BLOCK) costs_kernel(const RefDesc *refs, int r, int axis)
{
    constexpr int NS = Window<W>::NS;
    const RefDesc &D = refs[r];
    const int lane = threadIdx.x & 31;
    const int V = D.n_src;
    const int npix = D.width * D.height;
    __shared__ float2 slots[32 * NS];
    __shared__ float btabs[COST_BLOCK / 32][32 * NS];
    float *btab = btabs[threadIdx.x >> 5];
    fill_slot_table<W>(slots);
    __syncthreads();
    const int warps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int p = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); p < npix; p += warps) {
        const int x = p % D.width, y = p / D.width;
        PixelWindow<W> pw;
        load_window<W>(D, x, y, axis, lane, slots, btab, pw);
        const float d = D.depth[p];
        float mine = 0.0f;
        for (int v = 0; v + 1 < V; v += 2) {
            float na, nb;
            eval_pair<W, HW>(D, pw, slots, lane, v, d, v + 1, d, na, nb);
            if (lane == v) mine = na;
            if (lane == v + 1) mine = nb;
        }
        if (V & 1) {
            const float na = eval_one<W, HW>(D, pw, slots, lane, V - 1, d);
            if (lane == V - 1) mine = na;
        }
        if (lane < V) D.cost[(size_t)p * V + lane] = mine;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(D.evals, (unsigned long long)npix * V);
        atomicAdd(D.evals + 1, (unsigned long long)npix * V);
    }
}

// Windowed NCC for a list of queries, one warp per query.
template <int W, bool HW>
__global__ void __launch_bounds__(COST_BLOCK) eval_kernel(const RefDesc *refs, int r, int n,
                                                          const int4 *q, const float *depths,
                                                          float *out)
{
    constexpr int NS = Window<W>::NS;
    const RefDesc &D = refs[r];
    const int lane = threadIdx.x & 31;
    __shared__ float2 slots[32 * NS];
    __shared__ float btabs[COST_BLOCK / 32][32 * NS];
    float *btab = btabs[threadIdx.x >> 5];
    fill_slot_table<W>(slots);
    __syncthreads();
    const int warps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < n; i += warps) {
        const int4 t = q[i];  // x, y, view, axis
        PixelWindow<W> pw;
        load_window<W>(D, t.x, t.y, t.w, lane, slots, btab, pw);
        const float v = eval_one<W, HW>(D, pw, slots, lane, t.z, depths[i]);
        if (lane == 0) out[i] = v;
    }
}

}  // namespace pm
