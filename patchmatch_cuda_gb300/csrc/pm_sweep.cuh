// pm_sweep.cuh -- the PatchMatch kernels templated on the window side W (odd, 3..45).
//
//  sweep_kernel<W>  one directional sweep, topToDown / downToTop (patchMatch.cu:818-1209);
//                   one warp per line, several references per launch.
//  costs_kernel<W>  every view's cost at the current depth, computeAllCostGivenDepth
//                   (patchMatch.cu:775-816); one warp per pixel.
//  eval_kernel<W>   windowed NCC for arbitrary (x, y, view, depth, axis) queries.
#pragma once

#include "pm_device.cuh"

namespace pm {

constexpr int MAX_BATCH_REFS = 256;
constexpr int SWEEP_BLOCK = 128;   // 4 lines per CTA

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

template <int W>
__device__ __forceinline__ float eval_one(const RefDesc &D, const PixelWindow<W> &pw,
                                          const float (&fdx)[Window<W>::NS],
                                          const float (&fdy)[Window<W>::NS], int v, float d)
{
    constexpr int NS = Window<W>::NS;
    const WarpSetup A = warp_setup(D, v, d, pw.scale, pw.ox, pw.oy);
    const cudaTextureObject_t ta = D.tex[v];
    const float sw = D.src_w[v], sh = D.src_h[v];
    float j = 0.f, jj = 0.f, ij = 0.f;
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        if (pw.inb & ((uint64_t)1 << i)) {
            const float dx = fdx[i], dy = fdy[i];
            const float px = fmaf(A.c0x, dx, fmaf(A.c1x, dy, A.bx));
            const float py = fmaf(A.c0y, dx, fmaf(A.c1y, dy, A.by));
            const float pz = fmaf(A.c0z, dx, fmaf(A.c1z, dy, A.bz));
            const float r = __fdividef(1.0f, pz);
            const float s = sample_source(ta, px * r, py * r, sw, sh);
            j += s; jj = fmaf(s, s, jj); ij = fmaf(pw.rv[i], s, ij);
        }
    }
    j = warp_sum(j); jj = warp_sum(jj); ij = warp_sum(ij);
    return ncc_finalize(j, jj, ij, pw.si, pw.sii, pw.n);
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

template <int W>
__global__ void __launch_bounds__(SWEEP_BLOCK) sweep_kernel(const __grid_constant__ SweepArgs A)
{
    constexpr int NS = Window<W>::NS;
    const int lane = threadIdx.x & 31;
    const int gline = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    if (gline >= A.total_lines) return;  // warp-uniform
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
    float *cost = D.cost;
    float *bline = D.beta + (size_t)line * nsteps * V;

    float fdx[NS], fdy[NS];
    slot_offsets<W>(lane, fdx, fdy);

#define PM_PIXEL(k, x, y)                                    \
    do {                                                     \
        const int c_ = fwd ? (k) : nsteps - 1 - (k);         \
        x = rot ? c_ : line;                                 \
        y = rot ? line : c_;                                 \
    } while (0)

    // 1. backward messages, reverse processing order (patchMatch.cu:856-869, :1050-1059)
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
        int x, y;
        PM_PIXEL(k, x, y);
        const uint32_t pix = (uint32_t)(y * Wd + x);
        const float c_old = vl ? cost[(size_t)pix * V + lane] : 0.0f;
        const float b = vl ? bline[(size_t)k * V + lane] : 0.0f;
        const float d_cur = D.depth[pix];
        PixelWindow<W> pw;
        load_window<W>(D, x, y, axis, lane, fdx, fdy, pw);

        // forward message with the old costs, posterior, CDF (:905-923)
        float q = 0.0f;
        if (vl) {
            float c = c_old;
            if (c == 2.0f) c = 2.0f * draw_uniform(seed, pix, sweep, RNG_FWD_PRE, lane, batch);
            const float a = msg_forward(alpha, emission(c, a2), u_emit);
            const float z0 = a * b, z1 = (1.0f - a) * (1.0f - b);
            q = z0 / (z0 + z1);
        }
        float cdf = q;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float t = __shfl_up_sync(FULL_MASK, cdf, o);
            if (lane >= o) cdf += t;
        }
        cdf = cdf / __shfl_sync(FULL_MASK, cdf, V - 1);

        // random depth and view samples (:937-961)
        const float d_rand =
            draw_uniform(seed, pix, sweep, RNG_RAND_DEPTH, 0, batch) * D.depth_span + D.depth_near;
        const float u_mine = lane < S ? draw_uniform(seed, pix, sweep, RNG_SAMPLE, lane, batch) : 2.0f;
        float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
        int tested = 0, my_sel = -1;
        float cache_f = 0.0f, cache_r = 0.0f;  // lane v: NCC(v, d_former), NCC(v, d_rand)
        bool cached = false;
        for (int j = 0; j < S; ++j) {
            const float uj = __shfl_sync(FULL_MASK, u_mine, j);
            const unsigned bal = __ballot_sync(FULL_MASK, vl && uj <= cdf);
            const int view = bal ? __ffs(bal) - 1 : -1;
            if (lane == j) my_sel = view;
            if (view < 0) continue;
            ++tested;
            float nf, nr;
            if (__shfl_sync(FULL_MASK, (int)cached, view)) {
                // sampled again (with replacement): same arithmetic, same result
                nf = __shfl_sync(FULL_MASK, cache_f, view);
                nr = __shfl_sync(FULL_MASK, cache_r, view);
            } else {
                eval_pair<W>(D, pw, fdx, fdy, view, d_former, view, d_rand, nf, nr);
                n_done += 2;
                if (lane == view) { cache_f = nf; cache_r = nr; cached = true; }
            }
            c0 += nf;
            c1 += __shfl_sync(FULL_MASK, c_old, view);
            c2 += nr;
        }
        n_alg += 2 * tested;

        // argmin with ties to the later index (:972-979, :613-618)
        int idx = 1;
        if (tested > 0) {
            const float inv = 1.0f / (float)tested;
            c0 *= inv; c1 *= inv; c2 *= inv;
            idx = c0 < c1 ? 0 : 1;
            idx = (idx == 0 ? c0 : c1) < c2 ? idx : 2;
        }
        const float best = idx == 0 ? d_former : (idx == 1 ? d_cur : d_rand);
        if (lane == 0) D.depth[pix] = best;
        d_former = best;

        // refresh every view's cost at the chosen depth unless the current depth won (:983-994)
        float c_new = c_old;
        if (idx != 1) {
            n_alg += V;
            float mine = idx == 0 ? cache_f : cache_r;
            unsigned need = __ballot_sync(FULL_MASK, vl && !cached);
            while (need) {
                const int va = __ffs(need) - 1;
                need &= need - 1;
                if (need) {
                    const int vb = __ffs(need) - 1;
                    need &= need - 1;
                    float na, nb;
                    eval_pair<W>(D, pw, fdx, fdy, va, best, vb, best, na, nb);
                    n_done += 2;
                    if (lane == va) mine = na;
                    if (lane == vb) mine = nb;
                } else {
                    const float na = eval_one<W>(D, pw, fdx, fdy, va, best);
                    n_done += 1;
                    if (lane == va) mine = na;
                }
            }
            c_new = mine;
            if (vl) cost[(size_t)pix * V + lane] = c_new;
        }

        // forward message from the previous step's with the new costs (:996-999)
        if (vl) {
            float c = c_new;
            if (c == 2.0f) c = 2.0f * draw_uniform(seed, pix, sweep, RNG_FWD_POST, lane, batch);
            alpha = msg_forward(alpha, emission(c, a2), u_emit);
        }
        if (A.record_views && lane < S)
            D.view_sel[(size_t)lane * Wd * Hd + pix] = (uint8_t)(my_sel < 0 ? 255 : my_sel);
    }
#undef PM_PIXEL
    if (lane == 0) {
        atomicAdd(D.evals, n_alg);
        atomicAdd(D.evals + 1, n_done);
    }
}

// All views' costs at the current depth for every pixel of one reference.
template <int W>
__global__ void __launch_bounds__(SWEEP_BLOCK) costs_kernel(const RefDesc *refs, int r, int axis)
{
    constexpr int NS = Window<W>::NS;
    const RefDesc &D = refs[r];
    const int lane = threadIdx.x & 31;
    const int V = D.n_src;
    const int npix = D.width * D.height;
    float fdx[NS], fdy[NS];
    slot_offsets<W>(lane, fdx, fdy);
    const int warps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int p = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); p < npix; p += warps) {
        const int x = p % D.width, y = p / D.width;
        PixelWindow<W> pw;
        load_window<W>(D, x, y, axis, lane, fdx, fdy, pw);
        const float d = D.depth[p];
        float mine = 0.0f;
        for (int v = 0; v + 1 < V; v += 2) {
            float na, nb;
            eval_pair<W>(D, pw, fdx, fdy, v, d, v + 1, d, na, nb);
            if (lane == v) mine = na;
            if (lane == v + 1) mine = nb;
        }
        if (V & 1) {
            const float na = eval_one<W>(D, pw, fdx, fdy, V - 1, d);
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
template <int W>
__global__ void __launch_bounds__(SWEEP_BLOCK) eval_kernel(const RefDesc *refs, int r, int n,
                                                          const int4 *q, const float *depths,
                                                          float *out)
{
    constexpr int NS = Window<W>::NS;
    const RefDesc &D = refs[r];
    const int lane = threadIdx.x & 31;
    float fdx[NS], fdy[NS];
    slot_offsets<W>(lane, fdx, fdy);
    const int warps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < n; i += warps) {
        const int4 t = q[i];  // x, y, view, axis
        PixelWindow<W> pw;
        load_window<W>(D, t.x, t.y, t.w, lane, fdx, fdy, pw);
        const float v = eval_one<W>(D, pw, fdx, fdy, t.z, depths[i]);
        if (lane == 0) out[i] = v;
    }
}

}  // namespace pm
