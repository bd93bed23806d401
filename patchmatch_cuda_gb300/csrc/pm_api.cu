// pm_api.cu -- the C ABI of include/patchmatch_gb300.h.
//
// A handle owns one CUDA stream, its device buffers (stream-ordered allocations from the
// device's default memory pool, whose release threshold is raised so repeated
// create/destroy cycles reuse memory), one gather-capable CUDA array and texture object per
// source view, and a CUDA graph of the whole run schedule, captured on first use.
#include <cuda_fp16.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/patchmatch_gb300.h"
#include "pm_internal.h"

using namespace pm;

struct pm_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // a sweep's edge lines run on `side`, forked from and joined back to `stream`
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    pm_params p{};
    int W = 0, H = 0, V = 0, win = 0;
    int texel_bytes = 4;
    std::string err;

    float *d_ref = nullptr, *d_sum_i = nullptr, *d_sum_ii = nullptr, *d_c1 = nullptr;
    float *d_depth = nullptr, *d_cost = nullptr, *d_beta = nullptr;
    float2 *d_slopes = nullptr;          // slanted-plane mode: per-pixel slopes
    uint8_t *d_view_sel = nullptr;
    unsigned long long *d_evals = nullptr;
    float4 *d_hh = nullptr;
    RefDesc *d_desc = nullptr;
    RefDesc h_desc{};
    cudaArray_t arr[MAX_VIEWS] = {};
    cudaTextureObject_t tex[MAX_VIEWS] = {};
    cudaArray_t layered = nullptr;          // texture-filtering sampler: sources as layers
    cudaTextureObject_t tex_layered = 0;
    int layer_w = 0, layer_h = 0;
    int src_w[MAX_VIEWS] = {}, src_h[MAX_VIEWS] = {};
    SweepArgs *h_sweep_args = nullptr;   // pinned, one per sweep of the schedule

    int wpl[2] = {0, 0};                // warps per line: [vertical sweeps, horizontal sweeps]
    int wpl_edge[2] = {0, 0};           // the same for the launch of the lines along the edges
    // learned proposal
    pm_net *net = nullptr;
    ProposalGeom geom{};
    int prop_src[2] = {0, 0};           // the two sources nearest to the reference camera
    float *d_quarter[3] = {nullptr, nullptr, nullptr};  // reference, source 0, source 1
    float *d_prop_in = nullptr, *d_prop_out = nullptr;
    cudaGraphExec_t graph = nullptr;
    bool ran = false;
    bool has_depth = false;             // a depth map was initialised, set or computed
    float cam_K[9] = {}, cam_R[9] = {}, cam_t[3] = {};   // the reference camera
    pm_stats stats{};
};

namespace {

const char *kStatusStrings[] = {
    "ok", "invalid argument", "window size out of range", "too few views",
    "too many source views", "invalid image", "invalid camera", "CUDA error", "out of memory",
    "I/O error", "no CUDA device", "call out of order", "unsupported",
    "image too wide for the fixed scratch of pm_box_moments_noalloc"};

pm_status fail(pm_handle *h, pm_status s, const std::string &msg)
{
    if (h) h->err = msg;
    return s;
}

pm_status cuda_fail(pm_handle *h, cudaError_t e, const char *what)
{
    cudaGetLastError();  // clear sticky-free errors
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (h) h->err = m;
    return e == cudaErrorMemoryAllocation ? PM_ERR_OUT_OF_MEMORY : PM_ERR_CUDA;
}

#define PM_CUDA(h, expr)                                        \
    do {                                                        \
        cudaError_t e_ = (expr);                                \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #expr); \
    } while (0)

// ---- camera setup in double precision (image.cpp:4-61) --------------------------------------
bool finite_all(const float *v, int n)
{
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

void mul3(const double *a, const double *b, double *o)
{
    double t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            t[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
    std::memcpy(o, t, sizeof t);
}

bool inv3(const double *m, double *o)
{
    const double c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8],
                 c02 = m[3] * m[7] - m[4] * m[6];
    const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    if (!(std::fabs(det) > 1e-300) || !std::isfinite(det)) return false;
    const double id = 1.0 / det;
    o[0] = c00 * id; o[1] = (m[2] * m[7] - m[1] * m[8]) * id; o[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    o[3] = c01 * id; o[4] = (m[0] * m[8] - m[2] * m[6]) * id; o[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    o[6] = c02 * id; o[7] = (m[1] * m[6] - m[0] * m[7]) * id; o[8] = (m[0] * m[4] - m[1] * m[3]) * id;
    return true;
}

// H1 = K_s R_s R_r^T K_r^-1, H2 = K_s R_s (C_s - C_r) n^T K_r^-1 with C = -R^T t.
// e_out (may be null): e = K_s T_rel, the translation term slanted planes use.
void relative_homographies(const pm_view &ref, const double *k_ref_inv, const pm_view &src,
                           double nx, double nz, double out[18], double *e_out = nullptr)
{
    double rr[9], tr[3], ks[9], rs[9], ts[3];
    for (int i = 0; i < 9; ++i) { rr[i] = ref.R[i]; ks[i] = src.K[i]; rs[i] = src.R[i]; }
    for (int i = 0; i < 3; ++i) { tr[i] = ref.t[i]; ts[i] = src.t[i]; }
    double cr[3], cs[3], rrt[9], rrel[9], h1[9];
    for (int i = 0; i < 3; ++i) {
        cr[i] = -(rr[i] * tr[0] + rr[3 + i] * tr[1] + rr[6 + i] * tr[2]);
        cs[i] = -(rs[i] * ts[0] + rs[3 + i] * ts[1] + rs[6 + i] * ts[2]);
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) rrt[3 * i + j] = rr[3 * j + i];
    mul3(rs, rrt, rrel);
    mul3(ks, rrel, h1);
    mul3(h1, k_ref_inv, h1);
    const double dc[3] = {cs[0] - cr[0], cs[1] - cr[1], cs[2] - cr[2]};
    double trel[3], kt[3], nk[3];
    for (int i = 0; i < 3; ++i) trel[i] = rs[3 * i] * dc[0] + rs[3 * i + 1] * dc[1] + rs[3 * i + 2] * dc[2];
    for (int i = 0; i < 3; ++i) kt[i] = ks[3 * i] * trel[0] + ks[3 * i + 1] * trel[1] + ks[3 * i + 2] * trel[2];
    for (int j = 0; j < 3; ++j) nk[j] = nx * k_ref_inv[j] + nz * k_ref_inv[6 + j];
    for (int i = 0; i < 9; ++i) out[i] = h1[i];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out[9 + 3 * i + j] = kt[i] * nk[j];
    if (e_out)
        for (int i = 0; i < 3; ++i) e_out[i] = kt[i];
}

// Prefilter taps (GaussianBlurCUDA.cu:99-130).
int prefilter_taps(int mode, float sigma, float *w)
{
    int kw = (int)(5.0f * sigma);
    if (kw % 2 == 0) kw += 1;
    int radius = (kw - 1) >> 1;
    if (kw > 45) { radius = 22; kw = 45; }
    else if (kw < 5) { radius = 2; kw = 5; }
    if (mode == PM_PREFILTER_BOX) {
        for (int i = 0; i < kw; ++i) w[i] = 1.0f / (float)kw;
    } else {
        double sum = 0.0, tmp[45];
        for (int i = -radius; i <= radius; ++i) {
            tmp[i + radius] = std::exp(-0.5 * (double)(i * i) / ((double)sigma * sigma));
            sum += tmp[i + radius];
        }
        for (int i = 0; i < kw; ++i) w[i] = (float)(tmp[i] / sum);
    }
    return radius;
}

// ---- a small cache of gather-capable CUDA arrays, so handle churn does not reallocate ----
struct ArrayKey {
    int device, w, h, bytes, layers;  // layers 0: a plain 2-D gather array
};
std::mutex g_array_mutex;
std::vector<std::pair<ArrayKey, cudaArray_t>> g_free_arrays;
bool g_pool_ready[64] = {};

cudaError_t acquire_array(int device, int w, int h, int bytes, cudaArray_t *out, int layers = 0)
{
    {
        std::lock_guard<std::mutex> lk(g_array_mutex);
        for (size_t i = 0; i < g_free_arrays.size(); ++i) {
            const ArrayKey &k = g_free_arrays[i].first;
            if (k.device == device && k.w == w && k.h == h && k.bytes == bytes && k.layers == layers) {
                *out = g_free_arrays[i].second;
                g_free_arrays.erase(g_free_arrays.begin() + (long)i);
                return cudaSuccess;
            }
        }
    }
    cudaChannelFormatDesc fmt = bytes == 1   ? cudaCreateChannelDesc<unsigned char>()
                                : bytes == 2 ? cudaCreateChannelDescHalf()
                                             : cudaCreateChannelDesc<float>();
    if (layers > 0)
        return cudaMalloc3DArray(out, &fmt, make_cudaExtent((size_t)w, (size_t)h, (size_t)layers),
                                 cudaArrayLayered);
    return cudaMallocArray(out, &fmt, (size_t)w, (size_t)h, cudaArrayTextureGather);
}

void release_array(int device, int w, int h, int bytes, cudaArray_t a, int layers = 0)
{
    std::lock_guard<std::mutex> lk(g_array_mutex);
    if (g_free_arrays.size() < 256) g_free_arrays.push_back({ArrayKey{device, w, h, bytes, layers}, a});
    else cudaFreeArray(a);
}

cudaError_t prepare_pool(int device)
{
    if (device < 0 || device >= 64 || g_pool_ready[device]) return cudaSuccess;
    cudaMemPool_t pool;
    cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, device);
    if (e != cudaSuccess) return e;
    uint64_t threshold = UINT64_MAX;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    if (e == cudaSuccess) g_pool_ready[device] = true;
    return e;
}

template <typename T>
cudaError_t dalloc(T **p, size_t bytes, cudaStream_t s)
{
    return cudaMallocAsync((void **)p, bytes ? bytes : 16, s);
}

int window_side(const pm_handle *h) { return 2 * h->p.half_window + 1; }

bool hw_of(const pm_handle *h) { return h->p.sampler == PM_SAMPLER_HARDWARE; }

bool pl_of(const pm_handle *h) { return h->p.planes != 0; }

cudaError_t enqueue_costs(pm_handle *h, int axis)
{
    LaunchReq req{};
    req.kind = LaunchKind::Costs;
    req.stream = h->stream;
    req.refs = h->d_desc;
    req.ref_index = 0;
    req.axis = axis;
    const int npix = h->W * h->H;
    req.grid = (npix + COST_BLOCK / 32 - 1) / (COST_BLOCK / 32);
    return launch_window(window_side(h), hw_of(h), pl_of(h), req);
}

// Window axis of a sweep direction: 1 for the horizontal sweeps (transposed windows).
inline int orient(int dir) { return (dir == PM_DIR_LEFT_TO_RIGHT || dir == PM_DIR_RIGHT_TO_LEFT) ? 1 : 0; }

// Depth refinement of descriptor `ref` of `refs` on stream s (refine_kernel).
cudaError_t enqueue_refine(const pm_handle *h, const RefDesc *refs, int ref, int axis, int trials, float sigma,
                           uint32_t sweep_id, int samples, cudaStream_t s)
{
    LaunchReq req{};
    req.kind = LaunchKind::Refine;
    req.stream = s;
    req.refs = refs;
    req.ref_index = ref;
    req.axis = axis;
    req.trials = trials;
    req.sigma = sigma;
    req.sweep_id = sweep_id;
    req.samples = samples;
    const int npix = h->W * h->H;
    req.grid = (npix + COST_BLOCK / 32 - 1) / (COST_BLOCK / 32);
    return launch_window(window_side(h), hw_of(h), pl_of(h), req);
}

// The refinement that ends a schedule of `nsweeps` sweeps: on the last sweep's orientation and
// sampled views (one sample when that sweep is in the first iteration after a random
// initialisation), keyed by sweep id nsweeps.
cudaError_t enqueue_final_refine(const pm_handle *h, const RefDesc *refs, int ref, int nsweeps, bool one_sample_first,
                                 cudaStream_t s)
{
    if (h->p.refine_trials <= 0 || nsweeps <= 0) return cudaSuccess;
    const int k = nsweeps - 1;
    const int samples = (k / 4 == 0 && one_sample_first) ? 1 : h->p.num_samples;
    return enqueue_refine(h, refs, ref, orient(k % 4), h->p.refine_trials, h->p.refine_sigma, (uint32_t)nsweeps,
                          samples, s);
}

void fill_sweep_args(SweepArgs &a, const RefDesc *refs, const int *lines, int nrefs, int dir,
                     uint32_t sweep_id, int num_samples, int record)
{
    a.refs = refs;
    a.nrefs = nrefs;
    a.dir = dir;
    a.sweep_id = sweep_id;
    a.num_samples = num_samples;
    a.record_views = record;
    a.perturb = 0.0f;
    a.decay = std::exp2(-0.25f * (float)sweep_id);
    a.line_mode = LINES_ALL;
    a.line_start[0] = 0;
    for (int i = 0; i < nrefs; ++i) a.line_start[i + 1] = a.line_start[i] + lines[i];
    a.total_lines = a.line_start[nrefs];
}

// The same sweep restricted to the lines of `mode` (lines: each reference's lines of the sweep).
SweepArgs sweep_args_mode(const SweepArgs &all, const int *lines, int win, int mode)
{
    SweepArgs a = all;
    a.line_mode = mode;
    a.line_start[0] = 0;
    for (int i = 0; i < a.nrefs; ++i) a.line_start[i + 1] = a.line_start[i] + mode_lines(mode, lines[i], win / 2);
    a.total_lines = a.line_start[a.nrefs];
    return a;
}

cudaError_t enqueue_sweep(int win, bool hw, bool pl, int wpl, const SweepArgs &a, cudaStream_t s)
{
    if (a.total_lines == 0) return cudaSuccess;
    LaunchReq req{};
    req.kind = LaunchKind::Sweep;
    req.stream = s;
    req.sweep = &a;
    req.grid = a.total_lines;
    req.block = 32 * wpl;
    return launch_window(win, hw, pl, req);
}

// One sweep of every line (`all`, LINES_ALL), as two concurrent launches when it has both
// interior and edge lines: the interior lines on s with wpl warps per line, the edge lines on
// `side` with wpl_edge, forked from s and joined back to it (graph edges under stream capture).
cudaError_t enqueue_sweep_split(int win, bool hw, bool pl, int wpl, int wpl_edge, const SweepArgs &all,
                                const int *lines, cudaStream_t s, cudaStream_t side, cudaEvent_t fork,
                                cudaEvent_t join)
{
    const SweepArgs ai = sweep_args_mode(all, lines, win, LINES_INTERIOR);
    const SweepArgs ae = sweep_args_mode(all, lines, win, LINES_EDGES);
    if (!side || ai.total_lines == 0 || ae.total_lines == 0) return enqueue_sweep(win, hw, pl, wpl, all, s);
    cudaError_t e = cudaEventRecord(fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(side, fork, 0);
    if (e == cudaSuccess) e = enqueue_sweep(win, hw, pl, wpl_edge, ae, side);
    if (e == cudaSuccess) e = cudaEventRecord(join, side);
    if (e == cudaSuccess) e = enqueue_sweep(win, hw, pl, wpl, ai, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, join, 0);
    return e;
}


// ---- warps-per-line tuner ----------------------------------------------------------------
// A line's steps are sequential, so a sweep takes ceil(lines / resident lines) line-times;
// more warps per line shorten a line-time but fit fewer lines. The tuner times one sweep
// of the real workload for each candidate and remembers the winner per shape.
// A shape the tuner remembers: the kernel (window, sampler, plane mode) and the work per sweep.
struct TuneKey {
    int device, win, n_src, num_samples, lines, steps, texel_bytes;
    bool hw, pl;
    bool operator==(const TuneKey &o) const
    {
        return device == o.device && win == o.win && n_src == o.n_src && num_samples == o.num_samples &&
               lines == o.lines && steps == o.steps && texel_bytes == o.texel_bytes && hw == o.hw && pl == o.pl;
    }
};
std::mutex g_tune_mutex;
std::vector<std::pair<TuneKey, int>> g_tuned;

int tuned_lookup(const TuneKey &k)
{
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    for (auto &e : g_tuned)
        if (e.first == k) return e.second;
    return 0;
}

void tuned_store(const TuneKey &k, int wpl)
{
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    g_tuned.push_back({k, wpl});
}

int lines_of(const pm_handle *h, int dir)
{
    return (dir == PM_DIR_LEFT_TO_RIGHT || dir == PM_DIR_RIGHT_TO_LEFT) ? h->H : h->W;
}

// A sweep of the handle's reference: interior and edge lines as two concurrent launches.
cudaError_t enqueue_handle_sweep(pm_handle *h, const SweepArgs &a, int wpl, int wpl_edge)
{
    const int lines = lines_of(h, a.dir);
    return enqueue_sweep_split(h->win, hw_of(h), pl_of(h), wpl, wpl_edge, a, &lines, h->stream, h->side, h->fork,
                               h->join);
}

// The whole run: initial depth, initial costs, iterations x 4 sweeps (patchMatch.cu:307-394).
// Half-width of the local random search in sweep k: perturbation x 2^(-k/4) (0: the
// reference's uniform search only).
float sweep_perturb(const pm_handle *h, int k)
{
    return h->p.perturbation > 0.0f ? h->p.perturbation * std::exp2(-0.25f * (float)k) : 0.0f;
}

// Sweeps the schedule runs: num_iterations x 4, or fewer when num_sweeps says so.
int schedule_sweeps(const pm_handle *h)
{
    const int all = 4 * h->p.num_iterations;
    return h->p.num_sweeps > 0 && h->p.num_sweeps < all ? h->p.num_sweeps : all;
}

// Learned initialisation on stream s: plane-sweep input, network, depth from its output.
cudaError_t enqueue_proposal_init(pm_handle *h, cudaStream_t s)
{
    if (!h->net || !h->d_prop_in) return cudaErrorInvalidValue;
    const ProposalGeom &g = h->geom;
    cudaError_t e = launch_sweep_input(g, h->d_quarter[0], h->d_quarter[1], h->d_quarter[2], h->d_prop_in, s);
    if (e != cudaSuccess) return e;
    if (pm_net_forward(h->net, h->d_prop_in, h->d_prop_out, s) != PM_OK) return cudaErrorLaunchFailure;
    return launch_proposal_init(h->d_desc, 0, h->W * h->H, g, h->d_prop_out, h->p.proposal_threshold, s);
}

// The whole run: initial depth, initial costs, iterations x 4 sweeps (patchMatch.cu:307-394).
cudaError_t enqueue_schedule(pm_handle *h)
{
    cudaError_t e = cudaMemsetAsync(h->d_evals, 0, 2 * sizeof(unsigned long long), h->stream);
    if (e != cudaSuccess) return e;
    if (h->p.init_mode == PM_INIT_PROPOSAL) e = enqueue_proposal_init(h, h->stream);
    else e = launch_init_depth(h->d_desc, 0, h->W * h->H, h->stream);
    if (e != cudaSuccess) return e;
    e = enqueue_costs(h, 1);
    if (e != cudaSuccess) return e;
    const int nsweeps = schedule_sweeps(h);
    for (int k = 0; k < nsweeps; ++k) {
        const int it = k / 4, d = k % 4;
        SweepArgs &a = h->h_sweep_args[k];
        const int lines = lines_of(h, d);
        // the first iteration samples one view after a random initialisation
        // (patchMatch.cu:307-316); a learned initialisation starts with meaningful costs and
        // samples numOfSamples from the start
        const int s_first = h->p.init_mode == PM_INIT_RANDOM ? 1 : 0;
        fill_sweep_args(a, h->d_desc, &lines, 1, d, (uint32_t)k, it == 0 ? s_first : 0, k == nsweeps - 1 ? 1 : 0);
        a.perturb = sweep_perturb(h, k);
        e = enqueue_handle_sweep(h, a, h->wpl[orient(d)], h->wpl_edge[orient(d)]);
        if (e != cudaSuccess) return e;
    }
    return enqueue_final_refine(h, h->d_desc, 0, nsweeps, h->p.init_mode == PM_INIT_RANDOM, h->stream);
}

// Picks warps per line for both sweep orientations, for the interior lines' launch and for the
// edge lines' one: the caller's choice (both the same), a remembered result, or timing
// candidates on the handle's own buffers (the run initialises them afterwards). The best counts
// depend on how far the state has converged (early sweeps refresh more views per step), so
// candidates are timed from two states, each restored before every trial: the state after the
// schedule's first iteration and the one after its third, weighted 1 : 3 like the schedule's
// sweeps after its first iteration. Every pair of counts is timed on single sweeps; the pairs
// near the best are then timed on whole iterations.
cudaError_t tune_warps_per_line(pm_handle *h)
{
    if (h->wpl[0] && h->wpl[1]) return cudaSuccess;
    if (h->p.threads_per_line) {
        h->wpl[0] = h->wpl[1] = h->wpl_edge[0] = h->wpl_edge[1] = h->p.threads_per_line / 32;
        h->stats.threads_per_line = h->p.threads_per_line;
        for (int i = 0; i < 4; ++i) h->stats.warps_per_line[i] = h->p.threads_per_line / 32;
        return cudaSuccess;
    }
    TuneKey keys[2];
    int picks[2];
    bool need = false;
    for (int o = 0; o < 2; ++o) {
        const int dir = o == 0 ? PM_DIR_TOP_TO_BOTTOM : PM_DIR_LEFT_TO_RIGHT;
        keys[o] = TuneKey{h->device, h->win, h->V, h->p.num_samples, lines_of(h, dir), o == 0 ? h->H : h->W,
                          h->texel_bytes, hw_of(h), pl_of(h)};
        picks[o] = tuned_lookup(keys[o]);  // interior warps | edge warps << 8
        need = need || !picks[o];
    }
    if (need) {
        const size_t npix = (size_t)h->W * h->H;
        const size_t state_floats = npix * (1 + (size_t)h->V) + (pl_of(h) ? 2 * npix : 0);
        float *snap = nullptr;  // two states
        cudaError_t e = cudaMallocAsync((void **)&snap, 2 * state_floats * sizeof(float), h->stream);
        if (e != cudaSuccess) return e;
        auto copy_state = [&](int which, bool save) {
            float *parts[3] = {h->d_depth, h->d_cost, (float *)h->d_slopes};
            const size_t n[3] = {npix, npix * h->V, pl_of(h) ? 2 * npix : 0};
            size_t off = which * state_floats;
            cudaError_t r = cudaSuccess;
            for (int i = 0; i < 3 && r == cudaSuccess; ++i) {
                if (!n[i]) continue;
                r = save ? cudaMemcpyAsync(snap + off, parts[i], n[i] * sizeof(float), cudaMemcpyDeviceToDevice, h->stream)
                         : cudaMemcpyAsync(parts[i], snap + off, n[i] * sizeof(float), cudaMemcpyDeviceToDevice, h->stream);
                off += n[i];
            }
            return r;
        };
        // the schedule's first three iterations from the initial depth and costs, at a middle
        // count of warps, with the states after the first and the third kept
        e = launch_init_depth(h->d_desc, 0, h->W * h->H, h->stream);
        if (e == cudaSuccess) e = enqueue_costs(h, 1);
        for (int k = 0; k < 12 && e == cudaSuccess; ++k) {
            SweepArgs a;
            const int d = k % 4, lines = lines_of(h, d);
            const int s_first = h->p.init_mode == PM_INIT_RANDOM ? 1 : 0;
            fill_sweep_args(a, h->d_desc, &lines, 1, d, (uint32_t)k, k < 4 ? s_first : 0, 0);
            e = enqueue_handle_sweep(h, a, 3, 4);
            if (e == cudaSuccess && k == 3) e = copy_state(0, true);
        }
        if (e == cudaSuccess) e = copy_state(1, true);
        std::vector<int> cand[2];  // each orientation's candidate pairs (interior | edge << 8)
        for (int o = 0; o < 2 && e == cudaSuccess; ++o) {
            if (picks[o]) {
                cand[o].push_back(picks[o]);
                continue;
            }
            const int dir = o == 0 ? PM_DIR_TOP_TO_BOTTOM : PM_DIR_LEFT_TO_RIGHT;
            SweepArgs a[2];
            const int lines = lines_of(h, dir);
            fill_sweep_args(a[0], h->d_desc, &lines, 1, dir, 4u + (uint32_t)dir, 0, 0);
            fill_sweep_args(a[1], h->d_desc, &lines, 1, dir, 12u + (uint32_t)dir, 0, 0);
            // score: the faster of two trials from each state, weighted 1 : 3
            auto score = [&](int wpl, int wpl_edge, float &out) {
                out = 0.0f;
                cudaError_t r = cudaSuccess;
                for (int st = 0; st < 2 && r == cudaSuccess; ++st) {
                    float best_of = 1e30f;
                    for (int rep = 0; rep < 2 && r == cudaSuccess; ++rep) {
                        float ms = 0.0f;
                        r = copy_state(st, false);
                        if (r == cudaSuccess) r = cudaEventRecord(h->ev[2], h->stream);
                        if (r == cudaSuccess) r = enqueue_handle_sweep(h, a[st], wpl, wpl_edge);
                        if (r == cudaSuccess) r = cudaEventRecord(h->ev[3], h->stream);
                        if (r == cudaSuccess) r = cudaEventSynchronize(h->ev[3]);
                        if (r == cudaSuccess) r = cudaEventElapsedTime(&ms, h->ev[2], h->ev[3]);
                        best_of = std::min(best_of, ms);
                    }
                    out += (st == 0 ? 1.0f : 3.0f) * best_of;
                }
                return r;
            };
            // every pair (interior warps, edge-line warps = interior .. interior + 2): the best
            // counts of the two launches depend on each other (how much room the interior launch
            // leaves decides where the edge blocks fit)
            std::vector<std::pair<float, int>> pairs;
            for (int wpl = 1; wpl <= MAX_WARPS_PER_LINE && e == cudaSuccess; ++wpl)
                for (int we = wpl; we <= std::min(wpl + 2, MAX_WARPS_PER_LINE) && e == cudaSuccess; ++we) {
                    float sc = 0.0f;
                    e = score(wpl, we, sc);
                    pairs.push_back({sc, wpl | (we << 8)});
                }
            std::sort(pairs.begin(), pairs.end());
            for (auto &pr : pairs)
                if (cand[o].size() < 8 && pr.first <= 1.10f * pairs.front().first) cand[o].push_back(pr.second);
        }
        // single sweeps from saved states do not rank near pairs as the schedule's sequence of
        // sweeps does: each orientation's candidates (its pairs within 10 % of the best single-
        // sweep score, at most 8) are timed on whole iterations (all four sweeps in the
        // schedule's order, from both states, weighted 1 : 3), the other orientation at its best
        // single-sweep pair; the fastest wins, a pair within 0.5 % of it with fewer warps first
        auto iteration_score = [&](const int c[4], float &out) {
            out = 0.0f;
            cudaError_t r = cudaSuccess;
            for (int st = 0; st < 2 && r == cudaSuccess; ++st) {
                float ms = 0.0f;
                r = copy_state(st, false);
                if (r == cudaSuccess) r = cudaEventRecord(h->ev[2], h->stream);
                for (int d = 0; d < 4 && r == cudaSuccess; ++d) {
                    SweepArgs a;
                    const int lines = lines_of(h, d), o = orient(d);
                    fill_sweep_args(a, h->d_desc, &lines, 1, d, (st == 0 ? 4u : 12u) + (uint32_t)d, 0, 0);
                    r = enqueue_handle_sweep(h, a, c[2 * o], c[2 * o + 1]);
                }
                if (r == cudaSuccess) r = cudaEventRecord(h->ev[3], h->stream);
                if (r == cudaSuccess) r = cudaEventSynchronize(h->ev[3]);
                if (r == cudaSuccess) r = cudaEventElapsedTime(&ms, h->ev[2], h->ev[3]);
                out += (st == 0 ? 1.0f : 3.0f) * ms;
            }
            return r;
        };
        int chosen[2] = {cand[0].empty() ? 0 : cand[0][0], cand[1].empty() ? 0 : cand[1][0]};
        bool warmed = false;
        for (int o = 0; o < 2 && e == cudaSuccess; ++o) {
            if (cand[o].size() < 2) continue;
            std::vector<std::pair<float, int>> scored;
            for (int pr : cand[o]) {
                int c[4] = {chosen[0] & 0xFF, chosen[0] >> 8, chosen[1] & 0xFF, chosen[1] >> 8};
                c[2 * o] = pr & 0xFF;
                c[2 * o + 1] = pr >> 8;
                float sc = 0.0f;
                if (!warmed) { e = iteration_score(c, sc); warmed = true; }  // warms the caches
                if (e == cudaSuccess) e = iteration_score(c, sc);
                if (e != cudaSuccess) break;
                scored.push_back({sc, pr});
            }
            if (e != cudaSuccess) break;
            float best = 1e30f;
            for (auto &x : scored) best = std::min(best, x.first);
            int fewest = 1 << 30;
            for (auto &x : scored) {
                const int warps = (x.second & 0xFF) + (x.second >> 8);
                if (x.first <= 1.005f * best && warps < fewest) { fewest = warps; chosen[o] = x.second; }
            }
        }
        if (e == cudaSuccess) { picks[0] = chosen[0]; picks[1] = chosen[1]; }
        if (e == cudaSuccess)
            for (int o = 0; o < 2; ++o) tuned_store(keys[o], picks[o]);
        const cudaError_t ef = cudaFreeAsync(snap, h->stream);
        if (e == cudaSuccess) e = ef;
        if (e != cudaSuccess) return e;
    }
    for (int o = 0; o < 2; ++o) {
        h->wpl[o] = picks[o] & 0xFF;
        h->wpl_edge[o] = picks[o] >> 8;
        h->stats.warps_per_line[2 * o] = h->wpl[o];
        h->stats.warps_per_line[2 * o + 1] = h->wpl_edge[o];
    }
    h->stats.threads_per_line = 32 * std::max(h->wpl[0], h->wpl[1]);
    return cudaSuccess;
}

// Warps per line for a batched launch: the most that still keeps every line resident.
int batch_wpl(int win, bool hw, bool pl, int total_lines, int device)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    for (int wpl = MAX_WARPS_PER_LINE; wpl > 1; --wpl) {
        int occ = 0;
        LaunchReq r{};
        r.kind = LaunchKind::SweepOccupancy;
        r.block = 32 * wpl;
        r.occupancy = &occ;
        if (launch_window(win, hw, pl, r) == cudaSuccess && total_lines <= occ * sms) return wpl;
    }
    return 1;
}

pm_status set_device(pm_handle *h)
{
    PM_CUDA(h, cudaSetDevice(h->device));
    return PM_OK;
}

}  // namespace

extern "C" {

void pm_default_params(pm_params *p)
{
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->depth_near = -1.0f;
    p->depth_far = -1.0f;
    p->half_window = 5;
    p->num_samples = 3;
    p->sp_alpha = 0.45f;
    p->gaussian_sigma = 1.0f;
    p->prefilter = PM_PREFILTER_NONE;
    p->num_iterations = 3;
    p->orientation_x = 0.0f;
    p->orientation_z = 1.0f;
    p->seed = 0x5EEDull;
    p->precision = PM_PRECISION_FP32;
    p->init_mode = PM_INIT_RANDOM;
    p->num_sweeps = 0;
    p->proposal_threshold = 0.5f;
    p->perturbation = 0.0f;
    p->refine_trials = 0;
    p->refine_sigma = 0.05f;
    p->planes = 0;
    p->plane_depth_step = 0.02f;
    p->plane_slope_step = 0.25f;
    p->threads_per_line = 0;
    p->quirks = 1;
    p->sampler = PM_SAMPLER_HARDWARE;
    p->gpu_id = -1;
    p->block_dim_x = 32;
    p->block_dim_y = 16;
}

int pm_struct_sizes(size_t *out, int n)
{
    const size_t sizes[] = {sizeof(pm_view), sizeof(pm_params), sizeof(pm_stats), sizeof(pm_fuse_params),
                            sizeof(pm_depth_view)};
    const int total = (int)(sizeof sizes / sizeof sizes[0]);
    if (!out || n <= 0) return 0;
    const int k = n < total ? n : total;
    for (int i = 0; i < k; ++i) out[i] = sizes[i];
    return k;
}

const char *pm_status_string(pm_status s)
{
    const int i = (int)s;
    return (i >= 0 && i < (int)(sizeof kStatusStrings / sizeof *kStatusStrings)) ? kStatusStrings[i]
                                                                                 : "unknown status";
}

const char *pm_last_error(const pm_handle *h) { return h ? h->err.c_str() : ""; }

pm_status pm_destroy(pm_handle *h)
{
    if (!h) return PM_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    for (int v = 0; v < MAX_VIEWS; ++v) {
        if (h->tex[v]) cudaDestroyTextureObject(h->tex[v]);
        if (h->arr[v]) release_array(h->device, h->src_w[v], h->src_h[v], h->texel_bytes, h->arr[v]);
    }
    if (h->tex_layered) cudaDestroyTextureObject(h->tex_layered);
    if (h->layered) release_array(h->device, h->layer_w, h->layer_h, h->texel_bytes, h->layered, h->V);
    void *bufs[] = {h->d_ref, h->d_sum_i, h->d_sum_ii, h->d_c1, h->d_depth, h->d_cost, h->d_beta, h->d_slopes,
                    h->d_view_sel, h->d_evals, h->d_hh, h->d_desc, h->d_quarter[0],
                    h->d_quarter[1], h->d_quarter[2], h->d_prop_in, h->d_prop_out};
    for (void *b : bufs)
        if (b) cudaFreeAsync(b, h->stream);
    if (h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    if (h->side) {
        cudaStreamSynchronize(h->side);
        cudaStreamDestroy(h->side);
    }
    for (cudaEvent_t e : h->ev)
        if (e) cudaEventDestroy(e);
    if (h->fork) cudaEventDestroy(h->fork);
    if (h->join) cudaEventDestroy(h->join);
    if (h->h_sweep_args) cudaFreeHost(h->h_sweep_args);
    delete h;
    return PM_OK;
}

pm_status pm_create(const pm_view *views, int n_views, int ref_id, const pm_params *params,
                    pm_handle **out)
{
    if (!out) return PM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!views || !params) return PM_ERR_INVALID_ARGUMENT;
    if (n_views < 2) return PM_ERR_TOO_FEW_VIEWS;
    if (ref_id < 0 || ref_id >= n_views) return PM_ERR_INVALID_ARGUMENT;
    if (n_views - 1 > PM_MAX_SOURCE_VIEWS) return PM_ERR_TOO_MANY_VIEWS;
    const pm_params &p = *params;
    if (p.half_window < 1 || p.half_window > PM_MAX_HALF_WINDOW) return PM_ERR_WINDOW_SIZE;
    if (p.num_samples < 1 || p.num_samples > 32 || p.num_iterations < 1 ||
        !(p.depth_near > 0.0f) || !(p.depth_far > p.depth_near) || !std::isfinite(p.depth_far) ||
        !(p.sp_alpha > 0.0f) || !std::isfinite(p.orientation_x) || !std::isfinite(p.orientation_z) ||
        p.prefilter < PM_PREFILTER_NONE || p.prefilter > PM_PREFILTER_GAUSSIAN ||
        (p.prefilter == PM_PREFILTER_GAUSSIAN && !(p.gaussian_sigma > 0.0f)) ||
        (p.precision != PM_PRECISION_FP32 && p.precision != PM_PRECISION_MIXED) ||
        (p.init_mode != PM_INIT_RANDOM && p.init_mode != PM_INIT_PROPOSAL) || p.num_sweeps < 0 ||
        !(p.proposal_threshold >= 0.0f && p.proposal_threshold <= 1.0f) ||
        !(p.perturbation >= 0.0f && p.perturbation < 1.0f) ||
        p.refine_trials < 0 || p.refine_trials > PM_MAX_REFINE_TRIALS ||
        (p.refine_trials > 0 && !(p.refine_sigma > 0.0f && std::isfinite(p.refine_sigma))) ||
        (p.planes != 0 && p.planes != 1) ||
        (p.planes && !(p.plane_depth_step >= 0.0f && p.plane_depth_step < 1.0f)) ||
        (p.planes && !(p.plane_slope_step >= 0.0f && p.plane_slope_step <= 2.0f)) ||
        (p.sampler != PM_SAMPLER_EXACT && p.sampler != PM_SAMPLER_HARDWARE) ||
        (p.texel_format != PM_TEXELS_AUTO && p.texel_format != PM_TEXELS_U8 &&
         p.texel_format != PM_TEXELS_F16 && p.texel_format != PM_TEXELS_F32) ||
        (p.texel_format == PM_TEXELS_U8 && p.prefilter != PM_PREFILTER_NONE) ||
        (p.threads_per_line % 32 != 0 || p.threads_per_line < 0 ||
         p.threads_per_line > 32 * MAX_WARPS_PER_LINE))
        return PM_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < n_views; ++i) {
        const pm_view &v = views[i];
        if (!v.gray || v.width < 1 || v.height < 1 || v.stride < v.width || v.width > 32768 ||
            v.height > 32768)
            return PM_ERR_IMAGE;
        if (!finite_all(v.K, 9) || !finite_all(v.R, 9) || !finite_all(v.t, 3)) return PM_ERR_CAMERA;
    }
    const pm_view &ref = views[ref_id];
    if ((long long)ref.width * ref.height * (n_views - 1) > (1ll << 31)) return PM_ERR_IMAGE;

    int device = p.gpu_id;
    if (device < 0) {
        if (cudaGetDevice(&device) != cudaSuccess) return PM_ERR_NO_DEVICE;
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0 || device >= count) return PM_ERR_NO_DEVICE;

    pm_handle *h = new pm_handle();
    h->device = device;
    h->p = p;
    h->W = ref.width;
    h->H = ref.height;
    h->V = n_views - 1;
    h->win = 2 * p.half_window + 1;
    for (int k = 0; k < 9; ++k) {
        h->cam_K[k] = ref.K[k];
        h->cam_R[k] = ref.R[k];
    }
    for (int k = 0; k < 3; ++k) h->cam_t[k] = ref.t[k];
    const bool filtered = p.prefilter != PM_PREFILTER_NONE;
    h->texel_bytes = p.texel_format != PM_TEXELS_AUTO ? p.texel_format
                     : p.precision == PM_PRECISION_FP32 ? (filtered ? 4 : 1) : (filtered ? 2 : 1);
    // The texture unit filters FP16 texels in reduced precision (about 2e-3): gather instead.
    if (h->texel_bytes == 2) h->p.sampler = PM_SAMPLER_EXACT;

    // camera setup
    double kr[9], kr_inv[9];
    for (int i = 0; i < 9; ++i) kr[i] = ref.K[i];
    if (!inv3(kr, kr_inv)) { pm_destroy(h); return PM_ERR_CAMERA; }
    constexpr int HHF = 4 * HH_F4;  // floats per view: H1, H2, e, padding
    std::vector<float> hh((size_t)h->V * HHF, 0.0f);
    int si = 0;
    for (int i = 0; i < n_views; ++i) {
        if (i == ref_id) continue;
        double o[18], ev[3];
        relative_homographies(ref, kr_inv, views[i], p.orientation_x, p.orientation_z, o, ev);
        for (int k = 0; k < 18; ++k) {
            if (!std::isfinite(o[k])) { pm_destroy(h); return PM_ERR_CAMERA; }
            hh[(size_t)si * HHF + k] = (float)o[k];
        }
        for (int k = 0; k < 3; ++k) {
            if (!std::isfinite(ev[k])) { pm_destroy(h); return PM_ERR_CAMERA; }
            hh[(size_t)si * HHF + 18 + k] = (float)ev[k];
        }
        h->src_w[si] = views[i].width;
        h->src_h[si] = views[i].height;
        ++si;
    }
    // proposal: the two sources whose camera centres are nearest the reference's, and their
    // homographies for fronto-parallel planes
    {
        auto centre = [](const pm_view &v, double c[3]) {
            for (int i = 0; i < 3; ++i)
                c[i] = -((double)v.R[i] * v.t[0] + (double)v.R[3 + i] * v.t[1] + (double)v.R[6 + i] * v.t[2]);
        };
        double cr[3];
        centre(ref, cr);
        std::vector<std::pair<double, int>> dist;
        int k = 0;
        for (int i = 0; i < n_views; ++i) {
            if (i == ref_id) continue;
            double c[3];
            centre(views[i], c);
            dist.push_back({(c[0] - cr[0]) * (c[0] - cr[0]) + (c[1] - cr[1]) * (c[1] - cr[1]) +
                                (c[2] - cr[2]) * (c[2] - cr[2]),
                            k++});
        }
        std::sort(dist.begin(), dist.end());
        h->prop_src[0] = dist[0].second;
        h->prop_src[1] = dist.size() > 1 ? dist[1].second : dist[0].second;
        ProposalGeom &g = h->geom;
        g.w4 = h->W / 4;
        g.h4 = h->H / 4;
        g.wp = (g.w4 + 15) / 16 * 16;
        g.hp = (g.h4 + 15) / 16 * 16;
        g.inv_far = 1.0f / p.depth_far;
        g.inv_range = 1.0f / p.depth_near - 1.0f / p.depth_far;
        for (int j = 0; j < 2; ++j) {
            int vi = -1;
            for (int i = 0, s2 = 0; i < n_views; ++i) {
                if (i == ref_id) continue;
                if (s2++ == h->prop_src[j]) vi = i;
            }
            double o[18];
            relative_homographies(ref, kr_inv, views[vi], 0.0, 1.0, o);
            for (int q = 0; q < 18; ++q) g.hh[j][q] = (float)o[q];
            g.sw4[j] = views[vi].width / 4;
            g.sh4[j] = views[vi].height / 4;
        }
    }

    pm_status st = set_device(h);
    if (st != PM_OK) { pm_destroy(h); return st; }
    cudaError_t e = prepare_pool(device);
    if (e != cudaSuccess) { st = cuda_fail(h, e, "memory pool"); pm_destroy(h); return st; }
#define PM_TRY(expr)                                                     \
    do {                                                                 \
        cudaError_t e_ = (expr);                                         \
        if (e_ != cudaSuccess) {                                         \
            pm_status s_ = cuda_fail(h, e_, #expr);                      \
            if (h->stream) cudaStreamSynchronize(h->stream);             \
            pm_destroy(h);                                               \
            return s_;                                                   \
        }                                                                \
    } while (0)
    PM_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    PM_TRY(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
    for (cudaEvent_t &ev : h->ev) PM_TRY(cudaEventCreate(&ev));
    PM_TRY(cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming));
    PM_TRY(cudaEventCreateWithFlags(&h->join, cudaEventDisableTiming));
    PM_TRY(cudaMallocHost((void **)&h->h_sweep_args, sizeof(SweepArgs) * 4 * (size_t)p.num_iterations));
    PM_TRY(cudaEventRecord(h->ev[0], h->stream));

    const size_t npix = (size_t)h->W * h->H;
    cudaStream_t s = h->stream;
    PM_TRY(dalloc(&h->d_ref, npix * 4, s));
    PM_TRY(dalloc(&h->d_sum_i, npix * 4, s));
    PM_TRY(dalloc(&h->d_sum_ii, npix * 4, s));
    PM_TRY(dalloc(&h->d_c1, npix * 4, s));
    PM_TRY(dalloc(&h->d_depth, npix * 4, s));
    PM_TRY(dalloc(&h->d_cost, npix * h->V * 4, s));
    PM_TRY(dalloc(&h->d_beta, npix * h->V * 4, s));
    if (p.planes) PM_TRY(dalloc(&h->d_slopes, npix * sizeof(float2), s));
    PM_TRY(dalloc(&h->d_view_sel, npix * (size_t)p.num_samples, s));
    PM_TRY(dalloc(&h->d_evals, 2 * sizeof(unsigned long long), s));
    PM_TRY(dalloc(&h->d_hh, hh.size() * 4, s));
    PM_TRY(dalloc(&h->d_desc, sizeof(RefDesc), s));
    if (h->geom.w4 > 0 && h->geom.h4 > 0) {
        PM_TRY(dalloc(&h->d_quarter[0], (size_t)h->geom.w4 * h->geom.h4 * 4 + 16, s));
        for (int j = 0; j < 2; ++j)
            PM_TRY(dalloc(&h->d_quarter[1 + j], (size_t)std::max(1, h->geom.sw4[j] * h->geom.sh4[j]) * 4 + 16, s));
    }
    PM_TRY(cudaMemsetAsync(h->d_view_sel, 255, npix * (size_t)p.num_samples, s));
    PM_TRY(cudaMemsetAsync(h->d_evals, 0, 2 * sizeof(unsigned long long), s));
    PM_TRY(cudaMemcpyAsync(h->d_hh, hh.data(), hh.size() * 4, cudaMemcpyHostToDevice, s));

    // images: u8 upload -> float texels (-> prefilter) -> reference maps / source arrays
    int max_w = 0, max_h = 0;
    for (int i = 0; i < n_views; ++i) {
        max_w = std::max(max_w, views[i].width);
        max_h = std::max(max_h, views[i].height);
    }
    const size_t max_pix = (size_t)max_w * max_h;
    int src_max_w = 0, src_max_h = 0;
    for (int i = 0; i < n_views; ++i) {
        if (i == ref_id) continue;
        src_max_w = std::max(src_max_w, views[i].width);
        src_max_h = std::max(src_max_h, views[i].height);
    }
    void *d_layer = nullptr;
    if (h->p.sampler == PM_SAMPLER_HARDWARE)
        PM_TRY(dalloc((uint8_t **)&d_layer, (size_t)src_max_w * src_max_h * h->texel_bytes, s));
    uint8_t *d_u8 = nullptr;
    float *d_f0 = nullptr, *d_f1 = nullptr, *d_f2 = nullptr;
    double *d_row_i = nullptr, *d_row_ii = nullptr;
    PM_TRY(dalloc(&d_u8, max_pix, s));
    PM_TRY(dalloc(&d_f0, max_pix * 4, s));
    PM_TRY(dalloc(&d_f1, max_pix * 4, s));
    PM_TRY(dalloc(&d_f2, max_pix * 4, s));
    PM_TRY(dalloc(&d_row_i, npix * 8, s));
    PM_TRY(dalloc(&d_row_ii, npix * 8, s));
    float taps[45];
    const int radius = filtered ? prefilter_taps(p.prefilter, p.gaussian_sigma, taps) : 0;
    si = 0;
    for (int i = 0; i < n_views; ++i) {
        const pm_view &v = views[i];
        PM_TRY(cudaMemcpy2DAsync(d_u8, (size_t)v.width, v.gray, (size_t)v.stride, (size_t)v.width,
                                 (size_t)v.height, cudaMemcpyHostToDevice, s));
        const bool is_ref = i == ref_id;
        if (h->d_quarter[0]) {
            const int sidx = is_ref ? -1 : (i < ref_id ? i : i - 1);
            if (is_ref) PM_TRY(launch_quarter(d_u8, v.width, h->geom.w4, h->geom.h4, h->d_quarter[0], s));
            for (int j = 0; j < 2; ++j)
                if (!is_ref && sidx == h->prop_src[j])
                    PM_TRY(launch_quarter(d_u8, v.width, h->geom.sw4[j], h->geom.sh4[j], h->d_quarter[1 + j], s));
        }
        float *texels = is_ref && !filtered ? h->d_ref : d_f0;
        PM_TRY(launch_u8_to_float(d_u8, v.width, texels, v.width, v.height, s));
        if (filtered) {
            float *dst = is_ref ? h->d_ref : d_f1;
            PM_TRY(launch_filter(d_f0, d_f2, dst, v.width, v.height, radius, taps, s));
            texels = dst;
        }
        if (is_ref) {
            PM_TRY(launch_box_moments(h->d_ref, d_row_i, d_row_ii, h->d_sum_i, h->d_sum_ii,
                                      h->d_c1, v.width, v.height, p.half_window, s));
            continue;
        }
        // source texels in the array's format
        const void *src_texels = d_u8;
        size_t src_pitch = (size_t)v.width;
        if (h->texel_bytes == 2) {
            PM_TRY(launch_float_to_half(texels, d_f2, v.width * v.height, s));
            src_texels = d_f2;
            src_pitch = (size_t)v.width * 2;
        } else if (h->texel_bytes == 4) {
            src_texels = texels;
            src_pitch = (size_t)v.width * 4;
        }
        if (h->p.sampler == PM_SAMPLER_HARDWARE) {
            // one layer per source, zero-padded to the largest source (the reference's layout,
            // patchMatch.cu:72-95); the padding reads as the border's zero
            if (!h->layered) {
                h->layer_w = src_max_w;
                h->layer_h = src_max_h;
                PM_TRY(acquire_array(device, h->layer_w, h->layer_h, h->texel_bytes, &h->layered, h->V));
            }
            const size_t lp = (size_t)h->layer_w * h->texel_bytes;
            PM_TRY(cudaMemsetAsync(d_layer, 0, lp * h->layer_h, s));
            PM_TRY(cudaMemcpy2DAsync(d_layer, lp, src_texels, src_pitch, src_pitch, (size_t)v.height,
                                     cudaMemcpyDeviceToDevice, s));
            cudaMemcpy3DParms cp{};
            cp.srcPtr = make_cudaPitchedPtr(d_layer, lp, (size_t)h->layer_w, (size_t)h->layer_h);
            cp.dstArray = h->layered;
            cp.dstPos = make_cudaPos(0, 0, (size_t)si);
            cp.extent = make_cudaExtent((size_t)h->layer_w, (size_t)h->layer_h, 1);
            cp.kind = cudaMemcpyDeviceToDevice;
            PM_TRY(cudaMemcpy3DAsync(&cp, s));
            ++si;
            continue;
        }
        cudaArray_t arr = nullptr;
        PM_TRY(acquire_array(device, v.width, v.height, h->texel_bytes, &arr));
        h->arr[si] = arr;
        PM_TRY(cudaMemcpy2DToArrayAsync(arr, 0, 0, src_texels, src_pitch, src_pitch, (size_t)v.height,
                                        cudaMemcpyDeviceToDevice, s));
        cudaResourceDesc rd{};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        cudaTextureDesc td{};
        td.addressMode[0] = cudaAddressModeBorder;
        td.addressMode[1] = cudaAddressModeBorder;
        td.filterMode = cudaFilterModePoint;
        td.readMode = h->texel_bytes == 1 ? cudaReadModeNormalizedFloat : cudaReadModeElementType;
        td.normalizedCoords = 0;
        PM_TRY(cudaCreateTextureObject(&h->tex[si], &rd, &td, nullptr));
        ++si;
    }
    if (h->p.sampler == PM_SAMPLER_HARDWARE) {
        cudaResourceDesc rd{};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = h->layered;
        cudaTextureDesc td{};
        td.addressMode[0] = cudaAddressModeBorder;
        td.addressMode[1] = cudaAddressModeBorder;
        td.addressMode[2] = cudaAddressModeBorder;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = h->texel_bytes == 1 ? cudaReadModeNormalizedFloat : cudaReadModeElementType;
        td.normalizedCoords = 0;
        PM_TRY(cudaCreateTextureObject(&h->tex_layered, &rd, &td, nullptr));
    }
    if (d_layer) PM_TRY(cudaFreeAsync(d_layer, s));
    PM_TRY(cudaFreeAsync(d_u8, s));
    PM_TRY(cudaFreeAsync(d_f0, s));
    PM_TRY(cudaFreeAsync(d_f1, s));
    PM_TRY(cudaFreeAsync(d_f2, s));
    PM_TRY(cudaFreeAsync(d_row_i, s));
    PM_TRY(cudaFreeAsync(d_row_ii, s));

    RefDesc &D = h->h_desc;
    std::memset(&D, 0, sizeof D);
    D.width = h->W;
    D.height = h->H;
    D.n_src = h->V;
    D.num_samples = p.num_samples;
    D.depth_near = p.depth_near;
    D.depth_span = p.depth_far - p.depth_near;
    D.a2 = p.sp_alpha * p.sp_alpha;
    D.u_emit = (float)std::exp(-0.5 * (double)0.83f * (double)0.83f / (double)D.a2);
    D.nx = p.orientation_x;
    D.nz = p.orientation_z;
    D.ik00 = (float)kr_inv[0];
    D.ik02 = (float)kr_inv[2];
    D.ik11 = (float)kr_inv[4];
    D.ik12 = (float)kr_inv[5];
    D.planes = p.planes;
    D.plane_dstep = p.plane_depth_step;
    D.plane_sstep = p.plane_slope_step;
    D.slopes = h->d_slopes;
    D.quirks = p.quirks ? 1 : 0;
    D.record_sweep = -1;
    D.hw_filter = h->p.sampler == PM_SAMPLER_HARDWARE ? 1 : 0;
    D.batch_id = 0;
    D.seed = p.seed;
    D.ref = h->d_ref;
    D.sum_i = h->d_sum_i;
    D.sum_ii = h->d_sum_ii;
    D.c1 = h->d_c1;
    D.depth = h->d_depth;
    D.cost = h->d_cost;
    D.beta = h->d_beta;
    D.view_sel = h->d_view_sel;
    D.evals = h->d_evals;
    D.hh = h->d_hh;
    D.tex_layered = h->tex_layered;
    for (int v = 0; v < h->V; ++v) {
        D.tex[v] = h->tex[v];
        D.src_w[v] = (float)h->src_w[v];
        D.src_h[v] = (float)h->src_h[v];
    }
    PM_TRY(cudaMemcpyAsync(h->d_desc, &D, sizeof D, cudaMemcpyHostToDevice, s));
    PM_TRY(cudaEventRecord(h->ev[1], s));
    PM_TRY(cudaStreamSynchronize(s));
#undef PM_TRY
    cudaEventElapsedTime(&h->stats.ms_prepare, h->ev[0], h->ev[1]);
    h->stats.texel_bytes = h->texel_bytes;
    *out = h;
    return PM_OK;
}

pm_status pm_run_async(pm_handle *h)
{
    if (!h) return PM_ERR_INVALID_ARGUMENT;
    if (h->p.init_mode == PM_INIT_PROPOSAL && !h->net)
        return fail(h, PM_ERR_STATE, "init_mode is PM_INIT_PROPOSAL but no network is attached");
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    if (!h->graph) {
        const cudaError_t et = tune_warps_per_line(h);
        if (et != cudaSuccess) return cuda_fail(h, et, "warps-per-line tuning");
        cudaGraph_t g = nullptr;
        PM_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        const cudaError_t e = enqueue_schedule(h);
        const cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
        if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(h, e, "schedule capture"); }
        if (e2 != cudaSuccess) return cuda_fail(h, e2, "cudaStreamEndCapture");
        const cudaError_t e3 = cudaGraphInstantiate(&h->graph, g, 0);
        cudaGraphDestroy(g);
        if (e3 != cudaSuccess) { h->graph = nullptr; return cuda_fail(h, e3, "cudaGraphInstantiate"); }
    }
    PM_CUDA(h, cudaEventRecord(h->ev[2], h->stream));
    PM_CUDA(h, cudaGraphLaunch(h->graph, h->stream));
    PM_CUDA(h, cudaEventRecord(h->ev[3], h->stream));
    h->ran = true;
    h->has_depth = true;
    return PM_OK;
}

pm_status pm_synchronize(pm_handle *h)
{
    if (!h) return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_run(pm_handle *h)
{
    pm_status st = pm_run_async(h);
    if (st != PM_OK) return st;
    st = pm_synchronize(h);
    if (st != PM_OK) return st;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, h->ev[2], h->ev[3]) == cudaSuccess) h->stats.ms_total = ms;
    unsigned long long ev[2];
    PM_CUDA(h, cudaMemcpy(ev, h->d_evals, sizeof ev, cudaMemcpyDeviceToHost));
    h->stats.cost_evals = ev[0];
    h->stats.cost_evals_done = ev[1];
    return PM_OK;
}

}  // extern "C"

// A batch of references on one device: groups of equal window side, sampler and plane mode, each with a
// device array of descriptors; every sweep of a group is one launch over the lines of all of
// its references.
struct pm_batch {
    struct Group {
        std::vector<pm_handle *> refs;
        RefDesc *d_descs = nullptr;
        int win = 0;
        bool hw = false;
        bool pl = false;      // slanted planes
        int wpl[2] = {0, 0};  // warps per line: vertical, horizontal sweeps (0: occupancy rule)
    };
    std::vector<pm_handle *> hs;
    std::vector<Group> groups;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    int launches = 0;
};

namespace {

// Initialisation, initial costs and every sweep of the batch on stream s.
cudaError_t enqueue_batch(pm_batch *b, cudaStream_t s)
{
    b->launches = 0;
    for (pm_batch::Group &g : b->groups) {
        const int m = (int)g.refs.size();
        int max_sweeps = 0;
        for (int i = 0; i < m; ++i) {
            pm_handle *h = g.refs[i];
            cudaError_t e = cudaMemsetAsync(h->d_evals, 0, 2 * sizeof(unsigned long long), s);
            if (e == cudaSuccess)
                e = h->p.init_mode == PM_INIT_PROPOSAL ? enqueue_proposal_init(h, s)
                                                      : launch_init_depth(g.d_descs, i, h->W * h->H, s);
            if (e != cudaSuccess) return e;
            LaunchReq req{};
            req.kind = LaunchKind::Costs;
            req.stream = s;
            req.refs = g.d_descs;
            req.ref_index = i;
            req.axis = 1;
            req.grid = (h->W * h->H + COST_BLOCK / 32 - 1) / (COST_BLOCK / 32);
            e = launch_window(h->win, hw_of(h), pl_of(h), req);
            if (e != cudaSuccess) return e;
            b->launches += 2;
            max_sweeps = std::max(max_sweeps, schedule_sweeps(h));
        }
        for (int k = 0; k < max_sweeps; ++k) {
            const int it = k / 4, d = k % 4;
            // references still sweeping at k, in descriptor order
            std::vector<int> lines(m, 0);
            for (int i = 0; i < m; ++i) lines[i] = schedule_sweeps(g.refs[i]) > k ? lines_of(g.refs[i], d) : 0;
            SweepArgs a;
            // one view sample in the first iteration after a random initialisation
            // (patchMatch.cu:307-316); a group mixing both initialisations follows its first
            // reference. Every sweep records the sampled views; a reference's last writes last.
            const int s_first = g.refs[0]->p.init_mode == PM_INIT_RANDOM ? 1 : 0;
            fill_sweep_args(a, g.d_descs, lines.data(), m, d, (uint32_t)k, it == 0 ? s_first : 0, 1);
            a.perturb = sweep_perturb(g.refs[0], k);
            const int wpl = g.wpl[orient(d)] ? g.wpl[orient(d)]
                                              : batch_wpl(g.win, g.hw, g.pl, a.total_lines, b->hs[0]->device);
            const cudaError_t e = enqueue_sweep(g.win, g.hw, g.pl, wpl, a, s);
            if (e != cudaSuccess) return e;
            ++b->launches;
        }
        for (int i = 0; i < m; ++i) {
            pm_handle *h = g.refs[i];
            if (h->p.refine_trials <= 0) continue;
            const cudaError_t e = enqueue_final_refine(h, g.d_descs, i, schedule_sweeps(h),
                                                       g.refs[0]->p.init_mode == PM_INIT_RANDOM, s);
            if (e != cudaSuccess) return e;
            ++b->launches;
        }
    }
    return cudaGetLastError();
}

// Warps per line for each group and orientation: the fastest of 1 .. MAX_WARPS_PER_LINE on one
// sweep of the whole group, every trial from the same state (each reference's initialisation
// and initial costs, restored before each launch; the first of two launches warms the caches).
cudaError_t tune_batch(pm_batch *b, cudaEvent_t e0, cudaEvent_t e1)
{
    cudaStream_t s = b->stream;
    for (pm_batch::Group &g : b->groups) {
        // a state to sweep: random initialisation and initial costs of every reference
        cudaError_t e = cudaSuccess;
        const int m = (int)g.refs.size();
        for (int i = 0; i < m && e == cudaSuccess; ++i) {
            pm_handle *h = g.refs[i];
            e = launch_init_depth(g.d_descs, i, h->W * h->H, s);
            LaunchReq req{};
            req.kind = LaunchKind::Costs;
            req.stream = s;
            req.refs = g.d_descs;
            req.ref_index = i;
            req.axis = 1;
            req.grid = (h->W * h->H + COST_BLOCK / 32 - 1) / (COST_BLOCK / 32);
            if (e == cudaSuccess) e = launch_window(h->win, hw_of(h), pl_of(h), req);
        }
        if (e != cudaSuccess) return e;
        // snapshot of every reference's depth, costs and (slanted planes) slopes
        std::vector<std::pair<void *, size_t>> parts;
        for (pm_handle *h : g.refs) {
            const size_t npix = (size_t)h->W * h->H;
            parts.push_back({h->d_depth, npix * sizeof(float)});
            parts.push_back({h->d_cost, npix * h->V * sizeof(float)});
            if (g.pl) parts.push_back({h->d_slopes, npix * sizeof(float2)});
        }
        size_t total = 0;
        for (auto &pt : parts) total += pt.second;
        char *snap = nullptr;
        e = cudaMallocAsync((void **)&snap, total, s);
        if (e != cudaSuccess) return e;
        auto copy_state = [&](bool save) {
            size_t off = 0;
            cudaError_t r = cudaSuccess;
            for (auto &pt : parts) {
                if (r == cudaSuccess)
                    r = save ? cudaMemcpyAsync(snap + off, pt.first, pt.second, cudaMemcpyDeviceToDevice, s)
                             : cudaMemcpyAsync(pt.first, snap + off, pt.second, cudaMemcpyDeviceToDevice, s);
                off += pt.second;
            }
            return r;
        };
        e = copy_state(true);
        for (int o = 0; o < 2 && e == cudaSuccess; ++o) {
            const int d = o == 0 ? PM_DIR_TOP_TO_BOTTOM : PM_DIR_LEFT_TO_RIGHT;
            std::vector<int> lines;
            for (pm_handle *h : g.refs) lines.push_back(lines_of(h, d));
            float best_ms = 1e30f;
            for (int wpl = 1; wpl <= MAX_WARPS_PER_LINE && e == cudaSuccess; ++wpl) {
                SweepArgs a;
                fill_sweep_args(a, g.d_descs, lines.data(), m, d, 0xFFFFFFF0u, 0, 0);
                float ms = 0.0f;
                for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {
                    e = copy_state(false);
                    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
                    if (e == cudaSuccess) e = enqueue_sweep(g.win, g.hw, g.pl, wpl, a, s);
                    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
                    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                }
                if (e == cudaSuccess && ms < best_ms) {
                    best_ms = ms;
                    g.wpl[o] = wpl;
                }
            }
        }
        const cudaError_t ef = cudaFreeAsync(snap, s);
        if (e == cudaSuccess) e = ef;
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

pm_status batch_setup(pm_handle *const *hs, int n, pm_batch *b)
{
    if (!hs || n < 1) return PM_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < n; ++i) {
        if (!hs[i]) return PM_ERR_INVALID_ARGUMENT;
        if (hs[i]->device != hs[0]->device) return PM_ERR_UNSUPPORTED;
        if (hs[i]->p.init_mode == PM_INIT_PROPOSAL && !hs[i]->net) return PM_ERR_STATE;
    }
    pm_status st = set_device(hs[0]);
    if (st != PM_OK) return st;
    for (int i = 0; i < n; ++i) PM_CUDA(hs[i], cudaStreamSynchronize(hs[i]->stream));
    b->hs.assign(hs, hs + n);
    b->stream = hs[0]->stream;
    std::vector<int> done(n, 0);
    for (int g0 = 0; g0 < n; ++g0) {
        if (done[g0]) continue;
        std::vector<pm_handle *> grp;
        for (int i = g0; i < n; ++i)
            if (!done[i] && hs[i]->win == hs[g0]->win && hw_of(hs[i]) == hw_of(hs[g0]) &&
                pl_of(hs[i]) == pl_of(hs[g0])) {
                grp.push_back(hs[i]);
                done[i] = 1;
            }
        for (size_t start = 0; start < grp.size(); start += MAX_BATCH_REFS) {
            pm_batch::Group g;
            g.refs.assign(grp.begin() + start, grp.begin() + std::min(grp.size(), start + MAX_BATCH_REFS));
            g.win = grp[0]->win;
            g.hw = hw_of(grp[0]);
            g.pl = pl_of(grp[0]);
            PM_CUDA(hs[0], cudaMalloc((void **)&g.d_descs, sizeof(RefDesc) * g.refs.size()));
            for (size_t i = 0; i < g.refs.size(); ++i) {
                // each reference records the views of its own last sweep only, as a single run does
                RefDesc d = g.refs[i]->h_desc;
                d.record_sweep = schedule_sweeps(g.refs[i]) - 1;
                PM_CUDA(hs[0], cudaMemcpy(g.d_descs + i, &d, sizeof(RefDesc), cudaMemcpyHostToDevice));
            }
            b->groups.push_back(g);
        }
    }
    return PM_OK;
}

void batch_free(pm_batch *b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (pm_batch::Group &g : b->groups)
        if (g.d_descs) cudaFree(g.d_descs);
}

pm_status batch_finish(pm_batch *b)
{
    PM_CUDA(b->hs[0], cudaStreamSynchronize(b->stream));
    for (pm_handle *h : b->hs) {
        unsigned long long ev[2];
        PM_CUDA(h, cudaMemcpy(ev, h->d_evals, sizeof ev, cudaMemcpyDeviceToHost));
        h->stats.cost_evals = ev[0];
        h->stats.cost_evals_done = ev[1];
        h->ran = true;
        h->has_depth = true;
    }
    return PM_OK;
}

}  // namespace

extern "C" {

pm_status pm_run_batch(pm_handle *const *hs, int n)
{
    pm_batch b;
    pm_status st = batch_setup(hs, n, &b);
    if (st == PM_OK) {
        const cudaError_t e = enqueue_batch(&b, b.stream);
        st = e == cudaSuccess ? batch_finish(&b) : cuda_fail(hs[0], e, "batch schedule");
    }
    batch_free(&b);
    return st;
}

pm_status pm_batch_create(pm_handle *const *hs, int n, pm_batch **out)
{
    if (!out) return PM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    pm_batch *b = new pm_batch();
    pm_status st = batch_setup(hs, n, b);
    if (st == PM_OK) {
        pm_handle *h0 = hs[0];
        cudaError_t e = tune_batch(b, h0->ev[2], h0->ev[3]);
        cudaGraph_t g = nullptr;
        if (e == cudaSuccess) e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t e1 = enqueue_batch(b, b->stream);
            const cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
            e = e1 != cudaSuccess ? e1 : e2;
        }
        if (e == cudaSuccess) {
            // kernel launches per run: the graph's kernel nodes (the proposal network's
            // included)
            size_t n_nodes = 0;
            e = cudaGraphGetNodes(g, nullptr, &n_nodes);
            std::vector<cudaGraphNode_t> nodes(n_nodes);
            if (e == cudaSuccess && n_nodes) e = cudaGraphGetNodes(g, nodes.data(), &n_nodes);
            int kernels = 0;
            for (size_t i = 0; e == cudaSuccess && i < n_nodes; ++i) {
                cudaGraphNodeType t;
                if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
            }
            b->launches = kernels;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) st = cuda_fail(h0, e, "batch graph");
    }
    if (st != PM_OK) {
        batch_free(b);
        delete b;
        return st;
    }
    *out = b;
    return PM_OK;
}

pm_status pm_batch_run(pm_batch *b)
{
    if (!b) return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(b->hs[0]);
    if (st != PM_OK) return st;
    PM_CUDA(b->hs[0], cudaGraphLaunch(b->graph, b->stream));
    return batch_finish(b);
}

pm_status pm_batch_info(const pm_batch *b, int *launches, int *groups, int *wpl, int max_groups)
{
    if (!b) return PM_ERR_INVALID_ARGUMENT;
    if (launches) *launches = b->launches;
    if (groups) *groups = (int)b->groups.size();
    if (wpl)
        for (int i = 0; i < (int)b->groups.size() && i < max_groups; ++i) {
            wpl[2 * i] = b->groups[i].wpl[0];
            wpl[2 * i + 1] = b->groups[i].wpl[1];
        }
    return PM_OK;
}

pm_status pm_batch_destroy(pm_batch *b)
{
    if (!b) return PM_OK;
    set_device(b->hs[0]);
    cudaStreamSynchronize(b->stream);
    batch_free(b);
    delete b;
    return PM_OK;
}

pm_status pm_get_depth(pm_handle *h, float *dst, size_t dst_pitch)
{
    if (!h || !dst) return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    if (dst_pitch == 0) dst_pitch = (size_t)h->W * 4;
    if (dst_pitch < (size_t)h->W * 4) return PM_ERR_INVALID_ARGUMENT;
    PM_CUDA(h, cudaMemcpy2DAsync(dst, dst_pitch, h->d_depth, (size_t)h->W * 4, (size_t)h->W * 4,
                                 (size_t)h->H, cudaMemcpyDeviceToHost, h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_get_view_selection(pm_handle *h, uint8_t *dst)
{
    if (!h || !dst) return PM_ERR_INVALID_ARGUMENT;
    if (!h->ran) return fail(h, PM_ERR_STATE, "no run has recorded a view selection yet");
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    PM_CUDA(h, cudaMemcpyAsync(dst, h->d_view_sel, (size_t)h->W * h->H * h->p.num_samples,
                               cudaMemcpyDeviceToHost, h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_save_depth(pm_handle *h, const char *path)
{
    if (!h || !path) return PM_ERR_INVALID_ARGUMENT;
    std::vector<float> d((size_t)h->W * h->H);
    pm_status st = pm_get_depth(h, d.data(), 0);
    if (st != PM_OK) return st;
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(h, PM_ERR_IO, std::string("cannot open ") + path);
    std::fprintf(f, "%d&%d&%d&", h->W, h->H, 1);
    const size_t wrote = std::fwrite(d.data(), sizeof(float), d.size(), f);
    const int closed = std::fclose(f);
    if (wrote != d.size() || closed != 0) return fail(h, PM_ERR_IO, std::string("short write to ") + path);
    return PM_OK;
}

pm_status pm_get_stats(const pm_handle *h, pm_stats *out)
{
    if (!h || !out) return PM_ERR_INVALID_ARGUMENT;
    *out = h->stats;
    return PM_OK;
}

pm_status pm_get_stream(const pm_handle *h, void **stream)
{
    if (!h || !stream) return PM_ERR_INVALID_ARGUMENT;
    *stream = (void *)h->stream;
    return PM_OK;
}

pm_status pm_get_size(const pm_handle *h, int *width, int *height, int *n_src)
{
    if (!h) return PM_ERR_INVALID_ARGUMENT;
    if (width) *width = h->W;
    if (height) *height = h->H;
    if (n_src) *n_src = h->V;
    return PM_OK;
}

pm_status pm_init_depth(pm_handle *h)
{
    if (!h) return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    if (h->p.init_mode == PM_INIT_PROPOSAL) {
        if (!h->net) return fail(h, PM_ERR_STATE, "init_mode is PM_INIT_PROPOSAL but no network is attached");
        PM_CUDA(h, enqueue_proposal_init(h, h->stream));
    } else {
        PM_CUDA(h, launch_init_depth(h->d_desc, 0, h->W * h->H, h->stream));
    }
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    h->has_depth = true;
    return PM_OK;
}

pm_status pm_compute_costs(pm_handle *h, int axis)
{
    if (!h || (axis != 0 && axis != 1)) return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    PM_CUDA(h, enqueue_costs(h, axis));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_refine(pm_handle *h, int trials, float sigma, uint32_t sweep_id, int num_samples, int axis)
{
    if (!h || trials < 0 || trials > PM_MAX_REFINE_TRIALS || !(sigma > 0.0f && std::isfinite(sigma)) ||
        num_samples < 0 || num_samples > h->p.num_samples || (axis != 0 && axis != 1))
        return PM_ERR_INVALID_ARGUMENT;
    if (!h->has_depth) return fail(h, PM_ERR_STATE, "pm_refine needs a depth map");
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    PM_CUDA(h, enqueue_refine(h, h->d_desc, 0, axis, trials, sigma, sweep_id, num_samples, h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_run_sweep(pm_handle *h, int direction, uint32_t sweep_id, int num_samples,
                       int record_views)
{
    if (!h || direction < 0 || direction > 3 || num_samples < 0 || num_samples > 32)
        return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    SweepArgs a;
    const int lines = lines_of(h, direction);
    fill_sweep_args(a, h->d_desc, &lines, 1, direction, sweep_id, num_samples, record_views ? 1 : 0);
    a.perturb = sweep_perturb(h, (int)sweep_id);
    if (record_views && num_samples > h->p.num_samples) return PM_ERR_INVALID_ARGUMENT;
    if (!h->wpl[orient(direction)]) {
        // the tuner sweeps the handle's own buffers: keep the caller's state (depth, costs and,
        // with slanted planes, the slopes) and put it back afterwards
        const size_t npix = (size_t)h->W * h->H;
        std::vector<float> d(npix), c(npix * h->V);
        std::vector<float2> sl(pl_of(h) ? npix : 0);
        PM_CUDA(h, cudaMemcpyAsync(d.data(), h->d_depth, d.size() * 4, cudaMemcpyDeviceToHost, h->stream));
        PM_CUDA(h, cudaMemcpyAsync(c.data(), h->d_cost, c.size() * 4, cudaMemcpyDeviceToHost, h->stream));
        if (!sl.empty())
            PM_CUDA(h, cudaMemcpyAsync(sl.data(), h->d_slopes, sl.size() * sizeof(float2), cudaMemcpyDeviceToHost,
                                       h->stream));
        PM_CUDA(h, cudaStreamSynchronize(h->stream));
        PM_CUDA(h, tune_warps_per_line(h));
        PM_CUDA(h, cudaMemcpyAsync(h->d_depth, d.data(), d.size() * 4, cudaMemcpyHostToDevice, h->stream));
        PM_CUDA(h, cudaMemcpyAsync(h->d_cost, c.data(), c.size() * 4, cudaMemcpyHostToDevice, h->stream));
        if (!sl.empty())
            PM_CUDA(h, cudaMemcpyAsync(h->d_slopes, sl.data(), sl.size() * sizeof(float2), cudaMemcpyHostToDevice,
                                       h->stream));
        PM_CUDA(h, cudaStreamSynchronize(h->stream));  // the host copies must outlive the transfers
    }
    PM_CUDA(h, cudaEventRecord(h->ev[2], h->stream));
    PM_CUDA(h, enqueue_handle_sweep(h, a, h->wpl[orient(direction)], h->wpl_edge[orient(direction)]));
    PM_CUDA(h, cudaEventRecord(h->ev[3], h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, h->ev[2], h->ev[3]) == cudaSuccess) h->stats.ms_sweeps = ms;
    unsigned long long ev[2];
    PM_CUDA(h, cudaMemcpy(ev, h->d_evals, sizeof ev, cudaMemcpyDeviceToHost));
    h->stats.cost_evals = ev[0];
    h->stats.cost_evals_done = ev[1];
    if (record_views) h->ran = true;
    return PM_OK;
}

pm_status pm_set_depth(pm_handle *h, const float *src)
{
    if (!h || !src) return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    PM_CUDA(h, cudaMemcpyAsync(h->d_depth, src, (size_t)h->W * h->H * 4, cudaMemcpyHostToDevice, h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    h->has_depth = true;
    return PM_OK;
}

pm_status pm_fusion_create_from_engines(pm_handle *const *hs, int n, pm_fusion **out)
{
    if (!out) return PM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!hs || n < 1 || n > PM_MAX_FUSE_REFS) return PM_ERR_INVALID_ARGUMENT;
    std::vector<FuseSource> src((size_t)n);
    for (int i = 0; i < n; ++i) {
        const pm_handle *h = hs[i];
        if (!h) return PM_ERR_INVALID_ARGUMENT;
        if (h->device != hs[0]->device) return PM_ERR_INVALID_ARGUMENT;
        if (!h->has_depth) return PM_ERR_STATE;
        FuseSource &f = src[(size_t)i];
        f = FuseSource{};
        f.d_depth = h->d_depth;
        f.d_intensity = h->d_ref;
        f.width = h->W;
        f.height = h->H;
        for (int k = 0; k < 9; ++k) {
            f.K[k] = h->cam_K[k];
            f.R[k] = h->cam_R[k];
        }
        for (int k = 0; k < 3; ++k) f.t[k] = h->cam_t[k];
        f.wait_stream = h->stream;
    }
    return fusion_create(src.data(), n, hs[0]->device, out);
}

pm_status pm_get_costs(pm_handle *h, float *dst)
{
    if (!h || !dst) return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    PM_CUDA(h, cudaMemcpyAsync(dst, h->d_cost, (size_t)h->W * h->H * h->V * 4, cudaMemcpyDeviceToHost, h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_set_costs(pm_handle *h, const float *src)
{
    if (!h || !src) return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    PM_CUDA(h, cudaMemcpyAsync(h->d_cost, src, (size_t)h->W * h->H * h->V * 4, cudaMemcpyHostToDevice, h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_get_ref_maps(pm_handle *h, float *ref, float *sum_i, float *sum_ii)
{
    if (!h) return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    const size_t bytes = (size_t)h->W * h->H * 4;
    if (ref) PM_CUDA(h, cudaMemcpyAsync(ref, h->d_ref, bytes, cudaMemcpyDeviceToHost, h->stream));
    if (sum_i) PM_CUDA(h, cudaMemcpyAsync(sum_i, h->d_sum_i, bytes, cudaMemcpyDeviceToHost, h->stream));
    if (sum_ii) PM_CUDA(h, cudaMemcpyAsync(sum_ii, h->d_sum_ii, bytes, cudaMemcpyDeviceToHost, h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_get_source_texels(pm_handle *h, int view, float *dst)
{
    if (!h || !dst || view < 0 || view >= h->V) return PM_ERR_INVALID_ARGUMENT;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    const int w = h->src_w[view], hgt = h->src_h[view], b = h->texel_bytes;
    std::vector<uint8_t> raw((size_t)w * hgt * b);
    if (h->layered) {
        cudaMemcpy3DParms cp{};
        cp.srcArray = h->layered;
        cp.srcPos = make_cudaPos(0, 0, (size_t)view);
        cp.dstPtr = make_cudaPitchedPtr(raw.data(), (size_t)w * b, (size_t)w, (size_t)hgt);
        cp.extent = make_cudaExtent((size_t)w, (size_t)hgt, 1);
        cp.kind = cudaMemcpyDeviceToHost;
        PM_CUDA(h, cudaMemcpy3DAsync(&cp, h->stream));
    } else {
        PM_CUDA(h, cudaMemcpy2DFromArrayAsync(raw.data(), (size_t)w * b, h->arr[view], 0, 0,
                                              (size_t)w * b, (size_t)hgt, cudaMemcpyDeviceToHost,
                                              h->stream));
    }
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    const size_t n = (size_t)w * hgt;
    if (b == 1) {
        for (size_t i = 0; i < n; ++i) dst[i] = (float)raw[i] / 255.0f;
    } else if (b == 2) {
        const __half *hp = (const __half *)raw.data();
        for (size_t i = 0; i < n; ++i) dst[i] = __half2float(hp[i]);
    } else {
        std::memcpy(dst, raw.data(), n * 4);
    }
    return PM_OK;
}

namespace {
pm_status eval_costs(pm_handle *h, int n, const int *xs, const int *ys, const int *views, const float *depths,
                     const float *slopes, const int *axes, float *out);
}

pm_status pm_eval_costs(pm_handle *h, int n, const int *xs, const int *ys, const int *views,
                        const float *depths, const int *axes, float *out)
{
    return eval_costs(h, n, xs, ys, views, depths, nullptr, axes, out);
}

pm_status pm_eval_costs_planes(pm_handle *h, int n, const int *xs, const int *ys, const int *views,
                               const float *depths, const float *slopes, const int *axes, float *out)
{
    if (h && !h->d_slopes) return fail(h, PM_ERR_STATE, "the handle was created without slanted planes");
    if (n > 0 && !slopes) return PM_ERR_INVALID_ARGUMENT;
    return eval_costs(h, n, xs, ys, views, depths, slopes, axes, out);
}

}  // extern "C"

namespace {
pm_status eval_costs(pm_handle *h, int n, const int *xs, const int *ys, const int *views, const float *depths,
                     const float *slopes, const int *axes, float *out)
{
    if (!h || n < 0 || (n > 0 && (!xs || !ys || !views || !depths || !axes || !out)))
        return PM_ERR_INVALID_ARGUMENT;
    if (n == 0) return PM_OK;
    std::vector<int4> q((size_t)n);
    for (int i = 0; i < n; ++i) {
        if (xs[i] < 0 || xs[i] >= h->W || ys[i] < 0 || ys[i] >= h->H || views[i] < 0 ||
            views[i] >= h->V || (axes[i] != 0 && axes[i] != 1))
            return fail(h, PM_ERR_INVALID_ARGUMENT, "query out of range");
        q[(size_t)i] = make_int4(xs[i], ys[i], views[i], axes[i]);
    }
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    int4 *d_q = nullptr;
    float *d_d = nullptr, *d_o = nullptr;
    float2 *d_s = nullptr;
    cudaStream_t s = h->stream;
    PM_CUDA(h, cudaMallocAsync((void **)&d_q, sizeof(int4) * n, s));
    PM_CUDA(h, cudaMallocAsync((void **)&d_d, sizeof(float) * n, s));
    PM_CUDA(h, cudaMallocAsync((void **)&d_o, sizeof(float) * n, s));
    if (slopes) PM_CUDA(h, cudaMallocAsync((void **)&d_s, sizeof(float2) * n, s));
    PM_CUDA(h, cudaMemcpyAsync(d_q, q.data(), sizeof(int4) * n, cudaMemcpyHostToDevice, s));
    PM_CUDA(h, cudaMemcpyAsync(d_d, depths, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    if (slopes) PM_CUDA(h, cudaMemcpyAsync(d_s, slopes, sizeof(float2) * n, cudaMemcpyHostToDevice, s));
    LaunchReq req{};
    req.kind = LaunchKind::Eval;
    req.stream = s;
    req.refs = h->d_desc;
    req.ref_index = 0;
    req.n = n;
    req.queries = d_q;
    req.depths = d_d;
    req.slopes = d_s;
    req.out = d_o;
    req.grid = std::min((n + COST_BLOCK / 32 - 1) / (COST_BLOCK / 32), 65535);
    PM_CUDA(h, launch_window(h->win, hw_of(h), pl_of(h), req));
    PM_CUDA(h, cudaMemcpyAsync(out, d_o, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    PM_CUDA(h, cudaFreeAsync(d_q, s));
    PM_CUDA(h, cudaFreeAsync(d_d, s));
    PM_CUDA(h, cudaFreeAsync(d_o, s));
    if (d_s) PM_CUDA(h, cudaFreeAsync(d_s, s));
    PM_CUDA(h, cudaStreamSynchronize(s));
    return PM_OK;
}
}  // namespace

extern "C" {

pm_status pm_get_slopes(pm_handle *h, float *dst)
{
    if (!h || !dst) return PM_ERR_INVALID_ARGUMENT;
    if (!h->d_slopes) return fail(h, PM_ERR_STATE, "the handle was created without slanted planes");
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    PM_CUDA(h, cudaMemcpyAsync(dst, h->d_slopes, (size_t)h->W * h->H * sizeof(float2), cudaMemcpyDeviceToHost,
                               h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_set_slopes(pm_handle *h, const float *src)
{
    if (!h || !src) return PM_ERR_INVALID_ARGUMENT;
    if (!h->d_slopes) return fail(h, PM_ERR_STATE, "the handle was created without slanted planes");
    const size_t n = (size_t)h->W * h->H * 2;
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(src[i])) return fail(h, PM_ERR_INVALID_ARGUMENT, "slopes must be finite");
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    PM_CUDA(h, cudaMemcpyAsync(h->d_slopes, src, n * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_get_normals(pm_handle *h, float *dst)
{
    if (!h || !dst) return PM_ERR_INVALID_ARGUMENT;
    std::vector<float> sl((size_t)h->W * h->H * 2);
    pm_status st = pm_get_slopes(h, sl.data());
    if (st != PM_OK) return st;
    for (size_t i = 0; i < (size_t)h->W * h->H; ++i) {
        const double a = sl[2 * i], b = sl[2 * i + 1];
        const double inv = 1.0 / std::sqrt(a * a + b * b + 1.0);
        dst[3 * i] = (float)(a * inv);
        dst[3 * i + 1] = (float)(b * inv);
        dst[3 * i + 2] = (float)inv;
    }
    return PM_OK;
}

pm_status pm_sample_source(pm_handle *h, int view, int n, const float *xs, const float *ys,
                           float *out)
{
    if (!h || view < 0 || view >= h->V || n < 0 || (n > 0 && (!xs || !ys || !out)))
        return PM_ERR_INVALID_ARGUMENT;
    if (n == 0) return PM_OK;
    pm_status st = set_device(h);
    if (st != PM_OK) return st;
    float *d = nullptr;
    cudaStream_t s = h->stream;
    PM_CUDA(h, cudaMallocAsync((void **)&d, sizeof(float) * 3 * (size_t)n, s));
    PM_CUDA(h, cudaMemcpyAsync(d, xs, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    PM_CUDA(h, cudaMemcpyAsync(d + n, ys, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    PM_CUDA(h, launch_sample(h->d_desc, 0, view, n, d, d + n, d + 2 * (size_t)n, s));
    PM_CUDA(h, cudaMemcpyAsync(out, d + 2 * (size_t)n, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    PM_CUDA(h, cudaFreeAsync(d, s));
    PM_CUDA(h, cudaStreamSynchronize(s));
    return PM_OK;
}

pm_status pm_transpose_layers(const float *d_in, size_t in_pitch, float *d_out, size_t out_pitch,
                              int width, int height, int layers, void *stream)
{
    if (!d_in || !d_out || width < 1 || height < 1 || layers < 1 ||
        in_pitch < (size_t)width * 4 || out_pitch < (size_t)height * 4)
        return PM_ERR_INVALID_ARGUMENT;
    cudaError_t e = launch_transpose(d_in, in_pitch, d_out, out_pitch, width, height, layers,
                                     (cudaStream_t)stream);
    if (e != cudaSuccess) { cudaGetLastError(); return PM_ERR_CUDA; }
    return PM_OK;
}

pm_status pm_set_proposal(pm_handle *h, pm_net *net)
{
    if (!h) return PM_ERR_INVALID_ARGUMENT;
    if (net) {
        int b = 0, hh = 0, ww = 0;
        if (pm_net_size(net, &b, &hh, &ww) != PM_OK || b != 1 || hh != h->geom.hp || ww != h->geom.wp)
            return fail(h, PM_ERR_INVALID_ARGUMENT, "proposal network size does not match the handle");
        const pm_status st = set_device(h);
        if (st != PM_OK) return st;
        const size_t n = (size_t)h->geom.hp * h->geom.wp;
        if (!h->d_prop_in) PM_CUDA(h, cudaMalloc((void **)&h->d_prop_in, n * PROPOSAL_IN_CH * sizeof(float)));
        if (!h->d_prop_out) PM_CUDA(h, cudaMalloc((void **)&h->d_prop_out, n * 2 * sizeof(float)));
    }
    if (h->net != net && h->graph) {  // the captured schedule holds the old network's launches
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    h->net = net;
    return PM_OK;
}

pm_status pm_proposal_input(pm_handle *h, float *d_out, int *height, int *width)
{
    if (!h) return PM_ERR_INVALID_ARGUMENT;
    if (height) *height = h->geom.hp;
    if (width) *width = h->geom.wp;
    if (!d_out) return PM_OK;
    if (!h->d_quarter[0]) return fail(h, PM_ERR_UNSUPPORTED, "image smaller than 4 x 4");
    const pm_status st = set_device(h);
    if (st != PM_OK) return st;
    PM_CUDA(h, launch_sweep_input(h->geom, h->d_quarter[0], h->d_quarter[1], h->d_quarter[2], d_out, h->stream));
    PM_CUDA(h, cudaStreamSynchronize(h->stream));
    return PM_OK;
}

pm_status pm_philox(uint64_t seed, int n, const uint32_t *counters, uint32_t *out)
{
    if (n < 0 || (n > 0 && (!counters || !out))) return PM_ERR_INVALID_ARGUMENT;
    if (n == 0) return PM_OK;
    uint32_t *d = nullptr;
    if (cudaMalloc((void **)&d, sizeof(uint32_t) * 8 * (size_t)n) != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_OUT_OF_MEMORY;
    }
    cudaError_t e = cudaMemcpy(d, counters, sizeof(uint32_t) * 4 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_philox(seed, n, d, d + 4 * (size_t)n, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(out, d + 4 * (size_t)n, sizeof(uint32_t) * 4 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) { cudaGetLastError(); return PM_ERR_CUDA; }
    return PM_OK;
}

pm_status pm_texture_peak(double *samples_per_s)
{
    if (!samples_per_s) return PM_ERR_INVALID_ARGUMENT;
    const cudaError_t e = measure_texture_peak(samples_per_s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_CUDA;
    }
    return PM_OK;
}

pm_status pm_check_reciprocal(int exp_shift, unsigned long long *mismatches)
{
    if (!mismatches || exp_shift < -120 || exp_shift > 120) return PM_ERR_INVALID_ARGUMENT;
    unsigned long long *d = nullptr;
    if (cudaMalloc((void **)&d, sizeof *d) != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_OUT_OF_MEMORY;
    }
    cudaError_t e = cudaMemset(d, 0, sizeof *d);
    if (e == cudaSuccess) e = launch_check_rcp(exp_shift, d, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(mismatches, d, sizeof *d, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) { cudaGetLastError(); return PM_ERR_CUDA; }
    return PM_OK;
}

}  // extern "C"
