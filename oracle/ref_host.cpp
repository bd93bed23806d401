/*
 * ref_host.cpp -- the reference's own kernels run on the CPU. TEST INFRASTRUCTURE ONLY: it
 * pins the oracle (pm_oracle.c) to the reference's code and writes golden vectors
 * (tests/golden/make_ref_golden.py). Nothing in the engine uses it.
 *
 * The kernels come unchanged from the reference's sources (ref_kernels.inc, assembled by
 * ref_extract.sh): sumI_II_RowsKernel / sumI_II_ColsKernel (array2d_refImg.cu:11-67),
 * generate_kernel_float (array2d_wrapper.cu:3-20), computeNCC, findMinCost,
 * readImageIntoSharedMemory, computeMessageBackward / computeMessageForward,
 * computeAllCostGivenDepth, topToDown and downToTop (patchMatch.cu:409-1209), and
 * GaussianBlurCUDA's convolutionRowsKernel / convolutionColsKernel / CreateFilterKernel
 * (GaussianBlurCUDA.cu:39-70, :99-130; ref_blur.inc). This file
 * plays the host side the reference's PatchMatch class plays (patchMatch.cu:51-407): the
 * packed source layers and the homography table as textures (:51-130, :152-205), the
 * reference-window sums (array2d_refImg.cu:70-131), the transposes before and after the
 * rotated sweeps (:236-261), the launch configuration (one block of 32 threads per 32 lines,
 * :39-49) and the sweep schedule (:307-394). A block's threads run as 32 host threads; blocks
 * run one after another (their shared arrays are the kernels' static locals).
 *
 * Built twice by the Makefile: with PMR_REAL = float the reference computes as written; with
 * PMR_REAL = double every `float` of the extracted code is widened to double (a mechanical
 * change of type only), which gives the reference's rules without float rounding -- the
 * build the FP64 oracle must agree with to rounding level.
 */
#include "ref_host_shim.h"

#ifndef PMR_WIDE
#define PMR_WIDE 0
#endif

#include <algorithm>
#include <atomic>
#include <barrier>
#include <chrono>
#include <thread>
#include <type_traits>
#include <vector>

thread_local pmr_dim3 threadIdx, blockIdx;
thread_local unsigned long long pmr_point_fetches = 0, pmr_point_outside = 0;
pmr_dim3 blockDim, gridDim;
uint64_t pmr_seed;
alignas(64) unsigned char pmr_dynamic_shared[1 << 18];

static std::barrier<> *g_barrier = nullptr;
void pmr_block_barrier()
{
    if (g_barrier) g_barrier->arrive_and_wait();
}

// The reference is built with --use_fast_math (cmakelists_32bit.txt:11): float results and
// operands below the smallest normal float are zero. The float build runs its kernel threads
// in the host's flush-to-zero mode to match (x86-64 MXCSR FTZ and DAZ, AArch64 FPCR FZ).
static void flush_denormals()
{
#if defined(__x86_64__)
    __builtin_ia32_ldmxcsr(__builtin_ia32_stmxcsr() | 0x8040u);
#elif defined(__aarch64__)
    __builtin_aarch64_set_fpcr(__builtin_aarch64_get_fpcr() | (1u << 24));
#endif
}

#if PMR_WIDE
// The widened build keeps the one float behaviour that changes decisions: an emission
// exp(-c^2 / (2 alpha^2)) below the smallest normal float is stored as 0 by the float reference
// (patchMatch.cu:683, :708), so a step whose every view underflows has a NaN posterior CDF in
// both. The extracted code's only exp calls are the messages' (:673, :683, :697, :708).
static inline double pmr_exp_flushed(double x)
{
    const double e = exp(x);
    return e < 1.17549435e-38 ? 0.0 : e;
}
#define exp pmr_exp_flushed
#define float double
#endif
#include "ref_kernels.inc"
// GaussianBlurCUDA's kernels in a namespace of their own: their texture is named tex32F0 too.
namespace ref_blur {
#include "ref_blur.inc"
}
#if PMR_WIDE
#undef float
#undef exp
#endif

namespace {

constexpr int BLOCK = 32;  // N of patchMatch.cu:37: the reference's block width

// Point fetches (homography-table reads) of the last launch, summed over its threads, and the
// launch's wall time.
std::atomic<unsigned long long> g_fetches{0}, g_outside{0};
double g_launch_seconds = 0.0;

// Runs blocks [b0, b1) of a grid of `blocks` blocks of BLOCK host threads, one block at a time.
template <class F>
void launch_lines(int blocks, F &&kernel, int b0 = 0, int b1 = -1)
{
    blockDim = {BLOCK, 1, 1};
    gridDim = {(unsigned)blocks, 1, 1};
    g_fetches = 0;
    g_outside = 0;
    std::barrier<> bar(BLOCK);
    g_barrier = &bar;
    const auto t0 = std::chrono::steady_clock::now();
    for (int b = b0; b < (b1 < 0 ? blocks : std::min(b1, blocks)); ++b) {
        std::vector<std::thread> th;
        th.reserve(BLOCK);
        for (int t = 0; t < BLOCK; ++t)
            th.emplace_back([&, b, t] {
                if (!PMR_WIDE) flush_denormals();
                threadIdx = {(unsigned)t, 0, 0};
                blockIdx = {(unsigned)b, 0, 0};
                pmr_point_fetches = pmr_point_outside = 0;
                kernel();
                g_fetches += pmr_point_fetches;
                g_outside += pmr_point_outside;
            });
        for (auto &x : th) x.join();
    }
    g_launch_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    g_barrier = nullptr;
}

// Runs f on a host thread of its own in the build's floating-point mode, so that the caller's
// thread (the Python interpreter's) keeps its own.
template <class F>
void on_kernel_thread(F &&f)
{
    std::thread th([&] {
        if (!PMR_WIDE) flush_denormals();
        f();
    });
    th.join();
}

// A 2-D launch of independent threads (no shared memory, no barrier): run in turn.
template <class F>
void launch_2d(int w, int h, int bx, int by, F &&kernel)
{
    blockDim = {(unsigned)bx, (unsigned)by, 1};
    gridDim = {(unsigned)((w + bx - 1) / bx), (unsigned)((h + by - 1) / by), 1};
    on_kernel_thread([&] {
        for (unsigned gy = 0; gy < gridDim.y; ++gy)
            for (unsigned gx = 0; gx < gridDim.x; ++gx)
                for (int ty = 0; ty < by; ++ty)
                    for (int tx = 0; tx < bx; ++tx) {
                        blockIdx = {gx, gy, 0};
                        threadIdx = {(unsigned)tx, (unsigned)ty, 0};
                        kernel();
                    }
    });
}

// A pitched 2-D array of `layers` stacked layers (the reference's Array2D_wrapper), with one
// guard layer in front of it. When the posterior CDF of a step is NaN (every view's emission
// underflowed: costs above ~6 at the leading-edge windows) no view sample finds a view, and the
// reference reads the cost table at layer -1 (patchMatch.cu:966, :1147): outside its allocation
// on the GPU, so the value is undefined. Here the read stays inside the buffer and yields -1;
// the averaged costs are then (inf, -inf, inf) and findMinCost keeps the current depth, the
// definition the oracle and the engine use for a step whose samples find no view.
template <class T>
struct Pitched {
    int width = 0, height = 0, layers = 1;
    std::vector<T> v;
    void init(int w, int h, int l = 1)
    {
        width = w;
        height = h;
        layers = l;
        v.assign((size_t)w * h * (l + 1), T(0));
        std::fill(v.begin(), v.begin() + (size_t)w * h, T(-1));
    }
    size_t front() const { return (size_t)width * height; }
    size_t size() const { return (size_t)width * height * layers; }
    T *ptr() { return v.data() + front(); }
    T *begin() { return ptr(); }
    T *end() { return ptr() + size(); }
    int pitch() const { return width * (int)sizeof(T); }
    T &at(int layer, int row, int col) { return v[front() + ((size_t)layer * height + row) * width + col]; }
    T &operator[](size_t i) { return v[front() + i]; }
};

// cudaTranspose::transpose2dData per layer (cudaTranspose.h:9-71): out(l, c, r) = in(l, r, c).
template <class T>
void transpose(Pitched<T> &in, Pitched<T> &out)
{
    out.init(in.height, in.width, in.layers);
    for (int l = 0; l < in.layers; ++l)
        for (int r = 0; r < in.height; ++r)
            for (int c = 0; c < in.width; ++c) out.at(l, c, r) = in.at(l, r, c);
}

}  // namespace

extern "C" {

/* One reference image and its sources as the reference's PatchMatch object holds them. */
typedef struct pmr_problem {
    int width, height, n_src, half_window;
    const uint8_t *ref;          /* height x width */
    const uint8_t *src;          /* n_src layers of src_height x src_width, zero-padded */
    int src_width, src_height;
    const double *hh;            /* n_src x 18: H1 then H2, row-major (Image::init_relative) */
    double orientation[3];       /* plane normal (orientationX, 0, orientationZ) */
    double inv_k[4];             /* K_ref^-1 (0,0), (0,2), (1,1), (1,2) */
    double depth_near, depth_far, sp_alpha;
    uint64_t seed;
    int fixed_point_weights;     /* source texture: 1/256 fixed-point linear weights */
} pmr_problem;

int pmr_real_bytes(void) { return (int)sizeof(pmr_real); }

}  // extern "C"

namespace {

using PR = pmr_real;

// The address mode the reference's host code gives each of its textures (patchMatch.cu:192-204,
// array2d_refImg.cu:109-113): 0 outside the array.
template <class Tex>
void set_border(Tex &t)
{
    for (auto &m : t.addressMode) m = cudaAddressModeBorder;
}

// The device-side state of one PatchMatch object (textures, constants, reference maps).
struct Device {
    const pmr_problem *p;
    std::vector<PR> hh;  // the homography table texture's texels
    Pitched<PR> ref_i, sum_i, sum_ii;      // the reference maps (Array2d_refImg)
    Pitched<PR> ref_i_t, sum_i_t, sum_ii_t;  // transposed copies (patchMatch.cu:176-179)

    explicit Device(const pmr_problem *pp) : p(pp)
    {
        pmr_seed = p->seed;
        // textures and constants (patchMatch.cu:152-205)
        allImgsTexture.data = p->src;
        allImgsTexture.width = p->src_width;
        allImgsTexture.height = p->src_height;
        allImgsTexture.layers = p->n_src;
        set_border(allImgsTexture);
        allImgsTexture.filterMode = cudaFilterModeLinear;
        allImgsTexture.fixed_point_weights = p->fixed_point_weights;
        refImgTexture.data = p->ref;
        refImgTexture.width = p->width;
        refImgTexture.height = p->height;
        refImgTexture.layers = 1;
        set_border(refImgTexture);
        refImgTexture.filterMode = cudaFilterModeLinear;
        refImgTexture.fixed_point_weights = 0;  // sampled at texel centres: exact either way
        hh.assign(p->hh, p->hh + 18 * (size_t)p->n_src);
        transformTexture.data = hh.data();
        transformTexture.width = 18;
        transformTexture.height = p->n_src;
        transformTexture.layers = 1;
        set_border(transformTexture);
        transformTexture.filterMode = cudaFilterModePoint;
        orientation[0] = (PR)p->orientation[0];
        orientation[1] = (PR)p->orientation[1];
        orientation[2] = (PR)p->orientation[2];
        for (int i = 0; i < 4; ++i) inverseK[i] = (PR)p->inv_k[i];
        box_moments();
        transpose(ref_i, ref_i_t);
        transpose(sum_i, sum_i_t);
        transpose(sum_ii, sum_ii_t);
    }

    // Array2d_refImg::filterImage<FR> (array2d_refImg.cu:100-131): the row pass from the
    // u8 reference, then the column pass over each row sum bound as a float texture.
    template <int FR>
    void box_moments_fr()
    {
        const int w = p->width, h = p->height;
        ref_i.init(w, h);
        sum_i.init(w, h);
        sum_ii.init(w, h);
        tex32F0.data = p->ref;
        tex32F0.width = w;
        tex32F0.height = h;
        tex32F0.layers = 1;
        set_border(tex32F0);  // array2d_refImg.cu:109-110
        tex32F0.filterMode = cudaFilterModeLinear;
        launch_2d(w, h, 16, 12, [&] {
            sumI_II_RowsKernel<FR>(ref_i.ptr(), sum_i.ptr(), sum_ii.ptr(), w, h, sum_i.pitch());
        });
        for (Pitched<PR> *m : {&sum_i, &sum_ii}) {
            std::vector<PR> copy(m->begin(), m->end());  // the temporary array the texture is bound to
            tex32F0_float.data = copy.data();
            tex32F0_float.width = w;
            tex32F0_float.height = h;
            tex32F0_float.layers = 1;
            set_border(tex32F0_float);  // array2d_refImg.cu:112-113
            tex32F0_float.filterMode = cudaFilterModeLinear;
            launch_2d(w, h, 16, 12, [&] { sumI_II_ColsKernel<FR>(m->ptr(), w, h, m->pitch()); });
        }
    }

    void box_moments();
};

#define PMR_FR_CASES(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11)

void Device::box_moments()
{
    switch (p->half_window) {
#define X(n) case n: box_moments_fr<n>(); break;
        PMR_FR_CASES(X)
#undef X
    default: break;
    }
}

// Reference-side layout conversions: costs are V stacked layers of height x width
// (Array2D_wrapper with depth V), the engine's and oracle's are pixel-major.
void costs_to_layers(const double *cost, int w, int h, int V, Pitched<PR> &out)
{
    out.init(w, h, V);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
            for (int v = 0; v < V; ++v) out.at(v, y, x) = (PR)cost[((size_t)y * w + x) * V + v];
}

void layers_to_costs(Pitched<PR> &in, double *cost)
{
    const int w = in.width, h = in.height, V = in.layers;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
            for (int v = 0; v < V; ++v) cost[((size_t)y * w + x) * V + v] = (double)in.at(v, y, x);
}

template <int WS>
void initial_costs_w(Device &dev, Pitched<PR> &depth_t, Pitched<PR> &cost_t)
{
    // computeAllCostGivenDepth on the transposed maps (patchMatch.cu:338-343)
    const pmr_problem *p = dev.p;
    const int tw = p->height, th = p->width;  // transposed width and height
    launch_lines((tw - 1) / BLOCK + 1, [&] {
        computeAllCostGivenDepth<WS>(cost_t.ptr(), cost_t.pitch(), dev.ref_i_t.ptr(), dev.sum_i_t.ptr(),
                                     dev.sum_ii_t.ptr(), dev.sum_i_t.pitch(), tw, th, depth_t.ptr(), depth_t.pitch(),
                                     (unsigned)p->n_src);
    });
}

// One sweep as run<W> launches it (patchMatch.cu:331-390): rotated sweeps on the transposed
// depth and cost maps.
template <int WS>
void sweep_w(Device &dev, int dir, int S, Pitched<PR> &depth, Pitched<PR> &cost, std::vector<curandState> &rs,
             uint8_t *view_sel, int line_begin, int line_end)
{
    const pmr_problem *p = dev.p;
    const bool rotated = dir == 0 || dir == 2;
    const bool down = dir == 0 || dir == 1;  // topToDown
    const PR a2 = (PR)((float)p->sp_alpha * (float)p->sp_alpha);
    const int state_pitch = p->width * (int)sizeof(curandState);
    Pitched<PR> d_t, c_t, spmap;
    Pitched<PR> &d = rotated ? d_t : depth;
    Pitched<PR> &c = rotated ? c_t : cost;
    if (rotated) {
        transpose(depth, d_t);
        transpose(cost, c_t);
    }
    Pitched<PR> &ri = rotated ? dev.ref_i_t : dev.ref_i;
    Pitched<PR> &si = rotated ? dev.sum_i_t : dev.sum_i;
    Pitched<PR> &sii = rotated ? dev.sum_ii_t : dev.sum_ii;
    const int w = d.width, h = d.height, V = p->n_src;
    spmap.init(w, h, V);
    Pitched<uint8_t> used;
    if (view_sel) {
        used.init(w, h, S);
        std::fill(used.begin(), used.end(), (uint8_t)255);
    }
    const int b0 = std::max(0, line_begin) / BLOCK;
    const int b1 = line_end < 0 ? -1 : (std::min(line_end, w) + BLOCK - 1) / BLOCK;
    launch_lines((w - 1) / BLOCK + 1, [&] {
        if (down)
            topToDown<WS>(c.ptr(), ri.ptr(), si.ptr(), sii.ptr(), si.pitch(), w, h, d.ptr(), d.pitch(), spmap.ptr(),
                          spmap.pitch(), S, rs.data(), state_pitch, (PR)p->depth_near, (PR)p->depth_far,
                          p->half_window, rotated, (unsigned)V, a2);
        else
            downToTop<WS>(c.ptr(), ri.ptr(), si.ptr(), sii.ptr(), si.pitch(), w, h, d.ptr(), d.pitch(), spmap.ptr(),
                          spmap.pitch(), S, rs.data(), state_pitch, (PR)p->depth_near, (PR)p->depth_far,
                          p->half_window, rotated, (unsigned)V, a2, view_sel ? used.ptr() : nullptr,
                          view_sel ? used.pitch() : 0);
    }, b0, b1);
    if (rotated) {
        transpose(d_t, depth);
        transpose(c_t, cost);
    }
    if (view_sel) memcpy(view_sel, used.ptr(), used.size());
}

#define PMR_W_CASES(X) X(3) X(5) X(7) X(9) X(11) X(13) X(15) X(17) X(19) X(21) X(23)

std::vector<curandState> make_states(const pmr_problem *p, const uint32_t *counts)
{
    const size_t n = (size_t)p->width * p->height;
    std::vector<curandState> rs(n);
    for (size_t i = 0; i < n; ++i) rs[i] = {(uint32_t)i, counts ? counts[i] : 0u};
    return rs;
}

void store_counts(const std::vector<curandState> &rs, uint32_t *counts)
{
    if (counts)
        for (size_t i = 0; i < rs.size(); ++i) counts[i] = rs[i].count;
}

bool supported(const pmr_problem *p)
{
    return p && p->half_window >= 1 && p->half_window <= 11 && p->n_src >= 1 && p->n_src <= 32 && p->width >= 1 &&
           p->height >= 1 && (size_t)BLOCK * p->n_src * sizeof(PR) + BLOCK * 8 <= sizeof(pmr_dynamic_shared);
}

Pitched<PR> depth_maps(const pmr_problem *p, const double *depth)
{
    Pitched<PR> d;
    d.init(p->width, p->height);
    for (size_t i = 0; i < d.size(); ++i) d[i] = (PR)depth[i];
    return d;
}

}  // namespace

extern "C" {

/* Reference-window maps: I, S_I, S_II (height x width), Array2d_refImg::filterImage. */
int pmr_box_moments(const pmr_problem *p, double *img, double *sum_i, double *sum_ii)
{
    if (!supported(p)) return -1;
    Device dev(p);
    for (size_t i = 0; i < dev.sum_i.size(); ++i) {
        if (img) img[i] = (double)dev.ref_i[i];
        sum_i[i] = (double)dev.sum_i[i];
        sum_ii[i] = (double)dev.sum_ii[i];
    }
    return 0;
}

/* Initial depth (Array2D_wrapper::randNumGen, array2d_wrapper.cu:3-20) from the per-pixel
 * random states whose draw counts are counts[] (updated). */
int pmr_init_depth(const pmr_problem *p, uint32_t *counts, double *depth)
{
    if (!supported(p)) return -1;
    pmr_seed = p->seed;
    std::vector<curandState> rs = make_states(p, counts);
    Pitched<PR> d;
    d.init(p->width, p->height);
    const int state_pitch = p->width * (int)sizeof(curandState);
    launch_2d(p->width, p->height, 32, 16, [&] {
        generate_kernel_float(rs.data(), state_pitch, d.ptr(), d.pitch(), p->width, p->height, (PR)p->depth_near,
                              (PR)p->depth_far);
    });
    for (size_t i = 0; i < d.size(); ++i) depth[i] = (double)d[i];
    store_counts(rs, counts);
    return 0;
}

/* computeAllCostGivenDepth: every view's cost at depth (height x width), written pixel-major
 * (height x width x n_src). */
int pmr_initial_costs(const pmr_problem *p, const double *depth, double *cost)
{
    if (!supported(p)) return -1;
    Device dev(p);
    Pitched<PR> d = depth_maps(p, depth), d_t, c_t;
    transpose(d, d_t);
    c_t.init(p->height, p->width, p->n_src);
    switch (2 * p->half_window + 1) {
#define X(n) case n: initial_costs_w<n>(dev, d_t, c_t); break;
        PMR_W_CASES(X)
#undef X
    default: return -1;
    }
    Pitched<PR> c;
    transpose(c_t, c);
    layers_to_costs(c, cost);
    return 0;
}

/* One sweep in direction dir (0 left-to-right, 1 top-to-bottom, 2 right-to-left, 3
 * bottom-to-top) with S view samples, in place on depth and pixel-major costs; counts[] are
 * the per-pixel random states' draw counts (updated). view_sel (S x height x width, written
 * only by bottom-to-top sweeps, as the reference records usedImgsID) may be NULL. Only the
 * blocks of 32 lines that hold lines [line_begin, line_end) run (line_end < 0: all). Returns
 * the number of homography-table fetches outside the table (view samples that found no view);
 * *evals (if not NULL) receives the number of computeNCC calls and *seconds the wall time of
 * the kernel launch alone (not the host's layout conversions around it). */
long long pmr_sweep(const pmr_problem *p, int dir, int S, double *depth, double *cost, uint32_t *counts,
                    uint8_t *view_sel, int line_begin, int line_end, long long *evals, double *seconds)
{
    if (!supported(p) || dir < 0 || dir > 3 || S < 1) return -1;
    Device dev(p);
    std::vector<curandState> rs = make_states(p, counts);
    Pitched<PR> d = depth_maps(p, depth), c;
    costs_to_layers(cost, p->width, p->height, p->n_src, c);
    uint8_t *vs = dir == 3 ? view_sel : nullptr;
    switch (2 * p->half_window + 1) {
#define X(n) case n: sweep_w<n>(dev, dir, S, d, c, rs, vs, line_begin, line_end); break;
        PMR_W_CASES(X)
#undef X
    default: return -1;
    }
    for (size_t i = 0; i < d.size(); ++i) depth[i] = (double)d[i];
    layers_to_costs(c, cost);
    store_counts(rs, counts);
    if (evals) *evals = (long long)(g_fetches.load() / 18);
    if (seconds) *seconds = g_launch_seconds;
    return (long long)g_outside.load();
}

/* PatchMatch::run<W> (patchMatch.cu:307-394) from the random initial depth: iteration 0
 * samples one view and first computes every cost; each iteration sweeps left-to-right,
 * top-to-bottom, right-to-left, bottom-to-top; the last sweep records the sampled views.
 * Returns the homography-table fetches outside the table, or -1. */
long long pmr_run(const pmr_problem *p, int iterations, int S, double *depth, double *cost, uint8_t *view_sel)
{
    if (!supported(p) || iterations < 1 || S < 1) return -1;
    std::vector<uint32_t> counts((size_t)p->width * p->height, 0u);
    if (pmr_init_depth(p, counts.data(), depth) != 0) return -1;
    if (pmr_initial_costs(p, depth, cost) != 0) return -1;
    long long outside = 0;
    for (int it = 0; it < iterations; ++it)
        for (int dir = 0; dir < 4; ++dir) {
            const long long o = pmr_sweep(p, dir, it == 0 ? 1 : S, depth, cost, counts.data(),
                                          it == iterations - 1 ? view_sel : nullptr, 0, -1, nullptr, nullptr);
            if (o < 0) return -1;
            outside += o;
        }
    return outside;
}

/* computeNCC for arbitrary queries (x, y, view, depth, axis): the reference tile of the
 * query's line is loaded by the reference's loader for all 32 threads of its block, then the
 * query's thread evaluates, as computeAllCostGivenDepth (axis 1: rotated) and topToDown
 * (axis 0) call it. scale = nx (ik00 (x + 1/2) + ik02) + nz, the kernels' plane scale. */
int pmr_ncc(const pmr_problem *p, int n, const int *xs, const int *ys, const int *views, const double *depths,
            const int *axes, double *out)
{
    if (!supported(p)) return -1;
    Device dev(p);
    static PR tile[BLOCK * 3 * 23];
    int status = 0;
    on_kernel_thread([&] {
    for (int i = 0; i < n; ++i) {
        const bool rot = axes[i] != 0;
        const int row = rot ? xs[i] : ys[i], col = rot ? ys[i] : xs[i];
        const int w = rot ? p->height : p->width, h = rot ? p->width : p->height;
        const int hw = p->half_window;
        const int t = col % BLOCK, col0 = col - t;
        PR s_i[BLOCK], s_ii[BLOCK];
        s_i[t] = (PR)dev.sum_i.at(0, ys[i], xs[i]);
        s_ii[t] = (PR)dev.sum_ii.at(0, ys[i], xs[i]);
        // the kernels' plane scale at image column x (patchMatch.cu:798-800, :876-883)
        const PR scale = orientation[0] * (inverseK[0] * (xs[i] + 0.5) + inverseK[1]) +
                         orientation[1] * (inverseK[2] * (ys[i] + 0.5) + inverseK[3]) + orientation[2];
        const PR rmh = (PR)row - (PR)hw + (PR)0.5, cmh = (PR)col - (PR)hw + (PR)0.5;
        PR r = 0;
        switch (2 * hw + 1) {
#define X(WS)                                                                                                   \
    case WS:                                                                                                    \
        for (int k = 0; k < BLOCK; ++k) readImageIntoSharedMemory_block<WS>(tile, row, col0 + k, k, rot);     \
        r = computeNCC<WS>(t, tile, s_i, s_ii, views[i], rmh, cmh, (PR)depths[i], rot, hw, w, h, scale);       \
        break;
            PMR_W_CASES(X)
#undef X
        default: status = -1; return;
        }
        out[i] = (double)r;
    }
    });
    return status;
}

/* computeMessageForward / computeMessageBackward (patchMatch.cu:669-715) for one pixel and V
 * views: msg[v] is updated in place from cost[v]; a cost of exactly 2 is replaced by
 * 2 U(0, 1] drawn from the state (id, *count). */
int pmr_messages(int forward, int V, double *msg, const double *cost, double sp_alpha, uint64_t seed,
                 uint32_t id, uint32_t *count)
{
    if (V < 1 || V > 32) return -1;
    pmr_seed = seed;
    static PR spmap[BLOCK * 32];
    PR mc[32];
    for (int v = 0; v < V; ++v) {
        spmap[v * BLOCK] = (PR)msg[v];
        mc[v] = (PR)cost[v];
    }
    curandState st[1] = {{id, *count}};
    const PR a2 = (PR)((float)sp_alpha * (float)sp_alpha);
    const int row = 0, col = 0, tid = 0, pitch = (int)sizeof(PR);  // layer v is row v
    on_kernel_thread([&] {
        if (forward)
            computeMessageForward(spmap, row, col, tid, mc, pitch, a2, 1, V, st);
        else
            computeMessageBackward(spmap, row, col, tid, mc, pitch, a2, 1, V, st);
    });
    for (int v = 0; v < V; ++v) msg[v] = (double)spmap[v * BLOCK];
    *count = st[0].count;
    return 0;
}

/* findMinCost (patchMatch.cu:613-618). */
int pmr_find_min_cost(const double cost[3])
{
    PR c[3] = {(PR)cost[0], (PR)cost[1], (PR)cost[2]};
    return findMinCost(c);
}

// GaussianBlurCUDA::Filter(float *dst, const float *src) (GaussianBlurCUDA.cu:185-191) of an
// object made for (width, height, sigma) (:73-89): CreateFilterKernel (:99-130) fills g_Kernel,
// Filter switches on the radius (:152-183) and FilterImage<FR> (:132-149) runs the row pass
// over the source bound to tex32F0, then the column pass over the row pass's output, in blocks
// of 16 x 12 threads (:13-14, :134-135). The texture keeps the defaults of its declaration
// (:22; the class sets no mode): point filtering, clamp addressing. Writes the taps' count to
// *taps (the filter width); returns -1 where Filter runs no pass (a radius outside 2..22).
int pmr_blur(int width, int height, double sigma, const double *src, double *dst, int *taps)
{
    namespace B = ref_blur;
    auto &tex = B::tex32F0;
    PR filter_kernel[KERNEL_MAX_WIDTH];  // float as written, double in the widened build
    int kw = 0;
    B::GaussianBlurCUDA_CreateFilterKernel((PR)sigma, filter_kernel, kw);
    *taps = kw;
    for (int i = 0; i < kw; ++i) B::g_Kernel[i] = filter_kernel[i];
    const size_t n = (size_t)width * height;
    std::vector<PR> in(src, src + n), tmp(n), out(n);
    tex.width = width;
    tex.height = height;
    tex.layers = 1;
    auto filter = [&](auto fr) {
        constexpr int FR = decltype(fr)::value;
        tex.data = in.data();
        launch_2d(width, height, THREADS_NUMBER_H, THREADS_NUMBER_V,
                  [&] { B::convolutionRowsKernel<FR>(tmp.data(), width, height); });
        tex.data = tmp.data();
        launch_2d(width, height, THREADS_NUMBER_H, THREADS_NUMBER_V,
                  [&] { B::convolutionColsKernel<FR>(out.data(), width, height); });
    };
    switch (kw >> 1) {
#define X(n) case n: filter(std::integral_constant<int, n>{}); break;
        X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12)
        X(13) X(14) X(15) X(16) X(17) X(18) X(19) X(20) X(21) X(22)
#undef X
    default: return -1;
    }
    for (size_t i = 0; i < n; ++i) dst[i] = (double)out[i];
    return 0;
}

}  // extern "C"
