// pm_fuse.cu -- consistency filtering of several references' depth maps and their fusion into
// one point cloud. The reference has no counterpart: its output stops at one depth map per run
// (patchMatch.cu:263-407, main.cpp:124-128); this is the step after the path, run over the
// depth maps a batch leaves on the device.
//
// For pixel (x, y) of reference i with depth d and every other reference j: the pixel centre
// (x + 1/2, y + 1/2) at depth d is projected into j; j's depth d_j at the pixel containing the
// projection is taken; that pixel's centre at depth d_j is projected back into i. j agrees when
// the round trip lands within max_reproj_px of the start and its depth in i within
// max_rel_depth * d. A pixel with at least min_consistent agreeing references is kept; its fused
// depth is (d + the agreeing round-trip depths) / (1 + their count), and its point the
// back-projection of the fused depth. The point cloud lists the kept pixels reference by
// reference in row-major order.
//
// The per-pixel arithmetic is FP32 with explicit round-to-nearest operations (no contraction)
// in a fixed order and a correctly rounded reciprocal, so a CPU restatement in the same order
// gives the same bits from the same FP32 matrices (pm_fusion_geometry). The round trip's
// reprojection test is division-free: |q - qz (u, v)|^2 < max_reproj_px^2 qz^2.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "patchmatch_gb300.h"
#include "pm_internal.h"

namespace pm {
namespace {

constexpr int FUSE_THREADS = 256;
// Projection depths outside this range are rejected, so that rcp_nr (correct rounding for a
// normal argument with a normal reciprocal) equals 1 / z exactly.
constexpr float RCP_MIN = 1e-30f, RCP_MAX = 1e30f;
// Blocks per scan tile (one CTA of 1024 threads scans a tile).
constexpr int SCAN_TILE_LOG2 = 10;

struct FuseRefDev {
    const float *depth;       // width * height, row-major
    const float *tex_f;       // intensity in [0, 1], or null
    const uint8_t *tex_u8;    // intensity 0..255, or null
    float *fused;             // fused depth of kept pixels, 0 elsewhere
    uint8_t *count;           // agreeing references per pixel
    int width, height, blocks;
    float bp[12];             // R^T K^-1 (row-major 3x3), then the centre -R^T t
};

__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }

// m (3x3 row-major, then a translation) applied to depth * (u, v, 1): component k is
// depth * (m[3k] u + m[3k+1] v + m[3k+2]) + m[9+k].
__device__ __forceinline__ float apply_row(const float *m, int k, float u, float v, float depth)
{
    const float r = add(add(mul(m[3 * k], u), mul(m[3 * k + 1], v)), m[3 * k + 2]);
    return add(mul(depth, r), m[9 + k]);
}

__global__ void __launch_bounds__(FUSE_THREADS)
fuse_check_kernel(const FuseRefDev *__restrict__ refs, const float *__restrict__ pairs, int n,
                  float max_err2, float max_rel, int min_consistent, uint32_t *__restrict__ block_kept,
                  uint32_t *__restrict__ tile_kept)
{
    __shared__ float s_fwd[PM_MAX_FUSE_REFS * 12];   // i -> j
    __shared__ float s_bwd[PM_MAX_FUSE_REFS * 12];   // j -> i
    __shared__ const float *s_depth[PM_MAX_FUSE_REFS];
    __shared__ int2 s_size[PM_MAX_FUSE_REFS];
    const int i = blockIdx.y;
    const FuseRefDev &R = refs[i];
    const int W = R.width, npix = R.width * R.height;
    if ((int)blockIdx.x >= R.blocks) {
        if (threadIdx.x == 0) block_kept[(size_t)i * gridDim.x + blockIdx.x] = 0;
        return;
    }
    for (int t = threadIdx.x; t < n * 12; t += blockDim.x) {
        const int j = t / 12, k = t % 12;
        s_fwd[t] = pairs[((size_t)i * n + j) * 12 + k];
        s_bwd[t] = pairs[((size_t)j * n + i) * 12 + k];
    }
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        s_depth[j] = refs[j].depth;
        s_size[j] = make_int2(refs[j].width, refs[j].height);
    }
    __syncthreads();

    const int pix = blockIdx.x * FUSE_THREADS + threadIdx.x;
    bool keep = false;
    if (pix < npix) {
        const int x = pix % W, y = pix / W;
        const float d = R.depth[pix];
        int count = 0;
        float acc = d;
        const bool valid = d > 0.0f && d < INFINITY;
        if (valid) {
            const float u = add((float)x, 0.5f), v = add((float)y, 0.5f);
            const float tol = mul(max_rel, d);
            for (int j = 0; j < n; ++j) {
                if (j == i) continue;
                const float *A = s_fwd + 12 * j;
                const float pz = apply_row(A, 2, u, v, d);
                if (!(pz > RCP_MIN && pz < RCP_MAX)) continue;
                const float rz = rcp_nr(pz);   // correctly rounded in this range
                const float uj = mul(apply_row(A, 0, u, v, d), rz);
                const float vj = mul(apply_row(A, 1, u, v, d), rz);
                const int2 sz = s_size[j];
                if (!(uj >= 0.0f && uj < (float)sz.x && vj >= 0.0f && vj < (float)sz.y)) continue;
                const int ix = min((int)uj, sz.x - 1), iy = min((int)vj, sz.y - 1);
                const float dj = __ldg(s_depth[j] + (size_t)iy * sz.x + ix);
                if (!(dj > 0.0f && dj < INFINITY)) continue;
                const float *B = s_bwd + 12 * j;
                const float uc = add((float)ix, 0.5f), vc = add((float)iy, 0.5f);
                const float qz = apply_row(B, 2, uc, vc, dj);
                if (!(qz > 0.0f)) continue;
                // |q / qz - (u, v)|^2 < max_err2 without dividing: |q - qz (u, v)|^2 < max_err2 qz^2
                const float ex = add(apply_row(B, 0, uc, vc, dj), -mul(u, qz));
                const float ey = add(apply_row(B, 1, uc, vc, dj), -mul(v, qz));
                const float err2 = add(mul(ex, ex), mul(ey, ey));
                if (err2 < mul(max_err2, mul(qz, qz)) && fabsf(add(qz, -d)) < tol) {
                    ++count;
                    acc = add(acc, qz);
                }
            }
        }
        float fused = 0.0f;
        if (valid && count >= min_consistent) {
            fused = __fdiv_rn(acc, (float)(count + 1));
            keep = fused > 0.0f && fused < INFINITY;
            if (!keep) fused = 0.0f;
        }
        R.fused[pix] = fused;
        R.count[pix] = (uint8_t)min(count, 255);
    }
    const int kept = __syncthreads_count(keep);
    if (threadIdx.x == 0) {
        const size_t blk = (size_t)i * gridDim.x + blockIdx.x;
        block_kept[blk] = (uint32_t)kept;
        if (kept) atomicAdd(tile_kept + (blk >> SCAN_TILE_LOG2), (uint32_t)kept);   // integer: order-free
    }
}

// Exclusive scan of one value per thread over a CTA of 1024 threads; *total gets the sum.
__device__ __forceinline__ unsigned long long cta_exclusive_scan(unsigned long long val, unsigned long long *s_warp,
                                                                 unsigned long long *total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long inc = val;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        unsigned long long w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        s_warp[lane] = w;   // inclusive over warps
    }
    __syncthreads();
    const unsigned long long out = (wid ? s_warp[wid - 1] : 0ull) + inc - val;
    *total = s_warp[31];
    __syncthreads();        // s_warp may be reused by the caller
    return out;
}

// Exclusive scan of the tiles' kept counts (at most a few thousand tiles) into tile_base, and
// the total; one CTA.
__global__ void __launch_bounds__(1024)
fuse_scan_tiles_kernel(const uint32_t *__restrict__ tile_kept, int ntiles, unsigned long long *__restrict__ tile_base,
                       unsigned long long *__restrict__ total)
{
    __shared__ unsigned long long s_warp[32];
    unsigned long long carry = 0;
    for (int base = 0; base < ntiles; base += 1024) {
        const int k = base + threadIdx.x;
        unsigned long long chunk;
        const unsigned long long ex = cta_exclusive_scan(k < ntiles ? tile_kept[k] : 0ull, s_warp, &chunk);
        if (k < ntiles) tile_base[k] = carry + ex;
        carry += chunk;
    }
    if (threadIdx.x == 0) *total = carry;
}

// Offsets of the blocks of one tile (1024 blocks per CTA): the tile's base plus the exclusive
// scan of its blocks' counts.
__global__ void __launch_bounds__(1024)
fuse_scan_blocks_kernel(const uint32_t *__restrict__ block_kept, int nblocks,
                        const unsigned long long *__restrict__ tile_base, unsigned long long *__restrict__ offsets)
{
    __shared__ unsigned long long s_warp[32];
    const int k = (blockIdx.x << SCAN_TILE_LOG2) + threadIdx.x;
    unsigned long long chunk;
    const unsigned long long ex = cta_exclusive_scan(k < nblocks ? block_kept[k] : 0ull, s_warp, &chunk);
    if (k < nblocks) offsets[k] = tile_base[blockIdx.x] + ex;
}

// Writes the kept pixels' points (x, y, z, intensity) at their block's offset, in pixel order.
__global__ void __launch_bounds__(FUSE_THREADS)
fuse_points_kernel(const FuseRefDev *__restrict__ refs, const unsigned long long *__restrict__ offsets,
                   float4 *__restrict__ points)
{
    __shared__ int s_warp[FUSE_THREADS / 32];
    const int i = blockIdx.y;
    const FuseRefDev &R = refs[i];
    const int npix = R.width * R.height;
    if ((int)blockIdx.x >= R.blocks) return;
    const int pix = blockIdx.x * FUSE_THREADS + threadIdx.x;
    const float depth = pix < npix ? R.fused[pix] : 0.0f;
    const bool keep = depth > 0.0f;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned ball = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) s_warp[wid] = __popc(ball);
    __syncthreads();
    int before = 0;
    for (int w = 0; w < wid; ++w) before += s_warp[w];
    if (!keep) return;
    const unsigned long long idx =
        offsets[(size_t)i * gridDim.x + blockIdx.x] + before + __popc(ball & ((1u << lane) - 1u));
    const int x = pix % R.width, y = pix / R.width;
    const float u = add((float)x, 0.5f), v = add((float)y, 0.5f);
    float inten = 0.0f;
    if (R.tex_f) inten = R.tex_f[pix];
    else if (R.tex_u8) inten = __fdiv_rn((float)R.tex_u8[pix], 255.0f);
    points[idx] = make_float4(apply_row(R.bp, 0, u, v, depth), apply_row(R.bp, 1, u, v, depth),
                              apply_row(R.bp, 2, u, v, depth), inten);
}

bool inv3(const double *m, double *o)
{
    const double c0 = m[4] * m[8] - m[5] * m[7], c1 = m[5] * m[6] - m[3] * m[8], c2 = m[3] * m[7] - m[4] * m[6];
    const double det = m[0] * c0 + m[1] * c1 + m[2] * c2;
    if (!(std::fabs(det) > 1e-300) || !std::isfinite(det)) return false;
    const double r = 1.0 / det;
    o[0] = c0 * r; o[1] = (m[2] * m[7] - m[1] * m[8]) * r; o[2] = (m[1] * m[5] - m[2] * m[4]) * r;
    o[3] = c1 * r; o[4] = (m[0] * m[8] - m[2] * m[6]) * r; o[5] = (m[2] * m[3] - m[0] * m[5]) * r;
    o[6] = c2 * r; o[7] = (m[1] * m[6] - m[0] * m[7]) * r; o[8] = (m[0] * m[4] - m[1] * m[3]) * r;
    return true;
}

void mat3(const double *a, const double *b, double *o)
{
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) o[3 * r + c] = a[3 * r] * b[c] + a[3 * r + 1] * b[3 + c] + a[3 * r + 2] * b[6 + c];
}

void vec3(const double *a, const double *v, double *o)
{
    for (int r = 0; r < 3; ++r) o[r] = a[3 * r] * v[0] + a[3 * r + 1] * v[1] + a[3 * r + 2] * v[2];
}

void transpose3(const double *a, double *o)
{
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) o[3 * r + c] = a[3 * c + r];
}

}  // namespace
}  // namespace pm

struct pm_fusion {
    int device = 0;
    int n = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    std::vector<pm::FuseSource> src;
    std::vector<float> pairs, bp;
    std::vector<pm::FuseRefDev> h_refs;
    pm::FuseRefDev *d_refs = nullptr;
    float *d_pairs = nullptr;
    uint32_t *d_block_kept = nullptr, *d_tile_kept = nullptr;
    unsigned long long *d_offsets = nullptr, *d_tile_base = nullptr, *d_total = nullptr, *h_total = nullptr;
    int ntiles = 0;
    float4 *d_points = nullptr;
    std::vector<void *> owned;      // device buffers this object allocated
    int max_blocks = 0;
    long long total_pix = 0;
    long long n_points = -1;
    float ms_check = 0.0f, ms_total = 0.0f;
    std::string err;
};

namespace {

pm_status fuse_fail(pm_fusion *f, pm_status s, const std::string &msg)
{
    if (f) f->err = msg;
    return s;
}

pm_status fuse_cuda(pm_fusion *f, cudaError_t e, const char *what)
{
    cudaGetLastError();
    if (f) f->err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? PM_ERR_OUT_OF_MEMORY : PM_ERR_CUDA;
}

#define FUSE_CUDA(f, expr, what)                            \
    do {                                                    \
        cudaError_t e_ = (expr);                            \
        if (e_ != cudaSuccess) return fuse_cuda(f, e_, what); \
    } while (0)

template <typename T>
cudaError_t fuse_alloc(pm_fusion *f, T **p, size_t bytes)
{
    void *q = nullptr;
    const cudaError_t e = cudaMalloc(&q, bytes ? bytes : 16);
    if (e == cudaSuccess) {
        f->owned.push_back(q);
        *p = (T *)q;
    }
    return e;
}

void fuse_free(pm_fusion *f)
{
    if (!f) return;
    if (f->stream) cudaStreamSynchronize(f->stream);
    for (void *q : f->owned) cudaFree(q);
    f->owned.clear();
    if (f->h_total) cudaFreeHost(f->h_total);
    for (cudaEvent_t &e : f->ev)
        if (e) cudaEventDestroy(e);
    if (f->stream) cudaStreamDestroy(f->stream);
}

// Pair matrices and back-projections in FP64 from the FP32 cameras, rounded to FP32.
pm_status fuse_geometry(pm_fusion *f)
{
    const int n = f->n;
    f->pairs.assign((size_t)n * n * 12, 0.0f);
    f->bp.assign((size_t)n * 12, 0.0f);
    std::vector<double> K(9 * n), Ki(9 * n), R(9 * n), Rt(9 * n), T(3 * n);
    for (int i = 0; i < n; ++i) {
        const pm::FuseSource &s = f->src[(size_t)i];
        for (int k = 0; k < 9; ++k) {
            K[9 * i + k] = s.K[k];
            R[9 * i + k] = s.R[k];
        }
        for (int k = 0; k < 3; ++k) T[3 * i + k] = s.t[k];
        if (!pm::inv3(&K[9 * i], &Ki[9 * i])) return fuse_fail(f, PM_ERR_CAMERA, "singular K");
        pm::transpose3(&R[9 * i], &Rt[9 * i]);
        double W[9], C[3];
        pm::mat3(&Rt[9 * i], &Ki[9 * i], W);
        pm::vec3(&Rt[9 * i], &T[3 * i], C);
        for (int k = 0; k < 9; ++k) f->bp[(size_t)i * 12 + k] = (float)W[k];
        for (int k = 0; k < 3; ++k) f->bp[(size_t)i * 12 + 9 + k] = (float)(-C[k]);
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            // A = K_j R_j R_i^T K_i^-1, b = K_j (t_j - R_j R_i^T t_i)
            double RjRit[9], KR[9], A[9], RRt[3], bb[3], b[3];
            pm::mat3(&R[9 * j], &Rt[9 * i], RjRit);
            pm::mat3(&K[9 * j], RjRit, KR);
            pm::mat3(KR, &Ki[9 * i], A);
            pm::vec3(RjRit, &T[3 * i], RRt);
            for (int k = 0; k < 3; ++k) bb[k] = T[3 * j + k] - RRt[k];
            pm::vec3(&K[9 * j], bb, b);
            float *o = &f->pairs[((size_t)i * n + j) * 12];
            for (int k = 0; k < 9; ++k) o[k] = (float)A[k];
            for (int k = 0; k < 3; ++k) o[9 + k] = (float)b[k];
            for (int k = 0; k < 12; ++k)
                if (!std::isfinite(o[k])) return fuse_fail(f, PM_ERR_CAMERA, "non-finite pair geometry");
        }
    return PM_OK;
}

}  // namespace

namespace pm {

pm_status fusion_create(const FuseSource *sources, int n, int device, pm_fusion **out)
{
    if (!out) return PM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!sources || n < 1 || n > PM_MAX_FUSE_REFS) return PM_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < n; ++i) {
        const FuseSource &s = sources[i];
        if (s.width < 1 || s.height < 1 || s.width > 32768 || s.height > 32768 || (!s.d_depth && !s.h_depth))
            return PM_ERR_IMAGE;
        for (int k = 0; k < 9; ++k)
            if (!std::isfinite(s.K[k]) || !std::isfinite(s.R[k])) return PM_ERR_CAMERA;
        for (int k = 0; k < 3; ++k)
            if (!std::isfinite(s.t[k])) return PM_ERR_CAMERA;
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return PM_ERR_NO_DEVICE;
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return PM_ERR_NO_DEVICE;
    if (device >= count) return PM_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return PM_ERR_NO_DEVICE;

    pm_fusion *f = new pm_fusion();
    f->device = device;
    f->n = n;
    f->src.assign(sources, sources + n);
    pm_status st = fuse_geometry(f);
    auto bail = [&](pm_status s) {
        fuse_free(f);
        delete f;
        return s;
    };
    if (st != PM_OK) return bail(st);
#define FUSE_TRY(expr)                                  \
    do {                                                \
        cudaError_t e_ = (expr);                        \
        if (e_ != cudaSuccess) return bail(fuse_cuda(f, e_, #expr)); \
    } while (0)
    FUSE_TRY(cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking));
    for (cudaEvent_t &e : f->ev) FUSE_TRY(cudaEventCreate(&e));
    FUSE_TRY(cudaMallocHost(&f->h_total, sizeof(unsigned long long)));
    f->h_refs.resize((size_t)n);
    for (int i = 0; i < n; ++i) {
        const FuseSource &s = sources[i];
        FuseRefDev &r = f->h_refs[(size_t)i];
        const size_t npix = (size_t)s.width * s.height;
        r.width = s.width;
        r.height = s.height;
        r.blocks = (int)((npix + FUSE_THREADS - 1) / FUSE_THREADS);
        f->max_blocks = std::max(f->max_blocks, r.blocks);
        f->total_pix += (long long)npix;
        for (int k = 0; k < 12; ++k) r.bp[k] = f->bp[(size_t)i * 12 + k];
        if (s.d_depth) {
            r.depth = s.d_depth;
        } else {
            float *d = nullptr;
            FUSE_TRY(fuse_alloc(f, &d, npix * 4));
            FUSE_TRY(cudaMemcpyAsync(d, s.h_depth, npix * 4, cudaMemcpyHostToDevice, f->stream));
            r.depth = d;
        }
        r.tex_f = s.d_intensity;
        r.tex_u8 = nullptr;
        if (!s.d_intensity && s.h_gray) {
            uint8_t *g = nullptr;
            FUSE_TRY(fuse_alloc(f, &g, npix));
            FUSE_TRY(cudaMemcpyAsync(g, s.h_gray, npix, cudaMemcpyHostToDevice, f->stream));
            r.tex_u8 = g;
        }
        FUSE_TRY(fuse_alloc(f, &r.fused, npix * 4));
        FUSE_TRY(fuse_alloc(f, &r.count, npix));
    }
    const size_t nblk = (size_t)f->max_blocks * n;
    if (nblk > (size_t)INT_MAX) return bail(fuse_fail(f, PM_ERR_IMAGE, "too many pixels for one fusion"));
    FUSE_TRY(fuse_alloc(f, &f->d_refs, sizeof(FuseRefDev) * n));
    FUSE_TRY(fuse_alloc(f, &f->d_pairs, f->pairs.size() * 4));
    FUSE_TRY(fuse_alloc(f, &f->d_block_kept, nblk * 4));
    FUSE_TRY(fuse_alloc(f, &f->d_offsets, nblk * 8));
    f->ntiles = (int)((nblk + (1u << pm::SCAN_TILE_LOG2) - 1) >> pm::SCAN_TILE_LOG2);
    FUSE_TRY(fuse_alloc(f, &f->d_tile_kept, (size_t)f->ntiles * 4));
    FUSE_TRY(fuse_alloc(f, &f->d_tile_base, (size_t)f->ntiles * 8));
    FUSE_TRY(fuse_alloc(f, &f->d_total, 8));
    FUSE_TRY(fuse_alloc(f, &f->d_points, (size_t)f->total_pix * sizeof(float4)));
    FUSE_TRY(cudaMemcpyAsync(f->d_refs, f->h_refs.data(), sizeof(FuseRefDev) * n, cudaMemcpyHostToDevice, f->stream));
    FUSE_TRY(cudaMemcpyAsync(f->d_pairs, f->pairs.data(), f->pairs.size() * 4, cudaMemcpyHostToDevice, f->stream));
    FUSE_TRY(cudaStreamSynchronize(f->stream));
#undef FUSE_TRY
    *out = f;
    return PM_OK;
}

}  // namespace pm

extern "C" {

void pm_default_fuse_params(pm_fuse_params *p)
{
    if (!p) return;
    p->max_reproj_px = 1.0f;
    p->max_rel_depth = 0.01f;
    p->min_consistent = 2;
}

pm_status pm_fusion_create(const pm_depth_view *views, int n, int gpu_id, pm_fusion **out)
{
    if (!out) return PM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!views || n < 1 || n > PM_MAX_FUSE_REFS) return PM_ERR_INVALID_ARGUMENT;
    std::vector<pm::FuseSource> src((size_t)n);
    for (int i = 0; i < n; ++i) {
        const pm_depth_view &v = views[i];
        pm::FuseSource &s = src[(size_t)i];
        s = pm::FuseSource{};
        s.h_depth = v.depth;
        s.h_gray = v.gray;
        s.width = v.width;
        s.height = v.height;
        for (int k = 0; k < 9; ++k) {
            s.K[k] = v.K[k];
            s.R[k] = v.R[k];
        }
        for (int k = 0; k < 3; ++k) s.t[k] = v.t[k];
    }
    return pm::fusion_create(src.data(), n, gpu_id, out);
}

pm_status pm_fusion_run(pm_fusion *f, const pm_fuse_params *p)
{
    if (!f || !p) return PM_ERR_INVALID_ARGUMENT;
    if (!(p->max_reproj_px >= 0.0f) || !(p->max_rel_depth >= 0.0f) || p->min_consistent < 0 ||
        !std::isfinite(p->max_reproj_px) || !std::isfinite(p->max_rel_depth))
        return fuse_fail(f, PM_ERR_INVALID_ARGUMENT, "fusion thresholds must be finite and >= 0");
    FUSE_CUDA(f, cudaSetDevice(f->device), "cudaSetDevice");
    for (const pm::FuseSource &s : f->src)   // engines' depth maps are read where they are
        if (s.wait_stream) FUSE_CUDA(f, cudaStreamSynchronize(s.wait_stream), "engine stream");
    const dim3 grid((unsigned)f->max_blocks, (unsigned)f->n);
    const int nblk = f->max_blocks * f->n;
    const float err2 = p->max_reproj_px * p->max_reproj_px;
    FUSE_CUDA(f, cudaMemsetAsync(f->d_tile_kept, 0, (size_t)f->ntiles * 4, f->stream), "tile counts");
    FUSE_CUDA(f, cudaEventRecord(f->ev[0], f->stream), "event");
    pm::fuse_check_kernel<<<grid, pm::FUSE_THREADS, 0, f->stream>>>(f->d_refs, f->d_pairs, f->n, err2,
                                                                     p->max_rel_depth, p->min_consistent,
                                                                     f->d_block_kept, f->d_tile_kept);
    FUSE_CUDA(f, cudaGetLastError(), "fuse_check_kernel");
    FUSE_CUDA(f, cudaEventRecord(f->ev[1], f->stream), "event");
    pm::fuse_scan_tiles_kernel<<<1, 1024, 0, f->stream>>>(f->d_tile_kept, f->ntiles, f->d_tile_base, f->d_total);
    FUSE_CUDA(f, cudaGetLastError(), "fuse_scan_tiles_kernel");
    pm::fuse_scan_blocks_kernel<<<f->ntiles, 1024, 0, f->stream>>>(f->d_block_kept, nblk, f->d_tile_base,
                                                                   f->d_offsets);
    FUSE_CUDA(f, cudaGetLastError(), "fuse_scan_blocks_kernel");
    pm::fuse_points_kernel<<<grid, pm::FUSE_THREADS, 0, f->stream>>>(f->d_refs, f->d_offsets, f->d_points);
    FUSE_CUDA(f, cudaGetLastError(), "fuse_points_kernel");
    FUSE_CUDA(f, cudaEventRecord(f->ev[2], f->stream), "event");
    FUSE_CUDA(f, cudaMemcpyAsync(f->h_total, f->d_total, 8, cudaMemcpyDeviceToHost, f->stream), "total");
    FUSE_CUDA(f, cudaStreamSynchronize(f->stream), "fusion");
    f->n_points = (long long)*f->h_total;
    FUSE_CUDA(f, cudaEventElapsedTime(&f->ms_check, f->ev[0], f->ev[1]), "timing");
    FUSE_CUDA(f, cudaEventElapsedTime(&f->ms_total, f->ev[0], f->ev[2]), "timing");
    return PM_OK;
}

pm_status pm_fusion_info(const pm_fusion *f, int64_t *num_points, float *ms_check, float *ms_total,
                         int *launches)
{
    if (!f) return PM_ERR_INVALID_ARGUMENT;
    if (f->n_points < 0) return PM_ERR_STATE;
    if (num_points) *num_points = f->n_points;
    if (ms_check) *ms_check = f->ms_check;
    if (ms_total) *ms_total = f->ms_total;
    if (launches) *launches = 4;
    return PM_OK;
}

pm_status pm_fusion_get_points(pm_fusion *f, float *xyzi, int64_t capacity)
{
    if (!f || (!xyzi && capacity > 0) || capacity < 0) return PM_ERR_INVALID_ARGUMENT;
    if (f->n_points < 0) return fuse_fail(f, PM_ERR_STATE, "pm_fusion_run has not run");
    const int64_t m = std::min<int64_t>(capacity, f->n_points);
    if (m > 0) {
        FUSE_CUDA(f, cudaSetDevice(f->device), "cudaSetDevice");
        FUSE_CUDA(f, cudaMemcpyAsync(xyzi, f->d_points, (size_t)m * sizeof(float4), cudaMemcpyDeviceToHost, f->stream),
                  "points");
        FUSE_CUDA(f, cudaStreamSynchronize(f->stream), "points");
    }
    return PM_OK;
}

pm_status pm_fusion_get_depth(pm_fusion *f, int ref, float *fused, uint8_t *count)
{
    if (!f || ref < 0 || ref >= f->n) return PM_ERR_INVALID_ARGUMENT;
    if (f->n_points < 0) return fuse_fail(f, PM_ERR_STATE, "pm_fusion_run has not run");
    const pm::FuseRefDev &r = f->h_refs[(size_t)ref];
    const size_t npix = (size_t)r.width * r.height;
    FUSE_CUDA(f, cudaSetDevice(f->device), "cudaSetDevice");
    if (fused) FUSE_CUDA(f, cudaMemcpyAsync(fused, r.fused, npix * 4, cudaMemcpyDeviceToHost, f->stream), "fused");
    if (count) FUSE_CUDA(f, cudaMemcpyAsync(count, r.count, npix, cudaMemcpyDeviceToHost, f->stream), "count");
    FUSE_CUDA(f, cudaStreamSynchronize(f->stream), "depth");
    return PM_OK;
}

pm_status pm_fusion_geometry(const pm_fusion *f, float *pairs, float *backproject)
{
    if (!f) return PM_ERR_INVALID_ARGUMENT;
    if (pairs) std::copy(f->pairs.begin(), f->pairs.end(), pairs);
    if (backproject) std::copy(f->bp.begin(), f->bp.end(), backproject);
    return PM_OK;
}

pm_status pm_fusion_write_ply(pm_fusion *f, const char *path)
{
    if (!f || !path) return PM_ERR_INVALID_ARGUMENT;
    if (f->n_points < 0) return fuse_fail(f, PM_ERR_STATE, "pm_fusion_run has not run");
    std::vector<float> pts((size_t)f->n_points * 4);
    pm_status st = pm_fusion_get_points(f, pts.data(), f->n_points);
    if (st != PM_OK) return st;
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return fuse_fail(f, PM_ERR_IO, std::string("cannot open ") + path);
    std::fprintf(fp,
                 "ply\nformat binary_little_endian 1.0\nelement vertex %lld\nproperty float x\nproperty float y\n"
                 "property float z\nproperty uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n",
                 f->n_points);
    bool ok = true;
    for (long long k = 0; k < f->n_points && ok; ++k) {
        unsigned char rec[15];
        const float *q = &pts[(size_t)k * 4];
        for (int c = 0; c < 3; ++c) {   // little-endian IEEE floats, byte by byte
            uint32_t bits;
            std::memcpy(&bits, &q[c], 4);
            for (int b = 0; b < 4; ++b) rec[4 * c + b] = (unsigned char)(bits >> (8 * b));
        }
        const float g = std::fmin(std::fmax(q[3], 0.0f), 1.0f) * 255.0f + 0.5f;
        rec[12] = rec[13] = rec[14] = (unsigned char)g;
        ok = std::fwrite(rec, 1, sizeof rec, fp) == sizeof rec;
    }
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? PM_OK : fuse_fail(f, PM_ERR_IO, std::string("cannot write ") + path);
}

const char *pm_fusion_last_error(const pm_fusion *f) { return f ? f->err.c_str() : ""; }

pm_status pm_fusion_destroy(pm_fusion *f)
{
    if (!f) return PM_ERR_INVALID_ARGUMENT;
    cudaSetDevice(f->device);
    fuse_free(f);
    delete f;
    return PM_OK;
}

}  // extern "C"
