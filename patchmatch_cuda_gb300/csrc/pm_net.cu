// pm_net.cu -- the learned depth proposal: a BF16 encoder-decoder network whose convolutions
// run on the tensor-core GEMM (pm_gemm.cu), trained on the GPU by its own forward and backward
// kernels, and its C ABI. No counterpart in the reference, whose initial depth is uniformly
// random (array2d_wrapper.cu:3-20); the proposal replaces that initialisation.
//
// Network (all 3x3 convolutions with zero padding and ReLU, NHWC BF16 activations):
//   encoder  L0: 17 -> 32 -> 32 | L1: s2 -> 64 -> 64 | L2: s2 -> 96 -> 96 | L3: s2 -> 128 -> 128
//            L4: s2 -> 128 -> 128
//   decoder  each level: nearest 2x upsampling of the level below, concatenated with the
//            encoder's output of the level (written straight into one buffer), two convs:
//            D3: 256 -> 128 -> 128 | D2: 224 -> 96 -> 96 | D1: 160 -> 64 -> 64 | D0: 96 -> 32 -> 32
//   head     1x1 conv 32 -> 2 (no activation): the normalised inverse depth (after a sigmoid)
//            and the confidence logit.
// Input: 17 channels at a quarter of the reference resolution, padded to multiples of 16: the
// reference image and two source images warped onto 8 fronto-parallel depths.
//
// A convolution is im2col (BF16 rows of 9 Cin taps, padded to a multiple of 64) followed by
// the GEMM with the bias and ReLU in its epilogue. Backward per layer: ReLU mask -> dZ (BF16,
// and transposed), dW = dZ^T col (split-K over pixels with FP32 atomics), dcol = dZ W (FP32),
// then a col2im gather adds dX into the input's gradient. Adam updates FP32 master weights,
// repacked to BF16 for the GEMMs after every step.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/patchmatch_gb300.h"
#include "pm_internal.h"

typedef __nv_bfloat16 bf16;

namespace {
__device__ unsigned g_gemm_err;
}

namespace pm {
namespace net {

constexpr int IN_CH = 17;
constexpr int OUT_CH = 2;
constexpr int HEAD_N = 16;  // the head's GEMM width (2 used)

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

// ---- kernels ---------------------------------------------------------------------------------

// im2col of a k x k (k = 1 or 3) convolution with zero padding (k - 1) / 2 and stride s:
// col[p][t * C + c] for output pixel p, tap t, channel c; zero past 9C (or C) and for rows >= P.
__global__ void im2col_kernel(const bf16 *__restrict__ in, int cs, int co, int C, int B, int H, int W,
                              int Ho, int Wo, int ksize, int stride, bf16 *__restrict__ col, int Kpad,
                              int P)
{
    const int chunks = Kpad / 8;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)P * chunks) return;
    const int p = (int)(i / chunks), k0 = (int)(i % chunks) * 8;
    const int b = p / (Ho * Wo), r = p % (Ho * Wo), oy = r / Wo, ox = r % Wo;
    const int pad = (ksize - 1) / 2, K = ksize * ksize * C;
    if ((C & 7) == 0 && (cs & 7) == 0 && (co & 7) == 0) {
        // the 8 elements are 8 consecutive channels of one tap: one 16-byte load
        uint4 w = make_uint4(0, 0, 0, 0);
        if (k0 < K) {
            const int t = k0 / C, c = k0 % C;
            const int iy = oy * stride + t / ksize - pad, ix = ox * stride + t % ksize - pad;
            if (iy >= 0 && iy < H && ix >= 0 && ix < W)
                w = *(const uint4 *)(in + ((size_t)(b * H + iy) * W + ix) * cs + co + c);
        }
        *(uint4 *)(col + (size_t)p * Kpad + k0) = w;
        return;
    }
    __align__(16) bf16 v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int k = k0 + j;
        bf16 x = __float2bfloat16(0.0f);
        if (k < K) {
            const int t = k / C, c = k % C;
            const int iy = oy * stride + t / ksize - pad, ix = ox * stride + t % ksize - pad;
            if (iy >= 0 && iy < H && ix >= 0 && ix < W)
                x = in[((size_t)(b * H + iy) * W + ix) * cs + co + c];
        }
        v[j] = x;
    }
    *(uint4 *)(col + (size_t)p * Kpad + k0) = *(const uint4 *)v;
}

// Nearest 2x upsampling of src (B, h, w, C) into dst (B, 2h, 2w) channels [co, co + C).
__global__ void upsample2x_kernel(const bf16 *__restrict__ src, int scs, int sco, int C, int B, int h,
                                  int w, bf16 *__restrict__ dst, int dcs, int dco)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)B * 4 * h * w * C;
    if (i >= n) return;
    const int c = (int)(i % C);
    const long long q = i / C;
    const int W2 = 2 * w, H2 = 2 * h;
    const int x = (int)(q % W2), y = (int)((q / W2) % H2), b = (int)(q / ((long long)W2 * H2));
    dst[((size_t)(b * H2 + y) * W2 + x) * dcs + dco + c] =
        src[((size_t)(b * h + y / 2) * w + x / 2) * scs + sco + c];
}

// Gradient of the upsampling: g_src (B, h, w, C) += sum of the 4 children in g_dst.
__global__ void upsample2x_back_kernel(const float *__restrict__ gdst, int dcs, int dco, int C, int B,
                                       int h, int w, float *__restrict__ gsrc, int scs, int sco)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)B * h * w * C;
    if (i >= n) return;
    const int c = (int)(i % C);
    const long long q = i / C;
    const int x = (int)(q % w), y = (int)((q / w) % h), b = (int)(q / ((long long)w * h));
    const int W2 = 2 * w, H2 = 2 * h;
    float s = 0.0f;
#pragma unroll
    for (int d = 0; d < 4; ++d)
        s += gdst[((size_t)(b * H2 + 2 * y + (d >> 1)) * W2 + 2 * x + (d & 1)) * dcs + dco + c];
    gsrc[((size_t)(b * h + y) * w + x) * scs + sco + c] += s;
}

// ReLU gradient: dZ = g * (y > 0) (or g when the layer has no activation), as BF16 rows
// [Ppad x N64] and transposed [128 x Ppad] (zero padding), plus the bias gradient.
__global__ void relu_back_kernel(const float *__restrict__ g, int gcs, int gco, const bf16 *__restrict__ y,
                                 int ycs, int yco, int yf32, int relu, int P, int Ppad, int N, int N64,
                                 bf16 *__restrict__ dz, bf16 *__restrict__ dzt, float *__restrict__ dbias)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)Ppad * N64) return;
    const int p = (int)(i / N64), c = (int)(i % N64);
    float v = 0.0f;
    if (p < P && c < N) {
        v = g[(size_t)p * gcs + gco + c];
        if (relu) {
            const float yv = yf32 ? ((const float *)y)[(size_t)p * ycs + yco + c]
                                  : __bfloat162float(y[(size_t)p * ycs + yco + c]);
            if (!(yv > 0.0f)) v = 0.0f;
        }
    }
    const bf16 b = __float2bfloat16(v);
    dz[(size_t)p * N64 + c] = b;
    if (c < 128) dzt[(size_t)c * Ppad + p] = c < N ? b : __float2bfloat16(0.0f);
    if (dbias && c < N && p < P) atomicAdd(dbias + c, v);
}

// out[c][r] = in[r][c] for a rows x cols BF16 matrix (32 x 32 tiles through shared memory).
__global__ void transpose_bf16_kernel(const bf16 *__restrict__ in, int rows, int cols, bf16 *__restrict__ out)
{
    __shared__ bf16 t[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int r = by + j, c = bx + threadIdx.x;
        t[j][threadIdx.x] = (r < rows && c < cols) ? in[(size_t)r * cols + c] : __float2bfloat16(0.0f);
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = bx + j, r = by + threadIdx.x;
        if (c < cols && r < rows) out[(size_t)c * rows + r] = t[threadIdx.x][j];
    }
}

// col2im gather: gin[b, iy, ix, co + c] += sum over taps of dcol[output pixel][t * C + c].
__global__ void col2im_add_kernel(const float *__restrict__ dcol, int Kpad, int C, int B, int H, int W,
                                  int Ho, int Wo, int ksize, int stride, float *__restrict__ gin, int cs,
                                  int co)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)B * H * W * C) return;
    const int c = (int)(i % C);
    const long long q = i / C;
    const int ix = (int)(q % W), iy = (int)((q / W) % H), b = (int)(q / ((long long)W * H));
    const int pad = (ksize - 1) / 2;
    float s = 0.0f;
    for (int t = 0; t < ksize * ksize; ++t) {
        const int ky = t / ksize, kx = t % ksize;
        const int ny = iy + pad - ky, nx = ix + pad - kx;  // = oy * stride, ox * stride
        if (ny < 0 || nx < 0 || ny % stride || nx % stride) continue;
        const int oy = ny / stride, ox = nx / stride;
        if (oy >= Ho || ox >= Wo) continue;
        s += dcol[(size_t)((b * Ho + oy) * Wo + ox) * Kpad + t * C + c];
    }
    gin[((size_t)(b * H + iy) * W + ix) * cs + co + c] += s;
}

// Packs FP32 master weights [Cout x K] into the GEMM's BF16 operands: w [Npad x Kpad] and
// wt [Kpad x N64] (zero padding), and the bias into FP32 [Npad].
__global__ void pack_kernel(const float *__restrict__ master, int cout, int K, int Npad, int Kpad, int N64,
                            bf16 *__restrict__ w, bf16 *__restrict__ wt, float *__restrict__ bias)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Npad * Kpad) {
        const int n = i / Kpad, k = i % Kpad;
        const float v = (n < cout && k < K) ? master[(size_t)n * K + k] : 0.0f;
        w[i] = __float2bfloat16(v);
    }
    if (i < Kpad * N64) {
        const int k = i / N64, n = i % N64;
        const float v = (n < cout && k < K) ? master[(size_t)n * K + k] : 0.0f;
        wt[i] = __float2bfloat16(v);
    }
    if (i < Npad) bias[i] = i < cout ? master[(size_t)cout * K + i] : 0.0f;
}

// grad[n][k] = dwbuf[n][k] for n < cout, k < K; clears dwbuf.
__global__ void unpack_grad_kernel(float *__restrict__ dwbuf, int Kpad, int cout, int K, float *__restrict__ grad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 128 * Kpad) return;
    const int n = i / Kpad, k = i % Kpad;
    if (n < cout && k < K) grad[(size_t)n * K + k] = dwbuf[i];
    dwbuf[i] = 0.0f;
}

__device__ __forceinline__ float sigmoid(float x) { return 1.0f / (1.0f + __expf(-x)); }

// Loss on the head's output o[p][0..1]: s = sigmoid(o0) predicts the normalised inverse depth
// t in [0, 1] with an L1 loss on the relative inverse-depth error |inv_p - inv_t| / inv_t
// (inv = inv_far + s inv_range; the relative error of the depth itself, to first order);
// q = sigmoid(o1) the probability that the prediction's depth is within `conf_tol` relative of
// the target's (binary cross-entropy, weight `conf_w`). Targets below 0 are masked. Writes
// dL/do and accumulates the loss terms and the count into acc[0..2].
__global__ void loss_kernel(const float *__restrict__ o, int ocs, const float *__restrict__ target, int P,
                            float inv_far, float inv_range, float conf_tol, float conf_w, float scale,
                            float *__restrict__ go, int gcs, float *__restrict__ acc)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    float l1 = 0.0f, bce = 0.0f, cnt = 0.0f;
    if (p < P) {
        const float t = target[p];
        float g0 = 0.0f, g1 = 0.0f;
        if (t >= 0.0f) {
            const float s = sigmoid(o[(size_t)p * ocs]), q = sigmoid(o[(size_t)p * ocs + 1]);
            const float inv_p = inv_far + s * inv_range, inv_t = inv_far + t * inv_range;
            const float y = fabsf(inv_p - inv_t) <= conf_tol * inv_t ? 1.0f : 0.0f;
            l1 = fabsf(inv_p - inv_t) / inv_t;
            bce = -(y * __logf(fmaxf(q, 1e-7f)) + (1.0f - y) * __logf(fmaxf(1.0f - q, 1e-7f)));
            g0 = (s > t ? 1.0f : (s < t ? -1.0f : 0.0f)) * inv_range / inv_t * s * (1.0f - s) * scale;
            g1 = conf_w * (q - y) * scale;
            cnt = 1.0f;
        }
        go[(size_t)p * gcs] = g0;
        go[(size_t)p * gcs + 1] = g1;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        l1 += __shfl_xor_sync(0xffffffffu, l1, off);
        bce += __shfl_xor_sync(0xffffffffu, bce, off);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    }
    if ((threadIdx.x & 31) == 0 && cnt > 0.0f) {
        atomicAdd(acc, l1);
        atomicAdd(acc + 1, bce);
        atomicAdd(acc + 2, cnt);
    }
}

// Adam on the flat FP32 parameters (bias-corrected step sizes precomputed on the host).
__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, size_t n, float lr_t, float b1, float b2, float eps)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr_t * mi / (sqrtf(vi) + eps);
}

// FP32 input [P x 17] (valid pixels) -> BF16 [P x 17].
__global__ void to_bf16_kernel(const float *__restrict__ in, bf16 *__restrict__ out, size_t n)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16(in[i]);
}

// Head output -> (sigmoid(o0), sigmoid(o1)) per pixel.
__global__ void head_out_kernel(const float *__restrict__ o, int ocs, int P, float *__restrict__ out)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    out[2 * p] = sigmoid(o[(size_t)p * ocs]);
    out[2 * p + 1] = sigmoid(o[(size_t)p * ocs + 1]);
}

inline unsigned blocks(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// ---- the network -----------------------------------------------------------------------------

// A tensor view: base (BF16 or FP32) with channel stride cs, channel offset co, C channels.
struct View {
    void *p = nullptr;
    int cs = 0, co = 0, C = 0;
};

struct Layer {
    int cin, cout, ksize, stride, relu;
    int B, H, W, Ho, Wo, P, Ppad;   // input H x W, output Ho x Wo
    int K, Kpad, Npad, N64;
    size_t woff;                    // master offset: weights [cout x K], then bias [cout]
    View in, out, gin, gout;        // activations (BF16; the head's output FP32) and gradients
    bool out_f32 = false;
    bf16 *col = nullptr, *w = nullptr, *wt = nullptr;
    float *bias = nullptr;
};

struct Net {
    int B, H, W;                     // batch and level-0 size (multiples of 16)
    std::vector<Layer> layers;
    struct Up { View src, dst, gsrc, gdst; int B, h, w; };
    std::vector<Up> ups;
    size_t nparam = 0;
    float *master = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    int adam_t = 0;
    std::vector<void *> allocs;
    bf16 *x = nullptr;               // input, [P0 x 17]
    float *out = nullptr;            // head output FP32 [P0pad x 16]
    float *gout_head = nullptr;
    bf16 *dz = nullptr, *dzt = nullptr, *colt = nullptr;
    float *dcol = nullptr, *dwbuf = nullptr, *acc = nullptr;
    float *prob = nullptr;           // [P0 x 2] sigmoid outputs
    size_t dz_n = 0, dzt_n = 0, colt_n = 0, dcol_n = 0, dw_n = 0;
    std::vector<float *> grad_bufs;  // zeroed before each backward
    std::vector<size_t> grad_sizes;
    unsigned *err = nullptr;
    cudaStream_t stream = nullptr;
};

template <typename T>
cudaError_t dalloc(Net &n, T **p, size_t count)
{
    void *q = nullptr;
    const cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 256);
    if (e != cudaSuccess) return e;
    n.allocs.push_back(q);
    *p = (T *)q;
    return cudaMemset(q, 0, count * sizeof(T) + 256);
}

cudaError_t build(Net &n)
{
    const int B = n.B;
    const int ch[5] = {32, 64, 96, 128, 128};
    int hs[5], ws[5];
    for (int l = 0; l < 5; ++l) {
        hs[l] = n.H >> l;
        ws[l] = n.W >> l;
    }
    auto P = [&](int l) { return B * hs[l] * ws[l]; };
    cudaError_t e;
    // activation buffers (BF16) and their gradients (FP32)
    auto act = [&](int l, int C, View &v, View &g) -> cudaError_t {
        bf16 *p;
        float *gp;
        cudaError_t r = dalloc(n, &p, (size_t)round_up(P(l), 128) * C);
        if (r != cudaSuccess) return r;
        r = dalloc(n, &gp, (size_t)round_up(P(l), 128) * C);
        if (r != cudaSuccess) return r;
        n.grad_bufs.push_back(gp);
        n.grad_sizes.push_back((size_t)round_up(P(l), 128) * C);
        v.p = p; v.cs = C; v.co = 0; v.C = C;
        g.p = gp; g.cs = C; g.co = 0; g.C = C;
        return cudaSuccess;
    };
    if ((e = dalloc(n, &n.x, (size_t)round_up(P(0), 128) * IN_CH)) != cudaSuccess) return e;
    View X{n.x, IN_CH, 0, IN_CH}, noG{};
    // concat buffers: Cat_l = [up (decoder width of level l+1) | skip_l]
    const int upw[4] = {ch[1], ch[2], ch[3], ch[4]};
    View cat[4], gcat[4];
    for (int l = 0; l < 4; ++l)
        if ((e = act(l, upw[l] + ch[l], cat[l], gcat[l])) != cudaSuccess) return e;
    auto slice = [](View v, int co, int C) { v.co = co; v.C = C; return v; };
    View A[5], gA[5], Bt[5], gB[5], D[4], gD[4];
    for (int l = 0; l < 5; ++l)
        if ((e = act(l, ch[l], A[l], gA[l])) != cudaSuccess) return e;
    if ((e = act(4, ch[4], Bt[4], gB[4])) != cudaSuccess) return e;  // bottleneck output
    for (int l = 0; l < 4; ++l) {
        if ((e = act(l, ch[l], D[l], gD[l])) != cudaSuccess) return e;     // decoder first conv
        if ((e = act(l, ch[l], Bt[l], gB[l])) != cudaSuccess) return e;    // decoder output
    }
    auto add = [&](int cin, int cout, int ks, int st, int relu, int l_in, View in, View gin, View out,
                   View gout) {
        Layer L{};
        L.cin = cin; L.cout = cout; L.ksize = ks; L.stride = st; L.relu = relu;
        L.B = B; L.H = hs[l_in]; L.W = ws[l_in];
        L.Ho = L.H / st; L.Wo = L.W / st;
        L.P = B * L.Ho * L.Wo; L.Ppad = round_up(L.P, 128);
        L.K = ks * ks * cin; L.Kpad = round_up(L.K, 64);
        L.Npad = cout < 16 ? 16 : cout; L.N64 = round_up(L.Npad, 64);
        L.woff = n.nparam;
        n.nparam += (size_t)cout * L.K + cout;
        L.in = in; L.gin = gin; L.out = out; L.gout = gout;
        n.layers.push_back(L);
    };
    // encoder
    add(IN_CH, ch[0], 3, 1, 1, 0, X, noG, A[0], gA[0]);
    add(ch[0], ch[0], 3, 1, 1, 0, A[0], gA[0], slice(cat[0], upw[0], ch[0]), slice(gcat[0], upw[0], ch[0]));
    for (int l = 1; l < 4; ++l) {
        add(ch[l - 1], ch[l], 3, 2, 1, l - 1, slice(cat[l - 1], upw[l - 1], ch[l - 1]),
            slice(gcat[l - 1], upw[l - 1], ch[l - 1]), A[l], gA[l]);
        add(ch[l], ch[l], 3, 1, 1, l, A[l], gA[l], slice(cat[l], upw[l], ch[l]), slice(gcat[l], upw[l], ch[l]));
    }
    add(ch[3], ch[4], 3, 2, 1, 3, slice(cat[3], upw[3], ch[3]), slice(gcat[3], upw[3], ch[3]), A[4], gA[4]);
    add(ch[4], ch[4], 3, 1, 1, 4, A[4], gA[4], Bt[4], gB[4]);
    // decoder
    for (int l = 3; l >= 0; --l) {
        Net::Up u;
        u.src = Bt[l + 1]; u.gsrc = gB[l + 1];
        u.dst = slice(cat[l], 0, upw[l]); u.gdst = slice(gcat[l], 0, upw[l]);
        u.B = B; u.h = hs[l + 1]; u.w = ws[l + 1];
        n.ups.push_back(u);
        add(upw[l] + ch[l], ch[l], 3, 1, 1, l, cat[l], gcat[l], D[l], gD[l]);
        add(ch[l], ch[l], 3, 1, 1, l, D[l], gD[l], Bt[l], gB[l]);
    }
    // head
    if ((e = dalloc(n, &n.out, (size_t)round_up(P(0), 128) * HEAD_N)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.gout_head, (size_t)round_up(P(0), 128) * HEAD_N)) != cudaSuccess) return e;
    add(ch[0], OUT_CH, 1, 1, 0, 0, Bt[0], gB[0], View{n.out, HEAD_N, 0, HEAD_N}, View{n.gout_head, HEAD_N, 0, HEAD_N});
    n.layers.back().out_f32 = true;
    // per-layer GEMM operands and shared scratch
    for (Layer &L : n.layers) {
        if ((e = dalloc(n, &L.col, (size_t)L.Ppad * L.Kpad)) != cudaSuccess) return e;
        if ((e = dalloc(n, &L.w, (size_t)L.Npad * L.Kpad)) != cudaSuccess) return e;
        if ((e = dalloc(n, &L.wt, (size_t)L.Kpad * L.N64)) != cudaSuccess) return e;
        if ((e = dalloc(n, &L.bias, (size_t)L.Npad)) != cudaSuccess) return e;
        n.dz_n = std::max(n.dz_n, (size_t)L.Ppad * L.N64);
        n.dzt_n = std::max(n.dzt_n, (size_t)128 * L.Ppad);
        n.colt_n = std::max(n.colt_n, (size_t)L.Kpad * L.Ppad);
        n.dcol_n = std::max(n.dcol_n, (size_t)L.Ppad * L.Kpad);
        n.dw_n = std::max(n.dw_n, (size_t)128 * L.Kpad);
    }
    if ((e = dalloc(n, &n.dz, n.dz_n)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.dzt, n.dzt_n)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.colt, n.colt_n)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.dcol, n.dcol_n)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.dwbuf, n.dw_n)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.acc, 4)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.prob, (size_t)P(0) * 2)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.master, n.nparam)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.grad, n.nparam)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.adam_m, n.nparam)) != cudaSuccess) return e;
    if ((e = dalloc(n, &n.adam_v, n.nparam)) != cudaSuccess) return e;
    return cudaGetSymbolAddress((void **)&n.err, g_gemm_err);
}

// Deterministic He initialisation (host, splitmix64 -> Box-Muller), biases zero.
void init_params(Net &n, uint64_t seed, std::vector<float> &h)
{
    h.assign(n.nparam, 0.0f);
    uint64_t s = seed;
    auto next = [&]() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return (double)((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
    };
    for (const Layer &L : n.layers) {
        const double sd = std::sqrt(2.0 / L.K) * (L.relu ? 1.0 : 0.1);
        for (size_t i = 0; i < (size_t)L.cout * L.K; ++i) {
            const double u1 = std::max(next(), 1e-300), u2 = next();
            h[L.woff + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
}

cudaError_t pack_all(Net &n)
{
    for (Layer &L : n.layers) {
        const int m = std::max(L.Npad * L.Kpad, L.Kpad * L.N64);
        pack_kernel<<<blocks(m), 256, 0, n.stream>>>(n.master + L.woff, L.cout, L.K, L.Npad, L.Kpad, L.N64, L.w,
                                                     L.wt, L.bias);
    }
    return cudaGetLastError();
}

cudaError_t forward(Net &n, const float *input)
{
    cudaStream_t s = n.stream;
    const size_t nin = (size_t)n.B * n.H * n.W * IN_CH;
    to_bf16_kernel<<<blocks((long long)nin), 256, 0, s>>>(input, n.x, nin);
    size_t up = 0;
    for (size_t li = 0; li < n.layers.size(); ++li) {
        Layer &L = n.layers[li];
        // a decoder level's first conv reads the concat buffer: fill its upsampled part first
        if (up < n.ups.size() && L.in.p == n.ups[up].dst.p && L.in.co == 0 && L.in.C > n.ups[up].dst.C) {
            const Net::Up &u = n.ups[up++];
            const long long cnt = (long long)u.B * 4 * u.h * u.w * u.src.C;
            upsample2x_kernel<<<blocks(cnt), 256, 0, s>>>((const bf16 *)u.src.p, u.src.cs, u.src.co, u.src.C,
                                                           u.B, u.h, u.w, (bf16 *)u.dst.p, u.dst.cs, u.dst.co);
        }
        im2col_kernel<<<blocks((long long)L.P * (L.Kpad / 8)), 256, 0, s>>>(
            (const bf16 *)L.in.p, L.in.cs, L.in.co, L.cin, L.B, L.H, L.W, L.Ho, L.Wo, L.ksize, L.stride, L.col,
            L.Kpad, L.P);
        cudaError_t e;
        if (L.out_f32)
            e = launch_gemm_bf16(L.col, L.Kpad, L.w, L.Kpad, L.Ppad, L.Npad, L.Kpad, L.out.p, L.out.cs,
                                 GEMM_STORE_F32, L.bias, 0, 1, n.err, s);
        else
            e = launch_gemm_bf16(L.col, L.Kpad, L.w, L.Kpad, L.Ppad, L.Npad, L.Kpad,
                                 (bf16 *)L.out.p + L.out.co, L.out.cs, GEMM_STORE_BF16, L.bias, L.relu, 1,
                                 n.err, s);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

// Gradients of the loss into n.grad (overwritten).
cudaError_t backward(Net &n)
{
    cudaStream_t s = n.stream;
    for (size_t i = 0; i < n.grad_bufs.size(); ++i)
        cudaMemsetAsync(n.grad_bufs[i], 0, n.grad_sizes[i] * sizeof(float), s);
    cudaMemsetAsync(n.grad, 0, n.nparam * sizeof(float), s);
    size_t up = n.ups.size();
    for (int li = (int)n.layers.size() - 1; li >= 0; --li) {
        Layer &L = n.layers[li];
        relu_back_kernel<<<blocks((long long)L.Ppad * L.N64), 256, 0, s>>>(
            (const float *)L.gout.p, L.gout.cs, L.gout.co, (const bf16 *)L.out.p, L.out.cs, L.out.co,
            L.out_f32 ? 1 : 0, L.relu, L.P, L.Ppad, L.cout, L.N64, n.dz, n.dzt, n.grad + L.woff + (size_t)L.cout * L.K);
        const dim3 tb(32, 8), tg((L.Kpad + 31) / 32, (L.Ppad + 31) / 32);
        transpose_bf16_kernel<<<tg, tb, 0, s>>>(L.col, L.Ppad, L.Kpad, n.colt);
        // dW (rows >= cout of dz^T are zero) with K = pixels split over CTAs
        const int ktiles = L.Ppad / 64, ntiles = (L.Kpad + 127) / 128;
        const int splits = std::max(1, std::min(ktiles, 2 * 152 / ntiles));
        cudaError_t e = launch_gemm_bf16(n.dzt, L.Ppad, n.colt, L.Ppad, 128, L.Kpad, L.Ppad, n.dwbuf, L.Kpad,
                                         GEMM_ATOMIC_F32, nullptr, 0, splits, n.err, s);
        if (e != cudaSuccess) return e;
        unpack_grad_kernel<<<blocks(128LL * L.Kpad), 256, 0, s>>>(n.dwbuf, L.Kpad, L.cout, L.K, n.grad + L.woff);
        if (L.gin.p) {
            e = launch_gemm_bf16(n.dz, L.N64, L.wt, L.N64, L.Ppad, L.Kpad, L.N64, n.dcol, L.Kpad, GEMM_STORE_F32,
                                 nullptr, 0, 1, n.err, s);
            if (e != cudaSuccess) return e;
            col2im_add_kernel<<<blocks((long long)L.B * L.H * L.W * L.cin), 256, 0, s>>>(
                n.dcol, L.Kpad, L.cin, L.B, L.H, L.W, L.Ho, L.Wo, L.ksize, L.stride, (float *)L.gin.p, L.gin.cs,
                L.gin.co);
        }
        // the gradient of a concat buffer's upsampled part flows to the level below
        if (up > 0 && L.in.p == n.ups[up - 1].dst.p && L.in.co == 0 && L.in.C > n.ups[up - 1].dst.C) {
            const Net::Up &u = n.ups[--up];
            const long long cnt = (long long)u.B * u.h * u.w * u.src.C;
            upsample2x_back_kernel<<<blocks(cnt), 256, 0, s>>>((const float *)u.gdst.p, u.gdst.cs, u.gdst.co,
                                                                u.src.C, u.B, u.h, u.w, (float *)u.gsrc.p,
                                                                u.gsrc.cs, u.gsrc.co);
        }
    }
    return cudaGetLastError();
}

cudaError_t loss(Net &n, const float *target, float inv_far, float inv_range)
{
    const int P0 = n.B * n.H * n.W;
    cudaMemsetAsync(n.acc, 0, 4 * sizeof(float), n.stream);
    // the gradient is that of (sum over valid pixels) / P0; Adam's steps do not depend on a
    // constant factor, and pm_net_gradients reports the loss terms as means over valid pixels
    loss_kernel<<<blocks(P0), 256, 0, n.stream>>>(n.out, HEAD_N, target, P0, inv_far, inv_range, 0.02f, 0.1f,
                                                   1.0f / (float)P0, n.gout_head, HEAD_N, n.acc);
    return cudaGetLastError();
}

}  // namespace net
}  // namespace pm

struct pm_net {
    pm::net::Net n;
    std::string err;
};

using pm::net::Net;

extern "C" {

pm_status pm_gemm_bf16(const void *d_a, int lda, const void *d_b, int ldb, int m, int n, int k,
                       void *d_c, int ldc, int mode, const float *d_bias, int relu, int splits,
                       void *stream)
{
    if (!d_a || !d_b || !d_c || mode < 0 || mode > 2) return PM_ERR_INVALID_ARGUMENT;
    unsigned *err = nullptr;
    if (cudaGetSymbolAddress((void **)&err, g_gemm_err) != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_CUDA;
    }
    const cudaError_t e = pm::launch_gemm_bf16(d_a, lda, d_b, ldb, m, n, k, d_c, ldc, mode, d_bias,
                                               relu, splits, err, (cudaStream_t)stream);
    if (e == cudaErrorInvalidValue) {
        cudaGetLastError();
        return PM_ERR_INVALID_ARGUMENT;
    }
    return e == cudaSuccess ? PM_OK : PM_ERR_CUDA;
}

pm_status pm_gemm_error(unsigned *out, int clear)
{
    if (!out) return PM_ERR_INVALID_ARGUMENT;
    if (cudaMemcpyFromSymbol(out, g_gemm_err, sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_CUDA;
    }
    if (clear) {
        const unsigned z = 0;
        if (cudaMemcpyToSymbol(g_gemm_err, &z, sizeof z) != cudaSuccess) {
            cudaGetLastError();
            return PM_ERR_CUDA;
        }
    }
    return PM_OK;
}

pm_status pm_net_create(int batch, int height, int width, uint64_t seed, pm_net **out)
{
    if (!out || batch < 1 || height < 16 || width < 16 || height % 16 || width % 16 || batch > 4096)
        return PM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (pm::gemm_prepare() != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_CUDA;
    }
    pm_net *h = new pm_net();
    h->n.B = batch;
    h->n.H = height;
    h->n.W = width;
    cudaError_t e = pm::net::build(h->n);
    std::vector<float> init;
    if (e == cudaSuccess) {
        pm::net::init_params(h->n, seed, init);
        e = cudaMemcpy(h->n.master, init.data(), init.size() * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = pm::net::pack_all(h->n);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->n.stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        pm_net_destroy(h);
        return e == cudaErrorMemoryAllocation ? PM_ERR_OUT_OF_MEMORY : PM_ERR_CUDA;
    }
    *out = h;
    return PM_OK;
}

pm_status pm_net_destroy(pm_net *h)
{
    if (!h) return PM_OK;
    cudaDeviceSynchronize();
    for (void *p : h->n.allocs) cudaFree(p);
    delete h;
    return PM_OK;
}

pm_status pm_net_num_params(const pm_net *h, size_t *n)
{
    if (!h || !n) return PM_ERR_INVALID_ARGUMENT;
    *n = h->n.nparam;
    return PM_OK;
}

pm_status pm_net_size(const pm_net *h, int *batch, int *height, int *width)
{
    if (!h) return PM_ERR_INVALID_ARGUMENT;
    if (batch) *batch = h->n.B;
    if (height) *height = h->n.H;
    if (width) *width = h->n.W;
    return PM_OK;
}

pm_status pm_net_get_params(pm_net *h, float *dst, size_t n)
{
    if (!h || !dst || n != h->n.nparam) return PM_ERR_INVALID_ARGUMENT;
    if (cudaMemcpy(dst, h->n.master, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return PM_ERR_CUDA;
    return PM_OK;
}

pm_status pm_net_set_params(pm_net *h, const float *src, size_t n)
{
    if (!h || !src || n != h->n.nparam) return PM_ERR_INVALID_ARGUMENT;
    if (cudaMemcpy(h->n.master, src, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return PM_ERR_CUDA;
    if (pm::net::pack_all(h->n) != cudaSuccess || cudaStreamSynchronize(h->n.stream) != cudaSuccess)
        return PM_ERR_CUDA;
    h->n.adam_t = 0;
    cudaMemset(h->n.adam_m, 0, n * sizeof(float));
    cudaMemset(h->n.adam_v, 0, n * sizeof(float));
    return PM_OK;
}

pm_status pm_net_forward(pm_net *h, const float *d_input, float *d_out, void *stream)
{
    if (!h || !d_input) return PM_ERR_INVALID_ARGUMENT;
    Net &n = h->n;
    n.stream = (cudaStream_t)stream;
    cudaError_t e = pm::net::forward(n, d_input);
    const int P0 = n.B * n.H * n.W;
    if (e == cudaSuccess && d_out) {
        pm::net::head_out_kernel<<<pm::net::blocks(P0), 256, 0, n.stream>>>(n.out, pm::net::HEAD_N, P0, d_out);
        e = cudaGetLastError();
    }
    n.stream = nullptr;
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorInvalidValue ? PM_ERR_INVALID_ARGUMENT : PM_ERR_CUDA;
    }
    return PM_OK;
}

pm_status pm_net_gradients(pm_net *h, const float *d_input, const float *d_target, float inv_far,
                           float inv_range, float *grad_out, size_t n_grad, float *loss_out)
{
    if (!h || !d_input || !d_target || (grad_out && n_grad != h->n.nparam)) return PM_ERR_INVALID_ARGUMENT;
    Net &n = h->n;
    cudaError_t e = pm::net::forward(n, d_input);
    if (e == cudaSuccess) e = pm::net::loss(n, d_target, inv_far, inv_range);
    if (e == cudaSuccess) e = pm::net::backward(n);
    float acc[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(acc, n.acc, sizeof acc, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && grad_out) e = cudaMemcpy(grad_out, n.grad, n_grad * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_CUDA;
    }
    unsigned err = 0;
    cudaMemcpyFromSymbol(&err, g_gemm_err, sizeof err);
    if (err) return PM_ERR_CUDA;
    if (loss_out) {
        const float cnt = acc[2] > 0.0f ? acc[2] : 1.0f;
        loss_out[0] = acc[0] / cnt;
        loss_out[1] = acc[1] / cnt;
        loss_out[2] = acc[2];
    }
    return PM_OK;
}

pm_status pm_net_train_step(pm_net *h, const float *d_input, const float *d_target, float inv_far,
                            float inv_range, float lr, float *loss_out)
{
    pm_status st = pm_net_gradients(h, d_input, d_target, inv_far, inv_range, nullptr, 0, loss_out);
    if (st != PM_OK) return st;
    Net &n = h->n;
    const float b1 = 0.9f, b2 = 0.999f;
    ++n.adam_t;
    const float lr_t = lr * std::sqrt(1.0f - std::pow(b2, (float)n.adam_t)) / (1.0f - std::pow(b1, (float)n.adam_t));
    pm::net::adam_kernel<<<pm::net::blocks((long long)n.nparam), 256, 0, n.stream>>>(
        n.master, n.grad, n.adam_m, n.adam_v, n.nparam, lr_t, b1, b2, 1e-8f);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = pm::net::pack_all(n);
    if (e == cudaSuccess) e = cudaStreamSynchronize(n.stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_CUDA;
    }
    return PM_OK;
}

pm_status pm_net_layout(const pm_net *h, int *n_layers, int *desc, int max_layers)
{
    if (!h || !n_layers) return PM_ERR_INVALID_ARGUMENT;
    *n_layers = (int)h->n.layers.size();
    if (desc) {
        for (int i = 0; i < *n_layers && i < max_layers; ++i) {
            const pm::net::Layer &L = h->n.layers[i];
            int *d = desc + 8 * i;
            d[0] = L.cin; d[1] = L.cout; d[2] = L.ksize; d[3] = L.stride; d[4] = L.relu;
            d[5] = (int)L.woff; d[6] = L.H; d[7] = L.W;
        }
    }
    return PM_OK;
}

}  // extern "C"
