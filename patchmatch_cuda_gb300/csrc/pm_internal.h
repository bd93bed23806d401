// pm_internal.h -- host-side declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "patchmatch_gb300.h"
#include "pm_sweep.cuh"

namespace pm {

enum class LaunchKind { Sweep, Costs, Eval, SweepOccupancy, Refine };

struct LaunchReq {
    LaunchKind kind;
    cudaStream_t stream;
    int grid;
    int block;                 // Sweep: 32 * warps per line
    int *occupancy;            // SweepOccupancy: active CTAs per SM for `block`
    // Sweep
    const SweepArgs *sweep;
    // Costs / Eval
    const RefDesc *refs;
    int ref_index;
    int axis;
    int n;
    const int4 *queries;
    const float *depths;
    const float2 *slopes;      // Eval: per-query plane slopes, or null
    float *out;
    // Refine (axis, refs, ref_index as Costs)
    int trials;
    float sigma;
    uint32_t sweep_id;
    int samples;
};

// Window-size, sampler and plane-mode dispatch, split over translation units so they compile
// in parallel. Each returns cudaErrorInvalidValue when W is not in its group. The _hw groups
// sample through texture-unit bilinear filtering, the others through exact gathers; the _pl
// groups hold the slanted-plane kernels.
#define PM_DECLARE_GROUPS(g)                                          \
    cudaError_t launch_group_##g(int W, const LaunchReq &req);        \
    cudaError_t launch_group_##g##_hw(int W, const LaunchReq &req);   \
    cudaError_t launch_group_##g##_pl(int W, const LaunchReq &req);   \
    cudaError_t launch_group_##g##_hw_pl(int W, const LaunchReq &req);
PM_DECLARE_GROUPS(a)  // 3 .. 11
PM_DECLARE_GROUPS(b)  // 13 .. 17
PM_DECLARE_GROUPS(c)  // 19 .. 25
PM_DECLARE_GROUPS(d)  // 27 .. 45
#undef PM_DECLARE_GROUPS

inline cudaError_t launch_window(int W, bool hw, bool pl, const LaunchReq &req)
{
#define PM_PICK(g)                                                                      \
    return hw ? (pl ? launch_group_##g##_hw_pl(W, req) : launch_group_##g##_hw(W, req)) \
              : (pl ? launch_group_##g##_pl(W, req) : launch_group_##g(W, req));
    if (W <= 11) PM_PICK(a)
    if (W <= 17) PM_PICK(b)
    if (W <= 25) PM_PICK(c)
    PM_PICK(d)
#undef PM_PICK
}

// Prefilter, moments, conversions, init, transpose, Philox (pm_prep.cu).
cudaError_t launch_u8_to_float(const uint8_t *in, int in_pitch, float *out, int w, int h,
                               cudaStream_t s);
cudaError_t launch_filter(const float *in, float *tmp, float *out, int w, int h, int radius,
                          const float *weights, cudaStream_t s);
cudaError_t launch_box_moments(const float *img, double *row_i, double *row_ii, float *sum_i,
                               float *sum_ii, float *c1, int w, int h, int hw, cudaStream_t s);
cudaError_t launch_float_to_half(const float *in, void *out, int n, cudaStream_t s);
cudaError_t launch_init_depth(const RefDesc *refs, int r, int npix, cudaStream_t s);
cudaError_t launch_sample(const RefDesc *refs, int r, int view, int n, const float *xs,
                          const float *ys, float *out, cudaStream_t s);
cudaError_t launch_transpose(const float *in, size_t in_pitch, float *out, size_t out_pitch,
                             int w, int h, int layers, cudaStream_t s);
cudaError_t launch_philox(uint64_t seed, int n, const uint32_t *ctr, uint32_t *out,
                          cudaStream_t s);
cudaError_t launch_check_rcp(int exp_shift, unsigned long long *mismatches, cudaStream_t s);
cudaError_t measure_texture_peak(double *samples_per_s);

// Consistency filtering and fusion (pm_fuse.cu). A source's depth map is either on the device
// already (an engine's, read in place after its stream is synchronised) or copied from the host
// at creation.
struct FuseSource {
    const float *d_depth;        // device depth map, or null
    const float *d_intensity;    // device intensity in [0, 1], or null
    const float *h_depth;        // host depth map (when d_depth is null)
    const uint8_t *h_gray;       // host intensity 0..255, or null
    int width, height;
    float K[9], R[9], t[3];
    cudaStream_t wait_stream;    // synchronised before every run, or null
};
pm_status fusion_create(const FuseSource *sources, int n, int device, pm_fusion **out);

// Learned proposal (pm_proposal.cu): quarter-resolution images, the plane-sweep input of the
// network (17 channels), and the initial depth from its output.
constexpr int PROPOSAL_IN_CH = 17;
constexpr int PROPOSAL_PLANES = 8;
struct ProposalGeom {
    int w4, h4;          // quarter-resolution reference size
    int wp, hp;          // network size (w4, h4 rounded up to multiples of 16)
    int sw4[2], sh4[2];  // quarter-resolution size of the two sources
    float inv_far, inv_range;
    float hh[2][18];     // H1, H2 of the two sources for the plane normal (0, 0, 1)
};
cudaError_t launch_quarter(const uint8_t *img, int pitch, int w4, int h4, float *out, cudaStream_t s);
cudaError_t launch_sweep_input(const ProposalGeom &g, const float *ref_q, const float *src0, const float *src1,
                               float *out, cudaStream_t s);
cudaError_t launch_proposal_init(const RefDesc *refs, int r, int npix, const ProposalGeom &g, const float *prob,
                                 float threshold, cudaStream_t s);

// BF16 tensor-core GEMM C[M, N] (+)= A[M, K] . B[N, K]^T (pm_gemm.cu). M % 128 == 0,
// N % 16 == 0, K % 64 == 0, leading dimensions multiples of 8 elements, 16-byte aligned
// pointers. splits > 1 (GEMM_ATOMIC_F32 only) divides K over the grid. *err is set to 1 if a
// CTA's pipeline wait times out.
enum GemmMode { GEMM_STORE_BF16 = 0, GEMM_STORE_F32 = 1, GEMM_ATOMIC_F32 = 2 };
cudaError_t gemm_prepare();  // one-time host set-up; call before capturing GEMMs in a graph
cudaError_t launch_gemm_bf16(const void *A, int lda, const void *B, int ldb, int M, int N, int K,
                             void *C, int ldc, int mode, const float *bias, int relu, int splits,
                             unsigned *err, cudaStream_t s);

}  // namespace pm
