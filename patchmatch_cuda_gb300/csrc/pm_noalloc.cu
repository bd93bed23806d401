// pm_noalloc.cu -- reference-window moments without any device allocation.
//
// Some callers cannot allocate device memory: code running inside a CUDA stream capture
// that must not add allocation nodes, callers whose memory budget is fixed up front by a
// host framework that owns every allocation, or plugins that are handed buffers and must
// not touch the allocator. pm_box_moments_noalloc computes the same reference-window box
// sums (and the variance term c1) as the engine's preparation step, but keeps its
// intermediate row sums in a fixed scratch array compiled into this library instead of
// allocating one.
//
// The scratch array is a file-scope __device__ variable: every device that loads the library
// holds PM_NOALLOC_SCRATCH_DOUBLES doubles (8 MiB) until the process exits, whether or not the
// entry point is called. Host code cannot use the array's name as a device address, so the
// first call on each device (with that device current) resolves the address once with
// cudaGetSymbolAddress; make that first call before any stream capture. The address is kept
// for the life of the process: after cudaDeviceReset the library's module may load at another
// address, so the entry point must not be called on a device that was reset. Every call on a
// device shares the one array, so calls whose work overlaps on the GPU (different streams, or
// threads) race; serialise them. The row pass rewrites every scratch element the column pass
// then reads, so nothing needs clearing between calls.
#include <algorithm>
#include <mutex>

#include "../../include/patchmatch_gb300.h"
#include "pm_internal.h"

namespace {

constexpr size_t kScratchDoubles = PM_NOALLOC_SCRATCH_DOUBLES;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

std::mutex g_addr_mutex;
double *g_scratch_addr[64] = {};

// Row sums of I and I*I over rows [row0, row0 + rows) of the image, for the strip that
// starts at image row row0; rows outside the image are written as zero.
__global__ void strip_rows_kernel(const float *__restrict__ img, size_t pitch, int w, int h,
                                  int hw, int row0, int rows, double *__restrict__ ri,
                                  double *__restrict__ rii)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || r >= rows) return;
    const int y = row0 + r;
    double a = 0.0, b = 0.0;
    if (y >= 0 && y < h) {
        const float *row = (const float *)((const char *)img + (size_t)y * pitch);
        for (int k = -hw; k <= hw; ++k) {
            const int xx = x + k;
            const double v = (xx >= 0 && xx < w) ? (double)row[xx] : 0.0;
            a += v;
            b += v * v;
        }
    }
    ri[(size_t)r * w + x] = a;
    rii[(size_t)r * w + x] = b;
}

// Column sums for image rows [y0, y1); the strip buffer starts at image row y0 - hw.
__global__ void strip_cols_kernel(const double *__restrict__ ri, const double *__restrict__ rii,
                                  int w, int h, int hw, int y0, int y1, float *__restrict__ si,
                                  float *__restrict__ sii, float *__restrict__ c1, size_t out_pitch)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = y0 + blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= y1) return;
    double a = 0.0, b = 0.0;
    for (int k = -hw; k <= hw; ++k) {
        const int r = y + k - (y0 - hw);  // strip row of image row y + k
        a += ri[(size_t)r * w + x];
        b += rii[(size_t)r * w + x];
    }
    const int nx = min(x + hw, w - 1) - max(x - hw, 0) + 1;
    const int ny = min(y + hw, h - 1) - max(y - hw, 0) + 1;
    const double v = b - a * a / (double)(nx * ny);
    const size_t o = (size_t)y * (out_pitch / sizeof(float)) + x;
    if (si) si[o] = (float)a;
    if (sii) sii[o] = (float)b;
    if (c1) c1[o] = v < 0.00001 ? 0.0f : (float)v;
}

// Device address of the scratch array for the current device, resolved once per device.
pm_status scratch_address(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return PM_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lk(g_addr_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return PM_ERR_CUDA;
        }
        g_scratch_addr[dev] = (double *)p;
    }
    *out = g_scratch_addr[dev];
    return PM_OK;
}

}  // namespace

extern "C" pm_status pm_box_moments_noalloc(const float *d_ref, size_t ref_pitch, int width,
                                            int height, int half_window, float *d_sum_i,
                                            float *d_sum_ii, float *d_c1, size_t out_pitch,
                                            void *stream)
{
    if (!d_ref || width < 1 || height < 1 || (!d_sum_i && !d_sum_ii && !d_c1))
        return PM_ERR_INVALID_ARGUMENT;
    if (half_window < 1 || half_window > PM_MAX_HALF_WINDOW) return PM_ERR_WINDOW_SIZE;
    if (ref_pitch < (size_t)width * sizeof(float) || out_pitch < (size_t)width * sizeof(float) ||
        ref_pitch % sizeof(float) != 0 || out_pitch % sizeof(float) != 0)
        return PM_ERR_INVALID_ARGUMENT;
    // One strip of image rows needs (rows + 2 * half_window) * width * 2 doubles of scratch;
    // at least two rows per strip must fit.
    const size_t per_row = (size_t)width * 2;
    const size_t max_rows = kScratchDoubles / per_row;
    if (max_rows < (size_t)(2 * half_window + 2)) return PM_ERR_SCRATCH_LIMIT;
    double *scratch = nullptr;
    pm_status st = scratch_address(&scratch);
    if (st != PM_OK) return st;
    // a strip's row pass launches (rows + 7) / 8 blocks along y, at most 65535
    const size_t grid_rows = (size_t)65535 * 8 - 2 * (size_t)half_window;
    const int strip = (int)std::min<size_t>(std::min<size_t>((size_t)height, max_rows - 2 * (size_t)half_window),
                                            grid_rows);
    cudaStream_t s = (cudaStream_t)stream;
    const dim3 b(32, 8);
    for (int y0 = 0; y0 < height; y0 += strip) {
        const int y1 = std::min(height, y0 + strip);
        const int rows = (y1 - y0) + 2 * half_window;
        double *ri = scratch, *rii = scratch + (size_t)rows * width;
        strip_rows_kernel<<<dim3((width + 31) / 32, (rows + 7) / 8), b, 0, s>>>(
            d_ref, ref_pitch, width, height, half_window, y0 - half_window, rows, ri, rii);
        strip_cols_kernel<<<dim3((width + 31) / 32, (y1 - y0 + 7) / 8), b, 0, s>>>(
            ri, rii, width, height, half_window, y0, y1, d_sum_i, d_sum_ii, d_c1, out_pitch);
    }
    return cudaGetLastError() == cudaSuccess ? PM_OK : PM_ERR_CUDA;
}
