// noalloc.cu — the spline adjoint (translate) for callers that cannot
// allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: hosts that hand
// every byte of device memory to their own pool or arena and forbid
// allocations outside it, and latency-bound callers for whom the implicit
// device synchronisation of cudaMalloc and cudaFree is not acceptable.
// mgr_translate3d_noalloc serves them: the caller passes the force field
// and the gradient buffer, and every intermediate (per-axis transposed
// spline rows and the two separable pass buffers) lives in one fixed,
// file-scope device array.
//
// The array is kNoAllocScratchBytes (16 MiB) on every GPU that loads this
// library's device code and stays reserved until the process exits.  All
// calls share it and it keeps the contents of the last call; calls whose
// kernels overlap on the GPU (different streams, or different host threads
// on one device) race on it and must be serialised by the caller.
#include <mutex>
#include <string>

#include "../../include/mgr.h"
#include "mgr_kernels.hh"

namespace mgr {

void set_last_error(const std::string &msg);

static constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
static constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

std::mutex g_scratch_mutex;
void *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  In host code
// `g_noalloc_scratch` names a host-side stand-in, not device memory, so the
// address is looked up once per device with that device current.
cudaError_t scratch_on_current_device(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

// cubic B-spline value with unfused double operations, so the device
// rounds exactly as the reference's host code (bspline<3,0>::apply,
// mia/core/splinekernel/bspline.cc:328-345)
__device__ double b3_unfused(double x)
{
    x = fabs(x);
    if (x <= 1.0) return __dsub_rn(2.0 / 3.0, __dmul_rn(__dmul_rn(x, x), __dsub_rn(1.0, __dmul_rn(0.5, x))));
    if (x < 2.0) {
        const double dx = __dsub_rn(2.0, x);
        return __dmul_rn(__dmul_rn(__dmul_rn(dx, dx), dx), 1.0 / 6.0);
    }
    return 0.0;
}

// voxel coordinate i*scale + 1 - o as the reference's get_derivative_row
// forms it (mia/3d/transform/spline.cc:697-729)
__device__ double row_x(int i, double scale, int o)
{
    return __dsub_rn(__dadd_rn(__dmul_rn(double(i), scale), 1.0), double(o));
}

// transposed rows of one axis: per voxel the first coefficient and up to 4
// float weights, per coefficient the contiguous voxel range
__global__ void k_noalloc_rows(int n, int nc, double scale, int *as, float *aw, int *rows)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        const double c = __dadd_rn(__dmul_rn(double(t), scale), 1.0);
        const int o0 = max(0, int(floor(c)) - 2), o1 = min(nc - 1, int(floor(c)) + 2);
        int start = -1;
        float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int o = o0; o <= o1; ++o) {
            const double x = row_x(t, scale, o);
            if (fabs(x) < 2.0) {
                if (start < 0) start = o;
                const int k = o - start;
                if (k < 4) w[k] = float(b3_unfused(x));
            }
        }
        as[t] = start < 0 ? 0 : start;
        for (int k = 0; k < 4; ++k) aw[size_t(t) * 4 + k] = w[k];
    }
    if (t < nc) {
        // the voxels i with |i scale + 1 - t| < 2: x grows with i, so the
        // scan starts below the first of them and ends where x reaches 2
        int first = -1, len = 0;
        const int i0 = max(0, int(floor((double(t) - 3.0) / scale)) - 1);
        for (int i = i0; i < n; ++i) {
            const double x = row_x(i, scale, t);
            if (x >= 2.0) break;
            if (fabs(x) < 2.0) {
                if (first < 0) first = i;
                if (b3_unfused(x) > 0) ++len;
                else break;
            }
        }
        rows[2 * t] = first < 0 ? 0 : first;
        rows[2 * t + 1] = len;
    }
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

}  // namespace mgr

using namespace mgr;

extern "C" mgr_status mgr_translate3d_noalloc(const int size[3], const int csize[3], const float *d_force,
                                              double *d_grad, void *stream)
{
    if (!size || !csize || !d_force || !d_grad) {
        set_last_error("mgr_translate3d_noalloc: null argument");
        return MGR_ERR_ARG;
    }
    for (int k = 0; k < 3; ++k) {
        if (size[k] < 2 || csize[k] < 4) {
            set_last_error("mgr_translate3d_noalloc: image dimensions must be >= 2 and coefficient "
                           "dimensions >= 4");
            return MGR_ERR_ARG;
        }
    }
    const int nx = size[0], ny = size[1], nz = size[2];
    const int ncx = csize[0], ncy = csize[1], ncz = csize[2];
    // scratch layout: per axis (start, weights, rows), then the z and y pass buffers
    size_t need = 0;
    size_t off_as[3], off_aw[3], off_rows[3];
    for (int k = 0; k < 3; ++k) {
        off_as[k] = need;
        need += align256(size_t(size[k]) * sizeof(int));
        off_aw[k] = need;
        need += align256(size_t(size[k]) * 4 * sizeof(float));
        off_rows[k] = need;
        need += align256(size_t(csize[k]) * 2 * sizeof(int));
    }
    const size_t off_t1 = need;
    need += align256(size_t(ncz) * ny * nx * 3 * sizeof(float));
    const size_t off_t2 = need;
    need += align256(size_t(ncz) * ncy * nx * 3 * sizeof(float));
    if (need > kNoAllocScratchBytes) {
        set_last_error("mgr_translate3d_noalloc: this size needs " + std::to_string(need) +
                       " bytes of scratch, more than the fixed " + std::to_string(kNoAllocScratchBytes) +
                       " bytes; use mgr_level_translate instead");
        return MGR_ERR_ARG;
    }
    // an error left by earlier work of this thread is reported as such and
    // not taken for a failure of this call's launches
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("mgr_translate3d_noalloc: a CUDA error from earlier work is pending on this "
                                   "thread: ") + cudaGetErrorString(e));
        return MGR_ERR_CUDA;
    }
    void *base = nullptr;
    e = scratch_on_current_device(&base);
    if (e != cudaSuccess) {
        set_last_error(std::string("mgr_translate3d_noalloc: scratch address: ") + cudaGetErrorString(e));
        return MGR_ERR_CUDA;
    }
    unsigned char *s = static_cast<unsigned char *>(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    EvalArgs a{};
    a.dim = 3;
    a.cost_weight = 1.0;
    for (int k = 0; k < 3; ++k) {
        a.n[k] = size[k];
        a.nc[k] = csize[k];
        int *as = reinterpret_cast<int *>(s + off_as[k]);
        float *aw = reinterpret_cast<float *>(s + off_aw[k]);
        int *rows = reinterpret_cast<int *>(s + off_rows[k]);
        // every table entry is written by this kernel: nothing needs clearing
        const double scale = double(float(csize[k] - 3) / float(size[k] - 1));
        const int m = size[k] > csize[k] ? size[k] : csize[k];
        k_noalloc_rows<<<(m + 127) / 128, 128, 0, st>>>(size[k], csize[k], scale, as, aw, rows);
        count_launch();
        a.ax[k].as = as;
        a.ax[k].aw = reinterpret_cast<const float4 *>(aw);
        a.ax[k].rows = reinterpret_cast<const int2 *>(rows);
        a.ax[k].n = size[k];
        a.ax[k].nc = csize[k];
    }
    // the three separable passes assign every element of their outputs
    launch_translate(a, d_force, d_grad, reinterpret_cast<float *>(s + off_t1), reinterpret_cast<float *>(s + off_t2),
                     st);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("mgr_translate3d_noalloc: launch: ") + cudaGetErrorString(e));
        return MGR_ERR_CUDA;
    }
    (void)nz;
    (void)ncx;
    return MGR_OK;
}
