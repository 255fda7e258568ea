// prefilter.cu — cubic B-spline prefilter (causal/anticausal IIR, pole
// sqrt(3)-2, mirror boundary) and the image min/max used by the
// interpolator's clamp.  Restates T3DConvoluteInterpolator::prefilter
// (mia/3d/interpolator.cxx:98-164) with CSplineBoundaryCondition::filter_line
// (mia/core/boundary_conditions.cc:62-103) and CMirrorOnBoundary
// (mia/core/splinebc/bc.cc:67-88): x lines, then y lines, then z lines, each
// line filtered with the reference's operations (in float, see
// k_prefilter_lines) and stored back as float.
#include <cudaTypedefs.h>

#include <algorithm>
#include "mgr_common.cuh"
#include "mgr_kernels.hh"

namespace mgr {

// One block of PF_NT threads owns up to `lb` (<= 64) lines of length n,
// staged in shared memory (odd pitch) by independent coalesced loads: along
// the line for x lines, across the lines (consecutive x) for y and z lines.
// One thread per line runs the recursion, then the block stores the lines
// back the way it loaded them.  The reference filters each line in a double
// buffer; FP64 arithmetic runs at a small fraction of the FP32 rate on this
// GPU, so the recursion runs in float with the same operations: the pole's
// magnitude (0.268) damps the rounding of every step, and the result differs
// from the double filter by a few float ulp of the coefficient (the parity
// tests bound the warped image and costs, which read these coefficients, at
// 1e-5 / 1e-4).
// axis 0: lines along x (rows, consecutive rows per block);
// axis 1/2: lines along y/z (columns of consecutive x per block).
constexpr int PF_NT = 256;

__global__ void __launch_bounds__(PF_NT) k_prefilter_lines(float *__restrict__ img, int nx, int ny, int nz,
                                                           int axis, int lb)
{
    extern __shared__ float sl[];
    const int t = threadIdx.x;
    const size_t nxy = size_t(nx) * ny;
    int n, nl;
    size_t base, lstride, estride;
    if (axis == 0) {
        n = nx;
        const int l0 = blockIdx.x * lb;
        nl = min(lb, ny * nz - l0);
        base = size_t(l0) * nx;
        lstride = size_t(nx);
        estride = 1;
    } else {
        const int xb = blockIdx.x * lb;
        const int other = blockIdx.y;
        n = (axis == 1) ? ny : nz;
        base = (axis == 1) ? size_t(other) * nxy + xb : size_t(other) * nx + xb;
        lstride = 1;
        estride = (axis == 1) ? size_t(nx) : nxy;
        nl = min(lb, nx - xb);
    }
    const int pitch = n | 1;
    const bool along = axis == 0;
#pragma unroll 4
    for (int e = t; e < nl * n; e += PF_NT) {
        const int l = along ? e / n : e % nl, k = along ? e % n : e / nl;
        sl[l * pitch + k] = img[base + l * lstride + k * estride];
    }
    __syncthreads();
    if (t < nl && n >= 2) {
        float *c = sl + t * pitch;
        const float p = float(1.7320508075688772 - 2.0);   // sqrt(3) - 2
        const float lambda = float(2.0 - (1.7320508075688772 - 2.0) - 1.0 / (1.7320508075688772 - 2.0));
        for (int k = 0; k < n; ++k) c[k] *= lambda;
        // mirror initial value: sum of (p^k + p^(2n-2-k)) c[k]; the powers
        // below the float range contribute nothing
        float zn = p;
        const float iz = 1.0f / p;
        float z2n = powf(p, float(n - 1));
        float sum = c[0] + z2n * c[n - 1];
        z2n *= z2n * iz;
        for (int k = 1; k < n - 1; ++k) {
            sum += (zn + z2n) * c[k];
            zn *= p;
            z2n *= iz;
        }
        c[0] = sum / (1.0f - zn * zn);
        for (int k = 1; k < n; ++k) c[k] += p * c[k - 1];
        c[n - 1] = (p / (p * p - 1.0f)) * (p * c[n - 2] + c[n - 1]);
        for (int k = n - 2; k >= 0; --k) c[k] = p * (c[k + 1] - c[k]);
    }
    __syncthreads();
    for (int e = t; e < nl * n; e += PF_NT) {
        const int l = along ? e / n : e % nl, k = along ? e % n : e / nl;
        img[base + l * lstride + k * estride] = sl[l * pitch + k];
    }
}

// min/max of the source image with the reference's rule that the lower
// clamp bound is at most 0 (interpolator.cxx:109-112).  Per-block results
// go to `part`; the last block to finish reduces them in a fixed order.
__global__ void __launch_bounds__(256) k_minmax(const float *__restrict__ img, size_t n, float2 *part,
                                                unsigned int *counter, float *out_minmax)
{
    __shared__ float smin[256], smax[256];
    __shared__ bool last;
    float mn = INFINITY, mx = -INFINITY;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const float v = img[i];
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
    }
    smin[threadIdx.x] = mn;
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            smin[threadIdx.x] = fminf(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmaxf(smax[threadIdx.x], smax[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x] = make_float2(smin[0], smax[0]);
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        float a = INFINITY, b = -INFINITY;
        for (unsigned i = 0; i < gridDim.x; ++i) {
            const volatile float *v = reinterpret_cast<volatile float *>(part) + 2 * i;
            a = fminf(a, v[0]);
            b = fmaxf(b, v[1]);
        }
        if (0.0f < a) a = 0.0f;
        out_minmax[0] = a;
        out_minmax[1] = b;
        *counter = 0;
    }
}

// lines per block: at most 64 and 64 KB of staged lines, fewer while the
// launch would have less than two blocks per SM (the recursion of the
// block's lines is its critical path)
static int lines_per_block(int n, int lines_total, int blocks_per_line_group)
{
    int lb = 64;
    while (lb > 1 && size_t(lb) * (n | 1) * sizeof(float) > 64 * 1024) lb >>= 1;
    const int nsm = device_sm_count();
    while (lb > 8 && size_t((lines_total + lb - 1) / lb) * blocks_per_line_group < size_t(2 * nsm)) lb >>= 1;
    return lb;
}

void launch_prefilter(float *img, int dim, int nx, int ny, int nz, cudaStream_t st)
{
    if (dim == 2) nz = 1;
    // (a per-device setting: set on every call, once per level)
    cudaFuncSetAttribute(k_prefilter_lines, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    {
        const int nlines = ny * nz;
        const int lb = lines_per_block(nx, nlines, 1);
        const size_t sm = size_t(lb) * (nx | 1) * sizeof(float);
        k_prefilter_lines<<<(nlines + lb - 1) / lb, PF_NT, sm, st>>>(img, nx, ny, nz, 0, lb);
        count_launch();
    }
    {
        const int lb = lines_per_block(ny, nx, nz);
        const size_t sm = size_t(lb) * (ny | 1) * sizeof(float);
        k_prefilter_lines<<<dim3((nx + lb - 1) / lb, nz), PF_NT, sm, st>>>(img, nx, ny, nz, 1, lb);
        count_launch();
    }
    if (dim == 3 && nz > 1) {
        const int lb = lines_per_block(nz, nx, ny);
        const size_t sm = size_t(lb) * (nz | 1) * sizeof(float);
        k_prefilter_lines<<<dim3((nx + lb - 1) / lb, ny), PF_NT, sm, st>>>(img, nx, ny, nz, 2, lb);
        count_launch();
    }
}

__global__ void k_pad_mirror(const float *__restrict__ img, float *__restrict__ pad, int nx, int ny, int nz,
                             int pitch, int rows, int hz, size_t total)
{
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
        const int px = int(i % pitch);
        const size_t r = i / pitch;
        const int py = int(r % rows), pz = int(r / rows);
        const int x = px - PAD_H, y = py - PAD_H, z = pz - hz;
        float v = 0.0f;
        if (x < nx + PAD_H) {
            const int gx = mirror_fold(x, nx), gy = mirror_fold(y, ny), gz = mirror_fold(z, nz);
            v = img[(size_t(gz) * ny + gy) * nx + gx];
        }
        pad[i] = v;
    }
}

bool encode_pad_tmap(CUtensorMap *map, const float *pad, int nx, int ny, int nz)
{
    // resolved once, thread-safe (levels are made on several host threads)
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        return PFN_cuTensorMapEncodeTiled_v12000(nullptr);
    }();
    if (!fn) return false;
    const int P = pad_pitch(nx);
    const cuuint64_t dims[3] = {cuuint64_t(P), cuuint64_t(ny + 2 * PAD_H), cuuint64_t(nz + 2 * PAD_H)};
    const cuuint64_t strides[2] = {cuuint64_t(P) * 4, cuuint64_t(P) * (ny + 2 * PAD_H) * 4};
    const cuuint32_t box[3] = {64, 16, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(pad), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t pad_floats(int dim, int nx, int ny, int nz)
{
    const int planes = dim == 3 ? nz + 2 * PAD_H : 1;
    return size_t(pad_pitch(nx)) * (ny + 2 * PAD_H) * planes;
}

void launch_pad_mirror(const float *img, float *pad, int dim, int nx, int ny, int nz, cudaStream_t st)
{
    if (dim == 2) nz = 1;
    const size_t total = pad_floats(dim, nx, ny, nz);
    const int nb = int(std::min<size_t>(4096, (total + 255) / 256));
    k_pad_mirror<<<nb, 256, 0, st>>>(img, pad, nx, ny, nz, pad_pitch(nx), ny + 2 * PAD_H, dim == 3 ? PAD_H : 0,
                                     total);
    count_launch();
}

void launch_minmax(const float *img, size_t n, float2 *part, int nblocks, unsigned int *counter,
                   float *out, cudaStream_t st)
{
    k_minmax<<<nblocks, 256, 0, st>>>(img, n, part, counter, out);
    count_launch();
}

}  // namespace mgr
