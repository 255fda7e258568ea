// mgr_common.cuh — device helpers shared by the 2D and 3D kernels of
// libmgr (B-spline registration cost+gradient on sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mgr {

// ---------------------------------------------------------------------
// cubic B-spline arithmetic
// ---------------------------------------------------------------------

// Start index of the 4-tap window of a coordinate, with the reference's
// fixed-point floor: the coordinate is rounded to the nearest multiple of
// 2^-16 (ties to even) before flooring (mia/core/splinekernel.cc:164-192,
// 250-255).  For a float coordinate, x*65536 is exact and rint() rounds it
// exactly as the reference's 1.5*2^36 double trick does.
__device__ __forceinline__ int ffloor16(float x)
{
    return __float2int_rn(x * 65536.0f) >> 16;
}

// Cubic B-spline weights at fractional offset f, in the reference's
// evaluation order (mia/core/splinekernel/bspline.cc:258-285).
__device__ __forceinline__ void bspline3_weights(float f, float w[4])
{
    const float ob6 = 1.0f / 6.0f;
    const float xm1 = 1.0f - f;
    const float w0 = (xm1 * xm1) * (xm1 * ob6);
    const float w3 = (f * f) * (f * ob6);
    w[0] = w0;
    w[3] = w3;
    w[1] = ((xm1 - w0) - w0) + w3;
    w[2] = ((f - w3) - w3) + w0;
}

// Mirror halo of the padded copy of the prefiltered moving image that the
// split path's warp kernel stages from (voxels per side; the padded rows are
// 128-byte aligned so that any 16-byte aligned row segment can be copied
// with one bulk copy).
constexpr int PAD_H = 16;

__host__ __device__ inline int pad_pitch(int nx)
{
    return ((nx + 2 * PAD_H + 31) / 32) * 32;
}

// Shared-memory box in which the warp kernel stages the moving image's tap
// footprint of one tile: rows of stage_bx floats (a multiple of 32, so that
// the bank of a tap depends only on its x position and lanes on different
// rows do not conflict), stage_by rows per plane, stage_bz planes.  A tile
// whose footprint does not fit reads its taps from global memory.
__host__ __device__ constexpr int stage_bx(int tx)
{
    return ((tx + 24 + 31) / 32) * 32;
}
__host__ __device__ constexpr int stage_by(int ty)
{
    return ty + 10;
}
__host__ __device__ constexpr int stage_bz(int dim, int tz)
{
    return dim == 3 ? tz + 10 : 1;
}
__host__ __device__ constexpr int stage_floats(int dim, int tx, int ty, int tz)
{
    return stage_bx(tx) * stage_by(ty) * stage_bz(dim, tz);
}

// Mirror boundary index folding with period 2w-2
// (mia/core/splinebc/bc.cc:52-64).
__device__ __forceinline__ int mirror_fold(int i, int w)
{
    const int w2 = 2 * w - 2;
    int idx = i < 0 ? -i : i;
    idx = (w == 1) ? 0 : ((idx < w2) ? idx : idx % w2);
    if (w <= idx) idx = w2 - idx;
    return idx;
}

// clamp to [mn, mx] with the reference's comparison order
// (bounded<>, mia/3d/interpolator.cxx:177-185)
__device__ __forceinline__ float clamp_ref(float r, float mn, float mx)
{
    return (r >= mn) ? ((r <= mx) ? r : mx) : mn;
}

// Tricubic B-spline interpolation of a prefiltered volume at p, mirror BC.
__device__ __forceinline__ float sample3(const float *__restrict__ c, int nx, int ny, int nz,
                                         float px, float py, float pz, float mn, float mx)
{
    const int fx = ffloor16(px), fy = ffloor16(py), fz = ffloor16(pz);
    float wx[4], wy[4], wz[4];
    bspline3_weights(px - float(fx), wx);
    bspline3_weights(py - float(fy), wy);
    bspline3_weights(pz - float(fz), wz);
    int ix[4], iy[4], iz[4];
    const int sx = fx - 1, sy = fy - 1, sz = fz - 1;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        ix[k] = sx + k;
        iy[k] = sy + k;
        iz[k] = sz + k;
    }
    // the mirror fold runs only near the border (a real branch, so the
    // interior path does not pay for the modulo)
    if (sx < 0 || sx + 3 >= nx) {
#pragma unroll
        for (int k = 0; k < 4; ++k) ix[k] = mirror_fold(ix[k], nx);
    }
    if (sy < 0 || sy + 3 >= ny) {
#pragma unroll
        for (int k = 0; k < 4; ++k) iy[k] = mirror_fold(iy[k], ny);
    }
    if (sz < 0 || sz + 3 >= nz) {
#pragma unroll
        for (int k = 0; k < 4; ++k) iz[k] = mirror_fold(iz[k], nz);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) iy[k] *= nx;
    const size_t nxy = size_t(nx) * ny;
    float acc = 0.0f;
#pragma unroll
    for (int kz = 0; kz < 4; ++kz) {
        const float *__restrict__ pl = c + size_t(iz[kz]) * nxy;
        float ay = 0.0f;
#pragma unroll
        for (int ky = 0; ky < 4; ++ky) {
            const float *__restrict__ row = pl + iy[ky];
            const float r = wx[0] * __ldg(row + ix[0]) + wx[1] * __ldg(row + ix[1]) +
                            wx[2] * __ldg(row + ix[2]) + wx[3] * __ldg(row + ix[3]);
            ay += wy[ky] * r;
        }
        acc += wz[kz] * ay;
    }
    return clamp_ref(acc, mn, mx);
}

// Bicubic variant (mia/2d/interpolator.cxx:216-311).
__device__ __forceinline__ float sample2(const float *__restrict__ c, int nx, int ny, float px,
                                         float py, float mn, float mx)
{
    const int fx = ffloor16(px), fy = ffloor16(py);
    float wx[4], wy[4];
    bspline3_weights(px - float(fx), wx);
    bspline3_weights(py - float(fy), wy);
    int ix[4], iy[4];
    const int sx = fx - 1, sy = fy - 1;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        ix[k] = sx + k;
        iy[k] = sy + k;
    }
    if (sx < 0 || sx + 3 >= nx) {
#pragma unroll
        for (int k = 0; k < 4; ++k) ix[k] = mirror_fold(ix[k], nx);
    }
    if (sy < 0 || sy + 3 >= ny) {
#pragma unroll
        for (int k = 0; k < 4; ++k) iy[k] = mirror_fold(iy[k], ny);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) iy[k] *= nx;
    float acc = 0.0f;
#pragma unroll
    for (int ky = 0; ky < 4; ++ky) {
        const float *__restrict__ row = c + iy[ky];
        const float r = wx[0] * __ldg(row + ix[0]) + wx[1] * __ldg(row + ix[1]) +
                        wx[2] * __ldg(row + ix[2]) + wx[3] * __ldg(row + ix[3]);
        acc += wy[ky] * r;
    }
    return clamp_ref(acc, mn, mx);
}

// Tricubic / bicubic sample from a shared-memory footprint of the
// prefiltered image whose elements already hold the mirror-folded values:
// `base` points at the first tap (fx-1, fy-1, fz-1) and rows / planes are
// `sy` / `sz` floats apart.  Same weights and summation order as sample3 /
// sample2.
__device__ __forceinline__ float staged_sample3(const float *base, int sy, int sz, float px, float py, float pz,
                                                int fx, int fy, int fz, float mn, float mx)
{
    float wx[4], wy[4], wz[4];
    bspline3_weights(px - float(fx), wx);
    bspline3_weights(py - float(fy), wy);
    bspline3_weights(pz - float(fz), wz);
    float acc = 0.0f;
#pragma unroll
    for (int kz = 0; kz < 4; ++kz) {
        const float *pl = base + kz * sz;
        float ay = 0.0f;
#pragma unroll
        for (int ky = 0; ky < 4; ++ky) {
            const float *row = pl + ky * sy;
            const float r = wx[0] * row[0] + wx[1] * row[1] + wx[2] * row[2] + wx[3] * row[3];
            ay += wy[ky] * r;
        }
        acc += wz[kz] * ay;
    }
    return clamp_ref(acc, mn, mx);
}

__device__ __forceinline__ float staged_sample2(const float *base, int sy, float px, float py, int fx, int fy,
                                                float mn, float mx)
{
    float wx[4], wy[4];
    bspline3_weights(px - float(fx), wx);
    bspline3_weights(py - float(fy), wy);
    float acc = 0.0f;
#pragma unroll
    for (int ky = 0; ky < 4; ++ky) {
        const float *row = base + ky * sy;
        const float r = wx[0] * row[0] + wx[1] * row[1] + wx[2] * row[2] + wx[3] * row[3];
        acc += wy[ky] * r;
    }
    return clamp_ref(acc, mn, mx);
}

// ---------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of K doubles per thread into red[0..K-1] (thread 0 holds
// the result after the final __syncthreads).  `scratch` holds
// K * (blockDim.x/32) doubles.  Order is fixed, so the result is
// reproducible from run to run.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double *scratch)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) scratch[k * nw + wid] = v[k];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = lane < nw ? scratch[k * nw + lane] : 0.0;
            s = warp_sum(s);
            v[k] = s;
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------
// per-axis tables (built on the host, see tables.cc)
// ---------------------------------------------------------------------
struct Axis {
    const int *fs;      // forward start index per voxel coordinate
    const float4 *fw;   // forward weights (4th zero on the last voxel)
    const int *as;      // adjoint start per voxel coordinate
    const float4 *aw;   // adjoint weights (float rows of translate)
    const int2 *rows;   // per coefficient: voxel range [first, first+len)
    const int *ftile0;  // per tile: first coefficient of the forward footprint
    const int *atile0;  // per tile: first coefficient of the adjoint footprint
    const int2 *gtile;  // per coefficient: tiles [lo, hi] whose adjoint footprint holds it
    const int *glist;   // 3D, per coefficient: GATHER_LMAX offsets into the partial slots, this axis' part
    const int *glen;    // 3D, per coefficient: entries of glist (-1: longer than GATHER_LMAX)
    int n;              // voxels
    int nc;             // coefficients
    int t;              // tile length (voxels)
    int nt;             // number of tiles
    int fc;             // forward footprint length (max over tiles)
    int ac;             // adjoint footprint length (max over tiles)
};

// longest per-axis list of tiles whose adjoint footprint holds a coefficient
// that the 3D gather reads from the tables (longer lists take a slower path)
constexpr int GATHER_LMAX = 24;
// planes of the 3D warp kernel's shared-memory tap ring (split3.cu); the
// tile-fit rule (mgr_level::tile_fits) counts them.  12 keeps three warp
// blocks per SM at the usual spacings (14 measured slower: 2 blocks per SM
// at rate 5)
#ifndef MGR_RING_PLANES
#define MGR_RING_PLANES 12
#endif
constexpr int WARP_RING_PLANES = MGR_RING_PLANES;

// scalars written by the cost finalisation (double[16])
enum {
    SC_VALUE = 0,      // image cost value() (unweighted), NCC with the 1e-10 threshold
    SC_FORCE_COST = 1, // force-pass cost (2D full cost returns this)
    SC_K1 = 2,         // NCC: 2*cov/(var_a*var_b)  (gradient helper, 1e-5 threshold)
    SC_K2 = 3,         // NCC: cov/var_a
    SC_MA = 4,         // NCC: mean of the warped image
    SC_MB = 5,         // NCC: mean of the reference
    SC_FSCALE = 6,     // SSD: force scale (1/N with norm, else 1)
    SC_PEN = 7,        // penalty value (unweighted)
    SC_COST_IMG = 8,   // weighted image cost
    SC_COST_PEN = 9,   // weighted penalty cost
    SC_NSLOTS = 16
};

}  // namespace mgr
