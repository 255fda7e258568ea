// warp3_common.cuh — device helpers of the 3D warp kernels (split3.cu,
// fused3.cu): the tricubic tap sum from global memory and from the shared-
// memory ring of tap planes that bulk tensor copies fill, and the bounded
// mbarrier wait.
#pragma once

#include "mgr_common.cuh"

namespace mgr {
namespace {

// Tricubic sample at (px, py, pz) read from global memory: the taps come
// from the mirror-padded copy coef_pad while they lie inside it, else the
// indices are folded on the unpadded image (sample3).  Same weights and
// summation order as sample3.  This is the path of voxels whose taps are
// not in the shared-memory ring below.
__device__ __noinline__ float taps3_global(const EvalArgs &a, float px, float py, float pz, float mn, float mx)
{
    const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
    const int fx = ffloor16(px), fy = ffloor16(py), fz = ffloor16(pz);
    const int sx = fx - 1, sy = fy - 1, sz = fz - 1;
    constexpr int H = PAD_H;
    if (sx >= -H && sx + 3 < nx + H && sy >= -H && sy + 3 < ny + H && sz >= -H && sz + 3 < nz + H) {
        float wx[4], wy[4], wz[4];
        bspline3_weights(px - float(fx), wx);
        bspline3_weights(py - float(fy), wy);
        bspline3_weights(pz - float(fz), wz);
        const int P = pad_pitch(nx);
        const size_t PL = size_t(P) * a.pad_rows;
        const float *__restrict__ b = a.coef_pad + (size_t(sz + H) * a.pad_rows + (sy + H)) * P + (sx + H);
        float acc = 0.0f;
#pragma unroll
        for (int kz = 0; kz < 4; ++kz) {
            float ay = 0.0f;
#pragma unroll
            for (int ky = 0; ky < 4; ++ky) {
                const float *__restrict__ row = b + kz * PL + ky * P;
                const float r = wx[0] * __ldg(row) + wx[1] * __ldg(row + 1) + wx[2] * __ldg(row + 2) +
                                wx[3] * __ldg(row + 3);
                ay += wy[ky] * r;
            }
            acc += wz[kz] * ay;
        }
        return clamp_ref(acc, mn, mx);
    }
    return sample3(a.coef_img, nx, ny, nz, px, py, pz, mn, mx);
}

// Shared-memory ring of tap planes of the 3D warp kernel: RING_N planes of
// RING_Y rows of RING_X floats (a row holds the x extent of a tile's taps
// plus the alignment of the copies; its pitch is a multiple of the 32
// banks, so a warp whose lanes straddle two rows or planes reads without
// bank conflicts).  A tile whose taps do not fit (large variation of the
// displacement over the tile) reads them from global memory instead.
constexpr int RING_N = WARP_RING_PLANES;
constexpr int RING_Y = 16;
constexpr int RING_X = 64;
constexpr int RING_PLANE = RING_Y * RING_X;

__device__ __forceinline__ int ring_slot(int k)
{
    return k % RING_N;
}

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Bounded wait on phase `parity` of an mbarrier: false after LIMIT tries
// (the copy engine did not deliver), so that no wait is endless.
template <int LIMIT = (1 << 20)>
__device__ __forceinline__ bool mbar_wait(unsigned mb, unsigned parity)
{
    for (int it = 0; it < LIMIT; ++it) {
        unsigned done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(mb), "r"(parity)
                     : "memory");
        if (done) return true;
    }
    return false;
}

// Tricubic sample from the ring: `row`/`col` locate the first tap inside a
// plane and `slot0` is the ring slot of the first tap plane; the weights and
// the summation order are those of sample3.
__device__ __forceinline__ float taps3_ring(const float *ring, int slot0, int row, int col, float fx, float fy,
                                           float fz, float mn, float mx)
{
    float wx[4], wy[4], wz[4];
    bspline3_weights(fx, wx);
    bspline3_weights(fy, wy);
    bspline3_weights(fz, wz);
    const float *base = ring + row * RING_X + col;
    float acc = 0.0f;
#pragma unroll
    for (int kz = 0; kz < 4; ++kz) {
        int sl = slot0 + kz;
        sl = sl >= RING_N ? sl - RING_N : sl;
        const float *pl = base + sl * RING_PLANE;
        float ay = 0.0f;
#pragma unroll
        for (int ky = 0; ky < 4; ++ky) {
            const float *r = pl + ky * RING_X;
            ay += wy[ky] * (wx[0] * r[0] + wx[1] * r[1] + wx[2] * r[2] + wx[3] * r[3]);
        }
        acc += wz[kz] * ay;
    }
    return clamp_ref(acc, mn, mx);
}


}  // namespace
}  // namespace mgr
