// fused3.cu — the 3D SSD evaluation with the warp and the adjoint fused:
// one pass per tile computes the warped image, the central-difference
// gradient and the force, and contracts the force onto the tile's adjoint
// footprint (MGR_PATH_FUSED).
//
// The reference's chain is warp, evaluate_force, translate
// (C3DImageFullCost::do_evaluate, mia/3d/fullcost/image.cc:67-78): the force
// at a voxel is the SSD residual times the central differences of the
// warped image (mia/template/ssd.hh:126-181, mia/3d/image.cc:347-466), so a
// voxel's force needs the warped values of its six face neighbours.  A
// block computes them itself: its 320 threads sample the warped image on
// 32 x 10 columns (x0-1 .. x0+30, y0-1 .. y0+8) and walk the planes
// z0-1 .. z0+TZ; the forces of the 30 x 8 x TZ interior voxels follow one
// plane behind the walk (x neighbours by warp shuffle, y neighbours from
// the rows of the last three planes in shared memory, z neighbours held in
// registers).  The sampling (displacement from the coefficient footprint,
// tricubic taps from the ring of tap planes that bulk tensor copies fill)
// and the contraction (z while walking, then y and x in shared memory into
// the tile's partial slot, summed per coefficient by the gather kernel)
// are those of the split kernels.  The halo costs 32 * 10 * (TZ + 2)
// samples for 30 * 8 * TZ voxels; in exchange the warped image is neither
// written nor read back, the reference is read once and one launch goes.
//
// SSD only: the NCC force at a voxel is scaled by constants of the whole
// image's sums (mia/3d/cost/ncc.cc:88-128), which a single pass only knows
// when every tile has finished.
#include <algorithm>
#include <string>

#include "../../include/mgr.h"
#include "mgr_cost.cuh"
#include "warp3_common.cuh"

namespace mgr {

namespace {

constexpr int FWARPS = 10;            // rows y0-1 .. y0+8
constexpr int NTF = FWARPS * 32;      // threads per block
constexpr int FTX = 30;               // interior voxels of a row: lanes 1..30
constexpr int FTY = 8;                // interior rows: warps 1..8
constexpr unsigned FFULL = 0xffffffffu;

}  // namespace

size_t fused3_smem(const EvalArgs &a);

template <int TZ>
__device__ __forceinline__ void fused3_body(const EvalArgs &a, int bx, int by, int bz, int ntiles, int tile,
                                            int with_gradient)
{
    extern __shared__ __align__(16) float smf[];
    __shared__ double red[5 * FWARPS];
    __shared__ float wsum[FWARPS];
    __shared__ int zs[TZ + 2];
    __shared__ float4 zw[TZ + 2];
    __shared__ float urng[FWARPS][6];
    __shared__ int boxs[8];
    __shared__ __align__(8) unsigned long long mbar[RING_N];
    __shared__ int nissued;
    __shared__ volatile int ring_failed;
    __shared__ bool is_last;
    __shared__ int asx[FTX], asy[FTY], azs[TZ];
    __shared__ float4 awx[FTX], awy[FTY], azw[TZ];
    __shared__ float Wp[3][FWARPS][32];   // warped rows of the last three walked planes

    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
    const int ncx = a.nc[0], ncy = a.nc[1], ncz = a.nc[2];
    const int x0 = bx * FTX, y0 = by * FTY, z0 = bz * TZ;
    const int tid = threadIdx.x, lane = tid & 31, wy = tid >> 5;
    // this thread's sample column (clamped into the image where the halo
    // leaves it: those samples are computed but never used)
    const int xs = x0 - 1 + lane, ys = y0 - 1 + wy;
    const int xc = min(max(xs, 0), nx - 1), yc = min(max(ys, 0), ny - 1);
    // walked planes zlo .. zhi, interior planes z0 .. zi1
    const int zlo = max(z0 - 1, 0), zi1 = min(z0 + TZ, nz) - 1, zhi = min(z0 + TZ, nz - 1);
    const int nwalk = zhi - zlo + 1;
    const bool interior = lane >= 1 && lane <= FTX && xs < nx && wy >= 1 && wy <= FTY && ys < ny;
    const int ex = min(FTX, nx - x0), ey = min(FTY, ny - y0);
    // the forward footprint of the sample box: each halo column, row or
    // plane reaches at most one coefficient beyond the tile's (spacing >= 1)
    const int cx0 = X.fs[max(x0 - 1, 0)], cy0 = Y.fs[max(y0 - 1, 0)], cz0 = Z.fs[zlo];
    const int FX = X.fc + 2, FY = Y.fc + 2, FZ = Z.fc + 2;
    const int AXc = X.ac, AYc = Y.ac, AZc = Z.ac;
    const int ax0 = X.atile0[bx], ay0 = Y.atile0[by], az0 = Z.atile0[bz];
    const int fsx = X.fs[xc], fsy = Y.fs[yc];
    const float4 fwx = X.fw[xc], wyv = Y.fw[yc];
    const float mn = a.minmax[0], mxv = a.minmax[1];
    const size_t N = size_t(nx) * ny * nz;
    const float fscale = a.ssd_norm ? float(1.0 / double(N)) : 1.0f;

    // shared memory: Az (the z-contracted forces, written during the walk),
    // then the walk's coefficient footprint, x stage and tap ring, which the
    // y stage's Ay reuses after the walk
    float *Az = smf;                                  // [3][AZc][FTY][32]
    float *C = Az + 3 * AZc * FTY * 32;               // [3][FZ][FY][FX]
    float *Tx = C + 3 * FZ * FY * FX;                 // [3][FZ][FY][32]
    float *ring;
    {
        const int off = 3 * AZc * FTY * 32 + 3 * FZ * FY * (FX + 32);
        const unsigned ra = smem_u32(smf + off);
        ring = smf + off + ((((ra + 127u) & ~127u) - ra) >> 2);
    }
    float *Ay = C;                                    // [3][AZc][AYc][33], after the walk

    if (tid < TZ + 2) {
        const int z = min(zlo + tid, zhi);
        zs[tid] = Z.fs[z] - cz0;
        zw[tid] = Z.fw[z];
    }
    if (tid < FTX) {
        const int xx = min(x0 + tid, nx - 1);
        asx[tid] = X.as[xx] - ax0;
        awx[tid] = X.aw[xx];
    }
    if (tid < FTY) {
        const int yy = min(y0 + tid, ny - 1);
        asy[tid] = Y.as[yy] - ay0;
        awy[tid] = Y.aw[yy];
    }
    if (tid < TZ) {
        const int zz = min(z0 + tid, nz - 1);
        azs[tid] = Z.as[zz] - az0;
        azw[tid] = Z.aw[zz];
    }
    // coefficient footprint: rows (iz, iy) of 3 FX consecutive floats
    {
        const int w3 = 3 * FX, nel = FZ * FY * w3;
        for (int e = tid; e < nel; e += NTF) {
            const int r = e / w3, j = e - r * w3;
            const int ix = j / 3, c = j - 3 * ix;
            const int iz = r / FY, iy = r - iz * FY;
            float v = 0.0f;
            if (cx0 + ix < ncx && cy0 + iy < ncy && cz0 + iz < ncz)
                v = a.params_f[((size_t(cz0 + iz) * ncy + (cy0 + iy)) * ncx + cx0) * 3 + j];
            C[(c * FZ * FY + r) * FX + ix] = v;
        }
    }
    __syncthreads();
    // x stage: Tx[c][kz][jy][lane]
    {
        const int sx = fsx - cx0;
        for (int r = wy; r < 3 * FZ * FY; r += FWARPS) {
            const float *c = C + r * FX + sx;
            Tx[r * 32 + lane] = fwx.x * c[0] + fwx.y * c[1] + fwx.z * c[2] + fwx.w * c[3];
        }
        if (tid == 0) {
            for (int k = 0; k < RING_N; ++k)
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[k])) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        }
    }
    __syncthreads();
    const int sy = fsy - cy0;
    auto qat = [&](int c, int kz) {
        const float *t = Tx + ((c * FZ + kz) * FY + sy) * 32 + lane;
        return wyv.x * t[0] + wyv.y * t[32] + wyv.z * t[64] + wyv.w * t[96];
    };
    float q[3][4];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int m = 0; m < 4; ++m) q[c][m] = qat(c, m);
    int cur = 0;
    auto advance = [&](int t) {
        const int s = zs[t];
        while (cur < s) {
            ++cur;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                q[c][0] = q[c][1];
                q[c][1] = q[c][2];
                q[c][2] = q[c][3];
                q[c][3] = qat(c, cur + 3);
            }
        }
    };
    {
        // the range of u over the samples of the block (convex combinations
        // of this thread's q values; 0 joins it on the image's last plane)
        float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        const int kend = zs[nwalk - 1] + 3;
        for (int kz = 0; kz <= kend; ++kz)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float v = qat(c, kz);
                lo[c] = fminf(lo[c], v);
                hi[c] = fmaxf(hi[c], v);
            }
        const bool last_plane = zhi == nz - 1;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (last_plane) {
                lo[c] = fminf(lo[c], 0.0f);
                hi[c] = fmaxf(hi[c], 0.0f);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo[c] = fminf(lo[c], __shfl_xor_sync(FFULL, lo[c], o));
                hi[c] = fmaxf(hi[c], __shfl_xor_sync(FFULL, hi[c], o));
            }
        }
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                urng[wy][c] = lo[c];
                urng[wy][3 + c] = hi[c];
            }
    }
    __syncthreads();
    constexpr int H = PAD_H;
    auto issue_plane = [&](int k) {   // thread 0: plane k of the box into its ring slot
        const int slot = ring_slot(k);
        const unsigned mb = smem_u32(&mbar[slot]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb),
                     "r"(unsigned(RING_PLANE) * 4u)
                     : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];\n" ::"r"(smem_u32(ring + slot * RING_PLANE)),
            "l"(reinterpret_cast<unsigned long long>(&a.tmap)), "r"(boxs[1] + H), "r"(boxs[2] + H), "r"(boxs[3] + k + H),
            "r"(mb)
            : "memory");
    };
    if (tid == 0) {
        float ulo[3], uhi[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            ulo[c] = urng[0][c];
            uhi[c] = urng[0][3 + c];
            for (int w = 1; w < FWARPS; ++w) {
                ulo[c] = fminf(ulo[c], urng[w][c]);
                uhi[c] = fmaxf(uhi[c], urng[w][3 + c]);
            }
        }
        // the sample box: columns max(x0-1,0) .. min(x0+30,nx-1), rows
        // max(y0-1,0) .. min(y0+8,ny-1), planes zlo .. zhi
        const int sxl = max(x0 - 1, 0), sxh = min(x0 + 30, nx - 1);
        const int syl = max(y0 - 1, 0), syh = min(y0 + 8, ny - 1);
        const float big = 1.0e6f;
        bool ok = a.has_tmap != 0 && *(volatile unsigned *)&a.counters[6] == 0u;
#pragma unroll
        for (int c = 0; c < 3; ++c) ok = ok && fabsf(ulo[c]) < big && fabsf(uhi[c]) < big;
        int bxs = 0, xe = 0, ylo = 0, yhi = 0, dzl = 0, dzh = 0;
        if (ok) {
            const int xlo = int(floorf(float(sxl) - uhi[0])) - 1;
            xe = int(floorf(float(sxh) - ulo[0])) + 3;
            bxs = ((xlo + H) & ~3) - H;
            ylo = int(floorf(float(syl) - uhi[1])) - 1;
            yhi = int(floorf(float(syh) - ulo[1])) + 3;
            dzl = int(floorf(-uhi[2])) - 1;
            dzh = int(floorf(-ulo[2])) + 3;
            ok = bxs >= -H && xe <= nx + H - 1 && xe - bxs + 1 <= RING_X && ylo >= -H && yhi <= ny + H - 1 &&
                 yhi - ylo + 1 <= RING_Y && zlo + dzl >= -H && zhi + dzh <= nz + H - 1 &&
                 dzh - dzl + 1 <= RING_N - 2;
        }
        boxs[0] = ok;
        boxs[1] = bxs;
        boxs[2] = ylo;
        boxs[3] = zlo + dzl;
        boxs[4] = nwalk + dzh - dzl;
        boxs[5] = dzh - dzl + 1;
        boxs[6] = RING_X;
        boxs[7] = yhi - ylo + 1;
        nissued = 0;
        ring_failed = 0;
        if (ok) {
            for (int k = 0; k < min(boxs[4], RING_N); ++k) issue_plane(k);
            nissued = min(boxs[4], RING_N);
        }
    }
    __syncthreads();

    const float px0 = float(xc), py0 = float(yc);
    const size_t nxy = size_t(nx) * ny;
    const float *rin = a.ref + size_t(min(ys, ny - 1)) * nx + min(xs, nx - 1);
    const bool staged = boxs[0] != 0;
    const int bx0 = boxs[1], bylo = boxs[2], bzbase = boxs[3], nplanes = boxs[4], span = boxs[5];
    const int bw4 = boxs[6], brows = boxs[7];
    bool ring_ok = staged;
    int kwait = 0;
    // force state: warped values of the planes below / at / above the one
    // whose force comes next, the reference there, the z running sums
    float wprev = 0.0f, wcur = 0.0f, rcur = 0.0f, ssd = 0.0f;
    float acc[3][4];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[c][k] = 0.0f;
    int acur = 0;   // azs[0] == 0
    auto emit = [&](int kz, int c, float v) {
        if (interior) Az[((c * AZc + kz) * FTY + (wy - 1)) * 32 + (lane - 1)] = v;
    };
    // the force of plane zf (interior, uniform over the block) from the
    // warped values below (wb), at (wc) and above (wa) this column
    auto force_plane = [&](int zf, float wb, float wc, float wa, float b) {
        const int slot = (zf - zlo) % 3;
        float left = __shfl_up_sync(FFULL, wc, 1), right = __shfl_down_sync(FFULL, wc, 1);
        float f[3] = {0.0f, 0.0f, 0.0f};
        if (interior) {
            float g[3];
            g[0] = (xs > 0 && xs < nx - 1) ? 0.5f * (right - left) : 0.0f;
            g[1] = (ys > 0 && ys < ny - 1) ? 0.5f * (Wp[slot][wy + 1][lane] - Wp[slot][wy - 1][lane]) : 0.0f;
            g[2] = (zf > 0 && zf < nz - 1) ? 0.5f * (wa - wb) : 0.0f;
            const float d = wc - b;
            ssd += d * d;
#pragma unroll
            for (int k = 0; k < 3; ++k) f[k] = (g[k] * d) * fscale;
        }
        if (!with_gradient) return;
        const int t = zf - z0;
        const int s = azs[t];
        while (acur < s) {   // uniform over the block
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                emit(acur, c, acc[c][0]);
                acc[c][0] = acc[c][1];
                acc[c][1] = acc[c][2];
                acc[c][2] = acc[c][3];
                acc[c][3] = 0.0f;
            }
            ++acur;
        }
        const float4 w = azw[t];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            acc[c][0] += w.x * f[c];
            acc[c][1] += w.y * f[c];
            acc[c][2] += w.z * f[c];
            acc[c][3] += w.w * f[c];
        }
    };

    for (int t = 0; t < nwalk; ++t) {
        const int zp = zlo + t;
        // the reference of this plane, for the force one step later
        const float rpre = (interior && zp >= z0 && zp <= zi1) ? __ldg(rin + size_t(zp) * nxy) : 0.0f;
        advance(t);
        if (ring_ok) {
            while (kwait <= t + span - 1) {
                if (ring_failed || !mbar_wait(smem_u32(&mbar[ring_slot(kwait)]), unsigned(kwait / RING_N) & 1u)) {
                    if (!ring_failed) {
                        ring_failed = 1;
                        atomicOr(&a.counters[6], 1u);
                    }
                    ring_ok = false;
                    break;
                }
                ++kwait;
            }
        }
        const float4 wz = zw[t];
        float u[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) u[c] = wz.x * q[c][0] + wz.y * q[c][1] + wz.z * q[c][2] + wz.w * q[c][3];
        const float px = px0 - u[0], py = py0 - u[1], pz = float(zp) - u[2];
        const int fx = ffloor16(px), fy = ffloor16(py), fz = ffloor16(pz);
        const int col = fx - 1 - bx0, row = fy - 1 - bylo, kk = fz - 1 - bzbase;
        float wv;
        if (ring_ok && col >= 0 && col + 3 < bw4 && row >= 0 && row + 3 < brows && kk >= t && kk + 3 <= t + span - 1)
            wv = taps3_ring(ring, ring_slot(kk), row, col, px - float(fx), py - float(fy), pz - float(fz), mn, mxv);
        else
            wv = taps3_global(a, px, py, pz, mn, mxv);
        Wp[t % 3][wy][lane] = wv;
        __syncthreads();   // the plane's rows are written; every warp is done with ring plane t
        if (staged && tid == 0 && t + RING_N < nplanes && !ring_failed && ring_ok) {
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            issue_plane(t + RING_N);
            ++nissued;
        }
        if (t > 0 && zp - 1 >= z0) force_plane(zp - 1, wprev, wcur, wv, rcur);
        wprev = wcur;
        wcur = wv;
        rcur = rpre;
    }
    // the last interior plane when it is the image's last plane (no plane
    // above it: its z difference is zero)
    if (zhi == zi1) force_plane(zhi, wprev, wcur, 0.0f, rcur);
    if (staged && tid == 0) {
        const int issued = nissued;
        while (kwait < issued) {
            if (!mbar_wait(smem_u32(&mbar[ring_slot(kwait)]), unsigned(kwait / RING_N) & 1u)) {
                atomicOr(&a.counters[6], 1u);
                break;
            }
            ++kwait;
        }
    }
    // tile sum of the interior voxels' squared residuals: a float tree per
    // warp, the warps in double in a fixed order
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ssd += __shfl_xor_sync(FFULL, ssd, o);
    if (lane == 0) wsum[wy] = ssd;
    // the remaining z running sums
    if (with_gradient) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (acur + k < AZc)
#pragma unroll
                for (int c = 0; c < 3; ++c) emit(acur + k, c, acc[c][k]);
        for (int kz = acur + 4; kz < AZc; ++kz)
#pragma unroll
            for (int c = 0; c < 3; ++c) emit(kz, c, 0.0f);
    }
    __syncthreads();   // Az complete; the walk's shared memory is free for Ay
    if (tid == 0) {
        double v = 0.0;
        for (int w = 0; w < FWARPS; ++w) v += double(wsum[w]);
        a.tile_sums[size_t(tile) * 5] = v;
        for (int k = 1; k < 5; ++k) a.tile_sums[size_t(tile) * 5 + k] = 0.0;
        __threadfence();
        is_last = (atomicAdd(&a.counters[0], 1u) == unsigned(ntiles - 1));
    }
    if (with_gradient) {
        float *part = a.partial + size_t(tile) * a.slot;
        constexpr int AYP = 33;
        // y stage, one thread per (c, kz, column) of Az
        for (int e = tid; e < 3 * AZc * 32; e += NTF) {
            const int l = e & 31, ck = e >> 5;
            const float *src = Az + ck * FTY * 32 + l;
            float *dst = Ay + ck * AYc * AYP + l;
            float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
            int oc = 0;
            for (int yy = 0; yy < ey; ++yy) {
                const int o = asy[yy];
                while (oc < o) {
                    dst[oc * AYP] = s0;
                    s0 = s1;
                    s1 = s2;
                    s2 = s3;
                    s3 = 0.0f;
                    ++oc;
                }
                const float4 w = awy[yy];
                const float f = src[yy * 32];
                s0 += w.x * f;
                s1 += w.y * f;
                s2 += w.z * f;
                s3 += w.w * f;
            }
            if (oc < AYc) dst[oc * AYP] = s0;
            if (oc + 1 < AYc) dst[(oc + 1) * AYP] = s1;
            if (oc + 2 < AYc) dst[(oc + 2) * AYP] = s2;
            if (oc + 3 < AYc) dst[(oc + 3) * AYP] = s3;
            for (int jy = oc + 4; jy < AYc; ++jy) dst[jy * AYP] = 0.0f;
        }
        __syncthreads();
        // x stage, one thread per (c, kz, jy) row of Ay, into the partial
        // slot ((kz AYc + jy) AXc + ix) 3 + c
        for (int e = tid; e < 3 * AZc * AYc; e += NTF) {
            const int c = e / (AZc * AYc), kzjy = e - c * (AZc * AYc);
            const float *src = Ay + (c * AZc * AYc + kzjy) * AYP;
            float *dst = part + size_t(kzjy) * AXc * 3 + c;
            float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
            int oc = 0;
            for (int l = 0; l < ex; ++l) {
                const int o = asx[l];
                while (oc < o) {
                    dst[oc * 3] = s0;
                    s0 = s1;
                    s1 = s2;
                    s2 = s3;
                    s3 = 0.0f;
                    ++oc;
                }
                const float4 w = awx[l];
                const float f = src[l];
                s0 += w.x * f;
                s1 += w.y * f;
                s2 += w.z * f;
                s3 += w.w * f;
            }
            if (oc < AXc) dst[oc * 3] = s0;
            if (oc + 1 < AXc) dst[(oc + 1) * 3] = s1;
            if (oc + 2 < AXc) dst[(oc + 2) * 3] = s2;
            if (oc + 3 < AXc) dst[(oc + 3) * 3] = s3;
            for (int ix = oc + 4; ix < AXc; ++ix) dst[ix * 3] = 0.0f;
        }
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        reduce_tile_sums(a, ntiles, N, red);
        if (tid == 0) a.counters[0] = 0;
    }
}

template <int TZ>
__global__ void __launch_bounds__(NTF, 2) k_fused3(const __grid_constant__ EvalArgs a, int with_gradient)
{
    const int tile = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    fused3_body<TZ>(a, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.x * gridDim.y * gridDim.z, tile,
                    with_gradient);
}

// dynamic shared memory of a block: Az, then the larger of (footprint, x
// stage, 128 bytes of alignment slack, tap ring) and Ay
size_t fused3_smem(const EvalArgs &a)
{
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const size_t FX = X.fc + 2, FY = Y.fc + 2, FZ = Z.fc + 2;
    const size_t az = size_t(3) * Z.ac * FTY * 32;
    const size_t walk = 3 * FZ * FY * (FX + 32) + 32 + size_t(RING_N) * RING_PLANE;
    const size_t ay = size_t(3) * Z.ac * Y.ac * 33;
    return (az + std::max(walk, ay)) * sizeof(float);
}

bool tile_supported_fused3(int tx, int ty, int tz)
{
    return tx == FTX && ty == FTY && (tz == 4 || tz == 8 || tz == 16 || tz == 32);
}

namespace {
template <int TZ>
void launch_fused3_z(const EvalArgs &a, int with_gradient, size_t sm, cudaStream_t st)
{
    raise_smem_limit(reinterpret_cast<const void *>(k_fused3<TZ>), sm);
    k_fused3<TZ><<<dim3(a.ax[0].nt, a.ax[1].nt, a.ax[2].nt), NTF, sm, st>>>(a, with_gradient);
}
}  // namespace

void launch_fused3(const EvalArgs &a, int with_gradient, cudaStream_t st)
{
    launch_params_f32(a, st);
    const size_t sm = fused3_smem(a);
    switch (a.ax[2].t) {
    case 4: launch_fused3_z<4>(a, with_gradient, sm, st); break;
    case 8: launch_fused3_z<8>(a, with_gradient, sm, st); break;
    case 32: launch_fused3_z<32>(a, with_gradient, sm, st); break;
    default: launch_fused3_z<16>(a, with_gradient, sm, st); break;
    }
    count_launch();
}

}  // namespace mgr
