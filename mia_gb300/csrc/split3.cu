// split3.cu — the 3D split evaluation path.
//
// A tile is 32 (x) x 8 (y) x TZ (z) voxels and a block of 256 threads: lane
// = x, warp = y, and every thread walks its z column.  All threads of a
// block stand on the same z plane at the same step, so the z tables are
// uniform and the per-thread sliding windows below advance in lock step.
//
//   k_warp3<TZ>       the tile's coefficient footprint is contracted along x
//       and y in shared memory (C3DSplineTransformation::init_grid,
//       mia/3d/transform/spline.cc:541-653, x then y then z); each thread
//       keeps the four z coefficients of its column that the current voxel
//       needs in registers and slides them as z advances, giving u(x); the
//       prefiltered moving image is sampled with the tricubic B-spline at
//       x - u(x) (mia/3d/interpolator.cxx:250-287, mirror boundary, clamp
//       to [min(0, min src), max src]) from a bricked, mirror-padded copy,
//       so the interior needs no index folding and every tap address is an
//       immediate offset; the warped image is written and
//       the SSD / NCC sums are accumulated; the last block finalises the
//       cost.
//   k_adjoint3<TZ>    central differences of the warped image (x neighbours
//       by warp shuffle, y neighbours from the rows of the adjacent warps, z
//       neighbours carried in registers; mia/3d/image.cc:347-466), the SSD /
//       NCC force (mia/template/ssd.hh:126-181, mia/3d/cost/ncc.cc:88-128),
//       and the transposed spline contraction (translate,
//       spline.cc:731-791) in the reference's order: z while walking (four
//       running sums per component, the lowest one final when the window
//       moves on), then y and x in shared memory; the result goes to the
//       tile's partial slot (no atomics).
//   k_gather3         per 4x4x4 block of coefficients: the fixed-order sum of
//       the partial slots that hold each coefficient, the divcurl stencil
//       (C3DPPDivcurlMatrixImpl::evaluate / multiply,
//       mia/3d/ppmatrix.cc:292-599) over a shared-memory copy of the
//       parameters with a 3-node halo, the penalty weight and sign
//       (mia/3d/splinetransformpenalty.cc:60-71) and the full-cost weight
//       (mia/template/fullcost.cxx:37-45).
#include "mgr_cost.cuh"

namespace mgr {

namespace {

constexpr int NT3 = 256;   // threads per tile block: 8 warps
constexpr int TX3 = 32;    // tile x (lanes)
constexpr int TY3 = 8;     // tile y (warps)
constexpr unsigned FULL = 0xffffffffu;

// Packed (two lanes of a float2) cubic B-spline weights, the operations and
// their order as bspline3_weights: the x and y weights of a sample point in
// one pass.
__device__ __forceinline__ void bspline3_weights2(float2 f, float2 w[4])
{
    const float2 one = make_float2(1.0f, 1.0f), neg = make_float2(-1.0f, -1.0f);
    const float2 ob6 = make_float2(1.0f / 6.0f, 1.0f / 6.0f);
    const float2 xm1 = __ffma2_rn(neg, f, one);
    const float2 w0 = __fmul2_rn(__fmul2_rn(xm1, xm1), __fmul2_rn(xm1, ob6));
    const float2 w3 = __fmul2_rn(__fmul2_rn(f, f), __fmul2_rn(f, ob6));
    w[0] = w0;
    w[3] = w3;
    w[1] = __fadd2_rn(__ffma2_rn(neg, w0, __ffma2_rn(neg, w0, xm1)), w3);
    w[2] = __fadd2_rn(__ffma2_rn(neg, w3, __ffma2_rn(neg, w3, f)), w0);
}

// Tricubic sample at (px, py, pz) from the bricked pair copy: the 4 x 4 x 4
// taps of the start position lie in one brick at compile-time pitches (two
// 8-byte loads per tap row, immediate offsets).  Each row's sum is kept as a
// pair (even taps, odd taps) through the y and z contractions, in packed
// FP32 FMAs, and the pair is added at the end.  Sample points whose taps
// leave the padded box fold their indices on the unpadded image (sample3).
__device__ __forceinline__ float taps3(const EvalArgs &a, float px, float py, float pz, float mn, float mx)
{
    const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
    const int fx = ffloor16(px), fy = ffloor16(py), fz = ffloor16(pz);
    const int gx = fx - 1 + BRK_H, gy = fy - 1 + BRK_H, gz = fz - 1 + BRK_H;
    if (unsigned(gx) <= unsigned(nx + 2 * BRK_H - 4) && unsigned(gy) <= unsigned(ny + 2 * BRK_H - 4) &&
        unsigned(gz) <= unsigned(nz + 2 * BRK_H - 4)) {
        float2 wxy[4];
        bspline3_weights2(make_float2(px - float(fx), py - float(fy)), wxy);
        float wz[4];
        bspline3_weights(pz - float(fz), wz);
        const int bi = ((gz / BRK_CZ) * a.bny + gy / BRK_CY) * a.bnx + gx / BRK_CX;
        const float2 *__restrict__ b = a.brick + size_t(bi) * BRK_N +
                                       ((gz % BRK_CZ) * BRK_Y + (gy % BRK_CY)) * BRK_X + (gx % BRK_CX);
        const float2 wx01 = make_float2(wxy[0].x, wxy[1].x), wx23 = make_float2(wxy[2].x, wxy[3].x);
        float2 acc2 = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int kz = 0; kz < 4; ++kz) {
            float2 s2 = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int ky = 0; ky < 4; ++ky) {
                const float2 *__restrict__ row = b + (kz * BRK_Y + ky) * BRK_X;
                float2 r = __fmul2_rn(wx01, __ldg(row));
                r = __ffma2_rn(wx23, __ldg(row + 2), r);
                s2 = __ffma2_rn(make_float2(wxy[ky].y, wxy[ky].y), r, s2);
            }
            acc2 = __ffma2_rn(make_float2(wz[kz], wz[kz]), s2, acc2);
        }
        return clamp_ref(acc2.x + acc2.y, mn, mx);
    }
    return sample3(a.coef_img, nx, ny, nz, px, py, pz, mn, mx);
}

}  // namespace

// ---------------------------------------------------------------------
// warp
// ---------------------------------------------------------------------
template <int TZ>
__device__ __forceinline__ void warp3_body(const EvalArgs &a, int bx, int by, int bz, int ntiles, int tile)
{
    extern __shared__ __align__(16) float sm3[];
    __shared__ double red[5 * (NT3 / 32)];
    __shared__ float wsum[5][NT3 / 32];
    __shared__ int zs[TZ];
    __shared__ float4 zw[TZ];
    __shared__ bool is_last;
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
    const int x0 = bx * TX3, y0 = by * TY3, z0 = bz * TZ;
    const int ey = min(TY3, ny - y0);
    const int FX = X.fc, FY = Y.fc, FZ = Z.fc;
    const int ncx = a.nc[0], ncy = a.nc[1], ncz = a.nc[2];
    const int tid = threadIdx.x, lane = tid & 31, wy = tid >> 5;
    const int ez = min(TZ, nz - z0);
    // every table entry and scalar the tile needs, loaded up front so that
    // the loads overlap (the data is cold at the start of an evaluation)
    const int cx0 = X.ftile0[bx], cy0 = Y.ftile0[by], cz0 = Z.ftile0[bz];
    const int x = min(x0 + lane, nx - 1), y = min(y0 + wy, ny - 1);
    const int fsx = X.fs[x], fsy = Y.fs[y];
    const float4 fwx = X.fw[x], wyv = Y.fw[y];
    int fsz = 0;
    float4 fwz = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (tid < TZ) {
        const int z = min(z0 + tid, nz - 1);
        fsz = Z.fs[z];
        fwz = Z.fw[z];
    }
    const float mn = a.minmax[0], mxv = a.minmax[1];
    const float ca = float(a.centers[0]), cb = float(a.centers[1]);

    float *C = sm3;                        // [3][FZ][FY][FX]
    float *Tx = C + 3 * FZ * FY * FX;      // [3][FZ][FY][32]
    // coefficient footprint: rows (iz, iy) of 3 FX consecutive doubles
    // (parameters are interleaved per node); each thread issues its loads
    // as one batch before storing
    {
        const int w3 = 3 * FX, nel = FZ * FY * w3;
        auto src = [&](int e, int &dst) -> const double * {
            const int r = e / w3, j = e - r * w3;
            const int ix = j / 3, c = j - 3 * ix;
            const int iz = r / FY, iy = r - iz * FY;
            dst = (c * FZ * FY + r) * FX + ix;
            if (cx0 + ix >= ncx || cy0 + iy >= ncy || cz0 + iz >= ncz) return nullptr;
            return a.params + ((size_t(cz0 + iz) * ncy + (cy0 + iy)) * ncx + cx0) * 3 + j;
        };
        constexpr int K = 4;
        double v[K];
        int dst[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int e = tid + k * NT3;
            v[k] = 0.0;
            dst[k] = -1;
            if (e < nel) {
                const double *p = src(e, dst[k]);
                if (p) v[k] = *p;
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (dst[k] >= 0) C[dst[k]] = float(v[k]);
        for (int e = tid + K * NT3; e < nel; e += NT3) {
            int d;
            const double *p = src(e, d);
            C[d] = p ? float(*p) : 0.0f;
        }
    }
    if (tid < TZ) {
        zs[tid] = fsz - cz0;
        zw[tid] = fwz;
    }
    __syncthreads();
    // x stage: Tx[c][kz][jy][lane]
    {
        const int sx = fsx - cx0;
        for (int r = wy; r < 3 * FZ * FY; r += NT3 / 32) {
            const float *c = C + r * FX + sx;
            Tx[r * 32 + lane] = fwx.x * c[0] + fwx.y * c[1] + fwx.z * c[2] + fwx.w * c[3];
        }
    }
    __syncthreads();
    // y stage on demand: q(c, kz) for this thread's (x, y)
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
    int cur = 0;   // the window's first z coefficient (zs[0] == 0)

    const bool inxy = (x0 + lane < nx) && (y0 + wy < ny);
    const float px0 = float(x0 + lane), py0 = float(y0 + wy);
    const size_t nxy = size_t(nx) * ny;
    const size_t col = size_t(min(y0 + wy, ny - 1)) * nx + min(x0 + lane, nx - 1) + size_t(z0) * nxy;
    float *wout = a.warped + col;
    const float *rin = a.ref + col;
    float acc[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int t = 0; t < ez; ++t) {
        const int s = zs[t];
        while (cur < s) {   // uniform over the block
            ++cur;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                q[c][0] = q[c][1];
                q[c][1] = q[c][2];
                q[c][2] = q[c][3];
                q[c][3] = qat(c, cur + 3);
            }
        }
        const float4 wz = zw[t];
        float u[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) u[c] = wz.x * q[c][0] + wz.y * q[c][1] + wz.z * q[c][2] + wz.w * q[c][3];
        if (inxy) {
            const int z = z0 + t;
            const float wv = taps3(a, px0 - u[0], py0 - u[1], float(z) - u[2], mn, mxv);
            *wout = wv;
            const float b = __ldg(rin);
            if (a.cost == 0) {
                const float d = wv - b;
                acc[0] += d * d;
            } else {
                const float da = wv - ca, db = b - cb;
                acc[0] += da;
                acc[1] += db;
                acc[2] += da * da;
                acc[3] += db * db;
                acc[4] += da * db;
            }
        }
        wout += nxy;
        rin += nxy;
    }
    // tile sums: a float tree within each warp (5 levels), the warps' sums
    // added in double in a fixed order by thread 0 (FP64 is slow here, so
    // it is kept off the per-thread path)
    const int ncomp = a.cost == 0 ? 1 : 5;
#pragma unroll
    for (int k = 0; k < 5; ++k)
        if (k < ncomp) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(FULL, acc[k], o);
            if (lane == 0) wsum[k][wy] = acc[k];
        }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            double v = 0.0;
            if (k < ncomp)
                for (int w = 0; w < NT3 / 32; ++w) v += double(wsum[k][w]);
            a.tile_sums[size_t(tile) * 5 + k] = v;
        }
        __threadfence();
        is_last = (atomicAdd(&a.counters[0], 1u) == unsigned(ntiles - 1));
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        reduce_tile_sums(a, ntiles, size_t(nx) * ny * nz, red);
        if (tid == 0) a.counters[0] = 0;
    }
}

// ---------------------------------------------------------------------
// gradient + force + adjoint
// ---------------------------------------------------------------------
template <int TZ>
__device__ __forceinline__ void adjoint3_body(const EvalArgs &a, int bx, int by, int bz, int tile_index)
{
    extern __shared__ __align__(16) float sm3[];
    __shared__ int asx[TX3], asy[TY3], azs[TZ];
    __shared__ float4 awx[TX3], awy[TY3], azw[TZ];
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
    const int x0 = bx * TX3, y0 = by * TY3, z0 = bz * TZ;
    const int ex = min(TX3, nx - x0), ey = min(TY3, ny - y0), ez = min(TZ, nz - z0);
    const int AXc = X.ac, AYc = Y.ac, AZc = Z.ac;
    const int ax0 = X.atile0[bx], ay0 = Y.atile0[by], az0 = Z.atile0[bz];
    const int tid = threadIdx.x, lane = tid & 31, wy = tid >> 5;
    float *part = a.partial + size_t(tile_index) * a.slot;
    constexpr int AYP = TX3 + 1;              // Ay row pitch (odd: the x stage reads columns)
    float *Az = sm3;                          // [3][AZc][8][32]
    float *Ay = Az + 3 * AZc * TY3 * TX3;     // [3][AZc][AYc][AYP]

    // tables, scalars and the first planes of the column, loaded up front
    const int x = x0 + lane, y = y0 + wy;
    const bool inxy = x < nx && y < ny;
    const size_t nxy = size_t(nx) * ny;
    const size_t col = size_t(min(y, ny - 1)) * nx + min(x, nx - 1);
    const float *__restrict__ W = a.warped;
    const float *__restrict__ R = a.ref;
    const double *sc = a.scalars;
    const float k1 = float(sc[SC_K1]), k2 = float(sc[SC_K2]);
    const float ma = float(sc[SC_MA]), mb = float(sc[SC_MB]), fscale = float(sc[SC_FSCALE]);
    const bool bx_in = x > 0 && x < nx - 1, by_in = y > 0 && y < ny - 1;
    // column pointers at the current plane
    const float *__restrict__ wc = W + size_t(z0) * nxy + col;
    const float *__restrict__ rc = R + size_t(z0) * nxy + col;
    const int ynm = (y > 0) ? -nx : 0, ynp = (y + 1 < ny) ? nx : 0;
    float wm = (z0 > 0) ? __ldg(wc - nxy) : 0.0f;
    float w0 = __ldg(wc);
    if (tid < TX3) {
        const int xx = min(x0 + tid, nx - 1);
        asx[tid] = X.as[xx] - ax0;
        awx[tid] = X.aw[xx];
    }
    if (tid < TY3) {
        const int yy = min(y0 + tid, ny - 1);
        asy[tid] = Y.as[yy] - ay0;
        awy[tid] = Y.aw[yy];
    }
    if (tid < TZ) {
        const int zz = min(z0 + tid, nz - 1);
        azs[tid] = Z.as[zz] - az0;
        azw[tid] = Z.aw[zz];
    }
    __syncthreads();

    float acc[3][4];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[c][k] = 0.0f;
    int cur = 0;   // azs[0] == 0
    auto emit = [&](int kz, int c, float v) { Az[((c * AZc + kz) * TY3 + wy) * TX3 + lane] = v; };
    for (int t = 0; t < ez; ++t) {
        const int z = z0 + t;
        const float wp = (z + 1 < nz) ? __ldg(wc + nxy) : 0.0f;
        float left = __shfl_up_sync(FULL, w0, 1), right = __shfl_down_sync(FULL, w0, 1);
        if (lane == 0 && x > 0) left = __ldg(wc - 1);
        if (lane == TX3 - 1 && x + 1 < nx) right = __ldg(wc + 1);
        float f[3] = {0.0f, 0.0f, 0.0f};
        if (inxy) {
            const float ym = __ldg(wc + ynm), yp = __ldg(wc + ynp);
            float g[3];
            g[0] = bx_in ? 0.5f * (right - left) : 0.0f;
            g[1] = by_in ? 0.5f * (yp - ym) : 0.0f;
            g[2] = (z > 0 && z < nz - 1) ? 0.5f * (wp - wm) : 0.0f;
            const float b = __ldg(rc);
            if (a.cost == 0) {
                const float d = w0 - b;
#pragma unroll
                for (int k = 0; k < 3; ++k) f[k] = (g[k] * d) * fscale;
            } else {
                const float s = k1 * (k2 * (w0 - ma) - (b - mb));
#pragma unroll
                for (int k = 0; k < 3; ++k) f[k] = s * g[k];
            }
        }
        wc += nxy;
        rc += nxy;
        const int s = azs[t];
        while (cur < s) {   // uniform over the block
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                emit(cur, c, acc[c][0]);
                acc[c][0] = acc[c][1];
                acc[c][1] = acc[c][2];
                acc[c][2] = acc[c][3];
                acc[c][3] = 0.0f;
            }
            ++cur;
        }
        const float4 w = azw[t];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            acc[c][0] += w.x * f[c];
            acc[c][1] += w.y * f[c];
            acc[c][2] += w.z * f[c];
            acc[c][3] += w.w * f[c];
        }
        wm = w0;
        w0 = wp;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (cur + k < AZc)
#pragma unroll
            for (int c = 0; c < 3; ++c) emit(cur + k, c, acc[c][k]);
    for (int kz = cur + 4; kz < AZc; ++kz)
#pragma unroll
        for (int c = 0; c < 3; ++c) emit(kz, c, 0.0f);
    __syncthreads();
    // y stage, one thread per (c, kz, lane) column of Az: the transposed
    // contraction over the tile's rows as a sliding window of four sums
    // (the row starts are the same for every thread, so the window moves in
    // lock step); Ay rows have an odd pitch for the x stage
    for (int e = tid; e < 3 * AZc * TX3; e += NT3) {
        const int l = e & (TX3 - 1), ck = e >> 5;
        const float *src = Az + ck * TY3 * TX3 + l;
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
            const float f = src[yy * TX3];
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
    // x stage, one thread per (c, kz, jy) row of Ay, the same sliding window
    // over the lanes, straight into the partial slot
    // ((kz AYc + jy) AXc + ix) 3 + c
    for (int e = tid; e < 3 * AZc * AYc; e += NT3) {
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

// ---------------------------------------------------------------------
// gather + penalty
// ---------------------------------------------------------------------
namespace {
constexpr int GT3 = 256;
constexpr int GB = 4;             // coefficients per block edge
constexpr int GH = 3;             // stencil half width
constexpr int GP = GB + 2 * GH;   // 10: halo tile edge
constexpr int GPX = 12;           // padded row pitch (float4) of the halo tile
constexpr int GLMAX = 24;         // longest staged per-axis tile list
}  // namespace

__device__ __forceinline__ void gather3_body(const EvalArgs &a, int with_gradient, int image_from_dense, int blk,
                                             int nblk)
{
    __shared__ float4 Ps[GP * GP * GPX];
    __shared__ float4 Pt[343 * 2];
    __shared__ float pacc[4][12][64];
    __shared__ int gl[3][GB][GLMAX];   // per axis and coefficient of the block: slot offset part per tile
    __shared__ int gn[3][GB];          // list lengths (-1: too long, use the tables directly)
    __shared__ double red[GT3 / 32];
    __shared__ bool is_last;
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int ncx = a.nc[0], ncy = a.nc[1], ncz = a.nc[2];
    const int nbx = (ncx + GB - 1) / GB, nby = (ncy + GB - 1) / GB;
    const int bxi = blk % nbx, byi = (blk / nbx) % nby, bzi = blk / (nbx * nby);
    const int cx0 = bxi * GB, cy0 = byi * GB, cz0 = bzi * GB;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int sub = w >> 1;                   // 4 groups of 64 threads split the work of a coefficient
    const int li = ((w & 1) << 5) | lane;     // coefficient of the block
    const int lx = li & 3, ly = (li >> 2) & 3, lz = li >> 4;
    const int cx = cx0 + lx, cy = cy0 + ly, cz = cz0 + lz;
    const bool valid = cx < ncx && cy < ncy && cz < ncz;
    const size_t i = valid ? (size_t(cz) * ncy + cy) * ncx + cx : 0;

    // per axis a and coefficient c0 + k of the block: the tiles t whose
    // adjoint footprint holds it and the part of the slot offset that
    // depends on that axis (tile term, local term), so that the offset of
    // slot entry (tx, ty, tz) is gl[0] + gl[1] + gl[2] (partial is indexed
    // as ((tz nty + ty) ntx + tx) slot + ((lz acy + ly) acx + lx) 3)
    if (with_gradient && !image_from_dense && tid < 3 * GB) {
        const int ax = tid / GB, k = tid - ax * GB;
        const Axis &A = a.ax[ax];
        const int c = (ax == 0 ? cx0 : ax == 1 ? cy0 : cz0) + k;
        int cnt = 0;
        if (c < A.nc) {
            const int2 g = A.gtile[c];
            cnt = max(g.y - g.x + 1, 0);
            const long long nslots = (long long)X.nt * Y.nt * Z.nt * a.slot;
            if (cnt > GLMAX || nslots >= (1LL << 31)) {
                cnt = -1;
            } else {
                const int tstride = ax == 0 ? a.slot : ax == 1 ? X.nt * a.slot : X.nt * Y.nt * a.slot;
                const int lstride = ax == 0 ? 3 : ax == 1 ? X.ac * 3 : X.ac * Y.ac * 3;
                for (int j = 0; j < cnt; ++j) {
                    const int t = g.x + j;
                    gl[ax][k][j] = t * tstride + (c - A.atile0[t]) * lstride;
                }
            }
        }
        gn[ax][k] = cnt;
    }
    if (a.has_penalty) {
        // parameters of the block with a 3-node halo and the 7^3 cells of
        // the penalty table, each thread's loads issued as one batch
        constexpr int KP = (GP * GP * GP + GT3 - 1) / GT3;
        double pv[KP][3];
#pragma unroll
        for (int k = 0; k < KP; ++k) {
            const int e = tid + k * GT3;
            pv[k][0] = pv[k][1] = pv[k][2] = 0.0;
            if (e < GP * GP * GP) {
                const int hx = e % GP, hy = (e / GP) % GP, hz = e / (GP * GP);
                const int gx = cx0 - GH + hx, gy = cy0 - GH + hy, gz = cz0 - GH + hz;
                if (gx >= 0 && gx < ncx && gy >= 0 && gy < ncy && gz >= 0 && gz < ncz) {
                    const double *p = a.params + ((size_t(gz) * ncy + gy) * ncx + gx) * 3;
                    pv[k][0] = p[0];
                    pv[k][1] = p[1];
                    pv[k][2] = p[2];
                }
            }
        }
        constexpr int KT = (343 + GT3 - 1) / GT3;
        float tv[KT][6];
#pragma unroll
        for (int k = 0; k < KT; ++k) {
            const int e = tid + k * GT3;
            if (e < 343) {
                const int dx = e % 7 - 3, dy = (e / 7) % 7 - 3, dz = e / 49 - 3;
                const float *P = a.ptable + (((dz + 4) * 9 + (dy + 4)) * 9 + (dx + 4)) * 6;
#pragma unroll
                for (int j = 0; j < 6; ++j) tv[k][j] = P[j];
            }
        }
#pragma unroll
        for (int k = 0; k < KP; ++k) {
            const int e = tid + k * GT3;
            if (e < GP * GP * GP) {
                const int hx = e % GP, hy = (e / GP) % GP, hz = e / (GP * GP);
                Ps[(hz * GP + hy) * GPX + hx] = make_float4(float(pv[k][0]), float(pv[k][1]), float(pv[k][2]), 0.0f);
            }
        }
#pragma unroll
        for (int k = 0; k < KT; ++k) {
            const int e = tid + k * GT3;
            if (e < 343) {
                Pt[2 * e] = make_float4(tv[k][0], tv[k][1], tv[k][2], tv[k][3]);
                Pt[2 * e + 1] = make_float4(tv[k][4], tv[k][5], 0.0f, 0.0f);
            }
        }
    }
    __syncthreads();
    // R0..R5, T0..T2: the nine products of the 3x3 cell with c_j, summed
    // over the 7^3 neighbours j = i - d (zero outside the grid)
    float R0 = 0, R1 = 0, R2 = 0, R3 = 0, R4 = 0, R5 = 0, T0 = 0, T1 = 0, T2 = 0;
    if (valid && a.has_penalty) {
        for (int p = sub; p < 49; p += 4) {
            const int dz = p / 7 - 3, dy = p % 7 - 3;
            const float4 *prow = Ps + ((lz + GH - dz) * GP + (ly + GH - dy)) * GPX + (lx + GH);
            const float4 *trow = Pt + p * 14;
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const float4 cj = prow[3 - k];     // dx = k - 3
                const float4 t0 = trow[2 * k], t1 = trow[2 * k + 1];
                R0 += t0.x * cj.x;
                R1 += t0.y * cj.y;
                R2 += t0.z * cj.y;
                R3 += t0.w * cj.z;
                R4 += t1.x * cj.z;
                R5 += t1.y * cj.x;
                T0 += t1.y * cj.z;
                T1 += t0.y * cj.x;
                T2 += t0.w * cj.y;
            }
        }
    }
    float S[3] = {0.0f, 0.0f, 0.0f};
    if (valid && with_gradient && !image_from_dense) {
        // the tiles whose slot holds this coefficient: a contiguous range per
        // axis; the per-axis parts of the slot offsets come from the lists
        // staged above, the rest is independent loads
        const int nX = gn[0][lx], nY = gn[1][ly], nZ = gn[2][lz];
        if (nX >= 0 && nY >= 0 && nZ >= 0) {
            const int tot = nX * nY * nZ;
            for (int k0 = sub; k0 < tot; k0 += 16) {
                float v[4][3];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int k = k0 + 4 * u;
                    v[u][0] = v[u][1] = v[u][2] = 0.0f;
                    if (k < tot) {
                        const int jx = k % nX, r = k / nX;
                        const int jy = r % nY, jz = r / nY;
                        const float *p = a.partial + (size_t(gl[2][lz][jz] + gl[1][ly][jy]) + gl[0][lx][jx]);
                        v[u][0] = p[0];
                        v[u][1] = p[1];
                        v[u][2] = p[2];
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    S[0] += v[u][0];
                    S[1] += v[u][1];
                    S[2] += v[u][2];
                }
            }
        } else {
            const int2 gx = X.gtile[cx], gy = Y.gtile[cy], gz = Z.gtile[cz];
            const int mX = gx.y - gx.x + 1, mY = gy.y - gy.x + 1, mZ = gz.y - gz.x + 1;
            const int total = (mX > 0 && mY > 0 && mZ > 0) ? mX * mY * mZ : 0;
            for (int k = sub; k < total; k += 4) {
                const int tx = gx.x + k % mX, ty = gy.x + (k / mX) % mY, tz = gz.x + k / (mX * mY);
                const int lxo = cx - X.atile0[tx], lyo = cy - Y.atile0[ty], lzo = cz - Z.atile0[tz];
                const size_t t = (size_t(tz) * Y.nt + ty) * X.nt + tx;
                const float *p = a.partial + t * a.slot + ((size_t(lzo) * Y.ac + lyo) * X.ac + lxo) * 3;
                S[0] += p[0];
                S[1] += p[1];
                S[2] += p[2];
            }
        }
    }
    pacc[sub][0][li] = R0;
    pacc[sub][1][li] = R1;
    pacc[sub][2][li] = R2;
    pacc[sub][3][li] = R3;
    pacc[sub][4][li] = R4;
    pacc[sub][5][li] = R5;
    pacc[sub][6][li] = T0;
    pacc[sub][7][li] = T1;
    pacc[sub][8][li] = T2;
    pacc[sub][9][li] = S[0];
    pacc[sub][10][li] = S[1];
    pacc[sub][11][li] = S[2];
    __syncthreads();
    double pval = 0.0;
    if (sub == 0 && valid) {
        float v9[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) v9[k] = pacc[0][k][li] + pacc[1][k][li] + pacc[2][k][li] + pacc[3][k][li];
        double gp[3] = {0.0, 0.0, 0.0};
        if (a.has_penalty) {
            const float ci0 = float(a.params[i * 3]), ci1 = float(a.params[i * 3 + 1]), ci2 = float(a.params[i * 3 + 2]);
            float v;
            if (with_gradient)
                v = ci0 * v9[0] + ci0 * v9[1] + ci1 * v9[2] + ci1 * v9[3] + ci2 * v9[4] + ci2 * v9[5];
            else
                v = ci0 * v9[0] + ci1 * v9[2] + ci2 * v9[4] + ci0 * v9[1] + ci0 * v9[6] + ci1 * v9[3];
            pval = v;
            const float g0 = v9[6] + (2.0f * v9[0] + v9[1]);
            const float g1 = v9[7] + (2.0f * v9[2] + v9[3]);
            const float g2 = v9[8] + (2.0f * v9[4] + v9[5]);
            gp[0] = -a.pen_weight * double(g0);
            gp[1] = -a.pen_weight * double(g1);
            gp[2] = -a.pen_weight * double(g2);
        }
        if (with_gradient) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double gi = image_from_dense ? a.grad_image[i * 3 + k] : a.cost_weight * (-double(v9[9 + k]));
                a.grad_total[i * 3 + k] = gi + gp[k];
                if (a.grad_image && !image_from_dense) a.grad_image[i * 3 + k] = gi;
                if (a.grad_penalty) a.grad_penalty[i * 3 + k] = gp[k];
            }
        }
    }
    pval = warp_sum(pval);
    if (lane == 0) red[w] = pval;
    __syncthreads();
    if (tid == 0) {
        a.pen_part[blk] = red[0] + red[1];
        __threadfence();
        is_last = (atomicAdd(&a.counters[1], 1u) == unsigned(nblk - 1));
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        double sv[1] = {0.0};
        for (unsigned b = tid; b < unsigned(nblk); b += GT3) sv[0] += ((volatile double *)a.pen_part)[b];
        block_sum<1>(sv, red);
        if (tid == 0) {
            double *sc = a.scalars;
            const double pen = a.has_penalty ? sv[0] : 0.0;
            sc[SC_PEN] = pen;
            sc[SC_COST_IMG] = a.cost_weight * sc[SC_VALUE];
            sc[SC_COST_PEN] = a.has_penalty ? a.pen_weight * pen : 0.0;
            if (a.costs) {
                a.costs[0] = sc[SC_COST_IMG];
                a.costs[1] = sc[SC_COST_PEN];
            }
            a.counters[1] = 0;
        }
    }
}

// ---------------------------------------------------------------------
// kernels: one pair (grid = tiles) and a batch of pairs (grid = work list
// of (pair, tile) items; pairs whose minimizer has finished are skipped)
// ---------------------------------------------------------------------
#ifndef MGR_WARP_MINB
#define MGR_WARP_MINB 3
#endif

template <int TZ>
__global__ void __launch_bounds__(NT3, MGR_WARP_MINB) k_warp3(EvalArgs a)
{
    const int tile = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    warp3_body<TZ>(a, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.x * gridDim.y * gridDim.z, tile);
}

template <int TZ>
__global__ void __launch_bounds__(NT3) k_adjoint3(EvalArgs a)
{
    const int tile = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    adjoint3_body<TZ>(a, blockIdx.x, blockIdx.y, blockIdx.z, tile);
}

__global__ void __launch_bounds__(GT3) k_gather3(EvalArgs a, int with_gradient, int image_from_dense)
{
    gather3_body(a, with_gradient, image_from_dense, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void decode_tile3(const EvalArgs &a, int t, int &bx, int &by, int &bz, int &nt)
{
    const int ntx = a.ax[0].nt, nty = a.ax[1].nt, ntz = a.ax[2].nt;
    bx = t % ntx;
    by = (t / ntx) % nty;
    bz = t / (ntx * nty);
    nt = ntx * nty * ntz;
}

template <int TZ>
__global__ void __launch_bounds__(NT3, MGR_WARP_MINB) k_warp3_batch(const EvalArgs *__restrict__ args,
                                                                    const int2 *__restrict__ items,
                                                                    const int *__restrict__ active)
{
    const int2 it = items[blockIdx.x];
    if (!active[it.x]) return;
    const EvalArgs &a = args[it.x];
    int bx, by, bz, nt;
    decode_tile3(a, it.y, bx, by, bz, nt);
    warp3_body<TZ>(a, bx, by, bz, nt, it.y);
}

template <int TZ>
__global__ void __launch_bounds__(NT3) k_adjoint3_batch(const EvalArgs *__restrict__ args,
                                                        const int2 *__restrict__ items, const int *__restrict__ active)
{
    const int2 it = items[blockIdx.x];
    if (!active[it.x]) return;
    const EvalArgs &a = args[it.x];
    int bx, by, bz, nt;
    decode_tile3(a, it.y, bx, by, bz, nt);
    adjoint3_body<TZ>(a, bx, by, bz, it.y);
}

__global__ void __launch_bounds__(GT3) k_gather3_batch(const EvalArgs *__restrict__ args,
                                                       const int2 *__restrict__ items, const int *__restrict__ active,
                                                       const int *__restrict__ nblocks)
{
    const int2 it = items[blockIdx.x];
    if (!active[it.x]) return;
    gather3_body(args[it.x], 1, 0, it.y, nblocks[it.x]);
}

// ---------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------
size_t split3_smem(const EvalArgs &a, int which)
{
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    if (which == 0) return size_t(3) * Z.fc * Y.fc * (X.fc + TX3) * sizeof(float);
    return size_t(3) * Z.ac * (TY3 * TX3 + Y.ac * (TX3 + 1)) * sizeof(float);
}

bool tile_supported3(int tx, int ty, int tz)
{
    return tx == TX3 && ty == TY3 && (tz == 4 || tz == 8 || tz == 16);
}

namespace {

template <int TZ>
void launch_warp3_z(const EvalArgs &a, size_t sm, cudaStream_t st)
{
    cudaFuncSetAttribute(k_warp3<TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    k_warp3<TZ><<<dim3(a.ax[0].nt, a.ax[1].nt, a.ax[2].nt), NT3, sm, st>>>(a);
}

template <int TZ>
void launch_adjoint3_z(const EvalArgs &a, size_t sm, cudaStream_t st)
{
    cudaFuncSetAttribute(k_adjoint3<TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    k_adjoint3<TZ><<<dim3(a.ax[0].nt, a.ax[1].nt, a.ax[2].nt), NT3, sm, st>>>(a);
}

template <int TZ>
void batch3_z(const EvalArgs *args, const int2 *items, int nitems, const int *active, size_t sm, int which,
              cudaStream_t st)
{
    if (which == 0)
        k_warp3_batch<TZ><<<nitems, NT3, sm, st>>>(args, items, active);
    else
        k_adjoint3_batch<TZ><<<nitems, NT3, sm, st>>>(args, items, active);
}

template <int TZ>
void prepare3_z(size_t sm_warp, size_t sm_adj)
{
    cudaFuncSetAttribute(k_warp3_batch<TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm_warp));
    cudaFuncSetAttribute(k_adjoint3_batch<TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm_adj));
}

}  // namespace

void launch_warp3(const EvalArgs &a, cudaStream_t st)
{
    const size_t sm = split3_smem(a, 0);
    switch (a.ax[2].t) {
    case 4: launch_warp3_z<4>(a, sm, st); break;
    case 8: launch_warp3_z<8>(a, sm, st); break;
    default: launch_warp3_z<16>(a, sm, st); break;
    }
    count_launch();
}

void launch_adjoint3(const EvalArgs &a, cudaStream_t st)
{
    const size_t sm = split3_smem(a, 1);
    switch (a.ax[2].t) {
    case 4: launch_adjoint3_z<4>(a, sm, st); break;
    case 8: launch_adjoint3_z<8>(a, sm, st); break;
    default: launch_adjoint3_z<16>(a, sm, st); break;
    }
    count_launch();
}

int gather3_blocks(const EvalArgs &a)
{
    return ((a.nc[0] + GB - 1) / GB) * ((a.nc[1] + GB - 1) / GB) * ((a.nc[2] + GB - 1) / GB);
}

void launch_gather3(const EvalArgs &a, int with_gradient, int dense, cudaStream_t st)
{
    k_gather3<<<gather3_blocks(a), GT3, 0, st>>>(a, with_gradient, dense);
    count_launch();
}

void prepare_split3_batch(int tz, size_t sm_warp, size_t sm_adj)
{
    switch (tz) {
    case 4: prepare3_z<4>(sm_warp, sm_adj); break;
    case 8: prepare3_z<8>(sm_warp, sm_adj); break;
    default: prepare3_z<16>(sm_warp, sm_adj); break;
    }
}

void launch_split3_batch(int tz, const EvalArgs *args, const int2 *items, int nitems, const int *active, size_t sm,
                         int which, cudaStream_t st)
{
    switch (tz) {
    case 4: batch3_z<4>(args, items, nitems, active, sm, which, st); break;
    case 8: batch3_z<8>(args, items, nitems, active, sm, which, st); break;
    default: batch3_z<16>(args, items, nitems, active, sm, which, st); break;
    }
    count_launch();
}

void launch_gather3_batch(const EvalArgs *args, const int2 *items, int nitems, const int *active, const int *nblocks,
                          cudaStream_t st)
{
    k_gather3_batch<<<nitems, GT3, 0, st>>>(args, items, active, nblocks);
    count_launch();
}

}  // namespace mgr
