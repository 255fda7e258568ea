// split.cu — the split evaluation path (default):
//
//   k_warp_t<D,TX,TY,TZ>     per voxel tile: the tile's coefficient footprint
//       is contracted along z, y, x in shared memory (C3DSplineTransformation::
//       init_grid, mia/3d/transform/spline.cc:541-653) to the displacement
//       u(x); the prefiltered moving image is sampled with the tricubic
//       B-spline at x - u(x) (mia/3d/interpolator.cxx:250-287, mirror
//       boundary, clamp); the warped image is written and the SSD / NCC sums
//       accumulated; the last block to finish finalises the cost.
//   k_adjoint_t<D,TX,TY,TZ>  per voxel tile: central differences of the
//       warped image (mia/3d/image.cc:347-466), the SSD / NCC force
//       (mia/template/ssd.hh:126-181, mia/3d/cost/ncc.cc:88-128), and the
//       transposed spline contraction (translate, spline.cc:731-791) of the
//       force onto the tile's coefficient footprint, x then y then z, each
//       stage as a sliding 4-coefficient window over monotone start indices;
//       the result goes to the tile's partial slot (no atomics).
// The per-coefficient gather of the partial slots and the divcurl penalty
// follow in gather.cu.
#include "mgr_cost.cuh"

namespace mgr {

namespace {

constexpr int NT = 256;

struct RowMap {
    int ix, r0, rstep;
    bool act;
};

// rows of runtime width `w`: thread -> (column ix, first row r0), rows
// advance by rstep; threads beyond rstep*w idle
__device__ __forceinline__ RowMap row_map(int w)
{
    RowMap m;
    m.ix = threadIdx.x % w;
    m.r0 = threadIdx.x / w;
    m.rstep = NT / w;
    m.act = m.r0 < m.rstep;
    return m;
}

// Transposed B-spline contraction of one line of `len` samples onto nout
// coefficients: sample i contributes w_i[k] * in[i*stride] to coefficient
// start_i + k (k < 4), start_i non-decreasing.  Four running sums are kept;
// when the start advances the lowest one is final and emitted.  Every output
// in [0, nout) is emitted exactly once, in increasing order.
template <class Emit>
__device__ __forceinline__ void window_contract(int len, const int *start, const float4 *w, const float *in,
                                                int stride, int nout, Emit emit)
{
    int oc = 0;
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    for (int i = 0; i < len; ++i) {
        const int o = start[i];
        while (oc < o) {
            emit(oc, a0);
            a0 = a1;
            a1 = a2;
            a2 = a3;
            a3 = 0.0f;
            ++oc;
        }
        const float4 ww = w[i];
        const float f = in[i * stride];
        a0 += ww.x * f;
        a1 += ww.y * f;
        a2 += ww.z * f;
        a3 += ww.w * f;
    }
    if (oc < nout) emit(oc, a0);
    if (oc + 1 < nout) emit(oc + 1, a1);
    if (oc + 2 < nout) emit(oc + 2, a2);
    if (oc + 3 < nout) emit(oc + 3, a3);
    for (int o = oc + 4; o < nout; ++o) emit(o, 0.0f);
}

}  // namespace

// ---------------------------------------------------------------------
// warp
// ---------------------------------------------------------------------
// tile (bx, by, bz) of a pair with `ntiles` tiles, `tile` its linear index
template <int D, int TX, int TY, int TZ>
__device__ __forceinline__ void warp_body(const EvalArgs &a, int bx, int by, int bz, int ntiles, int tile)
{
    static_assert(NT % TX == 0, "a thread keeps its x column");
    extern __shared__ __align__(128) float sm[];
    __shared__ double red[5 * (NT / 32)];
    __shared__ float cred[NT / 32][6];
    __shared__ bool is_last;
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ int fsx[TX], fsy[TY], fsz[TZ];
    __shared__ float4 fwx[TX], fwy[TY], fwz[TZ];
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int nx = a.n[0], ny = a.n[1], nz = (D == 3) ? a.n[2] : 1;
    const int x0 = bx * TX, y0 = by * TY, z0 = bz * TZ;
    const int ex = min(TX, nx - x0), ey = min(TY, ny - y0), ez = min(TZ, nz - z0);
    const int FX = X.fc, FY = Y.fc, FZ = (D == 3) ? Z.fc : 1;
    const int cx0 = X.ftile0[bx], cy0 = Y.ftile0[by], cz0 = (D == 3) ? Z.ftile0[bz] : 0;
    const int ncx = a.nc[0], ncy = a.nc[1], ncz = (D == 3) ? a.nc[2] : 1;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

    float *C = sm;                                       // [D][FZ][FY][FX]
    float *T1 = C + D * FZ * FY * FX;                    // [D][TZ][FY][FX]   (3D)
    float *T2 = T1 + ((D == 3) ? D * TZ * FY * FX : 0);  // [D][TZ][TY][FX]
    // after C, T1, T2, rounded up to 32 floats (the host sizes it the same way)
    float *Fp = sm + ((D * FZ * FY * FX + ((D == 3) ? D * TZ * FY * FX : 0) + D * TZ * TY * FX + 31) & ~31);

    if (tid == 0) {
        const unsigned mb = static_cast<unsigned>(__cvta_generic_to_shared(&mbar));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb) : "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    }
    // per-tile forward tables (voxels past the image edge repeat the last one)
    if (tid < TX) {
        const int x = min(x0 + tid, nx - 1);
        fsx[tid] = X.fs[x] - cx0;
        fwx[tid] = X.fw[x];
    }
    if (tid < TY) {
        const int y = min(y0 + tid, ny - 1);
        fsy[tid] = Y.fs[y] - cy0;
        fwy[tid] = Y.fw[y];
    }
    if (D == 3 && tid < TZ) {
        const int z = min(z0 + tid, nz - 1);
        fsz[tid] = Z.fs[z] - cz0;
        fwz[tid] = Z.fw[z];
    }
    const RowMap m = row_map(FX);
    // coefficient footprint, rows (comp, iz, iy); parameters are double,
    // interleaved per node
    if (m.act) {
        const int gx = cx0 + m.ix;
        for (int r = m.r0; r < D * FZ * FY; r += m.rstep) {
            const int comp = r / (FZ * FY), rr = r - comp * FZ * FY;
            const int iz = rr / FY, iy = rr - iz * FY;
            const int gy = cy0 + iy, gz = cz0 + iz;
            float v = 0.0f;
            if (gx < ncx && gy < ncy && gz < ncz)
                v = float(a.params[((size_t(gz) * ncy + gy) * ncx + gx) * D + comp]);
            C[r * FX + m.ix] = v;
        }
    }
    __syncthreads();
    if (D == 3) {
        if (m.act) {
            const int st = FY * FX;
            for (int r = m.r0; r < D * TZ * FY; r += m.rstep) {
                const int comp = r / (TZ * FY), rr = r - comp * TZ * FY;
                const int zz = rr / FY, iy = rr - zz * FY;
                const int s = fsz[zz];
                const float4 w = fwz[zz];
                const float *c = C + (comp * FZ * FY + iy) * FX + m.ix + s * st;
                T1[r * FX + m.ix] = w.x * c[0] + w.y * c[st] + w.z * c[2 * st] + w.w * c[3 * st];
            }
        }
        __syncthreads();
    }
    // y stage.  The displacement of every voxel of the tile is a convex
    // combination (partition-of-unity weights) of the T2 entries of its
    // component, so their per-component range bounds the sample points.
    {
        float cmin[3] = {3.4e38f, 3.4e38f, 3.4e38f}, cmax[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        const float *Src = (D == 3) ? T1 : C;  // [D][TZ][FY][FX] (2D: TZ = FZ = 1)
        if (m.act) {
            for (int r = m.r0; r < D * TZ * TY; r += m.rstep) {
                const int comp = r / (TZ * TY), rr = r - comp * (TZ * TY);
                const int zz = rr / TY, yy = rr - zz * TY;
                const int s = fsy[yy];
                const float4 w = fwy[yy];
                const float *c = Src + ((comp * TZ + zz) * FY + s) * FX + m.ix;
                const float v = w.x * c[0] + w.y * c[FX] + w.z * c[2 * FX] + w.w * c[3 * FX];
                T2[r * FX + m.ix] = v;
#pragma unroll
                for (int k = 0; k < D; ++k)
                    if (comp == k) {
                        cmin[k] = fminf(cmin[k], v);
                        cmax[k] = fmaxf(cmax[k], v);
                    }
            }
        }
#pragma unroll
        for (int k = 0; k < D; ++k) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                cmin[k] = fminf(cmin[k], __shfl_xor_sync(0xffffffffu, cmin[k], o));
                cmax[k] = fmaxf(cmax[k], __shfl_xor_sync(0xffffffffu, cmax[k], o));
            }
        }
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < D; ++k) {
                cred[wid][k] = cmin[k];
                cred[wid][3 + k] = cmax[k];
            }
        }
    }
    __syncthreads();

    // footprint of the interpolation taps.  A sample point x - u(x) lies in
    // [x_lo - max T2, x_hi - min T2] per axis (plus a rounding margin); its taps
    // span [floor - 1, floor + 3].  The box is staged from the padded image
    // when it lies within the halo and fits the shared-memory budget.
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    bool staged = true;
    {
        const int v0[3] = {x0, y0, z0}, v1[3] = {x0 + ex - 1, y0 + ey - 1, z0 + ez - 1};
        const int nn[3] = {nx, ny, nz};
#pragma unroll
        for (int k = 0; k < D; ++k) {
            float c0 = cred[0][k], c1 = cred[0][3 + k];
            for (int w = 1; w < NT / 32; ++w) {
                c0 = fminf(c0, cred[w][k]);
                c1 = fmaxf(c1, cred[w][3 + k]);
            }
            const float mg = 0.01f + 1e-5f * (fabsf(c0) + fabsf(c1) + float(v1[k]));
            const float pmin = float(v0[k]) - c1 - mg, pmax = float(v1[k]) - c0 + mg;
            if (!(pmin > -1e6f && pmax < 1e6f)) {
                staged = false;
                continue;
            }
            lo[k] = int(floorf(pmin)) - 1;
            hi[k] = int(floorf(pmax)) + 3;
            if (lo[k] < -PAD_H || hi[k] > nn[k] - 1 + PAD_H) staged = false;
        }
        if (D == 2) lo[2] = hi[2] = 0;
    }
    // x origin aligned to 16 bytes in the padded rows; row length in floats
    constexpr int SBX = stage_bx(TX), SBY = stage_by(TY), SBZ = stage_bz(D, TZ);
    const int sx0 = ((lo[0] + PAD_H) & ~3) - PAD_H;
    const int SP = ((hi[0] - sx0 + 1) + 3) & ~3;
    const int FPY = hi[1] - lo[1] + 1, FPZ = hi[2] - lo[2] + 1;
    if (staged && (SP > SBX || FPY > SBY || FPZ > SBZ)) staged = false;
    const unsigned mb = static_cast<unsigned>(__cvta_generic_to_shared(&mbar));
    if (staged && wid == 0) {
        // one bulk copy per footprint row (16-byte aligned, multiple of 16
        // bytes), completion counted on the mbarrier
        const int rows = FPY * FPZ;
        if (lane == 0) {
            const unsigned bytes = unsigned(rows) * unsigned(SP) * 4u;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb), "r"(bytes) : "memory");
        }
        __syncwarp();
        const int P = pad_pitch(nx), PY = a.pad_rows;
        const int hz = (D == 3) ? PAD_H : 0;
        for (int r = lane; r < rows; r += 32) {
            const int j = r % FPY, k = r / FPY;
            const float *src = a.coef_pad + (size_t(lo[2] + k + hz) * PY + (lo[1] + j + PAD_H)) * P + (sx0 + PAD_H);
            const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(Fp + (k * SBY + j) * SBX));
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                         "l"(src), "r"(unsigned(SP) * 4u), "r"(mb)
                         : "memory");
        }
    }
    __syncthreads();
    if (staged) {
        // bounded wait for the copies (phase 0); on time-out the status flag
        // is raised and the copies are waited for once more before the block
        // may leave
        unsigned done = 0;
        for (int it = 0; it < (1 << 22) && !done; ++it)
            asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
                         : "=r"(done)
                         : "r"(mb)
                         : "memory");
        if (!done) {
            atomicOr(&a.counters[6], 1u);
            for (int it = 0; it < (1 << 22) && !done; ++it)
                asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
                             : "=r"(done)
                             : "r"(mb)
                             : "memory");
        }
    }

    // x stage, tricubic sample, warped image, sums: a thread keeps its x
    // column and walks the rows (y, z) of the tile
    float acc[5] = {0, 0, 0, 0, 0};
    const float mn = a.minmax[0], mxv = a.minmax[1];
    const float ca = float(a.centers[0]), cb = float(a.centers[1]);
    const int xx = tid % TX;
    const int x = x0 + xx;
    const int s = fsx[xx];
    const float4 w = fwx[xx];
    for (int r = tid / TX; r < TY * TZ; r += NT / TX) {
        const int yy = r % TY, zz = r / TY;
        if (xx >= ex || yy >= ey || zz >= ez) continue;
        const int y = y0 + yy, z = z0 + zz;
        float p[3];
#pragma unroll
        for (int comp = 0; comp < D; ++comp) {
            const float *c = T2 + ((comp * TZ + zz) * TY + yy) * FX + s;
            const float u = w.x * c[0] + w.y * c[1] + w.z * c[2] + w.w * c[3];
            p[comp] = float(comp == 0 ? x : (comp == 1 ? y : z)) - u;
        }
        const int fx = ffloor16(p[0]), fy = ffloor16(p[1]), fz = (D == 3) ? ffloor16(p[2]) : 0;
        float wv;
        const bool in_box = staged && fx - 1 >= lo[0] && fx + 2 <= hi[0] && fy - 1 >= lo[1] && fy + 2 <= hi[1] &&
                            (D == 2 || (fz - 1 >= lo[2] && fz + 2 <= hi[2]));
        if (in_box) {
            const int pz = (D == 3) ? fz - 1 - lo[2] : 0;
            const float *base = Fp + (pz * SBY + (fy - 1 - lo[1])) * SBX + (fx - 1 - sx0);
            if (D == 3)
                wv = staged_sample3(base, SBX, SBX * SBY, p[0], p[1], p[2], fx, fy, fz, mn, mxv);
            else
                wv = staged_sample2(base, SBX, p[0], p[1], fx, fy, mn, mxv);
        } else if (D == 3) {
            wv = sample3(a.coef_img, nx, ny, nz, p[0], p[1], p[2], mn, mxv);
        } else {
            wv = sample2(a.coef_img, nx, ny, p[0], p[1], mn, mxv);
        }
        const size_t idx = (size_t(z) * ny + y) * nx + x;
        a.warped[idx] = wv;
        const float b = a.ref[idx];
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
    double dv[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) dv[k] = acc[k];
    block_sum<5>(dv, red);
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < 5; ++k) a.tile_sums[size_t(tile) * 5 + k] = dv[k];
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
template <int D, int TX, int TY, int TZ>
__device__ __forceinline__ void adjoint_body(const EvalArgs &a, int bx, int by, int bz, int tile_index)
{
    extern __shared__ __align__(128) float sm[];
    constexpr int HX = TX + 2, HY = TY + 2, HZ = (D == 3) ? TZ + 2 : 1;
    constexpr int TXP = TX + 1;
    __shared__ int asx[TX], asy[TY], asz[TZ];
    __shared__ float4 awx[TX], awy[TY], awz[TZ];
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int nx = a.n[0], ny = a.n[1], nz = (D == 3) ? a.n[2] : 1;
    const int x0 = bx * TX, y0 = by * TY, z0 = bz * TZ;
    const int ex = min(TX, nx - x0), ey = min(TY, ny - y0), ez = min(TZ, nz - z0);
    const int AXc = X.ac, AYc = Y.ac, AZc = (D == 3) ? Z.ac : 1;
    const int ax0 = X.atile0[bx], ay0 = Y.atile0[by], az0 = (D == 3) ? Z.atile0[bz] : 0;
    const int tid = threadIdx.x;
    float *part = a.partial + size_t(tile_index) * a.slot;

    float *Wh = sm;                          // [HZ][HY][HX]
    float *F = Wh + HZ * HY * HX;            // [D][TZ][TY][TXP]
    float *AX = F + D * TZ * TY * TXP;       // [D][TZ][TY][AXc]
    float *AY = AX + D * TZ * TY * AXc;      // [D][TZ][AYc][AXc]   (3D)

    if (tid < TX) {
        const int x = min(x0 + tid, nx - 1);
        asx[tid] = X.as[x] - ax0;
        awx[tid] = X.aw[x];
    }
    if (tid < TY) {
        const int y = min(y0 + tid, ny - 1);
        asy[tid] = Y.as[y] - ay0;
        awy[tid] = Y.aw[y];
    }
    if (D == 3 && tid < TZ) {
        const int z = min(z0 + tid, nz - 1);
        asz[tid] = Z.as[z] - az0;
        awz[tid] = Z.aw[z];
    }
    // warped image with a one-voxel halo, zero outside the image
    for (int e = tid; e < HZ * HY * HX; e += NT) {
        const int hx = e % HX, hy = (e / HX) % HY, hz = e / (HX * HY);
        const int x = x0 - 1 + hx, y = y0 - 1 + hy, z = (D == 3) ? z0 - 1 + hz : 0;
        float v = 0.0f;
        if (x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz) v = a.warped[(size_t(z) * ny + y) * nx + x];
        Wh[e] = v;
    }
    __syncthreads();
    {
        const double *sc = a.scalars;
        const float k1 = float(sc[SC_K1]), k2 = float(sc[SC_K2]);
        const float ma = float(sc[SC_MA]), mb = float(sc[SC_MB]), fscale = float(sc[SC_FSCALE]);
        constexpr int NV = TX * TY * TZ;
        for (int v = tid; v < NV; v += NT) {
            const int xx = v % TX, yy = (v / TX) % TY, zz = v / (TX * TY);
            float f[3] = {0.0f, 0.0f, 0.0f};
            if (xx < ex && yy < ey && zz < ez) {
                const int x = x0 + xx, y = y0 + yy, z = z0 + zz;
                const int c = (((D == 3) ? zz + 1 : 0) * HY + yy + 1) * HX + xx + 1;
                const float w = Wh[c];
                float g[3];
                g[0] = (x > 0 && x < nx - 1) ? 0.5f * (Wh[c + 1] - Wh[c - 1]) : 0.0f;
                g[1] = (y > 0 && y < ny - 1) ? 0.5f * (Wh[c + HX] - Wh[c - HX]) : 0.0f;
                if (D == 3) g[2] = (z > 0 && z < nz - 1) ? 0.5f * (Wh[c + HX * HY] - Wh[c - HX * HY]) : 0.0f;
                const float b = a.ref[(size_t(z) * ny + y) * nx + x];
                if (a.cost == 0) {
                    const float d = w - b;
#pragma unroll
                    for (int k = 0; k < D; ++k) f[k] = (g[k] * d) * fscale;
                } else {
                    const float s = k1 * (k2 * (w - ma) - (b - mb));
#pragma unroll
                    for (int k = 0; k < D; ++k) f[k] = s * g[k];
                }
            }
#pragma unroll
            for (int k = 0; k < D; ++k) F[((k * TZ + zz) * TY + yy) * TXP + xx] = f[k];
        }
    }
    __syncthreads();
    // x: rows (comp, zz, yy)
    for (int r = tid; r < D * TZ * TY; r += NT) {
        float *out = AX + r * AXc;
        window_contract(ex, asx, awx, F + r * TXP, 1, AXc, [&](int o, float v) { out[o] = v; });
    }
    __syncthreads();
    // y: columns (comp*TZ + zz, ox)
    for (int c = tid; c < D * TZ * AXc; c += NT) {
        const int ox = c % AXc, cz = c / AXc;
        const float *in = AX + cz * TY * AXc + ox;
        if (D == 3) {
            float *out = AY + cz * AYc * AXc + ox;
            window_contract(ey, asy, awy, in, AXc, AYc, [&](int o, float v) { out[o * AXc] = v; });
        } else {
            const int comp = cz;
            window_contract(ey, asy, awy, in, AXc, AYc,
                            [&](int o, float v) { part[(size_t(o) * AXc + ox) * D + comp] = v; });
        }
    }
    if (D == 3) {
        __syncthreads();
        // z: columns (oy, ox, comp), comp fastest so the slot writes coalesce
        for (int c = tid; c < D * AYc * AXc; c += NT) {
            const int comp = c % D, rest = c / D;
            const int ox = rest % AXc, oy = rest / AXc;
            const float *in = AY + (comp * TZ * AYc + oy) * AXc + ox;
            window_contract(ez, asz, awz, in, AYc * AXc, AZc, [&](int o, float v) {
                part[((size_t(o) * AYc + oy) * AXc + ox) * D + comp] = v;
            });
        }
    }
}

// ---------------------------------------------------------------------
// kernels: one pair (grid = tiles) and a batch of pairs (grid = work list
// of (pair, tile) items; pairs whose minimizer has finished are skipped)
// ---------------------------------------------------------------------
template <int D, int TX, int TY, int TZ>
__global__ void __launch_bounds__(NT) k_warp_t(EvalArgs a)
{
    const int tile = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    warp_body<D, TX, TY, TZ>(a, blockIdx.x, blockIdx.y, D == 3 ? blockIdx.z : 0,
                             gridDim.x * gridDim.y * gridDim.z, tile);
}

template <int D, int TX, int TY, int TZ>
__global__ void __launch_bounds__(NT) k_adjoint_t(EvalArgs a)
{
    const int tile = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    adjoint_body<D, TX, TY, TZ>(a, blockIdx.x, blockIdx.y, D == 3 ? blockIdx.z : 0, tile);
}

__device__ __forceinline__ void decode_tile(const EvalArgs &a, int D, int t, int &bx, int &by, int &bz, int &nt)
{
    const int ntx = a.ax[0].nt, nty = a.ax[1].nt, ntz = D == 3 ? a.ax[2].nt : 1;
    bx = t % ntx;
    by = (t / ntx) % nty;
    bz = t / (ntx * nty);
    nt = ntx * nty * ntz;
}

template <int D, int TX, int TY, int TZ>
__global__ void __launch_bounds__(NT) k_warp_batch(const EvalArgs *__restrict__ args, const int2 *__restrict__ items,
                                                   const int *__restrict__ active)
{
    const int2 it = items[blockIdx.x];
    if (!active[it.x]) return;
    const EvalArgs &a = args[it.x];
    int bx, by, bz, nt;
    decode_tile(a, D, it.y, bx, by, bz, nt);
    warp_body<D, TX, TY, TZ>(a, bx, by, bz, nt, it.y);
}

template <int D, int TX, int TY, int TZ>
__global__ void __launch_bounds__(NT) k_adjoint_batch(const EvalArgs *__restrict__ args,
                                                      const int2 *__restrict__ items, const int *__restrict__ active)
{
    const int2 it = items[blockIdx.x];
    if (!active[it.x]) return;
    const EvalArgs &a = args[it.x];
    int bx, by, bz, nt;
    decode_tile(a, D, it.y, bx, by, bz, nt);
    adjoint_body<D, TX, TY, TZ>(a, bx, by, bz, it.y);
}

// ---------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------
static size_t warp_smem(const EvalArgs &a)
{
    const int D = a.dim;
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int TZ = (D == 3) ? Z.t : 1, FZ = (D == 3) ? Z.fc : 1;
    size_t f = size_t(D) * FZ * Y.fc * X.fc;
    if (D == 3) f += size_t(D) * TZ * Y.fc * X.fc;
    f += size_t(D) * TZ * Y.t * X.fc;
    f = (f + 31) & ~size_t(31);
    f += stage_floats(D, X.t, Y.t, D == 3 ? Z.t : 1);
    return f * sizeof(float);
}

static size_t adjoint_smem(const EvalArgs &a)
{
    const int D = a.dim;
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int TZ = (D == 3) ? Z.t : 1, HZ = (D == 3) ? Z.t + 2 : 1;
    size_t f = size_t(HZ) * (Y.t + 2) * (X.t + 2);
    f += size_t(D) * TZ * Y.t * (X.t + 1);
    f += size_t(D) * TZ * Y.t * X.ac;
    if (D == 3) f += size_t(D) * TZ * Y.ac * X.ac;
    return f * sizeof(float);
}

static dim3 tile_grid(const EvalArgs &a)
{
    return dim3(a.ax[0].nt, a.ax[1].nt, a.dim == 3 ? a.ax[2].nt : 1);
}

template <int D, int TX, int TY, int TZ>
static void launch_tile(const EvalArgs &a, int which, cudaStream_t st)
{
    if (which == 0) {
        const size_t sm = warp_smem(a);
        raise_smem_limit(reinterpret_cast<const void *>(k_warp_t<D, TX, TY, TZ>), sm);
        k_warp_t<D, TX, TY, TZ><<<tile_grid(a), NT, sm, st>>>(a);
    } else {
        const size_t sm = adjoint_smem(a);
        raise_smem_limit(reinterpret_cast<const void *>(k_adjoint_t<D, TX, TY, TZ>), sm);
        k_adjoint_t<D, TX, TY, TZ><<<tile_grid(a), NT, sm, st>>>(a);
    }
    count_launch();
}

// the 2D tile shapes compiled in (tile_supported() must match); 3D runs
// the z-walking kernels of split3.cu
static bool dispatch(const EvalArgs &a, int which, cudaStream_t st)
{
    if (a.dim == 3) {
        if (which == 0)
            launch_warp3(a, st);
        else
            launch_adjoint3(a, st);
        return true;
    }
    const int tx = a.ax[0].t, ty = a.ax[1].t;
#define MGR_TILE2(X_, Y_)                                  \
    if (tx == X_ && ty == Y_) {                            \
        launch_tile<2, X_, Y_, 1>(a, which, st);           \
        return true;                                       \
    }
    MGR_TILE2(32, 8)
    MGR_TILE2(32, 16)
    MGR_TILE2(64, 8)
    MGR_TILE2(64, 16)
    MGR_TILE2(32, 32)
#undef MGR_TILE2
    return false;
}

bool tile_supported(int dim, int tx, int ty, int tz)
{
    static const int t2[][2] = {{32, 8}, {32, 16}, {64, 8}, {64, 16}, {32, 32}};
    if (dim == 3) return tile_supported3(tx, ty, tz);
    for (auto &t : t2)
        if (t[0] == tx && t[1] == ty) return true;
    return false;
}

void launch_warp(const EvalArgs &a, cudaStream_t st)
{
    dispatch(a, 0, st);
}

void launch_adjoint(const EvalArgs &a, cudaStream_t st)
{
    dispatch(a, 1, st);
}

size_t split_smem(const EvalArgs &a, int which)
{
    if (a.dim == 3) return split3_smem(a, which);
    return which == 0 ? warp_smem(a) : adjoint_smem(a);
}

template <int D, int TX, int TY, int TZ>
static void launch_batch_tile(const EvalArgs *args, const int2 *items, int nitems, const int *active,
                              size_t sm, int which, cudaStream_t st)
{
    if (which == 0)
        k_warp_batch<D, TX, TY, TZ><<<nitems, NT, sm, st>>>(args, items, active);
    else
        k_adjoint_batch<D, TX, TY, TZ><<<nitems, NT, sm, st>>>(args, items, active);
    count_launch();
}

template <int D, int TX, int TY, int TZ>
static void prepare_batch_tile(size_t sm_warp, size_t sm_adj)
{
    cudaFuncSetAttribute(k_warp_batch<D, TX, TY, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm_warp));
    cudaFuncSetAttribute(k_adjoint_batch<D, TX, TY, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm_adj));
}

void prepare_split_batch(int dim, int tx, int ty, int tz, size_t sm_warp, size_t sm_adj)
{
    if (dim == 3) {
        prepare_split3_batch(tz, sm_warp, sm_adj);
        return;
    }
#define MGR_PTILE2(X_, Y_) \
    if (tx == X_ && ty == Y_) prepare_batch_tile<2, X_, Y_, 1>(sm_warp, sm_adj);
    MGR_PTILE2(32, 8)
    MGR_PTILE2(32, 16)
    MGR_PTILE2(64, 8)
    MGR_PTILE2(64, 16)
    MGR_PTILE2(32, 32)
#undef MGR_PTILE2
}

bool launch_split_batch(int dim, int tx, int ty, int tz, const EvalArgs *args, const int2 *items, int nitems,
                        const int *active, size_t sm, int which, cudaStream_t st)
{
    if (dim == 3) {
        if (!tile_supported3_batch(tx, ty, tz)) return false;
        launch_split3_batch(tz, args, items, nitems, active, sm, which, st);
        return true;
    }
#define MGR_BTILE2(X_, Y_)                                                      \
    if (tx == X_ && ty == Y_) {                                                 \
        launch_batch_tile<2, X_, Y_, 1>(args, items, nitems, active, sm, which, st); \
        return true;                                                            \
    }
    MGR_BTILE2(32, 8)
    MGR_BTILE2(32, 16)
    MGR_BTILE2(64, 8)
    MGR_BTILE2(64, 16)
    MGR_BTILE2(32, 32)
#undef MGR_BTILE2
    return false;
}

}  // namespace mgr
