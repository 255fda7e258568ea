// eval.cu — cost+gradient kernels of the spline registration path.
//
// SPLIT path (per evaluation, three launches):
//   k_warp<D>    per voxel tile: displacement u(x) by separable contraction
//                of the tile's coefficient footprint in shared memory, the
//                tricubic B-spline sample of the prefiltered moving image at
//                x - u(x) (mirror boundary, clamp), the warped image, and
//                the SSD / NCC sums; the last block finalises the cost.
//   k_adjoint<D> per voxel tile: central-difference gradient of the warped
//                image (normal component zero on faces), the SSD / NCC
//                force, and the separable transposed B-spline contraction of
//                the force onto the tile's coefficient footprint, written to
//                the tile's partial slot (no atomics).
//   k_gather<D>  per coefficient: fixed-order sum of the partial slots that
//                hold it (deterministic), the divcurl penalty value and
//                gradient, and the weighted total gradient.
//
// Reference routines restated: C3DSplineTransformation::init_grid
// (mia/3d/transform/spline.cc:541-653), the warp (mia/3d/transform.cc:280-353,
// mia/3d/interpolator.cxx:250-287), get_gradient (mia/3d/image.cc:347-466),
// the SSD force (mia/template/ssd.hh:126-181), the NCC force
// (mia/3d/cost/ncc.cc:88-128, mia/core/nccsum.cc:31-120), translate
// (spline.cc:731-791), and C3DPPDivcurlMatrixImpl::evaluate / multiply
// (mia/3d/ppmatrix.cc:292-599); 2D counterparts in mia/2d/.
#include "mgr_common.cuh"
#include "mgr_kernels.hh"

namespace mgr {

namespace {

__device__ __forceinline__ float aw_at(const float4 *aw, int i, int k)
{
    return reinterpret_cast<const float *>(aw)[i * 4 + k];
}

// final cost from the reduced sums; thread 0 of the last block only
__device__ void finalise_cost(const EvalArgs &a, const double s[5], size_t N)
{
    double *sc = a.scalars;
    if (a.cost == 0) {
        const double scale = a.ssd_norm ? 0.5 / double(N) : 0.5;
        sc[SC_VALUE] = scale * s[0];
        sc[SC_FORCE_COST] = scale * s[0];
        sc[SC_FSCALE] = a.ssd_norm ? double(float(1.0 / double(N))) : 1.0;
        sc[SC_K1] = sc[SC_K2] = sc[SC_MA] = sc[SC_MB] = 0.0;
    } else {
        // sums of da = a - ca, db = b - cb (centred to limit cancellation)
        const double n = double(N);
        const double sa = s[0], sb = s[1], saa = s[2], sbb = s[3], sab = s[4];
        const double ma = a.center_a + sa / n, mb = a.center_b + sb / n;
        const double s2a = saa - sa * sa / n;
        const double s2b = sbb - sb * sb / n;
        const double cab = sab - sa * sb / n;
        const double p1 = s2a * s2b;
        double v = 1.0;
        if (p1 > 1e-10) v = 1.0 - cab * cab / p1;
        else if (s2a < 1e-5 && s2b < 1e-5) v = 0.0;
        sc[SC_VALUE] = v;
        double fv = 1.0, k1 = 0.0, k2 = 0.0, hma = 0.0, hmb = 0.0;
        if (p1 > 1e-5) {
            fv = 1.0 - cab * cab / p1;
            k1 = 2.0 * (cab / p1);
            k2 = cab / s2a;
            hma = ma;
            hmb = mb;
        } else if (s2a < 1e-5 && s2b < 1e-5) {
            fv = 0.0;
        }
        sc[SC_FORCE_COST] = fv;
        sc[SC_K1] = k1;
        sc[SC_K2] = k2;
        sc[SC_MA] = hma;
        sc[SC_MB] = hmb;
        sc[SC_FSCALE] = 1.0;
    }
}

// reduce per-tile sums in a fixed order; called by every thread of the last
// block
__device__ void reduce_tile_sums(const EvalArgs &a, int ntiles, size_t N, double *red)
{
    double v[5] = {0, 0, 0, 0, 0};
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
        const volatile double *p = a.tile_sums + size_t(t) * 5;
#pragma unroll
        for (int k = 0; k < 5; ++k) v[k] += p[k];
    }
    block_sum<5>(v, red);
    if (threadIdx.x == 0) finalise_cost(a, v, N);
}

}  // namespace

// ---------------------------------------------------------------------
// warp
// ---------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(256) k_warp(EvalArgs a)
{
    extern __shared__ float sm[];
    __shared__ double red[5 * 8];
    __shared__ bool is_last;
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int nx = a.n[0], ny = a.n[1], nz = (D == 3) ? a.n[2] : 1;
    const int TX = X.t, TY = Y.t, TZ = (D == 3) ? Z.t : 1;
    const int bx = blockIdx.x, by = blockIdx.y, bz = (D == 3) ? blockIdx.z : 0;
    const int x0 = bx * TX, y0 = by * TY, z0 = bz * TZ;
    const int ex = min(TX, nx - x0), ey = min(TY, ny - y0), ez = min(TZ, nz - z0);
    const int FX = X.fc, FY = Y.fc, FZ = (D == 3) ? Z.fc : 1;
    const int cx0 = X.ftile0[bx], cy0 = Y.ftile0[by], cz0 = (D == 3) ? Z.ftile0[bz] : 0;
    const int ncx = a.nc[0], ncy = a.nc[1], ncz = (D == 3) ? a.nc[2] : 1;

    float *C = sm;                                   // D x FZ x FY x FX
    float *T1 = C + D * FZ * FY * FX;                // D x TZ x FY x FX   (3D)
    float *T2 = T1 + ((D == 3) ? D * TZ * FY * FX : 0); // D x TZ x TY x FX
    const int fbox = FZ * FY * FX;

    // coefficient footprint (params are double, interleaved per node)
    for (int e = threadIdx.x; e < D * fbox; e += blockDim.x) {
        const int comp = e / fbox, r = e - comp * fbox;
        const int iz = r / (FY * FX), iy = (r / FX) % FY, ix = r % FX;
        const int gx = cx0 + ix, gy = cy0 + iy, gz = cz0 + iz;
        float v = 0.0f;
        if (gx < ncx && gy < ncy && gz < ncz)
            v = float(a.params[((size_t(gz) * ncy + gy) * ncx + gx) * D + comp]);
        C[e] = v;
    }
    __syncthreads();
    const float *Cy = C;   // source of the y stage
    if (D == 3) {
        const int nt1 = D * TZ * FY * FX;
        for (int e = threadIdx.x; e < nt1; e += blockDim.x) {
            const int comp = e / (TZ * FY * FX), r = e % (TZ * FY * FX);
            const int zz = r / (FY * FX), iy = (r / FX) % FY, ix = r % FX;
            float v = 0.0f;
            if (zz < ez) {
                const int z = z0 + zz;
                const int s = Z.fs[z] - cz0;
                const float4 w = Z.fw[z];
                const float *c = C + comp * fbox + iy * FX + ix;
                v = w.x * c[(s)*FY * FX] + w.y * c[(s + 1) * FY * FX] + w.z * c[(s + 2) * FY * FX] +
                    w.w * c[(s + 3) * FY * FX];
            }
            T1[e] = v;
        }
        __syncthreads();
        Cy = T1;
    }
    {
        const int nt2 = D * TZ * TY * FX;
        for (int e = threadIdx.x; e < nt2; e += blockDim.x) {
            const int comp = e / (TZ * TY * FX), r = e % (TZ * TY * FX);
            const int zz = r / (TY * FX), yy = (r / FX) % TY, ix = r % FX;
            float v = 0.0f;
            if (zz < ez && yy < ey) {
                const int y = y0 + yy;
                const int s = Y.fs[y] - cy0;
                const float4 w = Y.fw[y];
                const float *c = Cy + (comp * TZ + zz) * FY * FX + ix;
                if (D == 2) c = Cy + comp * fbox + ix;
                v = w.x * c[s * FX] + w.y * c[(s + 1) * FX] + w.z * c[(s + 2) * FX] + w.w * c[(s + 3) * FX];
            }
            T2[e] = v;
        }
    }
    __syncthreads();

    // x stage, sample, write, sums
    float acc[5] = {0, 0, 0, 0, 0};
    const float mn = a.minmax[0], mxv = a.minmax[1];
    const float ca = float(a.center_a), cb = float(a.center_b);
    const int nvox = TZ * TY * TX;
    for (int v = threadIdx.x; v < nvox; v += blockDim.x) {
        const int zz = v / (TY * TX), yy = (v / TX) % TY, xx = v % TX;
        if (zz >= ez || yy >= ey || xx >= ex) continue;
        const int x = x0 + xx, y = y0 + yy, z = z0 + zz;
        const int s = X.fs[x] - cx0;
        const float4 w = X.fw[x];
        float u[3];
#pragma unroll
        for (int comp = 0; comp < D; ++comp) {
            const float *c = T2 + ((comp * TZ + zz) * TY + yy) * FX + s;
            u[comp] = w.x * c[0] + w.y * c[1] + w.z * c[2] + w.w * c[3];
        }
        float wv;
        if (D == 3)
            wv = sample3(a.coef_img, nx, ny, nz, float(x) - u[0], float(y) - u[1], float(z) - u[2], mn, mxv);
        else
            wv = sample2(a.coef_img, nx, ny, float(x) - u[0], float(y) - u[1], mn, mxv);
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
    const int ntiles = gridDim.x * gridDim.y * gridDim.z;
    const int tile = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 5; ++k) a.tile_sums[size_t(tile) * 5 + k] = dv[k];
        __threadfence();
        is_last = (atomicAdd(&a.counters[0], 1u) == unsigned(ntiles - 1));
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        reduce_tile_sums(a, ntiles, size_t(nx) * ny * nz, red);
        if (threadIdx.x == 0) a.counters[0] = 0;
    }
}

// ---------------------------------------------------------------------
// gradient + force + adjoint onto the tile's coefficient footprint
// ---------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void voxel_force(const EvalArgs &a, const float *Wh, int hx, int hy, int hz,
                                            int HX, int HY, int x, int y, int z, float sc_a, float k2,
                                            float ma, float mb, float fscale, float F[3])
{
    const int nx = a.n[0], ny = a.n[1], nz = (D == 3) ? a.n[2] : 1;
    const int c = (hz * HY + hy) * HX + hx;
    const float w = Wh[c];
    float g[3];
    g[0] = (x > 0 && x < nx - 1) ? 0.5f * (Wh[c + 1] - Wh[c - 1]) : 0.0f;
    g[1] = (y > 0 && y < ny - 1) ? 0.5f * (Wh[c + HX] - Wh[c - HX]) : 0.0f;
    if (D == 3) g[2] = (z > 0 && z < nz - 1) ? 0.5f * (Wh[c + HX * HY] - Wh[c - HX * HY]) : 0.0f;
    const float b = a.ref[(size_t(z) * ny + y) * nx + x];
    if (a.cost == 0) {
        const float d = w - b;
#pragma unroll
        for (int k = 0; k < D; ++k) F[k] = (g[k] * d) * fscale;
    } else {
        const float s = sc_a * (k2 * (w - ma) - (b - mb));
#pragma unroll
        for (int k = 0; k < D; ++k) F[k] = s * g[k];
    }
}

template <int D>
__global__ void __launch_bounds__(256) k_adjoint(EvalArgs a)
{
    extern __shared__ float sm[];
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int nx = a.n[0], ny = a.n[1], nz = (D == 3) ? a.n[2] : 1;
    const int TX = X.t, TY = Y.t, TZ = (D == 3) ? Z.t : 1;
    const int bx = blockIdx.x, by = blockIdx.y, bz = (D == 3) ? blockIdx.z : 0;
    const int x0 = bx * TX, y0 = by * TY, z0 = bz * TZ;
    const int ex = min(TX, nx - x0), ey = min(TY, ny - y0), ez = min(TZ, nz - z0);
    const int AXc = X.ac, AYc = Y.ac, AZc = (D == 3) ? Z.ac : 1;
    const int ax0 = X.atile0[bx], ay0 = Y.atile0[by], az0 = (D == 3) ? Z.atile0[bz] : 0;
    const int HX = TX + 2, HY = TY + 2, HZ = (D == 3) ? TZ + 2 : 1;

    float *Wh = sm;                              // HZ x HY x HX
    float *F = Wh + HZ * HY * HX;                // D x TZ x TY x TX
    float *AX = F + D * TZ * TY * TX;            // D x TZ x TY x AXc
    float *AY = AX + D * TZ * TY * AXc;          // D x TZ x AYc x AXc (3D)

    // warped image with a one-voxel halo (clamped to the image)
    for (int e = threadIdx.x; e < HZ * HY * HX; e += blockDim.x) {
        const int hz = e / (HY * HX), hy = (e / HX) % HY, hx = e % HX;
        const int x = x0 - 1 + hx, y = y0 - 1 + hy, z = (D == 3) ? z0 - 1 + hz : 0;
        float v = 0.0f;
        if (x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz) v = a.warped[(size_t(z) * ny + y) * nx + x];
        Wh[e] = v;
    }
    __syncthreads();
    const double *sc = a.scalars;
    const float k1 = float(sc[SC_K1]), k2 = float(sc[SC_K2]);
    const float ma = float(sc[SC_MA]), mb = float(sc[SC_MB]), fscale = float(sc[SC_FSCALE]);
    const int nvox = TZ * TY * TX;
    for (int v = threadIdx.x; v < nvox; v += blockDim.x) {
        const int zz = v / (TY * TX), yy = (v / TX) % TY, xx = v % TX;
        float f[3] = {0.0f, 0.0f, 0.0f};
        if (zz < ez && yy < ey && xx < ex)
            voxel_force<D>(a, Wh, xx + 1, yy + 1, (D == 3) ? zz + 1 : 0, HX, HY, x0 + xx, y0 + yy, z0 + zz, k1,
                           k2, ma, mb, fscale, f);
#pragma unroll
        for (int k = 0; k < D; ++k) F[k * nvox + v] = f[k];
    }
    __syncthreads();
    // x contraction
    {
        const int n = D * TZ * TY * AXc;
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            const int comp = e / (TZ * TY * AXc), r = e % (TZ * TY * AXc);
            const int zz = r / (TY * AXc), yy = (r / AXc) % TY, ox = r % AXc;
            const int o = ax0 + ox;
            float s = 0.0f;
            if (o < a.nc[0]) {
                const int2 row = X.rows[o];
                const int i0 = max(row.x, x0), i1 = min(row.x + row.y, x0 + ex);
                const float *f = F + comp * nvox + (zz * TY + yy) * TX;
                for (int i = i0; i < i1; ++i) s += aw_at(X.aw, i, o - X.as[i]) * f[i - x0];
            }
            AX[e] = s;
        }
    }
    __syncthreads();
    // y contraction
    float *outY = (D == 3) ? AY : nullptr;
    {
        const int n = D * TZ * AYc * AXc;
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            const int comp = e / (TZ * AYc * AXc), r = e % (TZ * AYc * AXc);
            const int zz = r / (AYc * AXc), oy = (r / AXc) % AYc, ox = r % AXc;
            const int o = ay0 + oy;
            float s = 0.0f;
            if (o < a.nc[1]) {
                const int2 row = Y.rows[o];
                const int i0 = max(row.x, y0), i1 = min(row.x + row.y, y0 + ey);
                const float *f = AX + (comp * TZ + zz) * TY * AXc + ox;
                for (int i = i0; i < i1; ++i) s += aw_at(Y.aw, i, o - Y.as[i]) * f[(i - y0) * AXc];
            }
            if (D == 3) {
                outY[e] = s;
            } else {
                const int tile = blockIdx.y * gridDim.x + blockIdx.x;
                a.partial[size_t(tile) * a.slot + (size_t(oy) * AXc + ox) * D + comp] = s;
            }
        }
    }
    if (D == 3) {
        __syncthreads();
        const int n = D * AZc * AYc * AXc;
        const int tile = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            const int comp = e / (AZc * AYc * AXc), r = e % (AZc * AYc * AXc);
            const int oz = r / (AYc * AXc), oy = (r / AXc) % AYc, ox = r % AXc;
            const int o = az0 + oz;
            float s = 0.0f;
            if (o < a.nc[2]) {
                const int2 row = Z.rows[o];
                const int i0 = max(row.x, z0), i1 = min(row.x + row.y, z0 + ez);
                const float *f = AY + comp * TZ * AYc * AXc + oy * AXc + ox;
                for (int i = i0; i < i1; ++i) s += aw_at(Z.aw, i, o - Z.as[i]) * f[(i - z0) * AYc * AXc];
            }
            a.partial[size_t(tile) * a.slot + ((size_t(oz) * AYc + oy) * AXc + ox) * D + comp] = s;
        }
    }
}

// ---------------------------------------------------------------------
// gather + divcurl penalty + costs
// ---------------------------------------------------------------------
// P table (3D): cell (dx,dy,dz) at ((dz*9 + dy)*9 + dx)*6 holding
// (xx, xy, yy, yz, zz, xz).
template <int D>
__global__ void __launch_bounds__(256) k_gather(EvalArgs a, int with_gradient, int image_from_dense)
{
    extern __shared__ float sm[];     // 3D penalty table
    __shared__ double red[8];
    __shared__ bool is_last;
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int ncx = a.nc[0], ncy = a.nc[1], ncz = (D == 3) ? a.nc[2] : 1;
    const size_t ncoef = size_t(ncx) * ncy * ncz;
    if (D == 3 && a.has_penalty) {
        for (int e = threadIdx.x; e < 9 * 9 * 9 * 6; e += blockDim.x) sm[e] = a.ptable[e];
        __syncthreads();
    }
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    float pval = 0.0f;
    if (i < ncoef) {
        const int cx = int(i % ncx), cy = int((i / ncx) % ncy), cz = (D == 3) ? int(i / (size_t(ncx) * ncy)) : 0;
        double gimg[3] = {0.0, 0.0, 0.0};
        if (with_gradient) {
            if (image_from_dense) {
#pragma unroll
                for (int k = 0; k < D; ++k) gimg[k] = a.grad_image[i * D + k];
            } else {
                float s[3] = {0.0f, 0.0f, 0.0f};
                const int2 gx = X.gtile[cx], gy = Y.gtile[cy];
                const int2 gz = (D == 3) ? Z.gtile[cz] : make_int2(0, 0);
                const int AXc = X.ac, AYc = Y.ac;
                for (int tz = gz.x; tz <= gz.y; ++tz) {
                    const int lz = (D == 3) ? cz - Z.atile0[tz] : 0;
                    for (int ty = gy.x; ty <= gy.y; ++ty) {
                        const int ly = cy - Y.atile0[ty];
                        for (int tx = gx.x; tx <= gx.y; ++tx) {
                            const int lx = cx - X.atile0[tx];
                            const size_t t = (size_t(tz) * Y.nt + ty) * X.nt + tx;
                            const float *p = a.partial + t * a.slot + ((size_t(lz) * AYc + ly) * AXc + lx) * D;
#pragma unroll
                            for (int k = 0; k < D; ++k) s[k] += p[k];
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < D; ++k) gimg[k] = a.cost_weight * (-double(s[k]));
            }
        }
        double gpen[3] = {0.0, 0.0, 0.0};
        if (a.has_penalty) {
            float g[3] = {0.0f, 0.0f, 0.0f};
            float ci[3];
#pragma unroll
            for (int k = 0; k < D; ++k) ci[k] = float(a.params[i * D + k]);
            if (D == 3) {
                float r0 = 0, r1 = 0, r2 = 0, r3 = 0, r4 = 0, r5 = 0;
                const int ks = 4;
                for (int zj = max(0, cz - ks); zj < min(cz + ks, ncz); ++zj) {
                    const int dz = cz - zj + ks;
                    for (int yj = max(0, cy - ks); yj < min(cy + ks, ncy); ++yj) {
                        const int dy = cy - yj + ks;
                        const int xs = max(0, cx - ks), xe = min(cx + ks, ncx);
                        const double *pj = a.params + ((size_t(zj) * ncy + yj) * ncx) * 3;
                        for (int xj = xs; xj < xe; ++xj) {
                            const float *P = sm + ((dz * 9 + dy) * 9 + (cx - xj + ks)) * 6;
                            const float cjx = float(pj[xj * 3]), cjy = float(pj[xj * 3 + 1]), cjz = float(pj[xj * 3 + 2]);
                            const float vxx = P[0], vxy = P[1], vyy = P[2], vyz = P[3], vzz = P[4], vxz = P[5];
                            if (with_gradient) {
                                const float ax = vxx * cjx, az = vxz * cjx;
                                const float bxy = vxy * cjy, byy = vyy * cjy;
                                const float cyz = vyz * cjz, czz = vzz * cjz;
                                r0 += ax; r1 += bxy; r2 += byy; r3 += cyz; r4 += czz; r5 += az;
                                g[0] += cjz * vxz + (2.0f * ax + bxy);
                                g[1] += cjx * vxy + (2.0f * byy + cyz);
                                g[2] += cjy * vyz + (2.0f * czz + az);
                            } else {
                                // operator* cross terms: ci.x cj.y vxy, ci.x cj.z vxz, ci.y cj.z vyz
                                r0 += cjx * vxx; r2 += cjy * vyy; r4 += cjz * vzz;
                                r1 += cjy * vxy; r5 += cjz * vxz; r3 += cjz * vyz;
                            }
                        }
                    }
                }
                if (with_gradient)
                    pval = ci[0] * r0 + ci[0] * r1 + ci[1] * r2 + ci[1] * r3 + ci[2] * r4 + ci[2] * r5;
                else
                    pval = ci[0] * r0 + ci[1] * r2 + ci[2] * r4 + ci[0] * r1 + ci[0] * r5 + ci[1] * r3;
            } else {
                float r1 = 0, r2 = 0, r3 = 0;
                for (int e = a.pen_rowptr[i]; e < a.pen_rowptr[i + 1]; ++e) {
                    const int j = a.pen_col[e];
                    const float4 v = a.pen_val[e];
                    const float cjx = float(a.params[size_t(j) * 2]), cjy = float(a.params[size_t(j) * 2 + 1]);
                    const float aa = cjx * v.x, bb = cjy * v.y, cxx = cjx * v.z, cyy = cjy * v.z;
                    g[0] += aa + aa + cyy;
                    g[1] += bb + bb + cxx;
                    r1 += aa;
                    r2 += cyy;
                    r3 += bb;
                }
                pval = ci[0] * r1 + ci[0] * r2 + ci[1] * r3;
            }
#pragma unroll
            for (int k = 0; k < D; ++k) gpen[k] = -a.pen_weight * double(g[k]);
        }
        if (with_gradient) {
#pragma unroll
            for (int k = 0; k < D; ++k) {
                a.grad_total[i * D + k] = gimg[k] + gpen[k];
                if (a.grad_image && !image_from_dense) a.grad_image[i * D + k] = gimg[k];
                if (a.grad_penalty) a.grad_penalty[i * D + k] = gpen[k];
            }
        }
    }
    // penalty value: block partial, last block reduces in fixed order
    double pv[1] = {double(pval)};
    block_sum<1>(pv, red);
    if (threadIdx.x == 0) {
        a.pen_part[blockIdx.x] = pv[0];
        __threadfence();
        is_last = (atomicAdd(&a.counters[1], 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        double s[1] = {0.0};
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) s[0] += ((volatile double *)a.pen_part)[b];
        block_sum<1>(s, red);
        if (threadIdx.x == 0) {
            double *sc = a.scalars;
            const double pen = a.has_penalty ? s[0] : 0.0;
            sc[SC_PEN] = pen;
            const double img = (D == 2 && with_gradient) ? sc[SC_FORCE_COST] : sc[SC_VALUE];
            sc[SC_COST_IMG] = a.cost_weight * img;
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
// plain per-step kernels (the reference's step structure, one kernel each)
// ---------------------------------------------------------------------
// force field from the warped image (TCost::evaluate_force)
template <int D>
__global__ void __launch_bounds__(256) k_force(EvalArgs a, float *force)
{
    const int nx = a.n[0], ny = a.n[1], nz = (D == 3) ? a.n[2] : 1;
    const size_t N = size_t(nx) * ny * nz;
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= N) return;
    const int x = int(i % nx), y = int((i / nx) % ny), z = int(i / (size_t(nx) * ny));
    const float *W = a.warped;
    float g[3];
    g[0] = (x > 0 && x < nx - 1) ? 0.5f * (W[i + 1] - W[i - 1]) : 0.0f;
    g[1] = (y > 0 && y < ny - 1) ? 0.5f * (W[i + nx] - W[i - nx]) : 0.0f;
    if (D == 3) {
        const size_t sl = size_t(nx) * ny;
        g[2] = (z > 0 && z < nz - 1) ? 0.5f * (W[i + sl] - W[i - sl]) : 0.0f;
    }
    const double *sc = a.scalars;
    const float w = W[i], b = a.ref[i];
    if (a.cost == 0) {
        const float fs = float(sc[SC_FSCALE]);
        const float d = w - b;
#pragma unroll
        for (int k = 0; k < D; ++k) force[i * D + k] = (g[k] * d) * fs;
    } else {
        const float s = float(sc[SC_K1]) * (float(sc[SC_K2]) * (w - float(sc[SC_MA])) - (b - float(sc[SC_MB])));
#pragma unroll
        for (int k = 0; k < D; ++k) force[i * D + k] = s * g[k];
    }
}

// separable translate, one pass per axis.  pass 0 (3D): z rows,
// F[N][3] -> t1[ncz][ny][nx][3]; pass 1: y rows -> t2[ncz][ncy][nx][3];
// pass 2: x rows -> grad (negated, weighted).  2D: pass 1 (y) reads F,
// pass 2 (x) writes grad.
template <int D>
__global__ void __launch_bounds__(256) k_translate_pass(EvalArgs a, int pass, const float *in, float *out,
                                                        double *grad)
{
    const int nx = a.n[0], ny = a.n[1];
    const int ncx = a.nc[0], ncy = a.nc[1], ncz = (D == 3) ? a.nc[2] : 1;
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (pass == 0) {  // 3D only
        const size_t n = size_t(ncz) * ny * nx;
        if (i >= n) return;
        const int x = int(i % nx), y = int((i / nx) % ny), oz = int(i / (size_t(nx) * ny));
        const int2 row = a.ax[2].rows[oz];
        float s[3] = {0, 0, 0};
        for (int z = row.x; z < row.x + row.y; ++z) {
            const float w = aw_at(a.ax[2].aw, z, oz - a.ax[2].as[z]);
            const float *f = in + ((size_t(z) * ny + y) * nx + x) * 3;
            s[0] += w * f[0];
            s[1] += w * f[1];
            s[2] += w * f[2];
        }
        float *o = out + i * 3;
        o[0] = s[0]; o[1] = s[1]; o[2] = s[2];
    } else if (pass == 1) {
        const int nzl = (D == 3) ? ncz : 1;
        const size_t n = size_t(nzl) * ncy * nx;
        if (i >= n) return;
        const int x = int(i % nx), oy = int((i / nx) % ncy), zl = int(i / (size_t(nx) * ncy));
        const int2 row = a.ax[1].rows[oy];
        float s[3] = {0, 0, 0};
        for (int y = row.x; y < row.x + row.y; ++y) {
            const float w = aw_at(a.ax[1].aw, y, oy - a.ax[1].as[y]);
            const float *f = in + ((size_t(zl) * ny + y) * nx + x) * D;
#pragma unroll
            for (int k = 0; k < D; ++k) s[k] += w * f[k];
        }
        float *o = out + i * D;
#pragma unroll
        for (int k = 0; k < D; ++k) o[k] = s[k];
    } else {
        const size_t n = size_t(ncz) * ncy * ncx;
        if (i >= n) return;
        const int ox = int(i % ncx);
        const size_t line = i / ncx;  // (cz, cy)
        const int2 row = a.ax[0].rows[ox];
        float s[3] = {0, 0, 0};
        for (int x = row.x; x < row.x + row.y; ++x) {
            const float w = aw_at(a.ax[0].aw, x, ox - a.ax[0].as[x]);
            const float *f = in + (line * nx + x) * D;
#pragma unroll
            for (int k = 0; k < D; ++k) s[k] += w * f[k];
        }
#pragma unroll
        for (int k = 0; k < D; ++k) grad[i * D + k] = a.cost_weight * (-double(s[k]));
    }
}

// dense displacement grid, one separable pass per kernel (init_grid):
// pass 0: x over coefficients -> t1[ncz][ncy][nx][3]; pass 1: y ->
// t2[ncz][ny][nx][3]; pass 2: z -> grid[N][3] = X - u.
__global__ void __launch_bounds__(256) k_grid_pass(EvalArgs a, int pass, const float *in, float *out)
{
    const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
    const int ncx = a.nc[0], ncy = a.nc[1], ncz = a.nc[2];
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (pass == 0) {
        const size_t n = size_t(ncz) * ncy * nx;
        if (i >= n) return;
        const int x = int(i % nx);
        const size_t line = i / nx;
        const int s = a.ax[0].fs[x];
        const float4 w = a.ax[0].fw[x];
        const float ww[4] = {w.x, w.y, w.z, w.w};
        float r[3] = {0, 0, 0};
        for (int k = 0; k < 4; ++k) {
            const int c = s + k;
            if (c < 0 || c >= ncx) continue;
            const double *p = a.params + (line * ncx + c) * 3;
            r[0] += ww[k] * float(p[0]);
            r[1] += ww[k] * float(p[1]);
            r[2] += ww[k] * float(p[2]);
        }
        out[i * 3] = r[0]; out[i * 3 + 1] = r[1]; out[i * 3 + 2] = r[2];
    } else if (pass == 1) {
        const size_t n = size_t(ncz) * ny * nx;
        if (i >= n) return;
        const int x = int(i % nx), y = int((i / nx) % ny), cz = int(i / (size_t(nx) * ny));
        const int s = a.ax[1].fs[y];
        const float4 w = a.ax[1].fw[y];
        const float ww[4] = {w.x, w.y, w.z, w.w};
        float r[3] = {0, 0, 0};
        for (int k = 0; k < 4; ++k) {
            const int c = s + k;
            if (c < 0 || c >= ncy) continue;
            const float *p = in + ((size_t(cz) * ncy + c) * nx + x) * 3;
            r[0] += ww[k] * p[0]; r[1] += ww[k] * p[1]; r[2] += ww[k] * p[2];
        }
        out[i * 3] = r[0]; out[i * 3 + 1] = r[1]; out[i * 3 + 2] = r[2];
    } else {
        const size_t n = size_t(nz) * ny * nx;
        if (i >= n) return;
        const int x = int(i % nx), y = int((i / nx) % ny), z = int(i / (size_t(nx) * ny));
        const int s = a.ax[2].fs[z];
        const float4 w = a.ax[2].fw[z];
        const float ww[4] = {w.x, w.y, w.z, w.w};
        float r[3] = {float(x), float(y), float(z)};
        for (int k = 0; k < 4; ++k) {
            const int c = s + k;
            if (c < 0 || c >= ncz) continue;
            const float *p = in + ((size_t(c) * ny + y) * nx + x) * 3;
            r[0] -= ww[k] * p[0]; r[1] -= ww[k] * p[1]; r[2] -= ww[k] * p[2];
        }
        out[i * 3] = r[0]; out[i * 3 + 1] = r[1]; out[i * 3 + 2] = r[2];
    }
}

// warp from a dense grid (3D) or from on_grid per pixel (2D), plus sums
template <int D>
__global__ void __launch_bounds__(256) k_warp_plain(EvalArgs a, const float *grid)
{
    __shared__ double red[5 * 8];
    __shared__ bool is_last;
    const int nx = a.n[0], ny = a.n[1], nz = (D == 3) ? a.n[2] : 1;
    const size_t N = size_t(nx) * ny * nz;
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    float acc[5] = {0, 0, 0, 0, 0};
    if (i < N) {
        const float mn = a.minmax[0], mxv = a.minmax[1];
        float wv;
        if (D == 3) {
            wv = sample3(a.coef_img, nx, ny, nz, grid[i * 3], grid[i * 3 + 1], grid[i * 3 + 2], mn, mxv);
        } else {
            const int x = int(i % nx), y = int(i / nx);
            const int sx = a.ax[0].fs[x], sy = a.ax[1].fs[y];
            const float4 wx = a.ax[0].fw[x], wy = a.ax[1].fw[y];
            const float wxx[4] = {wx.x, wx.y, wx.z, wx.w}, wyy[4] = {wy.x, wy.y, wy.z, wy.w};
            float u[2] = {0, 0};
            for (int j = 0; j < 4; ++j) {
                if (sy + j >= a.nc[1]) break;
                float h[2] = {0, 0};
                for (int k = 0; k < 4; ++k) {
                    if (sx + k >= a.nc[0]) break;
                    const double *p = a.params + (size_t(sy + j) * a.nc[0] + sx + k) * 2;
                    h[0] += wxx[k] * float(p[0]);
                    h[1] += wxx[k] * float(p[1]);
                }
                u[0] += wyy[j] * h[0];
                u[1] += wyy[j] * h[1];
            }
            wv = sample2(a.coef_img, nx, ny, float(x) - u[0], float(y) - u[1], mn, mxv);
        }
        a.warped[i] = wv;
        const float b = a.ref[i];
        if (a.cost == 0) {
            const float d = wv - b;
            acc[0] = d * d;
        } else {
            const float da = wv - float(a.center_a), db = b - float(a.center_b);
            acc[0] = da; acc[1] = db; acc[2] = da * da; acc[3] = db * db; acc[4] = da * db;
        }
    }
    double dv[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) dv[k] = acc[k];
    block_sum<5>(dv, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 5; ++k) a.tile_sums[size_t(blockIdx.x) * 5 + k] = dv[k];
        __threadfence();
        is_last = (atomicAdd(&a.counters[0], 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        reduce_tile_sums(a, gridDim.x, N, red);
        if (threadIdx.x == 0) a.counters[0] = 0;
    }
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
    return f * sizeof(float);
}

static size_t adjoint_smem(const EvalArgs &a)
{
    const int D = a.dim;
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int TZ = (D == 3) ? Z.t : 1, HZ = (D == 3) ? Z.t + 2 : 1;
    size_t f = size_t(HZ) * (Y.t + 2) * (X.t + 2);
    f += size_t(D) * TZ * Y.t * X.t;
    f += size_t(D) * TZ * Y.t * X.ac;
    if (D == 3) f += size_t(D) * TZ * Y.ac * X.ac;
    return f * sizeof(float);
}

static dim3 tile_grid(const EvalArgs &a)
{
    return dim3(a.ax[0].nt, a.ax[1].nt, a.dim == 3 ? a.ax[2].nt : 1);
}

void launch_warp(const EvalArgs &a, cudaStream_t st)
{
    const size_t sm = warp_smem(a);
    if (a.dim == 3) {
        cudaFuncSetAttribute(k_warp<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
        k_warp<3><<<tile_grid(a), 256, sm, st>>>(a);
    } else {
        cudaFuncSetAttribute(k_warp<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
        k_warp<2><<<tile_grid(a), 256, sm, st>>>(a);
    }
    count_launch();
}

void launch_adjoint(const EvalArgs &a, cudaStream_t st)
{
    const size_t sm = adjoint_smem(a);
    if (a.dim == 3) {
        cudaFuncSetAttribute(k_adjoint<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
        k_adjoint<3><<<tile_grid(a), 256, sm, st>>>(a);
    } else {
        cudaFuncSetAttribute(k_adjoint<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
        k_adjoint<2><<<tile_grid(a), 256, sm, st>>>(a);
    }
    count_launch();
}

int gather_blocks(const EvalArgs &a)
{
    const size_t ncoef = size_t(a.nc[0]) * a.nc[1] * (a.dim == 3 ? a.nc[2] : 1);
    return int((ncoef + 255) / 256);
}

static void gather_impl(const EvalArgs &a, int with_gradient, int dense, cudaStream_t st)
{
    const int nb = gather_blocks(a);
    if (a.dim == 3) {
        const size_t sm = (a.has_penalty ? 9 * 9 * 9 * 6 : 0) * sizeof(float);
        k_gather<3><<<nb, 256, sm, st>>>(a, with_gradient, dense);
    } else {
        k_gather<2><<<nb, 256, 0, st>>>(a, with_gradient, dense);
    }
    count_launch();
}

void launch_gather(const EvalArgs &a, int with_gradient, cudaStream_t st)
{
    gather_impl(a, with_gradient, 0, st);
}

void launch_force(const EvalArgs &a, float *force, cudaStream_t st)
{
    const size_t N = size_t(a.n[0]) * a.n[1] * (a.dim == 3 ? a.n[2] : 1);
    const int nb = int((N + 255) / 256);
    if (a.dim == 3) k_force<3><<<nb, 256, 0, st>>>(a, force);
    else k_force<2><<<nb, 256, 0, st>>>(a, force);
    count_launch();
}

void launch_translate(const EvalArgs &a, const float *force, double *grad, float *tmp1, float *tmp2,
                      cudaStream_t st)
{
    const int nx = a.n[0], ny = a.n[1];
    const int ncx = a.nc[0], ncy = a.nc[1];
    if (a.dim == 3) {
        const int ncz = a.nc[2];
        size_t n = size_t(ncz) * ny * nx;
        k_translate_pass<3><<<int((n + 255) / 256), 256, 0, st>>>(a, 0, force, tmp1, nullptr);
        n = size_t(ncz) * ncy * nx;
        k_translate_pass<3><<<int((n + 255) / 256), 256, 0, st>>>(a, 1, tmp1, tmp2, nullptr);
        n = size_t(ncz) * ncy * ncx;
        k_translate_pass<3><<<int((n + 255) / 256), 256, 0, st>>>(a, 2, tmp2, nullptr, grad);
        count_launch(3);
    } else {
        size_t n = size_t(ncy) * nx;
        k_translate_pass<2><<<int((n + 255) / 256), 256, 0, st>>>(a, 1, force, tmp2, nullptr);
        n = size_t(ncy) * ncx;
        k_translate_pass<2><<<int((n + 255) / 256), 256, 0, st>>>(a, 2, tmp2, nullptr, grad);
        count_launch(2);
    }
}

void launch_plain_eval(const EvalArgs &a, float *grid, float *force, float *tmp1, float *tmp2,
                       cudaStream_t st)
{
    const int nx = a.n[0], ny = a.n[1], nz = a.dim == 3 ? a.n[2] : 1;
    const size_t N = size_t(nx) * ny * nz;
    const int nb = int((N + 255) / 256);
    if (a.dim == 3) {
        const int ncy = a.nc[1], ncz = a.nc[2];
        size_t n = size_t(ncz) * ncy * nx;
        k_grid_pass<<<int((n + 255) / 256), 256, 0, st>>>(a, 0, nullptr, tmp1);
        n = size_t(ncz) * ny * nx;
        k_grid_pass<<<int((n + 255) / 256), 256, 0, st>>>(a, 1, tmp1, tmp2);
        k_grid_pass<<<nb, 256, 0, st>>>(a, 2, tmp2, grid);
        k_warp_plain<3><<<nb, 256, 0, st>>>(a, grid);
        count_launch(4);
    } else {
        k_warp_plain<2><<<nb, 256, 0, st>>>(a, nullptr);
        count_launch(1);
    }
    launch_force(a, force, st);
    launch_translate(a, force, a.grad_image, tmp1, tmp2, st);
    gather_impl(a, 1, 1, st);
}

int plain_sum_blocks(const EvalArgs &a)
{
    const size_t N = size_t(a.n[0]) * a.n[1] * (a.dim == 3 ? a.n[2] : 1);
    return int((N + 255) / 256);
}

}  // namespace mgr
