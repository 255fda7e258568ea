// eval.cu — the plain evaluation path: one kernel per step of the
// reference's evaluation (C3DImageFullCost::do_evaluate,
// mia/3d/fullcost/image.cc:67-78): the three init_grid passes
// (mia/3d/transform/spline.cc:541-653), the warp from the dense grid
// (mia/3d/transform.cc:280-353; 2D: on_grid per pixel,
// mia/2d/transform/spline.cc:640-666), the image gradient and force
// (mia/3d/image.cc:347-466, mia/template/ssd.hh:126-181,
// mia/3d/cost/ncc.cc:88-128), the three translate passes
// (spline.cc:731-791), then the shared gather/penalty kernel.  It is the
// straightforward per-pair GPU port that the split path is measured
// against, and it also serves mgr_level_force and mgr_level_translate.
#include "mgr_cost.cuh"

namespace mgr {

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
            const float da = wv - float(a.centers[0]), db = b - float(a.centers[1]);
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
    if (a.dim == 3) launch_params_f32(a, st);   // read by the gather's penalty
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
    launch_gather_mode(a, 1, 1, st);
}

int plain_sum_blocks(const EvalArgs &a)
{
    const size_t N = size_t(a.n[0]) * a.n[1] * (a.dim == 3 ? a.n[2] : 1);
    return int((N + 255) / 256);
}

}  // namespace mgr
