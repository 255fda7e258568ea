// gather.cu — per-coefficient gather of the tile partials, the divcurl
// penalty (value and gradient) and the final weighted costs.
//
// One block owns 32 consecutive coefficients (lane = coefficient, so
// neighbour loads coalesce along x).  The eight warps split the work of
// those 32 coefficients: the (dz, dy) rows of the 3D penalty stencil
// (C3DPPDivcurlMatrixImpl::evaluate / multiply, mia/3d/ppmatrix.cc:292-599;
// the P cell of an offset is read as a broadcast), the cells of the 2D
// boundary-clipped CSR row (mia/2d/ppmatrix.cc:328-352), and the partial
// slots of the split path that hold the coefficient.  Warp 0 combines the
// per-warp sums in a fixed order (deterministic, no atomics), applies the
// penalty weight and sign (C3DSplineTransformPenalty::value_and_gradient,
// mia/3d/splinetransformpenalty.cc:60-71) and the full-cost weight
// (mia/template/fullcost.cxx:37-45), and the last block finalises the costs.
#include "mgr_cost.cuh"

namespace mgr {

namespace {
constexpr int GT = 256;   // threads per block
constexpr int GW = GT / 32;
constexpr int GC = 32;    // coefficients per block
constexpr int NPART = 12; // per warp: penalty g[3], r[6]; image s[3]
}  // namespace

// block `blk` of the pair's `nblk` gather blocks
template <int D>
__device__ __forceinline__ void gather_body(const EvalArgs &a, int with_gradient, int image_from_dense, int blk,
                                            int nblk)
{
    extern __shared__ float sm[];            // 3D: P table (9^3 x 6)
    __shared__ float part[GW][NPART][GC];
    __shared__ double red[GW];
    __shared__ bool is_last;
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int ncx = a.nc[0], ncy = a.nc[1], ncz = (D == 3) ? a.nc[2] : 1;
    const size_t ncoef = size_t(ncx) * ncy * ncz;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (D == 3 && a.has_penalty) {
        for (int e = tid; e < 9 * 9 * 9 * 6; e += GT) sm[e] = a.ptable[e];
        __syncthreads();
    }
    const size_t i = size_t(blk) * GC + lane;
    const bool valid = i < ncoef;
    const int cx = valid ? int(i % ncx) : 0;
    const int cy = valid ? int((i / ncx) % ncy) : 0;
    const int cz = (D == 3 && valid) ? int(i / (size_t(ncx) * ncy)) : 0;

    float g[3] = {0.0f, 0.0f, 0.0f};
    float r[6] = {0, 0, 0, 0, 0, 0};
    float s[3] = {0.0f, 0.0f, 0.0f};
    if (valid && a.has_penalty) {
        if (D == 3) {
            for (int p = w; p < 49; p += GW) {
                const int dz = p / 7 - 3, dy = p % 7 - 3;
                const int zj = cz - dz, yj = cy - dy;
                if (zj < 0 || zj >= ncz || yj < 0 || yj >= ncy) continue;
                const double *row = a.params + ((size_t(zj) * ncy + yj) * ncx) * 3;
                const float *Prow = sm + (((dz + 4) * 9 + (dy + 4)) * 9 + 4) * 6;
#pragma unroll
                for (int dx = -3; dx <= 3; ++dx) {
                    const int xj = cx - dx;
                    if (xj < 0 || xj >= ncx) continue;
                    const float *P = Prow + dx * 6;
                    const float cjx = float(row[xj * 3]), cjy = float(row[xj * 3 + 1]), cjz = float(row[xj * 3 + 2]);
                    const float vxx = P[0], vxy = P[1], vyy = P[2], vyz = P[3], vzz = P[4], vxz = P[5];
                    if (with_gradient) {
                        const float ax = vxx * cjx, az = vxz * cjx;
                        const float bxy = vxy * cjy, byy = vyy * cjy;
                        const float cyz = vyz * cjz, czz = vzz * cjz;
                        r[0] += ax; r[1] += bxy; r[2] += byy; r[3] += cyz; r[4] += czz; r[5] += az;
                        g[0] += cjz * vxz + (2.0f * ax + bxy);
                        g[1] += cjx * vxy + (2.0f * byy + cyz);
                        g[2] += cjy * vyz + (2.0f * czz + az);
                    } else {
                        // operator*: ci.x cj.y vxy, ci.x cj.z vxz, ci.y cj.z vyz
                        r[0] += cjx * vxx; r[2] += cjy * vyy; r[4] += cjz * vzz;
                        r[1] += cjy * vxy; r[5] += cjz * vxz; r[3] += cjz * vyz;
                    }
                }
            }
        } else {
            for (int e = a.pen_rowptr[i] + w; e < a.pen_rowptr[i + 1]; e += GW) {
                const int j = a.pen_col[e];
                const float4 v = a.pen_val[e];
                const float cjx = float(a.params[size_t(j) * 2]), cjy = float(a.params[size_t(j) * 2 + 1]);
                const float aa = cjx * v.x, bb = cjy * v.y, cxx = cjx * v.z, cyy = cjy * v.z;
                g[0] += aa + aa + cyy;
                g[1] += bb + bb + cxx;
                r[0] += aa;
                r[1] += cyy;
                r[2] += bb;
            }
        }
    }
    if (valid && with_gradient && !image_from_dense) {
        const int2 gx = X.gtile[cx], gy = Y.gtile[cy];
        const int2 gz = (D == 3) ? Z.gtile[cz] : make_int2(0, 0);
        const int nX = gx.y - gx.x + 1, nY = gy.y - gy.x + 1, nZ = gz.y - gz.x + 1;
        const int total = (nX > 0 && nY > 0 && nZ > 0) ? nX * nY * nZ : 0;
        for (int k = w; k < total; k += GW) {
            const int tx = gx.x + k % nX, ty = gy.x + (k / nX) % nY, tz = gz.x + k / (nX * nY);
            const int lx = cx - X.atile0[tx], ly = cy - Y.atile0[ty];
            const int lz = (D == 3) ? cz - Z.atile0[tz] : 0;
            const size_t t = (size_t(tz) * Y.nt + ty) * X.nt + tx;
            const float *p = a.partial + t * a.slot + ((size_t(lz) * Y.ac + ly) * X.ac + lx) * D;
#pragma unroll
            for (int c = 0; c < D; ++c) s[c] += p[c];
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) part[w][k][lane] = g[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) part[w][3 + k][lane] = r[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) part[w][9 + k][lane] = s[k];
    __syncthreads();
    if (w == 0) {
        double pval = 0.0;
        if (valid) {
            float G[3] = {0.0f, 0.0f, 0.0f}, R[6] = {0, 0, 0, 0, 0, 0}, S[3] = {0.0f, 0.0f, 0.0f};
            for (int p = 0; p < GW; ++p) {
#pragma unroll
                for (int k = 0; k < 3; ++k) G[k] += part[p][k][lane];
#pragma unroll
                for (int k = 0; k < 6; ++k) R[k] += part[p][3 + k][lane];
#pragma unroll
                for (int k = 0; k < 3; ++k) S[k] += part[p][9 + k][lane];
            }
            double gp[3] = {0.0, 0.0, 0.0};
            if (a.has_penalty) {
                float ci[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
                for (int k = 0; k < D; ++k) ci[k] = float(a.params[i * D + k]);
                float v;
                if (D == 3) {
                    if (with_gradient)
                        v = ci[0] * R[0] + ci[0] * R[1] + ci[1] * R[2] + ci[1] * R[3] + ci[2] * R[4] + ci[2] * R[5];
                    else
                        v = ci[0] * R[0] + ci[1] * R[2] + ci[2] * R[4] + ci[0] * R[1] + ci[0] * R[5] + ci[1] * R[3];
                } else {
                    v = ci[0] * R[0] + ci[0] * R[1] + ci[1] * R[2];
                }
                pval = v;
#pragma unroll
                for (int k = 0; k < D; ++k) gp[k] = (a.pen_grad_sign * a.pen_weight) * double(G[k]);
            }
            if (with_gradient) {
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const double gi = image_from_dense ? a.grad_image[i * D + k] : a.cost_weight * (-double(S[k]));
                    a.grad_total[i * D + k] = gi + gp[k];
                    if (a.grad_image && !image_from_dense) a.grad_image[i * D + k] = gi;
                    if (a.grad_penalty) a.grad_penalty[i * D + k] = gp[k];
                }
            }
        }
        pval = warp_sum(pval);
        if (lane == 0) {
            a.pen_part[blk] = pval;
            __threadfence();
            is_last = (atomicAdd(&a.counters[1], 1u) == unsigned(nblk - 1));
        }
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        double sv[1] = {0.0};
        for (unsigned b = tid; b < unsigned(nblk); b += GT) sv[0] += ((volatile double *)a.pen_part)[b];
        block_sum<1>(sv, red);
        if (tid == 0) {
            double *sc = a.scalars;
            const double pen = a.has_penalty ? sv[0] : 0.0;
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

template <int D>
__global__ void __launch_bounds__(GT) k_gather_b(EvalArgs a, int with_gradient, int image_from_dense)
{
    gather_body<D>(a, with_gradient, image_from_dense, blockIdx.x, gridDim.x);
}

// batch: work list of (pair, block) items; finished pairs are skipped
template <int D>
__global__ void __launch_bounds__(GT) k_gather_batch(const EvalArgs *__restrict__ args, const int2 *__restrict__ items,
                                                     const int *__restrict__ active, const int *__restrict__ nblocks)
{
    const int2 it = items[blockIdx.x];
    if (!active[it.x]) return;
    gather_body<D>(args[it.x], 1, 0, it.y, nblocks[it.x]);
}

void launch_gather_batch(int dim, const EvalArgs *args, const int2 *items, int nitems, const int *active,
                         const int *nblocks, int has_penalty, cudaStream_t st)
{
    (void)has_penalty;
    if (dim == 3) {
        launch_gather3_batch(args, items, nitems, active, nblocks, st);
        return;
    }
    k_gather_batch<2><<<nitems, GT, 0, st>>>(args, items, active, nblocks);
    count_launch();
}

int gather_blocks(const EvalArgs &a)
{
    if (a.dim == 3) return gather3_blocks(a);
    const size_t ncoef = size_t(a.nc[0]) * a.nc[1];
    return int((ncoef + GC - 1) / GC);
}

void launch_gather_mode(const EvalArgs &a, int with_gradient, int dense, cudaStream_t st)
{
    if (a.dim == 3) {
        launch_gather3(a, with_gradient, dense, st);
        return;
    }
    k_gather_b<2><<<gather_blocks(a), GT, 0, st>>>(a, with_gradient, dense);
    count_launch();
}

void launch_gather(const EvalArgs &a, int with_gradient, cudaStream_t st)
{
    launch_gather_mode(a, with_gradient, 0, st);
}

}  // namespace mgr
