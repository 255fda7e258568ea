// mgr_cost.cuh — cost finalisation shared by the split and plain paths.
#pragma once

#include "mgr_common.cuh"
#include "mgr_kernels.hh"

namespace mgr {

// Final SSD / NCC cost and force constants from the reduced sums (thread 0
// of the last block only).  SSD: s[0] = sum (a-b)^2; value 0.5*s (x 1/N with
// norm) as FEvalSSD (mia/template/ssd.hh:54-99).  NCC: s = sums of
// da = a - c_a, db = b - c_b, da^2, db^2, da*db about provisional centres;
// value and gradient helper as NCCSums::value / get_grad_helper of the SSE2
// build (mia/core/nccsum.cc:31-120: 1e-10 and 1e-5 thresholds).
__device__ __forceinline__ void finalise_cost(const EvalArgs &a, const double s[5], size_t N)
{
    double *sc = a.scalars;
    if (a.cost == 0) {
        const double scale = a.ssd_norm ? 0.5 / double(N) : 0.5;
        sc[SC_VALUE] = scale * s[0];
        sc[SC_FORCE_COST] = scale * s[0];
        sc[SC_FSCALE] = a.ssd_norm ? double(float(1.0 / double(N))) : 1.0;
        sc[SC_K1] = sc[SC_K2] = sc[SC_MA] = sc[SC_MB] = 0.0;
        return;
    }
    const double n = double(N);
    const double sa = s[0], sb = s[1], saa = s[2], sbb = s[3], sab = s[4];
    const double ma = a.centers[0] + sa / n, mb = a.centers[1] + sb / n;
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

// Reduce the per-tile sums in a fixed order (every thread of the last block
// calls this), then finalise the cost.
__device__ __forceinline__ void reduce_tile_sums(const EvalArgs &a, int ntiles, size_t N, double *red)
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

__device__ __forceinline__ float aw_at(const float4 *aw, int i, int k)
{
    return reinterpret_cast<const float *>(aw)[i * 4 + k];
}

}  // namespace mgr
