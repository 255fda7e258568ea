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
//       to [min(0, min src), max src]); the taps are read from a ring of z
//       planes in shared memory that bulk copies fill ahead of the walk from
//       a mirror-padded copy (the box of a plane follows from the range of
//       u over the tile), so the interior needs no index folding and the
//       gather costs shared-memory wavefronts instead of L1 lines; each
//       thread samples two planes per step (two independent tap chains in
//       flight); the warped image is written and the SSD / NCC sums are
//       accumulated; the last block finalises the cost.
//   k_adjoint3<TZ>    central differences of the warped image (x neighbours
//       by warp shuffle, y neighbours from the rows of the adjacent warps, z
//       neighbours carried in registers; mia/3d/image.cc:347-466), the SSD /
//       NCC force (mia/template/ssd.hh:126-181, mia/3d/cost/ncc.cc:88-128),
//       and the transposed spline contraction (translate,
//       spline.cc:731-791): z while walking (four running sums per
//       component, the lowest one final when the window moves on), then x
//       and y in shared memory (the reference contracts y before x; the
//       order changes only the rounding, and x first keeps the intermediate
//       small); the result goes to the tile's partial slot (no atomics).
//   k_gather3         per 4x4x4 block of coefficients: the fixed-order sum of
//       the partial slots that hold each coefficient, the divcurl stencil
//       (C3DPPDivcurlMatrixImpl::evaluate / multiply,
//       mia/3d/ppmatrix.cc:292-599) over a shared-memory copy of the
//       parameters with a 3-node halo, the penalty weight and sign
//       (mia/3d/splinetransformpenalty.cc:60-71) and the full-cost weight
//       (mia/template/fullcost.cxx:37-45).
#include <algorithm>
#include <string>

#include "../../include/mgr.h"
#include "mgr_cost.cuh"
#include "warp3_common.cuh"

#include <type_traits>

// the one-pair adjoint kernel: minimum resident blocks per SM (a cap of 40
// registers, no spills) and the unroll factor of its plane walk (measured
// at 192x192x128 SSD and 256^3 NCC against no unroll and no cap; the
// batched kernels keep both off)
#ifndef MGR_ADJ_MINB
#define MGR_ADJ_MINB 6
#endif
#define MGR_ADJ_BOUNDS __launch_bounds__(NT3, MGR_ADJ_MINB)
#ifndef MGR_ADJ_UNROLL
#define MGR_ADJ_UNROLL 2
#endif

namespace mgr {

void set_last_error(const std::string &msg);

namespace {

constexpr int NT3 = 256;   // threads per tile block: 8 warps
constexpr int TX3 = 32;    // tile x (lanes)
constexpr int TY3 = 8;     // tile y (warps)
constexpr unsigned FULL = 0xffffffffu;

// Programmatic dependent launch.  A kernel launched with
// cudaLaunchAttributeProgrammaticStreamSerialization may start while the
// kernel before it in the stream is still running; pdl_wait returns once
// that kernel has completed and its writes are visible (at once for a
// kernel launched without the attribute).  Before it a kernel reads only
// the level's fixed tables.  pdl_trigger, issued by every block after its
// pdl_wait, lets the next kernel be launched: so no kernel starts before the
// one two places back in the stream has completed.
__device__ __forceinline__ void pdl_wait()
{
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
}
__device__ __forceinline__ void pdl_trigger()
{
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

}  // namespace

// ---------------------------------------------------------------------
// warp
// ---------------------------------------------------------------------
// COST: the image cost when known at compile time (MGR_COST_SSD / NCC; the
// one-pair kernels are compiled per cost), -1 to read it from a
template <int TZ, int COST>
__device__ __forceinline__ void warp3_body(const EvalArgs &a, int bx, int by, int bz, int ntiles, int tile)
{
    const int cost = COST >= 0 ? COST : a.cost;
    extern __shared__ __align__(16) float sm3[];
    __shared__ double red[5 * (NT3 / 32)];
    __shared__ float wsum[5][NT3 / 32];
    __shared__ float csc[2];   // NCC centres (converted once per block)
    __shared__ int zs[TZ];
    __shared__ float4 zw[TZ];
    __shared__ float urng[NT3 / 32][6];   // per warp: footprint min / max per component
    __shared__ int boxs[8];               // staged, xs, ylo, zbase, nplanes, span, w4, rows
    __shared__ __align__(8) unsigned long long mbar[RING_N];
    __shared__ unsigned rdone[RING_N];    // warps done with the ring slot's current plane
    __shared__ int nissued;               // planes whose copies were issued
    __shared__ volatile int ring_failed;  // a wait of this block gave up
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
    if (tid == 0) {
        csc[0] = float(a.centers[0]);
        csc[1] = float(a.centers[1]);
    }

    // the parameters' float copy comes from the kernel before this one
    pdl_wait();
    pdl_trigger();
    float *C = sm3;                        // [3][FZ][FY][FX]
    float *Tx = C + 3 * FZ * FY * FX;      // [3][FZ][FY][32]
    // [RING_N][RING_Y][RING_X]: the tensor copies want a 128-byte aligned
    // destination, so the ring starts at the next 128-byte boundary of the
    // shared window after Tx (the launch reserves the 128 bytes of slack)
    float *ring;
    {
        const int off = 3 * FZ * FY * (FX + 32);
        const unsigned ra = smem_u32(sm3 + off);
        ring = sm3 + off + ((((ra + 127u) & ~127u) - ra) >> 2);
    }
    // coefficient footprint: rows (iz, iy) of 3 FX consecutive floats
    // (parameters are interleaved per node); each thread issues its loads
    // as one batch before storing
    {
        const int w3 = 3 * FX, nel = FZ * FY * w3;
        auto src = [&](int e, int &dst) -> const float * {
            const int r = e / w3, j = e - r * w3;
            const int ix = j / 3, c = j - 3 * ix;
            const int iz = r / FY, iy = r - iz * FY;
            dst = (c * FZ * FY + r) * FX + ix;
            if (cx0 + ix >= ncx || cy0 + iy >= ncy || cz0 + iz >= ncz) return nullptr;
            return a.params_f + ((size_t(cz0 + iz) * ncy + (cy0 + iy)) * ncx + cx0) * 3 + j;
        };
        constexpr int K = 4;
        float v[K];
        int dst[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int e = tid + k * NT3;
            v[k] = 0.0f;
            dst[k] = -1;
            if (e < nel) {
                const float *p = src(e, dst[k]);
                if (p) v[k] = *p;
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (dst[k] >= 0) C[dst[k]] = v[k];
        for (int e = tid + K * NT3; e < nel; e += NT3) {
            int d;
            const float *p = src(e, d);
            C[d] = p ? *p : 0.0f;
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
        // the ring's barriers: one thread initialises them all (mbarrier and
        // bulk-copy instructions are issued by single threads here)
        if (tid == 0) {
            for (int k = 0; k < RING_N; ++k) {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[k])) : "memory");
                rdone[k] = 0;
            }
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
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
    auto advance = [&](int t) {   // the window moves to the coefficients of plane z0 + t (uniform)
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
    const bool inxy_t = (x0 + lane < nx) && (y0 + wy < ny);
    {
        // the range of u over the tile: along z, u is a combination of this
        // thread's q values over the window range 0 .. zs[ez-1] + 3 with
        // non-negative weights summing to 1 (to less than 1 on the last
        // plane of the image, where 0 joins the range)
        float lo[3], hi[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {   // the window's q values are kz = 0..3
            lo[c] = fminf(fminf(q[c][0], q[c][1]), fminf(q[c][2], q[c][3]));
            hi[c] = fmaxf(fmaxf(q[c][0], q[c][1]), fmaxf(q[c][2], q[c][3]));
        }
        const int kend = zs[ez - 1] + 3;
        for (int kz = 4; kz <= kend; ++kz)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float v = qat(c, kz);
                lo[c] = fminf(lo[c], v);
                hi[c] = fmaxf(hi[c], v);
            }
        const bool last_plane = z0 + ez == nz;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (last_plane) {
                lo[c] = fminf(lo[c], 0.0f);
                hi[c] = fmaxf(hi[c], 0.0f);
            }
            if (!inxy_t) {
                lo[c] = 3.0e38f;
                hi[c] = -3.0e38f;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo[c] = fminf(lo[c], __shfl_xor_sync(FULL, lo[c], o));
                hi[c] = fmaxf(hi[c], __shfl_xor_sync(FULL, hi[c], o));
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
    // tap box of the tile: x from xs (16-byte aligned in the padded rows),
    // rows from ylo, planes zbase .. zbase + nplanes - 1 of which step t
    // needs t .. t + span - 1; the ring is filled by bulk copies, one per
    // row, completion counted on the plane's mbarrier
    constexpr int H = PAD_H;
    auto issue_plane = [&](int k) {   // one thread: plane k of the box into its ring slot, one tensor copy
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
    // the displacement range of the tile: lane k < 6 of warp 0 reduces bound
    // k over the warps (lanes 0-2 the minima, 3-5 the maxima), lane 0 then
    // sets the box
    float urange = 0.0f;
    if (wy == 0 && lane < 6) {
        urange = urng[0][lane];
        for (int w = 1; w < NT3 / 32; ++w)
            urange = lane < 3 ? fminf(urange, urng[w][lane]) : fmaxf(urange, urng[w][lane]);
    }
    float ulo[3], uhi[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        ulo[c] = __shfl_sync(FULL, urange, c);
        uhi[c] = __shfl_sync(FULL, urange, 3 + c);
    }
    if (tid == 0) {
        // taps of a voxel at p = v - u: floor(p) - 1 .. floor(p) + 2; the
        // fixed-point floor may round p up to the next integer, one more
        // row / column / plane on the upper side
        const float big = 1.0e6f;
        // once a wait of this launch has given up (the flag the host reads
        // afterwards), later blocks read their taps from global memory, so
        // that a stalled copy engine costs one wait limit per launch, not
        // one per block
        bool ok = a.has_tmap != 0 && *(volatile unsigned *)&a.counters[6] == 0u;
#pragma unroll
        for (int c = 0; c < 3; ++c) ok = ok && fabsf(ulo[c]) < big && fabsf(uhi[c]) < big;
        int xs = 0, xe = 0, ylo = 0, yhi = 0, dzl = 0, dzh = 0;
        if (ok) {
            const int xlo = int(floorf(float(x0) - uhi[0])) - 1;
            xe = int(floorf(float(x0 + TX3 - 1) - ulo[0])) + 3;
            xs = ((xlo + H) & ~3) - H;
            ylo = int(floorf(float(y0) - uhi[1])) - 1;
            yhi = int(floorf(float(y0 + ey - 1) - ulo[1])) + 3;
            dzl = int(floorf(-uhi[2])) - 1;
            dzh = int(floorf(-ulo[2])) + 3;
            ok = xs >= -H && xe <= nx + H - 1 && xe - xs + 1 <= RING_X && ylo >= -H && yhi <= ny + H - 1 &&
                 yhi - ylo + 1 <= RING_Y && z0 + dzl >= -H && z0 + ez - 1 + dzh <= nz + H - 1 &&
                 dzh - dzl + 1 <= RING_N - 2;
        }
        boxs[0] = ok;
        boxs[1] = xs;
        boxs[2] = ylo;
        boxs[3] = z0 + dzl;
        boxs[4] = ez + dzh - dzl;
        boxs[5] = dzh - dzl + 1;
        boxs[6] = RING_X;
        boxs[7] = yhi - ylo + 1;
        ring_failed = 0;
        nissued = ok ? min(boxs[4], RING_N) : 0;
    }
    __syncthreads();
    // the box's first planes, issued by thread 0 after the barrier: the
    // other warps start their walks meanwhile, their waits on a plane end
    // once its copy has been issued and has landed
    if (tid == 0)
        for (int k = 0; k < nissued; ++k) issue_plane(k);

    const bool inxy = (x0 + lane < nx) && (y0 + wy < ny);
    const float px0 = float(x0 + lane), py0 = float(y0 + wy);
    const float ca = csc[0], cb = csc[1];
    const size_t nxy = size_t(nx) * ny;
    const size_t col = size_t(min(y0 + wy, ny - 1)) * nx + min(x0 + lane, nx - 1) + size_t(z0) * nxy;
    float *wout = a.warped + col;
    const float *rin = a.ref + col;
    float acc[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    const bool staged = boxs[0] != 0;
    const int bxs = boxs[1], bylo = boxs[2], bzbase = boxs[3], nplanes = boxs[4], span = boxs[5];
    const int brows = boxs[7];
    bool ring_ok = staged;
    // planes (bit t) of this thread's voxels whose taps are not read from
    // the ring: all of them when the tile was not staged, else the rare
    // voxel outside the box and, after a wait gave up, the rest of the walk.
    // They are sampled from global memory after the walk, so that the walk
    // itself makes no call (a call site costs the loop register spills).
    unsigned defer = 0u;
    int kwait = 0;      // planes below kwait have arrived
    // the reference is streamed three planes ahead of its use (registers
    // r0..r2), so the walk does not wait on its memory latency
    // two planes per step: the two voxels' tap gathers are independent
    // chains, so a warp keeps twice the loads in flight; the waits, the
    // displacement window and the refills are done per pair.  Per voxel the
    // arithmetic and the order of the sums are those of one plane per step.
    float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, r3 = 0.0f;
    if (inxy) {
        r0 = __ldg(rin);
        if (ez > 1) r1 = __ldg(rin + nxy);
        if (ez > 2) r2 = __ldg(rin + 2 * nxy);
        if (ez > 3) r3 = __ldg(rin + 3 * nxy);
    }
    // the sample at plane t from the ring; ok = false when its taps are
    // not there (the voxel is deferred)
    auto sample_ring = [&](int t, int st, const float u[3], bool &ok) -> float {
        const int z = z0 + t;
        const float px = px0 - u[0], py = py0 - u[1], pz = float(z) - u[2];
        const int fx = ffloor16(px), fy = ffloor16(py), fz = ffloor16(pz);
        const int col = fx - 1 - bxs, row = fy - 1 - bylo, dk = fz - 1 - bzbase - t;
        ok = ring_ok && unsigned(col) < unsigned(RING_X - 3) && unsigned(row) < unsigned(brows - 3) &&
             unsigned(dk) < unsigned(span - 3);
        // a voxel whose taps are not in the ring reads the ring's first taps
        // instead (the sample is discarded and the voxel deferred), so that
        // no branch separates the step's two tap chains
        const int c = ok ? col : 0, r = ok ? row : 0, d = ok ? dk : 0;
        // the slot of plane t + d: st is plane t's, d < RING_N
        const int sl = st + d >= RING_N ? st + d - RING_N : st + d;
        return taps3_ring(ring, sl, r, c, px - float(fx), py - float(fy), pz - float(fz), mn, mxv);
    };
    auto add_cost = [&](float wv, float b) {
        if (cost == 0) {
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
    };
    // this warp is done with planes t and t + 1 (t even: the pair's slots
    // st, st + 1 share the counter of slot st); the last warp refills both
    auto release = [&](int t, int st) {
        if (staged && t + RING_N < nplanes) {
            __syncwarp();
            if (lane == 0) {
                __threadfence_block();
                if (atomicAdd(&rdone[st], 1u) == unsigned(NT3 / 32 - 1)) {
                    rdone[st] = 0;
                    if (ring_ok && !ring_failed) {
                        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                        issue_plane(t + RING_N);
                        const bool second = t + 1 + RING_N < nplanes;
                        if (second) issue_plane(t + 1 + RING_N);
                        atomicAdd(&nissued, second ? 2 : 1);
                    }
                }
            }
        }
    };
    if (!staged && inxy) defer = ez >= 32 ? ~0u : (1u << ez) - 1u;
    static_assert(RING_N % 2 == 0, "the walk releases the ring's slots in pairs");
    for (int t = 0, st = 0; staged && t < ez; t += 2, st = st + 2 == RING_N ? 0 : st + 2) {
        const bool two = t + 1 < ez;
        float ua[3], ub[3] = {0.0f, 0.0f, 0.0f};
        advance(t);
        {
            const float4 wz = zw[t];
#pragma unroll
            for (int c = 0; c < 3; ++c) ua[c] = wz.x * q[c][0] + wz.y * q[c][1] + wz.z * q[c][2] + wz.w * q[c][3];
        }
        if (two) {
            advance(t + 1);
            const float4 wz = zw[t + 1];
#pragma unroll
            for (int c = 0; c < 3; ++c) ub[c] = wz.x * q[c][0] + wz.y * q[c][1] + wz.z * q[c][2] + wz.w * q[c][3];
        }
        if (ring_ok) {
            const int need = t + span - (two ? 0 : 1);
            while (kwait <= need) {
                if (!mbar_wait(smem_u32(&mbar[ring_slot(kwait)]), unsigned(kwait / RING_N) & 1u) || ring_failed) {
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
        if (inxy) {
            bool oka, okb = true;
            const float wa = sample_ring(t, st, ua, oka);
            float wb = 0.0f;
            if (two) wb = sample_ring(t + 1, st + 1, ub, okb);
            if (oka) {
                wout[0] = wa;
                add_cost(wa, r0);
            } else {
                defer |= 1u << t;
            }
            if (two) {
                if (okb) {
                    wout[nxy] = wb;
                    add_cost(wb, r1);
                } else {
                    defer |= 1u << (t + 1);
                }
            }
        }
        r0 = r2;
        r1 = r3;
        r2 = (inxy && t + 4 < ez) ? __ldg(rin + 4 * nxy) : 0.0f;
        r3 = (inxy && t + 5 < ez) ? __ldg(rin + 5 * nxy) : 0.0f;
        wout += 2 * nxy;
        rin += 2 * nxy;
        release(t, st);
    }
    // the deferred voxels, in plane order: the displacement from the y
    // stage's window at plane t (the walk's values: the window then starts
    // at coefficient zs[t]) and the taps from global memory
    if (defer) {
        float *const w0p = a.warped + col;
        const float *const r0p = a.ref + col;
        do {
            const int t = __ffs(defer) - 1;
            defer &= defer - 1u;
            const int s = zs[t];
            const float4 wz = zw[t];
            float u[3];
#pragma unroll
            for (int c = 0; c < 3; ++c)
                u[c] = wz.x * qat(c, s) + wz.y * qat(c, s + 1) + wz.z * qat(c, s + 2) + wz.w * qat(c, s + 3);
            const float wv = taps3_global(a, px0 - u[0], py0 - u[1], float(z0 + t) - u[2], mn, mxv);
            w0p[size_t(t) * nxy] = wv;
            add_cost(wv, __ldg(r0p + size_t(t) * nxy));
        } while (defer);
    }
    if (staged) __syncthreads();   // every warp is done with the ring
    if (staged && tid == 0) {
        // copies still in flight (only after a wait gave up) are waited for
        // before the block's shared memory is released: only the planes that
        // were issued, and within one wait limit in total (a plane whose
        // wait gives up ends the drain)
        const int issued = nissued;
        while (kwait < issued) {
            if (!mbar_wait(smem_u32(&mbar[ring_slot(kwait)]), unsigned(kwait / RING_N) & 1u)) {
                atomicOr(&a.counters[6], 1u);
                break;
            }
            ++kwait;
        }
    }
    // tile sums: a float tree within each warp (5 levels), the warps' sums
    // added in double in a fixed order by thread 0 (FP64 is slow here, so
    // it is kept off the per-thread path)
    const int ncomp = cost == 0 ? 1 : 5;
#pragma unroll
    for (int k = 0; k < 5; ++k)
        if (k < ncomp) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(FULL, acc[k], o);
            if (lane == 0) wsum[k][wy] = acc[k];
        }
    __syncthreads();
    // a deferred finalisation (the gather's for SSD, k_finalise3's for NCC)
    // needs no last-block pass here
    const bool finalise_here = !a.defer_cost;
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            double v = 0.0;
            if (k < ncomp)
                for (int w = 0; w < NT3 / 32; ++w) v += double(wsum[k][w]);
            a.tile_sums[size_t(tile) * 5 + k] = v;
        }
        is_last = false;
        if (finalise_here) {
            __threadfence();
            is_last = (atomicAdd(&a.counters[0], 1u) == unsigned(ntiles - 1));
        }
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
template <int TZ, int UNROLL>
__device__ __forceinline__ void adjoint3_body(const EvalArgs &a, int bx, int by, int bz, int tile_index)
{
    const int cost = a.cost;   // (a per-cost NCC kernel spills under the register cap)
    extern __shared__ __align__(16) float sm3[];
    __shared__ int asx[TX3], asy[TY3], azs[TZ];
    __shared__ float fsc[5];   // force constants (converted once per block)
    __shared__ float4 awx[TX3], awy[TY3], azw[TZ];
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
    const int x0 = bx * TX3, y0 = by * TY3, z0 = bz * TZ;
    const int ex = min(TX3, nx - x0), ey = min(TY3, ny - y0), ez = min(TZ, nz - z0);
    const int AXc = X.ac, AYc = Y.ac, AZc = Z.ac;
    const int ax0 = X.atile0[bx], ay0 = Y.atile0[by], az0 = Z.atile0[bz];
    const int tid = threadIdx.x, lane = tid & 31, wy = tid >> 5;
    float *part = a.partial + size_t(tile_index) * a.slot;
    constexpr int AZP = TX3 + 1;              // Az row pitch (odd: the x stage reads along the rows)
    float *Az = sm3;                          // [3][AZc][8][AZP]
    float *Ax = Az + 3 * AZc * TY3 * AZP;     // [3][AZc][8][AXc]

    // tables, scalars and the first planes of the column, loaded up front
    const int x = x0 + lane, y = y0 + wy;
    const bool inxy = x < nx && y < ny;
    const size_t nxy = size_t(nx) * ny;
    const size_t col = size_t(min(y, ny - 1)) * nx + min(x, nx - 1);
    const float *__restrict__ W = a.warped;
    const float *__restrict__ R = a.ref;
    const bool bx_in = x > 0 && x < nx - 1, by_in = y > 0 && y < ny - 1;
    // column pointers at the current plane
    const float *__restrict__ wc = W + size_t(z0) * nxy + col;
    const float *__restrict__ rc = R + size_t(z0) * nxy + col;
    const int ynm = (y > 0) ? -nx : 0, ynp = (y + 1 < ny) ? nx : 0;
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
    // the warped image and the cost's scalars come from the warp kernel
    pdl_wait();
    pdl_trigger();
    if (tid < 5) {
        const int slot[5] = {SC_K1, SC_K2, SC_MA, SC_MB, SC_FSCALE};
        fsc[tid] = float(a.scalars[slot[tid]]);
        // the SSD force scale from the settings, as the finalisation sets it
        // (with a deferred finalisation it is not set yet)
        if (tid == 4 && cost == 0) fsc[4] = a.ssd_norm ? float(1.0 / double(size_t(nx) * ny * nz)) : 1.0f;
    }
    float wm = (z0 > 0) ? __ldg(wc - nxy) : 0.0f;
    float w0 = __ldg(wc);
    __syncthreads();
    const float k1 = fsc[0], k2 = fsc[1], ma = fsc[2], mb = fsc[3], hscale = 0.5f * fsc[4];

    float acc[3][4];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[c][k] = 0.0f;
    int cur = 0;   // azs[0] == 0
    auto emit = [&](int kz, int c, float v) { Az[((c * AZc + kz) * TY3 + wy) * AZP + lane] = v; };
#pragma unroll UNROLL
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
            // central differences without their factor 1/2, which joins
            // the force's scale
            g[0] = bx_in ? right - left : 0.0f;
            g[1] = by_in ? yp - ym : 0.0f;
            g[2] = (z > 0 && z < nz - 1) ? wp - wm : 0.0f;
            const float b = __ldg(rc);
            const float s = cost == 0 ? (w0 - b) * hscale : 0.5f * (k1 * (k2 * (w0 - ma) - (b - mb)));
#pragma unroll
            for (int k = 0; k < 3; ++k) f[k] = g[k] * s;
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
    // x stage, one thread per (c, kz, row) row of Az: the transposed
    // contraction over the tile's columns as a sliding window of four sums
    // (the column starts are the same for every thread, so the window moves
    // in lock step).  Contracting x before y keeps the intermediate small
    // (AXc instead of 32 values per row): the block needs less shared
    // memory and the two stages fewer instructions.
    for (int e = tid; e < 3 * AZc * TY3; e += NT3) {
        if ((e & (TY3 - 1)) >= ey) continue;   // rows below the image: never read
        const float *src = Az + e * AZP;
        float *dst = Ax + e * AXc;
        float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
        int oc = 0;
        // all TX3 columns: the walk leaves 0 in the columns beyond the image,
        // whose coefficient start is the last column's
#pragma unroll 8
        for (int l = 0; l < TX3; ++l) {
            const int o = asx[l];
            while (oc < o) {
                dst[oc] = s0;
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
        if (oc < AXc) dst[oc] = s0;
        if (oc + 1 < AXc) dst[oc + 1] = s1;
        if (oc + 2 < AXc) dst[oc + 2] = s2;
        if (oc + 3 < AXc) dst[oc + 3] = s3;
        for (int ix = oc + 4; ix < AXc; ++ix) dst[ix] = 0.0f;
    }
    __syncthreads();
    // y stage, one thread per (c, kz, ix) column of Ax, the same sliding
    // window over the rows, straight into the partial slot
    // ((kz AYc + jy) AXc + ix) 3 + c
    for (int e = tid; e < 3 * AZc * AXc; e += NT3) {
        const int c = e / (AZc * AXc), r = e - c * (AZc * AXc);
        const int kz = r / AXc, ix = r - kz * AXc;
        const float *src = Ax + (c * AZc + kz) * TY3 * AXc + ix;
        float *dst = part + (size_t(kz) * AYc * AXc + ix) * 3 + c;
        const int pitch = AXc * 3;
        float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
        int oc = 0;
        for (int yy = 0; yy < ey; ++yy) {
            const int o = asy[yy];
            while (oc < o) {
                dst[oc * pitch] = s0;
                s0 = s1;
                s1 = s2;
                s2 = s3;
                s3 = 0.0f;
                ++oc;
            }
            const float4 w = awy[yy];
            const float f = src[yy * AXc];
            s0 += w.x * f;
            s1 += w.y * f;
            s2 += w.z * f;
            s3 += w.w * f;
        }
        if (oc < AYc) dst[oc * pitch] = s0;
        if (oc + 1 < AYc) dst[(oc + 1) * pitch] = s1;
        if (oc + 2 < AYc) dst[(oc + 2) * pitch] = s2;
        if (oc + 3 < AYc) dst[(oc + 3) * pitch] = s3;
        for (int jy = oc + 4; jy < AYc; ++jy) dst[jy * pitch] = 0.0f;
    }
}

// ---------------------------------------------------------------------
// gather + penalty
// ---------------------------------------------------------------------
#ifndef MGR_GATHER_THREADS
#define MGR_GATHER_THREADS 256
#endif
#ifdef MGR_GATHER_MINB
#define MGR_GATHER_BOUNDS __launch_bounds__(MGR_GATHER_THREADS, MGR_GATHER_MINB)
#else
#define MGR_GATHER_BOUNDS __launch_bounds__(MGR_GATHER_THREADS)
#endif
namespace {
constexpr int GT3 = MGR_GATHER_THREADS;
constexpr int GBX = 4, GBY = 4, GBZ = 2;   // coefficients per block: 32, lane = coefficient
constexpr int GH = 3;                      // stencil half width
constexpr int GPX = GBX + 2 * GH;          // 10: halo tile edges
constexpr int GPY = GBY + 2 * GH;          // 10
constexpr int GPZ = GBZ + 2 * GH;          // 8
constexpr int GPP = 12;                    // padded row pitch (float4) of the halo tile
constexpr int GSUB = GT3 / 32;             // the warps split each coefficient's work
constexpr int GNQ = 12;                    // per-warp partials: 9 penalty products, 3 image sums
constexpr int GSMAX = 64 / GSUB;           // partial slots per warp loaded in the first batch
// the per-warp partials fit beside the halo tables at 8 warps; with more
// warps they take the tables' place once the stencil is summed
constexpr int GTAB = GPZ * GPY * GPP + 343 * 2;   // float4: Ps, then Pt
constexpr bool GALIAS = GSUB * GNQ * 32 > 12 * 32 * 8;
static_assert(!GALIAS || GSUB * GNQ * 32 <= 4 * GTAB, "partials must fit in the tables' space");
}  // namespace

// Block: 4 x 4 x 2 coefficients, one per lane; the 8 warps split the 49
// (dz, dy) rows of the 7^3 divcurl stencil and the partial slots.  Loads are
// issued in two batches: the tables, the parameters with a 3-node halo and
// the penalty cells; then the partial slots, in flight while the stencil
// is summed.
__device__ __forceinline__ void gather3_body(const EvalArgs &a, int with_gradient, int image_from_dense, int blk,
                                             int nblk)
{
    __shared__ float4 PsPt[GTAB];
    __shared__ float pacc_own[GALIAS ? 1 : GSUB * GNQ * 32];
    __shared__ int gl[3][GBX][GATHER_LMAX];
    __shared__ int gn[3][GBX];
    __shared__ bool is_last;
    float4 *Ps = PsPt, *Pt = PsPt + GPZ * GPY * GPP;
    float (*pacc)[GNQ][32] = reinterpret_cast<float (*)[GNQ][32]>(GALIAS ? reinterpret_cast<float *>(PsPt) : pacc_own);
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    const int ncx = a.nc[0], ncy = a.nc[1], ncz = a.nc[2];
    const int nbx = (ncx + GBX - 1) / GBX, nby = (ncy + GBY - 1) / GBY;
    const int bxi = blk % nbx, byi = (blk / nbx) % nby, bzi = blk / (nbx * nby);
    const int cx0 = bxi * GBX, cy0 = byi * GBY, cz0 = bzi * GBZ;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int lx = lane & 3, ly = (lane >> 2) & 3, lz = lane >> 4;
    const int cx = cx0 + lx, cy = cy0 + ly, cz = cz0 + lz;
    const bool valid = cx < ncx && cy < ncy && cz < ncz;
    const size_t i = valid ? (size_t(cz) * ncy + cy) * ncx + cx : 0;
    const bool img = with_gradient && !image_from_dense;

    // fixed tables first: offset lists and penalty cells
    if (img && tid < 3 * GBX) {
        const int ax = tid / GBX, k = tid - ax * GBX;
        const Axis &A = a.ax[ax];
        const int c = (ax == 0 ? cx0 : ax == 1 ? cy0 : cz0) + k;
        int cnt = 0;
        if (c < A.nc && (ax < 2 || k < GBZ)) {
            cnt = A.glen[c];
            for (int j = 0; j < cnt; ++j) gl[ax][k][j] = A.glist[size_t(c) * GATHER_LMAX + j];
        }
        gn[ax][k] = cnt;
    }
    if (a.has_penalty) {
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
        for (int k = 0; k < KT; ++k) {
            const int e = tid + k * GT3;
            if (e < 343) {
                Pt[2 * e] = make_float4(tv[k][0], tv[k][1], tv[k][2], tv[k][3]);
                Pt[2 * e + 1] = make_float4(tv[k][4], tv[k][5], 0.0f, 0.0f);
            }
        }
    }
    // The divcurl stencil needs only the parameters' float copy, which
    // every launch order of this kernel has completed before any block of
    // it starts (the conversion kernel is never launched directly before
    // it; the kernel between them waits for the conversion before it lets
    // this one launch).  So the stencil runs before the dependency wait,
    // while the adjoint kernel finishes; the copy is read through the L2
    // (ld.global.cg), never from a line an earlier kernel left in L1.
    if (a.has_penalty) {
        constexpr int NH = GPX * GPY * GPZ;
        constexpr int KP = (NH + GT3 - 1) / GT3;
        float pv[KP][3];
#pragma unroll
        for (int k = 0; k < KP; ++k) {
            const int e = tid + k * GT3;
            pv[k][0] = pv[k][1] = pv[k][2] = 0.0f;
            if (e < NH) {
                const int hx = e % GPX, hy = (e / GPX) % GPY, hz = e / (GPX * GPY);
                const int gx = cx0 - GH + hx, gy = cy0 - GH + hy, gz = cz0 - GH + hz;
                if (gx >= 0 && gx < ncx && gy >= 0 && gy < ncy && gz >= 0 && gz < ncz) {
                    const float *p = a.params_f + ((size_t(gz) * ncy + gy) * ncx + gx) * 3;
                    pv[k][0] = __ldcg(p);
                    pv[k][1] = __ldcg(p + 1);
                    pv[k][2] = __ldcg(p + 2);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < KP; ++k) {
            const int e = tid + k * GT3;
            if (e < NH) {
                const int hx = e % GPX, hy = (e / GPX) % GPY, hz = e / (GPX * GPY);
                Ps[(hz * GPY + hy) * GPP + hx] = make_float4(pv[k][0], pv[k][1], pv[k][2], 0.0f);
            }
        }
    }
    __syncthreads();   // the offset lists, the parameter halo
    // R0..R5, T0..T2: the nine products of the 3x3 cell with c_j, summed
    // over the 7^3 neighbours j = i - d (zero outside the grid)
    float R0 = 0, R1 = 0, R2 = 0, R3 = 0, R4 = 0, R5 = 0, T0 = 0, T1 = 0, T2 = 0;
    if (valid && a.has_penalty) {
        for (int p = w; p < 49; p += GSUB) {
            const int dz = p / 7 - 3, dy = p % 7 - 3;
            const float4 *prow = Ps + ((lz + GH - dz) * GPY + (ly + GH - dy)) * GPP + (lx + GH);
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
    pdl_wait();
    pdl_trigger();
    // the adjoint's partial slots: this warp's share (entries k = w,
    // w + GSUB, ...) of the lane's coefficient, one batch of loads
    constexpr int SMAX = GSMAX;
    float sv[SMAX][3];
    int tot = 0, nX = 0, nY = 0, nZ = 0;
    bool lists = false;
    if (valid && img) {
        nX = gn[0][lx];
        nY = gn[1][ly];
        nZ = gn[2][lz];
        lists = nX >= 0 && nY >= 0 && nZ >= 0;
        if (lists) tot = nX * nY * nZ;
    }
#pragma unroll
    for (int u = 0; u < SMAX; ++u) {
        const int k = w + GSUB * u;
        sv[u][0] = sv[u][1] = sv[u][2] = 0.0f;
        if (k < tot) {
            const int jx = k % nX, r = k / nX;
            const int jy = r % nY, jz = r / nY;
            const float *p = a.partial + (size_t(gl[2][lz][jz] + gl[1][ly][jy]) + gl[0][lx][jx]);
            sv[u][0] = p[0];
            sv[u][1] = p[1];
            sv[u][2] = p[2];
        }
    }
    float S0 = 0.0f, S1 = 0.0f, S2 = 0.0f;
#pragma unroll
    for (int u = 0; u < SMAX; ++u) {
        S0 += sv[u][0];
        S1 += sv[u][1];
        S2 += sv[u][2];
    }
    if (valid && img) {
        if (lists) {
            for (int k = w + GSUB * SMAX; k < tot; k += GSUB) {
                const int jx = k % nX, r = k / nX;
                const int jy = r % nY, jz = r / nY;
                const float *p = a.partial + (size_t(gl[2][lz][jz] + gl[1][ly][jy]) + gl[0][lx][jx]);
                S0 += p[0];
                S1 += p[1];
                S2 += p[2];
            }
        } else {
            const int2 gx = X.gtile[cx], gy = Y.gtile[cy], gz = Z.gtile[cz];
            const int mX = gx.y - gx.x + 1, mY = gy.y - gy.x + 1, mZ = gz.y - gz.x + 1;
            const int mt = (mX > 0 && mY > 0 && mZ > 0) ? mX * mY * mZ : 0;
            for (int k = w; k < mt; k += GSUB) {
                const int tx = gx.x + k % mX, ty = gy.x + (k / mX) % mY, tz = gz.x + k / (mX * mY);
                const int lxo = cx - X.atile0[tx], lyo = cy - Y.atile0[ty], lzo = cz - Z.atile0[tz];
                const size_t t = (size_t(tz) * Y.nt + ty) * X.nt + tx;
                const float *p = a.partial + t * a.slot + ((size_t(lzo) * Y.ac + lyo) * X.ac + lxo) * 3;
                S0 += p[0];
                S1 += p[1];
                S2 += p[2];
            }
        }
    }
    // the lane's own parameters (the penalty value), read before the
    // partials may take the tables' place
    float ci[3] = {0.0f, 0.0f, 0.0f};
    if (w == 0 && a.has_penalty) {
        const float4 c4 = Ps[((lz + GH) * GPY + (ly + GH)) * GPP + (lx + GH)];
        ci[0] = c4.x;
        ci[1] = c4.y;
        ci[2] = c4.z;
    }
    if (GALIAS) __syncthreads();
    pacc[w][0][lane] = R0;
    pacc[w][1][lane] = R1;
    pacc[w][2][lane] = R2;
    pacc[w][3][lane] = R3;
    pacc[w][4][lane] = R4;
    pacc[w][5][lane] = R5;
    pacc[w][6][lane] = T0;
    pacc[w][7][lane] = T1;
    pacc[w][8][lane] = T2;
    pacc[w][9][lane] = S0;
    pacc[w][10][lane] = S1;
    pacc[w][11][lane] = S2;
    __syncthreads();
    // the warps' partials of each quantity summed in a fixed order (FP32,
    // warp k % GSUB sums quantity k into row 0), then warp 0 combines them
    // (the outputs are widened to double at the store)
    for (int k = w; k < GNQ; k += GSUB) {
        float t = pacc[0][k][lane];
#pragma unroll
        for (int ww = 1; ww < GSUB; ++ww) t += pacc[ww][k][lane];
        pacc[0][k][lane] = t;
    }
    __syncthreads();
    if (w == 0) {
        float pval = 0.0f;
        // parameters the conversion found non-finite: nothing is written to
        // the caller's buffers (uniform over the block)
        const bool bad = a.params_host && *(volatile unsigned *)&a.counters[7] != 0u;
        double gt[3] = {0.0, 0.0, 0.0};
        if (valid) {
            float v9[GNQ];
#pragma unroll
            for (int k = 0; k < GNQ; ++k) v9[k] = pacc[0][k][lane];
            float gp[3] = {0.0f, 0.0f, 0.0f};
            const float pw = float(a.pen_grad_sign * a.pen_weight), cw = float(a.cost_weight);
            if (a.has_penalty) {
                const float ci0 = ci[0], ci1 = ci[1], ci2 = ci[2];
                if (with_gradient)
                    pval = ci0 * v9[0] + ci0 * v9[1] + ci1 * v9[2] + ci1 * v9[3] + ci2 * v9[4] + ci2 * v9[5];
                else
                    pval = ci0 * v9[0] + ci1 * v9[2] + ci2 * v9[4] + ci0 * v9[1] + ci0 * v9[6] + ci1 * v9[3];
                gp[0] = pw * (v9[6] + (2.0f * v9[0] + v9[1]));
                gp[1] = pw * (v9[7] + (2.0f * v9[2] + v9[3]));
                gp[2] = pw * (v9[8] + (2.0f * v9[4] + v9[5]));
            }
            if (with_gradient && !bad) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const double gi = image_from_dense ? a.grad_image[i * 3 + k] : double(cw * -v9[9 + k]);
                    gt[k] = gi + double(gp[k]);
                    if (a.grad_image && !image_from_dense) a.grad_image[i * 3 + k] = gi;
                    if (a.grad_penalty) a.grad_penalty[i * 3 + k] = double(gp[k]);
                }
            }
        }
        if (with_gradient && !bad && !a.params_host) {
            if (valid)
#pragma unroll
                for (int k = 0; k < 3; ++k) a.grad_total[i * 3 + k] = gt[k];
        } else if (with_gradient && !bad) {
            // the total gradient into the caller's host memory: the lanes of
            // a row (ly, lz) hold four consecutive coefficients, 96
            // contiguous bytes of the output; a row whose four coefficients
            // are all in the grid and whose start is 16-byte aligned is
            // stored as six 16-byte pieces (few large writes over the
            // CPU-GPU link: an evaluation from host buffers took 153.9
            // instead of 158.0 us at 192x192x128), any other lane stores
            // its own three values
            __shared__ __align__(16) double gst[32 * 3];
#pragma unroll
            for (int k = 0; k < 3; ++k) gst[lane * 3 + k] = gt[k];
            __syncwarp();
            auto row_dst = [&](int r) -> double * {
                const int ry = cy0 + (r & 3), rz = cz0 + (r >> 2);
                return a.grad_total + ((size_t(rz) * ncy + ry) * ncx + cx0) * 3;
            };
            auto row_vec = [&](int r) -> bool {
                const int ry = cy0 + (r & 3), rz = cz0 + (r >> 2);
                return cx0 + GBX <= ncx && ry < ncy && rz < ncz &&
                       (reinterpret_cast<uintptr_t>(row_dst(r)) & 15u) == 0;
            };
            for (int c = lane; c < 48; c += 32) {
                const int r = c / 6, piece = c - r * 6;
                if (row_vec(r))
                    reinterpret_cast<double2 *>(row_dst(r))[piece] =
                        *reinterpret_cast<const double2 *>(&gst[r * 12 + piece * 2]);
            }
            if (valid && !row_vec(lane >> 2))
#pragma unroll
                for (int k = 0; k < 3; ++k) a.grad_total[i * 3 + k] = gt[k];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) pval += __shfl_xor_sync(FULL, pval, o);
        if (lane == 0) {
            a.pen_part[blk] = double(pval);
            __threadfence();
            is_last = (atomicAdd(&a.counters[1], 1u) == unsigned(nblk - 1));
        }
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        __shared__ double red[2 * (GT3 / 32)];
        // v[0]: a deferred SSD cost from the warp kernel's tile sums (the
        // fixed-order reduction of reduce_tile_sums: same striding, same
        // tree); v[1]: the blocks' penalty partials; one pass for both
        const bool fin = a.defer_cost && a.cost == 0;
        double v2[2] = {0.0, 0.0};
        if (fin) {
            const int ntw = a.ax[0].nt * a.ax[1].nt * a.ax[2].nt;
            for (int t = tid; t < ntw; t += GT3) v2[0] += ((volatile double *)a.tile_sums)[size_t(t) * 5];
        }
        for (unsigned b = tid; b < unsigned(nblk); b += GT3) v2[1] += ((volatile double *)a.pen_part)[b];
        block_sum<2>(v2, red);
        if (tid == 0) {
            if (fin) {
                const double s5[5] = {v2[0], 0.0, 0.0, 0.0, 0.0};
                finalise_cost(a, s5, size_t(a.n[0]) * a.n[1] * a.n[2]);
            }
            double *sc = a.scalars;
            const double pen = a.has_penalty ? v2[1] : 0.0;
            sc[SC_PEN] = pen;
            sc[SC_COST_IMG] = a.cost_weight * sc[SC_VALUE];
            sc[SC_COST_PEN] = a.has_penalty ? a.pen_weight * pen : 0.0;
            if (a.costs) {
                a.costs[0] = sc[SC_COST_IMG];
                a.costs[1] = sc[SC_COST_PEN];
            }
            if (a.host_out) {
                // the costs and both status flags to the caller's host
                // memory; the non-finite flag is cleared for the next call
                // (every block has read it before its arrival above)
                a.host_out[0] = sc[SC_COST_IMG];
                a.host_out[1] = sc[SC_COST_PEN];
                unsigned *hf = reinterpret_cast<unsigned *>(a.host_out + 2);
                hf[0] = *(volatile unsigned *)&a.counters[6];
                hf[1] = *(volatile unsigned *)&a.counters[7];
                a.counters[7] = 0;
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

template <int TZ, int COST>
__global__ void __launch_bounds__(NT3, MGR_WARP_MINB) k_warp3(const __grid_constant__ EvalArgs a)
{
    const int tile = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    warp3_body<TZ, COST>(a, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.x * gridDim.y * gridDim.z, tile);
}

template <int TZ>
__global__ void MGR_ADJ_BOUNDS k_adjoint3(EvalArgs a)
{
    const int tile = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    adjoint3_body<TZ, MGR_ADJ_UNROLL>(a, blockIdx.x, blockIdx.y, blockIdx.z, tile);
}

__global__ void MGR_GATHER_BOUNDS k_gather3(EvalArgs a, int with_gradient, int image_from_dense)
{
    gather3_body(a, with_gradient, image_from_dense, blockIdx.x, gridDim.x);
}

// The NCC cost and force constants from the warp kernel's tile sums, one
// block of NT3 threads: the reduction the warp kernel's last block makes
// otherwise (same striding, same order), so that the warp blocks end
// without a device-wide fence.  The adjoint kernel after it reads the
// constants.
__global__ void __launch_bounds__(NT3) k_finalise3(EvalArgs a)
{
    __shared__ double red[5 * (NT3 / 32)];
    pdl_wait();
    pdl_trigger();
    reduce_tile_sums(a, a.ax[0].nt * a.ax[1].nt * a.ax[2].nt, size_t(a.n[0]) * a.n[1] * a.n[2], red);
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
    warp3_body<TZ, -1>(a, bx, by, bz, nt, it.y);
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
    adjoint3_body<TZ, 1>(a, bx, by, bz, it.y);
}

// Persistent forms of the batched warp and adjoint kernels: a grid of
// resident blocks draws (pair, tile) items from a device queue (queue[0],
// one atomic per item); the last block to finish resets the queue for the
// next launch (queue[1] counts finished blocks), so the launch can be
// replayed from a CUDA graph.
__device__ __forceinline__ bool next_item(int *queue, int nitems, const int2 *items, int2 &it, int &slot)
{
    __syncthreads();   // every thread is done with the previous item's shared memory
    if (threadIdx.x == 0) slot = atomicAdd(&queue[0], 1);
    __syncthreads();
    const int i = slot;
    if (i >= nitems) return false;
    it = items[i];
    return true;
}

__device__ __forceinline__ void queue_done(int *queue)
{
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&queue[1], 1) == int(gridDim.x) - 1) {
            queue[0] = 0;
            queue[1] = 0;
            __threadfence();
        }
    }
}

template <int TZ>
__global__ void __launch_bounds__(NT3, MGR_WARP_MINB) k_warp3_queue(const EvalArgs *__restrict__ args,
                                                                    const int2 *__restrict__ items, int nitems,
                                                                    const int *__restrict__ active, int *queue)
{
    __shared__ int slot;
    int2 it;
    while (next_item(queue, nitems, items, it, slot)) {
        if (!active[it.x]) continue;
        const EvalArgs &a = args[it.x];
        int bx, by, bz, nt;
        decode_tile3(a, it.y, bx, by, bz, nt);
        warp3_body<TZ, -1>(a, bx, by, bz, nt, it.y);
    }
    queue_done(queue);
}

template <int TZ>
__global__ void __launch_bounds__(NT3) k_adjoint3_queue(const EvalArgs *__restrict__ args,
                                                        const int2 *__restrict__ items, int nitems,
                                                        const int *__restrict__ active, int *queue)
{
    __shared__ int slot;
    int2 it;
    while (next_item(queue, nitems, items, it, slot)) {
        if (!active[it.x]) continue;
        const EvalArgs &a = args[it.x];
        int bx, by, bz, nt;
        decode_tile3(a, it.y, bx, by, bz, nt);
        adjoint3_body<TZ, 1>(a, bx, by, bz, it.y);
    }
    queue_done(queue);
}

__global__ void MGR_GATHER_BOUNDS k_gather3_batch(const EvalArgs *__restrict__ args,
                                                       const int2 *__restrict__ items, const int *__restrict__ active,
                                                       const int *__restrict__ nblocks)
{
    const int2 it = items[blockIdx.x];
    if (!active[it.x]) return;
    gather3_body(args[it.x], 1, 0, it.y, nblocks[it.x]);
}

// float copy of the parameters (the warp and gather kernels read them as
// float, as the reference's spline evaluation does; FP64 conversions are
// slow on this GPU, so they are done once per evaluation)
__global__ void __launch_bounds__(256) k_params_f32(const double *__restrict__ p, float *__restrict__ f, size_t n)
{
    pdl_trigger();   // the warp kernel may start its set-up (it waits for this kernel)
    for (size_t i = blockIdx.x * size_t(256) + threadIdx.x; i < n; i += size_t(gridDim.x) * 256) f[i] = float(p[i]);
}

// ---------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------
// A launch that may start while the kernel before it in the stream is still
// running (programmatic stream serialisation; the kernel waits in pdl_wait
// before it reads that kernel's outputs), or a plain stream-ordered launch.
template <typename... KArgs, typename... Args>
static void launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

// The parameters read where the caller holds them (host memory that the
// device reads coherently): the device keeps a double and a float copy.  A
// non-finite value is stored as 0 in both and raises counters[7], so that
// the kernels after it run on finite parameters and the gather writes
// nothing to the caller's buffers.
__global__ void __launch_bounds__(256) k_params_host(const double *__restrict__ src, double *__restrict__ p,
                                                     float *__restrict__ f, size_t n, unsigned *__restrict__ bad)
{
    pdl_trigger();   // the warp kernel may start its set-up (it waits for this kernel)
    bool nonfinite = false;
    for (size_t i = blockIdx.x * size_t(256) + threadIdx.x; i < n; i += size_t(gridDim.x) * 256) {
        double v = src[i];
        if (!isfinite(v)) {
            nonfinite = true;
            v = 0.0;
        }
        p[i] = v;
        f[i] = float(v);
    }
    if (__any_sync(FULL, nonfinite) && (threadIdx.x & 31) == 0) atomicOr(bad, 1u);
}

void launch_params_f32(const EvalArgs &a, cudaStream_t st)
{
    const size_t n = size_t(a.nc[0]) * a.nc[1] * a.nc[2] * 3;
    const int nb = int(std::min<size_t>(1024, (n + 255) / 256));
    if (a.params_host)
        k_params_host<<<nb, 256, 0, st>>>(a.params_host, const_cast<double *>(a.params), a.params_f, n,
                                          a.counters + 7);
    else
        k_params_f32<<<nb, 256, 0, st>>>(a.params, a.params_f, n);
    count_launch();
}
size_t split3_smem(const EvalArgs &a, int which)
{
    const Axis &X = a.ax[0], &Y = a.ax[1], &Z = a.ax[2];
    if (which == 0)
        return size_t(3) * Z.fc * Y.fc * (X.fc + TX3) * sizeof(float) + 128 +
               size_t(RING_N) * RING_PLANE * sizeof(float);
    return size_t(3) * Z.ac * TY3 * (TX3 + 1 + X.ac) * sizeof(float);
}

namespace {

// the z-tile lengths the single-level kernels are compiled for:
// fn(std::integral_constant<int, TZ>{}) for the length tz, false when tz is
// not one of them.  The lengths between the powers of two let the
// autotuner fit a level's tiles to the waves of resident blocks: 128 planes
// in 20-plane tiles end with a row of 8-plane tiles that fills the last
// wave's gaps, where 16-plane tiles leave half of the last wave idle.
template <typename Fn>
bool with_tz(int tz, Fn &&fn)
{
    switch (tz) {
    case 4: fn(std::integral_constant<int, 4>{}); return true;
    case 8: fn(std::integral_constant<int, 8>{}); return true;
    case 12: fn(std::integral_constant<int, 12>{}); return true;
    case 16: fn(std::integral_constant<int, 16>{}); return true;
    case 20: fn(std::integral_constant<int, 20>{}); return true;
    case 24: fn(std::integral_constant<int, 24>{}); return true;
    case 32: fn(std::integral_constant<int, 32>{}); return true;
    default: return false;
    }
}

// the z-tile lengths of the batched and persistent kernels (the
// registration drivers run 16-plane tiles)
template <typename Fn>
bool with_tz_batch(int tz, Fn &&fn)
{
    switch (tz) {
    case 4: fn(std::integral_constant<int, 4>{}); return true;
    case 8: fn(std::integral_constant<int, 8>{}); return true;
    case 16: fn(std::integral_constant<int, 16>{}); return true;
    case 32: fn(std::integral_constant<int, 32>{}); return true;
    default: return false;
    }
}

}  // namespace

bool tile_supported3(int tx, int ty, int tz)
{
    return tx == TX3 && ty == TY3 && with_tz(tz, [](auto) {});
}

bool tile_supported3_batch(int tx, int ty, int tz)
{
    return tx == TX3 && ty == TY3 && with_tz_batch(tz, [](auto) {});
}

namespace {

template <int TZ, int COST>
void launch_warp3_zc(const EvalArgs &a, size_t sm, cudaStream_t st)
{
    raise_smem_limit(reinterpret_cast<const void *>(k_warp3<TZ, COST>), sm);
    launch_pdl(a.pdl != 0, k_warp3<TZ, COST>, dim3(a.ax[0].nt, a.ax[1].nt, a.ax[2].nt), dim3(NT3), sm, st, a);
}
template <int TZ>
void launch_warp3_z(const EvalArgs &a, size_t sm, cudaStream_t st)
{
    if (a.cost == MGR_COST_SSD)
        launch_warp3_zc<TZ, MGR_COST_SSD>(a, sm, st);
    else
        launch_warp3_zc<TZ, MGR_COST_NCC>(a, sm, st);
}

template <int TZ>
void launch_adjoint3_z(const EvalArgs &a, size_t sm, cudaStream_t st)
{
    raise_smem_limit(reinterpret_cast<const void *>(k_adjoint3<TZ>), sm);
    launch_pdl(a.pdl != 0, k_adjoint3<TZ>, dim3(a.ax[0].nt, a.ax[1].nt, a.ax[2].nt), dim3(NT3), sm, st, a);
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
    cudaFuncSetAttribute(k_warp3_queue<TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm_warp));
    cudaFuncSetAttribute(k_adjoint3_queue<TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm_adj));
}

// resident blocks of the persistent kernels (blocks per SM x SMs)
template <int TZ>
int queue_grid_z(int which, size_t sm)
{
    int per_sm = 0;
    if (which == 0)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_warp3_queue<TZ>, NT3, sm);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adjoint3_queue<TZ>, NT3, sm);
    return std::max(1, per_sm) * device_sm_count();
}

template <int TZ>
void queue3_z(const EvalArgs *args, const int2 *items, int nitems, const int *active, int *queue, int grid, size_t sm,
              int which, cudaStream_t st)
{
    if (which == 0)
        k_warp3_queue<TZ><<<grid, NT3, sm, st>>>(args, items, nitems, active, queue);
    else
        k_adjoint3_queue<TZ><<<grid, NT3, sm, st>>>(args, items, nitems, active, queue);
}

}  // namespace

void launch_warp3(const EvalArgs &a, cudaStream_t st)
{
    launch_params_f32(a, st);
    const size_t sm = split3_smem(a, 0);
    with_tz(a.ax[2].t, [&](auto z) { launch_warp3_z<decltype(z)::value>(a, sm, st); });
    count_launch();
    if (a.defer_cost && a.cost != MGR_COST_SSD) {
        launch_pdl(a.pdl != 0, k_finalise3, dim3(1), dim3(NT3), 0, st, a);
        count_launch();
    }
}

void launch_adjoint3(const EvalArgs &a, cudaStream_t st)
{
    const size_t sm = split3_smem(a, 1);
    with_tz(a.ax[2].t, [&](auto z) { launch_adjoint3_z<decltype(z)::value>(a, sm, st); });
    count_launch();
}

int gather3_blocks(const EvalArgs &a)
{
    return ((a.nc[0] + GBX - 1) / GBX) * ((a.nc[1] + GBY - 1) / GBY) * ((a.nc[2] + GBZ - 1) / GBZ);
}

void launch_gather3(const EvalArgs &a, int with_gradient, int dense, cudaStream_t st)
{
    launch_pdl(a.pdl != 0, k_gather3, dim3(gather3_blocks(a)), dim3(GT3), 0, st, a, with_gradient, dense);
    count_launch();
}

void prepare_split3_batch(int tz, size_t sm_warp, size_t sm_adj)
{
    with_tz_batch(tz, [&](auto z) { prepare3_z<decltype(z)::value>(sm_warp, sm_adj); });
}

void launch_split3_batch(int tz, const EvalArgs *args, const int2 *items, int nitems, const int *active, size_t sm,
                         int which, cudaStream_t st)
{
    with_tz_batch(tz, [&](auto z) { batch3_z<decltype(z)::value>(args, items, nitems, active, sm, which, st); });
    count_launch();
}

int split3_queue_grid(int tz, int which, size_t sm)
{
    int g = 0;
    with_tz_batch(tz, [&](auto z) { g = queue_grid_z<decltype(z)::value>(which, sm); });
    return g;
}

void launch_split3_queue(int tz, const EvalArgs *args, const int2 *items, int nitems, const int *active, int *queue,
                         int grid, size_t sm, int which, cudaStream_t st)
{
    with_tz_batch(tz, [&](auto z) { queue3_z<decltype(z)::value>(args, items, nitems, active, queue, grid, sm, which, st); });
    count_launch();
}

void launch_gather3_batch(const EvalArgs *args, const int2 *items, int nitems, const int *active, const int *nblocks,
                          cudaStream_t st)
{
    k_gather3_batch<<<nitems, GT3, 0, st>>>(args, items, active, nblocks);
    count_launch();
}

}  // namespace mgr

// Self-test of the bounded wait: one thread waits on phase 0 of an mbarrier
// that nothing arrives at (no copy is in flight), with the warp kernel's
// wait at a limit of SELFTEST_TRIES tries; it must give up and raise the
// flag, and the global timer (nanoseconds, independent of the SM clock)
// gives the time of one failed try.
namespace {
constexpr int SELFTEST_TRIES = 1024;

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void k_bounded_wait_selftest(unsigned *flag, long long *ns)
{
    __shared__ __align__(8) unsigned long long mb;
    const unsigned a = mgr::smem_u32(&mb);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
    const unsigned long long t0 = global_ns();
    if (!mgr::mbar_wait<SELFTEST_TRIES>(a, 0u)) atomicOr(flag, 1u);
    *ns = (long long)(global_ns() - t0);
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(a) : "memory");
}
}  // namespace

extern "C" mgr_status mgr_selftest_bounded_wait(int device, int *gave_up, double *us_per_try)
{
    if (!gave_up || !us_per_try) {
        mgr::set_last_error("mgr_selftest_bounded_wait: null argument");
        return MGR_ERR_ARG;
    }
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    unsigned *flag = nullptr;
    long long *ns = nullptr;
    unsigned f = 0;
    long long t = 0;
    if (e == cudaSuccess) e = cudaSetDevice(device);
    if (e == cudaSuccess) e = mgr::dev_malloc(reinterpret_cast<void **>(&flag), sizeof(unsigned));
    if (e == cudaSuccess) e = mgr::dev_malloc(reinterpret_cast<void **>(&ns), sizeof(long long));
    if (e == cudaSuccess) e = cudaMemset(flag, 0, sizeof(unsigned));
    if (e == cudaSuccess) {
        k_bounded_wait_selftest<<<1, 1>>>(flag, ns);
        mgr::count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&f, flag, sizeof f, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&t, ns, sizeof t, cudaMemcpyDeviceToHost);
    cudaFree(flag);
    cudaFree(ns);
    cudaSetDevice(prev);   // the caller's current device is left as it was
    if (e != cudaSuccess) {
        mgr::set_last_error(std::string("mgr_selftest_bounded_wait: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? MGR_ERR_OOM : MGR_ERR_CUDA;
    }
    *gave_up = f ? 1 : 0;
    *us_per_try = double(t) * 1e-3 / SELFTEST_TRIES;
    return MGR_OK;
}
