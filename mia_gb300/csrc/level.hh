// level.hh — the per-level state behind an mgr_level handle (device
// buffers, tables, stream); shared by the C ABI and the batched driver.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mgr.h"
#include "mgr_kernels.hh"
#include "tables.hh"
#include "tune.hh"

namespace mgr {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct StateError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
// a bounded device wait gave up (the kernel raised the level's status flag)
struct TimeoutError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void ck(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        std::string m = std::string(what) + ": " + cudaGetErrorString(e);
        if (e == cudaErrorMemoryAllocation) throw std::bad_alloc();
        throw CudaError(m);
    }
}

// Keep freed stream-ordered allocations of `device` cached in its default
// memory pool (up to a bound) so that repeated level setup does not map and
// unmap device memory.
void configure_pool(int device);

// Device buffer in stream-ordered memory: allocated on and freed on the
// stream given to alloc(), which must outlive the buffer.  Growing keeps the
// old contents only when the old allocation is large enough.
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t st = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count, cudaStream_t s)
    {
        if (count <= n && p) return;
        release();
        if (count == 0) return;
        ck(dev_malloc_async(reinterpret_cast<void **>(&p), count * sizeof(T), s), "cudaMallocAsync");
        st = s;
        n = count;
    }
    void upload(const std::vector<T> &h, cudaStream_t s)
    {
        alloc(h.size(), s);
        if (!h.empty()) ck(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
    }
};

// the per-axis tables of a level, packed with the other tables into one
// host blob and uploaded with one copy; `off` are byte offsets into it
struct AxisDev {
    AxisHost h;
    size_t off[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};   // fs, as, rows, ftile0, atile0, gtile, fw, aw, glist, glen
    const unsigned char *base = nullptr;

    template <class T>
    static size_t pack(std::vector<unsigned char> &blob, const std::vector<T> &v)
    {
        const size_t o = (blob.size() + 255) & ~size_t(255);
        blob.resize(o + v.size() * sizeof(T));
        if (!v.empty()) std::memcpy(blob.data() + o, v.data(), v.size() * sizeof(T));
        return o;
    }
    void pack_all(std::vector<unsigned char> &blob)
    {
        off[0] = pack(blob, h.fs);
        off[1] = pack(blob, h.as);
        off[2] = pack(blob, h.rows);
        off[3] = pack(blob, h.ftile0);
        off[4] = pack(blob, h.atile0);
        off[5] = pack(blob, h.gtile);
        off[6] = pack(blob, h.fw);
        off[7] = pack(blob, h.aw);
        off[8] = pack(blob, h.glist);
        off[9] = pack(blob, h.glen);
    }
    Axis view() const
    {
        Axis a;
        a.fs = reinterpret_cast<const int *>(base + off[0]);
        a.as = reinterpret_cast<const int *>(base + off[1]);
        a.rows = reinterpret_cast<const int2 *>(base + off[2]);
        a.ftile0 = reinterpret_cast<const int *>(base + off[3]);
        a.atile0 = reinterpret_cast<const int *>(base + off[4]);
        a.gtile = reinterpret_cast<const int2 *>(base + off[5]);
        a.fw = reinterpret_cast<const float4 *>(base + off[6]);
        a.aw = reinterpret_cast<const float4 *>(base + off[7]);
        a.glist = reinterpret_cast<const int *>(base + off[8]);
        a.glen = reinterpret_cast<const int *>(base + off[9]);
        a.n = h.n;
        a.nc = h.nc;
        a.t = h.t;
        a.nt = h.nt;
        a.fc = h.fc;
        a.ac = h.ac;
        return a;
    }
};

}  // namespace mgr

using namespace mgr;

struct mgr_level {
    mgr_level_desc d{};
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int n[3] = {1, 1, 1}, nc[3] = {1, 1, 1};
    size_t N = 0, ncoef = 0, nparams = 0;
    int path = MGR_PATH_SPLIT;
    int tile[3] = {32, 8, 16};
    AxisDev ax[3];
    DevBuf<unsigned char> axis_tables;   // the packed AxisDev tables
    // MGR_PATH_FUSED: the tables of the fused kernel's tiles (30 x 8 x TZ),
    // for its launch and the gather after it; the other kernels keep ax
    AxisDev axf[3];
    DevBuf<unsigned char> axis_tables_f;
    int slot_f = 0;
    DevBuf<float> coef, coef_pad, ref, warped, minmax, partial, ptable, pen_val, params_f;
    DevBuf<float2> mmpart;
    DevBuf<double> params, grad_total, grad_image, grad_penalty, scalars, costs, tile_sums, pen_part, means, mpart;
    DevBuf<unsigned int> counters;
    DevBuf<int> pen_rowptr, pen_col;
    DevBuf<float> grid, force, tmp1, tmp2;   // plain path and standalone force/translate
    // (rebind() below lists every DevBuf member)
    CUtensorMap tmap{};     // 3D: tensor map of coef_pad
    bool has_tmap = false;
    int slot = 0;
    bool images_set = false;
    bool tables_valid = false;
    bool timing = false;
    // 1: events around every kernel (launched one after another); 2: events
    // around the whole evaluation only (kernels overlap as in untimed runs)
    int timing_mode = 0, ev_mode = 0;
    // programmatic dependent launch of the split path's kernels (MGR_PDL=0
    // in the environment at level creation turns it off)
    bool pdl = true;
    // the device reads and writes the caller's host memory in place
    // (coherent_host_access): evaluate moves parameters, gradient and costs
    // with the kernels' own loads and stores instead of staged copies
    bool coherent = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool ev_recorded = false;
    // move the level to stream s: its later work and the stream-ordered
    // frees of all its buffers go to s (the caller has ordered s after the
    // work queued on the old stream)
    void rebind(cudaStream_t s)
    {
        if (own_stream) throw std::invalid_argument("a level with its own stream cannot be moved");
        stream = s;
        auto re = [s](auto &b) {
            if (b.p) b.st = s;
        };
        re(axis_tables);
        re(axis_tables_f);
        re(coef), re(coef_pad), re(ref), re(warped), re(minmax), re(partial), re(ptable), re(pen_val), re(params_f);
        re(mmpart);
        re(params), re(grad_total), re(grad_image), re(grad_penalty), re(scalars), re(costs), re(tile_sums);
        re(pen_part), re(means), re(mpart);
        re(counters);
        re(pen_rowptr), re(pen_col);
        re(grid), re(force), re(tmp1), re(tmp2);
    }
    void record(int k)
    {
        if (timing && (timing_mode == 1 || k == 0 || k == 3)) ck(cudaEventRecord(ev[k], stream), "cudaEventRecord");
    }
    // 4 doubles of pinned host memory for small read-backs (costs, status)
    double *host_small_p = nullptr;
    double *host_small()
    {
        if (!host_small_p) ck(host_malloc_pinned(reinterpret_cast<void **>(&host_small_p), 4 * sizeof(double)),
                              "cudaMallocHost");
        return host_small_p;
    }
    ~mgr_level()
    {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (host_small_p) cudaFreeHost(host_small_p);
    }

    // a level made on another level's images (the refine pass of a batched
    // registration level): the image buffers are that level's, which
    // outlives this one; only one of the two is evaluated at a time
    const mgr_level *images_from = nullptr;

    // the kernels' arguments; `fused`: with the fused kernel's tile tables
    EvalArgs args(bool fused = false) const
    {
        const mgr_level &I = images_from ? *images_from : *this;
        EvalArgs a{};
        a.tmap = I.tmap;
        a.has_tmap = I.has_tmap;
        a.dim = d.dim;
        for (int k = 0; k < 3; ++k) {
            a.n[k] = n[k];
            a.nc[k] = nc[k];
            a.ax[k] = fused ? axf[k].view() : ax[k].view();
        }
        a.coef_img = I.coef.p;
        a.coef_pad = I.coef_pad.p;
        a.pad_rows = n[1] + 2 * PAD_H;
        a.ref = I.ref.p;
        a.warped = I.warped.p;
        a.minmax = I.minmax.p;
        a.params = params.p;
        a.params_f = params_f.p;
        a.cost = d.cost;
        a.ssd_norm = d.ssd_norm;
        a.cost_weight = d.cost_weight;
        a.centers = I.means.p;
        a.partial = partial.p;
        a.slot = fused ? slot_f : slot;
        a.tile_sums = tile_sums.p;
        a.counters = counters.p;
        a.pdl = pdl && timing_mode != 1;
        a.scalars = scalars.p;
        a.has_penalty = d.has_penalty;
        double prod = double(d.size[0]) * d.size[1] * (d.dim == 3 ? d.size[2] : 1);
        a.pen_weight = d.pen_norm ? d.pen_weight / double(float(prod)) : d.pen_weight;
        a.pen_grad_sign = d.pen_corrected ? 1.0 : -1.0;
        a.pen_equal_w = d.pen_div == d.pen_curl;
        a.ptable = ptable.p;
        a.pen_rowptr = pen_rowptr.p;
        a.pen_col = pen_col.p;
        a.pen_val = reinterpret_cast<const float4 *>(pen_val.p);
        a.pen_part = pen_part.p;
        a.grad_total = grad_total.p;
        a.grad_image = nullptr;
        a.grad_penalty = nullptr;
        a.costs = costs.p;
        return a;
    }

    // whether tile t is compiled in and, in 3D, its blocks' shared memory
    // fits: `strict`, the warp block three to an SM and the adjoint block in
    // 64 KiB (the rule without measurements); else what a launch allows
    // (the autotuner measured the shape, occupancy included)
    bool tile_fits(const int t[3], bool strict = true) const
    {
        if (!tile_supported(d.dim, t[0], t[1], t[2])) return false;
        if (d.dim == 2) return true;
        AxisHost hx, hy, hz;
        build_axis(hx, n[0], nc[0], t[0]);
        build_axis(hy, n[1], nc[1], t[1]);
        build_axis(hz, n[2], nc[2], t[2]);
        const size_t w =
            (size_t(3) * hz.fc * hy.fc * (hx.fc + 32) + 32 + size_t(WARP_RING_PLANES) * 16 * 64) * sizeof(float);
        const size_t adj = size_t(3) * hz.ac * 8 * (33 + hx.ac) * sizeof(float);   // split3_smem(a, 1)
        if (strict) return w <= 74 * 1024 && adj <= 64 * 1024;
        return w + 128 <= 200 * 1024 && adj <= 200 * 1024;
    }

    // the tile of the autotuner's nearest case (tune.cc) when a launch
    // allows it, else 32x16 in 2D and in 3D the deepest z tile (16, 8, 4)
    // that fits three warp blocks to an SM
    void choose_tile()
    {
        int t[3];
        if (tuned_tile(d.dim, n, nc, t) && tile_fits(t, false)) {
            for (int k = 0; k < 3; ++k) tile[k] = t[k];
            return;
        }
        if (d.dim == 2) {
            tile[0] = 32;
            tile[1] = 16;
            tile[2] = 1;
            return;
        }
        static const int tzs[3] = {16, 8, 4};
        for (int k = 0; k < 3; ++k) {
            const int c[3] = {32, 8, tzs[k]};
            for (int j = 0; j < 3; ++j) tile[j] = c[j];
            if (tile_fits(c)) return;
        }
    }

    // the per-axis tables of tiles t into A (packed, uploaded to tables);
    // returns the number of tiles and sets the partial slot size
    int build_axis_set(const int t[3], AxisDev (&A)[3], DevBuf<unsigned char> &tables, int &slot_size)
    {
        const int D = d.dim;
        AxisDev *ax = A;
        std::vector<unsigned char> blob;
        for (int k = 0; k < D; ++k) build_axis(ax[k].h, n[k], nc[k], t[k]);
        if (D == 3) {
            // per axis and coefficient: the partial-slot offset parts of the
            // tiles that hold it, slot entry (tx, ty, tz) of coefficient
            // (cx, cy, cz) being at glist_x + glist_y + glist_z
            const int sl = D * ax[0].h.ac * ax[1].h.ac * ax[2].h.ac;
            const long long total = (long long)ax[0].h.nt * ax[1].h.nt * ax[2].h.nt * sl;
            const long long ts[3] = {sl, (long long)ax[0].h.nt * sl, (long long)ax[0].h.nt * ax[1].h.nt * sl};
            const long long ls[3] = {D, (long long)ax[0].h.ac * D, (long long)ax[0].h.ac * ax[1].h.ac * D};
            for (int k = 0; k < 3; ++k) {
                AxisHost &h = ax[k].h;
                h.glist.assign(size_t(h.nc) * GATHER_LMAX, 0);
                h.glen.assign(h.nc, -1);
                for (int c = 0; c < h.nc; ++c) {
                    const int lo = h.gtile[size_t(c) * 2], hi = h.gtile[size_t(c) * 2 + 1];
                    const int cnt = std::max(hi - lo + 1, 0);
                    if (cnt > GATHER_LMAX || total >= (1LL << 31)) continue;
                    for (int j = 0; j < cnt; ++j)
                        h.glist[size_t(c) * GATHER_LMAX + j] =
                            int((lo + j) * ts[k] + (c - h.atile0[lo + j]) * ls[k]);
                    h.glen[c] = cnt;
                }
            }
        }
        for (int k = 0; k < D; ++k) ax[k].pack_all(blob);
        // a fresh buffer: kernels queued earlier may still read the old one
        tables.release();
        tables.upload(blob, stream);
        for (int k = 0; k < D; ++k) ax[k].base = tables.p;
        slot_size = D * ax[0].h.ac * ax[1].h.ac * (D == 3 ? ax[2].h.ac : 1);
        return ax[0].h.nt * ax[1].h.nt * (D == 3 ? ax[2].h.nt : 1);
    }

    // the fused kernel's tile: 30 interior voxels in x (32 lanes with the
    // halo), 8 rows, the level's z tile
    void fused_tile(int t[3]) const
    {
        t[0] = 30;
        t[1] = 8;
        t[2] = tile[2];
    }

    void build_tables()
    {
        const int ntiles = build_axis_set(tile, ax, axis_tables, slot);
        size_t part = size_t(ntiles) * slot, sums = size_t(ntiles);
        if (path == MGR_PATH_FUSED) {
            int t[3];
            fused_tile(t);
            const int ntf = build_axis_set(t, axf, axis_tables_f, slot_f);
            part = std::max(part, size_t(ntf) * slot_f);
            sums = std::max(sums, size_t(ntf));
        }
        partial.alloc(part, stream);
        const size_t plain_blocks = (N + 255) / 256;
        tile_sums.alloc(std::max<size_t>(sums, plain_blocks) * 5, stream);
        pen_part.alloc(size_t(gather_blocks(args())) + 1, stream);
        tables_valid = true;
    }
};

namespace mgr {
// The tile of the registration drivers' split path, per pair (register.cu)
// and batched (batch.cu), so that both run the same kernels in the same
// order: 32x8x16 in 3D, 32x16 in 2D.  The autotuner's table times single
// evaluations, where the tile sets the latency of one launch; in the batch
// every launch carries all pairs and the deeper tile's lower per-item
// overhead wins (60-frame 2D series: 1733-1778 pairs/s with 32x16 against
// 1389-1415 with the tuned 32x8; the 3D cohort the same either way).
inline void registration_tile(int dim, int t[3])
{
    t[0] = 32;
    t[1] = dim == 3 ? 8 : 16;
    t[2] = dim == 3 ? 16 : 1;
}
// mgr_level_set_images_device without the final stream synchronisation
void level_set_images_async(mgr_level *L, const float *d_src, const float *d_ref);
// a new coefficient grid (and tile) on a level, images kept
void level_set_grid(mgr_level *L, const int csize[3], const int tile[3]);
// a level with the coefficient grid csize on the images of level S (same
// sizes, cost, penalty, path and tile; S must outlive it), made on stream st
mgr_level *level_create_on_images(const mgr_level *S, const int csize[3], cudaStream_t st);
}  // namespace mgr

namespace mgr {
// True when the device reads and writes pageable host memory coherently,
// translating through the host's page tables (Grace-based systems such as
// GB300, where the CPU-GPU link is cache coherent), unless the environment
// variable MGR_HOST_COPY is set to a value other than 0 (staged copies).
inline bool coherent_host_access(int device)
{
    int pageable = 0, host_tables = 0;
    const char *force_copy = std::getenv("MGR_HOST_COPY");
    bool ok = cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) == cudaSuccess &&
              cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) ==
                  cudaSuccess;
    cudaGetLastError();
    return ok && pageable == 1 && host_tables == 1 && !(force_copy && *force_copy && *force_copy != '0');
}

// Queue a read of the level's device status flag (counters[6], raised by a
// kernel whose bounded wait gave up) into *flag; after the stream has been
// synchronised, throw_if_flagged clears it and throws TimeoutError.
inline void read_status_flag(mgr_level *L, unsigned *flag)
{
    ck(cudaMemcpyAsync(flag, L->counters.p + 6, sizeof(unsigned), cudaMemcpyDeviceToHost, L->stream), "status D2H");
}
inline void throw_if_flagged(mgr_level *L, unsigned flag)
{
    if (flag) {
        ck(cudaMemsetAsync(L->counters.p + 6, 0, sizeof(unsigned), L->stream), "status reset");
        throw TimeoutError("a bounded device wait gave up (bulk copy did not complete)");
    }
}
}  // namespace mgr
