// level.hh — the per-level state behind an mgr_level handle (device
// buffers, tables, stream); shared by the C ABI and the batched driver.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mgr.h"
#include "mgr_kernels.hh"
#include "tables.hh"

namespace mgr {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct StateError : std::runtime_error {
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
        ck(cudaMallocAsync(reinterpret_cast<void **>(&p), count * sizeof(T), s), "cudaMallocAsync");
        st = s;
        n = count;
    }
    void upload(const std::vector<T> &h, cudaStream_t s)
    {
        alloc(h.size(), s);
        if (!h.empty()) ck(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
    }
};

struct AxisDev {
    AxisHost h;
    DevBuf<int> fs, as, rows, ftile0, atile0, gtile;
    DevBuf<float> fw, aw;
    void upload(cudaStream_t st)
    {
        fs.upload(h.fs, st);
        as.upload(h.as, st);
        rows.upload(h.rows, st);
        ftile0.upload(h.ftile0, st);
        atile0.upload(h.atile0, st);
        gtile.upload(h.gtile, st);
        fw.upload(h.fw, st);
        aw.upload(h.aw, st);
    }
    Axis view() const
    {
        Axis a;
        a.fs = fs.p;
        a.fw = reinterpret_cast<const float4 *>(fw.p);
        a.as = as.p;
        a.aw = reinterpret_cast<const float4 *>(aw.p);
        a.rows = reinterpret_cast<const int2 *>(rows.p);
        a.ftile0 = ftile0.p;
        a.atile0 = atile0.p;
        a.gtile = reinterpret_cast<const int2 *>(gtile.p);
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
    int tile[3] = {32, 8, 8};
    AxisDev ax[3];
    DevBuf<float> coef, ref, warped, minmax, partial, ptable, pen_val;
    DevBuf<float2> mmpart;
    DevBuf<double> params, grad_total, grad_image, grad_penalty, scalars, costs, tile_sums, pen_part, means, mpart;
    DevBuf<unsigned int> counters;
    DevBuf<int> pen_rowptr, pen_col;
    DevBuf<float> grid, force, tmp1, tmp2;   // plain path and standalone force/translate
    int slot = 0;
    bool images_set = false;
    bool tables_valid = false;
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool ev_recorded = false;
    void record(int k)
    {
        if (timing) ck(cudaEventRecord(ev[k], stream), "cudaEventRecord");
    }
    ~mgr_level()
    {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }

    EvalArgs args() const
    {
        EvalArgs a{};
        a.dim = d.dim;
        for (int k = 0; k < 3; ++k) {
            a.n[k] = n[k];
            a.nc[k] = nc[k];
            a.ax[k] = ax[k].view();
        }
        a.coef_img = coef.p;
        a.ref = ref.p;
        a.warped = warped.p;
        a.minmax = minmax.p;
        a.params = params.p;
        a.cost = d.cost;
        a.ssd_norm = d.ssd_norm;
        a.cost_weight = d.cost_weight;
        a.centers = means.p;
        a.partial = partial.p;
        a.slot = slot;
        a.tile_sums = tile_sums.p;
        a.counters = counters.p;
        a.scalars = scalars.p;
        a.has_penalty = d.has_penalty;
        double prod = double(d.size[0]) * d.size[1] * (d.dim == 3 ? d.size[2] : 1);
        a.pen_weight = d.pen_norm ? d.pen_weight / double(float(prod)) : d.pen_weight;
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

    void build_tables()
    {
        const int D = d.dim;
        for (int k = 0; k < D; ++k) {
            build_axis(ax[k].h, n[k], nc[k], tile[k]);
            ax[k].upload(stream);
        }
        const int ntiles = ax[0].h.nt * ax[1].h.nt * (D == 3 ? ax[2].h.nt : 1);
        slot = D * ax[0].h.ac * ax[1].h.ac * (D == 3 ? ax[2].h.ac : 1);
        partial.alloc(size_t(ntiles) * slot, stream);
        const size_t plain_blocks = (N + 255) / 256;
        tile_sums.alloc(std::max<size_t>(ntiles, plain_blocks) * 5, stream);
        pen_part.alloc(size_t(gather_blocks(args())) + 1, stream);
        tables_valid = true;
    }
};

namespace mgr {
// mgr_level_set_images_device without the final stream synchronisation
void level_set_images_async(mgr_level *L, const float *d_src, const float *d_ref);
}  // namespace mgr
