// api.cu — the C ABI of libmgr (include/mgr.h): per-level state, device
// memory, table upload and the evaluation pipelines.
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mgr.h"
#include "level.hh"
#include "trace.hh"

namespace mgr {

static std::atomic<unsigned long long> g_launches{0};
static thread_local bool g_capturing = false;
void count_launch(unsigned n)
{
    if (!g_capturing) g_launches.fetch_add(n, std::memory_order_relaxed);
}
void count_launch_pause(bool paused) { g_capturing = paused; }

static thread_local std::string g_err;
void set_last_error(const std::string &msg) { g_err = msg; }

// allocation accounting and failure injection (mgr_debug_fail_allocation)
static std::atomic<unsigned long long> g_allocs{0};
static std::atomic<long long> g_fail_in{0};   // 0: off; k: the k-th allocation from now fails

static bool injected_allocation_failure()
{
    g_allocs.fetch_add(1, std::memory_order_relaxed);
    long long k = g_fail_in.load();
    while (k > 0)
        if (g_fail_in.compare_exchange_weak(k, k - 1)) return k == 1;
    return false;
}

cudaError_t dev_malloc_async(void **p, size_t bytes, cudaStream_t s)
{
    if (injected_allocation_failure()) return cudaErrorMemoryAllocation;
    return cudaMallocAsync(p, bytes, s);
}

cudaError_t dev_malloc(void **p, size_t bytes)
{
    if (injected_allocation_failure()) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}

cudaError_t host_malloc_pinned(void **p, size_t bytes)
{
    if (injected_allocation_failure()) return cudaErrorMemoryAllocation;
    return cudaMallocHost(p, bytes);
}

void raise_smem_limit(const void *kernel, size_t bytes)
{
    struct Limit {
        const void *kernel;
        int device;
        size_t bytes;
    };
    static std::mutex mu;
    static std::vector<Limit> set;
    int device = 0;
    cudaGetDevice(&device);
    std::lock_guard<std::mutex> lk(mu);
    for (auto &l : set)
        if (l.kernel == kernel && l.device == device) {
            if (l.bytes >= bytes) return;
            cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
            l.bytes = bytes;
            return;
        }
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
    set.push_back({kernel, device, bytes});
}

// phase trace (MGR_TRACE=1)
namespace {
struct PhaseSum {
    std::string name;
    double ms;
    long n;
};
std::mutex g_trace_mu;
std::vector<PhaseSum> g_trace;
}  // namespace

bool trace_enabled()
{
    static const bool on = [] {
        const char *e = std::getenv("MGR_TRACE");
        return e && *e && std::strcmp(e, "0") != 0;
    }();
    return on;
}

void trace_add(const char *phase, double ms)
{
    std::lock_guard<std::mutex> lk(g_trace_mu);
    for (auto &p : g_trace)
        if (p.name == phase) {
            p.ms += ms;
            p.n += 1;
            return;
        }
    g_trace.push_back({phase, ms, 1});
}

void trace_count(const char *name, double value)
{
    if (trace_enabled()) trace_add(name, value);
}

void trace_report(const char *title)
{
    if (!trace_enabled()) return;
    std::lock_guard<std::mutex> lk(g_trace_mu);
    std::fprintf(stderr, "[mgr trace] %s\n", title);
    for (auto &p : g_trace) std::fprintf(stderr, "  %-28s %10.3f ms  %6ld calls\n", p.name.c_str(), p.ms, p.n);
    g_trace.clear();
}

void configure_pool(int device)
{
    static std::mutex mu;
    static std::vector<int> done;
    std::lock_guard<std::mutex> lk(mu);
    for (int d : done)
        if (d == device) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        // freed blocks stay cached up to this size instead of returning to
        // the device at every synchronisation
        uint64_t keep = 8ull << 30;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
    done.push_back(device);
}

static mgr_status fail(mgr_status s, const std::string &m)
{
    g_err = m;
    return s;
}

template <class F>
static mgr_status guarded(F f)
{
    try {
        f();
        return MGR_OK;
    } catch (const std::invalid_argument &e) {
        return fail(MGR_ERR_ARG, e.what());
    } catch (const std::bad_alloc &) {
        return fail(MGR_ERR_OOM, "device or host allocation failed");
    } catch (const StateError &e) {
        return fail(MGR_ERR_STATE, e.what());
    } catch (const TimeoutError &e) {
        return fail(MGR_ERR_TIMEOUT, e.what());
    } catch (const CudaError &e) {
        return fail(MGR_ERR_CUDA, e.what());
    } catch (const std::exception &e) {
        return fail(MGR_ERR_CUDA, e.what());
    }
}

static void check_launch(const char *what)
{
    ck(cudaGetLastError(), what);
}

}  // namespace mgr

using namespace mgr;

// the divcurl penalty table of the level's grid (3D: translation-invariant
// cells; 2D: boundary-clipped CSR rows, cached across levels of equal grid)
static void build_penalty(mgr_level *L)
{
    const mgr_level_desc &d = L->d;
    if (!d.has_penalty) return;
    const float range[3] = {float(d.size[0]), float(d.size[1]), float(d.dim == 3 ? d.size[2] : 1)};
    if (d.dim == 3) {
        std::vector<float> P = build_penalty3(L->nc, range, d.pen_div, d.pen_curl);
        L->ptable.release();   // kernels queued earlier may still read the old table
        L->ptable.upload(P, L->stream);
    } else {
        const auto t = penalty2_cached(L->nc, range, d.pen_div, d.pen_curl);
        L->pen_rowptr.release();
        L->pen_col.release();
        L->pen_val.release();
        L->pen_rowptr.upload(t->rowptr, L->stream);
        L->pen_col.upload(t->col, L->stream);
        L->pen_val.upload(t->val, L->stream);
    }
}

namespace mgr {
// A new coefficient grid on a level whose images stay (the second pass of a
// registration level after refine): parameter buffers, tables and penalty
// are rebuilt, the prefiltered images are kept.  All work is queued on the
// level's stream.
void level_set_grid(mgr_level *L, const int csize[3], const int tile[3])
{
    ck(cudaSetDevice(L->device), "cudaSetDevice");   // (callers may be helper threads)
    const int D = L->d.dim;
    for (int k = 0; k < D; ++k) {
        if (csize[k] <= 3) throw std::invalid_argument("coefficient grid must be larger than 3 per axis");
        L->nc[k] = csize[k];
        L->d.csize[k] = csize[k];
    }
    L->ncoef = size_t(L->nc[0]) * L->nc[1] * L->nc[2];
    L->nparams = L->ncoef * D;
    for (int k = 0; k < 3; ++k) L->tile[k] = tile[k];
    L->params.release();
    L->params_f.release();
    L->grad_total.release();
    L->grad_image.release();
    L->grad_penalty.release();
    L->params.alloc(L->nparams, L->stream);
    if (D == 3) L->params_f.alloc(L->nparams, L->stream);
    L->grad_total.alloc(L->nparams, L->stream);
    L->partial.release();
    L->tile_sums.release();
    L->pen_part.release();
    L->build_tables();
    build_penalty(L);
    check_launch("level set grid");
}
mgr_level *level_create_on_images(const mgr_level *S, const int csize[3], cudaStream_t st)
{
    ck(cudaSetDevice(S->device), "cudaSetDevice");
    std::unique_ptr<mgr_level> L(new mgr_level);
    L->d = S->d;
    const int D = S->d.dim;
    for (int k = 0; k < 3; ++k) {
        L->n[k] = S->n[k];
        L->nc[k] = k < D ? csize[k] : 1;
        if (k < D) {
            if (csize[k] <= 3) throw std::invalid_argument("coefficient grid must be larger than 3 per axis");
            L->d.csize[k] = csize[k];
        }
        L->tile[k] = S->tile[k];
    }
    L->N = S->N;
    L->ncoef = size_t(L->nc[0]) * L->nc[1] * L->nc[2];
    L->nparams = L->ncoef * D;
    L->path = S->path;
    L->device = S->device;
    L->coherent = S->coherent;
    L->pdl = S->pdl;
    L->stream = st;
    L->images_from = S;
    L->images_set = true;
    L->params.alloc(L->nparams, st);
    if (D == 3) L->params_f.alloc(L->nparams, st);
    L->grad_total.alloc(L->nparams, st);
    L->scalars.alloc(SC_NSLOTS, st);
    L->costs.alloc(2, st);
    L->counters.alloc(8, st);
    ck(cudaMemsetAsync(L->counters.p, 0, 8 * sizeof(unsigned), st), "memset");
    ck(cudaMemsetAsync(L->scalars.p, 0, SC_NSLOTS * sizeof(double), st), "memset");
    L->build_tables();
    build_penalty(L.get());
    check_launch("level create on images");
    return L.release();
}

}  // namespace mgr

extern "C" {

const char *mgr_last_error(void) { return g_err.c_str(); }

unsigned long long mgr_kernel_launch_count(void) { return g_launches.load(); }

mgr_status mgr_debug_fail_allocation(long long k)
{
    if (k < 0) return fail(MGR_ERR_ARG, "mgr_debug_fail_allocation: k must be >= 0");
    g_fail_in.store(k);
    return MGR_OK;
}

unsigned long long mgr_allocation_count(void) { return g_allocs.load(); }

mgr_status mgr_level_create(const mgr_level_desc *desc, int device, void *stream, mgr_level **out)
{
    if (!desc || !out) return fail(MGR_ERR_ARG, "null argument");
    *out = nullptr;
    std::unique_ptr<mgr_level> L(new mgr_level);
    mgr_status st = guarded([&] {
        const mgr_level_desc &d = *desc;
        if (d.dim != 2 && d.dim != 3) throw std::invalid_argument("dim must be 2 or 3");
        if (d.cost != MGR_COST_SSD && d.cost != MGR_COST_NCC) throw std::invalid_argument("unknown cost");
        if (!std::isfinite(d.cost_weight)) throw std::invalid_argument("cost weight must be finite");
        if (d.has_penalty && !(std::isfinite(d.pen_weight) && d.pen_weight > 0 && d.pen_div >= 0 && d.pen_curl >= 0))
            throw std::invalid_argument("penalty weight must be positive, div/curl non-negative");
        L->d = d;
        for (int k = 0; k < 3; ++k) {
            L->n[k] = (k < d.dim) ? d.size[k] : 1;
            if (k < d.dim) {
                if (d.size[k] < 2) throw std::invalid_argument("image dimensions must be >= 2");
                if (d.csize[k] > 0) {
                    if (d.csize[k] <= 3) throw std::invalid_argument("coefficient grid must be larger than 3 per axis");
                    L->nc[k] = d.csize[k];
                } else {
                    if (!(d.rate[k] >= 1.0f)) throw std::invalid_argument("spline rate must be >= 1");
                    const int c = csize_from_rate(d.size[k], d.rate[k]);
                    if (c - 2 <= 1)
                        throw std::invalid_argument("coefficient rate is too large for the image dimensions");
                    L->nc[k] = c;
                }
            }
        }
        L->N = size_t(L->n[0]) * L->n[1] * L->n[2];
        L->ncoef = size_t(L->nc[0]) * L->nc[1] * L->nc[2];
        L->nparams = L->ncoef * d.dim;
        L->choose_tile();
        L->device = device;
        ck(cudaSetDevice(device), "cudaSetDevice");
        configure_pool(device);
        L->coherent = coherent_host_access(device);
        {
            const char *e = std::getenv("MGR_PDL");
            L->pdl = !(e && std::strcmp(e, "0") == 0);
        }
        if (stream) {
            L->stream = static_cast<cudaStream_t>(stream);
        } else {
            ck(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking), "cudaStreamCreate");
            L->own_stream = true;
        }
        L->coef.alloc(L->N, L->stream);
        L->coef_pad.alloc(pad_floats(d.dim, L->n[0], L->n[1], L->n[2]), L->stream);
        if (d.dim == 3) L->has_tmap = encode_pad_tmap(&L->tmap, L->coef_pad.p, L->n[0], L->n[1], L->n[2]);
        L->ref.alloc(L->N, L->stream);
        L->warped.alloc(L->N, L->stream);
        L->minmax.alloc(2, L->stream);
        L->mmpart.alloc(1024, L->stream);
        L->params.alloc(L->nparams, L->stream);
        if (d.dim == 3) L->params_f.alloc(L->nparams, L->stream);
        L->grad_total.alloc(L->nparams, L->stream);
        L->scalars.alloc(SC_NSLOTS, L->stream);
        L->costs.alloc(2, L->stream);
        L->means.alloc(2, L->stream);
        L->mpart.alloc(2 * 1024, L->stream);
        L->counters.alloc(8, L->stream);
        ck(cudaMemsetAsync(L->counters.p, 0, 8 * sizeof(unsigned), L->stream), "memset");
        ck(cudaMemsetAsync(L->scalars.p, 0, SC_NSLOTS * sizeof(double), L->stream), "memset");
        L->build_tables();
        build_penalty(L.get());
        check_launch("level create");
    });
    if (st == MGR_OK) *out = L.release();
    else mgr_level_destroy(L.release());   // buffers made so far, and a stream the level created
    return st;
}

mgr_status mgr_level_destroy(mgr_level *lvl)
{
    if (!lvl) return MGR_OK;
    cudaSetDevice(lvl->device);
    // the buffers are freed in stream order, so a caller's stream needs no
    // synchronisation; a stream the level created is drained before it goes
    if (lvl->stream && lvl->own_stream) cudaStreamSynchronize(lvl->stream);
    const bool own = lvl->own_stream;
    cudaStream_t s = lvl->stream;
    delete lvl;
    if (own) cudaStreamDestroy(s);
    return MGR_OK;
}

mgr_status mgr_level_csize(const mgr_level *lvl, int csize[3], size_t *nparams)
{
    if (!lvl) return fail(MGR_ERR_ARG, "null level");
    if (csize)
        for (int k = 0; k < 3; ++k) csize[k] = lvl->nc[k];
    if (nparams) *nparams = lvl->nparams;
    return MGR_OK;
}

}  // extern "C"

// means of the two images in double (NCC provisional centres): per-block
// partial sums (blockIdx.y selects the image), then a fixed-order final sum
__global__ void __launch_bounds__(256) k_mean_part(const float *__restrict__ a, const float *__restrict__ b, size_t n,
                                                   double *part)
{
    __shared__ double red[8];
    const float *img = blockIdx.y ? b : a;
    double v[1] = {0.0};
    for (size_t i = blockIdx.x * size_t(256) + threadIdx.x; i < n; i += size_t(gridDim.x) * 256) v[0] += img[i];
    block_sum<1>(v, red);
    if (threadIdx.x == 0) part[blockIdx.y * gridDim.x + blockIdx.x] = v[0];
}

__global__ void __launch_bounds__(256) k_mean_final(const double *part, int nb, size_t n, double *out)
{
    __shared__ double red[8];
    double v[1] = {0.0};
    for (int i = threadIdx.x; i < nb; i += 256) v[0] += part[blockIdx.x * nb + i];
    block_sum<1>(v, red);
    if (threadIdx.x == 0) out[blockIdx.x] = v[0] / double(n);
}

namespace mgr {

// copy the images into the level, clamp bounds, centres and the prefilter,
// all queued on the level's stream (the sources must stay valid until the
// stream reaches them)
void level_set_images_async(mgr_level *L, const float *d_src, const float *d_ref)
{
    ck(cudaSetDevice(L->device), "cudaSetDevice");
    cudaStream_t st = L->stream;
    ck(cudaMemcpyAsync(L->coef.p, d_src, L->N * sizeof(float), cudaMemcpyDeviceToDevice, st), "copy src");
    if (d_ref != L->ref.p)
        ck(cudaMemcpyAsync(L->ref.p, d_ref, L->N * sizeof(float), cudaMemcpyDeviceToDevice, st), "copy ref");
    const int nb = int(std::min<size_t>(1024, (L->N + 255) / 256));
    launch_minmax(L->coef.p, L->N, L->mmpart.p, nb, L->counters.p + 4, L->minmax.p, st);
    k_mean_part<<<dim3(nb, 2), 256, 0, st>>>(L->coef.p, L->ref.p, L->N, L->mpart.p);
    k_mean_final<<<2, 256, 0, st>>>(L->mpart.p, nb, L->N, L->means.p);
    count_launch(2);
    launch_prefilter(L->coef.p, L->d.dim, L->n[0], L->n[1], L->n[2], st);
    launch_pad_mirror(L->coef.p, L->coef_pad.p, L->d.dim, L->n[0], L->n[1], L->n[2], st);
    check_launch("set_images kernels");
    L->images_set = true;
}

}  // namespace mgr

static void set_images_impl(mgr_level *L, const float *d_src, const float *d_ref)
{
    level_set_images_async(L, d_src, d_ref);
    // the caller may reuse its buffers once this returns
    ck(cudaStreamSynchronize(L->stream), "set_images sync");
}

static void upload_params(mgr_level *L, const double *params)
{
    // the copy starts first and the finiteness check runs while it is in
    // flight; no kernel is queued before the check has passed, and on
    // failure the copy is waited for (it reads the caller's buffer)
    ck(cudaMemcpyAsync(L->params.p, params, L->nparams * sizeof(double), cudaMemcpyHostToDevice, L->stream),
       "params H2D");
    // x - x is 0 for finite x and NaN otherwise: eight independent sums
    // (no branch per value, the loop vectorises) are 0 exactly when every
    // parameter is finite
    const size_t n = L->nparams;
    double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    size_t i = 0;
    for (; i + 8 <= n; i += 8)
        for (int k = 0; k < 8; ++k) acc[k] += params[i + k] - params[i + k];
    for (; i < n; ++i) acc[0] += params[i] - params[i];
    double all = 0.0;
    for (double v : acc) all += v;
    if (all != 0.0) {
        cudaStreamSynchronize(L->stream);
        throw std::invalid_argument("parameters must be finite");
    }
}

static void run_image_term(mgr_level *L, EvalArgs &a, bool with_gradient);

// Evaluation on a device that reads and writes the caller's host memory
// coherently (3D split path): the parameter conversion reads the caller's
// parameters, the gather writes the gradients into the caller's buffers and
// the costs and status flags into the level's pinned buffer; no staged copy
// and one synchronisation.  Non-finite parameters are found by the
// conversion: the kernels then run on zeros in their place, nothing is
// written to the caller's buffers and the call fails as the staged path does.
static void evaluate_in_place(mgr_level *L, const double *params, double *grad_total, double *grad_image,
                              double *grad_penalty, double *cost_image, double *cost_penalty)
{
    EvalArgs a = L->args();
    a.params_host = params;
    if (grad_total) a.grad_total = grad_total;
    a.grad_image = grad_image;
    a.grad_penalty = grad_penalty;
    double *hc = L->host_small();
    a.host_out = hc;
    run_image_term(L, a, true);
    check_launch("evaluate kernels");
    ck(cudaStreamSynchronize(L->stream), "evaluate sync");
    unsigned flags[2];
    std::memcpy(flags, hc + 2, sizeof flags);
    if (flags[1]) {
        if (flags[0]) ck(cudaMemsetAsync(L->counters.p + 6, 0, sizeof(unsigned), L->stream), "status reset");
        throw std::invalid_argument("parameters must be finite");
    }
    throw_if_flagged(L, flags[0]);
    if (cost_image) *cost_image = hc[0];
    if (cost_penalty) *cost_penalty = hc[1];
}

static void run_image_term(mgr_level *L, EvalArgs &a, bool with_gradient)
{
    cudaStream_t st = L->stream;
    if (!with_gradient) {
        launch_warp(a, st);
        return;
    }
    L->ev_recorded = L->timing;
    L->ev_mode = L->timing_mode;
    if (L->path == MGR_PATH_FUSED) {
        // the fused kernel and the gather on the fused tiles' tables; the
        // call's buffers as the caller set them in a
        EvalArgs af = L->args(true);
        af.params = a.params;
        af.grad_total = a.grad_total;
        af.grad_image = a.grad_image;
        af.grad_penalty = a.grad_penalty;
        af.costs = a.costs;
        L->record(0);
        {
            NvtxRange r("k_fused3");
            launch_fused3(af, 1, st);
        }
        L->record(1);
        L->record(2);
        {
            NvtxRange r("k_gather3");
            launch_gather(af, 1, st);
        }
        L->record(3);
        return;
    }
    if (L->path == MGR_PATH_PLAIN) {
        L->record(0);
        const size_t tsz = size_t(std::max(L->nc[2], 1)) * std::max(L->n[1], L->nc[1]) * L->n[0] * 3;
        if (L->d.dim == 3) L->grid.alloc(L->N * 3, L->stream);
        L->force.alloc(L->N * L->d.dim, L->stream);
        L->tmp1.alloc(tsz, L->stream);
        L->tmp2.alloc(tsz, L->stream);
        L->grad_image.alloc(L->nparams, L->stream);
        a.grad_image = L->grad_image.p;
        launch_plain_eval(a, L->grid.p, L->force.p, L->tmp1.p, L->tmp2.p, st);
        L->record(1);
        L->record(2);
        L->record(3);
        return;
    }
    L->record(0);
    // 3D: the cost is finalised after the warp kernel (its blocks end earlier)
    a.defer_cost = L->d.dim == 3;
    {
        NvtxRange r(L->d.dim == 3 ? "k_warp3" : "k_warp (2D)");
        launch_warp(a, st);
    }
    L->record(1);
    {
        NvtxRange r(L->d.dim == 3 ? "k_adjoint3" : "k_adjoint (2D)");
        launch_adjoint(a, st);
    }
    L->record(2);
    {
        NvtxRange r(L->d.dim == 3 ? "k_gather3" : "k_gather (2D)");
        launch_gather(a, 1, st);
    }
    L->record(3);
}

extern "C" {

mgr_status mgr_level_set_images(mgr_level *lvl, const float *src, const float *ref)
{
    NvtxRange nvtx_range("mgr_level_set_images");
    if (!lvl || !src || !ref) return fail(MGR_ERR_ARG, "null argument");
    return guarded([&] {
        for (size_t i = 0; i < lvl->N; ++i)
            if (!std::isfinite(src[i]) || !std::isfinite(ref[i]))
                throw std::invalid_argument("images must be finite");
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        lvl->warped.alloc(lvl->N, lvl->stream);
        ck(cudaMemcpyAsync(lvl->warped.p, src, lvl->N * sizeof(float), cudaMemcpyHostToDevice, lvl->stream), "src");
        ck(cudaMemcpyAsync(lvl->ref.p, ref, lvl->N * sizeof(float), cudaMemcpyHostToDevice, lvl->stream), "ref");
        set_images_impl(lvl, lvl->warped.p, lvl->ref.p);
    });
}

mgr_status mgr_level_set_images_device(mgr_level *lvl, const float *d_src, const float *d_ref)
{
    if (!lvl || !d_src || !d_ref) return fail(MGR_ERR_ARG, "null argument");
    return guarded([&] { set_images_impl(lvl, d_src, d_ref); });
}

mgr_status mgr_level_evaluate_device(mgr_level *lvl, const double *d_params, double *d_grad_total, double *d_costs)
{
    NvtxRange nvtx_range("mgr_level_evaluate_device");
    if (!lvl || !d_params || !d_grad_total) return fail(MGR_ERR_ARG, "null argument");
    return guarded([&] {
        if (!lvl->images_set) throw StateError("set_images must be called before evaluate");
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        EvalArgs a = lvl->args();
        a.params = d_params;
        a.grad_total = d_grad_total;
        a.costs = d_costs;
        run_image_term(lvl, a, true);
        check_launch("evaluate kernels");
    });
}

mgr_status mgr_level_evaluate(mgr_level *lvl, const double *params, double *grad_total, double *grad_image,
                              double *grad_penalty, double *cost_image, double *cost_penalty)
{
    NvtxRange nvtx_range("mgr_level_evaluate");
    if (!lvl || !params) return fail(MGR_ERR_ARG, "null argument");
    return guarded([&] {
        if (!lvl->images_set) throw StateError("set_images must be called before evaluate");
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        if (lvl->coherent && lvl->d.dim == 3 && lvl->path == MGR_PATH_SPLIT) {
            evaluate_in_place(lvl, params, grad_total, grad_image, grad_penalty, cost_image, cost_penalty);
            return;
        }
        upload_params(lvl, params);
        EvalArgs a = lvl->args();
        if (grad_image && lvl->path != MGR_PATH_PLAIN) {
            lvl->grad_image.alloc(lvl->nparams, lvl->stream);
            a.grad_image = lvl->grad_image.p;
        }
        if (grad_penalty) {
            lvl->grad_penalty.alloc(lvl->nparams, lvl->stream);
            a.grad_penalty = lvl->grad_penalty.p;
        }
        run_image_term(lvl, a, true);
        check_launch("evaluate kernels");
        cudaStream_t st = lvl->stream;
        const size_t bytes = lvl->nparams * sizeof(double);
        if (grad_total) ck(cudaMemcpyAsync(grad_total, lvl->grad_total.p, bytes, cudaMemcpyDeviceToHost, st), "D2H");
        if (grad_image) ck(cudaMemcpyAsync(grad_image, lvl->grad_image.p, bytes, cudaMemcpyDeviceToHost, st), "D2H");
        if (grad_penalty)
            ck(cudaMemcpyAsync(grad_penalty, lvl->grad_penalty.p, bytes, cudaMemcpyDeviceToHost, st), "D2H");
        // costs and status flag into the level's pinned buffer: asynchronous
        // copies, one synchronisation
        double *hc = lvl->host_small();
        ck(cudaMemcpyAsync(hc, lvl->costs.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
        ck(cudaMemcpyAsync(hc + 2, lvl->counters.p + 6, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "D2H");
        ck(cudaStreamSynchronize(st), "evaluate sync");
        unsigned flag;
        std::memcpy(&flag, hc + 2, sizeof flag);
        throw_if_flagged(lvl, flag);
        if (cost_image) *cost_image = hc[0];
        if (cost_penalty) *cost_penalty = hc[1];
    });
}

mgr_status mgr_level_host_access(const mgr_level *lvl, int *in_place)
{
    if (!lvl || !in_place) return fail(MGR_ERR_ARG, "null argument");
    *in_place = lvl->coherent && lvl->d.dim == 3 && lvl->path == MGR_PATH_SPLIT ? 1 : 0;
    return MGR_OK;
}

mgr_status mgr_level_value(mgr_level *lvl, const double *params, double *cost_image, double *cost_penalty)
{
    NvtxRange nvtx_range("mgr_level_value");
    if (!lvl || !params) return fail(MGR_ERR_ARG, "null argument");
    return guarded([&] {
        if (!lvl->images_set) throw StateError("set_images must be called before value");
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        upload_params(lvl, params);
        EvalArgs a = lvl->args();
        a.defer_cost = lvl->d.dim == 3;   // the cost is finalised after the warp kernel
        launch_warp(a, lvl->stream);
        launch_gather(a, 0, lvl->stream);
        check_launch("value kernels");
        double *hc = lvl->host_small();
        ck(cudaMemcpyAsync(hc, lvl->costs.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, lvl->stream), "D2H");
        ck(cudaMemcpyAsync(hc + 2, lvl->counters.p + 6, sizeof(unsigned), cudaMemcpyDeviceToHost, lvl->stream),
           "D2H");
        ck(cudaStreamSynchronize(lvl->stream), "value sync");
        unsigned flag;
        std::memcpy(&flag, hc + 2, sizeof flag);
        throw_if_flagged(lvl, flag);
        if (cost_image) *cost_image = hc[0];
        if (cost_penalty) *cost_penalty = hc[1];
    });
}

mgr_status mgr_level_warp(mgr_level *lvl, const double *params, float *out)
{
    if (!lvl || !params || !out) return fail(MGR_ERR_ARG, "null argument");
    return guarded([&] {
        if (!lvl->images_set) throw StateError("set_images must be called before warp");
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        upload_params(lvl, params);
        EvalArgs a = lvl->args();
        launch_warp(a, lvl->stream);
        check_launch("warp kernel");
        ck(cudaMemcpyAsync(out, lvl->warped.p, lvl->N * sizeof(float), cudaMemcpyDeviceToHost, lvl->stream), "D2H");
        unsigned flag = 0;
        read_status_flag(lvl, &flag);
        ck(cudaStreamSynchronize(lvl->stream), "warp sync");
        throw_if_flagged(lvl, flag);
    });
}

mgr_status mgr_level_force(mgr_level *lvl, const double *params, float *force, double *cost)
{
    if (!lvl || !params || !force) return fail(MGR_ERR_ARG, "null argument");
    return guarded([&] {
        if (!lvl->images_set) throw StateError("set_images must be called before force");
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        upload_params(lvl, params);
        EvalArgs a = lvl->args();
        launch_warp(a, lvl->stream);
        lvl->force.alloc(lvl->N * lvl->d.dim, lvl->stream);
        launch_force(a, lvl->force.p, lvl->stream);
        check_launch("force kernels");
        ck(cudaMemcpyAsync(force, lvl->force.p, lvl->N * lvl->d.dim * sizeof(float), cudaMemcpyDeviceToHost,
                           lvl->stream), "D2H");
        double sc[SC_NSLOTS];
        ck(cudaMemcpyAsync(sc, lvl->scalars.p, sizeof sc, cudaMemcpyDeviceToHost, lvl->stream), "D2H");
        unsigned flag = 0;
        read_status_flag(lvl, &flag);
        ck(cudaStreamSynchronize(lvl->stream), "force sync");
        throw_if_flagged(lvl, flag);
        if (cost) *cost = sc[SC_FORCE_COST];
    });
}

mgr_status mgr_level_translate(mgr_level *lvl, const float *force, double *grad)
{
    if (!lvl || !force || !grad) return fail(MGR_ERR_ARG, "null argument");
    return guarded([&] {
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        cudaStream_t st = lvl->stream;
        const int D = lvl->d.dim;
        lvl->force.alloc(lvl->N * D, lvl->stream);
        const size_t tsz = size_t(std::max(lvl->nc[2], 1)) * std::max(lvl->n[1], lvl->nc[1]) * lvl->n[0] * 3;
        lvl->tmp1.alloc(tsz, lvl->stream);
        lvl->tmp2.alloc(tsz, lvl->stream);
        lvl->grad_image.alloc(lvl->nparams, lvl->stream);
        ck(cudaMemcpyAsync(lvl->force.p, force, lvl->N * D * sizeof(float), cudaMemcpyHostToDevice, st), "H2D");
        EvalArgs a = lvl->args();
        a.cost_weight = 1.0;
        launch_translate(a, lvl->force.p, lvl->grad_image.p, lvl->tmp1.p, lvl->tmp2.p, st);
        check_launch("translate kernels");
        ck(cudaMemcpyAsync(grad, lvl->grad_image.p, lvl->nparams * sizeof(double), cudaMemcpyDeviceToHost, st),
           "D2H");
        ck(cudaStreamSynchronize(st), "translate sync");
    });
}

mgr_status mgr_level_set_grid(mgr_level *lvl, const int csize[3])
{
    if (!lvl || !csize) return fail(MGR_ERR_ARG, "null argument");
    return guarded([&] {
        if (lvl->images_from) throw StateError("mgr_level_set_grid: level shares another level's images");
        const int D = lvl->d.dim;
        int cs[3] = {1, 1, 1};
        bool same = true;
        for (int k = 0; k < D; ++k) {
            if (csize[k] <= 3) throw std::invalid_argument("coefficient grid must be larger than 3 per axis");
            cs[k] = csize[k];
            same = same && cs[k] == lvl->nc[k];
        }
        if (same) return;
        // the tile follows the new coefficient spacing as at creation
        for (int k = 0; k < D; ++k) lvl->nc[k] = cs[k];
        lvl->choose_tile();
        level_set_grid(lvl, cs, lvl->tile);
        ck(cudaStreamSynchronize(lvl->stream), "set_grid sync");
    });
}

mgr_status mgr_level_set_path(mgr_level *lvl, int path, int tile_x, int tile_y, int tile_z)
{
    if (!lvl) return fail(MGR_ERR_ARG, "null level");
    if (path != MGR_PATH_SPLIT && path != MGR_PATH_PLAIN && path != MGR_PATH_FUSED)
        return fail(MGR_ERR_ARG, "unknown path");
    return guarded([&] {
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        if (path == MGR_PATH_FUSED) {
            if (lvl->d.dim != 3 || lvl->d.cost != MGR_COST_SSD)
                throw std::invalid_argument("the fused path evaluates 3D SSD only");
            if (lvl->images_from) throw StateError("the fused path needs the level's own images");
            for (int k = 0; k < 3; ++k)
                if (lvl->nc[k] - 3 > lvl->n[k] - 1)
                    throw std::invalid_argument("the fused path needs a coefficient spacing of at least one voxel");
        }
        // the shape is checked before anything changes: a refused call
        // leaves the level as it was
        int t[3] = {tile_x > 0 ? tile_x : lvl->tile[0], tile_y > 0 ? tile_y : lvl->tile[1],
                    tile_z > 0 ? tile_z : lvl->tile[2]};
        if (lvl->d.dim == 2) t[2] = 1;
        if (!tile_supported(lvl->d.dim, t[0], t[1], t[2]))
            throw std::invalid_argument("tile shape not compiled in (3D: 32x8xTZ, TZ in 4, 8, 12, 16, 20, 24, 32; "
                                        "2D: 32x8, 32x16, 64x8, 64x16, 32x32)");
        if (!lvl->tile_fits(t, false))
            throw std::invalid_argument("the tile's shared memory does not fit at this coefficient spacing");
        const bool fused_change = (path == MGR_PATH_FUSED) != (lvl->path == MGR_PATH_FUSED);
        lvl->path = path;
        bool changed = fused_change;
        for (int k = 0; k < 3; ++k)
            if (t[k] != lvl->tile[k]) {
                lvl->tile[k] = t[k];
                changed = true;
            }
        if (changed) {
            ck(cudaStreamSynchronize(lvl->stream), "sync");
            lvl->build_tables();
            ck(cudaStreamSynchronize(lvl->stream), "sync");
        }
        if (path == MGR_PATH_FUSED && fused3_smem(lvl->args(true)) > size_t(227) * 1024) {
            lvl->path = MGR_PATH_SPLIT;
            throw std::invalid_argument("the fused kernel's shared memory does not fit at this coefficient spacing");
        }
    });
}

mgr_status mgr_level_tile(const mgr_level *lvl, int tile[3])
{
    if (!lvl || !tile) return fail(MGR_ERR_ARG, "null argument");
    for (int k = 0; k < 3; ++k) tile[k] = lvl->tile[k];
    return MGR_OK;
}

mgr_status mgr_level_set_timing(mgr_level *lvl, int enable)
{
    if (!lvl) return fail(MGR_ERR_ARG, "null level");
    return guarded([&] {
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        if (enable < 0 || enable > 2) throw std::invalid_argument("timing mode must be 0, 1 or 2");
        if (enable)
            for (auto &e : lvl->ev)
                if (!e) ck(cudaEventCreate(&e), "cudaEventCreate");
        lvl->timing = enable != 0;
        lvl->timing_mode = enable;
    });
}

mgr_status mgr_level_kernel_times(mgr_level *lvl, double ms[4])
{
    if (!lvl || !ms) return fail(MGR_ERR_ARG, "null argument");
    return guarded([&] {
        if (!lvl->ev_recorded) throw StateError("no timed evaluation recorded");
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        ck(cudaEventSynchronize(lvl->ev[3]), "cudaEventSynchronize");
        float t;
        for (int k = 0; k < 3; ++k) {
            ms[k] = 0.0;
            if (lvl->ev_mode != 1) continue;   // whole-evaluation events only
            ck(cudaEventElapsedTime(&t, lvl->ev[k], lvl->ev[k + 1]), "elapsed");
            ms[k] = t;
        }
        ck(cudaEventElapsedTime(&t, lvl->ev[0], lvl->ev[3]), "elapsed");
        ms[3] = t;
    });
}

mgr_status mgr_level_sync(mgr_level *lvl)
{
    if (!lvl) return fail(MGR_ERR_ARG, "null level");
    return guarded([&] {
        ck(cudaSetDevice(lvl->device), "cudaSetDevice");
        unsigned flag = 0;
        read_status_flag(lvl, &flag);
        ck(cudaStreamSynchronize(lvl->stream), "sync");
        throw_if_flagged(lvl, flag);
    });
}

}  // extern "C"
