// register.cu — mgr_register: the multiresolution registration of one pair
// (TNonrigidRegisterImpl::run, mia/template/nonrigidregister.cxx:193-296)
// with the minimizer on the host and every cost+gradient evaluated on the
// GPU through an mgr_level.
#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mgr.h"
#include "driver.hh"
#include "level.hh"
#include "pyramid.hh"
#include "tables.hh"
#include "trace.hh"

namespace mgr {

void set_last_error(const std::string &msg);

namespace {

void ckm(mgr_status s)
{
    if (s == MGR_ERR_ARG) throw std::invalid_argument(mgr_last_error());
    if (s == MGR_ERR_TIMEOUT) throw TimeoutError(mgr_last_error());
    if (s == MGR_ERR_OOM) throw std::bad_alloc();
    if (s != MGR_OK) throw std::runtime_error(mgr_last_error());
}

struct LevelHandle {
    mgr_level *h = nullptr;
    ~LevelHandle()
    {
        if (h) mgr_level_destroy(h);
    }
};

}  // namespace

// One pair through all levels.  Images are device pointers (full size);
// returns the final cost and fills params/csize.
double register_pair_device(const mgr_level_desc &full, int levels, const mgr_minimizer_desc &mz,
                            const float *d_src, const float *d_ref, int path, int device,
                            std::vector<double> &params, int csize[3], int *evaluations, cudaStream_t st)
{
    const int dim = full.dim;
    const int nz = dim == 3 ? full.size[2] : 1;
    const size_t n_full = size_t(full.size[0]) * full.size[1] * nz;
    DevBuf<float> src_n, ref_n, src_l, ref_l;
    src_n.alloc(n_full, st);
    ref_n.alloc(n_full, st);
    int evals = 0;
    double cost = 0.0;
    TraceScope tr_norm("pair: normalize", st);
    const bool varied = normalize_pair(d_src, d_ref, n_full, src_n.p, ref_n.p, st, nullptr, nullptr);
    tr_norm.stop();
    if (!varied) {
        // both images of a single value: the identity transformation at full size
        for (int k = 0; k < 3; ++k) csize[k] = k < dim ? csize_from_rate(full.size[k], full.rate[k]) : 1;
        params.assign(size_t(csize[0]) * csize[1] * (dim == 3 ? csize[2] : 1) * dim, 0.0);
        if (evaluations) *evaluations = 0;
        return 0.0;
    }
    int prev_size[3] = {0, 0, 0};
    for (int shift = levels - 1; shift >= 0; --shift) {
        const int factor = 1 << shift;
        int size[3] = {1, 1, 1};
        for (int k = 0; k < dim; ++k) size[k] = full.size[k] / factor;
        if (shift == levels - 1) {
            for (int k = 0; k < 3; ++k) csize[k] = k < dim ? csize_from_rate(size[k], full.rate[k]) : 1;
            params.assign(size_t(csize[0]) * csize[1] * (dim == 3 ? csize[2] : 1) * dim, 0.0);
            for (int k = 0; k < dim; ++k)
                if (csize[k] - 2 <= 1)
                    throw std::invalid_argument("coefficient rate is too large for the image dimensions of the "
                                                "coarsest level: reduce the rate or the number of levels");
        } else {
            upscale_params(dim, prev_size, size, params);
        }
        const size_t n = size_t(size[0]) * size[1] * (dim == 3 ? size[2] : 1);
        TraceScope tr_scale("pair: scale filter", st);
        src_l.alloc(n, st);
        ref_l.alloc(n, st);
        scale_image(src_n.p, full.size, src_l.p, size, dim, st);
        scale_image(ref_n.p, full.size, ref_l.p, size, dim, st);
        tr_scale.stop();
        for (int pass = 0; pass < 2; ++pass) {
            mgr_level_desc d = full;
            for (int k = 0; k < 3; ++k) {
                d.size[k] = size[k];
                d.csize[k] = csize[k];
            }
            TraceScope tr_lvl("pair: level setup", st);
            LevelHandle lv;
            ckm(mgr_level_create(&d, device, st, &lv.h));
            int t[3];
            registration_tile(dim, t);
            if (lv.h->tile_fits(t)) ckm(mgr_level_set_path(lv.h, path, t[0], t[1], t[2]));
            else ckm(mgr_level_set_path(lv.h, path, 0, 0, 0));
            level_set_images_async(lv.h, src_l.p, ref_l.p);
            tr_lvl.stop();
            TraceScope tr_min("pair: minimizer", st);
            FDF fdf = [&](const std::vector<double> &x, std::vector<double> &g) {
                double ci = 0, cp = 0;
                ckm(mgr_level_evaluate(lv.h, x.data(), g.data(), nullptr, nullptr, &ci, &cp));
                return ci + cp;
            };
            MinResult r = minimize(params, mz, fdf);
            tr_min.stop();
            evals += r.evaluations;
            cost = r.f;
            round_params_to_float(params);
            if (pass == 1) break;
            int nc_new[3] = {1, 1, 1};
            for (int k = 0; k < dim; ++k) nc_new[k] = refine_csize(size[k], full.rate[k]);
            if (!refine_params(dim, csize, nc_new, params)) break;
            for (int k = 0; k < 3; ++k) csize[k] = nc_new[k];
        }
        for (int k = 0; k < 3; ++k) prev_size[k] = size[k];
    }
    if (evaluations) *evaluations = evals;
    return cost;
}

}  // namespace mgr

using namespace mgr;

extern "C" mgr_status mgr_register(const mgr_level_desc *desc, int levels, const mgr_minimizer_desc *mz,
                                   const float *src, const float *ref, int path, int device,
                                   double *params_out, size_t max_params, int csize_out[3], double *final_cost,
                                   int *evaluations)
{
    if (!desc || !mz || !src || !ref || !params_out || !csize_out) {
        set_last_error("mgr_register: null argument");
        return MGR_ERR_ARG;
    }
    try {
        if (levels < 1) throw std::invalid_argument("levels must be >= 1");
        if (desc->dim != 2 && desc->dim != 3) throw std::invalid_argument("dim must be 2 or 3");
        for (int k = 0; k < desc->dim; ++k) {
            if (desc->csize[k] != 0) throw std::invalid_argument("mgr_register derives the grid from the rate");
            if (desc->size[k] < 2) throw std::invalid_argument("image dimensions must be >= 2");
        }
        if (mz->kind != MGR_MIN_GSL_SD && mz->kind != MGR_MIN_GDSQ) throw std::invalid_argument("unknown minimizer");
        if (mz->maxiter < 1) throw std::invalid_argument("maxiter must be >= 1");
        ck(cudaSetDevice(device), "cudaSetDevice");
        configure_pool(device);
        cudaStream_t st;
        ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard()
            {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
        } guard{st};
        const int dim = desc->dim;
        const size_t n = size_t(desc->size[0]) * desc->size[1] * (dim == 3 ? desc->size[2] : 1);
        std::vector<double> params;
        int cs[3] = {1, 1, 1};
        double cost = 0.0;
        {
            DevBuf<float> d_src, d_ref;
            d_src.alloc(n, st);
            d_ref.alloc(n, st);
            ck(cudaMemcpyAsync(d_src.p, src, n * sizeof(float), cudaMemcpyHostToDevice, st), "H2D");
            ck(cudaMemcpyAsync(d_ref.p, ref, n * sizeof(float), cudaMemcpyHostToDevice, st), "H2D");
            cost = register_pair_device(*desc, levels, *mz, d_src.p, d_ref.p, path, device, params, cs, evaluations,
                                        st);
            trace_report("mgr_register");
        }
        if (params.size() > max_params) throw std::invalid_argument("params_out too small");
        std::copy(params.begin(), params.end(), params_out);
        for (int k = 0; k < 3; ++k) csize_out[k] = cs[k];
        if (final_cost) *final_cost = cost;
        return MGR_OK;
    } catch (const std::invalid_argument &e) {
        set_last_error(e.what());
        return MGR_ERR_ARG;
    } catch (const TimeoutError &e) {
        set_last_error(e.what());
        return MGR_ERR_TIMEOUT;
    } catch (const std::bad_alloc &) {
        set_last_error("allocation failed");
        return MGR_ERR_OOM;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return MGR_ERR_CUDA;
    }
}

extern "C" mgr_status mgr_scale_image(int dim, const int in_size[3], const float *in, const int out_size[3],
                                      float *out, int device)
{
    if (!in_size || !in || !out_size || !out || (dim != 2 && dim != 3)) {
        set_last_error("mgr_scale_image: invalid argument");
        return MGR_ERR_ARG;
    }
    for (int k = 0; k < dim; ++k)
        if (in_size[k] < 1 || out_size[k] < 1) {
            set_last_error("mgr_scale_image: sizes must be positive");
            return MGR_ERR_ARG;
        }
    float *d_in = nullptr, *d_out = nullptr;
    cudaStream_t st = nullptr;
    try {
        ck(cudaSetDevice(device), "cudaSetDevice");
        ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
        const size_t ni = size_t(in_size[0]) * in_size[1] * (dim == 3 ? in_size[2] : 1);
        const size_t no = size_t(out_size[0]) * out_size[1] * (dim == 3 ? out_size[2] : 1);
        ck(dev_malloc(reinterpret_cast<void **>(&d_in), ni * sizeof(float)), "cudaMalloc");
        ck(dev_malloc(reinterpret_cast<void **>(&d_out), no * sizeof(float)), "cudaMalloc");
        ck(cudaMemcpyAsync(d_in, in, ni * sizeof(float), cudaMemcpyHostToDevice, st), "H2D");
        scale_image(d_in, in_size, d_out, out_size, dim, st);
        ck(cudaMemcpyAsync(out, d_out, no * sizeof(float), cudaMemcpyDeviceToHost, st), "D2H");
        ck(cudaStreamSynchronize(st), "sync");
    } catch (const std::invalid_argument &e) {
        set_last_error(e.what());
        cudaFree(d_in);
        cudaFree(d_out);
        if (st) cudaStreamDestroy(st);
        return MGR_ERR_ARG;
    } catch (const std::exception &e) {
        const bool oom = dynamic_cast<const std::bad_alloc *>(&e) != nullptr;
        set_last_error(oom ? "mgr_scale_image: device allocation failed" : e.what());
        cudaFree(d_in);
        cudaFree(d_out);
        if (st) cudaStreamDestroy(st);
        return oom ? MGR_ERR_OOM : MGR_ERR_CUDA;
    }
    cudaFree(d_in);
    cudaFree(d_out);
    cudaStreamDestroy(st);
    return MGR_OK;
}

extern "C" mgr_status mgr_normalize_pair(const float *src, const float *ref, size_t n, float *src_out,
                                         float *ref_out, double *mean, double *sigma, int *applied, int device)
{
    if (!src || !ref || !src_out || !ref_out || n == 0) {
        set_last_error("mgr_normalize_pair: invalid argument");
        return MGR_ERR_ARG;
    }
    float *d[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaStream_t st = nullptr;
    mgr_status status = MGR_OK;
    try {
        ck(cudaSetDevice(device), "cudaSetDevice");
        ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto &p : d) ck(dev_malloc(reinterpret_cast<void **>(&p), n * sizeof(float)), "cudaMalloc");
        ck(cudaMemcpyAsync(d[0], src, n * sizeof(float), cudaMemcpyHostToDevice, st), "H2D");
        ck(cudaMemcpyAsync(d[1], ref, n * sizeof(float), cudaMemcpyHostToDevice, st), "H2D");
        const bool ok = normalize_pair(d[0], d[1], n, d[2], d[3], st, mean, sigma);
        if (applied) *applied = ok ? 1 : 0;
        if (ok) {
            ck(cudaMemcpyAsync(src_out, d[2], n * sizeof(float), cudaMemcpyDeviceToHost, st), "D2H");
            ck(cudaMemcpyAsync(ref_out, d[3], n * sizeof(float), cudaMemcpyDeviceToHost, st), "D2H");
        }
        ck(cudaStreamSynchronize(st), "sync");
    } catch (const std::bad_alloc &) {
        set_last_error("mgr_normalize_pair: device allocation failed");
        status = MGR_ERR_OOM;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        status = MGR_ERR_CUDA;
    }
    for (auto p : d) cudaFree(p);
    if (st) cudaStreamDestroy(st);
    return status;
}
