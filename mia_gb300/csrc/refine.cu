// refine.cu — the refinement of the spline transform's coefficient grid on
// the device (C3DSplineTransformation::refine, mia/3d/transform/spline.cc:
// 360-396; 2D mia/2d/transform/spline.cc:318-353), for several coefficient
// fields at once (the pairs of a batched registration).
//
// The steps and the order of every operation are those of the host
// restatement refine_params (driver.cc): parameters rounded to float, the
// per-component minimum and maximum, the mirror-boundary cubic prefilter of
// every x, y and z line in double, then the cubic B-spline resampling onto
// the finer grid as three separable stages (x taps, then y, then z, each sum
// from 0 in tap order), clamped to [min, max] and stored as float.  Each
// operation is rounded as written (__dmul_rn / __dadd_rn / __ddiv_rn: no
// fused multiply-add) and the powers p^(n-1) come from the host, so the
// values are those of the host code.
#include <algorithm>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mgr.h"
#include "driver.hh"
#include "mgr_common.cuh"
#include "mgr_kernels.hh"

namespace mgr {

void set_last_error(const std::string &msg);

namespace {

constexpr int RT = 256;

void ck(cudaError_t e, const char *what)
{
    if (e == cudaErrorMemoryAllocation) throw std::bad_alloc();
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

struct RefineJob {
    const double *in;
    double *coef;     // old grid, filtered in place
    double *r1, *r2;  // x resampled (oz, oy, nx), then y (oz, ny, nx)
    double *out;      // new grid
    float *mnmx;      // 2 x 3: per component min, max
    const int *ti[3];
    const double *tw[3];
    RefineFilterConsts fk[3];   // per axis of the old grid
    int no[3], nn[3];
};

__global__ void __launch_bounds__(RT) k_refine_prep(const RefineJob *jobs, int dim)
{
    const RefineJob &J = jobs[blockIdx.x];
    const size_t nold = size_t(J.no[0]) * J.no[1] * J.no[2];
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = threadIdx.x; i < nold; i += RT)
        for (int c = 0; c < dim; ++c) {
            const float v = float(J.in[i * dim + c]);
            J.coef[i * dim + c] = double(v);
            mn[c] = fminf(mn[c], v);
            mx[c] = fmaxf(mx[c], v);
        }
    __shared__ float smn[3][RT / 32], smx[3][RT / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = 0; c < dim; ++c) {
        float a = mn[c], b = mx[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = fminf(a, __shfl_xor_sync(0xffffffffu, a, o));
            b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
        }
        if (lane == 0) {
            smn[c][w] = a;
            smx[c][w] = b;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a[3], b[3];
        bool all_pos = true;
        for (int c = 0; c < dim; ++c) {
            a[c] = smn[c][0];
            b[c] = smx[c][0];
            for (int k = 1; k < RT / 32; ++k) {
                a[c] = fminf(a[c], smn[c][k]);
                b[c] = fmaxf(b[c], smx[c][k]);
            }
            if (!(0.0f < a[c])) all_pos = false;
        }
        // "if (T() < m_min) m_min = T()": the vector < compares all components
        for (int c = 0; c < dim; ++c) {
            J.mnmx[c] = all_pos ? 0.0f : a[c];
            J.mnmx[3 + c] = b[c];
        }
    }
}

// the mirror-boundary cubic prefilter of one line (stride s), in place
__device__ void filter_line_dev(double *c, size_t s, int n, const RefineFilterConsts &k)
{
    if (n < 2) return;
    const double p = k.p;
    for (int i = 0; i < n; ++i) c[i * s] = __dmul_rn(c[i * s], k.lambda);
    double zn = p;
    double z2n = k.z2n;
    double sum = __dadd_rn(c[0], __dmul_rn(z2n, c[(n - 1) * s]));
    z2n = __dmul_rn(z2n, __dmul_rn(z2n, k.iz));
    for (int i = 1; i < n - 1; ++i) {
        sum = __dadd_rn(sum, __dmul_rn(__dadd_rn(zn, z2n), c[i * s]));
        zn = __dmul_rn(zn, p);
        z2n = __dmul_rn(z2n, k.iz);
    }
    c[0] = __ddiv_rn(sum, __dsub_rn(1.0, __dmul_rn(zn, zn)));
    for (int i = 1; i < n; ++i) c[i * s] = __dadd_rn(c[i * s], __dmul_rn(p, c[(i - 1) * s]));
    c[(n - 1) * s] = __dmul_rn(k.q, __dadd_rn(__dmul_rn(p, c[(n - 2) * s]), c[(n - 1) * s]));
    for (int i = n - 2; i >= 0; --i) c[i * s] = __dmul_rn(p, __dsub_rn(c[(i + 1) * s], c[i * s]));
}

// one thread per (line, component) of axis `axis`, lines in the order of
// the host loops (the lines are independent, the order does not matter)
__global__ void __launch_bounds__(RT) k_refine_filter(const RefineJob *jobs, int dim, int axis)
{
    const RefineJob &J = jobs[blockIdx.y];
    const int ox = J.no[0], oy = J.no[1], oz = J.no[2];
    const int n = J.no[axis];
    const size_t lines = size_t(ox) * oy * oz / n;
    const size_t stride = (axis == 0 ? 1 : axis == 1 ? size_t(ox) : size_t(ox) * oy) * dim;
    for (size_t t = blockIdx.x * size_t(RT) + threadIdx.x; t < lines * dim; t += size_t(gridDim.x) * RT) {
        const int c = int(t % dim);
        const size_t l = t / dim;
        size_t base;
        if (axis == 0) base = l * ox;                                         // (z, y)
        else if (axis == 1) base = (l / ox) * size_t(ox) * oy + (l % ox);     // (z, x)
        else base = l;                                                        // (y, x)
        filter_line_dev(J.coef + base * dim + c, stride, n, J.fk[axis]);
    }
}

__device__ __forceinline__ double tap_sum(const double *w, double a0, double a1, double a2, double a3)
{
    double r = 0.0;
    r = __dadd_rn(r, __dmul_rn(w[0], a0));
    r = __dadd_rn(r, __dmul_rn(w[1], a1));
    r = __dadd_rn(r, __dmul_rn(w[2], a2));
    r = __dadd_rn(r, __dmul_rn(w[3], a3));
    return r;
}

// stage 0: x taps, r1[(z, y), x_new]; stage 1: y taps, r2[(z, y_new), x_new];
// stage 2: z taps, clamp, float: out[(z_new, y_new), x_new]
__global__ void __launch_bounds__(RT) k_refine_stage(const RefineJob *jobs, int dim, int stage)
{
    const RefineJob &J = jobs[blockIdx.y];
    const int ox = J.no[0], oy = J.no[1], oz = J.no[2];
    const int nx = J.nn[0], ny = J.nn[1], nz = J.nn[2];
    const size_t rows = stage == 0 ? size_t(oz) * oy : stage == 1 ? size_t(oz) * ny : size_t(nz) * ny;
    const size_t total = rows * nx * dim;
    for (size_t t = blockIdx.x * size_t(RT) + threadIdx.x; t < total; t += size_t(gridDim.x) * RT) {
        const int c = int(t % dim);
        const size_t e = t / dim;
        const int x = int(e % nx);
        const size_t row = e / nx;
        if (stage == 0) {
            const int *ix = J.ti[0] + size_t(x) * 4;
            const double *src = J.coef + row * size_t(ox) * dim + c;
            J.r1[t] = tap_sum(J.tw[0] + size_t(x) * 4, src[size_t(ix[0]) * dim], src[size_t(ix[1]) * dim],
                              src[size_t(ix[2]) * dim], src[size_t(ix[3]) * dim]);
        } else if (stage == 1) {
            const int y = int(row % ny), z = int(row / ny);
            const int *iy = J.ti[1] + size_t(y) * 4;
            const size_t rown = size_t(nx) * dim, col = size_t(x) * dim + c;
            const double *b = J.r1 + size_t(z) * oy * rown + col;
            J.r2[t] = tap_sum(J.tw[1] + size_t(y) * 4, b[iy[0] * rown], b[iy[1] * rown], b[iy[2] * rown],
                              b[iy[3] * rown]);
        } else {
            const int y = int(row % ny), z = int(row / ny);
            const size_t rown = size_t(nx) * dim, col = size_t(x) * dim + c;
            const double *b = J.r2 + size_t(y) * rown + col;
            double r;
            if (dim == 3) {
                const int *iz = J.ti[2] + size_t(z) * 4;
                const size_t pz = size_t(ny) * rown;
                r = tap_sum(J.tw[2] + size_t(z) * 4, b[iz[0] * pz], b[iz[1] * pz], b[iz[2] * pz], b[iz[3] * pz]);
            } else {
                r = __dadd_rn(0.0, __dmul_rn(J.tw[2][size_t(z) * 4], b[0]));
            }
            const double mn = J.mnmx[c], mx = J.mnmx[3 + c];
            r = (r >= mn) ? ((r <= mx) ? r : mx) : mn;
            J.out[t] = double(__double2float_rn(r));
        }
    }
}

}  // namespace

void refine_params_device(int dim, const std::vector<RefineJobSpec> &specs, cudaStream_t st)
{
    if (specs.empty()) return;
    if (dim != 2 && dim != 3) throw std::invalid_argument("refine: dim must be 2 or 3");
    const int nj = int(specs.size());
    // one device blob: the job table, the taps, the per-job min/max and the
    // double scratch of all jobs
    std::vector<RefineJob> jobs(nj);
    std::vector<std::vector<int>> ti(size_t(nj) * 3);
    std::vector<std::vector<double>> tw(size_t(nj) * 3);
    size_t tap_ints = 0, tap_dbls = 0, scratch = 0;
    size_t max_lines = 0, max_stage = 0;
    for (int j = 0; j < nj; ++j) {
        const RefineJobSpec &s = specs[j];
        RefineJob &J = jobs[j];
        for (int k = 0; k < 3; ++k) {
            J.no[k] = k < dim ? s.nc_old[k] : 1;
            J.nn[k] = k < dim ? s.nc_new[k] : 1;
            if (k < dim && (J.no[k] < 4 || J.nn[k] < 4))
                throw std::invalid_argument("refine: grids must have more than 3 coefficients per axis");
            std::vector<int> &I = ti[size_t(j) * 3 + k];
            std::vector<double> &W = tw[size_t(j) * 3 + k];
            if (k < dim) {
                refine_axis_taps(J.no[k], J.nn[k], I, W);
            } else {
                I.assign(size_t(J.nn[k]) * 4, 0);
                W.assign(size_t(J.nn[k]) * 4, 0.0);
                for (int i = 0; i < J.nn[k]; ++i) W[size_t(i) * 4] = 1.0;
            }
            J.fk[k] = refine_filter_consts(J.no[k]);
            tap_ints += I.size();
            tap_dbls += W.size();
        }
        const size_t nold = size_t(J.no[0]) * J.no[1] * J.no[2];
        scratch += (nold + size_t(J.no[2]) * J.no[1] * J.nn[0] + size_t(J.no[2]) * J.nn[1] * J.nn[0]) * dim;
        for (int k = 0; k < dim; ++k) max_lines = std::max(max_lines, nold / J.no[k] * dim);
        max_stage = std::max(max_stage, size_t(J.nn[2]) * J.nn[1] * J.nn[0] * dim);
        max_stage = std::max(max_stage, size_t(J.no[2]) * J.nn[1] * J.nn[0] * dim);
    }
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t o_jobs = 0;
    const size_t o_mm = up(o_jobs + sizeof(RefineJob) * nj);
    const size_t o_tw = up(o_mm + sizeof(float) * 6 * nj);
    const size_t o_ti = up(o_tw + sizeof(double) * tap_dbls);
    const size_t o_sc = up(o_ti + sizeof(int) * tap_ints);
    const size_t bytes = o_sc + sizeof(double) * scratch;
    unsigned char *d = nullptr;
    ck(dev_malloc_async(reinterpret_cast<void **>(&d), bytes, st), "cudaMallocAsync");
    std::vector<unsigned char> host(o_sc, 0);
    size_t pi = 0, pd = 0, ps = 0;
    for (int j = 0; j < nj; ++j) {
        RefineJob &J = jobs[j];
        J.in = specs[j].in;
        J.out = specs[j].out;
        J.mnmx = reinterpret_cast<float *>(d + o_mm) + 6 * j;
        for (int k = 0; k < 3; ++k) {
            const std::vector<int> &I = ti[size_t(j) * 3 + k];
            const std::vector<double> &W = tw[size_t(j) * 3 + k];
            std::memcpy(host.data() + o_ti + sizeof(int) * pi, I.data(), sizeof(int) * I.size());
            std::memcpy(host.data() + o_tw + sizeof(double) * pd, W.data(), sizeof(double) * W.size());
            J.ti[k] = reinterpret_cast<const int *>(d + o_ti) + pi;
            J.tw[k] = reinterpret_cast<const double *>(d + o_tw) + pd;
            pi += I.size();
            pd += W.size();
        }
        const size_t nold = size_t(J.no[0]) * J.no[1] * J.no[2];
        double *sc = reinterpret_cast<double *>(d + o_sc) + ps;
        J.coef = sc;
        J.r1 = sc + nold * dim;
        J.r2 = J.r1 + size_t(J.no[2]) * J.no[1] * J.nn[0] * dim;
        ps += (nold + size_t(J.no[2]) * J.no[1] * J.nn[0] + size_t(J.no[2]) * J.nn[1] * J.nn[0]) * dim;
    }
    std::memcpy(host.data() + o_jobs, jobs.data(), sizeof(RefineJob) * nj);
    ck(cudaMemcpyAsync(d, host.data(), host.size(), cudaMemcpyHostToDevice, st), "refine tables H2D");
    const RefineJob *dj = reinterpret_cast<const RefineJob *>(d + o_jobs);
    k_refine_prep<<<nj, RT, 0, st>>>(dj, dim);
    count_launch();
    const unsigned gl = unsigned(std::min<size_t>(64, (max_lines + RT - 1) / RT));
    for (int axis = 0; axis < dim; ++axis) {
        k_refine_filter<<<dim3(gl, nj), RT, 0, st>>>(dj, dim, axis);
        count_launch();
    }
    const unsigned gs = unsigned(std::min<size_t>(512, (max_stage + RT - 1) / RT));
    for (int stage = 0; stage < 3; ++stage) {
        k_refine_stage<<<dim3(gs, nj), RT, 0, st>>>(dj, dim, stage);
        count_launch();
    }
    ck(cudaGetLastError(), "refine kernels");
    cudaFreeAsync(d, st);
}

}  // namespace mgr

using namespace mgr;

namespace {

mgr_status refine_args(int dim, const int nc_old[3], const int nc_new[3], const void *in, const void *out,
                       const int *grown, const char *who)
{
    if ((dim != 2 && dim != 3) || !nc_old || !nc_new || !in || !out || !grown) {
        set_last_error(std::string(who) + ": invalid argument");
        return MGR_ERR_ARG;
    }
    for (int k = 0; k < dim; ++k)
        if (nc_old[k] < 4 || nc_new[k] < 4) {
            set_last_error(std::string(who) + ": grids must have more than 3 coefficients per axis");
            return MGR_ERR_ARG;
        }
    return MGR_OK;
}

}  // namespace

extern "C" mgr_status mgr_refine_coefficients(int dim, const int nc_old[3], const int nc_new[3], const double *in,
                                              double *out, int *grown)
{
    const mgr_status a = refine_args(dim, nc_old, nc_new, in, out, grown, "mgr_refine_coefficients");
    if (a != MGR_OK) return a;
    try {
        const size_t n = size_t(nc_old[0]) * nc_old[1] * (dim == 3 ? nc_old[2] : 1) * dim;
        std::vector<double> p(in, in + n);
        *grown = refine_params(dim, nc_old, nc_new, p) ? 1 : 0;
        if (*grown) std::copy(p.begin(), p.end(), out);
        return MGR_OK;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return MGR_ERR_ARG;
    }
}

extern "C" mgr_status mgr_refine_coefficients_device(int dim, const int nc_old[3], const int nc_new[3],
                                                     const double *d_in, double *d_out, int *grown, void *stream)
{
    const mgr_status a = refine_args(dim, nc_old, nc_new, d_in, d_out, grown, "mgr_refine_coefficients_device");
    if (a != MGR_OK) return a;
    try {
        *grown = refine_grows(dim, nc_old, nc_new) ? 1 : 0;
        if (!*grown) return MGR_OK;
        RefineJobSpec j;
        for (int k = 0; k < 3; ++k) {
            j.nc_old[k] = nc_old[k];
            j.nc_new[k] = nc_new[k];
        }
        j.in = d_in;
        j.out = d_out;
        refine_params_device(dim, std::vector<RefineJobSpec>{j}, static_cast<cudaStream_t>(stream));
        return MGR_OK;
    } catch (const std::invalid_argument &e) {
        set_last_error(e.what());
        return MGR_ERR_ARG;
    } catch (const std::bad_alloc &) {
        set_last_error("mgr_refine_coefficients_device: device allocation failed");
        return MGR_ERR_OOM;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return MGR_ERR_CUDA;
    }
}
