// pyramid.cu — image preparation of the registration driver on the GPU:
//
// * joint intensity normalisation of the pair (FScaleFilterCreator,
//   mia/template/nonrigidregister.cxx:147-184): sums over both images in
//   double, then y = float(a*x + b) with a = 1/sigma, b = -mean/sigma, where
//   a and b pass through the reference's 6-significant-digit filter string;
// * the `scale` filter that builds each multiresolution level
//   (C3DScale / C2DScale, mia/3d/filter/scale.cc:95-155,
//   mia/2d/filter/scale.cc:50-90; C1DScalar::downscale,
//   mia/core/scaler1d.cc): per axis and per line a binomial
//   "gauss:w=round(1/scale)" smoothing with half-sample symmetric borders
//   (mia/core/spacialkernel/gauss.cc), the mirror-boundary cubic prefilter,
//   and cubic B-spline resampling at i*(n_in-1)/(n_out-1).  The reference
//   filters in double; here the lines are filtered in float (FP64 runs at a
//   small fraction of the FP32 rate on this GPU), which moves the result by
//   a few float ulp: the parity tests bound it at 1e-5 of the image maximum.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "mgr_common.cuh"
#include "mgr_kernels.hh"
#include "pyramid.hh"

namespace mgr {

int device_sm_count()
{
    static std::atomic<int> cache[64];   // per device, 0 until read (zero-initialised: static storage)
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152;
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n == 0) {
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
        cache[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

struct Wt4 {
    double x, y, z, w;
};

// per-block sums of a + b and a^2 + b^2 in double: block `blk` of `nblk`
// takes elements blk * 256 + t + k * nblk * 256
// ca, cb (optional): where the values read are also copied (host images
// read in place are then read only once over the CPU-GPU link)
__device__ __forceinline__ void pair_sums_body(const float *__restrict__ a, const float *__restrict__ b, size_t n,
                                               double *part, int blk, int nblk, float *ca = nullptr,
                                               float *cb = nullptr)
{
    __shared__ double red[2 * 8];
    double v[2] = {0.0, 0.0};
    for (size_t i = blk * size_t(256) + threadIdx.x; i < n; i += size_t(nblk) * 256) {
        const float xa = a[i], xb = b[i];
        if (ca) {
            ca[i] = xa;
            cb[i] = xb;
        }
        const double fa = xa, fb = xb;
        v[0] += fa + fb;
        v[1] += fa * fa + fb * fb;
    }
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        part[2 * blk] = v[0];
        part[2 * blk + 1] = v[1];
    }
}

__global__ void __launch_bounds__(256) k_pair_sums(const float *__restrict__ a, const float *__restrict__ b, size_t n,
                                                   double *part)
{
    pair_sums_body(a, b, n, part, blockIdx.x, gridDim.x);
}

// the normalisation of several pairs: per pair its images, block count of
// the sums, partial-sum slots and the linear map out = a * in + b
struct NormJob {
    const float *src, *ref;
    float *src_out, *ref_out;
    size_t n;
    double *part;
    int nb, varied;
    int copied;   // 1: the sums pass copied the images to src_out / ref_out; the map runs in place there
    double a, b;
};

__global__ void __launch_bounds__(256) k_pair_sums_batch(const NormJob *jobs)
{
    const NormJob &J = jobs[blockIdx.y];
    if (int(blockIdx.x) >= J.nb) return;
    pair_sums_body(J.src, J.ref, J.n, J.part, blockIdx.x, J.nb, J.copied ? J.src_out : nullptr,
                   J.copied ? J.ref_out : nullptr);
}

__global__ void __launch_bounds__(256) k_apply_linear_batch(const NormJob *jobs)
{
    const NormJob &J = jobs[blockIdx.y];
    if (!J.varied) return;
    float *out = blockIdx.z ? J.ref_out : J.src_out;
    const float *in = J.copied ? out : (blockIdx.z ? J.ref : J.src);
    for (size_t i = blockIdx.x * size_t(256) + threadIdx.x; i < J.n; i += size_t(gridDim.x) * 256)
        out[i] = float(fma(J.a, double(in[i]), J.b));
}

__global__ void k_apply_linear(const float *__restrict__ in, float *__restrict__ out, size_t n, double a, double b)
{
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        out[i] = float(fma(a, double(in[i]), b));
}

// One block of SCALE_NT threads owns lb consecutive lines (lb <= 64), in
// float.  Per line: binomial smoothing with half-sample symmetric borders,
// the mirror-boundary cubic prefilter in place, then the 4-tap resampling
// (n_out <= n_in).  The block stages its input lines in shared memory with
// independent coalesced loads (along the line for the x pass, across the
// lines of consecutive x otherwise), smooths and resamples element-parallel
// over all its lines, and runs only the prefilter's recursion one thread
// per line.  Lines sit at an odd pitch (no bank conflicts between lines).
// The arithmetic of every element is that of a sequential pass over the
// line.
constexpr int SCALE_NT = 256;

__global__ void __launch_bounds__(SCALE_NT) k_scale_lines(const float *__restrict__ in, float *__restrict__ out,
                                                          int lb, int n_in, int n_out, int nlines,
                                                          size_t in_line_stride, size_t in_elem_stride,
                                                          size_t out_line_stride, size_t out_elem_stride,
                                                          int lines_per_plane, size_t in_plane_stride,
                                                          size_t out_plane_stride, int gw, const float *gmask,
                                                          const int4 *idx, const float4 *wts)
{
    extern __shared__ float sl[];
    const int pitch = n_in | 1;
    const int tid = threadIdx.x;
    const int l0 = blockIdx.x * lb;
    const int nl = min(lb, nlines - l0);
    const bool along = in_elem_stride == 1;   // x pass: the lines are rows
    auto line_in = [&](int l) {
        const int g = l0 + l, pl = g / lines_per_plane, lp = g % lines_per_plane;
        return in + size_t(pl) * in_plane_stride + size_t(lp) * in_line_stride;
    };
    auto line_out = [&](int l) {
        const int g = l0 + l, pl = g / lines_per_plane, lp = g % lines_per_plane;
        return out + size_t(pl) * out_plane_stride + size_t(lp) * out_line_stride;
    };
    if (gw < 0) {   // the size does not change on this axis (C1DScalar copies)
        for (int e = tid; e < nl * n_in; e += SCALE_NT) {
            const int l = along ? e / n_in : e % nl, k = along ? e % n_in : e / nl;
            line_out(l)[k * out_elem_stride] = __ldg(line_in(l) + k * in_elem_stride);
        }
        return;
    }
    float *c_all = sl;
    float *s_all = sl + size_t(lb) * pitch;
#pragma unroll 4
    for (int e = tid; e < nl * n_in; e += SCALE_NT) {
        const int l = along ? e / n_in : e % nl, k = along ? e % n_in : e / nl;
        c_all[l * pitch + k] = __ldg(line_in(l) + k * in_elem_stride);
    }
    __syncthreads();
    const int m = 2 * gw + 1;
    for (int e = tid; e < nl * n_in; e += SCALE_NT) {
        const int l = along ? e / n_in : e % nl, i = along ? e % n_in : e / nl;
        const float *c = c_all + l * pitch;
        float h = 0.0f;
        for (int j = 0; j < m; ++j) {
            int k = i - gw + j;
            if (k < 0) k = -k - 1;
            if (k >= n_in) k = 2 * n_in - 1 - k;
            h = fmaf(gmask[j], c[k], h);
        }
        s_all[l * pitch + i] = h;
    }
    __syncthreads();
    if (tid < nl && n_in >= 2) {
        float *s = s_all + tid * pitch;
        const float p = -0.2679491924311227f;            // sqrt(3) - 2
        const float lambda = 6.0f;                       // 2 - p - 1/p
        for (int k = 0; k < n_in; ++k) s[k] *= lambda;
        float zn = p;
        const float iz = 1.0f / p;
        float z2n = powf(p, float(n_in - 1));
        float sum = fmaf(z2n, s[n_in - 1], s[0]);
        z2n *= z2n * iz;
        for (int k = 1; k < n_in - 1; ++k) {
            sum = fmaf(zn + z2n, s[k], sum);
            zn *= p;
            z2n *= iz;
        }
        s[0] = sum / (1.0f - zn * zn);
        for (int k = 1; k < n_in; ++k) s[k] = fmaf(p, s[k - 1], s[k]);
        s[n_in - 1] = (p / (p * p - 1.0f)) * fmaf(p, s[n_in - 2], s[n_in - 1]);
        for (int k = n_in - 2; k >= 0; --k) s[k] = p * (s[k + 1] - s[k]);
    }
    __syncthreads();
    for (int e = tid; e < nl * n_out; e += SCALE_NT) {
        const int l = along ? e / n_out : e % nl, i = along ? e % n_out : e / nl;
        const float *s = s_all + l * pitch;
        const int4 ix = idx[i];
        const float4 w = wts[i];
        line_out(l)[i * out_elem_stride] = fmaf(w.x, s[ix.x], fmaf(w.y, s[ix.y], fmaf(w.z, s[ix.z], w.w * s[ix.w])));
    }
}

namespace {

int fastfloor_h(double v)
{
    volatile double t = v + 68719476736.0 * 1.5;
    double tt = t;
    uint64_t bits;
    memcpy(&bits, &tt, sizeof bits);
    return int32_t(uint32_t(bits & 0xffffffffu)) >> 16;
}

int mirror_h(int index, int width)
{
    const int w2 = 2 * width - 2;
    int idx = index < 0 ? -index : index;
    idx = (width == 1) ? 0 : ((idx < w2) ? idx : idx % w2);
    if (width <= idx) idx = w2 - idx;
    return idx;
}

void ck(cudaError_t e, const char *what)
{
    if (e == cudaErrorMemoryAllocation) throw std::bad_alloc();
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

int num_sms() { return device_sm_count(); }

// per-axis resampling plan of C1DScalar (downscale): gauss half width and
// the 4 taps + weights of every output sample
struct AxisPlan {
    int gw = 0;
    std::vector<double> mask;
    std::vector<int4> idx;
    std::vector<Wt4> wts;
};

AxisPlan plan_axis(int n_in, int n_out)
{
    AxisPlan p;
    if (n_in == n_out) {
        p.gw = -1;
        p.mask.assign(1, 1.0);
        p.idx.assign(1, make_int4(0, 0, 0, 0));
        p.wts.assign(1, Wt4{1, 0, 0, 0});
        return p;
    }
    const double scale = double(n_out - 1) / double(n_in - 1);
    p.gw = int(std::floor(1.0 / scale + 0.5));
    const int m = 2 * p.gw + 1;
    std::vector<double> k(m, 0.0);
    k[0] = 1.0;
    if (m > 1) k[1] = 1.0;
    std::vector<double> tmp(m, 0.0);
    for (int i = 2; i < m; ++i) {
        k[i] = 1.0;
        for (int j = 1; j < i; ++j) tmp[j] = k[j - 1] + k[j];
        for (int j = 1; j < i; ++j) k[j] = tmp[j];
    }
    const double norm = std::pow(2.0, m - 1);
    for (auto &v : k) v /= norm;
    p.mask = k;
    const double dx = 1.0 / scale;
    for (int i = 0; i < n_out; ++i) {
        const double x = double(i) * dx;
        const int ix = fastfloor_h(x);
        const double f = x - ix;
        const double ob6 = 1.0 / 6.0, xm1 = 1 - f;
        const double w0 = (xm1 * xm1) * (xm1 * ob6), w3 = (f * f) * (f * ob6);
        const double w1 = ((xm1 - w0) - w0) + w3, w2 = ((f - w3) - w3) + w0;
        int id[4];
        for (int q = 0; q < 4; ++q) id[q] = ix - 1 + q;
        if (id[0] < 0 || id[3] >= n_in)
            for (int q = 0; q < 4; ++q) id[q] = mirror_h(id[q], n_in);
        p.idx.push_back(make_int4(id[0], id[1], id[2], id[3]));
        p.wts.push_back(Wt4{w0, w1, w2, w3});
    }
    return p;
}

void scale_axis(const float *in, float *out, const AxisPlan &p, int n_in, int n_out, int nlines, size_t ils,
                size_t ies, size_t ols, size_t oes, int lpp, size_t ips, size_t ops, cudaStream_t st)
{
    // the plan (mask, taps, weights) as float in one stream-ordered upload;
    // the host blob may go away once the pageable copy has been issued
    std::vector<float> mask(p.mask.begin(), p.mask.end());
    std::vector<float4> wts;
    for (const Wt4 &w : p.wts) wts.push_back(make_float4(float(w.x), float(w.y), float(w.z), float(w.w)));
    const size_t o_idx = ((mask.size() * sizeof(float) + 15) / 16) * 16;
    const size_t o_wts = o_idx + p.idx.size() * sizeof(int4);
    const size_t bytes = o_wts + wts.size() * sizeof(float4);
    std::vector<unsigned char> blob(bytes, 0);
    std::memcpy(blob.data(), mask.data(), mask.size() * sizeof(float));
    std::memcpy(blob.data() + o_idx, p.idx.data(), p.idx.size() * sizeof(int4));
    std::memcpy(blob.data() + o_wts, wts.data(), wts.size() * sizeof(float4));
    unsigned char *d = nullptr;
    ck(dev_malloc_async(reinterpret_cast<void **>(&d), bytes, st), "cudaMallocAsync");
    ck(cudaMemcpyAsync(d, blob.data(), bytes, cudaMemcpyHostToDevice, st), "H2D");
    // lines per block: at most 64 and 96 KB of staged lines, fewer while
    // the launch would have less than two blocks per SM (the block's line
    // recursion is its critical path)
    const int pitch = n_in | 1;
    int lb = 64;
    while (lb > 1 && size_t(lb) * 2 * pitch * sizeof(float) > 96 * 1024) lb >>= 1;
    while (lb > 8 && (nlines + lb - 1) / lb < 2 * num_sms()) lb >>= 1;
    const size_t sm = size_t(lb) * 2 * pitch * sizeof(float);
    if (sm > 200 * 1024) throw std::invalid_argument("scale: image line too long");
    cudaFuncSetAttribute(k_scale_lines, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    k_scale_lines<<<(nlines + lb - 1) / lb, SCALE_NT, sm, st>>>(in, out, lb, n_in, n_out, nlines, ils, ies, ols, oes, lpp,
                                                         ips, ops, p.gw, reinterpret_cast<const float *>(d),
                                                         reinterpret_cast<const int4 *>(d + o_idx),
                                                         reinterpret_cast<const float4 *>(d + o_wts));
    count_launch();
    ck(cudaGetLastError(), "scale kernel");
    cudaFreeAsync(d, st);
}

}  // namespace

std::string format_g6(double v)
{
    char buf[64];
    snprintf(buf, sizeof buf, "%g", v);
    return buf;
}

namespace {

int pair_sum_blocks(size_t n) { return int(std::min<size_t>(512, (n + 255) / 256)); }

// mean and sigma of the two images together from the per-block partial
// sums (added in block order) and the linear map a * x + b; false when
// sigma is 0
bool norm_map(const double *part, int nb, size_t n, double &a, double &b, double *mean_out, double *sigma_out)
{
    double sum = 0.0, sum2 = 0.0;
    for (int k = 0; k < nb; ++k) {
        sum += part[2 * k];
        sum2 += part[2 * k + 1];
    }
    const double nn = 2.0 * double(n);
    const double mean = sum / nn;
    const double sigma = std::sqrt((sum2 - sum * sum / nn) / (nn - 1));
    if (mean_out) *mean_out = mean;
    if (sigma_out) *sigma_out = sigma;
    if (sigma == 0.0) return false;
    // the reference passes a and b through "convert:...,b=<v>,a=<v>" with
    // the default stream precision (6 significant digits)
    b = std::stod(format_g6(-mean / sigma));
    a = std::stod(format_g6(1.0 / sigma));
    return true;
}

bool normalize_from_sums(const double *part, int nb, const float *d_src, const float *d_ref, size_t n,
                         float *d_src_out, float *d_ref_out, cudaStream_t st, double *mean_out, double *sigma_out)
{
    double a = 0.0, b = 0.0;
    if (!norm_map(part, nb, n, a, b, mean_out, sigma_out)) return false;
    const int nb2 = int(std::min<size_t>(4096, (n + 255) / 256));
    k_apply_linear<<<nb2, 256, 0, st>>>(d_src, d_src_out, n, a, b);
    k_apply_linear<<<nb2, 256, 0, st>>>(d_ref, d_ref_out, n, a, b);
    count_launch(2);
    ck(cudaGetLastError(), "normalize kernels");
    return true;
}

}  // namespace

bool normalize_pair(const float *d_src, const float *d_ref, size_t n, float *d_src_out, float *d_ref_out,
                    cudaStream_t st, double *mean_out, double *sigma_out)
{
    const int nb = pair_sum_blocks(n);
    double *d_part = nullptr;
    ck(dev_malloc_async(reinterpret_cast<void **>(&d_part), size_t(nb) * 2 * sizeof(double), st), "cudaMallocAsync");
    k_pair_sums<<<nb, 256, 0, st>>>(d_src, d_ref, n, d_part);
    count_launch();
    std::vector<double> part(size_t(nb) * 2);
    ck(cudaMemcpyAsync(part.data(), d_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
    cudaFreeAsync(d_part, st);
    ck(cudaStreamSynchronize(st), "sync");
    return normalize_from_sums(part.data(), nb, d_src, d_ref, n, d_src_out, d_ref_out, st, mean_out, sigma_out);
}

std::vector<char> normalize_pairs(const std::vector<const float *> &src, const std::vector<const float *> &ref,
                                  const std::vector<size_t> &n, const std::vector<float *> &src_out,
                                  const std::vector<float *> &ref_out, cudaStream_t st, bool copy_first)
{
    const size_t np = src.size();
    std::vector<char> varied(np, 0);
    if (np == 0) return varied;
    // one launch of the sums for all pairs (each pair with the block count
    // of its own launch, so the same partial sums), one copy back, one
    // launch of the linear maps
    std::vector<NormJob> jobs(np);
    size_t nparts = 0, maxnb = 1, maxn = 1;
    for (size_t i = 0; i < np; ++i) {
        NormJob &J = jobs[i];
        J.src = src[i];
        J.ref = ref[i];
        J.src_out = src_out[i];
        J.ref_out = ref_out[i];
        J.n = n[i];
        J.nb = pair_sum_blocks(n[i]);
        J.varied = 0;
        J.copied = copy_first ? 1 : 0;
        J.a = J.b = 0.0;
        nparts += size_t(J.nb) * 2;
        maxnb = std::max<size_t>(maxnb, J.nb);
        maxn = std::max<size_t>(maxn, n[i]);
    }
    const size_t o_part = ((sizeof(NormJob) * np + 255) / 256) * 256;
    unsigned char *d = nullptr;
    ck(dev_malloc_async(reinterpret_cast<void **>(&d), o_part + nparts * sizeof(double), st), "cudaMallocAsync");
    double *d_part = reinterpret_cast<double *>(d + o_part);
    size_t off = 0;
    std::vector<size_t> at(np);
    for (size_t i = 0; i < np; ++i) {
        at[i] = off;
        jobs[i].part = d_part + off;
        off += size_t(jobs[i].nb) * 2;
    }
    ck(cudaMemcpyAsync(d, jobs.data(), sizeof(NormJob) * np, cudaMemcpyHostToDevice, st), "H2D");
    k_pair_sums_batch<<<dim3(unsigned(maxnb), unsigned(np)), 256, 0, st>>>(reinterpret_cast<const NormJob *>(d));
    count_launch();
    std::vector<double> part(nparts);
    ck(cudaMemcpyAsync(part.data(), d_part, nparts * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "sync");
    bool any = false;
    for (size_t i = 0; i < np; ++i) {
        NormJob &J = jobs[i];
        J.varied = norm_map(part.data() + at[i], J.nb, J.n, J.a, J.b, nullptr, nullptr) ? 1 : 0;
        varied[i] = char(J.varied);
        any |= J.varied != 0;
    }
    if (any) {
        ck(cudaMemcpyAsync(d, jobs.data(), sizeof(NormJob) * np, cudaMemcpyHostToDevice, st), "H2D");
        const unsigned nb2 = unsigned(std::min<size_t>(4096, (maxn + 255) / 256));
        k_apply_linear_batch<<<dim3(nb2, unsigned(np), 2), 256, 0, st>>>(reinterpret_cast<const NormJob *>(d));
        count_launch();
        ck(cudaGetLastError(), "normalize kernels");
    }
    cudaFreeAsync(d, st);
    return varied;
}

void scale_image(const float *d_in, const int in_size[3], float *d_out, const int out_size[3], int dim,
                 cudaStream_t st)
{
    const int nx = in_size[0], ny = in_size[1], nz = dim == 3 ? in_size[2] : 1;
    const int mx = out_size[0], my = out_size[1], mz = dim == 3 ? out_size[2] : 1;
    if (nx == mx && ny == my && nz == mz) {
        ck(cudaMemcpyAsync(d_out, d_in, size_t(nx) * ny * nz * sizeof(float), cudaMemcpyDeviceToDevice, st), "copy");
        return;
    }
    for (int k = 0; k < dim; ++k)
        if (out_size[k] > in_size[k] || out_size[k] < 2)
            throw std::invalid_argument("scale: only downscaling to sizes >= 2 is supported");
    // x: lines = rows (y, z)
    float *t1 = nullptr, *t2 = nullptr;
    ck(dev_malloc_async(reinterpret_cast<void **>(&t1), size_t(mx) * ny * nz * sizeof(float), st), "cudaMallocAsync");
    const AxisPlan px = plan_axis(nx, mx);
    const AxisPlan py = plan_axis(ny, my);
    // (C1DScalar copies when the size does not change on an axis)
    scale_axis(d_in, t1, px, nx, mx, ny * nz, size_t(nx), 1, size_t(mx), 1, ny * nz, 0, 0, st);
    if (dim == 2) {
        // y: lines = columns x, stride mx
        scale_axis(t1, d_out, py, ny, my, mx, 1, size_t(mx), 1, size_t(mx), mx, 0, 0, st);
        cudaFreeAsync(t1, st);
        return;
    }
    ck(dev_malloc_async(reinterpret_cast<void **>(&t2), size_t(mx) * my * nz * sizeof(float), st), "cudaMallocAsync");
    // y: lines = (x, z): per plane z, mx lines of stride 1, element stride mx
    scale_axis(t1, t2, py, ny, my, mx * nz, 1, size_t(mx), 1, size_t(mx), mx, size_t(mx) * ny, size_t(mx) * my, st);
    // z: lines = (x, y): mx*my lines, element stride mx*my
    const AxisPlan pz = plan_axis(nz, mz);
    scale_axis(t2, d_out, pz, nz, mz, mx * my, 1, size_t(mx) * my, 1, size_t(mx) * my, mx * my, 0, 0, st);
    cudaFreeAsync(t1, st);
    cudaFreeAsync(t2, st);
}

}  // namespace mgr
