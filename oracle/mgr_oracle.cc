/*
 * mgr_oracle.cc — CPU restatement of MIA's B-spline nonrigid-registration
 * cost+gradient path (gerddie/mia).  TEST INFRASTRUCTURE ONLY: the checker
 * for the CUDA path and the timed CPU baseline.  Nothing in the product
 * library links or calls this file.
 *
 * Every routine names the reference routine (file:line, paths relative to
 * the reference project) whose arithmetic it restates.  The reference cannot
 * be compiled here (it needs Boost, GSL, Eigen3, FFTW3 and libxml2), so this
 * file is pinned against the known answers of the reference's own unit
 * tests (tests/golden/).
 *
 * Precision policy: the template parameter P selects the reference's
 * float/double mix (RefP) or all-double evaluation (F64P).  The build uses
 * -ffp-contract=off so that x86-64 and aarch64 round identically and match
 * the reference's SSE2 (non-FMA) x86-64 build.
 */
#include "mgr_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <thread>
#include <vector>

namespace {

/* ------------------------------------------------------------------ */
/* host threading: contiguous chunks, like the std::thread fallback of  */
/* pfor/preduce (mia/core/parallelcxx11.hh:158-240)                    */
/* ------------------------------------------------------------------ */
struct Pool {
    int threads = 1;
    template <class F> void pfor(int begin, int end, F f) const {
        int n = end - begin;
        if (n <= 0) return;
        int t = std::max(1, std::min(threads, n));
        if (t == 1) { f(begin, end); return; }
        std::vector<std::thread> ws;
        int chunk = (n + t - 1) / t;
        for (int k = 0; k < t; ++k) {
            int b = begin + k * chunk, e = std::min(end, b + chunk);
            if (b >= e) break;
            ws.emplace_back([=, &f] { f(b, e); });
        }
        for (auto &w : ws) w.join();
    }
};

/* ------------------------------------------------------------------ */
/* a1: cubic B-spline kernel                                           */
/* ------------------------------------------------------------------ */
/* fixed-point floor with 2^-16 resolution: the value is rounded to the
   nearest multiple of 2^-16 by adding 1.5*2^36, then the 16.16 fixed-point
   word is shifted (mia/core/splinekernel.cc:164-192). */
inline int fastfloor(double v)
{
    volatile double t = v + 68719476736.0 * 1.5;
    double tt = t;
    uint64_t bits;
    std::memcpy(&bits, &tt, sizeof bits);
    int32_t lo = static_cast<int32_t>(static_cast<uint32_t>(bits & 0xffffffffu));
    return lo >> 16;
}

/* CBSplineKernel3::get_weights, SSE2 evaluation order
   (mia/core/splinekernel/bspline.cc:258-285) */
inline void weights3(double x, double w[4])
{
    const double ob6 = 1.0 / 6.0;
    const double xm1 = 1 - x;
    const double w0 = (xm1 * xm1) * (xm1 * ob6);
    const double w3 = (x * x) * (x * ob6);
    w[0] = w0;
    w[3] = w3;
    w[1] = ((xm1 - w0) - w0) + w3;
    w[2] = ((x - w3) - w3) + w0;
}

/* CBSplineKernel3::get_derivative_weights (bspline.cc:287-293) */
inline void dweights3(double x, double w[4])
{
    w[3] = 0.5 * x * x;
    w[0] = x - 0.5 - w[3];
    w[2] = 1 + w[0] - 2.0 * w[3];
    w[1] = -w[0] - w[2] - w[3];
}

/* bspline<3,k>::apply (bspline.cc:328-393) */
inline double bspline3_at(double x, int deg)
{
    if (deg == 0) {
        const double ob6 = 1.0 / 6.0;
        x = std::fabs(x);
        if (x <= 1.0) return 2.0 / 3.0 - x * x * (1 - 0.5 * x);
        if (x < 2.0) { const double dx = 2.0 - x; return dx * dx * dx * ob6; }
        return 0.0;
    }
    if (deg == 1) {
        double ax = std::fabs(x);
        if (ax <= 1.0) return (1.5 * ax - 2) * x;
        if (ax <= 2.0) return (x > 0.0 ? -0.5 : 0.5) * (2 - ax) * (2 - ax);
        return 0.0;
    }
    if (deg == 2) {
        x = std::fabs(x);
        if (x > 2.0) return 0.0;
        if (x > 1.0) return 2.0 - x;
        return 3.0 * x - 2.0;
    }
    return 0.0;
}

/* CSplineKernel::get_start_idx_and_value_weights (splinekernel.cc:250-255),
   degree 3: shift 0, half degree 1 */
inline int start_weights(double x, double w[4])
{
    const int r = fastfloor(x);
    weights3(x - r, w);
    return r - 1;
}

/* ------------------------------------------------------------------ */
/* a2: mirror boundary + prefilter                                      */
/* ------------------------------------------------------------------ */
/* CMirrorOnBoundary::do_apply (mia/core/splinebc/bc.cc:52-64) */
inline int mirror_fold(int index, int width)
{
    const int w2 = 2 * width - 2;
    int idx = index < 0 ? -index : index;
    idx = (width == 1) ? 0 : ((idx < w2) ? idx : idx % w2);
    if (width <= idx) idx = w2 - idx;
    return idx;
}

const double kPole = std::sqrt(3.0) - 2.0;

/* CSplineBoundaryCondition::filter_line (mia/core/boundary_conditions.cc:62-103)
   with CMirrorOnBoundary::initial_coeff / initial_anti_coeff (bc.cc:67-88) */
void filter_line(double *c, int n)
{
    if (n < 2) return;
    const double p = kPole;
    double lambda = 1.0;
    lambda *= 2 - p - 1.0 / p;
    for (int i = 0; i < n; ++i) c[i] *= lambda;
    {
        double zn = p;
        const double iz = 1.0 / p;
        double z2n = std::pow(p, double(n - 1));
        double sum = c[0] + z2n * c[n - 1];
        z2n *= z2n * iz;
        for (int k = 1; k < n - 1; ++k) {
            sum += (zn + z2n) * c[k];
            zn *= p;
            z2n *= iz;
        }
        c[0] = sum / (1.0 - zn * zn);
    }
    for (int k = 1; k < n; ++k) c[k] += p * c[k - 1];
    c[n - 1] = (p / (p * p - 1.0)) * (p * c[n - 2] + c[n - 1]);
    for (int k = n - 2; k >= 0; --k) c[k] = p * (c[k + 1] - c[k]);
}

/* separable prefilter x, then y, then z; each line filtered in a double
   temporary and stored back in T after each axis
   (mia/3d/interpolator.cxx:98-164, mia/core/boundary_conditions.hh:247-300,
   2D: mia/2d/interpolator.cxx:91-132) */
template <class T>
void prefilter_nd(T *c, int nx, int ny, int nz, const Pool &pool)
{
    pool.pfor(0, nz, [&](int zb, int ze) {
        std::vector<double> buf(nx);
        for (int z = zb; z < ze; ++z)
            for (int y = 0; y < ny; ++y) {
                T *l = c + (size_t(z) * ny + y) * nx;
                for (int x = 0; x < nx; ++x) buf[x] = l[x];
                filter_line(buf.data(), nx);
                for (int x = 0; x < nx; ++x) l[x] = static_cast<T>(buf[x]);
            }
    });
    pool.pfor(0, nz, [&](int zb, int ze) {
        std::vector<double> buf(ny);
        for (int z = zb; z < ze; ++z)
            for (int x = 0; x < nx; ++x) {
                T *l = c + size_t(z) * ny * nx + x;
                for (int y = 0; y < ny; ++y) buf[y] = l[size_t(y) * nx];
                filter_line(buf.data(), ny);
                for (int y = 0; y < ny; ++y) l[size_t(y) * nx] = static_cast<T>(buf[y]);
            }
    });
    if (nz > 1)
        pool.pfor(0, ny, [&](int yb, int ye) {
            std::vector<double> buf(nz);
            const size_t sl = size_t(nx) * ny;
            for (int y = yb; y < ye; ++y)
                for (int x = 0; x < nx; ++x) {
                    T *l = c + size_t(y) * nx + x;
                    for (int z = 0; z < nz; ++z) buf[z] = l[z * sl];
                    filter_line(buf.data(), nz);
                    for (int z = 0; z < nz; ++z) l[z * sl] = static_cast<T>(buf[z]);
                }
        });
}

/* ------------------------------------------------------------------ */
/* precision policies                                                    */
/* ------------------------------------------------------------------ */
struct RefP {           /* the reference's own mix */
    typedef float Img;  /* images, coefficients, forces, grid */
    typedef float Crd;  /* transform scale and grid coordinates */
    typedef float RowW; /* transposed spline rows (translate) */
    typedef float Acc;  /* tricubic / separable accumulators */
};
struct F64P {
    typedef double Img;
    typedef double Crd;
    typedef double RowW;
    typedef double Acc;
};

/* ------------------------------------------------------------------ */
/* a5: B-spline interpolator with mirror BC and clamp                   */
/* ------------------------------------------------------------------ */
template <class P>
struct Interp {
    typedef typename P::Img T;
    typedef typename P::Acc A;
    int dim = 3, nx = 1, ny = 1, nz = 1;
    std::vector<T> coeff;
    T mn = 0, mx = 0;

    /* T3DConvoluteInterpolator ctor + prefilter (interpolator.cxx:67-164) */
    void init(const T *img, int d, int sx, int sy, int sz, const Pool &pool)
    {
        dim = d; nx = sx; ny = sy; nz = (d == 3) ? sz : 1;
        const size_t n = size_t(nx) * ny * nz;
        coeff.assign(img, img + n);
        mn = mx = img[0];
        for (size_t i = 1; i < n; ++i) {
            if (img[i] > mx) mx = img[i];
            if (img[i] < mn) mn = img[i];
        }
        if (T() < mn) mn = T();
        prefilter_nd(coeff.data(), nx, ny, nz, pool);
    }

    static void axis(double x, int width, int idx[4], A w[4])
    {
        double wd[4];
        const int s = start_weights(x, wd);
        for (int k = 0; k < 4; ++k) {
            int i = s + k;
            if (s < 0 || s + 3 >= width) i = mirror_fold(i, width);
            idx[k] = i;
            w[k] = static_cast<A>(wd[k]);
        }
    }

    /* operator()(x, cache) with add_3d<float,4> (interpolator.cxx:250-287,
       mia/3d/interpolator.cc:368-433): z first, then y, then x, then the
       four x lanes summed left to right (SSE2 build, no SSE3) */
    T operator()(double x, double y, double z) const
    {
        int ix[4], iy[4], iz[4];
        A wx[4], wy[4], wz[4];
        axis(x, nx, ix, wx);
        axis(y, ny, iy, wy);
        axis(z, nz, iz, wz);
        A t1[4][4];
        for (int yy = 0; yy < 4; ++yy)
            for (int xx = 0; xx < 4; ++xx) t1[yy][xx] = A(0);
        for (int zz = 0; zz < 4; ++zz)
            for (int yy = 0; yy < 4; ++yy) {
                const T *row = &coeff[(size_t(iz[zz]) * ny + iy[yy]) * nx];
                for (int xx = 0; xx < 4; ++xx) {
                    A prod = wz[zz] * static_cast<A>(row[ix[xx]]);
                    t1[yy][xx] = (zz == 0) ? prod : A(t1[yy][xx] + prod);
                }
            }
        A t2[4];
        for (int xx = 0; xx < 4; ++xx) t2[xx] = wy[0] * t1[0][xx];
        for (int yy = 1; yy < 4; ++yy)
            for (int xx = 0; xx < 4; ++xx) t2[xx] = A(t2[xx] + A(wy[yy] * t1[yy][xx]));
        for (int xx = 0; xx < 4; ++xx) t2[xx] = A(t2[xx] * wx[xx]);
        A r = A(A(A(t2[0] + t2[1]) + t2[2]) + t2[3]);
        return clamp(static_cast<T>(r));
    }

    /* 2D: add_2d_new (mia/2d/interpolator.cxx:216-250, 277-311) */
    T operator()(double x, double y) const
    {
        int ix[4], iy[4];
        A wx[4], wy[4];
        axis(x, nx, ix, wx);
        axis(y, ny, iy, wy);
        A r = A(0);
        for (int yy = 0; yy < 4; ++yy) {
            const T *row = &coeff[size_t(iy[yy]) * nx];
            A rx = A(0);
            for (int xx = 0; xx < 4; ++xx) rx = A(rx + A(wx[xx] * static_cast<A>(row[ix[xx]])));
            r = A(r + A(wy[yy] * rx));
        }
        return clamp(static_cast<T>(r));
    }

    /* bounded<> (interpolator.cxx:284) */
    T clamp(T r) const { return (r >= mn) ? ((r <= mx) ? r : mx) : mn; }
};

/* ------------------------------------------------------------------ */
/* a3/a4/a9/a12: the spline transformation                              */
/* ------------------------------------------------------------------ */
struct Row { int first; std::vector<double> w; };

template <class P>
struct Spline {
    typedef typename P::Img T;
    typedef typename P::Crd C;
    typedef typename P::Acc A;
    typedef typename P::RowW RW;
    int dim = 3;
    int n[3] = {1, 1, 1};     /* image size */
    int nc[3] = {1, 1, 1};    /* coefficient grid */
    C scale[3] = {1, 1, 1};
    std::vector<int> start[3];
    std::vector<std::array<double, 4>> wts[3];
    std::vector<int> nw[3];
    std::vector<Row> rows[3];
    std::vector<T> coef;      /* nc product * dim, interleaved */

    /* csize from the rate: floor((n-1+rate)/rate) + 2
       (mia/3d/transform/spline.cc:130-147, mia/2d/transform/spline.cc:103-118) */
    static int csize_from_rate(int size, float rate)
    {
        float f = (float(size - 1) + rate) / rate;
        return int(f) + 2;
    }

    /* C3DSplineTransformation::get_derivative_row (spline.cc:697-729) */
    static std::vector<Row> derivative_rows(int nin, int nout, double sc)
    {
        std::vector<Row> res;
        for (int o = 0; o < nout; ++o) {
            Row v;
            v.first = -1;
            for (int i = 0; i < nin; ++i) {
                double x = double(i) * sc + 1.0 - double(o);
                if (std::fabs(x) < 2.0) {
                    if (v.first < 0) v.first = i;
                    double y = bspline3_at(x, 0);
                    if (y > 0)
                        v.w.push_back(static_cast<double>(static_cast<RW>(y)));
                    else
                        break;
                }
            }
            res.push_back(v);
        }
        return res;
    }

    /* reinit (spline.cc:224-275; 2D spline.cc:170-203) */
    void init(int d, const int size[3], const int csize[3])
    {
        dim = d;
        for (int a = 0; a < 3; ++a) {
            n[a] = (a < d) ? size[a] : 1;
            nc[a] = (a < d) ? csize[a] : 1;
        }
        for (int a = 0; a < d; ++a) {
            scale[a] = C(nc[a] - 1 - 2) / C(n[a] - 1);
            start[a].resize(n[a]);
            wts[a].resize(n[a]);
            nw[a].assign(n[a], 4);
            for (int i = 0; i < n[a]; ++i) {
                C xc = C(C(i) * scale[a]) + C(1);
                double w[4];
                start[a][i] = start_weights(double(xc), w);
                for (int k = 0; k < 4; ++k) wts[a][i][k] = w[k];
            }
            nw[a][n[a] - 1] = 3;
            rows[a] = derivative_rows(n[a], nc[a], double(scale[a]));
        }
        coef.assign(size_t(nc[0]) * nc[1] * nc[2] * d, T(0));
    }

    size_t ncoef() const { return size_t(nc[0]) * nc[1] * nc[2]; }

    void set_params(const double *p)
    {
        const size_t m = ncoef() * dim;
        for (size_t i = 0; i < m; ++i) coef[i] = static_cast<T>(p[i]);
    }

    /* init_grid: u(x) by x, y, z saxpy passes (spline.cc:541-653); the
       grid returned is X - u.  Output u only (3 per voxel). */
    void displacement3(std::vector<T> &u, const Pool &pool) const
    {
        const int nx = n[0], ny = n[1], nz = n[2];
        const int cx = nc[0], cy = nc[1], cz = nc[2];
        std::vector<T> tmp(size_t(nx) * cy * cz * 3);
        pool.pfor(0, cz, [&](int zb, int ze) {
            for (int z = zb; z < ze; ++z)
                for (int y = 0; y < cy; ++y)
                    for (int x = 0; x < nx; ++x) {
                        A acc[3] = {A(0), A(0), A(0)};
                        const int s = start[0][x];
                        for (int i = 0; i < nw[0][x]; ++i) {
                            if (s + i < 0 || s + i >= cx) continue;
                            const A w = static_cast<A>(wts[0][x][i]);
                            const T *c = &coef[((size_t(z) * cy + y) * cx + s + i) * 3];
                            for (int k = 0; k < 3; ++k) acc[k] = A(acc[k] + A(w * A(c[k])));
                        }
                        T *o = &tmp[((size_t(z) * cy + y) * nx + x) * 3];
                        for (int k = 0; k < 3; ++k) o[k] = T(acc[k]);
                    }
        });
        std::vector<T> tmp2(size_t(nx) * ny * cz * 3);
        pool.pfor(0, cz, [&](int zb, int ze) {
            for (int z = zb; z < ze; ++z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x) {
                        A acc[3] = {A(0), A(0), A(0)};
                        const int s = start[1][y];
                        for (int i = 0; i < nw[1][y]; ++i) {
                            if (s + i < 0 || s + i >= cy) continue;
                            const A w = static_cast<A>(wts[1][y][i]);
                            const T *c = &tmp[((size_t(z) * cy + s + i) * nx + x) * 3];
                            for (int k = 0; k < 3; ++k) acc[k] = A(acc[k] + A(w * A(c[k])));
                        }
                        T *o = &tmp2[((size_t(z) * ny + y) * nx + x) * 3];
                        for (int k = 0; k < 3; ++k) o[k] = T(acc[k]);
                    }
        });
        u.assign(size_t(nx) * ny * nz * 3, T(0));
        pool.pfor(0, nz, [&](int zb, int ze) {
            for (int z = zb; z < ze; ++z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x) {
                        A acc[3] = {A(0), A(0), A(0)};
                        const int s = start[2][z];
                        for (int i = 0; i < nw[2][z]; ++i) {
                            if (s + i < 0 || s + i >= cz) continue;
                            const A w = static_cast<A>(wts[2][z][i]);
                            const T *c = &tmp2[((size_t(s + i) * ny + y) * nx + x) * 3];
                            for (int k = 0; k < 3; ++k) acc[k] = A(acc[k] + A(w * A(c[k])));
                        }
                        T *o = &u[((size_t(z) * ny + y) * nx + x) * 3];
                        for (int k = 0; k < 3; ++k) o[k] = T(acc[k]);
                    }
        });
    }

    /* on_grid (mia/2d/transform/spline.cc:640-666) */
    void displacement2(std::vector<T> &u, const Pool &pool) const
    {
        const int nx = n[0], ny = n[1];
        u.assign(size_t(nx) * ny * 2, T(0));
        pool.pfor(0, ny, [&](int yb, int ye) {
            for (int y = yb; y < ye; ++y)
                for (int x = 0; x < nx; ++x) {
                    A r[2] = {A(0), A(0)};
                    const int sy = start[1][y], sx = start[0][x];
                    for (int j = 0; j < nw[1][y] && sy + j < nc[1]; ++j) {
                        A hr[2] = {A(0), A(0)};
                        for (int i = 0; i < nw[0][x] && sx + i < nc[0]; ++i) {
                            const T *c = &coef[(size_t(sy + j) * nc[0] + sx + i) * 2];
                            const A w = static_cast<A>(wts[0][x][i]);
                            hr[0] = A(hr[0] + A(w * A(c[0])));
                            hr[1] = A(hr[1] + A(w * A(c[1])));
                        }
                        const A w = static_cast<A>(wts[1][y][j]);
                        r[0] = A(r[0] + A(w * hr[0]));
                        r[1] = A(r[1] + A(w * hr[1]));
                    }
                    T *o = &u[(size_t(y) * nx + x) * 2];
                    o[0] = T(r[0]);
                    o[1] = T(r[1]);
                }
        });
    }

    /* translate (spline.cc:731-791): separable transposed rows, z first in
       3D; the sum is negated */
    void translate3(const T *force, double *g, const Pool &pool) const
    {
        const int nx = n[0], ny = n[1], nz = n[2];
        const int cx = nc[0], cy = nc[1], cz = nc[2];
        (void)nz;
        std::vector<T> tmp(size_t(nx) * ny * cz * 3, T(0));
        pool.pfor(0, cz, [&](int zb, int ze) {
            for (int iz = zb; iz < ze; ++iz) {
                const Row &r = rows[2][iz];
                int i = r.first;
                T *o = &tmp[size_t(iz) * nx * ny * 3];
                for (size_t k = 0; k < r.w.size(); ++k, ++i) {
                    const A w = static_cast<A>(r.w[k]);
                    const T *f = &force[size_t(i) * nx * ny * 3];
                    for (size_t e = 0; e < size_t(nx) * ny * 3; ++e)
                        o[e] = T(A(o[e]) + A(w * A(f[e])));
                }
            }
        });
        std::vector<T> tmp2(size_t(nx) * cy * cz * 3);
        pool.pfor(0, cz, [&](int zb, int ze) {
            for (int iz = zb; iz < ze; ++iz)
                for (int x = 0; x < nx; ++x)
                    for (int oy = 0; oy < cy; ++oy) {
                        const Row &r = rows[1][oy];
                        A acc[3] = {A(0), A(0), A(0)};
                        for (size_t k = 0; k < r.w.size(); ++k) {
                            const T *f = &tmp[((size_t(iz) * ny + r.first + k) * nx + x) * 3];
                            const A w = static_cast<A>(r.w[k]);
                            for (int c = 0; c < 3; ++c) acc[c] = A(acc[c] + A(w * A(f[c])));
                        }
                        T *o = &tmp2[((size_t(iz) * cy + oy) * nx + x) * 3];
                        for (int c = 0; c < 3; ++c) o[c] = T(acc[c]);
                    }
        });
        pool.pfor(0, cz, [&](int zb, int ze) {
            for (int iz = zb; iz < ze; ++iz)
                for (int iy = 0; iy < cy; ++iy)
                    for (int ox = 0; ox < cx; ++ox) {
                        const Row &r = rows[0][ox];
                        A acc[3] = {A(0), A(0), A(0)};
                        for (size_t k = 0; k < r.w.size(); ++k) {
                            const T *f = &tmp2[((size_t(iz) * cy + iy) * nx + r.first + k) * 3];
                            const A w = static_cast<A>(r.w[k]);
                            for (int c = 0; c < 3; ++c) acc[c] = A(acc[c] + A(w * A(f[c])));
                        }
                        double *o = &g[((size_t(iz) * cy + iy) * cx + ox) * 3];
                        for (int c = 0; c < 3; ++c) o[c] = -double(acc[c]);
                    }
        });
    }

    /* 2D translate (mia/2d/transform/spline.cc:540-576): y rows first */
    void translate2(const T *force, double *g, const Pool &pool) const
    {
        const int nx = n[0], ny = n[1];
        const int cx = nc[0], cy = nc[1];
        (void)ny;
        std::vector<T> tmp(size_t(nx) * cy * 2);
        pool.pfor(0, nx, [&](int xb, int xe) {
            for (int x = xb; x < xe; ++x)
                for (int oy = 0; oy < cy; ++oy) {
                    const Row &r = rows[1][oy];
                    A acc[2] = {A(0), A(0)};
                    for (size_t k = 0; k < r.w.size(); ++k) {
                        const T *f = &force[((size_t(r.first + k)) * nx + x) * 2];
                        const A w = static_cast<A>(r.w[k]);
                        acc[0] = A(acc[0] + A(w * A(f[0])));
                        acc[1] = A(acc[1] + A(w * A(f[1])));
                    }
                    T *o = &tmp[(size_t(oy) * nx + x) * 2];
                    o[0] = T(acc[0]);
                    o[1] = T(acc[1]);
                }
        });
        for (int oy = 0; oy < cy; ++oy)
            for (int ox = 0; ox < cx; ++ox) {
                const Row &r = rows[0][ox];
                A acc[2] = {A(0), A(0)};
                for (size_t k = 0; k < r.w.size(); ++k) {
                    const T *f = &tmp[(size_t(oy) * nx + r.first + k) * 2];
                    const A w = static_cast<A>(r.w[k]);
                    acc[0] = A(acc[0] + A(w * A(f[0])));
                    acc[1] = A(acc[1] + A(w * A(f[1])));
                }
                g[(size_t(oy) * cx + ox) * 2] = -double(acc[0]);
                g[(size_t(oy) * cx + ox) * 2 + 1] = -double(acc[1]);
            }
    }
};

/* ------------------------------------------------------------------ */
/* a6: central-difference gradient, normal component zero on faces      */
/* (mia/3d/image.cc:347-466, mia/2d/image.cc:273-279,351-391)           */
/* ------------------------------------------------------------------ */
template <class T>
void gradient_nd(const T *img, T *g, int dim, int nx, int ny, int nz, const Pool &pool)
{
    if (dim == 2) nz = 1;
    const size_t sy = nx, sz = size_t(nx) * ny;
    pool.pfor(0, nz, [&](int zb, int ze) {
        for (int z = zb; z < ze; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) {
                    const size_t i = z * sz + y * sy + x;
                    T *o = g + i * dim;
                    o[0] = (x > 0 && x < nx - 1) ? T(0.5 * T(img[i + 1] - img[i - 1])) : T(0);
                    o[1] = (y > 0 && y < ny - 1) ? T(0.5 * T(img[i + sy] - img[i - sy])) : T(0);
                    if (dim == 3)
                        o[2] = (z > 0 && z < nz - 1) ? T(0.5 * T(img[i + sz] - img[i - sz])) : T(0);
                }
    });
}

/* ------------------------------------------------------------------ */
/* a7: SSD (mia/template/ssd.hh:54-194)                                 */
/* ------------------------------------------------------------------ */
template <class T>
double ssd_value(const T *a, const T *b, size_t n, bool norm)
{
    const double scale = norm ? 0.5 / n : 0.5;
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) {
        double d = double(a[i]) - double(b[i]);
        s = s + d * d;
    }
    return scale * s;
}

/* FEvalForce: force = grad * delta * scale, cost accumulated in the image
   type (float in the reference) */
template <class T>
double ssd_force(const T *a, const T *b, const T *grad, T *force, int dim, size_t n, bool norm)
{
    const T scale = norm ? T(1.0 / n) : T(1.0);
    T cost = T(0);
    for (size_t i = 0; i < n; ++i) {
        const T delta = T(a[i] - b[i]);
        for (int k = 0; k < dim; ++k) force[i * dim + k] = T(T(grad[i * dim + k] * delta) * scale);
        cost = T(cost + T(T(delta * delta) * scale));
    }
    return 0.5 * double(cost);
}

/* ------------------------------------------------------------------ */
/* a8: NCC (mia/3d/cost/ncc.cc:38-138, mia/core/nccsum.{hh,cc}, SSE2)    */
/* ------------------------------------------------------------------ */
struct NCCSums {
    double sa = 0, sb = 0, sa2 = 0, sb2 = 0, sab = 0, n = 0;
    void add(double a, double b) { sa += a; sb += b; sa2 += a * a; sb2 += b * b; sab += a * b; n += 1.0; }
    NCCSums &operator+=(const NCCSums &o)
    {
        sa += o.sa; sb += o.sb; sa2 += o.sa2; sb2 += o.sb2; sab += o.sab; n += o.n;
        return *this;
    }
    /* NCCSums::value (nccsum.cc:31-71) */
    double value() const
    {
        double result = 1.0;
        if (n > 0) {
            const double ma = sa / n, mb = sb / n;
            const double s2a = sa2 - sa * ma, s2b = sb2 - sb * mb;
            const double p0 = ma * mb, p1 = s2a * s2b;
            const double cab = sab - p0 * n;
            if (p1 > 1e-10) result = 1.0 - cab * cab / p1;
            else if (s2a < 1e-5 && s2b < 1e-5) result = 0.0;
        }
        return result;
    }
    /* NCCSums::get_grad_helper (nccsum.cc:73-120); helper = (2*cab/p1,
       cab/s2a, ma, mb) */
    double helper(double h[4]) const
    {
        double result = 1.0;
        h[0] = h[1] = h[2] = h[3] = 0.0;
        if (n > 0) {
            const double ma = sa / n, mb = sb / n;
            const double s2a = sa2 - sa * ma, s2b = sb2 - sb * mb;
            const double p0 = ma * mb, p1 = s2a * s2b;
            const double cab = sab - p0 * n;
            if (p1 > 1e-5) {
                result = 1.0 - cab * cab / p1;
                h[0] = 2.0 * (cab / p1);
                h[1] = cab / s2a;
                h[2] = ma;
                h[3] = mb;
            } else if (s2a < 1e-5 && s2b < 1e-5) {
                result = 0.0;
            }
        }
        return result;
    }
};

/* preduce over z-slabs (3D) or rows (2D), combined in slab order */
template <class T>
NCCSums ncc_sums(const T *a, const T *b, size_t n, size_t slab, const Pool &pool)
{
    const int nslab = int(n / slab);
    std::vector<NCCSums> part(std::max(1, pool.threads));
    std::vector<int> used(part.size(), 0);
    const int t = std::max(1, std::min(pool.threads, nslab));
    const int chunk = (nslab + t - 1) / t;
    pool.pfor(0, nslab, [&](int zb, int ze) {
        NCCSums s;
        for (int z = zb; z < ze; ++z)
            for (size_t i = size_t(z) * slab; i < size_t(z + 1) * slab; ++i) s.add(double(a[i]), double(b[i]));
        part[zb / chunk] = s;
    });
    NCCSums total;
    for (int k = 0; k < t; ++k) total += part[k];
    return total;
}

template <class T>
double ncc_force(const T *a, const T *b, const T *grad, T *force, int dim, size_t n,
                 const NCCSums &s)
{
    double h[4];
    const double v = s.helper(h);
    for (size_t i = 0; i < n; ++i) {
        const float sc = float(h[0] * (h[1] * (double(a[i]) - h[2]) - (double(b[i]) - h[3])));
        const T scale = T(sc);
        for (int k = 0; k < dim; ++k) force[i * dim + k] = T(scale * grad[i * dim + k]);
    }
    return v;
}

/* F64 NCC force keeps the scale in double */
template <>
double ncc_force<double>(const double *a, const double *b, const double *grad, double *force,
                         int dim, size_t n, const NCCSums &s)
{
    double h[4];
    const double v = s.helper(h);
    for (size_t i = 0; i < n; ++i) {
        const double scale = h[0] * (h[1] * (a[i] - h[2]) - (b[i] - h[3]));
        for (int k = 0; k < dim; ++k) force[i * dim + k] = scale * grad[i * dim + k];
    }
    return v;
}

/* ------------------------------------------------------------------ */
/* a11: divcurl matrices                                                */
/* ------------------------------------------------------------------ */
/* simpson() (mia/core/simpson.hh:36-51) and integrate2()
   (mia/core/splinekernel.cc:287-315) for the cubic kernel (radius 2) */
double integrate2(double s1, double s2, int d1, int d2, double n, double x0, double L)
{
    double sum = 0.0;
    x0 /= n;
    L /= n;
    const double r = 2.0;
    double a = s1 - r, b = s1 + r;
    if (a < s2 - r) a = s2 - r;
    if (a < x0) a = x0;
    if (b > s2 + r) b = s2 + r;
    if (b > L) b = L;
    if (b <= a) return sum;
    const size_t intervals = size_t(8 * (b - a));
    auto f = [&](double x) { return bspline3_at(x - s1, d1) * bspline3_at(x - s2, d2); };
    const double dx = (b - a) / intervals;
    sum = 0.5 * (f(a) + f(b));
    double x = a + dx;
    for (size_t i = 1; i < intervals; ++i, x += dx) sum += f(x);
    x = a + .5 * dx;
    for (size_t i = 0; i < intervals; ++i, x += dx) sum += 2 * f(x);
    sum = sum * dx / 3.0;
    return sum * n;
}

/* CIntegralCache2 (mia/3d/ppmatrix.cc:121-165), including the shadowed
   `result` that makes the first lookup of each delta return 0 */
struct IntegralCache2 {
    int shift = 4, d1, d2;
    std::vector<bool> valid;
    std::vector<double> values;
    IntegralCache2(int a, int b) : d1(a), d2(b), valid(9, false), values(9, 0.0) {}
    double get(int delta)
    {
        delta += shift;
        if (delta < 0 || delta >= int(valid.size())) return 0;
        double result = 0;
        if (valid[delta])
            result = values[delta];
        else {
            values[delta] = integrate2(shift, delta, d1, d2, 1, 0, 2 * shift);
            valid[delta] = true;
        }
        return result;
    }
};

struct Cell3 { double vxx = 0, vxz = 0, vxy = 0, vyy = 0, vyz = 0, vzz = 0; };

/* C3DPPDivcurlMatrixImpl (mia/3d/ppmatrix.cc:175-599) */
struct PPMatrix3 {
    int nx, ny, nz, ks = 4;
    std::vector<Cell3> P;   /* 9x9x9, index (x + 9*(y + 9*z)) */

    void reset(const int csize[3], const float range[3], double wdiv, double wrot)
    {
        nx = csize[0]; ny = csize[1]; nz = csize[2];
        P.assign(9 * 9 * 9, Cell3());
        const float h1x = float(csize[0] - 1) / range[0];
        const float h1y = float(csize[1] - 1) / range[1];
        const float h1z = float(csize[2] - 1) / range[2];
        const float h2x = h1x * h1x, h2y = h1y * h1y, h2z = h1z * h1z;
        const float h3x = h1x * h2x, h3y = h1y * h2y, h3z = h1z * h2z;
        const float h4x = h1x * h3x, h4y = h1y * h3y, h4z = h1z * h3z;
        const double gs = 1.0 / double(float(h1x * h1y) * h1z);
        IntegralCache2 rc00(0, 0), rc11(1, 1), rc22(2, 2), rc21(2, 1), rc12(1, 2), rc01(0, 1), rc10(1, 0);
        const double wsum = wdiv + wrot;
        const double wdelta = 2 * (wdiv - wrot);
        size_t pi = 0;
        for (int z = -ks; z <= ks; ++z) {
            const double r00z = rc00.get(z);
            const double r01z = h1z * rc01.get(z);
            const double r11z = h2z * rc11.get(z);
            const double r12z = h3z * rc12.get(z);
            const double r22z = h4z * rc22.get(z);
            for (int y = -ks; y <= ks; ++y) {
                const double r00y = rc00.get(y);
                const double r01y = h1y * rc01.get(y);
                const double r10y = h1y * rc10.get(y);
                const double r11y = h2y * rc11.get(y);
                const double r12y = h3y * rc12.get(y);
                const double r21y = h3y * rc21.get(y);
                const double r22y = h4y * rc22.get(y);
                for (int x = -ks; x <= ks; ++x, ++pi) {
                    const double r00x = rc00.get(x);
                    const double r01x = h1x * rc01.get(x);
                    const double r10x = h1x * rc10.get(x);
                    const double r11x = h2x * rc11.get(x);
                    const double r21x = h3x * rc21.get(x);
                    const double r22x = h4x * rc22.get(x);
                    Cell3 c;
                    const double r200200 = r22x * r00y * r00z;
                    const double r020020 = r00x * r22y * r00z;
                    const double r002002 = r00x * r00y * r22z;
                    const double r110110 = r11x * r11y * r00z;
                    const double r101101 = r11x * r00y * r11z;
                    const double r011011 = r00x * r11y * r11z;
                    c.vxx = gs * (r002002 * wrot + r011011 * 2.0 * wrot + r020020 * wrot +
                                  r101101 * wsum + r110110 * wsum + r200200 * wdiv);
                    c.vyy = gs * (r002002 * wrot + r011011 * wsum + r020020 * wdiv +
                                  r101101 * 2 * wrot + r110110 * wsum + r200200 * wrot);
                    c.vzz = gs * (r002002 * wdiv + r011011 * wsum + r020020 * wrot +
                                  r101101 * wsum + r110110 * wrot * 2 + r200200 * wrot);
                    if (wdelta != 0.0) {
                        c.vxy = gs * wdelta * (r21x * r01y * r00z + r10x * r12y * r00z + r01x * r10y * r11z);
                        c.vxz = gs * wdelta * (r21x * r00y * r01z + r10x * r11y * r01z + r10x * r00y * r12z);
                        c.vyz = gs * wdelta * (r11x * r10y * r01z + r00x * r21y * r01z + r00x * r10y * r12z);
                    }
                    P[pi] = c;
                }
            }
        }
    }
    const Cell3 &cell(int dx, int dy, int dz) const { return P[dx + 9 * (dy + 9 * dz)]; }

    /* EvaluateGradientAndValue, SSE2 order (ppmatrix.cc:363-489, 578-587) */
    double evaluate(const double *c, double *g, const Pool &pool) const
    {
        std::vector<double> values(nz, 0.0);
        pool.pfor(0, nz, [&](int zb, int ze) {
            for (int zi = zb; zi < ze; ++zi) {
                double res[6] = {0, 0, 0, 0, 0, 0};
                for (int yi = 0; yi < ny; ++yi)
                    for (int xi = 0; xi < nx; ++xi) {
                        const double *ci = &c[((size_t(zi) * ny + yi) * nx + xi) * 3];
                        double gg[3] = {0, 0, 0};
                        for (int zj = std::max(0, zi - ks); zj < std::min(zi + ks, nz); ++zj) {
                            const int dz = zi - zj + ks;
                            for (int yj = std::max(0, yi - ks); yj < std::min(yi + ks, ny); ++yj) {
                                const int dy = yi - yj + ks;
                                const int xs = std::max(0, xi - ks), xe = std::min(xi + ks, nx);
                                for (int xj = xs; xj < xe; ++xj) {
                                    const Cell3 &p = cell(xi - xj + ks, dy, dz);
                                    const double *cj = &c[((size_t(zj) * ny + yj) * nx + xj) * 3];
                                    const double ax = p.vxx * cj[0], az = p.vxz * cj[0];
                                    const double bxy = p.vxy * cj[1], byy = p.vyy * cj[1];
                                    const double cyz = p.vyz * cj[2], czz = p.vzz * cj[2];
                                    res[0] += ci[0] * ax;
                                    res[1] += ci[0] * bxy;
                                    res[2] += ci[1] * byy;
                                    res[3] += ci[1] * cyz;
                                    res[4] += ci[2] * czz;
                                    res[5] += ci[2] * az;
                                    gg[0] += cj[2] * p.vxz + (2.0 * ax + bxy);
                                    gg[1] += cj[0] * p.vxy + (2.0 * byy + cyz);
                                    gg[2] += cj[1] * p.vyz + (2.0 * czz + az);
                                }
                            }
                        }
                        if (g) {
                            double *o = &g[((size_t(zi) * ny + yi) * nx + xi) * 3];
                            o[0] = gg[0]; o[1] = gg[1]; o[2] = gg[2];
                        }
                    }
                values[zi] = res[0] + res[1] + res[2] + res[3] + res[4] + res[5];
            }
        });
        double v = 0.0;
        for (int z = 0; z < nz; ++z) v += values[z];
        return v;
    }

    /* multiply (ppmatrix.cc:292-361) */
    double multiply(const double *c, bool equal_w) const
    {
        double r1 = 0, r2 = 0, r3 = 0, r4 = 0, r5 = 0, r6 = 0;
        for (int zi = 0; zi < nz; ++zi)
            for (int yi = 0; yi < ny; ++yi)
                for (int xi = 0; xi < nx; ++xi) {
                    const double *ci = &c[((size_t(zi) * ny + yi) * nx + xi) * 3];
                    for (int zj = std::max(0, zi - ks); zj < std::min(zi + ks, nz); ++zj) {
                        const int dz = zi - zj + ks;
                        for (int yj = std::max(0, yi - ks); yj < std::min(yi + ks, ny); ++yj) {
                            const int dy = yi - yj + ks;
                            const int xs = std::max(0, xi - ks), xe = std::min(xi + ks, nx);
                            for (int xj = xs; xj < xe; ++xj) {
                                const Cell3 &p = cell(xi - xj + ks, dy, dz);
                                const double *cj = &c[((size_t(zj) * ny + yj) * nx + xj) * 3];
                                r1 += ci[0] * cj[0] * p.vxx;
                                r2 += ci[1] * cj[1] * p.vyy;
                                r3 += ci[2] * cj[2] * p.vzz;
                                if (!equal_w) {
                                    r4 += ci[0] * cj[1] * p.vxy;
                                    r5 += ci[0] * cj[2] * p.vxz;
                                    r6 += ci[1] * cj[2] * p.vyz;
                                }
                            }
                        }
                    }
                }
        return r1 + r2 + r3 + r4 + r5 + r6;
    }
};

/* CIntegralCache (mia/2d/ppmatrix.cc:100-172): boundary-clipped integrals
   cached by (skip, delta) */
struct IntegralCache {
    int max_skip = 4, row_length = 4, hr = 2;
    std::map<int, double> values;
    double get(int s1, int s2, int d1, int d2, int range)
    {
        bool swapped = false;
        if (s2 < s1) { swapped = true; std::swap(s1, s2); }
        int delta = s2 - s1;
        if (delta >= row_length) return 0.0;
        int skip = 0;
        const int dlow = hr - s1;
        if (dlow > 0) {
            skip = s2 - hr;
            if (skip > 0) skip = 0;
        } else {
            const int dhigh = hr + s2 - range;
            if (dhigh > 0) skip = hr + s1 - range;
            if (skip < 0) skip = 0;
        }
        if (std::abs(skip) >= max_skip) return 0.0;
        if (swapped) { delta = -delta; std::swap(s1, s2); }
        const int index = skip * 2 * row_length + delta + row_length;
        auto pv = values.find(index);
        if (pv != values.end()) return pv->second;
        double r = values[index] = integrate2(s1, s2, d1, d2, 1, 0, range);
        return r;
    }
};

struct Cell2 { double vx, vy, v12; size_t i, j; };

/* C2DPPDivcurlMatrixImpl (mia/2d/ppmatrix.cc:182-352) */
struct PPMatrix2 {
    int nx, ny;
    std::vector<Cell2> P;
    void reset(const int csize[2], const float range[2], double wd, double wr)
    {
        nx = csize[0]; ny = csize[1];
        P.clear();
        const float h1x = float(csize[0] - 1) / range[0];
        const float h1y = float(csize[1] - 1) / range[1];
        const double gs = 1.0 / double(h1x * h1y);
        const float h2x = h1x * h1x, h2y = h1y * h1y;
        const float h3x = h1x * h2x, h3y = h1y * h2y;
        const float h4x = h1x * h3x, h4y = h1y * h3y;
        const int kr = 4;
        IntegralCache rc22, rc21, rc01, rc12, rc10, rc00, rc11;
        for (int l = 0; l < ny; ++l)
            for (int n = std::max(0, l - kr); n < std::min(l + kr, ny); ++n) {
                const double r00y = rc00.get(l, n, 0, 0, ny);
                const double r01y = h1y * rc01.get(l, n, 0, 1, ny);
                const double r11y = h2y * rc11.get(l, n, 1, 1, ny);
                const double r21y = h3y * rc21.get(l, n, 2, 1, ny);
                const double r22y = h4y * rc22.get(l, n, 2, 2, ny);
                for (int k = 0; k < nx; ++k)
                    for (int m = std::max(0, k - kr); m < std::min(k + kr, nx); ++m) {
                        const double r00x = rc00.get(k, m, 0, 0, nx);
                        const double r01x = h1x * rc01.get(k, m, 0, 1, nx);
                        const double r11x = h2x * rc11.get(k, m, 1, 1, nx);
                        const double r21x = h3x * rc21.get(k, m, 2, 1, nx);
                        const double r22x = h4x * rc22.get(k, m, 2, 2, nx);
                        Cell2 c;
                        c.vx = gs * (wd * (r22x * r00y + r11x * r11y) + wr * (r11x * r11y + r00x * r22y));
                        c.v12 = 2 * gs * (wd - wr) * (r21x * r01y + r01x * r21y);
                        c.vy = gs * (wd * (r00x * r22y + r11x * r11y) + wr * (r22x * r00y + r11x * r11y));
                        c.i = k + size_t(l) * nx;
                        c.j = m + size_t(n) * nx;
                        if (c.vx != 0.0 || c.v12 != 0.0 || c.vy != 0.0) P.push_back(c);
                    }
            }
    }
    /* evaluate (float coefficients, ppmatrix.cc:328-352); gradient += */
    double evaluate(const double *c, double *g) const
    {
        double r1 = 0, r2 = 0, r3 = 0;
        for (const Cell2 &p : P) {
            const double *ci = &c[p.i * 2], *cj = &c[p.j * 2];
            const double a = cj[0] * p.vx, b = cj[1] * p.vy;
            const double cx = cj[0] * p.v12, cy = cj[1] * p.v12;
            if (g) {
                g[2 * p.i] += a + a + cy;
                g[2 * p.i + 1] += b + b + cx;
            }
            r1 += ci[0] * a;
            r2 += ci[0] * cy;
            r3 += ci[1] * b;
        }
        return r1 + r2 + r3;
    }
    /* multiply (ppmatrix.cc:245-262) */
    double multiply(const double *c) const
    {
        double r1 = 0, r2 = 0, r3 = 0;
        for (const Cell2 &p : P) {
            const double *ci = &c[p.i * 2], *cj = &c[p.j * 2];
            r1 += ci[0] * cj[0] * p.vx;
            r2 += ci[0] * cj[1] * p.v12;
            r3 += ci[1] * cj[1] * p.vy;
        }
        return r1 + r2 + r3;
    }
};

/* ------------------------------------------------------------------ */
/* a10/a13: one level = spline transform + image full cost + penalty    */
/* ------------------------------------------------------------------ */
struct LevelBase {
    OrcLevelDesc d;
    Pool pool;
    virtual ~LevelBase() {}
    virtual void set_images(const float *src, const float *ref) = 0;
    virtual double evaluate(const double *p, double *gi, double *gp, double *ci, double *cp) = 0;
    virtual double value(const double *p, double *ci, double *cp) = 0;
    virtual void warp(const double *p, float *out) = 0;
    virtual void displacement(const double *p, float *u) = 0;
    virtual void force(const double *p, float *f) = 0;
    virtual void translate(const float *f, double *g) = 0;
    virtual int csize(int cs[3]) const = 0;
};

template <class P>
struct Level : LevelBase {
    typedef typename P::Img T;
    Spline<P> tr;
    std::vector<T> src, ref;
    Interp<P> interp;
    PPMatrix3 pp3;
    PPMatrix2 pp2;
    size_t N = 0;
    int dim = 3;
    bool prefilter_each_eval = true;   /* the reference builds a new
                                          interpolator per warp
                                          (mia/3d/transform.cc:306) */

    void init(const OrcLevelDesc &desc)
    {
        d = desc;
        dim = d.dim;
        pool.threads = std::max(1, d.threads);
        int cs[3] = {1, 1, 1};
        for (int a = 0; a < dim; ++a)
            cs[a] = d.csize[a] > 0 ? d.csize[a] : Spline<P>::csize_from_rate(d.size[a], d.rate[a]);
        tr.init(dim, d.size, cs);
        N = size_t(tr.n[0]) * tr.n[1] * tr.n[2];
        if (d.has_penalty) {
            float range[3] = {float(d.size[0]), float(d.size[1]), float(dim == 3 ? d.size[2] : 1)};
            if (dim == 3) pp3.reset(cs, range, d.pen_div, d.pen_curl);
            else pp2.reset(cs, range, d.pen_div, d.pen_curl);
        }
    }
    int csize(int cs[3]) const override
    {
        for (int a = 0; a < 3; ++a) cs[a] = tr.nc[a];
        return int(tr.ncoef() * dim);
    }
    void set_images(const float *s, const float *r) override
    {
        src.assign(s, s + N);
        ref.assign(r, r + N);
        interp.init(src.data(), dim, tr.n[0], tr.n[1], tr.n[2], pool);
    }

    void disp(std::vector<T> &u)
    {
        if (dim == 3) tr.displacement3(u, pool);
        else tr.displacement2(u, pool);
    }

    /* t(*src): C3DTransformation::do_transform / F3DTransformer
       (mia/3d/transform.cc:280-353; 2D transform.cc:258-293) */
    void do_warp(std::vector<T> &w)
    {
        if (prefilter_each_eval) interp.init(src.data(), dim, tr.n[0], tr.n[1], tr.n[2], pool);
        std::vector<T> u;
        disp(u);
        w.assign(N, T(0));
        const int nx = tr.n[0], ny = tr.n[1], nz = tr.n[2];
        typedef typename P::Crd Cd;
        pool.pfor(0, nz, [&](int zb, int ze) {
            for (int z = zb; z < ze; ++z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x) {
                        const size_t i = (size_t(z) * ny + y) * nx + x;
                        if (dim == 3) {
                            const Cd gx = Cd(Cd(x) - Cd(u[i * 3]));
                            const Cd gy = Cd(Cd(y) - Cd(u[i * 3 + 1]));
                            const Cd gz = Cd(Cd(z) - Cd(u[i * 3 + 2]));
                            w[i] = interp(double(gx), double(gy), double(gz));
                        } else {
                            const Cd gx = Cd(Cd(x) - Cd(u[i * 2]));
                            const Cd gy = Cd(Cd(y) - Cd(u[i * 2 + 1]));
                            w[i] = interp(double(gx), double(gy));
                        }
                    }
        });
    }

    double cost_force(const std::vector<T> &w, std::vector<T> &f)
    {
        std::vector<T> g(N * dim);
        gradient_nd(w.data(), g.data(), dim, tr.n[0], tr.n[1], tr.n[2], pool);
        f.assign(N * dim, T(0));
        if (d.cost == ORC_COST_SSD)
            return ssd_force(w.data(), ref.data(), g.data(), f.data(), dim, N, d.ssd_norm != 0);
        const size_t slab = (dim == 3) ? size_t(tr.n[0]) * tr.n[1] : size_t(tr.n[0]);
        NCCSums s = ncc_sums(w.data(), ref.data(), N, slab, pool);
        return ncc_force(w.data(), ref.data(), g.data(), f.data(), dim, N, s);
    }

    double cost_value(const std::vector<T> &w)
    {
        if (d.cost == ORC_COST_SSD) return ssd_value(w.data(), ref.data(), N, d.ssd_norm != 0);
        const size_t slab = (dim == 3) ? size_t(tr.n[0]) * tr.n[1] : size_t(tr.n[0]);
        return ncc_sums(w.data(), ref.data(), N, slab, pool).value();
    }

    double pen_weight() const
    {
        double prod = d.size[0] * double(d.size[1]) * (dim == 3 ? d.size[2] : 1);
        return d.pen_norm ? d.pen_weight / double(float(prod)) : d.pen_weight;
    }

    /* coefficients as the penalty sees them: the transform's stored vectors */
    std::vector<double> coef_d() const
    {
        return std::vector<double>(tr.coef.begin(), tr.coef.end());
    }

    double evaluate(const double *p, double *gi, double *gp, double *ci, double *cp) override
    {
        tr.set_params(p);
        const size_t m = tr.ncoef() * dim;
        /* C3DImageFullCost::do_evaluate (mia/3d/fullcost/image.cc:67-78),
           C2DImageFullCost::do_evaluate (mia/2d/fullcost/image.cc:81-105) */
        std::vector<T> w, f;
        do_warp(w);
        double c = cost_force(w, f);
        std::vector<double> g(m, 0.0);
        if (dim == 3) tr.translate3(f.data(), g.data(), pool);
        else tr.translate2(f.data(), g.data(), pool);
        if (dim == 3) c = cost_value(w);
        /* TFullCost::evaluate weight (mia/template/fullcost.cxx:37-45) */
        const double cw = d.cost_weight;
        const double cost_img = cw * c;
        if (gi)
            for (size_t k = 0; k < m; ++k) gi[k] = cw * g[k];
        /* penalty value_and_gradient (mia/3d/splinetransformpenalty.cc:60-71) */
        double cost_pen = 0.0;
        if (d.has_penalty) {
            std::vector<double> cc = coef_d(), pg(m, 0.0);
            const double w8 = pen_weight();
            double v = (dim == 3) ? pp3.evaluate(cc.data(), pg.data(), pool) : pp2.evaluate(cc.data(), pg.data());
            cost_pen = w8 * v;
            if (gp)
                for (size_t k = 0; k < m; ++k) gp[k] = -w8 * pg[k];
        } else if (gp) {
            std::fill(gp, gp + m, 0.0);
        }
        if (ci) *ci = cost_img;
        if (cp) *cp = cost_pen;
        return cost_img + cost_pen;
    }

    double value(const double *p, double *ci, double *cp) override
    {
        tr.set_params(p);
        std::vector<T> w;
        do_warp(w);
        const double cost_img = d.cost_weight * cost_value(w);
        double cost_pen = 0.0;
        if (d.has_penalty) {
            std::vector<double> cc = coef_d();
            const double w8 = pen_weight();
            const double v = (dim == 3) ? pp3.multiply(cc.data(), d.pen_div == d.pen_curl) : pp2.multiply(cc.data());
            cost_pen = w8 * v;
        }
        if (ci) *ci = cost_img;
        if (cp) *cp = cost_pen;
        return cost_img + cost_pen;
    }

    void warp(const double *p, float *out) override
    {
        tr.set_params(p);
        std::vector<T> w;
        do_warp(w);
        for (size_t i = 0; i < N; ++i) out[i] = float(w[i]);
    }
    void displacement(const double *p, float *out) override
    {
        tr.set_params(p);
        std::vector<T> u;
        disp(u);
        for (size_t i = 0; i < N * dim; ++i) out[i] = float(u[i]);
    }
    void force(const double *p, float *out) override
    {
        tr.set_params(p);
        std::vector<T> w, f;
        do_warp(w);
        cost_force(w, f);
        for (size_t i = 0; i < N * dim; ++i) out[i] = float(f[i]);
    }
    void translate(const float *f, double *g) override
    {
        std::vector<T> ff(f, f + N * dim);
        if (dim == 3) tr.translate3(ff.data(), g, pool);
        else tr.translate2(ff.data(), g, pool);
    }
};

}  // namespace

struct OrcLevel {
    std::unique_ptr<LevelBase> impl;
};

extern "C" {

int orc_fastfloor(double x) { return fastfloor(x); }
void orc_bspline3_weights(double x, double w[4]) { weights3(x, w); }
void orc_bspline3_dweights(double x, double w[4]) { dweights3(x, w); }
/* CBSplineKernel3::get_derivative_weights(x, w, degree) (bspline.cc:295-326) */
void orc_bspline3_deriv_weights(double x, int degree, double w[4])
{
    switch (degree) {
    case 0: weights3(x, w); break;
    case 1: dweights3(x, w); break;
    case 2: w[3] = x; w[0] = 1 - x; w[2] = 1 - 3.0 * x; w[1] = 3 * x - 2; break;
    case 3: w[3] = 1.0; w[0] = -1.0; w[2] = -3.0; w[1] = 3.0; break;
    default: w[0] = w[1] = w[2] = w[3] = 0.0;
    }
}
double orc_bspline3_at(double x, int degree) { return bspline3_at(x, degree); }
int orc_mirror_fold(int index, int width) { return mirror_fold(index, width); }
void orc_filter_line(double *coeff, int n) { filter_line(coeff, n); }

void orc_prefilter(const float *in, float *out, int dim, const int size[3])
{
    Pool pool;
    const int nz = dim == 3 ? size[2] : 1;
    std::copy(in, in + size_t(size[0]) * size[1] * nz, out);
    prefilter_nd(out, size[0], size[1], nz, pool);
}

void orc_prefilter_vec_d(const double *in, double *out, int ncomp, int dim, const int size[3])
{
    Pool pool;
    const int nz = dim == 3 ? size[2] : 1;
    const size_t n = size_t(size[0]) * size[1] * nz;
    std::vector<double> comp(n);
    for (int c = 0; c < ncomp; ++c) {
        for (size_t i = 0; i < n; ++i) comp[i] = in[i * ncomp + c];
        prefilter_nd(comp.data(), size[0], size[1], nz, pool);
        for (size_t i = 0; i < n; ++i) out[i * ncomp + c] = comp[i];
    }
}

double orc_simpson_integrate2(double s1, double s2, int deg1, int deg2, double x0, double L)
{
    return integrate2(s1, s2, deg1, deg2, 1, x0, L);
}

void orc_divcurl_table3(const int csize[3], const float range[3], double wdiv, double wrot, double *out)
{
    PPMatrix3 m;
    m.reset(csize, range, wdiv, wrot);
    for (size_t c = 0; c < m.P.size(); ++c) {
        const Cell3 &p = m.P[c];
        double *o = out + c * 6;
        o[0] = p.vxx; o[1] = p.vxy; o[2] = p.vyy; o[3] = p.vyz; o[4] = p.vzz; o[5] = p.vxz;
    }
}

size_t orc_divcurl_cells2(const int csize[2], const float range[2], double wd, double wr, int *i, int *j,
                          double *v, size_t cap)
{
    PPMatrix2 m;
    m.reset(csize, range, wd, wr);
    /* the cells grouped by row i in list order, as the reference's
       evaluation visits them row by row */
    std::vector<size_t> order(m.P.size());
    for (size_t k = 0; k < order.size(); ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return m.P[a].i < m.P[b].i; });
    for (size_t k = 0; k < order.size() && k < cap; ++k) {
        const Cell2 &p = m.P[order[k]];
        i[k] = int(p.i);
        j[k] = int(p.j);
        v[3 * k] = p.vx; v[3 * k + 1] = p.vy; v[3 * k + 2] = p.v12;
    }
    return m.P.size();
}

void orc_gradient(const float *img, float *grad, int dim, const int size[3])
{
    Pool pool;
    gradient_nd(img, grad, dim, size[0], size[1], dim == 3 ? size[2] : 1, pool);
}

double orc_ssd_value(const float *a, const float *b, size_t n, int norm)
{
    return ssd_value(a, b, n, norm != 0);
}

double orc_ssd_force(const float *a, const float *b, float *force, int dim, const int size[3], int norm)
{
    Pool pool;
    const int nz = dim == 3 ? size[2] : 1;
    const size_t n = size_t(size[0]) * size[1] * nz;
    std::vector<float> g(n * dim);
    gradient_nd(a, g.data(), dim, size[0], size[1], nz, pool);
    return ssd_force(a, b, g.data(), force, dim, n, norm != 0);
}

void orc_ncc_sums(const float *a, const float *b, size_t n, double s[6])
{
    NCCSums x;
    for (size_t i = 0; i < n; ++i) x.add(a[i], b[i]);
    s[0] = x.sa; s[1] = x.sb; s[2] = x.sa2; s[3] = x.sb2; s[4] = x.sab; s[5] = x.n;
}

double orc_ncc_value(const float *a, const float *b, size_t n)
{
    NCCSums x;
    for (size_t i = 0; i < n; ++i) x.add(a[i], b[i]);
    return x.value();
}

double orc_ncc_force(const float *a, const float *b, float *force, int dim, const int size[3])
{
    Pool pool;
    const int nz = dim == 3 ? size[2] : 1;
    const size_t n = size_t(size[0]) * size[1] * nz;
    std::vector<float> g(n * dim);
    gradient_nd(a, g.data(), dim, size[0], size[1], nz, pool);
    NCCSums x;
    for (size_t i = 0; i < n; ++i) x.add(a[i], b[i]);
    return ncc_force(a, b, g.data(), force, dim, n, x);
}

double orc_divcurl_matrix(int dim, const int csize[3], const float range[3], double wdiv,
                          double wrot, const double *coeffs, double *grad, int as_float, int mode)
{
    Pool pool;
    const size_t nn = size_t(csize[0]) * csize[1] * (dim == 3 ? csize[2] : 1);
    std::vector<double> c(coeffs, coeffs + nn * dim);
    if (as_float)
        for (auto &v : c) v = double(float(v));
    if (dim == 3) {
        PPMatrix3 m;
        m.reset(csize, range, wdiv, wrot);
        if (mode == 1) return m.multiply(c.data(), wdiv == wrot);
        return m.evaluate(c.data(), grad, pool);
    }
    PPMatrix2 m;
    m.reset(csize, range, wdiv, wrot);
    if (mode == 1) return m.multiply(c.data());
    if (grad) std::fill(grad, grad + nn * 2, 0.0);
    return m.evaluate(c.data(), grad);
}

OrcLevel *orc_level_create(const OrcLevelDesc *desc)
{
    OrcLevel *l = new OrcLevel;
    if (desc->precision == ORC_PREC_F64) {
        auto *p = new Level<F64P>();
        p->init(*desc);
        l->impl.reset(p);
    } else {
        auto *p = new Level<RefP>();
        p->init(*desc);
        l->impl.reset(p);
    }
    return l;
}

void orc_level_destroy(OrcLevel *lvl) { delete lvl; }
int orc_level_csize(const OrcLevel *lvl, int csize[3]) { return lvl->impl->csize(csize); }
void orc_level_set_images(OrcLevel *lvl, const float *src, const float *ref) { lvl->impl->set_images(src, ref); }
double orc_level_evaluate(OrcLevel *lvl, const double *params, double *g_img, double *g_pen,
                          double *cost_img, double *cost_pen)
{
    return lvl->impl->evaluate(params, g_img, g_pen, cost_img, cost_pen);
}
double orc_level_value(OrcLevel *lvl, const double *params, double *cost_img, double *cost_pen)
{
    return lvl->impl->value(params, cost_img, cost_pen);
}
void orc_level_warp(OrcLevel *lvl, const double *params, float *out) { lvl->impl->warp(params, out); }
void orc_level_displacement(OrcLevel *lvl, const double *params, float *u) { lvl->impl->displacement(params, u); }
void orc_level_force(OrcLevel *lvl, const double *params, float *force) { lvl->impl->force(params, force); }
void orc_level_translate(OrcLevel *lvl, const float *force, double *g) { lvl->impl->translate(force, g); }

}  // extern "C"

/* ===================================================================== */
/* registration driver (TNonrigidRegisterImpl::run and its helpers)       */
/* ===================================================================== */
namespace {

/* Binomial "gauss:w=" kernel (mia/core/spacialkernel/gauss.cc:27-57) and
   its half-sample symmetric application (gauss.cc:72-137), restated as
   out[i] = sum_j mask[j] * in[reflect(i - w + j)]. */
std::vector<double> gauss_mask(int w)
{
    const int n = 2 * w + 1;
    std::vector<double> k(n, 0.0), tmp(n, 0.0);
    k[0] = 1.0;
    if (n > 1) k[1] = 1.0;
    for (int i = 2; i < n; ++i) {
        k[i] = 1.0;
        for (int j = 1; j < i; ++j) tmp[j] = k[j - 1] + k[j];
        for (int j = 1; j < i; ++j) k[j] = tmp[j];
    }
    const double norm = std::pow(2.0, n - 1);
    for (double &v : k) v /= norm;
    return k;
}

/* C1DScalar (mia/core/scaler1d.cc): copy when the size is kept, else
   gauss smoothing, mirror prefilter and cubic B-spline sampling at i*dx */
void scale_line(const std::vector<double> &in, std::vector<double> &out)
{
    const int n = int(in.size()), m = int(out.size());
    if (n == m) {
        out = in;
        return;
    }
    const double scale = double(m - 1) / double(n - 1);
    const int w = int(std::floor(1.0 / scale + 0.5));
    const std::vector<double> mask = gauss_mask(w);
    std::vector<double> c(n, 0.0);
    for (int i = 0; i < n; ++i) {
        double h = 0.0;
        for (int j = 0; j < 2 * w + 1; ++j) {
            int k = i - w + j;
            if (k < 0) k = -k - 1;
            if (k >= n) k = 2 * n - 1 - k;
            h += mask[j] * in[k];
        }
        c[i] = h;
    }
    filter_line(c.data(), n);
    const double dx = 1.0 / scale;
    for (int i = 0; i < m; ++i) {
        const double x = double(i) * dx;
        const int ix = fastfloor(x);
        double wt[4];
        weights3(x - ix, wt);
        int id[4];
        for (int q = 0; q < 4; ++q) id[q] = ix - 1 + q;
        if (id[0] < 0 || id[3] >= n)
            for (int q = 0; q < 4; ++q) id[q] = mirror_fold(id[q], n);
        double v = 0.0;
        for (int q = 0; q < 4; ++q) v += wt[q] * c[id[q]];
        out[i] = v;
    }
}

/* C3DScale::operator() / do_scale (mia/3d/filter/scale.cc:30-118),
   C2DScale (mia/2d/filter/scale.cc:50-90): x, y, z passes over double
   temporaries, float result */
void scale_image_cpu(const float *in, int dim, const int is[3], float *out, const int os[3])
{
    const int nx = is[0], ny = is[1], nz = dim == 3 ? is[2] : 1;
    const int mx = os[0], my = os[1], mz = dim == 3 ? os[2] : 1;
    if (nx == mx && ny == my && nz == mz) {
        std::copy(in, in + size_t(nx) * ny * nz, out);
        return;
    }
    std::vector<double> t1(size_t(mx) * ny * nz), t2(size_t(mx) * my * nz);
    std::vector<double> a, b;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            a.assign(in + (size_t(z) * ny + y) * nx, in + (size_t(z) * ny + y + 1) * nx);
            b.assign(mx, 0.0);
            scale_line(a, b);
            std::copy(b.begin(), b.end(), t1.begin() + (size_t(z) * ny + y) * mx);
        }
    for (int z = 0; z < nz; ++z)
        for (int x = 0; x < mx; ++x) {
            a.resize(ny);
            for (int y = 0; y < ny; ++y) a[y] = t1[(size_t(z) * ny + y) * mx + x];
            b.assign(my, 0.0);
            scale_line(a, b);
            for (int y = 0; y < my; ++y) t2[(size_t(z) * my + y) * mx + x] = b[y];
        }
    if (dim == 2) {
        for (size_t i = 0; i < size_t(mx) * my; ++i) out[i] = float(t2[i]);
        return;
    }
    for (int y = 0; y < my; ++y)
        for (int x = 0; x < mx; ++x) {
            a.resize(nz);
            for (int z = 0; z < nz; ++z) a[z] = t2[(size_t(z) * my + y) * mx + x];
            b.assign(mz, 0.0);
            scale_line(a, b);
            for (int z = 0; z < mz; ++z) out[(size_t(z) * my + y) * mx + x] = float(b[z]);
        }
}

/* FScaleFilterCreator + the "convert:repn=float,map=linear" filter
   (mia/template/nonrigidregister.cxx:147-184, mia/template/convert.cxx:
   78-92): a and b are written with the stream's default precision */
bool normalize_cpu(const float *s, const float *r, size_t n, float *so, float *ro, double *mean_o,
                   double *sigma_o)
{
    double sum = 0.0, sum2 = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const double fa = s[i], fb = r[i];
        sum += fa + fb;
        sum2 += fa * fa + fb * fb;
    }
    const double nn = 2.0 * double(n);
    const double mean = sum / nn;
    const double sigma = std::sqrt((sum2 - sum * sum / nn) / (nn - 1));
    if (mean_o) *mean_o = mean;
    if (sigma_o) *sigma_o = sigma;
    if (sigma == 0.0) return false;
    char buf[64];
    snprintf(buf, sizeof buf, "%g", -mean / sigma);
    const long double b = std::strtold(buf, nullptr);
    snprintf(buf, sizeof buf, "%g", 1.0 / sigma);
    const long double a = std::strtold(buf, nullptr);
    for (size_t i = 0; i < n; ++i) {
        so[i] = float(a * (long double)s[i] + b);
        ro[i] = float(a * (long double)r[i] + b);
    }
    return true;
}

/* refine(): grid size (mia/3d/transform/spline.cc:363-364) */
int refine_csize_cpu(int size, float rate) { return int((float(size) + rate - 1.0f) / rate) + 2; }

/* refine() interpolation (spline.cc:360-396, 2D spline.cc:318-353) with a
   vector-valued T3DConvoluteInterpolator: double coefficients, clamp to the
   componentwise min/max (min set to 0 only if all components are > 0) */
bool refine_cpu(int dim, const int nco[3], const int ncn[3], std::vector<double> &p)
{
    bool any = false;
    for (int k = 0; k < dim; ++k)
        if (ncn[k] > nco[k]) any = true;
    if (!any) return false;
    const int ox = nco[0], oy = nco[1], oz = dim == 3 ? nco[2] : 1;
    const size_t no = size_t(ox) * oy * oz;
    std::vector<double> comp(no);
    std::vector<std::vector<double>> coef(dim);
    float mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    Pool pool;
    for (int c = 0; c < dim; ++c) {
        for (size_t i = 0; i < no; ++i) comp[i] = double(float(p[i * dim + c]));
        mn[c] = mx[c] = float(comp[0]);
        for (size_t i = 1; i < no; ++i) {
            mn[c] = std::min(mn[c], float(comp[i]));
            mx[c] = std::max(mx[c], float(comp[i]));
        }
        prefilter_nd(comp.data(), ox, oy, oz, pool);
        coef[c] = comp;
    }
    bool allpos = true;
    for (int c = 0; c < dim; ++c)
        if (!(0.0f < mn[c])) allpos = false;
    if (allpos)
        for (int c = 0; c < dim; ++c) mn[c] = 0.0f;
    const int nx = ncn[0], ny = ncn[1], nz = dim == 3 ? ncn[2] : 1;
    float dxs[3] = {1, 1, 1};
    for (int k = 0; k < dim; ++k) dxs[k] = float(nco[k] - 3) / float(ncn[k] - 3);
    std::vector<double> out(size_t(nx) * ny * nz * dim);
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const float P[3] = {dxs[0] * (float(x) - 1.0f) + 1.0f, dxs[1] * (float(y) - 1.0f) + 1.0f,
                                    dxs[2] * (float(z) - 1.0f) + 1.0f};
                int idx[3][4];
                double wt[3][4];
                const int width[3] = {ox, oy, oz};
                for (int k = 0; k < 3; ++k) {
                    if (k >= dim) {
                        idx[k][0] = 0;
                        wt[k][0] = 1.0;
                        continue;
                    }
                    const int s = start_weights(double(P[k]), wt[k]);
                    for (int q = 0; q < 4; ++q) {
                        int i = s + q;
                        if (s < 0 || s + 3 >= width[k]) i = mirror_fold(i, width[k]);
                        idx[k][q] = i;
                    }
                }
                const int kzn = dim == 3 ? 4 : 1;
                for (int c = 0; c < dim; ++c) {
                    double r = 0.0;
                    for (int kz = 0; kz < kzn; ++kz) {
                        double ry = 0.0;
                        for (int ky = 0; ky < 4; ++ky) {
                            double rx = 0.0;
                            for (int kx = 0; kx < 4; ++kx)
                                rx += wt[0][kx] * coef[c][(size_t(idx[2][kz]) * oy + idx[1][ky]) * ox + idx[0][kx]];
                            ry += wt[1][ky] * rx;
                        }
                        r += wt[2][kz] * ry;
                    }
                    r = (r >= mn[c]) ? ((r <= mx[c]) ? r : mx[c]) : mn[c];
                    out[((size_t(z) * ny + y) * nx + x) * dim + c] = double(float(r));
                }
            }
    p.swap(out);
    return true;
}

typedef std::function<double(const std::vector<double> &, std::vector<double> &)> Fdf;

/* GSL steepest descent (multimin/steepest_descent.c) as driven by
   CGSLFDFMinimizer::do_run (mia/core/minimizer/gsl.cc:122-156) */
double run_gsl_sd(std::vector<double> &x, const OrcMinimizer &mz, const Fdf &fdf, int *evals)
{
    const size_t n = x.size();
    std::vector<double> g(n), x1(n), g1(n);
    double f = fdf(x, g);
    int ne = 1;
    double step = mz.step;
    int iter = 0;
    for (;;) {
        ++iter;
        double gn = 0.0;
        for (double v : g) gn += v * v;
        gn = std::sqrt(gn);
        if (gn == 0.0) break;
        bool failed = false, noprog = false;
        double f1 = 0.0;
        for (int trial = 0;; ++trial) {
            const double a = -step / gn;
            bool eq = true;
            for (size_t i = 0; i < n; ++i) {
                x1[i] = x[i] + a * g[i];
                if (x1[i] != x[i]) eq = false;
            }
            if (eq || trial >= 2000) {
                noprog = true;
                break;
            }
            f1 = fdf(x1, g1);
            ++ne;
            if (f1 > f) {
                failed = true;
                step *= mz.tol;
                continue;
            }
            break;
        }
        if (noprog) break;
        step *= failed ? mz.tol : 2.0;
        x.swap(x1);
        g.swap(g1);
        f = f1;
        double gn2 = 0.0;
        for (double v : g) gn2 += v * v;
        if (std::sqrt(gn2) < mz.eps || iter >= mz.maxiter) break;
    }
    if (evals) *evals += ne;
    return f;
}

/* CGDSQMinimizer::do_run (mia/core/minimizer/gdsq.cc:60-122) */
double run_gdsq(std::vector<double> &x, const OrcMinimizer &mz, const Fdf &fdf, int *evals)
{
    auto test_tol = [](const std::vector<double> &v, double tol, int cause) {
        for (double e : v)
            if (std::fabs(e) >= tol) return 0;
        return cause;
    };
    const size_t n = x.size();
    std::vector<double> g(n), gt(n), xw(x);
    double f_old = fdf(xw, g);
    int ne = 1;
    double step = mz.step;
    unsigned iter = 0;
    int success = test_tol(g, mz.xtol, 1);
    while (iter++ < unsigned(mz.maxiter) && step > mz.min_step && !success) {
        for (size_t i = 0; i < n; ++i) xw[i] += -step * g[i];
        const double f = fdf(xw, gt);
        ++ne;
        if (f < f_old) {
            for (size_t i = 0; i < n; ++i) g[i] *= -step;
            double sum = 0.0;
            for (size_t i = 0; i < n; ++i) sum += g[i] * gt[i];
            const double aux = f_old - f + sum;
            if (aux <= 0.0) step *= mz.scale;
            else {
                double nn = 0.0;
                for (double v : g) nn += v * v;
                step = 0.5 * std::sqrt(nn) / aux;
            }
            x = xw;
            g = gt;
            const double frel = f_old - f;
            f_old = f;
            success |= test_tol(gt, mz.gtol, 2);
            if (frel < mz.ftolr) success |= 4;
        } else {
            xw = x;
            step /= mz.scale;
        }
        success |= test_tol(g, mz.xtol / step, 1);
    }
    if (evals) *evals += ne;
    return f_old;
}

}  // namespace

extern "C" {

int orc_normalize_pair(const float *src, const float *ref, size_t n, float *so, float *ro, double *mean,
                       double *sigma)
{
    return normalize_cpu(src, ref, n, so, ro, mean, sigma) ? 1 : 0;
}

void orc_scale_image(const float *in, int dim, const int in_size[3], float *out, const int out_size[3])
{
    scale_image_cpu(in, dim, in_size, out, out_size);
}

int orc_refine(int dim, const int nco[3], const int ncn[3], const double *p, double *out, size_t max_out)
{
    std::vector<double> v(p, p + size_t(nco[0]) * nco[1] * (dim == 3 ? nco[2] : 1) * dim);
    if (!refine_cpu(dim, nco, ncn, v)) return 0;
    if (v.size() > max_out) return -1;
    std::copy(v.begin(), v.end(), out);
    return int(v.size());
}

int orc_register(const OrcLevelDesc *desc, int levels, const OrcMinimizer *mz, const float *src,
                 const float *ref, double *params_out, int max_params, int csize_out[3], double *final_cost,
                 int *evals_out)
{
    const int dim = desc->dim;
    const int fs[3] = {desc->size[0], desc->size[1], dim == 3 ? desc->size[2] : 1};
    const size_t nf = size_t(fs[0]) * fs[1] * fs[2];
    std::vector<float> sn(nf), rn(nf);
    int evals = 0;
    double cost = 0.0;
    int cs[3] = {1, 1, 1};
    std::vector<double> p;
    if (!normalize_cpu(src, ref, nf, sn.data(), rn.data(), nullptr, nullptr)) {
        for (int k = 0; k < dim; ++k) cs[k] = Spline<RefP>::csize_from_rate(fs[k], desc->rate[k]);
        p.assign(size_t(cs[0]) * cs[1] * cs[2] * dim, 0.0);
    } else {
        int prev[3] = {0, 0, 0};
        for (int shift = levels - 1; shift >= 0; --shift) {
            int sz[3] = {1, 1, 1};
            for (int k = 0; k < dim; ++k) sz[k] = fs[k] / (1 << shift);
            if (shift == levels - 1) {
                for (int k = 0; k < dim; ++k) cs[k] = Spline<RefP>::csize_from_rate(sz[k], desc->rate[k]);
                p.assign(size_t(cs[0]) * cs[1] * cs[2] * dim, 0.0);
            } else {
                /* do_upscale (spline.cc:399-412; 2D :356-370) */
                float mxs[3];
                for (int k = 0; k < dim; ++k)
                    mxs[k] = dim == 3 ? float(sz[k]) / float(prev[k]) : (float(sz[k]) - 1) / (float(prev[k]) - 1);
                for (size_t i = 0; i < p.size(); ++i) p[i] = double(mxs[i % dim] * float(p[i]));
            }
            const size_t n = size_t(sz[0]) * sz[1] * sz[2];
            std::vector<float> sl(n), rl(n);
            scale_image_cpu(sn.data(), dim, fs, sl.data(), sz);
            scale_image_cpu(rn.data(), dim, fs, rl.data(), sz);
            for (int pass = 0; pass < 2; ++pass) {
                OrcLevelDesc d = *desc;
                for (int k = 0; k < 3; ++k) {
                    d.size[k] = sz[k];
                    d.csize[k] = cs[k];
                }
                OrcLevel *lv = orc_level_create(&d);
                orc_level_set_images(lv, sl.data(), rl.data());
                Fdf fdf = [&](const std::vector<double> &x, std::vector<double> &g) {
                    std::vector<double> gp(g.size());
                    double ci = 0, cp = 0;
                    orc_level_evaluate(lv, x.data(), g.data(), gp.data(), &ci, &cp);
                    for (size_t i = 0; i < g.size(); ++i) g[i] += gp[i];
                    return ci + cp;
                };
                cost = (mz->kind == ORC_MIN_GDSQ) ? run_gdsq(p, *mz, fdf, &evals) : run_gsl_sd(p, *mz, fdf, &evals);
                orc_level_destroy(lv);
                for (double &v : p) v = double(float(v));
                if (pass == 1) break;
                int ncn[3] = {1, 1, 1};
                for (int k = 0; k < dim; ++k) ncn[k] = refine_csize_cpu(sz[k], desc->rate[k]);
                if (!refine_cpu(dim, cs, ncn, p)) break;
                for (int k = 0; k < 3; ++k) cs[k] = ncn[k];
            }
            for (int k = 0; k < 3; ++k) prev[k] = sz[k];
        }
    }
    if (int(p.size()) > max_params) return -1;
    std::copy(p.begin(), p.end(), params_out);
    for (int k = 0; k < 3; ++k) csize_out[k] = cs[k];
    if (final_cost) *final_cost = cost;
    if (evals_out) *evals_out = evals;
    return int(p.size());
}

}  // extern "C"

extern "C" {
/* The analytic problem of the reference's gdsq test
   (mia/core/minimizer/test_gdsq.cc:25-80):
   f = p2 (x - p0)^2 + p3 (y - p1)^2 + p4 with p = (1, 2, 10, 20, 30). */
double orc_minimize_test_problem(const OrcMinimizer *mz, double x[2], int *evals)
{
    const double pp[5] = {1.0, 2.0, 10.0, 20.0, 30.0};
    Fdf fdf = [&](const std::vector<double> &v, std::vector<double> &g) {
        g[0] = 2.0 * pp[2] * (v[0] - pp[0]);
        g[1] = 2.0 * pp[3] * (v[1] - pp[1]);
        return pp[2] * (v[0] - pp[0]) * (v[0] - pp[0]) + pp[3] * (v[1] - pp[1]) * (v[1] - pp[1]) + pp[4];
    };
    std::vector<double> v(x, x + 2);
    int ne = 0;
    const double f = (mz->kind == ORC_MIN_GDSQ) ? run_gdsq(v, *mz, fdf, &ne) : run_gsl_sd(v, *mz, fdf, &ne);
    x[0] = v[0];
    x[1] = v[1];
    if (evals) *evals = ne;
    return f;
}
}
