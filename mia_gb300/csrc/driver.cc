// driver.cc — minimizers and spline level transitions of the registration
// driver (host code; compiled with -ffp-contract=off so the arithmetic
// rounds as the reference's x86-64 build).
#include "driver.hh"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>

namespace mgr {

namespace {

double nrm2(const std::vector<double> &v)
{
    // BLAS dnrm2 computes a scaled sum of squares; for the stopping tests
    // and step rules only its value matters
    double s = 0.0;
    for (double e : v) s += e * e;
    return std::sqrt(s);
}

}  // namespace

// GSL's steepest descent (multimin/steepest_descent.c, GSL 2.x): a trial
// point x1 = x - step * g/|g|; if f(x1) > f(x) the step is multiplied by
// `tol` and the trial repeated, otherwise the move is accepted and the step
// is doubled (or multiplied by `tol` after a failed trial).  The driver
// stops when |g| < eps or after `maxiter` accepted iterations
// (mia/core/minimizer/gsl.cc:122-156).
MinResult minimize_gsl_sd(std::vector<double> &x, const mgr_minimizer_desc &mz, const FDF &fdf)
{
    MinResult r;
    const size_t n = x.size();
    std::vector<double> g(n), x1(n), g1(n);
    double f = fdf(x, g);
    r.evaluations = 1;
    double step = mz.step;
    const double tol = mz.tol;
    int iter = 0;
    bool cont = true;
    const int max_trials = 2000;   // a trial loop cannot exceed the double range of `step`
    while (cont) {
        ++iter;
        const double gnorm = nrm2(g);
        if (gnorm == 0.0) {
            r.status = 1;
            break;
        }
        bool failed = false;
        bool noprog = false;
        double f1 = 0.0;
        for (int trial = 0;; ++trial) {
            const double a = -step / gnorm;
            bool equal = true;
            for (size_t i = 0; i < n; ++i) {
                const double dx = a * g[i];
                x1[i] = x[i] + dx;
                if (x1[i] != x[i]) equal = false;
            }
            if (equal || trial >= max_trials) {
                noprog = true;
                break;
            }
            f1 = fdf(x1, g1);
            ++r.evaluations;
            if (f1 > f) {
                failed = true;
                step *= tol;
                continue;
            }
            break;
        }
        if (noprog) {
            r.status = 1;
            break;
        }
        step *= failed ? tol : 2.0;
        x.swap(x1);
        g.swap(g1);
        f = f1;
        const bool converged = nrm2(g) < mz.eps;
        cont = !converged && iter < mz.maxiter;
        if (!converged && iter >= mz.maxiter) r.status = 2;
    }
    r.f = f;
    r.iterations = iter;
    return r;
}

MinResult minimize_gdsq(std::vector<double> &x, const mgr_minimizer_desc &mz, const FDF &fdf)
{
    enum { SUCCESS_XTOLA = 1, SUCCESS_GTOLA = 2, SUCCESS_FTOLR = 4 };
    auto test_tol = [](const std::vector<double> &dx, double tol, int cause) {
        for (double v : dx)
            if (std::fabs(v) >= tol) return 0;
        return cause;
    };
    MinResult r;
    const size_t n = x.size();
    std::vector<double> g(n), gt(n), xwork(x);
    const double f_init = fdf(xwork, g);
    r.evaluations = 1;
    double step = mz.step;
    double f_old = f_init;
    unsigned iter = 0;
    int success = test_tol(g, mz.xtol, SUCCESS_XTOLA);
    while (iter++ < unsigned(mz.maxiter) && step > mz.min_step && !success) {
        for (size_t i = 0; i < n; ++i) xwork[i] += -step * g[i];
        const double f = fdf(xwork, gt);
        ++r.evaluations;
        if (f < f_old) {
            for (size_t i = 0; i < n; ++i) g[i] *= -step;
            double sum = 0.0;
            for (size_t i = 0; i < n; ++i) sum += g[i] * gt[i];
            const double aux = f_old - f + sum;
            if (aux <= 0.0) step *= mz.scale;
            else step = 0.5 * nrm2(g) / aux;
            x = xwork;
            g = gt;
            const double frel = f_old - f;
            f_old = f;
            success |= test_tol(gt, mz.gtol, SUCCESS_GTOLA);
            if (frel < mz.ftolr) success |= SUCCESS_FTOLR;
        } else {
            xwork = x;
            step /= mz.scale;
        }
        success |= test_tol(g, mz.xtol / step, SUCCESS_XTOLA);
    }
    r.f = f_old;
    r.iterations = int(std::min<unsigned>(iter, unsigned(mz.maxiter)));
    return r;
}

MinResult minimize(std::vector<double> &x, const mgr_minimizer_desc &mz, const FDF &fdf)
{
    if (mz.kind == MGR_MIN_GDSQ) return minimize_gdsq(x, mz, fdf);
    return minimize_gsl_sd(x, mz, fdf);
}

int refine_csize(int size, float rate)
{
    const float f = (float(size) + rate - 1.0f) / rate;
    return int(f) + 2;
}

void round_params_to_float(std::vector<double> &p)
{
    for (double &v : p) v = double(float(v));
}

void upscale_params(int dim, const int old_size[3], const int new_size[3], std::vector<double> &p)
{
    float mx[3];
    for (int k = 0; k < dim; ++k) {
        if (dim == 3) mx[k] = float(new_size[k]) / float(old_size[k]);
        else mx[k] = (float(new_size[k]) - 1) / (float(old_size[k]) - 1);
    }
    for (size_t i = 0; i < p.size(); ++i) p[i] = double(mx[i % dim] * float(p[i]));
}

namespace {

int fastfloor(double v)
{
    volatile double t = v + 68719476736.0 * 1.5;
    double tt = t;
    uint64_t bits;
    std::memcpy(&bits, &tt, sizeof bits);
    return int32_t(uint32_t(bits & 0xffffffffu)) >> 16;
}

int mirror(int index, int width)
{
    const int w2 = 2 * width - 2;
    int idx = index < 0 ? -index : index;
    idx = (width == 1) ? 0 : ((idx < w2) ? idx : idx % w2);
    if (width <= idx) idx = w2 - idx;
    return idx;
}

void filter_line(double *c, int n)
{
    if (n < 2) return;
    const RefineFilterConsts k = refine_filter_consts(n);
    const double p = k.p;
    for (int i = 0; i < n; ++i) c[i] *= k.lambda;
    double zn = p;
    const double iz = k.iz;
    double z2n = k.z2n;
    double sum = c[0] + z2n * c[n - 1];
    z2n *= z2n * iz;
    for (int k2 = 1; k2 < n - 1; ++k2) {
        sum += (zn + z2n) * c[k2];
        zn *= p;
        z2n *= iz;
    }
    c[0] = sum / (1.0 - zn * zn);
    for (int k2 = 1; k2 < n; ++k2) c[k2] += p * c[k2 - 1];
    c[n - 1] = k.q * (p * c[n - 2] + c[n - 1]);
    for (int k2 = n - 2; k2 >= 0; --k2) c[k2] = p * (c[k2 + 1] - c[k2]);
}

void axis_taps(double x, int width, int idx[4], double w[4])
{
    const int r = fastfloor(x);
    const double f = x - r;
    const double ob6 = 1.0 / 6.0, xm1 = 1 - f;
    const double w0 = (xm1 * xm1) * (xm1 * ob6), w3 = (f * f) * (f * ob6);
    w[0] = w0;
    w[3] = w3;
    w[1] = ((xm1 - w0) - w0) + w3;
    w[2] = ((f - w3) - w3) + w0;
    for (int k = 0; k < 4; ++k) idx[k] = r - 1 + k;
    if (idx[0] < 0 || idx[3] >= width)
        for (int k = 0; k < 4; ++k) idx[k] = mirror(idx[k], width);
}

}  // namespace

RefineFilterConsts refine_filter_consts(int n)
{
    RefineFilterConsts k;
    k.p = std::sqrt(3.0) - 2.0;
    k.lambda = 2 - k.p - 1.0 / k.p;
    k.iz = 1.0 / k.p;
    k.q = k.p / (k.p * k.p - 1.0);
    k.z2n = std::pow(k.p, double(n - 1));
    return k;
}

void refine_axis_taps(int n_old, int n_new, std::vector<int> &idx, std::vector<double> &w)
{
    const float dx = float(n_old - 1 - 2) / float(n_new - 1 - 2);
    const float shift = 1.0f;
    idx.assign(size_t(n_new) * 4, 0);
    w.assign(size_t(n_new) * 4, 0.0);
    for (int i = 0; i < n_new; ++i) axis_taps(dx * (float(i) - shift) + shift, n_old, &idx[size_t(i) * 4], &w[size_t(i) * 4]);
}

bool refine_grows(int dim, const int nc_old[3], const int nc_new[3])
{
    for (int k = 0; k < dim; ++k)
        if (nc_new[k] > nc_old[k]) return true;
    return false;
}

bool refine_params(int dim, const int nc_old[3], const int nc_new[3], std::vector<double> &p)
{
    if (!refine_grows(dim, nc_old, nc_new)) return false;
    const int ox = nc_old[0], oy = nc_old[1], oz = dim == 3 ? nc_old[2] : 1;
    const size_t nold = size_t(ox) * oy * oz;
    // coefficients of the vector-valued interpolator: per component, x,
    // then y, then z lines filtered in double (coefficient type C3DDVector)
    std::vector<double> coef(nold * dim);
    for (size_t i = 0; i < nold * dim; ++i) coef[i] = double(float(p[i]));
    float mn[3], mx[3];
    for (int c = 0; c < dim; ++c) {
        mn[c] = mx[c] = float(coef[c]);
        for (size_t i = 1; i < nold; ++i) {
            const float v = float(coef[i * dim + c]);
            if (v > mx[c]) mx[c] = v;
            if (v < mn[c]) mn[c] = v;
        }
    }
    // "if (T() < m_min) m_min = T()": vector < compares all components
    bool all_pos = true;
    for (int c = 0; c < dim; ++c)
        if (!(0.0f < mn[c])) all_pos = false;
    if (all_pos)
        for (int c = 0; c < dim; ++c) mn[c] = 0.0f;
    std::vector<double> line;
    for (int c = 0; c < dim; ++c) {
        line.resize(ox);
        for (int z = 0; z < oz; ++z)
            for (int y = 0; y < oy; ++y) {
                for (int x = 0; x < ox; ++x) line[x] = coef[((size_t(z) * oy + y) * ox + x) * dim + c];
                filter_line(line.data(), ox);
                for (int x = 0; x < ox; ++x) coef[((size_t(z) * oy + y) * ox + x) * dim + c] = line[x];
            }
        line.resize(oy);
        for (int z = 0; z < oz; ++z)
            for (int x = 0; x < ox; ++x) {
                for (int y = 0; y < oy; ++y) line[y] = coef[((size_t(z) * oy + y) * ox + x) * dim + c];
                filter_line(line.data(), oy);
                for (int y = 0; y < oy; ++y) coef[((size_t(z) * oy + y) * ox + x) * dim + c] = line[y];
            }
        if (dim == 3) {
            line.resize(oz);
            for (int y = 0; y < oy; ++y)
                for (int x = 0; x < ox; ++x) {
                    for (int z = 0; z < oz; ++z) line[z] = coef[((size_t(z) * oy + y) * ox + x) * dim + c];
                    filter_line(line.data(), oz);
                    for (int z = 0; z < oz; ++z) coef[((size_t(z) * oy + y) * ox + x) * dim + c] = line[z];
                }
        }
    }
    const int nx = nc_new[0], ny = nc_new[1], nz = dim == 3 ? nc_new[2] : 1;
    // taps of every new grid line on each axis (an axis the 2D grid lacks
    // has the single tap 0 with weight 1)
    const int nn[3] = {nx, ny, nz}, no[3] = {ox, oy, oz};
    std::vector<int> ti[3];
    std::vector<double> tw[3];
    for (int k = 0; k < 3; ++k) {
        if (k < dim) {
            refine_axis_taps(no[k], nn[k], ti[k], tw[k]);
        } else {
            ti[k].assign(size_t(nn[k]) * 4, 0);
            tw[k].assign(size_t(nn[k]) * 4, 0.0);
            for (int i = 0; i < nn[k]; ++i) tw[k][size_t(i) * 4] = 1.0;
        }
    }
    // The interpolation sums x taps, then y, then z (each sum from 0 in tap
    // order).  Done as three stages over whole lines, each partial sum is
    // computed once instead of once per output point, with the same
    // operands in the same order: the same values.
    const int kz_n = dim == 3 ? 4 : 1;
    const size_t rowo = size_t(ox) * dim, rown = size_t(nx) * dim;
    std::vector<double> r1(size_t(oz) * oy * rown);   // x resampled
    for (size_t row = 0; row < size_t(oz) * oy; ++row) {
        const double *src = &coef[row * rowo];
        double *o = &r1[row * rown];
        for (int x = 0; x < nx; ++x) {
            const int *ix = &ti[0][size_t(x) * 4];
            const double *wx = &tw[0][size_t(x) * 4];
            for (int c = 0; c < dim; ++c) {
                double r = 0.0;
                r += wx[0] * src[size_t(ix[0]) * dim + c];
                r += wx[1] * src[size_t(ix[1]) * dim + c];
                r += wx[2] * src[size_t(ix[2]) * dim + c];
                r += wx[3] * src[size_t(ix[3]) * dim + c];
                o[size_t(x) * dim + c] = r;
            }
        }
    }
    std::vector<double> r2(size_t(oz) * ny * rown);   // then y
    for (int z = 0; z < oz; ++z)
        for (int y = 0; y < ny; ++y) {
            const int *iy = &ti[1][size_t(y) * 4];
            const double *wy = &tw[1][size_t(y) * 4];
            const double *a0 = &r1[(size_t(z) * oy + iy[0]) * rown], *a1 = &r1[(size_t(z) * oy + iy[1]) * rown];
            const double *a2 = &r1[(size_t(z) * oy + iy[2]) * rown], *a3 = &r1[(size_t(z) * oy + iy[3]) * rown];
            double *o = &r2[(size_t(z) * ny + y) * rown];
            for (size_t i = 0; i < rown; ++i) {
                double r = 0.0;
                r += wy[0] * a0[i];
                r += wy[1] * a1[i];
                r += wy[2] * a2[i];
                r += wy[3] * a3[i];
                o[i] = r;
            }
        }
    std::vector<double> out(size_t(nx) * ny * nz * dim);   // then z, clamped, stored as float
    for (int z = 0; z < nz; ++z) {
        const int *iz = &ti[2][size_t(z) * 4];
        const double *wz = &tw[2][size_t(z) * 4];
        for (int y = 0; y < ny; ++y) {
            const double *a[4];
            for (int kz = 0; kz < 4; ++kz) a[kz] = &r2[(size_t(iz[kz]) * ny + y) * rown];
            double *o = &out[(size_t(z) * ny + y) * rown];
            for (int x = 0; x < nx; ++x)
                for (int c = 0; c < dim; ++c) {
                    const size_t i = size_t(x) * dim + c;
                    double r = 0.0;
                    if (kz_n == 4) {
                        r += wz[0] * a[0][i];
                        r += wz[1] * a[1][i];
                        r += wz[2] * a[2][i];
                        r += wz[3] * a[3][i];
                    } else {
                        r += wz[0] * a[0][i];
                    }
                    r = (r >= mn[c]) ? ((r <= mx[c]) ? r : mx[c]) : mn[c];
                    o[i] = double(float(r));
                }
        }
    }
    p.swap(out);
    return true;
}

}  // namespace mgr
