// tables.cc — host set-up of the per-level tables: per-axis spline weights
// (forward and transposed), tile footprints, and the divcurl penalty
// matrix.  All of it runs once per level (when the transformation or image
// size changes), as the reference's reinit() and penalty initialize() do.
//
// Compiled with -ffp-contract=off so the float/double expressions round as
// the reference's SSE2 x86-64 build does on both x86-64 and aarch64.
#include "tables.hh"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>

namespace mgr {

namespace {

// fixed-point floor with 2^-16 resolution (mia/core/splinekernel.cc:164-192)
int fastfloor(double v)
{
    volatile double t = v + 68719476736.0 * 1.5;
    double tt = t;
    uint64_t bits;
    std::memcpy(&bits, &tt, sizeof bits);
    return int32_t(uint32_t(bits & 0xffffffffu)) >> 16;
}

// CBSplineKernel3::get_weights, SSE2 order (bspline.cc:258-285)
void weights3(double x, double w[4])
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

// bspline<3,k>::apply (bspline.cc:328-375)
double bspline3(double x, int deg)
{
    if (deg == 0) {
        x = std::fabs(x);
        if (x <= 1.0) return 2.0 / 3.0 - x * x * (1 - 0.5 * x);
        if (x < 2.0) {
            const double dx = 2.0 - x;
            return dx * dx * dx * (1.0 / 6.0);
        }
        return 0.0;
    }
    if (deg == 1) {
        const double ax = std::fabs(x);
        if (ax <= 1.0) return (1.5 * ax - 2) * x;
        if (ax <= 2.0) return (x > 0.0 ? -0.5 : 0.5) * (2 - ax) * (2 - ax);
        return 0.0;
    }
    x = std::fabs(x);
    if (x > 2.0) return 0.0;
    if (x > 1.0) return 2.0 - x;
    return 3.0 * x - 2.0;
}

// integrate2 + simpson for the cubic kernel (mia/core/splinekernel.cc:287-315,
// mia/core/simpson.hh:36-51)
double integrate2(double s1, double s2, int d1, int d2, double x0, double L)
{
    double a = s1 - 2.0, b = s1 + 2.0;
    if (a < s2 - 2.0) a = s2 - 2.0;
    if (a < x0) a = x0;
    if (b > s2 + 2.0) b = s2 + 2.0;
    if (b > L) b = L;
    if (b <= a) return 0.0;
    const size_t intervals = size_t(8 * (b - a));
    auto f = [&](double x) { return bspline3(x - s1, d1) * bspline3(x - s2, d2); };
    const double dx = (b - a) / intervals;
    double sum = 0.5 * (f(a) + f(b));
    double x = a + dx;
    for (size_t i = 1; i < intervals; ++i, x += dx) sum += f(x);
    x = a + .5 * dx;
    for (size_t i = 0; i < intervals; ++i, x += dx) sum += 2 * f(x);
    return sum * dx / 3.0;
}

}  // namespace

int csize_from_rate(int size, float rate)
{
    // floor((n - 1 + rate) / rate) in float, plus the 2-coefficient border
    // (mia/3d/transform/spline.cc:133, mia/2d/transform/spline.cc:105-106)
    const float f = (float(size - 1) + rate) / rate;
    return int(f) + 2;
}

void build_axis(AxisHost &ax, int n, int nc, int tile)
{
    if (n < 2) throw std::invalid_argument("image dimension must be >= 2");
    if (nc < 4) throw std::invalid_argument("coefficient grid dimension must be >= 4");
    ax.n = n;
    ax.nc = nc;
    ax.t = tile;
    ax.nt = (n + tile - 1) / tile;
    // C3DSplineTransformation::reinit (spline.cc:224-275): float scale,
    // float coordinate, fixed-point floor, double weights, 3 taps on the
    // last voxel
    const float scale = float(nc - 3) / float(n - 1);
    ax.scale = scale;
    ax.fs.resize(n);
    ax.fw.resize(size_t(n) * 4);
    for (int i = 0; i < n; ++i) {
        const float xc = float(i) * scale + 1.0f;
        const int r = fastfloor(double(xc));
        double w[4];
        weights3(double(xc) - r, w);
        ax.fs[i] = r - 1;
        for (int k = 0; k < 4; ++k) ax.fw[size_t(i) * 4 + k] = float(w[k]);
    }
    ax.fw[size_t(n - 1) * 4 + 3] = 0.0f;
    // get_derivative_row (spline.cc:697-729): double coordinate, float
    // weights, contiguous voxel range per coefficient
    ax.rows.assign(size_t(nc) * 2, 0);
    ax.as.assign(n, INT32_MAX);
    ax.aw.assign(size_t(n) * 4, 0.0f);
    std::vector<std::vector<std::pair<int, float>>> per_voxel(n);
    for (int o = 0; o < nc; ++o) {
        int first = -1, len = 0;
        for (int i = 0; i < n; ++i) {
            const double x = double(i) * double(scale) + 1.0 - double(o);
            if (std::fabs(x) < 2.0) {
                if (first < 0) first = i;
                const double y = bspline3(x, 0);
                if (y > 0) {
                    ++len;
                    per_voxel[i].push_back({o, float(y)});
                } else {
                    break;
                }
            }
        }
        ax.rows[size_t(o) * 2] = first < 0 ? 0 : first;
        ax.rows[size_t(o) * 2 + 1] = len;
    }
    for (int i = 0; i < n; ++i) {
        auto &v = per_voxel[i];
        if (v.empty()) throw std::runtime_error("voxel without spline support");
        const int s = v.front().first;
        ax.as[i] = s;
        for (auto &p : v) {
            const int k = p.first - s;
            if (k < 0 || k > 3) throw std::runtime_error("non-contiguous spline support");
            ax.aw[size_t(i) * 4 + k] = p.second;
        }
    }
    // tile footprints
    ax.ftile0.resize(ax.nt);
    ax.atile0.resize(ax.nt);
    std::vector<int> aend(ax.nt);
    ax.fc = 0;
    ax.ac = 0;
    for (int b = 0; b < ax.nt; ++b) {
        const int v0 = b * tile, v1 = std::min(n, v0 + tile) - 1;
        ax.ftile0[b] = ax.fs[v0];
        ax.fc = std::max(ax.fc, ax.fs[v1] + 3 - ax.fs[v0] + 1);
        ax.atile0[b] = ax.as[v0];
        aend[b] = std::min(nc - 1, ax.as[v1] + 3);
        // the slot holds the full 4-wide window of the last voxel, even where
        // it reaches past the grid (those entries are zero and never read)
        ax.ac = std::max(ax.ac, ax.as[v1] + 3 - ax.atile0[b] + 1);
        if (ax.fs[v0] < 0) throw std::runtime_error("negative forward start index");
    }
    ax.gtile.assign(size_t(nc) * 2, 0);
    for (int o = 0; o < nc; ++o) {
        int lo = -1, hi = -2;
        for (int b = 0; b < ax.nt; ++b)
            if (ax.atile0[b] <= o && o <= aend[b]) {
                if (lo < 0) lo = b;
                hi = b;
            }
        if (lo < 0) { lo = 0; hi = -1; }  // no tile: empty range
        ax.gtile[size_t(o) * 2] = lo;
        ax.gtile[size_t(o) * 2 + 1] = hi;
    }
}

// C3DPPDivcurlMatrixImpl::reset (mia/3d/ppmatrix.cc:175-290), including
// CIntegralCache2's first-lookup-returns-0 behaviour (ppmatrix.cc:147-165).
std::vector<float> build_penalty3(const int csize[3], const float range[3], double wdiv, double wrot)
{
    struct Cache {
        int d1, d2;
        bool valid[9] = {false};
        double val[9] = {0};
        double get(int delta)
        {
            delta += 4;
            if (delta < 0 || delta >= 9) return 0;
            double r = 0;
            if (valid[delta]) r = val[delta];
            else {
                val[delta] = integrate2(4, delta, d1, d2, 0, 8);
                valid[delta] = true;
            }
            return r;
        }
    };
    Cache rc00{0, 0}, rc11{1, 1}, rc22{2, 2}, rc21{2, 1}, rc12{1, 2}, rc01{0, 1}, rc10{1, 0};
    const float h1x = float(csize[0] - 1) / range[0];
    const float h1y = float(csize[1] - 1) / range[1];
    const float h1z = float(csize[2] - 1) / range[2];
    const float h2x = h1x * h1x, h2y = h1y * h1y, h2z = h1z * h1z;
    const float h3x = h1x * h2x, h3y = h1y * h2y, h3z = h1z * h2z;
    const float h4x = h1x * h3x, h4y = h1y * h3y, h4z = h1z * h3z;
    const double gs = 1.0 / double(float(h1x * h1y) * h1z);
    const double wsum = wdiv + wrot, wdelta = 2 * (wdiv - wrot);
    std::vector<float> P(9 * 9 * 9 * 6, 0.0f);
    size_t pi = 0;
    for (int z = -4; z <= 4; ++z) {
        const double r00z = rc00.get(z), r01z = h1z * rc01.get(z), r11z = h2z * rc11.get(z);
        const double r12z = h3z * rc12.get(z), r22z = h4z * rc22.get(z);
        for (int y = -4; y <= 4; ++y) {
            const double r00y = rc00.get(y), r01y = h1y * rc01.get(y), r10y = h1y * rc10.get(y);
            const double r11y = h2y * rc11.get(y), r12y = h3y * rc12.get(y), r21y = h3y * rc21.get(y);
            const double r22y = h4y * rc22.get(y);
            for (int x = -4; x <= 4; ++x, ++pi) {
                const double r00x = rc00.get(x), r01x = h1x * rc01.get(x), r10x = h1x * rc10.get(x);
                const double r11x = h2x * rc11.get(x), r21x = h3x * rc21.get(x), r22x = h4x * rc22.get(x);
                const double r200200 = r22x * r00y * r00z, r020020 = r00x * r22y * r00z;
                const double r002002 = r00x * r00y * r22z, r110110 = r11x * r11y * r00z;
                const double r101101 = r11x * r00y * r11z, r011011 = r00x * r11y * r11z;
                const double vxx = gs * (r002002 * wrot + r011011 * 2.0 * wrot + r020020 * wrot +
                                         r101101 * wsum + r110110 * wsum + r200200 * wdiv);
                const double vyy = gs * (r002002 * wrot + r011011 * wsum + r020020 * wdiv +
                                         r101101 * 2 * wrot + r110110 * wsum + r200200 * wrot);
                const double vzz = gs * (r002002 * wdiv + r011011 * wsum + r020020 * wrot +
                                         r101101 * wsum + r110110 * wrot * 2 + r200200 * wrot);
                double vxy = 0, vxz = 0, vyz = 0;
                if (wdelta != 0.0) {
                    vxy = gs * wdelta * (r21x * r01y * r00z + r10x * r12y * r00z + r01x * r10y * r11z);
                    vxz = gs * wdelta * (r21x * r00y * r01z + r10x * r11y * r01z + r10x * r00y * r12z);
                    vyz = gs * wdelta * (r11x * r10y * r01z + r00x * r21y * r01z + r00x * r10y * r12z);
                }
                float *c = &P[pi * 6];
                c[0] = float(vxx);
                c[1] = float(vxy);
                c[2] = float(vyy);
                c[3] = float(vyz);
                c[4] = float(vzz);
                c[5] = float(vxz);
            }
        }
    }
    return P;
}

// C2DPPDivcurlMatrixImpl::reset (mia/2d/ppmatrix.cc:182-243) with the
// (skip, delta)-keyed CIntegralCache (ppmatrix.cc:113-172); cells grouped
// by row i in list order (CSR).
void build_penalty2(const int csize[2], const float range[2], double wd, double wr, std::vector<int> &rowptr,
                    std::vector<int> &col, std::vector<float> &val)
{
    struct Cache {
        std::map<int, double> values;
        double get(int s1, int s2, int d1, int d2, int range)
        {
            bool swapped = false;
            if (s2 < s1) { swapped = true; std::swap(s1, s2); }
            int delta = s2 - s1;
            if (delta >= 4) return 0.0;
            int skip = 0;
            const int dlow = 2 - s1;
            if (dlow > 0) {
                skip = s2 - 2;
                if (skip > 0) skip = 0;
            } else {
                const int dhigh = 2 + s2 - range;
                if (dhigh > 0) skip = 2 + s1 - range;
                if (skip < 0) skip = 0;
            }
            if (std::abs(skip) >= 4) return 0.0;
            if (swapped) { delta = -delta; std::swap(s1, s2); }
            const int index = skip * 8 + delta + 4;
            auto pv = values.find(index);
            if (pv != values.end()) return pv->second;
            const double r = values[index] = integrate2(s1, s2, d1, d2, 0, range);
            return r;
        }
    };
    const int nx = csize[0], ny = csize[1];
    const float h1x = float(nx - 1) / range[0], h1y = float(ny - 1) / range[1];
    const double gs = 1.0 / double(h1x * h1y);
    const float h2x = h1x * h1x, h2y = h1y * h1y, h3x = h1x * h2x, h3y = h1y * h2y;
    const float h4x = h1x * h3x, h4y = h1y * h3y;
    Cache rc22, rc21, rc01, rc12, rc10, rc00, rc11;
    struct Cell { int i, j; float vx, vy, v12; };
    std::vector<Cell> cells;
    for (int l = 0; l < ny; ++l)
        for (int n = std::max(0, l - 4); n < std::min(l + 4, ny); ++n) {
            const double r00y = rc00.get(l, n, 0, 0, ny), r01y = h1y * rc01.get(l, n, 0, 1, ny);
            const double r11y = h2y * rc11.get(l, n, 1, 1, ny), r21y = h3y * rc21.get(l, n, 2, 1, ny);
            const double r22y = h4y * rc22.get(l, n, 2, 2, ny);
            for (int k = 0; k < nx; ++k)
                for (int m = std::max(0, k - 4); m < std::min(k + 4, nx); ++m) {
                    const double r00x = rc00.get(k, m, 0, 0, nx), r01x = h1x * rc01.get(k, m, 0, 1, nx);
                    const double r11x = h2x * rc11.get(k, m, 1, 1, nx), r21x = h3x * rc21.get(k, m, 2, 1, nx);
                    const double r22x = h4x * rc22.get(k, m, 2, 2, nx);
                    const double vx = gs * (wd * (r22x * r00y + r11x * r11y) + wr * (r11x * r11y + r00x * r22y));
                    const double v12 = 2 * gs * (wd - wr) * (r21x * r01y + r01x * r21y);
                    const double vy = gs * (wd * (r00x * r22y + r11x * r11y) + wr * (r22x * r00y + r11x * r11y));
                    if (vx != 0.0 || v12 != 0.0 || vy != 0.0)
                        cells.push_back({k + l * nx, m + n * nx, float(vx), float(vy), float(v12)});
                }
        }
    std::stable_sort(cells.begin(), cells.end(), [](const Cell &a, const Cell &b) { return a.i < b.i; });
    rowptr.assign(size_t(nx) * ny + 1, 0);
    col.resize(cells.size());
    val.resize(cells.size() * 4);
    for (const Cell &c : cells) rowptr[c.i + 1]++;
    for (size_t i = 0; i < size_t(nx) * ny; ++i) rowptr[i + 1] += rowptr[i];
    for (size_t e = 0; e < cells.size(); ++e) {
        col[e] = cells[e].j;
        val[e * 4] = cells[e].vx;
        val[e * 4 + 1] = cells[e].vy;
        val[e * 4 + 2] = cells[e].v12;
        val[e * 4 + 3] = 0.0f;
    }
}

std::shared_ptr<const Penalty2Table> penalty2_cached(const int csize[2], const float range[2], double wd, double wr)
{
    struct Entry {
        int c0, c1;
        float r0, r1;
        double wd, wr;
        std::shared_ptr<const Penalty2Table> t;
    };
    static std::mutex mu;
    static std::deque<Entry> cache;
    std::lock_guard<std::mutex> lk(mu);
    for (const Entry &e : cache)
        if (e.c0 == csize[0] && e.c1 == csize[1] && e.r0 == range[0] && e.r1 == range[1] && e.wd == wd && e.wr == wr)
            return e.t;
    std::shared_ptr<Penalty2Table> t(new Penalty2Table);
    build_penalty2(csize, range, wd, wr, t->rowptr, t->col, t->val);
    if (cache.size() >= 64) cache.pop_front();   // bounded: the oldest table goes first
    cache.push_back(Entry{csize[0], csize[1], range[0], range[1], wd, wr, t});
    return t;
}

}  // namespace mgr
