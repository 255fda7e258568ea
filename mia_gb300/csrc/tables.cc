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

// Value of the cubic B-spline at x (bspline<3,0>::apply,
// mia/core/splinekernel/bspline.cc:328-345): the transposed rows of
// build_axis carry these values rounded to float, so the expression and
// its rounding are kept.
double bspline3_value(double x)
{
    x = std::fabs(x);
    if (x <= 1.0) return 2.0 / 3.0 - x * x * (1 - 0.5 * x);
    if (x < 2.0) {
        const double dx = 2.0 - x;
        return dx * dx * dx * (1.0 / 6.0);
    }
    return 0.0;
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
                const double y = bspline3_value(x);
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

// ---------------------------------------------------------------------
// divcurl penalty
// ---------------------------------------------------------------------
// The `divcurl` spline penalty (mia/3d/ppmatrix.cc, mia/2d/ppmatrix.cc)
// of a spline field u = sum_i c_i B(x - i) (B the cubic B-spline per axis,
// coordinates in coefficient units) is the energy
//
//   E(u) = int wdiv |grad(div u)|^2 + wrot |grad(curl u)|^2 dx,
//
// a quadratic form in the coefficients with one d x d block per pair of
// coefficients (i, j).  Every second derivative of u is a sum of
// coefficients times products of per-axis B-spline derivatives, so every
// entry of a block is a sum of terms
//
//   w * prod_axes J_a(alpha_a, beta_a; i_a, j_a),
//   J(p, q; s, t) = h^(p+q) int B^(p)(x - s) B^(q)(x - t) dx,
//
// where alpha and beta are the derivative orders taken at i and at j (two
// per term: each term pairs one second derivative at i with one at j) and
// h = (n_c - 1) / range converts coefficient units to image units.  The
// builders tabulate J per axis and derivative pair and assemble the blocks
// from a term list that follows from the two operators:
//
//   grad(div u):  for every axis a the form sum_c d_a d_c u_c, so block
//                 (c, c') gets wdiv * K(a + c, a + c') summed over a;
//   grad(curl u): |curl v|^2 = |grad v|^2 - tr(grad v grad v) for
//                 v = d_a u, so block (c, c) gets wrot * K(a + b, a + b)
//                 for every axis a and every b != c, and the pair of
//                 blocks (c, c'), (c', c) gets -2 wrot K(a + c', a + c);
//
// with K(alpha, beta) the product of the J over the axes.  Conventions of
// the reference that these tables follow (they decide values, not only
// rounding):
//
//   R1  quadrature: J is the composite Simpson sum on 8 panels per unit
//       interval of the supports' overlap (the reference integrates with
//       mia/core/splinekernel.cc:287-315 and mia/core/simpson.hh:36-51);
//       for these piecewise polynomials that is not the exact integral;
//   R2  powers of h are float products h, h*h, h*(h*h), ... and the global
//       factor is 1 / (h_x h_y [h_z]) of the float product
//       (mia/3d/ppmatrix.cc:191-197, mia/2d/ppmatrix.cc:195-199);
//   R3  cross entries store both orderings of the pair in one number and
//       write the curl part in the derivative order of the div part,
//       2 (wdiv - wrot) sum_a K(a + c, a + c'): the two orders agree by
//       integration by parts when the integrals cover the whole overlap;
//       the reference uses this form also for the boundary-clipped 2D
//       integrals, where they do not;
//   R4  in the (x, y) entry the term of the last axis is taken in the
//       opposite order, K(a + y, a + x) (mia/3d/ppmatrix.cc:269-272,
//       mia/2d/ppmatrix.cc:230); with whole-overlap 3D integrals the two
//       orders agree to rounding, with the clipped 2D ones they do not;
//   R5  3D integrals run over the whole overlap for every pair (no image
//       boundary), so one 9^3 table of offsets d = i - j serves the grid;
//       2D integrals are clipped to [0, n_c] on each axis, so 2D blocks
//       depend on the position and are listed per pair (i, j), the rows of
//       i in order of j;
//   R6  offsets of 4 or more coefficients have disjoint supports and are
//       zero (the reference's 3D table keeps them, its 2D list drops every
//       pair whose three values are all zero, mia/2d/ppmatrix.cc:237).
namespace {

// B^(p)(x) of the cubic B-spline, p = 0, 1, 2, from its polynomial pieces
// in t = |x|: (4 - 6 t^2 + 3 t^3) / 6 on [0, 1] and (2 - t)^3 / 6 on [1, 2]
double cubic_bspline_derivative(double x, int p)
{
    const double t = std::fabs(x);
    if (t >= 2.0) return 0.0;
    const double sgn = x < 0.0 ? -1.0 : 1.0;
    if (t <= 1.0) {
        if (p == 0) return (4.0 + t * t * (3.0 * t - 6.0)) / 6.0;
        if (p == 1) return sgn * t * (1.5 * t - 2.0);
        return 3.0 * t - 2.0;
    }
    const double r = 2.0 - t;
    if (p == 0) return r * r * r / 6.0;
    if (p == 1) return -0.5 * sgn * r * r;
    return r;
}

// J(p, q; s, t) without the factor h^(p+q), over the overlap of the two
// supports inside [lo, hi] (R1)
double overlap_integral(int p, int q, double s, double t, double lo, double hi)
{
    const double a = std::max(std::max(s, t) - 2.0, lo);
    const double b = std::min(std::min(s, t) + 2.0, hi);
    if (!(b > a)) return 0.0;
    const int panels = int(8.0 * (b - a));
    const double w = (b - a) / panels;
    auto f = [&](double x) { return cubic_bspline_derivative(x - s, p) * cubic_bspline_derivative(x - t, q); };
    double ends = f(a) + f(b), inner = 0.0, mid = 0.0;
    for (int k = 0; k < panels; ++k) {
        const double x = a + k * w;
        if (k > 0) inner += f(x);
        mid += f(x + 0.5 * w);
    }
    return (ends + 2.0 * inner + 4.0 * mid) * w / 6.0;
}

// h^k for k = 0..4 as float products (R2)
void float_powers(float h, float hp[5])
{
    hp[0] = 1.0f;
    for (int k = 1; k < 5; ++k) hp[k] = h * hp[k - 1];
}

// one term of a block entry: weight and the derivative orders at i and j
struct PenaltyTerm {
    double w;
    int alpha[3];
    int beta[3];
};

// the terms of block entry (c, cp), c <= cp, in a d-dimensional field
std::vector<PenaltyTerm> divcurl_terms(int dim, int c, int cp, double wdiv, double wrot)
{
    std::vector<PenaltyTerm> terms;
    auto orders = [](int a, int b, int o[3]) {
        o[0] = o[1] = o[2] = 0;
        ++o[a];
        ++o[b];
    };
    if (c == cp) {
        for (int a = 0; a < dim; ++a) {
            PenaltyTerm t{wdiv, {0, 0, 0}, {0, 0, 0}};
            orders(a, c, t.alpha);
            orders(a, c, t.beta);
            terms.push_back(t);
            for (int b = 0; b < dim; ++b) {
                if (b == c) continue;
                PenaltyTerm r{wrot, {0, 0, 0}, {0, 0, 0}};
                orders(a, b, r.alpha);
                orders(a, b, r.beta);
                terms.push_back(r);
            }
        }
        return terms;
    }
    const double w = 2.0 * (wdiv - wrot);   // R3
    if (w == 0.0) return terms;
    for (int a = 0; a < dim; ++a) {
        PenaltyTerm t{w, {0, 0, 0}, {0, 0, 0}};
        orders(a, c, t.alpha);
        orders(a, cp, t.beta);
        if (c == 0 && cp == 1 && a == dim - 1) std::swap(t.alpha, t.beta);   // R4
        terms.push_back(t);
    }
    return terms;
}

// the stored entries of a block: 3D (xx, xy, yy, yz, zz, xz), 2D (xx, yy, xy)
constexpr int kEntries3[6][2] = {{0, 0}, {0, 1}, {1, 1}, {1, 2}, {2, 2}, {0, 2}};
constexpr int kEntries2[3][2] = {{0, 0}, {1, 1}, {0, 1}};

}  // namespace

std::vector<double> penalty3_cells(const int csize[3], const float range[3], double wdiv, double wrot)
{
    // J per axis, derivative pair and offset d = -4..4 over the whole
    // overlap (R5), scaled by the float power of h (R2)
    double J[3][3][3][9];
    float hg = 1.0f;
    for (int a = 0; a < 3; ++a) {
        const float h = float(csize[a] - 1) / range[a];
        float hp[5];
        float_powers(h, hp);
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q)
                for (int d = -4; d <= 4; ++d)
                    J[a][p][q][d + 4] = double(hp[p + q]) * overlap_integral(p, q, 0.0, double(d), -1e30, 1e30);
        hg = a == 0 ? h : hg * h;
    }
    const double gscale = 1.0 / double(hg);
    std::vector<PenaltyTerm> terms[6];
    for (int e = 0; e < 6; ++e) terms[e] = divcurl_terms(3, kEntries3[e][0], kEntries3[e][1], wdiv, wrot);
    std::vector<double> P(size_t(9 * 9 * 9) * 6, 0.0);
    for (int dz = 0; dz < 9; ++dz)
        for (int dy = 0; dy < 9; ++dy)
            for (int dx = 0; dx < 9; ++dx) {
                const int d[3] = {dx, dy, dz};
                double *cell = &P[(size_t(dz * 9 + dy) * 9 + dx) * 6];
                for (int e = 0; e < 6; ++e) {
                    double v = 0.0;
                    for (const PenaltyTerm &t : terms[e]) {
                        double prod = t.w;
                        for (int a = 0; a < 3; ++a) prod *= J[a][t.alpha[a]][t.beta[a]][d[a]];
                        v += prod;
                    }
                    cell[e] = gscale * v;
                }
            }
    return P;
}

std::vector<float> build_penalty3(const int csize[3], const float range[3], double wdiv, double wrot)
{
    const std::vector<double> P = penalty3_cells(csize, range, wdiv, wrot);
    return std::vector<float>(P.begin(), P.end());
}

void penalty2_cells(const int csize[2], const float range[2], double wd, double wr, std::vector<int> &rowptr,
                    std::vector<int> &col, std::vector<double> &val)
{
    const int n[2] = {csize[0], csize[1]};
    // J per axis and derivative pair for the coefficient s and its
    // neighbours t = s - 4 .. s + 3, clipped to [0, n_c] (R5)
    std::vector<double> J[2];
    auto jat = [&](int a, int p, int q, int s, int t) -> double {
        return J[a][((size_t(p) * 3 + q) * n[a] + s) * 8 + (t - s + 4)];
    };
    float hg = 1.0f;
    for (int a = 0; a < 2; ++a) {
        const float h = float(n[a] - 1) / range[a];
        float hp[5];
        float_powers(h, hp);
        J[a].assign(size_t(9) * n[a] * 8, 0.0);
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q)
                for (int s = 0; s < n[a]; ++s)
                    for (int t = std::max(0, s - 4); t < std::min(n[a], s + 4); ++t)
                        J[a][((size_t(p) * 3 + q) * n[a] + s) * 8 + (t - s + 4)] =
                            double(hp[p + q]) * overlap_integral(p, q, double(s), double(t), 0.0, double(n[a]));
        hg = a == 0 ? h : hg * h;
    }
    const double gscale = 1.0 / double(hg);
    std::vector<PenaltyTerm> terms[3];
    for (int e = 0; e < 3; ++e) terms[e] = divcurl_terms(2, kEntries2[e][0], kEntries2[e][1], wd, wr);
    const int nx = n[0], ny = n[1];
    rowptr.assign(size_t(nx) * ny + 1, 0);
    col.clear();
    val.clear();
    for (int l = 0; l < ny; ++l)
        for (int k = 0; k < nx; ++k) {
            for (int m2 = std::max(0, l - 4); m2 < std::min(l + 4, ny); ++m2)
                for (int m1 = std::max(0, k - 4); m1 < std::min(k + 4, nx); ++m1) {
                    const int s[2] = {k, l}, t[2] = {m1, m2};
                    double v[3];
                    for (int e = 0; e < 3; ++e) {
                        double acc = 0.0;
                        for (const PenaltyTerm &tm : terms[e]) {
                            double prod = tm.w;
                            for (int a = 0; a < 2; ++a) prod *= jat(a, tm.alpha[a], tm.beta[a], s[a], t[a]);
                            acc += prod;
                        }
                        v[e] = gscale * acc;
                    }
                    if (v[0] == 0.0 && v[1] == 0.0 && v[2] == 0.0) continue;   // R6
                    col.push_back(m1 + m2 * nx);
                    val.push_back(v[0]);
                    val.push_back(v[1]);
                    val.push_back(v[2]);
                }
            rowptr[size_t(l) * nx + k + 1] = int(col.size());
        }
}

void build_penalty2(const int csize[2], const float range[2], double wd, double wr, std::vector<int> &rowptr,
                    std::vector<int> &col, std::vector<float> &val)
{
    std::vector<double> v;
    penalty2_cells(csize, range, wd, wr, rowptr, col, v);
    // device layout: (xx, yy, xy, 0) per cell
    val.assign(v.size() / 3 * 4, 0.0f);
    for (size_t e = 0; e < v.size() / 3; ++e) {
        val[e * 4] = float(v[e * 3]);
        val[e * 4 + 1] = float(v[e * 3 + 1]);
        val[e * 4 + 2] = float(v[e * 3 + 2]);
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
