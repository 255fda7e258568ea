// level_loop.cc — the MIA-side adapter of INTEGRATION.md, driven through
// include/mgr.h only (no MIA headers), over the registration driver's level
// loop (TNonrigidRegisterImpl::run, mia/template/nonrigidregister.cxx:
// 239-294): joint normalisation, for every level the `scale` filter and the
// full cost's set_size, the transformation upscaled with its old coefficient
// grid (mia/3d/transform/spline.cc:399-412), a minimisation, refine() growing
// the grid within the level (:360-396) and a second minimisation.
//
// The adapter part is what a maintainer adds to MIA: a GPU-backed `image`
// full cost that follows the transformation's grid (mgr_level_set_grid),
// reads the divcurl parameters from the transformation's creator string and
// evaluates image term and penalty in one call, and a GPU-backed `divcurl`
// penalty that returns that call's penalty, weighted and signed by the
// penalty wrapper (mia/3d/splinetransformpenalty.cc:52-71).  Every
// evaluation is checked against a level created afresh for the
// transformation's current grid with the penalty weight and the
// reference's sign inside the library: image cost and gradient equal bit
// for bit, penalty cost equal, penalty gradient within float rounding of
// the weight.
//
//   level_loop <2|3>      prints "ok ..." and exits 0 when every check holds
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mgr.h"

namespace {

int failures = 0;

void check(mgr_status s, const char *what)
{
    if (s != MGR_OK) {
        std::fprintf(stderr, "%s: status %d: %s\n", what, int(s), mgr_last_error());
        std::exit(2);
    }
}

void expect(bool ok, const char *what, double a, double b)
{
    if (!ok) {
        ++failures;
        if (failures < 20) std::fprintf(stderr, "mismatch: %s: %.17g vs %.17g\n", what, a, b);
    }
}

size_t prod(const int s[3], int dim) { return size_t(s[0]) * s[1] * (dim == 3 ? s[2] : 1); }

// the spline transformation as the driver sees it (C3DSplineTransformation)
struct Transformation {
    int dim = 3;
    int size[3] = {1, 1, 1};     // image size (range)
    int csize[3] = {1, 1, 1};    // coefficient grid
    float rate = 8.0f;
    std::string creator;         // get_creator_string(): the plugin string it was made from
    std::vector<double> p;       // parameters, x fastest, components interleaved

    void create(const int s[3], float r, const std::string &init)
    {
        rate = r;
        creator = init;
        for (int k = 0; k < 3; ++k) {
            size[k] = k < dim ? s[k] : 1;
            // (n - 1 + rate) / rate in float, plus the border (spline.cc:133)
            csize[k] = k < dim ? int((float(s[k] - 1) + r) / r) + 2 : 1;
        }
        p.assign(prod(csize, dim) * dim, 0.0);
    }
    // set_parameters: the coefficients are stored as float vectors
    void set_parameters(const std::vector<double> &x)
    {
        p = x;
        for (double &v : p) v = double(float(v));
    }
    // upscale: the same grid, coefficients times the size ratio (3D: new /
    // old; 2D: (new - 1) / (old - 1), mia/2d/transform/spline.cc:356-370)
    void upscale(const int ns[3])
    {
        float mx[3];
        for (int k = 0; k < dim; ++k)
            mx[k] = dim == 3 ? float(ns[k]) / float(size[k]) : (float(ns[k]) - 1) / (float(size[k]) - 1);
        for (size_t i = 0; i < p.size(); ++i) p[i] = double(mx[i % dim] * float(p[i]));
        for (int k = 0; k < dim; ++k) size[k] = ns[k];
    }
    // refine: the grid the rate asks for at this size, when larger
    bool refine()
    {
        int nn[3] = {1, 1, 1};
        for (int k = 0; k < dim; ++k) nn[k] = int((float(size[k]) + rate - 1.0f) / rate) + 2;
        std::vector<double> out(prod(nn, dim) * dim);
        int grown = 0;
        check(mgr_refine_coefficients(dim, csize, nn, p.data(), out.data(), &grown), "refine");
        if (!grown) return false;
        p.swap(out);
        for (int k = 0; k < 3; ++k) csize[k] = nn[k];
        return true;
    }
};

// the parameters of the transformation's divcurl penalty, read from its
// creator string "spline:...,penalty=[divcurl:weight=W,div=D,curl=C,norm=N]"
struct DivcurlParams {
    bool present = false;
    double weight = 1.0, div = 1.0, curl = 1.0;
    bool norm = false;
};

DivcurlParams parse_divcurl(const std::string &creator)
{
    DivcurlParams d;
    const size_t a = creator.find("penalty=[divcurl");
    if (a == std::string::npos) return d;
    d.present = true;
    const size_t b = creator.find(']', a);
    const std::string args = creator.substr(a, b - a);
    auto num = [&](const char *key, double &v) {
        const size_t k = args.find(key);
        if (k != std::string::npos) v = std::atof(args.c_str() + k + std::strlen(key));
    };
    num("weight=", d.weight);
    num("div=", d.div);
    num("curl=", d.curl);
    double n = 0;
    num("norm=", n);
    d.norm = n != 0;
    return d;
}

// what one evaluation of the full cost left for the penalty of the same
// coefficients (evaluate_fdf asks the transformation's penalty right after
// the full costs, on the same thread)
struct PenaltyRecord {
    std::vector<float> coeffs;
    double value = 0;            // unweighted c^T P c
    std::vector<double> grad;    // its derivative, unweighted, + sign
    bool with_grad = false;
};
thread_local PenaltyRecord g_penalty;

// the GPU-backed `image` full cost (weight 1 here)
struct GpuImageFullCost {
    int dim, cost;
    std::vector<float> src_full, ref_full;
    int full[3];
    int size[3] = {0, 0, 0};
    std::vector<float> src, ref;
    mgr_level *lvl = nullptr;
    DivcurlParams pen;

    ~GpuImageFullCost() { mgr_level_destroy(lvl); }
    // do_set_size: the images at the level's size (the `scale` filter); the
    // level itself waits for the first evaluation, which knows the grid
    void set_size(const int s[3])
    {
        for (int k = 0; k < 3; ++k) size[k] = k < dim ? s[k] : 1;
        const size_t n = prod(size, dim);
        src.resize(n);
        ref.resize(n);
        if (prod(full, dim) == n) {
            src = src_full;
            ref = ref_full;
        } else {
            check(mgr_scale_image(dim, full, src_full.data(), size, src.data(), 0), "scale src");
            check(mgr_scale_image(dim, full, ref_full.data(), size, ref.data(), 0), "scale ref");
        }
        mgr_level_destroy(lvl);
        lvl = nullptr;
    }
    void follow(const Transformation &t)
    {
        if (!lvl) {
            pen = parse_divcurl(t.creator);
            mgr_level_desc d{};
            d.dim = dim;
            for (int k = 0; k < 3; ++k) {
                d.size[k] = size[k];
                d.csize[k] = k < dim ? t.csize[k] : 0;
                d.rate[k] = t.rate;
            }
            d.cost = cost;
            d.cost_weight = 1.0;
            // the penalty's own weight, normalisation and sign are applied
            // by the penalty wrapper: the level returns c^T P c and its
            // derivative
            d.has_penalty = pen.present;
            d.pen_weight = 1.0;
            d.pen_div = pen.div;
            d.pen_curl = pen.curl;
            d.pen_norm = 0;
            d.pen_corrected = 1;
            check(mgr_level_create(&d, 0, nullptr, &lvl), "level create");
            check(mgr_level_set_images(lvl, src.data(), ref.data()), "set images");
            return;
        }
        int cs[3];
        size_t np = 0;
        check(mgr_level_csize(lvl, cs, &np), "csize");
        bool same = true;
        for (int k = 0; k < dim; ++k) same = same && cs[k] == t.csize[k];
        if (!same) check(mgr_level_set_grid(lvl, t.csize), "set grid");   // refine() grew it
    }
    void record(const Transformation &t, double pv, const std::vector<double> *pg)
    {
        g_penalty.coeffs.assign(t.p.begin(), t.p.end());
        g_penalty.value = pv;
        g_penalty.with_grad = pg != nullptr;
        if (pg) g_penalty.grad = *pg;
    }
    double evaluate(const Transformation &t, std::vector<double> &grad)
    {
        follow(t);
        std::vector<double> gp(t.p.size());
        double ci = 0, cp = 0;
        check(mgr_level_evaluate(lvl, t.p.data(), nullptr, grad.data(), gp.data(), &ci, &cp), "evaluate");
        record(t, cp, &gp);
        return ci;
    }
    double value(const Transformation &t)
    {
        follow(t);
        double ci = 0, cp = 0;
        check(mgr_level_value(lvl, t.p.data(), &ci, &cp), "value");
        record(t, cp, nullptr);
        return ci;
    }
};

// the GPU-backed `divcurl` penalty: value_and_gradient of the wrapper with
// the recorded evaluation as do_value_and_gradient
struct GpuDivcurlPenalty {
    DivcurlParams pen;
    int range[3];
    int dim;
    double weight() const
    {
        double vol = 1.0;
        for (int k = 0; k < dim; ++k) vol *= range[k];
        return pen.norm ? pen.weight / vol : pen.weight;
    }
    bool recorded_for(const Transformation &t) const
    {
        if (g_penalty.coeffs.size() != t.p.size()) return false;
        for (size_t i = 0; i < t.p.size(); ++i)
            if (g_penalty.coeffs[i] != float(t.p[i])) return false;
        return true;
    }
    double value_and_gradient(const Transformation &t, std::vector<double> &g) const
    {
        if (!recorded_for(t) || !g_penalty.with_grad) {
            std::fprintf(stderr, "penalty asked for coefficients the full cost did not evaluate\n");
            std::exit(3);
        }
        const double w = weight();
        for (size_t i = 0; i < g.size(); ++i) g[i] = -w * g_penalty.grad[i];
        return w * g_penalty.value;
    }
    double value(const Transformation &t) const
    {
        if (!recorded_for(t)) std::exit(3);
        return weight() * g_penalty.value;
    }
};

// the blob phantom of the tests, on the host
std::vector<float> phantom(const int s[3], int dim, double shift)
{
    std::vector<float> img(prod(s, dim));
    const int nz = dim == 3 ? s[2] : 1;
    size_t i = 0;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < s[1]; ++y)
            for (int x = 0; x < s[0]; ++x, ++i) {
                double v = 0;
                for (int b = 0; b < 5; ++b) {
                    const double cx = s[0] * (0.2 + 0.15 * b) + shift, cy = s[1] * (0.7 - 0.1 * b),
                                 cz = nz * (0.3 + 0.1 * b);
                    const double r2 = (x - cx) * (x - cx) + (y - cy) * (y - cy) + (dim == 3 ? (z - cz) * (z - cz) : 0);
                    v += (60.0 + 25.0 * b) * std::exp(-r2 / (2.0 * (3.0 + b) * (3.0 + b)));
                }
                img[i] = float(v);
            }
    return img;
}

}  // namespace

int main(int argc, char **argv)
{
    const int dim = argc > 1 ? std::atoi(argv[1]) : 3;
    const int full[3] = {dim == 3 ? 48 : 96, dim == 3 ? 40 : 80, dim == 3 ? 40 : 1};
    const float rate = dim == 3 ? 8.0f : 16.0f;
    const int levels = dim == 3 ? 3 : 2;
    const std::string init = "spline:rate=" + std::to_string(int(rate)) + ",penalty=[divcurl:weight=2.5,div=1.5,curl=0.5]";
    const int cost = dim == 3 ? MGR_COST_NCC : MGR_COST_SSD;

    GpuImageFullCost fc;
    fc.dim = dim;
    fc.cost = cost;
    for (int k = 0; k < 3; ++k) fc.full[k] = full[k];
    std::vector<float> mov = phantom(full, dim, 1.5), ref = phantom(full, dim, 0.0);
    // joint normalisation of the pair (FScaleFilterCreator, nonrigidregister.cxx:147-184)
    fc.src_full.resize(mov.size());
    fc.ref_full.resize(ref.size());
    double mean = 0, sigma = 0;
    int applied = 0;
    check(mgr_normalize_pair(mov.data(), ref.data(), mov.size(), fc.src_full.data(), fc.ref_full.data(), &mean,
                             &sigma, &applied, 0),
          "normalize");

    Transformation t;
    t.dim = dim;
    GpuDivcurlPenalty pen;
    pen.dim = dim;
    int evals = 0, grids = 0, refines = 0;
    int last_grid[3] = {0, 0, 0};

    // evaluate_fdf (nonrigidregister.cxx:415-439) through the adapter, and
    // the same evaluation on a level made afresh for the current grid
    auto fdf = [&](const std::vector<double> &x, std::vector<double> &g) {
        t.set_parameters(x);
        std::vector<double> gi(x.size(), 0.0), gp(x.size(), 0.0);
        const double ci = fc.evaluate(t, gi);
        const double cp = pen.value_and_gradient(t, gp);
        for (size_t i = 0; i < g.size(); ++i) g[i] = gi[i] + gp[i];
        ++evals;
        if (std::memcmp(last_grid, t.csize, sizeof last_grid) != 0) {
            ++grids;
            std::memcpy(last_grid, t.csize, sizeof last_grid);
        }
        mgr_level_desc d{};
        d.dim = dim;
        for (int k = 0; k < 3; ++k) {
            d.size[k] = fc.size[k];
            d.csize[k] = k < dim ? t.csize[k] : 0;
            d.rate[k] = rate;
        }
        d.cost = cost;
        d.cost_weight = 1.0;
        d.has_penalty = 1;
        d.pen_weight = pen.pen.weight;
        d.pen_div = pen.pen.div;
        d.pen_curl = pen.pen.curl;
        mgr_level *ref_lvl = nullptr;
        check(mgr_level_create(&d, 0, nullptr, &ref_lvl), "reference level");
        check(mgr_level_set_images(ref_lvl, fc.src.data(), fc.ref.data()), "reference images");
        std::vector<double> ri(x.size()), rp(x.size()), rt(x.size());
        double rci = 0, rcp = 0;
        check(mgr_level_evaluate(ref_lvl, t.p.data(), rt.data(), ri.data(), rp.data(), &rci, &rcp), "reference eval");
        mgr_level_destroy(ref_lvl);
        expect(ci == rci, "image cost", ci, rci);
        expect(cp == rcp, "penalty cost", cp, rcp);
        double e = 0, n = 0;
        for (size_t i = 0; i < x.size(); ++i) {
            expect(gi[i] == ri[i], "image gradient", gi[i], ri[i]);
            e += (gp[i] - rp[i]) * (gp[i] - rp[i]);
            n += rp[i] * rp[i];
        }
        expect(e <= 1e-12 * n, "penalty gradient (relative L2 squared)", e, n);
        return ci + cp;
    };
    // a few steps of descent along the normalised gradient: enough to move
    // the coefficients, the check is on every evaluation
    auto minimise = [&](int steps) {
        std::vector<double> x = t.p, g(x.size());
        double f = fdf(x, g), step = 0.5;
        for (int it = 0; it < steps; ++it) {
            double gmax = 0;
            for (double v : g) gmax = std::fmax(gmax, std::fabs(v));
            if (gmax == 0) break;
            std::vector<double> y(x.size()), gy(x.size());
            for (size_t i = 0; i < x.size(); ++i) y[i] = x[i] - step * g[i] / gmax;
            const double fy = fdf(y, gy);
            if (fy < f) {
                x = y;
                g = gy;
                f = fy;
            } else {
                step *= 0.5;
            }
        }
        t.set_parameters(x);
    };

    for (int shift = levels - 1; shift >= 0; --shift) {
        int s[3] = {1, 1, 1};
        for (int k = 0; k < dim; ++k) s[k] = full[k] >> shift;
        fc.set_size(s);
        if (shift == levels - 1)
            t.create(s, rate, init);
        else
            t.upscale(s);
        pen.pen = parse_divcurl(t.creator);
        for (int k = 0; k < 3; ++k) pen.range[k] = t.size[k];
        minimise(4);
        if (t.refine()) {
            ++refines;
            minimise(4);
        }
    }
    std::printf("%s dim=%d levels=%d evaluations=%d grids=%d refines=%d mismatches=%d final grid %dx%dx%d\n",
                failures ? "FAIL" : "ok", dim, levels, evals, grids, refines, failures, t.csize[0], t.csize[1],
                t.csize[2]);
    return failures ? 1 : 0;
}
