// driver.hh — host side of the registration driver: minimizers and the
// spline transformation's level transitions (upscale, refine).
#pragma once

#include <functional>
#include <vector>

#include "../../include/mgr.h"

namespace mgr {

// f(x, g): cost and gradient at x (the minimizer problem's fdf)
using FDF = std::function<double(const std::vector<double> &, std::vector<double> &)>;

struct MinResult {
    double f = 0.0;      // cost at the returned x
    int iterations = 0;
    int evaluations = 0;
    int status = 0;      // 0 success/stopped, 1 no progress, 2 max iterations
};

// gsl_multimin_fdfminimizer_steepest_descent as CGSLFDFMinimizer::do_run
// drives it (mia/core/minimizer/gsl.cc:122-156)
MinResult minimize_gsl_sd(std::vector<double> &x, const mgr_minimizer_desc &mz, const FDF &fdf);
// CGDSQMinimizer::do_run (mia/core/minimizer/gdsq.cc:60-122)
MinResult minimize_gdsq(std::vector<double> &x, const mgr_minimizer_desc &mz, const FDF &fdf);
MinResult minimize(std::vector<double> &x, const mgr_minimizer_desc &mz, const FDF &fdf);

// coefficient grid that C2D/C3DSplineTransformation::refine targets
// (mia/3d/transform/spline.cc:363-364, mia/2d/transform/spline.cc:321-322)
int refine_csize(int size, float rate);

// spline parameters stored as float coefficients (set_parameters /
// get_parameters round trip)
void round_params_to_float(std::vector<double> &p);

// do_upscale (mia/3d/transform/spline.cc:399-412; 2D spline.cc:356-370):
// coefficients scaled by size/range (3D) or (size-1)/(range-1) (2D), the
// grid is kept
void upscale_params(int dim, const int old_size[3], const int new_size[3], std::vector<double> &p);

// refine (mia/3d/transform/spline.cc:360-396; 2D spline.cc:318-353): the
// coefficient field is interpolated onto the finer grid `nc_new` with the
// cubic B-spline (mirror boundary, per-component clamp).  Returns false and
// leaves p unchanged when no axis grows.
bool refine_params(int dim, const int nc_old[3], const int nc_new[3], std::vector<double> &p);

// whether refine_params moves the coefficients to `nc_new` (some axis grows)
bool refine_grows(int dim, const int nc_old[3], const int nc_new[3]);

// the constants of refine's line prefilter for a line of n coefficients
// (pole p = sqrt(3) - 2, gain lambda, 1/p, p / (p^2 - 1), p^(n-1))
struct RefineFilterConsts {
    double p, lambda, iz, q, z2n;
};
RefineFilterConsts refine_filter_consts(int n);

// refine's resampling taps on one axis: 4 coefficient indices (mirrored at
// the borders) and cubic B-spline weights per line of the new grid
void refine_axis_taps(int n_old, int n_new, std::vector<int> &idx, std::vector<double> &w);

}  // namespace mgr
