/*
 * mgr_oracle.h — C interface of the CPU oracle for the B-spline nonrigid
 * registration cost+gradient path of MIA (gerddie/mia).
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a CPU restatement of the
 * reference algorithm, used by the tests as the checker and by bench.py as
 * the timed CPU baseline.  The product library (libmgr.so) never links or
 * calls it.
 *
 * Two precisions are provided:
 *   ORC_PREC_REF  — the reference's own float/double mix (float images,
 *                   float coefficients and forces, double weights and sums);
 *   ORC_PREC_F64  — every quantity in double, used to state the error of a
 *                   result against an FP64 evaluation of the same algorithm.
 */
#ifndef MGR_ORACLE_H
#define MGR_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_PREC_REF = 0, ORC_PREC_F64 = 1 };
enum { ORC_COST_SSD = 0, ORC_COST_NCC = 1 };

/* ---- primitives (each follows one reference routine) ------------------ */
int    orc_fastfloor(double x);
void   orc_bspline3_weights(double x, double w[4]);
void   orc_bspline3_dweights(double x, double w[4]);
void   orc_bspline3_deriv_weights(double x, int degree, double w[4]);
double orc_bspline3_at(double x, int degree);
int    orc_mirror_fold(int index, int width);
void   orc_filter_line(double *coeff, int n);
void   orc_prefilter(const float *in, float *out, int dim, const int size[3]);
void   orc_prefilter_vec_d(const double *in, double *out, int ncomp, int dim, const int size[3]);
double orc_simpson_integrate2(double s1, double s2, int deg1, int deg2, double x0, double L);
void   orc_gradient(const float *img, float *grad, int dim, const int size[3]);
double orc_ssd_value(const float *a, const float *b, size_t n, int norm);
double orc_ssd_force(const float *a, const float *b, float *force, int dim, const int size[3], int norm);
double orc_ncc_value(const float *a, const float *b, size_t n);
double orc_ncc_force(const float *a, const float *b, float *force, int dim, const int size[3]);
void   orc_ncc_sums(const float *a, const float *b, size_t n, double sums[6]);

/* divcurl matrix on an explicit coefficient grid; coefficient vectors are
   interleaved (x,y[,z]) per node, x fastest; `grad` may be NULL.  With
   `as_float` the coefficients are first rounded to float (the registration
   path stores them as float vectors).  `mode` 0 = value+gradient
   (evaluate), 1 = value only (operator*). */
double orc_divcurl_matrix(int dim, const int csize[3], const float range[3],
                          double wdiv, double wrot, const double *coeffs,
                          double *grad, int as_float, int mode);

/* the divcurl P tables themselves (for checks of other builders): 3D the
   9x9x9 cells of offsets i - j, six doubles each (xx, xy, yy, yz, zz, xz),
   cell index (dx + 4) + 9 ((dy + 4) + 9 (dz + 4)); 2D the nonzero cells
   (i, j, xx, yy, xy) grouped by row i; returns the number of cells, of
   which at most `cap` are written. */
void   orc_divcurl_table3(const int csize[3], const float range[3], double wdiv, double wrot, double *out);
size_t orc_divcurl_cells2(const int csize[2], const float range[2], double wd, double wr, int *i, int *j,
                          double *v, size_t cap);

/* ---- one registration level (transform + image full cost + penalty) -- */
typedef struct OrcLevel OrcLevel;

typedef struct {
    int    dim;            /* 2 or 3 */
    int    size[3];        /* image size (x,y,z); z ignored for dim 2 */
    int    csize[3];       /* coefficient grid incl. border; 0 = from rate */
    float  rate[3];        /* spline coefficient rate (c_rate) */
    int    cost;           /* ORC_COST_SSD / ORC_COST_NCC */
    int    ssd_norm;       /* ssd plugin `norm` */
    double cost_weight;    /* image full-cost weight */
    int    has_penalty;    /* divcurl spline penalty present */
    double pen_weight;     /* penalty `weight` */
    double pen_div;        /* penalty `div` */
    double pen_curl;       /* penalty `curl` */
    int    pen_norm;       /* penalty `norm` */
    int    precision;      /* ORC_PREC_* */
    int    threads;        /* host threads (z-slab / row parallel for) */
} OrcLevelDesc;

OrcLevel *orc_level_create(const OrcLevelDesc *desc);
void      orc_level_destroy(OrcLevel *lvl);
int       orc_level_csize(const OrcLevel *lvl, int csize[3]);   /* returns #params */
void      orc_level_set_images(OrcLevel *lvl, const float *src, const float *ref);
/* cost+gradient exactly as TNonrigRegGradientProblem::evaluate_fdf:
   g_img = weighted image-cost gradient, g_pen = penalty gradient (reference
   sign), returns cost_img + cost_pen.  Either gradient pointer may be NULL. */
double    orc_level_evaluate(OrcLevel *lvl, const double *params, double *g_img,
                             double *g_pen, double *cost_img, double *cost_pen);
/* value only, as TNonrigRegGradientProblem::do_f */
double    orc_level_value(OrcLevel *lvl, const double *params, double *cost_img,
                          double *cost_pen);
void      orc_level_warp(OrcLevel *lvl, const double *params, float *out);
void      orc_level_displacement(OrcLevel *lvl, const double *params, float *u);
void      orc_level_force(OrcLevel *lvl, const double *params, float *force);
void      orc_level_translate(OrcLevel *lvl, const float *force, double *g);

/* ---- registration driver -------------------------------------------- */
enum { ORC_MIN_GSL_SD = 0, ORC_MIN_GDSQ = 1 };
typedef struct {
    int    kind;
    int    maxiter;
    double step;
    double tol;       /* gsl: step factor after a failed trial */
    double eps;       /* gsl: stop when |g| < eps */
    double scale;     /* gdsq */
    double xtol, gtol, ftolr, min_step;   /* gdsq */
} OrcMinimizer;

int  orc_normalize_pair(const float *src, const float *ref, size_t n, float *src_out, float *ref_out,
                        double *mean, double *sigma);
void orc_scale_image(const float *in, int dim, const int in_size[3], float *out, const int out_size[3]);
int  orc_refine(int dim, const int nc_old[3], const int nc_new[3], const double *params, double *out,
                size_t max_out);
/* TNonrigidRegisterImpl::run for the spline transformation; returns the
   number of parameters written or -1 */
int  orc_register(const OrcLevelDesc *desc, int levels, const OrcMinimizer *mz, const float *src,
                  const float *ref, double *params_out, int max_params, int csize_out[3],
                  double *final_cost, int *evals_out);
/* the minimizers on the analytic problem of the reference's gdsq test */
double orc_minimize_test_problem(const OrcMinimizer *mz, double x[2], int *evals);

#ifdef __cplusplus
}
#endif
#endif
