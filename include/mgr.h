/*
 * mgr.h — C ABI of libmgr.so: GB300 (sm_103a) implementation of MIA's
 * B-spline nonrigid-registration cost+gradient path.
 *
 * One `mgr_level` holds one image pair at one resolution level on one GPU
 * stream: the `spline` transformation (bspline:d=3 coefficients), the
 * `image` full cost with the `ssd` or `ncc` image cost, and the optional
 * `divcurl` spline penalty.  Every call returns an mgr_status; on failure
 * mgr_last_error() returns a message for the calling thread.  No call throws
 * and no call falls back to the CPU: without a usable GPU the calls fail
 * with MGR_ERR_CUDA.
 *
 * Parameter vectors are laid out as MIA's CDoubleVector for a spline
 * transformation: one (x, y[, z]) double triple per coefficient, x fastest
 * over the coefficient grid (mia/3d/transform/spline.cc:329-358).  Images
 * are float, x fastest.  Host pointers are copied synchronously; the
 * *_device variants take device pointers, run asynchronously on the level's
 * stream and return before completion.
 */
#ifndef MGR_H
#define MGR_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MGR_OK = 0,
    MGR_ERR_ARG = 1,      /* invalid argument (std::invalid_argument in MIA) */
    MGR_ERR_CUDA = 2,     /* CUDA runtime failure or no GPU */
    MGR_ERR_OOM = 3,      /* device allocation failed */
    MGR_ERR_TIMEOUT = 4,  /* a bounded device wait gave up */
    MGR_ERR_STATE = 5     /* call out of order (e.g. evaluate before set_images) */
} mgr_status;

enum { MGR_COST_SSD = 0, MGR_COST_NCC = 1 };

/* Evaluation strategy of the image term.
   MGR_PATH_SPLIT: warp kernel (displacement + tricubic sample + cost sums),
                   then one fused gradient/force/adjoint kernel, then the
                   per-coefficient gather (default, fastest).
   MGR_PATH_PLAIN: one kernel per reference step (dense grid, warp, image
                   gradient, force, separable translate, value) — the plain
                   per-pair drop-in used as the comparison baseline.
   MGR_PATH_FUSED: 3D SSD only: one kernel computes, per tile, the warped
                   image with a one-voxel halo, the force and its adjoint
                   contraction (the warped image is neither stored nor read
                   back), then the per-coefficient gather.  The value-only
                   entry points of such a level run the split path's warp. */
enum { MGR_PATH_SPLIT = 0, MGR_PATH_PLAIN = 1, MGR_PATH_FUSED = 2 };

/* Level description; field names follow the plugin parameters:
   spline:rate, image:cost/weight, ssd:norm, divcurl:weight/div/curl/norm. */
typedef struct {
    int    dim;          /* 2 or 3 */
    int    size[3];      /* image size (x,y,z); size[2] ignored for dim 2 */
    int    csize[3];     /* coefficient grid incl. border; 0 = derive from rate */
    float  rate[3];      /* spline `rate` (coefficient spacing), >= 1 */
    int    cost;         /* MGR_COST_SSD / MGR_COST_NCC */
    int    ssd_norm;     /* ssd `norm` (divide by the number of voxels) */
    double cost_weight;  /* image full-cost `weight` */
    int    has_penalty;  /* 1 if the transformation carries a divcurl penalty */
    double pen_weight;   /* divcurl `weight` */
    double pen_div;      /* divcurl `div` */
    double pen_curl;     /* divcurl `curl` */
    int    pen_norm;     /* divcurl `norm` (divide by the image volume) */
    int    pen_corrected;/* 0: the penalty gradient as the reference returns it,
                            -weight * gradient (mia/3d/splinetransformpenalty.cc:
                            60-71); 1: +weight * gradient, the derivative of the
                            penalty value */
} mgr_level_desc;

typedef struct mgr_level mgr_level;

/* Thread-local message of the last failed call on this thread. */
const char *mgr_last_error(void);

/* Replaces: C3DSplineTransformation ctor + reinit
   (mia/3d/transform/spline.cc:102-147, 224-275), the divcurl penalty
   initialize (mia/3d/splinetransformpenalty.cc:43-49) and the image full
   cost set_size (mia/3d/fullcost/image.cc:80-98).  `stream` is a
   cudaStream_t or NULL for a stream owned by the level.  A caller's stream
   must outlive the level: the level's device buffers are allocated and
   freed in its order. */
mgr_status mgr_level_create(const mgr_level_desc *desc, int device, void *stream,
                            mgr_level **out);
/* Releases the level.  Its device buffers are freed in stream order: on a
   caller's stream, work already queued that reads them completes first and
   destroy does not wait for it; a stream the level created is drained. */
mgr_status mgr_level_destroy(mgr_level *lvl);

/* Coefficient grid and number of parameters (degrees_of_freedom,
   mia/3d/transform/spline.cc:414-418). */
mgr_status mgr_level_csize(const mgr_level *lvl, int csize[3], size_t *nparams);

/* A new coefficient grid for the level's images (kept, with their
   prefiltered coefficients): the spline tables and the divcurl table are
   rebuilt for `csize` (dim entries, each > 3).  Follows the transformation
   where its grid changes while the image size stays: the coefficient grid
   that C3DSplineTransformation::refine grows within a level
   (mia/3d/transform/spline.cc:360-396) and the coarser grid that upscale
   keeps for the next level's size (:399-412, before that level's
   set_size).  A grid equal to the current one changes nothing.  Returns
   after the rebuild; parameters and gradients of later calls have the new
   size. */
mgr_status mgr_level_set_grid(mgr_level *lvl, const int csize[3]);

/* Replaces: C3DImageFullCost::do_reinit + TCost::set_reference
   (mia/3d/fullcost/image.cc:112-128, mia/core/cost.cxx:43-48) and the
   interpolator prefilter (mia/3d/interpolator.cxx:98-164), done once here
   instead of on every warp.  Host pointers, `size` voxels each. */
mgr_status mgr_level_set_images(mgr_level *lvl, const float *src, const float *ref);
mgr_status mgr_level_set_images_device(mgr_level *lvl, const float *d_src, const float *d_ref);

/* Replaces: TNonrigRegGradientProblem::evaluate_fdf
   (mia/template/nonrigidregister.cxx:415-439) = TFullCost::evaluate of the
   image cost (C3DImageFullCost::do_evaluate, mia/3d/fullcost/image.cc:67-78:
   warp, evaluate_force, translate, value) plus the penalty's
   value_and_gradient (mia/3d/splinetransformpenalty.cc:60-71, with its
   reference sign).  Any output pointer may be NULL.
   grad_total = grad_image + grad_penalty, as evaluate_fdf returns it.
   Non-finite parameters: MGR_ERR_ARG, and the output buffers are not
   written. */
mgr_status mgr_level_evaluate(mgr_level *lvl, const double *params, double *grad_total,
                              double *grad_image, double *grad_penalty,
                              double *cost_image, double *cost_penalty);

/* How mgr_level_evaluate moves the caller's host data.  *in_place = 1: the
   level's device reads and writes pageable host memory coherently through
   the host's page tables (Grace-based systems such as GB300) and the level
   is a 3D split-path level; the kernels read `params` and write the
   gradients where the caller holds them, with no staged copy.  *in_place =
   0: the call stages them through device buffers.  MGR_HOST_COPY=1 in the
   environment when the level is created keeps the staged copies.  The
   results are the same bit for bit.  Has no counterpart in the reference. */
mgr_status mgr_level_host_access(const mgr_level *lvl, int *in_place);

/* Device variant: params / grad_total are device pointers (nparams doubles),
   d_costs receives {cost_image, cost_penalty} (2 doubles, device).  The
   kernels are only queued on the level's stream (no synchronisation, no
   finite check of the parameters); a bounded device wait that gave up is
   reported by the next mgr_level_sync. */
mgr_status mgr_level_evaluate_device(mgr_level *lvl, const double *d_params,
                                     double *d_grad_total, double *d_costs);

/* Replaces: TNonrigRegGradientProblem::do_f (nonrigidregister.cxx:376-396):
   C3DImageFullCost::do_value + get_energy_penalty (C3DPPDivcurlMatrix
   operator*, mia/3d/ppmatrix.cc:292-361). */
mgr_status mgr_level_value(mgr_level *lvl, const double *params, double *cost_image,
                           double *cost_penalty);

/* Replaces: Transformation::operator()(image) for the spline transformation
   (mia/3d/transform.cc:280-323) — the warped moving image. */
mgr_status mgr_level_warp(mgr_level *lvl, const double *params, float *out);

/* Replaces: TCost::evaluate_force (mia/core/cost.cxx:37-41) on the warped
   image; writes dim floats per voxel and returns the force-pass cost. */
mgr_status mgr_level_force(mgr_level *lvl, const double *params, float *force,
                           double *cost);

/* Replaces: C3DSplineTransformation::translate / C2DSplineTransformation::
   translate (mia/3d/transform/spline.cc:731-791,
   mia/2d/transform/spline.cc:540-576) for a caller-supplied force field. */
mgr_status mgr_level_translate(mgr_level *lvl, const float *force, double *grad);

/* Select the evaluation strategy (MGR_PATH_*) and, for MGR_PATH_SPLIT, the
   tile shape (0 = autotuned default).  Compiled shapes: 3D 32 x 8 x TZ with
   TZ in {4, 8, 12, 16, 20, 24, 32}; 2D 32 x 8, 32 x 16, 64 x 8, 64 x 16,
   32 x 32; any other shape is MGR_ERR_ARG.  Has no counterpart in the
   reference: it chooses between implementations of the same result. */
mgr_status mgr_level_set_path(mgr_level *lvl, int path, int tile_x, int tile_y, int tile_z);

/* The tile shape the level's split path uses: the autotuner's choice for
   the nearest tuned case (mia_gb300/tiles.json) when it fits the level's
   coefficient spacing, else the shared-memory fit rule; or the shape last
   given to mgr_level_set_path. */
mgr_status mgr_level_tile(const mgr_level *lvl, int tile[3]);

/* Kernel timing for profiling: with `enable` = 1, every evaluation records
   CUDA events around each of its kernels on the level's stream (the
   kernels then run one after another); with `enable` = 2, events around the
   whole evaluation only (the 3D split path's kernels keep their overlapped
   launches, as in an untimed evaluation); 0 turns timing off.
   mgr_level_kernel_times waits for the last evaluation and writes the
   device time in milliseconds of its kernels: ms[0] warp, ms[1]
   gradient/force/adjoint, ms[2] gather+penalty, ms[3] the whole image and
   penalty term (plain path and `enable` = 2: ms[3] only, the others 0).
   Has no counterpart in the reference (it replaces its optional TRACE
   logging of timings). */
mgr_status mgr_level_set_timing(mgr_level *lvl, int enable);
mgr_status mgr_level_kernel_times(mgr_level *lvl, double ms[4]);

/* Spline adjoint (translate, 3D) for callers that cannot allocate device
   memory.  No counterpart in the reference.  Such callers are hosts that
   hand all device memory to their own pool or arena and forbid other
   allocations, and latency-bound callers that cannot afford the implicit
   device synchronisation of cudaMalloc/cudaFree.  The caller passes the
   force field (d_force: size[0]*size[1]*size[2] voxels x 3 floats, device)
   and receives the negated transposed-spline contraction in d_grad (csize
   product x 3 doubles, device): bit for bit the result of
   mgr_level_translate for the same sizes (the same per-axis rows and the
   same three passes).  It runs asynchronously on `stream` (NULL: the legacy
   default stream) of the calling thread's current device and calls no
   allocating function.  Its intermediates live in one fixed 16 MiB device
   array per GPU, which the CUDA runtime sets up when it first loads this
   library's device code on that GPU (under lazy loading, the default, that
   is the first call) and which stays reserved until the process exits;
   sizes needing more are rejected with MGR_ERR_ARG.  The first call on a
   device also looks up that array's device address (once per device), so
   make the first call on each device outside any stream capture.  Calls
   share the array and it keeps the last call's contents: calls whose
   kernels overlap on the GPU (other streams, other host threads) race on
   it and must be serialised by the caller. */
mgr_status mgr_translate3d_noalloc(const int size[3], const int csize[3], const float *d_force,
                                   double *d_grad, void *stream);

/* ---- registration driver ------------------------------------------- */

enum { MGR_MIN_GSL_SD = 0, MGR_MIN_GDSQ = 1 };

/* Minimizer parameters, named as the plugin parameters:
   gsl:opt=gd  -> kind MGR_MIN_GSL_SD, iter=maxiter, step, tol, eps
                  (defaults 100, 0.001, 0.1, 0.01; mia/core/minimizer/gsl.cc:252-273)
   gdsq        -> kind MGR_MIN_GDSQ, maxiter, step, scale, xtola=xtol,
                  gtola=gtol, ftolr, min_step (defaults 100, 0.1, 2, 0, 0, 0,
                  1e-6; mia/core/minimizer/gdsq.cc:127-147) */
typedef struct {
    int    kind;
    int    maxiter;
    double step;
    double tol;
    double eps;
    double scale;
    double xtol, gtol, ftolr, min_step;
} mgr_minimizer_desc;

/* Replaces: TNonrigidRegisterImpl::run (mia/template/nonrigidregister.cxx:
   193-296) for the spline transformation with the image (+ divcurl) cost:
   joint mean-0/sigma-1 normalisation of the pair, `levels` resolution
   levels (size / 2^shift; the `scale` filter builds each level), upscale of
   the transformation between levels, the minimizer on every level and again
   after a refine() that grows the coefficient grid.  `desc` describes the
   full-size problem (desc->csize must be 0: the grid follows `rate`).
   `path` selects the evaluation kernels (MGR_PATH_*); the minimizer runs on
   the host and evaluates through mgr_level_evaluate (one device round trip
   per evaluation: the plain per-pair drop-in).  Writes the final
   coefficient grid, its parameters (max_params doubles), the cost at the
   returned parameters and the number of cost+gradient evaluations.  The
   grid has at most size + 2 coefficients per axis (rate >= 1), so
   prod(size[k] + 2) * dim doubles always suffice; a smaller buffer that
   cannot hold the result is MGR_ERR_ARG after the run. */
mgr_status mgr_register(const mgr_level_desc *desc, int levels, const mgr_minimizer_desc *mz,
                        const float *src, const float *ref, int path, int device,
                        double *params_out, size_t max_params, int csize_out[3],
                        double *final_cost, int *evaluations);

/* Registration of many pairs at once; replaces the per-pair loop of the
   series programs (src/2dmyoset-all2one-nonrigid.cc:124-190,
   src/3dmany2one-nonrigid.cc:118-187), which run one mgr_register-like
   registration per pair in host threads.  All pairs must have the same
   dimension, cost and penalty; sizes may differ.  Each pair follows the same
   levels / refine / minimizer sequence as mgr_register, but the minimizers
   run as device state machines and one step evaluates every unfinished
   pair with one launch per kernel over a (pair, tile) work list.
   `use_graphs` is a set of flags: 1, the steps of each level are captured
   as a CUDA graph; 2 (3D), the warp and adjoint kernels run as persistent
   launches — as many blocks as stay resident, drawing (pair, tile) items
   from a device queue — instead of one block per item (same results bit
   for bit).
   csize_out holds 3 ints per pair; params_out[p] receives max_params[p]
   doubles at most (sized as for mgr_register). */
mgr_status mgr_register_batch(int npairs, const mgr_level_desc *descs, int levels,
                              const mgr_minimizer_desc *mz, const float *const *srcs,
                              const float *const *refs, int device, int use_graphs,
                              double *const *params_out, const size_t *max_params, int *csize_out,
                              double *final_costs, int *evaluations);

/* mgr_register_batch with the images already in device memory (device
   pointers on `device`); no counterpart in the reference, which holds its
   images in host memory. */
mgr_status mgr_register_batch_device(int npairs, const mgr_level_desc *descs, int levels,
                                     const mgr_minimizer_desc *mz, const float *const *d_srcs,
                                     const float *const *d_refs, int device, int use_graphs,
                                     double *const *params_out, const size_t *max_params, int *csize_out,
                                     double *final_costs, int *evaluations);

/* Replaces: the `scale` filter that builds a multiresolution level
   (C3DScale::operator(), mia/3d/filter/scale.cc:95-118; C2DScale,
   mia/2d/filter/scale.cc:50-90); downscaling only.  Host images, run on
   `device`. */
mgr_status mgr_scale_image(int dim, const int in_size[3], const float *in, const int out_size[3],
                           float *out, int device);

/* Replaces: FScaleFilterCreator + the linear convert filter it builds
   (mia/template/nonrigidregister.cxx:147-184): the joint mean-0/sigma-1
   normalisation of a pair.  Writes the normalised images (host), the mean
   and sigma; *applied = 0 when both images hold one value (then nothing is
   written to the outputs). */
mgr_status mgr_normalize_pair(const float *src, const float *ref, size_t n, float *src_out,
                              float *ref_out, double *mean, double *sigma, int *applied, int device);

/* Replaces: C2D/C3DSplineTransformation::refine (mia/3d/transform/spline.cc:
   360-396, mia/2d/transform/spline.cc:318-353), the coefficient grid growing
   between the two passes of a registration level: the dim-vector
   coefficients on the grid nc_old (x fastest, components interleaved,
   rounded to float) prefiltered and resampled onto nc_new, clamped to the
   per-component range, stored as float values.  When no axis grows,
   *grown = 0 and nothing is written; otherwise prod(nc_new) * dim values go
   to out.  Host arrays; the host restatement the per-pair driver uses. */
mgr_status mgr_refine_coefficients(int dim, const int nc_old[3], const int nc_new[3], const double *in,
                                   double *out, int *grown);

/* mgr_refine_coefficients on the device (device pointers, work queued on
   `stream`, nothing waited for): the same operations, each rounded as
   written, so the same values.  The batched driver refines its pairs this
   way. */
mgr_status mgr_refine_coefficients_device(int dim, const int nc_old[3], const int nc_new[3], const double *d_in,
                                          double *d_out, int *grown, void *stream);

/* Replaces: the `xml` transformation IO plugin (mia/3d/transio/xml.cc:55-73,
   mia/2d/transio/xml.cc; fields as mia/3d/transio/serialization.hh:35-83):
   writes a spline transformation — the creator string (e.g.
   "spline:rate=8"), the image size, the attributes (name/value strings) and
   the parameters (prod(csize) * dim, interleaved, x fastest) — as a Boost
   XML archive layout; the coefficient grid is stored as the attribute
   "csize".  Host code only. */
mgr_status mgr_transform_save(const char *path, int dim, const int size[3], const int csize[3],
                              const char *creator, const double *params, size_t nparams,
                              const char *const *attr_names, const char *const *attr_values, int nattr);

/* Reads what mgr_transform_save wrote.  Writes dim, size, csize,
   *nparams; the creator string and the attributes ("name\tvalue\n" lines,
   csize excluded) when their buffers are given (MGR_ERR_ARG, naming the
   size needed, when a string does not fit with its terminating zero); the
   parameters when `params` is given (params_cap >= *nparams).  Call with
   params = NULL to learn *nparams first. */
mgr_status mgr_transform_load(const char *path, int *dim, int size[3], int csize[3], char *creator,
                              size_t creator_cap, char *attrs, size_t attrs_cap, double *params,
                              size_t params_cap, size_t *nparams);

/* Wait for all work queued on the level's stream; MGR_ERR_TIMEOUT when a
   bounded device wait of that work gave up (the flag is then cleared). */
mgr_status mgr_level_sync(mgr_level *lvl);

/* Self-test of the bounded device waits (no counterpart in the reference):
   one thread waits on a barrier that nothing completes, with the warp
   kernel's wait at a limit of 1024 tries.  *gave_up = 1 when the wait ended
   by its limit and raised its flag (the expected result); *us_per_try is
   the time of one failed try, read from the GPU's global nanosecond timer,
   from which the production limit (2^20 tries) takes its duration.  The
   device stays usable afterwards and the calling thread's current device is
   restored. */
mgr_status mgr_selftest_bounded_wait(int device, int *gave_up, double *us_per_try);

/* Number of kernels this library has launched in the calling process
   (for launch accounting in benchmarks). */
unsigned long long mgr_kernel_launch_count(void);

/* Test aids for the out-of-memory paths (no counterpart in the reference,
   whose allocations throw std::bad_alloc).  After mgr_debug_fail_allocation(k)
   with k > 0, the k-th device or page-locked host allocation this library
   makes from then on fails as an exhausted device would, and the call that
   made it returns MGR_ERR_OOM; k = 0 disarms.  Process-wide.
   mgr_allocation_count is the number of such allocations the library has
   made so far in the process. */
mgr_status mgr_debug_fail_allocation(long long k);
unsigned long long mgr_allocation_count(void);

#ifdef __cplusplus
}
#endif
#endif
