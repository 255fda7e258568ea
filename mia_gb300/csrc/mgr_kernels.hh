// mgr_kernels.hh — host-side launchers of the libmgr kernels.
#pragma once

#include <cuda.h>

#include <vector>
#include <cuda_runtime.h>
#include <stddef.h>

#include "mgr_common.cuh"

namespace mgr {

// launch accounting (mgr_kernel_launch_count); while a thread records a
// graph it pauses its own counting (count_launch_pause), and the graph's
// launches are counted when it runs
void count_launch(unsigned n = 1);
// SMs of the current device (cached per device, thread-safe)
int device_sm_count();
void count_launch_pause(bool paused);

// Every device and page-locked host allocation of the library goes through
// these three, so that mgr_debug_fail_allocation can make a chosen one fail
// as an out-of-memory would (the allocation-failure paths are tested
// without exhausting a device).
cudaError_t dev_malloc_async(void **p, size_t bytes, cudaStream_t s);
cudaError_t dev_malloc(void **p, size_t bytes);
cudaError_t host_malloc_pinned(void **p, size_t bytes);

// cudaFuncSetAttribute(kernel, MaxDynamicSharedMemorySize, bytes) on the
// current device, made only when `bytes` exceeds what was set for that
// kernel and device before (the limit only grows): a launch of an
// evaluation then makes no driver call for it
void raise_smem_limit(const void *kernel, size_t bytes);

void launch_prefilter(float *img, int dim, int nx, int ny, int nz, cudaStream_t st);
// padded copy with the mirror fold applied in the halo (layout of coef_pad)
void launch_pad_mirror(const float *img, float *pad, int dim, int nx, int ny, int nz, cudaStream_t st);
// the padded image's size in floats
size_t pad_floats(int dim, int nx, int ny, int nz);
void launch_minmax(const float *img, size_t n, float2 *part, int nblocks, unsigned int *counter,
                   float *out, cudaStream_t st);

// 3D: tensor map of the padded copy (box 64 x 16 x 1 floats, the
// warp kernel's shared-memory ring planes); false if the driver offers no
// tensor-map encoder (the kernel then reads its taps from global memory)
bool encode_pad_tmap(CUtensorMap *map, const float *pad, int nx, int ny, int nz);

// ---- the evaluation pipeline ----------------------------------------
struct EvalArgs {
    CUtensorMap tmap;      // 3D: encode_pad_tmap of coef_pad (first: 64-byte aligned)
    int has_tmap;
    int dim;
    int n[3];              // image size
    int nc[3];             // coefficient grid
    Axis ax[3];            // per-axis tables (ax[2] unused in 2D)
    const float *coef_img; // prefiltered moving image
    const float *coef_pad; // the same with a mirror halo of PAD_H voxels (3D: all axes, 2D: x and y)
    int pad_rows;          // rows per plane of coef_pad (ny + 2 PAD_H); the row pitch is pad_pitch(nx)
    const float *ref;      // reference image
    float *warped;         // warped moving image (N)
    const float *minmax;   // device {min, max} clamp bounds
    const double *params;  // spline parameters, interleaved, device
    float *params_f;       // 3D: their float copy (launch_params_f32), read by the warp and gather kernels
    int cost;              // MGR_COST_SSD / NCC
    int ssd_norm;
    double cost_weight;
    const double *centers; // device {mean src, mean ref}: NCC provisional centres
                           // (sums are taken around them to reduce cancellation)
    // tile partials and reductions
    float *partial;        // per tile adjoint footprint partials
    int slot;              // floats per tile slot
    double *tile_sums;     // per warp tile: 5 doubles
    unsigned int *counters;// [0] warp, [1] gather, [2] penalty value
    double *scalars;       // SC_* slots
    // penalty
    int has_penalty;
    double pen_weight;     // effective weight (norm already applied)
    double pen_grad_sign;  // -1: the reference's penalty gradient sign, +1: corrected
    int pen_equal_w;       // div == curl (multiply skips the cross terms)
    const float *ptable;   // 3D: 9x9x9 cells x 6 floats (xx, xy, yy, yz, zz, xz)
    const int *pen_rowptr; // 2D: CSR rows of the boundary-clipped matrix
    const int *pen_col;
    const float4 *pen_val; // 2D: (vx, vy, v12, 0)
    double *pen_part;      // per gather block: penalty value partial
    // outputs (device)
    double *grad_total;
    double *grad_image;    // optional
    double *grad_penalty;  // optional
    double *costs;         // optional {cost_image, cost_penalty}
    // caller's host memory read and written in place (a device with
    // coherent access to pageable host memory, 3D split path): params_host
    // is read by the parameter conversion (launch_params_f32), and the
    // gather's last block writes {cost_image, cost_penalty, status flags}
    // to host_out; the gradient pointers above may then be host memory too
    const double *params_host;
    double *host_out;
    // 1: the cost is finalised after the warp kernel from its tile sums
    // (the warp blocks then end without a device-wide fence and last-block
    // reduction): an SSD cost by the gather's last block (the adjoint takes
    // its force scale from the settings), an NCC cost by k_finalise3, which
    // launch_warp3 queues right after the warp kernel; 0: the warp kernel's
    // last block finalises the cost
    int defer_cost;
    // 1: the 3D split path's warp, adjoint and gather kernels are launched
    // with programmatic stream serialisation (each may start while the one
    // before it finishes, and waits for it before reading its outputs)
    int pdl;
};

// SPLIT path: warp (+cost sums), gradient/force/adjoint, gather(+penalty)
void launch_warp(const EvalArgs &a, cudaStream_t st);
void launch_adjoint(const EvalArgs &a, cudaStream_t st);
void launch_gather(const EvalArgs &a, int with_gradient, cudaStream_t st);
// dense = 1: the image gradient is read from a.grad_image (plain path)
void launch_gather_mode(const EvalArgs &a, int with_gradient, int dense, cudaStream_t st);
int  gather_blocks(const EvalArgs &a);
// tile shapes compiled into the split path
bool tile_supported(int dim, int tx, int ty, int tz);

// batched split path: one launch per phase over a work list of
// (pair, tile) items (which = 0 warp, 1 adjoint) or (pair, block) items
// (gather); pairs with active[pair] == 0 are skipped
size_t split_smem(const EvalArgs &a, int which);
void prepare_split_batch(int dim, int tx, int ty, int tz, size_t sm_warp, size_t sm_adj);
bool launch_split_batch(int dim, int tx, int ty, int tz, const EvalArgs *args, const int2 *items, int nitems,
                        const int *active, size_t smem, int which, cudaStream_t st);
void launch_gather_batch(int dim, const EvalArgs *args, const int2 *items, int nitems, const int *active,
                         const int *nblocks, int has_penalty, cudaStream_t st);

// 3D split path (split3.cu): tiles of 32 x 8 x tz voxels, z-walking threads;
// launch_warp3 converts the parameters to float first (launch_params_f32)
void launch_params_f32(const EvalArgs &a, cudaStream_t st);
// (the batched driver's minimizer writes the float copy with each trial point)
bool tile_supported3(int tx, int ty, int tz);
bool tile_supported3_batch(int tx, int ty, int tz);
size_t split3_smem(const EvalArgs &a, int which);
void launch_warp3(const EvalArgs &a, cudaStream_t st);
void launch_adjoint3(const EvalArgs &a, cudaStream_t st);
// persistent batched 3D warp (which = 0) and adjoint (1) kernels: `grid`
// resident blocks draw the items from the device queue queue[0..1] (zero
// before the first launch; the last block resets it)
int split3_queue_grid(int tz, int which, size_t sm);
void launch_split3_queue(int tz, const EvalArgs *args, const int2 *items, int nitems, const int *active, int *queue,
                         int grid, size_t sm, int which, cudaStream_t st);
// the fused SSD kernel (fused3.cu): warp, force and adjoint in one pass per
// 30 x 8 x TZ tile; with_gradient = 0 sums the cost only
bool tile_supported_fused3(int tx, int ty, int tz);
size_t fused3_smem(const EvalArgs &a);
void launch_fused3(const EvalArgs &a, int with_gradient, cudaStream_t st);
int gather3_blocks(const EvalArgs &a);
void launch_gather3(const EvalArgs &a, int with_gradient, int dense, cudaStream_t st);
void prepare_split3_batch(int tz, size_t sm_warp, size_t sm_adj);
void launch_split3_batch(int tz, const EvalArgs *args, const int2 *items, int nitems, const int *active, size_t sm,
                         int which, cudaStream_t st);
void launch_gather3_batch(const EvalArgs *args, const int2 *items, int nitems, const int *active, const int *nblocks,
                          cudaStream_t st);

// standalone pieces for tests and the plain path
void launch_force(const EvalArgs &a, float *force, cudaStream_t st);       // force field from `warped`
void launch_translate(const EvalArgs &a, const float *force, double *grad, float *tmp1,
                      float *tmp2, cudaStream_t st);                         // plain separable adjoint
void launch_plain_eval(const EvalArgs &a, float *grid, float *force, float *tmp1, float *tmp2,
                       cudaStream_t st);                                     // PLAIN path image term

// refine_params (driver.cc) on the device for several coefficient fields
// at once (same operations, each rounded as written: the same values).
// in: nc_old product x dim parameters, out: nc_new product x dim; device
// pointers, work queued on st (refine.cu)
struct RefineJobSpec {
    int nc_old[3], nc_new[3];
    const double *in;
    double *out;
};
void refine_params_device(int dim, const std::vector<RefineJobSpec> &jobs, cudaStream_t st);

}  // namespace mgr
