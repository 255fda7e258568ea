// pyramid.hh — multiresolution image preparation (see pyramid.cu).
#pragma once

#include <vector>

#include <cuda_runtime.h>
#include <stddef.h>

#include <string>

namespace mgr {

// %g formatting (6 significant digits), as a C++ stream writes a double
std::string format_g6(double v);

// Joint mean-0 / sigma-1 normalisation of a pair; returns false (and writes
// nothing) when both images hold a single value.
bool normalize_pair(const float *d_src, const float *d_ref, size_t n, float *d_src_out, float *d_ref_out,
                    cudaStream_t st, double *mean_out, double *sigma_out);

// normalize_pair for several pairs with one host synchronisation for all
// the sums (the same partial sums per pair, so the same results); returns
// per pair whether its images vary (0: both images of one value, nothing
// written, or with copy_first the images copied unchanged); copy_first: the
// sums pass also copies the images to the outputs and the linear map runs
// there in place (inputs in host memory are then read once)
std::vector<char> normalize_pairs(const std::vector<const float *> &src, const std::vector<const float *> &ref,
                                  const std::vector<size_t> &n, const std::vector<float *> &src_out,
                                  const std::vector<float *> &ref_out, cudaStream_t st,
                                  bool copy_first = false);

// The `scale` filter (downscaling only); a copy when the sizes agree.
void scale_image(const float *d_in, const int in_size[3], float *d_out, const int out_size[3], int dim,
                 cudaStream_t st);

}  // namespace mgr
