// lbm_fixed.h - launchers of the fixed arithmetic of FP64 handles (lbm_fixed.cu).
#pragma once

#include <cuda_runtime.h>

#include "lbm_fixed_cell.cuh"

namespace lbm {

// One fused step (part 0: flow kernel, 1: thermal kernel, 2: both) on q60 fused buffers.
// first: the inputs are the FP64 module arrays.  g: deviation geometry (deviation_geo).
// wide: 64-bit cell indices in the interior-row kernels even where 32-bit ones fit.
void fixed_fused_step(const Geo& g, const PhysX& X, const FixedArrays& A, int dim, bool first, const long long* fprev,
                      const long long* gprev, long long* fnext, long long* gnext, cudaStream_t s, int part = 2,
                      bool wide = false);
// The FP64 module arrays of the current step from the q60 fused buffers and the lag.
void fixed_materialize(const Geo& g, const PhysX& X, const FixedArrays& A, int dim, const long long* fcur,
                       const long long* gcur, cudaStream_t s);
// Convert the q60 fused buffers in place to the FP64 post-collision populations of the
// plain method's layout (the handle then continues from its module arrays).
void fixed_post_to_double(const PhysX& X, long long* fbuf, long long* gbuf, long long n, int q, int qt,
                          cudaStream_t s);

// Fused step (3D, nx <= 512): thermal collision of step s and flow collision of step s+1 in
// one launch.  In: f_post_s, g_post_{s-1}, B_prev (bin); out: f_post_{s+1}, g_post_s, B_prev
// (bout, a second set of buffers).
bool fixed_fused_supported(const Geo& g, int dim);
void fixed_fused_pass(const Geo& g, const PhysX& X, const long long* fin, const long long* gin, long long* fout,
                      long long* gout, const long long* const bin[3], long long* const bout[3], cudaStream_t s);

}  // namespace lbm
