// lbm_fixed.cu - kernels of the fixed arithmetic of FP64 handles (lbm_params.arith =
// LBM_ARITH_FIXED): the two-kernel fused step and the materialisation of the module arrays,
// with the per-cell bodies of lbm_fixed_cell.cuh (q60 integer arithmetic on the integer
// pipes, FP64 accuracy).  The fused buffers hold q60 deviations; the module arrays stay the
// plain method's FP64 arrays, so diagnostics, state transfer and restart files are shared
// with the plain method.
#include <cuda_runtime.h>

#include "lbm_fixed.h"
#include "lbm_fixed_cell.cuh"

namespace lbm {

using namespace fxa;

__device__ __forceinline__ bool fixed_cell_of_thread(const Geo& g, long long& c, int& i, int& j, int& k) {
    c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return false;
    cell_coords(g, c, i, j, k);
    return true;
}

template <int D, bool FIRST>
__global__ void __launch_bounds__(128) k_xflow(Geo g, PhysX X, FixedArrays A, const long long* __restrict__ fin,
                                               const long long* __restrict__ gin, long long* __restrict__ fout) {
    long long c;
    int i, j, k;
    if (!fixed_cell_of_thread(g, c, i, j, k)) return;
    flow_cell<D, FIRST>(g, X, A, fin, gin, fout, c, i, j, k);
}

template <int D, bool FIRST>
__global__ void __launch_bounds__(128) k_xthermal(Geo g, PhysX X, FixedArrays A, const long long* __restrict__ fin,
                                                  const long long* __restrict__ gin, long long* __restrict__ gout) {
    long long c;
    int i, j, k;
    if (!fixed_cell_of_thread(g, c, i, j, k)) return;
    thermal_cell<D, FIRST>(g, X, A, fin, gin, gout, c, i, j, k);
}

template <int D>
__global__ void k_xmaterialize(Geo g, PhysX X, FixedArrays A, const long long* __restrict__ fin,
                               const long long* __restrict__ gin) {
    long long c;
    int i, j, k;
    if (!fixed_cell_of_thread(g, c, i, j, k)) return;
    materialize_cell<D>(g, X, A, fin, gin, c, i, j, k);
}

// q60 deviations of a fused buffer -> the FP64 populations they stand for, in place.
__global__ void k_xpost_to_double(long long* buf, long long n, int q, PhysX X, int thermal) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)q * n) return;
    const int a = (int)(e / n);
    const long long rest = thermal ? X.wt[a] : X.w[a];
    const double v = to_double(Qb(buf[e]) + Qb(rest));
    buf[e] = __double_as_longlong(v);
}

static inline unsigned xblocks(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

void fixed_fused_step(const Geo& g, const PhysX& X, const FixedArrays& A, int dim, bool first, const long long* fprev,
                      const long long* gprev, long long* fnext, long long* gnext, cudaStream_t s, int part) {
    const int bs = 128;
    const unsigned nb = xblocks(g.ncell, bs);
    const bool fl = part != 1, th = part != 0;
    if (dim == 2) {
        if (first) {
            if (fl) k_xflow<2, true><<<nb, bs, 0, s>>>(g, X, A, fprev, gprev, fnext);
            if (th) k_xthermal<2, true><<<nb, bs, 0, s>>>(g, X, A, fnext, gprev, gnext);
        } else {
            if (fl) k_xflow<2, false><<<nb, bs, 0, s>>>(g, X, A, fprev, gprev, fnext);
            if (th) k_xthermal<2, false><<<nb, bs, 0, s>>>(g, X, A, fnext, gprev, gnext);
        }
    } else {
        if (first) {
            if (fl) k_xflow<3, true><<<nb, bs, 0, s>>>(g, X, A, fprev, gprev, fnext);
            if (th) k_xthermal<3, true><<<nb, bs, 0, s>>>(g, X, A, fnext, gprev, gnext);
        } else {
            if (fl) k_xflow<3, false><<<nb, bs, 0, s>>>(g, X, A, fprev, gprev, fnext);
            if (th) k_xthermal<3, false><<<nb, bs, 0, s>>>(g, X, A, fnext, gprev, gnext);
        }
    }
}

void fixed_materialize(const Geo& g, const PhysX& X, const FixedArrays& A, int dim, const long long* fcur,
                       const long long* gcur, cudaStream_t s) {
    const unsigned nb = xblocks(g.ncell, 128);
    if (dim == 2) k_xmaterialize<2><<<nb, 128, 0, s>>>(g, X, A, fcur, gcur);
    else k_xmaterialize<3><<<nb, 128, 0, s>>>(g, X, A, fcur, gcur);
}

void fixed_post_to_double(const PhysX& X, long long* fbuf, long long* gbuf, long long n, int q, int qt,
                          cudaStream_t s) {
    k_xpost_to_double<<<xblocks((long long)q * n, 256), 256, 0, s>>>(fbuf, n, q, X, 0);
    k_xpost_to_double<<<xblocks((long long)qt * n, 256), 256, 0, s>>>(gbuf, n, qt, X, 1);
}

}  // namespace lbm
