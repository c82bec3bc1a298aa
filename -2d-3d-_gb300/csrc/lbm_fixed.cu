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

// Resident blocks per SM asked of the interior flow kernel: 4 (128 registers, no spill) ran
// faster on GB300 than 5 (96 registers and a spill) or 6, at 128^3, 256^3 and 384^3.
#ifndef LBM_XFLOW_MIN_BLOCKS
#define LBM_XFLOW_MIN_BLOCKS 4
#endif

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

// Interior cells (no pull needs a boundary rule) of the steady-state step: block (bx, j, k)
// holds cells i = bx*128 + t of the interior row (j, k), so warps start at row starts (rows
// are 2 KB-aligned when nx is a multiple of 32); threads on the x faces (i = 0, nx-1) do
// nothing, the face kernels take every face cell.  Keeping the boundary code out of these
// kernels keeps them small (instruction fetch) and in fewer registers.
__device__ __forceinline__ bool fixed_interior_cell(const Geo& g, long long& c, int& i, int& j, int& k) {
    i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    j = (int)blockIdx.y + 1;
    k = g.nz > 1 ? (int)blockIdx.z + 1 : 0;
    if (i < 1 || i >= g.nx - 1) return false;
    c = (long long)i + (long long)g.nx * ((long long)j + (long long)g.ny * (long long)k);
    return true;
}

// Face cells: x faces (i = 0, nx-1; all j, k), then y faces (j = 0, ny-1; 0 < i < nx-1; all
// k), then in 3D the z faces (k = 0, nz-1; 0 < i < nx-1; 0 < j < ny-1).
__host__ __device__ __forceinline__ long long fixed_face_count(const Geo& g) {
    const long long nx = g.nx, ny = g.ny, nz = g.nz;
    long long f = 2 * ny * nz + 2 * (nx - 2) * nz;
    if (nz > 1) f += 2 * (nx - 2) * (ny - 2);
    return f;
}
__device__ __forceinline__ bool fixed_face_cell(const Geo& g, long long& c, int& i, int& j, int& k) {
    long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= fixed_face_count(g)) return false;
    const long long nx = g.nx, ny = g.ny, nz = g.nz;
    const long long nxf = 2 * ny * nz, nyf = 2 * (nx - 2) * nz;
    if (f < nxf) {
        i = (f & 1) ? g.nx - 1 : 0;
        j = (int)((f >> 1) % ny);
        k = (int)((f >> 1) / ny);
    } else if ((f -= nxf) < nyf) {
        j = (f & 1) ? g.ny - 1 : 0;
        i = 1 + (int)((f >> 1) % (nx - 2));
        k = (int)((f >> 1) / (nx - 2));
    } else {
        f -= nyf;
        k = (f & 1) ? g.nz - 1 : 0;
        i = 1 + (int)((f >> 1) % (nx - 2));
        j = 1 + (int)((f >> 1) / (nx - 2));
    }
    c = (long long)i + (long long)g.nx * ((long long)j + (long long)g.ny * (long long)k);
    return true;
}

template <int D>
__global__ void __launch_bounds__(128, LBM_XFLOW_MIN_BLOCKS) k_xflow_in(Geo g, PhysX X, FixedArrays A, const long long* __restrict__ fin,
                                                     const long long* __restrict__ gin, long long* __restrict__ fout) {
    long long c;
    int i, j, k;
    if (!fixed_interior_cell(g, c, i, j, k)) return;
    flow_cell<D, false, 1>(g, X, A, fin, gin, fout, c, i, j, k);
}

template <int D>
__global__ void __launch_bounds__(128) k_xflow_face(Geo g, PhysX X, FixedArrays A, const long long* __restrict__ fin,
                                                    const long long* __restrict__ gin, long long* __restrict__ fout) {
    long long c;
    int i, j, k;
    if (!fixed_face_cell(g, c, i, j, k)) return;
    flow_cell<D, false, 2>(g, X, A, fin, gin, fout, c, i, j, k);
}

template <int D>
__global__ void __launch_bounds__(128, 6) k_xthermal_in(Geo g, PhysX X, FixedArrays A,
                                                        const long long* __restrict__ fin,
                                                        const long long* __restrict__ gin, long long* __restrict__ gout) {
    long long c;
    int i, j, k;
    if (!fixed_interior_cell(g, c, i, j, k)) return;
    thermal_cell<D, false, 1>(g, X, A, fin, gin, gout, c, i, j, k);
}

template <int D>
__global__ void __launch_bounds__(128) k_xthermal_face(Geo g, PhysX X, FixedArrays A,
                                                       const long long* __restrict__ fin,
                                                       const long long* __restrict__ gin, long long* __restrict__ gout) {
    long long c;
    int i, j, k;
    if (!fixed_face_cell(g, c, i, j, k)) return;
    thermal_cell<D, false, 2>(g, X, A, fin, gin, gout, c, i, j, k);
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

// Steady-state step of one dimension: interior kernel and face kernel for each half.
template <int D>
static void steady_step(const Geo& g, const PhysX& X, const FixedArrays& A, const long long* fprev,
                        const long long* gprev, long long* fnext, long long* gnext, cudaStream_t s, bool fl, bool th) {
    const dim3 bin(128), gin_grid((unsigned)((g.nx + 127) / 128), (unsigned)(g.ny - 2), D == 3 ? (unsigned)(g.nz - 2) : 1u);
    const unsigned nf = xblocks(fixed_face_count(g), 128);
    if (fl) {
        k_xflow_in<D><<<gin_grid, bin, 0, s>>>(g, X, A, fprev, gprev, fnext);
        k_xflow_face<D><<<nf, 128, 0, s>>>(g, X, A, fprev, gprev, fnext);
    }
    if (th) {
        k_xthermal_in<D><<<gin_grid, bin, 0, s>>>(g, X, A, fnext, gprev, gnext);
        k_xthermal_face<D><<<nf, 128, 0, s>>>(g, X, A, fnext, gprev, gnext);
    }
}

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
            steady_step<2>(g, X, A, fprev, gprev, fnext, gnext, s, fl, th);
        }
    } else {
        if (first) {
            if (fl) k_xflow<3, true><<<nb, bs, 0, s>>>(g, X, A, fprev, gprev, fnext);
            if (th) k_xthermal<3, true><<<nb, bs, 0, s>>>(g, X, A, fnext, gprev, gnext);
        } else {
            steady_step<3>(g, X, A, fprev, gprev, fnext, gnext, s, fl, th);
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
