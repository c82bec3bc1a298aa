// lbm_reduce.cu - FP64 diagnostics reductions and layout transforms.
//
// Each diagnostic of the reference (check, calNuRe, RBcalc_Nu_global, the sums of
// RBcalc_Nu_wall_avg) is a sum over cells of a per-cell term.  Here every thread forms
// the reference's per-cell term in FP64 (from FP64 or FP32 fields), accumulates a
// grid-stride slice, the warp folds its partials with __shfl_down_sync, the block folds
// the warps through shared memory, and block b writes its partials to slot b.  The host
// adds the per-block partials in block order, so results are reproducible run to run
// (the reference's OpenMP reductions combine thread partials in an unspecified order,
// so only the per-cell terms, not the sums, can match it bit for bit).
#include <cuda_runtime.h>

#include <cmath>

#include "lbm_internal.h"

namespace lbm {

constexpr int kRedThreads = 256;
constexpr int kRedMaxBlocks = 152 * 8;  // 8 blocks of 256 threads per SM on 152 SMs

int diag_blocks(long long ncell) {
    long long nb = (ncell + kRedThreads - 1) / kRedThreads;
    if (nb > kRedMaxBlocks) nb = kRedMaxBlocks;
    if (nb < 1) nb = 1;
    return (int)nb;
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    return x;
}

template <int N>
__device__ __forceinline__ void block_store(double (&acc)[N], double* out) {
    __shared__ double sh[kRedThreads / 32][N];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < N; ++s) acc[s] = warp_sum(acc[s]);
    if (lane == 0) {
#pragma unroll
        for (int s = 0; s < N; ++s) sh[wid][s] = acc[s];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int s = 0; s < N; ++s) {
            double x = (lane < kRedThreads / 32) ? sh[lane][s] : 0.0;
            x = warp_sum(x);
            if (lane == 0) out[(long long)blockIdx.x * N + s] = x;
        }
    }
}

template <class S>
__device__ __forceinline__ double ld(const S* p, long long c) {
    return (double)p[c];
}

// A cell is "bad" when it holds a non-finite temperature or velocity or a density <= 0
// (the reference's restart check, 3DRB.F90:1423, extended to the running state).
template <class S>
__device__ __forceinline__ double bad_cell(const DiagFields<S>& F, long long c, bool d3) {
    const double u = ld(F.u, c), v = ld(F.v, c), T = ld(F.T, c);
    const double w = d3 ? ld(F.w, c) : 0.0;
    const double r = F.rho ? ld(F.rho, c) : 1.0;
    return (isfinite(u) && isfinite(v) && isfinite(w) && isfinite(T) && r > 0.0) ? 0.0 : 1.0;
}

template <class S, int OP>
__global__ void __launch_bounds__(kRedThreads) k_diag(Geo g, DiagScalars D, DiagFields<S> F, double* partials) {
    double acc[DIAG_NSUM] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const bool d3 = D.d3 != 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    if (OP == DIAG_NU_COLD_MID_SIDE) {
        // one thread per (j,k) row: cold (right) wall term and x mid-plane term
        const long long nrow = (long long)g.ny * g.nz;
        for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < nrow; row += stride) {
            const int j = (int)(row % g.ny), k = (int)(row / g.ny);
            auto T = [&](int i) { return ld(F.T, cell_index(g, i, j, k)); };
            auto U = [&](int i) { return ld(F.u, cell_index(g, i, j, k)); };
            const int nx = g.nx;
            // Nu_cold (2DRB.F90:1908-1912, 3DRB.F90:1990-1997)
            const double qx_wall = (-8.0 * D.Tcold + 9.0 * T(nx - 1) - T(nx - 2)) / (3.0 * D.dy);
            acc[0] += qx_wall / D.deltaT;
            // Nu_middle (2DRB.F90:1916-1931, 3DRB.F90:2000-2021)
            if (nx % 2 == 1) {
                const int im = (nx + 1) / 2 - 1;
                acc[1] += (D.coef * U(im) * (T(im) - D.Tref) + (T(im - 1) - T(im + 1)) / (2.0 * D.dy)) / D.deltaT;
            } else {
                const int iL = nx / 2 - 1, iR = iL + 1;
                if (d3)
                    acc[1] += (D.coef * 0.5 * (U(iL) * (T(iL) - D.Tref) + U(iR) * (T(iR) - D.Tref)) + (T(iL) - T(iR)) / D.dy) / D.deltaT;
                else
                    acc[1] += (D.coef * (0.5 * (U(iL) * (T(iL) - D.Tref) + U(iR) * (T(iR) - D.Tref))) + (T(iL) - T(iR)) / D.dy) / D.deltaT;
            }
        }
        block_store(acc, partials);
        return;
    }
    if (OP == DIAG_NU_COLD_MID) {
        // one thread per (i,k) column: cold wall term and mid-plane term
        const long long ncol = (long long)g.nx * g.nz;
        for (long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x; col < ncol; col += stride) {
            const int i = (int)(col % g.nx), k = (int)(col / g.nx);
            auto T = [&](int j) { return ld(F.T, cell_index(g, i, j, k)); };
            auto V = [&](int j) { return ld(F.v, cell_index(g, i, j, k)); };
            const int ny = g.ny;
            // Nu_cold (2DRB.F90:2423-2428, 3DRB.F90:2145-2152)
            const double qy_wall = (-8.0 * D.Tcold + 9.0 * T(ny - 1) - T(ny - 2)) / (3.0 * D.dy);
            acc[0] += qy_wall / D.deltaT;
            // Nu_middle (2DRB.F90:2433-2457, 3DRB.F90:2156-2180)
            if (ny % 2 == 1) {
                const int jm = (ny + 1) / 2 - 1;
                acc[1] += (D.coef * V(jm) * (T(jm) - D.Tref) - (T(jm + 1) - T(jm - 1)) / (2.0 * D.dy)) / D.deltaT;
            } else {
                const int jB = ny / 2 - 1, jT = jB + 1;
                if (d3)
                    acc[1] += (D.coef * 0.5 * (V(jB) * (T(jB) - D.Tref) + V(jT) * (T(jT) - D.Tref)) + (T(jB) - T(jT)) / D.dy) / D.deltaT;
                else
                    acc[1] += (D.coef * (0.5 * (V(jB) * (T(jB) - D.Tref) + V(jT) * (T(jT) - D.Tref))) + (T(jB) - T(jT)) / D.dy) / D.deltaT;
            }
        }
        block_store(acc, partials);
        return;
    }
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < g.ncell; c += stride) {
        if (OP == DIAG_CHECK) {
            // check (2DRB.F90:1233-1246, 3DRB.F90:1491-1520)
            const double u = ld(F.u, c), v = ld(F.v, c), T = ld(F.T, c);
            const double du = u - ld(F.up, c), dv = v - ld(F.vp, c);
            double e1 = du * du + dv * dv, e2 = u * u + v * v;
            if (d3) {
                const double w = ld(F.w, c), dw = w - ld(F.wp, c);
                e1 = e1 + dw * dw;
                e2 = e2 + w * w;
                F.wp[c] = F.w[c];
            }
            acc[0] += e1;
            acc[1] += e2;
            acc[2] += fabs(T - ld(F.Tp, c));
            acc[3] += fabs(T);
            acc[4] += bad_cell(F, c, d3);
            F.up[c] = F.u[c];
            F.vp[c] = F.v[c];
            F.Tp[c] = F.T[c];
        } else if (OP == DIAG_NURE) {
            // calNuRe (2DRB.F90:1631-1663, 3DRB.F90:1731-1768)
            const double u = ld(F.u, c), v = ld(F.v, c), T = ld(F.T, c);
            acc[0] += (D.side ? u : v) * T;
            double r = u * u + v * v;
            if (d3) {
                const double w = ld(F.w, c);
                r = r + w * w;
            }
            acc[1] += r;
            acc[4] += bad_cell(F, c, d3);
        } else if (OP == DIAG_NU_GLOBAL_SIDE) {
            // SideHeatedcalc_Nu_global (2DRB.F90:1700-1720, 3DRB.F90:1801-1817)
            int i, j, k;
            cell_coords(g, c, i, j, k);
            auto T = [&](int ii) { return ld(F.T, cell_index(g, ii, j, k)); };
            double dTdx;
            if (i == 0) dTdx = (-3.0 * T(0) - T(1) + 4.0 * D.Thot) / (3.0 * D.dy);
            else if (i == g.nx - 1) dTdx = (-4.0 * D.Tcold + 3.0 * T(g.nx - 1) + T(g.nx - 2)) / (3.0 * D.dy);
            else dTdx = (T(i - 1) - T(i + 1)) / (2.0 * D.dy);
            acc[0] += D.coef * ld(F.u, c) * (T(i) - D.Tref) + dTdx;
        } else {
            // RBcalc_Nu_global (2DRB.F90:2268-2288, 3DRB.F90:1851-1866)
            int i, j, k;
            cell_coords(g, c, i, j, k);
            auto T = [&](int jj) { return ld(F.T, cell_index(g, i, jj, k)); };
            double dTdy;
            if (j == 0) dTdy = (3.0 * T(0) + T(1) - 4.0 * D.Thot) / (3.0 * D.dy);
            else if (j == g.ny - 1) dTdy = (4.0 * D.Tcold - 3.0 * T(g.ny - 1) - T(g.ny - 2)) / (3.0 * D.dy);
            else dTdy = (T(j + 1) - T(j - 1)) / (2.0 * D.dy);
            acc[0] += D.coef * ld(F.v, c) * (T(j) - D.Tref) - dTdy;
        }
    }
    block_store(acc, partials);
}

template <class S>
void diag_reduce(DiagOp op, const Geo& g, const DiagScalars& D, const DiagFields<S>& F, double* partials, int nb,
                 cudaStream_t s) {
    switch (op) {
        case DIAG_CHECK: k_diag<S, DIAG_CHECK><<<nb, kRedThreads, 0, s>>>(g, D, F, partials); break;
        case DIAG_NURE: k_diag<S, DIAG_NURE><<<nb, kRedThreads, 0, s>>>(g, D, F, partials); break;
        case DIAG_NU_GLOBAL: k_diag<S, DIAG_NU_GLOBAL><<<nb, kRedThreads, 0, s>>>(g, D, F, partials); break;
        case DIAG_NU_COLD_MID: k_diag<S, DIAG_NU_COLD_MID><<<nb, kRedThreads, 0, s>>>(g, D, F, partials); break;
        case DIAG_NU_GLOBAL_SIDE: k_diag<S, DIAG_NU_GLOBAL_SIDE><<<nb, kRedThreads, 0, s>>>(g, D, F, partials); break;
        case DIAG_NU_COLD_MID_SIDE:
            k_diag<S, DIAG_NU_COLD_MID_SIDE><<<nb, kRedThreads, 0, s>>>(g, D, F, partials);
            break;
    }
}

template <class S>
__global__ void k_wall_columns(Geo g, DiagScalars D, const S* __restrict__ T, double* Tb, double* Nub) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.nx) return;
    // 3DRB.F90:2067-2087 (2D: 2DRB.F90:2330-2336 is the nz = 1 case of the same sums)
    double tb = 0.0, nb = 0.0;
    for (int k = 0; k < g.nz; ++k) tb = tb + (double)T[cell_index(g, i, 0, k)];
    for (int k = 0; k < g.nz; ++k) {
        const double qy_wall = (8.0 * D.Thot - 9.0 * (double)T[cell_index(g, i, 0, k)] + (double)T[cell_index(g, i, 1, k)]) / (3.0 * D.dy);
        nb = nb + qy_wall / D.deltaT;
    }
    Tb[i] = tb / (double)g.nz;
    Nub[i] = nb / (double)g.nz;
}

template <class S>
void diag_wall_columns(const Geo& g, const DiagScalars& D, const S* T, double* Tb, double* Nub, cudaStream_t s) {
    k_wall_columns<S><<<(g.nx + 127) / 128, 128, 0, s>>>(g, D, T, Tb, Nub);
}

template <class S>
__global__ void k_wall_rows(Geo g, DiagScalars D, const S* __restrict__ T, double* Tl, double* Nul) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.ny) return;
    // 3DRB.F90:1905-1925 (2D: 2DRB.F90:1776-1781 is the nz = 1 case of the same sums)
    double tl = 0.0, nl = 0.0;
    for (int k = 0; k < g.nz; ++k) tl = tl + (double)T[cell_index(g, 0, j, k)];
    for (int k = 0; k < g.nz; ++k) {
        const double qx_wall = (8.0 * D.Thot - 9.0 * (double)T[cell_index(g, 0, j, k)] + (double)T[cell_index(g, 1, j, k)]) / (3.0 * D.dy);
        nl = nl + qx_wall / D.deltaT;
    }
    Tl[j] = tl / (double)g.nz;
    Nul[j] = nl / (double)g.nz;
}

template <class S>
void diag_wall_rows(const Geo& g, const DiagScalars& D, const S* T, double* Tl, double* Nul, cudaStream_t s) {
    k_wall_rows<S><<<(g.ny + 127) / 128, 128, 0, s>>>(g, D, T, Tl, Nul);
}

// The plane `idx` normal to `axis` of a field, contiguous in FP64:
//   axis 0: out[j + ny k] = f(idx, j, k);  axis 1: out[i + nx k];  axis 2: out[i + nx j].
template <class S>
__global__ void k_gather_plane(Geo g, const S* __restrict__ f, int axis, int idx, double* out) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n1 = axis == 0 ? g.ny : g.nx, n2 = axis == 2 ? g.ny : g.nz;
    if (e >= n1 * n2) return;
    const int a = (int)(e % n1), b = (int)(e / n1);
    const long long c = axis == 0 ? cell_index(g, idx, a, b) : (axis == 1 ? cell_index(g, a, idx, b) : cell_index(g, a, b, idx));
    out[e] = (double)f[c];
}

template <class S>
void diag_gather_plane(const Geo& g, const S* f, int axis, int idx, double* out, cudaStream_t s) {
    const long long n1 = axis == 0 ? g.ny : g.nx, n2 = axis == 2 ? g.ny : g.nz;
    k_gather_plane<S><<<(unsigned)((n1 * n2 + 255) / 256), 256, 0, s>>>(g, f, axis, idx, out);
}

template void diag_reduce<double>(DiagOp, const Geo&, const DiagScalars&, const DiagFields<double>&, double*, int, cudaStream_t);
template void diag_reduce<float>(DiagOp, const Geo&, const DiagScalars&, const DiagFields<float>&, double*, int, cudaStream_t);
template void diag_wall_columns<double>(const Geo&, const DiagScalars&, const double*, double*, double*, cudaStream_t);
template void diag_wall_columns<float>(const Geo&, const DiagScalars&, const float*, double*, double*, cudaStream_t);
template void diag_wall_rows<double>(const Geo&, const DiagScalars&, const double*, double*, double*, cudaStream_t);
template void diag_wall_rows<float>(const Geo&, const DiagScalars&, const float*, double*, double*, cudaStream_t);
template void diag_gather_plane<double>(const Geo&, const double*, int, int, double*, cudaStream_t);
template void diag_gather_plane<float>(const Geo&, const float*, int, int, double*, cudaStream_t);

// ---- fine-grid |psi| search (calc_psi_absmax_fine_spline, 2DRB.F90:2873-2998) ----------
// The reference interpolates psi on a grid of nFinePerUnit points per unit length with
// natural cubic splines: first along x on every coarse row, then along y on every fine x
// column, and keeps the first point of largest |psi| in (x outer, y inner) order.  Here a
// thread per (fine x, coarse row) evaluates the row splines, and a block per fine x builds
// its column spline in shared memory and scans the fine y points; ties go to the smallest
// (k, l), which is the sequential scan's choice.
__device__ double d_splint(int n, const double* xa, const double* ya, const double* y2a, double x) {
    int klo = 1, khi = n;
    while (khi - klo > 1) {
        const int k = (khi + klo) / 2;
        if (xa[k - 1] > x) khi = k;
        else klo = k;
    }
    const double h = xa[khi - 1] - xa[klo - 1];
    if (h == 0.0) return ya[klo - 1];
    const double a = (xa[khi - 1] - x) / h;
    const double b = (x - xa[klo - 1]) / h;
    return a * ya[klo - 1] + b * ya[khi - 1] +
           ((a * a * a - a) * y2a[klo - 1] + (b * b * b - b) * y2a[khi - 1]) * (h * h) / 6.0;
}

__device__ void d_spline_natural(int n, const double* x, const double* y, double* y2, double* u) {
    y2[0] = 0.0;
    u[0] = 0.0;
    for (int i = 2; i <= n - 1; ++i) {
        const double sig = (x[i - 1] - x[i - 2]) / (x[i] - x[i - 2]);
        const double p = sig * y2[i - 2] + 2.0;
        y2[i - 1] = (sig - 1.0) / p;
        u[i - 1] = (6.0 * ((y[i] - y[i - 1]) / (x[i] - x[i - 1]) - (y[i - 1] - y[i - 2]) / (x[i - 1] - x[i - 2])) /
                        (x[i] - x[i - 2]) - sig * u[i - 2]) / p;
    }
    y2[n - 1] = 0.0;
    for (int k = n - 1; k >= 1; --k) y2[k - 1] = y2[k - 1] * y2[k] + u[k - 1];
}

// psi_xfine(k, j) for k < nFineX, j < ny: rows[j] = [0, psi(1..nx, j), 0], y2rows[j] its spline
__global__ void k_psi_rows(int nx, int ny, int nFineX, double xLen, const double* xExt, const double* rows,
                           const double* y2rows, double* xfine) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nFineX * ny) return;
    const int k = (int)(e % nFineX), j = (int)(e / nFineX);
    const double xq = xLen * (double)k / (double)(nFineX - 1);
    xfine[(long long)k * ny + j] = d_splint(nx + 2, xExt, rows + (size_t)j * (nx + 2), y2rows + (size_t)j * (nx + 2), xq);
}

__global__ void k_psi_columns(int ny, int nFineX, int nFineY, double yLen, const double* yExt, const double* xfine,
                              double* best_val, int* best_l) {
    extern __shared__ double sh[];
    const int n = ny + 2;
    double* col = sh;
    double* y2 = sh + n;
    double* uu = sh + 2 * n;
    __shared__ double red_v[256];
    __shared__ int red_l[256];
    const int k = blockIdx.x;
    if (threadIdx.x == 0) {
        col[0] = 0.0;
        col[n - 1] = 0.0;
        for (int j = 0; j < ny; ++j) col[j + 1] = xfine[(long long)k * ny + j];
        d_spline_natural(n, yExt, col, y2, uu);
    }
    __syncthreads();
    double bv = -1.0;
    int bl = 0x7fffffff;
    for (int l = threadIdx.x; l < nFineY; l += blockDim.x) {
        const double yq = yLen * (double)l / (double)(nFineY - 1);
        const double a = fabs(d_splint(n, yExt, col, y2, yq));
        if (a > bv) {  // the first (smallest l) of this thread's largest values
            bv = a;
            bl = l;
        }
    }
    red_v[threadIdx.x] = bv;
    red_l[threadIdx.x] = bl;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            const double v2 = red_v[threadIdx.x + o];
            const int l2 = red_l[threadIdx.x + o];
            if (v2 > red_v[threadIdx.x] || (v2 == red_v[threadIdx.x] && l2 < red_l[threadIdx.x])) {
                red_v[threadIdx.x] = v2;
                red_l[threadIdx.x] = l2;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        best_val[k] = red_v[0];
        best_l[k] = red_l[0];
    }
}

int psi_fine_search(int nx, int ny, double xLen, double yLen, int nFineX, int nFineY, const double* xExt,
                    const double* yExt, const double* rows, const double* y2rows, double* xfine, double* best_val,
                    int* best_l, cudaStream_t s) {
    const long long ne = (long long)nFineX * ny;
    k_psi_rows<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(nx, ny, nFineX, xLen, xExt, rows, y2rows, xfine);
    const size_t shm = (size_t)3 * (ny + 2) * sizeof(double);
    if (shm > 48 * 1024) return LBM_ERR_PARAM;
    k_psi_columns<<<nFineX, 256, shm, s>>>(ny, nFineX, nFineY, yLen, yExt, xfine, best_val, best_l);
    return cudaGetLastError() == cudaSuccess ? LBM_OK : LBM_ERR_CUDA;
}

// ---- layout transforms ----------------------------------------------------------------
__global__ void k_aos_to_soa(const double* __restrict__ aos, double* __restrict__ soa, int q, long long n) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)q * n) return;
    const long long c = e / q;
    const int a = (int)(e - c * q);
    soa[(long long)a * n + c] = aos[e];
}

__global__ void k_soa_to_aos(const double* __restrict__ soa, double* __restrict__ aos, int q, long long n) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)q * n) return;
    const long long c = e / q;
    const int a = (int)(e - c * q);
    aos[e] = soa[(long long)a * n + c];
}

__global__ void k_copy_doubles(const double* __restrict__ src, double* __restrict__ dst, long long n) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) dst[e] = src[e];
}

void copy_doubles(const double* src, double* dst, long long n, cudaStream_t s) {
    k_copy_doubles<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, n);
}

void aos_to_soa(const double* aos, double* soa, int q, long long ncell, cudaStream_t s) {
    const long long tot = (long long)q * ncell;
    k_aos_to_soa<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(aos, soa, q, ncell);
}

void soa_to_aos(const double* soa, double* aos, int q, long long ncell, cudaStream_t s) {
    const long long tot = (long long)q * ncell;
    k_soa_to_aos<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(soa, aos, q, ncell);
}

}  // namespace lbm
