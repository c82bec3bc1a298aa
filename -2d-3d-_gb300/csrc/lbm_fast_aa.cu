// lbm_fast_aa.cu - the in-place (AA) access pattern of the FP32/FP16 storage forms, and
// the pattern's helpers shared with the FP64 plain method (face snapshots, module view).
//
// One population array per lattice (fbuf[0], gbuf[0]) whose layout alternates between the
// streamed and the swapped form (lbm_device.cuh).  A step is the two-kernel step of
// lbm_fast.cu with the same per-cell arithmetic in the same order; only the slots a cell
// reads and writes change, so every state equals the two-buffer state bit for bit.  The
// population memory is half the two-buffer form's: the arrays are also the module arrays.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lbm_fast.h"
#include "lbm_fast_cells.cuh"
#include "lbm_fast_pairs.cuh"

namespace lbm {

// Coherent loads for the array a kernel also writes (the read-only path may not be used
// for memory the same kernel stores to).
template <class S> __device__ __forceinline__ float ldA(const S* p, long long i);
template <> __device__ __forceinline__ float ldA<float>(const float* p, long long i) { return p[i]; }
template <> __device__ __forceinline__ float ldA<__half>(const __half* p, long long i) { return __half2float(p[i]); }

// The value the module array of storage type S holds for an arithmetic value x.
template <class S> __device__ __forceinline__ float roundS(float x) { return x; }
template <> __device__ __forceinline__ float roundS<__half>(float x) { return __half2float(__float2half_rn(x)); }

// conversions of the generic helpers (S = double for the FP64 plain method)
template <class S> __device__ __forceinline__ double to_d(S x) { return (double)x; }
template <> __device__ __forceinline__ double to_d<__half>(__half x) { return (double)__half2float(x); }

// ------------------------------------------------------------------------------------
// face snapshots: slot (opp(a), source) of every cell on the far face of a periodic axis,
// stored at [a][face index of the destination cell] (the pull wraps along that axis only,
// so source and destination share their other indices)
// ------------------------------------------------------------------------------------
template <int Q, class S>
__global__ void k_aa_face(Geo g, const S* __restrict__ arr, S* __restrict__ face, int axis) {
    const long long nf = aa_face_cells(g, axis);
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)Q * nf) return;
    const int a = (int)(e / nf);
    const long long f = e - (long long)a * nf;
    const int ea = axis == 0 ? Lat<Q>::ex(a) : (axis == 1 ? Lat<Q>::ey(a) : Lat<Q>::ez(a));
    if (ea == 0) return;
    int i, j, k;
    if (axis == 0) {
        j = (int)(f % g.ny); k = (int)(f / g.ny); i = ea > 0 ? g.nx - 1 : 0;
    } else if (axis == 1) {
        i = (int)(f % g.nx); k = (int)(f / g.nx); j = ea > 0 ? g.ny - 1 : 0;
    } else {
        i = (int)(f % g.nx); j = (int)(f / g.nx); k = ea > 0 ? g.nz - 1 : 0;
    }
    face[e] = arr[(long long)Lat<Q>::opp(a) * g.ncell + cell_index(g, i, j, k)];
}

template <int Q, class S>
static void face_launch(const Geo& g, const void* arr, void* const face[3], cudaStream_t s) {
    for (int ax = 0; ax < 3; ++ax) {
        if (!face[ax]) continue;
        const long long cnt = (long long)Q * aa_face_cells(g, ax);
        k_aa_face<Q, S><<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(g, (const S*)arr, (S*)face[ax], ax);
    }
}

template <class S>
static void face_dispatch(const Geo& g, int q, const void* arr, void* const face[3], cudaStream_t s) {
    switch (q) {
        case 19: face_launch<19, S>(g, arr, face, s); break;
        case 9: face_launch<9, S>(g, arr, face, s); break;
        case 7: face_launch<7, S>(g, arr, face, s); break;
        default: face_launch<5, S>(g, arr, face, s); break;
    }
}

void aa_snapshot(const Geo& g, int q, bool, int precision, const void* arr, void* const face[3], cudaStream_t s) {
    if (precision == LBM_FP64) face_dispatch<double>(g, q, arr, face, s);
    else if (precision == LBM_FP32) face_dispatch<float>(g, q, arr, face, s);
    else face_dispatch<__half>(g, q, arr, face, s);
}

// ------------------------------------------------------------------------------------
// module view: the streamed population of (cell, a) read through the array's layout
// ------------------------------------------------------------------------------------
template <int Q, bool THERMAL, class S, class T>
__global__ void k_aa_view(Geo g, const S* __restrict__ arr, int par, int raw, double* __restrict__ out, int soa,
                          int dev, double w0, double w1) {
    const long long n = g.ncell;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)Q * n) return;
    const long long c = e / Q;
    const int a = (int)(e - c * Q);
    int i, j, k;
    cell_coords(g, c, i, j, k);
    auto ld = [&](int b, long long cc) { return (T)to_d<S>(arr[(long long)(par ? Lat<Q>::opp(b) : b) * n + cc]); };
    T v;
    if (THERMAL) v = par ? pull_thermal<Q, T>(g, a, i, j, k, c, ld) : aa_local_thermal<Q, T>(g, a, i, j, k, c, raw != 0, ld);
    else v = par ? pull_flow<Q, T>(g, a, i, j, k, c, ld) : ld(a, c);
    double r = (double)v;
    if (dev) {
        const double rest = THERMAL ? (a == 0 ? w0 : w1) : wrest<(Q == 9 || Q == 5) ? 9 : 19>(a);
        r = rest + (double)roundS<S>((float)v);
    }
    out[soa ? (long long)a * n + c : e] = r;
}

template <class S, class T>
static void view_launch(const Geo& g, int q, bool thermal, const void* arr, int par, bool raw, double* out, bool soa,
                        bool dev, double w0, double w1, cudaStream_t s) {
    const unsigned nb = (unsigned)(((long long)q * g.ncell + 255) / 256);
    const S* p = (const S*)arr;
    const int r = raw ? 1 : 0, so = soa ? 1 : 0, dv = dev ? 1 : 0;
    if (thermal) {
        if (q == 7) k_aa_view<7, true, S, T><<<nb, 256, 0, s>>>(g, p, par, r, out, so, dv, w0, w1);
        else k_aa_view<5, true, S, T><<<nb, 256, 0, s>>>(g, p, par, r, out, so, dv, w0, w1);
    } else {
        if (q == 19) k_aa_view<19, false, S, T><<<nb, 256, 0, s>>>(g, p, par, r, out, so, dv, w0, w1);
        else k_aa_view<9, false, S, T><<<nb, 256, 0, s>>>(g, p, par, r, out, so, dv, w0, w1);
    }
}

void aa_module_view(const Geo& g, int q, bool thermal, int precision, const void* arr, int par, bool raw, double* out,
                    bool soa, bool dev, double w0, double w1, cudaStream_t s) {
    if (precision == LBM_FP64) view_launch<double, double>(g, q, thermal, arr, par, raw, out, soa, false, w0, w1, s);
    else if (precision == LBM_FP32) view_launch<float, float>(g, q, thermal, arr, par, raw, out, soa, dev, w0, w1, s);
    else view_launch<__half, float>(g, q, thermal, arr, par, raw, out, soa, dev, w0, w1, s);
}

// ------------------------------------------------------------------------------------
// FP32/FP16 step kernels, one cell per thread (the arithmetic of flow_cell_2k and
// thermal_cell_2k).  ODD: the kernel's own array is in the swapped layout.  FIRST is a
// template parameter as in the two-buffer kernels: with FMA contraction allowed, a value
// merged from two paths at run time could be rounded differently downstream.
// ------------------------------------------------------------------------------------
template <int D, class S, bool ODD, bool FIRST>
__global__ void __launch_bounds__(128) k_aa_flow_f(Geo g, PhysF P, FastArgs<S> A, S* f, const S* __restrict__ gs,
                                                   AAFace<S> wf, int gpar, int graw) {
    long long c;
    int i, j, k;
    if (!fcell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    float d[Q], dp[Q], dr, rho, u, v, w = 0.0f, T;
    if (ODD) {
        auto lf = [&](int b, long long cc) { return ldA(f, Lat<Q>::opp(b) * n + cc); };
        auto wr = [&](int ax, int b, long long) {
            return ldA(aa_face_ptr(wf, ax), b * aa_face_cells(g, ax) + aa_face_index(g, ax, i, j, k));
        };
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = pull_flow_w<Q, float>(g, a, i, j, k, c, lf, wr);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldA(f, a * n + c);
    }
    if (FIRST) {
        rho = A.rho[c];
        dr = rho - 1.0f;
        u = A.u[c];
        v = A.v[c];
        if (D == 3) w = A.w[c];
        T = A.T[c];
    } else {
        float ts = 0.0f;
        if (gpar) {
            auto lg = [&](int b, long long cc) { return ldS(gs, Lat<QT>::opp(b) * n + cc); };
#pragma unroll
            for (int a = 0; a < QT; ++a) ts += pull_thermal<QT, float>(g, a, i, j, k, c, lg);
        } else {
            auto lg = [&](int b, long long cc) { return ldS(gs, b * n + cc); };
#pragma unroll
            for (int a = 0; a < QT; ++a) ts += aa_local_thermal<QT, float>(g, a, i, j, k, c, graw != 0, lg);
        }
        T = ts + P.Tref;
        float Fy;
        fmacro<D>(d, A.lag_in[c], P, dr, rho, u, v, w, Fy);
    }
    const float Fy = rho * P.gBeta * (T - P.Tref);
    if (D == 2) {
        A.lag_out[c] = Fy;
        fcollide_2d(d, dr, rho, u, v, Fy, P, dp);
    } else {
        fcollide_3d(d, dr, rho, u, v, w, Fy, P, dp);
    }
    if (ODD) {
        auto st = [&](int b, long long cc, float val) { f[b * n + cc] = toS<S>(val); };
#pragma unroll
        for (int a = 0; a < Q; ++a) aa_push<Q, false, float>(g, a, i, j, k, c, dp[a], st);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) f[Lat<Q>::opp(a) * n + c] = toS<S>(dp[a]);
    }
}

template <int D, class S, bool ODD, bool FIRST>
__global__ void __launch_bounds__(128) k_aa_thermal_f(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fs, S* gg,
                                                      AAFace<S> wg, int fpar, int graw) {
    long long c;
    int i, j, k;
    if (!fcell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    float d[Q], G[QT], GP[QT];
    if (fpar) {
        auto lf = [&](int b, long long cc) { return ldS(fs, Lat<Q>::opp(b) * n + cc); };
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, float>(g, a, i, j, k, c, lf);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldS(fs, a * n + c);
    }
    float e[QT];
    if (ODD) {
        auto lg = [&](int b, long long cc) { return ldA(gg, Lat<QT>::opp(b) * n + cc); };
        auto wr = [&](int ax, int b, long long) {
            return ldA(aa_face_ptr(wg, ax), b * aa_face_cells(g, ax) + aa_face_index(g, ax, i, j, k));
        };
#pragma unroll
        for (int a = 0; a < QT; ++a) e[a] = pull_thermal_w<QT, float>(g, a, i, j, k, c, lg, wr);
    } else {
        auto lg = [&](int b, long long cc) { return ldA(gg, b * n + cc); };
#pragma unroll
        for (int a = 0; a < QT; ++a) e[a] = aa_local_thermal<QT, float>(g, a, i, j, k, c, graw != 0, lg);
    }
    float Tprev;
    if (FIRST) {
        // the module array holds each value rounded to the storage type
#pragma unroll
        for (int a = 0; a < QT; ++a) G[a] = roundS<S>(e[a]) + wT<QT>(P, a) * P.Tref;
        Tprev = A.T[c];
    } else {
        float ts = 0.0f;
#pragma unroll
        for (int a = 0; a < QT; ++a) {
            G[a] = e[a] + wT<QT>(P, a) * P.Tref;
            ts += G[a];
        }
        Tprev = ts;
    }
    float dr, rho, u, v, w, Fy;
    fmacro<D>(d, D == 2 ? A.lag_in[c] : Tprev, P, dr, rho, u, v, w, Fy);
    if (D == 2) {
        float Bx = A.Bin0[c], By = A.Bin1[c];
        fcollideT_2d(G, u, v, Tprev, Bx, By, P, GP);
        A.Bout0[c] = Bx;
        A.Bout1[c] = By;
    } else {
        float Bx = A.Bin0[c], By = A.Bin1[c], Bz = A.Bin2[c];
        fcollideT_3d(G, u, v, w, Tprev, Bx, By, Bz, P, GP);
        A.Bout0[c] = Bx;
        A.Bout1[c] = By;
        A.Bout2[c] = Bz;
        A.lag_out[c] = Tprev;
    }
    if (ODD) {
        auto st = [&](int b, long long cc, float val) { gg[b * n + cc] = toS<S>(val); };
#pragma unroll
        for (int a = 0; a < QT; ++a) aa_push<QT, true, float>(g, a, i, j, k, c, GP[a] - wT<QT>(P, a) * P.Tref, st);
    } else {
#pragma unroll
        for (int a = 0; a < QT; ++a) gg[Lat<QT>::opp(a) * n + c] = toS<S>(GP[a] - wT<QT>(P, a) * P.Tref);
    }
}

// Module scalars (rho, u, v, w, T) of the current step, populations left in place.
template <int D, class S>
__global__ void k_aa_materialize_f(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fs,
                                   const S* __restrict__ gs, int fpar, int gpar, int graw) {
    long long c;
    int i, j, k;
    if (!fcell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    float d[Q];
    if (fpar) {
        auto lf = [&](int b, long long cc) { return ldS(fs, Lat<Q>::opp(b) * n + cc); };
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, float>(g, a, i, j, k, c, lf);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldS(fs, a * n + c);
    }
    float ts = 0.0f;
    if (gpar) {
        auto lg = [&](int b, long long cc) { return ldS(gs, Lat<QT>::opp(b) * n + cc); };
#pragma unroll
        for (int a = 0; a < QT; ++a) ts += pull_thermal<QT, float>(g, a, i, j, k, c, lg) + wT<QT>(P, a) * P.Tref;
    } else {
        auto lg = [&](int b, long long cc) { return ldS(gs, b * n + cc); };
#pragma unroll
        for (int a = 0; a < QT; ++a)
            ts += aa_local_thermal<QT, float>(g, a, i, j, k, c, graw != 0, lg) + wT<QT>(P, a) * P.Tref;
    }
    float dr, rho, u, v, w, Fy;
    fmacro<D>(d, A.lag_in[c], P, dr, rho, u, v, w, Fy);
    A.rho[c] = rho;
    A.u[c] = u;
    A.v[c] = v;
    if (D == 3) A.w[c] = w;
    A.T[c] = ts;
}

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
template <class S>
static FastArgs<S> aa_args(const FastState& F) {
    FastArgs<S> a;
    a.fref = (S*)F.fref;
    a.gref = (S*)F.gref;
    a.rho = F.rho; a.u = F.u; a.v = F.v; a.w = F.w; a.T = F.T;
    a.Bin0 = F.B[0][0]; a.Bin1 = F.B[0][1]; a.Bin2 = F.B[0][2];
    a.Bout0 = F.B[0][0]; a.Bout1 = F.B[0][1]; a.Bout2 = F.B[0][2];
    a.lag_in = F.L[0];
    a.lag_out = F.L[0];
    return a;
}

template <class S>
static AAFace<S> aa_faces(void* const face[3]) {
    return AAFace<S>{(const S*)face[0], (const S*)face[1], (const S*)face[2]};
}

static bool any_face(void* const face[3]) { return face[0] || face[1] || face[2]; }

template <int D, class S, bool FIRST>
static void aa_step_launch(FastState& F, const Geo& g, const PhysF& pf, cudaStream_t s, int part) {
    AAState& st = F.AA;
    const FastArgs<S> A = aa_args<S>(F);
    S* f = (S*)F.fbuf[0];
    S* gg = (S*)F.gbuf[0];
    const unsigned nb = (unsigned)((g.ncell + 127) / 128);
    const int raw = st.graw ? 1 : 0;
    if (part != 1) {
        if (st.fpar && any_face(st.face_f)) aa_snapshot(g, F.q, false, F.precision, f, st.face_f, s);
        const AAFace<S> wf = aa_faces<S>(st.face_f);
        if (st.fpar) k_aa_flow_f<D, S, true, FIRST><<<nb, 128, 0, s>>>(g, pf, A, f, gg, wf, st.gpar, raw);
        else k_aa_flow_f<D, S, false, FIRST><<<nb, 128, 0, s>>>(g, pf, A, f, gg, wf, st.gpar, raw);
        st.fpar ^= 1;
    }
    if (part != 0) {
        if (st.gpar && any_face(st.face_g)) aa_snapshot(g, F.qt, true, F.precision, gg, st.face_g, s);
        const AAFace<S> wg = aa_faces<S>(st.face_g);
        if (st.gpar) k_aa_thermal_f<D, S, true, FIRST><<<nb, 128, 0, s>>>(g, pf, A, f, gg, wg, st.fpar, raw);
        else k_aa_thermal_f<D, S, false, FIRST><<<nb, 128, 0, s>>>(g, pf, A, f, gg, wg, st.fpar, raw);
        if (st.gpar) st.graw = true;
        st.gpar ^= 1;
    }
}

template <int D, class S>
static void aa_step_first(FastState& F, const Geo& g, const PhysF& pf, bool first, cudaStream_t s, int part) {
    if (first) aa_step_launch<D, S, true>(F, g, pf, s, part);
    else aa_step_launch<D, S, false>(F, g, pf, s, part);
}

void fast_step_aa(FastState& F, const Geo& g, const PhysF& pf, int dim, bool first, cudaStream_t s, int part) {
    if (F.precision == LBM_FP16) {
        if (dim == 2) aa_step_first<2, __half>(F, g, pf, first, s, part);
        else aa_step_first<3, __half>(F, g, pf, first, s, part);
    } else {
        if (dim == 2) aa_step_first<2, float>(F, g, pf, first, s, part);
        else aa_step_first<3, float>(F, g, pf, first, s, part);
    }
}

void fast_materialize_aa(FastState& F, const Geo& g, const PhysF& pf, int dim, cudaStream_t s) {
    const unsigned nb = (unsigned)((g.ncell + 127) / 128);
    const AAState& st = F.AA;
    const int raw = st.graw ? 1 : 0;
    if (F.precision == LBM_FP16) {
        const FastArgs<__half> A = aa_args<__half>(F);
        const __half *f = (const __half*)F.fbuf[0], *gg = (const __half*)F.gbuf[0];
        if (dim == 2) k_aa_materialize_f<2, __half><<<nb, 128, 0, s>>>(g, pf, A, f, gg, st.fpar, st.gpar, raw);
        else k_aa_materialize_f<3, __half><<<nb, 128, 0, s>>>(g, pf, A, f, gg, st.fpar, st.gpar, raw);
    } else {
        const FastArgs<float> A = aa_args<float>(F);
        const float *f = (const float*)F.fbuf[0], *gg = (const float*)F.gbuf[0];
        if (dim == 2) k_aa_materialize_f<2, float><<<nb, 128, 0, s>>>(g, pf, A, f, gg, st.fpar, st.gpar, raw);
        else k_aa_materialize_f<3, float><<<nb, 128, 0, s>>>(g, pf, A, f, gg, st.fpar, st.gpar, raw);
    }
}

}  // namespace lbm
