// lbm_fused.cu - one kernel launch per time step for the FP32 / FP16 storage forms.
//
// The reference's step order (collision, streaming, bounceback, macro, collisionT,
// streamingT, bouncebackT, macroT, 3DRB.F90:227-241) makes the flow collision of step
// n+1 at a cell depend on the thermal collision of step n at its six face neighbours
// (T_n is the sum of the streamed g_post_n), and those on the flow populations around
// them: a cone of radius 2.  This kernel evaluates it in one pass with the thermal
// stage staged in shared memory:
//
//   state read : f_post_n (pulled), g_post_{n-1} (pulled), B_prev_{n-1}  [+ 2D F_y,n]
//   state write: g_post_n, B_prev_n, f_post_{n+1}                         [+ 3D T lag / 2D F_y,n+1]
//
// A block owns a TX x TY tile of the xy plane and marches a chunk of z planes.  For each
// plane it pulls f_post_n and g_post_{n-1} of the tile plus a one-cell halo ring (the
// halo loads are L2 hits: the neighbouring tiles load the same lines), forms rho_n, u_n,
// T_{n-1}, runs the thermal MRT collision, and keeps g_post_n of three consecutive planes
// in a shared-memory ring.  One plane behind, the tile's cells sum the streamed g_post_n
// from the ring (with the thermal wall rules) into T_n and run the flow MRT collision on
// the f_n they pulled one iteration earlier and kept in registers.  Every population is
// read from and written to HBM once per step; the halo's thermal work is recomputed.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lbm_fast.h"
#include "lbm_fast_math.cuh"

namespace lbm {

template <class S>
struct FusedArgs {
    const S* fin;    // f_post_n       (F[cur^1])
    const S* gin;    // g_post_{n-1}   (G[cur])
    const float *Bin0, *Bin1, *Bin2;
    const float* lag_in;  // 2D: F_y,n (L[cur^1])
    S* fout;         // f_post_{n+1}   (F[cur])
    S* gout;         // g_post_n       (G[cur^1])
    float *Bout0, *Bout1, *Bout2;
    float* lag_out;  // 3D: T_{n-1} -> L[cur^1]; 2D: F_y,n+1 -> L[cur]
    const unsigned long long* tick;  // step counter n: g_post_n rounds with n, f_post_{n+1} with n+1
};

template <int D>
struct Tile;
template <> struct Tile<3> { static constexpr int TX = 32, TY = 8, MINB = 2; };
template <> struct Tile<2> { static constexpr int TX = 32, TY = 4, MINB = 4; };

// A stored population as a pull reads it back (ldS).
__device__ __forceinline__ float stored_value(float h) { return h; }
__device__ __forceinline__ float stored_value(__half h) { return __half2float(h); }

// Thermal stage at one cell: pulls, macro, thermal collision.  Returns g_post_n as the
// next pull reads it (the stored deviations, rounded to the storage type and back; halo
// cells round with the owner's random bits, so they hold the owner's values) and, through
// the references, the flow state f_n (deviations), rho_n, u_n.
template <int D, class S>
__device__ __forceinline__ void thermal_cell(const Geo& g, const PhysF& P, const FusedArgs<S>& A, int x, int y, int z,
                                             bool owner, float* d, float& dr, float& rho, float& u, float& v, float& w,
                                             float* GP) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    const long long c = cell_index(g, x, y, z);
    auto lf = [&](int a, long long cc) { return ldS(A.fin, a * n + cc); };
    auto lg = [&](int a, long long cc) { return ldS(A.gin, a * n + cc); };
#pragma unroll
    for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, float>(g, a, x, y, z, c, lf);
    float G[QT], Tprev = 0.0f;
#pragma unroll
    for (int a = 0; a < QT; ++a) {
        G[a] = pull_thermal<QT, float>(g, a, x, y, z, c, lg) + wT<QT>(P, a) * P.Tref;
        Tprev += G[a];
    }
    float Fy;
    fmacro<D>(d, D == 2 ? A.lag_in[c] : Tprev, P, dr, rho, u, v, w, Fy);
    if (D == 2) {
        float Bx = A.Bin0[c], By = A.Bin1[c];
        fcollideT_2d(G, u, v, Tprev, Bx, By, P, GP);
        if (owner) {
            A.Bout0[c] = Bx;
            A.Bout1[c] = By;
        }
    } else {
        float Bx = A.Bin0[c], By = A.Bin1[c], Bz = A.Bin2[c];
        fcollideT_3d(G, u, v, w, Tprev, Bx, By, Bz, P, GP);
        if (owner) {
            A.Bout0[c] = Bx;
            A.Bout1[c] = By;
            A.Bout2[c] = Bz;
            A.lag_out[c] = Tprev;
        }
    }
    float ev[QT];
    S hs[QT];
#pragma unroll
    for (int a = 0; a < QT; ++a) ev[a] = GP[a] - wT<QT>(P, a) * P.Tref;
    round_cell<QT>(ev, hs, P.sr != 0, sr_seed(*A.tick, c, 1));
#pragma unroll
    for (int a = 0; a < QT; ++a) {
        if (owner) A.gout[a * n + c] = hs[a];
        GP[a] = stored_value(hs[a]);
    }
}

// Wrap a coordinate along a periodic axis; return -1 when it is outside a walled axis.
__device__ __forceinline__ int wrap_or_skip(int v, int n, bool periodic) {
    if (v >= 0 && v < n) return v;
    if (!periodic) return -1;
    return v < 0 ? v + n : v - n;
}

// Per-thread placement of one block: own cell and halo-ring cell.
struct Place {
    int tx, ty, x, y;       // own cell (local, global)
    bool own_xy;
    int hx, hy, hgx, hgy;   // halo cell (local ring coordinates, global)
    bool halo;
    bool perx, pery, perz;
    int kb, ke;             // z planes owned by the block
};

// Thermal stage of plane kp into the ring slot `sgs` (layout [QT][HY][HX]); the own
// cell's (dr, rho, u, v, w) go to `keep` when keep_own is set.
template <int D, class S, int HX, int HY>
__device__ __forceinline__ void thermal_plane(const Geo& g, const PhysF& P, const FusedArgs<S>& A, const Place& pl,
                                              float* sgs, int kp, bool keep_own, float* keep) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const int gz = (D == 3) ? wrap_or_skip(kp, g.nz, pl.perz) : 0;
    if (gz < 0) return;
    const bool owned = (D == 2) || (kp >= pl.kb && kp < pl.ke);
    float d[Q], GP[QT], dr, rho, u, v, w;
    if (pl.own_xy) {
        thermal_cell<D, S>(g, P, A, pl.x, pl.y, gz, owned, d, dr, rho, u, v, w, GP);
#pragma unroll
        for (int a = 0; a < QT; ++a) sgs[(a * HY + pl.ty + 1) * HX + pl.tx + 1] = GP[a];
        if (keep_own) {
            keep[0] = dr; keep[1] = rho; keep[2] = u; keep[3] = v; keep[4] = w;
        }
    }
    if (pl.halo) {
        thermal_cell<D, S>(g, P, A, pl.hgx, pl.hgy, gz, false, d, dr, rho, u, v, w, GP);
#pragma unroll
        for (int a = 0; a < QT; ++a) sgs[(a * HY + pl.hy) * HX + pl.hx] = GP[a];
    }
}

// Flow stage of the own cell on plane k: f_n pulled again (the thermal stage loaded the
// same lines one plane earlier), T_n summed from the ring's stored deviations with the
// thermal wall rules in pull_thermal's order and form (so T_n equals the two-kernel
// step's bit for bit), then the MRT collision.  m = (dr, rho, u, v, w) of the cell from the
// thermal stage, whose macro step takes the same pulled f and the same lagged T.
template <int D, class S, int HX, int HY>
__device__ __forceinline__ void flow_cell(const Geo& g, const PhysF& P, const FusedArgs<S>& A, const Place& pl,
                                          const float* s_prev, const float* s_cur, const float* s_next, int k,
                                          const float* m) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    if (!pl.own_xy) return;
    const long long n = g.ncell;
    const int x = pl.x, y = pl.y, lx = pl.tx + 1, ly = pl.ty + 1;
    const long long c = cell_index(g, x, y, k);
    float ts = 0.0f;
#pragma unroll
    for (int a = 0; a < QT; ++a) {
        const int ex = Lat<QT>::ex(a), ey = Lat<QT>::ey(a), ez = Lat<QT>::ez(a);
        int axis = -1;
        bool low = false;
        if (ex != 0 && !pl.perx && (x - ex < 0 || x - ex >= g.nx)) { axis = 0; low = x - ex < 0; }
        if (ey != 0 && !pl.pery && (y - ey < 0 || y - ey >= g.ny)) { axis = 1; low = y - ey < 0; }
        if (ez != 0 && !pl.perz && (k - ez < 0 || k - ez >= g.nz)) { axis = 2; low = k - ez < 0; }
        if (a == 0 || axis < 0) {
            const float* sl = ez > 0 ? s_prev : (ez < 0 ? s_next : s_cur);
            ts += sl[(a * HY + ly - ey) * HX + lx - ex];
        } else {
            const float eopp = s_cur[(Lat<QT>::opp(a) * HY + ly) * HX + lx];
            ts += (pick3(g.bct, axis) == LBM_BCT_CONST) ? (-eopp + (float)(low ? pick3(g.bcT_lo, axis) : pick3(g.bcT_hi, axis)))
                                                         : eopp;
        }
    }
    const float Tn = ts + P.Tref;  // sum of deviations + Tref * sum(wT)
    float d[Q], dp[Q];
    auto lf = [&](int a, long long cc) { return ldS(A.fin, a * n + cc); };
#pragma unroll
    for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, float>(g, a, x, y, k, c, lf);
    const float Fy = m[1] * P.gBeta * (Tn - P.Tref);
    if (D == 2) {
        A.lag_out[c] = Fy;
        fcollide_2d(d, m[0], m[1], m[2], m[3], Fy, P, dp);
    } else {
        fcollide_3d(d, m[0], m[1], m[2], m[3], m[4], Fy, P, dp);
    }
    S hs[Q];
    round_cell<Q>(dp, hs, P.sr != 0, sr_seed(*A.tick + 1, c, 0));
#pragma unroll
    for (int a = 0; a < Q; ++a) A.fout[a * n + c] = hs[a];
}

template <int D, class S>
__global__ void __launch_bounds__(Tile<D>::TX * Tile<D>::TY, Tile<D>::MINB)
    k_fused(Geo g, PhysF P, FusedArgs<S> A, int kchunk) {
    constexpr int TX = Tile<D>::TX, TY = Tile<D>::TY;
    constexpr int HX = TX + 2, HY = TY + 2, NH = 2 * HX + 2 * TY;
    constexpr int QT = (D == 2) ? 5 : 7;
    constexpr int NS = (D == 2) ? 1 : 3;  // planes in the ring
    constexpr int SLOT = QT * HY * HX;
    __shared__ float sg[NS * SLOT];

    Place pl;
    const int t = threadIdx.x;
    pl.tx = t % TX;
    pl.ty = t / TX;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    pl.x = x0 + pl.tx;
    pl.y = y0 + pl.ty;
    pl.own_xy = pl.x < g.nx && pl.y < g.ny;
    pl.perx = g.bct[0] == LBM_BCT_PERIODIC;
    pl.pery = g.bct[1] == LBM_BCT_PERIODIC;
    pl.perz = D == 3 && g.bct[2] == LBM_BCT_PERIODIC;
    pl.kb = (D == 3) ? blockIdx.z * kchunk : 0;
    pl.ke = (D == 3) ? min(g.nz, pl.kb + kchunk) : 1;
    pl.hx = pl.hy = pl.hgx = pl.hgy = -1;
    if (t < NH) {
        if (t < HX) { pl.hx = t; pl.hy = 0; }
        else if (t < 2 * HX) { pl.hx = t - HX; pl.hy = HY - 1; }
        else { const int r = t - 2 * HX; pl.hx = (r & 1) ? HX - 1 : 0; pl.hy = 1 + (r >> 1); }
        pl.hgx = wrap_or_skip(x0 + pl.hx - 1, g.nx, pl.perx);
        pl.hgy = wrap_or_skip(y0 + pl.hy - 1, g.ny, pl.pery);
    }
    pl.halo = pl.hgx >= 0 && pl.hgy >= 0;

    float mc[5] = {0.f, 1.f, 0.f, 0.f, 0.f}, mn[5] = {0.f, 1.f, 0.f, 0.f, 0.f};
    if (D == 2) {
        thermal_plane<D, S, HX, HY>(g, P, A, pl, sg, 0, true, mc);
        __syncthreads();
        flow_cell<D, S, HX, HY>(g, P, A, pl, sg, sg, sg, 0, mc);
        return;
    }
    // 3D: ring slot of plane kp is (kp - kb + 1) mod 3
    const int kb = pl.kb, ke = pl.ke;
    thermal_plane<D, S, HX, HY>(g, P, A, pl, sg + 0 * SLOT, kb - 1, false, mn);
    thermal_plane<D, S, HX, HY>(g, P, A, pl, sg + 1 * SLOT, kb, true, mc);
    for (int k = kb; k < ke; ++k) {
        const int sp = (k - kb) % 3, sc = (k - kb + 1) % 3, sn = (k - kb + 2) % 3;
        thermal_plane<D, S, HX, HY>(g, P, A, pl, sg + sn * SLOT, k + 1, k + 1 < ke, mn);
        __syncthreads();
        flow_cell<D, S, HX, HY>(g, P, A, pl, sg + sp * SLOT, sg + sc * SLOT, sg + sn * SLOT, k, mc);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 5; ++q) mc[q] = mn[q];
    }
}

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
bool fast_fused_supported(const Geo& g, int dim) {
    const int TX = 32;
    // a periodic x axis needs whole tiles so that the wrapped halo lands in the ring
    if ((g.bct[0] == LBM_BCT_PERIODIC) && (g.nx % TX) != 0) return false;
    const int TY = dim == 3 ? 8 : 4;
    if ((g.bct[1] == LBM_BCT_PERIODIC) && (g.ny % TY) != 0) return false;
    return true;
}

void fast_fused_step(FastState& F, const Geo& g0, const PhysC& P, int dim, cudaStream_t s) {
    const PhysF pf = fast_physf(F, P);
    const Geo g = dev_geo(g0, P);
    const int c = F.cur;
    auto launch = [&](auto tag) {
        using S = decltype(tag);
        FusedArgs<S> A;
        A.fin = (const S*)F.fbuf[c ^ 1];
        A.gin = (const S*)F.gbuf[c];
        A.Bin0 = F.B[c][0]; A.Bin1 = F.B[c][1]; A.Bin2 = F.B[c][2];
        A.fout = (S*)F.fbuf[c];
        A.gout = (S*)F.gbuf[c ^ 1];
        A.Bout0 = F.B[c ^ 1][0]; A.Bout1 = F.B[c ^ 1][1]; A.Bout2 = F.B[c ^ 1][2];
        A.tick = F.tick;
        if (dim == 2) {
            A.lag_in = F.L[c ^ 1];
            A.lag_out = F.L[c];
        } else {
            A.lag_in = nullptr;
            A.lag_out = F.L[c ^ 1];
        }
        if (dim == 3) {
            const int kc = F.kchunk > 0 ? F.kchunk : 16;
            dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + kc - 1) / kc);
            k_fused<3, S><<<grid, 256, 0, s>>>(g, pf, A, kc);
        } else {
            dim3 grid((g.nx + 31) / 32, (g.ny + 3) / 4, 1);
            k_fused<2, S><<<grid, 128, 0, s>>>(g, pf, A, 1);
        }
    };
    if (F.precision == LBM_FP16) launch(__half());
    else launch(float());
    fast_tick(F, s);
    F.cur ^= 1;
}

}  // namespace lbm
