// lbm_ensemble.cu - one flow launch and one thermal launch per time step for any number of
// FP32/FP16 lattices of uneven sizes and parameters (the batched form).
//
// A grid of about SMs x grid_mul persistent blocks walks a packed tile table: tile t is
// (member m, first cell c0) and covers tile_cells consecutive cells of member m.  Each
// block reads the member's descriptor (geometry, relaxation rates, buffer pointers and
// parity), then runs the same per-cell bodies as the single-lattice two-kernel step
// (lbm_fast_cells.cuh) on its cells.  Small lattices therefore fill the GPU together
// instead of one launch each.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <vector>

#include "lbm_ensemble.h"
#include "lbm_fast_cells.cuh"

namespace lbm {

template <class S>
struct EnsMember {
    Geo g;      // wall terms in deviation form
    PhysF P;
    S* f[2];
    S* gp[2];
    float* B[2][3];
    float* L[2];
    unsigned long long* tick;  // the member's step counter (stochastic rounding of FP16)
    int cur;    // buffer parity when the table was built
};

// Fixed-offset pulls for the cells off the faces (lbm_fast_cells.cuh), and two resident
// blocks per SM (the 3D thermal kernel otherwise takes 242 registers, one block): measured
// on GB300, 64 2D RB instances (8.4 M cells) 1.4x faster in FP32 and 2.8x in FP16, twelve
// 3D instances of 64^3-192^3 (23.5 M cells) 2.1x in FP32.
template <int D>
constexpr bool kEnsInner = true;

// Cell coordinates of a thread's cells in a tile, stepped instead of divided: one division
// at the tile's first cell, then (i, j, k) advance by blockDim.x cells with carries (i by
// less than a row; j may wrap several planes on narrow lattices).
struct CellWalk {
    long long c;
    int i, j, k, di, dj;
    __device__ __forceinline__ CellWalk(const Geo& g, long long c0) : c(c0) {
        cell_coords(g, c0, i, j, k);
        di = (int)(blockDim.x % (unsigned)g.nx);
        dj = (int)(blockDim.x / (unsigned)g.nx);
    }
    __device__ __forceinline__ void next(const Geo& g) {
        c += blockDim.x;
        i += di;
        j += dj;
        if (i >= g.nx) {
            i -= g.nx;
            j += 1;
        }
        while (j >= g.ny) {
            j -= g.ny;
            k += 1;
        }
    }
};

template <int D, class S>
__global__ void __launch_bounds__(256, 2) k_ens_flow(const EnsMember<S>* __restrict__ mem, const int2* __restrict__ tiles,
                                                  int ntiles, int tile_cells, int flip) {
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tt = tiles[t];
        const EnsMember<S>& m = mem[tt.x];
        const Geo g = m.g;
        const PhysF P = m.P;
        const int cur = m.cur ^ flip, nxt = cur ^ 1;
        FastArgs<S> A{};
        A.lag_in = m.L[cur];
        A.lag_out = m.L[nxt];
        A.tick = m.tick;
        const long long c0 = (long long)tt.y * tile_cells;
        const long long ce = min(c0 + tile_cells, g.ncell);
        for (CellWalk w(g, c0 + threadIdx.x); w.c < ce; w.next(g))
            flow_cell_2k<D, false, S, kEnsInner<D>>(g, P, A, m.f[cur], m.gp[cur], m.f[nxt], w.c, w.i, w.j, w.k);
    }
}

template <int D, class S>
__global__ void __launch_bounds__(256, 2) k_ens_thermal(const EnsMember<S>* __restrict__ mem,
                                                     const int2* __restrict__ tiles, int ntiles, int tile_cells,
                                                     int flip) {
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tt = tiles[t];
        const EnsMember<S>& m = mem[tt.x];
        const Geo g = m.g;
        const PhysF P = m.P;
        const int cur = m.cur ^ flip, nxt = cur ^ 1;
        FastArgs<S> A{};
        A.Bin0 = m.B[cur][0]; A.Bin1 = m.B[cur][1]; A.Bin2 = m.B[cur][2];
        A.Bout0 = m.B[nxt][0]; A.Bout1 = m.B[nxt][1]; A.Bout2 = m.B[nxt][2];
        A.lag_in = m.L[nxt];
        A.lag_out = m.L[nxt];
        A.tick = m.tick;
        const long long c0 = (long long)tt.y * tile_cells;
        const long long ce = min(c0 + tile_cells, g.ncell);
        for (CellWalk w(g, c0 + threadIdx.x); w.c < ce; w.next(g))
            thermal_cell_2k<D, false, S, kEnsInner<D>>(g, P, A, m.f[nxt], m.gp[cur], m.gp[nxt], w.c, w.i, w.j, w.k);
    }
}

// Every member's step counter advances by one after a batched step.
template <class S>
__global__ void k_ens_tick(const EnsMember<S>* __restrict__ mem, int nmem) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < nmem) *mem[m].tick += 1ULL;
}

template <class S>
static cudaError_t build_typed(EnsPlan& plan, const std::vector<EnsMemberHost>& members) {
    for (int di = 0; di < 2; ++di) {
        const int dim = di == 0 ? 2 : 3;
        std::vector<EnsMember<S>> hm;
        std::vector<int2> tiles;
        for (const EnsMemberHost& mh : members) {
            if (mh.dim != dim) continue;
            EnsMember<S> m{};
            m.g = dev_geo(mh.geo, mh.phys);
            m.P = fast_physf(*mh.F, mh.phys);
            m.tick = mh.F->tick;
            for (int b = 0; b < 2; ++b) {
                m.f[b] = (S*)mh.F->fbuf[b];
                m.gp[b] = (S*)mh.F->gbuf[b];
                for (int c = 0; c < 3; ++c) m.B[b][c] = mh.F->B[b][c];
                m.L[b] = mh.F->L[b];
            }
            m.cur = mh.F->cur;
            const int idx = (int)hm.size();
            const long long nt = (m.g.ncell + plan.cfg.tile_cells - 1) / plan.cfg.tile_cells;
            for (long long t = 0; t < nt; ++t) tiles.push_back(make_int2(idx, (int)t));
            plan.cells += m.g.ncell;
            hm.push_back(m);
        }
        plan.nmembers[di] = (int)hm.size();
        plan.ntiles[di] = (int)tiles.size();
        if (hm.empty()) continue;
        cudaError_t e = cudaMalloc(&plan.d_members[di], hm.size() * sizeof(EnsMember<S>));
        if (e != cudaSuccess) return e;
        e = cudaMalloc((void**)&plan.d_tiles[di], tiles.size() * sizeof(int2));
        if (e != cudaSuccess) return e;
        e = cudaMemcpy(plan.d_members[di], hm.data(), hm.size() * sizeof(EnsMember<S>), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
        e = cudaMemcpy(plan.d_tiles[di], tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void ens_free(EnsPlan& plan) {
    for (int di = 0; di < 2; ++di) {
        if (plan.d_members[di]) cudaFree(plan.d_members[di]);
        if (plan.d_tiles[di]) cudaFree(plan.d_tiles[di]);
        plan.d_members[di] = nullptr;
        plan.d_tiles[di] = nullptr;
        plan.nmembers[di] = plan.ntiles[di] = 0;
    }
    plan.cells = 0;
}

cudaError_t ens_build(EnsPlan& plan, const std::vector<EnsMemberHost>& members, const EnsLaunchCfg& cfg, int sms) {
    ens_free(plan);
    plan.cfg = cfg;
    plan.sms = sms > 0 ? sms : 152;
    plan.precision = members.empty() ? LBM_FP32 : members[0].F->precision;
    return plan.precision == LBM_FP16 ? build_typed<__half>(plan, members) : build_typed<float>(plan, members);
}

template <class S>
static void step_typed(const EnsPlan& plan, int flip, cudaStream_t s) {
    const int blk = plan.cfg.block, tc = plan.cfg.tile_cells;
    for (int stage = 0; stage < 2; ++stage) {
        for (int di = 0; di < 2; ++di) {
            if (plan.ntiles[di] == 0) continue;
            const int grid = min(plan.ntiles[di], plan.sms * plan.cfg.grid_mul);
            const EnsMember<S>* mem = (const EnsMember<S>*)plan.d_members[di];
            if (stage == 0) {
                if (di == 0) k_ens_flow<2, S><<<grid, blk, 0, s>>>(mem, plan.d_tiles[di], plan.ntiles[di], tc, flip);
                else k_ens_flow<3, S><<<grid, blk, 0, s>>>(mem, plan.d_tiles[di], plan.ntiles[di], tc, flip);
            } else {
                if (di == 0) k_ens_thermal<2, S><<<grid, blk, 0, s>>>(mem, plan.d_tiles[di], plan.ntiles[di], tc, flip);
                else k_ens_thermal<3, S><<<grid, blk, 0, s>>>(mem, plan.d_tiles[di], plan.ntiles[di], tc, flip);
            }
        }
    }
    for (int di = 0; di < 2; ++di) {
        if (plan.nmembers[di] == 0) continue;
        k_ens_tick<S><<<(plan.nmembers[di] + 127) / 128, 128, 0, s>>>((const EnsMember<S>*)plan.d_members[di],
                                                                      plan.nmembers[di]);
    }
}

void ens_step(const EnsPlan& plan, int flip, cudaStream_t s) {
    if (plan.precision == LBM_FP16) step_typed<__half>(plan, flip, s);
    else step_typed<float>(plan, flip, s);
}

}  // namespace lbm
