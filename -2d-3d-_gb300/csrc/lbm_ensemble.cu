// lbm_ensemble.cu - one flow launch and one thermal launch per time step for any number of
// FP32/FP16 lattices of uneven sizes and parameters (the batched form).
//
// A grid of about SMs x grid_mul persistent blocks walks a packed tile table: tile t is
// (member m, first cell c0) and covers tile_cells consecutive cells of member m.  Each
// block reads the member's descriptor (geometry, relaxation rates, buffer pointers and
// parity), then runs the same per-cell bodies as the single-lattice two-kernel step
// (lbm_fast_cells.cuh, or the paired bodies of lbm_fast_pairs.cuh for members with even
// nx) on its cells.  Small lattices therefore fill the GPU together instead of one launch
// each.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <vector>

#include "lbm_ensemble.h"
#include "lbm_fast_pairs.cuh"

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

// Fixed-offset pulls for the cells off the faces (lbm_fast_cells.cuh).  Resident blocks of
// 256 threads per SM: three, except two for the paired 3D bodies (about 115 registers);
// four for the paired 2D bodies spills 48-60 bytes and measured no faster on GB300.
// With the member descriptor and buffer arguments staged in shared memory the one-cell
// kernels take 66-80 registers, against 96-128 with register copies of the descriptor
// (the 3D thermal kernel took 242 without a bound), and none spills.
#ifndef LBM_ENS_PAIR2D_BLOCKS
#define LBM_ENS_PAIR2D_BLOCKS 3
#endif
template <int D>
constexpr bool kEnsInner = true;
template <int D, bool PAIR>
constexpr int kEnsBlocks = (D == 3 && PAIR) ? 2 : (D == 2 && PAIR) ? LBM_ENS_PAIR2D_BLOCKS : 3;

// Cell coordinates of a thread's cells in a tile, stepped instead of divided: one division
// at the thread's first cell, then (i, j, k) advance by `stride` cells with carries (i by
// less than a row; j may wrap several planes on narrow lattices).
struct CellWalk {
    long long c;
    int i, j, k, di, dj, stride;
    __device__ __forceinline__ CellWalk(const Geo& g, long long c0, int stride_) : c(c0), stride(stride_) {
        cell_coords(g, c0, i, j, k);
        di = (int)((unsigned)stride % (unsigned)g.nx);
        dj = (int)((unsigned)stride / (unsigned)g.nx);
    }
    __device__ __forceinline__ void next(const Geo& g) {
        c += stride;
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

// The member descriptor of a block's current tile and the buffer arguments of this step,
// staged in shared memory: the cell bodies read geometry, constants and buffer pointers
// from there as the single-lattice kernels read them from the kernel parameters, instead of
// holding register copies across the cell loop.  `args` (thread 0) fills the arguments from
// the descriptor in global memory.
template <class S>
struct EnsStage {
    EnsMember<S> m;
    FastArgs<S> A;
};

template <class S, class ARGS>
__device__ __forceinline__ const EnsStage<S>& stage_member(const EnsMember<S>* __restrict__ mem, int idx,
                                                           unsigned* __restrict__ sh, ARGS args) {
    static_assert(sizeof(EnsMember<S>) % 4 == 0, "descriptor copied in 32-bit words");
    EnsStage<S>& st = *reinterpret_cast<EnsStage<S>*>(sh);
    const unsigned* src = reinterpret_cast<const unsigned*>(mem + idx);
    __syncthreads();  // the block's previous tile is done with the staged copy
    for (int w = threadIdx.x; w < (int)(sizeof(EnsMember<S>) / 4); w += blockDim.x) sh[w] = __ldg(src + w);
    if (threadIdx.x == 0) {
        FastArgs<S> A{};
        args(mem[idx], A);
        st.A = A;
    }
    __syncthreads();
    return st;
}

// PAIR: the thread's cells are c and c + 1 (same row: nx even, tiles start on even cells,
// c even), walked with a stride of two cells per thread.
template <int D, class S, bool PAIR>
__global__ void __launch_bounds__(256, (kEnsBlocks<D, PAIR>)) k_ens_flow(const EnsMember<S>* __restrict__ mem,
                                                                       const int2* __restrict__ tiles, int ntiles,
                                                                       int tile_cells, int flip) {
    constexpr int W = PAIR ? 2 : 1;
    __shared__ __align__(16) unsigned sh[(sizeof(EnsStage<S>) + 3) / 4];
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tt = tiles[t];
        const EnsStage<S>& st = stage_member<S>(mem, tt.x, sh, [flip](const EnsMember<S>& gm, FastArgs<S>& A) {
            const int c = gm.cur ^ flip;
            A.lag_in = gm.L[c];
            A.lag_out = gm.L[c ^ 1];
            A.tick = gm.tick;
        });
        const EnsMember<S>& m = st.m;
        const FastArgs<S>& A = st.A;
        const Geo& g = m.g;
        const PhysF& P = m.P;
        const int cur = m.cur ^ flip, nxt = cur ^ 1;
        const long long c0 = (long long)tt.y * tile_cells;
        const long long ce = min(c0 + tile_cells, g.ncell);
        for (CellWalk w(g, c0 + W * (long long)threadIdx.x, W * (int)blockDim.x); w.c < ce; w.next(g)) {
            if constexpr (PAIR)
                flow_pair_2k<D, S>(g, P, A, m.f[cur], m.gp[cur], m.f[nxt], w.c, w.i, w.j, w.k);
            else
                flow_cell_2k<D, false, S, kEnsInner<D>>(g, P, A, m.f[cur], m.gp[cur], m.f[nxt], w.c, w.i, w.j, w.k);
        }
    }
}

template <int D, class S, bool PAIR>
__global__ void __launch_bounds__(256, (kEnsBlocks<D, PAIR>)) k_ens_thermal(const EnsMember<S>* __restrict__ mem,
                                                                          const int2* __restrict__ tiles, int ntiles,
                                                                          int tile_cells, int flip) {
    constexpr int W = PAIR ? 2 : 1;
    __shared__ __align__(16) unsigned sh[(sizeof(EnsStage<S>) + 3) / 4];
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tt = tiles[t];
        const EnsStage<S>& st = stage_member<S>(mem, tt.x, sh, [flip](const EnsMember<S>& gm, FastArgs<S>& A) {
            const int c = gm.cur ^ flip, n = c ^ 1;
            A.Bin0 = gm.B[c][0]; A.Bin1 = gm.B[c][1]; A.Bin2 = gm.B[c][2];
            A.Bout0 = gm.B[n][0]; A.Bout1 = gm.B[n][1]; A.Bout2 = gm.B[n][2];
            A.lag_in = gm.L[n];
            A.lag_out = gm.L[n];
            A.tick = gm.tick;
        });
        const EnsMember<S>& m = st.m;
        const FastArgs<S>& A = st.A;
        const Geo& g = m.g;
        const PhysF& P = m.P;
        const int cur = m.cur ^ flip, nxt = cur ^ 1;
        const long long c0 = (long long)tt.y * tile_cells;
        const long long ce = min(c0 + tile_cells, g.ncell);
        for (CellWalk w(g, c0 + W * (long long)threadIdx.x, W * (int)blockDim.x); w.c < ce; w.next(g)) {
            if constexpr (PAIR)
                thermal_pair_2k<D, S>(g, P, A, m.f[nxt], m.gp[cur], m.gp[nxt], w.c, w.i, w.j, w.k);
            else
                thermal_cell_2k<D, false, S, kEnsInner<D>>(g, P, A, m.f[nxt], m.gp[cur], m.gp[nxt], w.c, w.i, w.j,
                                                           w.k);
        }
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
    // a member pairs when the configuration pairs, its rows hold whole pairs, and every tile
    // starts on an even cell
    for (int li = 0; li < kEnsLists; ++li) {
        const int dim = (li & 1) ? 3 : 2;
        const bool paired = (li & 2) != 0;
        const bool pairing = (plan.cfg.pairs & (dim == 3 ? 2 : 1)) != 0 && plan.cfg.tile_cells % 2 == 0;
        std::vector<EnsMember<S>> hm;
        std::vector<int2> tiles;
        for (const EnsMemberHost& mh : members) {
            if (mh.dim != dim || (pairing && mh.geo.nx % 2 == 0) != paired) continue;
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
        plan.nmembers[li] = (int)hm.size();
        plan.ntiles[li] = (int)tiles.size();
        if (hm.empty()) continue;
        cudaError_t e = cudaMalloc(&plan.d_members[li], hm.size() * sizeof(EnsMember<S>));
        if (e != cudaSuccess) return e;
        e = cudaMalloc((void**)&plan.d_tiles[li], tiles.size() * sizeof(int2));
        if (e != cudaSuccess) return e;
        e = cudaMemcpy(plan.d_members[li], hm.data(), hm.size() * sizeof(EnsMember<S>), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
        e = cudaMemcpy(plan.d_tiles[li], tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void ens_free(EnsPlan& plan) {
    for (int li = 0; li < kEnsLists; ++li) {
        if (plan.d_members[li]) cudaFree(plan.d_members[li]);
        if (plan.d_tiles[li]) cudaFree(plan.d_tiles[li]);
        plan.d_members[li] = nullptr;
        plan.d_tiles[li] = nullptr;
        plan.nmembers[li] = plan.ntiles[li] = 0;
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

template <int D, class S, bool PAIR>
static void launch_list(const EnsPlan& plan, int li, int stage, int flip, cudaStream_t s) {
    const int grid = min(plan.ntiles[li], plan.sms * plan.cfg.grid_mul);
    const EnsMember<S>* mem = (const EnsMember<S>*)plan.d_members[li];
    if (stage == 0)
        k_ens_flow<D, S, PAIR><<<grid, plan.cfg.block, 0, s>>>(mem, plan.d_tiles[li], plan.ntiles[li],
                                                               plan.cfg.tile_cells, flip);
    else
        k_ens_thermal<D, S, PAIR><<<grid, plan.cfg.block, 0, s>>>(mem, plan.d_tiles[li], plan.ntiles[li],
                                                                  plan.cfg.tile_cells, flip);
}

template <class S>
static void step_typed(const EnsPlan& plan, int flip, cudaStream_t s) {
    for (int stage = 0; stage < 2; ++stage) {
        for (int li = 0; li < kEnsLists; ++li) {
            if (plan.ntiles[li] == 0) continue;
            switch (li) {
                case 0: launch_list<2, S, false>(plan, li, stage, flip, s); break;
                case 1: launch_list<3, S, false>(plan, li, stage, flip, s); break;
                case 2: launch_list<2, S, true>(plan, li, stage, flip, s); break;
                default: launch_list<3, S, true>(plan, li, stage, flip, s); break;
            }
        }
    }
    for (int li = 0; li < kEnsLists; ++li) {
        if (plan.nmembers[li] == 0) continue;
        k_ens_tick<S><<<(plan.nmembers[li] + 127) / 128, 128, 0, s>>>((const EnsMember<S>*)plan.d_members[li],
                                                                      plan.nmembers[li]);
    }
}

void ens_step(const EnsPlan& plan, int flip, cudaStream_t s) {
    if (plan.precision == LBM_FP16) step_typed<__half>(plan, flip, s);
    else step_typed<float>(plan, flip, s);
}

}  // namespace lbm
