// lbm_fast.h - FP32 / FP16 population storage with FP32 arithmetic.
//
// Populations are stored as deviations from the rest state: d_a = f_a - w_a and
// e_a = g_a - wT_a*Tref, so that the stored numbers carry only the flow and thermal
// signal and FP16 keeps ~3 significant digits of it.  Arithmetic is FP32 in the same
// moment space as the reference (same M, same relaxation, same Guo source); the lag
// state (B_prev, and the 3D T lag / 2D stored force) is kept in FP32.
//
// Buffers come in pairs indexed by one parity `cur`:
//   F[cur] = f_post_N, G[cur] = g_post_N, B[cur] = B_prev_N,
//   L[cur] = lag (3D: T_{N-1}; 2D: the force F_y,N stored by the flow collision).
// In single-kernel mode the handle runs one flow collision ahead ("ahead"):
//   F[cur^1] = f_post_{N+1} and, in 2D, L[cur^1] = F_y,N+1.
#pragma once

#include <cuda_runtime.h>

#include <functional>

#include "lbm_internal.h"

namespace lbm {

struct PhysF;

struct FastState {
    int precision = LBM_FP32;  // LBM_FP32 or LBM_FP16
    int dim = 3, q = 19, qt = 7;
    size_t esize = 4;          // bytes per stored population
    void* fbuf[2] = {nullptr, nullptr};
    void* gbuf[2] = {nullptr, nullptr};
    float* B[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    float* L[2] = {nullptr, nullptr};
    // module form (after initial / materialisation): populations as deviations
    void* fref = nullptr;
    void* gref = nullptr;
    float *rho = nullptr, *u = nullptr, *v = nullptr, *w = nullptr, *T = nullptr;
    float *up = nullptr, *vp = nullptr, *wp = nullptr, *Tp = nullptr;
    int cur = 0;
    bool fused_valid = false;   // the fused buffers hold the current state
    bool ahead = false;         // single-kernel phase: F[cur^1] already holds f_post_{N+1}
    bool single_kernel = false; // one-launch fused step (lbm_fused.cu); off: the two-kernel step is faster today
    int kchunk = 16;            // z planes per block of the fused kernel (3D)
    // Form of the non-first two-kernel step, chosen by fast_allocate from GB300 timings:
    // one cell per thread, except two cells per thread for 2D FP32; staged rows
    // (lbm_fast_tma.cu) on request.
    bool pairs = false;
    bool tma = false;
    bool rows = false;          // interior-row and face-row launches (LBM_OPT_ROWS)
    bool wide = false;          // 64-bit cell indices where 32-bit ones fit (LBM_OPT_WIDE_INDEX)
    int* err = nullptr;         // device flag: a bounded wait of a staged kernel gave up
    // In-place (AA) pattern: fbuf[0] / gbuf[0] are the only population arrays and also the
    // module arrays (fref, gref alias them); B and L have one buffer each.
    bool aa = false;
    AAState AA;
    // FP16 storage rounds new populations stochastically (lbm_fast_math.cuh, storeS), with
    // random bits keyed on this device step counter (steps since initial; continuation
    // records keep it).
    bool sr = false;
    unsigned long long* tick = nullptr;
};

using AllocFn = std::function<int(void**, size_t)>;

int fast_allocate(FastState& F, const lbm_params& p, const Geo& g, const AllocFn& alloc);
void fast_initial(FastState& F, const Geo& g, const PhysC& P, const InitC& I, int dim, cudaStream_t s);
// Two-kernel step (flow collision, then thermal).  first: read the module arrays.
// part: 0 = flow kernel only, 1 = thermal kernel only, 2 = both.
void fast_step(FastState& F, const Geo& g, const PhysC& P, int dim, bool first, cudaStream_t s, int part = 2);
// Single-kernel mode: enter (one flow collision ahead), then one launch per step.
void fast_enter(FastState& F, const Geo& g, const PhysC& P, int dim, cudaStream_t s);
void fast_fused_step(FastState& F, const Geo& g, const PhysC& P, int dim, cudaStream_t s);
bool fast_fused_supported(const Geo& g, int dim);
// The staged two-kernel step applies (nx a multiple of 8, a tile row within the budget).
bool fast_tma_supported(const Geo& g, int dim, int precision);
// Read and clear the device error flag of the staged kernels (synchronises the stream).
int fast_take_error(FastState& F, cudaStream_t s);
// Run the bounded mbarrier wait of the staged kernels on a barrier that never completes,
// with `limit` polls: it gives up and sets the error flag (lbm_selftest_wait_timeout).
void fast_wait_selftest(FastState& F, unsigned limit, cudaStream_t s);
// Physics constants of the step kernels of this handle (adds the rounding mode).
PhysF fast_physf(const FastState& F, const PhysC& P);
// Advance the step counter by one step (after a step's thermal kernel).
void fast_tick(FastState& F, cudaStream_t s);
// In-place pattern step and materialisation (lbm_fast_aa.cu); g is the deviation geometry.
void fast_step_aa(FastState& F, const Geo& g, const PhysF& pf, int dim, bool first, cudaStream_t s, int part);
void fast_materialize_aa(FastState& F, const Geo& g, const PhysF& pf, int dim, cudaStream_t s);
// Rebuild the module arrays (f, g, rho, u, v, w, T) of the current step; leaves the fused
// buffers valid.  In-place pattern: the module scalars only (the arrays are the populations).
void fast_materialize(FastState& F, const Geo& g, const PhysC& P, int dim, cudaStream_t s);
inline bool fast_fused_valid(const FastState& F) { return F.fused_valid; }
inline bool fast_at_origin(const FastState& F) { return F.cur == 0; }
DiagFields<float> fast_diag_fields(const FastState& F);
// Export a field to an FP64 device buffer in the reference's Fortran layout (AoS for
// populations, or direction-major SoA with soa = true); import the reverse.  Return LBM_OK
// or LBM_ERR_STATE / LBM_ERR_PARAM.
int fast_export(const FastState& F, const Geo& g, const PhysC& P, int dim, int field, double* out, cudaStream_t s,
                bool soa = false);
int fast_import(FastState& F, const Geo& g, const PhysC& P, int dim, int field, const double* in, cudaStream_t s,
                bool soa = false);

}  // namespace lbm
