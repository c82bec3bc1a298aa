// lbm_fast.h - FP32 / FP16 population storage with FP32 arithmetic.
//
// Populations are stored as deviations from the rest state: d_a = f_a - w_a and
// e_a = g_a - wT_a*Tref, so that the stored numbers carry only the flow and thermal
// signal and FP16 keeps ~3 significant digits of it.  Arithmetic is FP32 in the same
// moment space as the reference (same M, same relaxation, same Guo source); the lag
// state (B_prev, and the 3D T lag / 2D stored force) is kept in FP32.
#pragma once

#include <cuda_runtime.h>

#include <functional>

#include "lbm_internal.h"

namespace lbm {

struct FastState {
    int precision = LBM_FP32;  // LBM_FP32 or LBM_FP16
    int dim = 3, q = 19, qt = 7;
    size_t esize = 4;          // bytes per stored population
    // fused buffers (type float or __half, stored as raw bytes)
    void* fbuf[2] = {nullptr, nullptr};
    void* gbuf[2] = {nullptr, nullptr};
    // module form (after initial / materialisation): populations as deviations
    void* fref = nullptr;
    void* gref = nullptr;
    float *rho = nullptr, *u = nullptr, *v = nullptr, *w = nullptr, *T = nullptr;
    float *up = nullptr, *vp = nullptr, *wp = nullptr, *Tp = nullptr;
    float *Bx = nullptr, *By = nullptr, *Bz = nullptr;
    float* lag = nullptr;  // 3D: T of the previous step; 2D: stored force F_y
    bool fused_valid = false;
    int cur = 0;
};

using AllocFn = std::function<int(void**, size_t)>;

int fast_allocate(FastState& F, const lbm_params& p, const Geo& g, const AllocFn& alloc);
void fast_initial(FastState& F, const Geo& g, const PhysC& P, const InitC& I, int dim, cudaStream_t s);
// part: 0 = flow kernel only, 1 = thermal kernel only (then advances the buffers), 2 = both
void fast_step(FastState& F, const Geo& g, const PhysC& P, int dim, bool first, cudaStream_t s, int part = 2);
void fast_materialize(FastState& F, const Geo& g, const PhysC& P, int dim, cudaStream_t s);
inline bool fast_fused_valid(const FastState& F) { return F.fused_valid; }
inline bool fast_at_origin(const FastState& F) { return F.cur == 0; }
DiagFields<float> fast_diag_fields(const FastState& F);
// Export a field to an FP64 device buffer in the reference's Fortran layout (AoS for
// populations); import the reverse.  Return LBM_OK or LBM_ERR_STATE.
int fast_export(const FastState& F, const Geo& g, const PhysC& P, int dim, int field, double* out, cudaStream_t s);
int fast_import(FastState& F, const Geo& g, const PhysC& P, int dim, int field, const double* in, cudaStream_t s);

}  // namespace lbm
