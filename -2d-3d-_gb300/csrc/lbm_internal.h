// lbm_internal.h - structures and launchers shared by the kernels and the host API.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "lbm_device.cuh"

namespace lbm {

// Physics constants of one run, in the form the kernels consume (all from commondata).
struct PhysC {
    double gBeta, Tref;
    double Snu, Sq, Se, Seps, Spi, Sm;  // flow relaxation rates
    double Qk, Qnu, SG, paraA;          // thermal relaxation, M1G factor, legacy a_T
    double omegaT0, omegaT1, geqc;      // thermal weights and g^eq coefficient
    int use_g, legacy;
    int ha;                             // SideHeatedHa: magnetic force in the 2D collision
    double B2, sinphi, cosphi;          // B2sigemarho, sin(phi), cos(phi)
    // Factors of the Guo source that depend on the rates only, rounded once on the host in
    // the reference's order instead of once per cell: 3D (1 - Se/2)*38, (1 - Seps/2)*(-11),
    // (1 - Sq/2)*(-2/3), 1 - Snu/2, 1 - Spi/2; 2D 6 - 3 Snu, 1 - Sq/2, 2 - Snu (and 1 - Snu/2).
    double hSe38, hSeps11, hSq23, hSnu, hSpi;
    double h6Snu, hSq, h2Snu;
};

// The kernels' physics constants from the parameters and the derived commondata constants.
// Host code, compiled without floating-point contraction: the rate-only factors are rounded
// once here in the reference's order.
inline PhysC make_physc(const lbm_params& p, const lbm_constants& c) {
    PhysC P{};
    P.gBeta = c.gBeta;
    P.Tref = c.Tref;
    P.Snu = c.Snu;
    P.Sq = c.Sq;
    P.Se = c.Se;
    P.Seps = c.Seps;
    P.Spi = c.Spi;
    P.Sm = c.Sm;
    P.Qk = c.Qk;
    P.Qnu = c.Qnu;
    P.SG = c.SG;
    P.paraA = c.paraA;
    P.omegaT0 = c.omegaT0;
    P.omegaT1 = c.omegaT1;
    P.geqc = c.thermalGeqCoeff;
    P.use_g = p.use_g ? 1 : 0;
    P.legacy = p.legacy_thermal ? 1 : 0;
    P.ha = p.side_heated_ha ? 1 : 0;
    P.B2 = c.B2sigemarho;
    P.sinphi = c.sinphi;
    P.cosphi = c.cosphi;
    P.hSe38 = (1.0 - 0.5 * c.Se) * 38.0;
    P.hSeps11 = (1.0 - 0.5 * c.Seps) * (-11.0);
    P.hSq23 = (1.0 - 0.5 * c.Sq) * (-2.0 / 3.0);
    P.hSnu = 1.0 - 0.5 * c.Snu;
    P.hSpi = 1.0 - 0.5 * c.Spi;
    P.h6Snu = 6.0 - 3.0 * c.Snu;
    P.hSq = 1.0 - 0.5 * c.Sq;
    P.h2Snu = 2.0 - c.Snu;
    return P;
}

// Geometry and boundary switches of one run (host code).  The anti-bounce-back source of a
// constant-temperature wall is 2 wT Tw (2DRB.F90:1052-1059, 1094-1101; 3DRB.F90:1265-1271,
// 1309-1315), written in the legacy scheme as (4 + a_T)/10 Tw (2D) or (6 + a_T)/21 Tw (3D).
inline Geo make_geo(const lbm_params& p, const lbm_constants& c) {
    Geo g{};
    g.nx = p.nx;
    g.ny = p.ny;
    g.nz = p.dim == 3 ? p.nz : 1;
    g.ncell = (long long)g.nx * g.ny * g.nz;
    for (int a = 0; a < 3; ++a) {
        g.bcf[a] = p.bc_flow[a];
        g.bct[a] = p.bc_thermal[a];
        if (p.dim == 2 && a == 2) {
            g.bcf[a] = LBM_BC_NOSLIP;
            g.bct[a] = LBM_BCT_ADIABATIC;
        }
        if (p.legacy_thermal) {
            const double cc = p.dim == 2 ? (4.0 + c.paraA) / 10.0 : (6.0 + c.paraA) / 21.0;
            g.bcT_lo[a] = cc * p.Thot;
            g.bcT_hi[a] = cc * p.Tcold;
        } else {
            g.bcT_lo[a] = 2.0 * c.omegaT1 * p.Thot;
            g.bcT_hi[a] = 2.0 * c.omegaT1 * p.Tcold;
        }
    }
    return g;
}

// The same geometry with the thermal wall terms of populations stored as deviations from the
// rest state (e = g - wT Tref): the wall term minus 2 wT Tref.
inline Geo deviation_geo(const Geo& g, const lbm_constants& c) {
    Geo d = g;
    for (int a = 0; a < 3; ++a) {
        d.bcT_lo[a] = g.bcT_lo[a] - 2.0 * c.omegaT1 * c.Tref;
        d.bcT_hi[a] = g.bcT_hi[a] - 2.0 * c.omegaT1 * c.Tref;
    }
    return d;
}

// Inputs of `initial` that depend on host-side math (sin/cos of the RB perturbation).
struct InitC {
    double L, Thot, Tcold;
    int perturb;
    double pert_amp;
    const double* sx;  // sin(2 pi x/xLen) (2D) or cos(...) (3D), per i
    const double* sy;  // sin(pi y/yLen), per j
    double noise_amp;
    uint64_t seed;
};

// FP64 device arrays: the reference's module state (f, g, f_post, g_post, rho, u, v, w,
// T, B_prev, F, up..Tp) plus the lag field of the fused path.
struct ExactArrays {
    double *f, *g, *fpost, *gpost;
    double *rho, *u, *v, *w, *T;
    double *Bx, *By, *Bz;
    double *Fx, *Fy;   // 2D: force stored by collision
    double *Tlag;      // 3D fused: T of the previous step
    // fused: the momentum sums sum_a e_a f_a of the last macro step (no force term), written
    // by the thermal kernel of step n and read by the flow kernel of step n+1, which pulls
    // the same f_n: they are its moments m3, m5, m7 (and rho its m0), bit for bit
    double *jx, *jy, *jz;
    double *up, *vp, *wp, *Tp;
};

enum Stage {
    STAGE_COLLISION = 0, STAGE_STREAMING, STAGE_BOUNCEBACK, STAGE_MACRO,
    STAGE_COLLISIONT, STAGE_STREAMINGT, STAGE_BOUNCEBACKT, STAGE_MACROT
};

// ---- in-place (AA) access pattern --------------------------------------------------------
// State of the pattern for one lattice: the layout parity of the flow and thermal arrays
// (0 streamed, 1 swapped; lbm_device.cuh) and the face snapshots that an odd sweep reads
// across periodic faces.
struct AAState {
    int fpar = 0, gpar = 0;
    bool graw = false;  // the thermal array's streamed slots were filled by pushes (raw values)
    void* face_f[3] = {nullptr, nullptr, nullptr};  // per periodic flow axis: q * face cells
    void* face_g[3] = {nullptr, nullptr, nullptr};
};

// Storage precision of an array handed to the pattern's helpers (LBM_FP64/FP32/FP16).
// Snapshot the face slots of every periodic axis of one array before its odd sweep.
void aa_snapshot(const Geo& g, int q, bool thermal, int precision, const void* arr, void* const face[3],
                 cudaStream_t s);
// The module (streamed) view of one array into FP64: AoS (Fortran order) or SoA.  dev:
// the array stores deviations from the rest state (FP32/FP16 forms; w0/w1 are the thermal
// rest values) and each value is rounded to the storage type as the module array holds it.
void aa_module_view(const Geo& g, int q, bool thermal, int precision, const void* arr, int par, bool raw, double* out,
                    bool soa, bool dev, double w0, double w1, cudaStream_t s);

// ---- exact FP64 kernels (lbm_exact.cu) ------------------------------------------------
void exact_initial(const Geo& g, const PhysC& P, const InitC& I, const ExactArrays& A, int dim, cudaStream_t s);
void exact_stage(int stage, const Geo& g, const PhysC& P, const ExactArrays& A, int dim, cudaStream_t s);
// part: 0 = flow kernel only, 1 = thermal kernel only, 2 = both (one full step)
void exact_fused_step(const Geo& g, const PhysC& P, const ExactArrays& A, int dim, bool first, const double* fprev,
                      const double* gprev, double* fnext, double* gnext, cudaStream_t s, int part = 2);
void exact_materialize(const Geo& g, const PhysC& P, const ExactArrays& A, int dim, const double* fcur,
                       const double* gcur, cudaStream_t s);

// In-place pattern: part 0 = flow sweep, 1 = thermal sweep, 2 = both; flips the parities.
void exact_aa_step(const Geo& g, const PhysC& P, const ExactArrays& A, int dim, bool first, AAState& S,
                   cudaStream_t s, int part = 2);
// Module scalars (rho, u, v, w, T) of the current step from the in-place arrays A.f, A.g.
void exact_aa_materialize(const Geo& g, const PhysC& P, const ExactArrays& A, int dim, const AAState& S,
                          cudaStream_t s);

// Restart: rebuild T, rho, u, v, w, B_prev and the 2D force from the SoA populations A.f,
// A.g (reconstruct_macro_from_fg); sets *bad = 1 when some cell has rho <= 0.
void exact_reconstruct(const Geo& g, const PhysC& P, const ExactArrays& A, int dim, unsigned int* bad,
                       cudaStream_t s);

// ---- reductions (lbm_reduce.cu) ---------------------------------------------------------
// Fields read by the diagnostics (FP64 or FP32 device arrays of ncell values).
template <class S>
struct DiagFields {
    const S *u, *v, *w, *T, *rho;
    S *up, *vp, *wp, *Tp;
};

enum DiagOp {
    DIAG_CHECK = 0, DIAG_NURE = 1, DIAG_NU_GLOBAL = 2, DIAG_NU_COLD_MID = 3,
    DIAG_NU_GLOBAL_SIDE = 4, DIAG_NU_COLD_MID_SIDE = 5
};

// Number of partial-sum slots a reduction launch writes: nblocks * DIAG_NSUM doubles.
constexpr int DIAG_NSUM = 5;
int diag_blocks(long long ncell);

struct DiagScalars {
    double Thot, Tcold, Tref, dy, coef, deltaT;
    int side;  // side-heated cell: Nu uses u instead of v
    int d3;
};

// Launch one reduction; partial sums (DIAG_NSUM per block, fixed order) go to `partials`.
template <class S>
void diag_reduce(DiagOp op, const Geo& g, const DiagScalars& D, const DiagFields<S>& F, double* partials,
                 int nblocks, cudaStream_t s);
// Per-column wall profile for RBcalc_Nu_wall_avg: Tb[i] = mean_k T(i,1,k) and
// Nu_bot[i] = mean_k (8Thot - 9T(i,1,k) + T(i,2,k))/(3dy)/deltaT, k summed in order.
template <class S>
void diag_wall_columns(const Geo& g, const DiagScalars& D, const S* T, double* Tb, double* Nub, cudaStream_t s);

// Per-row hot (left) wall profile for SideHeatedcalc_Nu_wall_avg: Tl[j] = mean_k T(1,j,k)
// and Nu_left[j] = mean_k (8Thot - 9T(1,j,k) + T(2,j,k))/(3dx)/deltaT, k summed in order.
template <class S>
void diag_wall_rows(const Geo& g, const DiagScalars& D, const S* T, double* Tl, double* Nul, cudaStream_t s);
// Copy the plane `idx` normal to `axis` of a field into `out` (FP64, contiguous).
template <class S>
void diag_gather_plane(const Geo& g, const S* f, int axis, int idx, double* out, cudaStream_t s);

// Fine-grid |psi| search of calc_psi_absmax_fine_spline on device arrays: xExt (nx+2),
// yExt (ny+2), rows (ny x (nx+2)) and their spline second derivatives y2rows; scratch xfine
// (nFineX x ny); per fine x column k the largest |psi| and the first fine y index holding it.
int psi_fine_search(int nx, int ny, double xLen, double yLen, int nFineX, int nFineY, const double* xExt,
                    const double* yExt, const double* rows, const double* y2rows, double* xfine, double* best_val,
                    int* best_l, cudaStream_t s);

// ---- layout transforms (lbm_reduce.cu) -------------------------------------------------
// Fortran AoS f(0:q-1, cells) <-> device SoA f[q][cells], FP64.  Either side may be host
// memory that the device reads and writes coherently (cudaDevAttrPageableMemoryAccess).
void copy_doubles(const double* src, double* dst, long long n, cudaStream_t s);
void aos_to_soa(const double* aos, double* soa, int q, long long ncell, cudaStream_t s);
void soa_to_aos(const double* soa, double* aos, int q, long long ncell, cudaStream_t s);

}  // namespace lbm
