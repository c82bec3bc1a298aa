// lbm_api.cpp - host side of the C ABI declared in include/lbm_gpu.h.
//
// A handle owns one lattice resident in HBM, a CUDA stream and (after the first
// lbm_step) a captured CUDA graph that replays a chunk of fused steps.  State lives in
// one of two forms:
//   * "module" form: the reference's arrays after a full iteration (f, g, rho, u, v, w,
//     T, B_prev, F), used by the stage entry points, the diagnostics and state transfer;
//   * "fused" form: post-collision buffers f_post_N / g_post_N plus the lag fields,
//     advanced by the fused kernels.
// lbm_step leaves the handle in fused form; any call that needs the module arrays first
// rebuilds them with one materialisation pass (bit-identical to what the reference
// holds after iteration N, so stepping resumes on the same trajectory).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <utility>
#include <cmath>
#include <cstdio>
#include <limits>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/lbm_gpu.h"
#include "lbm_ensemble.h"
#include "lbm_fast.h"
#include "lbm_fixed.h"
#include "lbm_internal.h"
#include "lbm_records.h"

using namespace lbm;

namespace {

const double kPi = 3.141592653589793115997963468544185161590576171875;  // acos(-1.0d0)
constexpr int kChunkSteps = 32;  // fused steps per captured graph (even: ends on buffer 0)

}  // namespace

struct lbm_handle {
    lbm_params p;
    lbm_constants c;
    int dim = 3, q = 19, qt = 7;
    int device = 0;
    cudaStream_t stream = nullptr;
    Geo geo{};
    PhysC phys{};
    DiagScalars dsc{};
    std::string err;
    int64_t itc = 0;
    bool initialised = false;
    // convergence history: the reference's once-per-run flags (first_write, zone_started)
    bool conv_started = false, conv_zone_started = false;

    // FP64 plain method
    ExactArrays A{};
    double* fbuf[2] = {nullptr, nullptr};
    double* gbuf[2] = {nullptr, nullptr};
    bool fused_valid = false;  // true: current state is in the fused buffers
    int cur = 0;               // fused buffer index holding f_post_N / g_post_N
    AAState aa;                // in-place pattern: A.f / A.g are the only population arrays
    // fixed arithmetic (arith = LBM_ARITH_FIXED): fbuf / gbuf hold q60 deviations
    // (lbm_fixed_cell.cuh); the lag state lives in xb0..xb2 (B_prev) and xlag (3D T lag,
    // 2D stored force), q60 as well
    bool fixed = false;
    PhysX px{};
    Geo xgeo{};  // geometry with the thermal wall terms of deviations
    long long *xb0 = nullptr, *xb1 = nullptr, *xb2 = nullptr, *xlag = nullptr;
    // fused passes (lbm_fixed.cu k_xfused): B_prev double-buffered, the graph of a chunk of
    // passes and the state it was captured from
    // LBM_OPT_SINGLE_KERNEL on a fixed handle.  Off by default: on GB300 the fused pass reads
    // a third less DRAM but executes about 1.4x the integer instructions (the thermal halo is
    // recomputed with 64-bit products) and runs at half the two-kernel rate (256^3: 4.08 ms
    // against 2.14 ms per step).
    bool xfused = false;
    long long *xb0b = nullptr, *xb1b = nullptr, *xb2b = nullptr;
    cudaGraph_t xgraph = nullptr;
    cudaGraphExec_t xgraph_exec = nullptr;
    int xgraph_key = -1;

    // FP32 / FP16 storage forms
    FastState F{};

    // captured chunk of fused steps
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_key = 0;  // in-place pattern: the layout state the chunk was captured from

    // scratch
    double* d_part = nullptr;
    std::vector<double> h_part;
    double* d_tb = nullptr;
    double* d_nub = nullptr;
    double* d_tl = nullptr;   // side-heated wall profile: mean T and Nu of the hot (left) wall per row
    double* d_nul = nullptr;
    double* d_stage = nullptr;  // AoS staging for state transfer
    size_t stage_cap = 0;
    double* d_sx = nullptr;
    double* d_sy = nullptr;
    std::vector<void*> allocs;

    // batched stepping
    lbm_ensemble* ensemble = nullptr;  // the ensemble this handle is a member of
    cudaEvent_t order_ev = nullptr;    // orders the handle's stream against the ensemble's

    int reload_form = -1;  // form used by the last lbm_reload (0 reference, 1 continuation)

    // State transfer straight between the caller's host arrays and the device arrays: the
    // layout kernels read and write pageable host memory coherently (Grace + NVLink-C2C:
    // cudaDevAttrPageableMemoryAccess), instead of a staged copy through the driver.
    bool host_access = false;   // the device can
    bool host_direct = false;   // and lbm_set_state reads the caller's array so (LBM_OPT_HOST_DIRECT bit 0)
    bool host_direct_wr = false;  // and lbm_get_state writes it so (bit 1)
    bool wide_index = false;      // fixed arithmetic: 64-bit cell indices everywhere (LBM_OPT_WIDE_INDEX)
};

// ------------------------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------------------------
// NVTX range around an entry point (stepping, diagnostics, state transfer, restart files),
// so a timeline from a profiler shows where the host-side calls begin and end.  The
// header-only NVTX API costs a branch when no tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

static int fail(lbm_handle* h, int status, const std::string& msg) {
    if (h) h->err = msg;
    return status;
}

static int cuda_fail(lbm_handle* h, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(h, e == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA, m);
}

#define CK(h, call)                                              \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #call); \
    } while (0)

#define CK_LAUNCH(h, what)                                     \
    do {                                                       \
        cudaError_t e_ = cudaGetLastError();                   \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, what); \
    } while (0)

template <class T>
static int dalloc(lbm_handle* h, T** ptr, size_t count) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T) > 0 ? count * sizeof(T) : 1);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return cuda_fail(h, e, "cudaMalloc");
    }
    h->allocs.push_back(p);
    *ptr = (T*)p;
    return LBM_OK;
}

static int validate(const lbm_params* p) {
    if (!p) return LBM_ERR_PARAM;
    if (p->dim != 2 && p->dim != 3) return LBM_ERR_PARAM;
    if (p->nx < 5 || p->ny < 5) return LBM_ERR_PARAM;
    if (p->dim == 2 && p->nz != 1) return LBM_ERR_PARAM;
    if (p->dim == 3 && p->nz < 2) return LBM_ERR_PARAM;
    if ((long long)p->nx * p->ny * (long long)p->nz > (1LL << 31)) return LBM_ERR_PARAM;
    if (!(p->Ra > 0) || !(p->Pr > 0) || !(p->Mach > 0)) return LBM_ERR_PARAM;
    if (!(p->Thot > p->Tcold)) return LBM_ERR_PARAM;
    if (p->cell != LBM_CELL_RB && p->cell != LBM_CELL_SIDE) return LBM_ERR_PARAM;
    // only the boundary switches the reference defines (3DRB.F90:14-37, 2DRB.F90:15-32)
    if (p->bc_flow[0] != LBM_BC_NOSLIP && p->bc_flow[0] != LBM_BC_PERIODIC) return LBM_ERR_PARAM;
    if (p->bc_flow[1] != LBM_BC_NOSLIP) return LBM_ERR_PARAM;
    if (p->bc_thermal[0] < LBM_BCT_CONST || p->bc_thermal[0] > LBM_BCT_PERIODIC) return LBM_ERR_PARAM;
    if (p->bc_thermal[1] != LBM_BCT_CONST && p->bc_thermal[1] != LBM_BCT_ADIABATIC) return LBM_ERR_PARAM;
    if (p->dim == 3) {
        if (p->bc_flow[2] != LBM_BC_NOSLIP && p->bc_flow[2] != LBM_BC_PERIODIC) return LBM_ERR_PARAM;
        if (p->bc_thermal[2] != LBM_BCT_ADIABATIC && p->bc_thermal[2] != LBM_BCT_PERIODIC) return LBM_ERR_PARAM;
    }
    if (p->precision < LBM_FP64 || p->precision > LBM_FP16) return LBM_ERR_PARAM;
    if (p->pattern != LBM_PATTERN_AB && p->pattern != LBM_PATTERN_AA) return LBM_ERR_PARAM;
    // the fixed arithmetic: FP64 handles, two-buffer pattern, without the magnetic force
    if (p->arith != LBM_ARITH_REFERENCE && p->arith != LBM_ARITH_FIXED) return LBM_ERR_PARAM;
    if (p->arith == LBM_ARITH_FIXED &&
        (p->precision != LBM_FP64 || p->pattern != LBM_PATTERN_AB || p->side_heated_ha))
        return LBM_ERR_PARAM;
    // the magnetic force exists in the 2D program only (2DRB.F90:88-92); the FP32/FP16 forms
    // carry only F_y in their lag state
    if (p->side_heated_ha && (p->dim != 2 || p->precision != LBM_FP64 || !std::isfinite(p->Ha) ||
                              !std::isfinite(p->phi_deg)))
        return LBM_ERR_PARAM;
    return LBM_OK;
}

// ------------------------------------------------------------------------------------
// parameters
// ------------------------------------------------------------------------------------
extern "C" int lbm_params_default(int dim, lbm_params* out) {
    if (!out || (dim != 2 && dim != 3)) return LBM_ERR_PARAM;
    std::memset(out, 0, sizeof(*out));
    out->dim = dim;
    if (dim == 2) {  // 2DRB.F90:11-38, 61-71
        out->nx = 320; out->ny = 160; out->nz = 1;
        out->Ra = 5.0e4;
        out->bc_flow[0] = LBM_BC_PERIODIC;
        out->bc_thermal[0] = LBM_BCT_PERIODIC;
    } else {  // RayleighBenardCell variant of 3DRB.F90:9-47, 73-83
        out->nx = 120; out->ny = 120; out->nz = 120;
        out->Ra = 1.0e7;
        out->bc_flow[0] = LBM_BC_NOSLIP;
        out->bc_thermal[0] = LBM_BCT_ADIABATIC;
    }
    out->Pr = 0.71;
    out->Mach = 0.1;
    out->Thot = 0.5;
    out->Tcold = -0.5;
    out->cell = LBM_CELL_RB;
    out->bc_flow[1] = LBM_BC_NOSLIP;
    out->bc_flow[2] = LBM_BC_NOSLIP;
    out->bc_thermal[1] = LBM_BCT_CONST;
    out->bc_thermal[2] = LBM_BCT_ADIABATIC;
    out->use_g = 1;
    out->legacy_thermal = 0;
    out->precision = LBM_FP64;
    out->pattern = LBM_PATTERN_AB;
    out->seed = 20261203ULL;
    out->noise_amp = 0.0;
    out->side_heated_ha = 0;
    out->Ha = 20.0;
    out->phi_deg = 0.0;
    return LBM_OK;
}

// commondata (2DRB.F90:61-115) / commondata3d (3DRB.F90:73-123), same operation order.
extern "C" int lbm_derive_constants(const lbm_params* p, lbm_constants* c) {
    if (!c || validate(p) != LBM_OK) return LBM_ERR_PARAM;
    std::memset(c, 0, sizeof(*c));
    const double L = (p->cell == LBM_CELL_SIDE) ? (double)p->nx : (double)p->ny;
    c->lengthUnit = L;
    c->Tref = 0.5 * (p->Thot + p->Tcold);
    c->tauf = 0.5 + p->Mach * L * std::sqrt(3.0 * p->Pr / p->Ra);
    c->viscosity = (c->tauf - 0.5) / 3.0;
    c->diffusivity = c->viscosity / p->Pr;
    c->heatFluxScale = L / c->diffusivity;
    c->velocityScaleCompare = L / c->diffusivity;
    const double gBeta1 = p->Ra * c->viscosity * c->diffusivity / L;
    c->gBeta = gBeta1 / L / L;
    c->timeUnit = std::sqrt(L / c->gBeta);
    c->velocityUnit = std::sqrt(c->gBeta * L);
    c->Snu = 1.0 / c->tauf;
    c->Sq = 8.0 * (2.0 * c->tauf - 1.0) / (8.0 * c->tauf - 1.0);
    if (p->dim == 2) {
        c->paraA = 20.0 * std::sqrt(3.0) * c->diffusivity - 4.0;
        if (p->legacy_thermal) {
            if ((c->paraA >= 1.0) || (c->paraA <= -4.0)) return LBM_ERR_PARAM;  // 2DRB.F90:404-414
            c->Qk = 3.0 - std::sqrt(3.0);
            c->Qnu = 4.0 * std::sqrt(3.0) - 6.0;
            c->thermalGeqCoeff = 10.0 / (4.0 + c->paraA);
            c->omegaT0 = (1.0 - c->paraA) / 5.0;
            c->omegaT1 = (c->paraA + 4.0) / 20.0;
        } else {
            c->taug = 0.5 + (c->tauf - 0.5) / p->Pr;
            c->Qnu = 1.0;
            c->Qk = 1.0 / c->taug;
            c->thermalGeqCoeff = 3.0;
            c->omegaT0 = 1.0 / 3.0;
            c->omegaT1 = 1.0 / 6.0;
        }
    } else {
        c->cs2T = 0.25;
        c->paraA = 42.0 * std::sqrt(3.0) * c->diffusivity - 6.0;
        c->Se = 1.0 / c->tauf;
        c->Seps = 1.0 / c->tauf;
        c->Spi = 1.0 / c->tauf;
        c->Sm = 8.0 * (2.0 * c->tauf - 1.0) / (8.0 * c->tauf - 1.0);
        if (p->legacy_thermal) {
            if ((c->paraA >= 1.0) || (c->paraA <= -6.0)) return LBM_ERR_PARAM;  // 3DRB.F90:379-388
            c->Qk = 3.0 - std::sqrt(3.0);
            c->Qnu = 4.0 * std::sqrt(3.0) - 6.0;
            c->thermalGeqCoeff = 7.0 / ((6.0 + c->paraA) * c->cs2T);
            c->omegaT0 = (1.0 - c->paraA) / 7.0;
            c->omegaT1 = (6.0 + c->paraA) / 42.0;
        } else {
            c->taug = 0.5 + c->diffusivity / c->cs2T;
            c->Qnu = 1.0;
            c->Qk = 1.0 / c->taug;
            c->thermalGeqCoeff = 1.0 / c->cs2T;
            c->omegaT0 = 1.0 / 4.0;
            c->omegaT1 = 1.0 / 8.0;
        }
    }
    c->SG = 1.0 - 0.5 * c->Qk;
    if (p->side_heated_ha) {
        // 2DRB.F90:67, 89-91: pi = acos(-1), phi = deg*(pi/180), B2sigemarho = Ha**2 nu / L^2
        const double pi = std::acos(-1.0);
        c->phi = p->phi_deg * (pi / 180.0);
        c->B2sigemarho = (p->Ha * p->Ha * c->viscosity) / (L * L);
        c->sinphi = std::sin(c->phi);
        c->cosphi = std::cos(c->phi);
    }
    if (!(c->tauf > 0.5)) return LBM_ERR_PARAM;
    return LBM_OK;
}

// ------------------------------------------------------------------------------------
// lifecycle
// ------------------------------------------------------------------------------------
static void release(lbm_handle* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    if (h->xgraph_exec) cudaGraphExecDestroy(h->xgraph_exec);
    if (h->xgraph) cudaGraphDestroy(h->xgraph);
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    if (h->stream) cudaStreamDestroy(h->stream);
    h->stream = nullptr;
}

static int allocate(lbm_handle* h) {
    const long long n = h->geo.ncell;
    const bool d3 = h->dim == 3;
    int st;
#define AL(ptr, cnt)                                      \
    do {                                                  \
        if ((st = dalloc(h, &(ptr), (size_t)(cnt))) != LBM_OK) return st; \
    } while (0)
    if (h->p.precision == LBM_FP64 && h->p.pattern == LBM_PATTERN_AA) {
        // one array per lattice, which is also the module array; no f_post / g_post
        AL(h->A.f, h->q * n);
        AL(h->A.g, h->qt * n);
        h->fbuf[0] = h->A.f;
        h->gbuf[0] = h->A.g;
        h->A.fpost = nullptr;
        h->A.gpost = nullptr;
        for (int ax = 0; ax < 3; ++ax) {
            double* pf = nullptr;
            double* pg = nullptr;
            if (h->geo.bcf[ax] == LBM_BC_PERIODIC) AL(pf, (size_t)h->q * aa_face_cells(h->geo, ax));
            if (h->geo.bct[ax] == LBM_BCT_PERIODIC) AL(pg, (size_t)h->qt * aa_face_cells(h->geo, ax));
            h->aa.face_f[ax] = pf;
            h->aa.face_g[ax] = pg;
        }
    }
    if (h->p.precision == LBM_FP64) {
        if (h->p.pattern != LBM_PATTERN_AA) {
            AL(h->fbuf[0], h->q * n);
            AL(h->fbuf[1], h->q * n);
            AL(h->gbuf[0], h->qt * n);
            AL(h->gbuf[1], h->qt * n);
            AL(h->A.f, h->q * n);
            AL(h->A.g, h->qt * n);
            h->A.fpost = h->fbuf[0];
            h->A.gpost = h->gbuf[0];
        }
        AL(h->A.rho, n);
        AL(h->A.u, n);
        AL(h->A.v, n);
        AL(h->A.T, n);
        AL(h->A.Bx, n);
        AL(h->A.By, n);
        AL(h->A.up, n);
        AL(h->A.vp, n);
        AL(h->A.Tp, n);
        if (d3) {
            AL(h->A.w, n);
            AL(h->A.Bz, n);
            AL(h->A.wp, n);
            AL(h->A.Tlag, n);
            AL(h->A.jz, n);
        } else {
            AL(h->A.Fx, n);
            AL(h->A.Fy, n);
        }
        AL(h->A.jx, n);
        AL(h->A.jy, n);
        if (h->fixed) {
            AL(h->xb0, n);
            AL(h->xb1, n);
            if (d3) AL(h->xb2, n);
            AL(h->xlag, n);
            if (d3 && fixed_fused_supported(h->geo, h->dim)) {
                AL(h->xb0b, n);
                AL(h->xb1b, n);
                AL(h->xb2b, n);
            }
        }
    } else {
        st = fast_allocate(h->F, h->p, h->geo, [h](void** p, size_t bytes) {
            cudaError_t e = cudaMalloc(p, bytes > 0 ? bytes : 1);
            if (e != cudaSuccess) return cuda_fail(h, e, "cudaMalloc");
            h->allocs.push_back(*p);
            return LBM_OK;
        });
        if (st != LBM_OK) return st;
    }
    AL(h->d_part, (size_t)diag_blocks(n) * DIAG_NSUM);
    AL(h->d_tb, h->geo.nx);
    AL(h->d_nub, h->geo.nx);
    AL(h->d_tl, h->geo.ny);
    AL(h->d_nul, h->geo.ny);
    AL(h->d_sx, h->geo.nx);
    AL(h->d_sy, h->geo.ny);
#undef AL
    h->h_part.assign((size_t)diag_blocks(n) * DIAG_NSUM, 0.0);
    return LBM_OK;
}

extern "C" int lbm_create(const lbm_params* p, int device, lbm_handle** out) {
    if (!out) return LBM_ERR_PARAM;
    *out = nullptr;
    if (validate(p) != LBM_OK) return LBM_ERR_PARAM;
    lbm_handle* h = new (std::nothrow) lbm_handle();
    if (!h) return LBM_ERR_OOM;
    h->p = *p;
    if (lbm_derive_constants(p, &h->c) != LBM_OK) {
        delete h;
        return LBM_ERR_PARAM;
    }
    h->dim = p->dim;
    h->q = p->dim == 3 ? 19 : 9;
    h->qt = p->dim == 3 ? 7 : 5;
    h->device = device;
    const lbm_constants& c = h->c;

    h->geo = make_geo(*p, c);
    h->phys = make_physc(*p, c);
    if (p->arith == LBM_ARITH_FIXED) {
        h->fixed = true;
        h->xgeo = deviation_geo(h->geo, c);
        if (!make_physx(*p, c, h->px)) {  // a relaxation constant out of the q60 range
            delete h;
            return LBM_ERR_PARAM;
        }
    }
    DiagScalars& D = h->dsc;
    D.Thot = p->Thot;
    D.Tcold = p->Tcold;
    D.Tref = c.Tref;
    D.dy = 1.0 / c.lengthUnit;
    D.deltaT = p->Thot - p->Tcold;
    D.coef = c.velocityScaleCompare;
    D.side = p->cell == LBM_CELL_SIDE;
    D.d3 = p->dim == 3;

    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        delete h;
        return LBM_ERR_CUDA;
    }
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete h;
        return LBM_ERR_CUDA;
    }
    int st = allocate(h);
    if (st != LBM_OK) {
        release(h);
        delete h;
        return st;
    }
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) == cudaSuccess && pageable) {
        // reads of the caller's array by the layout kernels only: writes into freshly
        // allocated host memory fault its pages in from the GPU side, measured at 3-4.5 GB/s
        // on GB300 against 9-27 GB/s for a staged copy (reads: 195-204 against 166-184 GB/s)
        h->host_access = true;
        h->host_direct = true;
    }
    *out = h;
    return LBM_OK;
}

extern "C" int lbm_ensemble_remove(lbm_ensemble* e, lbm_handle* h);

extern "C" int lbm_destroy(lbm_handle* h) {
    if (!h) return LBM_ERR_PARAM;
    if (h->ensemble) lbm_ensemble_remove(h->ensemble, h);
    if (h->order_ev) cudaEventDestroy(h->order_ev);
    release(h);
    delete h;
    return LBM_OK;
}

extern "C" const char* lbm_last_error(const lbm_handle* h) { return h ? h->err.c_str() : "null handle"; }

extern "C" const char* lbm_status_string(int s) {
    switch (s) {
        case LBM_OK: return "LBM_OK";
        case LBM_ERR_PARAM: return "LBM_ERR_PARAM";
        case LBM_ERR_CUDA: return "LBM_ERR_CUDA";
        case LBM_ERR_OOM: return "LBM_ERR_OOM";
        case LBM_ERR_DIVERGED: return "LBM_ERR_DIVERGED";
        case LBM_ERR_TIMEOUT: return "LBM_ERR_TIMEOUT";
        case LBM_ERR_STATE: return "LBM_ERR_STATE";
        case LBM_ERR_TOO_LARGE: return "LBM_ERR_TOO_LARGE";
        default: return "unknown status";
    }
}

extern "C" int lbm_get_params(const lbm_handle* h, lbm_params* out) {
    if (!h || !out) return LBM_ERR_PARAM;
    *out = h->p;
    return LBM_OK;
}

extern "C" int lbm_get_constants(const lbm_handle* h, lbm_constants* out) {
    if (!h || !out) return LBM_ERR_PARAM;
    *out = h->c;
    return LBM_OK;
}

extern "C" int64_t lbm_itc(const lbm_handle* h) { return h ? h->itc : -1; }

// A staged FP32/FP16 kernel whose bounded wait gave up leaves a device flag set.
static int take_device_error(lbm_handle* h) {
    if (h->p.precision == LBM_FP64) return LBM_OK;
    const int st = fast_take_error(h->F, h->stream);
    if (st == LBM_ERR_TIMEOUT) return fail(h, st, "a staged kernel timed out waiting for its bulk copies");
    if (st != LBM_OK) return fail(h, st, "reading the device error flag failed");
    return LBM_OK;
}

extern "C" int lbm_selftest_wait_timeout(lbm_handle* h, int64_t polls) {
    if (!h || polls <= 0 || polls > (1LL << 24)) return LBM_ERR_PARAM;
    if (h->p.precision == LBM_FP64) return fail(h, LBM_ERR_STATE, "the staged kernels exist for FP32/FP16 handles");
    CK(h, cudaSetDevice(h->device));
    fast_wait_selftest(h->F, (unsigned)polls, h->stream);
    CK_LAUNCH(h, "wait self-test");
    return LBM_OK;
}

extern "C" int lbm_sync(lbm_handle* h) {
    if (!h) return LBM_ERR_PARAM;
    CK(h, cudaSetDevice(h->device));
    CK(h, cudaStreamSynchronize(h->stream));
    return take_device_error(h);
}

// ------------------------------------------------------------------------------------
// initial (2DRB.F90:371-663, 3DRB.F90:342-643)
// ------------------------------------------------------------------------------------
extern "C" int lbm_initial(lbm_handle* h) {
    if (!h) return LBM_ERR_PARAM;
    CK(h, cudaSetDevice(h->device));
    const lbm_params& p = h->p;
    const double L = h->c.lengthUnit;
    InitC I{};
    I.L = L;
    I.Thot = p.Thot;
    I.Tcold = p.Tcold;
    I.noise_amp = p.noise_amp;
    I.seed = p.seed;
    I.sx = h->d_sx;
    I.sy = h->d_sy;
    // RB sinusoidal perturbation, only for small Ra (2DRB.F90:567-581: Ra < 1e4;
    // 3DRB.F90:545-556: Ra <= 1e4).  sin/cos come from the host libm.
    const bool small_ra = h->dim == 2 ? (p.Ra < 1.0e4) : (p.Ra <= 1.0e4);
    I.perturb = (p.cell == LBM_CELL_RB && p.bc_thermal[1] == LBM_BCT_CONST && small_ra) ? 1 : 0;
    I.pert_amp = 1.0e-3 * (p.Thot - p.Tcold);
    if (I.perturb) {
        const int nx = h->geo.nx, ny = h->geo.ny;
        std::vector<double> sx(nx), sy(ny);
        const double xLen = (double)nx / L, yLen = (double)ny / L;
        for (int i = 1; i <= nx; ++i) {
            const double xp = ((double)i - 0.5) / L;
            sx[i - 1] = h->dim == 3 ? std::cos(2.0 * kPi * xp / xLen) : std::sin(2.0 * kPi * xp / xLen);
        }
        for (int j = 1; j <= ny; ++j) {
            const double yp = ((double)j - 0.5) / L;
            sy[j - 1] = std::sin(kPi * yp / yLen);
        }
        CK(h, cudaMemcpyAsync(h->d_sx, sx.data(), nx * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        CK(h, cudaMemcpyAsync(h->d_sy, sy.data(), ny * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    if (h->p.precision == LBM_FP64) {
        if (h->p.pattern != LBM_PATTERN_AA) {
            h->A.fpost = h->fbuf[0];
            h->A.gpost = h->gbuf[0];
        }
        h->cur = 0;
        h->fused_valid = false;
        h->aa.fpar = h->aa.gpar = 0;  // module data in the streamed layout
        h->aa.graw = false;
        exact_initial(h->geo, h->phys, I, h->A, h->dim, h->stream);
    } else {
        fast_initial(h->F, h->geo, h->phys, I, h->dim, h->stream);
    }
    CK_LAUNCH(h, "initial");
    h->itc = 0;
    h->initialised = true;
    return LBM_OK;
}

// The arrays the fixed-arithmetic kernels read and write.
static FixedArrays fixed_arrays(const lbm_handle* h) {
    const ExactArrays& A = h->A;
    FixedArrays X{};
    X.f = A.f;
    X.g = A.g;
    X.rho = A.rho;
    X.u = A.u;
    X.v = A.v;
    X.w = A.w;
    X.T = A.T;
    X.Bx = A.Bx;
    X.By = A.By;
    X.Bz = A.Bz;
    X.Tlag = A.Tlag;
    X.Fx = A.Fx;
    X.Fy = A.Fy;
    X.xb0 = h->xb0;
    X.xb1 = h->xb1;
    X.xb2 = h->xb2;
    X.xlag = h->xlag;
    return X;
}

// Rebuild the module arrays from the fused buffers (no-op when already there).  The fixed
// arithmetic keeps its q60 buffers as the state: the module arrays are a rounded FP64 copy,
// so how often a caller reads diagnostics does not change the run.
static int materialize(lbm_handle* h) {
    if (h->p.precision != LBM_FP64) {
        fast_materialize(h->F, h->geo, h->phys, h->dim, h->stream);
        CK_LAUNCH(h, "materialize");
        return LBM_OK;
    }
    if (!h->fused_valid) return LBM_OK;
    if (h->fixed) {
        fixed_materialize(h->xgeo, h->px, fixed_arrays(h), h->dim, (const long long*)h->fbuf[h->cur],
                          (const long long*)h->gbuf[h->cur], h->stream);
        CK_LAUNCH(h, "materialize");
        return LBM_OK;
    }
    if (h->p.pattern == LBM_PATTERN_AA) {
        // the arrays are the module populations; the state stays where it is
        exact_aa_materialize(h->geo, h->phys, h->A, h->dim, h->aa, h->stream);
        CK_LAUNCH(h, "materialize");
        return LBM_OK;
    }
    exact_materialize(h->geo, h->phys, h->A, h->dim, h->fbuf[h->cur], h->gbuf[h->cur], h->stream);
    CK_LAUNCH(h, "materialize");
    h->A.fpost = h->fbuf[h->cur];
    h->A.gpost = h->gbuf[h->cur];
    h->fused_valid = false;
    return LBM_OK;
}

// Fixed arithmetic: make the FP64 module arrays the state again (before a stage kernel or a
// state load): materialise, turn the q60 fused buffers into the FP64 post-collision arrays
// the stage kernels read, and start the next fused step from the module arrays.
static int release_fixed(lbm_handle* h) {
    if (!h->fixed || !h->fused_valid) return LBM_OK;
    int st = materialize(h);
    if (st != LBM_OK) return st;
    fixed_post_to_double(h->px, (long long*)h->fbuf[h->cur], (long long*)h->gbuf[h->cur], h->geo.ncell, h->q, h->qt,
                         h->stream);
    CK_LAUNCH(h, "post-collision conversion");
    h->A.fpost = h->fbuf[h->cur];
    h->A.gpost = h->gbuf[h->cur];
    h->fused_valid = false;
    return LBM_OK;
}

// ------------------------------------------------------------------------------------
// stage entry points
// ------------------------------------------------------------------------------------
static int stage(lbm_handle* h, int which) {
    if (!h) return LBM_ERR_PARAM;
    if (!h->initialised) return fail(h, LBM_ERR_STATE, "lbm_initial has not been called");
    if (h->p.precision != LBM_FP64)
        return fail(h, LBM_ERR_STATE, "stage entry points exist for the FP64 plain method only");
    if (h->p.pattern == LBM_PATTERN_AA)
        return fail(h, LBM_ERR_STATE, "stage entry points need the two-buffer pattern (separate f and f_post)");
    CK(h, cudaSetDevice(h->device));
    int st = h->fixed ? release_fixed(h) : materialize(h);
    if (st != LBM_OK) return st;
    if (which == STAGE_COLLISION) h->itc += 1;
    exact_stage(which, h->geo, h->phys, h->A, h->dim, h->stream);
    CK_LAUNCH(h, "stage kernel");
    return LBM_OK;
}

extern "C" int lbm_collision(lbm_handle* h) { return stage(h, STAGE_COLLISION); }
extern "C" int lbm_streaming(lbm_handle* h) { return stage(h, STAGE_STREAMING); }
extern "C" int lbm_bounceback(lbm_handle* h) { return stage(h, STAGE_BOUNCEBACK); }
extern "C" int lbm_macro(lbm_handle* h) { return stage(h, STAGE_MACRO); }
extern "C" int lbm_collisionT(lbm_handle* h) { return stage(h, STAGE_COLLISIONT); }
extern "C" int lbm_streamingT(lbm_handle* h) { return stage(h, STAGE_STREAMINGT); }
extern "C" int lbm_bouncebackT(lbm_handle* h) { return stage(h, STAGE_BOUNCEBACKT); }
extern "C" int lbm_macroT(lbm_handle* h) { return stage(h, STAGE_MACROT); }

// ------------------------------------------------------------------------------------
// fused stepping
// ------------------------------------------------------------------------------------
// FP32/FP16 handles advance with the single fused kernel (lbm_fused.cu) unless it is
// switched off or the geometry needs whole tiles it does not have.
static bool use_single(const lbm_handle* h) {
    return h->p.precision != LBM_FP64 && !h->F.aa && h->F.single_kernel && fast_fused_supported(h->geo, h->dim);
}

static bool in_place(const lbm_handle* h) { return h->p.pattern == LBM_PATTERN_AA; }

static const AAState& aa_state(const lbm_handle* h) { return h->p.precision == LBM_FP64 ? h->aa : h->F.AA; }

static void enqueue_one(lbm_handle* h, bool first) {
    const int nxt = h->cur ^ 1;
    if (h->p.precision == LBM_FP64 && in_place(h)) {
        exact_aa_step(h->geo, h->phys, h->A, h->dim, first, h->aa, h->stream);
    } else if (h->p.precision == LBM_FP64 && h->fixed) {
        fixed_fused_step(h->xgeo, h->px, fixed_arrays(h), h->dim, first, (const long long*)h->fbuf[h->cur],
                         (const long long*)h->gbuf[h->cur], (long long*)h->fbuf[nxt], (long long*)h->gbuf[nxt],
                         h->stream, 2, h->wide_index);
        h->cur = nxt;
    } else if (h->p.precision == LBM_FP64) {
        exact_fused_step(h->geo, h->phys, h->A, h->dim, first, h->fbuf[h->cur], h->gbuf[h->cur], h->fbuf[nxt],
                         h->gbuf[nxt], h->stream);
        h->cur = nxt;
    } else if (first || !use_single(h)) {
        fast_step(h->F, h->geo, h->phys, h->dim, first, h->stream);
    } else {
        if (!h->F.ahead) fast_enter(h->F, h->geo, h->phys, h->dim, h->stream);
        fast_fused_step(h->F, h->geo, h->phys, h->dim, h->stream);
    }
}

// In-place pattern: a chunk (an even number of steps) starts and ends with the flow array
// in the streamed layout; the thermal array's layout and its push flag are part of what
// was captured, so a chunk replays only from the state it was captured in.
static int layout_key(const lbm_handle* h) {
    const AAState& S = aa_state(h);
    return 1 + S.gpar + 2 * (S.graw ? 1 : 0);
}

static bool at_graph_origin(const lbm_handle* h) {
    if (in_place(h)) return aa_state(h).fpar == 0;
    return h->p.precision == LBM_FP64 ? h->cur == 0 : fast_at_origin(h->F);
}

static void drop_chunk(lbm_handle* h) {
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->graph_exec = nullptr;
    h->graph = nullptr;
}

static int capture_chunk(lbm_handle* h) {
    h->graph_key = in_place(h) ? layout_key(h) : 0;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < kChunkSteps; ++s) enqueue_one(h, false);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
    h->graph = g;
    CK(h, cudaGraphInstantiate(&h->graph_exec, g, 0));
    return LBM_OK;
}

// ---- fused passes of the fixed arithmetic (3D) --------------------------------------------
// Between lbm_step calls the handle is in the two-kernel state (f_post_N, g_post_N).  A run of
// steps enters the fused state (f_post_{N+1}, g_post_N) with the flow half of one step, runs
// one fused pass per further step, and leaves with the thermal half of the last step.
static bool use_xfused(const lbm_handle* h) {
    return h->fixed && h->xfused && h->xb0b && fixed_fused_supported(h->geo, h->dim);
}

static void x_enter(lbm_handle* h) {
    const int nxt = h->cur ^ 1;
    fixed_fused_step(h->xgeo, h->px, fixed_arrays(h), h->dim, false, (const long long*)h->fbuf[h->cur],
                     (const long long*)h->gbuf[h->cur], (long long*)h->fbuf[nxt], nullptr, h->stream, 0,
                     h->wide_index);
    h->cur = nxt;  // f is one step ahead: fbuf[cur] = f_post_{N+1}, gbuf[cur ^ 1] = g_post_N
}

static void x_pass(lbm_handle* h) {
    const int c = h->cur, o = c ^ 1;
    const long long* bin[3] = {h->xb0, h->xb1, h->xb2};
    long long* const bout[3] = {h->xb0b, h->xb1b, h->xb2b};
    fixed_fused_pass(h->xgeo, h->px, (const long long*)h->fbuf[c], (const long long*)h->gbuf[o], (long long*)h->fbuf[o],
                     (long long*)h->gbuf[c], bin, bout, h->stream);
    h->cur = o;
    std::swap(h->xb0, h->xb0b);
    std::swap(h->xb1, h->xb1b);
    std::swap(h->xb2, h->xb2b);
}

static void x_exit(lbm_handle* h) {
    const int c = h->cur;
    fixed_fused_step(h->xgeo, h->px, fixed_arrays(h), h->dim, false, nullptr, (const long long*)h->gbuf[c ^ 1],
                     (long long*)h->fbuf[c], (long long*)h->gbuf[c], h->stream, 1, h->wide_index);
}

// Capture key of a chunk of fused passes: the buffer parity and which B_prev set is current.
static int x_key(const lbm_handle* h) { return h->cur + 2 * (h->xb0 < h->xb0b ? 1 : 0); }

static int x_run(lbm_handle* h, int64_t passes) {
    while (passes > 0) {
        if (passes >= kChunkSteps) {
            if (h->xgraph_exec && h->xgraph_key != x_key(h)) {
                CK(h, cudaStreamSynchronize(h->stream));
                cudaGraphExecDestroy(h->xgraph_exec);
                cudaGraphDestroy(h->xgraph);
                h->xgraph_exec = nullptr;
                h->xgraph = nullptr;
            }
            if (!h->xgraph_exec) {
                h->xgraph_key = x_key(h);
                CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
                for (int s = 0; s < kChunkSteps; ++s) x_pass(h);
                cudaGraph_t g = nullptr;
                cudaError_t e = cudaStreamEndCapture(h->stream, &g);
                if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
                h->xgraph = g;
                CK(h, cudaGraphInstantiate(&h->xgraph_exec, g, 0));
            }
            // a chunk holds an even number of passes: the buffer parity and the current B_prev
            // set after it are those before it
            CK(h, cudaGraphLaunch(h->xgraph_exec, h->stream));
            passes -= kChunkSteps;
        } else {
            x_pass(h);
            passes -= 1;
        }
    }
    return LBM_OK;
}

extern "C" int lbm_step(lbm_handle* h, int64_t nsteps) {
    NvtxRange range_("lbm_step");
    if (!h) return LBM_ERR_PARAM;
    if (nsteps < 0) return fail(h, LBM_ERR_PARAM, "nsteps < 0");
    if (!h->initialised) return fail(h, LBM_ERR_STATE, "lbm_initial has not been called");
    if (nsteps == 0) return LBM_OK;
    CK(h, cudaSetDevice(h->device));
    int64_t done = 0;
    const bool fused = h->p.precision == LBM_FP64 ? h->fused_valid : fast_fused_valid(h->F);
    if (!fused) {
        enqueue_one(h, true);
        if (h->p.precision == LBM_FP64) h->fused_valid = true;
        done = 1;
    }
    // enter the single-kernel phase outside any captured graph
    if (use_single(h) && !h->F.ahead && done < nsteps) fast_enter(h->F, h->geo, h->phys, h->dim, h->stream);
    if (use_xfused(h) && nsteps - done >= 2) {
        x_enter(h);
        int st = x_run(h, nsteps - done - 1);
        if (st != LBM_OK) return st;
        x_exit(h);
        done = nsteps;
    }
    while (done < nsteps) {
        if (at_graph_origin(h) && nsteps - done >= kChunkSteps) {
            if (h->graph_exec && in_place(h) && h->graph_key != layout_key(h)) {
                CK(h, cudaStreamSynchronize(h->stream));
                drop_chunk(h);
            }
            if (!h->graph_exec) {
                int st = capture_chunk(h);
                if (st != LBM_OK) return st;
            }
            CK(h, cudaGraphLaunch(h->graph_exec, h->stream));
            done += kChunkSteps;
            // a chunk holds odd thermal sweeps: the thermal array's slots are pushed values now
            if (in_place(h)) (h->p.precision == LBM_FP64 ? h->aa : h->F.AA).graw = true;
        } else {
            enqueue_one(h, false);
            done += 1;
        }
    }
    CK_LAUNCH(h, "fused step");
    h->itc += nsteps;
    return LBM_OK;
}

// ------------------------------------------------------------------------------------
// diagnostics
// ------------------------------------------------------------------------------------
static int run_reduce(lbm_handle* h, DiagOp op, double sums[DIAG_NSUM]) {
    NvtxRange range_("diagnostic reduction");
    const int nb = diag_blocks(op == DIAG_NU_COLD_MID ? (long long)h->geo.nx * h->geo.nz : h->geo.ncell);
    if (h->p.precision == LBM_FP64) {
        DiagFields<double> F{h->A.u, h->A.v, h->A.w, h->A.T, h->A.rho, h->A.up, h->A.vp, h->A.wp, h->A.Tp};
        diag_reduce<double>(op, h->geo, h->dsc, F, h->d_part, nb, h->stream);
    } else {
        DiagFields<float> F = fast_diag_fields(h->F);
        diag_reduce<float>(op, h->geo, h->dsc, F, h->d_part, nb, h->stream);
    }
    CK_LAUNCH(h, "reduction");
    CK(h, cudaMemcpyAsync(h->h_part.data(), h->d_part, (size_t)nb * DIAG_NSUM * sizeof(double), cudaMemcpyDeviceToHost,
                          h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (int s = 0; s < DIAG_NSUM; ++s) sums[s] = 0.0;
    for (int b = 0; b < nb; ++b)
        for (int s = 0; s < DIAG_NSUM; ++s) sums[s] += h->h_part[(size_t)b * DIAG_NSUM + s];
    return LBM_OK;
}

static int diag_prologue(lbm_handle* h) {
    if (!h) return LBM_ERR_PARAM;
    if (!h->initialised) return fail(h, LBM_ERR_STATE, "lbm_initial has not been called");
    CK(h, cudaSetDevice(h->device));
    int st = take_device_error(h);
    if (st != LBM_OK) return st;
    return materialize(h);
}

extern "C" int lbm_check(lbm_handle* h, double* errU, double* errT) {
    int st = diag_prologue(h);
    if (st != LBM_OK) return st;
    if (!errU || !errT) return fail(h, LBM_ERR_PARAM, "null output");
    double s[DIAG_NSUM];
    if ((st = run_reduce(h, DIAG_CHECK, s)) != LBM_OK) return st;
    if (h->dim == 3) {  // 3DRB.F90:1511-1520
        *errU = (s[1] > 1.0e-30) ? std::sqrt(s[0]) / std::sqrt(s[1]) : std::sqrt(s[0]);
        *errT = (s[3] > 1.0e-30) ? s[2] / s[3] : s[2];
    } else {  // 2DRB.F90:1244-1245
        *errU = std::sqrt(s[0]) / std::sqrt(s[1]);
        *errT = s[2] / s[3];
    }
    if (s[4] != 0.0 || !std::isfinite(s[0]) || !std::isfinite(s[2]))
        return fail(h, LBM_ERR_DIVERGED, "non-finite field or rho <= 0 in " + std::to_string((long long)s[4]) + " cells");
    return LBM_OK;
}

// caseTag of check: '("Ra=",ES10.3E2,",nx=",I0,",ny=",I0[,",nz=",I0],",useG=",L1,",old=",L1)'
// (2DRB.F90:1252-1253, 3DRB.F90:1523-1524).
extern "C" int lbm_case_tag(const lbm_handle* h, char* buf, size_t len) {
    if (!h || !buf) return LBM_ERR_PARAM;
    char ra[32];
    int st = lbm_format_fortran_es(h->p.Ra, 10, 3, 2, ra, sizeof(ra));
    if (st != LBM_OK) return st;
    std::string t = std::string("Ra=") + ra + ",nx=" + std::to_string(h->p.nx) + ",ny=" + std::to_string(h->p.ny);
    if (h->dim == 3) t += ",nz=" + std::to_string(h->p.nz);
    t += std::string(",useG=") + (h->p.use_g ? "T" : "F") + ",old=" + (h->p.legacy_thermal ? "T" : "F");
    if (t.size() + 1 > len) return LBM_ERR_PARAM;
    std::memcpy(buf, t.c_str(), t.size() + 1);
    return LBM_OK;
}

extern "C" int lbm_append_convergence_tecplot(lbm_handle* h, const char* filename, int64_t itc, double errorU,
                                              double errorT) {
    if (!h || !filename) return LBM_ERR_PARAM;
    const int st = lbm_append_convergence_tecplot_host(filename, h->conv_started ? 0 : 1, h->dim, itc, errorU, errorT);
    h->conv_started = true;
    return st == LBM_OK ? LBM_OK : fail(h, st, std::string("cannot write ") + filename);
}

extern "C" int lbm_append_convergence_master_tecplot(lbm_handle* h, const char* filename, const char* zone, int64_t itc,
                                                     double errorU, double errorT) {
    if (!h || !filename || !zone) return LBM_ERR_PARAM;
    const int st = lbm_append_convergence_master_tecplot_host(filename, h->conv_zone_started ? 0 : 1, h->dim, zone, itc,
                                                              errorU, errorT);
    h->conv_zone_started = true;
    return st == LBM_OK ? LBM_OK : fail(h, st, std::string("cannot write ") + filename);
}

// check as the reference's subroutine does it: the errors, then the record appended to the
// run's file and (under the case tag) to the master file, then echoed to standard output
// (2DRB.F90:1244-1258, 3DRB.F90:1511-1526).  A diverged field is still logged (its errors
// are NaN) and reported as LBM_ERR_DIVERGED.
extern "C" int lbm_check_log(lbm_handle* h, const char* dir, int echo, double* errU, double* errT) {
    if (!h || !errU || !errT) return LBM_ERR_PARAM;
    const int chk = lbm_check(h, errU, errT);
    if (chk != LBM_OK && chk != LBM_ERR_DIVERGED) return chk;
    const std::string d = (dir && *dir) ? std::string(dir) + "/" : std::string();
    const bool d3 = h->dim == 3;
    int st = lbm_append_convergence_tecplot(h, (d + (d3 ? "convergence3D.plt" : "convergence.plt")).c_str(), h->itc,
                                            *errU, *errT);
    if (st != LBM_OK) return st;
    char tag[256];
    if ((st = lbm_case_tag(h, tag, sizeof(tag))) != LBM_OK) return fail(h, st, "case tag");
    st = lbm_append_convergence_master_tecplot(h, (d + (d3 ? "convergence_all_3D.plt" : "convergence_all.plt")).c_str(),
                                               tag, h->itc, *errU, *errT);
    if (st != LBM_OK) return st;
    if (echo) {
        char line[128];
        if (lbm_convergence_line(h->itc, *errU, *errT, line, sizeof(line)) == LBM_OK) {
            std::fputs(line, stdout);
            std::fflush(stdout);
        }
    }
    return chk;
}

extern "C" int lbm_calNuRe(lbm_handle* h, double* Nu, double* Re) {
    int st = diag_prologue(h);
    if (st != LBM_OK) return st;
    if (!Nu || !Re) return fail(h, LBM_ERR_PARAM, "null output");
    double s[DIAG_NSUM];
    if ((st = run_reduce(h, DIAG_NURE, s)) != LBM_OK) return st;
    const double N = (double)h->geo.ncell;
    *Nu = s[0] / N * h->c.lengthUnit / h->c.diffusivity + 1.0;
    *Re = std::sqrt(s[1] / N) * h->c.lengthUnit / h->c.viscosity;
    if (s[4] != 0.0 || !std::isfinite(*Nu) || !std::isfinite(*Re))
        return fail(h, LBM_ERR_DIVERGED, "non-finite field or rho <= 0 in " + std::to_string((long long)s[4]) + " cells");
    return LBM_OK;
}

extern "C" int lbm_RBcalc_Nu_global(lbm_handle* h, double* Nu) {
    int st = diag_prologue(h);
    if (st != LBM_OK) return st;
    if (!Nu) return fail(h, LBM_ERR_PARAM, "null output");
    double s[DIAG_NSUM];
    if ((st = run_reduce(h, DIAG_NU_GLOBAL, s)) != LBM_OK) return st;
    *Nu = (s[0] / (double)h->geo.ncell) / h->dsc.deltaT;
    return std::isfinite(*Nu) ? LBM_OK : fail(h, LBM_ERR_DIVERGED, "non-finite Nu_global");
}

// fit_adiabatic_wall_T4 (2DRB.F90:1953-1991)
static double fit_adiabatic_wall_T4(double y0, const double y[4], const double tt[4]) {
    double s[4];
    for (int k = 0; k < 4; ++k) s[k] = (y[k] - y0) * (y[k] - y0);
    double S0 = 4.0, S1 = 0.0, S2 = 0.0, B0 = 0.0, B1 = 0.0;
    for (int k = 0; k < 4; ++k) {
        S1 = S1 + s[k];
        S2 = S2 + s[k] * s[k];
        B0 = B0 + tt[k];
        B1 = B1 + tt[k] * s[k];
    }
    const double D = S0 * S2 - S1 * S1;
    return (B0 * S2 - B1 * S1) / D;
}

// fit_parabola_ls5: 2D form (2DRB.F90:1999-2080) solves for (quadratic, linear,
// constant); 3D form (3DRB.F90:2257-2334) for (constant, linear, quadratic) and also
// rejects a parabola of the wrong curvature.
static void fit_parabola_ls5(bool d3, const double y[5], const double f[5], int mode, double* fstar, double* ystar) {
    const double epsD = 1.0e-20, epsA = 1.0e-14;
    int kb = 0;
    for (int k = 1; k < 5; ++k) {
        if (mode == 1 ? (f[k] > f[kb]) : (f[k] < f[kb])) kb = k;
    }
    double S0 = 0, S1 = 0, S2 = 0, S3 = 0, S4 = 0, F0 = 0, F1 = 0, F2 = 0;
    for (int k = 0; k < 5; ++k) {
        S0 = S0 + 1.0;
        S1 = S1 + y[k];
        S2 = S2 + y[k] * y[k];
        S3 = S3 + y[k] * y[k] * y[k];
        S4 = S4 + y[k] * y[k] * y[k] * y[k];
        F0 = F0 + f[k];
        if (d3) {
            F1 = F1 + f[k] * y[k];
            F2 = F2 + f[k] * y[k] * y[k];
        } else {
            F1 = F1 + y[k] * f[k];
            F2 = F2 + y[k] * y[k] * f[k];
        }
    }
    double ymin = y[0], ymax = y[0];
    for (int k = 1; k < 5; ++k) {
        ymin = y[k] < ymin ? y[k] : ymin;
        ymax = y[k] > ymax ? y[k] : ymax;
    }
    *ystar = y[kb];
    *fstar = f[kb];
    if (!d3) {
        const double D = S4 * (S2 * S0 - S1 * S1) - S3 * (S3 * S0 - S1 * S2) + S2 * (S3 * S1 - S2 * S2);
        const double DA = F2 * (S2 * S0 - S1 * S1) - S3 * (F1 * S0 - S1 * F0) + S2 * (F1 * S1 - S2 * F0);
        const double DB = S4 * (F1 * S0 - S1 * F0) - F2 * (S3 * S0 - S1 * S2) + S2 * (S3 * F0 - F1 * S2);
        const double DC = S4 * (S2 * F0 - F1 * S1) - S3 * (S3 * F0 - F1 * S2) + F2 * (S3 * S1 - S2 * S2);
        if (std::fabs(D) > epsD) {
            const double A = DA / D, B = DB / D, C = DC / D;
            if (std::fabs(A) > epsA) {
                const double ys = -B / (2.0 * A);
                if (ys >= ymin && ys <= ymax) {
                    *ystar = ys;
                    *fstar = C - B * B / (4.0 * A);
                }
            }
        }
        return;
    }
    const double D = S0 * (S2 * S4 - S3 * S3) - S1 * (S1 * S4 - S2 * S3) + S2 * (S1 * S3 - S2 * S2);
    const double DA = F0 * (S2 * S4 - S3 * S3) - S1 * (F1 * S4 - S3 * F2) + S2 * (F1 * S3 - S2 * F2);
    const double DB = S0 * (F1 * S4 - S3 * F2) - F0 * (S1 * S4 - S2 * S3) + S2 * (S1 * F2 - F1 * S2);
    const double DC = S0 * (S2 * F2 - F1 * S3) - S1 * (S1 * F2 - F1 * S2) + F0 * (S1 * S3 - S2 * S2);
    if (std::fabs(D) <= epsD) return;
    const double A = DA / D, B = DB / D, C = DC / D;
    if (std::fabs(C) <= epsA || (mode == 1 && C >= 0.0) || (mode == -1 && C <= 0.0)) return;
    const double ys = -B / (2.0 * C);
    if (ys < ymin || ys > ymax) return;
    *ystar = ys;
    *fstar = A + B * ys + C * ys * ys;
}

extern "C" int lbm_RBcalc_Nu_wall_avg(lbm_handle* h, lbm_nu_wall* out) {
    int st = diag_prologue(h);
    if (st != LBM_OK) return st;
    if (!out) return fail(h, LBM_ERR_PARAM, "null output");
    const int nx = h->geo.nx, nz = h->geo.nz;
    const bool d3 = h->dim == 3;
    if (h->p.precision == LBM_FP64) diag_wall_columns<double>(h->geo, h->dsc, h->A.T, h->d_tb, h->d_nub, h->stream);
    else diag_wall_columns<float>(h->geo, h->dsc, fast_diag_fields(h->F).T, h->d_tb, h->d_nub, h->stream);
    CK_LAUNCH(h, "wall columns");
    std::vector<double> Tb(nx + 2, 0.0), Nub(nx + 2, 0.0);
    CK(h, cudaMemcpyAsync(Tb.data() + 1, h->d_tb, nx * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(Nub.data() + 1, h->d_nub, nx * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    const double L = h->c.lengthUnit, dy = h->dsc.dy, deltaT = h->dsc.deltaT, Thot = h->p.Thot;
    std::vector<double> xp(nx + 2);
    xp[0] = 0.0 / L;
    xp[nx + 1] = (double)nx / L;
    for (int i = 1; i <= nx; ++i) xp[i] = ((double)i - 0.5) / L;
    // (1) hot wall mean (2DRB.F90:2329-2337, 3DRB.F90:2067-2080)
    double sum_hot = 0.0;
    for (int i = 1; i <= nx; ++i) sum_hot = sum_hot + Nub[i];
    out->Nu_hot = sum_hot / (double)nx;
    // (1.1) corner extension by the 4-point adiabatic fit
    double xf[4], Tf[4];
    for (int m = 0; m < 4; ++m) { xf[m] = xp[1 + m]; Tf[m] = Tb[1 + m]; }
    const double T_wl = fit_adiabatic_wall_T4(0.0, xf, Tf);
    for (int m = 0; m < 4; ++m) { xf[m] = xp[nx - 3 + m]; Tf[m] = Tb[nx - 3 + m]; }
    const double T_wr = fit_adiabatic_wall_T4(xp[nx + 1], xf, Tf);
    std::vector<double> ext(Nub);
    ext[0] = (2.0 * (Thot - T_wl) / dy) / deltaT;
    ext[nx + 1] = (2.0 * (Thot - T_wr) / dy) / deltaT;
    // (1.2) grid extremes, (1.3)/(1.4) 5-point least-squares parabola around them
    int imax = 0, imin = 0;
    double vmax = ext[0], vmin = ext[0];
    for (int i = 1; i <= nx + 1; ++i) {
        if (ext[i] > vmax) { vmax = ext[i]; imax = i; }
        if (ext[i] < vmin) { vmin = ext[i]; imin = i; }
    }
    auto pick = [nx](int ic, int ii[5]) {
        for (int m = 0; m < 5; ++m) ii[m] = (ic <= 2) ? m : (ic >= nx - 1 ? nx - 3 + m : ic - 2 + m);
    };
    int ii[5];
    double xk[5], fk[5], fstar, xstar;
    pick(imax, ii);
    for (int m = 0; m < 5; ++m) { xk[m] = xp[ii[m]]; fk[m] = ext[ii[m]]; }
    fit_parabola_ls5(d3, xk, fk, +1, &fstar, &xstar);
    out->Nu_hot_max = fstar;
    out->Nu_hot_max_position = xstar;
    pick(imin, ii);
    for (int m = 0; m < 5; ++m) { xk[m] = xp[ii[m]]; fk[m] = ext[ii[m]]; }
    fit_parabola_ls5(d3, xk, fk, -1, &fstar, &xstar);
    out->Nu_hot_min = fstar;
    out->Nu_hot_min_position = xstar;
    // (2) cold wall and mid-plane means
    double s[DIAG_NSUM];
    if ((st = run_reduce(h, DIAG_NU_COLD_MID, s)) != LBM_OK) return st;
    out->Nu_cold = s[0] / (double)(nx * nz);
    out->Nu_middle = s[1] / (double)(nx * nz);
    return std::isfinite(out->Nu_hot) && std::isfinite(out->Nu_cold) ? LBM_OK
                                                                      : fail(h, LBM_ERR_DIVERGED, "non-finite wall Nu");
}

// ------------------------------------------------------------------------------------
// side-heated cell diagnostics and mid-line / mid-plane velocity maxima
// ------------------------------------------------------------------------------------
// Node coordinates of one axis (3DRB.F90:444-465, 2DRB.F90:463-476): c[0] = 0,
// c[n+1] = n/L, c[i] = (i - 1/2)/L.
static std::vector<double> node_coords(int n, double L) {
    std::vector<double> c((size_t)n + 2);
    for (int i = 0; i <= n + 1; ++i) {
        const double raw = i == 0 ? 0.0 : (i == n + 1 ? (double)n : (double)i - 0.5);
        c[(size_t)i] = raw / L;
    }
    return c;
}

extern "C" int lbm_SideHeatedcalc_Nu_global(lbm_handle* h, double* Nu) {
    int st = diag_prologue(h);
    if (st != LBM_OK) return st;
    if (!Nu) return fail(h, LBM_ERR_PARAM, "null output");
    double s[DIAG_NSUM];
    if ((st = run_reduce(h, DIAG_NU_GLOBAL_SIDE, s)) != LBM_OK) return st;
    *Nu = (s[0] / (double)h->geo.ncell) / h->dsc.deltaT;
    return std::isfinite(*Nu) ? LBM_OK : fail(h, LBM_ERR_DIVERGED, "non-finite Nu_global");
}

// SideHeatedcalc_Nu_wall_avg (2DRB.F90:1746-1941, 3DRB.F90:1889-2038): the hot wall is
// the left face x = 0; its profile runs along y.
extern "C" int lbm_SideHeatedcalc_Nu_wall_avg(lbm_handle* h, lbm_nu_wall* out) {
    int st = diag_prologue(h);
    if (st != LBM_OK) return st;
    if (!out) return fail(h, LBM_ERR_PARAM, "null output");
    const int ny = h->geo.ny, nz = h->geo.nz;
    const bool d3 = h->dim == 3;
    if (ny < 5) return fail(h, LBM_ERR_PARAM, "the wall fits need ny >= 5");
    if (h->p.precision == LBM_FP64) diag_wall_rows<double>(h->geo, h->dsc, h->A.T, h->d_tl, h->d_nul, h->stream);
    else diag_wall_rows<float>(h->geo, h->dsc, fast_diag_fields(h->F).T, h->d_tl, h->d_nul, h->stream);
    CK_LAUNCH(h, "wall rows");
    std::vector<double> Tl(ny + 2, 0.0), Nul(ny + 2, 0.0);
    CK(h, cudaMemcpyAsync(Tl.data() + 1, h->d_tl, ny * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(Nul.data() + 1, h->d_nul, ny * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    const double dx = h->dsc.dy, deltaT = h->dsc.deltaT, Thot = h->p.Thot;
    const std::vector<double> yp = node_coords(ny, h->c.lengthUnit);
    double sum_hot = 0.0;
    for (int j = 1; j <= ny; ++j) sum_hot = sum_hot + Nul[j];
    out->Nu_hot = sum_hot / (double)ny;
    double yf[4], Tf[4];
    for (int m = 0; m < 4; ++m) { yf[m] = yp[1 + m]; Tf[m] = Tl[1 + m]; }
    const double T_wb = fit_adiabatic_wall_T4(0.0, yf, Tf);
    for (int m = 0; m < 4; ++m) { yf[m] = yp[ny - 3 + m]; Tf[m] = Tl[ny - 3 + m]; }
    const double T_wt = fit_adiabatic_wall_T4(yp[ny + 1], yf, Tf);
    std::vector<double> ext(Nul);
    ext[0] = (2.0 * (Thot - T_wb) / dx) / deltaT;
    ext[ny + 1] = (2.0 * (Thot - T_wt) / dx) / deltaT;
    int jmax = 0, jmin = 0;
    double vmax = ext[0], vmin = ext[0];
    for (int j = 1; j <= ny + 1; ++j) {
        if (ext[j] > vmax) { vmax = ext[j]; jmax = j; }
        if (ext[j] < vmin) { vmin = ext[j]; jmin = j; }
    }
    int jj[5];
    double yk[5], fk[5], fstar, ystar;
    for (int m = 0; m < 5; ++m) jj[m] = jmax <= 2 ? m : (jmax >= ny - 1 ? ny - 3 + m : jmax - 2 + m);
    for (int m = 0; m < 5; ++m) { yk[m] = yp[jj[m]]; fk[m] = ext[jj[m]]; }
    fit_parabola_ls5(d3, yk, fk, +1, &fstar, &ystar);
    out->Nu_hot_max = fstar;
    out->Nu_hot_max_position = ystar;
    // the minimum's window ends at it (2DRB.F90:1880-1884, 3DRB.F90:1974-1978)
    for (int m = 0; m < 5; ++m) jj[m] = jmin >= 4 ? jmin - 4 + m : m;
    for (int m = 0; m < 5; ++m) { yk[m] = yp[jj[m]]; fk[m] = ext[jj[m]]; }
    fit_parabola_ls5(d3, yk, fk, -1, &fstar, &ystar);
    out->Nu_hot_min = fstar;
    out->Nu_hot_min_position = ystar;
    double s[DIAG_NSUM];
    if ((st = run_reduce(h, DIAG_NU_COLD_MID_SIDE, s)) != LBM_OK) return st;
    out->Nu_cold = s[0] / (double)(ny * nz);
    out->Nu_middle = s[1] / (double)(ny * nz);
    return std::isfinite(out->Nu_hot) && std::isfinite(out->Nu_cold) ? LBM_OK
                                                                      : fail(h, LBM_ERR_DIVERGED, "non-finite wall Nu");
}

static int ensure_stage(lbm_handle* h, size_t count);

// The plane `idx` (0-based) normal to `axis` of velocity component `comp` (0 u, 1 v, 2 w),
// to host memory.
static int fetch_plane(lbm_handle* h, int comp, int axis, int idx, std::vector<double>& out) {
    const Geo& g = h->geo;
    const size_t n1 = axis == 0 ? g.ny : g.nx, n2 = axis == 2 ? g.ny : g.nz;
    int st = ensure_stage(h, n1 * n2);
    if (st != LBM_OK) return st;
    if (h->p.precision == LBM_FP64) {
        const double* f = comp == 0 ? h->A.u : (comp == 1 ? h->A.v : h->A.w);
        diag_gather_plane<double>(g, f, axis, idx, h->d_stage, h->stream);
    } else {
        const DiagFields<float> F = fast_diag_fields(h->F);
        const float* f = comp == 0 ? F.u : (comp == 1 ? F.v : F.w);
        diag_gather_plane<float>(g, f, axis, idx, h->d_stage, h->stream);
    }
    CK_LAUNCH(h, "gather plane");
    out.resize(n1 * n2);
    CK(h, cudaMemcpyAsync(out.data(), h->d_stage, n1 * n2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return LBM_OK;
}

// calc_{u,v,w}mid_max_common (3DRB.F90:2399-2518): the grid maximum, over the mid plane
// normal to the component's axis, of the component interpolated to that plane.
static int mid_max_3d(lbm_handle* h, int comp, lbm_mid_max* out) {
    const Geo& g = h->geo;
    const double L = h->c.lengthUnit;
    const int n[3] = {g.nx, g.ny, g.nz};
    const std::vector<double> cx = node_coords(g.nx, L), cy = node_coords(g.ny, L), cz = node_coords(g.nz, L);
    const std::vector<double>& c = comp == 0 ? cx : (comp == 1 ? cy : cz);
    const int nn = n[comp];
    // find_bracketing_index (3DRB.F90:2525-2545)
    const double target = 0.5 * c[(size_t)nn + 1];
    int iL = 1;
    while (iL < nn && c[(size_t)iL + 1] < target) iL = iL + 1;
    const int iR = iL + 1 < nn ? iL + 1 : nn;
    double weight = std::fabs(c[(size_t)iR] - c[(size_t)iL]) <= 1.0e-14 ? 0.0 : (target - c[(size_t)iL]) / (c[(size_t)iR] - c[(size_t)iL]);
    weight = std::max(0.0, std::min(1.0, weight));
    std::vector<double> pL, pR;
    int st = fetch_plane(h, comp, comp, iL - 1, pL);
    if (st != LBM_OK) return st;
    if (iR != iL && (st = fetch_plane(h, comp, comp, iR - 1, pR)) != LBM_OK) return st;
    // loop order of the reference: outer over the later axis, inner over the earlier one
    const int a1 = comp == 0 ? 1 : 0, a2 = comp == 2 ? 1 : 2;
    const int n1 = n[a1], n2 = n[a2];
    double vmax = -std::numeric_limits<double>::max();
    int b1 = 1, b2 = 1;
    for (int q2 = 1; q2 <= n2; ++q2)
        for (int q1 = 1; q1 <= n1; ++q1) {
            const size_t e = (size_t)(q1 - 1) + (size_t)n1 * (size_t)(q2 - 1);
            const double val = iL == iR ? pL[e] : (1.0 - weight) * pL[e] + weight * pR[e];
            if (val > vmax) {
                vmax = val;
                b1 = q1;
                b2 = q2;
            }
        }
    const std::vector<double>& c1 = a1 == 0 ? cx : cy;
    const std::vector<double>& c2 = a2 == 1 ? cy : cz;
    out->value = vmax * h->dsc.coef;
    out->pos1 = c1[(size_t)b1];
    out->pos2 = c2[(size_t)b2];
    out->mid = target;
    return std::isfinite(vmax) ? LBM_OK : fail(h, LBM_ERR_DIVERGED, "non-finite velocity");
}

// 2D mid-line maxima with the 5-point parabola (2DRB.F90:2081-2238, 2484-2575).
// comp 0: u on the line x = mid (rb: x = 0.5, interpolated, maximum position folded into
// the lower half); comp 1: v on the line y = mid.
static int mid_max_2d(lbm_handle* h, int comp, bool rb, lbm_mid_max* out) {
    const Geo& g = h->geo;
    const int nx = g.nx, ny = g.ny;
    const double L = h->c.lengthUnit;
    const std::vector<double> xp = node_coords(nx, L), yp = node_coords(ny, L);
    const int nline = comp == 0 ? ny : nx, nacross = comp == 0 ? nx : ny;
    const std::vector<double>& along = comp == 0 ? yp : xp;   // coordinate along the line
    const std::vector<double>& across = comp == 0 ? xp : yp;  // coordinate of the line
    std::vector<double> line((size_t)nline + 1), pa, pb;
    double mid;
    int st;
    if (comp == 0 && rb) {
        const double targetX = 0.5;
        mid = targetX;
        int iL = 1;
        while (iL < nx && xp[(size_t)iL + 1] < targetX) iL = iL + 1;
        const int iR = iL + 1 < nx ? iL + 1 : nx;
        if ((st = fetch_plane(h, 0, 0, iL - 1, pa)) != LBM_OK) return st;
        if (std::fabs(xp[(size_t)iL] - targetX) <= 1.0e-14 || iR == iL) {
            for (int j = 1; j <= ny; ++j) line[(size_t)j] = pa[(size_t)j - 1];
        } else {
            if ((st = fetch_plane(h, 0, 0, iR - 1, pb)) != LBM_OK) return st;
            const double w = (targetX - xp[(size_t)iL]) / (xp[(size_t)iR] - xp[(size_t)iL]);
            for (int j = 1; j <= ny; ++j) line[(size_t)j] = (1.0 - w) * pa[(size_t)j - 1] + w * pb[(size_t)j - 1];
        }
    } else if (nacross % 2 == 1) {
        const int m = (nacross + 1) / 2;
        mid = across[(size_t)m];
        if ((st = fetch_plane(h, comp, comp, m - 1, pa)) != LBM_OK) return st;
        for (int q = 1; q <= nline; ++q) line[(size_t)q] = pa[(size_t)q - 1];
    } else {
        const int mL = nacross / 2, mR = mL + 1;
        mid = 0.5 * (across[(size_t)mL] + across[(size_t)mR]);
        if ((st = fetch_plane(h, comp, comp, mL - 1, pa)) != LBM_OK) return st;
        if ((st = fetch_plane(h, comp, comp, mR - 1, pb)) != LBM_OK) return st;
        for (int q = 1; q <= nline; ++q) line[(size_t)q] = 0.5 * (pa[(size_t)q - 1] + pb[(size_t)q - 1]);
    }
    int q0 = 1;
    double vmax = line[1];
    for (int q = 2; q <= nline; ++q)
        if (line[(size_t)q] > vmax) {
            vmax = line[(size_t)q];
            q0 = q;
        }
    double sk[5], fk[5], fstar, sstar;
    for (int m = 0; m < 5; ++m) {
        const int q = q0 <= 2 ? 1 + m : (q0 >= nline - 1 ? nline - 4 + m : q0 - 2 + m);
        sk[m] = along[(size_t)q];
        fk[m] = line[(size_t)q];
    }
    fit_parabola_ls5(false, sk, fk, +1, &fstar, &sstar);
    if (comp == 0 && rb) {
        const double yLen = yp[(size_t)ny + 1];
        if (sstar > 0.5 * yLen) sstar = yLen - sstar;
    }
    out->value = fstar * h->dsc.coef;
    out->pos1 = sstar;
    out->pos2 = 0.0;
    out->mid = mid;
    return std::isfinite(fstar) ? LBM_OK : fail(h, LBM_ERR_DIVERGED, "non-finite velocity");
}

static int mid_max(lbm_handle* h, int comp, bool rb, lbm_mid_max* out) {
    int st = diag_prologue(h);
    if (st != LBM_OK) return st;
    if (!out) return fail(h, LBM_ERR_PARAM, "null output");
    if (comp == 2 && h->dim != 3) return fail(h, LBM_ERR_PARAM, "w exists in 3D only");
    if (h->dim == 2 && (h->geo.nx < 5 || h->geo.ny < 5)) return fail(h, LBM_ERR_PARAM, "the fit needs 5 points");
    return h->dim == 3 ? mid_max_3d(h, comp, out) : mid_max_2d(h, comp, rb, out);
}

extern "C" int lbm_SideHeatedcalc_umid_max(lbm_handle* h, lbm_mid_max* out) { return mid_max(h, 0, false, out); }
extern "C" int lbm_SideHeatedcalc_vmid_max(lbm_handle* h, lbm_mid_max* out) { return mid_max(h, 1, false, out); }
extern "C" int lbm_SideHeatedcalc_wmid_max(lbm_handle* h, lbm_mid_max* out) { return mid_max(h, 2, false, out); }
extern "C" int lbm_RBcalc_umid_max(lbm_handle* h, lbm_mid_max* out) { return mid_max(h, 0, true, out); }
extern "C" int lbm_RBcalc_vmid_max(lbm_handle* h, lbm_mid_max* out) { return mid_max(h, 1, true, out); }
extern "C" int lbm_RBcalc_wmid_max(lbm_handle* h, lbm_mid_max* out) { return mid_max(h, 2, true, out); }

// ------------------------------------------------------------------------------------
// state transfer
// ------------------------------------------------------------------------------------
static int ensure_stage(lbm_handle* h, size_t count) {
    if (h->stage_cap >= count) return LBM_OK;
    if (h->d_stage) {
        for (auto it = h->allocs.begin(); it != h->allocs.end(); ++it)
            if (*it == h->d_stage) {
                h->allocs.erase(it);
                break;
            }
        cudaFree(h->d_stage);
        h->d_stage = nullptr;
        h->stage_cap = 0;
    }
    int st = dalloc(h, &h->d_stage, count);
    if (st != LBM_OK) return st;
    h->stage_cap = count;
    return LBM_OK;
}

static double* scalar_ptr(lbm_handle* h, int field) {
    ExactArrays& A = h->A;
    const bool d3 = h->dim == 3;
    switch (field) {
        case LBM_FIELD_RHO: return A.rho;
        case LBM_FIELD_U: return A.u;
        case LBM_FIELD_V: return A.v;
        case LBM_FIELD_W: return d3 ? A.w : nullptr;
        case LBM_FIELD_T: return A.T;
        case LBM_FIELD_BX_PREV: return A.Bx;
        case LBM_FIELD_BY_PREV: return A.By;
        case LBM_FIELD_BZ_PREV: return d3 ? A.Bz : nullptr;
        case LBM_FIELD_FX: return d3 ? nullptr : A.Fx;
        case LBM_FIELD_FY: return d3 ? nullptr : A.Fy;
        default: return nullptr;
    }
}

static int state_io(lbm_handle* h, int field, double* dst, const double* src, size_t count) {
    NvtxRange range_("state transfer");
    if (!h || (!dst && !src)) return LBM_ERR_PARAM;
    if (!h->initialised) return fail(h, LBM_ERR_STATE, "lbm_initial has not been called");
    CK(h, cudaSetDevice(h->device));
    // fixed arithmetic: a load makes the module arrays the state; the post-collision arrays
    // exist only in FP64 form
    const bool post = field == LBM_FIELD_F_POST || field == LBM_FIELD_G_POST;
    int st = (h->fixed && (src || post)) ? release_fixed(h) : materialize(h);
    if (st != LBM_OK) return st;
    const long long n = h->geo.ncell;
    const bool pop = field == LBM_FIELD_F || field == LBM_FIELD_G || field == LBM_FIELD_F_POST || field == LBM_FIELD_G_POST;
    const int qq = (field == LBM_FIELD_F || field == LBM_FIELD_F_POST) ? h->q : h->qt;
    const size_t want = pop ? (size_t)qq * n : (size_t)n;
    if (count != want) return fail(h, LBM_ERR_PARAM, "count does not match the field size");
    if (in_place(h) && (field == LBM_FIELD_F_POST || field == LBM_FIELD_G_POST))
        return fail(h, LBM_ERR_STATE, "the in-place pattern keeps no post-collision array");
    if (h->p.precision != LBM_FP64) {
        if ((st = ensure_stage(h, want)) != LBM_OK) return st;
        if (dst) {
            st = fast_export(h->F, h->geo, h->phys, h->dim, field, h->d_stage, h->stream);
            if (st != LBM_OK) return fail(h, st, "field not available for this precision");
            CK_LAUNCH(h, "export");
            CK(h, cudaMemcpyAsync(dst, h->d_stage, want * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            CK(h, cudaStreamSynchronize(h->stream));
        } else {
            CK(h, cudaMemcpyAsync(h->d_stage, src, want * sizeof(double), cudaMemcpyHostToDevice, h->stream));
            st = fast_import(h->F, h->geo, h->phys, h->dim, field, h->d_stage, h->stream);
            if (st != LBM_OK) return fail(h, st, "field not settable for this precision");
            CK_LAUNCH(h, "import");
            CK(h, cudaStreamSynchronize(h->stream));
        }
        return LBM_OK;
    }
    if (src) h->fused_valid = false;  // the module arrays are the state again
    if (pop) {
        double* soa = field == LBM_FIELD_F ? h->A.f : field == LBM_FIELD_G ? h->A.g : field == LBM_FIELD_F_POST ? h->A.fpost : h->A.gpost;
        const bool th = field == LBM_FIELD_G;
        if ((st = ensure_stage(h, want)) != LBM_OK) return st;
        if (dst && in_place(h)) {
            aa_module_view(h->geo, qq, th, LBM_FP64, soa, th ? h->aa.gpar : h->aa.fpar, h->aa.graw, h->d_stage, false,
                           false, 0.0, 0.0, h->stream);
            CK_LAUNCH(h, "module view");
            CK(h, cudaMemcpyAsync(dst, h->d_stage, want * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        } else if (dst && h->host_direct_wr) {
            soa_to_aos(soa, dst, qq, n, h->stream);  // written straight into the caller's array
            CK_LAUNCH(h, "soa_to_aos");
        } else if (dst) {
            soa_to_aos(soa, h->d_stage, qq, n, h->stream);
            CK_LAUNCH(h, "soa_to_aos");
            CK(h, cudaMemcpyAsync(dst, h->d_stage, want * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        } else {
            if (h->host_direct) {
                aos_to_soa(src, soa, qq, n, h->stream);  // read straight from the caller's array
            } else {
                CK(h, cudaMemcpyAsync(h->d_stage, src, want * sizeof(double), cudaMemcpyHostToDevice, h->stream));
                aos_to_soa(h->d_stage, soa, qq, n, h->stream);
            }
            CK_LAUNCH(h, "aos_to_soa");
            if (th) {  // module data in the streamed layout
                h->aa.gpar = 0;
                h->aa.graw = false;
            } else {
                h->aa.fpar = 0;
            }
        }
        CK(h, cudaStreamSynchronize(h->stream));
        return LBM_OK;
    }
    double* d = scalar_ptr(h, field);
    if (!d) return fail(h, LBM_ERR_PARAM, "field not defined for this dimension");
    if (dst ? h->host_direct_wr : h->host_direct) {
        copy_doubles(dst ? d : src, dst ? dst : d, (long long)want, h->stream);
        CK_LAUNCH(h, "field copy");
    } else if (dst) {
        CK(h, cudaMemcpyAsync(dst, d, want * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    } else {
        CK(h, cudaMemcpyAsync(d, src, want * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    }
    CK(h, cudaStreamSynchronize(h->stream));
    return LBM_OK;
}

extern "C" int lbm_get_state(lbm_handle* h, int field, double* host, size_t count) {
    if (!host) return LBM_ERR_PARAM;
    return state_io(h, field, host, nullptr, count);
}

extern "C" int lbm_set_state(lbm_handle* h, int field, const double* host, size_t count) {
    if (!host) return LBM_ERR_PARAM;
    return state_io(h, field, nullptr, host, count);
}

// ------------------------------------------------------------------------------------
// restart files: backupData / reload (3DRB.F90:1638-1665, 602-623; 2DRB.F90:1402-1430,
// 621-637) with reconstruct_macro_from_fg (3DRB.F90:1392-1463, 2DRB.F90:1144-1200)
// ------------------------------------------------------------------------------------
namespace {

constexpr int64_t kContMagic = 0x31544E4F434D424CLL;  // "LBMCONT1" read as little-endian bytes
constexpr int64_t kContVersion = 1;
constexpr int kContHeader = 16;                       // int64 words of the header record
constexpr size_t kIoChunk = size_t(64) << 20;         // host staging per copy

// forms of the continuation records
constexpr int kFormExact = 0;      // FP64 module arrays (f, g come from the two reference records)
constexpr int kFormFastFused = 1;  // FP32/FP16 fused buffers F[cur], G[cur], B[cur], L[cur]
constexpr int kFormFastModule = 2; // FP32/FP16 module arrays fref, gref, rho, u, v, w, T, B, L
constexpr int kFormFastAA = 3;     // FP32/FP16 in-place arrays as they lie, module scalars, B, L
                                   // (header words 11-14: flow / thermal layout, push flag, fused)

struct Pinned {
    void* p = nullptr;
    size_t cap = 0;
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
};

struct ContArray {
    void* dptr;
    size_t bytes;
};

struct FileCloser {
    FILE* fp = nullptr;
    ~FileCloser() {
        if (fp) std::fclose(fp);
    }
};

}  // namespace

// Device arrays of the continuation records, in file order, for one form.
static std::vector<ContArray> cont_arrays(lbm_handle* h, int form) {
    const size_t n = (size_t)h->geo.ncell;
    const bool d3 = h->dim == 3;
    std::vector<ContArray> v;
    if (form == kFormExact) {
        ExactArrays& A = h->A;
        const size_t b = n * sizeof(double);
        v = {{A.rho, b}, {A.u, b}, {A.v, b}};
        if (d3) v.push_back({A.w, b});
        v.push_back({A.T, b});
        v.push_back({A.Bx, b});
        v.push_back({A.By, b});
        if (d3) v.push_back({A.Bz, b});
        else {
            v.push_back({A.Fx, b});
            v.push_back({A.Fy, b});
        }
        v.push_back({A.up, b});
        v.push_back({A.vp, b});
        if (d3) v.push_back({A.wp, b});
        v.push_back({A.Tp, b});
        return v;
    }
    FastState& F = h->F;
    const size_t b = n * sizeof(float);
    const int c = F.cur;
    if (form == kFormFastFused) {
        v = {{F.fbuf[c], (size_t)h->q * n * F.esize}, {F.gbuf[c], (size_t)h->qt * n * F.esize}};
    } else if (form == kFormFastAA) {
        v = {{F.fbuf[0], (size_t)h->q * n * F.esize}, {F.gbuf[0], (size_t)h->qt * n * F.esize}, {F.rho, b}, {F.u, b},
             {F.v, b}};
        if (d3) v.push_back({F.w, b});
        v.push_back({F.T, b});
    } else {
        v = {{F.fref, (size_t)h->q * n * F.esize}, {F.gref, (size_t)h->qt * n * F.esize}, {F.rho, b}, {F.u, b},
             {F.v, b}};
        if (d3) v.push_back({F.w, b});
        v.push_back({F.T, b});
    }
    for (int a = 0; a < h->dim; ++a) v.push_back({F.B[c][a], b});
    v.push_back({F.L[c], b});
    v.push_back({F.up, b});
    v.push_back({F.vp, b});
    if (d3) v.push_back({F.wp, b});
    v.push_back({F.Tp, b});
    return v;
}

static int pinned_for(lbm_handle* h, Pinned& pin, size_t largest) {
    const size_t want = largest < kIoChunk ? largest : kIoChunk;
    CK(h, cudaMallocHost(&pin.p, want > 0 ? want : 1));
    pin.cap = want > 0 ? want : 1;
    return LBM_OK;
}

// One record of `bytes` bytes of device memory, staged through pinned host memory.
static int write_device_record(lbm_handle* h, FILE* fp, const void* dptr, size_t bytes, Pinned& pin) {
    RecordWriter w;
    if (!w.begin(fp, bytes)) return fail(h, LBM_ERR_IO, "write failed");
    for (size_t off = 0; off < bytes;) {
        const size_t k = bytes - off < pin.cap ? bytes - off : pin.cap;
        CK(h, cudaMemcpyAsync(pin.p, (const char*)dptr + off, k, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        if (!w.put(pin.p, k)) return fail(h, LBM_ERR_IO, "write failed");
        off += k;
    }
    if (!w.end()) return fail(h, LBM_ERR_IO, "write failed");
    return LBM_OK;
}

static int read_device_record(lbm_handle* h, FILE* fp, void* dptr, size_t bytes, Pinned& pin) {
    RecordReader r;
    if (!r.begin(fp)) return fail(h, LBM_ERR_IO, "restart file truncated");
    for (size_t off = 0; off < bytes;) {
        const size_t k = bytes - off < pin.cap ? bytes - off : pin.cap;
        if (r.get(pin.p, k) != k) return fail(h, LBM_ERR_IO, "restart record shorter than the lattice");
        CK(h, cudaMemcpyAsync((char*)dptr + off, pin.p, k, cudaMemcpyHostToDevice, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        off += k;
    }
    if (!r.ok || !r.at_end()) return fail(h, LBM_ERR_IO, "restart record longer than the lattice");
    return LBM_OK;
}

static void cont_header(const lbm_handle* h, int form, size_t narrays, int64_t hdr[kContHeader]) {
    for (int k = 0; k < kContHeader; ++k) hdr[k] = 0;
    hdr[0] = kContMagic;
    hdr[1] = kContVersion;
    hdr[2] = h->dim;
    hdr[3] = h->geo.nx;
    hdr[4] = h->geo.ny;
    hdr[5] = h->geo.nz;
    hdr[6] = h->p.precision;
    hdr[7] = form;
    hdr[8] = h->itc;
    hdr[9] = (int64_t)narrays;
    hdr[10] = h->p.precision == LBM_FP64 ? 8 : (int64_t)h->F.esize;
    if (form == kFormFastAA) {
        hdr[11] = h->F.AA.fpar;
        hdr[12] = h->F.AA.gpar;
        hdr[13] = h->F.AA.graw ? 1 : 0;
        hdr[14] = h->F.fused_valid ? 1 : 0;
    }
    if (h->p.precision != LBM_FP64) {  // the step counter that keys FP16 stochastic rounding
        unsigned long long t = 0;
        if (cudaMemcpy(&t, h->F.tick, sizeof(t), cudaMemcpyDeviceToHost) == cudaSuccess) hdr[15] = (int64_t)t;
    }
}

extern "C" int lbm_backupData(lbm_handle* h, const char* path, int flags) {
    NvtxRange range_("lbm_backupData");
    if (!h || !path) return LBM_ERR_PARAM;
    if (flags != LBM_BACKUP_REFERENCE && flags != LBM_BACKUP_CONTINUE) return fail(h, LBM_ERR_PARAM, "unknown flags");
    if (!h->initialised) return fail(h, LBM_ERR_STATE, "lbm_initial has not been called");
    CK(h, cudaSetDevice(h->device));
    int st = materialize(h);
    if (st != LBM_OK) return st;
    const size_t n = (size_t)h->geo.ncell;
    const bool fp64 = h->p.precision == LBM_FP64;
    Pinned pin;
    if ((st = pinned_for(h, pin, (size_t)h->q * n * sizeof(double))) != LBM_OK) return st;
    FileCloser file;
    file.fp = std::fopen(path, "wb");
    if (!file.fp) return fail(h, LBM_ERR_IO, std::string("cannot open ") + path + " for writing");
    // the reference's two records: f then g, direction outermost, x fastest, FP64
    for (int which = 0; which < 2; ++which) {
        const int qq = which == 0 ? h->q : h->qt;
        const double* src = nullptr;
        if (fp64 && !in_place(h)) {
            src = which == 0 ? h->A.f : h->A.g;
        } else if (fp64) {
            // the module view of the in-place array
            if ((st = ensure_stage(h, (size_t)qq * n)) != LBM_OK) return st;
            aa_module_view(h->geo, qq, which == 1, LBM_FP64, which == 0 ? h->A.f : h->A.g,
                           which == 0 ? h->aa.fpar : h->aa.gpar, h->aa.graw, h->d_stage, true, false, 0.0, 0.0,
                           h->stream);
            CK_LAUNCH(h, "module view");
            src = h->d_stage;
        } else {
            if ((st = ensure_stage(h, (size_t)qq * n)) != LBM_OK) return st;
            st = fast_export(h->F, h->geo, h->phys, h->dim, which == 0 ? LBM_FIELD_F : LBM_FIELD_G, h->d_stage,
                             h->stream, true);
            if (st != LBM_OK) return fail(h, st, "population export failed");
            CK_LAUNCH(h, "export");
            src = h->d_stage;
        }
        if ((st = write_device_record(h, file.fp, src, (size_t)qq * n * sizeof(double), pin)) != LBM_OK) return st;
    }
    if (flags == LBM_BACKUP_CONTINUE) {
        const int form = fp64 ? kFormExact : (h->F.aa ? kFormFastAA : (h->F.fused_valid ? kFormFastFused : kFormFastModule));
        std::vector<ContArray> arrays = cont_arrays(h, form);
        int64_t hdr[kContHeader];
        cont_header(h, form, arrays.size(), hdr);
        RecordWriter w;
        if (!(w.begin(file.fp, sizeof(hdr)) && w.put(hdr, sizeof(hdr)) && w.end()))
            return fail(h, LBM_ERR_IO, "write failed");
        for (const ContArray& a : arrays)
            if ((st = write_device_record(h, file.fp, a.dptr, a.bytes, pin)) != LBM_OK) return st;
    }
    const int rc = std::fclose(file.fp);
    file.fp = nullptr;
    if (rc != 0) return fail(h, LBM_ERR_IO, "write failed");
    return LBM_OK;
}

// Record layout of a restart file, read without touching the handle.
struct RestartScan {
    size_t len_f = 0, len_g = 0;
    bool has_cont = false;
    int64_t hdr[kContHeader] = {};
    std::vector<size_t> lens;
};

static bool scan_restart(FILE* fp, RestartScan& s) {
    RecordReader r;
    if (!r.begin(fp) || !r.skip_rest()) return false;
    s.len_f = r.total;
    RecordReader r2;
    if (!r2.begin(fp) || !r2.skip_rest()) return false;
    s.len_g = r2.total;
    RecordReader r3;
    if (!r3.begin(fp)) return true;  // end of file: the reference's two records only
    if (r3.get(s.hdr, sizeof(s.hdr)) != sizeof(s.hdr) || !r3.ok || !r3.at_end()) return true;
    if (s.hdr[0] != kContMagic) return true;
    for (int64_t k = 0; k < s.hdr[9] && k < 64; ++k) {
        RecordReader ra;
        if (!ra.begin(fp) || !ra.skip_rest()) return true;
        s.lens.push_back(ra.total);
    }
    s.has_cont = (int64_t)s.lens.size() == s.hdr[9];
    return true;
}

static std::string cont_mismatch(lbm_handle* h, const RestartScan& s) {
    const int64_t* H = s.hdr;
    if (H[1] != kContVersion) return "unknown continuation version";
    if (H[2] != h->dim || H[3] != h->geo.nx || H[4] != h->geo.ny || H[5] != h->geo.nz)
        return "continuation records were written for another lattice size";
    if (H[6] != h->p.precision) return "continuation records were written for another storage precision";
    const bool fp64 = h->p.precision == LBM_FP64;
    if (fp64 ? H[7] != kFormExact
             : (h->F.aa ? H[7] != kFormFastAA : (H[7] != kFormFastFused && H[7] != kFormFastModule)))
        return "continuation records were written for another storage form or access pattern";
    if (H[7] == kFormFastAA && (H[11] < 0 || H[11] > 1 || H[12] < 0 || H[12] > 1 || H[13] < 0 || H[13] > 1))
        return "continuation header holds an unknown layout state";
    std::vector<ContArray> arrays = cont_arrays(h, (int)H[7]);
    if (arrays.size() != s.lens.size()) return "continuation record count differs";
    for (size_t k = 0; k < arrays.size(); ++k)
        if (arrays[k].bytes != s.lens[k]) return "continuation record length differs";
    return "";
}

extern "C" int lbm_reload(lbm_handle* h, const char* path, int mode) {
    NvtxRange range_("lbm_reload");
    if (!h || !path) return LBM_ERR_PARAM;
    if (mode != LBM_RELOAD_REFERENCE && mode != LBM_RELOAD_CONTINUE && mode != LBM_RELOAD_AUTO)
        return fail(h, LBM_ERR_PARAM, "unknown reload mode");
    if (h->ensemble) return fail(h, LBM_ERR_STATE, "remove the handle from its ensemble before reloading it");
    CK(h, cudaSetDevice(h->device));
    FileCloser file;
    file.fp = std::fopen(path, "rb");
    if (!file.fp) return fail(h, LBM_ERR_IO, std::string("cannot open ") + path);
    // check the whole file before the state is touched
    RestartScan scan;
    if (!scan_restart(file.fp, scan)) return fail(h, LBM_ERR_IO, "not a restart file (two Fortran records expected)");
    const size_t n = (size_t)h->geo.ncell;
    if (scan.len_f != (size_t)h->q * n * sizeof(double) || scan.len_g != (size_t)h->qt * n * sizeof(double))
        return fail(h, LBM_ERR_IO, "restart records do not match the lattice size");
    std::string why = scan.has_cont ? cont_mismatch(h, scan) : "no continuation records in the file";
    bool cont = false;
    if (mode == LBM_RELOAD_CONTINUE) {
        if (!scan.has_cont) return fail(h, LBM_ERR_IO, why);
        if (!why.empty()) return fail(h, LBM_ERR_PARAM, why);
        cont = true;
    } else if (mode == LBM_RELOAD_AUTO) {
        cont = scan.has_cont && why.empty();
    }
    int st;
    if (!h->initialised && (st = lbm_initial(h)) != LBM_OK) return st;
    CK(h, cudaStreamSynchronize(h->stream));
    std::rewind(file.fp);
    const bool fp64 = h->p.precision == LBM_FP64;
    Pinned pin;
    if ((st = pinned_for(h, pin, (size_t)h->q * n * sizeof(double))) != LBM_OK) return st;
    // from here on a failure leaves the state partly overwritten
    h->initialised = false;
    auto lost = [h](int s) {
        h->err = "reload failed, lattice state lost: " + h->err;
        return s;
    };
    // a temporary set of FP64 module arrays for FP32/FP16 handles (reference reconstruction)
    std::vector<void*> tmp;
    struct TmpFree {
        std::vector<void*>& v;
        ~TmpFree() {
            for (void* p : v) cudaFree(p);
        }
    } tmp_free{tmp};
    ExactArrays X = h->A;
    if (!fp64 && !cont) {
        auto talloc = [&](double** p, size_t cnt) {
            void* q = nullptr;
            cudaError_t e = cudaMalloc(&q, cnt * sizeof(double));
            if (e != cudaSuccess) return cuda_fail(h, e, "cudaMalloc");
            tmp.push_back(q);
            *p = (double*)q;
            return LBM_OK;
        };
        X = ExactArrays{};
        double** scal[] = {&X.rho, &X.u, &X.v, &X.w, &X.T, &X.Bx, &X.By, &X.Bz, &X.Fx, &X.Fy};
        if ((st = talloc(&X.f, (size_t)h->q * n)) != LBM_OK || (st = talloc(&X.g, (size_t)h->qt * n)) != LBM_OK)
            return lost(st);
        for (double** p : scal)
            if ((st = talloc(p, n)) != LBM_OK) return lost(st);
    }
    // records 1 and 2: f and g
    if (fp64 || !cont) {
        if ((st = read_device_record(h, file.fp, X.f, (size_t)h->q * n * sizeof(double), pin)) != LBM_OK) return lost(st);
        if ((st = read_device_record(h, file.fp, X.g, (size_t)h->qt * n * sizeof(double), pin)) != LBM_OK) return lost(st);
    } else {
        RecordReader r1, r2;
        if (!(r1.begin(file.fp) && r1.skip_rest() && r2.begin(file.fp) && r2.skip_rest()))
            return lost(fail(h, LBM_ERR_IO, "restart file truncated"));
    }
    if (fp64) {
        if (!in_place(h)) {
            h->A.fpost = h->fbuf[0];
            h->A.gpost = h->gbuf[0];
        }
        h->cur = 0;
        h->fused_valid = false;
        h->aa.fpar = h->aa.gpar = 0;  // the records are module data: the streamed layout
        h->aa.graw = false;
    } else {
        h->F.cur = 0;
        h->F.ahead = false;
    }
    if (cont) {
        RecordReader rh;
        if (!(rh.begin(file.fp) && rh.skip_rest())) return lost(fail(h, LBM_ERR_IO, "restart file truncated"));
        const int form = (int)scan.hdr[7];
        for (const ContArray& a : cont_arrays(h, form))
            if ((st = read_device_record(h, file.fp, a.dptr, a.bytes, pin)) != LBM_OK) return lost(st);
        if (!fp64) h->F.fused_valid = form == kFormFastFused;
        if (form == kFormFastAA) {
            h->F.AA.fpar = (int)scan.hdr[11];
            h->F.AA.gpar = (int)scan.hdr[12];
            h->F.AA.graw = scan.hdr[13] != 0;
            h->F.fused_valid = scan.hdr[14] != 0;
        }
        if (!fp64) {
            const unsigned long long t = (unsigned long long)scan.hdr[15];
            CK(h, cudaMemcpyAsync(h->F.tick, &t, sizeof(t), cudaMemcpyHostToDevice, h->stream));
            CK(h, cudaStreamSynchronize(h->stream));
        }
        h->itc = scan.hdr[8];
        h->reload_form = 1;
        h->initialised = true;
        return LBM_OK;
    }
    // reference reconstruction
    unsigned int* bad = (unsigned int*)h->d_part;
    CK(h, cudaMemsetAsync(bad, 0, sizeof(unsigned int), h->stream));
    exact_reconstruct(h->geo, h->phys, X, h->dim, bad, h->stream);
    CK_LAUNCH(h, "reconstruct");
    if (!fp64) {
        const bool d3 = h->dim == 3;
        FastState& F = h->F;
        if ((st = fast_import(F, h->geo, h->phys, h->dim, LBM_FIELD_F, X.f, h->stream, true)) != LBM_OK ||
            (st = fast_import(F, h->geo, h->phys, h->dim, LBM_FIELD_G, X.g, h->stream, true)) != LBM_OK)
            return lost(fail(h, st, "population import failed"));
        std::vector<std::pair<int, const double*>> fields = {
            {LBM_FIELD_RHO, X.rho}, {LBM_FIELD_U, X.u}, {LBM_FIELD_V, X.v}, {LBM_FIELD_T, X.T}};
        if (d3) {
            fields.push_back({LBM_FIELD_W, X.w});
            fields.push_back({LBM_FIELD_BX_PREV, X.Bx});
            fields.push_back({LBM_FIELD_BY_PREV, X.By});
            fields.push_back({LBM_FIELD_BZ_PREV, X.Bz});
        } else {
            fields.push_back({LBM_FIELD_FY, X.Fy});
            if (h->p.use_g) {
                fields.push_back({LBM_FIELD_BX_PREV, X.Bx});
                fields.push_back({LBM_FIELD_BY_PREV, X.By});
            }
        }
        for (auto& fv : fields)
            if ((st = fast_import(F, h->geo, h->phys, h->dim, fv.first, fv.second, h->stream)) != LBM_OK)
                return lost(fail(h, st, "field import failed"));
        CK(h, cudaMemsetAsync(F.tick, 0, sizeof(unsigned long long), h->stream));  // a new start: itc = 0
        CK_LAUNCH(h, "import");
    }
    // initial after a reload: up = vp = wp = Tp = 0 (3DRB.F90:627-632, steadyFlow)
    const size_t es = fp64 ? sizeof(double) : sizeof(float);
    void* prev[4] = {fp64 ? (void*)h->A.up : (void*)h->F.up, fp64 ? (void*)h->A.vp : (void*)h->F.vp,
                     fp64 ? (void*)h->A.wp : (void*)h->F.wp, fp64 ? (void*)h->A.Tp : (void*)h->F.Tp};
    for (void* p : prev)
        if (p) CK(h, cudaMemsetAsync(p, 0, n * es, h->stream));
    unsigned int hbad = 0;
    CK(h, cudaMemcpyAsync(&hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (hbad) return fail(h, LBM_ERR_DIVERGED, "non-positive rho found during restart reconstruction");
    h->itc = 0;
    h->reload_form = 0;
    h->initialised = true;
    return LBM_OK;
}

extern "C" int lbm_reload_form(const lbm_handle* h) { return h ? h->reload_form : -1; }

// ------------------------------------------------------------------------------------
// measurement hooks
// ------------------------------------------------------------------------------------
extern "C" int lbm_get_stream(lbm_handle* h, void** stream) {
    if (!h || !stream) return LBM_ERR_PARAM;
    *stream = (void*)h->stream;
    return LBM_OK;
}

extern "C" int lbm_time_kernels(lbm_handle* h, int64_t nsteps, double* ms_flow, double* ms_thermal) {
    if (!h || !ms_flow || !ms_thermal || nsteps <= 0) return LBM_ERR_PARAM;
    if (!h->initialised) return fail(h, LBM_ERR_STATE, "lbm_initial has not been called");
    CK(h, cudaSetDevice(h->device));
    const bool fused = h->p.precision == LBM_FP64 ? h->fused_valid : fast_fused_valid(h->F);
    if (!fused) {
        int st = lbm_step(h, 1);
        if (st != LBM_OK) return st;
    }
    std::vector<cudaEvent_t> ev((size_t)(2 * nsteps + 1));
    for (auto& e : ev) CK(h, cudaEventCreate(&e));
    CK(h, cudaEventRecord(ev[0], h->stream));
    for (int64_t k = 0; k < nsteps; ++k) {
        if (h->p.precision == LBM_FP64 && in_place(h)) {
            exact_aa_step(h->geo, h->phys, h->A, h->dim, false, h->aa, h->stream, 0);
            CK(h, cudaEventRecord(ev[2 * k + 1], h->stream));
            exact_aa_step(h->geo, h->phys, h->A, h->dim, false, h->aa, h->stream, 1);
        } else if (use_xfused(h)) {
            // one fused pass per step: its time goes to the first slot, the second is empty
            if (k == 0) x_enter(h);
            CK(h, cudaEventRecord(ev[2 * k + 1], h->stream));
            x_pass(h);
            if (k == nsteps - 1) {
                CK(h, cudaEventRecord(ev[2 * k + 2], h->stream));
                x_exit(h);
                continue;
            }
        } else if (h->p.precision == LBM_FP64 && h->fixed) {
            const int nxt = h->cur ^ 1;
            const FixedArrays X = fixed_arrays(h);
            const long long *fc = (const long long*)h->fbuf[h->cur], *gc = (const long long*)h->gbuf[h->cur];
            long long *fn = (long long*)h->fbuf[nxt], *gn = (long long*)h->gbuf[nxt];
            fixed_fused_step(h->xgeo, h->px, X, h->dim, false, fc, gc, fn, gn, h->stream, 0, h->wide_index);
            CK(h, cudaEventRecord(ev[2 * k + 1], h->stream));
            fixed_fused_step(h->xgeo, h->px, X, h->dim, false, fc, gc, fn, gn, h->stream, 1, h->wide_index);
            h->cur = nxt;
        } else if (h->p.precision == LBM_FP64) {
            const int nxt = h->cur ^ 1;
            exact_fused_step(h->geo, h->phys, h->A, h->dim, false, h->fbuf[h->cur], h->gbuf[h->cur], h->fbuf[nxt],
                             h->gbuf[nxt], h->stream, 0);
            CK(h, cudaEventRecord(ev[2 * k + 1], h->stream));
            exact_fused_step(h->geo, h->phys, h->A, h->dim, false, h->fbuf[h->cur], h->gbuf[h->cur], h->fbuf[nxt],
                             h->gbuf[nxt], h->stream, 1);
            h->cur = nxt;
        } else if (use_single(h)) {
            // one kernel per step: its time goes to the first slot, the second is empty
            if (!h->F.ahead) fast_enter(h->F, h->geo, h->phys, h->dim, h->stream);
            CK(h, cudaEventRecord(ev[2 * k + 1], h->stream));
            fast_fused_step(h->F, h->geo, h->phys, h->dim, h->stream);
        } else {
            fast_step(h->F, h->geo, h->phys, h->dim, false, h->stream, 0);
            CK(h, cudaEventRecord(ev[2 * k + 1], h->stream));
            fast_step(h->F, h->geo, h->phys, h->dim, false, h->stream, 1);
        }
        CK(h, cudaEventRecord(ev[2 * k + 2], h->stream));
    }
    CK_LAUNCH(h, "timed steps");
    CK(h, cudaEventSynchronize(ev.back()));
    double tf = 0.0, tt = 0.0;
    for (int64_t k = 0; k < nsteps; ++k) {
        float a = 0.f, b = 0.f;
        CK(h, cudaEventElapsedTime(&a, ev[2 * k], ev[2 * k + 1]));
        CK(h, cudaEventElapsedTime(&b, ev[2 * k + 1], ev[2 * k + 2]));
        if (use_single(h) || use_xfused(h)) {
            tf += b;  // the fused kernel sits between the middle and the last event
        } else {
            tf += a;
            tt += b;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    *ms_flow = tf / (double)nsteps;
    *ms_thermal = tt / (double)nsteps;
    h->itc += nsteps;
    return LBM_OK;
}

extern "C" int lbm_set_option(lbm_handle* h, int option, int value) {
    if (!h) return LBM_ERR_PARAM;
    switch (option) {
        case LBM_OPT_HOST_DIRECT:
            if (value < 0 || value > 3) return fail(h, LBM_ERR_PARAM, "host-direct option: 0..3");
            if (value != 0 && !h->host_access)
                return fail(h, LBM_ERR_STATE, "the device cannot access pageable host memory");
            h->host_direct = (value & 1) != 0;
            h->host_direct_wr = (value & 2) != 0;
            break;
        case LBM_OPT_SINGLE_KERNEL:
            if (h->fixed) {  // fused passes of the fixed arithmetic (3D), or its two-kernel step
                h->xfused = value != 0;
                break;
            }
            if (h->p.precision == LBM_FP64) return fail(h, LBM_ERR_STATE, "the plain FP64 method has no single-kernel form");
            if (h->F.single_kernel != (value != 0)) {
                // leave the one-ahead phase and drop the graph captured for the other form
                h->F.ahead = false;
                h->F.single_kernel = value != 0;
            }
            break;
        case LBM_OPT_KCHUNK:
            if (value < 1) return fail(h, LBM_ERR_PARAM, "kchunk must be >= 1");
            h->F.kchunk = value;
            break;
        case LBM_OPT_PAIRS:
            if (h->p.precision == LBM_FP64) return fail(h, LBM_ERR_STATE, "the plain FP64 method has no paired form");
            h->F.pairs = value != 0;
            break;
        case LBM_OPT_WIDE_INDEX:
            if (h->p.precision == LBM_FP64 && !h->fixed)
                return fail(h, LBM_ERR_STATE, "the plain FP64 method indexes with 64-bit integers only");
            h->wide_index = value != 0;  // the captured chunk is dropped below
            h->F.wide = value != 0;
            break;
        case LBM_OPT_ROWS:
            if (h->p.precision == LBM_FP64) return fail(h, LBM_ERR_STATE, "the FP64 forms choose their own launches");
            h->F.rows = value != 0;
            break;
        case LBM_OPT_STAGED:
            if (h->p.precision == LBM_FP64) return fail(h, LBM_ERR_STATE, "the plain FP64 method has no staged form");
            h->F.tma = value != 0;
            break;
        case LBM_OPT_FP16_ROUNDING:
            if (h->p.precision != LBM_FP16) return fail(h, LBM_ERR_STATE, "the rounding option is for FP16 storage");
            if (h->ensemble) return fail(h, LBM_ERR_STATE, "remove the handle from its ensemble before changing its rounding");
            h->F.sr = value != 0;
            break;
        default:
            return fail(h, LBM_ERR_PARAM, "unknown option");
    }
    if (h->graph_exec) {
        CK(h, cudaStreamSynchronize(h->stream));
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
    }
    if (h->graph) {
        cudaGraphDestroy(h->graph);
        h->graph = nullptr;
    }
    return LBM_OK;
}

// ------------------------------------------------------------------------------------
// device footprint (for admission against an HBM budget)
// ------------------------------------------------------------------------------------
extern "C" int lbm_footprint(const lbm_params* p, size_t* bytes) {
    if (!bytes || validate(p) != LBM_OK) return LBM_ERR_PARAM;
    const size_t n = (size_t)p->nx * p->ny * (size_t)(p->dim == 3 ? p->nz : 1);
    const size_t q = p->dim == 3 ? 19 : 9, qt = p->dim == 3 ? 7 : 5;
    size_t b = 0;
    const bool aa = p->pattern == LBM_PATTERN_AA;
    const size_t es = p->precision == LBM_FP64 ? 8 : (p->precision == LBM_FP16 ? 2 : 4);
    if (p->precision == LBM_FP64) {
        b += 8 * n * (aa ? q + qt : 3 * q + 3 * qt);         // AA: f, g | f_post A/B, g_post A/B, f, g
        b += 8 * n * (p->dim == 3 ? 16 : 13);                // rho u v T Bx By up vp Tp jx jy (+w Bz wp Tlag jz | Fx Fy)
        if (p->arith == LBM_ARITH_FIXED) b += 8 * n * (p->dim == 3 ? 4 : 3);  // q60 B_prev and lag
    } else {
        const size_t nb = aa ? 1 : 2;
        b += es * n * (aa ? q + qt : 3 * q + 3 * qt);        // AA: f, g | F A/B, G A/B, f, g (module)
        b += 4 * n * nb * ((p->dim == 3 ? 3 : 2) + 1);       // B_prev, lag (A/B: two each)
        b += 4 * n * (p->dim == 3 ? 9 : 7);                  // rho u v T up vp Tp (+w wp)
    }
    if (aa) {  // face snapshots of the periodic axes
        const size_t fx = (size_t)p->ny * (p->dim == 3 ? p->nz : 1), fz = (size_t)p->nx * p->ny;
        if (p->bc_flow[0] == LBM_BC_PERIODIC) b += es * q * fx;
        if (p->bc_thermal[0] == LBM_BCT_PERIODIC) b += es * qt * fx;
        if (p->dim == 3 && p->bc_flow[2] == LBM_BC_PERIODIC) b += es * q * fz;
        if (p->dim == 3 && p->bc_thermal[2] == LBM_BCT_PERIODIC) b += es * qt * fz;
    }
    b += 8 * ((size_t)diag_blocks((long long)n) * DIAG_NSUM + 3 * (size_t)p->nx + (size_t)p->ny);
    *bytes = b;
    return LBM_OK;
}

// ------------------------------------------------------------------------------------
// batched stepping of many lattices
// ------------------------------------------------------------------------------------
struct lbm_ensemble {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<lbm_handle*> members;
    EnsPlan plan;
    EnsLaunchCfg cfg;
    bool dirty = true;
    int flip = 0;
    int sms = 152;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    std::string err;
};

static int efail(lbm_ensemble* e, int st, const std::string& m) {
    if (e) e->err = m;
    return st;
}

#define ECK(e, call)                                                                              \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return efail((e), e_ == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA,        \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                      \
    } while (0)

static void drop_graph(lbm_ensemble* e) {
    if (e->graph_exec) cudaGraphExecDestroy(e->graph_exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    e->graph_exec = nullptr;
    e->graph = nullptr;
}

extern "C" int lbm_ensemble_create(int device, lbm_ensemble** out) {
    if (!out) return LBM_ERR_PARAM;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return LBM_ERR_CUDA;
    lbm_ensemble* e = new (std::nothrow) lbm_ensemble();
    if (!e) return LBM_ERR_OOM;
    e->device = device;
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming) != cudaSuccess) {
        delete e;
        return LBM_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, device);
    *out = e;
    return LBM_OK;
}

extern "C" int lbm_ensemble_destroy(lbm_ensemble* e) {
    if (!e) return LBM_ERR_PARAM;
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->stream);
    for (lbm_handle* h : e->members) h->ensemble = nullptr;
    drop_graph(e);
    ens_free(e->plan);
    cudaEventDestroy(e->done);
    cudaStreamDestroy(e->stream);
    delete e;
    return LBM_OK;
}

extern "C" const char* lbm_ensemble_last_error(const lbm_ensemble* e) { return e ? e->err.c_str() : "null ensemble"; }

extern "C" int lbm_ensemble_add(lbm_ensemble* e, lbm_handle* h) {
    if (!e || !h) return LBM_ERR_PARAM;
    if (h->p.precision == LBM_FP64) return efail(e, LBM_ERR_STATE, "the batched form takes FP32/FP16 handles");
    if (h->p.pattern == LBM_PATTERN_AA) return efail(e, LBM_ERR_STATE, "the batched form takes two-buffer handles");
    if (h->device != e->device) return efail(e, LBM_ERR_PARAM, "handle is on another device");
    if (!h->initialised) return efail(e, LBM_ERR_STATE, "lbm_initial has not been called on the handle");
    if (h->ensemble) return efail(e, LBM_ERR_STATE, "handle already belongs to an ensemble");
    if (!e->members.empty() && e->members[0]->p.precision != h->p.precision)
        return efail(e, LBM_ERR_PARAM, "all members of an ensemble share one storage precision");
    if (!h->order_ev && cudaEventCreateWithFlags(&h->order_ev, cudaEventDisableTiming) != cudaSuccess)
        return efail(e, LBM_ERR_CUDA, "cudaEventCreate");
    // wait for the ensemble's queued work before the member is used again on its own stream
    cudaSetDevice(e->device);
    ECK(e, cudaStreamSynchronize(e->stream));
    e->members.push_back(h);
    h->ensemble = e;
    e->dirty = true;
    return LBM_OK;
}

extern "C" int lbm_ensemble_remove(lbm_ensemble* e, lbm_handle* h) {
    if (!e || !h) return LBM_ERR_PARAM;
    for (size_t i = 0; i < e->members.size(); ++i) {
        if (e->members[i] == h) {
            cudaSetDevice(e->device);
            cudaStreamSynchronize(e->stream);
            e->members.erase(e->members.begin() + (long)i);
            h->ensemble = nullptr;
            e->dirty = true;
            return LBM_OK;
        }
    }
    return efail(e, LBM_ERR_PARAM, "handle is not a member");
}

extern "C" int lbm_ensemble_size(const lbm_ensemble* e) { return e ? (int)e->members.size() : -1; }

extern "C" int lbm_ensemble_get_stream(lbm_ensemble* e, void** stream) {
    if (!e || !stream) return LBM_ERR_PARAM;
    *stream = (void*)e->stream;
    return LBM_OK;
}

static int ens_rebuild(lbm_ensemble* e) {
    std::vector<EnsMemberHost> mh;
    for (lbm_handle* h : e->members) mh.push_back(EnsMemberHost{h->geo, h->phys, &h->F, h->dim});
    drop_graph(e);
    ECK(e, ens_build(e->plan, mh, e->cfg, e->sms));
    e->flip = 0;
    e->dirty = false;
    return LBM_OK;
}

extern "C" int lbm_ensemble_step(lbm_ensemble* e, int64_t nsteps) {
    NvtxRange range_("lbm_ensemble_step");
    if (!e || nsteps < 0) return LBM_ERR_PARAM;
    if (e->members.empty() || nsteps == 0) return LBM_OK;
    ECK(e, cudaSetDevice(e->device));
    // a member not in the fused form takes its first step (reading the module arrays) alone
    for (lbm_handle* h : e->members) {
        if (!h->F.fused_valid) {
            enqueue_one(h, true);
            h->itc += 1;
            e->dirty = true;
        }
        h->F.ahead = false;
    }
    if (e->dirty) {
        int st = ens_rebuild(e);
        if (st != LBM_OK) return st;
    }
    for (lbm_handle* h : e->members) {
        ECK(e, cudaEventRecord(h->order_ev, h->stream));
        ECK(e, cudaStreamWaitEvent(e->stream, h->order_ev, 0));
    }
    int64_t done = 0;
    while (done < nsteps) {
        if (e->flip == 0 && nsteps - done >= kChunkSteps) {
            if (!e->graph_exec) {
                ECK(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
                for (int s = 0; s < kChunkSteps; ++s) ens_step(e->plan, s & 1, e->stream);
                cudaGraph_t g = nullptr;
                ECK(e, cudaStreamEndCapture(e->stream, &g));
                e->graph = g;
                ECK(e, cudaGraphInstantiate(&e->graph_exec, g, 0));
            }
            ECK(e, cudaGraphLaunch(e->graph_exec, e->stream));
            done += kChunkSteps;
        } else {
            ens_step(e->plan, e->flip, e->stream);
            e->flip ^= 1;
            done += 1;
        }
    }
    ECK(e, cudaGetLastError());
    ECK(e, cudaEventRecord(e->done, e->stream));
    for (lbm_handle* h : e->members) {
        ECK(e, cudaStreamWaitEvent(h->stream, e->done, 0));
        h->F.cur ^= (int)(nsteps & 1);
        h->F.fused_valid = true;
        h->itc += nsteps;
    }
    return LBM_OK;
}

extern "C" int lbm_ensemble_sync(lbm_ensemble* e) {
    if (!e) return LBM_ERR_PARAM;
    ECK(e, cudaSetDevice(e->device));
    ECK(e, cudaStreamSynchronize(e->stream));
    return LBM_OK;
}

extern "C" int lbm_ensemble_configure(lbm_ensemble* e, int block, int tile_cells, int grid_mul, int pairs) {
    if (!e) return LBM_ERR_PARAM;
    if ((block != 128 && block != 256) || tile_cells <= 0 || tile_cells % block != 0 || grid_mul < 1 ||
        grid_mul > 64 || pairs < 0 || pairs > 3)
        return efail(e, LBM_ERR_PARAM, "lbm_ensemble_configure: block 128 or 256, tile_cells a positive multiple "
                                       "of block, grid_mul 1..64, pairs 0..3");
    e->cfg = EnsLaunchCfg{block, tile_cells, grid_mul, pairs};
    e->dirty = true;
    return LBM_OK;
}

extern "C" int lbm_ensemble_get_launch(const lbm_ensemble* e, int* block, int* tile_cells, int* grid_mul,
                                       int* pairs) {
    if (!e) return LBM_ERR_PARAM;
    if (block) *block = e->cfg.block;
    if (tile_cells) *tile_cells = e->cfg.tile_cells;
    if (grid_mul) *grid_mul = e->cfg.grid_mul;
    if (pairs) *pairs = e->cfg.pairs;
    return LBM_OK;
}

// Time `nsteps` batched steps per launch configuration and keep the fastest.  The steps
// are real steps: every member advances by ncand * nsteps steps.
extern "C" int lbm_ensemble_autotune(lbm_ensemble* e, int nsteps, int* best_block, int* best_tile, int* best_grid) {
    if (!e || nsteps <= 0) return LBM_ERR_PARAM;
    if (e->members.empty()) return LBM_OK;
    // pairs: bit 0 pairs the 2D members, bit 1 the 3D members
    const EnsLaunchCfg cands[] = {{128, 1024, 16, 1}, {128, 1024, 32, 1}, {128, 1024, 64, 1}, {128, 512, 64, 1},
                                  {128, 2048, 32, 1}, {256, 2048, 16, 1}, {256, 4096, 8, 1},  {128, 1024, 32, 3},
                                  {128, 1024, 16, 0}, {128, 1024, 32, 0}, {128, 512, 64, 0},  {256, 2048, 8, 0}};
    ECK(e, cudaSetDevice(e->device));
    int st = lbm_ensemble_step(e, 1);  // first steps and ordering
    if (st != LBM_OK) return st;
    cudaEvent_t a, b;
    ECK(e, cudaEventCreate(&a));
    ECK(e, cudaEventCreate(&b));
    float best = 1e30f;
    EnsLaunchCfg bestc = e->cfg;
    for (const EnsLaunchCfg& c : cands) {
        e->cfg = c;
        if ((st = ens_rebuild(e)) != LBM_OK) return st;
        ens_step(e->plan, 0, e->stream);  // warm
        ens_step(e->plan, 1, e->stream);
        ECK(e, cudaEventRecord(a, e->stream));
        for (int s = 0; s < nsteps; ++s) ens_step(e->plan, s & 1, e->stream);
        ECK(e, cudaEventRecord(b, e->stream));
        ECK(e, cudaEventSynchronize(b));
        float ms = 0.f;
        ECK(e, cudaEventElapsedTime(&ms, a, b));
        if (ms < best) {
            best = ms;
            bestc = c;
        }
        const int adv = 2 + nsteps;
        for (lbm_handle* h : e->members) {
            h->F.cur ^= (adv & 1);
            h->itc += adv;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    ECK(e, cudaEventRecord(e->done, e->stream));
    for (lbm_handle* h : e->members) ECK(e, cudaStreamWaitEvent(h->stream, e->done, 0));
    e->cfg = bestc;
    e->dirty = true;
    if (best_block) *best_block = bestc.block;
    if (best_tile) *best_tile = bestc.tile_cells;
    if (best_grid) *best_grid = bestc.grid_mul;
    return LBM_OK;
}
