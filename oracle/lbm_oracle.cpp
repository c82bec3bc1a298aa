// lbm_oracle.cpp - CPU oracle (test infrastructure only; see lbm_oracle.h).
//
// A literal restatement of the reference's hot path in C++:
//   2D: 2DRB.F90 (commondata 48-194, initial 371-663, step 675-1134, check 1213-1260,
//       calNuRe 1610-1675, RBcalc_Nu_global 2251-2297, RBcalc_Nu_wall_avg 2308-2473,
//       fit_adiabatic_wall_T4 1953-1991, fit_parabola_ls5 1999-2080)
//   3D: 3DRB.F90 (commondata3d 55-187, initial 342-643, init_lattice_constants 650-679,
//       step 689-1381, check 1475-1528, calNuRe 1712-1778, RBcalc_Nu_global 1839-1878,
//       RBcalc_Nu_wall_avg 2049-2210, fits 2219-2334)
// Arrays keep the Fortran layout: f(0:q-1,1:nx,1:ny[,1:nz]) direction-fastest, and
// f_post/g_post carry one ghost layer (0:nx+1, ...), zero-filled, as in the reference.
// Every floating-point expression keeps the reference's left-to-right order; build with
// -ffp-contract=off so that no multiply-add is fused.
// Reductions (check, calNuRe, Nu) run serially in loop order so results are reproducible;
// the reference's OpenMP reductions combine partial sums in an unspecified order.

#include "lbm_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <new>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kPi = 3.141592653589793115997963468544185161590576171875;  // acos(-1.0d0)

struct Lattice {
    int q, qt;
    int ex[19], ey[19], ez[19], opp[19];
    int exT[7], eyT[7], ezT[7], oppT[7];
    double omega[19], omegaT[7];
};

}  // namespace

struct ora_handle {
    lbm_params p;
    lbm_constants c;
    Lattice L;
    bool d3;
    int nx, ny, nz;
    size_t ncell, npad;
    std::vector<double> f, fpost, g, gpost;
    std::vector<double> rho, u, v, w, T, up, vp, wp, Tp;
    std::vector<double> Bx, By, Bz, Fx, Fy;
    std::vector<double> xp, yp, zp;
    long long itc;

    // cell (1-based) -> linear index; padded (0-based incl. ghosts) -> linear index
    inline size_t C(int i, int j, int k) const {
        return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
    }
    inline size_t P(int i, int j, int k) const {
        return (size_t)i + (size_t)(nx + 2) * ((size_t)j + (size_t)(ny + 2) * (size_t)(d3 ? k : 0));
    }
};

// ------------------------------------------------------------------------------------
// commondata / commondata3d parameter block (2DRB.F90:61-115, 3DRB.F90:73-123)
// ------------------------------------------------------------------------------------
static int derive(const lbm_params* p, lbm_constants* c) {
    if (!p || !c) return LBM_ERR_PARAM;
    if (p->dim != 2 && p->dim != 3) return LBM_ERR_PARAM;
    if (p->nx < 5 || p->ny < 5) return LBM_ERR_PARAM;
    if (p->dim == 2 && p->nz != 1) return LBM_ERR_PARAM;
    if (p->dim == 3 && p->nz < 2) return LBM_ERR_PARAM;
    if (!(p->Ra > 0) || !(p->Pr > 0) || !(p->Mach > 0)) return LBM_ERR_PARAM;
    if (p->cell != LBM_CELL_RB && p->cell != LBM_CELL_SIDE) return LBM_ERR_PARAM;
    // boundary switches that exist in the reference
    if (p->bc_flow[0] != LBM_BC_NOSLIP && p->bc_flow[0] != LBM_BC_PERIODIC) return LBM_ERR_PARAM;
    if (p->bc_flow[1] != LBM_BC_NOSLIP) return LBM_ERR_PARAM;
    if (p->bc_thermal[0] < 0 || p->bc_thermal[0] > 2) return LBM_ERR_PARAM;
    if (p->bc_thermal[1] != LBM_BCT_CONST && p->bc_thermal[1] != LBM_BCT_ADIABATIC) return LBM_ERR_PARAM;
    if (p->dim == 3) {
        if (p->bc_flow[2] != LBM_BC_NOSLIP && p->bc_flow[2] != LBM_BC_PERIODIC) return LBM_ERR_PARAM;
        if (p->bc_thermal[2] != LBM_BCT_ADIABATIC && p->bc_thermal[2] != LBM_BCT_PERIODIC) return LBM_ERR_PARAM;
    }
    std::memset(c, 0, sizeof(*c));
    const double L = (p->cell == LBM_CELL_SIDE) ? (double)p->nx : (double)p->ny;
    c->lengthUnit = L;
    c->Tref = 0.5 * (p->Thot + p->Tcold);
    c->tauf = 0.5 + p->Mach * L * std::sqrt(3.0 * p->Pr / p->Ra);
    c->viscosity = (c->tauf - 0.5) / 3.0;
    c->diffusivity = c->viscosity / p->Pr;
    c->heatFluxScale = L / c->diffusivity;
    c->velocityScaleCompare = L / c->diffusivity;
    double gBeta1 = p->Ra * c->viscosity * c->diffusivity / L;
    c->gBeta = gBeta1 / L / L;
    c->timeUnit = std::sqrt(L / c->gBeta);
    c->velocityUnit = std::sqrt(c->gBeta * L);
    if (p->dim == 2) {
        c->paraA = 20.0 * std::sqrt(3.0) * c->diffusivity - 4.0;
        c->Snu = 1.0 / c->tauf;
        c->Sq = 8.0 * (2.0 * c->tauf - 1.0) / (8.0 * c->tauf - 1.0);
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
        c->Snu = 1.0 / c->tauf;
        c->Spi = 1.0 / c->tauf;
        c->Sq = 8.0 * (2.0 * c->tauf - 1.0) / (8.0 * c->tauf - 1.0);
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
    c->SG = 1.0 - 0.5 * c->Qk;  // collisionT: SG = 1 - 0.5*Qk (2DRB.F90:915, 3DRB.F90:1113)
    if (p->side_heated_ha) {
        if (p->dim != 2) return LBM_ERR_PARAM;
        const double pi = std::acos(-1.0);                             // 2DRB.F90:67
        c->phi = p->phi_deg * (pi / 180.0);                            // 2DRB.F90:90
        c->B2sigemarho = (p->Ha * p->Ha * c->viscosity) / (L * L);     // 2DRB.F90:91
        c->sinphi = std::sin(c->phi);
        c->cosphi = std::cos(c->phi);
    }
    if (!(c->tauf > 0.5)) return LBM_ERR_PARAM;
    return LBM_OK;
}

static void init_lattice(ora_handle* h) {
    Lattice& L = h->L;
    std::memset(&L, 0, sizeof(L));
    if (!h->d3) {
        // D2Q9: 2DRB.F90:189-190; weights 2DRB.F90:506-512
        static const int ex[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
        static const int ey[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
        static const int opp[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
        L.q = 9;
        L.qt = 5;
        for (int a = 0; a < 9; ++a) { L.ex[a] = ex[a]; L.ey[a] = ey[a]; L.opp[a] = opp[a]; }
        L.omega[0] = 4.0 / 9.0;
        for (int a = 1; a <= 4; ++a) L.omega[a] = 1.0 / 9.0;
        for (int a = 5; a <= 8; ++a) L.omega[a] = 1.0 / 36.0;
        for (int a = 0; a < 5; ++a) { L.exT[a] = ex[a]; L.eyT[a] = ey[a]; L.oppT[a] = opp[a]; }
        L.omegaT[0] = h->c.omegaT0;
        for (int a = 1; a <= 4; ++a) L.omegaT[a] = h->c.omegaT1;
    } else {
        // D3Q19 / D3Q7: 3DRB.F90:655-676
        static const int ex[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
        static const int ey[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
        static const int ez[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
        static const int opp[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
        L.q = 19;
        L.qt = 7;
        for (int a = 0; a < 19; ++a) { L.ex[a] = ex[a]; L.ey[a] = ey[a]; L.ez[a] = ez[a]; L.opp[a] = opp[a]; }
        L.omega[0] = 1.0 / 3.0;
        for (int a = 1; a <= 6; ++a) L.omega[a] = 1.0 / 18.0;
        for (int a = 7; a <= 18; ++a) L.omega[a] = 1.0 / 36.0;
        for (int a = 0; a < 7; ++a) { L.exT[a] = ex[a]; L.eyT[a] = ey[a]; L.ezT[a] = ez[a]; L.oppT[a] = opp[a]; }
        L.omegaT[0] = h->c.omegaT0;
        for (int a = 1; a <= 6; ++a) L.omegaT[a] = h->c.omegaT1;
    }
}

// splitmix64 of (seed ^ cell index) -> xi in [0,1) with 53 random bits.
static inline double noise_xi(uint64_t seed, uint64_t idx) {
    uint64_t z = (seed ^ idx) + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

extern "C" int ora_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

extern "C" int ora_create(const lbm_params* p, ora_handle** out) {
    if (!out) return LBM_ERR_PARAM;
    *out = nullptr;
    lbm_constants c;
    int st = derive(p, &c);
    if (st != LBM_OK) return st;
    ora_handle* h = new (std::nothrow) ora_handle();
    if (!h) return LBM_ERR_OOM;
    h->p = *p;
    h->c = c;
    h->d3 = (p->dim == 3);
    h->nx = p->nx;
    h->ny = p->ny;
    h->nz = h->d3 ? p->nz : 1;
    init_lattice(h);
    h->ncell = (size_t)h->nx * h->ny * h->nz;
    h->npad = (size_t)(h->nx + 2) * (h->ny + 2) * (h->d3 ? (h->nz + 2) : 1);
    try {
        h->f.assign((size_t)h->L.q * h->ncell, 0.0);
        h->fpost.assign((size_t)h->L.q * h->npad, 0.0);
        h->g.assign((size_t)h->L.qt * h->ncell, 0.0);
        h->gpost.assign((size_t)h->L.qt * h->npad, 0.0);
        for (auto* a : {&h->rho, &h->u, &h->v, &h->T, &h->up, &h->vp, &h->Tp, &h->Bx, &h->By})
            a->assign(h->ncell, 0.0);
        if (h->d3) {
            for (auto* a : {&h->w, &h->wp, &h->Bz}) a->assign(h->ncell, 0.0);
        } else {
            for (auto* a : {&h->Fx, &h->Fy}) a->assign(h->ncell, 0.0);
        }
    } catch (...) {
        delete h;
        return LBM_ERR_OOM;
    }
    h->itc = 0;
    *out = h;
    return LBM_OK;
}

extern "C" void ora_destroy(ora_handle* h) { delete h; }

extern "C" int ora_constants(const ora_handle* h, lbm_constants* out) {
    if (!h || !out) return LBM_ERR_PARAM;
    *out = h->c;
    return LBM_OK;
}

// ------------------------------------------------------------------------------------
// initial (2DRB.F90:371-663 / 3DRB.F90:342-643), loadInitField = 0
// ------------------------------------------------------------------------------------
extern "C" int ora_initial(ora_handle* h) {
    const lbm_params& p = h->p;
    const lbm_constants& c = h->c;
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const double Lu = c.lengthUnit;
    h->itc = 0;
    // xp(0)=0, xp(nx+1)=nx, xp(i)=i-0.5, then xp = xp/lengthUnit (2DRB.F90:463-475)
    h->xp.assign(nx + 2, 0.0);
    h->yp.assign(ny + 2, 0.0);
    h->zp.assign(nz + 2, 0.0);
    h->xp[0] = 0.0;
    h->xp[nx + 1] = (double)nx;
    for (int i = 1; i <= nx; ++i) h->xp[i] = (double)i - 0.5;
    for (auto& x : h->xp) x = x / Lu;
    h->yp[0] = 0.0;
    h->yp[ny + 1] = (double)ny;
    for (int j = 1; j <= ny; ++j) h->yp[j] = (double)j - 0.5;
    for (auto& y : h->yp) y = y / Lu;
    if (h->d3) {
        h->zp[0] = 0.0;
        h->zp[nz + 1] = (double)nz;
        for (int k = 1; k <= nz; ++k) h->zp[k] = (double)k - 0.5;
        for (auto& z : h->zp) z = z / Lu;
    }
    std::fill(h->rho.begin(), h->rho.end(), 1.0);
    std::fill(h->u.begin(), h->u.end(), 0.0);
    std::fill(h->v.begin(), h->v.end(), 0.0);
    std::fill(h->T.begin(), h->T.end(), 0.0);
    std::fill(h->Bx.begin(), h->Bx.end(), 0.0);
    std::fill(h->By.begin(), h->By.end(), 0.0);
    if (h->d3) {
        std::fill(h->w.begin(), h->w.end(), 0.0);
        std::fill(h->Bz.begin(), h->Bz.end(), 0.0);
    }
    const std::vector<double>& xp = h->xp;
    const std::vector<double>& yp = h->yp;
    // VerticalWallsConstT: T linear in x (2DRB.F90:545-552, 3DRB.F90:525-534)
    if (p.bc_thermal[0] == LBM_BCT_CONST) {
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i)
                    h->T[h->C(i, j, k)] = p.Thot + (xp[i] - xp[0]) / (xp[nx + 1] - xp[0]) * (p.Tcold - p.Thot);
    }
    // HorizontalWallsConstT: T linear in y, RB sinusoidal perturbation at small Ra
    // (2DRB.F90:555-583, 3DRB.F90:537-558)
    if (p.bc_thermal[1] == LBM_BCT_CONST) {
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i)
                    h->T[h->C(i, j, k)] = p.Thot + (yp[j] - yp[0]) / (yp[ny + 1] - yp[0]) * (p.Tcold - p.Thot);
        if (p.cell == LBM_CELL_RB) {
            bool perturb = h->d3 ? (p.Ra <= 1.0e4) : (p.Ra < 1.0e4);
            if (perturb) {
                double xLen = xp[nx + 1];
                double yLen = yp[ny + 1];
                double amp = 1.0e-3 * (p.Thot - p.Tcold);
                for (int k = 1; k <= nz; ++k)
                    for (int j = 1; j <= ny; ++j)
                        for (int i = 1; i <= nx; ++i) {
                            double sx = h->d3 ? std::cos(2.0 * kPi * xp[i] / xLen) : std::sin(2.0 * kPi * xp[i] / xLen);
                            size_t ci = h->C(i, j, k);
                            h->T[ci] = h->T[ci] + amp * sx * std::sin(kPi * yp[j] / yLen);
                        }
            }
        }
    }
    // Seeded noise (no counterpart in the reference, which has no random numbers).
    if (p.noise_amp != 0.0) {
        for (size_t ci = 0; ci < h->ncell; ++ci) {
            double xi = noise_xi(p.seed, (uint64_t)ci);
            h->T[ci] = h->T[ci] + p.noise_amp * (2.0 * xi - 1.0);
        }
    }
    const Lattice& L = h->L;
    // equilibrium populations (2DRB.F90:593-607, 3DRB.F90:587-603)
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                size_t ci = h->C(i, j, k);
                double uu = h->u[ci], vv = h->v[ci], TT = h->T[ci], rr = h->rho[ci];
                if (!h->d3) {
                    double us2 = uu * uu + vv * vv;
                    for (int a = 0; a < 9; ++a) {
                        double un = uu * L.ex[a] + vv * L.ey[a];
                        h->f[a + 9 * ci] = rr * L.omega[a] * (1.0 + 3.0 * un + 4.5 * un * un - 1.5 * us2);
                    }
                    for (int a = 0; a < 5; ++a) {
                        double un = uu * L.ex[a] + vv * L.ey[a];
                        h->g[a + 5 * ci] = L.omegaT[a] * TT * (1.0 + c.thermalGeqCoeff * un);
                    }
                } else {
                    double ww = h->w[ci];
                    double u2Loc = uu * uu + vv * vv + ww * ww;
                    for (int a = 0; a < 19; ++a) {
                        double eu = (double)L.ex[a] * uu + (double)L.ey[a] * vv + (double)L.ez[a] * ww;
                        h->f[a + 19 * ci] = L.omega[a] * rr * (1.0 + 3.0 * eu + 4.5 * eu * eu - 1.5 * u2Loc);
                    }
                    for (int a = 0; a < 7; ++a) {
                        double eu = (double)L.exT[a] * uu + (double)L.eyT[a] * vv + (double)L.ezT[a] * ww;
                        h->g[a + 7 * ci] = L.omegaT[a] * TT * (1.0 + c.thermalGeqCoeff * eu);
                    }
                }
                if (p.use_g) {
                    h->Bx[ci] = uu * TT;
                    h->By[ci] = vv * TT;
                    if (h->d3) h->Bz[ci] = h->w[ci] * TT;
                }
            }
    std::fill(h->up.begin(), h->up.end(), 0.0);
    std::fill(h->vp.begin(), h->vp.end(), 0.0);
    std::fill(h->Tp.begin(), h->Tp.end(), 0.0);
    if (h->d3) std::fill(h->wp.begin(), h->wp.end(), 0.0);
    std::fill(h->fpost.begin(), h->fpost.end(), 0.0);
    std::fill(h->gpost.begin(), h->gpost.end(), 0.0);
    if (!h->d3) {
        std::fill(h->Fx.begin(), h->Fx.end(), 0.0);
        std::fill(h->Fy.begin(), h->Fy.end(), 0.0);
    }
    return LBM_OK;
}

// Hand-expanded moment transforms, kept verbatim from the reference so that the
// collisions and the known-answer matrix extraction share one statement of them.
// D2Q9 m = M f (2DRB.F90:688-696)
static inline void d2q9_forward(const double* F, double* m) {
    m[0] = F[0] + F[1] + F[2] + F[3] + F[4] + F[5] + F[6] + F[7] + F[8];
    m[1] = -4.0 * F[0] - F[1] - F[2] - F[3] - F[4] + 2.0 * (F[5] + F[6] + F[7] + F[8]);
    m[2] = 4.0 * F[0] - 2.0 * (F[1] + F[2] + F[3] + F[4]) + F[5] + F[6] + F[7] + F[8];
    m[3] = F[1] - F[3] + F[5] - F[6] - F[7] + F[8];
    m[4] = -2.0 * F[1] + 2.0 * F[3] + F[5] - F[6] - F[7] + F[8];
    m[5] = F[2] - F[4] + F[5] + F[6] - F[7] - F[8];
    m[6] = -2.0 * F[2] + 2.0 * F[4] + F[5] + F[6] - F[7] - F[8];
    m[7] = F[1] - F[2] + F[3] - F[4];
    m[8] = F[5] - F[6] + F[7] - F[8];
}

// D2Q9 f_post = M^-1 m_post (2DRB.F90:743-759)
static inline void d2q9_inverse(const double* m_post, double* FP) {
    FP[0] = m_post[0] / 9.0 - m_post[1] / 9.0 + m_post[2] / 9.0;
    FP[1] = m_post[0] / 9.0 - m_post[1] / 36.0 - m_post[2] / 18.0 + m_post[3] / 6.0 - m_post[4] / 6.0
            + m_post[7] / 4.0;
    FP[2] = m_post[0] / 9.0 - m_post[1] / 36.0 - m_post[2] / 18.0
            + m_post[5] / 6.0 - m_post[6] / 6.0 - m_post[7] / 4.0;
    FP[3] = m_post[0] / 9.0 - m_post[1] / 36.0 - m_post[2] / 18.0 - m_post[3] / 6.0 + m_post[4] / 6.0
            + m_post[7] / 4.0;
    FP[4] = m_post[0] / 9.0 - m_post[1] / 36.0 - m_post[2] / 18.0
            - m_post[5] / 6.0 + m_post[6] / 6.0 - m_post[7] / 4.0;
    FP[5] = m_post[0] / 9.0 + m_post[1] / 18.0 + m_post[2] / 36.0 + m_post[3] / 6.0 + m_post[4] / 12.0
            + m_post[5] / 6.0 + m_post[6] / 12.0 + m_post[8] / 4.0;
    FP[6] = m_post[0] / 9.0 + m_post[1] / 18.0 + m_post[2] / 36.0 - m_post[3] / 6.0 - m_post[4] / 12.0
            + m_post[5] / 6.0 + m_post[6] / 12.0 - m_post[8] / 4.0;
    FP[7] = m_post[0] / 9.0 + m_post[1] / 18.0 + m_post[2] / 36.0 - m_post[3] / 6.0 - m_post[4] / 12.0
            - m_post[5] / 6.0 - m_post[6] / 12.0 + m_post[8] / 4.0;
    FP[8] = m_post[0] / 9.0 + m_post[1] / 18.0 + m_post[2] / 36.0 + m_post[3] / 6.0 + m_post[4] / 12.0
            - m_post[5] / 6.0 - m_post[6] / 12.0 - m_post[8] / 4.0;
}

// D2Q5 n = N g (2DRB.F90:951-955)
static inline void d2q5_forward(const double* G, double* n) {
    n[0] = G[0] + G[1] + G[2] + G[3] + G[4];
    n[1] = G[1] - G[3];
    n[2] = G[2] - G[4];
    n[3] = -4.0 * G[0] + G[1] + G[2] + G[3] + G[4];
    n[4] = G[1] - G[2] + G[3] - G[4];
}

// D2Q5 g_post = N^-1 n_post (2DRB.F90:970-974)
static inline void d2q5_inverse(const double* n_post, double* GP) {
    GP[0] = 0.2 * n_post[0] - 0.2 * n_post[3];
    GP[1] = 0.2 * n_post[0] + 0.5 * n_post[1] + 0.05 * n_post[3] + 0.25 * n_post[4];
    GP[2] = 0.2 * n_post[0] + 0.5 * n_post[2] + 0.05 * n_post[3] - 0.25 * n_post[4];
    GP[3] = 0.2 * n_post[0] - 0.5 * n_post[1] + 0.05 * n_post[3] + 0.25 * n_post[4];
    GP[4] = 0.2 * n_post[0] - 0.5 * n_post[2] + 0.05 * n_post[3] - 0.25 * n_post[4];
}

// D3Q19 m = M f (3DRB.F90:714-775)
static inline void d3q19_forward(const double* f, double* m) {
    m[0] = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8] + f[9] + f[10] + f[11] + f[12]
           + f[13] + f[14] + f[15] + f[16] + f[17] + f[18];
    m[1] = -30.0 * f[0] - 11.0 * (f[1] + f[2] + f[3] + f[4] + f[5] + f[6])
           + 8.0 * (f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18]);
    m[2] = 12.0 * f[0] - 4.0 * (f[1] + f[2] + f[3] + f[4] + f[5] + f[6])
           + (f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18]);
    m[3] = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    m[4] = -4.0 * f[1] + 4.0 * f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    m[5] = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
    m[6] = -4.0 * f[3] + 4.0 * f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
    m[7] = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
    m[8] = -4.0 * f[5] + 4.0 * f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
    m[9] = 2.0 * (f[1] + f[2]) - (f[3] + f[4] + f[5] + f[6])
           + (f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14])
           - 2.0 * (f[15] + f[16] + f[17] + f[18]);
    m[10] = -4.0 * (f[1] + f[2]) + 2.0 * (f[3] + f[4] + f[5] + f[6])
            + (f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14])
            - 2.0 * (f[15] + f[16] + f[17] + f[18]);
    m[11] = (f[3] + f[4]) - (f[5] + f[6]) + (f[7] + f[8] + f[9] + f[10]) - (f[11] + f[12] + f[13] + f[14]);
    m[12] = -2.0 * (f[3] + f[4]) + 2.0 * (f[5] + f[6]) + (f[7] + f[8] + f[9] + f[10])
            - (f[11] + f[12] + f[13] + f[14]);
    m[13] = f[7] - f[8] - f[9] + f[10];
    m[14] = f[15] - f[16] - f[17] + f[18];
    m[15] = f[11] - f[12] - f[13] + f[14];
    m[16] = f[7] - f[8] + f[9] - f[10] - f[11] + f[12] - f[13] + f[14];
    m[17] = -f[7] - f[8] + f[9] + f[10] + f[15] - f[16] + f[17] - f[18];
    m[18] = f[11] + f[12] - f[13] - f[14] - f[15] - f[16] + f[17] + f[18];
}

// D3Q19 f_post = M^-1 m_post (3DRB.F90:861-943)
static inline void d3q19_inverse(const double* mp, double* fp) {
    fp[0] = mp[0] / 19.0 - 5.0 * mp[1] / 399.0 + mp[2] / 21.0;
    fp[1] = mp[0] / 19.0 - 11.0 * mp[1] / 2394.0 - mp[2] / 63.0 + mp[3] / 10.0 - mp[4] / 10.0
            + mp[9] / 18.0 - mp[10] / 18.0;
    fp[2] = mp[0] / 19.0 - 11.0 * mp[1] / 2394.0 - mp[2] / 63.0 - mp[3] / 10.0 + mp[4] / 10.0
            + mp[9] / 18.0 - mp[10] / 18.0;
    fp[3] = mp[0] / 19.0 - 11.0 * mp[1] / 2394.0 - mp[2] / 63.0 + mp[5] / 10.0 - mp[6] / 10.0
            - mp[9] / 36.0 + mp[10] / 36.0 + mp[11] / 12.0 - mp[12] / 12.0;
    fp[4] = mp[0] / 19.0 - 11.0 * mp[1] / 2394.0 - mp[2] / 63.0 - mp[5] / 10.0 + mp[6] / 10.0
            - mp[9] / 36.0 + mp[10] / 36.0 + mp[11] / 12.0 - mp[12] / 12.0;
    fp[5] = mp[0] / 19.0 - 11.0 * mp[1] / 2394.0 - mp[2] / 63.0 + mp[7] / 10.0 - mp[8] / 10.0
            - mp[9] / 36.0 + mp[10] / 36.0 - mp[11] / 12.0 + mp[12] / 12.0;
    fp[6] = mp[0] / 19.0 - 11.0 * mp[1] / 2394.0 - mp[2] / 63.0 - mp[7] / 10.0 + mp[8] / 10.0
            - mp[9] / 36.0 + mp[10] / 36.0 - mp[11] / 12.0 + mp[12] / 12.0;
    fp[7] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 + mp[3] / 10.0 + mp[4] / 40.0
            + mp[5] / 10.0 + mp[6] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 + mp[11] / 12.0
            + mp[12] / 24.0 + mp[13] / 4.0 + mp[16] / 8.0 - mp[17] / 8.0;
    fp[8] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 - mp[3] / 10.0 - mp[4] / 40.0
            + mp[5] / 10.0 + mp[6] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 + mp[11] / 12.0
            + mp[12] / 24.0 - mp[13] / 4.0 - mp[16] / 8.0 - mp[17] / 8.0;
    fp[9] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 + mp[3] / 10.0 + mp[4] / 40.0
            - mp[5] / 10.0 - mp[6] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 + mp[11] / 12.0
            + mp[12] / 24.0 - mp[13] / 4.0 + mp[16] / 8.0 + mp[17] / 8.0;
    fp[10] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 - mp[3] / 10.0 - mp[4] / 40.0
             - mp[5] / 10.0 - mp[6] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 + mp[11] / 12.0
             + mp[12] / 24.0 + mp[13] / 4.0 - mp[16] / 8.0 + mp[17] / 8.0;
    fp[11] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 + mp[3] / 10.0 + mp[4] / 40.0
             + mp[7] / 10.0 + mp[8] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 - mp[11] / 12.0
             - mp[12] / 24.0 + mp[15] / 4.0 - mp[16] / 8.0 + mp[18] / 8.0;
    fp[12] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 - mp[3] / 10.0 - mp[4] / 40.0
             + mp[7] / 10.0 + mp[8] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 - mp[11] / 12.0
             - mp[12] / 24.0 - mp[15] / 4.0 + mp[16] / 8.0 + mp[18] / 8.0;
    fp[13] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 + mp[3] / 10.0 + mp[4] / 40.0
             - mp[7] / 10.0 - mp[8] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 - mp[11] / 12.0
             - mp[12] / 24.0 - mp[15] / 4.0 - mp[16] / 8.0 - mp[18] / 8.0;
    fp[14] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 - mp[3] / 10.0 - mp[4] / 40.0
             - mp[7] / 10.0 - mp[8] / 40.0 + mp[9] / 36.0 + mp[10] / 72.0 - mp[11] / 12.0
             - mp[12] / 24.0 + mp[15] / 4.0 + mp[16] / 8.0 - mp[18] / 8.0;
    fp[15] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 + mp[5] / 10.0 + mp[6] / 40.0
             + mp[7] / 10.0 + mp[8] / 40.0 - mp[9] / 18.0 - mp[10] / 36.0 + mp[14] / 4.0
             + mp[17] / 8.0 - mp[18] / 8.0;
    fp[16] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 - mp[5] / 10.0 - mp[6] / 40.0
             + mp[7] / 10.0 + mp[8] / 40.0 - mp[9] / 18.0 - mp[10] / 36.0 - mp[14] / 4.0
             - mp[17] / 8.0 - mp[18] / 8.0;
    fp[17] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 + mp[5] / 10.0 + mp[6] / 40.0
             - mp[7] / 10.0 - mp[8] / 40.0 - mp[9] / 18.0 - mp[10] / 36.0 - mp[14] / 4.0
             + mp[17] / 8.0 + mp[18] / 8.0;
    fp[18] = mp[0] / 19.0 + 4.0 * mp[1] / 1197.0 + mp[2] / 252.0 - mp[5] / 10.0 - mp[6] / 40.0
             - mp[7] / 10.0 - mp[8] / 40.0 - mp[9] / 18.0 - mp[10] / 36.0 + mp[14] / 4.0
             - mp[17] / 8.0 + mp[18] / 8.0;
}

// D3Q7 n = N g (3DRB.F90:1141-1147)
static inline void d3q7_forward(const double* g, double* n) {
    n[0] = g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6];
    n[1] = g[1] - g[2];
    n[2] = g[3] - g[4];
    n[3] = g[5] - g[6];
    n[4] = -6.0 * g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6];
    n[5] = 2.0 * g[1] + 2.0 * g[2] - g[3] - g[4] - g[5] - g[6];
    n[6] = g[3] + g[4] - g[5] - g[6];
}

// D3Q7 g_post = N^-1 n_post (3DRB.F90:1181-1191)
static inline void d3q7_inverse(const double* n_post, double* gp) {
    gp[0] = n_post[0] / 7.0 - n_post[4] / 7.0;
    gp[1] = n_post[0] / 7.0 + n_post[1] / 2.0 + n_post[4] / 42.0 + n_post[5] / 6.0;
    gp[2] = n_post[0] / 7.0 - n_post[1] / 2.0 + n_post[4] / 42.0 + n_post[5] / 6.0;
    gp[3] = n_post[0] / 7.0 + n_post[2] / 2.0 + n_post[4] / 42.0 - n_post[5] / 12.0 + n_post[6] / 4.0;
    gp[4] = n_post[0] / 7.0 - n_post[2] / 2.0 + n_post[4] / 42.0 - n_post[5] / 12.0 + n_post[6] / 4.0;
    gp[5] = n_post[0] / 7.0 + n_post[3] / 2.0 + n_post[4] / 42.0 - n_post[5] / 12.0 - n_post[6] / 4.0;
    gp[6] = n_post[0] / 7.0 - n_post[3] / 2.0 + n_post[4] / 42.0 - n_post[5] / 12.0 - n_post[6] / 4.0;
}

// ------------------------------------------------------------------------------------
// 2D stages (2DRB.F90:675-1134)
// ------------------------------------------------------------------------------------
static void collision2d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny;
    const lbm_constants& c = h->c;
    const double Snu = c.Snu, Sq = c.Sq, gBeta = c.gBeta, Tref = c.Tref;
    const bool ha = h->p.side_heated_ha != 0;
    const double B2 = c.B2sigemarho, sphi = c.sinphi, cphi = c.cosphi;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j) {
        double m[9], m_post[9], meq[9], s[9], fSource[9];
        for (int i = 1; i <= nx; ++i) {
            size_t ci = h->C(i, j, 1);
            const double* F = &h->f[9 * ci];
            double* FP = &h->fpost[9 * h->P(i, j, 0)];
            double rho = h->rho[ci], u = h->u[ci], v = h->v[ci], T = h->T[ci];
            d2q9_forward(F, m);

            meq[0] = rho;
            meq[1] = rho * (-2.0 + 3.0 * (u * u + v * v));
            meq[2] = rho * (1.0 - 3.0 * (u * u + v * v));
            meq[3] = rho * u;
            meq[4] = -(rho * u);
            meq[5] = rho * v;
            meq[6] = -(rho * v);
            meq[7] = rho * (u * u - v * v);
            meq[8] = rho * (u * v);

            s[0] = 0.0; s[1] = Snu; s[2] = Snu; s[3] = 0.0; s[4] = Sq;
            s[5] = 0.0; s[6] = Sq;  s[7] = Snu; s[8] = Snu;

            double Fx = 0.0;
            double Fy = rho * gBeta * (T - Tref);
            if (ha) {  // SideHeatedHa (2DRB.F90:722-726)
                Fx = 0.0 + B2 * (v * sphi * cphi - u * sphi * sphi);
                Fy = rho * gBeta * (T - Tref) + rho * B2 * (u * sphi * cphi - v * cphi * cphi);
            }
            h->Fx[ci] = Fx;
            h->Fy[ci] = Fy;

            fSource[0] = 0.0;
            fSource[1] = (6.0 - 3.0 * s[1]) * (u * Fx + v * Fy);
            fSource[2] = -((6.0 - 3.0 * s[2]) * (u * Fx + v * Fy));
            fSource[3] = (1.0 - 0.5 * s[3]) * Fx;
            fSource[4] = -((1.0 - 0.5 * s[4]) * Fx);
            fSource[5] = (1.0 - 0.5 * s[5]) * Fy;
            fSource[6] = -((1.0 - 0.5 * s[6]) * Fy);
            fSource[7] = (2.0 - s[7]) * (u * Fx - v * Fy);
            fSource[8] = (1.0 - 0.5 * s[8]) * (u * Fy + v * Fx);

            for (int a = 0; a < 9; ++a) m_post[a] = m[a] - s[a] * (m[a] - meq[a]) + fSource[a];

            d2q9_inverse(m_post, FP);
        }
    }
}

static void streaming2d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny;
    const Lattice& L = h->L;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            size_t ci = h->C(i, j, 1);
            for (int a = 0; a < 9; ++a) h->f[a + 9 * ci] = h->fpost[a + 9 * h->P(i - L.ex[a], j - L.ey[a], 0)];
        }
}

static void bounceback2d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny;
    auto F = [h](int a, int i, int j) -> double& { return h->f[a + 9 * h->C(i, j, 1)]; };
    auto FP = [h](int a, int i, int j) -> double { return h->fpost[a + 9 * h->P(i, j, 0)]; };
    if (h->p.bc_flow[0] == LBM_BC_PERIODIC) {  // VerticalWallsPeriodicalU (2DRB.F90:816-831)
        for (int j = 1; j <= ny; ++j) {
            F(1, 1, j) = FP(1, nx, j);
            F(5, 1, j) = FP(5, nx, j);
            F(8, 1, j) = FP(8, nx, j);
            F(3, nx, j) = FP(3, 1, j);
            F(6, nx, j) = FP(6, 1, j);
            F(7, nx, j) = FP(7, 1, j);
        }
    }
    if (h->p.bc_flow[0] == LBM_BC_NOSLIP) {  // VerticalWallsNoslip (2DRB.F90:833-847)
        for (int j = 1; j <= ny; ++j) {
            F(1, 1, j) = FP(3, 1, j);
            F(5, 1, j) = FP(7, 1, j);
            F(8, 1, j) = FP(6, 1, j);
            F(3, nx, j) = FP(1, nx, j);
            F(6, nx, j) = FP(8, nx, j);
            F(7, nx, j) = FP(5, nx, j);
        }
    }
    // HorizontalWallsNoslip (2DRB.F90:849-863)
    for (int i = 1; i <= nx; ++i) {
        F(2, i, 1) = FP(4, i, 1);
        F(5, i, 1) = FP(7, i, 1);
        F(6, i, 1) = FP(8, i, 1);
        F(4, i, ny) = FP(2, i, ny);
        F(7, i, ny) = FP(5, i, ny);
        F(8, i, ny) = FP(6, i, ny);
    }
}

static void macro2d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            size_t ci = h->C(i, j, 1);
            const double* F = &h->f[9 * ci];
            double rho = F[0] + F[1] + F[2] + F[3] + F[4] + F[5] + F[6] + F[7] + F[8];
            h->rho[ci] = rho;
            h->u[ci] = (F[1] - F[3] + F[5] - F[6] - F[7] + F[8] + 0.5 * h->Fx[ci]) / rho;
            h->v[ci] = (F[2] - F[4] + F[5] + F[6] - F[7] - F[8] + 0.5 * h->Fy[ci]) / rho;
        }
}

static void collisionT2d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny;
    const lbm_constants& c = h->c;
    const bool useG = h->p.use_g != 0, legacy = h->p.legacy_thermal != 0;
    const double SG = c.SG, Qk = c.Qk, Qnu = c.Qnu, paraA = c.paraA;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j) {
        double n[5], n_post[5], neq[5], q[5];
        for (int i = 1; i <= nx; ++i) {
            size_t ci = h->C(i, j, 1);
            double u = h->u[ci], v = h->v[ci], T = h->T[ci];
            double Bx = u * T;
            double By = v * T;
            double dBx, dBy;
            if (useG) {
                dBx = Bx - h->Bx[ci];
                dBy = By - h->By[ci];
                h->Bx[ci] = Bx;
                h->By[ci] = By;
            } else {
                dBx = 0.0;
                dBy = 0.0;
            }
            const double* G = &h->g[5 * ci];
            double* GP = &h->gpost[5 * h->P(i, j, 0)];
            d2q5_forward(G, n);
            neq[0] = T;
            neq[1] = T * u;
            neq[2] = T * v;
            neq[3] = legacy ? T * paraA : T * (-2.0 / 3.0);
            neq[4] = 0.0;
            q[0] = 0.0; q[1] = Qk; q[2] = Qk; q[3] = Qnu; q[4] = Qnu;
            n_post[0] = n[0] - q[0] * (n[0] - neq[0]);
            n_post[1] = n[1] - q[1] * (n[1] - neq[1]) + SG * dBx;
            n_post[2] = n[2] - q[2] * (n[2] - neq[2]) + SG * dBy;
            n_post[3] = n[3] - q[3] * (n[3] - neq[3]);
            n_post[4] = n[4] - q[4] * (n[4] - neq[4]);
            d2q5_inverse(n_post, GP);
        }
    }
}

static void streamingT2d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny;
    const Lattice& L = h->L;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            size_t ci = h->C(i, j, 1);
            for (int a = 0; a < 5; ++a) h->g[a + 5 * ci] = h->gpost[a + 5 * h->P(i - L.ex[a], j - L.ey[a], 0)];
        }
}

static void bouncebackT2d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny;
    const lbm_constants& c = h->c;
    const double Thot = h->p.Thot, Tcold = h->p.Tcold;
    const bool legacy = h->p.legacy_thermal != 0;
    const double* omegaT = h->L.omegaT;
    auto G = [h](int a, int i, int j) -> double& { return h->g[a + 5 * h->C(i, j, 1)]; };
    auto GP = [h](int a, int i, int j) -> double { return h->gpost[a + 5 * h->P(i, j, 0)]; };
    const int bx = h->p.bc_thermal[0], by = h->p.bc_thermal[1];
    if (bx == LBM_BCT_PERIODIC)  // 2DRB.F90:1031-1042
        for (int j = 1; j <= ny; ++j) {
            G(1, 1, j) = GP(1, nx, j);
            G(3, nx, j) = GP(3, 1, j);
        }
    if (bx == LBM_BCT_CONST)  // 2DRB.F90:1044-1062
        for (int j = 1; j <= ny; ++j) {
            if (legacy) {
                G(1, 1, j) = -GP(3, 1, j) + (4.0 + c.paraA) / 10.0 * Thot;
                G(3, nx, j) = -GP(1, nx, j) + (4.0 + c.paraA) / 10.0 * Tcold;
            } else {
                G(1, 1, j) = -GP(3, 1, j) + 2.0 * omegaT[3] * Thot;
                G(3, nx, j) = -GP(1, nx, j) + 2.0 * omegaT[1] * Tcold;
            }
        }
    if (bx == LBM_BCT_ADIABATIC)  // 2DRB.F90:1064-1073
        for (int j = 1; j <= ny; ++j) {
            G(1, 1, j) = GP(3, 1, j);
            G(3, nx, j) = GP(1, nx, j);
        }
    if (by == LBM_BCT_ADIABATIC)  // 2DRB.F90:1075-1084
        for (int i = 1; i <= nx; ++i) {
            G(2, i, 1) = GP(4, i, 1);
            G(4, i, ny) = GP(2, i, ny);
        }
    if (by == LBM_BCT_CONST)  // 2DRB.F90:1086-1104
        for (int i = 1; i <= nx; ++i) {
            if (legacy) {
                G(2, i, 1) = -GP(4, i, 1) + (4.0 + c.paraA) / 10.0 * Thot;
                G(4, i, ny) = -GP(2, i, ny) + (4.0 + c.paraA) / 10.0 * Tcold;
            } else {
                G(2, i, 1) = -GP(4, i, 1) + 2.0 * omegaT[4] * Thot;
                G(4, i, ny) = -GP(2, i, ny) + 2.0 * omegaT[2] * Tcold;
            }
        }
}

static void macroT2d(ora_handle* h) {
#pragma omp parallel for schedule(static)
    for (long long ci = 0; ci < (long long)h->ncell; ++ci) {
        const double* G = &h->g[5 * ci];
        h->T[ci] = G[0] + G[1] + G[2] + G[3] + G[4];
    }
}

// ------------------------------------------------------------------------------------
// 3D stages (3DRB.F90:689-1381)
// ------------------------------------------------------------------------------------
static void collision3d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const lbm_constants& c = h->c;
    const double gBeta = c.gBeta, Tref = c.Tref;
    double s[19];
    s[0] = 0.0;   s[1] = c.Se;   s[2] = c.Seps; s[3] = 0.0;   s[4] = c.Sq;
    s[5] = 0.0;   s[6] = c.Sq;   s[7] = 0.0;    s[8] = c.Sq;  s[9] = c.Snu;
    s[10] = c.Spi; s[11] = c.Snu; s[12] = c.Spi; s[13] = c.Snu; s[14] = c.Snu;
    s[15] = c.Snu; s[16] = c.Sm; s[17] = c.Sm; s[18] = c.Sm;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j) {
            double m[19], meq[19], m_post[19], fSource[19];
            for (int i = 1; i <= nx; ++i) {
                size_t ci = h->C(i, j, k);
                const double* f = &h->f[19 * ci];
                double* fp = &h->fpost[19 * h->P(i, j, k)];
                double rhoLoc = h->rho[ci], uLoc = h->u[ci], vLoc = h->v[ci], wLoc = h->w[ci];
                double u2 = uLoc * uLoc + vLoc * vLoc + wLoc * wLoc;

                d3q19_forward(f, m);

                meq[0] = rhoLoc;
                meq[1] = rhoLoc * (-11.0 + 19.0 * u2);
                meq[2] = rhoLoc * (3.0 - 11.0 * u2 / 2.0);
                meq[3] = rhoLoc * uLoc;
                meq[4] = -2.0 * rhoLoc * uLoc / 3.0;
                meq[5] = rhoLoc * vLoc;
                meq[6] = -2.0 * rhoLoc * vLoc / 3.0;
                meq[7] = rhoLoc * wLoc;
                meq[8] = -2.0 * rhoLoc * wLoc / 3.0;
                meq[9] = rhoLoc * (2.0 * uLoc * uLoc - vLoc * vLoc - wLoc * wLoc);
                meq[10] = -0.5 * meq[9];
                meq[11] = rhoLoc * (vLoc * vLoc - wLoc * wLoc);
                meq[12] = -0.5 * meq[11];
                meq[13] = rhoLoc * uLoc * vLoc;
                meq[14] = rhoLoc * vLoc * wLoc;
                meq[15] = rhoLoc * uLoc * wLoc;
                meq[16] = 0.0;
                meq[17] = 0.0;
                meq[18] = 0.0;

                double FxLoc = 0.0;
                double FyLoc = rhoLoc * gBeta * (h->T[ci] - Tref);
                double FzLoc = 0.0;
                double uDotF = uLoc * FxLoc + vLoc * FyLoc + wLoc * FzLoc;

                fSource[0] = 0.0;
                fSource[1] = (1.0 - 0.5 * s[1]) * 38.0 * uDotF;
                fSource[2] = (1.0 - 0.5 * s[2]) * (-11.0) * uDotF;
                fSource[3] = (1.0 - 0.5 * s[3]) * FxLoc;
                fSource[4] = (1.0 - 0.5 * s[4]) * (-2.0 / 3.0) * FxLoc;
                fSource[5] = (1.0 - 0.5 * s[5]) * FyLoc;
                fSource[6] = (1.0 - 0.5 * s[6]) * (-2.0 / 3.0) * FyLoc;
                fSource[7] = (1.0 - 0.5 * s[7]) * FzLoc;
                fSource[8] = (1.0 - 0.5 * s[8]) * (-2.0 / 3.0) * FzLoc;
                fSource[9] = (1.0 - 0.5 * s[9]) * (4.0 * uLoc * FxLoc - 2.0 * vLoc * FyLoc - 2.0 * wLoc * FzLoc);
                fSource[10] = (1.0 - 0.5 * s[10]) * (-2.0 * uLoc * FxLoc + vLoc * FyLoc + wLoc * FzLoc);
                fSource[11] = (1.0 - 0.5 * s[11]) * (2.0 * vLoc * FyLoc - 2.0 * wLoc * FzLoc);
                fSource[12] = (1.0 - 0.5 * s[12]) * (-(vLoc * FyLoc) + wLoc * FzLoc);
                fSource[13] = (1.0 - 0.5 * s[13]) * (uLoc * FyLoc + vLoc * FxLoc);
                fSource[14] = (1.0 - 0.5 * s[14]) * (vLoc * FzLoc + wLoc * FyLoc);
                fSource[15] = (1.0 - 0.5 * s[15]) * (uLoc * FzLoc + wLoc * FxLoc);
                fSource[16] = 0.0;
                fSource[17] = 0.0;
                fSource[18] = 0.0;

                for (int a = 0; a < 19; ++a) m_post[a] = m[a] - s[a] * (m[a] - meq[a]) + fSource[a];

                d3q19_inverse(m_post, fp);
            }
        }
}

static void streaming3d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const Lattice& L = h->L;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                size_t ci = h->C(i, j, k);
                for (int a = 0; a < 19; ++a)
                    h->f[a + 19 * ci] = h->fpost[a + 19 * h->P(i - L.ex[a], j - L.ey[a], k - L.ez[a])];
            }
}

static void bounceback3d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const Lattice& L = h->L;
    auto F = [h](int a, int i, int j, int k) -> double& { return h->f[a + 19 * h->C(i, j, k)]; };
    auto FP = [h](int a, int i, int j, int k) -> double { return h->fpost[a + 19 * h->P(i, j, k)]; };
    if (h->p.bc_flow[0] == LBM_BC_PERIODIC)  // 3DRB.F90:992-1002
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int a = 0; a < 19; ++a) {
                    if (L.ex[a] == 1) F(a, 1, j, k) = FP(a, nx, j, k);
                    if (L.ex[a] == -1) F(a, nx, j, k) = FP(a, 1, j, k);
                }
    if (h->p.bc_flow[0] == LBM_BC_NOSLIP)  // 3DRB.F90:1005-1015
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int a = 0; a < 19; ++a) {
                    if (L.ex[a] == 1) F(a, 1, j, k) = FP(L.opp[a], 1, j, k);
                    if (L.ex[a] == -1) F(a, nx, j, k) = FP(L.opp[a], nx, j, k);
                }
    // HorizontalWallsNoslip (3DRB.F90:1018-1028)
    for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i)
            for (int a = 0; a < 19; ++a) {
                if (L.ey[a] == 1) F(a, i, 1, k) = FP(L.opp[a], i, 1, k);
                if (L.ey[a] == -1) F(a, i, ny, k) = FP(L.opp[a], i, ny, k);
            }
    if (h->p.bc_flow[2] == LBM_BC_PERIODIC)  // 3DRB.F90:1031-1041
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i)
                for (int a = 0; a < 19; ++a) {
                    if (L.ez[a] == 1) F(a, i, j, 1) = FP(a, i, j, nz);
                    if (L.ez[a] == -1) F(a, i, j, nz) = FP(a, i, j, 1);
                }
    if (h->p.bc_flow[2] == LBM_BC_NOSLIP)  // 3DRB.F90:1044-1054
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i)
                for (int a = 0; a < 19; ++a) {
                    if (L.ez[a] == 1) F(a, i, j, 1) = FP(L.opp[a], i, j, 1);
                    if (L.ez[a] == -1) F(a, i, j, nz) = FP(L.opp[a], i, j, nz);
                }
}

static void macro3d(ora_handle* h) {
    const double gBeta = h->c.gBeta, Tref = h->c.Tref;
#pragma omp parallel for schedule(static)
    for (long long ci = 0; ci < (long long)h->ncell; ++ci) {
        const double* f = &h->f[19 * ci];
        double rho = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8] + f[9] + f[10] + f[11] + f[12]
                     + f[13] + f[14] + f[15] + f[16] + f[17] + f[18];
        h->rho[ci] = rho;
        double FyLoc = rho * gBeta * (h->T[ci] - Tref);
        h->u[ci] = (f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14]) / rho;
        h->v[ci] = (f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18] + 0.5 * FyLoc) / rho;
        h->w[ci] = (f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18]) / rho;
    }
}

static void collisionT3d(ora_handle* h) {
    const lbm_constants& c = h->c;
    const bool useG = h->p.use_g != 0, legacy = h->p.legacy_thermal != 0;
    const double SG = c.SG, Qk = c.Qk, Qnu = c.Qnu, paraA = c.paraA;
    const int nx = h->nx, ny = h->ny, nz = h->nz;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j) {
            double n[7], neq[7], q[7], n_post[7];
            for (int i = 1; i <= nx; ++i) {
                size_t ci = h->C(i, j, k);
                double u = h->u[ci], v = h->v[ci], w = h->w[ci], T = h->T[ci];
                double Bx = u * T, By = v * T, Bz = w * T;
                double dBx, dBy, dBz;
                if (useG) {
                    dBx = Bx - h->Bx[ci];
                    dBy = By - h->By[ci];
                    dBz = Bz - h->Bz[ci];
                    h->Bx[ci] = Bx;
                    h->By[ci] = By;
                    h->Bz[ci] = Bz;
                } else {
                    dBx = 0.0;
                    dBy = 0.0;
                    dBz = 0.0;
                }
                const double* g = &h->g[7 * ci];
                double* gp = &h->gpost[7 * h->P(i, j, k)];
                d3q7_forward(g, n);
                neq[0] = T;
                neq[1] = Bx;
                neq[2] = By;
                neq[3] = Bz;
                neq[4] = legacy ? paraA * T : -0.75 * T;
                neq[5] = 0.0;
                neq[6] = 0.0;
                q[0] = 0.0; q[1] = Qk; q[2] = Qk; q[3] = Qk; q[4] = Qnu; q[5] = Qnu; q[6] = Qnu;
                n_post[0] = n[0] - q[0] * (n[0] - neq[0]);
                n_post[1] = n[1] - q[1] * (n[1] - neq[1]) + SG * dBx;
                n_post[2] = n[2] - q[2] * (n[2] - neq[2]) + SG * dBy;
                n_post[3] = n[3] - q[3] * (n[3] - neq[3]) + SG * dBz;
                n_post[4] = n[4] - q[4] * (n[4] - neq[4]);
                n_post[5] = n[5] - q[5] * (n[5] - neq[5]);
                n_post[6] = n[6] - q[6] * (n[6] - neq[6]);
                d3q7_inverse(n_post, gp);
            }
        }
}

static void streamingT3d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const Lattice& L = h->L;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                size_t ci = h->C(i, j, k);
                for (int a = 0; a < 7; ++a)
                    h->g[a + 7 * ci] = h->gpost[a + 7 * h->P(i - L.exT[a], j - L.eyT[a], k - L.ezT[a])];
            }
}

static void bouncebackT3d(ora_handle* h) {
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const Lattice& L = h->L;
    const lbm_constants& c = h->c;
    const double Thot = h->p.Thot, Tcold = h->p.Tcold;
    const bool legacy = h->p.legacy_thermal != 0;
    auto G = [h](int a, int i, int j, int k) -> double& { return h->g[a + 7 * h->C(i, j, k)]; };
    auto GP = [h](int a, int i, int j, int k) -> double { return h->gpost[a + 7 * h->P(i, j, k)]; };
    const int bx = h->p.bc_thermal[0], by = h->p.bc_thermal[1], bz = h->p.bc_thermal[2];
    if (bx == LBM_BCT_PERIODIC)  // 3DRB.F90:1248-1258
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int a = 0; a < 7; ++a) {
                    if (L.exT[a] == 1) G(a, 1, j, k) = GP(a, nx, j, k);
                    if (L.exT[a] == -1) G(a, nx, j, k) = GP(a, 1, j, k);
                }
    if (bx == LBM_BCT_CONST)  // 3DRB.F90:1261-1276
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int a = 0; a < 7; ++a) {
                    if (legacy) {
                        if (L.exT[a] == 1) G(a, 1, j, k) = -GP(L.oppT[a], 1, j, k) + (6.0 + c.paraA) / 21.0 * Thot;
                        if (L.exT[a] == -1) G(a, nx, j, k) = -GP(L.oppT[a], nx, j, k) + (6.0 + c.paraA) / 21.0 * Tcold;
                    } else {
                        if (L.exT[a] == 1) G(a, 1, j, k) = -GP(L.oppT[a], 1, j, k) + 2.0 * L.omegaT[a] * Thot;
                        if (L.exT[a] == -1) G(a, nx, j, k) = -GP(L.oppT[a], nx, j, k) + 2.0 * L.omegaT[a] * Tcold;
                    }
                }
    if (bx == LBM_BCT_ADIABATIC)  // 3DRB.F90:1279-1289
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int a = 0; a < 7; ++a) {
                    if (L.exT[a] == 1) G(a, 1, j, k) = GP(L.oppT[a], 1, j, k);
                    if (L.exT[a] == -1) G(a, nx, j, k) = GP(L.oppT[a], nx, j, k);
                }
    if (by == LBM_BCT_ADIABATIC)  // 3DRB.F90:1292-1302
        for (int k = 1; k <= nz; ++k)
            for (int i = 1; i <= nx; ++i)
                for (int a = 0; a < 7; ++a) {
                    if (L.eyT[a] == 1) G(a, i, 1, k) = GP(L.oppT[a], i, 1, k);
                    if (L.eyT[a] == -1) G(a, i, ny, k) = GP(L.oppT[a], i, ny, k);
                }
    if (by == LBM_BCT_CONST)  // 3DRB.F90:1305-1320
        for (int k = 1; k <= nz; ++k)
            for (int i = 1; i <= nx; ++i)
                for (int a = 0; a < 7; ++a) {
                    if (legacy) {
                        if (L.eyT[a] == 1) G(a, i, 1, k) = -GP(L.oppT[a], i, 1, k) + (6.0 + c.paraA) / 21.0 * Thot;
                        if (L.eyT[a] == -1) G(a, i, ny, k) = -GP(L.oppT[a], i, ny, k) + (6.0 + c.paraA) / 21.0 * Tcold;
                    } else {
                        if (L.eyT[a] == 1) G(a, i, 1, k) = -GP(L.oppT[a], i, 1, k) + 2.0 * L.omegaT[a] * Thot;
                        if (L.eyT[a] == -1) G(a, i, ny, k) = -GP(L.oppT[a], i, ny, k) + 2.0 * L.omegaT[a] * Tcold;
                    }
                }
    if (bz == LBM_BCT_PERIODIC)  // 3DRB.F90:1323-1333
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i)
                for (int a = 0; a < 7; ++a) {
                    if (L.ezT[a] == 1) G(a, i, j, 1) = GP(a, i, j, nz);
                    if (L.ezT[a] == -1) G(a, i, j, nz) = GP(a, i, j, 1);
                }
    if (bz == LBM_BCT_ADIABATIC)  // 3DRB.F90:1336-1346
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i)
                for (int a = 0; a < 7; ++a) {
                    if (L.ezT[a] == 1) G(a, i, j, 1) = GP(L.oppT[a], i, j, 1);
                    if (L.ezT[a] == -1) G(a, i, j, nz) = GP(L.oppT[a], i, j, nz);
                }
}

static void macroT3d(ora_handle* h) {
#pragma omp parallel for schedule(static)
    for (long long ci = 0; ci < (long long)h->ncell; ++ci) {
        const double* g = &h->g[7 * ci];
        h->T[ci] = g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6];
    }
}

// ------------------------------------------------------------------------------------
// public stage entry points
// ------------------------------------------------------------------------------------
extern "C" void ora_collision(ora_handle* h) { h->d3 ? collision3d(h) : collision2d(h); }
extern "C" void ora_streaming(ora_handle* h) { h->d3 ? streaming3d(h) : streaming2d(h); }
extern "C" void ora_bounceback(ora_handle* h) { h->d3 ? bounceback3d(h) : bounceback2d(h); }
extern "C" void ora_macro(ora_handle* h) { h->d3 ? macro3d(h) : macro2d(h); }
extern "C" void ora_collisionT(ora_handle* h) { h->d3 ? collisionT3d(h) : collisionT2d(h); }
extern "C" void ora_streamingT(ora_handle* h) { h->d3 ? streamingT3d(h) : streamingT2d(h); }
extern "C" void ora_bouncebackT(ora_handle* h) { h->d3 ? bouncebackT3d(h) : bouncebackT2d(h); }
extern "C" void ora_macroT(ora_handle* h) { h->d3 ? macroT3d(h) : macroT2d(h); }

// ------------------------------------------------------------------------------------
// restart: reconstruct_macro_from_fg (2DRB.F90:1144-1200, 3DRB.F90:1392-1463), called by
// initial after loadInitField = 1 has read f and g (2DRB.F90:621-637, 3DRB.F90:602-623);
// initial then zeroes up, vp, wp, Tp (steadyFlow, 3DRB.F90:627-632) and the time loop
// starts from itc = 0.  The three fixed-point iterations of the reference do not depend
// on u, so one pass gives the same values.  Returns 1 if some cell had rho <= 0 (the
// reference stops there), else 0.
// ------------------------------------------------------------------------------------
extern "C" int ora_reconstruct_macro_from_fg(ora_handle* h) {
    ora_macroT(h);
    const double gBeta = h->c.gBeta, Tref = h->c.Tref;
    const bool useG = h->p.use_g != 0;
    const bool ha = h->p.side_heated_ha != 0;
    const double B2 = h->c.B2sigemarho, sphi = h->c.sinphi, cphi = h->c.cosphi;
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (long long ci = 0; ci < (long long)h->ncell; ++ci) {
        const double T = h->T[ci];
        if (h->d3) {
            const double* f = &h->f[19 * ci];
            const double rho = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8] + f[9] + f[10] + f[11]
                               + f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18];
            const double momx = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
            const double momy = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
            const double momz = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
            h->rho[ci] = rho;
            double u = 0.0, v = 0.0, w = 0.0;
            if (rho > 0.0) {
                const double FxLoc = 0.0, FyLoc = rho * gBeta * (T - Tref), FzLoc = 0.0;
                u = (momx + 0.5 * FxLoc) / rho;
                v = (momy + 0.5 * FyLoc) / rho;
                w = (momz + 0.5 * FzLoc) / rho;
            } else {
                bad = 1;
            }
            h->u[ci] = u;
            h->v[ci] = v;
            h->w[ci] = w;
            h->Bx[ci] = useG ? u * T : 0.0;
            h->By[ci] = useG ? v * T : 0.0;
            h->Bz[ci] = useG ? w * T : 0.0;
        } else {
            const double* f = &h->f[9 * ci];
            const double rho = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8];
            const double momx = f[1] - f[3] + f[5] - f[6] - f[7] + f[8];
            const double momy = f[2] - f[4] + f[5] + f[6] - f[7] - f[8];
            h->rho[ci] = rho;
            double u = 0.0, v = 0.0, Fx = 0.0, Fy = 0.0;
            if (rho > 0.0) {
                u = momx / rho;
                v = momy / rho;
                for (int iter = 1; iter <= 3; ++iter) {  // 2DRB.F90:1165-1177
                    Fx = 0.0;
                    Fy = rho * gBeta * (T - Tref);
                    if (ha) {
                        Fx = B2 * (v * sphi * cphi - u * sphi * sphi);
                        Fy = rho * gBeta * (T - Tref) + rho * B2 * (u * sphi * cphi - v * cphi * cphi);
                    }
                    u = (momx + 0.5 * Fx) / rho;
                    v = (momy + 0.5 * Fy) / rho;
                }
            } else {
                bad = 1;
            }
            h->u[ci] = u;
            h->v[ci] = v;
            h->Fx[ci] = Fx;
            h->Fy[ci] = Fy;
            if (useG) {  // 2DRB.F90:1189-1192: without EnableUseG B_prev is left as it is
                h->Bx[ci] = u * T;
                h->By[ci] = v * T;
            }
        }
    }
    std::fill(h->up.begin(), h->up.end(), 0.0);
    std::fill(h->vp.begin(), h->vp.end(), 0.0);
    std::fill(h->wp.begin(), h->wp.end(), 0.0);
    std::fill(h->Tp.begin(), h->Tp.end(), 0.0);
    h->itc = 0;
    return bad;
}

extern "C" void ora_step(ora_handle* h, long long nsteps) {
    for (long long s = 0; s < nsteps; ++s) {
        h->itc += 1;
        ora_collision(h);
        ora_streaming(h);
        ora_bounceback(h);
        ora_macro(h);
        ora_collisionT(h);
        ora_streamingT(h);
        ora_bouncebackT(h);
        ora_macroT(h);
    }
}

// ------------------------------------------------------------------------------------
// diagnostics
// ------------------------------------------------------------------------------------
// check (2DRB.F90:1213-1260, 3DRB.F90:1475-1528)
extern "C" int ora_check(ora_handle* h, double* errU, double* errT) {
    double error1 = 0.0, error2 = 0.0, error5 = 0.0, error6 = 0.0;
    for (size_t ci = 0; ci < h->ncell; ++ci) {
        double du = h->u[ci] - h->up[ci], dv = h->v[ci] - h->vp[ci];
        if (h->d3) {
            double dw = h->w[ci] - h->wp[ci];
            error1 = error1 + du * du + dv * dv + dw * dw;
            error2 = error2 + h->u[ci] * h->u[ci] + h->v[ci] * h->v[ci] + h->w[ci] * h->w[ci];
            h->wp[ci] = h->w[ci];
        } else {
            error1 = error1 + du * du + dv * dv;
            error2 = error2 + h->u[ci] * h->u[ci] + h->v[ci] * h->v[ci];
        }
        error5 = error5 + std::fabs(h->T[ci] - h->Tp[ci]);
        error6 = error6 + std::fabs(h->T[ci]);
        h->up[ci] = h->u[ci];
        h->vp[ci] = h->v[ci];
        h->Tp[ci] = h->T[ci];
    }
    if (h->d3) {
        *errU = (error2 > 1.0e-30) ? std::sqrt(error1) / std::sqrt(error2) : std::sqrt(error1);
        *errT = (error6 > 1.0e-30) ? error5 / error6 : error5;
    } else {
        *errU = std::sqrt(error1) / std::sqrt(error2);
        *errT = error5 / error6;
    }
    return (std::isfinite(error1) && std::isfinite(error5)) ? LBM_OK : LBM_ERR_DIVERGED;
}

// calNuRe (2DRB.F90:1610-1675, 3DRB.F90:1712-1778)
extern "C" int ora_calNuRe(ora_handle* h, double* Nu, double* Re) {
    const lbm_constants& c = h->c;
    const std::vector<double>& ucomp = (h->p.cell == LBM_CELL_SIDE) ? h->u : h->v;
    double s = 0.0;
    for (size_t ci = 0; ci < h->ncell; ++ci) s = s + ucomp[ci] * h->T[ci];
    double ncell = (double)(long long)h->ncell;
    *Nu = s / ncell * c.lengthUnit / c.diffusivity + 1.0;
    double r = 0.0;
    for (size_t ci = 0; ci < h->ncell; ++ci) {
        if (h->d3)
            r = r + h->u[ci] * h->u[ci] + h->v[ci] * h->v[ci] + h->w[ci] * h->w[ci];
        else
            r = r + (h->u[ci] * h->u[ci] + h->v[ci] * h->v[ci]);
    }
    *Re = std::sqrt(r / ncell) * c.lengthUnit / c.viscosity;
    return (std::isfinite(*Nu) && std::isfinite(*Re)) ? LBM_OK : LBM_ERR_DIVERGED;
}

// RBcalc_Nu_global (2DRB.F90:2251-2297, 3DRB.F90:1839-1878)
extern "C" int ora_RBcalc_Nu_global(ora_handle* h, double* Nu) {
    const lbm_constants& c = h->c;
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const double dy = 1.0 / c.lengthUnit;
    const double deltaT = h->p.Thot - h->p.Tcold;
    const double coef = c.velocityScaleCompare;
    const double Thot = h->p.Thot, Tcold = h->p.Tcold, Tref = c.Tref;
    double sum_qy = 0.0;
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                auto T = [h, i, k](int jj) { return h->T[h->C(i, jj, k)]; };
                double dTdy;
                if (j == 1)
                    dTdy = (3.0 * T(1) + T(2) - 4.0 * Thot) / (3.0 * dy);
                else if (j == ny)
                    dTdy = (4.0 * Tcold - 3.0 * T(ny) - T(ny - 1)) / (3.0 * dy);
                else
                    dTdy = (T(j + 1) - T(j - 1)) / (2.0 * dy);
                double qy = coef * h->v[h->C(i, j, k)] * (T(j) - Tref) - dTdy;
                sum_qy = sum_qy + qy;
            }
    *Nu = (sum_qy / (double)(long long)h->ncell) / deltaT;
    return std::isfinite(*Nu) ? LBM_OK : LBM_ERR_DIVERGED;
}

// fit_adiabatic_wall_T4 (2DRB.F90:1953-1991; identical in 3DRB.F90)
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
    double D = S0 * S2 - S1 * S1;
    return (B0 * S2 - B1 * S1) / D;
}

// fit_parabola_ls5, 2D form (2DRB.F90:1999-2080): quadratic coefficient first.
static void fit_parabola_ls5_2d(const double y[5], const double f[5], int mode, double* fstar, double* ystar) {
    const double epsD = 1.0e-20, epsA = 1.0e-14;
    int kbest = 0;
    for (int k = 1; k < 5; ++k) {
        if (mode == 1) {
            if (f[k] > f[kbest]) kbest = k;
        } else {
            if (f[k] < f[kbest]) kbest = k;
        }
    }
    double S0 = 0, S1 = 0, S2 = 0, S3 = 0, S4 = 0, F0 = 0, F1 = 0, F2 = 0;
    for (int k = 0; k < 5; ++k) {
        S0 = S0 + 1.0;
        S1 = S1 + y[k];
        S2 = S2 + y[k] * y[k];
        S3 = S3 + y[k] * y[k] * y[k];
        S4 = S4 + y[k] * y[k] * y[k] * y[k];
        F0 = F0 + f[k];
        F1 = F1 + y[k] * f[k];
        F2 = F2 + y[k] * y[k] * f[k];
    }
    double D = S4 * (S2 * S0 - S1 * S1) - S3 * (S3 * S0 - S1 * S2) + S2 * (S3 * S1 - S2 * S2);
    double DA = F2 * (S2 * S0 - S1 * S1) - S3 * (F1 * S0 - S1 * F0) + S2 * (F1 * S1 - S2 * F0);
    double DB = S4 * (F1 * S0 - S1 * F0) - F2 * (S3 * S0 - S1 * S2) + S2 * (S3 * F0 - F1 * S2);
    double DC = S4 * (S2 * F0 - F1 * S1) - S3 * (S3 * F0 - F1 * S2) + F2 * (S3 * S1 - S2 * S2);
    if (std::fabs(D) > epsD) {
        double A = DA / D, B = DB / D, Cc = DC / D;
        if (std::fabs(A) > epsA) {
            double ys = -B / (2.0 * A);
            double ymin = y[0], ymax = y[0];
            for (int k = 1; k < 5; ++k) {
                ymin = std::min(ymin, y[k]);
                ymax = std::max(ymax, y[k]);
            }
            if (ys >= ymin && ys <= ymax) {
                *ystar = ys;
                *fstar = Cc - B * B / (4.0 * A);
            } else {
                *ystar = y[kbest];
                *fstar = f[kbest];
            }
            return;
        }
    }
    *ystar = y[kbest];
    *fstar = f[kbest];
}

// fit_parabola_ls5, 3D form (3DRB.F90:2257-2334): constant coefficient first.
static void fit_parabola_ls5_3d(const double y[5], const double f[5], int mode, double* fstar, double* ystar) {
    const double epsD = 1.0e-20, epsA = 1.0e-14;
    int kbest = 0;
    for (int k = 1; k < 5; ++k) {
        if (mode == 1) {
            if (f[k] > f[kbest]) kbest = k;
        } else {
            if (f[k] < f[kbest]) kbest = k;
        }
    }
    double S0 = 0, S1 = 0, S2 = 0, S3 = 0, S4 = 0, F0 = 0, F1 = 0, F2 = 0;
    for (int k = 0; k < 5; ++k) {
        S0 = S0 + 1.0;
        S1 = S1 + y[k];
        S2 = S2 + y[k] * y[k];
        S3 = S3 + y[k] * y[k] * y[k];
        S4 = S4 + y[k] * y[k] * y[k] * y[k];
        F0 = F0 + f[k];
        F1 = F1 + f[k] * y[k];
        F2 = F2 + f[k] * y[k] * y[k];
    }
    double D = S0 * (S2 * S4 - S3 * S3) - S1 * (S1 * S4 - S2 * S3) + S2 * (S1 * S3 - S2 * S2);
    double DA = F0 * (S2 * S4 - S3 * S3) - S1 * (F1 * S4 - S3 * F2) + S2 * (F1 * S3 - S2 * F2);
    double DB = S0 * (F1 * S4 - S3 * F2) - F0 * (S1 * S4 - S2 * S3) + S2 * (S1 * F2 - F1 * S2);
    double DC = S0 * (S2 * F2 - F1 * S3) - S1 * (S1 * F2 - F1 * S2) + F0 * (S1 * S3 - S2 * S2);
    if (std::fabs(D) <= epsD) {
        *ystar = y[kbest];
        *fstar = f[kbest];
        return;
    }
    double A = DA / D, B = DB / D, Cq = DC / D;
    double ymin = y[0], ymax = y[0];
    for (int k = 1; k < 5; ++k) {
        ymin = std::min(ymin, y[k]);
        ymax = std::max(ymax, y[k]);
    }
    if (std::fabs(Cq) <= epsA || (mode == 1 && Cq >= 0.0) || (mode == -1 && Cq <= 0.0)) {
        *ystar = y[kbest];
        *fstar = f[kbest];
        return;
    }
    double ys = -B / (2.0 * Cq);
    if (ys < ymin || ys > ymax) {
        *ystar = y[kbest];
        *fstar = f[kbest];
        return;
    }
    *ystar = ys;
    *fstar = A + B * ys + Cq * ys * ys;
}

// RBcalc_Nu_wall_avg (2DRB.F90:2308-2473, 3DRB.F90:2049-2210)
extern "C" int ora_RBcalc_Nu_wall_avg(ora_handle* h, lbm_nu_wall* out) {
    const lbm_constants& c = h->c;
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const double dy = 1.0 / c.lengthUnit;
    const double deltaT = h->p.Thot - h->p.Tcold;
    const double Thot = h->p.Thot, Tcold = h->p.Tcold, Tref = c.Tref;
    const double coef = h->d3 ? c.heatFluxScale : c.velocityScaleCompare;
    const std::vector<double>& xp = h->xp;
    auto T = [h](int i, int j, int k) { return h->T[h->C(i, j, k)]; };
    auto V = [h](int i, int j, int k) { return h->v[h->C(i, j, k)]; };
    std::vector<double> Nu_bot(nx + 2, 0.0), Tb(nx + 2, 0.0);
    double sum_hot = 0.0;
    for (int i = 1; i <= nx; ++i) {
        if (h->d3) {
            double tb = 0.0;
            for (int k = 1; k <= nz; ++k) tb = tb + T(i, 1, k);
            Tb[i] = tb / (double)nz;
            double nb = 0.0;
            for (int k = 1; k <= nz; ++k) {
                double qy_wall = (8.0 * Thot - 9.0 * T(i, 1, k) + T(i, 2, k)) / (3.0 * dy);
                nb = nb + qy_wall / deltaT;
            }
            Nu_bot[i] = nb / (double)nz;
        } else {
            Tb[i] = T(i, 1, 1);
            double qy_wall = (8.0 * Thot - 9.0 * T(i, 1, 1) + T(i, 2, 1)) / (3.0 * dy);
            Nu_bot[i] = qy_wall / deltaT;
        }
        sum_hot = sum_hot + Nu_bot[i];
    }
    out->Nu_hot = sum_hot / (double)nx;
    double xfit[4], Tfit[4];
    for (int m = 0; m < 4; ++m) { xfit[m] = xp[1 + m]; Tfit[m] = Tb[1 + m]; }
    double T_wl = fit_adiabatic_wall_T4(0.0, xfit, Tfit);
    for (int m = 0; m < 4; ++m) { xfit[m] = xp[nx - 3 + m]; Tfit[m] = Tb[nx - 3 + m]; }
    double T_wr = fit_adiabatic_wall_T4(xp[nx + 1], xfit, Tfit);
    std::vector<double> ext(Nu_bot);
    ext[0] = (2.0 * (Thot - T_wl) / dy) / deltaT;
    ext[nx + 1] = (2.0 * (Thot - T_wr) / dy) / deltaT;
    int imax = 0, imin = 0;
    double vmax = ext[0], vmin = ext[0];
    for (int i = 1; i <= nx + 1; ++i) {
        if (ext[i] > vmax) { vmax = ext[i]; imax = i; }
        if (ext[i] < vmin) { vmin = ext[i]; imin = i; }
    }
    auto pick = [nx](int ic, int ii[5]) {
        if (ic <= 2) { for (int m = 0; m < 5; ++m) ii[m] = m; }
        else if (ic >= nx - 1) { for (int m = 0; m < 5; ++m) ii[m] = nx - 3 + m; }
        else { for (int m = 0; m < 5; ++m) ii[m] = ic - 2 + m; }
    };
    int ii[5];
    double xk[5], fk[5], fstar, xstar;
    pick(imax, ii);
    for (int m = 0; m < 5; ++m) { xk[m] = xp[ii[m]]; fk[m] = ext[ii[m]]; }
    if (h->d3) fit_parabola_ls5_3d(xk, fk, +1, &fstar, &xstar); else fit_parabola_ls5_2d(xk, fk, +1, &fstar, &xstar);
    out->Nu_hot_max = fstar;
    out->Nu_hot_max_position = xstar;
    pick(imin, ii);
    for (int m = 0; m < 5; ++m) { xk[m] = xp[ii[m]]; fk[m] = ext[ii[m]]; }
    if (h->d3) fit_parabola_ls5_3d(xk, fk, -1, &fstar, &xstar); else fit_parabola_ls5_2d(xk, fk, -1, &fstar, &xstar);
    out->Nu_hot_min = fstar;
    out->Nu_hot_min_position = xstar;

    double sum_cold = 0.0;
    for (int i = 1; i <= nx; ++i)
        for (int k = 1; k <= nz; ++k) {
            double qy_wall = (-8.0 * Tcold + 9.0 * T(i, ny, k) - T(i, ny - 1, k)) / (3.0 * dy);
            sum_cold = sum_cold + qy_wall / deltaT;
        }
    out->Nu_cold = sum_cold / (double)(nx * nz);

    double sum_mid = 0.0;
    if (ny % 2 == 1) {
        int jMid = (ny + 1) / 2;
        for (int k = 1; k <= nz; ++k)
            for (int i = 1; i <= nx; ++i)
                sum_mid = sum_mid + (coef * V(i, jMid, k) * (T(i, jMid, k) - Tref)
                                     - (T(i, jMid + 1, k) - T(i, jMid - 1, k)) / (2.0 * dy)) / deltaT;
    } else {
        int jB = ny / 2, jT = jB + 1;
        for (int k = 1; k <= nz; ++k)
            for (int i = 1; i <= nx; ++i) {
                if (h->d3)
                    sum_mid = sum_mid + (coef * 0.5 * (V(i, jB, k) * (T(i, jB, k) - Tref) + V(i, jT, k) * (T(i, jT, k) - Tref))
                                         + (T(i, jB, k) - T(i, jT, k)) / dy) / deltaT;
                else
                    sum_mid = sum_mid + (coef * (0.5 * (V(i, jB, k) * (T(i, jB, k) - Tref) + V(i, jT, k) * (T(i, jT, k) - Tref)))
                                         + (T(i, jB, k) - T(i, jT, k)) / dy) / deltaT;
            }
    }
    out->Nu_middle = sum_mid / (double)(nx * nz);
    return std::isfinite(out->Nu_hot) ? LBM_OK : LBM_ERR_DIVERGED;
}

// SideHeatedcalc_Nu_global (2DRB.F90:1686-1734, 3DRB.F90:1789-1828)
extern "C" int ora_SideHeatedcalc_Nu_global(ora_handle* h, double* Nu) {
    const lbm_constants& c = h->c;
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const double dx = 1.0 / c.lengthUnit;
    const double deltaT = h->p.Thot - h->p.Tcold;
    const double coef = c.velocityScaleCompare;
    const double Thot = h->p.Thot, Tcold = h->p.Tcold, Tref = c.Tref;
    double sum_qx = 0.0;
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                auto T = [h, j, k](int ii) { return h->T[h->C(ii, j, k)]; };
                double dTdx;
                if (i == 1)
                    dTdx = (-3.0 * T(1) - T(2) + 4.0 * Thot) / (3.0 * dx);
                else if (i == nx)
                    dTdx = (-4.0 * Tcold + 3.0 * T(nx) + T(nx - 1)) / (3.0 * dx);
                else
                    dTdx = (T(i - 1) - T(i + 1)) / (2.0 * dx);
                double qx = coef * h->u[h->C(i, j, k)] * (T(i) - Tref) + dTdx;
                sum_qx = sum_qx + qx;
            }
    *Nu = (sum_qx / (double)(long long)h->ncell) / deltaT;
    return std::isfinite(*Nu) ? LBM_OK : LBM_ERR_DIVERGED;
}

// SideHeatedcalc_Nu_wall_avg (2DRB.F90:1746-1941, 3DRB.F90:1889-2038)
extern "C" int ora_SideHeatedcalc_Nu_wall_avg(ora_handle* h, lbm_nu_wall* out) {
    const lbm_constants& c = h->c;
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const double dx = 1.0 / c.lengthUnit;
    const double deltaT = h->p.Thot - h->p.Tcold;
    const double Thot = h->p.Thot, Tcold = h->p.Tcold, Tref = c.Tref;
    const double coef = h->d3 ? c.heatFluxScale : c.velocityScaleCompare;
    const std::vector<double>& yp = h->yp;
    auto T = [h](int i, int j, int k) { return h->T[h->C(i, j, k)]; };
    auto U = [h](int i, int j, int k) { return h->u[h->C(i, j, k)]; };
    std::vector<double> Nu_left(ny + 2, 0.0), Tl(ny + 2, 0.0);
    double sum_hot = 0.0;
    for (int j = 1; j <= ny; ++j) {
        if (h->d3) {
            double tl = 0.0;
            for (int k = 1; k <= nz; ++k) tl = tl + T(1, j, k);
            Tl[j] = tl / (double)nz;
            double nl = 0.0;
            for (int k = 1; k <= nz; ++k) {
                double qx_wall = (8.0 * Thot - 9.0 * T(1, j, k) + T(2, j, k)) / (3.0 * dx);
                nl = nl + qx_wall / deltaT;
            }
            Nu_left[j] = nl / (double)nz;
        } else {
            Tl[j] = T(1, j, 1);
            double qx_wall = (8.0 * Thot - 9.0 * T(1, j, 1) + T(2, j, 1)) / (3.0 * dx);
            Nu_left[j] = qx_wall / deltaT;
        }
        sum_hot = sum_hot + Nu_left[j];
    }
    out->Nu_hot = sum_hot / (double)ny;
    double yfit[4], Tfit[4];
    for (int m = 0; m < 4; ++m) { yfit[m] = yp[1 + m]; Tfit[m] = Tl[1 + m]; }
    double T_wb = fit_adiabatic_wall_T4(0.0, yfit, Tfit);
    for (int m = 0; m < 4; ++m) { yfit[m] = yp[ny - 3 + m]; Tfit[m] = Tl[ny - 3 + m]; }
    double T_wt = fit_adiabatic_wall_T4(yp[ny + 1], yfit, Tfit);
    std::vector<double> ext(Nu_left);
    ext[0] = (2.0 * (Thot - T_wb) / dx) / deltaT;
    ext[ny + 1] = (2.0 * (Thot - T_wt) / dx) / deltaT;
    int jmax = 0, jmin = 0;
    double vmax = ext[0], vmin = ext[0];
    for (int j = 1; j <= ny + 1; ++j) {
        if (ext[j] > vmax) { vmax = ext[j]; jmax = j; }
        if (ext[j] < vmin) { vmin = ext[j]; jmin = j; }
    }
    int jj[5];
    if (jmax <= 2) { for (int m = 0; m < 5; ++m) jj[m] = m; }
    else if (jmax >= ny - 1) { for (int m = 0; m < 5; ++m) jj[m] = ny - 3 + m; }
    else { for (int m = 0; m < 5; ++m) jj[m] = jmax - 2 + m; }
    double yk[5], fk[5], fstar, ystar;
    for (int m = 0; m < 5; ++m) { yk[m] = yp[jj[m]]; fk[m] = ext[jj[m]]; }
    if (h->d3) fit_parabola_ls5_3d(yk, fk, +1, &fstar, &ystar); else fit_parabola_ls5_2d(yk, fk, +1, &fstar, &ystar);
    out->Nu_hot_max = fstar;
    out->Nu_hot_max_position = ystar;
    if (jmin >= 4) { for (int m = 0; m < 5; ++m) jj[m] = jmin - 4 + m; }
    else { for (int m = 0; m < 5; ++m) jj[m] = m; }
    for (int m = 0; m < 5; ++m) { yk[m] = yp[jj[m]]; fk[m] = ext[jj[m]]; }
    if (h->d3) fit_parabola_ls5_3d(yk, fk, -1, &fstar, &ystar); else fit_parabola_ls5_2d(yk, fk, -1, &fstar, &ystar);
    out->Nu_hot_min = fstar;
    out->Nu_hot_min_position = ystar;

    double sum_cold = 0.0;
    for (int j = 1; j <= ny; ++j)
        for (int k = 1; k <= nz; ++k) {
            double qx_wall = (-8.0 * Tcold + 9.0 * T(nx, j, k) - T(nx - 1, j, k)) / (3.0 * dx);
            sum_cold = sum_cold + qx_wall / deltaT;
        }
    out->Nu_cold = sum_cold / (double)(ny * nz);

    double sum_mid = 0.0;
    if (nx % 2 == 1) {
        int iMid = (nx + 1) / 2;
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                sum_mid = sum_mid + (coef * U(iMid, j, k) * (T(iMid, j, k) - Tref)
                                     + (T(iMid - 1, j, k) - T(iMid + 1, j, k)) / (2.0 * dx)) / deltaT;
    } else {
        int iL = nx / 2, iR = iL + 1;
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j) {
                if (h->d3)
                    sum_mid = sum_mid + (coef * 0.5 * (U(iL, j, k) * (T(iL, j, k) - Tref) + U(iR, j, k) * (T(iR, j, k) - Tref))
                                         + (T(iL, j, k) - T(iR, j, k)) / dx) / deltaT;
                else
                    sum_mid = sum_mid + (coef * (0.5 * (U(iL, j, k) * (T(iL, j, k) - Tref) + U(iR, j, k) * (T(iR, j, k) - Tref)))
                                         + (T(iL, j, k) - T(iR, j, k)) / dx) / deltaT;
            }
    }
    out->Nu_middle = sum_mid / (double)(ny * nz);
    return std::isfinite(out->Nu_hot) ? LBM_OK : LBM_ERR_DIVERGED;
}

// Mid-line / mid-plane velocity maxima.  comp: 0 u, 1 v, 2 w; rb: the RB form of the 2D
// u line.  out = {value * velocityScaleCompare, position 1, position 2, mid coordinate}.
//   2D: SideHeatedcalc_umid_max / vmid_max (2DRB.F90:2081-2238), RBcalc_umid_max /
//       vmid_max (2DRB.F90:2484-2655);
//   3D: calc_{u,v,w}mid_max_common with find_bracketing_index and interp_scalar_*
//       (3DRB.F90:2399-2617), shared by the SideHeated and RB entry points.
extern "C" int ora_mid_max(ora_handle* h, int comp, int rb, lbm_mid_max* out) {
    const double coef = h->c.velocityScaleCompare;
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const std::vector<double>& xp = h->xp;
    const std::vector<double>& yp = h->yp;
    const std::vector<double>& zp = h->zp;
    const std::vector<double>& field = comp == 0 ? h->u : (comp == 1 ? h->v : h->w);
    auto F = [h, &field](int i, int j, int k) { return field[h->C(i, j, k)]; };
    if (h->d3) {
        const std::vector<double>& cc = comp == 0 ? xp : (comp == 1 ? yp : zp);
        const int n = comp == 0 ? nx : (comp == 1 ? ny : nz);
        const double target = 0.5 * cc[n + 1];
        int iL = 1;
        while (iL < n && cc[iL + 1] < target) iL = iL + 1;
        const int iR = std::min(iL + 1, n);
        double weight;
        if (std::fabs(cc[iR] - cc[iL]) <= 1.0e-14) weight = 0.0;
        else weight = (target - cc[iL]) / (cc[iR] - cc[iL]);
        weight = std::max(0.0, std::min(1.0, weight));
        auto interp = [&](int a, int b) {
            int iA, jA, kA, iB, jB, kB;
            if (comp == 0) { iA = iL; iB = iR; jA = jB = a; kA = kB = b; }
            else if (comp == 1) { jA = iL; jB = iR; iA = iB = a; kA = kB = b; }
            else { kA = iL; kB = iR; iA = iB = a; jA = jB = b; }
            if (iL == iR) return F(iA, jA, kA);
            return (1.0 - weight) * F(iA, jA, kA) + weight * F(iB, jB, kB);
        };
        double vmax = -std::numeric_limits<double>::max();
        int b1 = 1, b2 = 1;
        const int n1 = comp == 0 ? ny : nx, n2 = comp == 2 ? ny : nz;
        for (int q2 = 1; q2 <= n2; ++q2)
            for (int q1 = 1; q1 <= n1; ++q1) {
                const double val = interp(q1, q2);
                if (val > vmax) { vmax = val; b1 = q1; b2 = q2; }
            }
        out->value = vmax * coef;
        out->pos1 = comp == 0 ? yp[b1] : xp[b1];
        out->pos2 = comp == 2 ? yp[b2] : zp[b2];
        out->mid = target;
        return std::isfinite(vmax) ? LBM_OK : LBM_ERR_DIVERGED;
    }
    if (comp == 2) return LBM_ERR_PARAM;
    std::vector<double> line;
    double mid;
    if (comp == 0) {
        line.assign(ny + 1, 0.0);
        if (rb) {
            const double targetX = 0.5;
            mid = targetX;
            int iL = 1;
            while (iL < nx && xp[iL + 1] < targetX) iL = iL + 1;
            const int iR = std::min(iL + 1, nx);
            if (std::fabs(xp[iL] - targetX) <= 1.0e-14 || iR == iL) {
                for (int j = 1; j <= ny; ++j) line[j] = F(iL, j, 1);
            } else {
                const double w = (targetX - xp[iL]) / (xp[iR] - xp[iL]);
                for (int j = 1; j <= ny; ++j) line[j] = (1.0 - w) * F(iL, j, 1) + w * F(iR, j, 1);
            }
        } else if (nx % 2 == 1) {
            const int iMid = (nx + 1) / 2;
            mid = xp[iMid];
            for (int j = 1; j <= ny; ++j) line[j] = F(iMid, j, 1);
        } else {
            const int iL = nx / 2, iR = iL + 1;
            mid = 0.5 * (xp[iL] + xp[iR]);
            for (int j = 1; j <= ny; ++j) line[j] = 0.5 * (F(iL, j, 1) + F(iR, j, 1));
        }
    } else {
        line.assign(nx + 1, 0.0);
        if (ny % 2 == 1) {
            const int jMid = (ny + 1) / 2;
            mid = yp[jMid];
            for (int i = 1; i <= nx; ++i) line[i] = F(i, jMid, 1);
        } else {
            const int jB = ny / 2, jT = jB + 1;
            mid = 0.5 * (yp[jB] + yp[jT]);
            for (int i = 1; i <= nx; ++i) line[i] = 0.5 * (F(i, jB, 1) + F(i, jT, 1));
        }
    }
    const int nl = (int)line.size() - 1;
    const std::vector<double>& along = comp == 0 ? yp : xp;
    int q0 = 1;
    double gmax = line[1];
    for (int q = 2; q <= nl; ++q)
        if (line[q] > gmax) { gmax = line[q]; q0 = q; }
    int qq[5];
    if (q0 <= 2) { for (int m = 0; m < 5; ++m) qq[m] = 1 + m; }
    else if (q0 >= nl - 1) { for (int m = 0; m < 5; ++m) qq[m] = nl - 4 + m; }
    else { for (int m = 0; m < 5; ++m) qq[m] = q0 - 2 + m; }
    double sk[5], fk[5], fstar, sstar;
    for (int m = 0; m < 5; ++m) { sk[m] = along[qq[m]]; fk[m] = line[qq[m]]; }
    fit_parabola_ls5_2d(sk, fk, +1, &fstar, &sstar);
    if (comp == 0 && rb) {
        const double yLen = yp[ny + 1];
        if (sstar > 0.5 * yLen) sstar = yLen - sstar;
    }
    out->value = fstar * coef;
    out->pos1 = sstar;
    out->pos2 = 0.0;
    out->mid = mid;
    return std::isfinite(fstar) ? LBM_OK : LBM_ERR_DIVERGED;
}

// ------------------------------------------------------------------------------------
// state transfer
// ------------------------------------------------------------------------------------
static std::vector<double>* scalar_field(ora_handle* h, int field) {
    switch (field) {
        case LBM_FIELD_RHO: return &h->rho;
        case LBM_FIELD_U: return &h->u;
        case LBM_FIELD_V: return &h->v;
        case LBM_FIELD_W: return h->d3 ? &h->w : nullptr;
        case LBM_FIELD_T: return &h->T;
        case LBM_FIELD_BX_PREV: return &h->Bx;
        case LBM_FIELD_BY_PREV: return &h->By;
        case LBM_FIELD_BZ_PREV: return h->d3 ? &h->Bz : nullptr;
        case LBM_FIELD_FX: return h->d3 ? nullptr : &h->Fx;
        case LBM_FIELD_FY: return h->d3 ? nullptr : &h->Fy;
        default: return nullptr;
    }
}

static void copy_io(double* dst, const double* src, double* field, size_t count) {
    if (dst) {
        for (size_t n = 0; n < count; ++n) dst[n] = field[n];
    } else {
        for (size_t n = 0; n < count; ++n) field[n] = src[n];
    }
}

static int state_io(ora_handle* h, int field, double* dst, const double* src, size_t count) {
    const int q = h->L.q, qt = h->L.qt;
    if (field == LBM_FIELD_F || field == LBM_FIELD_G) {
        int qq = (field == LBM_FIELD_F) ? q : qt;
        std::vector<double>& a = (field == LBM_FIELD_F) ? h->f : h->g;
        if (count != (size_t)qq * h->ncell) return LBM_ERR_PARAM;
        copy_io(dst, src, a.data(), count);
        return LBM_OK;
    }
    if (field == LBM_FIELD_F_POST || field == LBM_FIELD_G_POST) {
        int qq = (field == LBM_FIELD_F_POST) ? q : qt;
        std::vector<double>& a = (field == LBM_FIELD_F_POST) ? h->fpost : h->gpost;
        if (count != (size_t)qq * h->ncell) return LBM_ERR_PARAM;
        for (int k = 1; k <= h->nz; ++k)
            for (int j = 1; j <= h->ny; ++j)
                for (int i = 1; i <= h->nx; ++i) {
                    size_t ci = h->C(i, j, k), pi = h->P(i, j, k);
                    for (int s = 0; s < qq; ++s) {
                        if (dst) dst[s + qq * ci] = a[s + qq * pi];
                        else a[s + qq * pi] = src[s + qq * ci];
                    }
                }
        return LBM_OK;
    }
    std::vector<double>* a = scalar_field(h, field);
    if (!a || count != h->ncell) return LBM_ERR_PARAM;
    copy_io(dst, src, a->data(), count);
    return LBM_OK;
}

extern "C" int ora_get_state(ora_handle* h, int field, double* dst, size_t count) {
    if (!h || !dst) return LBM_ERR_PARAM;
    return state_io(h, field, dst, nullptr, count);
}

extern "C" int ora_set_state(ora_handle* h, int field, const double* src, size_t count) {
    if (!h || !src) return LBM_ERR_PARAM;
    return state_io(h, field, nullptr, src, count);
}

// ------------------------------------------------------------------------------------
// transforms as matrices (for known-answer tests)
// ------------------------------------------------------------------------------------
extern "C" int ora_transform_matrices(int lattice, double* M, double* Minv) {
    const int q = lattice;
    if (!M || !Minv || (q != 9 && q != 5 && q != 19 && q != 7)) return LBM_ERR_PARAM;
    for (int col = 0; col < q; ++col) {
        double e[19] = {0}, m[19] = {0}, out[19] = {0};
        e[col] = 1.0;
        switch (q) {
            case 9: d2q9_forward(e, m); d2q9_inverse(e, out); break;
            case 5: d2q5_forward(e, m); d2q5_inverse(e, out); break;
            case 19: d3q19_forward(e, m); d3q19_inverse(e, out); break;
            default: d3q7_forward(e, m); d3q7_inverse(e, out); break;
        }
        for (int r = 0; r < q; ++r) {
            M[r * q + col] = m[r];       // column col of M is M * e_col
            Minv[r * q + col] = out[r];  // column col of Minv is Minv * e_col
        }
    }
    return LBM_OK;
}
