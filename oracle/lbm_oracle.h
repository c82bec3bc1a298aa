/*
 * lbm_oracle.h - CPU oracle for the coupled thermal MRT lattice-Boltzmann step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a literal C++ restatement of the reference Fortran
 * (2DRB/2DRB.F90 and 2DRB/3DRB.F90): the same eight separate passes per time step, the
 * same Fortran array-of-structures layout f(alpha,i,j,k) with ghost-padded f_post/g_post,
 * the same expression order and literal divisions, the same boundary order and quirks.
 * It is used by the tests as the parity checker and by bench.py as the timed CPU baseline
 * ("port" of the reference's OpenMP build, which cannot be compiled here: no Fortran
 * compiler).  Nothing in the product library links or calls it.
 *
 * Parity status: unpinned by the reference's own tests (the reference ships no tests,
 * fixtures or golden vectors).  It is pinned by known-answer tests (transform matrices
 * against ChaiPRE2020.F90:263-276 and the algorithm guide's D3Q7 matrix, conservation,
 * rest-state invariance) kept under tests/.
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H

#include "../include/lbm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_handle ora_handle;

int  ora_create(const lbm_params* p, ora_handle** out);
void ora_destroy(ora_handle* h);
int  ora_constants(const ora_handle* h, lbm_constants* out);
int  ora_set_threads(int n);

int ora_initial(ora_handle* h);
void ora_collision(ora_handle* h);
void ora_streaming(ora_handle* h);
void ora_bounceback(ora_handle* h);
void ora_macro(ora_handle* h);
void ora_collisionT(ora_handle* h);
void ora_streamingT(ora_handle* h);
void ora_bouncebackT(ora_handle* h);
void ora_macroT(ora_handle* h);
/* nsteps iterations of the time loop body (3DRB.F90:227-243), without check/output. */
void ora_step(ora_handle* h, long long nsteps);

/* Restart: rebuild T, rho, u, v, w, B_prev (and the 2D force) from f and g as
 * reconstruct_macro_from_fg does; zero up..Tp and itc.  Returns 1 if some rho <= 0. */
int ora_reconstruct_macro_from_fg(ora_handle* h);

int ora_check(ora_handle* h, double* errU, double* errT);
int ora_calNuRe(ora_handle* h, double* Nu, double* Re);
int ora_RBcalc_Nu_global(ora_handle* h, double* Nu);
int ora_RBcalc_Nu_wall_avg(ora_handle* h, lbm_nu_wall* out);
int ora_SideHeatedcalc_Nu_global(ora_handle* h, double* Nu);
int ora_SideHeatedcalc_Nu_wall_avg(ora_handle* h, lbm_nu_wall* out);
/* comp: 0 u, 1 v, 2 w; rb: 1 for the RB form of the 2D u line (RBcalc_umid_max). */
int ora_mid_max(ora_handle* h, int comp, int rb, lbm_mid_max* out);

int ora_get_state(ora_handle* h, int field, double* dst, size_t count);
int ora_set_state(ora_handle* h, int field, const double* src, size_t count);

/* Apply the oracle's hand-expanded transforms to unit vectors: M (forward) and Minv
 * (inverse), row-major q x q.  lattice: 9 = D2Q9, 5 = D2Q5, 19 = D3Q19, 7 = D3Q7. */
int ora_transform_matrices(int lattice, double* M, double* Minv);

#ifdef __cplusplus
}
#endif

#endif
