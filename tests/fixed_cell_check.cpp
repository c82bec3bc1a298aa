// Host stepper of the fixed arithmetic (csrc/lbm_fixed_cell.cuh) for test_cpu_fixed.py and
// the GPU tests of that form: the same cell bodies the GPU kernels run (flow_cell,
// thermal_cell, materialize_cell), looped over the cells in order on the CPU.  Integer
// arithmetic rounds identically on both, so the GPU must reproduce this stepper bit for bit;
// the CPU test compares it with the oracle at the form's tolerance.
//
// fixed_run: module arrays in the reference's Fortran layout in (after `initial` or any
// state), nsteps fused steps (the first from the module arrays), module arrays out.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "lbm_fixed_cell.cuh"

using namespace lbm;
using namespace lbm::fxa;

namespace {

// A row of the steady-state step's interior-row kernels (0 < j < ny-1, and 0 < k < nz-1 in
// 3D); the other rows go to the face-row kernels.  The stepper takes the same path per cell as
// the GPU (PATH 3: select-based x rule; PATH 2: full boundary rule), and the first step the
// any-cell path of the first-step kernels.
static bool interior_row(const Geo& g, int j, int k) {
    return j > 0 && j < g.ny - 1 && (g.nz == 1 || (k > 0 && k < g.nz - 1));
}

template <int D>
void run(const Geo& g, const PhysX& X, FixedArrays& A, long long nsteps, std::vector<long long>* fb,
         std::vector<long long>* gb) {
    const long long n = g.ncell;
    int cur = 0;
    for (long long s = 0; s < nsteps; ++s) {
        const int nxt = cur ^ 1;
        for (long long c = 0; c < n; ++c) {
            const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / ((long long)g.nx * g.ny));
            if (s == 0) flow_cell<D, true>(g, X, A, fb[cur].data(), gb[cur].data(), fb[nxt].data(), c, i, j, k);
            else if (interior_row(g, j, k))
                flow_cell<D, false, 3>(g, X, A, fb[cur].data(), gb[cur].data(), fb[nxt].data(), c, i, j, k);
            else flow_cell<D, false, 2>(g, X, A, fb[cur].data(), gb[cur].data(), fb[nxt].data(), c, i, j, k);
        }
        for (long long c = 0; c < n; ++c) {
            const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / ((long long)g.nx * g.ny));
            if (s == 0) thermal_cell<D, true>(g, X, A, fb[nxt].data(), gb[cur].data(), gb[nxt].data(), c, i, j, k);
            else if (interior_row(g, j, k))
                thermal_cell<D, false, 3>(g, X, A, fb[nxt].data(), gb[cur].data(), gb[nxt].data(), c, i, j, k);
            else thermal_cell<D, false, 2>(g, X, A, fb[nxt].data(), gb[cur].data(), gb[nxt].data(), c, i, j, k);
        }
        cur = nxt;
    }
    if (nsteps > 0) {
        for (long long c = 0; c < n; ++c) {
            const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / ((long long)g.nx * g.ny));
            materialize_cell<D>(g, X, A, fb[cur].data(), gb[cur].data(), c, i, j, k);
        }
    }
}

}  // namespace

// Arrays: f (q per cell), g (qt per cell), then rho, u, v, w, T, Bx, By, Bz, Fx, Fy, Tlag per
// cell (unused ones may be null: w, Bz, Tlag in 2D; Fx, Fy in 3D).  Returns 0, or 1 when the
// parameters leave the range of the fixed arithmetic.
extern "C" int fixed_run(const lbm_params* p, const lbm_constants* c, long long nsteps, double* f, double* g,
                         double* rho, double* u, double* v, double* w, double* T, double* Bx, double* By, double* Bz,
                         double* Fx, double* Fy, double* Tlag) {
    PhysX X;
    if (!make_physx(*p, *c, X)) return 1;
    const Geo geo = deviation_geo(make_geo(*p, *c), *c);
    const int d3 = p->dim == 3;
    const int q = d3 ? 19 : 9, qt = d3 ? 7 : 5;
    const long long n = geo.ncell;
    std::vector<double> fs((size_t)q * n), gs((size_t)qt * n);
    for (long long x = 0; x < n; ++x) {
        for (int a = 0; a < q; ++a) fs[(size_t)a * n + x] = f[a + (size_t)q * x];
        for (int a = 0; a < qt; ++a) gs[(size_t)a * n + x] = g[a + (size_t)qt * x];
    }
    std::vector<double> zero((size_t)n, 0.0), wz((size_t)n, 0.0), bz((size_t)n, 0.0), tl((size_t)n, 0.0),
        fx((size_t)n, 0.0), fy((size_t)n, 0.0);
    std::vector<long long> xb0(n), xb1(n), xb2(n), xlag(n);
    std::vector<long long> fb[2] = {std::vector<long long>((size_t)q * n), std::vector<long long>((size_t)q * n)};
    std::vector<long long> gb[2] = {std::vector<long long>((size_t)qt * n), std::vector<long long>((size_t)qt * n)};
    FixedArrays A{};
    A.f = fs.data();
    A.g = gs.data();
    A.rho = rho;
    A.u = u;
    A.v = v;
    A.w = d3 ? w : wz.data();
    A.T = T;
    A.Bx = Bx;
    A.By = By;
    A.Bz = d3 ? Bz : bz.data();
    A.Tlag = d3 && Tlag ? Tlag : tl.data();
    A.Fx = !d3 && Fx ? Fx : fx.data();
    A.Fy = !d3 && Fy ? Fy : fy.data();
    A.xb0 = xb0.data();
    A.xb1 = xb1.data();
    A.xb2 = xb2.data();
    A.xlag = xlag.data();
    if (d3) run<3>(geo, X, A, nsteps, fb, gb);
    else run<2>(geo, X, A, nsteps, fb, gb);
    for (long long x = 0; x < n; ++x) {
        for (int a = 0; a < q; ++a) f[a + (size_t)q * x] = fs[(size_t)a * n + x];
        for (int a = 0; a < qt; ++a) g[a + (size_t)qt * x] = gs[(size_t)a * n + x];
    }
    return 0;
}

// The constants of the fixed arithmetic, for inspection by the tests: 0 in range, 1 not.
extern "C" int fixed_constants_ok(const lbm_params* p, const lbm_constants* c) {
    PhysX X;
    return make_physx(*p, *c, X) ? 0 : 1;
}
