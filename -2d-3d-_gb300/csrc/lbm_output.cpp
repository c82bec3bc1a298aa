// lbm_output.cpp - the reference's snapshot writers and stream-function post-processing,
// on host arrays in the Fortran layout (x fastest).
//
//   output_binary       3DRB.F90:1599-1627, 2DRB.F90:1357-1389  (unformatted sequential records)
//   output_Tecplot      2DRB.F90:1443-1570 (2D fields), 3DRB.F90:1676-1700 (seven 3D files):
//     write_full_fields_plt      3DRB.F90:3018-3099
//     write_midplane_{x,y,z}     3DRB.F90:2619-2719
//     write_midplane_stream_*    3DRB.F90:2721-3016
//   calc_psi_vort_and_output   2DRB.F90:2657-2780, output_Tecplot_psi_vort 2DRB.F90:2782-2871
//   output_psi_center_abs      2DRB.F90:3085-3165 (4-point Lagrange interpolation)
//   spline_natural / splint    2DRB.F90:3000-3083 (the fine-grid |psi| search runs on the GPU)
//   append_convergence_tecplot, append_convergence_master_tecplot  2DRB.F90:1269-1343,
//     3DRB.F90:1533-1591 (formatted text: the convergence history that check appends)
//
// The Tecplot files are the reference's stream-access binary: "#!TDV101", int32 control
// words, strings as one int32 per character and a 0, float32 zone / end-of-header markers,
// then the points in x-fastest order with every variable as a float64.  Every arithmetic
// expression keeps the reference's operation order (the unit is compiled without
// floating-point contraction), so the numbers in the files are the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbm_gpu.h"
#include "lbm_records.h"

namespace lbm {
namespace {

// Node coordinates xp(0:n+1)/L (3DRB.F90:444-465, 2DRB.F90:463-476).
std::vector<double> node_coords(int n, double L) {
    std::vector<double> c((size_t)n + 2);
    for (int i = 0; i <= n + 1; ++i) {
        const double raw = i == 0 ? 0.0 : (i == n + 1 ? (double)n : (double)i - 0.5);
        c[(size_t)i] = raw / L;
    }
    return c;
}

class Stream {
  public:
    explicit Stream(const char* path) : fp_(path ? std::fopen(path, "wb") : nullptr) {}
    ~Stream() {
        if (fp_) std::fclose(fp_);
    }
    bool ok() const { return fp_ != nullptr && good_; }
    void raw(const void* p, size_t n) {
        if (fp_ && std::fwrite(p, 1, n, fp_) != n) good_ = false;
    }
    void i4(int32_t v) { raw(&v, 4); }
    void f4(float v) { raw(&v, 4); }
    void f8(double v) { raw(&v, 8); }
    // dumpstring / dumpstring_to_unit: one int32 per character of the trimmed string, then 0
    void str(const char* s) {
        size_t n = std::strlen(s);
        while (n > 0 && s[n - 1] == ' ') --n;
        for (size_t i = 0; i < n; ++i) i4((int32_t)(unsigned char)s[i]);
        i4(0);
    }
    bool close() {
        if (!fp_) return false;
        const bool ok = good_ && std::fclose(fp_) == 0;
        fp_ = nullptr;
        return ok;
    }

  private:
    FILE* fp_;
    bool good_ = true;
};

// Header and zone record common to every Tecplot file of the reference.
void tecplot_header(Stream& s, const char* title, const std::vector<const char*>& vars, int ni, int nj, int nk) {
    const float zoneMarker = 299.0f, eohMarker = 357.0f;
    s.raw("#!TDV101", 8);
    s.i4(1);
    s.str(title);
    s.i4((int32_t)vars.size());
    for (const char* v : vars) s.str(v);
    s.f4(zoneMarker);
    s.str("ZONE 001");
    s.i4(-1);
    s.i4(0);
    s.i4(1);
    s.i4(0);
    s.i4(0);
    s.i4(ni);
    s.i4(nj);
    s.i4(nk);
    s.i4(0);
    s.f4(eohMarker);
    s.f4(zoneMarker);
    for (size_t k = 0; k < vars.size(); ++k) s.i4(2);
    s.i4(0);
    s.i4(-1);
}

inline size_t at2(int i, int j, int ni) { return (size_t)(i - 1) + (size_t)ni * (size_t)(j - 1); }
inline size_t at3(int i, int j, int k, int nx, int ny) {
    return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
}

// find_bracketing_index (3DRB.F90:2525-2545) on coordinates c(0:n+1).
void bracket(const std::vector<double>& c, int n, double target, int& iL, int& iR, double& weight) {
    iL = 1;
    while (iL < n && c[(size_t)iL + 1] < target) iL = iL + 1;
    iR = iL + 1 < n ? iL + 1 : n;
    if (std::fabs(c[(size_t)iR] - c[(size_t)iL]) <= 1.0e-14) weight = 0.0;
    else weight = (target - c[(size_t)iL]) / (c[(size_t)iR] - c[(size_t)iL]);
    weight = std::fmax(0.0, std::fmin(1.0, weight));
}

// interp_scalar_{x,y,z} (3DRB.F90:2553-2617): the field on the mid plane normal to `axis`
// as a slice s(a,b) (a the earlier remaining axis), ni x nj.
std::vector<double> mid_slice(const double* f, int axis, int nx, int ny, int nz, int iL, int iR, double w) {
    const int n1 = axis == 0 ? ny : nx, n2 = axis == 2 ? ny : nz;
    std::vector<double> s((size_t)n1 * n2);
    for (int b = 1; b <= n2; ++b)
        for (int a = 1; a <= n1; ++a) {
            auto F = [&](int q) {
                if (axis == 0) return f[at3(q, a, b, nx, ny)];
                if (axis == 1) return f[at3(a, q, b, nx, ny)];
                return f[at3(a, b, q, nx, ny)];
            };
            s[at2(a, b, n1)] = iL == iR ? F(iL) : (1.0 - w) * F(iL) + w * F(iR);
        }
    return s;
}

// d/d(first slice index) and d/d(second) with the reference's one-sided ends (3DRB.F90:2776-2810).
double d_first(const std::vector<double>& s, int a, int b, int n1, double h) {
    if (n1 == 1) return 0.0;
    if (a == 1) {
        if (n1 == 2) return (s[at2(2, b, n1)] - s[at2(1, b, n1)]) / h;
        return (-3.0 * s[at2(1, b, n1)] + 4.0 * s[at2(2, b, n1)] - s[at2(3, b, n1)]) / (2.0 * h);
    }
    if (a == n1) {
        if (n1 == 2) return (s[at2(n1, b, n1)] - s[at2(n1 - 1, b, n1)]) / h;
        return (3.0 * s[at2(n1, b, n1)] - 4.0 * s[at2(n1 - 1, b, n1)] + s[at2(n1 - 2, b, n1)]) / (2.0 * h);
    }
    return (s[at2(a + 1, b, n1)] - s[at2(a - 1, b, n1)]) / (2.0 * h);
}
double d_second(const std::vector<double>& s, int a, int b, int n1, int n2, double h) {
    if (n2 == 1) return 0.0;
    if (b == 1) {
        if (n2 == 2) return (s[at2(a, 2, n1)] - s[at2(a, 1, n1)]) / h;
        return (-3.0 * s[at2(a, 1, n1)] + 4.0 * s[at2(a, 2, n1)] - s[at2(a, 3, n1)]) / (2.0 * h);
    }
    if (b == n2) {
        if (n2 == 2) return (s[at2(a, n2, n1)] - s[at2(a, n2 - 1, n1)]) / h;
        return (3.0 * s[at2(a, n2, n1)] - 4.0 * s[at2(a, n2 - 1, n1)] + s[at2(a, n2 - 2, n1)]) / (2.0 * h);
    }
    return (s[at2(a, b + 1, n1)] - s[at2(a, b - 1, n1)]) / (2.0 * h);
}

// Stream function of a slice by integrating the velocity s along the second index
// (Simpson rule with a quadratic mid-point, 3DRB.F90:2744-2764).
std::vector<double> psi_slice(const std::vector<double>& s, int n1, int n2, double h, double coef) {
    std::vector<double> psi((size_t)n1 * n2, 0.0);
    if (n2 == 1) return psi;
    for (int a = 1; a <= n1; ++a) {
        auto S = [&](int b) { return s[at2(a, b, n1)]; };
        const double v1 = S(1) * coef, v2 = S(2) * coef;
        psi[at2(a, 1, n1)] = h * (21.0 * v1 - v2) / 72.0;
        for (int b = 2; b <= n2; ++b) {
            const int m = b - 1;
            double mid;
            if (n2 == 2) mid = 0.5 * (S(1) + S(2)) * coef;
            else if (m == 1) mid = (3.0 / 8.0 * S(1) + 3.0 / 4.0 * S(2) - 1.0 / 8.0 * S(3)) * coef;
            else mid = (-1.0 / 8.0 * S(m - 1) + 3.0 / 4.0 * S(m) + 3.0 / 8.0 * S(m + 1)) * coef;
            const double inc = h / 6.0 * (S(b - 1) * coef + 4.0 * mid + S(b) * coef);
            psi[at2(a, b, n1)] = psi[at2(a, b - 1, n1)] + inc;
        }
    }
    return psi;
}

bool write_slice(const char* path, const char* title, const std::vector<const char*>& vars, int ni, int nj,
                 const double* c1, const double* c2, const std::vector<const std::vector<double>*>& fields) {
    Stream s(path);
    if (!s.ok()) return false;
    tecplot_header(s, title, vars, ni, nj, 1);
    for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
            s.f8(c1[i]);
            s.f8(c2[j]);
            for (const auto* f : fields) s.f8((*f)[at2(i, j, ni)]);
        }
    return s.close();
}

}  // namespace

// ---- splines (2DRB.F90:3000-3083), shared with the device search -------------------------
void spline_natural(int n, const double* x, const double* y, double* y2, double* u) {
    y2[0] = 0.0;
    u[0] = 0.0;
    for (int i = 2; i <= n - 1; ++i) {
        const double sig = (x[i - 1] - x[i - 2]) / (x[i] - x[i - 2]);
        const double p = sig * y2[i - 2] + 2.0;
        y2[i - 1] = (sig - 1.0) / p;
        u[i - 1] = (6.0 * ((y[i] - y[i - 1]) / (x[i] - x[i - 1]) - (y[i - 1] - y[i - 2]) / (x[i - 1] - x[i - 2])) /
                        (x[i] - x[i - 2]) - sig * u[i - 2]) / p;
    }
    y2[n - 1] = 0.0;
    for (int k = n - 1; k >= 1; --k) y2[k - 1] = y2[k - 1] * y2[k] + u[k - 1];
}

double splint(int n, const double* xa, const double* ya, const double* y2a, double x) {
    int klo = 1, khi = n;
    while (khi - klo > 1) {
        const int k = (khi + klo) / 2;
        if (xa[k - 1] > x) khi = k;
        else klo = k;
    }
    const double h = xa[khi - 1] - xa[klo - 1];
    if (h == 0.0) return ya[klo - 1];
    const double a = (xa[khi - 1] - x) / h;
    const double b = (x - xa[klo - 1]) / h;
    return a * ya[klo - 1] + b * ya[khi - 1] +
           ((a * a * a - a) * y2a[klo - 1] + (b * b * b - b) * y2a[khi - 1]) * (h * h) / 6.0;
}

}  // namespace lbm

using namespace lbm;

// ---- host-array writers ------------------------------------------------------------------
extern "C" int lbm_output_binary_host(const char* path, int dim, int nx, int ny, int nz, double velocityScaleCompare,
                                      const double* u, const double* v, const double* w, const double* T,
                                      const double* rho) {
    if (!path || !u || !v || !T || !rho || (dim == 3 && !w) || nx < 1 || ny < 1 || nz < 1) return LBM_ERR_PARAM;
    const size_t n = (size_t)nx * ny * (dim == 3 ? nz : 1);
    std::vector<double> rec(n);
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return LBM_ERR_IO;
    bool ok = true;
    auto record = [&](const double* a, bool scaled) {
        for (size_t c = 0; c < n; ++c) rec[c] = scaled ? velocityScaleCompare * a[c] : a[c];
        RecordWriter wr;
        ok = ok && wr.begin(fp, n * sizeof(double)) && wr.put(rec.data(), n * sizeof(double)) && wr.end();
    };
    record(u, true);
    record(v, true);
    if (dim == 3) record(w, true);
    record(T, false);
    record(rho, false);
    if (std::fclose(fp) != 0) ok = false;
    return ok ? LBM_OK : LBM_ERR_IO;
}

extern "C" int lbm_tecplot_fields_2d(const char* path, int nx, int ny, double lengthUnit, double velocityScaleCompare,
                                     const double* u, const double* v, const double* T) {
    if (!path || !u || !v || !T || nx < 1 || ny < 1) return LBM_ERR_PARAM;
    const std::vector<double> xp = node_coords(nx, lengthUnit), yp = node_coords(ny, lengthUnit);
    Stream s(path);
    if (!s.ok()) return LBM_ERR_IO;
    tecplot_header(s, "MyFirst", {"X", "Y", "U_nd", "V_nd", "T"}, nx, ny, 1);
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            s.f8(xp[(size_t)i]);
            s.f8(yp[(size_t)j]);
            s.f8(velocityScaleCompare * u[at2(i, j, nx)]);
            s.f8(velocityScaleCompare * v[at2(i, j, nx)]);
            s.f8(T[at2(i, j, nx)]);
        }
    return s.close() ? LBM_OK : LBM_ERR_IO;
}

extern "C" int lbm_tecplot_full_3d(const char* path, int nx, int ny, int nz, double lengthUnit, const double* u,
                                   const double* v, const double* w, const double* T) {
    if (!path || !u || !v || !w || !T || nx < 1 || ny < 1 || nz < 1) return LBM_ERR_PARAM;
    const std::vector<double> xp = node_coords(nx, lengthUnit), yp = node_coords(ny, lengthUnit),
                              zp = node_coords(nz, lengthUnit);
    Stream s(path);
    if (!s.ok()) return LBM_ERR_IO;
    tecplot_header(s, "full-field-3d", {"X", "Y", "Z", "U", "V", "W", "T"}, nx, ny, nz);
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                const size_t c = at3(i, j, k, nx, ny);
                s.f8(xp[(size_t)i]);
                s.f8(yp[(size_t)j]);
                s.f8(zp[(size_t)k]);
                s.f8(u[c]);
                s.f8(v[c]);
                s.f8(w[c]);
                s.f8(T[c]);
            }
    return s.close() ? LBM_OK : LBM_ERR_IO;
}

extern "C" int lbm_tecplot_midplane_3d(const char* path, int axis, int nx, int ny, int nz, double lengthUnit,
                                       double velocityScaleCompare, const double* u, const double* v, const double* w,
                                       const double* T) {
    if (!path || !u || !v || !w || !T || axis < 0 || axis > 2 || nx < 1 || ny < 1 || nz < 1) return LBM_ERR_PARAM;
    const std::vector<double> c[3] = {node_coords(nx, lengthUnit), node_coords(ny, lengthUnit), node_coords(nz, lengthUnit)};
    const int n[3] = {nx, ny, nz};
    int iL, iR;
    double wgt;
    bracket(c[axis], n[axis], 0.5 * c[axis][(size_t)n[axis] + 1], iL, iR, wgt);
    std::vector<double> su = mid_slice(u, axis, nx, ny, nz, iL, iR, wgt), sv = mid_slice(v, axis, nx, ny, nz, iL, iR, wgt),
                        sw = mid_slice(w, axis, nx, ny, nz, iL, iR, wgt), st = mid_slice(T, axis, nx, ny, nz, iL, iR, wgt);
    for (std::vector<double>* s : {&su, &sv, &sw})
        for (double& x : *s) x = velocityScaleCompare * x;
    const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    static const char* titles[3] = {"midX-fields", "midY-fields", "midZ-fields"};
    static const char* names[3] = {"X", "Y", "Z"};
    return write_slice(path, titles[axis], {names[a1], names[a2], "U_nd", "V_nd", "W_nd", "T"}, n[a1], n[a2],
                       c[a1].data(), c[a2].data(), {&su, &sv, &sw, &st})
               ? LBM_OK
               : LBM_ERR_IO;
}

extern "C" int lbm_tecplot_midplane_stream_3d(const char* path, int axis, int nx, int ny, int nz, double lengthUnit,
                                              double velocityScaleCompare, const double* u, const double* v,
                                              const double* w) {
    if (!path || !u || !v || !w || axis < 0 || axis > 2 || nx < 1 || ny < 1 || nz < 1) return LBM_ERR_PARAM;
    const std::vector<double> c[3] = {node_coords(nx, lengthUnit), node_coords(ny, lengthUnit), node_coords(nz, lengthUnit)};
    const int n[3] = {nx, ny, nz};
    int iL, iR;
    double wgt;
    bracket(c[axis], n[axis], 0.5 * c[axis][(size_t)n[axis] + 1], iL, iR, wgt);
    const double h = 1.0 / lengthUnit, coef = velocityScaleCompare;
    const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    const int n1 = n[a1], n2 = n[a2];
    // integrated component (along the second slice index) and the other in-plane component:
    //   x: v along z, w;  y: u along z, w;  z: u along y, v
    const double* fi = axis == 0 ? v : u;
    const double* fo = axis == 2 ? v : w;
    const std::vector<double> si = mid_slice(fi, axis, nx, ny, nz, iL, iR, wgt);
    const std::vector<double> so = mid_slice(fo, axis, nx, ny, nz, iL, iR, wgt);
    const std::vector<double> psi = psi_slice(si, n1, n2, h, coef);
    std::vector<double> vort((size_t)n1 * n2);
    for (int b = 1; b <= n2; ++b)
        for (int a = 1; a <= n1; ++a) {
            // x: coef*(dw/dy - dv/dz); y: coef*(du/dz - dw/dx); z: coef*(dv/dx - du/dy)
            double t1, t2;
            if (axis == 0) {
                t1 = d_first(so, a, b, n1, h);
                t2 = d_second(si, a, b, n1, n2, h);
            } else if (axis == 1) {
                t1 = d_second(si, a, b, n1, n2, h);
                t2 = d_first(so, a, b, n1, h);
            } else {
                t1 = d_first(so, a, b, n1, h);
                t2 = d_second(si, a, b, n1, n2, h);
            }
            vort[at2(a, b, n1)] = coef * (t1 - t2);
        }
    static const char* titles[3] = {"midX-psi-vort", "midY-psi-vort", "midZ-psi-vort"};
    static const char* psin[3] = {"PSI_YZ", "PSI_XZ", "PSI_XY"};
    static const char* vortn[3] = {"VORT_X", "VORT_Y", "VORT_Z"};
    static const char* names[3] = {"X", "Y", "Z"};
    return write_slice(path, titles[axis], {names[a1], names[a2], psin[axis], vortn[axis]}, n1, n2, c[a1].data(),
                       c[a2].data(), {&psi, &vort})
               ? LBM_OK
               : LBM_ERR_IO;
}

// calc_psi_vort_and_output (2DRB.F90:2657-2740): psi by Simpson integration of u along y,
// vorticity with one-sided wall stencils.
extern "C" int lbm_psi_vort_2d(int nx, int ny, double lengthUnit, double velocityScaleCompare, const double* u,
                               const double* v, double* psi, double* vort) {
    if (!u || !v || !psi || !vort || nx < 2 || ny < 3) return LBM_ERR_PARAM;
    const double dx = 1.0 / lengthUnit, dy = 1.0 / lengthUnit, coef = velocityScaleCompare;
    auto U = [&](int i, int j) { return u[at2(i, j, nx)]; };
    auto V = [&](int i, int j) { return v[at2(i, j, nx)]; };
    for (int i = 1; i <= nx; ++i) {
        const double u1 = U(i, 1) * coef, u2 = U(i, 2) * coef;
        psi[at2(i, 1, nx)] = dy * (21.0 * u1 - u2) / 72.0;
        for (int j = 2; j <= ny; ++j) {
            const int m = j - 1;
            double u_mid;
            if (m == 1) u_mid = (3.0 / 8.0 * U(i, 1) + 3.0 / 4.0 * U(i, 2) - 1.0 / 8.0 * U(i, 3)) * coef;
            else u_mid = (-1.0 / 8.0 * U(i, m - 1) + 3.0 / 4.0 * U(i, m) + 3.0 / 8.0 * U(i, m + 1)) * coef;
            const double inc = dy / 6.0 * ((U(i, j - 1) * coef) + 4.0 * u_mid + (U(i, j) * coef));
            psi[at2(i, j, nx)] = psi[at2(i, j - 1, nx)] + inc;
        }
    }
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            double dv_dx, du_dy;
            if (i == 1) dv_dx = (3.0 * V(1, j) + V(2, j) - 4.0 * 0.0) / (3.0 * dx);
            else if (i == nx) dv_dx = (-3.0 * V(nx, j) - V(nx - 1, j) + 4.0 * 0.0) / (3.0 * dx);
            else dv_dx = (V(i + 1, j) - V(i - 1, j)) / (2.0 * dx);
            if (j == 1) du_dy = (3.0 * U(i, 1) + U(i, 2) - 4.0 * 0.0) / (3.0 * dy);
            else if (j == ny) du_dy = (-3.0 * U(i, ny) - U(i, ny - 1) + 4.0 * 0.0) / (3.0 * dy);
            else du_dy = (U(i, j + 1) - U(i, j - 1)) / (2.0 * dy);
            vort[at2(i, j, nx)] = coef * (dv_dx - du_dy);
        }
    return LBM_OK;
}

// output_Tecplot_psi_vort (2DRB.F90:2782-2871)
extern "C" int lbm_tecplot_psi_vort_2d(const char* path, int nx, int ny, double lengthUnit, const double* psi,
                                       const double* vort) {
    if (!path || !psi || !vort || nx < 1 || ny < 1) return LBM_ERR_PARAM;
    const std::vector<double> xp = node_coords(nx, lengthUnit), yp = node_coords(ny, lengthUnit);
    Stream s(path);
    if (!s.ok()) return LBM_ERR_IO;
    tecplot_header(s, "psi-vort", {"X", "Y", "PSI", "VORT"}, nx, ny, 1);
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            s.f8(xp[(size_t)i]);
            s.f8(yp[(size_t)j]);
            s.f8(psi[at2(i, j, nx)]);
            s.f8(vort[at2(i, j, nx)]);
        }
    return s.close() ? LBM_OK : LBM_ERR_IO;
}

// output_psi_center_abs (2DRB.F90:3085-3165): psi at the cavity centre by 4 x 4 Lagrange
// interpolation on the coarse grid.
extern "C" int lbm_psi_center_2d(int nx, int ny, double lengthUnit, const double* psi, double* psi_center) {
    if (!psi || !psi_center || nx < 1 || ny < 1) return LBM_ERR_PARAM;
    const std::vector<double> xp = node_coords(nx, lengthUnit), yp = node_coords(ny, lengthUnit);
    auto lagrange4 = [](double xq, const double* xk, const double* fk) {
        double fq = 0.0;
        for (int a = 0; a < 4; ++a) {
            double basis = 1.0;
            for (int b = 0; b < 4; ++b)
                if (b != a) basis = basis * (xq - xk[b]) / (xk[a] - xk[b]);
            fq = fq + fk[a] * basis;
        }
        return fq;
    };
    const double x0 = 0.5 * xp[(size_t)nx + 1], y0 = 0.5 * yp[(size_t)ny + 1];
    if (nx < 4 || ny < 4) {
        *psi_center = psi[at2((nx + 1) / 2, (ny + 1) / 2, nx)];
        return LBM_OK;
    }
    int i0 = 1;
    while (i0 < nx && xp[(size_t)i0 + 1] <= x0) i0 = i0 + 1;
    i0 = std::max(1, std::min(i0 - 1, nx - 3));
    int j0 = 1;
    while (j0 < ny && yp[(size_t)j0 + 1] <= y0) j0 = j0 + 1;
    j0 = std::max(1, std::min(j0 - 1, ny - 3));
    double x4[4], y4[4], f4[4], gx[4];
    for (int p = 0; p < 4; ++p) x4[p] = xp[(size_t)(i0 + p)];
    for (int q = 0; q < 4; ++q) y4[q] = yp[(size_t)(j0 + q)];
    for (int q = 0; q < 4; ++q) {
        for (int p = 0; p < 4; ++p) f4[p] = psi[at2(i0 + p, j0 + q, nx)];
        gx[q] = lagrange4(x0, x4, f4);
    }
    *psi_center = lagrange4(y0, y4, gx);
    return LBM_OK;
}

// ---- fine-grid |psi| search (calc_psi_absmax_fine_spline, 2DRB.F90:2873-2998) -------------
namespace lbm {
int psi_fine_search(int nx, int ny, double xLen, double yLen, int nFineX, int nFineY, const double* xExt,
                    const double* yExt, const double* rows, const double* y2rows, double* xfine, double* best_val,
                    int* best_l, cudaStream_t s);
}

extern "C" int lbm_psi_absmax_fine_spline(int nx, int ny, double lengthUnit, const double* psi, int nFinePerUnit,
                                          double* psi_abs_max, double* x_at_max, double* y_at_max,
                                          double* psi_center_abs_fine) {
    if (!psi || !psi_abs_max || !x_at_max || !y_at_max || !psi_center_abs_fine || nx < 1 || ny < 1 ||
        nFinePerUnit < 1 || ny + 2 > 2048)
        return LBM_ERR_PARAM;
    const std::vector<double> xp = node_coords(nx, lengthUnit), yp = node_coords(ny, lengthUnit);
    const double xLen = xp[(size_t)nx + 1], yLen = yp[(size_t)ny + 1];
    const double xCenter = 0.5 * xLen, yCenter = 0.5 * yLen;
    const int nFineX = std::max(2, (int)std::lround(xLen * (double)nFinePerUnit) + 1);
    const int nFineY = std::max(2, (int)std::lround(yLen * (double)nFinePerUnit) + 1);
    const int nXExt = nx + 2, nYExt = ny + 2;
    std::vector<double> xExt(nXExt), yExt(nYExt);
    xExt[0] = 0.0;
    xExt[nXExt - 1] = xp[(size_t)nx + 1];
    for (int i = 1; i <= nx; ++i) xExt[i] = xp[(size_t)i];
    yExt[0] = 0.0;
    yExt[nYExt - 1] = yp[(size_t)ny + 1];
    for (int j = 1; j <= ny; ++j) yExt[j] = yp[(size_t)j];
    // row splines and the centre line, as the reference's first loop (host, sequential)
    std::vector<double> rows((size_t)ny * nXExt), y2rows((size_t)ny * nXExt), work(nXExt > nYExt ? nXExt : nYExt),
        centre_x(ny);
    for (int j = 1; j <= ny; ++j) {
        double* row = &rows[(size_t)(j - 1) * nXExt];
        row[0] = 0.0;
        row[nXExt - 1] = 0.0;
        for (int i = 1; i <= nx; ++i) row[i] = psi[at2(i, j, nx)];
        double* y2 = &y2rows[(size_t)(j - 1) * nXExt];
        spline_natural(nXExt, xExt.data(), row, y2, work.data());
        centre_x[(size_t)j - 1] = splint(nXExt, xExt.data(), row, y2, xCenter);
    }
    std::vector<double> col(nYExt), y2col(nYExt);
    col[0] = 0.0;
    col[nYExt - 1] = 0.0;
    for (int j = 1; j <= ny; ++j) col[j] = centre_x[(size_t)j - 1];
    spline_natural(nYExt, yExt.data(), col.data(), y2col.data(), work.data());
    *psi_center_abs_fine = std::fabs(splint(nYExt, yExt.data(), col.data(), y2col.data(), yCenter));
    // the fine grid on the GPU
    double *d_x = nullptr, *d_y = nullptr, *d_rows = nullptr, *d_y2 = nullptr, *d_fine = nullptr, *d_best = nullptr;
    int* d_l = nullptr;
    int st = LBM_OK;
    auto alloc = [&](void** p, size_t b) {
        if (st == LBM_OK && cudaMalloc(p, b) != cudaSuccess) st = LBM_ERR_OOM;
    };
    alloc((void**)&d_x, nXExt * sizeof(double));
    alloc((void**)&d_y, nYExt * sizeof(double));
    alloc((void**)&d_rows, rows.size() * sizeof(double));
    alloc((void**)&d_y2, y2rows.size() * sizeof(double));
    alloc((void**)&d_fine, (size_t)nFineX * ny * sizeof(double));
    alloc((void**)&d_best, (size_t)nFineX * sizeof(double));
    alloc((void**)&d_l, (size_t)nFineX * sizeof(int));
    std::vector<double> best(nFineX);
    std::vector<int> bl(nFineX);
    if (st == LBM_OK) {
        bool ok = cudaMemcpy(d_x, xExt.data(), nXExt * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
                  cudaMemcpy(d_y, yExt.data(), nYExt * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
                  cudaMemcpy(d_rows, rows.data(), rows.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
                  cudaMemcpy(d_y2, y2rows.data(), y2rows.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess;
        if (!ok) st = LBM_ERR_CUDA;
    }
    if (st == LBM_OK)
        st = psi_fine_search(nx, ny, xLen, yLen, nFineX, nFineY, d_x, d_y, d_rows, d_y2, d_fine, d_best, d_l, 0);
    if (st == LBM_OK) {
        bool ok = cudaMemcpy(best.data(), d_best, (size_t)nFineX * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess &&
                  cudaMemcpy(bl.data(), d_l, (size_t)nFineX * sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
        if (!ok) st = LBM_ERR_CUDA;
    }
    for (void* p : {(void*)d_x, (void*)d_y, (void*)d_rows, (void*)d_y2, (void*)d_fine, (void*)d_best, (void*)d_l})
        if (p) cudaFree(p);
    if (st != LBM_OK) return st;
    // the reference's scan: x outer, y inner, strictly larger |psi| replaces
    double vmax = -1.0, xm = 0.0, ym = 0.0;
    for (int k = 0; k < nFineX; ++k)
        if (best[(size_t)k] > vmax) {
            vmax = best[(size_t)k];
            xm = xLen * (double)k / (double)(nFineX - 1);
            ym = yLen * (double)bl[(size_t)k] / (double)(nFineY - 1);
        }
    *psi_abs_max = vmax;
    *x_at_max = xm;
    *y_at_max = ym;
    return LBM_OK;
}

// ---- handle-level writers ------------------------------------------------------------------
namespace {

struct Fields {
    lbm_params p;
    lbm_constants c;
    size_t n = 0;
    std::vector<double> u, v, w, T, rho;
};

int fetch(lbm_handle* h, Fields& F, bool with_T, bool with_rho) {
    int st = lbm_get_params(h, &F.p);
    if (st != LBM_OK) return st;
    if ((st = lbm_get_constants(h, &F.c)) != LBM_OK) return st;
    F.n = (size_t)F.p.nx * F.p.ny * (F.p.dim == 3 ? F.p.nz : 1);
    F.u.resize(F.n);
    F.v.resize(F.n);
    if ((st = lbm_get_state(h, LBM_FIELD_U, F.u.data(), F.n)) != LBM_OK) return st;
    if ((st = lbm_get_state(h, LBM_FIELD_V, F.v.data(), F.n)) != LBM_OK) return st;
    if (F.p.dim == 3) {
        F.w.resize(F.n);
        if ((st = lbm_get_state(h, LBM_FIELD_W, F.w.data(), F.n)) != LBM_OK) return st;
    }
    if (with_T) {
        F.T.resize(F.n);
        if ((st = lbm_get_state(h, LBM_FIELD_T, F.T.data(), F.n)) != LBM_OK) return st;
    }
    if (with_rho) {
        F.rho.resize(F.n);
        if ((st = lbm_get_state(h, LBM_FIELD_RHO, F.rho.data(), F.n)) != LBM_OK) return st;
    }
    return LBM_OK;
}

// ------------------------------------------------------------------------------------
// Fortran formatted output of the convergence records.  ESw.d[Ee]: a minus sign for negative
// values, one nonzero digit (0 for zero), '.', d digits, then the exponent: 'E', sign and two
// digits; without Ee a three-digit exponent takes the place of the letter ("-100"); with Ee
// exactly e digits.  NaN and Infinity are spelled out.  Iw right-justifies an integer in w
// columns, I0 writes it in as few as it needs.  A value that does not fit its field is
// written as w asterisks.  The decimal digits are the correctly rounded ones, as gfortran
// and the C library both produce.
// ------------------------------------------------------------------------------------
std::string fit(const std::string& s, int w) {
    if (w <= 0) return s;
    if ((int)s.size() > w) return std::string((size_t)w, '*');
    return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

std::string fortran_es(double x, int w, int d, int e) {
    if (std::isnan(x)) return fit("NaN", w);
    if (std::isinf(x)) return fit(x < 0 ? "-Infinity" : "Infinity", w);
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.*E", d, x);
    const std::string c(buf);
    const size_t at = c.find('E');
    const std::string mant = c.substr(0, at);
    const char sign = c[at + 1];
    std::string digits = c.substr(at + 2);
    while (digits.size() > 2 && digits[0] == '0') digits.erase(0, 1);
    std::string out;
    if (e > 0) {
        if ((int)digits.size() > e) return std::string((size_t)w, '*');
        while ((int)digits.size() < e) digits.insert(0, "0");
        out = mant + "E" + sign + digits;
    } else {
        out = digits.size() <= 2 ? mant + "E" + sign + digits : mant + sign + digits;
    }
    return fit(out, w);
}

std::string fortran_i(long long v, int w) { return fit(std::to_string(v), w); }

// write(u,'(I12,1X,ES24.16,1X,ES24.16)') itc, errorU, errorT
std::string convergence_line(long long itc, double errU, double errT) {
    return fortran_i(itc, 12) + " " + fortran_es(errU, 24, 16, 0) + " " + fortran_es(errT, 24, 16, 0) + "\n";
}

bool file_exists(const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fclose(f);
    return true;
}

// Write `text` to `path`: replacing the file (status='replace') or appending to an existing
// one (status='old', position='append': a missing file is an error, as in the reference).
int write_text(const char* path, const std::string& text, bool replace) {
    if (!replace && !file_exists(path)) return LBM_ERR_IO;
    FILE* f = std::fopen(path, replace ? "wb" : "ab");
    if (!f) return LBM_ERR_IO;
    const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
    return (std::fclose(f) == 0 && ok) ? LBM_OK : LBM_ERR_IO;
}

std::string numbered(const char* prefix, const char* tag, long long number, const char* ext) {
    char num[32];
    std::snprintf(num, sizeof(num), "%012lld", number);  // write(filename,'(i12.12)')
    return std::string(prefix) + "-" + tag + num + ext;
}

}  // namespace

extern "C" int lbm_format_fortran_es(double x, int w, int d, int e, char* buf, size_t len) {
    if (!buf || len == 0 || w <= 0 || d < 0 || e < 0) return LBM_ERR_PARAM;
    const std::string s = fortran_es(x, w, d, e);
    if (s.size() + 1 > len) return LBM_ERR_PARAM;
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return LBM_OK;
}

extern "C" int lbm_append_convergence_tecplot_host(const char* filename, int first, int dim, int64_t itc, double errorU,
                                                   double errorT) {
    if (!filename || (dim != 2 && dim != 3)) return LBM_ERR_PARAM;
    const std::string line = convergence_line((long long)itc, errorU, errorT);
    if (first) {  // the run's first record replaces the file (2DRB.F90:1283-1290, 3DRB.F90:1543-1549)
        const std::string head = std::string("VARIABLES = \"itc\" \"errorU\" \"errorT\"\n") + "ZONE T=\"" +
                                 (dim == 3 ? "conv3d" : "conv") + "\", F=POINT\n";
        return write_text(filename, head + line, true);
    }
    return write_text(filename, line, false);
}

extern "C" int lbm_append_convergence_master_tecplot_host(const char* filename, int first, int dim, const char* zone,
                                                          int64_t itc, double errorU, double errorT) {
    if (!filename || !zone || (dim != 2 && dim != 3)) return LBM_ERR_PARAM;
    int st;
    if (first) {  // a title the first time the file is made, a new zone for every run (2DRB.F90:1322-1337)
        if (!file_exists(filename)) {
            const std::string head = std::string("TITLE = \"Convergence comparison") + (dim == 3 ? " 3D" : "") +
                                     "\"\nVARIABLES = \"itc\" \"errorU\" \"errorT\"\n";
            if ((st = write_text(filename, head, true)) != LBM_OK) return st;
        }
        std::string z(zone);
        while (!z.empty() && z.back() == ' ') z.pop_back();  // trim(zoneName)
        if ((st = write_text(filename, "ZONE T=\"" + z + "\", F=POINT\n", false)) != LBM_OK) return st;
    }
    return write_text(filename, convergence_line((long long)itc, errorU, errorT), false);
}

extern "C" int lbm_convergence_line(int64_t itc, double errorU, double errorT, char* buf, size_t len) {
    if (!buf) return LBM_ERR_PARAM;
    const std::string s = convergence_line((long long)itc, errorU, errorT);
    if (s.size() + 1 > len) return LBM_ERR_PARAM;
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return LBM_OK;
}

extern "C" int lbm_output_binary(lbm_handle* h, const char* path) {
    if (!h || !path) return LBM_ERR_PARAM;
    Fields F;
    int st = fetch(h, F, true, true);
    if (st != LBM_OK) return st;
    return lbm_output_binary_host(path, F.p.dim, F.p.nx, F.p.ny, F.p.dim == 3 ? F.p.nz : 1, F.c.velocityScaleCompare,
                                  F.u.data(), F.v.data(), F.p.dim == 3 ? F.w.data() : nullptr, F.T.data(),
                                  F.rho.data());
}

extern "C" int lbm_output_Tecplot(lbm_handle* h, const char* prefix, int64_t number) {
    if (!h || !prefix) return LBM_ERR_PARAM;
    Fields F;
    int st = fetch(h, F, true, false);
    if (st != LBM_OK) return st;
    const double L = F.c.lengthUnit, vsc = F.c.velocityScaleCompare;
    const int nx = F.p.nx, ny = F.p.ny, nz = F.p.nz;
    if (F.p.dim == 2)
        return lbm_tecplot_fields_2d(numbered(prefix, "", number, ".plt").c_str(), nx, ny, L, vsc, F.u.data(),
                                     F.v.data(), F.T.data());
    const double *u = F.u.data(), *v = F.v.data(), *w = F.w.data(), *T = F.T.data();
    if ((st = lbm_tecplot_full_3d(numbered(prefix, "fullField-", number, ".plt").c_str(), nx, ny, nz, L, u, v, w, T)))
        return st;
    static const char* mids[3] = {"midX-", "midY-", "midZ-"};
    static const char* streams[3] = {"midXpsiVort-", "midYpsiVort-", "midZpsiVort-"};
    for (int a = 0; a < 3; ++a)
        if ((st = lbm_tecplot_midplane_3d(numbered(prefix, mids[a], number, ".plt").c_str(), a, nx, ny, nz, L, vsc, u, v,
                                          w, T)))
            return st;
    for (int a = 0; a < 3; ++a)
        if ((st = lbm_tecplot_midplane_stream_3d(numbered(prefix, streams[a], number, ".plt").c_str(), a, nx, ny, nz, L,
                                                 vsc, u, v, w)))
            return st;
    return LBM_OK;
}

extern "C" int lbm_calc_psi_vort_and_output(lbm_handle* h, const char* prefix, int64_t number, int nFinePerUnit,
                                            lbm_psi_summary* out) {
    if (!h || !out) return LBM_ERR_PARAM;
    Fields F;
    int st = fetch(h, F, false, false);
    if (st != LBM_OK) return st;
    if (F.p.dim != 2) return LBM_ERR_PARAM;
    const int nx = F.p.nx, ny = F.p.ny;
    const double L = F.c.lengthUnit;
    std::vector<double> psi(F.n), vort(F.n);
    if ((st = lbm_psi_vort_2d(nx, ny, L, F.c.velocityScaleCompare, F.u.data(), F.v.data(), psi.data(), vort.data())))
        return st;
    double centre = 0.0;
    if ((st = lbm_psi_center_2d(nx, ny, L, psi.data(), &centre))) return st;
    out->psi_center = centre;
    out->psi_center_abs = std::fabs(centre);
    if (prefix && (st = lbm_tecplot_psi_vort_2d(numbered(prefix, "psiVort-", number, ".plt").c_str(), nx, ny, L,
                                                psi.data(), vort.data())))
        return st;
    return lbm_psi_absmax_fine_spline(nx, ny, L, psi.data(), nFinePerUnit, &out->psi_abs_max, &out->x_at_max,
                                      &out->y_at_max, &out->psi_center_abs_fine);
}
