// lbm_device.cuh - lattice tables, index arithmetic and the pull-with-boundary rule shared
// by every kernel of the library (exact FP64, FP32/FP16 storage, reductions).
//
// Layout in HBM: structure of arrays, one plane of `ncell` values per direction,
// cell index c = i + nx*(j + ny*k) with 0-based i,j,k (x fastest, so a warp reads 32
// consecutive cells of one direction: fully coalesced).  No ghost layers are stored;
// the reference's ghost-padded f_post (3DRB.F90:472) is replaced by the boundary rule
// below, evaluated inside the streaming pull.
#pragma once

#include <cstdint>

#include "../../include/lbm_gpu.h"

namespace lbm {

// ------------------------------------------------------------------------------------
// Lattice velocity sets.  D2Q9 order 0,E,N,W,S,NE,NW,SW,SE (2DRB.F90:189-190); D2Q5 is
// its first five.  D3Q19 / D3Q7 order and opposites from 3DRB.F90:655-667.  The tables
// are constexpr functions so that fully unrolled loops fold them into immediates.
// ------------------------------------------------------------------------------------
template <int Q> struct Lat;

template <> struct Lat<9> {
    static constexpr int D = 2;
    __host__ __device__ static constexpr int ex(int a) { return (a == 1 || a == 5 || a == 8) ? 1 : (a == 3 || a == 6 || a == 7) ? -1 : 0; }
    __host__ __device__ static constexpr int ey(int a) { return (a == 2 || a == 5 || a == 6) ? 1 : (a == 4 || a == 7 || a == 8) ? -1 : 0; }
    __host__ __device__ static constexpr int ez(int) { return 0; }
    __host__ __device__ static constexpr int opp(int a) { return a == 0 ? 0 : (a <= 4 ? ((a + 1) % 4) + 1 : ((a - 5 + 2) % 4) + 5); }
};
template <> struct Lat<5> {
    static constexpr int D = 2;
    __host__ __device__ static constexpr int ex(int a) { return Lat<9>::ex(a); }
    __host__ __device__ static constexpr int ey(int a) { return Lat<9>::ey(a); }
    __host__ __device__ static constexpr int ez(int) { return 0; }
    __host__ __device__ static constexpr int opp(int a) { return Lat<9>::opp(a); }
};
template <> struct Lat<19> {
    static constexpr int D = 3;
    __host__ __device__ static constexpr int ex(int a) {
        return (a == 1 || a == 7 || a == 9 || a == 11 || a == 13) ? 1 : (a == 2 || a == 8 || a == 10 || a == 12 || a == 14) ? -1 : 0;
    }
    __host__ __device__ static constexpr int ey(int a) {
        return (a == 3 || a == 7 || a == 8 || a == 15 || a == 17) ? 1 : (a == 4 || a == 9 || a == 10 || a == 16 || a == 18) ? -1 : 0;
    }
    __host__ __device__ static constexpr int ez(int a) {
        return (a == 5 || a == 11 || a == 12 || a == 15 || a == 16) ? 1 : (a == 6 || a == 13 || a == 14 || a == 17 || a == 18) ? -1 : 0;
    }
    __host__ __device__ static constexpr int opp(int a) {
        return a == 0 ? 0 : (a <= 6 ? (a % 2 == 1 ? a + 1 : a - 1)
                                    : (a <= 10 ? 17 - a : (a <= 14 ? 25 - a : 33 - a)));
    }
};
template <> struct Lat<7> {
    static constexpr int D = 3;
    __host__ __device__ static constexpr int ex(int a) { return Lat<19>::ex(a); }
    __host__ __device__ static constexpr int ey(int a) { return Lat<19>::ey(a); }
    __host__ __device__ static constexpr int ez(int a) { return Lat<19>::ez(a); }
    __host__ __device__ static constexpr int opp(int a) { return Lat<19>::opp(a); }
};

static_assert(Lat<9>::opp(1) == 3 && Lat<9>::opp(2) == 4 && Lat<9>::opp(3) == 1 && Lat<9>::opp(4) == 2, "d2q9 opp");
static_assert(Lat<9>::opp(5) == 7 && Lat<9>::opp(6) == 8 && Lat<9>::opp(7) == 5 && Lat<9>::opp(8) == 6, "d2q9 opp");
static_assert(Lat<19>::opp(7) == 10 && Lat<19>::opp(8) == 9 && Lat<19>::opp(11) == 14 && Lat<19>::opp(12) == 13, "d3q19 opp");
static_assert(Lat<19>::opp(15) == 18 && Lat<19>::opp(16) == 17 && Lat<19>::opp(5) == 6 && Lat<19>::opp(2) == 1, "d3q19 opp");

// ------------------------------------------------------------------------------------
// Geometry and boundary switches of one lattice, passed by value to every kernel.
// ------------------------------------------------------------------------------------
struct Geo {
    int nx, ny, nz;      // nz = 1 in 2D
    long long ncell;
    int bcf[3];          // LBM_BC_* per axis
    int bct[3];          // LBM_BCT_* per axis
    double bcT_lo[3];    // anti-bounce-back source term at the low face of each axis
    double bcT_hi[3];    // ... and at the high face
};

// Select element `axis` of a 3-array without a runtime-indexed access (which would copy a
// by-value kernel parameter to local memory).
template <class T>
__host__ __device__ __forceinline__ T pick3(const T (&a)[3], int axis) {
    return axis == 0 ? a[0] : (axis == 1 ? a[1] : a[2]);
}

__host__ __device__ inline long long cell_index(const Geo& g, int i, int j, int k) {
    return (long long)i + (long long)g.nx * ((long long)j + (long long)g.ny * (long long)k);
}

// Index checks of the CPU builds of the shared cell code (compiled with -DLBM_CHECK by the
// host tests, together with the address and undefined-behaviour sanitizers); nothing in a
// GPU build.
#if defined(LBM_CHECK) && !defined(__CUDA_ARCH__)
}  // namespace lbm
#include <cassert>
namespace lbm {
#define LBM_CHECK_CELL(g, cc) assert((cc) >= 0 && (cc) < (g).ncell)
#else
#define LBM_CHECK_CELL(g, cc) ((void)0)
#endif

// Pull of direction `a` into cell (i,j,k) from a post-collision array, with the
// reference's boundary handling folded in.
//
// The reference streams from a zero ghost layer and then overwrites the incoming
// directions face by face in a fixed order: x faces, then y, then z
// (3DRB.F90:987-1058, 2DRB.F90:811-866).  For a direction whose source lies outside
// the lattice along one or more axes the last of those faces wins, so the value is
// the boundary rule of the last out-of-range axis:
//   no-slip  : f_post(opp(a)) of the same cell (half-way bounce-back);
//   periodic : f_post(a) of the cell wrapped along that axis only, other indices
//              unchanged (the reference's same-row copy, 2DRB.F90:821-828).
// LOAD(dir, cell) returns the stored value converted to the arithmetic type.
template <int Q, class T, class LOAD, class WRAP>
__device__ __forceinline__ T pull_flow_w(const Geo& g, int a, int i, int j, int k, long long c, LOAD load, WRAP wrap) {
    const int si = i - Lat<Q>::ex(a), sj = j - Lat<Q>::ey(a), sk = k - Lat<Q>::ez(a);
    int axis = -1;
    if (Lat<Q>::ex(a) != 0 && (si < 0 || si >= g.nx)) axis = 0;
    if (Lat<Q>::ey(a) != 0 && (sj < 0 || sj >= g.ny)) axis = 1;
    if (Lat<Q>::ez(a) != 0 && (sk < 0 || sk >= g.nz)) axis = 2;
    if (axis < 0) {
        const long long off = (long long)(-Lat<Q>::ex(a)) + (long long)g.nx * ((long long)(-Lat<Q>::ey(a)) + (long long)g.ny * (long long)(-Lat<Q>::ez(a)));
        LBM_CHECK_CELL(g, c + off);
        return load(a, c + off);
    }
    if (pick3(g.bcf, axis) == LBM_BC_NOSLIP) return load(Lat<Q>::opp(a), c);
    if (axis == 0) return wrap(0, a, cell_index(g, si < 0 ? g.nx - 1 : 0, j, k));
    if (axis == 1) return wrap(1, a, cell_index(g, i, sj < 0 ? g.ny - 1 : 0, k));
    return wrap(2, a, cell_index(g, i, j, sk < 0 ? g.nz - 1 : 0));
}

// The same with the periodic source read like any other: WRAP(axis, dir, cell) is the hook
// the in-place (AA) pattern uses to read face values from a snapshot.
template <int Q, class T, class LOAD>
__device__ __forceinline__ T pull_flow(const Geo& g, int a, int i, int j, int k, long long c, LOAD load) {
    return pull_flow_w<Q, T>(g, a, i, j, k, c, load, [&](int, int d, long long cc) { return load(d, cc); });
}

// Thermal pull (D2Q5 / D3Q7, axis-aligned: at most one axis out of range), with the
// bouncebackT rules (3DRB.F90:1243-1351, 2DRB.F90:1026-1107):
//   constant T : -g_post(opp(a)) + bc term (2*omegaT*Tw, Tw = Thot low face / Tcold high);
//   adiabatic  :  g_post(opp(a));
//   periodic   :  g_post(a) of the wrapped cell.
template <int QT, class T, class LOAD, class WRAP>
__device__ __forceinline__ T pull_thermal_w(const Geo& g, int a, int i, int j, int k, long long c, LOAD load, WRAP wrap) {
    if (a == 0) return load(0, c);
    const int si = i - Lat<QT>::ex(a), sj = j - Lat<QT>::ey(a), sk = k - Lat<QT>::ez(a);
    int axis = -1;
    bool low = false;
    if (Lat<QT>::ex(a) != 0 && (si < 0 || si >= g.nx)) { axis = 0; low = si < 0; }
    if (Lat<QT>::ey(a) != 0 && (sj < 0 || sj >= g.ny)) { axis = 1; low = sj < 0; }
    if (Lat<QT>::ez(a) != 0 && (sk < 0 || sk >= g.nz)) { axis = 2; low = sk < 0; }
    if (axis < 0) {
        const long long off = (long long)(-Lat<QT>::ex(a)) + (long long)g.nx * ((long long)(-Lat<QT>::ey(a)) + (long long)g.ny * (long long)(-Lat<QT>::ez(a)));
        LBM_CHECK_CELL(g, c + off);
        return load(a, c + off);
    }
    const int bt = pick3(g.bct, axis);
    if (bt == LBM_BCT_CONST) return -load(Lat<QT>::opp(a), c) + (T)(low ? pick3(g.bcT_lo, axis) : pick3(g.bcT_hi, axis));
    if (bt == LBM_BCT_ADIABATIC) return load(Lat<QT>::opp(a), c);
    if (axis == 0) return wrap(0, a, cell_index(g, si < 0 ? g.nx - 1 : 0, j, k));
    if (axis == 1) return wrap(1, a, cell_index(g, i, sj < 0 ? g.ny - 1 : 0, k));
    return wrap(2, a, cell_index(g, i, j, sk < 0 ? g.nz - 1 : 0));
}

template <int QT, class T, class LOAD>
__device__ __forceinline__ T pull_thermal(const Geo& g, int a, int i, int j, int k, long long c, LOAD load) {
    return pull_thermal_w<QT, T>(g, a, i, j, k, c, load, [&](int, int d, long long cc) { return load(d, cc); });
}

// Row launches.  Interior rows (0 < j < ny-1, and 0 < k < nz-1 in 3D): block (bx, j-1, k-1)
// holds cells i = bx*blockDim.x + t of row (j, k), so warps start at row starts and every
// access of a warp is one contiguous run; only x can take a pull source outside the lattice
// there.  Face rows: the y faces (j = 0, ny-1; every k), then in 3D the z faces (k = 0,
// nz-1; 0 < j < ny-1); block (bx, r) holds cells i = bx*blockDim.x + t of face row r.
#if defined(__CUDACC__)
__device__ __forceinline__ bool row_interior_cell(const Geo& g, long long& c, int& i, int& j, int& k) {
    i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    j = (int)blockIdx.y + 1;
    k = g.nz > 1 ? (int)blockIdx.z + 1 : 0;
    if (i >= g.nx) return false;
    c = (long long)i + (long long)g.nx * ((long long)j + (long long)g.ny * (long long)k);
    return true;
}
#endif
__host__ __device__ __forceinline__ long long face_row_count(const Geo& g) {
    return 2LL * g.nz + (g.nz > 1 ? 2LL * (g.ny - 2) : 0LL);
}
#if defined(__CUDACC__)
__device__ __forceinline__ bool row_face_cell(const Geo& g, long long& c, int& i, int& j, int& k) {
    i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= g.nx) return false;
    const int r = (int)blockIdx.y;
    if (r < 2 * g.nz) {
        j = (r & 1) ? g.ny - 1 : 0;
        k = r >> 1;
    } else {
        const int s = r - 2 * g.nz;
        k = (s & 1) ? g.nz - 1 : 0;
        j = 1 + (s >> 1);
    }
    c = (long long)i + (long long)g.nx * ((long long)j + (long long)g.ny * (long long)k);
    return true;
}
#endif
// The row launches need interior rows: ny >= 3 and, in 3D, nz >= 3.
__host__ __device__ __forceinline__ bool row_launch_supported(const Geo& g) {
    return g.ny >= 3 && (g.nz == 1 || g.nz >= 3);
}

// Pulls of a cell whose row is interior (0 < j < ny-1 and, in 3D, 0 < k < nz-1): only the x
// axis can take a source outside the lattice, at i = 0 or nx-1.  The rule is pull_flow's /
// pull_thermal's for that case, written with selects so that every lane of a warp runs the
// same instructions (x-face lanes share warps with interior ones).
// I: the cell-index type (long long; int where every index of the arrays fits in 32 bits,
// which halves the address arithmetic).
template <int Q, class T, class LOAD, class I = long long>
__device__ __forceinline__ T pull_flow_xrow(const Geo& g, int a, int i, I c, LOAD load) {
    const I off = (I)Lat<Q>::ex(a) + (I)g.nx * ((I)Lat<Q>::ey(a) + (I)g.ny * (I)Lat<Q>::ez(a));
    if (Lat<Q>::ex(a) == 0) return load(a, c - off);
    const int si = i - Lat<Q>::ex(a);
    const bool out = si < 0 || si >= g.nx;
    if (g.bcf[0] == LBM_BC_NOSLIP) return out ? load(Lat<Q>::opp(a), c) : load(a, c - off);
    // periodic: the same-row copy from the other end of the row (j and k unchanged, also
    // for the diagonal directions: the reference's x-periodic copy, 2DRB.F90:821-828)
    return load(a, out ? c + (I)Lat<Q>::ex(a) * (I)(g.nx - 1) : c - off);
}
template <int QT, class T, class LOAD, class I = long long>
__device__ __forceinline__ T pull_thermal_xrow(const Geo& g, int a, int i, I c, LOAD load) {
    const I off = (I)Lat<QT>::ex(a) + (I)g.nx * ((I)Lat<QT>::ey(a) + (I)g.ny * (I)Lat<QT>::ez(a));
    if (Lat<QT>::ex(a) == 0) return load(a, c - off);
    const int si = i - Lat<QT>::ex(a);
    const bool out = si < 0 || si >= g.nx;
    const int bt = g.bct[0];
    if (bt == LBM_BCT_PERIODIC) return load(a, out ? c + (I)Lat<QT>::ex(a) * (I)(g.nx - 1) : c - off);
    const T v = out ? load(Lat<QT>::opp(a), c) : load(a, c - off);
    if (bt == LBM_BCT_CONST && out) return -v + (T)(si < 0 ? g.bcT_lo[0] : g.bcT_hi[0]);
    return v;
}

// ------------------------------------------------------------------------------------
// In-place (AA) access pattern.  One array per lattice; its layout alternates:
//   parity 0 ("streamed"): slot (a, x) holds the streamed population f_a(x), i.e. what the
//            pull above returns -- the reference's module array f;
//   parity 1 ("swapped") : slot (opp(a), x) holds the post-collision f_post_a(x).
// An even sweep reads a cell's own slots and writes its post-collision values back into
// the opposite slots of the same cell.  An odd sweep pulls through the swapped layout
// (dir d of cell s lives in slot (opp(d), s)) and pushes each post-collision value to
// every slot that the next pull resolves to it, so the array is streamed again.  Every
// slot an odd sweep writes is read in that sweep only by the cell that writes it, except
// across a periodic face: those reads come from a snapshot of the face slots taken before
// the sweep (aa_face_index indexes it).  The boundary rules are the pull's, so the
// sequence of states equals the two-buffer sequence value for value.
// ------------------------------------------------------------------------------------
// Index of cell (i,j,k) in the face plane normal to `axis`.
__device__ __forceinline__ long long aa_face_index(const Geo& g, int axis, int i, int j, int k) {
    return axis == 0 ? (long long)j + (long long)g.ny * k
                     : (axis == 1 ? (long long)i + (long long)g.nx * k : (long long)i + (long long)g.nx * j);
}
__host__ __device__ inline long long aa_face_cells(const Geo& g, int axis) {
    return axis == 0 ? (long long)g.ny * g.nz : (axis == 1 ? (long long)g.nx * g.nz : (long long)g.nx * g.ny);
}

// A cell that touches no face of the lattice: every pull source and push target of it is
// the neighbour at offset -e_a / +e_a, with no boundary rule.
__device__ __forceinline__ bool aa_inner(const Geo& g, int i, int j, int k) {
    return i > 0 && i < g.nx - 1 && j > 0 && j < g.ny - 1 && (g.nz == 1 || (k > 0 && k < g.nz - 1));
}
template <int Q>
__device__ __forceinline__ long long lat_off(const Geo& g, int a) {
    return (long long)Lat<Q>::ex(a) + (long long)g.nx * ((long long)Lat<Q>::ey(a) + (long long)g.ny * (long long)Lat<Q>::ez(a));
}

// Face snapshots of one array (one pointer per axis, null where the axis is not periodic).
template <class S>
struct AAFace {
    const S *p0, *p1, *p2;
};
template <class S>
__device__ __forceinline__ const S* aa_face_ptr(const AAFace<S>& w, int axis) {
    return axis == 0 ? w.p0 : (axis == 1 ? w.p1 : w.p2);
}

// Push of the post-collision value v of direction a at cell (i,j,k) (odd sweep).
// STORE(slot_dir, cell, value) writes the streamed layout.  Values are stored as they
// leave the collision: a slot filled across a constant-temperature wall holds the raw
// g_post, and the reader applies -g + 2 w T_w (aa_local_thermal), so the stored number and
// the arithmetic on it are those of the two-buffer pull.  THERMAL selects the thermal
// boundary table.
template <int Q, bool THERMAL, class T, class STORE>
__device__ __forceinline__ void aa_push(const Geo& g, int a, int i, int j, int k, long long c, T v, STORE store) {
    const int ex = Lat<Q>::ex(a), ey = Lat<Q>::ey(a), ez = Lat<Q>::ez(a);
    const int ti = i + ex, tj = j + ey, tk = k + ez;
    const bool ox = ex != 0 && (ti < 0 || ti >= g.nx);
    const bool oy = ey != 0 && (tj < 0 || tj >= g.ny);
    const bool oz = ez != 0 && (tk < 0 || tk >= g.nz);
    if (!ox && !oy && !oz) {
        store(a, c + (long long)ex + (long long)g.nx * ((long long)ey + (long long)g.ny * (long long)ez), v);
        return;
    }
    auto periodic = [&](int axis) {
        return THERMAL ? pick3(g.bct, axis) == LBM_BCT_PERIODIC : pick3(g.bcf, axis) == LBM_BC_PERIODIC;
    };
    // the pull of opp(a) into this cell has the target as its source and is resolved on
    // the last out-of-range axis of the target: a wall returns this value
    const int ax = oz ? 2 : (oy ? 1 : 0);
    if (!periodic(ax)) store(Lat<Q>::opp(a), c, v);
    // the cell wrapped along an out-of-range periodic axis pulls this value when no later
    // axis of its own source is out of range
    const bool iy = ey != 0 && (j - ey < 0 || j - ey >= g.ny);
    const bool iz = ez != 0 && (k - ez < 0 || k - ez >= g.nz);
    if (ox && periodic(0) && !iy && !iz) store(a, cell_index(g, ti < 0 ? g.nx - 1 : 0, j, k), v);
    if (oy && periodic(1) && !iz) store(a, cell_index(g, i, tj < 0 ? g.ny - 1 : 0, k), v);
    if (oz && periodic(2)) store(a, cell_index(g, i, j, tk < 0 ? g.nz - 1 : 0), v);
}

// Thermal population a of cell (i,j,k) from the streamed layout.  raw: the slot was filled
// by a push, so a constant-temperature wall's rule is still to be applied (slots written
// from module data -- initial, a state load -- already hold the module value).
template <int QT, class T, class LOAD>
__device__ __forceinline__ T aa_local_thermal(const Geo& g, int a, int i, int j, int k, long long c, bool raw, LOAD load) {
    const T v = load(a, c);
    if (a == 0 || !raw) return v;
    const int si = i - Lat<QT>::ex(a), sj = j - Lat<QT>::ey(a), sk = k - Lat<QT>::ez(a);
    int axis = -1;
    bool low = false;
    if (Lat<QT>::ex(a) != 0 && (si < 0 || si >= g.nx)) { axis = 0; low = si < 0; }
    if (Lat<QT>::ey(a) != 0 && (sj < 0 || sj >= g.ny)) { axis = 1; low = sj < 0; }
    if (Lat<QT>::ez(a) != 0 && (sk < 0 || sk >= g.nz)) { axis = 2; low = sk < 0; }
    if (axis < 0 || pick3(g.bct, axis) != LBM_BCT_CONST) return v;
    return -v + (T)(low ? pick3(g.bcT_lo, axis) : pick3(g.bcT_hi, axis));
}

// Decompose a linear thread index into (i,j,k).
__device__ __forceinline__ void cell_coords(const Geo& g, long long c, int& i, int& j, int& k) {
    const long long plane = (long long)g.nx * g.ny;
    k = (int)(c / plane);
    const long long r = c - (long long)k * plane;
    j = (int)(r / g.nx);
    i = (int)(r - (long long)j * g.nx);
}

// splitmix64 of (seed ^ cell) -> [0,1) with 53 random bits; integer-exact on host and device.
__host__ __device__ inline double noise_xi(uint64_t seed, uint64_t idx) {
    uint64_t z = (seed ^ idx) + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace lbm
