// Host check of the in-place (AA) access-pattern helpers of csrc/lbm_device.cuh, compiled as
// plain C++ (the device qualifiers are defined away).  On small lattices with every
// combination of boundary kinds it runs the two-buffer pull and the in-place sweeps side
// by side, with a random linear "collision" per cell and the cells of each sweep in a
// random order, and checks that
//   - every slot index is in range;
//   - an odd sweep writes every streamed slot exactly once and no cell writes a slot that
//     another cell reads in that sweep (periodic faces are read from the snapshot);
//   - after every step the module view of the in-place array equals the two-buffer pull,
//     bit for bit, thermal wall terms included.
// Exit status 0 and "ok" on success; the first failure is printed.
#define __host__
#define __device__
#define __forceinline__ inline
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>
#include <set>
#include <map>
#include <algorithm>
#include "lbm_device.cuh"
using namespace lbm;

static void die(const char* m, long long a = 0, long long b = 0) { std::printf("FAIL %s %lld %lld\n", m, a, b); std::exit(1); }

template <int Q, bool TH>
static void run(Geo g, int steps, unsigned seed) {
    const long long n = g.ncell;
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(-1, 1);
    std::vector<double> M((size_t)n * Q * Q);
    for (auto& x : M) x = U(rng) * 0.3;
    auto collide = [&](long long c, const double* in, double* out) {
        for (int r = 0; r < Q; ++r) { double s = 0; for (int q = 0; q < Q; ++q) s += M[(c * Q + r) * Q + q] * in[q]; out[r] = s; }
    };
    std::vector<double> module0((size_t)Q * n);
    for (auto& x : module0) x = U(rng);
    auto chk = [&](long long idx, long long size) { if (idx < 0 || idx >= size) die("index", idx, size); return idx; };
    auto pull = [&](const std::vector<double>& arr, int a, int i, int j, int k, long long c, bool swapped) {
        auto ld = [&](int b, long long cc) { return arr[chk((long long)(swapped ? Lat<Q>::opp(b) : b) * n + chk(cc, n), (long long)Q * n)]; };
        return TH ? pull_thermal<Q, double>(g, a, i, j, k, c, ld) : pull_flow<Q, double>(g, a, i, j, k, c, ld);
    };
    // A/B
    std::vector<double> fpost((size_t)Q * n), nf((size_t)Q * n);
    for (long long c = 0; c < n; ++c) { double in[Q], out[Q]; for (int a = 0; a < Q; ++a) in[a] = module0[a * n + c]; collide(c, in, out); for (int a = 0; a < Q; ++a) fpost[a * n + c] = out[a]; }
    std::vector<std::vector<double>> abv;
    for (int s = 0; s < steps; ++s) {
        std::vector<double> view((size_t)Q * n);
        for (long long c = 0; c < n; ++c) { int i, j, k; long long pl = (long long)g.nx * g.ny; k = c / pl; j = (c % pl) / g.nx; i = c % g.nx;
            for (int a = 0; a < Q; ++a) view[a * n + c] = pull(fpost, a, i, j, k, c, false); }
        abv.push_back(view);
        for (long long c = 0; c < n; ++c) { double in[Q], out[Q]; for (int a = 0; a < Q; ++a) in[a] = view[a * n + c]; collide(c, in, out); for (int a = 0; a < Q; ++a) nf[a * n + c] = out[a]; }
        fpost.swap(nf);
    }
    // AA
    std::vector<double> A = module0;
    int par = 0; bool raw = false;
    std::vector<double> face[3];
    bool per[3];
    for (int ax = 0; ax < 3; ++ax) { per[ax] = TH ? pick3(g.bct, ax) == LBM_BCT_PERIODIC : pick3(g.bcf, ax) == LBM_BC_PERIODIC;
        if (per[ax]) face[ax].assign((size_t)Q * aa_face_cells(g, ax), 0.0); }
    std::vector<int> order(n); for (long long c = 0; c < n; ++c) order[c] = (int)c;
    for (int s = 0; s < steps; ++s) {
        std::shuffle(order.begin(), order.end(), rng);
        if (par == 0) {
            for (int c : order) { int i, j, k; long long pl = (long long)g.nx * g.ny; k = c / pl; j = (c % pl) / g.nx; i = c % g.nx;
                double in[Q], out[Q];
                for (int a = 0; a < Q; ++a) {
                    auto ld = [&](int b, long long cc) { return A[chk((long long)b * n + chk(cc, n), (long long)Q * n)]; };
                    in[a] = TH ? aa_local_thermal<Q, double>(g, a, i, j, k, c, raw, ld) : ld(a, c);
                }
                collide(c, in, out);
                for (int a = 0; a < Q; ++a) A[chk((long long)Lat<Q>::opp(a) * n + c, (long long)Q * n)] = out[a];
            }
            par = 1;
        } else {
            // snapshot (k_aa_face logic)
            for (int ax = 0; ax < 3; ++ax) if (per[ax]) {
                const long long nfc = aa_face_cells(g, ax);
                for (long long e = 0; e < Q * nfc; ++e) { int a = e / nfc; long long f = e - (long long)a * nfc;
                    int ea = ax == 0 ? Lat<Q>::ex(a) : (ax == 1 ? Lat<Q>::ey(a) : Lat<Q>::ez(a)); if (!ea) continue;
                    int i, j, k;
                    if (ax == 0) { j = f % g.ny; k = f / g.ny; i = ea > 0 ? g.nx - 1 : 0; }
                    else if (ax == 1) { i = f % g.nx; k = f / g.nx; j = ea > 0 ? g.ny - 1 : 0; }
                    else { i = f % g.nx; j = f / g.nx; k = ea > 0 ? g.nz - 1 : 0; }
                    face[ax][e] = A[chk((long long)Lat<Q>::opp(a) * n + cell_index(g, i, j, k), (long long)Q * n)]; }
            }
            std::map<long long, int> writer; std::map<long long, std::set<int>> readers;
            for (int c : order) { int i, j, k; long long pl = (long long)g.nx * g.ny; k = c / pl; j = (c % pl) / g.nx; i = c % g.nx;
                double in[Q], out[Q];
                auto ld = [&](int b, long long cc) { long long slot = chk((long long)Lat<Q>::opp(b) * n + chk(cc, n), (long long)Q * n);
                    readers[slot].insert(c); if (writer.count(slot) && writer[slot] != c) die("read after foreign write", slot, c); return A[slot]; };
                auto wr = [&](int ax, int b, long long) { if (!per[ax]) die("face of non-periodic axis", ax, c);
                    return face[ax][chk((long long)b * aa_face_cells(g, ax) + aa_face_index(g, ax, i, j, k), (long long)face[ax].size())]; };
                for (int a = 0; a < Q; ++a) in[a] = TH ? pull_thermal_w<Q, double>(g, a, i, j, k, c, ld, wr) : pull_flow_w<Q, double>(g, a, i, j, k, c, ld, wr);
                collide(c, in, out);
                auto st = [&](int b, long long cc, double v) { long long slot = chk((long long)b * n + chk(cc, n), (long long)Q * n);
                    if (writer.count(slot)) die("slot written twice", slot, c);
                    for (int r : readers[slot]) if (r != c) die("write over a foreign read", slot, c);
                    writer[slot] = c; A[slot] = v; };
                for (int a = 0; a < Q; ++a) aa_push<Q, TH, double>(g, a, i, j, k, c, out[a], st);
            }
            // every streamed slot is written exactly once
            if ((long long)writer.size() != (long long)Q * n) die("streamed slots written", writer.size(), Q * n);
            par = 0; raw = true;
        }
        // module view vs A/B
        for (long long c = 0; c < n; ++c) { int i, j, k; long long pl = (long long)g.nx * g.ny; k = c / pl; j = (c % pl) / g.nx; i = c % g.nx;
            for (int a = 0; a < Q; ++a) {
                double v;
                if (par) v = pull(A, a, i, j, k, c, true);
                else { auto ld = [&](int b, long long cc) { return A[b * n + cc]; }; v = TH ? aa_local_thermal<Q, double>(g, a, i, j, k, c, raw, ld) : ld(a, c); }
                if (v != abv[s][a * n + c]) die("view differs", s, c * Q + a);
            } }
    }
}


int main() {
    int ncase = 0;
    for (int d = 2; d <= 3; ++d) for (int bx = 0; bx < 3; ++bx) for (int bz = 0; bz < 2; ++bz) for (int by = 0; by < 2; ++by) {
        if (d == 2 && bz) continue;
        Geo g{};
        g.nx = d == 2 ? 7 : 5; g.ny = 6; g.nz = d == 2 ? 1 : 4; g.ncell = (long long)g.nx * g.ny * g.nz;
        // flow: x no-slip/periodic, y no-slip, z no-slip/periodic; thermal: x const/adiabatic/periodic, y const/adiabatic
        g.bcf[0] = bx == 2 ? LBM_BC_PERIODIC : LBM_BC_NOSLIP; g.bcf[1] = LBM_BC_NOSLIP; g.bcf[2] = bz ? LBM_BC_PERIODIC : LBM_BC_NOSLIP;
        g.bct[0] = bx == 0 ? LBM_BCT_CONST : (bx == 1 ? LBM_BCT_ADIABATIC : LBM_BCT_PERIODIC);
        g.bct[1] = by ? LBM_BCT_ADIABATIC : LBM_BCT_CONST; g.bct[2] = bz ? LBM_BCT_PERIODIC : LBM_BCT_ADIABATIC;
        for (int a = 0; a < 3; ++a) { g.bcT_lo[a] = 0.37 + a; g.bcT_hi[a] = -0.21 - a; }
        if (d == 2) { run<9, false>(g, 6, 11 + ncase); run<5, true>(g, 6, 12 + ncase); }
        else { run<19, false>(g, 6, 13 + ncase); run<7, true>(g, 6, 14 + ncase); }
        ++ncase;
    }
    std::printf("ok: %d geometries, flow and thermal, 6 steps each\n", ncase);
    return 0;
}
