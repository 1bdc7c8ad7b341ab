// CPU oracle for the 2D path (TEST INFRASTRUCTURE ONLY). Pinned, like the 3D oracle, to
// golden vectors made by the reference's own 2D solver code run on the host
// (oracle/ref_emu, tests/golden/make_ref_golden.py): operators, transfers, smoothers,
// coarsest solve, V-cycle and GMRES agree bit for bit or to round-off.
//
// Restates, in the reference's own 8x8-blocked solver layout
// [cells | x-faces | y-faces] (common_cpx/form01mapping.cu:10-57):
//   the operator A   stoke/StokeFlowMapping.cu:30-139 (no definite fix: fixed rows are 0)
//   the energy E     fluid_topo/FluidEnergyGrad.cu:30-61 (5-point face Laplacian + P x)
//   coarsening       stoke/StokeFlowSubSystem.cu:100-160 (lap_coeff doubles per level)
//   transfers        stoke/StokeFlowSubSystem.cu:32-98, common_cpx/SubSystemUtils.cuh
//   smoother         stoke/StokeFlowSmoothing.cu:8-209 (5-DOF box, 2x2 velocity blocks)
//   coarsest solve   stoke/StokeFlowDirectSolve.cpp:6-179 (analytic dense matrix + LU)
//   V-cycle / GMRES  common_cpx/MultigridSolve.cpp:73-114, common_cpx/GMRES.cpp:20-110
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "krylov.h"

namespace orc2 {

using orc::KrylovStats;
using orc::VecOp;

// common_cpx/form01mapping.cu:10-57 (faces padded by 8 along their normal)
struct G2 {
    int nx = 0, ny = 0;
    int cell_size() const { return nx * ny; }
    int face_size(int d) const { return (nx + 8 * (d == 0)) * (ny + 8 * (d == 1)); }
    int node_size() const { return (nx + 8) * (ny + 8); }
    int size() const { return cell_size() + face_size(0) + face_size(1); }
    int face_off(int d) const { return cell_size() + (d == 1 ? face_size(0) : 0); }
    int cell_ind(int x, int y) const { return ((y >> 3) * (nx >> 3) + (x >> 3)) * 64 + ((y & 7) * 8 + (x & 7)); }
    int face_ind(int x, int y, int d) const {
        int b = (y >> 3) * ((nx >> 3) + (d == 0)) + (x >> 3);
        int ix = x & 7, iy = y & 7;
        return b * 64 + (d == 0 ? ix * 8 + iy : iy * 8 + ix);
    }
    int node_ind(int x, int y) const { return ((y >> 3) * ((nx >> 3) + 1) + (x >> 3)) * 64 + ((y & 7) * 8 + (x & 7)); }
    bool face_valid(int x, int y, int d) const {
        return x >= 0 && y >= 0 && (d == 0 ? (x <= nx && y < ny) : (x < nx && y <= ny));
    }
    bool cell_valid(int x, int y) const { return x >= 0 && y >= 0 && x < nx && y < ny; }
    // stored (padded) face range: x-faces x < nx+8, y < ny; y-faces x < nx, y < ny+8
    bool face_stored(int x, int y, int d) const {
        return x >= 0 && y >= 0 && (d == 0 ? (x < nx + 8 && y < ny) : (x < nx && y < ny + 8));
    }
};

struct Descr2 {
    G2 g;
    double lap = 1.0;
    std::vector<double> vol, pen;
    std::vector<uint8_t> fixed;
    void init(int n) {
        g.nx = g.ny = n;
        vol.assign(g.size(), 0.0);
        pen.assign(g.size(), 0.0);
        fixed.assign(g.size(), 0);
    }
    // StokeFlowDescriptor::finish (stoke/StokeFlowDescriptor.cpp:40-46)
    void finish() {
        for (int d = 0; d < 2; d++) {
            int off = g.face_off(d);
            int X = d == 0 ? g.nx + 8 : g.nx, Y = d == 0 ? g.ny : g.ny + 8;
            int xm = d == 0 ? g.nx + 1 : g.nx, ym = d == 0 ? g.ny : g.ny + 1;
            for (int x = 0; x < X; x++)
                for (int y = 0; y < Y; y++)
                    if (x >= xm || y >= ym) fixed[off + g.face_ind(x, y, d)] = 1;
        }
        for (int i = 0; i < g.size(); i++)
            if (fixed[i]) {
                vol[i] = 0.0;
                pen[i] = 0.0;
            }
    }
};

// ---------------------------------------------------------------- operators
// c = D1(fx, fy): -fx(x) + fx(x+1) + fy(y) - fy(y+1) (form01mapping.cu:203-252)
static void D1(const G2& g, const double* v, double* c) {
    const double *fx = v + g.face_off(0), *fy = v + g.face_off(1);
    for (int x = 0; x < g.nx; x++)
        for (int y = 0; y < g.ny; y++) {
            double d = -fx[g.face_ind(x, y, 0)];
            d += fx[g.face_ind(x + 1, y, 0)];
            d += fy[g.face_ind(x, y, 1)];
            d += -fy[g.face_ind(x, y + 1, 1)];
            c[g.cell_ind(x, y)] = d;
        }
}
// faces = Cod0(c): f(x) = c(x) - c(x-1), zero outside (form01mapping.cu:151-199)
static void Cod0(const G2& g, const double* c, double* v) {
    double *fx = v + g.face_off(0), *fy = v + g.face_off(1);
    std::fill(fx, fx + g.face_size(0), 0.0);
    std::fill(fy, fy + g.face_size(1), 0.0);
    auto cv = [&](int x, int y) { return g.cell_valid(x, y) ? c[g.cell_ind(x, y)] : 0.0; };
    for (int x = 0; x <= g.nx; x++)
        for (int y = 0; y < g.ny; y++) fx[g.face_ind(x, y, 0)] = cv(x, y) - cv(x - 1, y);
    for (int x = 0; x < g.nx; x++)
        for (int y = 0; y <= g.ny; y++) fy[g.face_ind(x, y, 1)] = cv(x, y) - cv(x, y - 1);
}
// node(x,y) = fx(x,y-1) - fx(x,y) - fy(x-1,y) + fy(x,y) on x <= nx, y <= ny (form01mapping.cu:256-300)
static void Cod1(const G2& g, const double* v, std::vector<double>& node) {
    const double *fx = v + g.face_off(0), *fy = v + g.face_off(1);
    node.assign(g.node_size(), 0.0);
    auto FX = [&](int x, int y) { return g.face_valid(x, y, 0) ? fx[g.face_ind(x, y, 0)] : 0.0; };
    auto FY = [&](int x, int y) { return g.face_valid(x, y, 1) ? fy[g.face_ind(x, y, 1)] : 0.0; };
    for (int x = 0; x <= g.nx; x++)
        for (int y = 0; y <= g.ny; y++) node[g.node_ind(x, y)] = FX(x, y - 1) - FX(x, y) - FY(x - 1, y) + FY(x, y);
}
// fx(x,y) = n(x,y+1) - n(x,y), fy(x,y) = n(x+1,y) - n(x,y) (form01mapping.cu:376-424)
static void D0(const G2& g, const std::vector<double>& node, double* v) {
    double *fx = v + g.face_off(0), *fy = v + g.face_off(1);
    std::fill(fx, fx + g.face_size(0), 0.0);
    std::fill(fy, fy + g.face_size(1), 0.0);
    for (int x = 0; x <= g.nx; x++)
        for (int y = 0; y < g.ny; y++) fx[g.face_ind(x, y, 0)] = node[g.node_ind(x, y + 1)] - node[g.node_ind(x, y)];
    for (int x = 0; x < g.nx; x++)
        for (int y = 0; y <= g.ny; y++) fy[g.face_ind(x, y, 1)] = node[g.node_ind(x + 1, y)] - node[g.node_ind(x, y)];
}

// StokeFlowMapping::applyMapping (stoke/StokeFlowMapping.cu:30-139)
void apply_A(const Descr2& D, double* Ap, const double* p) {
    const G2& g = D.g;
    const int n = g.size(), nc = g.cell_size(), f0 = g.face_off(0), f1 = g.face_off(1);
    std::vector<double> t(n), c(nc), node;
    std::fill(Ap, Ap + n, 0.0);
    // grad div v
    for (int i = f0; i < n; i++) t[i] = (i >= f1 ? -p[i] : p[i]) * D.vol[i];
    D1(g, t.data(), c.data());
    for (int i = 0; i < nc; i++) c[i] = D.fixed[i] ? 0.0 : c[i];
    for (int i = 0; i < nc; i++) c[i] = -c[i];
    Cod0(g, c.data(), t.data());
    for (int i = f0; i < n; i++) Ap[i] += D.fixed[i] ? 0.0 : t[i];
    // - curl curl v  (on the raw velocity)
    Cod1(g, p, node);
    D0(g, node, t.data());
    for (int i = f1; i < n; i++) t[i] = -t[i];
    for (int i = f0; i < n; i++) Ap[i] += t[i] * D.vol[i];
    // -grad p
    Cod0(g, p, t.data());
    for (int i = f0; i < n; i++) Ap[i] -= t[i] * D.vol[i];
    // div v
    for (int i = f0; i < n; i++) t[i] = (i >= f1 ? -p[i] : p[i]) * D.vol[i];
    D1(g, t.data(), c.data());
    for (int i = 0; i < nc; i++) Ap[i] += D.fixed[i] ? 0.0 : c[i];
    // penalty
    for (int i = 0; i < n; i++) Ap[i] += p[i] * D.pen[i];
}

// FluidEnergyGrad::applyMapping (fluid_topo/FluidEnergyGrad.cu:30-61): lap_coeff * fix(L5 u) + P x,
// L5 = 4 u - the four same-direction neighbours over the stored (padded) face arrays
// (faceLapMapping, common_cpx/form01mapping.cu:430-525)
void apply_E(const Descr2& D, double* Ap, const double* p) {
    const G2& g = D.g;
    const int n = g.size();
    std::fill(Ap, Ap + n, 0.0);
    for (int d = 0; d < 2; d++) {
        const double* f = p + g.face_off(d);
        int off = g.face_off(d);
        int X = d == 0 ? g.nx + 8 : g.nx, Y = d == 0 ? g.ny : g.ny + 8;
        auto F = [&](int x, int y) { return (x >= 0 && y >= 0 && x < X && y < Y) ? f[g.face_ind(x, y, d)] : 0.0; };
        for (int x = 0; x < X; x++)
            for (int y = 0; y < Y; y++) {
                int i = g.face_ind(x, y, d);
                double lap = 4.0 * F(x, y) - F(x - 1, y) - F(x + 1, y) - F(x, y - 1) - F(x, y + 1);
                Ap[off + i] += D.fixed[off + i] ? 0.0 : D.lap * lap;
            }
    }
    for (int i = 0; i < n; i++) Ap[i] += p[i] * D.pen[i];
}

// ---------------------------------------------------------------- coarsening and transfers
// children of coarse (X,Y): x in {2X, 2X+1}, y in {2Y, 2Y+1}; order (0,0),(1,0),(0,1),(1,1)
template <class T, class F>
static void down2(const G2& cg, const G2& fg, T* cv, const T* fv, F f) {
    for (int X = 0; X < cg.nx; X++)
        for (int Y = 0; Y < cg.ny; Y++) {
            T v[4];
            for (int q = 0; q < 4; q++) v[q] = fv[fg.cell_ind(2 * X + (q & 1), 2 * Y + (q >> 1))];
            cv[cg.cell_ind(X, Y)] = f(v, -1);
        }
    for (int d = 0; d < 2; d++) {
        T* c = cv + cg.face_off(d);
        const T* fa = fv + fg.face_off(d);
        int XX = d == 0 ? cg.nx + 8 : cg.nx, YY = d == 0 ? cg.ny : cg.ny + 8;
        for (int X = 0; X < XX; X++)
            for (int Y = 0; Y < YY; Y++) {
                T v[4];
                for (int q = 0; q < 4; q++) {
                    int x = 2 * X + (q & 1), y = 2 * Y + (q >> 1);
                    v[q] = fg.face_valid(x, y, d) ? fa[fg.face_ind(x, y, d)] : T(0);
                }
                c[cg.face_ind(X, Y, d)] = f(v, d);
            }
    }
}

// updateSubSystem (stoke/StokeFlowSubSystem.cu:100-152): fixed OR of 4, vol sum of 4 (cells)
// or of the 2 coincident children (faces), penalty sum of 4, then finish().
void update_subsystem(Descr2& c, const Descr2& f) {
    down2<uint8_t>(c.g, f.g, c.fixed.data(), f.fixed.data(), [](uint8_t* v, int) {
        return (uint8_t)(v[0] | v[1] | v[2] | v[3]);
    });
    down2<double>(c.g, f.g, c.vol.data(), f.vol.data(), [](double* v, int d) {
        if (d < 0) return v[0] + v[1] + v[2] + v[3];
        return d == 0 ? v[0] + v[2] : v[0] + v[1];
    });
    down2<double>(c.g, f.g, c.pen.data(), f.pen.data(), [](double* v, int) { return v[0] + v[1] + v[2] + v[3]; });
    c.finish();
}

// The GPU solver's own coarse penalties (its "flow rule", not in the reference): a coarse
// face that is not fixed takes 4 x the smallest penalty among its present children (none of
// which is fixed then: fixed is the OR of the children) instead of the sum.
void flow_penalties(Descr2& c, const Descr2& f) {
    const G2 &cg = c.g, &fg = f.g;
    for (int d = 0; d < 2; d++) {
        const int XX = d == 0 ? cg.nx + 8 : cg.nx, YY = d == 0 ? cg.ny : cg.ny + 8;
        for (int X = 0; X < XX; X++)
            for (int Y = 0; Y < YY; Y++) {
                if (!cg.face_valid(X, Y, d)) continue;
                const int i = cg.face_off(d) + cg.face_ind(X, Y, d);
                if (c.fixed[i]) continue;
                double lo = -1.0;
                for (int q = 0; q < 4; q++) {
                    const int x = 2 * X + (q & 1), y = 2 * Y + (q >> 1);
                    if (!fg.face_valid(x, y, d)) continue;
                    const double v = f.pen[fg.face_off(d) + fg.face_ind(x, y, d)];
                    if (lo < 0.0 || v < lo) lo = v;
                }
                if (lo >= 0.0) c.pen[i] = 4.0 * lo;
            }
    }
}

void restrict_r(const Descr2& c, const Descr2& f, double* rc, const double* rf) {
    down2<double>(c.g, f.g, rc, rf, [](double* v, int) { return v[0] + v[1] + v[2] + v[3]; });
    for (int i = 0; i < c.g.size(); i++)
        if (c.fixed[i]) rc[i] = 0.0;
}

void prolong(const Descr2& c, const Descr2& f, double* xf, const double* xc) {
    const G2 &fg = f.g, &cg = c.g;
    std::fill(xf, xf + fg.size(), 0.0);
    for (int x = 0; x < fg.nx; x++)
        for (int y = 0; y < fg.ny; y++) xf[fg.cell_ind(x, y)] = xc[cg.cell_ind(x >> 1, y >> 1)];
    for (int d = 0; d < 2; d++)
        for (int x = 0; x <= fg.nx; x++)
            for (int y = 0; y <= fg.ny; y++)
                if (fg.face_valid(x, y, d))
                    xf[fg.face_off(d) + fg.face_ind(x, y, d)] = xc[cg.face_off(d) + cg.face_ind(x >> 1, y >> 1, d)];
    for (int i = 0; i < fg.size(); i++)
        if (f.fixed[i]) xf[i] = 0.0;
}

// ---------------------------------------------------------------- smoother
// BlockInverse (stoke/StokeFlowSmoothing.cu:48-73): velocity block approximated by two
// 2x2 blocks [[4l+P0, -f],[-f, 4l+P1]] (f = l unless a face is fixed), Schur complement on p.
static void lap2x2inv(double* y, const double* x, double a, double b, double f) {
    double s = 1.0 / (a * b - f * f);
    y[0] = (b * x[0] + f * x[1]) * s;
    y[1] = (f * x[0] + a * x[1]) * s;
}
static void block_inverse(double* x, const double* r, const double* div, const double* pen, const uint8_t* fixed, double lap) {
    double f[2], vd[4], temp[4], pd = 0.0;
    f[0] = (fixed[0] || fixed[1]) ? 0.0 : lap;
    f[1] = (fixed[2] || fixed[3]) ? 0.0 : lap;
    for (int i = 0; i < 4; i++) vd[i] = 4.0 * lap + pen[i];
    lap2x2inv(temp, div, vd[0], vd[1], f[0]);
    lap2x2inv(temp + 2, div + 2, vd[2], vd[3], f[1]);
    for (int i = 0; i < 4; i++) x[i] = r[i];
    x[4] = r[4];
    for (int i = 0; i < 4; i++) x[4] -= temp[i] * r[i];
    double y[4];
    lap2x2inv(y, x, vd[0], vd[1], f[0]);
    lap2x2inv(y + 2, x + 2, vd[2], vd[3], f[1]);
    for (int i = 0; i < 4; i++) x[i] = y[i];
    for (int i = 0; i < 4; i++) pd += temp[i] * div[i];
    pd = -pd + pen[4];
    if (fixed[4])
        x[4] = 0.0;
    else
        x[4] /= pd;
    lap2x2inv(temp, div, vd[0], vd[1], f[0]);
    lap2x2inv(temp + 2, div + 2, vd[2], vd[3], f[1]);
    for (int i = 0; i < 4; i++) x[i] -= x[4] * temp[i];
}

// SmoothKernel for one colour: cells with (x + y + flag) even (stoke/StokeFlowSmoothing.cu:75-137)
void smooth_colour(const Descr2& D, int flag, double* d, const double* r) {
    const G2& g = D.g;
    std::fill(d, d + g.size(), 0.0);
    const int f0 = g.face_off(0), f1 = g.face_off(1);
    for (int x = 0; x < g.nx; x++)
        for (int y = 0; y < g.ny; y++) {
            if (((x & 1) ^ (y & 1) ^ flag) != 0) continue;
            int ind[5] = {f0 + g.face_ind(x, y, 0), f0 + g.face_ind(x + 1, y, 0), f1 + g.face_ind(x, y, 1),
                          f1 + g.face_ind(x, y + 1, 1), g.cell_ind(x, y)};
            double lr[5], lx[5], div[4], pen[5];
            uint8_t fx[5];
            for (int q = 0; q < 5; q++) {
                lr[q] = r[ind[q]];
                pen[q] = D.pen[ind[q]];
                fx[q] = D.fixed[ind[q]];
            }
            div[0] = -D.vol[ind[0]];
            div[1] = D.vol[ind[1]];
            div[2] = -D.vol[ind[2]];
            div[3] = D.vol[ind[3]];
            block_inverse(lx, lr, div, pen, fx, D.lap);
            for (int q = 0; q < 5; q++) d[ind[q]] = lx[q];
        }
}

// StokeFlowSmoothing::applyMapping (stoke/StokeFlowSmoothing.cu:172-209), iter_num 1, alpha 1
void smoother(const Descr2& D, int order, double* out, const double* p) {
    const int n = D.g.size();
    std::vector<double> r(p, p + n), d(n), Ad(n);
    std::fill(out, out + n, 0.0);
    for (int i = 0; i < 2; i++) {
        int flag = order ? 1 - i : i;
        smooth_colour(D, flag, d.data(), r.data());
        apply_A(D, Ad.data(), d.data());
        for (int q = 0; q < n; q++) {
            out[q] += d[q];
            r[q] -= Ad[q];
        }
    }
}

// ---------------------------------------------------------------- coarsest solve
// calcA + LU (stoke/StokeFlowDirectSolve.cpp:6-133)
struct Dense2 {
    int n = 0;
    std::vector<double> a;
    std::vector<int> piv;
    int info = 0;
};

static int lu(double* a, int* piv, int k) {
    int info = 0;
    for (int j = 0; j < k; j++) {
        int p = j;
        double m = std::fabs(a[j + (size_t)j * k]);
        for (int i = j + 1; i < k; i++)
            if (std::fabs(a[i + (size_t)j * k]) > m) {
                m = std::fabs(a[i + (size_t)j * k]);
                p = i;
            }
        piv[j] = p;
        if (a[p + (size_t)j * k] == 0.0) {
            if (!info) info = j + 1;
            continue;
        }
        if (p != j)
            for (int c = 0; c < k; c++) std::swap(a[j + (size_t)c * k], a[p + (size_t)c * k]);
        double inv = 1.0 / a[j + (size_t)j * k];
        for (int i = j + 1; i < k; i++) a[i + (size_t)j * k] *= inv;
        for (int c = j + 1; c < k; c++) {
            double u = a[j + (size_t)c * k];
            if (u != 0.0)
                for (int i = j + 1; i < k; i++) a[i + (size_t)c * k] -= a[i + (size_t)j * k] * u;
        }
    }
    return info;
}

void dense_setup(const Descr2& D, bool closed, Dense2& M) {
    const G2& g = D.g;
    const int size = g.size(), f0 = g.face_off(0), f1 = g.face_off(1);
    M.n = size;
    M.a.assign((size_t)size * size, 0.0);
    M.piv.assign(size, 0);
    double* A = M.a.data();
    auto at = [&](int r, int c) -> double& { return A[r + (size_t)c * size]; };
    const double lap = D.lap;
    for (int y = 0; y < g.ny; y++)
        for (int x = 0; x < g.nx; x++) {
            int ci = g.cell_ind(x, y);
            int fi;
            fi = f0 + g.face_ind(x, y, 0);
            at(ci, fi) = -D.vol[fi];
            at(fi, ci) = -D.vol[fi];
            fi = f0 + g.face_ind(x + 1, y, 0);
            at(ci, fi) = D.vol[fi];
            at(fi, ci) = D.vol[fi];
            fi = f1 + g.face_ind(x, y, 1);
            at(ci, fi) = -D.vol[fi];
            at(fi, ci) = -D.vol[fi];
            fi = f1 + g.face_ind(x, y + 1, 1);
            at(ci, fi) = D.vol[fi];
            at(fi, ci) = D.vol[fi];
        }
    if (closed)
        for (int j = 0; j < g.cell_size(); j++)
            for (int i = 0; i < g.cell_size(); i++) at(i, j) = 1.0;
    for (int x = 0; x <= g.nx; x++)
        for (int y = 0; y < g.ny; y++) {
            int fi = f0 + g.face_ind(x, y, 0);
            at(fi, fi) = 4.0 * lap;
            if (x != 0) at(f0 + g.face_ind(x - 1, y, 0), fi) = -lap;
            if (x != g.nx) at(f0 + g.face_ind(x + 1, y, 0), fi) = -lap;
            if (y != 0) at(f0 + g.face_ind(x, y - 1, 0), fi) = -lap;
            if (y != g.ny - 1) at(f0 + g.face_ind(x, y + 1, 0), fi) = -lap;
        }
    for (int y = 0; y <= g.ny; y++)
        for (int x = 0; x < g.nx; x++) {
            int fi = f1 + g.face_ind(x, y, 1);
            at(fi, fi) = 4.0 * lap;
            if (y != 0) at(f1 + g.face_ind(x, y - 1, 1), fi) = -lap;
            if (y != g.ny) at(f1 + g.face_ind(x, y + 1, 1), fi) = -lap;
            if (x != 0) at(f1 + g.face_ind(x - 1, y, 1), fi) = -lap;
            if (x != g.nx - 1) at(f1 + g.face_ind(x + 1, y, 1), fi) = -lap;
        }
    for (int i = 0; i < size; i++) at(i, i) += D.pen[i];
    for (int i = 0; i < size; i++)
        if (D.fixed[i])
            for (int j = 0; j < size; j++) at(i, j) = at(j, i) = 0.0;
    for (int i = 0; i < size; i++)
        if (D.fixed[i]) at(i, i) = 1.0;
    M.info = lu(A, M.piv.data(), size);
}

void dense_apply(const Dense2& M, double* out, const double* r) {
    const int k = M.n;
    std::copy(r, r + k, out);
    const double* a = M.a.data();
    for (int j = 0; j < k; j++)
        if (M.piv[j] != j) std::swap(out[j], out[M.piv[j]]);
    for (int j = 0; j < k; j++)
        for (int i = j + 1; i < k; i++) out[i] -= a[i + (size_t)j * k] * out[j];
    for (int j = k - 1; j >= 0; j--) {
        out[j] /= a[j + (size_t)j * k];
        for (int i = 0; i < j; i++) out[i] -= a[i + (size_t)j * k] * out[j];
    }
}

// ---------------------------------------------------------------- hierarchy, V-cycle
struct H2 {
    int l = 0;
    bool flow = false;  // coarse penalties by the GPU solver's rule instead of the sums
    std::vector<Descr2> lv;
    Descr2 energy;
    Dense2 dense;
    bool closed = true;
    std::vector<std::vector<double>> r, x, p, Ap;
    std::vector<double> b, sol;
};

// FluidSteadyState::init (stoke/FluidSteadyState.cpp:9-85): levels = log2(lowbit N) - 2
int level_count(int n) {
    int low = n & -n;
    int l = (int)std::lround(std::log2((double)low)) - 2;
    return l < 1 ? 1 : l;
}

void vcycle(H2& H) {
    for (int i = H.l - 1; i >= 0; i--) {
        const Descr2& D = H.lv[i];
        int n = D.g.size();
        auto &r = H.r[i], &x = H.x[i], &p = H.p[i], &Ap = H.Ap[i];
        std::fill(p.begin(), p.end(), 0.0);
        if (i > 0)
            smoother(D, 0, p.data(), r.data());
        else
            dense_apply(H.dense, p.data(), r.data());
        apply_A(D, Ap.data(), p.data());
        for (int q = 0; q < n; q++) {
            x[q] += p[q];
            r[q] -= Ap[q];
        }
        if (i != 0) {
            restrict_r(H.lv[i - 1], D, H.r[i - 1].data(), r.data());
            std::fill(H.x[i - 1].begin(), H.x[i - 1].end(), 0.0);
        }
    }
    for (int i = 0; i < H.l; i++) {
        const Descr2& D = H.lv[i];
        int n = D.g.size();
        auto &r = H.r[i], &x = H.x[i], &p = H.p[i], &Ap = H.Ap[i];
        if (i != 0) {
            prolong(H.lv[i - 1], D, p.data(), H.x[i - 1].data());
            apply_A(D, Ap.data(), p.data());
            for (int q = 0; q < n; q++) {
                x[q] += p[q];
                r[q] -= Ap[q];
            }
        }
        std::fill(p.begin(), p.end(), 0.0);
        if (i > 0) smoother(D, 1, p.data(), r.data());
        apply_A(D, Ap.data(), p.data());
        for (int q = 0; q < n; q++) {
            x[q] += p[q];
            r[q] -= Ap[q];
        }
    }
}

void mg_apply(H2& H, double* out, const double* in) {
    int t = H.l - 1;
    std::copy(in, in + H.lv[t].g.size(), H.r[t].begin());
    std::fill(H.x[t].begin(), H.x[t].end(), 0.0);
    vcycle(H);
    std::copy(H.x[t].begin(), H.x[t].end(), out);
}

}  // namespace orc2

using namespace orc2;

namespace {

inline int fidx2(int n, int d, int i, int j) { return i * (n + (d == 1)) + j; }

template <class T, class U>
void field_to_blocked2(const G2& g, const T* cell, const T* const f[2], U* out) {
    int n = g.nx;
    std::fill(out, out + g.size(), U(0));
    if (cell)
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) out[g.cell_ind(i, j)] = (U)cell[i * n + j];
    for (int d = 0; d < 2; d++) {
        if (!f || !f[d]) continue;
        U* o = out + g.face_off(d);
        for (int i = 0; i < n + (d == 0); i++)
            for (int j = 0; j < n + (d == 1); j++) o[g.face_ind(i, j, d)] = (U)f[d][fidx2(n, d, i, j)];
    }
}

}  // namespace

extern "C" {

int orc2_dof(int n) {
    G2 g;
    g.nx = g.ny = n;
    return g.size();
}
int orc2_levels(int n) { return orc2::level_count(n); }
int orc2_index(int n, int kind, int x, int y, int d) {
    G2 g;
    g.nx = g.ny = n;
    return kind == 0 ? g.cell_ind(x, y) : (kind == 1 ? g.face_ind(x, y, d) : g.node_ind(x, y));
}
void orc2_field_to_blocked(int n, const double* cell, const double* f0, const double* f1, double* out) {
    G2 g;
    g.nx = g.ny = n;
    const double* f[2] = {f0, f1};
    field_to_blocked2(g, cell, f, out);
}
void orc2_blocked_to_field(int n, const double* in, double* cell, double* f0, double* f1) {
    G2 g;
    g.nx = g.ny = n;
    if (cell)
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) cell[i * n + j] = in[g.cell_ind(i, j)];
    double* f[2] = {f0, f1};
    for (int d = 0; d < 2; d++) {
        if (!f[d]) continue;
        for (int i = 0; i < n + (d == 0); i++)
            for (int j = 0; j < n + (d == 1); j++) f[d][fidx2(n, d, i, j)] = in[g.face_off(d) + g.face_ind(i, j, d)];
    }
}

void* orc2_create(int n) {
    H2* H = new H2();
    H->l = orc2::level_count(n);
    H->lv.resize(H->l);
    for (int i = H->l - 1, m = n; i >= 0; i--, m /= 2) H->lv[i].init(m);
    for (int i = H->l - 2; i >= 0; i--) H->lv[i].lap = 2.0 * H->lv[i + 1].lap;
    H->energy.init(n);
    H->r.resize(H->l);
    H->x.resize(H->l);
    H->p.resize(H->l);
    H->Ap.resize(H->l);
    for (int i = 0; i < H->l; i++) {
        int s = H->lv[i].g.size();
        H->r[i].assign(s, 0.0);
        H->x[i].assign(s, 0.0);
        H->p[i].assign(s, 0.0);
        H->Ap[i].assign(s, 0.0);
    }
    H->b.assign(H->lv[H->l - 1].g.size(), 0.0);
    H->sol = H->b;
    return H;
}
void orc2_destroy(void* p) { delete (H2*)p; }

// FluidSteadyState::init_boundary (stoke/FluidSteadyState.cpp:87-108)
void orc2_init_boundary(void* p, const double* cell_vol, const int* cell_fixed, const double* fv0, const double* fv1,
                        const int* ff0, const int* ff1, int closed) {
    H2* H = (H2*)p;
    Descr2& D = H->lv[H->l - 1];
    const double* fv[2] = {fv0, fv1};
    const int* ff[2] = {ff0, ff1};
    std::vector<int> fi(D.g.size());
    field_to_blocked2(D.g, cell_vol, fv, D.vol.data());
    field_to_blocked2(D.g, cell_fixed, ff, fi.data());
    for (int i = 0; i < D.g.size(); i++) D.fixed[i] = fi[i] != 0;
    H->energy.vol = D.vol;
    H->energy.fixed = D.fixed;
    H->closed = closed != 0;
}

// FluidSteadyState::update_penalty (:122-140): finish, coarse subsystems, coarsest matrix
void orc2_update_penalty(void* p, const double* cell_pen, const double* fp0, const double* fp1) {
    H2* H = (H2*)p;
    Descr2& D = H->lv[H->l - 1];
    const double* fp[2] = {fp0, fp1};
    field_to_blocked2(D.g, cell_pen, fp, D.pen.data());
    D.finish();
    for (int i = H->l - 2; i >= 0; i--) {
        orc2::update_subsystem(H->lv[i], H->lv[i + 1]);
        if (H->flow) orc2::flow_penalties(H->lv[i], H->lv[i + 1]);
    }
    orc2::dense_setup(H->lv[0], H->closed, H->dense);
    H->energy.pen = D.pen;
    H->energy.finish();
}

// Selects the coarse penalties of the next orc2_update_penalty: the reference's sums (0) or
// the GPU solver's rule (1).
void orc2_set_flow(void* p, int flow) { ((H2*)p)->flow = flow != 0; }

void orc2_update_b(void* p, const double* cell_b, const double* fb0, const double* fb1) {
    H2* H = (H2*)p;
    const double* fb[2] = {fb0, fb1};
    field_to_blocked2(H->lv[H->l - 1].g, cell_b, fb, H->b.data());
}
void orc2_set_b_blocked(void* p, const double* b) {
    H2* H = (H2*)p;
    std::copy(b, b + H->b.size(), H->b.begin());
}
int orc2_level_dof(void* p, int level) { return ((H2*)p)->lv[level].g.size(); }

// GMRES with the reference's 2D basis size (40) and thresholds passed in
int orc2_solve(void* p, int max_iter, double abs_thr, double rel_thr, double norm_thr, int restarts, double true_tol,
               double* x_out, double* stats) {
    H2* H = (H2*)p;
    const Descr2& D = H->lv[H->l - 1];
    VecOp A = [&](double* out, const double* in) { orc2::apply_A(D, out, in); };
    VecOp M = [&](double* out, const double* in) { orc2::mg_apply(*H, out, in); };
    KrylovStats ks;
    orc::gmres_generic(D.g.size(), A, M, H->b.data(), H->sol.data(), max_iter, abs_thr, rel_thr, norm_thr, restarts, true_tol,
                       ks);
    if (x_out) std::copy(H->sol.begin(), H->sol.end(), x_out);
    if (stats) {
        stats[0] = ks.iters;
        stats[1] = ks.restarts;
        stats[2] = ks.rel_true;
        stats[3] = ks.abs_true;
        stats[4] = ks.precond_res;
    }
    return ks.iters;
}

void orc2_apply_A(void* p, int level, const double* x, double* y) { orc2::apply_A(((H2*)p)->lv[level], y, x); }
void orc2_apply_E(void* p, const double* x, double* y) { orc2::apply_E(((H2*)p)->energy, y, x); }
double orc2_energy(void* p, const double* x) {
    H2* H = (H2*)p;
    std::vector<double> Ex(H->energy.g.size());
    orc2::apply_E(H->energy, Ex.data(), x);
    double s = 0;
    for (size_t i = 0; i < Ex.size(); i++) s += Ex[i] * x[i];
    return 0.5 * s;
}
void orc2_level_descr(void* p, int level, double* vol, double* pen, uint8_t* fixed, double* lap) {
    const Descr2& D = ((H2*)p)->lv[level];
    if (vol) std::copy(D.vol.begin(), D.vol.end(), vol);
    if (pen) std::copy(D.pen.begin(), D.pen.end(), pen);
    if (fixed) std::copy(D.fixed.begin(), D.fixed.end(), fixed);
    if (lap) *lap = D.lap;
}
void orc2_restrict(void* p, int coarse_level, const double* rf, double* rc) {
    H2* H = (H2*)p;
    orc2::restrict_r(H->lv[coarse_level], H->lv[coarse_level + 1], rc, rf);
}
void orc2_prolong(void* p, int coarse_level, const double* xc, double* xf) {
    H2* H = (H2*)p;
    orc2::prolong(H->lv[coarse_level], H->lv[coarse_level + 1], xf, xc);
}
void orc2_smooth_colour(void* p, int level, int flag, const double* r, double* out) {
    orc2::smooth_colour(((H2*)p)->lv[level], flag, out, r);
}
void orc2_smooth(void* p, int level, int post, const double* r, double* out) { orc2::smoother(((H2*)p)->lv[level], post, out, r); }
void orc2_coarse_apply(void* p, const double* r, double* out) { orc2::dense_apply(((H2*)p)->dense, out, r); }
int orc2_coarse_info(void* p) { return ((H2*)p)->dense.info; }
void orc2_vcycle(void* p, const double* r, double* out) { orc2::mg_apply(*(H2*)p, out, r); }

// Reference 2D test 0 (fluid_topo/FluidTopoOptDriver.cpp:104-156)
void orc_bc_test0_2d(int n, double* cell_vol, int* cell_fixed, double* cell_b, double* fv0, double* fv1, int* ff0, int* ff1,
                     double* fb0, double* fb1) {
    size_t nc = (size_t)n * n, nf = (size_t)n * (n + 1);
    std::fill(cell_vol, cell_vol + nc, 1.0);
    std::fill(cell_fixed, cell_fixed + nc, 0);
    std::fill(cell_b, cell_b + nc, 0.0);
    double* fv[2] = {fv0, fv1};
    int* ff[2] = {ff0, ff1};
    double* fb[2] = {fb0, fb1};
    for (int d = 0; d < 2; d++) {
        std::fill(fv[d], fv[d] + nf, 1.0);
        std::fill(ff[d], ff[d] + nf, 0);
        std::fill(fb[d], fb[d] + nf, 0.0);
    }
    for (int i = 0; i < n; i++) {
        ff[0][fidx2(n, 0, 0, i)] = 1;
        ff[0][fidx2(n, 0, n, i)] = 1;
        ff[1][fidx2(n, 1, i, 0)] = 1;
        ff[1][fidx2(n, 1, i, n)] = 1;
    }
    const int O = 16;
    int in_half = n / 32, out_half = n / (4 * O);
    double e = 60;
    double r = e * (2 * in_half + 1) / (2 * out_half + 1) / O;
    for (int i = 0; i < n; i++) {
        if (std::abs(i - n / 2) > in_half) continue;
        cell_b[0 * n + i] = e;
        fb[0][fidx2(n, 0, 1, i)] = e;
    }
    for (int o = 0; o < O; o++)
        for (int i = 0; i < n; i++) {
            if (std::abs(i - n / (2 * O) * (2 * o + 1)) > out_half) continue;
            cell_b[(n - 1) * n + i] = -r;
            fb[0][fidx2(n, 0, n - 1, i)] = r;
        }
}

}  // extern "C"
