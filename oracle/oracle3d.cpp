// CPU oracle for the 3D hot path (TEST INFRASTRUCTURE ONLY; see oracle3d.h).
//
// Every function cites the reference file:line it restates. Vectors use the
// reference's own blocked DOF layout [cells | x-faces | y-faces | z-faces] so the
// oracle can be compared entry by entry with the reference's LinearMapping vectors.
#include "oracle3d.h"
#include "krylov.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <omp.h>

namespace orc {

// ---------------------------------------------------------------- layout
// common_cpx/grid3D.cu:54-60
int G3::cell_ind(int x, int y, int z) const {
    int nbx = nx >> 2, nby = ny >> 2;
    int bx = x >> 2, by = y >> 2, bz = z >> 2;
    int ix = x & 3, iy = y & 3, iz = z & 3;
    return ((bz * nby + by) * nbx + bx) * 64 + ((iz * 4 + iy) * 4 + ix);
}
// common_cpx/grid3D.cu:62-68 (faces padded by 4 along their normal; the
// intra-tile axis order is permuted per face axis)
int G3::face_ind(int x, int y, int z, int d) const {
    int nbx = (nx >> 2) + (d == 0), nby = (ny >> 2) + (d == 1);
    int bx = x >> 2, by = y >> 2, bz = z >> 2;
    int ix = x & 3, iy = y & 3, iz = z & 3;
    int in_tile = d == 0 ? (ix * 4 + iz) * 4 + iy : d == 1 ? (iy * 4 + iz) * 4 + ix : (iz * 4 + iy) * 4 + ix;
    return ((bz * nby + by) * nbx + bx) * 64 + in_tile;
}
// common_cpx/grid3D.cu:70-76
int G3::edge_ind(int x, int y, int z, int d) const {
    int nbx = (nx >> 2) + (d != 0), nby = (ny >> 2) + (d != 1);
    int bx = x >> 2, by = y >> 2, bz = z >> 2;
    int ix = x & 3, iy = y & 3, iz = z & 3;
    int in_tile = d == 0 ? (iz * 4 + iy) * 4 + ix : d == 1 ? (iz * 4 + ix) * 4 + iy : (iy * 4 + ix) * 4 + iz;
    return ((bz * nby + by) * nbx + bx) * 64 + in_tile;
}
// common_cpx/grid3D.cu:86-94
void G3::ind_cell(int i, int& x, int& y, int& z) const {
    int nbx = nx >> 2, nby = ny >> 2;
    int ix = i & 3, iy = (i >> 2) & 3, iz = (i >> 4) & 3;
    int b = i >> 6;
    x = ((b % nbx) << 2) + ix;
    y = (((b / nbx) % nby) << 2) + iy;
    z = ((b / nbx / nby) << 2) + iz;
}
// common_cpx/grid3D.cu:96-105
void G3::ind_face(int i, int d, int& x, int& y, int& z) const {
    int nbx = (nx >> 2) + (d == 0), nby = (ny >> 2) + (d == 1);
    int a = i & 3, b4 = (i >> 2) & 3, c = (i >> 4) & 3;
    int b = i >> 6;
    x = ((b % nbx) << 2) + (d == 0) * c + (d == 1) * a + (d == 2) * a;
    y = (((b / nbx) % nby) << 2) + (d == 0) * a + (d == 1) * c + (d == 2) * b4;
    z = ((b / nbx / nby) << 2) + (d == 0) * b4 + (d == 1) * b4 + (d == 2) * c;
}

// ---------------------------------------------------------------- descriptor
// stoke/StokeFlowDescriptor3D.cu:6-20 (init) and :37-50 (finish)
void Descr::init(int n) {
    g = G3(n, n, n);
    vol.assign(g.size(), 0.0);
    penalty.assign(g.size(), 0.0);
    fixed.assign(g.size(), 0);
}
void Descr::finish() {
    for (int d = 0; d < 3; d++) {
        int off = g.face_off(d);
#pragma omp parallel for
        for (int i = 0; i < g.face_size(d); i++) {
            int x, y, z;
            g.ind_face(i, d, x, y, z);
            if (!g.face_valid(x, y, z, d)) fixed[off + i] = 1;
        }
    }
#pragma omp parallel for
    for (int i = 0; i < g.size(); i++)
        if (fixed[i]) { vol[i] = 0.0; penalty[i] = 0.0; }
}

// ---------------------------------------------------------------- DEC operators
// Face arrays are addressed as (base pointer of axis d, face_ind).
struct Faces {
    double* f[3];
};
struct CFaces {
    const double* f[3];
};

static inline double fget(const G3& g, const double* a, int x, int y, int z, int d) {
    return g.face_valid(x, y, z, d) ? a[g.face_ind(x, y, z, d)] : 0.0;
}
static inline double eget(const G3& g, const double* a, int x, int y, int z, int d) {
    return g.edge_valid(x, y, z, d) ? a[g.edge_ind(x, y, z, d)] : 0.0;
}

// Divergence face -> cell (common_cpx/grid3D.cu:330-397).
static void D2(const G3& g, double* cell, CFaces F) {
#pragma omp parallel for collapse(2)
    for (int z = 0; z < g.nz; z++)
        for (int y = 0; y < g.ny; y++)
            for (int x = 0; x < g.nx; x++) {
                double div = -F.f[0][g.face_ind(x, y, z, 0)] + F.f[0][g.face_ind(x + 1, y, z, 0)];
                div += -F.f[1][g.face_ind(x, y, z, 1)] + F.f[1][g.face_ind(x, y + 1, z, 1)];
                div += -F.f[2][g.face_ind(x, y, z, 2)] + F.f[2][g.face_ind(x, y, z + 1, 2)];
                cell[g.cell_ind(x, y, z)] = div;
            }
}

// Gradient cell -> face, face(x) = c(x) - c(x-1), zero outside the domain
// (common_cpx/grid3D.cu:401-465; the atomics only merge the two tile halves).
static void Cod0(const G3& g, Faces F, const double* cell) {
    for (int d = 0; d < 3; d++) std::memset(F.f[d], 0, sizeof(double) * g.face_size(d));
    auto c = [&](int x, int y, int z) { return g.cell_valid(x, y, z) ? cell[g.cell_ind(x, y, z)] : 0.0; };
    for (int d = 0; d < 3; d++) {
        int ex = d == 0, ey = d == 1, ez = d == 2;
#pragma omp parallel for collapse(2)
        for (int z = 0; z < g.nz + ez; z++)
            for (int y = 0; y < g.ny + ey; y++)
                for (int x = 0; x < g.nx + ex; x++) F.f[d][g.face_ind(x, y, z, d)] = c(x, y, z) - c(x - ex, y - ey, z - ez);
    }
}

// Curl face -> edge (common_cpx/grid3D.cu:469-578).
static void Cod1(const G3& g, Faces E, CFaces F) {
    for (int d = 0; d < 3; d++) std::memset(E.f[d], 0, sizeof(double) * g.edge_size(d));
    const double *fx = F.f[0], *fy = F.f[1], *fz = F.f[2];
#pragma omp parallel for collapse(2)
    for (int z = 0; z <= g.nz; z++)
        for (int y = 0; y <= g.ny; y++)
            for (int x = 0; x <= g.nx; x++) {
                if (g.edge_valid(x, y, z, 0))
                    E.f[0][g.edge_ind(x, y, z, 0)] = fget(g, fy, x, y, z, 1) - fget(g, fy, x, y, z - 1, 1) -
                                                     fget(g, fz, x, y, z, 2) + fget(g, fz, x, y - 1, z, 2);
                if (g.edge_valid(x, y, z, 1))
                    E.f[1][g.edge_ind(x, y, z, 1)] = fget(g, fx, x, y, z - 1, 0) - fget(g, fx, x, y, z, 0) +
                                                     fget(g, fz, x, y, z, 2) - fget(g, fz, x - 1, y, z, 2);
                if (g.edge_valid(x, y, z, 2))
                    E.f[2][g.edge_ind(x, y, z, 2)] = fget(g, fx, x, y, z, 0) - fget(g, fx, x, y - 1, z, 0) +
                                                     fget(g, fy, x - 1, y, z, 1) - fget(g, fy, x, y, z, 1);
            }
}

// Curl edge -> face (common_cpx/grid3D.cu:219-326).
static void D1(const G3& g, Faces F, CFaces E) {
    for (int d = 0; d < 3; d++) std::memset(F.f[d], 0, sizeof(double) * g.face_size(d));
    const double *ex = E.f[0], *ey = E.f[1], *ez = E.f[2];
#pragma omp parallel for collapse(2)
    for (int z = 0; z <= g.nz; z++)
        for (int y = 0; y <= g.ny; y++)
            for (int x = 0; x <= g.nx; x++) {
                if (g.face_valid(x, y, z, 0))
                    F.f[0][g.face_ind(x, y, z, 0)] = eget(g, ey, x, y, z + 1, 1) - eget(g, ey, x, y, z, 1) +
                                                     eget(g, ez, x, y, z, 2) - eget(g, ez, x, y + 1, z, 2);
                if (g.face_valid(x, y, z, 1))
                    F.f[1][g.face_ind(x, y, z, 1)] = eget(g, ex, x, y, z, 0) - eget(g, ex, x, y, z + 1, 0) -
                                                     eget(g, ez, x, y, z, 2) + eget(g, ez, x + 1, y, z, 2);
                if (g.face_valid(x, y, z, 2))
                    F.f[2][g.face_ind(x, y, z, 2)] = -eget(g, ex, x, y, z, 0) + eget(g, ex, x, y + 1, z, 0) +
                                                     eget(g, ey, x, y, z, 1) - eget(g, ey, x + 1, y, z, 1);
            }
}

// ---------------------------------------------------------------- operators

static Faces faces_of(const G3& g, double* v) { return Faces{{v + g.face_off(0), v + g.face_off(1), v + g.face_off(2)}}; }
static CFaces cfaces_of(const G3& g, const double* v) {
    return CFaces{{v + g.face_off(0), v + g.face_off(1), v + g.face_off(2)}};
}
static Faces edges_of(const G3& g, double* v) { return Faces{{v, v + g.edge_size(0), v + g.edge_size(0) + g.edge_size(1)}}; }
static CFaces cedges_of(const G3& g, const double* v) {
    return CFaces{{v, v + g.edge_size(0), v + g.edge_size(0) + g.edge_size(1)}};
}

// Viscous part shared by A and E: Ap_f -= fix_f(G(fix_c(D(V u)))) ; Ap_f += V D1(Cod1(fix_f u)).
// stoke/StokeFlowMapping3D.cu:236-300 and fluid_topo/FluidEnergyGrad3D.cu:220-288.
static void viscous(const Descr& ds, double* Ap, const double* p, Work& w) {
    const G3& g = ds.g;
    const int nc = g.cell_size(), n = g.size();
    double* t = w.t.data();
    // grad div
    for (int i = nc; i < n; i++) t[i] = p[i] * ds.vol[i];
    D2(g, t, cfaces_of(g, t));
    for (int i = 0; i < nc; i++)
        if (ds.fixed[i]) t[i] = 0.0;
    Cod0(g, faces_of(g, t), t);
    for (int i = nc; i < n; i++) {
        double v = ds.fixed[i] ? 0.0 : t[i];
        Ap[i] -= v;
    }
    // curl curl
    for (int i = nc; i < n; i++) t[i] = ds.fixed[i] ? 0.0 : p[i];
    double* e = w.e.data();
    Cod1(g, edges_of(g, e), cfaces_of(g, t));
    D1(g, faces_of(g, t), cedges_of(g, e));
    for (int i = nc; i < n; i++) Ap[i] += t[i] * ds.vol[i];
}

// Operator A = StokeFlowMapping3DFixed::applyMapping (stoke/StokeFlowMapping3D.cu:218-348).
void apply_A(const Descr& ds, double* Ap, const double* p, Work& w) {
    const G3& g = ds.g;
    const int nc = g.cell_size(), n = g.size();
    w.ensure(g);
    std::fill(Ap, Ap + n, 0.0);
    viscous(ds, Ap, p, w);
    double* t = w.t.data();
    // -grad p  (:302-313)
    Cod0(g, faces_of(g, t), p);
    for (int i = nc; i < n; i++) Ap[i] -= t[i] * ds.vol[i];
    // div v (:315-332)
    for (int i = nc; i < n; i++) t[i] = p[i] * ds.vol[i];
    D2(g, t, cfaces_of(g, t));
    for (int i = 0; i < nc; i++) Ap[i] += ds.fixed[i] ? 0.0 : t[i];
    // penalty (:334-341) and definite fix (:343-347)
    for (int i = 0; i < n; i++) Ap[i] += p[i] * ds.penalty[i];
    for (int i = 0; i < n; i++)
        if (ds.fixed[i]) Ap[i] += p[i];
}

// Operator E = FluidEnergyGrad3D::applyMapping (fluid_topo/FluidEnergyGrad3D.cu:201-308).
void apply_E(const Descr& ds, double* Ap, const double* p, Work& w) {
    const int n = ds.g.size();
    w.ensure(ds.g);
    std::fill(Ap, Ap + n, 0.0);
    viscous(ds, Ap, p, w);
    for (int i = 0; i < n; i++) Ap[i] += p[i] * ds.penalty[i];
}

// ---------------------------------------------------------------- coarsening and transfers
// Eight fine children of coarse slot (X,Y,Z) for any DOF kind: x in {2X,2X+1}, ...
// (common_cpx/SubsystemUtils3D.cuh:8-186; the child bit order is bit0=x, bit1=y, bit2=z).
template <class T, class F>
static void down_sample(const G3& cg, const G3& fg, T* cv, const T* fv, F f) {
    // cells
#pragma omp parallel for collapse(2)
    for (int z = 0; z < cg.nz; z++)
        for (int y = 0; y < cg.ny; y++)
            for (int x = 0; x < cg.nx; x++) {
                T v[8];
                for (int k = 0; k < 8; k++)
                    v[k] = fv[fg.cell_ind(2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + ((k >> 2) & 1))];
                cv[cg.cell_ind(x, y, z)] = f(v, -1);
            }
    // faces: every coarse face slot of the padded array is written
    for (int d = 0; d < 3; d++) {
        T* c = cv + cg.face_off(d);
        const T* fa = fv + fg.face_off(d);
#pragma omp parallel for
        for (int i = 0; i < cg.face_size(d); i++) {
            int x, y, z;
            cg.ind_face(i, d, x, y, z);
            T v[8];
            for (int k = 0; k < 8; k++) {
                int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + ((k >> 2) & 1);
                v[k] = fg.face_valid(fx, fy, fz, d) ? fa[fg.face_ind(fx, fy, fz, d)] : T(0);
            }
            c[i] = f(v, d);
        }
    }
}

// updateSubSystem (stoke/StokeFlowSubSystem3D.cu:103-154): fixed = OR of 8,
// vol = sum of 8 (cells) / 4 coincident (faces), penalty = sum of 8; then finish().
void update_subsystem(Descr& c, const Descr& f) {
    down_sample<uint8_t>(c.g, f.g, c.fixed.data(), f.fixed.data(), [](uint8_t* v, int) {
        uint8_t s = 0;
        for (int k = 0; k < 8; k++) s |= v[k];
        return s;
    });
    down_sample<double>(c.g, f.g, c.vol.data(), f.vol.data(), [](double* v, int d) {
        if (d < 0) {
            double s = 0;
            for (int k = 0; k < 8; k++) s += v[k];
            return s;
        }
        int bit = 1 << d;  // the coincident children have a zero offset along the normal
        double s = 0;
        for (int k = 0; k < 8; k++)
            if (!(k & bit)) s += v[k];
        return s;
    });
    down_sample<double>(c.g, f.g, c.penalty.data(), f.penalty.data(), [](double* v, int) {
        double s = 0;
        for (int k = 0; k < 8; k++) s += v[k];
        return s;
    });
    c.finish();
}

// The GPU solver's own coarse penalties (its "flow rule", not in the reference): a coarse
// face takes 8 x the smallest penalty among its present, free children instead of the sum;
// cell penalties keep the sum. Applied after update_subsystem, which fixes the coarse
// unknowns, so fixed coarse faces stay at zero.
void flow_penalties(Descr& c, const Descr& f) {
    for (int d = 0; d < 3; d++) {
        double* cp = c.penalty.data() + c.g.face_off(d);
        const double* fp = f.penalty.data() + f.g.face_off(d);
        const uint8_t* ff = f.fixed.data() + f.g.face_off(d);
        const uint8_t* cf = c.fixed.data() + c.g.face_off(d);
        for (int i = 0; i < c.g.face_size(d); i++) {
            if (cf[i]) continue;
            int x, y, z;
            c.g.ind_face(i, d, x, y, z);
            double lo = -1.0;
            for (int k = 0; k < 8; k++) {
                const int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + ((k >> 2) & 1);
                if (!f.g.face_valid(fx, fy, fz, d)) continue;
                const int j = f.g.face_ind(fx, fy, fz, d);
                if (ff[j]) continue;
                if (lo < 0.0 || fp[j] < lo) lo = fp[j];
            }
            if (lo >= 0.0) cp[i] = 8.0 * lo;
        }
    }
}

// StokeFlowDownSample3D::applyMapping (stoke/StokeFlowSubSystem3D.cu:32-52).
void restrict_r(const Descr& c, const Descr& f, double* rc, const double* rf) {
    down_sample<double>(c.g, f.g, rc, rf, [](double* v, int) {
        double s = 0;
        for (int k = 0; k < 8; k++) s += v[k];
        return s;
    });
#pragma omp parallel for
    for (int i = 0; i < c.g.size(); i++)
        if (c.fixed[i]) rc[i] = 0.0;
}

// StokeFlowUpSample3D::applyMapping (stoke/StokeFlowSubSystem3D.cu:81-101 with
// common_cpx/SubsystemUtils3D.cuh:370-495): piecewise-constant injection.
void prolong(const Descr& c, const Descr& f, double* xf, const double* xc) {
    const G3 &fg = f.g, &cg = c.g;
    std::fill(xf, xf + fg.size(), 0.0);
#pragma omp parallel for collapse(2)
    for (int z = 0; z < fg.nz; z++)
        for (int y = 0; y < fg.ny; y++)
            for (int x = 0; x < fg.nx; x++) xf[fg.cell_ind(x, y, z)] = xc[cg.cell_ind(x >> 1, y >> 1, z >> 1)];
    for (int d = 0; d < 3; d++) {
        int ex = d == 0, ey = d == 1, ez = d == 2;
        double* fa = xf + fg.face_off(d);
        const double* ca = xc + cg.face_off(d);
#pragma omp parallel for collapse(2)
        for (int z = 0; z < fg.nz + ez; z++)
            for (int y = 0; y < fg.ny + ey; y++)
                for (int x = 0; x < fg.nx + ex; x++) fa[fg.face_ind(x, y, z, d)] = ca[cg.face_ind(x >> 1, y >> 1, z >> 1, d)];
    }
#pragma omp parallel for
    for (int i = 0; i < fg.size(); i++)
        if (f.fixed[i]) xf[i] = 0.0;
}

// ---------------------------------------------------------------- Vanka smoother
// StokeMask3D (stoke/StokeLike.cu:11-39): parity masks on cells and faces.
static bool stoke_mask(const G3& g, int i, int cell_flag, int face_flag) {
    int x, y, z;
    if (i < g.cell_size()) {
        g.ind_cell(i, x, y, z);
        return (x + y + z + cell_flag) % 2 == 0;
    }
    i -= g.cell_size();
    int d;
    for (d = 0; d < 3; d++) {
        if (i < g.face_size(d)) break;
        i -= g.face_size(d);
    }
    g.ind_face(i, d, x, y, z);
    return (x + y + z + face_flag) % 2 == 0;
}

// Packed 7-DOF index of red block t, local DOF l (GATHER/SHATTER, stoke/StokeLike.cu:98-166):
// l = 0..5 -> face (d = l>>1, +1 offset if l odd), l = 6 -> cell.
static int block_dof(const G3& g, int t, int l, int flag) {
    int b = t >> 5;
    int ix = (t & 1) << 1, iy = (t & 6) >> 1, iz = (t & 24) >> 3;
    ix += (iy + iz + flag) % 2;
    int nbx = g.nx >> 2, nby = g.ny >> 2;
    int x = ((b % nbx) << 2) + ix, y = (((b / nbx) % nby) << 2) + iy, z = ((b / nbx / nby) << 2) + iz;
    if (l < 6) {
        int d = l >> 1;
        x += (d == 0) * (l & 1);
        y += (d == 1) * (l & 1);
        z += (d == 2) * (l & 1);
        return g.face_off(d) + g.face_ind(x, y, z, d);
    }
    return g.cell_ind(x, y, z);
}

// Dense LU with partial pivoting, LAPACK getrf/getrs semantics on a column-major
// k x k block (the batched cuBLAS calls of common_cpx/DirectSolveBlockInverse.cuh:105-132
// and the dense cuSOLVER calls of stoke/StokeLike.cu:421-425,636-640).
static int lu_factor(double* a, int* piv, int k, int lda) {
    int info = 0;
    for (int j = 0; j < k; j++) {
        int p = j;
        double m = std::fabs(a[j + j * lda]);
        for (int i = j + 1; i < k; i++)
            if (std::fabs(a[i + j * lda]) > m) { m = std::fabs(a[i + j * lda]); p = i; }
        piv[j] = p;
        if (a[p + j * lda] == 0.0) {
            if (!info) info = j + 1;
            continue;
        }
        if (p != j)
            for (int c = 0; c < k; c++) std::swap(a[j + c * lda], a[p + c * lda]);
        double inv = 1.0 / a[j + j * lda];
        for (int i = j + 1; i < k; i++) a[i + j * lda] *= inv;
        for (int c = j + 1; c < k; c++) {
            double u = a[j + c * lda];
            if (u != 0.0)
                for (int i = j + 1; i < k; i++) a[i + c * lda] -= a[i + j * lda] * u;
        }
    }
    return info;
}
static void lu_solve(const double* a, const int* piv, int k, int lda, double* b) {
    for (int j = 0; j < k; j++)
        if (piv[j] != j) std::swap(b[j], b[piv[j]]);
    for (int j = 0; j < k; j++)
        for (int i = j + 1; i < k; i++) b[i] -= a[i + j * lda] * b[j];
    for (int j = k - 1; j >= 0; j--) {
        b[j] /= a[j + j * lda];
        for (int i = 0; i < j; i++) b[i] -= a[i + j * lda] * b[j];
    }
}


// B x = M_w A M_w x + M_b A M_b x (VelDiagPressureFullMapping3D, stoke/StokeLike.cu:41-96).
static void apply_B(const Descr& ds, int flag, double* y, const double* x, Work& w, std::vector<double>& tmp) {
    const G3& g = ds.g;
    int n = g.size();
    std::vector<double> xm(n), ym(n);
    std::fill(y, y + n, 0.0);
    for (int face_flag = 0; face_flag < 2; face_flag++) {
#pragma omp parallel for
        for (int i = 0; i < n; i++) xm[i] = stoke_mask(g, i, flag, face_flag) ? x[i] : 0.0;
        apply_A(ds, ym.data(), xm.data(), w);
#pragma omp parallel for
        for (int i = 0; i < n; i++)
            if (stoke_mask(g, i, flag, face_flag)) y[i] += ym[i];
    }
    (void)tmp;
}

// DirectSolveBlockInverse<7>::update with LinearMappingToBlockMatrix<7,7>
// (common_cpx/DirectSolveBlockInverse.cuh:116-132, BatchInverse.cuh:61-75): column l of
// every block is read off B applied to the vector holding 1 at local DOF l of EVERY red block.
//
// reorder_as_run: the reference packs the probe results into 7x7 blocks with
// BlockMatrixReorderKernel (common_cpx/BatchInverse.cuh:13-47), one 32-thread warp per 32
// blocks, staging 32 packed rows at a time in a two-chunk shared buffer. Its output
// schedule (end = start + 7, minus one after the first chunk) writes output chunk 33 of
// every warp after loading only row chunks 0-4, so entry (row 6, column 0) of the warp's
// block 22 - packed row 7*22+6 = 160, loaded with chunk 5 - is read from the buffer slot
// that still holds packed row 96 of chunk 3, i.e. entry (row 5, column 0) of block 13.
// Executed in lockstep, as a warp does, this is deterministic; reorder_as_run reproduces
// it, so that the oracle can be checked against the reference's own smoother as it runs.
// Without it the oracle builds the blocks the reference intends (the exact restriction of
// B), which is what the GPU solver's closed-form block solve implements.
void vanka_setup(const Descr& ds, int flag, Vanka& v, Work& w, bool reorder_as_run) {
    const G3& g = ds.g;
    v.flag = flag;
    v.nb = g.cell_size() / 2;
    v.dofs.resize(v.nb * 7);
#pragma omp parallel for
    for (int t = 0; t < v.nb; t++)
        for (int l = 0; l < 7; l++) v.dofs[t * 7 + l] = block_dof(g, t, l, flag);
    v.lu.assign(v.nb * 49, 0.0);
    v.piv.assign(v.nb * 7, 0);
    int n = g.size();
    std::vector<double> s(n), y(n), tmp;
    for (int l = 0; l < 7; l++) {
        std::fill(s.begin(), s.end(), 0.0);
#pragma omp parallel for
        for (int t = 0; t < v.nb; t++) s[v.dofs[t * 7 + l]] = 1.0;
        apply_B(ds, flag, y.data(), s.data(), w, tmp);
#pragma omp parallel for
        for (int t = 0; t < v.nb; t++)
            for (int m = 0; m < 7; m++) v.lu[t * 49 + l * 7 + m] = y[v.dofs[t * 7 + m]];
    }
    if (reorder_as_run)
        for (int t = 22; t < v.nb; t += 32) v.lu[t * 49 + 0 * 7 + 6] = v.lu[(t - 9) * 49 + 0 * 7 + 5];
#pragma omp parallel for
    for (int t = 0; t < v.nb; t++) lu_factor(&v.lu[t * 49], &v.piv[t * 7], 7, 7);
}

// VelDiagPressureFullSmoothing::applyMapping (stoke/StokeLike.cu:263-272).
void vanka_apply(const Vanka& v, int n, double* out, const double* r) {
    std::fill(out, out + n, 0.0);
#pragma omp parallel for
    for (int t = 0; t < v.nb; t++) {
        double b[7];
        for (int l = 0; l < 7; l++) b[l] = r[v.dofs[t * 7 + l]];
        lu_solve(&v.lu[t * 49], &v.piv[t * 7], 7, 7, b);
        for (int l = 0; l < 7; l++) out[v.dofs[t * 7 + l]] = b[l];
    }
}

// DescentSmoother::applyMapping (common_cpx/DescentSmoother.cu:31-47).
void descent_smoother(const Descr& ds, const Vanka* P[2], const int iters[2], double* out, const double* r_in, Work& w) {
    int n = ds.g.size();
    std::vector<double> r(r_in, r_in + n), d(n), Ad(n);
    std::fill(out, out + n, 0.0);
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < iters[i]; j++) {
            vanka_apply(*P[i], n, d.data(), r.data());
#pragma omp parallel for
            for (int q = 0; q < n; q++) out[q] += d[q];
            if (i == 1 && j == iters[i] - 1) break;
            apply_A(ds, Ad.data(), d.data(), w);
#pragma omp parallel for
            for (int q = 0; q < n; q++) r[q] -= Ad[q];
        }
}

// ---------------------------------------------------------------- coarsest dense solve
// DirectSolve3D::update (stoke/StokeLike.cu:427-641): the dense matrix is read off 2
// cell-parity probes and 7 face probes coloured by (x+2y+3z+magic[d]+flag) mod 7.

void dense_setup(const Descr& ds, bool closed, Dense& D, Work& w) {
    const G3& g = ds.g;
    const int n = g.size(), nc = g.cell_size();
    D.n = n;
    D.a.assign((size_t)n * n, 0.0);
    D.piv.assign(n, 0);
    std::vector<double> p(n), Ap(n);
    auto face_of = [&](int i, int& d, int& x, int& y, int& z) {
        int t = i - nc;
        for (d = 0; d < 3; d++) {
            if (t < g.face_size(d)) break;
            t -= g.face_size(d);
        }
        g.ind_face(t, d, x, y, z);
    };
    for (int flag = 0; flag < 2; flag++) {
        std::fill(p.begin(), p.end(), 0.0);
        for (int i = 0; i < nc; i++) {
            int x, y, z;
            g.ind_cell(i, x, y, z);
            p[i] = ((x + y + z + flag) % 2 == 0) ? 1.0 : 0.0;
        }
        apply_A(ds, Ap.data(), p.data(), w);
        for (int i = nc; i < n; i++) {
            int d, x, y, z;
            face_of(i, d, x, y, z);
            int x0 = x, y0 = y, z0 = z;
            if ((x + y + z + flag) % 2 == 1) {
                if (d == 0) x0--;
                if (d == 1) y0--;
                if (d == 2) z0--;
            }
            if (g.cell_valid(x0, y0, z0)) D.a[i + (size_t)g.cell_ind(x0, y0, z0) * n] = Ap[i];
        }
    }
    const int magic[3] = {2, 4, 5};
    for (int flag = 0; flag < 7; flag++) {
        std::fill(p.begin(), p.end(), 0.0);
        for (int d = 0; d < 3; d++) {
            int off = g.face_off(d);
            for (int i = 0; i < g.face_size(d); i++) {
                int x, y, z;
                g.ind_face(i, d, x, y, z);
                p[off + i] = ((x + 2 * y + 3 * z + magic[d] + flag) % 7 == 0) ? 1.0 : 0.0;
            }
        }
        apply_A(ds, Ap.data(), p.data(), w);
        auto in_padded = [&](int x, int y, int z, int d) {
            return x >= 0 && y >= 0 && z >= 0 && x < g.nx + 4 * (d == 0) && y < g.ny + 4 * (d == 1) && z < g.nz + 4 * (d == 2);
        };
        for (int i = 0; i < nc; i++) {
            int x, y, z;
            g.ind_cell(i, x, y, z);
            int d0 = -1, x0 = x, y0 = y, z0 = z;
            switch ((x + 2 * y + 3 * z + flag) % 7) {
                case 1: d0 = 1; y0++; break;
                case 2: d0 = 2; break;
                case 3: d0 = 1; break;
                case 4: d0 = 0; x0++; break;
                case 5: d0 = 0; break;
                case 6: d0 = 2; z0++; break;
                default: break;
            }
            if (d0 != -1 && in_padded(x0, y0, z0, d0)) D.a[i + (size_t)(g.face_off(d0) + g.face_ind(x0, y0, z0, d0)) * n] = Ap[i];
        }
        for (int i = nc; i < n; i++) {
            int d, x, y, z;
            face_of(i, d, x, y, z);
            int x0 = x, y0 = y, z0 = z;
            switch ((x + 2 * y + 3 * z + magic[d] + flag) % 7) {
                case 1: x0--; break;
                case 2: y0--; break;
                case 3: z0--; break;
                case 4: z0++; break;
                case 5: y0++; break;
                case 6: x0++; break;
                default: break;
            }
            if (in_padded(x0, y0, z0, d)) D.a[i + (size_t)(g.face_off(d) + g.face_ind(x0, y0, z0, d)) * n] = Ap[i];
        }
    }
    if (closed)
        for (int i = 0; i < nc; i++)
            for (int j = 0; j < nc; j++) D.a[i + (size_t)j * n] += 1.0;
    D.info = lu_factor(D.a.data(), D.piv.data(), n, n);
}

void dense_apply(const Dense& D, double* out, const double* r) {
    std::copy(r, r + D.n, out);
    lu_solve(D.a.data(), D.piv.data(), D.n, D.n, out);
}

// ---------------------------------------------------------------- hierarchy and V-cycle

// FluidSteadyState3D::init level count (stoke/FluidSteadyState3D.cpp:12-15).
int level_count(int n) {
    int low = n & -n;
    int l = (int)std::lround(std::log2((double)low)) - 1;
    return l < 1 ? 1 : l;
}

void hierarchy_init(Hierarchy& H, int n) {
    H.l = level_count(n);
    H.lv.resize(H.l);
    for (int i = H.l - 1, m = n; i >= 0; i--, m /= 2) H.lv[i].init(m);
    H.red.resize(H.l);
    H.black.resize(H.l);
    H.r.resize(H.l);
    H.x.resize(H.l);
    H.p.resize(H.l);
    H.Ap.resize(H.l);
    for (int i = 0; i < H.l; i++) {
        int s = H.lv[i].g.size();
        H.r[i].assign(s, 0.0);
        H.x[i].assign(s, 0.0);
        H.p[i].assign(s, 0.0);
        H.Ap[i].assign(s, 0.0);
    }
}

// FluidSteadyState3D::solve set-up half (stoke/FluidSteadyState3D.cpp:152-156):
// coarse descriptors, smoother blocks, coarsest LU.
void hierarchy_update(Hierarchy& H, bool flow, bool reorder_as_run) {
    for (int i = H.l - 2; i >= 0; i--) {
        update_subsystem(H.lv[i], H.lv[i + 1]);
        if (flow) flow_penalties(H.lv[i], H.lv[i + 1]);
    }
    for (int i = 1; i < H.l; i++) {
        vanka_setup(H.lv[i], 0, H.red[i], H.w, reorder_as_run);
        vanka_setup(H.lv[i], 1, H.black[i], H.w, reorder_as_run);
    }
    dense_setup(H.lv[0], H.closed, H.dense, H.w);
}

// MultigridSolve::Vcycle (common_cpx/MultigridSolve.cpp:73-106); presmoother = {red x2,
// black x2}, postsmoother = {black x2, red x2} (stoke/StokeLike.cu:361), coarsest = dense LU.
void vcycle(Hierarchy& H) {
    const int iters[2] = {2, 2};
    for (int i = H.l - 1; i >= 0; i--) {
        int n = H.lv[i].g.size();
        auto &r = H.r[i], &x = H.x[i], &p = H.p[i], &Ap = H.Ap[i];
        std::fill(p.begin(), p.end(), 0.0);
        if (i > 0) {
            const Vanka* P[2] = {&H.red[i], &H.black[i]};
            descent_smoother(H.lv[i], P, iters, p.data(), r.data(), H.w);
        } else {
            dense_apply(H.dense, p.data(), r.data());
        }
        apply_A(H.lv[i], Ap.data(), p.data(), H.w);
#pragma omp parallel for
        for (int q = 0; q < n; q++) { x[q] += p[q]; r[q] -= Ap[q]; }
        if (i != 0) {
            restrict_r(H.lv[i - 1], H.lv[i], H.r[i - 1].data(), r.data());
            std::fill(H.x[i - 1].begin(), H.x[i - 1].end(), 0.0);
        }
    }
    for (int i = 0; i < H.l; i++) {
        int n = H.lv[i].g.size();
        auto &r = H.r[i], &x = H.x[i], &p = H.p[i], &Ap = H.Ap[i];
        if (i != 0) {
            prolong(H.lv[i - 1], H.lv[i], p.data(), H.x[i - 1].data());
            apply_A(H.lv[i], Ap.data(), p.data(), H.w);
    #pragma omp parallel for
        for (int q = 0; q < n; q++) { x[q] += p[q]; r[q] -= Ap[q]; }
        }
        std::fill(p.begin(), p.end(), 0.0);
        if (i > 0) {
            const Vanka* P[2] = {&H.black[i], &H.red[i]};
            descent_smoother(H.lv[i], P, iters, p.data(), r.data(), H.w);
        }
        apply_A(H.lv[i], Ap.data(), p.data(), H.w);
#pragma omp parallel for
        for (int q = 0; q < n; q++) { x[q] += p[q]; r[q] -= Ap[q]; }
    }
}

// MultigridSolve::applyMapping (common_cpx/MultigridSolve.cpp:108-114).
void mg_apply(Hierarchy& H, double* out, const double* in) {
    int t = H.l - 1;
    std::copy(in, in + H.lv[t].g.size(), H.r[t].begin());
    std::fill(H.x[t].begin(), H.x[t].end(), 0.0);
    vcycle(H);
    std::copy(H.x[t].begin(), H.x[t].end(), out);
}

// ---------------------------------------------------------------- Krylov
// GMRES::Solve (common_cpx/GMRES.cpp:20-110) with A = the finest operator and the V-cycle
// as left preconditioner (stoke/FluidSteadyState3D.cpp:120-125); see krylov.h.
void gmres_solve(Hierarchy& H, const double* b, double* x, int max_iter, double abs_thres, double rel_thres,
                 double norm_thres, int restarts, double true_tol, SolveStats& st) {
    const int t = H.l - 1;
    const Descr& ds = H.lv[t];
    const int n = ds.g.size();
    VecOp A = [&](double* out, const double* in) { apply_A(ds, out, in, H.w); };
    VecOp M = [&](double* out, const double* in) { mg_apply(H, out, in); };
    KrylovStats ks;
    gmres_generic(n, A, M, b, x, max_iter, abs_thres, rel_thres, norm_thres, restarts, true_tol, ks);
    st.iters = ks.iters;
    st.restarts = ks.restarts;
    st.rel_true = ks.rel_true;
    st.abs_true = ks.abs_true;
    st.precond_res = ks.precond_res;
}

}  // namespace orc
