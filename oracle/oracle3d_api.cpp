// extern "C" surface of the CPU oracle (TEST INFRASTRUCTURE ONLY; see oracle3d.h).
//
// Host arrays use the simplex Field order: cells N^3 with index i*N*N + j*N + k
// (simplex/src/reservoir/Field.h:67-72); face axis d has N+1 entries along d
// (simplex/src/reservoir/FaceField.h:16). Blocked vectors use the reference's
// solver layout (common_cpx/grid3D.cu:24-146).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "oracle3d.h"
#include "topo_common.h"

using namespace orc;

namespace {

struct Handle {
    int n = 0;
    Hierarchy H;
    Descr energy;  // FluidEnergy3D's own descriptor (fluid_topo/FluidEnergy3D.cpp:5-31)
    std::vector<double> b, x;
    Work w;
};

inline int fidx(int n, int d, int i, int j, int k) {
    int cy = n + (d == 1), cz = n + (d == 2);
    return (i * cy + j) * cz + k;
}

// simplexSupport::simplex2solver for Field and FaceField (common_cpx/SimplexSupport.h:228-305).
template <class T, class U>
void field_to_blocked(const G3& g, const T* cell, const T* const f[3], U* out) {
    int n = g.nx;
    std::fill(out, out + g.size(), U(0));
    if (cell)
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++)
                for (int k = 0; k < n; k++) out[g.cell_ind(i, j, k)] = (U)cell[(i * n + j) * n + k];
    for (int d = 0; d < 3; d++) {
        if (!f || !f[d]) continue;
        U* o = out + g.face_off(d);
        for (int i = 0; i < n + (d == 0); i++)
            for (int j = 0; j < n + (d == 1); j++)
                for (int k = 0; k < n + (d == 2); k++) o[g.face_ind(i, j, k, d)] = (U)f[d][fidx(n, d, i, j, k)];
    }
}

// simplexSupport::solver2simplex (common_cpx/SimplexSupport.h:307-330).
void blocked_to_field(const G3& g, const double* in, double* cell, double* const f[3]) {
    int n = g.nx;
    if (cell)
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++)
                for (int k = 0; k < n; k++) cell[(i * n + j) * n + k] = in[g.cell_ind(i, j, k)];
    for (int d = 0; d < 3; d++) {
        if (!f || !f[d]) continue;
        const double* o = in + g.face_off(d);
        for (int i = 0; i < n + (d == 0); i++)
            for (int j = 0; j < n + (d == 1); j++)
                for (int k = 0; k < n + (d == 2); k++) f[d][fidx(n, d, i, j, k)] = o[g.face_ind(i, j, k, d)];
    }
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- layout
int orc3_dof(int n) { return G3(n, n, n).size(); }
int orc3_levels(int n) { return level_count(n); }
int orc3_level_n(int n, int level) {
    int l = level_count(n);
    return n >> (l - 1 - level);
}
// kind 0 = cell_ind, 1 = face_ind(d), 2 = edge_ind(d), 3 = ind_cell (x <- i), 4 = ind_face
int orc3_index(int n, int kind, int x, int y, int z, int d, int* out3) {
    G3 g(n, n, n);
    switch (kind) {
        case 0: return g.cell_ind(x, y, z);
        case 1: return g.face_ind(x, y, z, d);
        case 2: return g.edge_ind(x, y, z, d);
        case 3: g.ind_cell(x, out3[0], out3[1], out3[2]); return 0;
        case 4: g.ind_face(x, d, out3[0], out3[1], out3[2]); return 0;
    }
    return -1;
}
void orc3_field_to_blocked(int n, const double* cell, const double* f0, const double* f1, const double* f2, double* out) {
    const double* f[3] = {f0, f1, f2};
    field_to_blocked(G3(n, n, n), cell, f, out);
}
void orc3_blocked_to_field(int n, const double* in, double* cell, double* f0, double* f1, double* f2) {
    double* f[3] = {f0, f1, f2};
    blocked_to_field(G3(n, n, n), in, cell, f);
}

// ---------------------------------------------------------------- solver handle
// FluidSteadyState3D::init (stoke/FluidSteadyState3D.cpp:12-90) without the GMRES print.
void* orc3_create(int n) {
    Handle* h = new Handle();
    h->n = n;
    hierarchy_init(h->H, n);
    h->energy.init(n);
    h->b.assign(h->H.lv[h->H.l - 1].g.size(), 0.0);
    h->x = h->b;
    return h;
}
void orc3_destroy(void* p) { delete (Handle*)p; }

// FluidSteadyState3D::init_boundary (:92-114) and FluidEnergy3D::init_boundary (FluidEnergy3D.cpp:33-54).
void orc3_init_boundary(void* p, const double* cell_vol, const int* cell_fixed, const double* fv0, const double* fv1,
                        const double* fv2, const int* ff0, const int* ff1, const int* ff2, int closed) {
    Handle* h = (Handle*)p;
    Descr& ds = h->H.lv[h->H.l - 1];
    const double* fv[3] = {fv0, fv1, fv2};
    const int* ff[3] = {ff0, ff1, ff2};
    std::vector<int> fixed_i(ds.g.size());
    field_to_blocked(ds.g, cell_vol, fv, ds.vol.data());
    field_to_blocked(ds.g, cell_fixed, ff, fixed_i.data());
    for (int i = 0; i < ds.g.size(); i++) ds.fixed[i] = fixed_i[i] != 0;
    h->energy.vol = ds.vol;
    h->energy.fixed = ds.fixed;
    h->H.closed = closed != 0;
}

// FluidSteadyState3D::update_penalty (:130-150) and FluidEnergy3D::update_penalty.
// The reference calls finish() after setPenalty/toDevice, which also marks the
// padded faces fixed and zeroes vol/penalty on fixed DOFs.
void orc3_update_penalty(void* p, const double* cell_pen, const double* fp0, const double* fp1, const double* fp2) {
    Handle* h = (Handle*)p;
    Descr& ds = h->H.lv[h->H.l - 1];
    const double* fp[3] = {fp0, fp1, fp2};
    field_to_blocked(ds.g, cell_pen, fp, ds.penalty.data());
    ds.finish();
    h->energy.penalty = ds.penalty;
    h->energy.finish();
}

// FluidSteadyState3D::update_b (:116-127).
void orc3_update_b(void* p, const double* cell_b, const double* fb0, const double* fb1, const double* fb2) {
    Handle* h = (Handle*)p;
    const double* fb[3] = {fb0, fb1, fb2};
    field_to_blocked(h->H.lv[h->H.l - 1].g, cell_b, fb, h->b.data());
}
void orc3_set_b_blocked(void* p, const double* b) {
    Handle* h = (Handle*)p;
    std::copy(b, b + h->b.size(), h->b.begin());
}

// FluidSteadyState3D::solve set-up half (:152-156).
void orc3_setup(void* p) { hierarchy_update(((Handle*)p)->H); }
// The same with the GPU solver's coarse penalties (not the reference's).
void orc3_setup_flow(void* p) { hierarchy_update(((Handle*)p)->H, true); }
// The reference's set-up with its Vanka blocks as its block packing leaves them.
void orc3_setup_as_run(void* p) { hierarchy_update(((Handle*)p)->H, false, true); }

// GMRES::Solve with the reference thresholds passed in (common_cpx/GMRES.cpp:20-110).
// stats = {iters, restarts, rel_true, abs_true, precond_res, seconds}
int orc3_solve(void* p, int max_iter, double abs_thr, double rel_thr, double norm_thr, int restarts, double true_tol,
               double* x_out, double* stats) {
    Handle* h = (Handle*)p;
    SolveStats st;
    auto t0 = std::chrono::steady_clock::now();
    gmres_solve(h->H, h->b.data(), h->x.data(), max_iter, abs_thr, rel_thr, norm_thr, restarts, true_tol, st);
    double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (x_out) std::copy(h->x.begin(), h->x.end(), x_out);
    if (stats) {
        stats[0] = st.iters;
        stats[1] = st.restarts;
        stats[2] = st.rel_true;
        stats[3] = st.abs_true;
        stats[4] = st.precond_res;
        stats[5] = sec;
    }
    return st.iters;
}

// ---------------------------------------------------------------- components
// 'level' counts like the reference: 0 = coarsest, levels-1 = finest.
int orc3_level_dof(void* p, int level) { return ((Handle*)p)->H.lv[level].g.size(); }
void orc3_apply_A(void* p, int level, const double* x, double* y) {
    Handle* h = (Handle*)p;
    apply_A(h->H.lv[level], y, x, h->w);
}
void orc3_apply_E(void* p, const double* x, double* y) {
    Handle* h = (Handle*)p;
    apply_E(h->energy, y, x, h->w);
}
void orc3_level_descr(void* p, int level, double* vol, double* pen, uint8_t* fixed) {
    Descr& d = ((Handle*)p)->H.lv[level];
    if (vol) std::copy(d.vol.begin(), d.vol.end(), vol);
    if (pen) std::copy(d.penalty.begin(), d.penalty.end(), pen);
    if (fixed) std::copy(d.fixed.begin(), d.fixed.end(), fixed);
}
void orc3_update_subsystems(void* p) {
    Hierarchy& H = ((Handle*)p)->H;
    for (int i = H.l - 2; i >= 0; i--) update_subsystem(H.lv[i], H.lv[i + 1]);
}
void orc3_restrict(void* p, int coarse_level, const double* rf, double* rc) {
    Hierarchy& H = ((Handle*)p)->H;
    restrict_r(H.lv[coarse_level], H.lv[coarse_level + 1], rc, rf);
}
void orc3_prolong(void* p, int coarse_level, const double* xc, double* xf) {
    Hierarchy& H = ((Handle*)p)->H;
    prolong(H.lv[coarse_level], H.lv[coarse_level + 1], xf, xc);
}
// One colour's block solve (VelDiagPressureFullSmoothing) after orc3_setup.
void orc3_vanka_apply(void* p, int level, int flag, const double* r, double* out) {
    Hierarchy& H = ((Handle*)p)->H;
    const Vanka& v = flag ? H.black[level] : H.red[level];
    vanka_apply(v, H.lv[level].g.size(), out, r);
}
// Pre- (post=0) or post-smoother (post=1) of the V-cycle.
void orc3_smooth(void* p, int level, int post, const double* r, double* out) {
    Handle* h = (Handle*)p;
    Hierarchy& H = h->H;
    const int iters[2] = {2, 2};
    const Vanka* P[2] = {post ? &H.black[level] : &H.red[level], post ? &H.red[level] : &H.black[level]};
    descent_smoother(H.lv[level], P, iters, out, r, h->w);
}
void orc3_coarse_apply(void* p, const double* r, double* out) { dense_apply(((Handle*)p)->H.dense, out, r); }
int orc3_coarse_info(void* p) { return ((Handle*)p)->H.dense.info; }
void orc3_vcycle(void* p, const double* r, double* out) { mg_apply(((Handle*)p)->H, out, r); }

// FluidEnergy3D::compute_energy (fluid_topo/FluidEnergy3D.cpp:94-109): J = 1/2 x^T E x.
double orc3_energy(void* p, const double* x) {
    Handle* h = (Handle*)p;
    std::vector<double> Ex(h->energy.g.size());
    apply_E(h->energy, Ex.data(), x, h->w);
    double s = 0;
    for (size_t i = 0; i < Ex.size(); i++) s += Ex[i] * x[i];
    return 0.5 * s;
}

}  // extern "C"
