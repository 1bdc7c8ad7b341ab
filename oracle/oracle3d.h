// CPU oracle for the 3D Brinkman-Stokes hot path of Stokes_TO.
//
// TEST INFRASTRUCTURE ONLY. This is a plain FP64 restatement of the reference
// algorithm, used as the checker by the tests, by __graft_entry__.smoke() and as
// the timed CPU baseline of bench.py. The product (libstokes_gb300.so) never
// links, loads or calls it.
//
// Parity status: pinned. The blocked layout index math is checked against the
// reference's own compiled host functions, and every value this oracle computes (the
// descriptors of every level, A, E, restriction, prolongation, the Vanka block solves,
// the composite smoothers, the coarsest dense solve, the V-cycle and the GMRES solve)
// against golden vectors produced by the reference's own CUDA solver code, run on the
// host through oracle/ref_emu (tests/golden/make_ref_golden.py, tests/test_ref_golden_cpu.py).
// The reference's Vanka block packing misplaces one block entry in 32; vanka_setup's
// reorder_as_run reproduces that, the default builds the intended blocks.
#pragma once
#include <cstdint>
#include <vector>

namespace orc {

// Reference blocked grid (simplex/src/common_cpx/grid3D.cu:24-146).
struct G3 {
    int nx = 0, ny = 0, nz = 0;
    G3() {}
    G3(int a, int b, int c) : nx(a), ny(b), nz(c) {}
    int cell_size() const { return nx * ny * nz; }
    int face_size(int d) const { return (nx + 4 * (d == 0)) * (ny + 4 * (d == 1)) * (nz + 4 * (d == 2)); }
    int edge_size(int d) const { return (nx + 4 * (d != 0)) * (ny + 4 * (d != 1)) * (nz + 4 * (d != 2)); }
    int size() const { return cell_size() + face_size(0) + face_size(1) + face_size(2); }
    int face_off(int d) const {
        int o = cell_size();
        for (int p = 0; p < d; p++) o += face_size(p);
        return o;
    }
    int cell_ind(int x, int y, int z) const;
    int face_ind(int x, int y, int z, int d) const;
    int edge_ind(int x, int y, int z, int d) const;
    void ind_cell(int i, int& x, int& y, int& z) const;
    void ind_face(int i, int d, int& x, int& y, int& z) const;
    bool cell_valid(int x, int y, int z) const { return x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz; }
    bool face_valid(int x, int y, int z, int d) const {
        return x >= 0 && x < nx + (d == 0) && y >= 0 && y < ny + (d == 1) && z >= 0 && z < nz + (d == 2);
    }
    bool edge_valid(int x, int y, int z, int d) const {
        return x >= 0 && x < nx + (d != 0) && y >= 0 && y < ny + (d != 1) && z >= 0 && z < nz + (d != 2);
    }
};

// Per-level coefficient arrays (stoke/StokeFlowDescriptor3D.cu:6-65).
struct Descr {
    G3 g;
    std::vector<double> vol, penalty;
    std::vector<uint8_t> fixed;
    void init(int n);
    void finish();
};

struct Work {
    std::vector<double> t, e;
    void ensure(const G3& g) {
        t.resize(g.size());
        e.resize(g.edge_size(0) + g.edge_size(1) + g.edge_size(2));
    }
};

struct Vanka {
    int flag = 0, nb = 0;
    std::vector<double> lu;  // nb blocks, 7x7 column-major LU factors
    std::vector<int> piv;
    std::vector<int> dofs;  // nb*7 packed -> full index
};

struct Dense {
    int n = 0;
    std::vector<double> a;  // column-major n x n, LU factors after set-up
    std::vector<int> piv;
    int info = 0;
};

struct Hierarchy {
    int l = 0;
    std::vector<Descr> lv;  // lv[l-1] finest ... lv[0] coarsest
    std::vector<Vanka> red, black;
    Dense dense;
    bool closed = true;
    Work w;
    std::vector<std::vector<double>> r, x, p, Ap;
};

struct SolveStats {
    int iters = 0, restarts = 0;
    double rel_true = 0, abs_true = 0, precond_res = 0;
};

void apply_A(const Descr& ds, double* Ap, const double* p, Work& w);
void apply_E(const Descr& ds, double* Ap, const double* p, Work& w);
void update_subsystem(Descr& c, const Descr& f);
void restrict_r(const Descr& c, const Descr& f, double* rc, const double* rf);
void prolong(const Descr& c, const Descr& f, double* xf, const double* xc);
void vanka_setup(const Descr& ds, int flag, Vanka& v, Work& w, bool reorder_as_run = false);
void vanka_apply(const Vanka& v, int n, double* out, const double* r);
void descent_smoother(const Descr& ds, const Vanka* P[2], const int iters[2], double* out, const double* r_in, Work& w);
void dense_setup(const Descr& ds, bool closed, Dense& D, Work& w);
void dense_apply(const Dense& D, double* out, const double* r);
int level_count(int n);
void hierarchy_init(Hierarchy& H, int n);
// flow: the GPU solver's coarse penalties (8 x the smallest free child) instead of the sums;
// reorder_as_run: the Vanka blocks as the reference's block packing produces them (vanka_setup)
void flow_penalties(Descr& c, const Descr& f);
void hierarchy_update(Hierarchy& H, bool flow = false, bool reorder_as_run = false);
void vcycle(Hierarchy& H);
void mg_apply(Hierarchy& H, double* out, const double* in);
void gmres_solve(Hierarchy& H, const double* b, double* x, int max_iter, double abs_thres, double rel_thres,
                 double norm_thres, int restarts, double true_tol, SolveStats& st);

}  // namespace orc
