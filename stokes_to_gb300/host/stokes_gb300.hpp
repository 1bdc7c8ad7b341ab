// C++ mirror of the reference's solver classes over the libstokes_gb300 C ABI.
//
// FluidSteadyState<d> follows FluidSteadyState3D / FluidSteadyState
// (stoke/FluidSteadyState3D.h:11-38, stoke/FluidSteadyState.h): init, init_boundary,
// update_b, update_penalty, solve, with the solution in the public members p and vel.
// FluidEnergy<d> follows FluidEnergy3D / FluidEnergy (fluid_topo/FluidEnergy3D.h:10-44):
// compute_energy, compute_gradient_x, compute_gradient_q. Both work on host arrays in the
// simplex Field order (cell (i,j,k) at (i*N + j)*N + k; face axis d with N+1 entries
// along d). Errors throw stg::Error; a solve that stops short of the tolerance is kept
// (stats().status says so), as the reference keeps its last GMRES iterate.
#pragma once
#include <algorithm>
#include <array>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "stokes_gb300.h"

namespace stg {

class Error : public std::runtime_error {
   public:
    Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

   private:
    int code_;
};

inline int check(int rc, bool allow_not_converged = false) {
    if (rc == STG_OK || (allow_not_converged && rc == STG_E_NOT_CONVERGED)) return rc;
    throw Error(rc, std::string("stokes_gb300: ") + stg_last_error());
}

inline size_t cell_count(int dim, int n) { return dim == 3 ? (size_t)n * n * n : (size_t)n * n; }
inline size_t face_count(int dim, int n) { return dim == 3 ? (size_t)n * n * (n + 1) : (size_t)n * (n + 1); }

// Cell and face arrays of one problem in Field order.
template <int d>
struct Fields {
    int n = 0;
    std::vector<double> cell;
    std::array<std::vector<double>, d> face;
    void resize(int n_) {
        n = n_;
        cell.assign(cell_count(d, n), 0.0);
        for (auto& f : face) f.assign(face_count(d, n), 0.0);
    }
    std::array<const double*, d> cptr() const {
        std::array<const double*, d> a;
        for (int q = 0; q < d; q++) a[q] = face[q].data();
        return a;
    }
    std::array<double*, d> ptr() {
        std::array<double*, d> a;
        for (int q = 0; q < d; q++) a[q] = face[q].data();
        return a;
    }
};

// Boundary description (FluidTopoOptDriver{,3D}::init_boundary outputs).
template <int d>
struct Boundary {
    int n = 0;
    std::vector<double> cell_vol, cell_b;
    std::vector<int32_t> cell_fixed;
    std::array<std::vector<double>, d> face_vol, face_b;
    std::array<std::vector<int32_t>, d> face_fixed;
    bool closed = true;
    void resize(int n_) {
        n = n_;
        cell_vol.assign(cell_count(d, n), 0.0);
        cell_b.assign(cell_count(d, n), 0.0);
        cell_fixed.assign(cell_count(d, n), 0);
        for (int q = 0; q < d; q++) {
            face_vol[q].assign(face_count(d, n), 0.0);
            face_b[q].assign(face_count(d, n), 0.0);
            face_fixed[q].assign(face_count(d, n), 0);
        }
    }
};

// FluidSteadyState3D (d = 3) / FluidSteadyState (d = 2).
template <int d>
class FluidSteadyState {
   public:
    std::vector<double> p;                 // cell pressure after solve()
    std::array<std::vector<double>, d> vel;  // face velocity after solve()

    FluidSteadyState() = default;
    FluidSteadyState(const FluidSteadyState&) = delete;
    FluidSteadyState& operator=(const FluidSteadyState&) = delete;
    ~FluidSteadyState() {
        if (h_) stg_destroy(h_);
    }

    // FluidSteadyState3D::init(N) (stoke/FluidSteadyState3D.cpp:12-90)
    void init(int n, const stg_opts* opts = nullptr) {
        if (h_) stg_destroy(h_);
        h_ = nullptr;
        n_ = n;
        check(stg_create(d, n, opts, &h_));
        p.assign(cell_count(d, n), 0.0);
        for (auto& v : vel) v.assign(face_count(d, n), 0.0);
    }
    // init_boundary(cell_vol, cell_fixed, face_vol, face_fixed, closed) (:92-114)
    void init_boundary(const Boundary<d>& b) {
        std::array<const double*, d> fv;
        std::array<const int32_t*, d> ff;
        for (int q = 0; q < d; q++) {
            fv[q] = b.face_vol[q].data();
            ff[q] = b.face_fixed[q].data();
        }
        check(stg_set_boundary(h_, b.cell_vol.data(), b.cell_fixed.data(), fv.data(), ff.data(), b.closed ? 1 : 0));
    }
    // update_b(cell_b, face_b) (:116-127)
    void update_b(const double* cell_b, const std::array<const double*, d>& face_b) {
        check(stg_set_rhs(h_, cell_b, face_b.data()));
    }
    void update_b(const Boundary<d>& b) {
        std::array<const double*, d> fb;
        for (int q = 0; q < d; q++) fb[q] = b.face_b[q].data();
        update_b(b.cell_b.data(), fb);
    }
    // update_penalty(cell_penalty, face_penalty) (:130-150)
    void update_penalty(const double* cell_pen, const std::array<const double*, d>& face_pen) {
        check(stg_set_penalty(h_, cell_pen, face_pen.data()));
    }
    // solve() (:152-170); keep_on_device skips the copy to p / vel
    const stg_stats& solve(bool keep_on_device = false) {
        if (keep_on_device) {
            check(stg_solve(h_, nullptr, nullptr, &stats_), true);
        } else {
            std::array<double*, d> v;
            for (int q = 0; q < d; q++) v[q] = vel[q].data();
            check(stg_solve(h_, p.data(), v.data(), &stats_), true);
        }
        return stats_;
    }
    void download() {
        std::array<double*, d> v;
        for (int q = 0; q < d; q++) v[q] = vel[q].data();
        check(stg_get_solution(h_, p.data(), v.data()));
    }
    const stg_stats& stats() const { return stats_; }
    int n() const { return n_; }
    stg_t* handle() const { return h_; }

   private:
    stg_t* h_ = nullptr;
    int n_ = 0;
    stg_stats stats_{};
};

// FluidEnergy3D / FluidEnergy on the same handle (the energy operator shares the
// boundary and penalty of the solver, as the reference's init_boundary / update_penalty
// feed both).
template <int d>
class FluidEnergy {
   public:
    explicit FluidEnergy(const FluidSteadyState<d>& s) : s_(s) {}
    // compute_energy(vel, p): J = 1/2 x^T E x (fluid_topo/FluidEnergy3D.cpp:94-109);
    // no arguments: the last solution held on the device
    double compute_energy() const {
        double J = 0;
        check(stg_energy(s_.handle(), nullptr, nullptr, &J));
        return J;
    }
    double compute_energy(const std::vector<double>& p, const std::array<std::vector<double>, d>& vel) const {
        std::array<const double*, d> v;
        for (int q = 0; q < d; q++) v[q] = vel[q].data();
        double J = 0;
        check(stg_energy(s_.handle(), p.data(), v.data(), &J));
        return J;
    }
    // compute_gradient_x: E x (:71-80)
    void compute_gradient_x(Fields<d>& out) const {
        out.resize(s_.n());
        auto v = out.ptr();
        check(stg_energy_grad_x(s_.handle(), nullptr, nullptr, out.cell.data(), v.data()));
    }
    // compute_gradient_q: 1/2 x^2 (:82-91)
    void compute_gradient_q(Fields<d>& out) const {
        out.resize(s_.n());
        auto v = out.ptr();
        check(stg_energy_grad_q(s_.handle(), nullptr, nullptr, out.cell.data(), v.data()));
    }

   private:
    const FluidSteadyState<d>& s_;
};

// ------------------------------------------------------------------ boundary builders
inline size_t fidx(int dim, int n, int d, int i, int j, int k) {
    if (dim == 2) return (size_t)i * (n + (d == 1)) + j;
    return ((size_t)i * (n + (d == 1)) + j) * (n + (d == 2)) + k;
}
inline size_t cidx(int dim, int n, int i, int j, int k) { return dim == 2 ? (size_t)i * n + j : ((size_t)i * n + j) * n + k; }

template <int d>
void fix_domain_boundary(Boundary<d>& b) {
    const int n = b.n;
    for (int q = 0; q < d; q++) {
        const int ni = n + (q == 0), nj = n + (q == 1), nk = d == 3 ? n + (q == 2) : 1;
        for (int i = 0; i < ni; i++)
            for (int j = 0; j < nj; j++)
                for (int k = 0; k < nk; k++) {
                    const int c = q == 0 ? i : q == 1 ? j : k;
                    if (c == 0 || c == n) b.face_fixed[q][fidx(d, n, q, i, j, k)] = 1;
                }
    }
}

// Reference test 0: 2D FluidTopoOptDriver.cpp:104-156 (one inlet, 16 outlets on the
// right edge); 3D FluidTopoOptDriver3D.cpp:104-156 (index ranges fixed for 64^3).
template <int d>
Boundary<d> boundary_test0(int n);

template <>
inline Boundary<2> boundary_test0<2>(int n) {
    Boundary<2> b;
    b.resize(n);
    std::fill(b.cell_vol.begin(), b.cell_vol.end(), 1.0);
    for (auto& f : b.face_vol) std::fill(f.begin(), f.end(), 1.0);
    fix_domain_boundary(b);
    const int O = 16, in_half = n / 32, out_half = n / (4 * O);
    const double e = 60, r = e * (2 * in_half + 1) / (2 * out_half + 1) / O;
    for (int i = 0; i < n; i++) {
        if (std::abs(i - n / 2) > in_half) continue;
        b.cell_b[cidx(2, n, 0, i, 0)] = e;
        b.face_b[0][fidx(2, n, 0, 1, i, 0)] = e;
    }
    for (int o = 0; o < O; o++)
        for (int i = 0; i < n; i++) {
            if (std::abs(i - n / (2 * O) * (2 * o + 1)) > out_half) continue;
            b.cell_b[cidx(2, n, n - 1, i, 0)] = -r;
            b.face_b[0][fidx(2, n, 0, n - 1, i, 0)] = r;
        }
    return b;
}

template <>
inline Boundary<3> boundary_test0<3>(int n) {
    if (n != 64) throw Error(STG_E_INVALID, "3D test 0 is defined for -s 64 (its patches use fixed index ranges)");
    Boundary<3> b;
    b.resize(n);
    std::fill(b.cell_vol.begin(), b.cell_vol.end(), 1.0);
    for (auto& f : b.face_vol) std::fill(f.begin(), f.end(), 1.0);
    fix_domain_boundary(b);
    for (int j = 28; j < 36; j++)
        for (int k = 28; k < 36; k++) {
            b.cell_b[cidx(3, n, 0, j, k)] = 600;
            b.face_b[0][fidx(3, n, 0, 1, j, k)] = 600;
        }
    for (int j = 10; j < 18; j++)
        for (int k = 34; k < 42; k++) {
            b.cell_b[cidx(3, n, n - 1, j, k)] = -200;
            b.face_b[0][fidx(3, n, 0, n - 1, j, k)] = 200;
        }
    for (int i = 28; i < 36; i++)
        for (int j = 22; j < 30; j++) {
            b.cell_b[cidx(3, n, i, j, n - 1)] = -200;
            b.face_b[2][fidx(3, n, 2, i, j, n - 1)] = 200;
        }
    for (int i = 22; i < 30; i++)
        for (int j = 28; j < 36; j++) {
            b.cell_b[cidx(3, n, i, j, 0)] = -200;
            b.face_b[2][fidx(3, n, 2, i, j, 1)] = -200;
        }
    return b;
}

// Parabolic inlet g(s) = 1 - (2s/W)^2 (peak 1) on a centred W-cell segment (2D) or
// W x W patch (3D, product profile) of the x = 0 side, mirrored outlet at x = 1, every
// boundary face fixed; encoded as the reference encodes its inflow (a +g cell source
// and +g on the first interior x-face; outlet -g / +g).
template <int d>
Boundary<d> boundary_parabolic(int n, int width) {
    Boundary<d> b;
    b.resize(n);
    std::fill(b.cell_vol.begin(), b.cell_vol.end(), 1.0);
    for (auto& f : b.face_vol) std::fill(f.begin(), f.end(), 1.0);
    fix_domain_boundary(b);
    const int W = width, lo = n / 2 - W / 2;
    auto prof = [&](int t) {
        double s = (t + 0.5) - n / 2.0;
        return 1.0 - (2.0 * s / W) * (2.0 * s / W);
    };
    for (int j = lo; j < lo + W; j++)
        for (int k = (d == 3 ? lo : 0); k < (d == 3 ? lo + W : 1); k++) {
            const double g = d == 3 ? prof(j) * prof(k) : prof(j);
            b.cell_b[cidx(d, n, 0, j, k)] = g;
            b.face_b[0][fidx(d, n, 0, 1, j, k)] = g;
            b.cell_b[cidx(d, n, n - 1, j, k)] = -g;
            b.face_b[0][fidx(d, n, 0, n - 1, j, k)] = g;
        }
    return b;
}

// ------------------------------------------------------------------ output frames
// Frames in the layout and binary format of the reference drivers
// (FluidTopoOptDriver{,3D}::Write_Output_Files, FT/FluidTopoOptDriver3D.cpp:35-92, with
// simplex/src/common/Driver.h:57-70): <out>/<frame>/{grid (frame 0), velocity, x, psi_D,
// psi_N} and <out>/0/last_frame.txt. Encodings (simplex File::Write_Binary, raw
// little-endian values): Field<T,3> = int32 counts[3] + values; Grid<3> = int32
// cell_counts[3] + double dx + double domain_min[3]; Particles<3> = int32 n + n x
// {X[3], V[3], F[3]} doubles + n x {M, C} doubles + n x int32 I. 2D data go through the
// reference's 3D conversion (counts (N, N, 1), Grid cell_counts (N, N, 0), vectors
// padded with 0). Velocity is the face-to-cell average 0.5 (u(c) + u(c + e_axis))
// (Interpolation::Interpolate_Faces_To_Cells). dx = 1, domain_min = 0, as the drivers'
// grid.Initialize(N, 1.).
namespace frames {

template <class T>
void put(std::ostream& o, const T& v) {
    o.write(reinterpret_cast<const char*>(&v), sizeof(T));
}

inline void write_grid(const std::string& path, int dim, int n) {
    std::ofstream o(path, std::ios::binary);
    const int32_t c[3] = {n, n, dim == 3 ? n : 0};
    for (int q = 0; q < 3; q++) put(o, c[q]);
    put(o, 1.0);
    for (int q = 0; q < 3; q++) put(o, 0.0);
    if (!o) throw Error(STG_E_INVALID, "cannot write " + path);
}

// scalar cell field (Field order) as Field<double,3>
inline void write_scalar(const std::string& path, int dim, int n, const std::vector<double>& a) {
    std::ofstream o(path, std::ios::binary);
    const int32_t c[3] = {n, n, dim == 3 ? n : 1};
    for (int q = 0; q < 3; q++) put(o, c[q]);
    o.write(reinterpret_cast<const char*>(a.data()), (std::streamsize)(a.size() * sizeof(double)));
    if (!o) throw Error(STG_E_INVALID, "cannot write " + path);
}

// face velocity averaged to cells, as Field<Vector3d,3>
template <int d>
void write_velocity(const std::string& path, int n, const std::array<std::vector<double>, d>& vel) {
    std::ofstream o(path, std::ios::binary);
    const int32_t c[3] = {n, n, d == 3 ? n : 1};
    for (int q = 0; q < 3; q++) put(o, c[q]);
    const int nk = d == 3 ? n : 1;
    std::vector<double> buf((size_t)n * n * nk * 3, 0.0);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
            for (int k = 0; k < nk; k++) {
                const size_t cell = cidx(d, n, i, j, k);
                for (int a = 0; a < d; a++) {
                    const double lo = vel[a][fidx(d, n, a, i, j, k)];
                    const double hi = vel[a][fidx(d, n, a, i + (a == 0), j + (a == 1), k + (a == 2))];
                    buf[3 * cell + a] = 0.5 * (lo + hi);
                }
            }
    o.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)(buf.size() * sizeof(double)));
    if (!o) throw Error(STG_E_INVALID, "cannot write " + path);
}

inline void write_particles(const std::string& path, const std::vector<std::array<double, 3>>& X) {
    std::ofstream o(path, std::ios::binary);
    const int32_t np = (int32_t)X.size();
    put(o, np);
    if (np > 0) {
        for (auto& x : X)
            for (int q = 0; q < 3; q++) put(o, x[q]);
        const std::vector<double> zeros((size_t)np * 3, 0.0);
        o.write(reinterpret_cast<const char*>(zeros.data()), (std::streamsize)(zeros.size() * sizeof(double)));  // V
        o.write(reinterpret_cast<const char*>(zeros.data()), (std::streamsize)(zeros.size() * sizeof(double)));  // F
        o.write(reinterpret_cast<const char*>(zeros.data()), (std::streamsize)(np * sizeof(double)));           // M
        o.write(reinterpret_cast<const char*>(zeros.data()), (std::streamsize)(np * sizeof(double)));           // C
        const std::vector<int32_t> izero((size_t)np, 0);
        o.write(reinterpret_cast<const char*>(izero.data()), (std::streamsize)(np * sizeof(int32_t)));          // I
    }
    if (!o) throw Error(STG_E_INVALID, "cannot write " + path);
}

// One frame of a run: the design, the face velocity and the boundary markers (psi_D:
// centres of fixed cells; psi_N: centres of fixed faces, x-faces first).
template <int d>
void write_frame(const std::string& out, int frame, const Boundary<d>& b, const std::vector<double>& design,
                 const std::array<std::vector<double>, d>& vel, void (*mkdir_p)(const std::string&)) {
    const int n = b.n;
    const std::string dir = out + "/" + std::to_string(frame);
    mkdir_p(dir);
    {
        mkdir_p(out + "/0");
        std::ofstream t(out + "/0/last_frame.txt");
        t << frame;
    }
    if (frame == 0) write_grid(dir + "/grid", d, n);
    write_velocity<d>(dir + "/velocity", n, vel);
    write_scalar(dir + "/x", d, n, design);
    const int nk = d == 3 ? n : 1;
    std::vector<std::array<double, 3>> pd, pn;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
            for (int k = 0; k < nk; k++)
                if (b.cell_fixed[cidx(d, n, i, j, k)]) pd.push_back({i + 0.5, j + 0.5, d == 3 ? k + 0.5 : 0.0});
    write_particles(dir + "/psi_D", pd);
    for (int a = 0; a < d; a++) {
        const int ni = n + (a == 0), nj = n + (a == 1), nkk = d == 3 ? n + (a == 2) : 1;
        // the 2D driver walks y-faces with j outermost (FluidTopoOptDriver.cpp Write_Output_Files)
        if (d == 2 && a == 1) {
            for (int j = 0; j < nj; j++)
                for (int i = 0; i < ni; i++)
                    if (b.face_fixed[a][fidx(d, n, a, i, j, 0)]) pn.push_back({i + 0.5, (double)j, 0.0});
            continue;
        }
        for (int i = 0; i < ni; i++)
            for (int j = 0; j < nj; j++)
                for (int k = 0; k < nkk; k++)
                    if (b.face_fixed[a][fidx(d, n, a, i, j, k)])
                        pn.push_back({a == 0 ? (double)i : i + 0.5, a == 1 ? (double)j : j + 0.5,
                                      d == 3 ? (a == 2 ? (double)k : k + 0.5) : 0.0});
    }
    write_particles(dir + "/psi_N", pn);
}

}  // namespace frames

}  // namespace stg
