// fluid_topo: command-line driver of the flow topology optimization, drop-in for the
// reference's fluid_topo (fluid_topo/main.cpp:14-59) on libstokes_gb300.
//
//   fluid_topo -driver {0,1} -test k -s N -o dir -frac f -lf iterations
//
// takes the reference's flags with the reference's defaults (-driver 1, -test 2, -s 64,
// -lf 200, -o output; -frac has no usable default there and must be given in (0, 1]).
// -driver 0 runs the 2D problem (FluidTopoOptDriver), 1 the 3D one (FluidTopoOptDriver3D).
// Tests: 0 = the reference's test 0 (2D: one inlet, 16 outlets; 3D: the 64^3 patch case),
// 1 = parabolic inlet on a centred N/4 segment / patch with a mirrored outlet,
// 2 = the reference default (no boundary data; the solve returns zero).
// The loop follows OptimizerMMA::Optimize_MMA (simplex/src/optimization/OptimizerMma.h:96-128):
// iteration k evaluates the objective and its gradient at design k, writes frame k, then
// updates the design; MMA stops once the largest change is <= 1e-3 or after -lf iterations.
// Extra flags:
//   -opt mma|oc the reference's MMA (default for test 0: reference law, no filter) or an
//               optimality-criteria step with a hat filter (default otherwise)
//   -rmin r     filter radius in cells (default 1.5 with oc, none with mma; r <= 1 leaves
//               the design unfiltered)
//   -law ref|bp Brinkman law: the reference's alpha on rho^3 (FluidTopoOpt3D.cpp:110-123,
//               default for test 0) or amax 0.1 (1 - rho)/(0.1 + rho) (default otherwise)
//   -amax a     BP law maximum (1e4);  -move m  OC move limit (0.2)
//   -tol t      FP64 relative residual of every solve (1e-8 in 3D, 1e-10 in 2D)
//   -method plain|mixed   solver precision form (plain)
//   -inner m    FGMRES basis size per refinement step (30); each step of the basis holds two
//               FP32 vectors (V and Z) and an FP16 copy of V, 40 bytes per cell in 3D:
//               5.5 GB at 512^3
//   -basis16 0|1  keep the FP16 basis copies the 3D multi-dots read (default 1; 0 saves 8
//               bytes per cell and basis step: 32 bytes, 4.4 GB at 512^3)
//   -maxouter k FP64 refinement steps per solve (20); a solve that ends without reaching
//               -tol is logged with its residual and the loop goes on
//   -warm 0|1   start each forward / adjoint solve from the previous one (default 1; the
//               reference starts from zero, which -warm 0 reproduces)
//   -init uniform|noise   initial design: frac everywhere, or seeded smoothed noise
//   -seed s -sigma g      noise seed and Gaussian width in cells (1, 4)
//   -frames k   write a frame every k iterations (default 1, as the reference; 0: none)
//   -dump_boundary dir   write the boundary arrays of the test to dir and exit (no GPU)
// Output in -o: log.csv (iteration, objective, volume, change, V-cycles, solve times, the
// final FP64 relative residuals of both solves)
// and frames in the reference drivers' layout and binary format (frame k = design k
// with the velocity of its forward solve): k/x, k/velocity, k/psi_D, k/psi_N, 0/grid,
// 0/last_frame.txt.
#include <sys/stat.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "stokes_gb300.hpp"

namespace {

struct Args {
    std::map<std::string, std::string> kv;
    std::string get(const std::string& k, const std::string& def) const {
        auto it = kv.find(k);
        return it == kv.end() ? def : it->second;
    }
    int geti(const std::string& k, int def) const { return std::stoi(get(k, std::to_string(def))); }
    double getd(const std::string& k, double def) const {
        auto it = kv.find(k);
        return it == kv.end() ? def : std::stod(it->second);
    }
    bool has(const std::string& k) const { return kv.count(k) != 0; }
};

Args parse(int argc, char** argv) {
    static const char* known[] = {"-o",   "-s",    "-test", "-driver", "-lf",  "-frac",   "-rmin",  "-law",   "-amax",
                                  "-move", "-tol", "-method", "-init", "-seed", "-sigma", "-frames", "-verbose",
                                  "-dump_boundary", "-opt", "-warm", "-inner", "-maxouter", "-basis16"};
    Args a;
    for (int i = 1; i < argc; i++) {
        std::string k = argv[i];
        bool ok = false;
        for (const char* q : known) ok = ok || k == q;
        if (!ok || i + 1 >= argc) throw stg::Error(STG_E_INVALID, "unknown flag or missing value: " + k);
        a.kv[k] = argv[++i];
    }
    return a;
}

void make_dir(const std::string& d) {
    std::string cur;
    for (size_t i = 0; i <= d.size(); i++) {
        if (i == d.size() || d[i] == '/') {
            if (!cur.empty()) mkdir(cur.c_str(), 0755);
        }
        if (i < d.size()) cur += d[i];
    }
}

void write_raw(const std::string& path, const std::vector<const std::vector<double>*>& arrays) {
    std::ofstream f(path, std::ios::binary);
    for (auto* a : arrays) f.write(reinterpret_cast<const char*>(a->data()), (std::streamsize)(a->size() * sizeof(double)));
    if (!f) throw stg::Error(STG_E_INVALID, "cannot write " + path);
}

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

template <int d>
int run(const Args& a) {
    const int n = a.geti("-s", 64);
    const int test = a.geti("-test", 2);
    const int iters = a.geti("-lf", 200);
    const double frac = a.getd("-frac", -1.0);
    if (!(frac > 0.0 && frac <= 1.0)) throw stg::Error(STG_E_INVALID, "-frac must be given in (0, 1]");
    const std::string opt = a.get("-opt", test == 0 ? "mma" : "oc");
    if (opt != "mma" && opt != "oc") throw stg::Error(STG_E_INVALID, "-opt must be mma or oc");
    double rmin = a.getd("-rmin", opt == "oc" ? 1.5 : 0.0);
    if (rmin <= 1.0) rmin = 0.5;  // radius below one cell: the hat filter is the identity
    const std::string law_s = a.get("-law", test == 0 ? "ref" : "bp");
    const double move = a.getd("-move", 0.2);
    const std::string out = a.get("-o", "output");
    const int frames = a.geti("-frames", 1);

    stg_opts opts;
    stg_default_opts(&opts);
    opts.tol = a.getd("-tol", d == 3 ? 1e-8 : 1e-10);
    opts.method = a.get("-method", "plain") == "mixed" ? STG_METHOD_MIXED : STG_METHOD_PLAIN;
    opts.verbose = a.geti("-verbose", 0);
    opts.warm_start = a.geti("-warm", 1);
    opts.inner_max = a.geti("-inner", opts.inner_max);
    opts.max_outer = a.geti("-maxouter", opts.max_outer);
    opts.basis16 = a.geti("-basis16", opts.basis16);

    stg_alpha law{};
    if (law_s == "ref") {
        // FluidTopoOpt3D.h:42-46 and Init (alpha_os scaled by 32/N); FluidTopoOpt.h:43-46 in 2D
        law = stg_alpha{STG_ALPHA_REF, 5e2 / (n / 32.0), 1e-3, d == 3 ? 0.01 : 0.014, 0.0};
    } else if (law_s == "bp") {
        law = stg_alpha{STG_ALPHA_BP, 0.0, 0.0, 0.0, a.getd("-amax", 1e4)};
    } else {
        throw stg::Error(STG_E_INVALID, "-law must be ref or bp");
    }

    stg::Boundary<d> b;
    if (test == 0)
        b = stg::boundary_test0<d>(n);
    else if (test == 1)
        b = stg::boundary_parabolic<d>(n, n / 4);
    else {
        b.resize(n);  // reference default: empty boundary data
        std::fill(b.cell_vol.begin(), b.cell_vol.end(), 1.0);
        for (auto& f : b.face_vol) std::fill(f.begin(), f.end(), 1.0);
    }

    if (a.has("-dump_boundary")) {
        // cell_vol, cell_b, face_vol[d], face_b[d] as float64, then cell_fixed, face_fixed[d] as int32
        const std::string dir = a.get("-dump_boundary", ".");
        make_dir(dir);
        std::vector<const std::vector<double>*> dv = {&b.cell_vol, &b.cell_b};
        for (int q = 0; q < d; q++) dv.push_back(&b.face_vol[q]);
        for (int q = 0; q < d; q++) dv.push_back(&b.face_b[q]);
        write_raw(dir + "/boundary_f64.bin", dv);
        std::ofstream f(dir + "/boundary_i32.bin", std::ios::binary);
        f.write(reinterpret_cast<const char*>(b.cell_fixed.data()), (std::streamsize)(b.cell_fixed.size() * 4));
        for (int q = 0; q < d; q++)
            f.write(reinterpret_cast<const char*>(b.face_fixed[q].data()), (std::streamsize)(b.face_fixed[q].size() * 4));
        return 0;
    }

    stg::FluidSteadyState<d> fluid;
    fluid.init(n, &opts);
    fluid.init_boundary(b);
    fluid.update_b(b);
    stg::FluidEnergy<d> energy(fluid);
    stg_t* h = fluid.handle();

    const size_t nc = stg::cell_count(d, n);
    std::vector<double> x(nc, frac), x_old(nc);
    if (a.get("-init", "uniform") == "noise")
        stg::check(stg_density_noise(h, (uint64_t)a.geti("-seed", 1), a.getd("-sigma", 4.0), x.data()));

    make_dir(out);
    std::ofstream log(out + "/log.csv");
    log.precision(17);
    log << "iteration,objective,volume,change,v_cycles_forward,v_cycles_adjoint,solve_ms,iteration_ms,rel_residual_forward,"
           "rel_residual_adjoint\n";
    std::printf("fluid_topo %dD N=%d test %d: %s, %s law, rmin %.2f, frac %.3f, %d iterations, tol %.1e, %s\n", d, n, test,
                opt.c_str(), law_s.c_str(), rmin, frac, iters, opts.tol, stg_version());

    double J = 0;
    for (int it = 0; it < iters; it++) {
        const double t0 = now_ms();
        x_old = x;
        // physical density = H x (FluidTopoOpt3D::Update_Fluid with the filter in front)
        stg::check(stg_filter(h, rmin, x.data(), nullptr, 0));
        stg::check(stg_set_density(h, nullptr, &law));
        const stg_stats& fs = fluid.solve(true);
        const int vf = fs.inner_iters;
        const double sms = fs.solve_ms, rf = fs.rel_residual;
        J = energy.compute_energy();
        // adjoint solve and chain rule (Update_Grad), then H^T for the filter
        stg_stats as{};
        stg::check(stg_adjoint_sensitivity(h, &law, nullptr, &as), true);
        stg::check(stg_filter(h, rmin, nullptr, nullptr, 1));
        if (frames > 0 && it % frames == 0) {
            fluid.download();
            stg::frames::write_frame<d>(out, it, b, x, fluid.vel, make_dir);
        }
        double lam = 0, mma_change = 0;
        if (opt == "oc")
            stg::check(stg_oc_update(h, rmin, x.data(), nullptr, frac, move, 0.0, 1.0, x.data(), &lam));
        else  // the reference optimizer: coef 1e4, bounds [0.01, 1], move 0.2 (FluidTopoOpt3D::Init_MMA)
            stg::check(stg_mma_update(h, x.data(), nullptr, frac, 1e4, 0.01, 1.0, move, x.data(), &mma_change));
        double vol = 0, change = 0;
        for (size_t q = 0; q < nc; q++) {
            vol += x[q];
            change = std::max(change, std::fabs(x[q] - x_old[q]));
        }
        vol /= (double)nc;
        const double tms = now_ms() - t0;
        log << it << "," << J << "," << vol << "," << change << "," << vf << "," << as.inner_iters << "," << sms + as.solve_ms
            << "," << tms << "," << rf << "," << as.rel_residual << "\n";
        std::printf("iter %4d  J %.6e  vol %.4f  change %.3e  V-cycles %d+%d  %.1f ms\n", it, J, vol, change, vf,
                    as.inner_iters, tms);
        if (opt == "mma" && change <= 1e-3) break;  // Optimize_MMA's stopping test (tol 1e-3)
    }
    std::printf("final objective %.8e\n", J);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    try {
        Args a = parse(argc, argv);
        const int driver = a.geti("-driver", 1);
        if (driver == 0) return run<2>(a);
        if (driver == 1) return run<3>(a);
        throw stg::Error(STG_E_INVALID, "-driver must be 0 (2D) or 1 (3D)");
    } catch (const stg::Error& e) {
        std::fprintf(stderr, "fluid_topo: %s\n", e.what());
        return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "fluid_topo: %s\n", e.what());
        return 2;
    }
}
