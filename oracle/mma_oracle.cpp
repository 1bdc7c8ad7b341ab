// Method of Moving Asymptotes, one inequality constraint (TEST INFRASTRUCTURE ONLY).
//
// Restates the reference's vendored MMA solver (simplex/ext/mma/MMASolver.cpp:70-442,
// MIT, "dual interior point" variant of Aage & Lazarov's parallel MMA; Svanberg 1987) for
// m = 1, the case the reference optimizer runs (FT/FluidTopoOpt3D.cpp:74-83, n_cons = 1):
//   * asymptotes: L,U = x -/+ 0.5 (xmax - xmin) for the first two updates, then moved by
//     0.7 / 1.2 according to the sign of (x - x1)(x1 - x2), clamped to
//     [x - 100 w, x - 1e-5 w] / [x + 1e-5 w, x + 100 w], w = max(1e-5, xmax - xmin);
//   * bounds alpha = max(xmin, L + 0.1 (x - L), x - 0.5 w), beta likewise;
//   * convex approximations p = (U - x)^2 (max(0, df) + 0.001 |df| + 1e-5 / w),
//     q = (x - L)^2 (max(0, -df) + ...), for the objective and the constraint;
//   * the dual in lambda (a = 0, c = 1000, d = 0) solved by a primal-dual interior point
//     Newton method with epsilon = 1, 0.1, ... down to sqrt(n + 1) 1e-9.
// Parity of this restatement is pinned against the reference code itself
// (oracle/_ref/libref_mma.so, tests/golden/ref_mma.npz).
#include <algorithm>
#include <cmath>
#include <vector>

namespace {

struct Mma1 {
    int n = 0, iter = 0;
    std::vector<double> low, upp, alpha, beta, p0, q0, p1, q1, xold1, xold2;
    double b = 0, lam = 0, mu = 0, y = 0, z = 0;
    static constexpr double xmamieps = 1e-5, raa0 = 1e-5, move = 0.5, albefa = 0.1;
    static constexpr double asyminit = 0.5, asymdec = 0.7, asyminc = 1.2, a = 0.0, c = 1000.0;

    explicit Mma1(int n_) : n(n_), low(n_), upp(n_), alpha(n_), beta(n_), p0(n_), q0(n_), p1(n_), q1(n_), xold1(n_), xold2(n_) {}

    void gensub(const double* x, const double* df, double g, const double* dg, const double* xmin, const double* xmax) {
        iter++;
        for (int i = 0; i < n; i++) {
            if (iter < 3) {
                low[i] = x[i] - asyminit * (xmax[i] - xmin[i]);
                upp[i] = x[i] + asyminit * (xmax[i] - xmin[i]);
            } else {
                const double sgn = (x[i] - xold1[i]) * (xold1[i] - xold2[i]);
                const double gam = sgn < 0 ? asymdec : (sgn > 0 ? asyminc : 1.0);
                low[i] = x[i] - gam * (xold1[i] - low[i]);
                upp[i] = x[i] + gam * (upp[i] - xold1[i]);
                const double w = std::max(xmamieps, xmax[i] - xmin[i]);
                low[i] = std::min(std::max(low[i], x[i] - 100.0 * w), x[i] - 1e-5 * w);
                upp[i] = std::min(std::max(upp[i], x[i] + 1e-5 * w), x[i] + 100.0 * w);
                const double lo = xmin[i] - 1e-6, hi = xmax[i] + 1e-6;
                if (x[i] < lo) {
                    low[i] = x[i] - (hi - x[i]) / 0.9;
                    upp[i] = x[i] + (hi - x[i]) / 0.9;
                }
                if (x[i] > hi) {
                    low[i] = x[i] - (x[i] - lo) / 0.9;
                    upp[i] = x[i] + (x[i] - lo) / 0.9;
                }
            }
        }
        b = -g;
        for (int i = 0; i < n; i++) {
            alpha[i] = std::min(std::max(std::max(xmin[i], low[i] + albefa * (x[i] - low[i])), x[i] - move * (xmax[i] - xmin[i])),
                                xmax[i]);
            beta[i] = std::max(std::min(std::min(xmax[i], upp[i] - albefa * (upp[i] - x[i])), x[i] + move * (xmax[i] - xmin[i])),
                               xmin[i]);
            const double winv = 1.0 / std::max(xmamieps, xmax[i] - xmin[i]);
            const double du = upp[i] - x[i], dl = x[i] - low[i];
            const double pq0 = 0.001 * std::fabs(df[i]) + raa0 * winv;
            p0[i] = du * du * (std::max(0.0, df[i]) + pq0);
            q0[i] = dl * dl * (std::max(0.0, -df[i]) + pq0);
            const double pq1 = 0.001 * std::fabs(dg[i]) + raa0 * winv;
            p1[i] = du * du * (std::max(0.0, dg[i]) + pq1);
            q1[i] = dl * dl * (std::max(0.0, -dg[i]) + pq1);
            b += p1[i] / du + q1[i] / dl;
        }
    }

    // x(lambda): the minimiser of the Lagrangian on [alpha, beta]; y, z of the dual
    void xyz(double* x) {
        if (lam < 0) lam = 0;
        y = std::max(0.0, lam - c);
        z = std::max(0.0, 10.0 * (lam * a - 1.0));
        for (int i = 0; i < n; i++) {
            const double pl = p0[i] + p1[i] * lam, ql = q0[i] + q1[i] * lam;
            double v = (std::sqrt(pl) * low[i] + std::sqrt(ql) * upp[i]) / (std::sqrt(pl) + std::sqrt(ql));
            x[i] = std::min(std::max(v, alpha[i]), beta[i]);
        }
    }
    double constraint_sum(const double* x) const {
        double s = 0;
        for (int i = 0; i < n; i++) s += p1[i] / (upp[i] - x[i]) + q1[i] / (x[i] - low[i]);
        return s;
    }
    double dual_hess(const double* x) {
        double h = 0;
        for (int i = 0; i < n; i++) {
            const double pl = p0[i] + p1[i] * lam, ql = q0[i] + q1[i] * lam;
            const double du = upp[i] - x[i], dl = x[i] - low[i];
            const double pq = p1[i] / (du * du) - q1[i] / (dl * dl);
            double df2 = -1.0 / (2.0 * pl / (du * du * du) + 2.0 * ql / (dl * dl * dl));
            const double xp = (std::sqrt(pl) * low[i] + std::sqrt(ql) * upp[i]) / (std::sqrt(pl) + std::sqrt(ql));
            if (xp < alpha[i] || xp > beta[i]) df2 = 0.0;
            h += pq * df2 * pq;
        }
        if (lam < 0) lam = 0;
        if (lam > c) h += -1.0;
        h += -mu / lam;
        double corr = 1e-4 * h;
        if (-corr < 1e-7) corr = -1e-7;
        return h + corr;
    }

    void solve_dip(double* x) {
        lam = c / 2.0;
        mu = 1.0;
        const double tol = std::sqrt((double)n + 1.0) * 1e-9;
        double epsi = 1.0, err = 1.0;
        while (epsi > tol) {
            int loop = 0;
            while (err > 0.9 * epsi && loop < 100) {
                loop++;
                xyz(x);
                const double grad = -(-b - a * z - y + constraint_sum(x)) - epsi / lam;
                const double hess = dual_hess(x);
                const double s0 = grad / hess;
                const double s1 = -mu + epsi / lam - s0 * mu / lam;
                double theta = 1.005;
                theta = std::max(theta, -1.01 * s0 / lam);
                theta = std::max(theta, -1.01 * s1 / mu);
                theta = 1.0 / theta;
                lam += theta * s0;
                mu += theta * s1;
                xyz(x);
                const double r0 = -b - a * z - y + mu + constraint_sum(x);
                const double r1 = mu * lam - epsi;
                err = std::max(std::fabs(r0), std::fabs(r1));
            }
            epsi *= 0.1;
        }
    }

    void update(double* x, const double* df, double g, const double* dg, const double* xmin, const double* xmax) {
        gensub(x, df, g, dg, xmin, xmax);
        xold2 = xold1;
        std::copy(x, x + n, xold1.begin());
        solve_dip(x);
    }
};

}  // namespace

extern "C" {
void* orc_mma_create(int n) { return new Mma1(n); }
void orc_mma_destroy(void* p) { delete static_cast<Mma1*>(p); }
// one MMA update in place on x; returns the final dual variable lambda
double orc_mma_update(void* p, double* x, const double* dfdx, double g, const double* dgdx, const double* xmin,
                      const double* xmax) {
    Mma1* s = static_cast<Mma1*>(p);
    s->update(x, dfdx, g, dgdx, xmin, xmax);
    return s->lam;
}
}
