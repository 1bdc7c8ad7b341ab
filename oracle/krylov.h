// Reference GMRES restated generically (TEST INFRASTRUCTURE ONLY).
//
// GMRES::Solve (common_cpx/GMRES.cpp:20-110): left-preconditioned, classical
// Gram-Schmidt, x recomputed from the whole basis, stopping on the preconditioned
// residual with the thresholds of common_cpx/GMRES.h:15-17 (passed in). 'restarts' lets
// the oracle reach a tight tolerance by re-running the reference loop on the current
// true residual; restarts = 0 is exactly the reference.
#pragma once
#include <cmath>
#include <functional>
#include <vector>

namespace orc {

using VecOp = std::function<void(double* out, const double* in)>;

struct KrylovStats {
    int iters = 0, restarts = 0;
    double rel_true = 0, abs_true = 0, precond_res = 0;
};

inline double kdot(const double* a, const double* b, int n) {
    double s = 0;
#pragma omp parallel for reduction(+ : s)
    for (int i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

// min ||e0 e_1 - H y|| for the (i+1) x i Hessenberg by Givens rotations (the reference
// uses Eigen's colPivHouseholderQr, common_cpx/GMRES.cpp:84; same minimiser for full rank H)
inline void hessenberg_lsq(const std::vector<double>& Hm, int ld, int i, double e0, std::vector<double>& y, double& res) {
    std::vector<double> R((size_t)(i + 1) * i), g(i + 1, 0.0);
    for (int c = 0; c < i; c++)
        for (int r = 0; r <= i; r++) R[r + (size_t)c * (i + 1)] = Hm[r + (size_t)c * ld];
    g[0] = e0;
    for (int c = 0; c < i; c++) {
        double a = R[c + (size_t)c * (i + 1)], b = R[c + 1 + (size_t)c * (i + 1)];
        double h = std::hypot(a, b);
        double cs = h == 0 ? 1.0 : a / h, sn = h == 0 ? 0.0 : b / h;
        for (int k = c; k < i; k++) {
            double u = R[c + (size_t)k * (i + 1)], v = R[c + 1 + (size_t)k * (i + 1)];
            R[c + (size_t)k * (i + 1)] = cs * u + sn * v;
            R[c + 1 + (size_t)k * (i + 1)] = -sn * u + cs * v;
        }
        double u = g[c], v = g[c + 1];
        g[c] = cs * u + sn * v;
        g[c + 1] = -sn * u + cs * v;
    }
    y.assign(i, 0.0);
    for (int c = i - 1; c >= 0; c--) {
        double s = g[c];
        for (int k = c + 1; k < i; k++) s -= R[c + (size_t)k * (i + 1)] * y[k];
        double d = R[c + (size_t)c * (i + 1)];
        y[c] = d != 0.0 ? s / d : 0.0;
    }
    res = std::fabs(g[i]);
}

inline void gmres_generic(int n, const VecOp& A, const VecOp& M, const double* b, double* x, int max_iter, double abs_thres,
                          double rel_thres, double norm_thres, int restarts, double true_tol, KrylovStats& st) {
    std::vector<double> rr(n), Ax(n), Aq(n), q(n);
    std::fill(x, x + n, 0.0);
    double bn = std::sqrt(kdot(b, b, n));
    st = KrylovStats();
    for (int cyc = 0; cyc <= restarts; cyc++) {
        A(Ax.data(), x);
        for (int k = 0; k < n; k++) rr[k] = b[k] - Ax[k];
        double tr = std::sqrt(kdot(rr.data(), rr.data(), n));
        if (cyc > 0 && (bn == 0 || tr / bn <= true_tol)) break;
        if (cyc > 0) st.restarts++;
        std::vector<std::vector<double>> Q;
        Q.emplace_back(n);
        M(Q[0].data(), rr.data());
        double e0 = std::sqrt(kdot(Q[0].data(), Q[0].data(), n));
        if (e0 == 0) break;
        for (int k = 0; k < n; k++) Q[0][k] /= e0;
        std::vector<double> Hm((size_t)(max_iter + 1) * max_iter, 0.0), y;
        const int ld = max_iter + 1;
        int used = 0;
        bool stop = false;
        for (int i = 1; i < max_iter; i++) {
            A(Aq.data(), Q[i - 1].data());
            M(q.data(), Aq.data());
            std::vector<double> hcol(i);
            for (int j = 0; j < i; j++) hcol[j] = kdot(q.data(), Q[j].data(), n);
            for (int j = 0; j < i; j++) {
                Hm[j + (size_t)(i - 1) * ld] = hcol[j];
                const double* qj = Q[j].data();
                double hj = hcol[j];
#pragma omp parallel for
                for (int k = 0; k < n; k++) q[k] -= hj * qj[k];
            }
            double nq = std::sqrt(kdot(q.data(), q.data(), n));
            if (nq < norm_thres) stop = true;
            Hm[i + (size_t)(i - 1) * ld] = nq;
            Q.emplace_back(n);
            for (int k = 0; k < n; k++) Q[i][k] = nq > 0 ? q[k] / nq : 0.0;
            double res;
            hessenberg_lsq(Hm, ld, i, e0, y, res);
            used = i;
            st.iters++;
            st.precond_res = res;
            if (res < abs_thres) stop = true;
            if (res < rel_thres * e0) stop = true;
            if (stop) break;
        }
        for (int j = 0; j < used; j++) {
            const double* qj = Q[j].data();
            double yj = y[j];
#pragma omp parallel for
            for (int k = 0; k < n; k++) x[k] += yj * qj[k];
        }
    }
    A(Ax.data(), x);
    for (int k = 0; k < n; k++) rr[k] = b[k] - Ax[k];
    st.abs_true = std::sqrt(kdot(rr.data(), rr.data(), n));
    st.rel_true = bn > 0 ? st.abs_true / bn : 0.0;
}

}  // namespace orc
