// Design-loop oracle: alpha laws, face-penalty assembly, adjoint chain rule, density
// filter, optimality-criteria update, seeded densities and boundary builders.
// TEST INFRASTRUCTURE ONLY: the checker for the library's GPU kernels.
//
// Arrays are in the simplex Field order (simplex/src/reservoir/Field.h:67-72):
// 3D cell (i,j,k) -> (i*N + j)*N + k; face axis d has N+1 entries along d.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "topo_common.h"

namespace {

inline int cidx(int n, int i, int j, int k) { return (i * n + j) * n + k; }
inline int fidx(int n, int d, int i, int j, int k) {
    int cy = n + (d == 1), cz = n + (d == 2);
    return (i * cy + j) * cz + k;
}

// Reference alpha law (fluid_topo/FluidTopoOpt3D.cpp:110-123).
inline double alpha_ref(double s, double aos, double aus, double q) { return aos + (aus - aos) * s * (1 + q) / (s + q); }
inline double dalpha_ref(double s, double aos, double aus, double q) {
    return (aus - aos) * ((1 + q) / (s + q) - s * (1 + q) / ((s + q) * (s + q)));
}
// Borrvall-Petersson law alpha(rho) = amax * 0.1 (1 - rho) / (0.1 + rho).
inline double alpha_bp(double r, double amax) { return amax * 0.1 * (1.0 - r) / (0.1 + r); }
inline double dalpha_bp(double r, double amax) { return -amax * 0.1 * 1.1 / ((0.1 + r) * (0.1 + r)); }

}  // namespace

extern "C" {

double orc_uniform(uint64_t seed, uint64_t index) {
    uint64_t z = seed * 0x9E3779B97F4A7C15ull + index + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------- penalty assembly
// FluidTopoOpt3D::Update_Fluid (fluid_topo/FluidTopoOpt3D.cpp:145-159): each cell adds
// t = 1/2 alpha(.) to its 2*dim faces. law 0 = reference law on rho^3, law 1 = BP law on rho.
// p = {aos, aus, q} for law 0; p = {amax} for law 1.
void orc_face_penalty(int dim, int n, const double* rho, int law, const double* p, double* f0, double* f1, double* f2) {
    double* f[3] = {f0, f1, f2};
    if (dim == 3) {
        for (int d = 0; d < 3; d++) std::fill(f[d], f[d] + (size_t)n * n * (n + 1), 0.0);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++)
                for (int k = 0; k < n; k++) {
                    double r = rho[cidx(n, i, j, k)];
                    double t = 0.5 * (law == 0 ? alpha_ref(r * r * r, p[0], p[1], p[2]) : alpha_bp(r, p[0]));
                    for (int d = 0; d < 3; d++) {
                        f[d][fidx(n, d, i, j, k)] += t;
                        f[d][fidx(n, d, i + (d == 0), j + (d == 1), k + (d == 2))] += t;
                    }
                }
    } else {
        // 2D: cell (i,j) -> i*n + j; face axis d has (n+1) entries along d.
        for (int d = 0; d < 2; d++) std::fill(f[d], f[d] + (size_t)n * (n + 1), 0.0);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double r = rho[i * n + j];
                double t = 0.5 * (law == 0 ? alpha_ref(r * r * r, p[0], p[1], p[2]) : alpha_bp(r, p[0]));
                f[0][i * n + j] += t;
                f[0][(i + 1) * n + j] += t;
                f[1][i * (n + 1) + j] += t;
                f[1][i * (n + 1) + j + 1] += t;
            }
    }
}

// FluidTopoOpt3D::Update_Grad chain rule (fluid_topo/FluidTopoOpt3D.cpp:170-198):
// temp_f = -u_f lambda_f + 1/2 u_f^2; dJ/drho_c = 1/2 alpha'(.) (d./drho) sum_{faces of c} temp_f.
void orc_sensitivity(int dim, int n, const double* rho, int law, const double* p, const double* const u[3],
                     const double* const lam[3], double* grad) {
    auto temp = [&](int d, int idx) { return -u[d][idx] * lam[d][idx] + 0.5 * u[d][idx] * u[d][idx]; };
    if (dim == 3) {
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++)
                for (int k = 0; k < n; k++) {
                    double r = rho[cidx(n, i, j, k)];
                    double t = law == 0 ? 0.5 * dalpha_ref(r * r * r, p[0], p[1], p[2]) * 3.0 * r * r : 0.5 * dalpha_bp(r, p[0]);
                    double s = 0;
                    for (int d = 0; d < 3; d++) {
                        s += temp(d, fidx(n, d, i, j, k));
                        s += temp(d, fidx(n, d, i + (d == 0), j + (d == 1), k + (d == 2)));
                    }
                    grad[cidx(n, i, j, k)] = s * t;
                }
    } else {
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double r = rho[i * n + j];
                double t = law == 0 ? 0.5 * dalpha_ref(r * r * r, p[0], p[1], p[2]) * 3.0 * r * r : 0.5 * dalpha_bp(r, p[0]);
                double s = temp(0, i * n + j) + temp(0, (i + 1) * n + j) + temp(1, i * (n + 1) + j) + temp(1, i * (n + 1) + j + 1);
                grad[i * n + j] = s * t;
            }
    }
}

// ---------------------------------------------------------------- density filter
// rho~_i = sum_j w_ij rho_j / sum_j w_ij, w_ij = max(0, rmin - |c_i - c_j|) over cells inside
// the domain (linear hat filter). mode 0 = forward, mode 1 = transpose (sensitivity chain).
void orc_filter(int dim, int n, double rmin, const double* in, double* out, int mode) {
    int R = (int)std::ceil(rmin) - 1;
    if (R < 0) R = 0;
    int nz = dim == 3 ? n : 1, kz = dim == 3 ? R : 0;
    auto idx = [&](int i, int j, int k) { return dim == 3 ? cidx(n, i, j, k) : i * n + j; };
    auto wsum = [&](int i, int j, int k) {
        double W = 0;
        for (int a = -R; a <= R; a++)
            for (int b = -R; b <= R; b++)
                for (int c = -kz; c <= kz; c++) {
                    int ii = i + a, jj = j + b, kk = k + c;
                    if (ii < 0 || jj < 0 || kk < 0 || ii >= n || jj >= n || kk >= nz) continue;
                    double w = rmin - std::sqrt((double)(a * a + b * b + c * c));
                    if (w > 0) W += w;
                }
        return W;
    };
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
            for (int k = 0; k < nz; k++) {
                double W = mode == 0 ? wsum(i, j, k) : 0.0, s = 0;
                for (int a = -R; a <= R; a++)
                    for (int b = -R; b <= R; b++)
                        for (int c = -kz; c <= kz; c++) {
                            int ii = i + a, jj = j + b, kk = k + c;
                            if (ii < 0 || jj < 0 || kk < 0 || ii >= n || jj >= n || kk >= nz) continue;
                            double w = rmin - std::sqrt((double)(a * a + b * b + c * c));
                            if (w <= 0) continue;
                            if (mode == 0)
                                s += w * in[idx(ii, jj, kk)];
                            else
                                s += w * in[idx(ii, jj, kk)] / wsum(ii, jj, kk);
                        }
                out[idx(i, j, k)] = mode == 0 ? s / W : s;
            }
}

// ---------------------------------------------------------------- optimality criteria
// x_new = clamp(x * sqrt(max(0,-dc) / (lambda dv)), max(lo, x - move), min(hi, x + move));
// lambda by bisection so that sum_j vw_j x_new_j (the volume of the filtered design,
// vw_j = sum_i w_ij / W_i) equals frac * ncell, on [0, 1e9] widened by decades while its
// upper end still overshoots the volume. Stops when (l2-l1) <= tol (l1+l2).
// Returns the number of bisection steps; lam_out receives the final lambda.
int orc_oc_update(int ncell, const double* x, const double* dc, const double* dv, const double* vw, double frac, double move,
                  double lo, double hi, double tol, int max_steps, double* x_new, double* lam_out) {
    double l1 = 0.0, l2 = 1e9;
    int steps = 0;
    double target = frac * ncell, lmid = 0;
    for (int k = 0; k < 60; k++) {
        double vol = 0;
        for (int i = 0; i < ncell; i++) {
            double B = std::max(0.0, -dc[i]) / (dv[i] * l2);
            double xn = x[i] * std::sqrt(B);
            vol += vw[i] * std::min(std::min(hi, x[i] + move), std::max(std::max(lo, x[i] - move), xn));
        }
        if (vol <= target) break;
        l1 = l2;
        l2 *= 10.0;
    }
    while ((l2 - l1) > tol * (l1 + l2) && steps < max_steps) {
        lmid = 0.5 * (l1 + l2);
        double vol = 0;
        for (int i = 0; i < ncell; i++) {
            double B = std::max(0.0, -dc[i]) / (dv[i] * lmid);
            double xn = x[i] * std::sqrt(B);
            xn = std::min(std::min(hi, x[i] + move), std::max(std::max(lo, x[i] - move), xn));
            x_new[i] = xn;
            vol += vw[i] * xn;
        }
        if (vol > target)
            l1 = lmid;
        else
            l2 = lmid;
        steps++;
    }
    lmid = 0.5 * (l1 + l2);
    for (int i = 0; i < ncell; i++) {
        double B = std::max(0.0, -dc[i]) / (dv[i] * lmid);
        double xn = x[i] * std::sqrt(B);
        x_new[i] = std::min(std::min(hi, x[i] + move), std::max(std::max(lo, x[i] - move), xn));
    }
    if (lam_out) *lam_out = lmid;
    return steps;
}

// ---------------------------------------------------------------- seeded densities
// rho0 ~ U[0,1) keyed by (seed, Field index); separable Gaussian (sigma, truncated at
// ceil(3 sigma), clamp-to-edge) along axis 0, 1, 2 in that order; clip to [0,1].
void orc_density_noise(int dim, int n, uint64_t seed, double sigma, double* out) {
    size_t nc = dim == 3 ? (size_t)n * n * n : (size_t)n * n;
    std::vector<double> a(nc), b(nc);
    for (size_t i = 0; i < nc; i++) a[i] = orc_uniform(seed, i);
    if (sigma > 0) {
        int R = (int)std::ceil(3.0 * sigma);
        std::vector<double> w(2 * R + 1);
        double s = 0;
        for (int t = -R; t <= R; t++) s += (w[t + R] = std::exp(-(double)(t * t) / (2.0 * sigma * sigma)));
        for (auto& v : w) v /= s;
        size_t st3[3] = {(size_t)n * n, (size_t)n, 1};
        size_t st2[2] = {(size_t)n, 1};
        for (int ax = 0; ax < dim; ax++) {
            size_t stride = dim == 3 ? st3[ax] : st2[ax];
            for (size_t i = 0; i < nc; i++) {
                int c = (int)((i / stride) % n);
                double acc = 0;
                for (int t = -R; t <= R; t++) {
                    int cc = std::min(n - 1, std::max(0, c + t));
                    acc += w[t + R] * a[i + (size_t)((long)cc - c) * stride];
                }
                b[i] = acc;
            }
            std::swap(a, b);
        }
    }
    for (size_t i = 0; i < nc; i++) out[i] = std::min(1.0, std::max(0.0, a[i]));
}

// ---------------------------------------------------------------- boundary builders
// Parabolic inlet / matching outlet in the reference's source-term encoding
// (pattern of fluid_topo/FluidTopoOptDriver3D.cpp:106-156): every boundary face fixed,
// vol = 1, inlet cells cell_b = +g with face_b(first interior x-face) = +g, outlet
// cells cell_b = -g with face_b(last interior x-face) = +g. 3D patch: centred N/4 x N/4
// on x = 0 with g = (1-(2s_j/W)^2)(1-(2s_k/W)^2); 2D: centred W-cell segment.
void orc_bc_parabolic(int dim, int n, int width, double* cell_vol, int* cell_fixed, double* cell_b, double* fv0, double* fv1,
                      double* fv2, int* ff0, int* ff1, int* ff2, double* fb0, double* fb1, double* fb2) {
    double* fv[3] = {fv0, fv1, fv2};
    int* ff[3] = {ff0, ff1, ff2};
    double* fb[3] = {fb0, fb1, fb2};
    int W = width;
    int lo = n / 2 - W / 2;
    auto prof = [&](int t) {
        double s = (t + 0.5) - n / 2.0;
        return 1.0 - (2.0 * s / W) * (2.0 * s / W);
    };
    if (dim == 3) {
        size_t nc = (size_t)n * n * n, nf = (size_t)n * n * (n + 1);
        std::fill(cell_vol, cell_vol + nc, 1.0);
        std::fill(cell_fixed, cell_fixed + nc, 0);
        std::fill(cell_b, cell_b + nc, 0.0);
        for (int d = 0; d < 3; d++) {
            std::fill(fv[d], fv[d] + nf, 1.0);
            std::fill(ff[d], ff[d] + nf, 0);
            std::fill(fb[d], fb[d] + nf, 0.0);
            for (int i = 0; i < n + (d == 0); i++)
                for (int j = 0; j < n + (d == 1); j++)
                    for (int k = 0; k < n + (d == 2); k++) {
                        int c = d == 0 ? i : d == 1 ? j : k;
                        if (c == 0 || c == n) ff[d][fidx(n, d, i, j, k)] = 1;
                    }
        }
        for (int j = lo; j < lo + W; j++)
            for (int k = lo; k < lo + W; k++) {
                double g = prof(j) * prof(k);
                cell_b[cidx(n, 0, j, k)] = g;
                fb[0][fidx(n, 0, 1, j, k)] = g;
                cell_b[cidx(n, n - 1, j, k)] = -g;
                fb[0][fidx(n, 0, n - 1, j, k)] = g;
            }
    } else {
        size_t nc = (size_t)n * n, nf = (size_t)n * (n + 1);
        std::fill(cell_vol, cell_vol + nc, 1.0);
        std::fill(cell_fixed, cell_fixed + nc, 0);
        std::fill(cell_b, cell_b + nc, 0.0);
        for (int d = 0; d < 2; d++) {
            std::fill(fv[d], fv[d] + nf, 1.0);
            std::fill(ff[d], ff[d] + nf, 0);
            std::fill(fb[d], fb[d] + nf, 0.0);
        }
        for (int j = 0; j < n; j++) {
            ff[0][0 * n + j] = 1;
            ff[0][n * n + j] = 1;
        }
        for (int i = 0; i < n; i++) {
            ff[1][i * (n + 1) + 0] = 1;
            ff[1][i * (n + 1) + n] = 1;
        }
        for (int j = lo; j < lo + W; j++) {
            double g = prof(j);
            cell_b[0 * n + j] = g;
            fb[0][1 * n + j] = g;
            cell_b[(n - 1) * n + j] = -g;
            fb[0][(n - 1) * n + j] = g;
        }
    }
}

// Reference test 0 (fluid_topo/FluidTopoOptDriver3D.cpp:99-157); valid for N >= 64.
void orc_bc_test0_3d(int n, double* cell_vol, int* cell_fixed, double* cell_b, double* fv0, double* fv1, double* fv2, int* ff0,
                     int* ff1, int* ff2, double* fb0, double* fb1, double* fb2) {
    double* fv[3] = {fv0, fv1, fv2};
    int* ff[3] = {ff0, ff1, ff2};
    double* fb[3] = {fb0, fb1, fb2};
    size_t nc = (size_t)n * n * n, nf = (size_t)n * n * (n + 1);
    std::fill(cell_vol, cell_vol + nc, 1.0);
    std::fill(cell_fixed, cell_fixed + nc, 0);
    std::fill(cell_b, cell_b + nc, 0.0);
    for (int d = 0; d < 3; d++) {
        std::fill(fv[d], fv[d] + nf, 1.0);
        std::fill(ff[d], ff[d] + nf, 0);
        std::fill(fb[d], fb[d] + nf, 0.0);
    }
    for (int j = 0; j < n; j++)
        for (int k = 0; k < n; k++) {
            ff[0][fidx(n, 0, 0, j, k)] = 1;
            ff[0][fidx(n, 0, n, j, k)] = 1;
        }
    for (int i = 0; i < n; i++)
        for (int k = 0; k < n; k++) {
            ff[1][fidx(n, 1, i, 0, k)] = 1;
            ff[1][fidx(n, 1, i, n, k)] = 1;
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            ff[2][fidx(n, 2, i, j, 0)] = 1;
            ff[2][fidx(n, 2, i, j, n)] = 1;
        }
    for (int j = 28; j < 36; j++)
        for (int k = 28; k < 36; k++) {
            cell_b[cidx(n, 0, j, k)] = 600;
            fb[0][fidx(n, 0, 1, j, k)] = 600;
        }
    for (int j = 10; j < 18; j++)
        for (int k = 34; k < 42; k++) {
            cell_b[cidx(n, n - 1, j, k)] = -200;
            fb[0][fidx(n, 0, n - 1, j, k)] = 200;
        }
    for (int i = 28; i < 36; i++)
        for (int j = 22; j < 30; j++) {
            cell_b[cidx(n, i, j, n - 1)] = -200;
            fb[2][fidx(n, 2, i, j, n - 1)] = 200;
        }
    for (int i = 22; i < 30; i++)
        for (int j = 28; j < 36; j++) {
            cell_b[cidx(n, i, j, 0)] = -200;
            fb[2][fidx(n, 2, i, j, 1)] = -200;
        }
}

}  // extern "C"
