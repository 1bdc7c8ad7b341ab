// 2D path (dim = 2) of libstokes_gb300.
//
// The 2D configuration is small (64^2: 13,312 unknowns) and latency-bound, so its
// vectors stay in the reference's own 8x8-blocked solver layout
// [cells | x-faces | y-faces] (common_cpx/form01mapping.cu:10-57) and every kernel is a
// thread per unknown. The algorithm is the reference's 2D one:
//   A          stoke/StokeFlowMapping.cu:30-139 (grad-div, node-based curl-curl on the raw
//              velocity, -grad p, div, penalty; no definite fix: fixed rows are zero)
//   E          fluid_topo/FluidEnergyGrad.cu:30-61 (5-point face Laplacian + P x)
//   coarsening stoke/StokeFlowSubSystem.cu:100-160 (lap_coeff doubles per level)
//   smoother   stoke/StokeFlowSmoothing.cu:8-209 (5-unknown box with two 2x2 velocity
//              blocks, colours (x + y + flag) even, r-form with a residual update per colour)
//   coarsest   stoke/StokeFlowDirectSolve.cpp:6-133 (analytic dense matrix), inverted on
//              the GPU by Gauss-Jordan and applied as a GEMV
//   V-cycle    common_cpx/MultigridSolve.cpp:73-106 in FP32; Krylov as in 3D (solve_core).
#include <cmath>
#include <vector>

#include "alpha.cuh"
#include "ctx.h"

namespace stg {

namespace {

constexpr int TPB = 256;

// common_cpx/form01mapping.cu:10-57 (faces padded by 8 along their normal)
struct G2d {
    int n = 0;
    __host__ __device__ int nc() const { return n * n; }
    __host__ __device__ int fs(int d) const { return (n + 8 * (d == 0)) * (n + 8 * (d == 1)); }
    __host__ __device__ int size() const { return nc() + fs(0) + fs(1); }
    __host__ __device__ int off(int d) const { return nc() + (d == 1 ? fs(0) : 0); }
    __host__ __device__ int cell(int x, int y) const { return ((y >> 3) * (n >> 3) + (x >> 3)) * 64 + ((y & 7) * 8 + (x & 7)); }
    __host__ __device__ int face(int x, int y, int d) const {
        int b = (y >> 3) * ((n >> 3) + (d == 0)) + (x >> 3);
        int ix = x & 7, iy = y & 7;
        return off(d) + b * 64 + (d == 0 ? ix * 8 + iy : iy * 8 + ix);
    }
    __host__ __device__ bool cell_ok(int x, int y) const { return x >= 0 && y >= 0 && x < n && y < n; }
    __host__ __device__ bool face_ok(int x, int y, int d) const {
        return x >= 0 && y >= 0 && (d == 0 ? (x <= n && y < n) : (x < n && y <= n));
    }
    // stored index -> kind (-1 cell, 0/1 face axis) and coordinates
    __host__ __device__ void decode(int t, int& kind, int& x, int& y) const {
        if (t < nc()) {
            kind = -1;
            int b = t >> 6, ix = t & 7, iy = (t >> 3) & 7;
            x = (b % (n >> 3)) * 8 + ix;
            y = (b / (n >> 3)) * 8 + iy;
            return;
        }
        t -= nc();
        int d = t < fs(0) ? 0 : 1;
        if (d == 1) t -= fs(0);
        int b = t >> 6, i = t & 63;
        int nbx = (n >> 3) + (d == 0);
        int ix = d == 0 ? i >> 3 : i & 7, iy = d == 0 ? i & 7 : i >> 3;
        kind = d;
        x = (b % nbx) * 8 + ix;
        y = (b / nbx) * 8 + iy;
    }
};

// ------------------------------------------------------------------ operator rows
template <class T>
struct Coef2 {
    const T* vol;
    const T* pen;
    const uint8_t* fixed;
};

template <class T>
__device__ __forceinline__ T fval(const G2d& g, const T* v, int x, int y, int d) {
    return g.face_ok(x, y, d) ? v[g.face(x, y, d)] : T(0);
}
template <class T>
__device__ __forceinline__ T vval(const G2d& g, const Coef2<T>& C, const T* v, int x, int y, int d) {
    if (!g.face_ok(x, y, d)) return T(0);
    int i = g.face(x, y, d);
    return C.vol[i] * v[i];
}
// fix_c D (V u) of cell (x, y); 0 outside the grid
template <class T>
__device__ __forceinline__ T divp(const G2d& g, const Coef2<T>& C, const T* v, int x, int y) {
    if (!g.cell_ok(x, y) || C.fixed[g.cell(x, y)]) return T(0);
    return (vval(g, C, v, x + 1, y, 0) - vval(g, C, v, x, y, 0)) + (vval(g, C, v, x, y + 1, 1) - vval(g, C, v, x, y, 1));
}
// node(x,y) = u(x,y-1) - u(x,y) - v(x-1,y) + v(x,y) on the raw velocity (form01mapping.cu:256-300)
template <class T>
__device__ __forceinline__ T node(const G2d& g, const T* v, int x, int y) {
    return fval(g, v, x, y - 1, 0) - fval(g, v, x, y, 0) - fval(g, v, x - 1, y, 1) + fval(g, v, x, y, 1);
}
template <class T>
__device__ __forceinline__ T cval(const G2d& g, const T* v, int x, int y) {
    return g.cell_ok(x, y) ? v[g.cell(x, y)] : T(0);
}

// one row of A (MODE 0), b - A x (MODE 1) or E (MODE 2, lap = lap_coeff of the energy)
template <class T, int MODE>
__device__ __forceinline__ T row(const G2d& g, const Coef2<T>& C, T lap, const T* v, int t) {
    int kind, x, y;
    g.decode(t, kind, x, y);
    const T pen = C.pen[t];
    if (kind < 0) {
        T out = pen * v[t];
        if (MODE != 2) out += divp(g, C, v, x, y);
        return out;
    }
    const int d = kind;
    if (!g.face_ok(x, y, d) || C.fixed[t]) return pen * v[t];  // zero rows (pen is 0 there)
    if (MODE == 2) {
        // 5-point Laplacian over the stored face array (faceLapMapping, form01mapping.cu:430-525)
        const int X = d == 0 ? g.n + 8 : g.n, Y = d == 0 ? g.n : g.n + 8;
        auto F = [&](int a, int b) { return (a >= 0 && b >= 0 && a < X && b < Y) ? v[g.face(a, b, d)] : T(0); };
        T l = T(4) * v[t] - F(x - 1, y) - F(x + 1, y) - F(x, y - 1) - F(x, y + 1);
        return lap * l + pen * v[t];
    }
    const T vol = C.vol[t];
    T gd, cc, gp;
    if (d == 0) {
        gd = -(divp(g, C, v, x, y) - divp(g, C, v, x - 1, y));
        cc = vol * (node(g, v, x, y + 1) - node(g, v, x, y));
        gp = vol * (cval(g, v, x, y) - cval(g, v, x - 1, y));
    } else {
        gd = -(divp(g, C, v, x, y) - divp(g, C, v, x, y - 1));
        cc = vol * (-(node(g, v, x + 1, y) - node(g, v, x, y)));
        gp = vol * (cval(g, v, x, y) - cval(g, v, x, y - 1));
    }
    return gd + cc - gp + pen * v[t];
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <class T, int MODE>
__global__ void k2_apply(G2d g, Coef2<T> C, T lap, const T* __restrict__ v, const T* __restrict__ b, T* __restrict__ out,
                         double* __restrict__ part) {
    __shared__ double sh[TPB / 32];
    int t = blockIdx.x * TPB + threadIdx.x;
    double acc = 0;
    if (t < g.size()) {
        T o = row<T, MODE == 1 ? 0 : MODE>(g, C, lap, v, t);
        if (MODE == 1) {
            o = b[t] - o;
            acc = (double)o * o;
        } else if (MODE == 2) {
            acc = (double)v[t] * o;
        }
        out[t] = o;
    }
    if (part) {
        acc = warp_sum(acc);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0;
            for (int w = 0; w < TPB / 32; w++) s += sh[w];
            part[blockIdx.x] = s;
        }
    }
}

// ------------------------------------------------------------------ smoother colour
// One colour of the 2D box smoother (the operator of stoke/StokeFlowSmoothing.cu:74-140):
// every cell of the colour solves for its 5 unknowns - the x-faces a (low) and b (high),
// the y-faces c (low) and d (high), the pressure p - with the box matrix
//
//     | K    g  |  | u |   | r_u |       K = diag(K_x, K_y),  K_x = | 4L+P_a   -s_x |
//     | g^T  P_p|  | p | = | r_p |                                  | -s_x   4L+P_b |
//
// where L is the level's Laplacian coefficient, s_x = L unless face a or b is fixed (0
// then), K_y likewise, and g = (-vol_a, vol_b, -vol_c, vol_d) holds the divergence
// weights. Block elimination: z = K^-1 r_u, w = K^-1 g, p = (r_p - g.z) / (P_p - g.w),
// u = z - p w; a fixed cell keeps p = 0. Each 2x2 block of K is inverted once and applied
// to both right-hand sides.
struct SymInv2 {
    float i00, i01, i11;  // inverse of [[d0, -s], [-s, d1]]
    __device__ __forceinline__ SymInv2(float d0, float d1, float s) {
        const float rdet = 1.f / (d0 * d1 - s * s);
        i00 = d1 * rdet;
        i11 = d0 * rdet;
        i01 = s * rdet;
    }
    __device__ __forceinline__ void apply(float v0, float v1, float& o0, float& o1) const {
        o0 = i00 * v0 + i01 * v1;
        o1 = i01 * v0 + i11 * v1;
    }
};

__global__ void k2_smooth(G2d g, Coef2<float> C, float lap, int flag, const float* __restrict__ r, float* __restrict__ dout) {
    const int c = blockIdx.x * TPB + threadIdx.x;
    if (c >= g.nc()) return;
    const int x = (c / 64 % (g.n >> 3)) * 8 + (c & 7), y = (c / 64 / (g.n >> 3)) * 8 + ((c >> 3) & 7);
    if ((((x & 1) ^ (y & 1) ^ flag)) != 0) return;
    const int fa = g.face(x, y, 0), fb = g.face(x + 1, y, 0), fc = g.face(x, y, 1), fd = g.face(x, y + 1, 1);
    const int cp = g.cell(x, y);
    const float sx = (C.fixed[fa] || C.fixed[fb]) ? 0.f : lap;
    const float sy = (C.fixed[fc] || C.fixed[fd]) ? 0.f : lap;
    const SymInv2 Kx(4.f * lap + C.pen[fa], 4.f * lap + C.pen[fb], sx);
    const SymInv2 Ky(4.f * lap + C.pen[fc], 4.f * lap + C.pen[fd], sy);
    const float ga = -C.vol[fa], gb = C.vol[fb], gc = -C.vol[fc], gd = C.vol[fd];
    float za, zb, zc, zd, wa, wb, wc, wd;
    Kx.apply(r[fa], r[fb], za, zb);
    Ky.apply(r[fc], r[fd], zc, zd);
    Kx.apply(ga, gb, wa, wb);
    Ky.apply(gc, gd, wc, wd);
    const float schur = C.pen[cp] - (ga * wa + gb * wb + gc * wc + gd * wd);
    const float rhs_p = r[cp] - (ga * za + gb * zb + gc * zc + gd * zd);
    const float p = C.fixed[cp] ? 0.f : rhs_p / schur;
    dout[fa] = za - p * wa;
    dout[fb] = zb - p * wb;
    dout[fc] = zc - p * wc;
    dout[fd] = zd - p * wd;
    dout[cp] = p;
}

// ------------------------------------------------------------------ transfers and coarsening
// children of a coarse unknown: (2X + a, 2Y + b), order (0,0), (1,0), (0,1), (1,1)
template <class T>
__global__ void k2_restrict(G2d gc, G2d gf, const T* __restrict__ rf, const uint8_t* __restrict__ cfixed, T* __restrict__ rc) {
    int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= gc.size()) return;
    int kind, X, Y;
    gc.decode(t, kind, X, Y);
    T s = 0;
    for (int q = 0; q < 4; q++) {
        int x = 2 * X + (q & 1), y = 2 * Y + (q >> 1);
        if (kind < 0)
            s += rf[gf.cell(x, y)];
        else if (gf.face_ok(x, y, kind))
            s += rf[gf.face(x, y, kind)];
    }
    rc[t] = cfixed[t] ? T(0) : s;
}

template <class T>
__global__ void k2_prolong(G2d gf, G2d gc, const T* __restrict__ xc, const uint8_t* __restrict__ ffixed, T* __restrict__ xf) {
    int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= gf.size()) return;
    int kind, x, y;
    gf.decode(t, kind, x, y);
    T v = 0;
    if (kind < 0)
        v = xc[gc.cell(x >> 1, y >> 1)];
    else if (gf.face_ok(x, y, kind))
        v = xc[gc.face(x >> 1, y >> 1, kind)];
    xf[t] = ffixed[t] ? T(0) : v;
}

// finish(): padded faces fixed, vol and penalty zero on fixed (stoke/StokeFlowDescriptor.cpp:40-46)
__device__ __forceinline__ bool padded2(const G2d& g, int kind, int x, int y) {
    return kind >= 0 && !g.face_ok(x, y, kind);
}

// FLOW (the solver's own hierarchy): a coarse face takes 4 x the smallest penalty of its
// children instead of the sum, so channels narrower than a coarse cell stay open on the
// coarse levels (the 3D k_coarsen gives the reason; oracle/oracle2d.cpp flow_penalties
// restates the rule).
template <bool FLOW>
__global__ void k2_coarsen(G2d gc, G2d gf, const uint8_t* __restrict__ ff, const double* __restrict__ fvol,
                           const double* __restrict__ fpen, uint8_t* __restrict__ cf, double* __restrict__ cvol,
                           double* __restrict__ cpen, float* __restrict__ cvol32, float* __restrict__ cpen32) {
    int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= gc.size()) return;
    int kind, X, Y;
    gc.decode(t, kind, X, Y);
    uint8_t fx = 0;
    double v = 0, p = 0, lo = INFINITY;
    for (int q = 0; q < 4; q++) {
        int x = 2 * X + (q & 1), y = 2 * Y + (q >> 1);
        int i;
        if (kind < 0)
            i = gf.cell(x, y);
        else if (gf.face_ok(x, y, kind))
            i = gf.face(x, y, kind);
        else
            continue;
        fx |= ff[i];
        p += fpen[i];
        lo = fmin(lo, fpen[i]);
        // cells: sum of 4; faces: the 2 coincident children (zero offset along the normal)
        bool coincident = kind < 0 || (kind == 0 ? (q & 1) == 0 : (q >> 1) == 0);
        if (coincident) v += fvol[i];
    }
    if (FLOW && kind >= 0 && lo < INFINITY) p = 4.0 * lo;
    if (padded2(gc, kind, X, Y)) fx = 1;
    if (fx) v = p = 0;
    cf[t] = fx;
    cvol[t] = v;
    cpen[t] = p;
    cvol32[t] = (float)v;
    cpen32[t] = (float)p;
}

// fine descriptor from Field-order host inputs (staged on the device)
__global__ void k2_fine_descr(G2d g, const double* __restrict__ cvol, const int* __restrict__ cfix, const double* __restrict__ fv0,
                              const double* __restrict__ fv1, const int* __restrict__ ff0, const int* __restrict__ ff1,
                              uint8_t* __restrict__ fixed, double* __restrict__ vol) {
    int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= g.size()) return;
    int kind, x, y;
    g.decode(t, kind, x, y);
    const int n = g.n;
    uint8_t f = 0;
    double v = 0;
    if (kind < 0) {
        f = cfix ? (cfix[x * n + y] != 0) : 0;
        v = cvol ? cvol[x * n + y] : 0.0;
    } else if (g.face_ok(x, y, kind)) {
        int idx = kind == 0 ? x * n + y : x * (n + 1) + y;
        f = (kind == 0 ? ff0 : ff1)[idx] != 0;
        v = (kind == 0 ? fv0 : fv1)[idx];
    } else {
        f = 1;
    }
    fixed[t] = f;
    vol[t] = f ? 0.0 : v;
}

__global__ void k2_penalty_from_field(G2d g, const double* __restrict__ cp, const double* __restrict__ f0,
                                      const double* __restrict__ f1, const uint8_t* __restrict__ fixed,
                                      double* __restrict__ pen, float* __restrict__ pen32) {
    int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= g.size()) return;
    int kind, x, y;
    g.decode(t, kind, x, y);
    const int n = g.n;
    double v = 0;
    if (kind < 0)
        v = cp ? cp[x * n + y] : 0.0;
    else if (g.face_ok(x, y, kind))
        v = (kind == 0 ? f0 : f1) ? (kind == 0 ? f0 : f1)[kind == 0 ? x * n + y : x * (n + 1) + y] : 0.0;
    if (fixed[t]) v = 0;
    pen[t] = v;
    pen32[t] = (float)v;
}

__global__ void k2_field_to_blocked(G2d g, const double* __restrict__ cell, const double* __restrict__ f0,
                                    const double* __restrict__ f1, double* __restrict__ out) {
    int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= g.size()) return;
    int kind, x, y;
    g.decode(t, kind, x, y);
    const int n = g.n;
    double v = 0;
    if (kind < 0)
        v = cell ? cell[x * n + y] : 0.0;
    else if (g.face_ok(x, y, kind)) {
        const double* f = kind == 0 ? f0 : f1;
        v = f ? f[kind == 0 ? x * n + y : x * (n + 1) + y] : 0.0;
    }
    out[t] = v;
}

__global__ void k2_blocked_to_field(G2d g, const double* __restrict__ in, double* __restrict__ cell, double* __restrict__ f0,
                                    double* __restrict__ f1) {
    int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= g.size()) return;
    int kind, x, y;
    g.decode(t, kind, x, y);
    const int n = g.n;
    if (kind < 0) {
        if (cell) cell[x * n + y] = in[t];
    } else if (g.face_ok(x, y, kind)) {
        double* f = kind == 0 ? f0 : f1;
        if (f) f[kind == 0 ? x * n + y : x * (n + 1) + y] = in[t];
    }
}

// face penalty = 1/2 alpha(left cell) + 1/2 alpha(right cell), zero on fixed
// (fluid_topo/FluidTopoOpt.cpp:143-160)
__global__ void k2_face_penalty(G2d g, const double* __restrict__ rho, stg_alpha L, const uint8_t* __restrict__ fixed,
                                double* __restrict__ pen, float* __restrict__ pen32) {
    int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= g.size()) return;
    int kind, x, y;
    g.decode(t, kind, x, y);
    const int n = g.n;
    double v = 0;
    if (kind >= 0 && g.face_ok(x, y, kind)) {
        int lx = x - (kind == 0), ly = y - (kind == 1);
        double lo = g.cell_ok(lx, ly) ? 0.5 * alpha_of(rho[lx * n + ly], L) : 0.0;
        double hi = g.cell_ok(x, y) ? 0.5 * alpha_of(rho[x * n + y], L) : 0.0;
        v = lo + hi;
    }
    if (fixed[t]) v = 0;
    pen[t] = v;
    pen32[t] = (float)v;
}

// dJ/drho = 1/2 alpha'(rho) sum over the 4 faces of (-u lambda + 1/2 u^2)
// (fluid_topo/FluidTopoOpt.cpp:166-190)
__global__ void k2_sensitivity(G2d g, const double* __restrict__ rho, stg_alpha L, const double* __restrict__ u,
                               const double* __restrict__ lam, double* __restrict__ grad) {
    int t = blockIdx.x * TPB + threadIdx.x;
    const int n = g.n;
    if (t >= n * n) return;
    int x = t / n, y = t % n;
    const int fi[4] = {g.face(x, y, 0), g.face(x + 1, y, 0), g.face(x, y, 1), g.face(x, y + 1, 1)};
    double s = 0;
    for (int q = 0; q < 4; q++) s += -(u[fi[q]] * lam[fi[q]]) + (0.5 * u[fi[q]]) * u[fi[q]];
    grad[t] = s * (0.5 * dalpha_of(rho[t], L));
}

// calcA (stoke/StokeFlowDirectSolve.cpp:6-133) as a function of the entry (row i, col j),
// written into row i of the row-major augmented matrix [A | I] (ld = 2 nd)
__global__ void k2_calcA(G2d g, const double* __restrict__ vol, const double* __restrict__ pen,
                         const uint8_t* __restrict__ fixed, double lap, int closed, double* __restrict__ aug) {
    const int nd = g.size();
    long long e = (long long)blockIdx.x * TPB + threadIdx.x;
    if (e >= (long long)nd * nd) return;
    int i = (int)(e / nd), j = (int)(e % nd);
    double a = 0;
    if (fixed[i] || fixed[j]) {
        a = i == j ? 1.0 : 0.0;
    } else {
        int ki, xi, yi, kj, xj, yj;
        g.decode(i, ki, xi, yi);
        g.decode(j, kj, xj, yj);
        if (ki < 0 && kj < 0) {
            a = closed ? 1.0 : 0.0;
        } else if (ki < 0 || kj < 0) {
            // cell-face coupling: -vol (left / bottom face), +vol (right / top face)
            int cx = ki < 0 ? xi : xj, cy = ki < 0 ? yi : yj;
            int fk = ki < 0 ? kj : ki, fxx = ki < 0 ? xj : xi, fyy = ki < 0 ? yj : yi;
            int fidx = ki < 0 ? j : i;
            if (g.face_ok(fxx, fyy, fk)) {
                if (fk == 0 && fyy == cy && fxx == cx) a = -vol[fidx];
                if (fk == 0 && fyy == cy && fxx == cx + 1) a = vol[fidx];
                if (fk == 1 && fxx == cx && fyy == cy) a = -vol[fidx];
                if (fk == 1 && fxx == cx && fyy == cy + 1) a = vol[fidx];
            }
        } else if (ki == kj && g.face_ok(xi, yi, ki) && g.face_ok(xj, yj, kj)) {
            int dx = xj - xi, dy = yj - yi;
            const int d = ki;
            if (dx == 0 && dy == 0) {
                a = 4.0 * lap;
            } else if (abs(dx) + abs(dy) == 1) {
                // the column face's neighbour list (its x / y range limits) decides the entry
                bool ok;
                if (d == 0)
                    ok = (dx == 1 && xj != 0) || (dx == -1 && xj != g.n) || (dy == 1 && yj != 0) || (dy == -1 && yj != g.n - 1);
                else
                    ok = (dy == 1 && yj != 0) || (dy == -1 && yj != g.n) || (dx == 1 && xj != 0) || (dx == -1 && xj != g.n - 1);
                if (ok) a = -lap;
            }
        }
        if (i == j) a += pen[i];
    }
    aug[(long long)i * 2 * nd + j] = a;
    aug[(long long)i * 2 * nd + nd + j] = i == j ? 1.0 : 0.0;
}

// x = Ainv r (warp per row), FP32 in/out
__global__ void k2_gemv(int nd, const double* __restrict__ inv, int ld, const float* __restrict__ r, float* __restrict__ x) {
    int row = (blockIdx.x * TPB + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= nd) return;
    double s = 0;
    for (int c = lane; c < nd; c += 32) s += inv[(long long)row * ld + c] * (double)r[c];
    s = warp_sum(s);
    if (lane == 0) x[row] = (float)s;
}
__global__ void k2_gemv64(int nd, const double* __restrict__ inv, int ld, const double* __restrict__ r, double* __restrict__ x) {
    int row = (blockIdx.x * TPB + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= nd) return;
    double s = 0;
    for (int c = lane; c < nd; c += 32) s += inv[(long long)row * ld + c] * r[c];
    s = warp_sum(s);
    if (lane == 0) x[row] = s;
}

// x += p; r -= Ap
__global__ void k2_update(int n, const float* __restrict__ p, const float* __restrict__ Ap, float* __restrict__ x,
                          float* __restrict__ r) {
    int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= n) return;
    x[t] += p[t];
    r[t] -= Ap[t];
}

unsigned g1(long long n) { return (unsigned)((n + TPB - 1) / TPB); }

}  // namespace

// ====================================================================== 2D handle state
struct Level2 {
    G2d g;
    double lap = 1.0;
    uint8_t* fixed = nullptr;
    double *vol = nullptr, *pen = nullptr;
    float *vol32 = nullptr, *pen32 = nullptr;
    float *r = nullptr, *x = nullptr, *p = nullptr, *Ap = nullptr, *rs = nullptr, *d = nullptr, *Ad = nullptr;
    double *t0 = nullptr, *t1 = nullptr;
};

}  // namespace stg

struct Ctx2 {
    std::vector<stg::Level2> lv;
    double *aug0 = nullptr, *aug1 = nullptr;
    const double* inv = nullptr;
    int* info = nullptr;
};

namespace stg {

namespace {

Level2& fine2(stg_t* h) { return h->c2->lv.back(); }

Coef2<double> coef64(const Level2& L) { return Coef2<double>{L.vol, L.pen, L.fixed}; }
Coef2<float> coef32(const Level2& L) { return Coef2<float>{L.vol32, L.pen32, L.fixed}; }

int apply2_32(stg_t* h, Level2& L, const float* x, float* y) {
    k2_apply<float, 0><<<g1(L.g.size()), TPB, 0, h->st>>>(L.g, coef32(L), (float)L.lap, x, nullptr, y, nullptr);
    STG_LAUNCH_CK();
    return STG_OK;
}

// StokeFlowSmoothing::applyMapping, iter_num 1, alpha 1: out = sum of the two colour
// corrections, each followed by r -= A d
int smoother2(stg_t* h, Level2& L, int order, const float* r, float* out) {
    const int n = L.g.size();
    STG_CK(cudaMemcpyAsync(L.rs, r, sizeof(float) * n, cudaMemcpyDeviceToDevice, h->st));
    STG_CK(cudaMemsetAsync(out, 0, sizeof(float) * n, h->st));
    for (int i = 0; i < 2; i++) {
        int flag = order ? 1 - i : i;
        STG_CK(cudaMemsetAsync(L.d, 0, sizeof(float) * n, h->st));
        PROF(h, 1, 0.0, ([&] {
                 k2_smooth<<<g1(L.g.nc()), TPB, 0, h->st>>>(L.g, coef32(L), (float)L.lap, flag, L.rs, L.d);
                 STG_LAUNCH_CK();
                 return STG_OK;
             })());
        STG_TRY(apply2_32(h, L, L.d, L.Ad));
        k2_update<<<g1(n), TPB, 0, h->st>>>(n, L.d, L.Ad, out, L.rs);
        STG_LAUNCH_CK();
    }
    return STG_OK;
}

int coarse2(stg_t* h, const float* r, float* x) {
    Level2& C = h->c2->lv[0];
    const int nd = C.g.size();
    k2_gemv<<<g1(32ll * nd), TPB, 0, h->st>>>(nd, h->c2->inv, 2 * nd, r, x);
    STG_LAUNCH_CK();
    return STG_OK;
}

// MultigridSolve::Vcycle (common_cpx/MultigridSolve.cpp:73-106) in FP32
int vcycle2(stg_t* h) {
    auto& lv = h->c2->lv;
    const int L = (int)lv.size();
    for (int i = L - 1; i >= 0; i--) {
        Level2& F = lv[i];
        const int n = F.g.size();
        if (i > 0)
            STG_TRY(smoother2(h, F, 0, F.r, F.p));
        else
            STG_TRY(coarse2(h, F.r, F.p));
        STG_TRY(apply2_32(h, F, F.p, F.Ap));
        k2_update<<<g1(n), TPB, 0, h->st>>>(n, F.p, F.Ap, F.x, F.r);
        STG_LAUNCH_CK();
        if (i != 0) {
            Level2& C = lv[i - 1];
            k2_restrict<float><<<g1(C.g.size()), TPB, 0, h->st>>>(C.g, F.g, F.r, C.fixed, C.r);
            STG_LAUNCH_CK();
            STG_CK(cudaMemsetAsync(C.x, 0, sizeof(float) * C.g.size(), h->st));
        }
    }
    for (int i = 0; i < L; i++) {
        Level2& F = lv[i];
        const int n = F.g.size();
        if (i != 0) {
            Level2& C = lv[i - 1];
            k2_prolong<float><<<g1(n), TPB, 0, h->st>>>(F.g, C.g, C.x, F.fixed, F.p);
            STG_LAUNCH_CK();
            STG_TRY(apply2_32(h, F, F.p, F.Ap));
            k2_update<<<g1(n), TPB, 0, h->st>>>(n, F.p, F.Ap, F.x, F.r);
            STG_LAUNCH_CK();
        }
        if (i > 0) {
            STG_TRY(smoother2(h, F, 1, F.r, F.p));
            STG_TRY(apply2_32(h, F, F.p, F.Ap));
            k2_update<<<g1(n), TPB, 0, h->st>>>(n, F.p, F.Ap, F.x, F.r);
            STG_LAUNCH_CK();
        }
    }
    return STG_OK;
}

// ---------------------------------------------------------------- solve_core hooks
// FluidSteadyState::update_penalty set-up half (stoke/FluidSteadyState.cpp:122-140)
int setup2(stg_t* h) {
    if (!h->have_boundary || !h->have_penalty) {
        set_error("boundary and penalty must be set before the solver set-up");
        return STG_E_INVALID;
    }
    auto& lv = h->c2->lv;
    // coarsening and the analytic coarsest matrix touch fixed buffers only: replayed as a
    // CUDA graph; the Gauss-Jordan inverse follows as one cooperative launch
    auto body = [&]() -> int {
        for (int i = (int)lv.size() - 2; i >= 0; i--) {
            Level2 &c = lv[i], &f = lv[i + 1];
            if (h->hier_flow)
                k2_coarsen<true><<<g1(c.g.size()), TPB, 0, h->st>>>(c.g, f.g, f.fixed, f.vol, f.pen, c.fixed, c.vol, c.pen, c.vol32,
                                                                      c.pen32);
            else
                k2_coarsen<false><<<g1(c.g.size()), TPB, 0, h->st>>>(c.g, f.g, f.fixed, f.vol, f.pen, c.fixed, c.vol, c.pen, c.vol32,
                                                                       c.pen32);
            STG_LAUNCH_CK();
        }
        Level2& C = lv[0];
        const int nd = C.g.size();
        k2_calcA<<<g1((long long)nd * nd), TPB, 0, h->st>>>(C.g, C.vol, C.pen, C.fixed, C.lap, h->closed ? 1 : 0, h->c2->aug0);
        STG_LAUNCH_CK();
        return STG_OK;
    };
    GraphCache& G = h->sgraph;
    STG_TRY(graphed(h, G, (h->closed ? 2 : 1) | (h->hier_flow ? 4 : 0), body, [](bool) {}));
    // the inversion: one cooperative launch, outside the graph
    STG_TRY(gj_invert(h->st, lv[0].g.size(), h->c2->aug0, h->c2->aug1, h->c2->info, &h->c2->inv, true));
    h->updated = true;
    return STG_OK;
}

int resid2(stg_t* h, const d4* b, const d4* x, d4* r, double* nrm2_host) {
    Level2& F = fine2(h);
    unsigned nb = g1(F.g.size());
    k2_apply<double, 1><<<nb, TPB, 0, h->st>>>(F.g, coef64(F), F.lap, reinterpret_cast<const double*>(x),
                                               reinterpret_cast<const double*>(b), reinterpret_cast<double*>(r), h->d_parts);
    STG_LAUNCH_CK();
    STG_TRY(reduce_parts(h->st, h->d_parts, (int)nb, h->dnrm));
    STG_CK(cudaMemcpyAsync(nrm2_host, h->dnrm, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int precond2(stg_t* h, const float4* rhs, float4* out) {
    Level2& F = fine2(h);
    const int n = F.g.size();
    STG_CK(cudaMemcpyAsync(F.r, rhs, sizeof(float) * n, cudaMemcpyDeviceToDevice, h->st));
    STG_CK(cudaMemsetAsync(F.x, 0, sizeof(float) * n, h->st));
    // the V-cycle works on the level buffers only: replayed as a CUDA graph
    STG_TRY(graphed(h, h->vgraph, 1, [&] { return vcycle2(h); }, [](bool) {}));
    STG_CK(cudaMemcpyAsync(out, F.x, sizeof(float) * n, cudaMemcpyDeviceToDevice, h->st));
    return STG_OK;
}

int shift2(stg_t* h, const float4* v, const float4* z, float4* out) {
    Level2& L = fine2(h);
    k2_apply<float, 1><<<g1(L.g.size()), TPB, 0, h->st>>>(L.g, coef32(L), (float)L.lap, reinterpret_cast<const float*>(z),
                                                           reinterpret_cast<const float*>(v), reinterpret_cast<float*>(out), nullptr);
    STG_LAUNCH_CK();
    return STG_OK;
}

int apply2(stg_t* h, const float4* x, float4* y) {
    return apply2_32(h, fine2(h), reinterpret_cast<const float*>(x), reinterpret_cast<float*>(y));
}

}  // namespace

// ====================================================================== 2D entry points
// (called by the C ABI in solver.cu when the handle has dim == 2)
int create2d(stg_t* h) {
    const int n = h->n;
    h->c2 = new Ctx2();
    auto& lv = h->c2->lv;
    int low = n & -n;
    int L = (int)std::lround(std::log2((double)low)) - 2;  // FluidSteadyState::init (:12)
    if (L < 1) L = 1;
    lv.resize(L);
    for (int i = L - 1, m = n; i >= 0; i--, m /= 2) lv[i].g.n = m;
    lv[L - 1].lap = 1.0;
    for (int i = L - 2; i >= 0; i--) lv[i].lap = 2.0 * lv[i + 1].lap;  // createSubSystem (StokeFlowSubSystem.cu:155)
    for (auto& V : lv) {
        size_t s = V.g.size();
        STG_TRY(dalloc(&V.fixed, s));
        STG_TRY(dalloc(&V.vol, s));
        STG_TRY(dalloc(&V.pen, s));
        STG_TRY(dalloc(&V.vol32, s));
        STG_TRY(dalloc(&V.pen32, s));
        for (float** q : {&V.r, &V.x, &V.p, &V.Ap, &V.rs, &V.d, &V.Ad}) STG_TRY(dalloc(q, s));
    }
    const int nd = lv[0].g.size();
    if (nd > 8192) {
        set_error("N = %d leaves a %d-unknown coarsest level (N / 8 must have a larger power-of-two factor)", n, nd);
        return STG_E_UNSUPPORTED;
    }
    STG_TRY(dalloc(&h->c2->aug0, 2ull * nd * nd));
    STG_TRY(dalloc(&h->c2->aug1, 2ull * nd * nd));
    STG_TRY(dalloc(&h->c2->info, 1));
    Level2& F = lv.back();
    h->L = L;
    h->n4 = F.g.size() / 4;
    h->ncell = (size_t)n * n;
    h->nface = (size_t)n * (n + 1);
    h->setup = setup2;
    h->resid64 = resid2;
    h->precond = precond2;
    h->apply32 = apply2;
    h->shift32 = shift2;
    return STG_OK;
}

void destroy2d(stg_t* h) {
    if (!h->c2) return;
    for (auto& V : h->c2->lv) {
        cudaFree(V.fixed);
        cudaFree(V.vol);
        cudaFree(V.pen);
        cudaFree(V.vol32);
        cudaFree(V.pen32);
        for (float* q : {V.r, V.x, V.p, V.Ap, V.rs, V.d, V.Ad}) cudaFree(q);
        cudaFree(V.t0);
        cudaFree(V.t1);
    }
    cudaFree(h->c2->aug0);
    cudaFree(h->c2->aug1);
    cudaFree(h->c2->info);
    delete h->c2;
    h->c2 = nullptr;
}

long long dof2d(const stg_t* h, int level) { return h->c2->lv[level].g.size(); }
int level_n2d(const stg_t* h, int level) { return h->c2->lv[level].g.n; }

// inputs are device staging copies of the Field-order host arrays
int set_boundary2d(stg_t* h, const double* cvol, const int* cfix, const double* fv0, const double* fv1, const int* ff0,
                   const int* ff1) {
    Level2& F = fine2(h);
    k2_fine_descr<<<g1(F.g.size()), TPB, 0, h->st>>>(F.g, cvol, cfix, fv0, fv1, ff0, ff1, F.fixed, F.vol);
    STG_LAUNCH_CK();
    STG_TRY(f64_to_f32(h->st, F.g.size() / 4, reinterpret_cast<const d4*>(F.vol), 1.0, reinterpret_cast<float4*>(F.vol32)));
    return STG_OK;
}

int set_penalty2d(stg_t* h, const double* cp, const double* f0, const double* f1) {
    Level2& F = fine2(h);
    k2_penalty_from_field<<<g1(F.g.size()), TPB, 0, h->st>>>(F.g, cp, f0, f1, F.fixed, F.pen, F.pen32);
    STG_LAUNCH_CK();
    return STG_OK;
}

int set_density2d(stg_t* h, const double* rho, const stg_alpha& law) {
    Level2& F = fine2(h);
    k2_face_penalty<<<g1(F.g.size()), TPB, 0, h->st>>>(F.g, rho, law, F.fixed, F.pen, F.pen32);
    STG_LAUNCH_CK();
    return STG_OK;
}

int field_to_vec2d(stg_t* h, const double* cell, const double* f0, const double* f1, d4* out) {
    Level2& F = fine2(h);
    k2_field_to_blocked<<<g1(F.g.size()), TPB, 0, h->st>>>(F.g, cell, f0, f1, reinterpret_cast<double*>(out));
    STG_LAUNCH_CK();
    return STG_OK;
}

int vec_to_field2d(stg_t* h, const d4* in, double* cell, double* f0, double* f1) {
    Level2& F = fine2(h);
    k2_blocked_to_field<<<g1(F.g.size()), TPB, 0, h->st>>>(F.g, reinterpret_cast<const double*>(in), cell, f0, f1);
    STG_LAUNCH_CK();
    return STG_OK;
}

// E x (FluidEnergyGrad, lap_coeff 1 on the energy descriptor = fine coefficients)
int energy2d(stg_t* h, const d4* x, d4* out, double* part, int* nb) {
    Level2& F = fine2(h);
    *nb = (int)g1(F.g.size());
    k2_apply<double, 2><<<*nb, TPB, 0, h->st>>>(F.g, coef64(F), 1.0, reinterpret_cast<const double*>(x), nullptr,
                                                reinterpret_cast<double*>(out), part);
    STG_LAUNCH_CK();
    return STG_OK;
}

int sensitivity2d(stg_t* h, const double* rho, const stg_alpha& law, const d4* x, const d4* lam, double* grad) {
    Level2& F = fine2(h);
    k2_sensitivity<<<g1((long long)F.g.n * F.g.n), TPB, 0, h->st>>>(F.g, rho, law, reinterpret_cast<const double*>(x),
                                                                     reinterpret_cast<const double*>(lam), grad);
    STG_LAUNCH_CK();
    return STG_OK;
}

// ---------------------------------------------------------------- LinearMapping adapters (blocked layout = native)
int apply_A2d(stg_t* h, int level, double* out, const double* in) {
    Level2& L = h->c2->lv[level];
    k2_apply<double, 0><<<g1(L.g.size()), TPB, 0, h->st>>>(L.g, coef64(L), L.lap, in, nullptr, out, nullptr);
    STG_LAUNCH_CK();
    return STG_OK;
}

int apply_E2d(stg_t* h, double* out, const double* in) {
    int nb;
    return energy2d(h, reinterpret_cast<const d4*>(in), reinterpret_cast<d4*>(out), nullptr, &nb);
}

int vcycle2d(stg_t* h, double* out, const double* in) {
    Level2& F = fine2(h);
    const long long n4 = F.g.size() / 4;
    STG_TRY(f64_to_f32(h->st, n4, reinterpret_cast<const d4*>(in), 1.0, reinterpret_cast<float4*>(F.r)));
    STG_CK(cudaMemsetAsync(F.x, 0, sizeof(float) * F.g.size(), h->st));
    STG_TRY(vcycle2(h));
    STG_TRY(f32_to_f64(h->st, n4, reinterpret_cast<const float4*>(F.x), reinterpret_cast<d4*>(out)));
    return STG_OK;
}

int apply_op2d(stg_t* h, int op, int level, double* out, const double* in) {
    auto& lv = h->c2->lv;
    Level2& L = lv[level];
    switch (op) {
        case STG_OP_RESTRICT:
            if (level >= (int)lv.size() - 1) break;
            k2_restrict<double><<<g1(L.g.size()), TPB, 0, h->st>>>(L.g, lv[level + 1].g, in, L.fixed, out);
            STG_LAUNCH_CK();
            return STG_OK;
        case STG_OP_PROLONG: {
            if (level >= (int)lv.size() - 1) break;
            Level2& F = lv[level + 1];
            k2_prolong<double><<<g1(F.g.size()), TPB, 0, h->st>>>(F.g, L.g, in, F.fixed, out);
            STG_LAUNCH_CK();
            return STG_OK;
        }
        case STG_OP_SMOOTH_PRE:
        case STG_OP_SMOOTH_POST:
        case STG_OP_VANKA_RED:
        case STG_OP_VANKA_BLACK: {
            if (level == 0) break;
            const long long n4 = L.g.size() / 4;
            STG_TRY(f64_to_f32(h->st, n4, reinterpret_cast<const d4*>(in), 1.0, reinterpret_cast<float4*>(L.r)));
            if (op == STG_OP_SMOOTH_PRE || op == STG_OP_SMOOTH_POST) {
                STG_TRY(smoother2(h, L, op == STG_OP_SMOOTH_POST ? 1 : 0, L.r, L.x));
            } else {
                STG_CK(cudaMemsetAsync(L.x, 0, sizeof(float) * L.g.size(), h->st));
                k2_smooth<<<g1(L.g.nc()), TPB, 0, h->st>>>(L.g, coef32(L), (float)L.lap, op == STG_OP_VANKA_BLACK ? 1 : 0,
                                                             L.r, L.x);
                STG_LAUNCH_CK();
            }
            STG_TRY(f32_to_f64(h->st, n4, reinterpret_cast<const float4*>(L.x), reinterpret_cast<d4*>(out)));
            return STG_OK;
        }
        case STG_OP_COARSE: {
            if (level != 0) break;
            const int nd = L.g.size();
            k2_gemv64<<<g1(32ll * nd), TPB, 0, h->st>>>(nd, h->c2->inv, 2 * nd, in, out);
            STG_LAUNCH_CK();
            return STG_OK;
        }
        default: break;
    }
    set_error("operator %d not defined at level %d", op, level);
    return STG_E_INVALID;
}

int level_descr2d(stg_t* h, int level, double* vol, double* pen, uint8_t* fixed) {
    Level2& L = h->c2->lv[level];
    const size_t s = L.g.size();
    if (vol) STG_CK(cudaMemcpyAsync(vol, L.vol, sizeof(double) * s, cudaMemcpyDeviceToDevice, h->st));
    if (pen) STG_CK(cudaMemcpyAsync(pen, L.pen, sizeof(double) * s, cudaMemcpyDeviceToDevice, h->st));
    if (fixed) STG_CK(cudaMemcpyAsync(fixed, L.fixed, s, cudaMemcpyDeviceToDevice, h->st));
    return STG_OK;
}

}  // namespace stg
