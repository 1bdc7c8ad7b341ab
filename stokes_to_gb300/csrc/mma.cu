// Method of Moving Asymptotes design update on the GPU: the reference optimizer
// (OptimizerMMA::Optimize_MMA, simplex/src/optimization/OptimizerMma.h:96-128, around the
// vendored simplex/ext/mma/MMASolver.cpp:70-442) for the one volume constraint of
// FluidTopoOpt3D (FT/FluidTopoOpt3D.cpp:19-39, 74-83).
//
// Per update: one fused pass over the cells builds the convex subproblem (moving
// asymptotes, move bounds, the p/q coefficients of objective and constraint, the
// constraint constant b and the volume); the dual in the single multiplier lambda is
// then solved by the reference's primal-dual interior-point Newton iteration on the host
// (scalars only), every Newton step costing one FP64 reduction pass that evaluates
// x(lambda) per cell and returns the constraint sum and the dual Hessian; a last pass
// writes x(lambda) and the largest change. All cell arrays stay in HBM.
#include <cmath>
#include <vector>

#include "ctx.h"

namespace stg {

struct MmaArrays {
    double *low, *upp, *xold1, *xold2, *alpha, *beta, *p0, *q0, *p1, *q1;
};

namespace {

constexpr int TPB = 256;
constexpr int MGRID = 1216;  // 8 x 152 SMs

// constants of MMASolver (simplex/ext/mma/MMASolver.cpp:34-48) and OptimizerMMA
constexpr double XMAMIEPS = 1e-5, RAA0 = 1e-5, MMA_MOVE = 0.5, ALBEFA = 0.1;
constexpr double ASYMINIT = 0.5, ASYMDEC = 0.7, ASYMINC = 1.2, C_DUAL = 1000.0;

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// block sums of two values into part[block * 2 + {0,1}]
__device__ __forceinline__ void block_sum2(double a, double b, double* part) {
    __shared__ double sa[TPB / 32], sb[TPB / 32];
    a = warp_sum(a);
    b = warp_sum(b);
    if ((threadIdx.x & 31) == 0) {
        sa[threadIdx.x >> 5] = a;
        sb[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0, y = 0;
        for (int w = 0; w < TPB / 32; w++) {
            x += sa[w];
            y += sb[w];
        }
        part[2 * blockIdx.x] = x;
        part[2 * blockIdx.x + 1] = y;
    }
}


// GenSub (MMASolver.cpp:358-442) with the per-cell move bounds of Optimize_MMA
// [max(lo, x - movlim), min(hi, x + movlim)], then xold2 <- xold1 <- x. Partials: the
// constraint constant sum p1/(U-x) + q1/(x-L) and the volume sum x.
__global__ void k_mma_gensub(long long n, int iter, const double* __restrict__ x, const double* __restrict__ df, double dg,
                             double lo, double hi, double movlim, MmaArrays A, double* __restrict__ part) {
    double bs = 0, vs = 0;
    for (long long i = (long long)blockIdx.x * TPB + threadIdx.x; i < n; i += (long long)gridDim.x * TPB) {
        const double xv = x[i];
        const double xmin = fmax(lo, xv - movlim), xmax = fmin(hi, xv + movlim);
        double L, U;
        if (iter < 3) {
            L = xv - ASYMINIT * (xmax - xmin);
            U = xv + ASYMINIT * (xmax - xmin);
        } else {
            const double x1 = A.xold1[i], x2 = A.xold2[i];
            const double sgn = (xv - x1) * (x1 - x2);
            const double gam = sgn < 0 ? ASYMDEC : (sgn > 0 ? ASYMINC : 1.0);
            L = xv - gam * (x1 - A.low[i]);
            U = xv + gam * (A.upp[i] - x1);
            const double w = fmax(XMAMIEPS, xmax - xmin);
            L = fmin(fmax(L, xv - 100.0 * w), xv - 1e-5 * w);
            U = fmin(fmax(U, xv + 1e-5 * w), xv + 100.0 * w);
            const double xlo = xmin - 1e-6, xhi = xmax + 1e-6;
            if (xv < xlo) {
                L = xv - (xhi - xv) / 0.9;
                U = xv + (xhi - xv) / 0.9;
            }
            if (xv > xhi) {
                L = xv - (xv - xlo) / 0.9;
                U = xv + (xv - xlo) / 0.9;
            }
        }
        A.low[i] = L;
        A.upp[i] = U;
        A.alpha[i] = fmin(fmax(fmax(xmin, L + ALBEFA * (xv - L)), xv - MMA_MOVE * (xmax - xmin)), xmax);
        A.beta[i] = fmax(fmin(fmin(xmax, U - ALBEFA * (U - xv)), xv + MMA_MOVE * (xmax - xmin)), xmin);
        const double winv = 1.0 / fmax(XMAMIEPS, xmax - xmin);
        const double du = U - xv, dl = xv - L;
        const double d0 = df[i];
        const double pq0 = 0.001 * fabs(d0) + RAA0 * winv;
        A.p0[i] = du * du * (fmax(0.0, d0) + pq0);
        A.q0[i] = dl * dl * (fmax(0.0, -d0) + pq0);
        const double pq1 = 0.001 * fabs(dg) + RAA0 * winv;
        const double p1 = du * du * (fmax(0.0, dg) + pq1), q1 = dl * dl * (fmax(0.0, -dg) + pq1);
        A.p1[i] = p1;
        A.q1[i] = q1;
        bs += p1 / du + q1 / dl;
        vs += xv;
        A.xold2[i] = A.xold1[i];
        A.xold1[i] = xv;
    }
    block_sum2(bs, vs, part);
}

// x(lambda) of one cell (XYZofLAMBDA, MMASolver.cpp:328-355); xp is the unclamped minimiser
__device__ __forceinline__ double x_of(const MmaArrays& A, long long i, double lam, double& xp, double& pl, double& ql) {
    pl = A.p0[i] + A.p1[i] * lam;
    ql = A.q0[i] + A.q1[i] * lam;
    const double sp = sqrt(pl), sq = sqrt(ql);
    xp = (sp * A.low[i] + sq * A.upp[i]) / (sp + sq);
    return fmin(fmax(xp, A.alpha[i]), A.beta[i]);
}

// Partials at lambda: the constraint sum p1/(U-x) + q1/(x-L) (DualGrad / DualResidual) and
// the Hessian sum PQ^2 df2 (DualHess, MMASolver.cpp:208-300) at x(lambda).
__global__ void k_mma_dual(long long n, double lam, MmaArrays A, double* __restrict__ part) {
    double cs = 0, hs = 0;
    for (long long i = (long long)blockIdx.x * TPB + threadIdx.x; i < n; i += (long long)gridDim.x * TPB) {
        double xp, pl, ql;
        const double xi = x_of(A, i, lam, xp, pl, ql);
        const double du = A.upp[i] - xi, dl = xi - A.low[i];
        const double p1 = A.p1[i], q1 = A.q1[i];
        cs += p1 / du + q1 / dl;
        const double pq = p1 / (du * du) - q1 / (dl * dl);
        double df2 = -1.0 / (2.0 * pl / (du * du * du) + 2.0 * ql / (dl * dl * dl));
        if (xp < A.alpha[i] || xp > A.beta[i]) df2 = 0.0;
        hs += pq * df2 * pq;
    }
    block_sum2(cs, hs, part);
}

// x_new = x(lambda) and the block maxima of |x_new - x_old|
__global__ void k_mma_final(long long n, double lam, MmaArrays A, double* __restrict__ xout, double* __restrict__ part) {
    __shared__ double sm[TPB / 32];
    double mx = 0;
    for (long long i = (long long)blockIdx.x * TPB + threadIdx.x; i < n; i += (long long)gridDim.x * TPB) {
        double xp, pl, ql;
        const double xi = x_of(A, i, lam, xp, pl, ql);
        mx = fmax(mx, fabs(xi - A.xold1[i]));
        xout[i] = xi;
    }
    mx = warp_max(mx);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0;
        for (int w = 0; w < TPB / 32; w++) m = fmax(m, sm[w]);
        part[blockIdx.x] = m;
    }
}

unsigned mgrid(long long n) {
    long long g = (n + TPB - 1) / TPB;
    return (unsigned)(g < 1 ? 1 : (g > MGRID ? MGRID : g));
}

// deterministic host-side sums of the block partials (fixed order)
void host_sum2(const std::vector<double>& p, int nb, double& a, double& b) {
    a = b = 0;
    for (int q = 0; q < nb; q++) {
        a += p[2 * q];
        b += p[2 * q + 1];
    }
}

}  // namespace

}  // namespace stg

struct MmaState {
    int iter = 0;
    stg::MmaArrays A{};
    double* part = nullptr;
    std::vector<double> hpart;
};

namespace stg {

void mma_free(stg_t* h) {
    if (!h->mma) return;
    MmaArrays& A = h->mma->A;
    for (double* p : {A.low, A.upp, A.xold1, A.xold2, A.alpha, A.beta, A.p0, A.q0, A.p1, A.q1, h->mma->part}) cudaFree(p);
    delete h->mma;
    h->mma = nullptr;
}

int mma_reset(stg_t* h) {
    if (h->mma) h->mma->iter = 0;
    return STG_OK;
}

int mma_update(stg_t* h, const double* d_x, const double* d_df, double frac, double coef, double lo, double hi, double movlim,
               double* d_xout, double* change) {
    const long long n = (long long)h->ncell;
    if (!h->mma) {
        h->mma = new MmaState();
        MmaArrays& A = h->mma->A;
        for (double** p : {&A.low, &A.upp, &A.xold1, &A.xold2, &A.alpha, &A.beta, &A.p0, &A.q0, &A.p1, &A.q1})
            STG_TRY(dalloc(p, (size_t)n));
        STG_TRY(dalloc(&h->mma->part, 2 * MGRID));
        h->mma->hpart.resize(2 * MGRID);
    }
    MmaState& M = *h->mma;
    M.iter++;
    const unsigned g = mgrid(n);
    const double dg = coef / (double)n;  // FluidTopoOpt3D::Compute_Constraint_Grad
    k_mma_gensub<<<g, TPB, 0, h->st>>>(n, M.iter, d_x, d_df, dg, lo, hi, movlim, M.A, M.part);
    STG_LAUNCH_CK();
    auto fetch2 = [&](double& a, double& b) -> int {
        STG_CK(cudaMemcpyAsync(M.hpart.data(), M.part, sizeof(double) * 2 * g, cudaMemcpyDeviceToHost, h->st));
        STG_CK(cudaStreamSynchronize(h->st));
        host_sum2(M.hpart, (int)g, a, b);
        return STG_OK;
    };
    double bsum = 0, vsum = 0;
    STG_TRY(fetch2(bsum, vsum));
    const double gval = coef * (vsum / (double)n - frac);  // Compute_Constraint
    const double b = -gval + bsum;

    // SolveDIP (MMASolver.cpp:100-146), m = 1, a = 0, c = 1000
    double lam = C_DUAL / 2.0, mu = 1.0, epsi = 1.0, err = 1.0;
    const double tol = std::sqrt((double)n + 1.0) * 1e-9;
    double csum = 0, hsum = 0;
    k_mma_dual<<<g, TPB, 0, h->st>>>(n, lam, M.A, M.part);
    STG_LAUNCH_CK();
    STG_TRY(fetch2(csum, hsum));
    int steps = 0;
    while (epsi > tol) {
        int loop = 0;
        while (err > 0.9 * epsi && loop < 100) {
            loop++;
            steps++;
            const double y = std::max(0.0, lam - C_DUAL);
            const double grad = -(-b - y + csum) - epsi / lam;
            double hess = hsum;
            if (lam > C_DUAL) hess += -1.0;
            hess += -mu / lam;
            double corr = 1e-4 * hess;
            if (-corr < 1e-7) corr = -1e-7;
            hess += corr;
            const double s0 = grad / hess;
            const double s1 = -mu + epsi / lam - s0 * mu / lam;
            double theta = 1.005;
            theta = std::max(theta, -1.01 * s0 / lam);
            theta = std::max(theta, -1.01 * s1 / mu);
            theta = 1.0 / theta;
            lam += theta * s0;
            mu += theta * s1;
            if (lam < 0) lam = 0;
            k_mma_dual<<<g, TPB, 0, h->st>>>(n, lam, M.A, M.part);
            STG_LAUNCH_CK();
            STG_TRY(fetch2(csum, hsum));
            const double y2 = std::max(0.0, lam - C_DUAL);
            err = std::max(std::fabs(-b - y2 + mu + csum), std::fabs(mu * lam - epsi));
            if (!std::isfinite(err)) {
                set_error("MMA dual iteration produced a non-finite residual");
                return STG_E_NONFINITE;
            }
        }
        epsi *= 0.1;
    }
    k_mma_final<<<g, TPB, 0, h->st>>>(n, lam, M.A, d_xout, M.part);
    STG_LAUNCH_CK();
    STG_CK(cudaMemcpyAsync(M.hpart.data(), M.part, sizeof(double) * g, cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    double mx = 0;
    for (unsigned q = 0; q < g; q++) mx = std::max(mx, M.hpart[q]);
    if (change) *change = mx;
    (void)steps;
    return STG_OK;
}

}  // namespace stg
