// Design-loop kernels: Brinkman penalty from the density (FluidTopoOpt3D::Update_Fluid),
// the adjoint chain rule (FluidTopoOpt3D::Update_Grad), the density filter, the
// optimality-criteria volume pass and the seeded density generator.
//
// Cell arrays are in the simplex Field order: (i*N + j)*N + k in 3D, i*N + j in 2D.
#include <cooperative_groups.h>
#include <math.h>

#include "alpha.cuh"
#include "kernels.h"
#include "stencil.cuh"

namespace stg {

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ long long cidx(int n, int i, int j, int k) { return ((long long)i * n + j) * n + k; }

// face penalty = 1/2 alpha(left cell) + 1/2 alpha(right cell), zero on fixed / absent faces
__global__ void k_face_penalty(Geom g, const double* __restrict__ rho, stg_alpha L, const uint8_t* __restrict__ m,
                               d4* __restrict__ P64, float4* __restrict__ P32) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    const int n = g.n;
    int s = g.slot(i, j, k);
    uint8_t mm = m[s];
    double own = cell_ok(n, i, j, k) ? 0.5 * alpha_of(rho[cidx(n, i, j, k)], L) : 0.0;
    double f[3];
    for (int d = 0; d < 3; d++) {
        int li = i - (d == 0), lj = j - (d == 1), lk = k - (d == 2);
        double lo = (li >= 0 && lj >= 0 && lk >= 0 && cell_ok(n, li, lj, lk)) ? 0.5 * alpha_of(rho[cidx(n, li, lj, lk)], L) : 0.0;
        f[d] = lo + own;
    }
    double u = (mm & MU) ? 0.0 : f[0], v = (mm & MV) ? 0.0 : f[1], w = (mm & MW) ? 0.0 : f[2];
    store4(P64, s, 0.0, u, v, w);
    P32[s] = make_float4(0.f, (float)u, (float)v, (float)w);
}

// dJ/drho_c = 1/2 alpha'(rho_c) sum_{6 faces} (-u lambda + 1/2 u^2)   (FluidTopoOpt3D.cpp:264-281)
__global__ void k_sensitivity(Geom g, const double* __restrict__ rho, stg_alpha L, const d4* __restrict__ x,
                              const d4* __restrict__ lam, double* __restrict__ grad) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    const int n = g.n;
    if (t >= (long long)n * n * n) return;
    int k = (int)(t % n), j = (int)((t / n) % n), i = (int)(t / ((long long)n * n));
    const double* xs = reinterpret_cast<const double*>(x);
    const double* ls = reinterpret_cast<const double*>(lam);
    double sum = 0.0;
    for (int d = 0; d < 3; d++) {
        int s0 = g.slot(i, j, k), s1 = g.slot(i + (d == 0), j + (d == 1), k + (d == 2));
        double u0 = xs[4ll * s0 + 1 + d], l0 = ls[4ll * s0 + 1 + d];
        double u1 = xs[4ll * s1 + 1 + d], l1 = ls[4ll * s1 + 1 + d];
        sum += -(u0 * l0) + (0.5 * u0) * u0;
        sum += -(u1 * l1) + (0.5 * u1) * u1;
    }
    double r = rho[t];
    grad[t] = sum * (0.5 * dalpha_of(r, L));
}

// Linear hat filter: out_i = sum_j w_ij in_j / W_i (forward) or sum_j w_ji in_j / W_j
// (transpose), w_ij = max(0, rmin - |c_i - c_j|) over cells inside the domain, W_i =
// sum_j w_ij. W is computed once per call by k_filter_wsum, so the transpose reads it
// instead of re-summing every neighbour's weights. dim 2 runs the same loops with a
// single k plane (nz = 1, no k offsets). Loop order and arithmetic are the same in both
// kernels, so W_i and the sums are identical wherever they are formed.
__device__ __forceinline__ double hat_w(double rmin, int a, int b, int c) { return rmin - sqrt((double)(a * a + b * b + c * c)); }

// the weights rmin - |o| of every offset o, computed once on the host (IEEE sqrt, so the
// same values as hat_w); used when the stencil fits (radius R <= 3)
constexpr int WTAB_MAX = 343;
struct WTab {
    double w[WTAB_MAX];
};
template <bool TAB>
__device__ __forceinline__ double weight(const WTab& T, double rmin, int R, int Rz, int a, int b, int c) {
    if (TAB) return T.w[((a + R) * (2 * R + 1) + (b + R)) * (2 * Rz + 1) + (c + Rz)];
    return hat_w(rmin, a, b, c);
}

template <bool TAB>
__global__ void k_filter_wsum(int n, int nz, double rmin, int R, int Rz, WTab T, double* __restrict__ W) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= (long long)n * n * nz) return;
    int k = (int)(t % nz), j = (int)((t / nz) % n), i = (int)(t / ((long long)n * nz));
    double s = 0;
    for (int a = -R; a <= R; a++)
        for (int b = -R; b <= R; b++)
            for (int c = -Rz; c <= Rz; c++) {
                int ii = i + a, jj = j + b, kk = k + c;
                if (ii < 0 || jj < 0 || kk < 0 || ii >= n || jj >= n || kk >= nz) continue;
                double w = weight<TAB>(T, rmin, R, Rz, a, b, c);
                if (w > 0) s += w;
            }
    W[t] = s;
}

template <bool TAB>
__global__ void k_filter(int n, int nz, double rmin, int R, int Rz, WTab T, const double* __restrict__ in,
                         const double* __restrict__ W, double* __restrict__ out, int transpose) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= (long long)n * n * nz) return;
    int k = (int)(t % nz), j = (int)((t / nz) % n), i = (int)(t / ((long long)n * nz));
    double s = 0;
    for (int a = -R; a <= R; a++)
        for (int b = -R; b <= R; b++)
            for (int c = -Rz; c <= Rz; c++) {
                int ii = i + a, jj = j + b, kk = k + c;
                if (ii < 0 || jj < 0 || kk < 0 || ii >= n || jj >= n || kk >= nz) continue;
                double w = weight<TAB>(T, rmin, R, Rz, a, b, c);
                if (w <= 0) continue;
                const long long q = ((long long)ii * n + jj) * nz + kk;
                if (transpose)
                    s += w * in[q] / W[q];
                else
                    s += w * in[q];
            }
    out[t] = transpose ? s : s / W[t];
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One bisection probe of the OC update: x_new(lambda) and its filtered volume partials.
__global__ void k_oc(int ncell, const double* __restrict__ x, const double* __restrict__ dc, const double* __restrict__ vw,
                     double lam, double move, double lo, double hi, double* __restrict__ xnew, double* __restrict__ part) {
    __shared__ double sh[TPB / 32];
    double acc = 0;
    double inv_n = 1.0 / ncell;
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < ncell; t += (long long)gridDim.x * TPB) {
        double xi = x[t];
        double dv = vw[t] * inv_n;
        double B = fmax(0.0, -dc[t]) / (dv * lam);
        double xn = xi * sqrt(B);
        xn = fmin(fmin(hi, xi + move), fmax(fmax(lo, xi - move), xn));
        if (xnew) xnew[t] = xn;
        acc += vw[t] * xn;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < TPB / 32; w++) s += sh[w];
        part[blockIdx.x] = s;
    }
}

// seeded density: U[0,1) from a SplitMix64 hash of (seed, Field index)
__global__ void k_uniform(long long nc, uint64_t seed, double* __restrict__ out) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= nc) return;
    uint64_t z = seed * 0x9E3779B97F4A7C15ull + (uint64_t)t + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    out[t] = (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// 1D Gaussian along one axis (stride), clamp-to-edge; clip after the last axis
__global__ void k_blur(int n, long long nc, long long stride, const double* __restrict__ w, int R, const double* __restrict__ in,
                       double* __restrict__ out, int clip) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= nc) return;
    int c = (int)((t / stride) % n);
    double acc = 0;
    for (int q = -R; q <= R; q++) {
        int cc = min(n - 1, max(0, c + q));
        acc += w[q + R] * in[t + (long long)(cc - c) * stride];
    }
    out[t] = clip ? fmin(1.0, fmax(0.0, acc)) : acc;
}


// x_new(lambda) of the OC update for the cells of this thread (grid-stride, as k_oc) and
// the block's part of the filtered volume sum_j vw_j x_new_j.
__device__ __forceinline__ double oc_block_volume(int ncell, const double* __restrict__ x, const double* __restrict__ dc,
                                                  const double* __restrict__ vw, double lam, double move, double lo,
                                                  double hi, double* __restrict__ xnew, double* sh) {
    double acc = 0;
    const double inv_n = 1.0 / ncell;
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < ncell; t += (long long)gridDim.x * TPB) {
        const double xi = x[t];
        const double dv = vw[t] * inv_n;
        const double B = fmax(0.0, -dc[t]) / (dv * lam);
        double xn = xi * sqrt(B);
        xn = fmin(fmin(hi, xi + move), fmax(fmax(lo, xi - move), xn));
        if (xnew) xnew[t] = xn;
        acc += vw[t] * xn;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    double r = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < TPB / 32; w++) r += sh[w];
    __syncthreads();
    return r;  // valid in thread 0
}

// Sum of the block partials in the order of the partial reduction kernel (threads stride
// over the parts, warp tree, warps in order), formed by every block alike so that all
// blocks take the same bisection decision.
__device__ __forceinline__ double oc_reduce(const double* part, int nparts, double* sh) {
    double s = 0;
    for (int p = threadIdx.x; p < nparts; p += TPB) s += part[p];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0;
        for (int w = 0; w < TPB / 32; w++) r += sh[w];
        sh[TPB / 32] = r;
    }
    __syncthreads();
    const double r = sh[TPB / 32];
    __syncthreads();
    return r;
}

// The whole OC update in one cooperative launch: the multiplier bracket [0, 1e9] widened
// by decades while its upper end still overshoots the volume, then bisection to relative
// width 1e-9 (at most 200 steps), then x_new at the midpoint. One grid-wide barrier per
// probe; the partials alternate between two buffers so a probe never overwrites the ones
// the previous probe's reduction still reads.
__global__ void __launch_bounds__(TPB) k_oc_bisect(int ncell, const double* __restrict__ x, const double* __restrict__ dc,
                                                   const double* __restrict__ vw, double target, double move, double lo,
                                                   double hi, double* __restrict__ xnew, double* __restrict__ part,
                                                   double* __restrict__ lambda_out) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[TPB / 32 + 1];
    const int nparts = gridDim.x;
    int buf = 0;
    auto volume = [&](double lam) {
        const double b = oc_block_volume(ncell, x, dc, vw, lam, move, lo, hi, nullptr, sh);
        double* pp = part + buf * nparts;
        if (threadIdx.x == 0) pp[blockIdx.x] = b;
        grid.sync();
        const double v = oc_reduce(pp, nparts, sh);
        buf ^= 1;
        return v;
    };
    double l1 = 0.0, l2 = 1e9;
    for (int k = 0; k < 60; k++) {
        if (volume(l2) <= target) break;
        l1 = l2;
        l2 *= 10.0;
    }
    const double tol = 1e-9;
    int steps = 0;
    while ((l2 - l1) > tol * (l1 + l2) && steps < 200) {
        const double lmid = 0.5 * (l1 + l2);
        if (volume(lmid) > target)
            l1 = lmid;
        else
            l2 = lmid;
        steps++;
    }
    const double lmid = 0.5 * (l1 + l2);
    oc_block_volume(ncell, x, dc, vw, lmid, move, lo, hi, xnew, sh);
    if (blockIdx.x == 0 && threadIdx.x == 0) *lambda_out = lmid;
}

}  // namespace

int face_penalty_from_density(cudaStream_t st, const Geom& g, const double* rho, const stg_alpha& law, const uint8_t* m,
                              d4* P64, float4* P32) {
    k_face_penalty<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, rho, law, m, P64, P32);
    STG_LAUNCH_CK();
    return STG_OK;
}

int sensitivity(cudaStream_t st, const Geom& g, const double* rho, const stg_alpha& law, const d4* x, const d4* lam,
                double* grad) {
    long long nc = (long long)g.n * g.n * g.n;
    k_sensitivity<<<grid_for(nc, TPB), TPB, 0, st>>>(g, rho, law, x, lam, grad);
    STG_LAUNCH_CK();
    return STG_OK;
}

int density_filter(cudaStream_t st, int dim, int n, double rmin, const double* in, double* out, int transpose, double* W) {
    int R = (int)ceil(rmin) - 1;
    if (R < 0) R = 0;
    const int nz = dim == 3 ? n : 1, Rz = dim == 3 ? R : 0;
    long long nc = (long long)n * n * nz;
    WTab T{};
    const int nt = (2 * R + 1) * (2 * R + 1) * (2 * Rz + 1);
    const bool tab = nt <= WTAB_MAX;
    if (tab)
        for (int a = -R; a <= R; a++)
            for (int b = -R; b <= R; b++)
                for (int c = -Rz; c <= Rz; c++)
                    T.w[((a + R) * (2 * R + 1) + (b + R)) * (2 * Rz + 1) + (c + Rz)] = rmin - sqrt((double)(a * a + b * b + c * c));
    if (tab)
        k_filter_wsum<true><<<grid_for(nc, TPB), TPB, 0, st>>>(n, nz, rmin, R, Rz, T, W);
    else
        k_filter_wsum<false><<<grid_for(nc, TPB), TPB, 0, st>>>(n, nz, rmin, R, Rz, T, W);
    STG_LAUNCH_CK();
    if (tab)
        k_filter<true><<<grid_for(nc, TPB), TPB, 0, st>>>(n, nz, rmin, R, Rz, T, in, W, out, transpose);
    else
        k_filter<false><<<grid_for(nc, TPB), TPB, 0, st>>>(n, nz, rmin, R, Rz, T, in, W, out, transpose);
    STG_LAUNCH_CK();
    return STG_OK;
}

int oc_volume(cudaStream_t st, int ncell, const double* x, const double* dc, const double* vw, double lam, double move,
              double lo, double hi, double* xnew, double* parts, int* nparts) {
    long long g = (ncell + TPB - 1) / TPB;
    if (g > 1216) g = 1216;
    if (g < 1) g = 1;
    *nparts = (int)g;
    k_oc<<<(unsigned)g, TPB, 0, st>>>(ncell, x, dc, vw, lam, move, lo, hi, xnew, parts);
    STG_LAUNCH_CK();
    return STG_OK;
}

int oc_update_device(cudaStream_t st, int ncell, const double* x, const double* dc, const double* vw, double frac,
                     double move, double lo, double hi, double* xnew, double* parts, double* lambda_out) {
    // the grid of the probe kernel (k_oc), capped at what can be co-resident
    long long g = (ncell + TPB - 1) / TPB;
    if (g > 1216) g = 1216;
    if (g < 1) g = 1;
    int dev = 0, sms = 0, per_sm = 0;
    STG_CK(cudaGetDevice(&dev));
    STG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    STG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_oc_bisect, TPB, 0));
    if (per_sm < 1) {
        set_error("the OC bisection kernel cannot be made resident");
        return STG_E_CUDA;
    }
    if (g > (long long)sms * per_sm) g = (long long)sms * per_sm;
    double target = frac * ncell;
    void* args[] = {&ncell, &x, &dc, &vw, &target, &move, &lo, &hi, &xnew, &parts, &lambda_out};
    STG_CK(cudaLaunchCooperativeKernel((const void*)k_oc_bisect, dim3((unsigned)g), dim3(TPB), args, 0, st));
    return STG_OK;
}

int density_noise(cudaStream_t st, int dim, int n, uint64_t seed, const double* w, int R, double* out, double* tmp) {
    long long nc = dim == 3 ? (long long)n * n * n : (long long)n * n;
    unsigned gb = grid_for(nc, TPB);
    k_uniform<<<gb, TPB, 0, st>>>(nc, seed, out);
    STG_LAUNCH_CK();
    if (R >= 0 && w) {
        const long long strides3[3] = {(long long)n * n, n, 1}, strides2[2] = {n, 1};
        double* a = out;
        double* b = tmp;
        for (int ax = 0; ax < dim; ax++) {
            k_blur<<<gb, TPB, 0, st>>>(n, nc, dim == 3 ? strides3[ax] : strides2[ax], w, R, a, b, ax == dim - 1);
            STG_LAUNCH_CK();
            double* c = a;
            a = b;
            b = c;
        }
        // an odd number of passes leaves the result in tmp
        if (a != out) STG_CK(cudaMemcpyAsync(out, a, sizeof(double) * nc, cudaMemcpyDeviceToDevice, st));
    }
    return STG_OK;
}

}  // namespace stg
