// General-coefficient form of the 3D solver: per-face vol and fixed cells, the inputs
// FluidSteadyState3D::init_boundary (stoke/FluidSteadyState3D.cpp:92-114) accepts beyond
// the uniform vol and free cells of the drivers' problems.
//
// The uniform form's operators read one vol value per level and its smoother solves the
// Vanka blocks in closed form (they are arrow matrices only when every free face carries
// the same vol and no cell is fixed). Here every face carries its own vol (a per-slot
// d4 {cell vol, x-face, y-face, z-face vol}, coarsened like the reference's descriptors:
// faces sum their 4 coincident children, cells their 8) and the smoother is the
// reference's algorithm (StokeLike::GenerateJacobiPreconditioner, stoke/StokeLike.cu:345-372):
// the 7x7 block of B = M_w A M_w + M_b A M_b of every cell of a colour is read off 7 probes
// (DirectSolveBlockInverse<7>::update, common_cpx/DirectSolveBlockInverse.cuh:116-132),
// factored once per set-up by LU with partial pivoting (one thread per block, FP64), and
// applied as GATHER / solve / SHATTER inside the DescentSmoother composition
// {red x2, black x2} (common_cpx/DescentSmoother.cu:31-47). The V-cycle is
// MultigridSolve::Vcycle (common_cpx/MultigridSolve.cpp:73-106) in FP64; FGMRES and the
// FP64 refinement around it are those of the uniform form (solver.cu solve_core).
#include <algorithm>
#include <cmath>

#include "ctx.h"
#include "stencil.cuh"

namespace stg {

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ double block_sum64(double v) {
    __shared__ double sh[TPB / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < TPB / 32; w++) r += sh[w];
    return r;
}

// MODE 0: out = A x; 1: out = b - A x (x == nullptr: out = b); 2: out = E x. part: per-block
// partials of |out|^2 (mode 1) or x.out (mode 2).
template <int MODE>
__global__ void __launch_bounds__(TPB) k_op64v(Geom g, const d4* __restrict__ x, const uint8_t* __restrict__ m,
                                               const d4* __restrict__ P, const d4* __restrict__ V, const d4* __restrict__ b,
                                               d4* __restrict__ out, double* __restrict__ part) {
    const long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    double acc = 0.0;
    if (t < g.box()) {
        int i, j, k;
        g.box_ijk(t, i, j, k);
        const int s = g.slot(i, j, k);
        double o[4] = {0.0, 0.0, 0.0, 0.0};
        if (x) apply_rows_v<double, MODE == 2>(x, m, P, V, s, g.di(), g.dj(), o);
        if (MODE == 1) {
            double bp, bu, bv, bw;
            load4(b, s, bp, bu, bv, bw);
            o[0] = bp - o[0];
            o[1] = bu - o[1];
            o[2] = bv - o[2];
            o[3] = bw - o[3];
            acc = o[0] * o[0] + o[1] * o[1] + o[2] * o[2] + o[3] * o[3];
        } else if (MODE == 2) {
            double xp, xu, xv, xw;
            load4(x, s, xp, xu, xv, xw);
            acc = xp * o[0] + xu * o[1] + xv * o[2] + xw * o[3];
        }
        store4(out, s, o[0], o[1], o[2], o[3]);
    }
    if (part) {
        const double r = block_sum64(acc);
        if (threadIdx.x == 0) part[blockIdx.x] = r;
    }
}

// Coarse face vols: the 4 coincident children of a face (zero offset along its normal),
// cell vols: the 8 children (updateSubSystem, stoke/StokeFlowSubSystem3D.cu:103-154);
// then 0 on fixed or absent coarse unknowns (StokeFlowDescriptor3D::finish).
__global__ void k_coarsen_vol(Geom gc, Geom gf, const d4* __restrict__ Vf, const uint8_t* __restrict__ mc,
                              d4* __restrict__ Vc) {
    const long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= gc.box()) return;
    int I, J, K;
    gc.box_ijk(t, I, J, K);
    const int nf = gf.n;
    double c = 0, a[3] = {0, 0, 0};
    for (int q = 0; q < 8; q++) {
        const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + ((q >> 2) & 1);
        if (i > nf || j > nf || k > nf) continue;
        double vp, vu, vv, vw;
        load4(Vf, gf.slot(i, j, k), vp, vu, vv, vw);
        if (cell_ok(nf, i, j, k)) c += vp;
        if (!(q & 1) && face_ok(nf, 0, i, j, k)) a[0] += vu;
        if (!(q & 2) && face_ok(nf, 1, i, j, k)) a[1] += vv;
        if (!(q & 4) && face_ok(nf, 2, i, j, k)) a[2] += vw;
    }
    const int s = gc.slot(I, J, K);
    const uint8_t mm = mc[s];
    store4(Vc, s, (mm & MP) ? 0.0 : c, (mm & MU) ? 0.0 : a[0], (mm & MV) ? 0.0 : a[1], (mm & MW) ? 0.0 : a[2]);
}

// Per-slot vols from Field-order arrays, 0 on fixed or absent unknowns.
__global__ void k_vol_from_field(Geom g, const double* __restrict__ cell, const double* __restrict__ f0,
                                 const double* __restrict__ f1, const double* __restrict__ f2, const uint8_t* __restrict__ m,
                                 d4* __restrict__ V) {
    const long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    const int n = g.n;
    const int s = g.slot(i, j, k);
    const uint8_t mm = m[s];
    const double* f[3] = {f0, f1, f2};
    double o[4] = {0, 0, 0, 0};
    if (cell_ok(n, i, j, k) && !(mm & MP) && cell) o[0] = cell[((long long)i * n + j) * n + k];
    for (int d = 0; d < 3; d++) {
        if (!face_ok(n, d, i, j, k) || (mm & (MU << d))) continue;
        const long long ny = n + (d == 1), nz = n + (d == 2);
        o[d + 1] = f[d][((long long)i * ny + j) * nz + k];
    }
    store4(V, s, o[0], o[1], o[2], o[3]);
}

// ---------------------------------------------------------------- Vanka blocks
// Block t of colour `flag` is cell (i, j, k) with i + j + k + flag even: k = 2q + ((i + j +
// flag) & 1), t = (i n + j) n/2 + q. Its unknowns, in block order: the x-faces at i and
// i + 1, the y-faces at j and j + 1, the z-faces at k and k + 1, the pressure.
struct BlockDofs {
    int s[7];
    int c[7];
};
__device__ __forceinline__ BlockDofs block_dofs(const Geom& g, int t, int flag) {
    const int n = g.n, h = n / 2;
    const int q = t % h, j = (t / h) % n, i = t / (h * n);
    const int k = 2 * q + ((i + j + flag) & 1);
    BlockDofs b;
    const int s0 = g.slot(i, j, k);
    b.s[0] = s0;
    b.c[0] = 1;
    b.s[1] = g.slot(i + 1, j, k);
    b.c[1] = 1;
    b.s[2] = s0;
    b.c[2] = 2;
    b.s[3] = g.slot(i, j + 1, k);
    b.c[3] = 2;
    b.s[4] = s0;
    b.c[4] = 3;
    b.s[5] = g.slot(i, j, k + 1);
    b.c[5] = 3;
    b.s[6] = s0;
    b.c[6] = 0;
    return b;
}

// probe: 1 at block unknown l of every block of the colour (the rest of probe is zero)
__global__ void k_block_probe(Geom g, int flag, int l, double* __restrict__ probe) {
    const int nb = g.n * g.n * g.n / 2;
    const int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= nb) return;
    const BlockDofs b = block_dofs(g, t, flag);
    probe[4ll * b.s[l] + b.c[l]] = 1.0;
}

// StokeMask3D (stoke/StokeLike.cu:11-39): a cell is kept when i + j + k + flag is even,
// a face (of either axis, at slot (i,j,k)) when i + j + k + face_flag is even.
// ACC false: out = mask(in); true: out += mask(in)
template <bool ACC>
__global__ void k_parity_mask(Geom g, int flag, int face_flag, const d4* __restrict__ in, d4* __restrict__ out) {
    const long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    const int s = g.slot(i, j, k);
    const bool kc = ((i + j + k + flag) & 1) == 0, kf = ((i + j + k + face_flag) & 1) == 0;
    double p, u, v, w;
    load4(in, s, p, u, v, w);
    if (!kc) p = 0;
    if (!kf) u = v = w = 0;
    if (ACC) {
        double op, ou, ov, ow;
        load4(out, s, op, ou, ov, ow);
        p += op;
        u += ou;
        v += ov;
        w += ow;
    }
    store4(out, s, p, u, v, w);
}

// column l of every block (column-major 7x7: entry (row r, column l) at r + 7 l)
__global__ void k_block_gather(Geom g, int flag, int l, const double* __restrict__ y, double* __restrict__ blk) {
    const int nb = g.n * g.n * g.n / 2;
    const int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= nb) return;
    const BlockDofs b = block_dofs(g, t, flag);
    double* a = blk + 49ll * t;
    for (int r = 0; r < 7; r++) a[r + 7 * l] = y[4ll * b.s[r] + b.c[r]];
}

// LU with partial pivoting (largest magnitude in the column, first on ties), in place;
// piv[k] = the row swapped with row k. A zero pivot is left in place (the block solve then
// gives a non-finite value, as the reference's batched solve would).
__global__ void k_block_lu(int nb, double* __restrict__ blk, int8_t* __restrict__ piv) {
    const int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= nb) return;
    double a[49];
    double* g = blk + 49ll * t;
    for (int q = 0; q < 49; q++) a[q] = g[q];
    for (int k = 0; k < 7; k++) {
        int p = k;
        double best = fabs(a[k + 7 * k]);
        for (int r = k + 1; r < 7; r++) {
            const double v = fabs(a[r + 7 * k]);
            if (v > best) {
                best = v;
                p = r;
            }
        }
        piv[7ll * t + k] = (int8_t)p;
        if (p != k)
            for (int c = 0; c < 7; c++) {
                const double tmp = a[k + 7 * c];
                a[k + 7 * c] = a[p + 7 * c];
                a[p + 7 * c] = tmp;
            }
        const double d = a[k + 7 * k];
        if (d == 0.0) continue;
        const double inv = 1.0 / d;
        for (int r = k + 1; r < 7; r++) a[r + 7 * k] *= inv;
        for (int c = k + 1; c < 7; c++) {
            const double u = a[k + 7 * c];
            for (int r = k + 1; r < 7; r++) a[r + 7 * c] -= a[r + 7 * k] * u;
        }
    }
    for (int q = 0; q < 49; q++) g[q] = a[q];
}

// VelDiagPressureFullSmoothing::applyMapping (stoke/StokeLike.cu:263-272): out = SHATTER(
// B^-1 GATHER(r)) on the colour's blocks; out must be zero elsewhere (the caller clears it)
__global__ void k_block_solve(Geom g, int flag, const double* __restrict__ blk, const int8_t* __restrict__ piv,
                              const double* __restrict__ r, double* __restrict__ out) {
    const int nb = g.n * g.n * g.n / 2;
    const int t = blockIdx.x * TPB + threadIdx.x;
    if (t >= nb) return;
    const BlockDofs b = block_dofs(g, t, flag);
    const double* a = blk + 49ll * t;
    double x[7];
    for (int q = 0; q < 7; q++) x[q] = r[4ll * b.s[q] + b.c[q]];
    for (int k = 0; k < 7; k++) {
        const int p = piv[7ll * t + k];
        if (p != k) {
            const double tmp = x[k];
            x[k] = x[p];
            x[p] = tmp;
        }
    }
    for (int k = 0; k < 7; k++)
        for (int q = k + 1; q < 7; q++) x[q] -= a[q + 7 * k] * x[k];
    for (int k = 6; k >= 0; k--) {
        x[k] /= a[k + 7 * k];
        for (int q = 0; q < k; q++) x[q] -= a[q + 7 * k] * x[k];
    }
    for (int q = 0; q < 7; q++) out[4ll * b.s[q] + b.c[q]] = x[q];
}

// x += p, r -= Ap (the cycle's correction step)
__global__ void k_correct(long long n, double* __restrict__ x, const double* __restrict__ p, double* __restrict__ r,
                          const double* __restrict__ Ap) {
    const long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= n) return;
    x[t] += p[t];
    r[t] -= Ap[t];
}

// x += p only
__global__ void k_add(long long n, double* __restrict__ x, const double* __restrict__ p) {
    const long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= n) return;
    x[t] += p[t];
}

// the coarsest matrix's cell-cell diagonal of fixed cells (definite fix), which the probe
// assembly of DirectSolve3D never reads
__global__ void k_dense_fixed_cells(int nd, const int* __restrict__ slot_of, const int* __restrict__ comp_of,
                                    const uint8_t* __restrict__ m, double* __restrict__ A) {
    const int row = blockIdx.x * TPB + threadIdx.x;
    if (row >= nd) return;
    if (comp_of[row] == 0 && (m[slot_of[row]] & MP)) A[(long long)row * 2 * nd + row] += 1.0;
}

}  // namespace

// ---------------------------------------------------------------- launchers
int op64v(cudaStream_t st, const Geom& g, const d4* x, const uint8_t* m, const d4* P, const d4* V, const d4* b, d4* out,
          int mode, double* part, int* nb_out) {
    const unsigned nb = grid_for(g.box(), TPB);
    if (nb_out) *nb_out = (int)nb;
    if (mode == 0)
        k_op64v<0><<<nb, TPB, 0, st>>>(g, x, m, P, V, b, out, part);
    else if (mode == 1)
        k_op64v<1><<<nb, TPB, 0, st>>>(g, x, m, P, V, b, out, part);
    else
        k_op64v<2><<<nb, TPB, 0, st>>>(g, x, m, P, V, b, out, part);
    STG_LAUNCH_CK();
    return STG_OK;
}

int vol_from_field(cudaStream_t st, const Geom& g, const double* cell, const double* f0, const double* f1, const double* f2,
                   const uint8_t* m, d4* V) {
    k_vol_from_field<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, cell, f0, f1, f2, m, V);
    STG_LAUNCH_CK();
    return STG_OK;
}

namespace {

int gen_alloc(stg_t* h) {
    for (auto& L : h->lv) {
        const size_t ns = L.g.nslot;
        if (!L.V64 && dalloc(&L.V64, ns)) return STG_E_CUDA;
        if (!L.gr && (dalloc(&L.gr, ns) || dalloc(&L.gx, ns) || dalloc(&L.gp, ns) || dalloc(&L.gAp, ns))) return STG_E_CUDA;
        if (&L != &h->lv[0]) {
            const size_t nb = (size_t)L.g.n * L.g.n * L.g.n / 2;
            for (int c = 0; c < 2; c++)
                if (!L.vblk[c] && (dalloc(&L.vblk[c], 49 * nb) || dalloc(&L.vpiv[c], 7 * nb))) return STG_E_CUDA;
        }
    }
    const size_t ns = fine(h).g.nslot;
    for (auto& p : h->gtmp)
        if (!p && dalloc(&p, ns)) return STG_E_CUDA;
    return STG_OK;
}

// y = B s = M_w A M_w s + M_b A M_b s for the colour `flag` (VelDiagPressureFullMapping3D,
// stoke/StokeLike.cu:41-96)
int apply_B(stg_t* h, Level& L, int flag, const d4* s, d4* y, d4* t0, d4* t1) {
    const unsigned nb = grid_for(L.g.box(), TPB);
    STG_CK(cudaMemsetAsync(y, 0, sizeof(d4) * L.g.nslot, h->st));
    for (int ff = 0; ff < 2; ff++) {
        k_parity_mask<false><<<nb, TPB, 0, h->st>>>(L.g, flag, ff, s, t0);
        STG_LAUNCH_CK();
        STG_TRY(op64v(h->st, L.g, t0, L.m, L.P64, L.V64, nullptr, t1, 0, nullptr, nullptr));
        k_parity_mask<true><<<nb, TPB, 0, h->st>>>(L.g, flag, ff, t1, y);
        STG_LAUNCH_CK();
    }
    return STG_OK;
}

int vanka_setup(stg_t* h, Level& L) {
    const int nb = L.g.n * L.g.n * L.g.n / 2;
    d4 *probe = h->gtmp[0], *y = h->gtmp[1], *t0 = L.gp, *t1 = L.gAp;
    for (int flag = 0; flag < 2; flag++) {
        for (int l = 0; l < 7; l++) {
            STG_CK(cudaMemsetAsync(probe, 0, sizeof(d4) * L.g.nslot, h->st));
            k_block_probe<<<grid_for(nb, TPB), TPB, 0, h->st>>>(L.g, flag, l, reinterpret_cast<double*>(probe));
            STG_LAUNCH_CK();
            STG_TRY(apply_B(h, L, flag, probe, y, t0, t1));
            k_block_gather<<<grid_for(nb, TPB), TPB, 0, h->st>>>(L.g, flag, l, reinterpret_cast<const double*>(y), L.vblk[flag]);
            STG_LAUNCH_CK();
        }
        k_block_lu<<<grid_for(nb, TPB), TPB, 0, h->st>>>(nb, L.vblk[flag], L.vpiv[flag]);
        STG_LAUNCH_CK();
    }
    return STG_OK;
}

int correct(stg_t* h, long long n4, d4* x, const d4* p, d4* r, const d4* Ap) {
    k_correct<<<grid_for(4 * n4, TPB), TPB, 0, h->st>>>(4 * n4, reinterpret_cast<double*>(x), reinterpret_cast<const double*>(p),
                                                       reinterpret_cast<double*>(r), reinterpret_cast<const double*>(Ap));
    STG_LAUNCH_CK();
    return STG_OK;
}

}  // namespace

int gen_vanka(stg_t* h, Level& L, int flag, const d4* r, d4* out) {
    const int nb = L.g.n * L.g.n * L.g.n / 2;
    STG_CK(cudaMemsetAsync(out, 0, sizeof(d4) * L.g.nslot, h->st));
    k_block_solve<<<grid_for(nb, TPB), TPB, 0, h->st>>>(L.g, flag, L.vblk[flag], L.vpiv[flag], reinterpret_cast<const double*>(r),
                                                         reinterpret_cast<double*>(out));
    STG_LAUNCH_CK();
    return STG_OK;
}

// DescentSmoother::applyMapping (common_cpx/DescentSmoother.cu:31-47) with the two colours
// {red, black} (post: {black, red}), two steps each: out = smoother(r_in)
int gen_smooth(stg_t* h, Level& L, bool post, const d4* r_in, d4* out) {
    const long long n4 = L.g.nslot;
    d4 *r = h->gtmp[0], *d = h->gtmp[1], *Ad = h->gtmp[2];
    STG_CK(cudaMemcpyAsync(r, r_in, sizeof(d4) * n4, cudaMemcpyDeviceToDevice, h->st));
    STG_CK(cudaMemsetAsync(out, 0, sizeof(d4) * n4, h->st));
    for (int c = 0; c < 2; c++)
        for (int q = 0; q < 2; q++) {
            STG_TRY(gen_vanka(h, L, post ? 1 - c : c, r, d));
            if (c == 1 && q == 1) {  // the last step: out += d, no residual update
                k_add<<<grid_for(4 * n4, TPB), TPB, 0, h->st>>>(4 * n4, reinterpret_cast<double*>(out),
                                                               reinterpret_cast<const double*>(d));
                STG_LAUNCH_CK();
                return STG_OK;
            }
            STG_TRY(op64v(h->st, L.g, d, L.m, L.P64, L.V64, nullptr, Ad, 0, nullptr, nullptr));
            STG_TRY(correct(h, n4, out, d, r, Ad));
        }
    return STG_OK;
}

// MultigridSolve::Vcycle (common_cpx/MultigridSolve.cpp:73-106) in FP64 from a zero guess:
// the finest level's gr holds the right-hand side, its gx receives the result.
int gen_vcycle(stg_t* h) {
    const int Lc = h->L;
    for (int i = Lc - 1; i >= 0; i--) {
        Level& F = h->lv[i];
        const long long n4 = F.g.nslot;
        if (i == Lc - 1) STG_CK(cudaMemsetAsync(F.gx, 0, sizeof(d4) * n4, h->st));
        if (i > 0)
            STG_TRY(gen_smooth(h, F, false, F.gr, F.gp));
        else
            STG_TRY(dense_apply64(h->st, h->dense, F.g, F.gr, F.gp));
        STG_TRY(op64v(h->st, F.g, F.gp, F.m, F.P64, F.V64, nullptr, F.gAp, 0, nullptr, nullptr));
        STG_TRY(correct(h, n4, F.gx, F.gp, F.gr, F.gAp));
        if (i != 0) {
            Level& C = h->lv[i - 1];
            STG_TRY(restrict64(h->st, C.g, F.g, F.gr, C.m, C.gr));
            STG_CK(cudaMemsetAsync(C.gx, 0, sizeof(d4) * C.g.nslot, h->st));
        }
    }
    for (int i = 1; i < Lc; i++) {
        Level& F = h->lv[i];
        Level& C = h->lv[i - 1];
        const long long n4 = F.g.nslot;
        STG_TRY(prolong64(h->st, F.g, C.g, C.gx, F.m, F.gp));
        STG_TRY(op64v(h->st, F.g, F.gp, F.m, F.P64, F.V64, nullptr, F.gAp, 0, nullptr, nullptr));
        STG_TRY(correct(h, n4, F.gx, F.gp, F.gr, F.gAp));
        STG_TRY(gen_smooth(h, F, true, F.gr, F.gp));
        STG_TRY(op64v(h->st, F.g, F.gp, F.m, F.P64, F.V64, nullptr, F.gAp, 0, nullptr, nullptr));
        STG_TRY(correct(h, n4, F.gx, F.gp, F.gr, F.gAp));
    }
    return STG_OK;
}

// Set-up of the general form after the coarse masks and penalties are built: coarse vols,
// the coarsest inverse on the general operator (plus the fixed-cell diagonal), the Vanka
// blocks of every smoothed level.
int gen_setup(stg_t* h) {
    STG_TRY(gen_alloc(h));
    for (int i = h->L - 2; i >= 0; i--) {
        Level &c = h->lv[i], &f = h->lv[i + 1];
        k_coarsen_vol<<<grid_for(c.g.box(), TPB), TPB, 0, h->st>>>(c.g, f.g, f.V64, c.m, c.V64);
        STG_LAUNCH_CK();
    }
    Level& C0 = h->lv[0];
    STG_TRY(dense_setup_v(h->st, h->dense, C0.g, C0.V64, C0.m, C0.P64, h->closed ? 1 : 0,
                          [&](double* A, int nd) -> int {
                              k_dense_fixed_cells<<<grid_for(nd, TPB), TPB, 0, h->st>>>(nd, h->dense.slot_of,
                                                                                      h->dense.comp_of, C0.m, A);
                              STG_LAUNCH_CK();
                              return STG_OK;
                          }));
    for (int i = 1; i < h->L; i++) STG_TRY(vanka_setup(h, h->lv[i]));
    return STG_OK;
}

// ---------------------------------------------------------------- solve_core hooks
int gen_precond(stg_t* h, const float4* rhs, float4* out) {
    Level& F = fine(h);
    const long long n4 = F.g.nslot;
    STG_TRY(f32_to_f64(h->st, n4, rhs, F.gr));
    STG_TRY(gen_vcycle(h));
    STG_TRY(f64_to_f32(h->st, n4, F.gx, 1.0, out));
    return STG_OK;
}

int gen_apply32(stg_t* h, const float4* x, float4* y) {
    Level& F = fine(h);
    const long long n4 = F.g.nslot;
    STG_TRY(f32_to_f64(h->st, n4, x, h->gtmp[0]));
    STG_TRY(op64v(h->st, F.g, h->gtmp[0], F.m, F.P64, F.V64, nullptr, h->gtmp[1], 0, nullptr, nullptr));
    STG_TRY(f64_to_f32(h->st, n4, h->gtmp[1], 1.0, y));
    return STG_OK;
}

int gen_shift32(stg_t* h, const float4* v, const float4* z, float4* out) {
    Level& F = fine(h);
    const long long n4 = F.g.nslot;
    STG_TRY(f32_to_f64(h->st, n4, z, h->gtmp[0]));
    STG_TRY(f32_to_f64(h->st, n4, v, h->gtmp[1]));
    STG_TRY(op64v(h->st, F.g, h->gtmp[0], F.m, F.P64, F.V64, h->gtmp[1], h->gtmp[2], 1, nullptr, nullptr));
    STG_TRY(f64_to_f32(h->st, n4, h->gtmp[2], 1.0, out));
    return STG_OK;
}

int gen_resid64(stg_t* h, const d4* b, const d4* x, d4* r, double* nrm2_host) {
    Level& F = fine(h);
    int nb = 0;
    PROF(h, 5, 129.0 * F.g.box(), op64v(h->st, F.g, x, F.m, F.P64, F.V64, b, r, 1, h->d_parts, &nb));
    STG_TRY(reduce_parts(h->st, h->d_parts, nb, h->dnrm));
    STG_CK(cudaMemcpyAsync(nrm2_host, h->dnrm, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

}  // namespace stg
