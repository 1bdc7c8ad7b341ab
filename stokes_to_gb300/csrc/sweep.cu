// Fused smoothing sweep: one colour of the box-Vanka block-Jacobi step on the residual
// equation, x_out = x_in + SHATTER(B^-1 GATHER(r - A x_in)), in a single pass over HBM.
//
// The step is DescentSmoother's P_c applied to the current residual
// (common_cpx/DescentSmoother.cu:31-47, stoke/StokeLike.cu:220-278 and 345-372). The
// residual r - A x_in is never written out: a block owns a 32 (k) x 8 (j) column of slots
// and marches along i through a chunk of planes. Planes of x (tile + two-slot halo in j and k),
// r and P (tile + one-slot halo) are staged in shared-memory rings by asynchronous copies
// (cp.async) issued three planes ahead, the masks by register prefetch; while plane i+3
// streams in, the block forms the residual of plane i+1, the pressure update of every red
// cell of plane i (tile + one-slot low halo) and the new unknowns of plane i. Each sweep
// reads r, x, P and the mask once from HBM and writes x once.
//
// Block algebra. A red cell's block is read by DirectSolveBlockInverse<7> off
// B = M_w A M_w + M_b A M_b (stoke/StokeLike.cu:41-96, 345-372; the masks keep the faces
// of one parity). With one vol value on the free faces and no fixed cell, the face-face
// couplings inside a block cancel (grad-div against curl-curl) and B couples no two red
// blocks, so each block is an arrow matrix solved exactly by its Schur complement:
//   face rows  D_f u_f + c_f p = r_f,  D_f = vol*free_f*(4 + free(left cell) + free(right cell)) + P_f + F_f
//   pressure   sum_f b_f u_f + a p = r_p,  c_f = -vol*free_f (owner's left face) / +vol*free_f (right face),
//              b_f = free_c * c_f,  a = 2 (P_p + F_p) (the pressure diagonal is counted by both masks).
// Every face belongs to exactly one red block (the cell on its low side or on its high
// side, whichever has the colour); faces with neither are left unchanged, as SHATTER
// leaves them. If the Schur complement is 0 (the reference's LU meets a zero pivot) the
// pressure is left unchanged.
#include <cuda.h>
#include <cuda_fp16.h>

#include <type_traits>

#include "kernels.h"
#include "stencil.cuh"

namespace stg {

namespace {

constexpr int SK = 32, SJ = 8;           // output tile (k, j)
constexpr int XK = SK + 4, XJ = SJ + 4;  // x / mask region  [j0-2, j0+SJ+2) x [k0-2, k0+SK+2)
constexpr int RK = SK + 2, RJ = SJ + 2;  // r / rr / P region [j0-1, j0+SJ+1) x [k0-1, k0+SK+1)
constexpr int DK = SK + 1, DJ = SJ + 1;  // dp region        [j0-1, j0+SJ)   x [k0-1, k0+SK)
constexpr int NT = SK * SJ;
constexpr int XN = XJ * XK, RN = RJ * RK;
constexpr int DRED = (DK + 1) / 2;       // red cells per dp row (at most)
static_assert(XN <= 2 * NT && RN <= 2 * NT && DJ * DRED <= NT, "tile regions exceed two elements per thread");

// shared-memory rings: x by plane mod 4, P mod 3, r and rr mod 2, masks mod 5
struct Smem {
    float4 x[4][XN];
    float4 P[3][RN];
    float4 r[2][RN];
    float4 rr[2][RN];
    float dp[DJ * DK];
    float dpp[SJ * SK];
    uint8_t m[5][XN];
};

__device__ __forceinline__ int rx(int p) { return (p + 20) & 3; }
__device__ __forceinline__ int rp(int p) { return (p + 21) % 3; }
__device__ __forceinline__ int r2(int p) { return (p + 20) & 1; }
__device__ __forceinline__ int rm(int p) { return (p + 20) % 5; }

// 16-byte asynchronous global -> shared copy; zero-fills when !ok
__device__ __forceinline__ void cp16(void* dst, const void* src, bool ok) {
    unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    int n = ok ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Per-thread element of a staged region: its shared index, the (j,k) part of its slot
// offset and whether that (j,k) lies inside the allocation.
struct Elem {
    int sidx;   // -1: no element
    int jk;     // (j+1)*sz + (k+1)
    bool ok;    // j, k inside the allocation
    bool box;   // j, k inside [0, n]
};

__device__ __forceinline__ Elem make_elem(const Geom& g, int e, int nelem, int w, int j_org, int k_org) {
    Elem el;
    el.sidx = e < nelem ? e : -1;
    int j = j_org + e / w, k = k_org + e % w;
    el.jk = (j + 1) * g.sz + (k + 1);
    el.ok = e < nelem && j >= -1 && j <= g.n + 1 && k >= -1 && k <= g.n + 2;
    el.box = e < nelem && j >= 0 && j <= g.n && k >= 0 && k <= g.n;
    return el;
}

__device__ __forceinline__ bool plane_ok(int n, int p) { return p >= -1 && p <= n + 1; }

template <bool HAS_X, bool LAP>
__device__ __forceinline__ void residual_plane(Smem& S, const Elem (&R)[2], int n, float vol, int p) {
    const bool pin = p >= 0 && p <= n;
    const int xa = rx(p - 1), xb = rx(p), xc = rx(p + 1);
    const int ma = rm(p - 1), mb = rm(p), mc = rm(p + 1);
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int e = R[q].sidx;
        if (e < 0) continue;
        float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
        if (pin && R[q].box) {
            float4 rv = S.r[r2(p)][e];
            if (HAS_X && LAP) {
                // Laplacian form (stencil.cuh): six face neighbours, own row masked
                const int xi = e + (e / RK) * (XK - RK) + XK + 1;
                auto q = [&](int pl, int o) {
                    float4 v = S.x[pl][o];
                    return Q4<float>{v.x, v.y, v.z, v.w};
                };
                const float4 pv = S.P[rp(p)][e];
                float o[4];
                lap_core<float>(q(xb, xi), q(xa, xi), q(xc, xi), q(xb, xi - XK), q(xb, xi + XK), q(xb, xi - 1), q(xb, xi + 1),
                                Q4<float>{pv.x, pv.y, pv.z, pv.w}, vol, o);
                o[0] = rv.x - o[0];
                o[1] = rv.y - o[1];
                o[2] = rv.z - o[2];
                o[3] = rv.w - o[3];
                mask4<float>(S.m[mb][xi], o);
                out = make_float4(o[0], o[1], o[2], o[3]);
            } else if (HAS_X) {
                // rr region index e = rj*RK + rk  ->  x region index (rj+1)*XK + (rk+1)
                const int xi = e + (e / RK) * (XK - RK) + XK + 1;
                auto ld = [&](int a, int b, int c) {
                    const int pl = a < 0 ? xa : (a > 0 ? xc : xb);
                    const int ml = a < 0 ? ma : (a > 0 ? mc : mb);
                    const int o = xi + b * XK + c;
                    float4 v = S.x[pl][o];
                    return nb_make<float>(v.x, v.y, v.z, v.w, S.m[ml][o]);
                };
                uint8_t ms = S.m[mb][xi];
                float o[4];
                stencil_core<float, false>(ld, vol, ms, o);
                float4 xv = S.x[xb][xi];
                float4 pv = S.P[rp(p)][e];
                o[0] += (pv.x + ((ms & MP) ? 1.f : 0.f)) * xv.x;
                o[1] += (pv.y + ((ms & MU) ? 1.f : 0.f)) * xv.y;
                o[2] += (pv.z + ((ms & MV) ? 1.f : 0.f)) * xv.z;
                o[3] += (pv.w + ((ms & MW) ? 1.f : 0.f)) * xv.w;
                out = make_float4(rv.x - o[0], rv.y - o[1], rv.z - o[2], rv.w - o[3]);
            } else {
                out = rv;
            }
        }
        S.rr[r2(p)][e] = out;
    }
}

// pressure update of every red cell of plane p in the dp region, one thread per red cell.
// LAP: every present cell is free and every free face lies between two present cells, so a
// free face's diagonal is 6 vol + P; fixed faces (residual 0) drop out through vL / vR = 0.
template <bool LAP>
__device__ __forceinline__ void pressure_plane(Smem& S, int n, float vol, int p, int j0, int k0, int flag, int tid) {
    if (tid >= DJ * DRED) return;
    const int dj = tid / DRED, q = tid % DRED;
    const int j = j0 - 1 + dj;
    const int dk = ((p + j + flag - (k0 - 1)) & 1) + 2 * q;  // red: (p + j + k + flag) even
    const int k = k0 - 1 + dk;
    if (dk >= DK || p < 0 || j < 0 || k < 0 || !cell_ok(n, p, j, k)) return;
    const int ri = dj * RK + dk;                 // rr / P index of the cell
    const int xi = (dj + 1) * XK + (dk + 1);     // x / mask index of the cell
    float4 rc = S.rr[r2(p)][ri];
    float4 pc = S.P[rp(p)][ri];
    uint8_t m0 = S.m[rm(p)][xi];
    float out;
    if (LAP) {
        const float rL[3] = {rc.y, rc.z, rc.w};
        const float pL[3] = {pc.y, pc.z, pc.w};
        const uint8_t mhi[3] = {S.m[rm(p + 1)][xi], S.m[rm(p)][xi + XK], S.m[rm(p)][xi + 1]};
        const float rh[3] = {S.rr[r2(p + 1)][ri].y, S.rr[r2(p)][ri + RK].z, S.rr[r2(p)][ri + 1].w};
        const float ph[3] = {S.P[rp(p + 1)][ri].y, S.P[rp(p)][ri + RK].z, S.P[rp(p)][ri + 1].w};
        const uint8_t bit[3] = {MU, MV, MW};
        const float v6 = 6.f * vol;
        float num = rc.x, den = 2.f * pc.x;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            float vL = (m0 & bit[d]) ? 0.f : vol, vR = (mhi[d] & bit[d]) ? 0.f : vol;
            float iL = __fdividef(vL, v6 + pL[d]);
            float iR = __fdividef(vR, v6 + ph[d]);
            num += rL[d] * iL - rh[d] * iR;
            den -= vL * iL + vR * iR;
        }
        out = den != 0.f ? __fdividef(num, den) : 0.f;
    } else if (m0 & MP) {
        out = __fdividef(rc.x, 2.f * (pc.x + 1.f));
    } else {
        const float rL[3] = {rc.y, rc.z, rc.w};
        const float pL[3] = {pc.y, pc.z, pc.w};
        const uint8_t mlo[3] = {S.m[rm(p - 1)][xi], S.m[rm(p)][xi - XK], S.m[rm(p)][xi - 1]};
        const uint8_t mhi[3] = {S.m[rm(p + 1)][xi], S.m[rm(p)][xi + XK], S.m[rm(p)][xi + 1]};
        const float rh[3] = {S.rr[r2(p + 1)][ri].y, S.rr[r2(p)][ri + RK].z, S.rr[r2(p)][ri + 1].w};
        const float ph[3] = {S.P[rp(p + 1)][ri].y, S.P[rp(p)][ri + RK].z, S.P[rp(p)][ri + 1].w};
        const uint8_t bit[3] = {MU, MV, MW};
        float num = rc.x, den = 2.f * pc.x;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            bool fixL = m0 & bit[d], fixR = mhi[d] & bit[d];
            float vL = fixL ? 0.f : vol, vR = fixR ? 0.f : vol;
            float iL = __fdividef(1.f, vL * (5.f + ((mlo[d] & MP) ? 0.f : 1.f)) + pL[d] + (fixL ? 1.f : 0.f));
            float iR = __fdividef(1.f, vR * (5.f + ((mhi[d] & MP) ? 0.f : 1.f)) + ph[d] + (fixR ? 1.f : 0.f));
            num += vL * rL[d] * iL - vR * rh[d] * iR;
            den -= vL * vL * iL + vR * vR * iR;
        }
        out = den != 0.f ? __fdividef(num, den) : 0.f;
    }
    S.dp[dj * DK + dk] = out;
}

template <bool HAS_X, bool LAP>
__global__ void __launch_bounds__(NT, 3) k_sweep(Geom g, float vol, const float4* __restrict__ r, const float4* __restrict__ xin,
                                                float4* __restrict__ xout, const uint8_t* __restrict__ m,
                                                const float4* __restrict__ P, int flag, int chunk) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);
    const int n = g.n;
    const int tk = threadIdx.x, tj = threadIdx.y, tid = tj * SK + tk;
    const int k0 = blockIdx.x * SK, j0 = blockIdx.y * SJ, i0 = blockIdx.z * chunk;
    const int i1 = min(i0 + chunk, n + 1);
    const int j = j0 + tj, k = k0 + tk;
    const int plane = g.sy * g.sz;
    const Elem X[2] = {make_elem(g, tid, XN, XK, j0 - 2, k0 - 2), make_elem(g, tid + NT, XN, XK, j0 - 2, k0 - 2)};
    const Elem R[2] = {make_elem(g, tid, RN, RK, j0 - 1, k0 - 1), make_elem(g, tid + NT, RN, RK, j0 - 1, k0 - 1)};
    const bool out_ok = j <= n && k <= n;
    const int out_jk = (j + 1) * g.sz + (k + 1);
    const int oxi = (tj + 2) * XK + (tk + 2), ori = (tj + 1) * RK + (tk + 1), odi = (tj + 1) * DK + (tk + 1);

    auto issue_x = [&](int p) {
        const bool pok = plane_ok(n, p);
        const int base = (p + 1) * plane;
#pragma unroll
        for (int q = 0; q < 2; q++)
            if (X[q].sidx >= 0) {
                bool ok = pok && X[q].ok;
                cp16(&S.x[rx(p)][X[q].sidx], ok ? (const void*)(xin + base + X[q].jk) : (const void*)xin, ok);
            }
    };
    auto issue_r = [&](float4* dst, const float4* a, int p) {
        const bool pok = plane_ok(n, p);
        const int base = (p + 1) * plane;
#pragma unroll
        for (int q = 0; q < 2; q++)
            if (R[q].sidx >= 0) {
                bool ok = pok && R[q].ok;
                cp16(&dst[R[q].sidx], ok ? (const void*)(a + base + R[q].jk) : (const void*)a, ok);
            }
    };
    uint8_t mreg[2];
    auto fetch_m = [&](int p) {
        const bool pok = plane_ok(n, p);
        const int base = (p + 1) * plane;
#pragma unroll
        for (int q = 0; q < 2; q++) mreg[q] = (pok && X[q].ok) ? __ldg(m + base + X[q].jk) : (uint8_t)MALL;
    };
    auto store_m = [&](int p) {
#pragma unroll
        for (int q = 0; q < 2; q++)
            if (X[q].sidx >= 0) S.m[rm(p)][X[q].sidx] = mreg[q];
    };

    // prologue: planes i0-2 .. i0+2 staged, residual of i0-1 and i0, pressure of i0-1
    if (HAS_X)
        for (int p = i0 - 2; p <= i0 + 1; p++) issue_x(p);
    for (int p = i0 - 1; p <= i0 + 1; p++) issue_r(S.P[rp(p)], P, p);
    issue_r(S.r[r2(i0 - 1)], r, i0 - 1);
    issue_r(S.r[r2(i0)], r, i0);
    cp_commit();
    for (int p = i0 - 2; p <= i0 + 2; p++) {
        fetch_m(p);
        store_m(p);
    }
    cp_wait_all();
    __syncthreads();
    residual_plane<HAS_X, LAP>(S, R, n, vol, i0 - 1);
    __syncthreads();
    if (HAS_X) issue_x(i0 + 2);       // replaces plane i0-2
    issue_r(S.r[r2(i0 + 1)], r, i0 + 1);  // replaces r of i0-1
    cp_commit();
    residual_plane<HAS_X, LAP>(S, R, n, vol, i0);
    __syncthreads();
    pressure_plane<LAP>(S, n, vol, i0 - 1, j0, k0, flag, tid);
    __syncthreads();
    S.dpp[tid] = S.dp[odi];
    cp_wait_all();
    __syncthreads();

    for (int i = i0; i < i1; i++) {
        // stream plane i+3 (x, masks) and i+2 (P, r) while plane i is processed
        if (HAS_X) issue_x(i + 3);
        issue_r(S.P[rp(i + 2)], P, i + 2);
        issue_r(S.r[r2(i + 2)], r, i + 2);
        cp_commit();
        fetch_m(i + 3);
        residual_plane<HAS_X, LAP>(S, R, n, vol, i + 1);
        __syncthreads();
        pressure_plane<LAP>(S, n, vol, i, j0, k0, flag, tid);
        __syncthreads();
        if (out_ok) {
            float4 xo = HAS_X ? S.x[rx(i)][oxi] : make_float4(0.f, 0.f, 0.f, 0.f);
            float4 rv = S.rr[r2(i)][ori];
            float4 pv = S.P[rp(i)][ori];
            uint8_t m0 = S.m[rm(i)][oxi];
            const bool own_red = cell_ok(n, i, j, k) && ((i + j + k + flag) & 1) == 0;
            const float fc = (m0 & MP) ? 0.f : 1.f;
            const float dpown = S.dp[odi];
            if (own_red) xo.x += dpown;
            const float rf[3] = {rv.y, rv.z, rv.w};
            const float pf[3] = {pv.y, pv.z, pv.w};
            const uint8_t bit[3] = {MU, MV, MW};
            uint8_t mlo[3] = {0, 0, 0};
            if (!LAP) {
                mlo[0] = S.m[rm(i - 1)][oxi];
                mlo[1] = S.m[rm(i)][oxi - XK];
                mlo[2] = S.m[rm(i)][oxi - 1];
            }
            const float dplo[3] = {S.dpp[tid], S.dp[odi - DK], S.dp[odi - 1]};
            float upd[3];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                upd[d] = 0.f;
                int li = i - (d == 0), lj = j - (d == 1), lk = k - (d == 2);
                bool lower_red = !own_red && li >= 0 && lj >= 0 && lk >= 0 && cell_ok(n, li, lj, lk) &&
                                 ((li + lj + lk + flag) & 1) == 0;
                if (!own_red && !lower_red) continue;
                bool fix = m0 & bit[d];
                float v = fix ? 0.f : vol;
                // LAP: a free face has two present cells (fc = 1, lower cell present)
                float D = LAP ? (fix ? 1.f : 6.f * vol + pf[d])
                              : v * (4.f + fc + ((mlo[d] & MP) ? 0.f : 1.f)) + pf[d] + (fix ? 1.f : 0.f);
                float dpo = own_red ? dpown : dplo[d];
                float cf = own_red ? -v : v;
                upd[d] = __fdividef(rf[d] - cf * dpo, D);
            }
            xo.y += upd[0];
            xo.z += upd[1];
            xo.w += upd[2];
            xout[(i + 1) * plane + out_jk] = xo;
        }
        store_m(i + 3);
        cp_wait_all();
        __syncthreads();
        S.dpp[tid] = S.dp[odi];
    }
}

// ---------------------------------------------------------------- Laplacian-form sweep
// The same march and algebra in the Laplacian form (stencil.cuh), written so that the
// plane loop does little besides the arithmetic: ring slots are rotated element offsets
// into flat shared arrays (no modular ring indices), every per-thread index, validity
// flag and global offset is formed once before the march, global plane pointers advance
// by one plane per step, and the mask ring holds 4 planes (the Laplacian form reads no
// mask of the plane below).
struct SmemL {
    float4 x[4 * XN];
    float4 P[3 * RN];
    float4 r[2 * RN];
    float4 rr[2 * RN];
    float dp[DJ * DK];
    float dpp[SJ * SK];
    uint8_t m[4 * XN];
};

struct Stage {
    int s;   // shared index in the plane (-1: none)
    int jk;  // global offset in the plane
};

__device__ __forceinline__ Stage make_stage(const Geom& g, int e, int nelem, int w, int j_org, int k_org) {
    Stage st;
    int j = j_org + e / w, k = k_org + e % w;
    bool ok = e < nelem && j >= -1 && j <= g.n + 1 && k >= -1 && k <= g.n + 2;
    st.s = e < nelem ? e : -1;
    st.jk = ok ? (j + 1) * g.sz + (k + 1) : -1;  // -1: outside the allocation (zero fill)
    return st;
}

__device__ __forceinline__ void cp16s(unsigned dst, const void* src, bool ok) {
    int n = ok ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n) : "memory");
}

template <bool HAS_X>
__global__ void __launch_bounds__(NT, 3) k_sweep_lap(Geom g, float vol, const float4* __restrict__ r, const float4* __restrict__ xin,
                                                    float4* __restrict__ xout, const uint8_t* __restrict__ m,
                                                    const float4* __restrict__ P, int flag, int chunk) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemL& S = *reinterpret_cast<SmemL*>(smem_raw);
    const int n = g.n;
    const int tk = threadIdx.x, tj = threadIdx.y, tid = tj * SK + tk;
    const int k0 = blockIdx.x * SK, j0 = blockIdx.y * SJ, i0 = blockIdx.z * chunk;
    const int i1 = min(i0 + chunk, n + 1);
    const int j = j0 + tj, k = k0 + tk;
    const long long plane = (long long)g.sy * g.sz;
    const float v6 = 6.f * vol;

    // staging elements: x / mask region (X) and P / r region (R), two per thread
    const Stage X0 = make_stage(g, tid, XN, XK, j0 - 2, k0 - 2), X1 = make_stage(g, tid + NT, XN, XK, j0 - 2, k0 - 2);
    const Stage R0 = make_stage(g, tid, RN, RK, j0 - 1, k0 - 1), R1 = make_stage(g, tid + NT, RN, RK, j0 - 1, k0 - 1);
    const unsigned sx = (unsigned)__cvta_generic_to_shared(S.x), sP = (unsigned)__cvta_generic_to_shared(S.P),
                   sr = (unsigned)__cvta_generic_to_shared(S.r);

    // residual elements: rr/P index e and x/mask index xi, and whether (j,k) lies in [0,n]^2
    const int re0 = tid, re1 = tid + NT;
    const int rx0 = re0 + (re0 / RK) * (XK - RK) + XK + 1, rx1 = re1 + (re1 / RK) * (XK - RK) + XK + 1;
    auto in_box = [&](int e) {
        int jj = j0 - 1 + e / RK, kk = k0 - 1 + e % RK;
        return e < RN && jj >= 0 && jj <= n && kk >= 0 && kk <= n;
    };
    const bool rb0 = in_box(re0), rb1 = in_box(re1);

    // pressure-phase cell of this thread for the two plane parities
    const int pdj = tid / DRED, pq = tid % DRED, pj = j0 - 1 + pdj;
    const bool p_thread = tid < DJ * DRED;
    const int ppar0 = (pj + flag - (k0 - 1)) & 1;  // dk = ((p & 1) ^ ppar0) + 2 pq
    // (the two parities as scalars: a runtime-indexed array would live in local memory)
    const int pdk0 = 2 * pq, pdk1 = 2 * pq + 1;
    const bool pok0 = p_thread && pdk0 < DK && pj >= 0 && k0 - 1 + pdk0 >= 0 && pj < n && k0 - 1 + pdk0 < n;
    const bool pok1 = p_thread && pdk1 < DK && pj >= 0 && k0 - 1 + pdk1 >= 0 && pj < n && k0 - 1 + pdk1 < n;

    // update-phase slot
    const bool out_ok = j <= n && k <= n;
    const long long out_jk = (long long)(j + 1) * g.sz + (k + 1);
    const int oxi = (tj + 2) * XK + (tk + 2), ori = (tj + 1) * RK + (tk + 1), odi = (tj + 1) * DK + (tk + 1);
    const bool jk_cell = j < n && k < n;
    const int opar = (j + k + flag) & 1;  // own colour is red when ((i & 1) ^ opar) == 0
    const bool lo_j_ok = j >= 1 && k < n, lo_k_ok = k >= 1 && j < n;

    auto issue_x = [&](int slot, int p, const float4* src) {  // plane p of x into ring slot
        const bool pok = p >= -1 && p <= n + 1;
        if (X0.s >= 0) cp16s(sx + 16u * (slot + X0.s), (pok && X0.jk >= 0) ? (const void*)(src + X0.jk) : (const void*)xin, pok && X0.jk >= 0);
        if (X1.s >= 0) cp16s(sx + 16u * (slot + X1.s), (pok && X1.jk >= 0) ? (const void*)(src + X1.jk) : (const void*)xin, pok && X1.jk >= 0);
    };
    auto issue_r = [&](unsigned base, int slot, int p, const float4* src, const float4* any) {
        const bool pok = p >= -1 && p <= n + 1;
        if (R0.s >= 0) cp16s(base + 16u * (slot + R0.s), (pok && R0.jk >= 0) ? (const void*)(src + R0.jk) : (const void*)any, pok && R0.jk >= 0);
        if (R1.s >= 0) cp16s(base + 16u * (slot + R1.s), (pok && R1.jk >= 0) ? (const void*)(src + R1.jk) : (const void*)any, pok && R1.jk >= 0);
    };
    uint8_t mr0 = MALL, mr1 = MALL;
    auto fetch_m = [&](int p, const uint8_t* src) {
        const bool pok = p >= -1 && p <= n + 1;
        mr0 = (pok && X0.jk >= 0) ? __ldg(src + X0.jk) : (uint8_t)MALL;
        mr1 = (pok && X1.jk >= 0) ? __ldg(src + X1.jk) : (uint8_t)MALL;
    };
    auto store_m = [&](int slot) {
        if (X0.s >= 0) S.m[slot + X0.s] = mr0;
        if (X1.s >= 0) S.m[slot + X1.s] = mr1;
    };

    // residual of plane p: x slots (p-1, p, p+1), r / P / mask slots of p, into rr slot
    auto residual = [&](int p, int xa, int xb, int xc, int rs, int ps, int ms, int rrs) {
        const bool pin = p >= 0 && p <= n;
        auto one = [&](int e, int xi, bool box) {
            float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
            if (pin && box) {
                const float4 rv = S.r[rs + e];
                if (HAS_X) {
                    auto q = [&](int idx) {
                        const float4 v = S.x[idx];
                        return Q4<float>{v.x, v.y, v.z, v.w};
                    };
                    const float4 pv = S.P[ps + e];
                    float o[4];
                    lap_core<float>(q(xb + xi), q(xa + xi), q(xc + xi), q(xb + xi - XK), q(xb + xi + XK), q(xb + xi - 1),
                                    q(xb + xi + 1), Q4<float>{pv.x, pv.y, pv.z, pv.w}, vol, o);
                    o[0] = rv.x - o[0];
                    o[1] = rv.y - o[1];
                    o[2] = rv.z - o[2];
                    o[3] = rv.w - o[3];
                    mask4<float>(S.m[ms + xi], o);
                    out = make_float4(o[0], o[1], o[2], o[3]);
                } else {
                    out = rv;  // r is zero on fixed unknowns
                }
            }
            S.rr[rrs + e] = out;
        };
        one(re0, rx0, rb0);
        if (re1 < RN) one(re1, rx1, rb1);
    };

    // pressure update of the red cells of plane p (rr slots p, p+1; P slots p, p+1; mask slots p, p+1)
    auto pressure = [&](int p, int rr0, int rr1, int p0, int p1, int m0s, int m1s) {
        const int b = (p & 1) ^ ppar0;
        if (!(b ? pok1 : pok0) || p < 0 || p >= n) return;
        const int dk = b ? pdk1 : pdk0;
        const int ri = pdj * RK + dk, xi = (pdj + 1) * XK + (dk + 1);
        const float4 rc = S.rr[rr0 + ri], pc = S.P[p0 + ri];
        const uint8_t mo = S.m[m0s + xi];
        const float rL[3] = {rc.y, rc.z, rc.w}, pL[3] = {pc.y, pc.z, pc.w};
        const uint8_t mhi[3] = {S.m[m1s + xi], S.m[m0s + xi + XK], S.m[m0s + xi + 1]};
        const float rh[3] = {S.rr[rr1 + ri].y, S.rr[rr0 + ri + RK].z, S.rr[rr0 + ri + 1].w};
        const float ph[3] = {S.P[p1 + ri].y, S.P[p0 + ri + RK].z, S.P[p0 + ri + 1].w};
        const uint8_t bit[3] = {MU, MV, MW};
        float num = rc.x, den = 2.f * pc.x;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const float vL = (mo & bit[d]) ? 0.f : vol, vR = (mhi[d] & bit[d]) ? 0.f : vol;
            const float iL = __fdividef(vL, v6 + pL[d]), iR = __fdividef(vR, v6 + ph[d]);
            num += rL[d] * iL - rh[d] * iR;
            den -= vL * iL + vR * iR;
        }
        S.dp[pdj * DK + dk] = den != 0.f ? __fdividef(num, den) : 0.f;
    };

    // ring slots as element offsets (rotated each plane)
    int xm1 = 0 * XN, x0 = 1 * XN, x1 = 2 * XN, x2 = 3 * XN;  // x(i-1), x(i), x(i+1), x(i+2)
    int pm1 = 0 * RN, p0 = 1 * RN, p1 = 2 * RN;               // P(i-1), P(i), P(i+1)
    int r0 = 0 * RN, r1 = 1 * RN;                             // r(i), r(i+1)
    int rrm1 = 0 * RN, rr0 = 1 * RN;                          // rr(i-1), rr(i)
    int mm1 = 0 * XN, m0 = 1 * XN, m1 = 2 * XN, m2 = 3 * XN;  // masks of planes i-1 .. i+2

    // prologue: planes i0-2 .. i0+1 of x, i0-1 .. i0+1 of P, i0-1 and i0 of r, masks i0-1 .. i0+2
    const float4* gx = xin + (i0 - 1) * plane;  // plane p lives at (p + 1) * plane: this is plane i0-2
    if (HAS_X) {
        issue_x(xm1, i0 - 2, gx);
        issue_x(x0, i0 - 1, gx + plane);
        issue_x(x1, i0, gx + 2 * plane);
        issue_x(x2, i0 + 1, gx + 3 * plane);
    }
    const float4* gP = P + i0 * plane;
    issue_r(sP, pm1, i0 - 1, gP, P);
    issue_r(sP, p0, i0, gP + plane, P);
    issue_r(sP, p1, i0 + 1, gP + 2 * plane, P);
    const float4* gr = r + i0 * plane;
    issue_r(sr, r0, i0 - 1, gr, r);
    issue_r(sr, r1, i0, gr + plane, r);
    cp_commit();
    const uint8_t* gm = m + i0 * plane;  // plane i0-1
    fetch_m(i0 - 1, gm);
    store_m(mm1);
    fetch_m(i0, gm + plane);
    store_m(m0);
    fetch_m(i0 + 1, gm + 2 * plane);
    store_m(m1);
    fetch_m(i0 + 2, gm + 3 * plane);
    store_m(m2);
    cp_wait_all();
    __syncthreads();
    // residual of i0-1: x(i0-2, i0-1, i0) = slots (xm1, x0, x1), r(i0-1) = r0, P(i0-1) = pm1, mask(i0-1) = mm1
    residual(i0 - 1, xm1, x0, x1, r0, pm1, mm1, rrm1);
    __syncthreads();
    if (HAS_X) issue_x(xm1, i0 + 2, gx + 4 * plane);  // x(i0+2) replaces x(i0-2)
    issue_r(sr, r0, i0 + 1, gr + 2 * plane, r);       // r(i0+1) replaces r(i0-1)
    cp_commit();
    // residual of i0: x(i0-1, i0, i0+1) = (x0, x1, x2), r(i0) = r1, P(i0) = p0, mask(i0) = m0
    residual(i0, x0, x1, x2, r1, p0, m0, rr0);
    __syncthreads();
    pressure(i0 - 1, rrm1, rr0, pm1, p0, mm1, m0);
    __syncthreads();
    S.dpp[tid] = S.dp[odi];
    cp_wait_all();
    __syncthreads();
    // rotate to the loop's view at i = i0: x(i0-1..i0+2) = (x0, x1, x2, xm1), r(i0) = r1,
    // r(i0+1) = r0, rr(i0-1) = rrm1, rr(i0) = rr0, P(i0-1) = pm1, masks i0-1 .. i0+2 unchanged
    {
        int t = xm1;
        xm1 = x0;
        x0 = x1;
        x1 = x2;
        x2 = t;
        t = r0;
        r0 = r1;
        r1 = t;
    }
    gx += 5 * plane;  // plane i0+3
    gP += 3 * plane;  // plane i0+2
    gr += 3 * plane;  // plane i0+2
    gm += 4 * plane;  // plane i0+3
    float4* gout = xout + (i0 + 1) * plane + out_jk;

    for (int i = i0; i < i1; i++) {
        // stream x(i+3) into the slot of x(i-1), P(i+2) into P(i-1), r(i+2) into r(i)
        if (HAS_X) issue_x(xm1, i + 3, gx);
        issue_r(sP, pm1, i + 2, gP, P);
        issue_r(sr, r0, i + 2, gr, r);
        cp_commit();
        fetch_m(i + 3, gm);
        residual(i + 1, x0, x1, x2, r1, p1, m1, rrm1);
        __syncthreads();
        pressure(i, rr0, rrm1, p0, p1, m0, m1);
        __syncthreads();
        if (out_ok) {
            float4 xo = HAS_X ? S.x[x0 + oxi] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 rv = S.rr[rr0 + ori], pv = S.P[p0 + ori];
            const uint8_t mo = S.m[m0 + oxi];
            const bool cell = jk_cell && i < n;
            const bool own_col = ((i & 1) ^ opar) == 0;  // (i + j + k + flag) even
            const bool own_red = cell && own_col;
            const float dpown = S.dp[odi];
            if (own_red) xo.x += dpown;
            // the lower cells have the other colour: red exactly when the own colour is black
            const bool lo_ok[3] = {!own_col && i >= 1 && jk_cell, !own_col && lo_j_ok && i < n, !own_col && lo_k_ok && i < n};
            const float dplo[3] = {S.dpp[tid], S.dp[odi - DK], S.dp[odi - 1]};
            const float rf[3] = {rv.y, rv.z, rv.w}, pf[3] = {pv.y, pv.z, pv.w};
            const uint8_t bit[3] = {MU, MV, MW};
            float upd[3];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                upd[d] = 0.f;
                if (!own_red && !lo_ok[d]) continue;
                const bool fix = mo & bit[d];
                const float v = fix ? 0.f : vol;
                const float D = fix ? 1.f : v6 + pf[d];
                upd[d] = __fdividef(rf[d] - (own_red ? -v : v) * (own_red ? dpown : dplo[d]), D);
            }
            xo.y += upd[0];
            xo.z += upd[1];
            xo.w += upd[2];
            *gout = xo;
        }
        store_m(mm1);  // mask (i+3) into the slot of mask (i-1)
        cp_wait_all();
        __syncthreads();
        S.dpp[tid] = S.dp[odi];
        // rotate the rings and advance the plane pointers
        {
            int t = xm1;
            xm1 = x0;
            x0 = x1;
            x1 = x2;
            x2 = t;
            t = pm1;
            pm1 = p0;
            p0 = p1;
            p1 = t;
            t = r0;
            r0 = r1;
            r1 = t;
            t = rrm1;
            rrm1 = rr0;
            rr0 = t;
            t = mm1;
            mm1 = m0;
            m0 = m1;
            m1 = m2;
            m2 = t;
        }
        gx += plane;
        gP += plane;
        gr += plane;
        gm += plane;
        gout += plane;
    }
}

// ---------------------------------------------------------------- Laplacian-form sweep, TMA staging
// The Laplacian-form sweep with the planes of x, r and P staged by the tensor-memory
// accelerator: one thread issues one cp.async.bulk.tensor box load per plane and array
// (x: 36 x 12 slots, r and P: 34 x 10 slots, 16 bytes each) into the ring slot, with an
// mbarrier counting the bytes, instead of every thread issuing 16-byte copies. The boxes
// read zero outside the allocation, as the copies did. Everything else is k_sweep_lap.
constexpr int RNP = 344;  // r / P ring slot in float4s: RN padded to 128 bytes (TMA destinations)
constexpr int RNP16 = 352;  // P ring slot in FP16 quadruples (8 bytes): RN padded to 128 bytes
constexpr unsigned XBYTES = XN * 16, RBYTES = RN * 16, RBYTES16 = RN * 8;
static_assert(RNP >= RN && (RNP * 16) % 128 == 0 && (XN * 16) % 128 == 0, "TMA ring slots must be 128-byte aligned");
static_assert(RNP16 >= RN && (RNP16 * 8) % 128 == 0, "TMA ring slots must be 128-byte aligned");

// PB = false: P in FP32, separate rings for r and the computed residual rr (the adapters,
// which reproduce the reference smoother to FP32 rounding). PB = true (the solver's own
// sweeps): P staged from the level's FP16 copy (divided by a per-level power-of-two scale,
// multiplied back on reading), and rr written over r in place in a three-slot ring (rr(i),
// r(i+1) turning into rr(i+1), r(i+2) in flight): 68.4 -> 55.2 KB of shared memory, so
// four blocks (32 warps) share an SM instead of three. The kernel is latency- and
// issue-bound, and the extra warps hide the per-plane barriers. The smoother works with P
// to 2^-11 relative, which keeps the FP32 smoother's V-cycle count (BF16's 2^-8 did not);
// the V-cycle is a preconditioner inside FP64 refinement.
template <bool PB>
struct SmemT;
template <>
struct SmemT<false> {
    float4 x[4 * XN];
    float4 P[3 * RNP];
    float4 r[2 * RNP];
    float4 rr[2 * RN];
    float dp[DJ * DK];
    float dpp[SJ * SK];
    uint8_t m[4 * XN];
    unsigned long long bar;
};
template <>
struct SmemT<true> {
    float4 x[4 * XN];
    uint2 P[3 * RNP16];
    float4 r[3 * RNP];  // r and rr in one ring
    float dp[DJ * DK];
    float dpp[SJ * SK];
    uint8_t m[4 * XN];
    unsigned long long bar;
};

// a staged penalty quadruple as float4: FP32 as it is, or four FP16 values (x, y in the
// first word, z, w in the second, low half first) times the level's scale
__device__ __forceinline__ float4 ldv(const float4& v, float) { return v; }
__device__ __forceinline__ float4 ldv(const uint2& v, float sc) {
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&v.x)), b = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
    return make_float4(a.x * sc, a.y * sc, b.x * sc, b.y * sc);
}

// 3D box load of the tensor map at coordinates (c0, c1, c2) into shared memory, counted on bar
__device__ __forceinline__ void tma3(unsigned dst, const CUtensorMap* map, int c0, int c1, int c2, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

// arrive on bar expecting `bytes` of transfers in the current phase
__device__ __forceinline__ void arm_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

// waits for the phase of the given parity to complete; false after about a second
__device__ __forceinline__ bool wait_phase(unsigned bar, unsigned parity) {
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    while (true) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        unsigned long long t1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        if (t1 - t0 > 1000000000ull) return false;
    }
}

__device__ __forceinline__ void fail(int* err) {
    if (threadIdx.x == 0 && threadIdx.y == 0) atomicExch(err, 1);
}

// PRO (with HAS_X and PB): the sweep also applies the coarse-grid correction, x_in = x +
// inject(xc) (k_prolong_add32's injection: each unmasked unknown of a box slot adds its
// parent coarse slot's value), to every x plane as it lands in shared memory, so the
// first post-smoothing sweep replaces the prolongation pass; xout = x_in + the update.
template <bool HAS_X, bool PB, bool PRO = false>
__global__ void __launch_bounds__(NT, PB ? 4 : 3) k_sweep_tma(const __grid_constant__ CUtensorMap tmx,
                                                             const __grid_constant__ CUtensorMap tmr,
                                                             const __grid_constant__ CUtensorMap tmp, Geom g, float vol,
                                                             float4* __restrict__ xout, const uint8_t* __restrict__ m, int flag,
                                                             int chunk, int* __restrict__ err, const float* __restrict__ pscale,
                                                             const float4* __restrict__ xc, int c_plane, int c_sz) {
    static_assert(!PRO || (HAS_X && PB), "the fused prolongation needs x and the FP16 penalty ring");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SmemT<PB>& S = *reinterpret_cast<SmemT<PB>*>(smem_raw);
    float4* RR;  // the residual ring: its own array, or the r ring itself
    if constexpr (PB)
        RR = S.r;
    else
        RR = S.rr;
    constexpr int PSTR = PB ? RNP16 : RNP;               // P ring slot, elements
    constexpr unsigned PESZ = PB ? 8u : 16u;             // P element bytes
    constexpr unsigned PBYTES = PB ? RBYTES16 : RBYTES;  // bytes one P box load delivers
    const float psc = PB ? __ldg(pscale) : 1.f;          // the FP16 copy's scale
    const int n = g.n;
    const int tk = threadIdx.x, tj = threadIdx.y, tid = tj * SK + tk;
    const int k0 = blockIdx.x * SK, j0 = blockIdx.y * SJ, i0 = blockIdx.z * chunk;
    const int i1 = i0 + chunk >= n ? n + 1 : i0 + chunk;  // the last chunk also takes plane n
    const int j = j0 + tj, k = k0 + tk;
    const float v6 = 6.f * vol;

    // staging elements: x / mask region (X) and P / r region (R), two per thread
    const Stage X0 = make_stage(g, tid, XN, XK, j0 - 2, k0 - 2), X1 = make_stage(g, tid + NT, XN, XK, j0 - 2, k0 - 2);
    const unsigned sx = (unsigned)__cvta_generic_to_shared(S.x), sP = (unsigned)__cvta_generic_to_shared(S.P),
                   sr = (unsigned)__cvta_generic_to_shared(S.r);

    // residual elements: rr/P index e and x/mask index xi, and whether (j,k) lies in [0,n]^2
    const int re0 = tid, re1 = tid + NT;
    const int rx0 = re0 + (re0 / RK) * (XK - RK) + XK + 1, rx1 = re1 + (re1 / RK) * (XK - RK) + XK + 1;
    auto in_box = [&](int e) {
        int jj = j0 - 1 + e / RK, kk = k0 - 1 + e % RK;
        return e < RN && jj >= 0 && jj <= n && kk >= 0 && kk <= n;
    };
    const bool rb0 = in_box(re0), rb1 = in_box(re1);

    // pressure-phase cell of this thread for the two plane parities
    const int pdj = tid / DRED, pq = tid % DRED, pj = j0 - 1 + pdj;
    const bool p_thread = tid < DJ * DRED;
    const int ppar0 = (pj + flag - (k0 - 1)) & 1;  // dk = ((p & 1) ^ ppar0) + 2 pq
    // (the two parities as scalars: a runtime-indexed array would live in local memory)
    const int pdk0 = 2 * pq, pdk1 = 2 * pq + 1;
    const bool pok0 = p_thread && pdk0 < DK && pj >= 0 && k0 - 1 + pdk0 >= 0 && pj < n && k0 - 1 + pdk0 < n;
    const bool pok1 = p_thread && pdk1 < DK && pj >= 0 && k0 - 1 + pdk1 >= 0 && pj < n && k0 - 1 + pdk1 < n;

    // update-phase slot
    const bool out_ok = j <= n && k <= n;
    const long long out_jk = (long long)(j + 1) * g.sz + (k + 1);
    const int oxi = (tj + 2) * XK + (tk + 2), ori = (tj + 1) * RK + (tk + 1), odi = (tj + 1) * DK + (tk + 1);
    // the grid's tiles cover [0, n) in j and k: where a tile ends at n, its last lane in k
    // (last row in j) also writes the slot at k = n (j = n)
    const bool ext_k = tk == SK - 1 && k + 1 == n && j <= n, ext_j = tj == SJ - 1 && j + 1 == n && k <= n;

    // plane p of x (region origin j0-2, k0-2) or of r / P (origin j0-1, k0-1) into a ring
    // slot by one TMA box load each; out-of-allocation parts of a box read as zero
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&S.bar);
    auto tma_x = [&](int slot, int p) { tma3(sx + 16u * slot, &tmx, 4 * (k0 - 1), j0 - 1, p + 1, bar); };
    auto tma_r = [&](unsigned base, int slot, int p, const CUtensorMap* tm) { tma3(base + 16u * slot, tm, 4 * k0, j0, p + 1, bar); };
    auto tma_p = [&](int slot, int p) { tma3(sP + PESZ * slot, &tmp, 4 * k0, j0, p + 1, bar); };
    uint32_t phase = 0;
    // every thread waits for the current phase; a wait that gives up (about a second) makes
    // the whole block record the error and leave at the next barrier
    auto wait_loads = [&]() {
        const bool ok = wait_phase(bar, phase);
        phase ^= 1u;
        return ok;
    };
    // fused prolongation: the thread's two staged x elements, whether they lie in the
    // box's (j, k) range, and their parents' offsets in a coarse plane
    bool pin0 = false, pin1 = false;
    int cofs0 = 0, cofs1 = 0;
    if (PRO) {
        auto setup = [&](const Stage& X, int e, bool& pin, int& cofs) {
            const int jj = j0 - 2 + e / XK, kk = k0 - 2 + e % XK;
            pin = X.s >= 0 && jj >= 0 && jj <= n && kk >= 0 && kk <= n;
            cofs = pin ? ((jj >> 1) + 1) * c_sz + ((kk >> 1) + 1) : 0;
        };
        setup(X0, tid, pin0, cofs0);
        setup(X1, tid + NT, pin1, cofs1);
    }
    // the coarse values of plane p for the thread's two elements (zero outside the box)
    auto coarse = [&](int p, float4& v0, float4& v1) {
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        v0 = v1 = z;
        if (!PRO || p < 0 || p > n) return;
        const float4* cp = xc + (long long)((p >> 1) + 1) * c_plane;
        if (pin0) v0 = __ldg(cp + cofs0);
        if (pin1) v1 = __ldg(cp + cofs1);
    };
    // x plane p in ring slot xs += the coarse values v0, v1, with the masks ma, mb
    auto inject = [&](int xs, int p, const float4& v0, const float4& v1, uint8_t ma, uint8_t mb) {
        if (!PRO || p < 0 || p > n) return;
        auto add = [&](int idx, const float4& v, uint8_t mm) {
            float4 x = S.x[xs + idx];
            if (!(mm & MP)) x.x += v.x;
            if (!(mm & MU)) x.y += v.y;
            if (!(mm & MV)) x.z += v.z;
            if (!(mm & MW)) x.w += v.w;
            S.x[xs + idx] = x;
        };
        if (pin0) add(X0.s, v0, ma);
        if (pin1) add(X1.s, v1, mb);
    };
    auto prolong = [&](int xs, int p, uint8_t ma, uint8_t mb) {
        float4 v0, v1;
        coarse(p, v0, v1);
        inject(xs, p, v0, v1, ma, mb);
    };
    uint8_t mr0 = MALL, mr1 = MALL;
    auto fetch_m = [&](int p, const uint8_t* src) {
        const bool pok = p >= -1 && p <= n + 1;
        mr0 = (pok && X0.jk >= 0) ? __ldg(src + X0.jk) : (uint8_t)MALL;
        mr1 = (pok && X1.jk >= 0) ? __ldg(src + X1.jk) : (uint8_t)MALL;
    };
    auto store_m = [&](int slot) {
        if (X0.s >= 0) S.m[slot + X0.s] = mr0;
        if (X1.s >= 0) S.m[slot + X1.s] = mr1;
    };

    // residual of plane p: x slots (p-1, p, p+1), r / P / mask slots of p, into rr slot
    auto residual = [&](int p, int xa, int xb, int xc, int rs, int ps, int ms, int rrs) {
        const bool pin = p >= 0 && p <= n;
        auto one = [&](int e, int xi, bool box) {
            float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
            if (pin && box) {
                const float4 rv = S.r[rs + e];
                if (HAS_X) {
                    auto q = [&](int idx) {
                        const float4 v = S.x[idx];
                        return Q4<float>{v.x, v.y, v.z, v.w};
                    };
                    const float4 pv = ldv(S.P[ps + e], psc);
                    float o[4];
                    lap_core<float>(q(xb + xi), q(xa + xi), q(xc + xi), q(xb + xi - XK), q(xb + xi + XK), q(xb + xi - 1),
                                    q(xb + xi + 1), Q4<float>{pv.x, pv.y, pv.z, pv.w}, vol, o);
                    o[0] = rv.x - o[0];
                    o[1] = rv.y - o[1];
                    o[2] = rv.z - o[2];
                    o[3] = rv.w - o[3];
                    mask4<float>(S.m[ms + xi], o);
                    out = make_float4(o[0], o[1], o[2], o[3]);
                } else {
                    out = rv;  // r is zero on fixed unknowns
                }
            }
            RR[rrs + e] = out;
        };
        one(re0, rx0, rb0);
        if (re1 < RN) one(re1, rx1, rb1);
    };

    // pressure update of the red cells of plane p (rr slots p, p+1; P slots p, p+1; mask slots p, p+1)
    auto pressure = [&](int p, int rr0, int rr1, int p0, int p1, int m0s, int m1s) {
        const int b = (p & 1) ^ ppar0;
        if (!(b ? pok1 : pok0) || p < 0 || p >= n) return;
        const int dk = b ? pdk1 : pdk0;
        const int ri = pdj * RK + dk, xi = (pdj + 1) * XK + (dk + 1);
        const float4 rc = RR[rr0 + ri], pc = ldv(S.P[p0 + ri], psc);
        const uint8_t mo = S.m[m0s + xi];
        const float rL[3] = {rc.y, rc.z, rc.w}, pL[3] = {pc.y, pc.z, pc.w};
        const uint8_t mhi[3] = {S.m[m1s + xi], S.m[m0s + xi + XK], S.m[m0s + xi + 1]};
        const float rh[3] = {RR[rr1 + ri].y, RR[rr0 + ri + RK].z, RR[rr0 + ri + 1].w};
        const float ph[3] = {ldv(S.P[p1 + ri], psc).y, ldv(S.P[p0 + ri + RK], psc).z, ldv(S.P[p0 + ri + 1], psc).w};
        const uint8_t bit[3] = {MU, MV, MW};
        float num = rc.x, den = 2.f * pc.x;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const float vL = (mo & bit[d]) ? 0.f : vol, vR = (mhi[d] & bit[d]) ? 0.f : vol;
            const float iL = __fdividef(vL, v6 + pL[d]), iR = __fdividef(vR, v6 + ph[d]);
            num += rL[d] * iL - rh[d] * iR;
            den -= vL * iL + vR * iR;
        }
        S.dp[pdj * DK + dk] = den != 0.f ? __fdividef(num, den) : 0.f;
    };

    // ring slots as element offsets (rotated each plane)
    int xm1 = 0 * XN, x0 = 1 * XN, x1 = 2 * XN, x2 = 3 * XN;  // x(i-1), x(i), x(i+1), x(i+2)
    int pm1 = 0 * PSTR, p0 = 1 * PSTR, p1 = 2 * PSTR;         // P(i-1), P(i), P(i+1)
    int r0 = 0 * RNP, r1 = 1 * RNP;                           // r(i), r(i+1)
    int rrm1 = 0 * RN, rr0 = 1 * RN;                          // rr(i-1), rr(i)
    if constexpr (PB) {  // rr written over r in place: one ring of three slots
        rrm1 = r0;
        rr0 = r1;
    }
    int mm1 = 0 * XN, m0 = 1 * XN, m1 = 2 * XN, m2 = 3 * XN;  // masks of planes i-1 .. i+2

    // new x of slot (i, jj, kk) of the current plane (x / mask index xi, rr / P index ri,
    // dp index di of its own cell), written to dst: the pressure of an own red cell, and
    // each face whose red block is the own cell (red) or the cell below it (the own cell
    // black). dp is read only where that red cell exists, so the high-side slots (jj or
    // kk = n) read nothing outside the dp region; dpp (the cell below in i) only for the
    // thread's own (j, k).
    auto update = [&](int i, int jj, int kk, int xi, int ri, int di, float4* dst) {
        float4 xo = HAS_X ? S.x[x0 + xi] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 rv = RR[rr0 + ri], pv = ldv(S.P[p0 + ri], psc);
        const uint8_t mo = S.m[m0 + xi];
        const bool jkc = jj < n && kk < n;
        const bool own_col = ((i + jj + kk + flag) & 1) == 0;
        const bool own_red = jkc && i < n && own_col;
        const float dpown = own_red ? S.dp[di] : 0.f;
        if (own_red) xo.x += dpown;
        // the lower cells have the other colour: red exactly when the own colour is black
        const bool lo_ok[3] = {!own_col && i >= 1 && jkc, !own_col && jj >= 1 && kk < n && i < n,
                               !own_col && kk >= 1 && jj < n && i < n};
        const float dplo[3] = {lo_ok[0] ? S.dpp[tid] : 0.f, lo_ok[1] ? S.dp[di - DK] : 0.f, lo_ok[2] ? S.dp[di - 1] : 0.f};
        const float rf[3] = {rv.y, rv.z, rv.w}, pf[3] = {pv.y, pv.z, pv.w};
        const uint8_t bit[3] = {MU, MV, MW};
        float upd[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            upd[d] = 0.f;
            if (!own_red && !lo_ok[d]) continue;
            const bool fix = mo & bit[d];
            const float v = fix ? 0.f : vol;
            const float D = fix ? 1.f : v6 + pf[d];
            upd[d] = __fdividef(rf[d] - (own_red ? -v : v) * (own_red ? dpown : dplo[d]), D);
        }
        xo.y += upd[0];
        xo.z += upd[1];
        xo.w += upd[2];
        *dst = xo;
    };

    // prologue: planes i0-2 .. i0+1 of x, i0-1 .. i0+1 of P, i0-1 and i0 of r, masks i0-1 .. i0+2
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        arm_tx(bar, (HAS_X ? 4 * XBYTES : 0) + 3 * PBYTES + 2 * RBYTES);
        if (HAS_X) {
            tma_x(xm1, i0 - 2);
            tma_x(x0, i0 - 1);
            tma_x(x1, i0);
            tma_x(x2, i0 + 1);
        }
        tma_p(pm1, i0 - 1);
        tma_p(p0, i0);
        tma_p(p1, i0 + 1);
        tma_r(sr, r0, i0 - 1, &tmr);
        tma_r(sr, r1, i0, &tmr);
    }
    const long long plane = (long long)g.sy * g.sz;
    const uint8_t* gm = m + i0 * plane;  // plane i0-1
    fetch_m(i0 - 1, gm);
    store_m(mm1);
    fetch_m(i0, gm + plane);
    store_m(m0);
    fetch_m(i0 + 1, gm + 2 * plane);
    store_m(m1);
    fetch_m(i0 + 2, gm + 3 * plane);
    store_m(m2);
    if (__syncthreads_or(!wait_loads())) return fail(err);
    if (PRO) {
        // planes i0-1 .. i0+1 take their masks from the ring (the thread's own entries), i0-2
        // from memory
        auto ms = [&](int slot, const Stage& X) { return X.s >= 0 ? S.m[slot + X.s] : (uint8_t)MALL; };
        const uint8_t* g2 = m + (long long)(i0 - 1) * plane;  // plane i0-2
        const bool ok2 = i0 - 2 >= 0;
        prolong(xm1, i0 - 2, ok2 && X0.jk >= 0 ? __ldg(g2 + X0.jk) : (uint8_t)MALL, ok2 && X1.jk >= 0 ? __ldg(g2 + X1.jk) : (uint8_t)MALL);
        prolong(x0, i0 - 1, ms(mm1, X0), ms(mm1, X1));
        prolong(x1, i0, ms(m0, X0), ms(m0, X1));
        prolong(x2, i0 + 1, ms(m1, X0), ms(m1, X1));
        __syncthreads();
    }
    // residual of i0-1: x(i0-2, i0-1, i0) = slots (xm1, x0, x1), r(i0-1) = r0, P(i0-1) = pm1, mask(i0-1) = mm1
    residual(i0 - 1, xm1, x0, x1, r0, pm1, mm1, rrm1);
    __syncthreads();
    if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        arm_tx(bar, (HAS_X ? XBYTES : 0) + RBYTES);
        if (HAS_X) tma_x(xm1, i0 + 2);  // x(i0+2) replaces x(i0-2)
        tma_r(sr, PB ? 2 * RNP : r0, i0 + 1, &tmr);  // r(i0+1): the third slot, or replaces r(i0-1)
    }
    // residual of i0: x(i0-1, i0, i0+1) = (x0, x1, x2), r(i0) = r1, P(i0) = p0, mask(i0) = m0
    residual(i0, x0, x1, x2, r1, p0, m0, rr0);
    __syncthreads();
    pressure(i0 - 1, rrm1, rr0, pm1, p0, mm1, m0);
    __syncthreads();
    S.dpp[tid] = S.dp[odi];
    if (__syncthreads_or(!wait_loads())) return fail(err);
    if (PRO) {  // x(i0+2) landed in slot xm1; its masks are in ring slot m2
        prolong(xm1, i0 + 2, X0.s >= 0 ? S.m[m2 + X0.s] : (uint8_t)MALL, X1.s >= 0 ? S.m[m2 + X1.s] : (uint8_t)MALL);
        __syncthreads();
    }
    // rotate to the loop's view at i = i0: x(i0-1..i0+2) = (x0, x1, x2, xm1), r(i0) = r1,
    // r(i0+1) = r0, rr(i0-1) = rrm1, rr(i0) = rr0, P(i0-1) = pm1, masks i0-1 .. i0+2 unchanged
    {
        int t = xm1;
        xm1 = x0;
        x0 = x1;
        x1 = x2;
        x2 = t;
        if constexpr (PB) {  // rr(i0) in slot 1, r(i0+1) in slot 2, slot 0 (rr(i0-1)) free
            r0 = 0;
            r1 = rrm1 = 2 * RNP;
            rr0 = RNP;
        } else {
            t = r0;
            r0 = r1;
            r1 = t;
        }
    }
    gm += 4 * plane;  // plane i0+3
    float4* gout = xout + (i0 + 1) * plane + out_jk;

    for (int i = i0; i < i1; i++) {
        // stream x(i+3) into the slot of x(i-1), P(i+2) into P(i-1), r(i+2) into r(i)
        if (tid == 0) {
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            arm_tx(bar, (HAS_X ? XBYTES : 0) + PBYTES + RBYTES);
            if (HAS_X) tma_x(xm1, i + 3);
            tma_p(pm1, i + 2);
            tma_r(sr, r0, i + 2, &tmr);
        }
        fetch_m(i + 3, gm);
        // the coarse values for x(i+3) are loaded now and injected once it has landed, so
        // their latency hides behind this plane's work
        float4 pc0, pc1;
        coarse(i + 3, pc0, pc1);
        residual(i + 1, x0, x1, x2, r1, p1, m1, rrm1);
        __syncthreads();
        pressure(i, rr0, rrm1, p0, p1, m0, m1);
        __syncthreads();
        if (out_ok) {
            update(i, j, k, oxi, ori, odi, gout);
            // the last tile in k (j) also writes column k = n (row j = n): slots whose only
            // unknowns are the faces on the box's high side, updated by the cells below them
            if (ext_k) update(i, j, k + 1, oxi + 1, ori + 1, odi + 1, gout + 1);
            if (ext_j) update(i, j + 1, k, oxi + XK, ori + RK, odi + DK, gout + g.sz);
            if (ext_j && ext_k) update(i, j + 1, k + 1, oxi + XK + 1, ori + RK + 1, odi + DK + 1, gout + g.sz + 1);
        }
        store_m(mm1);  // mask (i+3) into the slot of mask (i-1)
        if (__syncthreads_or(!wait_loads())) return fail(err);
        S.dpp[tid] = S.dp[odi];
        if (PRO) {  // x(i+3) landed in slot xm1; its masks are still in registers
            inject(xm1, i + 3, pc0, pc1, mr0, mr1);
            __syncthreads();
        }
        // rotate the rings and advance the plane pointers
        {
            int t = xm1;
            xm1 = x0;
            x0 = x1;
            x1 = x2;
            x2 = t;
            t = pm1;
            pm1 = p0;
            p0 = p1;
            p1 = t;
            if constexpr (PB) {  // (rr(i), r(i+1), free) <- (r(i+1) now rr(i+1), r(i+2), rr(i))
                t = rr0;
                rr0 = r1;
                r1 = rrm1 = r0;
                r0 = t;
            } else {
                t = r0;
                r0 = r1;
                r1 = t;
                t = rrm1;
                rrm1 = rr0;
                rr0 = t;
            }
            t = mm1;
            mm1 = m0;
            m0 = m1;
            m1 = m2;
            m2 = t;
        }
        gm += plane;
        gout += plane;
    }
}

}  // namespace

namespace {

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                 const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// the driver's tensor-map encoder, fetched through the runtime (no link against the driver
// library); null when unavailable, in which case the sweep stages with cp.async
EncodeTiled encoder() {
    static EncodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
        cudaGetLastError();
    }
    return fn;
}

// tensor map of a slot array of g as FP32 [planes][rows][4 (n+4)], box (4 bk) x bj x 1
bool slot_map(EncodeTiled enc, CUtensorMap* map, const void* base, const Geom& g, int bk, int bj) {
    const cuuint64_t dims[3] = {(cuuint64_t)g.sz * 4, (cuuint64_t)g.sy, (cuuint64_t)g.sx};
    const cuuint64_t strides[2] = {(cuuint64_t)g.sz * 16, (cuuint64_t)g.sy * g.sz * 16};
    const cuuint32_t box[3] = {(cuuint32_t)(4 * bk), (cuuint32_t)bj, 1}, es[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the same for an FP16 slot array (four 2-byte values per slot)
bool slot_map16(EncodeTiled enc, CUtensorMap* map, const void* base, const Geom& g, int bk, int bj) {
    const cuuint64_t dims[3] = {(cuuint64_t)g.sz * 4, (cuuint64_t)g.sy, (cuuint64_t)g.sx};
    const cuuint64_t strides[2] = {(cuuint64_t)g.sz * 8, (cuuint64_t)g.sy * g.sz * 8};
    const cuuint32_t box[3] = {(cuuint32_t)(4 * bk), (cuuint32_t)bj, 1}, es[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// per device: kernel attributes set, and the flag a TMA sweep sets when its wait gave up
bool g_attr_set[MAX_DEVICES] = {}, g_tattr_set[MAX_DEVICES] = {};
int* g_sweep_err[MAX_DEVICES] = {};
int g_sms[MAX_DEVICES] = {};

// Planes per block of the TMA sweep on an n^3 box. On large boxes a block marches through
// its chunk plane after plane (plus about three planes of prologue), and the blocks run in
// waves of SMs x resident blocks, so the chunk minimises waves x (chunk + 3), the longest
// chain of planes an SM works through (at n = 256: 37 planes, 2.9 waves, 2 % faster than
// 32 planes and 3.4 waves). On the coarse levels, where the blocks are few and latency
// sets the time, that choice measured 2 % slower than the fixed lengths kept there.
int tma_chunk(int dev, int n, bool fp16_pen) {
    if (n < 192) return n >= 96 ? 8 : n >= 48 ? 4 : n >= 24 ? 2 : 1;
    if (!g_sms[dev] && cudaDeviceGetAttribute(&g_sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) g_sms[dev] = 0;
    const long long slots = (long long)(g_sms[dev] > 0 ? g_sms[dev] : 152) * (fp16_pen ? 4 : 3);
    const long long plane_blocks = (long long)((n + SK - 1) / SK) * ((n + SJ - 1) / SJ);
    int best = 1;
    long long best_cost = -1;
    for (int c = 1; c <= n; c++) {
        const long long blocks = plane_blocks * ((n + c - 1) / c);
        const long long cost = ((blocks + slots - 1) / slots) * (c + 3);
        if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            best = c;
        }
    }
    return best;
}

}  // namespace

bool sweep_tma_available() { return encoder() != nullptr; }

int sweep_status(cudaStream_t st, int* timed_out) {
    *timed_out = 0;
    const int dev = device_slot();
    if (dev < 0 || !g_sweep_err[dev]) return STG_OK;
    STG_CK(cudaMemcpyAsync(timed_out, g_sweep_err[dev], sizeof(int), cudaMemcpyDeviceToHost, st));
    STG_CK(cudaStreamSynchronize(st));
    return STG_OK;
}

int sweep32(cudaStream_t st, const Geom& g, float vol, const float4* r, const float4* xin, float4* xout, const uint8_t* m,
            const float4* P, int flag, bool lap, const __half* P16, const float* p16_scale, const float4* xc, const Geom* gc) {
    const int dev = device_slot();
    if (dev < 0) {
        set_error("sweep32: device ordinal beyond %d", MAX_DEVICES - 1);
        return STG_E_UNSUPPORTED;
    }
    const int smem = (int)sizeof(Smem), smem_l = (int)sizeof(SmemL);
    if (!g_attr_set[dev]) {
        STG_CK(cudaFuncSetAttribute(k_sweep<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        STG_CK(cudaFuncSetAttribute(k_sweep<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        STG_CK(cudaFuncSetAttribute(k_sweep_lap<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_l));
        STG_CK(cudaFuncSetAttribute(k_sweep_lap<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_l));
        g_attr_set[dev] = true;
    }
    // planes per block: long marches on big grids (prologue amortised), short ones on the
    // coarse levels, where the sequential march, not bandwidth, sets the time
    const int chunk = g.n >= 192 ? 32 : g.n >= 96 ? 8 : g.n >= 48 ? 4 : g.n >= 24 ? 2 : 1;
    dim3 grid((g.n + SK) / SK, (g.n + SJ) / SJ, (g.n + chunk) / chunk), block(SK, SJ);
    // the TMA sweep's tiles and chunks cover [0, n) and take the high-side slots (k, j or
    // i = n) with the last ones (at n = 256: 8 x 32 x 7 blocks of 37 planes)
    const int chunk_t = tma_chunk(dev, g.n, P16 != nullptr);
    const dim3 grid_t((g.n + SK - 1) / SK, (g.n + SJ - 1) / SJ, (g.n + chunk_t - 1) / chunk_t);
    if (lap && encoder()) {
        const int smem_t = (int)sizeof(SmemT<false>), smem_b = (int)sizeof(SmemT<true>);
        if (!g_tattr_set[dev]) {
            STG_CK(cudaFuncSetAttribute(k_sweep_tma<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_t));
            STG_CK(cudaFuncSetAttribute(k_sweep_tma<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_t));
            STG_CK(cudaFuncSetAttribute(k_sweep_tma<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_b));
            STG_CK(cudaFuncSetAttribute(k_sweep_tma<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_b));
            STG_CK(cudaFuncSetAttribute(k_sweep_tma<true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_b));
            STG_CK(cudaMalloc((void**)&g_sweep_err[dev], sizeof(int)));
            STG_CK(cudaMemset(g_sweep_err[dev], 0, sizeof(int)));
            g_tattr_set[dev] = true;
        }
        CUtensorMap mx{}, mr{}, mp{};
        const EncodeTiled enc = encoder();
        if (P16 && !p16_scale) P16 = nullptr;  // the FP16 copy needs its scale
        const bool ok = (!xin || slot_map(enc, &mx, xin, g, XK, XJ)) && slot_map(enc, &mr, r, g, RK, RJ) &&
                        (P16 ? slot_map16(enc, &mp, P16, g, RK, RJ) : slot_map(enc, &mp, P, g, RK, RJ));
        if (ok) {
            int* err = g_sweep_err[dev];
            if (xc && P16 && xin) {
                k_sweep_tma<true, true, true><<<grid_t, block, smem_b, st>>>(mx, mr, mp, g, vol, xout, m, flag, chunk_t, err, p16_scale,
                                                                             xc, gc->sy * gc->sz, gc->sz);
                STG_LAUNCH_CK();
                return STG_OK;
            }
            if (xc) {
                set_error("sweep32: the fused prolongation needs x and the FP16 penalty");
                return STG_E_UNSUPPORTED;
            }
            if (P16 && xin)
                k_sweep_tma<true, true><<<grid_t, block, smem_b, st>>>(mx, mr, mp, g, vol, xout, m, flag, chunk_t, err, p16_scale, nullptr, 0, 0);
            else if (P16)
                k_sweep_tma<false, true><<<grid_t, block, smem_b, st>>>(mr, mr, mp, g, vol, xout, m, flag, chunk_t, err, p16_scale, nullptr, 0, 0);
            else if (xin)
                k_sweep_tma<true, false><<<grid_t, block, smem_t, st>>>(mx, mr, mp, g, vol, xout, m, flag, chunk_t, err, nullptr, nullptr, 0, 0);
            else
                k_sweep_tma<false, false><<<grid_t, block, smem_t, st>>>(mr, mr, mp, g, vol, xout, m, flag, chunk_t, err, nullptr, nullptr, 0, 0);
            STG_LAUNCH_CK();
            return STG_OK;
        }
    }
    if (xc) {
        set_error("sweep32: the fused prolongation needs the TMA sweep");
        return STG_E_UNSUPPORTED;
    }
    if (xin && lap)
        k_sweep_lap<true><<<grid, block, smem_l, st>>>(g, vol, r, xin, xout, m, P, flag, chunk);
    else if (xin)
        k_sweep<true, false><<<grid, block, smem, st>>>(g, vol, r, xin, xout, m, P, flag, chunk);
    else if (lap)
        k_sweep_lap<false><<<grid, block, smem_l, st>>>(g, vol, r, xin, xout, m, P, flag, chunk);
    else
        k_sweep<false, false><<<grid, block, smem, st>>>(g, vol, r, xin, xout, m, P, flag, chunk);
    STG_LAUNCH_CK();
    return STG_OK;
}

}  // namespace stg
