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

}  // namespace

int sweep32(cudaStream_t st, const Geom& g, float vol, const float4* r, const float4* xin, float4* xout, const uint8_t* m,
            const float4* P, int flag, bool lap) {
    static bool attr_set = false;
    const int smem = (int)sizeof(Smem);
    if (!attr_set) {
        STG_CK(cudaFuncSetAttribute(k_sweep<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        STG_CK(cudaFuncSetAttribute(k_sweep<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        STG_CK(cudaFuncSetAttribute(k_sweep<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        STG_CK(cudaFuncSetAttribute(k_sweep<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr_set = true;
    }
    // planes per block: long marches on big grids (prologue amortised), short ones on the
    // coarse levels, where the sequential march, not bandwidth, sets the time
    const int chunk = g.n >= 192 ? 32 : g.n >= 96 ? 16 : g.n >= 48 ? 8 : g.n >= 24 ? 4 : 2;
    dim3 grid((g.n + SK) / SK, (g.n + SJ) / SJ, (g.n + chunk) / chunk), block(SK, SJ);
    if (xin && lap)
        k_sweep<true, true><<<grid, block, smem, st>>>(g, vol, r, xin, xout, m, P, flag, chunk);
    else if (xin)
        k_sweep<true, false><<<grid, block, smem, st>>>(g, vol, r, xin, xout, m, P, flag, chunk);
    else if (lap)
        k_sweep<false, true><<<grid, block, smem, st>>>(g, vol, r, xin, xout, m, P, flag, chunk);
    else
        k_sweep<false, false><<<grid, block, smem, st>>>(g, vol, r, xin, xout, m, P, flag, chunk);
    STG_LAUNCH_CK();
    return STG_OK;
}

}  // namespace stg
