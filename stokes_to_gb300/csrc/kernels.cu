// Grid kernels of the multigrid hierarchy: FP64/FP32 operator and residual, the
// colored box-Vanka block update, fused residual + restriction, prolongation,
// coarse re-discretisation and layout conversions.
#include <cuda_bf16.h>

#include "kernels.h"
#include "stencil.cuh"

namespace stg {

namespace {

constexpr int TPB = 256;

template <class T>
__device__ __forceinline__ T block_sum(T v) {
    __shared__ T sh[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    T r = 0;
    if (wid == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : T(0);
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;
}

// ------------------------------------------------------------------ operators
template <int MODE>
__global__ void __launch_bounds__(TPB) k_op64(Geom g, double vol, const d4* __restrict__ x, const uint8_t* __restrict__ m,
                                              const d4* __restrict__ P, const d4* __restrict__ b, d4* __restrict__ out,
                                              double* __restrict__ part) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    double acc = 0.0;
    if (t < g.box()) {
        int i, j, k;
        g.box_ijk(t, i, j, k);
        int s = g.slot(i, j, k);
        double o[4];
        if (MODE == 2)
            apply_rows<double, true>(x, m, P, s, g.di(), g.dj(), vol, o);
        else
            apply_rows<double, false>(x, m, P, s, g.di(), g.dj(), vol, o);
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
        double r = block_sum(acc);
        if (threadIdx.x == 0) part[blockIdx.x] = r;
    }
}

template <bool HAS_X, bool RESID>
__global__ void __launch_bounds__(TPB) k_op32(Geom g, float vol, const float4* __restrict__ r, const float4* __restrict__ x,
                                              const uint8_t* __restrict__ m, const float4* __restrict__ P,
                                              float4* __restrict__ out) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    int s = g.slot(i, j, k);
    float o[4] = {0.f, 0.f, 0.f, 0.f};
    if (HAS_X) apply_rows<float, false>(x, m, P, s, g.di(), g.dj(), vol, o);
    if (RESID) {
        float4 rv = __ldg(r + s);
        out[s] = make_float4(rv.x - o[0], rv.y - o[1], rv.z - o[2], rv.w - o[3]);
    } else {
        out[s] = make_float4(o[0], o[1], o[2], o[3]);
    }
}

// ------------------------------------------------------------------ box-Vanka
// Block of red cell c (7 unknowns: the six faces and the pressure), as extracted by
// DirectSolveBlockInverse<7> from B = M_w A M_w + M_b A M_b (stoke/StokeLike.cu:41-96,
// 345-372). With one vol value on the free faces and no fixed cell, the face-face
// couplings of B inside a block cancel (grad-div against curl-curl) and B's couplings to
// other red blocks vanish, so the block is an arrow matrix:
//   face rows   D_f u_f + c_f p = r_f ,  D_f = vol*free_f*(4 + free_cell(left) + free_cell(right)) + P_f + F_f
//   pressure    sum_f b_f u_f + a p = r_p,  c_f = -/+ vol*free_f (left/right face), b_f = free_c * c_f,
//               a = 2 (P_p + F_p)  (the pressure diagonal is counted by both masks)
// and is solved exactly by its Schur complement. (If the complement is 0 the
// reference's LU has a zero pivot; this kernel leaves the pressure unchanged there.)
// Pressure update of the arrow block of red cell c (its Schur-complement equation).
__device__ __forceinline__ float vanka_dp(const float4* __restrict__ rr, const uint8_t* __restrict__ m,
                                          const float4* __restrict__ P, int c, int di, int dj, float vol) {
    const int off[3] = {di, dj, 1};
    const uint8_t bit[3] = {MU, MV, MW};
    float4 rc = __ldg(rr + c);
    float4 pc = __ldg(P + c);
    uint8_t m0 = __ldg(m + c);
    if (m0 & MP) return rc.x / (2.f * (pc.x + 1.f));  // fixed cell: b = 0, a = 2 (P + 1)
    const float rL[3] = {rc.y, rc.z, rc.w};
    const float pL[3] = {pc.y, pc.z, pc.w};
    float num = rc.x, den = 2.f * pc.x;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        uint8_t mlo = __ldg(m + c - off[d]);
        uint8_t mhi = __ldg(m + c + off[d]);
        float4 rh = __ldg(rr + c + off[d]);
        float4 ph = __ldg(P + c + off[d]);
        float rhv = d == 0 ? rh.y : d == 1 ? rh.z : rh.w;
        float phv = d == 0 ? ph.y : d == 1 ? ph.z : ph.w;
        bool fixL = m0 & bit[d], fixR = mhi & bit[d];
        float vL = fixL ? 0.f : vol, vR = fixR ? 0.f : vol;
        float DL = vL * (5.f + ((mlo & MP) ? 0.f : 1.f)) + pL[d] + (fixL ? 1.f : 0.f);
        float DR = vR * (5.f + ((mhi & MP) ? 0.f : 1.f)) + phv + (fixR ? 1.f : 0.f);
        // b_f = c_f = -vL (left), +vR (right) for a free cell
        num -= (-vL) * rL[d] / DL + vR * rhv / DR;
        den -= vL * vL / DL + vR * vR / DR;
    }
    return den != 0.f ? num / den : 0.f;
}

// Tiled box-Vanka step. A block owns a 32 (k) x 8 (j) column of slots and marches along i
// through VT_CHUNK planes. Per plane it first forms the pressure update of every red cell
// of the plane over the tile plus a one-slot low halo in j and k (shared memory), then
// every slot updates its own unknowns: its pressure if its cell is red, and each face
// from the red cell that owns it (the cell itself, or its lower neighbour along the
// face normal), with the face diagonal D_f formed from the slot's own coefficients.
constexpr int VT_K = 32, VT_J = 8, VT_CHUNK = 16;

template <bool HAS_X>
__global__ void __launch_bounds__(VT_K* VT_J) k_vanka_tiled(Geom g, float vol, const float4* __restrict__ rr,
                                                          const float4* __restrict__ xin, float4* __restrict__ xout,
                                                          const uint8_t* __restrict__ m, const float4* __restrict__ P,
                                                          int flag) {
    __shared__ float dp_cur[VT_J + 1][VT_K + 1];
    __shared__ float dp_prev[VT_J][VT_K];
    const int n = g.n, di = g.di(), dj = g.dj();
    const int tk = threadIdx.x, tj = threadIdx.y, tid = tj * VT_K + tk;
    const int k0 = blockIdx.x * VT_K, j0 = blockIdx.y * VT_J, i0 = blockIdx.z * VT_CHUNK;
    const int i1 = min(i0 + VT_CHUNK, n + 1);
    const int k = k0 + tk, j = j0 + tj;
    const bool in_box = k <= n && j <= n;
    // pressure updates of plane i0 - 1 (owners of the x-faces of plane i0)
    {
        int i = i0 - 1;
        bool red = i >= 0 && cell_ok(n, i, j, k) && ((i + j + k + flag) & 1) == 0;
        dp_prev[tj][tk] = red ? vanka_dp(rr, m, P, g.slot(i, j, k), di, dj, vol) : 0.f;
    }
    for (int i = i0; i < i1; i++) {
        for (int e = tid; e < (VT_J + 1) * (VT_K + 1); e += VT_K * VT_J) {
            int jj = j0 - 1 + e / (VT_K + 1), kk = k0 - 1 + e % (VT_K + 1);
            bool red = jj >= 0 && kk >= 0 && cell_ok(n, i, jj, kk) && ((i + jj + kk + flag) & 1) == 0;
            dp_cur[e / (VT_K + 1)][e % (VT_K + 1)] = red ? vanka_dp(rr, m, P, g.slot(i, jj, kk), di, dj, vol) : 0.f;
        }
        __syncthreads();
        if (in_box) {
            int s = g.slot(i, j, k);
            float4 r = __ldg(rr + s);
            float4 pp = __ldg(P + s);
            uint8_t m0 = __ldg(m + s);
            float4 xo = HAS_X ? __ldg(xin + s) : make_float4(0.f, 0.f, 0.f, 0.f);
            const bool own_red = cell_ok(n, i, j, k) && ((i + j + k + flag) & 1) == 0;
            const float fc = (m0 & MP) ? 0.f : 1.f;
            if (own_red) xo.x += dp_cur[tj + 1][tk + 1];
            // faces: owner = this cell if red (left face, c_f = -vol), else the lower neighbour (right face, +vol)
            const float rf[3] = {r.y, r.z, r.w};
            const float pf[3] = {pp.y, pp.z, pp.w};
            const uint8_t bit[3] = {MU, MV, MW};
            const int offs[3] = {di, dj, 1};
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
                uint8_t mlo = __ldg(m + s - offs[d]);
                float D = v * (4.f + fc + ((mlo & MP) ? 0.f : 1.f)) + pf[d] + (fix ? 1.f : 0.f);
                float dpo = own_red ? dp_cur[tj + 1][tk + 1]
                                    : (d == 0 ? dp_prev[tj][tk] : d == 1 ? dp_cur[tj][tk + 1] : dp_cur[tj + 1][tk]);
                float cf = own_red ? -v : v;
                upd[d] = (rf[d] - cf * dpo) / D;
            }
            xo.y += upd[0];
            xo.z += upd[1];
            xo.w += upd[2];
            xout[s] = xo;
        }
        __syncthreads();
        dp_prev[tj][tk] = dp_cur[tj + 1][tk + 1];
        __syncthreads();
    }
}

// ------------------------------------------------------------------ transfers
// Restriction (stoke/StokeFlowSubSystem3D.cu:32-52 with common_cpx/SubsystemUtils3D.cuh:8-186):
// the coarse unknown of every kind at slot (I,J,K) sums the eight fine unknowns of the same
// kind at slots (2I+a, 2J+b, 2K+c), then fixed coarse unknowns are zeroed. Fused with the
// fine residual r - A x.
template <bool HAS_X>
__global__ void __launch_bounds__(TPB) k_restrict_res32(Geom gc, Geom gf, float volf, const float4* __restrict__ rf,
                                                        const float4* __restrict__ xf, const uint8_t* __restrict__ mf,
                                                        const float4* __restrict__ Pf, const uint8_t* __restrict__ mc,
                                                        float4* __restrict__ rc) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= gc.box()) return;
    int I, J, K;
    gc.box_ijk(t, I, J, K);
    const int nf = gf.n;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        int i = 2 * I + (c & 1), j = 2 * J + ((c >> 1) & 1), k = 2 * K + ((c >> 2) & 1);
        if (i > nf || j > nf || k > nf) continue;
        int s = gf.slot(i, j, k);
        float4 r = __ldg(rf + s);
        if (HAS_X) {
            float o[4];
            apply_rows<float, false>(xf, mf, Pf, s, gf.di(), gf.dj(), volf, o);
            r.x -= o[0];
            r.y -= o[1];
            r.z -= o[2];
            r.w -= o[3];
        }
        a0 += r.x;
        a1 += r.y;
        a2 += r.z;
        a3 += r.w;
    }
    int sc = gc.slot(I, J, K);
    uint8_t mm = __ldg(mc + sc);
    rc[sc] = make_float4((mm & MP) ? 0.f : a0, (mm & MU) ? 0.f : a1, (mm & MV) ? 0.f : a2, (mm & MW) ? 0.f : a3);
}

// Prolongation (stoke/StokeFlowSubSystem3D.cu:81-101 with SubsystemUtils3D.cuh:370-495):
// piecewise-constant injection from the parent slot, fixed fine unknowns zeroed.
template <class C>
__device__ __forceinline__ float4 parent_value(const C* xc, int sc);
template <>
__device__ __forceinline__ float4 parent_value<float4>(const float4* xc, int sc) {
    return __ldg(xc + sc);
}
template <>
__device__ __forceinline__ float4 parent_value<__nv_bfloat16>(const __nv_bfloat16* xc, int sc) {
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(xc + 4ll * sc);
    float2 a = __bfloat1622float2(h[0]), b = __bfloat1622float2(h[1]);
    return make_float4(a.x, a.y, b.x, b.y);
}

template <class C>
__global__ void __launch_bounds__(TPB) k_prolong_add32(Geom gf, Geom gc, const C* __restrict__ xc,
                                                       const uint8_t* __restrict__ mf, float4* __restrict__ xf) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= gf.box()) return;
    int i, j, k;
    gf.box_ijk(t, i, j, k);
    int s = gf.slot(i, j, k);
    float4 v = parent_value<C>(xc, gc.slot(i >> 1, j >> 1, k >> 1));
    uint8_t mm = __ldg(mf + s);
    float4 x = xf[s];
    if (!(mm & MP)) x.x += v.x;
    if (!(mm & MU)) x.y += v.y;
    if (!(mm & MV)) x.z += v.z;
    if (!(mm & MW)) x.w += v.w;
    xf[s] = x;
}

__global__ void k_to_bf16(Geom g, const float4* __restrict__ x, __nv_bfloat16* __restrict__ y) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    int s = g.slot(i, j, k);
    float4 v = __ldg(x + s);
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(y + 4ll * s);
    h[0] = __floats2bfloat162_rn(v.x, v.y);
    h[1] = __floats2bfloat162_rn(v.z, v.w);
}

__global__ void k_restrict64(Geom gc, Geom gf, const d4* __restrict__ rf, const uint8_t* __restrict__ mc, d4* __restrict__ rc) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= gc.box()) return;
    int I, J, K;
    gc.box_ijk(t, I, J, K);
    double a[4] = {0, 0, 0, 0};
    for (int c = 0; c < 8; c++) {
        int i = 2 * I + (c & 1), j = 2 * J + ((c >> 1) & 1), k = 2 * K + ((c >> 2) & 1);
        if (i > gf.n || j > gf.n || k > gf.n) continue;
        double p, u, v, w;
        load4(rf, gf.slot(i, j, k), p, u, v, w);
        a[0] += p;
        a[1] += u;
        a[2] += v;
        a[3] += w;
    }
    int sc = gc.slot(I, J, K);
    uint8_t mm = mc[sc];
    store4(rc, sc, (mm & MP) ? 0.0 : a[0], (mm & MU) ? 0.0 : a[1], (mm & MV) ? 0.0 : a[2], (mm & MW) ? 0.0 : a[3]);
}

__global__ void k_prolong64(Geom gf, Geom gc, const d4* __restrict__ xc, const uint8_t* __restrict__ mf, d4* __restrict__ xf) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= gf.box()) return;
    int i, j, k;
    gf.box_ijk(t, i, j, k);
    int s = gf.slot(i, j, k);
    double p, u, v, w;
    load4(xc, gc.slot(i >> 1, j >> 1, k >> 1), p, u, v, w);
    uint8_t mm = mf[s];
    store4(xf, s, (mm & MP) ? 0.0 : p, (mm & MU) ? 0.0 : u, (mm & MV) ? 0.0 : v, (mm & MW) ? 0.0 : w);
}

// updateSubSystem (stoke/StokeFlowSubSystem3D.cu:103-154) + finish(): fixed = OR over the
// eight children that exist, penalty = sum of the eight; not-present coarse unknowns are
// fixed and every fixed unknown carries zero penalty. (The vol sums reduce to the scalar
// 4*vol for the uniform form; cell vol never enters A.)
__global__ void k_coarsen(Geom gc, Geom gf, const uint8_t* __restrict__ mf, const d4* __restrict__ Pf, uint8_t* __restrict__ mc,
                          d4* __restrict__ Pc64, float4* __restrict__ Pc32) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= gc.box()) return;
    int I, J, K;
    gc.box_ijk(t, I, J, K);
    const int nf = gf.n;
    uint8_t mo = 0;
    double a[4] = {0, 0, 0, 0};
    for (int c = 0; c < 8; c++) {
        int i = 2 * I + (c & 1), j = 2 * J + ((c >> 1) & 1), k = 2 * K + ((c >> 2) & 1);
        if (i > nf || j > nf || k > nf) continue;
        int s = gf.slot(i, j, k);
        uint8_t present = (uint8_t)(~invalid_bits(nf, i, j, k) & MALL);
        mo |= (uint8_t)(mf[s] & present);
        double p, u, v, w;
        load4(Pf, s, p, u, v, w);
        a[0] += p;
        a[1] += u;
        a[2] += v;
        a[3] += w;
    }
    mo |= invalid_bits(gc.n, I, J, K);
    if (mo & MP) a[0] = 0;
    if (mo & MU) a[1] = 0;
    if (mo & MV) a[2] = 0;
    if (mo & MW) a[3] = 0;
    int sc = gc.slot(I, J, K);
    mc[sc] = mo;
    store4(Pc64, sc, a[0], a[1], a[2], a[3]);
    Pc32[sc] = make_float4((float)a[0], (float)a[1], (float)a[2], (float)a[3]);
}

// ------------------------------------------------------------------ layout conversions
__device__ __forceinline__ long long field_index(int n, int d, int i, int j, int k) {
    // d = -1: cell array; d = 0..2: face array of axis d (N+1 along d)
    long long cy = n + (d == 1), cz = n + (d == 2);
    return ((long long)i * cy + j) * cz + k;
}

__global__ void k_field_to_slots64(Geom g, const double* __restrict__ cell, const double* __restrict__ f0,
                                   const double* __restrict__ f1, const double* __restrict__ f2, d4* __restrict__ out) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    const int n = g.n;
    double p = (cell && cell_ok(n, i, j, k)) ? cell[field_index(n, -1, i, j, k)] : 0.0;
    double u = (f0 && face_ok(n, 0, i, j, k)) ? f0[field_index(n, 0, i, j, k)] : 0.0;
    double v = (f1 && face_ok(n, 1, i, j, k)) ? f1[field_index(n, 1, i, j, k)] : 0.0;
    double w = (f2 && face_ok(n, 2, i, j, k)) ? f2[field_index(n, 2, i, j, k)] : 0.0;
    store4(out, g.slot(i, j, k), p, u, v, w);
}

__global__ void k_slots_to_field64(Geom g, const d4* __restrict__ in, double* __restrict__ cell, double* __restrict__ f0,
                                   double* __restrict__ f1, double* __restrict__ f2) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    const int n = g.n;
    double p, u, v, w;
    load4(in, g.slot(i, j, k), p, u, v, w);
    if (cell && cell_ok(n, i, j, k)) cell[field_index(n, -1, i, j, k)] = p;
    if (f0 && face_ok(n, 0, i, j, k)) f0[field_index(n, 0, i, j, k)] = u;
    if (f1 && face_ok(n, 1, i, j, k)) f1[field_index(n, 1, i, j, k)] = v;
    if (f2 && face_ok(n, 2, i, j, k)) f2[field_index(n, 2, i, j, k)] = w;
}

__global__ void k_mask_from_field(Geom g, const int* __restrict__ cell, const int* __restrict__ f0, const int* __restrict__ f1,
                                  const int* __restrict__ f2, uint8_t* __restrict__ m) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.nslot) return;
    // halo slots: everything fixed / absent
    int k = (int)(t % g.sz) - 1;
    long long r = t / g.sz;
    int j = (int)(r % g.sy) - 1;
    int i = (int)(r / g.sy) - 1;
    const int n = g.n;
    if (i < 0 || j < 0 || k < 0 || i > n || j > n || k > n) {
        m[t] = MALL;
        return;
    }
    uint8_t b = invalid_bits(n, i, j, k);
    if (cell && cell_ok(n, i, j, k) && cell[field_index(n, -1, i, j, k)]) b |= MP;
    if (f0 && face_ok(n, 0, i, j, k) && f0[field_index(n, 0, i, j, k)]) b |= MU;
    if (f1 && face_ok(n, 1, i, j, k) && f1[field_index(n, 1, i, j, k)]) b |= MV;
    if (f2 && face_ok(n, 2, i, j, k) && f2[field_index(n, 2, i, j, k)]) b |= MW;
    m[t] = b;
}

__global__ void k_penalty_from_field(Geom g, const double* __restrict__ cell, const double* __restrict__ f0,
                                     const double* __restrict__ f1, const double* __restrict__ f2, const uint8_t* __restrict__ m,
                                     d4* __restrict__ P64, float4* __restrict__ P32) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    const int n = g.n;
    int s = g.slot(i, j, k);
    uint8_t mm = m[s];
    double p = (cell && !(mm & MP)) ? cell[field_index(n, -1, i, j, k)] : 0.0;
    double u = (f0 && !(mm & MU)) ? f0[field_index(n, 0, i, j, k)] : 0.0;
    double v = (f1 && !(mm & MV)) ? f1[field_index(n, 1, i, j, k)] : 0.0;
    double w = (f2 && !(mm & MW)) ? f2[field_index(n, 2, i, j, k)] : 0.0;
    store4(P64, s, p, u, v, w);
    P32[s] = make_float4((float)p, (float)u, (float)v, (float)w);
}

// Blocked (reference) index -> (slot, component) or -1 for a padding entry.
__device__ __forceinline__ int blocked_to_slot(const Geom& g, const Blocked& B, long long idx, int& comp) {
    int x, y, z;
    long long nc = B.cell_size(), nf = B.face_size();
    if (idx < nc) {
        B.ind_cell(idx, x, y, z);
        comp = 0;
        return g.slot(x, y, z);
    }
    idx -= nc;
    int d = (int)(idx / nf);
    idx -= (long long)d * nf;
    B.ind_face(idx, d, x, y, z);
    if (!face_ok(g.n, d, x, y, z)) return -1;
    comp = d + 1;
    return g.slot(x, y, z);
}

__global__ void k_blocked_to_slots64(Geom g, Blocked B, const double* __restrict__ in, double* __restrict__ out) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= B.size()) return;
    int comp;
    int s = blocked_to_slot(g, B, t, comp);
    if (s >= 0) out[4ll * s + comp] = in[t];
}

__global__ void k_slots_to_blocked64(Geom g, Blocked B, const double* __restrict__ in, double* __restrict__ out,
                                     const double* __restrict__ pad_src) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= B.size()) return;
    int comp;
    int s = blocked_to_slot(g, B, t, comp);
    out[t] = s >= 0 ? in[4ll * s + comp] : (pad_src ? pad_src[t] : 0.0);
}

__global__ void k_mask_to_blocked(Geom g, Blocked B, const uint8_t* __restrict__ m, uint8_t* __restrict__ out) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= B.size()) return;
    int comp;
    int s = blocked_to_slot(g, B, t, comp);
    out[t] = s >= 0 ? ((m[s] >> comp) & 1) : 1;
}

__global__ void k_vol_slots(Geom g, const uint8_t* __restrict__ m, double cell_vol, double vol, d4* __restrict__ out) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    int s = g.slot(i, j, k);
    uint8_t mm = m[s];
    store4(out, s, (mm & MP) ? 0.0 : cell_vol, (mm & MU) ? 0.0 : vol, (mm & MV) ? 0.0 : vol, (mm & MW) ? 0.0 : vol);
}

__global__ void k_half_square64(long long n, const double* __restrict__ x, double* __restrict__ out) {
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < n; t += (long long)gridDim.x * TPB)
        out[t] = (0.5 * x[t]) * x[t];
}

}  // namespace

// ------------------------------------------------------------------ launchers
int vol_slots(cudaStream_t st, const Geom& g, const uint8_t* m, double cell_vol, double vol, d4* out) {
    k_vol_slots<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, m, cell_vol, vol, out);
    STG_LAUNCH_CK();
    return STG_OK;
}

int half_square64(cudaStream_t st, long long n4, const d4* x, d4* out) {
    long long nb = (4 * n4 + TPB - 1) / TPB;
    k_half_square64<<<(unsigned)(nb > 4096 ? 4096 : nb), TPB, 0, st>>>(4 * n4, reinterpret_cast<const double*>(x),
                                                                        reinterpret_cast<double*>(out));
    STG_LAUNCH_CK();
    return STG_OK;
}

int op64(cudaStream_t st, const Geom& g, double vol, const d4* x, const uint8_t* m, const d4* P, const d4* b, d4* out,
         int mode, double* part, int* nblocks_out) {
    unsigned nb = grid_for(g.box(), TPB);
    if (nblocks_out) *nblocks_out = (int)nb;
    if (mode == 0)
        k_op64<0><<<nb, TPB, 0, st>>>(g, vol, x, m, P, b, out, part);
    else if (mode == 1)
        k_op64<1><<<nb, TPB, 0, st>>>(g, vol, x, m, P, b, out, part);
    else
        k_op64<2><<<nb, TPB, 0, st>>>(g, vol, x, m, P, b, out, part);
    STG_LAUNCH_CK();
    return STG_OK;
}

int resid32(cudaStream_t st, const Geom& g, float vol, const float4* r, const float4* x, const uint8_t* m, const float4* P,
            float4* rr) {
    unsigned nb = grid_for(g.box(), TPB);
    if (x)
        k_op32<true, true><<<nb, TPB, 0, st>>>(g, vol, r, x, m, P, rr);
    else
        k_op32<false, true><<<nb, TPB, 0, st>>>(g, vol, r, x, m, P, rr);
    STG_LAUNCH_CK();
    return STG_OK;
}

int apply32(cudaStream_t st, const Geom& g, float vol, const float4* x, const uint8_t* m, const float4* P, float4* y) {
    k_op32<true, false><<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, vol, nullptr, x, m, P, y);
    STG_LAUNCH_CK();
    return STG_OK;
}

int vanka32(cudaStream_t st, const Geom& g, float vol, const float4* rr, const float4* xin, float4* xout, const uint8_t* m,
            const float4* P, int flag) {
    dim3 grid((g.n + VT_K) / VT_K, (g.n + VT_J) / VT_J, (g.n + VT_CHUNK) / VT_CHUNK), block(VT_K, VT_J);
    if (xin)
        k_vanka_tiled<true><<<grid, block, 0, st>>>(g, vol, rr, xin, xout, m, P, flag);
    else
        k_vanka_tiled<false><<<grid, block, 0, st>>>(g, vol, rr, xin, xout, m, P, flag);
    STG_LAUNCH_CK();
    return STG_OK;
}

int restrict_resid32(cudaStream_t st, const Geom& gc, const Geom& gf, float volf, const float4* rf, const float4* xf,
                     const uint8_t* mf, const float4* Pf, const uint8_t* mc, float4* rc) {
    unsigned nb = grid_for(gc.box(), TPB);
    if (xf)
        k_restrict_res32<true><<<nb, TPB, 0, st>>>(gc, gf, volf, rf, xf, mf, Pf, mc, rc);
    else
        k_restrict_res32<false><<<nb, TPB, 0, st>>>(gc, gf, volf, rf, xf, mf, Pf, mc, rc);
    STG_LAUNCH_CK();
    return STG_OK;
}

int prolong_add32(cudaStream_t st, const Geom& gf, const Geom& gc, const float4* xc, const uint8_t* mf, float4* xf) {
    k_prolong_add32<float4><<<grid_for(gf.box(), TPB), TPB, 0, st>>>(gf, gc, xc, mf, xf);
    STG_LAUNCH_CK();
    return STG_OK;
}

int prolong_add_bf16(cudaStream_t st, const Geom& gf, const Geom& gc, const __nv_bfloat16* xc, const uint8_t* mf, float4* xf) {
    k_prolong_add32<__nv_bfloat16><<<grid_for(gf.box(), TPB), TPB, 0, st>>>(gf, gc, xc, mf, xf);
    STG_LAUNCH_CK();
    return STG_OK;
}

int to_bf16(cudaStream_t st, const Geom& g, const float4* x, __nv_bfloat16* y) {
    k_to_bf16<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, x, y);
    STG_LAUNCH_CK();
    return STG_OK;
}

int coarsen(cudaStream_t st, const Geom& gc, const Geom& gf, const uint8_t* mf, const d4* Pf, uint8_t* mc, d4* Pc64,
            float4* Pc32) {
    k_coarsen<<<grid_for(gc.box(), TPB), TPB, 0, st>>>(gc, gf, mf, Pf, mc, Pc64, Pc32);
    STG_LAUNCH_CK();
    return STG_OK;
}

int restrict64(cudaStream_t st, const Geom& gc, const Geom& gf, const d4* rf, const uint8_t* mc, d4* rc) {
    k_restrict64<<<grid_for(gc.box(), TPB), TPB, 0, st>>>(gc, gf, rf, mc, rc);
    STG_LAUNCH_CK();
    return STG_OK;
}

int prolong64(cudaStream_t st, const Geom& gf, const Geom& gc, const d4* xc, const uint8_t* mf, d4* xf) {
    k_prolong64<<<grid_for(gf.box(), TPB), TPB, 0, st>>>(gf, gc, xc, mf, xf);
    STG_LAUNCH_CK();
    return STG_OK;
}

int field_to_slots64(cudaStream_t st, const Geom& g, const double* cell, const double* f0, const double* f1, const double* f2,
                     d4* out) {
    k_field_to_slots64<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, cell, f0, f1, f2, out);
    STG_LAUNCH_CK();
    return STG_OK;
}

int slots_to_field64(cudaStream_t st, const Geom& g, const d4* in, double* cell, double* f0, double* f1, double* f2) {
    k_slots_to_field64<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, in, cell, f0, f1, f2);
    STG_LAUNCH_CK();
    return STG_OK;
}

int mask_from_field(cudaStream_t st, const Geom& g, const int* cell, const int* f0, const int* f1, const int* f2, uint8_t* m) {
    k_mask_from_field<<<grid_for(g.nslot, TPB), TPB, 0, st>>>(g, cell, f0, f1, f2, m);
    STG_LAUNCH_CK();
    return STG_OK;
}

int penalty_from_field(cudaStream_t st, const Geom& g, const double* cell, const double* f0, const double* f1, const double* f2,
                       const uint8_t* m, d4* P64, float4* P32) {
    k_penalty_from_field<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, cell, f0, f1, f2, m, P64, P32);
    STG_LAUNCH_CK();
    return STG_OK;
}

int blocked_to_slots64(cudaStream_t st, const Geom& g, const double* in, d4* out) {
    Blocked B{g.n};
    STG_CK(cudaMemsetAsync(out, 0, sizeof(d4) * g.nslot, st));
    k_blocked_to_slots64<<<grid_for(B.size(), TPB), TPB, 0, st>>>(g, B, in, reinterpret_cast<double*>(out));
    STG_LAUNCH_CK();
    return STG_OK;
}

int slots_to_blocked64(cudaStream_t st, const Geom& g, const d4* in, double* out, const double* pad_src) {
    Blocked B{g.n};
    k_slots_to_blocked64<<<grid_for(B.size(), TPB), TPB, 0, st>>>(g, B, reinterpret_cast<const double*>(in), out, pad_src);
    STG_LAUNCH_CK();
    return STG_OK;
}

int mask_to_blocked(cudaStream_t st, const Geom& g, const uint8_t* m, uint8_t* out) {
    Blocked B{g.n};
    k_mask_to_blocked<<<grid_for(B.size(), TPB), TPB, 0, st>>>(g, B, m, out);
    STG_LAUNCH_CK();
    return STG_OK;
}

}  // namespace stg
