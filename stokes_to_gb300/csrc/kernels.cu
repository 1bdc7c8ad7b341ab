// Grid kernels of the multigrid hierarchy: FP64/FP32 operator and residual, fused
// residual + restriction, prolongation, coarse re-discretisation and layout conversions.
// (The smoothing sweep lives in sweep.cu.)
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fp64bits.cuh"
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
// LAP: Laplacian form (stencil.cuh) for vectors zero on fixed unknowns; rows of fixed
// unknowns come out 0 (MODE 1: b - A x is 0 there as well, the fixed part of the
// solution being exactly b_f).
template <int MODE, bool LAP>
__global__ void __launch_bounds__(TPB) k_op64(Geom g, double vol, const d4* __restrict__ x, const uint8_t* __restrict__ m,
                                              const d4* __restrict__ P, const d4* __restrict__ b, d4* __restrict__ out,
                                              double* __restrict__ part) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    double acc = 0.0;
    if (t < g.box()) {
        int i, j, k;
        g.box_ijk(t, i, j, k);
        int s = g.slot(i, j, k);
        double o[4] = {0.0, 0.0, 0.0, 0.0};
        if (MODE == 3)
            ;  // x = 0
        else if (LAP)
            lap_rows<double>(x, P, s, g.di(), g.dj(), vol, o);
        else if (MODE == 2)
            apply_rows<double, true>(x, m, P, s, g.di(), g.dj(), vol, o);
        else
            apply_rows<double, false>(x, m, P, s, g.di(), g.dj(), vol, o);
        if (MODE == 1 || MODE == 3) {
            double bp, bu, bv, bw;
            load4(b, s, bp, bu, bv, bw);
            o[0] = bp - o[0];
            o[1] = bu - o[1];
            o[2] = bv - o[2];
            o[3] = bw - o[3];
        }
        if (LAP) mask4<double>(__ldg(m + s), o);
        if (MODE == 1 || MODE == 3) {
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

template <bool HAS_X, bool RESID, bool LAP>
__global__ void __launch_bounds__(TPB) k_op32(Geom g, float vol, const float4* __restrict__ r, const float4* __restrict__ x,
                                              const uint8_t* __restrict__ m, const float4* __restrict__ P,
                                              float4* __restrict__ out) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    int s = g.slot(i, j, k);
    float o[4] = {0.f, 0.f, 0.f, 0.f};
    if (HAS_X) {
        if (LAP)
            lap_rows<float>(x, P, s, g.di(), g.dj(), vol, o);
        else
            apply_rows<float, false>(x, m, P, s, g.di(), g.dj(), vol, o);
    }
    if (RESID) {
        float4 rv = __ldg(r + s);
        o[0] = rv.x - o[0];
        o[1] = rv.y - o[1];
        o[2] = rv.z - o[2];
        o[3] = rv.w - o[3];
    }
    if (LAP) mask4<float>(__ldg(m + s), o);
    out[s] = make_float4(o[0], o[1], o[2], o[3]);
}

// ------------------------------------------------------------------ transfers
// Restriction (stoke/StokeFlowSubSystem3D.cu:32-52 with common_cpx/SubsystemUtils3D.cuh:8-186):
// the coarse unknown of every kind at slot (I,J,K) sums the eight fine unknowns of the same
// kind at slots (2I+a, 2J+b, 2K+c), then fixed coarse unknowns are zeroed. Fused with the
// fine residual r - A x.
// One thread per fine slot: a 32 (k) x 8 (j) block covers the 16 x 4 coarse cells of one
// coarse plane I, each thread adds the residuals of its fine
// slot on planes 2I and 2I+1 (coalesced loads, neighbours through L1), and the 2 x 2 (j, k)
// children sums go through shared memory to the 64 writing threads.
template <bool HAS_X, bool LAP>
__global__ void __launch_bounds__(256) k_restrict_fine32(Geom gc, Geom gf, float volf, const float4* __restrict__ rf,
                                                         const float4* __restrict__ xf, const uint8_t* __restrict__ mf,
                                                         const float4* __restrict__ Pf, const uint8_t* __restrict__ mc,
                                                         float4* __restrict__ rc) {
    __shared__ float4 sv[8][32];
    const int tk = threadIdx.x, tj = threadIdx.y;
    const int k = blockIdx.x * 32 + tk, j = blockIdx.y * 8 + tj, I = blockIdx.z;
    const int nf = gf.n;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (j <= nf && k <= nf) {
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int i = 2 * I + q;
            if (i > nf) continue;
            const int s = gf.slot(i, j, k);
            float4 r = __ldg(rf + s);
            if (HAS_X) {
                float o[4];
                if (LAP) {
                    lap_rows<float>(xf, Pf, s, gf.di(), gf.dj(), volf, o);
                    o[0] = r.x - o[0];
                    o[1] = r.y - o[1];
                    o[2] = r.z - o[2];
                    o[3] = r.w - o[3];
                    mask4<float>(__ldg(mf + s), o);
                    r = make_float4(o[0], o[1], o[2], o[3]);
                } else {
                    apply_rows<float, false>(xf, mf, Pf, s, gf.di(), gf.dj(), volf, o);
                    r.x -= o[0];
                    r.y -= o[1];
                    r.z -= o[2];
                    r.w -= o[3];
                }
            }
            v.x += r.x;
            v.y += r.y;
            v.z += r.z;
            v.w += r.w;
        }
    }
    sv[tj][tk] = v;
    __syncthreads();
    const int t = tj * 32 + tk;
    if (t >= 64) return;
    const int cj = t >> 4, ck = t & 15;
    const int J = blockIdx.y * 4 + cj, K = blockIdx.x * 16 + ck;
    if (J > gc.n || K > gc.n) return;
    const float4 a = sv[2 * cj][2 * ck], b = sv[2 * cj][2 * ck + 1], c = sv[2 * cj + 1][2 * ck], d = sv[2 * cj + 1][2 * ck + 1];
    const int sc = gc.slot(I, J, K);
    const uint8_t mm = __ldg(mc + sc);
    rc[sc] = make_float4((mm & MP) ? 0.f : (a.x + b.x) + (c.x + d.x), (mm & MU) ? 0.f : (a.y + b.y) + (c.y + d.y),
                         (mm & MV) ? 0.f : (a.z + b.z) + (c.z + d.z), (mm & MW) ? 0.f : (a.w + b.w) + (c.w + d.w));
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

// Interpolated face value of component d (0 x, 1 y, 2 z) at fine slot (i, j, k): along the
// face normal the fine face lies on a coarse face (even index: weight 1) or midway between
// two (odd: 1/2 each); along each tangent the fine face centre lies a quarter of a coarse
// cell from the coarse face centre of the same parent and three quarters from the next one
// (weights 3/4 and 1/4). Coarse faces that are fixed, absent or in the halo hold zero.
template <class C>
__device__ __forceinline__ float face_interp(const C* xc, const Geom& gc, int d, int i, int j, int k) {
    const int f[3] = {i, j, k};
    int lo[3], hi[3];
    float wl[3], wh[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int c = f[a] >> 1, b = f[a] & 1;
        if (a == d) {
            lo[a] = c;
            hi[a] = c + 1;
            wl[a] = b ? 0.5f : 1.f;
            wh[a] = b ? 0.5f : 0.f;
        } else {
            lo[a] = c;
            hi[a] = b ? c + 1 : c - 1;
            wl[a] = 0.75f;
            wh[a] = 0.25f;
        }
    }
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int a0 = (q & 1) ? hi[0] : lo[0], a1 = (q & 2) ? hi[1] : lo[1], a2 = (q & 4) ? hi[2] : lo[2];
        const float w = ((q & 1) ? wh[0] : wl[0]) * ((q & 2) ? wh[1] : wl[1]) * ((q & 4) ? wh[2] : wl[2]);
        if (w == 0.f) continue;
        const float4 v = parent_value<C>(xc, gc.slot(a0, a1, a2));
        acc += w * (d == 0 ? v.y : d == 1 ? v.z : v.w);
    }
    return acc;
}

template <class C, bool LIN>
__global__ void __launch_bounds__(TPB) k_prolong_add32(Geom gf, Geom gc, const C* __restrict__ xc,
                                                       const uint8_t* __restrict__ mf, float4* __restrict__ xf) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= gf.box()) return;
    int i, j, k;
    gf.box_ijk(t, i, j, k);
    int s = gf.slot(i, j, k);
    float4 v = parent_value<C>(xc, gc.slot(i >> 1, j >> 1, k >> 1));
    if (LIN) {
        v.y = face_interp<C>(xc, gc, 0, i, j, k);
        v.z = face_interp<C>(xc, gc, 1, i, j, k);
        v.w = face_interp<C>(xc, gc, 2, i, j, k);
    }
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

// y = FP16(x / *scale) on the box slots (the sweeps' staged penalty copy)
__global__ void k_to_f16(Geom g, const float4* __restrict__ x, const float* __restrict__ scale, __half* __restrict__ y) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    int s = g.slot(i, j, k);
    const float4 v = __ldg(x + s);
    const float inv = 1.f / __ldg(scale);
    __half2* h = reinterpret_cast<__half2*>(y + 4ll * s);
    h[0] = __floats2half2_rn(v.x * inv, v.y * inv);
    h[1] = __floats2half2_rn(v.z * inv, v.w * inv);
}

// largest |x| over the box slots, as the bits of a non-negative float (atomicMax on them
// orders as the values do): a grid-stride pass, one atomic per block
__global__ void k_absmax(Geom g, const float4* __restrict__ x, unsigned* __restrict__ out) {
    __shared__ float sh[TPB / 32];
    float a = 0.f;
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < g.box(); t += (long long)gridDim.x * TPB) {
        int i, j, k;
        g.box_ijk(t, i, j, k);
        const float4 v = __ldg(x + g.slot(i, j, k));
        a = fmaxf(a, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
    }
    for (int o = 16; o > 0; o >>= 1) a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < TPB / 32; w++) a = fmaxf(a, sh[w]);
        atomicMax(out, __float_as_uint(a));
    }
}

// per-level FP16 scales: a power of two that brings the finest level's largest penalty to at
// most 2^15 (FP16 holds up to 65504), times 8 per level down (a coarse penalty is at most 8 x
// the largest of the finer level's)
__global__ void k_pscale(int nlev, const unsigned* __restrict__ maxbits, float* __restrict__ scale) {
    const float mx = __uint_as_float(*maxbits);
    float s = 1.f;
    while (s < 1e30f && mx > 32768.f * s) s *= 2.f;
    for (int l = nlev - 1; l >= 0; l--, s *= 8.f) scale[l] = s;
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
// FLOW (the solver's own hierarchy): a coarse velocity unknown takes 8 x the smallest
// penalty among its free children instead of the sum. The sum (the Galerkin penalty for
// piecewise-constant prolongation) closes every channel narrower than the coarse cell, so
// on optimised designs (solid 1e4, fluid ~0, channels a few cells wide) the coarse
// correction misses the flow and the restarted Krylov solve stagnates; the smallest penalty
// keeps the channel open and leaves the solid side to the smoother, whose blocks the large
// penalty makes diagonally dominant. The factor 8 keeps a uniform penalty's coarse value.
// On the 3D loop's iteration-5 design (fraction 0.15) the sum left the residual at 0.21
// (64^3) and 0.71 (128^3) after 600 V-cycles; the smallest penalty converges in 68 and 180.
// Harmonic and geometric means and a per-layer minimum (mean along the face normal) did no
// better; smooth (noise) densities take the same V-cycle count under every rule. The
// oracle restates the rule (oracle/oracle3d.cpp flow_penalties).
template <bool FLOW>
__global__ void k_coarsen(Geom gc, Geom gf, const uint8_t* __restrict__ mf, const d4* __restrict__ Pf, uint8_t* __restrict__ mc,
                          d4* __restrict__ Pc64, float4* __restrict__ Pc32) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= gc.box()) return;
    int I, J, K;
    gc.box_ijk(t, I, J, K);
    const int nf = gf.n;
    uint8_t mo = 0;
    double a[4] = {0, 0, 0, 0};
    double lo[3] = {INFINITY, INFINITY, INFINITY};  // FLOW: smallest free-child penalty (u, v, w)
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
        if (FLOW) {
            const uint8_t fr = (uint8_t)(present & ~mf[s]);
            if (fr & MU) lo[0] = fmin(lo[0], u);
            if (fr & MV) lo[1] = fmin(lo[1], v);
            if (fr & MW) lo[2] = fmin(lo[2], w);
        }
    }
    if (FLOW) {
#pragma unroll
        for (int d = 0; d < 3; d++)
            if (lo[d] < INFINITY) a[d + 1] = 8.0 * lo[d];
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

__global__ void k_fixed_nonzero(Geom g, const d4* __restrict__ x, const uint8_t* __restrict__ m, int* __restrict__ flag) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    int s = g.slot(i, j, k);
    uint8_t mm = __ldg(m + s);
    if (!mm) return;
    double p, u, v, w;
    load4(x, s, p, u, v, w);
    if (((mm & MP) && p != 0.0) || ((mm & MU) && u != 0.0) || ((mm & MV) && v != 0.0) || ((mm & MW) && w != 0.0))
        atomicOr(flag, 1);
}

__global__ void k_patch_fixed(Geom g, const d4* __restrict__ b, const uint8_t* __restrict__ m, d4* __restrict__ x) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    int s = g.slot(i, j, k);
    uint8_t mm = __ldg(m + s);
    if (!mm) return;
    double bp = 0, bu = 0, bv = 0, bw = 0, p, u, v, w;
    if (b) load4(b, s, bp, bu, bv, bw);
    load4(x, s, p, u, v, w);
    store4(x, s, (mm & MP) ? bp : p, (mm & MU) ? bu : u, (mm & MV) ? bv : v, (mm & MW) ? bw : w);
}

}  // namespace

// ------------------------------------------------------------------ launchers
int vol_slots(cudaStream_t st, const Geom& g, const uint8_t* m, double cell_vol, double vol, d4* out) {
    k_vol_slots<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, m, cell_vol, vol, out);
    STG_LAUNCH_CK();
    return STG_OK;
}

int fixed_nonzero(cudaStream_t st, const Geom& g, const d4* x, const uint8_t* m, int* flag) {
    STG_CK(cudaMemsetAsync(flag, 0, sizeof(int), st));
    k_fixed_nonzero<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, x, m, flag);
    STG_LAUNCH_CK();
    return STG_OK;
}

int zero_fixed(cudaStream_t st, const Geom& g, const uint8_t* m, d4* x) {
    k_patch_fixed<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, nullptr, m, x);
    STG_LAUNCH_CK();
    return STG_OK;
}

int patch_fixed(cudaStream_t st, const Geom& g, const d4* b, const uint8_t* m, d4* x) {
    k_patch_fixed<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, b, m, x);
    STG_LAUNCH_CK();
    return STG_OK;
}

// ------------------------------------------------------------------ double-float residual
// FP64 values as unevaluated sums hi + lo of two FP32 words (~46 significant bits). GB300
// executes FP64 arithmetic far slower than FP32, so the FP64 residual of the solver's
// refinement loop is evaluated in this arithmetic on double-float copies of x, b and the
// penalty, and only the result is formed in FP64.
struct F2 {
    float h, l;
};
__device__ __forceinline__ F2 f2(float h, float l) { return F2{h, l}; }
__device__ __forceinline__ F2 df_add(F2 a, F2 b) {
    const float s = a.h + b.h, bb = s - a.h;
    const float e = ((a.h - (s - bb)) + (b.h - bb)) + (a.l + b.l);
    const float h = s + e;
    return F2{h, e - (h - s)};
}
__device__ __forceinline__ F2 df_sub(F2 a, F2 b) { return df_add(a, F2{-b.h, -b.l}); }
__device__ __forceinline__ F2 df_mul(F2 a, F2 b) {
    const float p = a.h * b.h;
    const float e = fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p)));
    const float h = p + e;
    return F2{h, e - (h - p)};
}

// hi = fl32(a), lo = fl32(a - hi) componentwise (integer arithmetic, fp64bits.cuh); part
// (optional): per-block partials of |a|^2 from the FP32 squares of the hi words, summed in
// double-float arithmetic
__device__ __forceinline__ F2 warp_sum_f2(F2 v) {
    for (int o = 16; o > 0; o >>= 1) v = df_add(v, F2{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)});
    return v;
}

__global__ void __launch_bounds__(TPB) k_split64(long long n4, const d4* __restrict__ a, float4* __restrict__ hi,
                                                 float4* __restrict__ lo, double* __restrict__ part) {
    float acc = 0.f;
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < n4; t += (long long)gridDim.x * TPB) {
        double v[4];
        load4(a, (int)t, v[0], v[1], v[2], v[3]);
        float h[4], l[4];
#pragma unroll
        for (int c = 0; c < 4; c++) split_bits(v[c], h[c], l[c]);
        if (hi) hi[t] = make_float4(h[0], h[1], h[2], h[3]);
        lo[t] = make_float4(l[0], l[1], l[2], l[3]);
        acc += h[0] * h[0] + h[1] * h[1] + h[2] * h[2] + h[3] * h[3];
    }
    if (part) {
        __shared__ F2 sh[TPB / 32];
        const F2 v = warp_sum_f2(f2(acc, 0.f));
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            F2 b = sh[0];
            for (int w = 1; w < TPB / 32; w++) b = df_add(b, sh[w]);
            part[blockIdx.x] = f2d_bits(b.h) + f2d_bits(b.l);
        }
    }
}

// r = b - A x in the Laplacian form (rows of fixed unknowns 0, x zero on fixed unknowns),
// double-float arithmetic; HAS_X false: x = 0 (r = b). r in FP64 (r64), or rounded to FP32
// (r32, what the Krylov basis is built from). Per-block partials of |r|^2, summed in
// double-float arithmetic from the FP32 squares of the residual's high words.
template <bool HAS_X>
__global__ void __launch_bounds__(TPB) k_resid_df(Geom g, F2 vol, const float4* __restrict__ xh, const float4* __restrict__ xl,
                                                  const float4* __restrict__ bh, const float4* __restrict__ bl,
                                                  const float4* __restrict__ Ph, const float4* __restrict__ Pl,
                                                  const uint8_t* __restrict__ m, d4* __restrict__ r64, float4* __restrict__ r32,
                                                  double* __restrict__ part) {
    const long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    float acc = 0.f;
    if (t < g.box()) {
        int i, j, k;
        g.box_ijk(t, i, j, k);
        const int s = g.slot(i, j, k);
        const float4 b0 = __ldg(bh + s), b1 = __ldg(bl + s);
        const F2 bb[4] = {f2(b0.x, b1.x), f2(b0.y, b1.y), f2(b0.z, b1.z), f2(b0.w, b1.w)};
        F2 o[4] = {f2(0.f, 0.f), f2(0.f, 0.f), f2(0.f, 0.f), f2(0.f, 0.f)};
        if (HAS_X) {
            auto ld = [&](int q, F2 (&v)[4]) {
                const float4 a = __ldg(xh + q), b = __ldg(xl + q);
                v[0] = f2(a.x, b.x);
                v[1] = f2(a.y, b.y);
                v[2] = f2(a.z, b.z);
                v[3] = f2(a.w, b.w);
            };
            F2 c[4], xm[4], xp[4], ym[4], yp[4], zm[4], zp[4];
            ld(s, c);
            ld(s - g.di(), xm);
            ld(s + g.di(), xp);
            ld(s - g.dj(), ym);
            ld(s + g.dj(), yp);
            ld(s - 1, zm);
            ld(s + 1, zp);
            const float4 ph = __ldg(Ph + s), pl = __ldg(Pl + s);
            const F2 pen[4] = {f2(ph.x, pl.x), f2(ph.y, pl.y), f2(ph.z, pl.z), f2(ph.w, pl.w)};
            const F2 six = f2(6.f, 0.f);
            // the rows of stencil.cuh lap_core
            const F2 div = df_add(df_add(df_sub(xp[1], c[1]), df_sub(yp[2], c[2])), df_sub(zp[3], c[3]));
            o[0] = df_add(df_mul(vol, div), df_mul(pen[0], c[0]));
            const F2* lo_nb[3] = {xm, ym, zm};
#pragma unroll
            for (int d = 1; d <= 3; d++) {
                F2 l = df_mul(six, c[d]);
                l = df_sub(l, df_add(xm[d], xp[d]));
                l = df_sub(l, df_add(ym[d], yp[d]));
                l = df_sub(l, df_add(zm[d], zp[d]));
                const F2 gp = df_sub(c[0], lo_nb[d - 1][0]);
                o[d] = df_add(df_mul(vol, df_sub(l, gp)), df_mul(pen[d], c[d]));
            }
        }
        const uint8_t ms = __ldg(m + s);
        const uint8_t bit[4] = {MP, MU, MV, MW};
        F2 rd[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            rd[q] = (ms & bit[q]) ? f2(0.f, 0.f) : df_sub(bb[q], o[q]);
            acc += rd[q].h * rd[q].h;
        }
        if (r32) {
            r32[s] = make_float4(rd[0].h, rd[1].h, rd[2].h, rd[3].h);
        } else {
            double rv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) rv[q] = f2d_bits(rd[q].h) + f2d_bits(rd[q].l);
            store4(r64, s, rv[0], rv[1], rv[2], rv[3]);
        }
    }
    if (part) {
        __shared__ F2 sh[TPB / 32];
        const F2 v = warp_sum_f2(f2(acc, 0.f));
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            F2 b = sh[0];
            for (int w = 1; w < TPB / 32; w++) b = df_add(b, sh[w]);
            part[blockIdx.x] = f2d_bits(b.h) + f2d_bits(b.l);
        }
    }
}

// x = hi + lo in FP64 (one FP64 addition per element; the conversions by integer arithmetic)
__global__ void __launch_bounds__(TPB) k_df_to_f64(long long n4, const float4* __restrict__ hi, const float4* __restrict__ lo,
                                                   d4* __restrict__ x) {
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < n4; t += (long long)gridDim.x * TPB) {
        const float4 h = __ldg(hi + t), l = __ldg(lo + t);
        store4(x, (int)t, f2d_bits(h.x) + f2d_bits(l.x), f2d_bits(h.y) + f2d_bits(l.y), f2d_bits(h.z) + f2d_bits(l.z),
               f2d_bits(h.w) + f2d_bits(l.w));
    }
}

int split64(cudaStream_t st, long long n4, const d4* a, float4* hi, float4* lo, double* part, int* nblocks_out) {
    const unsigned nb = grid_for(n4, TPB) > 4096 ? 4096 : grid_for(n4, TPB);
    if (nblocks_out) *nblocks_out = (int)nb;
    k_split64<<<nb, TPB, 0, st>>>(n4, a, hi, lo, part);
    STG_LAUNCH_CK();
    return STG_OK;
}

int resid64_df(cudaStream_t st, const Geom& g, double vol, const float4* xh, const float4* xl, const float4* bh, const float4* bl,
               const float4* Ph, const float4* Pl, const uint8_t* m, d4* r, float4* r32, double* part, int* nblocks_out) {
    const unsigned nb = grid_for(g.box(), TPB);
    if (nblocks_out) *nblocks_out = (int)nb;
    const float vh = (float)vol;
    const F2 v2{vh, (float)(vol - (double)vh)};
    if (xh)
        k_resid_df<true><<<nb, TPB, 0, st>>>(g, v2, xh, xl, bh, bl, Ph, Pl, m, r, r32, part);
    else
        k_resid_df<false><<<nb, TPB, 0, st>>>(g, v2, xh, xl, bh, bl, Ph, Pl, m, r, r32, part);
    STG_LAUNCH_CK();
    return STG_OK;
}

int df_to_f64(cudaStream_t st, long long n4, const float4* hi, const float4* lo, d4* x) {
    const unsigned nb = grid_for(n4, TPB);
    k_df_to_f64<<<nb > 4096 ? 4096 : nb, TPB, 0, st>>>(n4, hi, lo, x);
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
         int mode, double* part, int* nblocks_out, bool lap) {
    unsigned nb = grid_for(g.box(), TPB);
    if (nblocks_out) *nblocks_out = (int)nb;
    if (mode == 0 && lap)
        k_op64<0, true><<<nb, TPB, 0, st>>>(g, vol, x, m, P, b, out, part);
    else if (mode == 0)
        k_op64<0, false><<<nb, TPB, 0, st>>>(g, vol, x, m, P, b, out, part);
    else if (mode == 1 && !x && lap)  // r = b with x = 0: no operator pass
        k_op64<3, true><<<nb, TPB, 0, st>>>(g, vol, x, m, P, b, out, part);
    else if (mode == 1 && !x)
        k_op64<3, false><<<nb, TPB, 0, st>>>(g, vol, x, m, P, b, out, part);
    else if (mode == 1 && lap)
        k_op64<1, true><<<nb, TPB, 0, st>>>(g, vol, x, m, P, b, out, part);
    else if (mode == 1)
        k_op64<1, false><<<nb, TPB, 0, st>>>(g, vol, x, m, P, b, out, part);
    else
        k_op64<2, false><<<nb, TPB, 0, st>>>(g, vol, x, m, P, b, out, part);
    STG_LAUNCH_CK();
    return STG_OK;
}

int resid32(cudaStream_t st, const Geom& g, float vol, const float4* r, const float4* x, const uint8_t* m, const float4* P,
            float4* rr, bool lap) {
    unsigned nb = grid_for(g.box(), TPB);
    if (x && lap)
        k_op32<true, true, true><<<nb, TPB, 0, st>>>(g, vol, r, x, m, P, rr);
    else if (x)
        k_op32<true, true, false><<<nb, TPB, 0, st>>>(g, vol, r, x, m, P, rr);
    else
        k_op32<false, true, false><<<nb, TPB, 0, st>>>(g, vol, r, x, m, P, rr);
    STG_LAUNCH_CK();
    return STG_OK;
}

int apply32(cudaStream_t st, const Geom& g, float vol, const float4* x, const uint8_t* m, const float4* P, float4* y, bool lap) {
    if (lap)
        k_op32<true, false, true><<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, vol, nullptr, x, m, P, y);
    else
        k_op32<true, false, false><<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, vol, nullptr, x, m, P, y);
    STG_LAUNCH_CK();
    return STG_OK;
}

int restrict_resid32(cudaStream_t st, const Geom& gc, const Geom& gf, float volf, const float4* rf, const float4* xf,
                     const uint8_t* mf, const float4* Pf, const uint8_t* mc, float4* rc, bool lap) {
    // fine box [0, nf]^3 in 32 x 8 (k, j) tiles, one coarse plane per z block
    const dim3 grid((gf.n + 1 + 31) / 32, (gf.n + 1 + 7) / 8, gc.n + 1), block(32, 8);
    if (xf && lap)
        k_restrict_fine32<true, true><<<grid, block, 0, st>>>(gc, gf, volf, rf, xf, mf, Pf, mc, rc);
    else if (xf)
        k_restrict_fine32<true, false><<<grid, block, 0, st>>>(gc, gf, volf, rf, xf, mf, Pf, mc, rc);
    else
        k_restrict_fine32<false, false><<<grid, block, 0, st>>>(gc, gf, volf, rf, xf, mf, Pf, mc, rc);
    STG_LAUNCH_CK();
    return STG_OK;
}

int prolong_add32(cudaStream_t st, const Geom& gf, const Geom& gc, const float4* xc, const uint8_t* mf, float4* xf,
                  bool linear) {
    if (linear)
        k_prolong_add32<float4, true><<<grid_for(gf.box(), TPB), TPB, 0, st>>>(gf, gc, xc, mf, xf);
    else
        k_prolong_add32<float4, false><<<grid_for(gf.box(), TPB), TPB, 0, st>>>(gf, gc, xc, mf, xf);
    STG_LAUNCH_CK();
    return STG_OK;
}

int prolong_add_bf16(cudaStream_t st, const Geom& gf, const Geom& gc, const __nv_bfloat16* xc, const uint8_t* mf, float4* xf,
                     bool linear) {
    if (linear)
        k_prolong_add32<__nv_bfloat16, true><<<grid_for(gf.box(), TPB), TPB, 0, st>>>(gf, gc, xc, mf, xf);
    else
        k_prolong_add32<__nv_bfloat16, false><<<grid_for(gf.box(), TPB), TPB, 0, st>>>(gf, gc, xc, mf, xf);
    STG_LAUNCH_CK();
    return STG_OK;
}

int to_f16(cudaStream_t st, const Geom& g, const float4* x, const float* scale, __half* y) {
    k_to_f16<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, x, scale, y);
    STG_LAUNCH_CK();
    return STG_OK;
}

int penalty_scales(cudaStream_t st, const Geom& fine, const float4* P, int nlev, unsigned* scratch, float* scale) {
    STG_CK(cudaMemsetAsync(scratch, 0, sizeof(unsigned), st));
    const unsigned nb = grid_for(fine.box(), TPB);
    k_absmax<<<nb > 1216 ? 1216 : nb, TPB, 0, st>>>(fine, P, scratch);
    STG_LAUNCH_CK();
    k_pscale<<<1, 1, 0, st>>>(nlev, scratch, scale);
    STG_LAUNCH_CK();
    return STG_OK;
}

int to_bf16(cudaStream_t st, const Geom& g, const float4* x, __nv_bfloat16* y) {
    k_to_bf16<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, x, y);
    STG_LAUNCH_CK();
    return STG_OK;
}

int coarsen(cudaStream_t st, const Geom& gc, const Geom& gf, const uint8_t* mf, const d4* Pf, uint8_t* mc, d4* Pc64,
            float4* Pc32, bool flow) {
    if (flow)
        k_coarsen<true><<<grid_for(gc.box(), TPB), TPB, 0, st>>>(gc, gf, mf, Pf, mc, Pc64, Pc32);
    else
        k_coarsen<false><<<grid_for(gc.box(), TPB), TPB, 0, st>>>(gc, gf, mf, Pf, mc, Pc64, Pc32);
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
