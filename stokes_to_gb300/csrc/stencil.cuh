// Device-side stencil of the reference Stokes operator A and energy operator E on the
// slot layout (internal.cuh).
//
// A = StokeFlowMapping3DFixed::applyMapping (stoke/StokeFlowMapping3D.cu:218-348):
//   Ap_f = -fix_f G fix_c D (V u) + V D1 Cod1 (fix_f u) - V G p + P u + F u
//   Ap_c =  fix_c D (V u) + P p + F p
// with D the face->cell divergence (common_cpx/grid3D.cu:330-397), G = Cod0 the
// cell->face difference c(x)-c(x-1) (:401-465), Cod1/D1 the face->edge->face curls
// (:469-578, :219-326), V the face vol, P the penalty and F the fixed mask.
// E = FluidEnergyGrad3D::applyMapping (fluid_topo/FluidEnergyGrad3D.cu:201-308) keeps
// the two viscous terms and P x only.
//
// Uniform-coefficient form: every free face carries the same vol value "vol" (fixed
// faces carry 0, as StokeFlowDescriptor3D::finish leaves them), so V u = vol * fix_f u.
// One thread evaluates all four rows of one slot from 13 slots: the 7-point
// neighbourhood plus the six edge-diagonal slots the curl and the divergence reach.
#pragma once
#include "internal.cuh"

namespace stg {

template <class T>
struct Vec4;
template <>
struct Vec4<float> {
    using type = float4;
};
template <>
struct Vec4<double> {
    using type = d4;
};

__device__ __forceinline__ void load4(const float4* a, int q, float& p, float& u, float& v, float& w) {
    float4 t = __ldg(a + q);
    p = t.x;
    u = t.y;
    v = t.z;
    w = t.w;
}
__device__ __forceinline__ void load4(const d4* a, int q, double& p, double& u, double& v, double& w) {
    const double2* b = reinterpret_cast<const double2*>(a + q);
    double2 t0 = __ldg(b), t1 = __ldg(b + 1);
    p = t0.x;
    u = t0.y;
    v = t1.x;
    w = t1.y;
}
__device__ __forceinline__ void store4(float4* a, int q, float p, float u, float v, float w) { a[q] = make_float4(p, u, v, w); }
__device__ __forceinline__ void store4(d4* a, int q, double p, double u, double v, double w) {
    double2* b = reinterpret_cast<double2*>(a + q);
    b[0] = make_double2(p, u);
    b[1] = make_double2(v, w);
}

// Masked unknowns of one slot: face values with fixed faces zeroed (fix_f u), the raw
// pressure, and whether the cell is free (fix_c).
template <class T>
struct Nb {
    T p, ux, uy, uz;
    bool mc;
};

template <class T, class V>
__device__ __forceinline__ Nb<T> nb_load(const V* x, const uint8_t* m, int q) {
    T p, u, v, w;
    load4(x, q, p, u, v, w);
    uint8_t mm = __ldg(m + q);
    Nb<T> r;
    r.p = p;
    r.ux = (mm & MU) ? T(0) : u;
    r.uy = (mm & MV) ? T(0) : v;
    r.uz = (mm & MW) ? T(0) : w;
    r.mc = !(mm & MP);
    return r;
}

// Viscous and pressure parts of A (or E when ENERGY) at one slot, without the diagonal
// P x + F x terms. ld(a, b, c) returns the masked unknowns of the slot at offset (a, b, c)
// along (i, j, k). out = {row p, row u, row v, row w}.
template <class T, bool ENERGY, class LD>
__device__ __forceinline__ void stencil_core(LD ld, T vol, uint8_t ms, T out[4]) {
    Nb<T> c0 = ld(0, 0, 0);
    Nb<T> xm = ld(-1, 0, 0), xp = ld(1, 0, 0);
    Nb<T> ym = ld(0, -1, 0), yp = ld(0, 1, 0);
    Nb<T> zm = ld(0, 0, -1), zp = ld(0, 0, 1);
    Nb<T> xp_ym = ld(1, -1, 0), xm_yp = ld(-1, 1, 0);
    Nb<T> xp_zm = ld(1, 0, -1), xm_zp = ld(-1, 0, 1);
    Nb<T> yp_zm = ld(0, 1, -1), ym_zp = ld(0, -1, 1);

    // fix_c D (V u) at the own cell and the three lower neighbours
    T dv0 = c0.mc ? vol * ((xp.ux - c0.ux) + (yp.uy - c0.uy) + (zp.uz - c0.uz)) : T(0);
    T dvx = xm.mc ? vol * ((c0.ux - xm.ux) + (xm_yp.uy - xm.uy) + (xm_zp.uz - xm.uz)) : T(0);
    T dvy = ym.mc ? vol * ((xp_ym.ux - ym.ux) + (c0.uy - ym.uy) + (ym_zp.uz - ym.uz)) : T(0);
    T dvz = zm.mc ? vol * ((xp_zm.ux - zm.ux) + (yp_zm.uy - zm.uy) + (c0.uz - zm.uz)) : T(0);

    // Cod1 edges (common_cpx/grid3D.cu:469-578) at the slot and its upper neighbours
    T ex0 = c0.uy - zm.uy - c0.uz + ym.uz;
    T exk = zp.uy - c0.uy - zp.uz + ym_zp.uz;
    T exj = yp.uy - yp_zm.uy - yp.uz + c0.uz;
    T ey0 = zm.ux - c0.ux + c0.uz - xm.uz;
    T eyk = c0.ux - zp.ux + zp.uz - xm_zp.uz;
    T eyi = xp_zm.ux - xp.ux + xp.uz - c0.uz;
    T ez0 = c0.ux - ym.ux + xm.uy - c0.uy;
    T ezj = yp.ux - c0.ux + xm_yp.uy - yp.uy;
    T ezi = xp.ux - xp_ym.ux + c0.uy - xp.uy;
    // D1 back to faces (common_cpx/grid3D.cu:219-326)
    T ccx = (eyk - ey0) + (ez0 - ezj);
    T ccy = (ex0 - exk) + (ezi - ez0);
    T ccz = (exj - ex0) + (ey0 - eyi);

    T gx = -(dv0 - dvx) + vol * ccx;
    T gy = -(dv0 - dvy) + vol * ccy;
    T gz = -(dv0 - dvz) + vol * ccz;
    if (!ENERGY) {
        gx -= vol * (c0.p - xm.p);
        gy -= vol * (c0.p - ym.p);
        gz -= vol * (c0.p - zm.p);
    }
    out[0] = ENERGY ? T(0) : dv0;
    out[1] = (ms & MU) ? T(0) : gx;
    out[2] = (ms & MV) ? T(0) : gy;
    out[3] = (ms & MW) ? T(0) : gz;
}

// General-coefficient form: every face carries its own vol (V u per face, V at the
// receiving face for the curl-curl and gradient terms), fixed faces carry vol 0 (as
// StokeFlowDescriptor3D::finish leaves them), cells may be fixed. The same 13 slots as
// stencil_core, each read with its three face vols.
template <class T>
struct NbV {
    T p, ux, uy, uz;     // p and the masked face values fix_f u
    T vux, vuy, vuz;     // V u of the three faces
    bool mc;
};

template <class T, class VV>
__device__ __forceinline__ NbV<T> nbv_load(const VV* x, const uint8_t* m, const VV* vol, int q) {
    T p, u, v, w, c, a, b, e;
    load4(x, q, p, u, v, w);
    load4(vol, q, c, a, b, e);
    uint8_t mm = __ldg(m + q);
    NbV<T> r;
    r.p = p;
    r.ux = (mm & MU) ? T(0) : u;
    r.uy = (mm & MV) ? T(0) : v;
    r.uz = (mm & MW) ? T(0) : w;
    r.vux = a * r.ux;
    r.vuy = b * r.uy;
    r.vuz = e * r.uz;
    r.mc = !(mm & MP);
    return r;
}

// A (or E) rows at slot s without the diagonal P x + F x terms; vx, vy, vz = the slot's face vols.
template <class T, bool ENERGY, class LD>
__device__ __forceinline__ void stencil_core_v(LD ld, T vx, T vy, T vz, uint8_t ms, T out[4]) {
    NbV<T> c0 = ld(0, 0, 0);
    NbV<T> xm = ld(-1, 0, 0), xp = ld(1, 0, 0);
    NbV<T> ym = ld(0, -1, 0), yp = ld(0, 1, 0);
    NbV<T> zm = ld(0, 0, -1), zp = ld(0, 0, 1);
    NbV<T> xp_ym = ld(1, -1, 0), xm_yp = ld(-1, 1, 0);
    NbV<T> xp_zm = ld(1, 0, -1), xm_zp = ld(-1, 0, 1);
    NbV<T> yp_zm = ld(0, 1, -1), ym_zp = ld(0, -1, 1);
    // fix_c D (V u) at the own cell and the three lower neighbours
    T dv0 = c0.mc ? ((xp.vux - c0.vux) + (yp.vuy - c0.vuy) + (zp.vuz - c0.vuz)) : T(0);
    T dvx = xm.mc ? ((c0.vux - xm.vux) + (xm_yp.vuy - xm.vuy) + (xm_zp.vuz - xm.vuz)) : T(0);
    T dvy = ym.mc ? ((xp_ym.vux - ym.vux) + (c0.vuy - ym.vuy) + (ym_zp.vuz - ym.vuz)) : T(0);
    T dvz = zm.mc ? ((xp_zm.vux - zm.vux) + (yp_zm.vuy - zm.vuy) + (c0.vuz - zm.vuz)) : T(0);
    // curl-curl of fix_f u, as in stencil_core
    T ex0 = c0.uy - zm.uy - c0.uz + ym.uz;
    T exk = zp.uy - c0.uy - zp.uz + ym_zp.uz;
    T exj = yp.uy - yp_zm.uy - yp.uz + c0.uz;
    T ey0 = zm.ux - c0.ux + c0.uz - xm.uz;
    T eyk = c0.ux - zp.ux + zp.uz - xm_zp.uz;
    T eyi = xp_zm.ux - xp.ux + xp.uz - c0.uz;
    T ez0 = c0.ux - ym.ux + xm.uy - c0.uy;
    T ezj = yp.ux - c0.ux + xm_yp.uy - yp.uy;
    T ezi = xp.ux - xp_ym.ux + c0.uy - xp.uy;
    T ccx = (eyk - ey0) + (ez0 - ezj);
    T ccy = (ex0 - exk) + (ezi - ez0);
    T ccz = (exj - ex0) + (ey0 - eyi);
    T gx = -(dv0 - dvx) + vx * ccx;
    T gy = -(dv0 - dvy) + vy * ccy;
    T gz = -(dv0 - dvz) + vz * ccz;
    if (!ENERGY) {
        gx -= vx * (c0.p - xm.p);
        gy -= vy * (c0.p - ym.p);
        gz -= vz * (c0.p - zm.p);
    }
    out[0] = ENERGY ? T(0) : dv0;
    out[1] = (ms & MU) ? T(0) : gx;
    out[2] = (ms & MV) ? T(0) : gy;
    out[3] = (ms & MW) ? T(0) : gz;
}

// Full rows of A x (or E x) at slot s in the general-coefficient form.
template <class T, bool ENERGY, class VV>
__device__ __forceinline__ void apply_rows_v(const VV* __restrict__ x, const uint8_t* __restrict__ m, const VV* __restrict__ P,
                                             const VV* __restrict__ vol, int s, int di, int dj, T out[4]) {
    const uint8_t ms = __ldg(m + s);
    T c, vx, vy, vz;
    load4(vol, s, c, vx, vy, vz);
    auto ld = [&](int a, int b, int e) { return nbv_load<T>(x, m, vol, s + a * di + b * dj + e); };
    stencil_core_v<T, ENERGY>(ld, vx, vy, vz, ms, out);
    T xp, xu, xv, xw, pp, pu, pv, pw;
    load4(x, s, xp, xu, xv, xw);
    load4(P, s, pp, pu, pv, pw);
    if (ENERGY) {
        out[0] += pp * xp;
        out[1] += pu * xu;
        out[2] += pv * xv;
        out[3] += pw * xw;
    } else {
        out[0] += (pp + ((ms & MP) ? T(1) : T(0))) * xp;
        out[1] += (pu + ((ms & MU) ? T(1) : T(0))) * xu;
        out[2] += (pv + ((ms & MV) ? T(1) : T(0))) * xv;
        out[3] += (pw + ((ms & MW) ? T(1) : T(0))) * xw;
    }
}

template <class T, bool ENERGY, class V>
__device__ __forceinline__ void stencil_rows(const V* __restrict__ x, const uint8_t* __restrict__ m, int s, int di, int dj,
                                             T vol, uint8_t ms, T out[4]) {
    auto ld = [&](int a, int b, int c) { return nb_load<T>(x, m, s + a * di + b * dj + c); };
    stencil_core<T, ENERGY>(ld, vol, ms, out);
}

template <class T>
__device__ __forceinline__ Nb<T> nb_make(T p, T u, T v, T w, uint8_t mm) {
    Nb<T> r;
    r.p = p;
    r.ux = (mm & MU) ? T(0) : u;
    r.uy = (mm & MV) ? T(0) : v;
    r.uz = (mm & MW) ? T(0) : w;
    r.mc = !(mm & MP);
    return r;
}

// ---------------------------------------------------------------- Laplacian form of A
// Applies when (1) the free faces share one vol value and no cell is fixed, (2) every
// face on the domain boundary is fixed, and (3) the vector is zero on every fixed or
// absent unknown. Then each free face lies between two present cells, fix_f u = u, and
// -fix_f G fix_c D (V u) + V D1 Cod1 (fix_f u) is exactly vol times the negative
// 7-point face Laplacian of u: the edge-diagonal terms of the two parts cancel
// identically (expanding ccx - (dv0 - dvx)/vol of stencil_core leaves
// 6 u - sum of the six x-face neighbours), so a row reads the slot and its six face
// neighbours. The rows of fixed and absent unknowns are masked by the caller (their
// reference value, (P + F) x = x, is 0 under (3)).
template <class T>
struct Q4 {
    T p, u, v, w;
};

template <class T>
__device__ __forceinline__ void lap_core(const Q4<T>& c, const Q4<T>& xm, const Q4<T>& xp, const Q4<T>& ym, const Q4<T>& yp,
                                         const Q4<T>& zm, const Q4<T>& zp, const Q4<T>& pen, T vol, T out[4]) {
    const T div = (xp.u - c.u) + (yp.v - c.v) + (zp.w - c.w);
    const T lu = T(6) * c.u - (xm.u + xp.u) - (ym.u + yp.u) - (zm.u + zp.u);
    const T lv = T(6) * c.v - (xm.v + xp.v) - (ym.v + yp.v) - (zm.v + zp.v);
    const T lw = T(6) * c.w - (xm.w + xp.w) - (ym.w + yp.w) - (zm.w + zp.w);
    out[0] = vol * div + pen.p * c.p;
    out[1] = vol * (lu - (c.p - xm.p)) + pen.u * c.u;
    out[2] = vol * (lv - (c.p - ym.p)) + pen.v * c.v;
    out[3] = vol * (lw - (c.p - zm.p)) + pen.w * c.w;
}

template <class T>
__device__ __forceinline__ void mask4(uint8_t ms, T o[4]) {
    if (ms & MP) o[0] = T(0);
    if (ms & MU) o[1] = T(0);
    if (ms & MV) o[2] = T(0);
    if (ms & MW) o[3] = T(0);
}

template <class T, class V>
__device__ __forceinline__ Q4<T> q4_load(const V* __restrict__ a, int s) {
    Q4<T> r;
    load4(a, s, r.p, r.u, r.v, r.w);
    return r;
}

// Unmasked Laplacian-form rows of A x at slot s (global-memory operands).
template <class T, class V>
__device__ __forceinline__ void lap_rows(const V* __restrict__ x, const V* __restrict__ P, int s, int di, int dj, T vol, T out[4]) {
    lap_core<T>(q4_load<T>(x, s), q4_load<T>(x, s - di), q4_load<T>(x, s + di), q4_load<T>(x, s - dj), q4_load<T>(x, s + dj),
                q4_load<T>(x, s - 1), q4_load<T>(x, s + 1), q4_load<T>(P, s), vol, out);
}

// Full row values: A x (ENERGY false) or E x (ENERGY true) at slot s.
template <class T, bool ENERGY, class V>
__device__ __forceinline__ void apply_rows(const V* __restrict__ x, const uint8_t* __restrict__ m, const V* __restrict__ P,
                                           int s, int di, int dj, T vol, T out[4]) {
    uint8_t ms = __ldg(m + s);
    stencil_rows<T, ENERGY>(x, m, s, di, dj, vol, ms, out);
    T xp, xu, xv, xw, pp, pu, pv, pw;
    load4(x, s, xp, xu, xv, xw);
    load4(P, s, pp, pu, pv, pw);
    if (ENERGY) {
        out[0] += pp * xp;
        out[1] += pu * xu;
        out[2] += pv * xv;
        out[3] += pw * xw;
    } else {
        out[0] += (pp + ((ms & MP) ? T(1) : T(0))) * xp;
        out[1] += (pu + ((ms & MU) ? T(1) : T(0))) * xu;
        out[2] += (pv + ((ms & MV) ? T(1) : T(0))) * xv;
        out[3] += (pw + ((ms & MW) ? T(1) : T(0))) * xw;
    }
}

}  // namespace stg
