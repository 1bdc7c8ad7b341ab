// Vector kernels of the device-resident Krylov solver: precision conversion, batched
// dot products and updates for the Arnoldi step, and deterministic reductions (fixed
// grid, partials summed in a fixed order, so repeated runs are bitwise identical).
#include <cuda_fp16.h>

#include "kernels.h"
#include "stencil.cuh"

namespace stg {

namespace {

constexpr int TPB = 256;
constexpr int RGRID = 1216;  // 8 x 152 SMs: reduction grid
constexpr int MAXV = 16;     // vectors per multi-dot / projection pass

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int NV>
__device__ __forceinline__ void block_sums(double (&v)[NV], double* out) {
    __shared__ double sh[NV][TPB / 32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
        double s = warp_sum(v[q]);
        if (lane == 0) sh[q][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0;
        for (int w = 0; w < TPB / 32; w++) s += sh[threadIdx.x][w];
        out[threadIdx.x] = s;
    }
}

// Double-float sums (hi + lo, two FP32 words) for the reductions of the Krylov kernels:
// GB300's FP64 pipe retires about two operations per SM and cycle, so FP64 warp and block
// sums over the 1216-block grid cost tens of microseconds per launch, while the FP32 pipe
// does the same error-free sums (two-sum, the lo words carried) in a few.
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float s = a.x + b.x, bb = s - a.x;
    const float e = ((a.x - (s - bb)) + (b.x - bb)) + (a.y + b.y);
    const float hi = s + e;
    return make_float2(hi, e - (hi - s));
}
__device__ __forceinline__ float2 warp_sum_df(float2 v) {
    for (int o = 16; o > 0; o >>= 1)
        v = df_add(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)));
    return v;
}
// block partials of NV per-thread FP32 sums, as double-float pairs out[0..NV)
template <int NV>
__device__ __forceinline__ void block_sums_df(const float (&v)[NV], float2* out) {
    __shared__ float2 sh[NV][TPB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
        const float2 s = warp_sum_df(make_float2(v[q], 0.f));
        if (lane == 0) sh[q][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        float2 s = sh[threadIdx.x][0];
        for (int w = 1; w < TPB / 32; w++) s = df_add(s, sh[threadIdx.x][w]);
        out[threadIdx.x] = s;
    }
}

// FP16 copies of basis vectors (four halves per slot, the vector times its scale)
struct TabH {
    const uint2* p[MAXV];
};

__device__ __forceinline__ float4 h4_load(const uint2* a, long long t) {
    const uint2 v = __ldg(a + t);
    const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&v.x)), hi = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}
__device__ __forceinline__ uint2 h4_pack(float4 a, float s) {
    const __half2 lo = __floats2half2_rn(a.x * s, a.y * s), hi = __floats2half2_rn(a.z * s, a.w * s);
    return make_uint2(*reinterpret_cast<const unsigned*>(&lo), *reinterpret_cast<const unsigned*>(&hi));
}

// Scale of the FP16 copy of a vector whose squared norm is at most nrm2 over 4 n4 values:
// a quarter of the scale that brings its root mean square to 1, so that no element, even
// one holding the whole norm, exceeds sqrt(4 n4) / 4 (below FP16's 65504 up to 1024^3
// slots) while typical elements stay far above FP16's subnormal range.
__device__ __forceinline__ float h16_scale(long long n4, double nrm2) {
    return nrm2 > 0 ? (float)(0.25 * sqrt(4.0 * (double)n4 / nrm2)) : 1.f;
}

__global__ void k_f64_to_f32(long long n4, const double* __restrict__ a, double scale, float* __restrict__ out) {
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < 4 * n4; t += (long long)gridDim.x * TPB)
        out[t] = (float)(a[t] * scale);
}
// out = a * scale for a vector a of norm 1 / scale, with out's FP16 copy and that copy's
// scale (FP32 arithmetic only)
__global__ void k_scale_h16(long long n4, const float4* __restrict__ a, float scale, float4* __restrict__ out, uint2* __restrict__ out16,
                            float* __restrict__ sc_out) {
    __shared__ float hs_sh;
    if (threadIdx.x == 0) hs_sh = h16_scale(n4, 1.0);
    __syncthreads();
    const float hs = hs_sh;
    if (blockIdx.x == 0 && threadIdx.x == 0) *sc_out = hs;
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < n4; t += (long long)gridDim.x * TPB) {
        const float4 v = __ldg(a + t);
        const float4 o = make_float4(v.x * scale, v.y * scale, v.z * scale, v.w * scale);
        out[t] = o;
        out16[t] = h4_pack(o, hs);
    }
}
__global__ void k_f32_to_f64(long long n4, const float* __restrict__ a, double* __restrict__ out) {
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < 4 * n4; t += (long long)gridDim.x * TPB)
        out[t] = (double)a[t];
}

struct Tab {
    const float4* p[MAXV];
};

// Double-float accumulator (hi + lo, two FP32 words, ~46 significant bits): the products
// c z of an FP64 coefficient split as ch + cl and an FP32 value z are added exactly up to
// the lo words (ch z by its FMA remainder, cl z rounded in FP32, a term 2^-24 smaller).
struct DF {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add_prod(float ch, float cl, float z) {
        const float p = ch * z;
        const float pe = fmaf(ch, z, -p) + cl * z;
        const float t = hi + p;  // two-sum of hi and p
        const float bb = t - hi;
        const float e = (hi - (t - bb)) + (p - bb);
        hi = t;
        lo += e + pe;
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// x += sum_q (alpha y_q) z_q. The sum runs in double-float arithmetic, not FP64: an FP32
// sum of the basis loses the outer refinement step's accuracy to cancellation among the
// terms, and GB300's FP64 pipe is far slower than HBM for this stream. With x non-null the
// sum is added to the FP64 x (and, with xh / xl, x's double-float copy rewritten from it);
// with x null the double-float pair (xh, xl) is the iterate and takes the sum in
// double-float arithmetic, with no FP64 operation per element. The coefficients are split
// into FP32 pairs once per block. e (optional): the FP32 value of the sum over alpha is
// stored (first = true) or added; e may be one of the z_q, since each element is read
// before it is written.
template <int NV>
__global__ void __launch_bounds__(TPB) k_axpy_multi_32to64(long long n4, Tab z, const double* __restrict__ y, double alpha,
                                                           d4* __restrict__ x, float4* __restrict__ xh, float4* __restrict__ xl,
                                                           float4* e, bool first) {
    __shared__ float csh[2 * NV + 1];
    if (threadIdx.x < NV) {
        const double c = alpha * y[threadIdx.x];
        const float h = (float)c;
        csh[threadIdx.x] = h;
        csh[NV + threadIdx.x] = (float)(c - (double)h);
    }
    if (threadIdx.x == NV) csh[2 * NV] = (float)(1.0 / alpha);
    __syncthreads();
    float ch[NV], cl[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) {
        ch[q] = csh[q];
        cl[q] = csh[NV + q];
    }
    const float ia = csh[2 * NV];
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < n4; t += (long long)gridDim.x * TPB) {
        DF s0, s1, s2, s3;
#pragma unroll
        for (int q = 0; q < NV; q++) {
            const float4 v = __ldg(z.p[q] + t);
            s0.add_prod(ch[q], cl[q], v.x);
            s1.add_prod(ch[q], cl[q], v.y);
            s2.add_prod(ch[q], cl[q], v.z);
            s3.add_prod(ch[q], cl[q], v.w);
        }
        if (e) {
            float4 ev = make_float4((s0.hi + s0.lo) * ia, (s1.hi + s1.lo) * ia, (s2.hi + s2.lo) * ia, (s3.hi + s3.lo) * ia);
            if (!first) {
                const float4 o = e[t];
                ev.x += o.x;
                ev.y += o.y;
                ev.z += o.z;
                ev.w += o.w;
            }
            e[t] = ev;
        }
        if (!x) {
            const float4 h = xh[t], l = xl[t];
            const float2 a0 = df_add(make_float2(h.x, l.x), make_float2(s0.hi, s0.lo));
            const float2 a1 = df_add(make_float2(h.y, l.y), make_float2(s1.hi, s1.lo));
            const float2 a2 = df_add(make_float2(h.z, l.z), make_float2(s2.hi, s2.lo));
            const float2 a3 = df_add(make_float2(h.w, l.w), make_float2(s3.hi, s3.lo));
            xh[t] = make_float4(a0.x, a1.x, a2.x, a3.x);
            xl[t] = make_float4(a0.y, a1.y, a2.y, a3.y);
            continue;
        }
        double2* xp = reinterpret_cast<double2*>(x + t);
        double2 a = xp[0], b = xp[1];
        a.x += s0.value();
        a.y += s1.value();
        b.x += s2.value();
        b.y += s3.value();
        xp[0] = a;
        xp[1] = b;
        if (xh) {
            const float4 hv = make_float4((float)a.x, (float)a.y, (float)b.x, (float)b.y);
            xh[t] = hv;
            xl[t] = make_float4((float)(a.x - (double)hv.x), (float)(a.y - (double)hv.y), (float)(b.x - (double)hv.z),
                                (float)(b.y - (double)hv.w));
        }
    }
}

// Per-thread partial sums are FP32 (a thread covers a few hundred products; GB300's FP64
// pipe cannot keep up with HBM for these streams); block and grid sums are double-float.
// With WW the pass also returns <w, w> in column NV.
template <int NV, bool WW>
__global__ void __launch_bounds__(TPB) k_multidot32(long long n4, Tab v, const float4* __restrict__ w, float2* __restrict__ part) {
    float acc[NV + 1];
#pragma unroll
    for (int q = 0; q <= NV; q++) acc[q] = 0.f;
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < n4; t += (long long)gridDim.x * TPB) {
        float4 a = __ldg(w + t);
#pragma unroll
        for (int q = 0; q < NV; q++) {
            float4 b = __ldg(v.p[q] + t);
            acc[q] += a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
        }
        if (WW) acc[NV] += a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w;
    }
    block_sums_df<NV + 1>(acc, part + (long long)blockIdx.x * (MAXV + 1));
}

// The FGMRES operator fused with the first multi-dot of the Arnoldi step, in the
// Laplacian form: w = v - A z over the box slots (rows of fixed unknowns 0), written out,
// and per-block partials of <V_q, w> and <w, w> (w never re-read from memory for them).
// H16: the dots read the basis vectors' FP16 copies (half the bytes) and are scaled back by
// 1/sc[q]; the products still accumulate in FP32. The dots only set the projection
// coefficients: the projection itself subtracts the FP32 vectors, so the Arnoldi relation
// A z_j = v_j - w holds as in FP32, and a dot's rounding (a few 1e-4 of |V_q| |w| at
// worst, far less for rounding errors uncorrelated with w) perturbs only the orthogonality
// of the new vector, which the second projection's dots (FP32) measure.
template <int NV, bool H16>
__global__ void __launch_bounds__(TPB) k_shift_dots(Geom g, float vol, const float4* __restrict__ v, const float4* __restrict__ z,
                                                    const uint8_t* __restrict__ m, const float4* __restrict__ P, Tab V, TabH VH,
                                                    const float* __restrict__ sc, float4* __restrict__ w, float2* __restrict__ part) {
    float acc[NV + 1];
#pragma unroll
    for (int q = 0; q <= NV; q++) acc[q] = 0.f;
    const long long nb = g.box();
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < nb; t += (long long)gridDim.x * TPB) {
        int i, j, k;
        g.box_ijk(t, i, j, k);
        const int s = g.slot(i, j, k);
        float o[4];
        lap_rows<float>(z, P, s, g.di(), g.dj(), vol, o);
        const float4 vv = __ldg(v + s);
        o[0] = vv.x - o[0];
        o[1] = vv.y - o[1];
        o[2] = vv.z - o[2];
        o[3] = vv.w - o[3];
        mask4<float>(__ldg(m + s), o);
        const float4 a = make_float4(o[0], o[1], o[2], o[3]);
        w[s] = a;
#pragma unroll
        for (int q = 0; q < NV; q++) {
            const float4 b = H16 ? h4_load(VH.p[q], s) : __ldg(V.p[q] + s);
            acc[q] += a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
        }
        acc[NV] += a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w;
    }
    if (H16) {
#pragma unroll
        for (int q = 0; q < NV; q++) acc[q] *= __frcp_rn(__ldg(sc + q));
    }
    block_sums_df<NV + 1>(acc, part + (long long)blockIdx.x * (MAXV + 1));
}

// w -= sum_q h[q] v_q ; partial ||w||^2 per block (computed after the update)
template <int NV>
__global__ void __launch_bounds__(TPB) k_multiaxpy32(long long n4, Tab v, const double* __restrict__ h, float4* __restrict__ w,
                                                     float2* __restrict__ part, int want_norm) {
    float c[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) c[q] = (float)h[q];
    float accf = 0.f;
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < n4; t += (long long)gridDim.x * TPB) {
        float4 a = w[t];
#pragma unroll
        for (int q = 0; q < NV; q++) {
            float4 b = __ldg(v.p[q] + t);
            a.x -= c[q] * b.x;
            a.y -= c[q] * b.y;
            a.z -= c[q] * b.z;
            a.w -= c[q] * b.w;
        }
        w[t] = a;
        if (want_norm) accf += a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w;
    }
    const float acc[1] = {accf};
    if (want_norm) block_sums_df<1>(acc, part + blockIdx.x);
}

// Projection step of classical Gram-Schmidt on unnormalised basis vectors:
// out = w - sum_q c_q v_q with c_q = sig2[q] * d[q] (d: the dot products <v_q, w> of the
// previous pass, sig2[q] = 1/||v_q||^2), in one pass. DOTS: the same pass also returns
// the dot products <v_q, out> (the re-orthogonalisation coefficients; the v_q are still
// in registers) and <out, out> in column NV. out may alias w.
// out16 (optional): the FP16 copy of out, scaled by h16_scale of nest (an upper estimate of
// ||out||^2 read from the device), the scale stored to *sc_out.
template <int NV, bool DOTS>
__global__ void __launch_bounds__(TPB) k_proj32(long long n4, Tab v, const double* __restrict__ d, const double* __restrict__ sig2,
                                                const float4* w, float4* out, float2* __restrict__ part, uint2* __restrict__ out16,
                                                const double* __restrict__ nest, float* __restrict__ sc_out) {
    // the coefficients and the FP16 scale in FP64 once per block (FP64 is slow on GB300)
    __shared__ float csh[NV + 1];
    if (threadIdx.x < NV) csh[threadIdx.x] = (float)(sig2[threadIdx.x] * d[threadIdx.x]);
    if (threadIdx.x == NV) csh[NV] = out16 ? h16_scale(n4, *nest) : 0.f;
    __syncthreads();
    const float hs = csh[NV];
    if (out16 && blockIdx.x == 0 && threadIdx.x == 0) *sc_out = hs;
    float c[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) c[q] = csh[q];
    float acc[NV + 1];
#pragma unroll
    for (int q = 0; q <= NV; q++) acc[q] = 0.f;
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < n4; t += (long long)gridDim.x * TPB) {
        float4 a = w[t];
        float4 b[NV];
#pragma unroll
        for (int q = 0; q < NV; q++) {
            b[q] = __ldg(v.p[q] + t);
            a.x -= c[q] * b[q].x;
            a.y -= c[q] * b[q].y;
            a.z -= c[q] * b[q].z;
            a.w -= c[q] * b[q].w;
        }
        out[t] = a;
        if (out16) out16[t] = h4_pack(a, hs);
        if (DOTS) {
#pragma unroll
            for (int q = 0; q < NV; q++) acc[q] += a.x * b[q].x + a.y * b[q].y + a.z * b[q].z + a.w * b[q].w;
        }
        acc[NV] += a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w;
    }
    block_sums_df<NV + 1>(acc, part + (long long)blockIdx.x * (MAXV + 1));
}

// sc (optional): the scale of x's FP16 copy, which keeps representing the scaled vector
__global__ void k_scale32(long long n4, const float4* __restrict__ x, const double* __restrict__ nrm2, float4* __restrict__ out,
                          float* __restrict__ sc) {
    double s0 = *nrm2;
    float s = s0 > 0 ? (float)(1.0 / sqrt(s0)) : 0.f;
    if (sc && s0 > 0 && blockIdx.x == 0 && threadIdx.x == 0) *sc = (float)((double)*sc * sqrt(s0));
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < n4; t += (long long)gridDim.x * TPB) {
        float4 a = __ldg(x + t);
        out[t] = make_float4(a.x * s, a.y * s, a.z * s, a.w * s);
    }
}

// Sums column q of a [nparts][stride] partial table in a fixed order.
__global__ void k_reduce_cols(const double* __restrict__ part, int nparts, int stride, int ncols, double* __restrict__ out) {
    __shared__ double sh[TPB / 32];
    for (int q = 0; q < ncols; q++) {
        double s = 0;
        for (int p = threadIdx.x; p < nparts; p += TPB) s += part[(long long)p * stride + q];
        s = warp_sum(s);
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 0) sh[wid] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double r = 0;
            for (int w = 0; w < TPB / 32; w++) r += sh[w];
            out[q] = r;
        }
        __syncthreads();
    }
}

// Sums column q of a [nparts][stride] table of double-float partials in a fixed order, one
// warp per column (no block barriers): columns 0 .. ncols-2 go to out[q], the last to
// *out_last (or to out[ncols-1] when out_last is null).
__global__ void k_reduce_cols_df(const float2* __restrict__ part, int nparts, int stride, int ncols, double* __restrict__ out,
                                 double* __restrict__ out_last) {
    const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (q >= ncols) return;
    float2 s = make_float2(0.f, 0.f);
    for (int p = lane; p < nparts; p += 32) s = df_add(s, part[(long long)p * stride + q]);
    s = warp_sum_df(s);
    if (lane == 0) {
        double* dst = (out_last && q == ncols - 1) ? out_last : out + q;
        *dst = (double)s.x + (double)s.y;
    }
}

__global__ void __launch_bounds__(TPB) k_dot64(long long n4, const d4* __restrict__ a, const d4* __restrict__ b,
                                               double* __restrict__ part) {
    double acc[1] = {0.0};
    const double* x = reinterpret_cast<const double*>(a);
    const double* y = reinterpret_cast<const double*>(b);
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < 4 * n4; t += (long long)gridDim.x * TPB)
        acc[0] += x[t] * y[t];
    block_sums<1>(acc, part + blockIdx.x);
}

unsigned rgrid(long long work) {
    long long g = (work + TPB - 1) / TPB;
    return (unsigned)(g < 1 ? 1 : (g > RGRID ? RGRID : g));
}

}  // namespace

int fill_bytes(cudaStream_t st, void* p, size_t bytes) {
    STG_CK(cudaMemsetAsync(p, 0, bytes, st));
    return STG_OK;
}

int f64_to_f32(cudaStream_t st, long long n4, const d4* a, double scale, float4* out) {
    k_f64_to_f32<<<rgrid(4 * n4), TPB, 0, st>>>(n4, reinterpret_cast<const double*>(a), scale, reinterpret_cast<float*>(out));
    STG_LAUNCH_CK();
    return STG_OK;
}

int scale_h16(cudaStream_t st, long long n4, const float4* a, float scale, float4* out, uint2* out16, float* sc_out) {
    k_scale_h16<<<rgrid(n4), TPB, 0, st>>>(n4, a, scale, out, out16, sc_out);
    STG_LAUNCH_CK();
    return STG_OK;
}

int f32_to_f64(cudaStream_t st, long long n4, const float4* a, d4* out) {
    k_f32_to_f64<<<rgrid(4 * n4), TPB, 0, st>>>(n4, reinterpret_cast<const float*>(a), reinterpret_cast<double*>(out));
    STG_LAUNCH_CK();
    return STG_OK;
}

// column sums of a table of double-float partials (the Krylov kernels' scratch, 8 bytes an entry)
static void rcols_df(cudaStream_t st, const double* scratch, int nparts, int stride, int ncols, double* out, double* out_last = nullptr) {
    k_reduce_cols_df<<<1, 32 * ncols, 0, st>>>(reinterpret_cast<const float2*>(scratch), nparts, stride, ncols, out, out_last);
}

int reduce_parts(cudaStream_t st, const double* parts, int nparts, double* out) {
    k_reduce_cols<<<1, TPB, 0, st>>>(parts, nparts, 1, 1, out);
    STG_LAUNCH_CK();
    return STG_OK;
}

// Calls K<NV>::run(args...) with NV = nb in [1, MAXV].
template <template <int> class K, class... A>
static void dispatch_nv(int nb, A&&... args) {
    switch (nb) {
        case 1: K<1>::run(args...); break;
        case 2: K<2>::run(args...); break;
        case 3: K<3>::run(args...); break;
        case 4: K<4>::run(args...); break;
        case 5: K<5>::run(args...); break;
        case 6: K<6>::run(args...); break;
        case 7: K<7>::run(args...); break;
        case 8: K<8>::run(args...); break;
        case 9: K<9>::run(args...); break;
        case 10: K<10>::run(args...); break;
        case 11: K<11>::run(args...); break;
        case 12: K<12>::run(args...); break;
        case 13: K<13>::run(args...); break;
        case 14: K<14>::run(args...); break;
        case 15: K<15>::run(args...); break;
        default: K<16>::run(args...); break;
    }
}

template <int NV>
struct AxpyL {
    static void run(cudaStream_t st, long long n4, const Tab& t, const double* y, double alpha, d4* x, float4* xh, float4* xl,
                    float4* e, bool first) {
        k_axpy_multi_32to64<NV><<<rgrid(n4), TPB, 0, st>>>(n4, t, y, alpha, x, xh, xl, e, first);
    }
};
template <int NV>
struct DotL {
    static void run(cudaStream_t st, long long n4, const Tab& t, const float4* w, double* part, bool ww) {
        if (ww)
            k_multidot32<NV, true><<<rgrid(n4), TPB, 0, st>>>(n4, t, w, reinterpret_cast<float2*>(part));
        else
            k_multidot32<NV, false><<<rgrid(n4), TPB, 0, st>>>(n4, t, w, reinterpret_cast<float2*>(part));
    }
};
template <int NV>
struct ProjL {
    static void run(cudaStream_t st, long long n4, const Tab& t, const double* d, const double* sig2, const float4* w, float4* out,
                    double* part, bool dots, uint2* out16, const double* nest, float* sc_out) {
        if (dots)
            k_proj32<NV, true><<<rgrid(n4), TPB, 0, st>>>(n4, t, d, sig2, w, out, reinterpret_cast<float2*>(part), out16, nest, sc_out);
        else
            k_proj32<NV, false><<<rgrid(n4), TPB, 0, st>>>(n4, t, d, sig2, w, out, reinterpret_cast<float2*>(part), out16, nest, sc_out);
    }
};

int axpy_last_chunk(int nz) { return nz > 0 ? ((nz - 1) / MAXV) * MAXV : 0; }

// Chunks of MAXV vectors from the last one down: e (when one of the z_q, a slot at the end
// of the basis) is written by the first chunk, which holds it, and only added to by the
// later ones; the double-float copy of x is written by the last chunk.
int axpy_multi_32to64(cudaStream_t st, long long n4, const float4* const* z, const double* y, int nz, double alpha, d4* x,
                      float4* xh, float4* xl, float4* e) {
    if (!x && (!xh || !xl)) {
        set_error("axpy_multi_32to64: no iterate");
        return STG_E_INVALID;
    }
    const int nchunk = (nz + MAXV - 1) / MAXV;
    for (int c = nchunk - 1; c >= 0; c--) {
        const int j0 = c * MAXV;
        int nb = nz - j0 < MAXV ? nz - j0 : MAXV;
        Tab t{};
        for (int q = 0; q < nb; q++) t.p[q] = z[j0 + q];
        const bool upd = c == 0 || !x;  // the copy is written by the last chunk, the pair iterate by every one
        dispatch_nv<AxpyL>(nb, st, n4, t, y + j0, alpha, x, upd ? xh : nullptr, upd ? xl : nullptr, e, c == nchunk - 1);
        STG_LAUNCH_CK();
    }
    return STG_OK;
}

template <int NV>
struct ShiftL {
    static void run(cudaStream_t st, const Geom& g, float vol, const float4* v, const float4* z, const uint8_t* m, const float4* P,
                    const Tab& t, const TabH& th, const float* sc, float4* w, double* part) {
        if (sc)
            k_shift_dots<NV, true><<<RGRID, TPB, 0, st>>>(g, vol, v, z, m, P, t, th, sc, w, reinterpret_cast<float2*>(part));
        else
            k_shift_dots<NV, false><<<RGRID, TPB, 0, st>>>(g, vol, v, z, m, P, t, th, sc, w, reinterpret_cast<float2*>(part));
    }
};

int shift_multidot32(cudaStream_t st, const Geom& g, float vol, const float4* v, const float4* z, const uint8_t* m, const float4* P,
                     long long n4, const float4* const* V, int nv, float4* w, double* h, double* scratch, double* ww,
                     const uint2* const* V16, const float* sc) {
    const int nb = nv < MAXV ? nv : MAXV;
    Tab t{};
    TabH th{};
    for (int q = 0; q < nb; q++) {
        t.p[q] = V[q];
        th.p[q] = V16 ? V16[q] : nullptr;
    }
    dispatch_nv<ShiftL>(nb, st, g, vol, v, z, m, P, t, th, V16 ? sc : nullptr, w, scratch);
    STG_LAUNCH_CK();
    rcols_df(st, scratch, RGRID, MAXV + 1, nb + 1, h, ww);  // the dots, and <w, w> in column nb
    STG_LAUNCH_CK();
    // basis vectors past the first MAXV: a plain multi-dot pass over the written w
    if (nv > MAXV) STG_TRY(multidot32(st, n4, V + MAXV, nv - MAXV, w, h + MAXV, scratch, nullptr));
    return STG_OK;
}

int multidot32(cudaStream_t st, long long n4, const float4* const* v, int nv, const float4* w, double* h, double* scratch,
               double* ww) {
    unsigned g = rgrid(n4);
    for (int j0 = 0; j0 < nv; j0 += MAXV) {
        int nb = nv - j0 < MAXV ? nv - j0 : MAXV;
        bool want_ww = ww && j0 == 0;
        Tab t{};
        for (int q = 0; q < nb; q++) t.p[q] = v[j0 + q];
        dispatch_nv<DotL>(nb, st, n4, t, w, scratch, want_ww);
        STG_LAUNCH_CK();
        rcols_df(st, scratch, (int)g, MAXV + 1, want_ww ? nb + 1 : nb, h + j0, want_ww ? ww : nullptr);
        STG_LAUNCH_CK();
    }
    return STG_OK;
}

template <int NV>
struct MaxpyL {
    static void run(cudaStream_t st, long long n4, const Tab& t, const double* h, float4* w, double* part, int want) {
        k_multiaxpy32<NV><<<rgrid(n4), TPB, 0, st>>>(n4, t, h, w, reinterpret_cast<float2*>(part), want);
    }
};

int multiaxpy32_norm(cudaStream_t st, long long n4, const float4* const* v, int nv, const double* h, float4* w, double* nrm2,
                     double* scratch) {
    if (nv < 1) {
        set_error("multiaxpy32_norm: empty basis");
        return STG_E_INVALID;
    }
    unsigned g = rgrid(n4);
    for (int j0 = 0; j0 < nv; j0 += MAXV) {
        int nb = nv - j0 < MAXV ? nv - j0 : MAXV;
        int last = j0 + nb >= nv;
        Tab t{};
        for (int q = 0; q < nb; q++) t.p[q] = v[j0 + q];
        dispatch_nv<MaxpyL>(nb, st, n4, t, h + j0, w, scratch, last);
        STG_LAUNCH_CK();
    }
    rcols_df(st, scratch, (int)g, 1, 1, nrm2);
    STG_LAUNCH_CK();
    return STG_OK;
}

int project32(cudaStream_t st, long long n4, const float4* const* v, int nv, const double* d, const double* sig2, const float4* w,
              float4* out, double* dots, double* nrm2, double* scratch, uint2* out16, const double* nest, float* sc_out) {
    if (nv < 1) {
        set_error("project32: empty basis");
        return STG_E_INVALID;
    }
    unsigned g = rgrid(n4);
    if (nv <= MAXV) {
        Tab t{};
        for (int q = 0; q < nv; q++) t.p[q] = v[q];
        dispatch_nv<ProjL>(nv, st, n4, t, d, sig2, w, out, scratch, dots != nullptr, out16, nest, sc_out);
        STG_LAUNCH_CK();
        if (dots)
            rcols_df(st, scratch, (int)g, MAXV + 1, nv + 1, dots, nrm2);  // the dots, and |out|^2 in column nv
        else
            rcols_df(st, scratch + nv, (int)g, MAXV + 1, 1, nrm2);
        STG_LAUNCH_CK();
        return STG_OK;
    }
    // more vectors than one pass holds: subtract in chunks, then a separate dot pass
    for (int j0 = 0; j0 < nv; j0 += MAXV) {
        int nb = nv - j0 < MAXV ? nv - j0 : MAXV;
        Tab t{};
        for (int q = 0; q < nb; q++) t.p[q] = v[j0 + q];
        const bool last = j0 + nb >= nv;  // the last chunk writes the FP16 copy
        dispatch_nv<ProjL>(nb, st, n4, t, d + j0, sig2 + j0, j0 == 0 ? w : out, out, scratch, false, last ? out16 : nullptr, nest,
                           sc_out);
        STG_LAUNCH_CK();
    }
    if (dots) return multidot32(st, n4, v, nv, out, dots, scratch, nrm2);
    rcols_df(st, scratch + (nv - ((nv - 1) / MAXV) * MAXV), (int)g, MAXV + 1, 1, nrm2);
    STG_LAUNCH_CK();
    return STG_OK;
}

int scale32(cudaStream_t st, long long n4, float4* x, const double* nrm2, float4* out, float* sc) {
    k_scale32<<<rgrid(n4), TPB, 0, st>>>(n4, x, nrm2, out, sc);
    STG_LAUNCH_CK();
    return STG_OK;
}

int dot64(cudaStream_t st, long long n4, const d4* a, const d4* b, double* out, double* scratch) {
    unsigned g = rgrid(4 * n4);
    k_dot64<<<g, TPB, 0, st>>>(n4, a, b, scratch);
    STG_LAUNCH_CK();
    k_reduce_cols<<<1, TPB, 0, st>>>(scratch, (int)g, 1, 1, out);
    STG_LAUNCH_CK();
    return STG_OK;
}

}  // namespace stg
