// Vector kernels of the device-resident Krylov solver: precision conversion, batched
// dot products and updates for the Arnoldi step, and deterministic reductions (fixed
// grid, partials summed in a fixed order, so repeated runs are bitwise identical).
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

__global__ void k_f64_to_f32(long long n4, const double* __restrict__ a, double scale, float* __restrict__ out) {
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < 4 * n4; t += (long long)gridDim.x * TPB)
        out[t] = (float)(a[t] * scale);
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

// x64 += sum_q (alpha y_q) z_q. The sum runs in double-float arithmetic, not FP64: an FP32
// sum of the basis loses the outer refinement step's accuracy to cancellation among the
// terms, and GB300's FP64 pipe is far slower than HBM for this stream; only the final
// addition to x is FP64. e (optional): the FP32 value of the sum over alpha is stored
// (first = true) or added; e may be one of the z_q, since each element is read before it is
// written.
template <int NV>
__global__ void __launch_bounds__(TPB) k_axpy_multi_32to64(long long n4, Tab z, const double* __restrict__ y, double alpha,
                                                           d4* __restrict__ x, float4* __restrict__ xh, float4* __restrict__ xl,
                                                           float4* e, bool first) {
    float ch[NV], cl[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) {
        const double c = alpha * y[q];
        ch[q] = (float)c;
        cl[q] = (float)(c - (double)ch[q]);
    }
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
        double2* xp = reinterpret_cast<double2*>(x + t);
        double2 a = xp[0], b = xp[1];
        const double d0 = s0.value(), d1 = s1.value(), d2 = s2.value(), d3 = s3.value();
        a.x += d0;
        a.y += d1;
        b.x += d2;
        b.y += d3;
        xp[0] = a;
        xp[1] = b;
        if (e) {
            const double ia = 1.0 / alpha;
            float4 ev = make_float4((float)(d0 * ia), (float)(d1 * ia), (float)(d2 * ia), (float)(d3 * ia));
            if (!first) {
                const float4 o = e[t];
                ev.x += o.x;
                ev.y += o.y;
                ev.z += o.z;
                ev.w += o.w;
            }
            e[t] = ev;
        }
        if (xh) {
            const float4 hv = make_float4((float)a.x, (float)a.y, (float)b.x, (float)b.y);
            xh[t] = hv;
            xl[t] = make_float4((float)(a.x - (double)hv.x), (float)(a.y - (double)hv.y), (float)(b.x - (double)hv.z),
                                (float)(b.y - (double)hv.w));
        }
    }
}

// Per-thread partial sums are FP32 (a thread covers a few hundred products; GB300's FP64
// pipe cannot keep up with HBM for these streams); block and grid sums are FP64.
// With WW the pass also returns <w, w> in column NV.
template <int NV, bool WW>
__global__ void __launch_bounds__(TPB) k_multidot32(long long n4, Tab v, const float4* __restrict__ w, double* __restrict__ part) {
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
    double d[NV + 1];
#pragma unroll
    for (int q = 0; q <= NV; q++) d[q] = acc[q];
    block_sums<NV + 1>(d, part + (long long)blockIdx.x * (MAXV + 1));
}

// The FGMRES operator fused with the first multi-dot of the Arnoldi step, in the
// Laplacian form: w = v - A z over the box slots (rows of fixed unknowns 0), written out,
// and per-block partials of <V_q, w> and <w, w> (w never re-read from memory for them).
template <int NV>
__global__ void __launch_bounds__(TPB) k_shift_dots(Geom g, float vol, const float4* __restrict__ v, const float4* __restrict__ z,
                                                    const uint8_t* __restrict__ m, const float4* __restrict__ P, Tab V,
                                                    float4* __restrict__ w, double* __restrict__ part) {
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
            const float4 b = __ldg(V.p[q] + s);
            acc[q] += a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
        }
        acc[NV] += a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w;
    }
    double d[NV + 1];
#pragma unroll
    for (int q = 0; q <= NV; q++) d[q] = acc[q];
    block_sums<NV + 1>(d, part + (long long)blockIdx.x * (MAXV + 1));
}

// w -= sum_q h[q] v_q ; partial ||w||^2 per block (computed after the update)
template <int NV>
__global__ void __launch_bounds__(TPB) k_multiaxpy32(long long n4, Tab v, const double* __restrict__ h, float4* __restrict__ w,
                                                     double* __restrict__ part, int want_norm) {
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
    double acc[1] = {(double)accf};
    if (want_norm) block_sums<1>(acc, part + blockIdx.x);
}

// Projection step of classical Gram-Schmidt on unnormalised basis vectors:
// out = w - sum_q c_q v_q with c_q = sig2[q] * d[q] (d: the dot products <v_q, w> of the
// previous pass, sig2[q] = 1/||v_q||^2), in one pass. DOTS: the same pass also returns
// the dot products <v_q, out> (the re-orthogonalisation coefficients; the v_q are still
// in registers) and <out, out> in column NV. out may alias w.
template <int NV, bool DOTS>
__global__ void __launch_bounds__(TPB) k_proj32(long long n4, Tab v, const double* __restrict__ d, const double* __restrict__ sig2,
                                                const float4* w, float4* out, double* __restrict__ part) {
    float c[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) c[q] = (float)(sig2[q] * d[q]);
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
        if (DOTS) {
#pragma unroll
            for (int q = 0; q < NV; q++) acc[q] += a.x * b[q].x + a.y * b[q].y + a.z * b[q].z + a.w * b[q].w;
        }
        acc[NV] += a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w;
    }
    double dd[NV + 1];
#pragma unroll
    for (int q = 0; q <= NV; q++) dd[q] = acc[q];
    block_sums<NV + 1>(dd, part + (long long)blockIdx.x * (MAXV + 1));
}

__global__ void k_scale32(long long n4, const float4* __restrict__ x, const double* __restrict__ nrm2, float4* __restrict__ out) {
    double s0 = *nrm2;
    float s = s0 > 0 ? (float)(1.0 / sqrt(s0)) : 0.f;
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

int f32_to_f64(cudaStream_t st, long long n4, const float4* a, d4* out) {
    k_f32_to_f64<<<rgrid(4 * n4), TPB, 0, st>>>(n4, reinterpret_cast<const float*>(a), reinterpret_cast<double*>(out));
    STG_LAUNCH_CK();
    return STG_OK;
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
            k_multidot32<NV, true><<<rgrid(n4), TPB, 0, st>>>(n4, t, w, part);
        else
            k_multidot32<NV, false><<<rgrid(n4), TPB, 0, st>>>(n4, t, w, part);
    }
};
template <int NV>
struct ProjL {
    static void run(cudaStream_t st, long long n4, const Tab& t, const double* d, const double* sig2, const float4* w, float4* out,
                    double* part, bool dots) {
        if (dots)
            k_proj32<NV, true><<<rgrid(n4), TPB, 0, st>>>(n4, t, d, sig2, w, out, part);
        else
            k_proj32<NV, false><<<rgrid(n4), TPB, 0, st>>>(n4, t, d, sig2, w, out, part);
    }
};

int axpy_last_chunk(int nz) { return nz > 0 ? ((nz - 1) / MAXV) * MAXV : 0; }

// Chunks of MAXV vectors from the last one down: e (when one of the z_q, a slot at the end
// of the basis) is written by the first chunk, which holds it, and only added to by the
// later ones; the double-float copy of x is written by the last chunk.
int axpy_multi_32to64(cudaStream_t st, long long n4, const float4* const* z, const double* y, int nz, double alpha, d4* x,
                      float4* xh, float4* xl, float4* e) {
    const int nchunk = (nz + MAXV - 1) / MAXV;
    for (int c = nchunk - 1; c >= 0; c--) {
        const int j0 = c * MAXV;
        int nb = nz - j0 < MAXV ? nz - j0 : MAXV;
        Tab t{};
        for (int q = 0; q < nb; q++) t.p[q] = z[j0 + q];
        const bool last = c == 0;
        dispatch_nv<AxpyL>(nb, st, n4, t, y + j0, alpha, x, last ? xh : nullptr, last ? xl : nullptr, e, c == nchunk - 1);
        STG_LAUNCH_CK();
    }
    return STG_OK;
}

template <int NV>
struct ShiftL {
    static void run(cudaStream_t st, const Geom& g, float vol, const float4* v, const float4* z, const uint8_t* m, const float4* P,
                    const Tab& t, float4* w, double* part) {
        k_shift_dots<NV><<<RGRID, TPB, 0, st>>>(g, vol, v, z, m, P, t, w, part);
    }
};

int shift_multidot32(cudaStream_t st, const Geom& g, float vol, const float4* v, const float4* z, const uint8_t* m, const float4* P,
                     long long n4, const float4* const* V, int nv, float4* w, double* h, double* scratch, double* ww) {
    const int nb = nv < MAXV ? nv : MAXV;
    Tab t{};
    for (int q = 0; q < nb; q++) t.p[q] = V[q];
    dispatch_nv<ShiftL>(nb, st, g, vol, v, z, m, P, t, w, scratch);
    STG_LAUNCH_CK();
    k_reduce_cols<<<1, TPB, 0, st>>>(scratch, RGRID, MAXV + 1, nb, h);
    STG_LAUNCH_CK();
    k_reduce_cols<<<1, TPB, 0, st>>>(scratch + nb, RGRID, MAXV + 1, 1, ww);
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
        k_reduce_cols<<<1, TPB, 0, st>>>(scratch, (int)g, MAXV + 1, nb, h + j0);
        STG_LAUNCH_CK();
        if (want_ww) {
            k_reduce_cols<<<1, TPB, 0, st>>>(scratch + nb, (int)g, MAXV + 1, 1, ww);
            STG_LAUNCH_CK();
        }
    }
    return STG_OK;
}

template <int NV>
struct MaxpyL {
    static void run(cudaStream_t st, long long n4, const Tab& t, const double* h, float4* w, double* part, int want) {
        k_multiaxpy32<NV><<<rgrid(n4), TPB, 0, st>>>(n4, t, h, w, part, want);
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
    k_reduce_cols<<<1, TPB, 0, st>>>(scratch, (int)g, 1, 1, nrm2);
    STG_LAUNCH_CK();
    return STG_OK;
}

int project32(cudaStream_t st, long long n4, const float4* const* v, int nv, const double* d, const double* sig2, const float4* w,
              float4* out, double* dots, double* nrm2, double* scratch) {
    if (nv < 1) {
        set_error("project32: empty basis");
        return STG_E_INVALID;
    }
    unsigned g = rgrid(n4);
    if (nv <= MAXV) {
        Tab t{};
        for (int q = 0; q < nv; q++) t.p[q] = v[q];
        dispatch_nv<ProjL>(nv, st, n4, t, d, sig2, w, out, scratch, dots != nullptr);
        STG_LAUNCH_CK();
        if (dots) {
            k_reduce_cols<<<1, TPB, 0, st>>>(scratch, (int)g, MAXV + 1, nv, dots);
            STG_LAUNCH_CK();
        }
        k_reduce_cols<<<1, TPB, 0, st>>>(scratch + nv, (int)g, MAXV + 1, 1, nrm2);
        STG_LAUNCH_CK();
        return STG_OK;
    }
    // more vectors than one pass holds: subtract in chunks, then a separate dot pass
    for (int j0 = 0; j0 < nv; j0 += MAXV) {
        int nb = nv - j0 < MAXV ? nv - j0 : MAXV;
        Tab t{};
        for (int q = 0; q < nb; q++) t.p[q] = v[j0 + q];
        dispatch_nv<ProjL>(nb, st, n4, t, d + j0, sig2 + j0, j0 == 0 ? w : out, out, scratch, false);
        STG_LAUNCH_CK();
    }
    if (dots) return multidot32(st, n4, v, nv, out, dots, scratch, nrm2);
    k_reduce_cols<<<1, TPB, 0, st>>>(scratch + (nv - ((nv - 1) / MAXV) * MAXV), (int)g, MAXV + 1, 1, nrm2);
    STG_LAUNCH_CK();
    return STG_OK;
}

int scale32(cudaStream_t st, long long n4, float4* x, const double* nrm2, float4* out) {
    k_scale32<<<rgrid(n4), TPB, 0, st>>>(n4, x, nrm2, out);
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
