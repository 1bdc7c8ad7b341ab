// Learned preconditioner: a 3-level 3D U-Net over the finest-level cells (new; no
// counterpart in the reference).
//
// Input per cell (i,j,k) of the n^3 grid: the physical density, the four unknowns of slot
// (i,j,k) of a residual vector (p and the three low faces) scaled by the residual's RMS,
// and the three face penalties as shares P / (P + 6 vol) of the diagonal of A. Output: a
// correction for the same four unknowns, scaled back. Architecture (c base
// channels; every convolution 3x3x3 + ReLU, BF16 weights and activations, FP32
// accumulation on the tensor cores, unet_kernels.cu):
//   level 0 (n^3):   in(16) -> c -> c = s0
//   level 1 (n/2):   avgpool(s0) -> 2c -> 2c = s1
//   level 2 (n/4):   avgpool(s1) -> 4c -> 4c
//   level 1:         [up(level 2), s1] (6c) -> 2c -> 2c
//   level 0:         [up(level 1), s0] (3c) -> c -> c -> 1x1 head -> 4 (FP32)
// Skip connections are channel slices of the concatenation buffers (the encoder writes its
// output straight into them). Training: relative squared error against the exact
// correction, Adam on FP32 master weights, BF16 working copies refreshed after every step.
#include <cuda_bf16.h>

#include <cmath>
#include <vector>

#include "ctx.h"

namespace stg {

int conv3_forward(cudaStream_t st, const __nv_bfloat16* in, int cin, int ldin, const __nv_bfloat16* w, const float* bias,
                  void* out, int cout, int ldout, int n, int relu, bool f32_out, int wtap);
int conv3_backward_weights(cudaStream_t st, const __nv_bfloat16* x, int cin, int ldx, const __nv_bfloat16* dy, int cout, int lddy,
                           float* dw, float* db, int n);
int conv3_flip_weights(cudaStream_t st, const __nv_bfloat16* w, int cout, int cin, __nv_bfloat16* wf);
int conv3_tc_status(cudaStream_t st, int* timed_out);

// error when a tensor-core convolution gave up waiting for its MMAs (bounded waits)
int tc_check(cudaStream_t st) {
    int t = 0;
    STG_TRY(conv3_tc_status(st, &t));
    if (t) {
        set_error("tensor-core convolution: MMA completion wait timed out");
        return STG_E_CUDA;
    }
    return STG_OK;
}

namespace {

constexpr int TPB = 256;
using bf16 = __nv_bfloat16;

unsigned nb(long long work) { return (unsigned)((work + TPB - 1) / TPB); }

int cuda_ck(cudaError_t e) { return e == cudaSuccess ? STG_OK : cuda_fail(e, "CUDA call", __FILE__, __LINE__); }

// ---------------------------------------------------------------- elementwise kernels
__device__ __forceinline__ float bf(bf16 x) { return __bfloat162float(x); }

// Network input of cell v = (i n + j) n + k: channel 0 the physical density (0 when the
// handle has none), 1..4 the unknowns (p, u, v, w) of slot (i,j,k) of r times sc[0],
// 5..7 the face penalties as P / (P + 6 vol) (the share of the penalty in the diagonal of
// A), 8..15 zero.
__global__ void k_pack_input(Geom g, int n, const double* __restrict__ rho, const float4* __restrict__ P, float six_vol,
                             const float4* __restrict__ r, const float* __restrict__ sc, bf16* __restrict__ in0) {
    const long long v = (long long)blockIdx.x * TPB + threadIdx.x;
    if (v >= (long long)n * n * n) return;
    const int k = (int)(v % n), j = (int)((v / n) % n), i = (int)(v / ((long long)n * n));
    const int s = g.slot(i, j, k);
    const float4 x = r[s], q = P[s];
    const float a = sc[0];
    __align__(16) bf16 o[16];
    o[0] = __float2bfloat16(rho ? (float)rho[v] : 0.f);
    o[1] = __float2bfloat16(x.x * a);
    o[2] = __float2bfloat16(x.y * a);
    o[3] = __float2bfloat16(x.z * a);
    o[4] = __float2bfloat16(x.w * a);
    o[5] = __float2bfloat16(q.y / (q.y + six_vol));
    o[6] = __float2bfloat16(q.z / (q.z + six_vol));
    o[7] = __float2bfloat16(q.w / (q.w + six_vol));
#pragma unroll
    for (int c = 8; c < 16; c++) o[c] = __float2bfloat16(0.f);
    uint4* d = reinterpret_cast<uint4*>(in0 + v * 16);
    d[0] = *reinterpret_cast<const uint4*>(o);
    d[1] = *reinterpret_cast<const uint4*>(o + 8);
}

// per-block partials of the sum of (e - z).p over the free cells and of their count
__global__ void k_pmean(Geom g, int n, const float4* __restrict__ e, const float4* __restrict__ z, const uint8_t* __restrict__ m,
                        double* __restrict__ part) {
    __shared__ double sh[2][TPB / 32];
    double s = 0, c = 0;
    const long long V = (long long)n * n * n;
    for (long long v = (long long)blockIdx.x * TPB + threadIdx.x; v < V; v += (long long)gridDim.x * TPB) {
        const int k = (int)(v % n), j = (int)((v / n) % n), i = (int)(v / ((long long)n * n));
        const int q = g.slot(i, j, k);
        if (!(m[q] & MP)) {
            s += (double)(e[q].x - z[q].x);
            c += 1.0;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sh[0][threadIdx.x >> 5] = s;
        sh[1][threadIdx.x >> 5] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int w = 0; w < TPB / 32; w++) {
            a += sh[0][w];
            b += sh[1][w];
        }
        part[blockIdx.x] = a;
        part[gridDim.x + blockIdx.x] = b;
    }
}

// training target of cell v: (e - z) at slot (i,j,k) divided by sc[1], with the mean
// pressure pm[0] / pm[1] over the free cells removed when pm != nullptr (closed domains:
// the constant pressure is the null space of A, so no residual can predict it)
__global__ void k_pack_target(Geom g, int n, const float4* __restrict__ e, const float4* __restrict__ z, const float* __restrict__ sc,
                              const double* __restrict__ pm, const uint8_t* __restrict__ m, float* __restrict__ tgt) {
    const long long v = (long long)blockIdx.x * TPB + threadIdx.x;
    if (v >= (long long)n * n * n) return;
    const int k = (int)(v % n), j = (int)((v / n) % n), i = (int)(v / ((long long)n * n));
    const int s = g.slot(i, j, k);
    const float4 a = e[s], b = z[s];
    const float w = sc[1] > 0.f ? 1.f / sc[1] : 0.f;
    const float p0 = (pm && pm[1] > 0 && !(m[s] & MP)) ? (float)(pm[0] / pm[1]) : 0.f;
    *reinterpret_cast<float4*>(tgt + v * 4) = make_float4((a.x - b.x - p0) * w, (a.y - b.y) * w, (a.z - b.z) * w, (a.w - b.w) * w);
}

// z[slot] += out[v] * sc[1] on the free unknowns of the cells (i,j,k) < n
__global__ void k_unpack_output(Geom g, int n, const float* __restrict__ out, const float* __restrict__ sc, const uint8_t* __restrict__ m,
                                float4* __restrict__ z) {
    const long long v = (long long)blockIdx.x * TPB + threadIdx.x;
    if (v >= (long long)n * n * n) return;
    const int k = (int)(v % n), j = (int)((v / n) % n), i = (int)(v / ((long long)n * n));
    const int s = g.slot(i, j, k);
    const float4 o = *reinterpret_cast<const float4*>(out + v * 4);
    const float w = sc[1];
    const uint8_t mm = m[s];
    float4 zz = z[s];
    if (!(mm & MP)) zz.x += o.x * w;
    if (!(mm & MU)) zz.y += o.y * w;
    if (!(mm & MV)) zz.z += o.z * w;
    if (!(mm & MW)) zz.w += o.w * w;
    z[s] = zz;
}

// per-block partial sums of x.x over n4 float4 entries (FP64)
__global__ void k_sumsq(long long n4, const float4* __restrict__ x, double* __restrict__ part) {
    __shared__ double sh[TPB / 32];
    double s = 0;
    for (long long e = (long long)blockIdx.x * TPB + threadIdx.x; e < n4; e += (long long)gridDim.x * TPB) {
        const float4 a = x[e];
        s += (double)(a.x * a.x + a.y * a.y) + (double)(a.z * a.z + a.w * a.w);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < TPB / 32; w++) t += sh[w];
        part[blockIdx.x] = t;
    }
}

// sc[0] = 1 / rms(r) (0 for r = 0), sc[1] = kappa * rms(r): the input and output scales
// of the network for a residual with squared norm *nr2 over `count` unknowns
__global__ void k_scales(const double* __restrict__ nr2, double count, const float* __restrict__ kappa, float* __restrict__ sc) {
    const double rms = sqrt(*nr2 / count);
    sc[0] = rms > 0 ? (float)(1.0 / rms) : 0.f;
    sc[1] = (float)(rms * (double)*kappa);
}

// noise on the free unknowns of the box: U(-1, 1) from a SplitMix64 hash of (seed, slot, component)
__global__ void k_noise_slots(Geom g, const uint8_t* __restrict__ m, uint64_t seed, float4* __restrict__ x) {
    const long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    const int s = g.slot(i, j, k);
    float r[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        uint64_t z = seed * 0x9E3779B97F4A7C15ull + (uint64_t)(4 * s + c) + 0x632BE59BD9B4E019ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z = z ^ (z >> 31);
        r[c] = 2.0f * (float)((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.f;
    }
    const uint8_t mm = m[s];
    x[s] = make_float4(mm & MP ? 0.f : r[0], mm & MU ? 0.f : r[1], mm & MV ? 0.f : r[2], mm & MW ? 0.f : r[3]);
}

// The resampling kernels below take one thread per (voxel, 8 BF16 or 4 FP32 channels):
// every channel count and row stride is a multiple of 8 and every row starts on 16 bytes.
__device__ __forceinline__ void vox_of(long long v, int nn, int& i, int& j, int& k) {
    const long long q = v / nn;
    k = (int)(v - q * nn);
    i = (int)(q / nn);
    j = (int)(q - (long long)i * nn);
}

// 2x2x2 average pooling of channels [0, C) of a (ld_in) into b (ld_out), coarse grid nc
__global__ void k_pool(const bf16* __restrict__ a, int ld_in, int C, bf16* __restrict__ b, int ld_out, int nc) {
    const int G = C / 8;
    const long long e = (long long)blockIdx.x * TPB + threadIdx.x;
    if (e >= (long long)nc * nc * nc * G) return;
    const int q = (int)(e % G);
    const long long v = e / G;
    int i, j, k;
    vox_of(v, nc, i, j, k);
    const int nf = 2 * nc;
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const long long fv = ((long long)(2 * i + (c >> 2)) * nf + 2 * j + ((c >> 1) & 1)) * nf + 2 * k + (c & 1);
        const uint4 x = *reinterpret_cast<const uint4*>(a + fv * ld_in + 8 * q);
        const bf16* h = reinterpret_cast<const bf16*>(&x);
#pragma unroll
        for (int u = 0; u < 8; u++) s[u] += bf(h[u]);
    }
    __align__(16) bf16 o[8];
#pragma unroll
    for (int u = 0; u < 8; u++) o[u] = __float2bfloat16(0.125f * s[u]);
    *reinterpret_cast<uint4*>(b + v * ld_out + 8 * q) = *reinterpret_cast<const uint4*>(o);
}

// g_fine[child][c] += g_coarse[parent][c] / 8 (pooling backward; FP32, 4 channels a thread)
__global__ void k_pool_bwd(const float* __restrict__ gc, int ldc, int C, float* __restrict__ gf, int ldf, int nc) {
    const int G = C / 4;
    const int nf = 2 * nc;
    const long long e = (long long)blockIdx.x * TPB + threadIdx.x;
    if (e >= (long long)nf * nf * nf * G) return;
    const int q = (int)(e % G);
    const long long v = e / G;
    int i, j, k;
    vox_of(v, nf, i, j, k);
    const long long pv = ((long long)(i >> 1) * nc + (j >> 1)) * nc + (k >> 1);
    const float4 g = *reinterpret_cast<const float4*>(gc + pv * ldc + 4 * q);
    float4* d = reinterpret_cast<float4*>(gf + v * ldf + 4 * q);
    float4 x = *d;
    x.x += 0.125f * g.x;
    x.y += 0.125f * g.y;
    x.z += 0.125f * g.z;
    x.w += 0.125f * g.w;
    *d = x;
}

// nearest up-sampling of channels [0, C) of the coarse a into b (fine grid 2 nc)
__global__ void k_up(const bf16* __restrict__ a, int ld_in, int C, bf16* __restrict__ b, int ld_out, int nc) {
    const int G = C / 8;
    const int nf = 2 * nc;
    const long long e = (long long)blockIdx.x * TPB + threadIdx.x;
    if (e >= (long long)nf * nf * nf * G) return;
    const int q = (int)(e % G);
    const long long v = e / G;
    int i, j, k;
    vox_of(v, nf, i, j, k);
    const long long pv = ((long long)(i >> 1) * nc + (j >> 1)) * nc + (k >> 1);
    *reinterpret_cast<uint4*>(b + v * ld_out + 8 * q) = *reinterpret_cast<const uint4*>(a + pv * ld_in + 8 * q);
}

// g_coarse[parent][c] = sum of the 8 children's g_fine (up-sampling backward, 4 channels a thread)
__global__ void k_up_bwd(const float* __restrict__ gf, int ldf, int C, float* __restrict__ gc, int ldc, int nc) {
    const int G = C / 4;
    const long long e = (long long)blockIdx.x * TPB + threadIdx.x;
    if (e >= (long long)nc * nc * nc * G) return;
    const int q = (int)(e % G);
    const long long v = e / G;
    int i, j, k;
    vox_of(v, nc, i, j, k);
    const int nf = 2 * nc;
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const long long fv = ((long long)(2 * i + (c >> 2)) * nf + 2 * j + ((c >> 1) & 1)) * nf + 2 * k + (c & 1);
        const float4 g = *reinterpret_cast<const float4*>(gf + fv * ldf + 4 * q);
        s.x += g.x;
        s.y += g.y;
        s.z += g.z;
        s.w += g.w;
    }
    *reinterpret_cast<float4*>(gc + v * ldc + 4 * q) = s;
}

// out = (y > 0) ? g : 0 as BF16 (ReLU backward, the conv input of the next backward pass),
// 8 channels a thread
__global__ void k_relu_grad(const float* __restrict__ g, int ldg, const bf16* __restrict__ y, int ldy, int C, long long V,
                            bf16* __restrict__ out) {
    const int G = C / 8;
    const long long e = (long long)blockIdx.x * TPB + threadIdx.x;
    if (e >= V * G) return;
    const int q = (int)(e % G);
    const long long v = e / G;
    const float4 g0 = *reinterpret_cast<const float4*>(g + v * ldg + 8 * q);
    const float4 g1 = *reinterpret_cast<const float4*>(g + v * ldg + 8 * q + 4);
    const uint4 yy = *reinterpret_cast<const uint4*>(y + v * ldy + 8 * q);
    const bf16* h = reinterpret_cast<const bf16*>(&yy);
    const float gg[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
    __align__(16) bf16 o[8];
#pragma unroll
    for (int u = 0; u < 8; u++) o[u] = __float2bfloat16(bf(h[u]) > 0.f ? gg[u] : 0.f);
    *reinterpret_cast<uint4*>(out + v * C + 8 * q) = *reinterpret_cast<const uint4*>(o);
}

// 1x1 head: out[v][o] = b[o] + sum_c W[o][c] x[v][c]  (4 outputs, FP32)
__global__ void k_head(const bf16* __restrict__ x, int C, const float* __restrict__ W, const float* __restrict__ b, long long V,
                       float* __restrict__ out) {
    const long long v = (long long)blockIdx.x * TPB + threadIdx.x;
    if (v >= V) return;
    float o[4] = {b[0], b[1], b[2], b[3]};
    for (int c = 0; c < C; c++) {
        const float xv = bf(x[v * C + c]);
#pragma unroll
        for (int q = 0; q < 4; q++) o[q] += W[q * C + c] * xv;
    }
    *reinterpret_cast<float4*>(out + v * 4) = make_float4(o[0], o[1], o[2], o[3]);
}

// partials of the relative squared error sum (out - tgt)^2 / *t2 (t2 = sum tgt^2, so the
// zero output scores 1 on every sample) and dout = 2 (out - tgt) / *t2
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ tgt, long long count, const double* __restrict__ t2,
                      float* __restrict__ dout, double* __restrict__ part) {
    __shared__ double sh[TPB / 32];
    double s = 0;
    const double inv = *t2 > 0 ? 1.0 / *t2 : 0.0;
    for (long long e = (long long)blockIdx.x * TPB + threadIdx.x; e < count; e += (long long)gridDim.x * TPB) {
        const float d = out[e] - tgt[e];
        s += (double)d * d * inv;
        dout[e] = (float)(2.0 * d * inv);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < TPB / 32; w++) t += sh[w];
        part[blockIdx.x] = t;
    }
}

// head backward: gx[v][c] = sum_o W[o][c] dout[v][o]; dW[o][c] += sum_v dout[v][o] x[v][c]; db[o] += sum_v dout
__global__ void k_head_bwd(const bf16* __restrict__ x, int C, const float* __restrict__ W, const float* __restrict__ dout, long long V,
                           float* __restrict__ gx, float* __restrict__ dW, float* __restrict__ db) {
    __shared__ float sw[4 * 64], sb[4];
    for (int e = threadIdx.x; e < 4 * C; e += TPB) sw[e] = 0.f;
    if (threadIdx.x < 4) sb[threadIdx.x] = 0.f;
    __syncthreads();
    const long long v = (long long)blockIdx.x * TPB + threadIdx.x;
    if (v < V) {
        const float4 d = *reinterpret_cast<const float4*>(dout + v * 4);
        const float dd[4] = {d.x, d.y, d.z, d.w};
        for (int c = 0; c < C; c++) {
            const float xv = bf(x[v * C + c]);
            float g = 0.f;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                g += W[q * C + c] * dd[q];
                atomicAdd(&sw[q * C + c], dd[q] * xv);
            }
            gx[v * C + c] = g;
        }
#pragma unroll
        for (int q = 0; q < 4; q++) atomicAdd(&sb[q], dd[q]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 4 * C; e += TPB) atomicAdd(&dW[e], sw[e]);
    if (threadIdx.x < 4) atomicAdd(&db[threadIdx.x], sb[threadIdx.x]);
}

// Adam on FP32 master parameters; optional BF16 working copy
__global__ void k_adam(long long n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       float lr, float b1, float b2, float c1, float c2, float eps, bf16* __restrict__ p16) {
    const long long e = (long long)blockIdx.x * TPB + threadIdx.x;
    if (e >= n) return;
    const float gg = g[e];
    const float mm = b1 * m[e] + (1.f - b1) * gg, vv = b2 * v[e] + (1.f - b2) * gg * gg;
    m[e] = mm;
    v[e] = vv;
    const float pp = p[e] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    p[e] = pp;
    if (p16) p16[e] = __float2bfloat16(pp);
}

__global__ void k_f32_to_bf16(long long n, const float* __restrict__ a, bf16* __restrict__ b) {
    const long long e = (long long)blockIdx.x * TPB + threadIdx.x;
    if (e < n) b[e] = __float2bfloat16(a[e]);
}

// deterministic initial weights: U(-s, s) from a SplitMix64 hash of (seed, index)
__global__ void k_init_uniform(long long n, uint64_t seed, float s, float* __restrict__ p) {
    const long long e = (long long)blockIdx.x * TPB + threadIdx.x;
    if (e >= n) return;
    uint64_t z = seed * 0x9E3779B97F4A7C15ull + (uint64_t)e + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    p[e] = s * (2.0f * (float)((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.f);
}

}  // namespace

// ---------------------------------------------------------------- network
constexpr int NCONV = 10;
constexpr int IN_CH = 16;    // input channels as stored (8 used)
constexpr int IN_USED = 8;   // channels of the host-side input of stg_net_forward_backward
constexpr int OUT_CH = 4;

struct Buf {
    std::vector<void*> ptrs;
    template <class T>
    int get(T** p, size_t count) {
        cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
        ptrs.push_back(*p);
        return STG_OK;
    }
    void release() {
        for (void* p : ptrs) cudaFree(p);
        ptrs.clear();
    }
};

}  // namespace stg

// The network of a handle: parameters (FP32 master, BF16 working copy, flipped BF16
// weights for the backward-data pass), Adam state, and activation buffers for one grid size.
struct NetState {
    int c = 16;
    int cin[stg::NCONV] = {}, cout[stg::NCONV] = {};
    long long woff[stg::NCONV] = {}, boff[stg::NCONV] = {}, hw_off = 0, hb_off = 0, kappa_off = 0, nparam = 0;
    float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;
    __nv_bfloat16 *p16 = nullptr, *wf = nullptr;
    int adam_t = 0;
    float kappa = 0.f;  // host copy of p[kappa_off]
    double *part = nullptr, *dsum = nullptr, *dloss = nullptr, *dt2 = nullptr;
    float* sc = nullptr;
    stg::Buf pbuf;
    // activations for grid n (train: also the gradient buffers)
    int n = 0;
    bool train = false;
    __nv_bfloat16 *in0 = nullptr, *a0 = nullptr, *cat0 = nullptr, *a0d = nullptr, *b0d = nullptr, *p0 = nullptr, *a1 = nullptr,
                  *cat1 = nullptr, *a1d = nullptr, *b1d = nullptr, *p1 = nullptr, *a2 = nullptr, *b2 = nullptr, *dy = nullptr;
    float *out = nullptr, *tgt = nullptr, *dout = nullptr, *G0a = nullptr, *G0b = nullptr, *G0cat = nullptr, *G1a = nullptr,
          *G1b = nullptr, *G1cat = nullptr, *G2a = nullptr, *G2b = nullptr;
    stg::Buf abuf;
    // fine-grid slot vectors of the training-pair generator
    float4 *s_e = nullptr, *s_r = nullptr, *s_z = nullptr, *s_r1 = nullptr;
    stg::Buf sbuf;
    ~NetState() {
        abuf.release();
        sbuf.release();
        pbuf.release();
    }
};

namespace stg {
namespace {

constexpr int NPART = 512;

int net_layout(NetState& N, int c) {
    N.c = c;
    const int ci[NCONV] = {IN_CH, c, c, 2 * c, 2 * c, 4 * c, 6 * c, 2 * c, 3 * c, c};
    const int co[NCONV] = {c, c, 2 * c, 2 * c, 4 * c, 4 * c, 2 * c, 2 * c, c, c};
    long long off = 0;
    for (int l = 0; l < NCONV; l++) {
        N.cin[l] = ci[l];
        N.cout[l] = co[l];
        N.woff[l] = off;
        off += 27LL * co[l] * ci[l];
        N.boff[l] = off;
        off += co[l];
    }
    N.hw_off = off;
    off += OUT_CH * c;
    N.hb_off = off;
    off += OUT_CH;
    N.kappa_off = off;
    off += 1;
    N.nparam = off;
    return STG_OK;
}

int refresh_working(NetState& N, cudaStream_t st) {
    k_f32_to_bf16<<<nb(N.nparam), TPB, 0, st>>>(N.nparam, N.p, N.p16);
    STG_LAUNCH_CK();
    for (int l = 0; l < NCONV; l++) STG_TRY(conv3_flip_weights(st, N.p16 + N.woff[l], N.cout[l], N.cin[l], N.wf + N.woff[l]));
    return STG_OK;
}

int net_alloc_params(NetState& N) {
    Buf& B = N.pbuf;
    STG_TRY(B.get(&N.p, N.nparam));
    STG_TRY(B.get(&N.g, N.nparam));
    STG_TRY(B.get(&N.m1, N.nparam));
    STG_TRY(B.get(&N.m2, N.nparam));
    STG_TRY(B.get(&N.p16, N.nparam));
    STG_TRY(B.get(&N.wf, N.nparam));
    STG_TRY(B.get(&N.part, 2 * NPART));
    STG_TRY(B.get(&N.dsum, 2));
    STG_TRY(B.get(&N.dloss, 1));
    STG_TRY(B.get(&N.dt2, 1));
    STG_TRY(B.get(&N.sc, 2));
    return STG_OK;
}

int reset_adam(NetState& N, cudaStream_t st) {
    N.adam_t = 0;
    STG_CK(cudaMemsetAsync(N.m1, 0, sizeof(float) * N.nparam, st));
    STG_CK(cudaMemsetAsync(N.m2, 0, sizeof(float) * N.nparam, st));
    return STG_OK;
}

// He-uniform weights U(-sqrt(6 / fan_in), +), zero biases, kappa 0 (set by the first training pair)
int net_init_params(NetState& N, cudaStream_t st, uint64_t seed) {
    STG_CK(cudaMemsetAsync(N.p, 0, sizeof(float) * N.nparam, st));
    for (int l = 0; l < NCONV; l++) {
        const int fan = 27 * (l == 0 ? IN_USED : N.cin[l]);
        const long long cnt = 27LL * N.cout[l] * N.cin[l];
        k_init_uniform<<<nb(cnt), TPB, 0, st>>>(cnt, seed + 1000003ull * (l + 1), std::sqrt(6.0f / fan), N.p + N.woff[l]);
        STG_LAUNCH_CK();
    }
    k_init_uniform<<<nb(OUT_CH * N.c), TPB, 0, st>>>(OUT_CH * N.c, seed + 77ull, std::sqrt(6.0f / N.c), N.p + N.hw_off);
    STG_LAUNCH_CK();
    N.kappa = 0.f;
    STG_TRY(reset_adam(N, st));
    return refresh_working(N, st);
}

long long vox3(int n) { return (long long)n * n * n; }

int net_buffers(NetState& N, int n, bool train) {
    if (n == N.n && (N.train || !train)) return STG_OK;
    N.abuf.release();
    N.n = 0;
    const int c = N.c;
    const long long V0 = vox3(n), V1 = vox3(n / 2), V2 = vox3(n / 4);
    Buf& B = N.abuf;
    STG_TRY(B.get(&N.in0, V0 * IN_CH));
    STG_TRY(B.get(&N.a0, V0 * c));
    STG_TRY(B.get(&N.cat0, V0 * 3 * c));
    STG_TRY(B.get(&N.a0d, V0 * c));
    STG_TRY(B.get(&N.b0d, V0 * c));
    STG_TRY(B.get(&N.p0, V1 * c));
    STG_TRY(B.get(&N.a1, V1 * 2 * c));
    STG_TRY(B.get(&N.cat1, V1 * 6 * c));
    STG_TRY(B.get(&N.a1d, V1 * 2 * c));
    STG_TRY(B.get(&N.b1d, V1 * 2 * c));
    STG_TRY(B.get(&N.p1, V2 * 2 * c));
    STG_TRY(B.get(&N.a2, V2 * 4 * c));
    STG_TRY(B.get(&N.b2, V2 * 4 * c));
    STG_TRY(B.get(&N.out, V0 * OUT_CH));
    if (train) {
        STG_TRY(B.get(&N.dy, std::max(V0 * c, std::max(V1 * 2 * c, V2 * 4 * c))));
        STG_TRY(B.get(&N.tgt, V0 * OUT_CH));
        STG_TRY(B.get(&N.dout, V0 * OUT_CH));
        STG_TRY(B.get(&N.G0a, V0 * c));
        STG_TRY(B.get(&N.G0b, V0 * c));
        STG_TRY(B.get(&N.G0cat, V0 * 3 * c));
        STG_TRY(B.get(&N.G1a, V1 * 2 * c));
        STG_TRY(B.get(&N.G1b, V1 * 2 * c));
        STG_TRY(B.get(&N.G1cat, V1 * 6 * c));
        STG_TRY(B.get(&N.G2a, V2 * 4 * c));
        STG_TRY(B.get(&N.G2b, V2 * 4 * c));
    }
    N.n = n;
    N.train = train;
    return STG_OK;
}

// conv l forward: in (ld ldin) -> out (ld ldout), ReLU, BF16
int conv_f(NetState& N, cudaStream_t st, int l, const bf16* in, int ldin, bf16* out, int ldout, int n) {
    return conv3_forward(st, in, N.cin[l], ldin, N.p16 + N.woff[l], N.p + N.boff[l], out, N.cout[l], ldout, n, 1, false, 0);
}

int pool(cudaStream_t st, const bf16* a, int ld_in, int C, bf16* b, int ld_out, int nc) {
    k_pool<<<nb(vox3(nc) * C / 8), TPB, 0, st>>>(a, ld_in, C, b, ld_out, nc);
    STG_LAUNCH_CK();
    return STG_OK;
}

int up(cudaStream_t st, const bf16* a, int ld_in, int C, bf16* b, int ld_out, int nc) {
    k_up<<<nb(vox3(2 * nc) * C / 8), TPB, 0, st>>>(a, ld_in, C, b, ld_out, nc);
    STG_LAUNCH_CK();
    return STG_OK;
}

// forward pass on N.in0 (grid n) -> N.out
int net_forward(NetState& N, cudaStream_t st, int n) {
    const int c = N.c, n1 = n / 2, n2 = n / 4;
    STG_TRY(conv_f(N, st, 0, N.in0, IN_CH, N.a0, c, n));
    STG_TRY(conv_f(N, st, 1, N.a0, c, N.cat0 + 2 * c, 3 * c, n));
    STG_TRY(pool(st, N.cat0 + 2 * c, 3 * c, c, N.p0, c, n1));
    STG_TRY(conv_f(N, st, 2, N.p0, c, N.a1, 2 * c, n1));
    STG_TRY(conv_f(N, st, 3, N.a1, 2 * c, N.cat1 + 4 * c, 6 * c, n1));
    STG_TRY(pool(st, N.cat1 + 4 * c, 6 * c, 2 * c, N.p1, 2 * c, n2));
    STG_TRY(conv_f(N, st, 4, N.p1, 2 * c, N.a2, 4 * c, n2));
    STG_TRY(conv_f(N, st, 5, N.a2, 4 * c, N.b2, 4 * c, n2));
    STG_TRY(up(st, N.b2, 4 * c, 4 * c, N.cat1, 6 * c, n2));
    STG_TRY(conv_f(N, st, 6, N.cat1, 6 * c, N.a1d, 2 * c, n1));
    STG_TRY(conv_f(N, st, 7, N.a1d, 2 * c, N.b1d, 2 * c, n1));
    STG_TRY(up(st, N.b1d, 2 * c, 2 * c, N.cat0, 3 * c, n1));
    STG_TRY(conv_f(N, st, 8, N.cat0, 3 * c, N.a0d, c, n));
    STG_TRY(conv_f(N, st, 9, N.a0d, c, N.b0d, c, n));
    k_head<<<nb(vox3(n)), TPB, 0, st>>>(N.b0d, c, N.p + N.hw_off, N.p + N.hb_off, vox3(n), N.out);
    STG_LAUNCH_CK();
    return STG_OK;
}

// dy = relu'(y) * g as BF16 (ld C)
int relu_grad(NetState& N, cudaStream_t st, const float* g, int ldg, const bf16* y, int ldy, int C, int n) {
    k_relu_grad<<<nb(vox3(n) * C / 8), TPB, 0, st>>>(g, ldg, y, ldy, C, vox3(n), N.dy);
    STG_LAUNCH_CK();
    return STG_OK;
}

// weight and bias gradients of conv l from its input x and N.dy
int conv_dw(NetState& N, cudaStream_t st, int l, const bf16* x, int ldx, int n) {
    return conv3_backward_weights(st, x, N.cin[l], ldx, N.dy, N.cout[l], N.cout[l], N.g + N.woff[l], N.g + N.boff[l], n);
}

// input gradient of conv l: dx (FP32, ld ldx) = the forward pass of N.dy with the flipped
// weights, in blocks of at most 64 output channels
int conv_dx(NetState& N, cudaStream_t st, int l, float* dx, int ldx, int n) {
    const int ci = N.cin[l], co = N.cout[l];
    const int blk = ci > 64 ? ci / 2 : ci;
    for (int b = 0; b < ci; b += blk)
        STG_TRY(conv3_forward(st, N.dy, co, co, N.wf + N.woff[l] + (size_t)b * co, nullptr, dx + b, blk, ldx, n, 0, true, ci * co));
    return STG_OK;
}

// backward pass from N.dout; gradients into N.g (zeroed here)
int net_backward(NetState& N, cudaStream_t st, int n) {
    const int c = N.c, n1 = n / 2, n2 = n / 4;
    const long long V0 = vox3(n), V1 = vox3(n1), V2 = vox3(n2);
    STG_CK(cudaMemsetAsync(N.g, 0, sizeof(float) * N.nparam, st));
    k_head_bwd<<<nb(V0), TPB, 0, st>>>(N.b0d, c, N.p + N.hw_off, N.dout, V0, N.G0a, N.g + N.hw_off, N.g + N.hb_off);
    STG_LAUNCH_CK();
    // level 0 decoder
    STG_TRY(relu_grad(N, st, N.G0a, c, N.b0d, c, c, n));
    STG_TRY(conv_dw(N, st, 9, N.a0d, c, n));
    STG_TRY(conv_dx(N, st, 9, N.G0b, c, n));
    STG_TRY(relu_grad(N, st, N.G0b, c, N.a0d, c, c, n));
    STG_TRY(conv_dw(N, st, 8, N.cat0, 3 * c, n));
    STG_TRY(conv_dx(N, st, 8, N.G0cat, 3 * c, n));
    k_up_bwd<<<nb(V1 * 2 * c / 4), TPB, 0, st>>>(N.G0cat, 3 * c, 2 * c, N.G1a, 2 * c, n1);
    STG_LAUNCH_CK();
    // level 1 decoder
    STG_TRY(relu_grad(N, st, N.G1a, 2 * c, N.b1d, 2 * c, 2 * c, n1));
    STG_TRY(conv_dw(N, st, 7, N.a1d, 2 * c, n1));
    STG_TRY(conv_dx(N, st, 7, N.G1b, 2 * c, n1));
    STG_TRY(relu_grad(N, st, N.G1b, 2 * c, N.a1d, 2 * c, 2 * c, n1));
    STG_TRY(conv_dw(N, st, 6, N.cat1, 6 * c, n1));
    STG_TRY(conv_dx(N, st, 6, N.G1cat, 6 * c, n1));
    k_up_bwd<<<nb(V2 * 4 * c / 4), TPB, 0, st>>>(N.G1cat, 6 * c, 4 * c, N.G2a, 4 * c, n2);
    STG_LAUNCH_CK();
    // level 2
    STG_TRY(relu_grad(N, st, N.G2a, 4 * c, N.b2, 4 * c, 4 * c, n2));
    STG_TRY(conv_dw(N, st, 5, N.a2, 4 * c, n2));
    STG_TRY(conv_dx(N, st, 5, N.G2b, 4 * c, n2));
    STG_TRY(relu_grad(N, st, N.G2b, 4 * c, N.a2, 4 * c, 4 * c, n2));
    STG_TRY(conv_dw(N, st, 4, N.p1, 2 * c, n2));
    STG_TRY(conv_dx(N, st, 4, N.G2a, 2 * c, n2));
    k_pool_bwd<<<nb(V1 * 2 * c / 4), TPB, 0, st>>>(N.G2a, 2 * c, 2 * c, N.G1cat + 4 * c, 6 * c, n2);
    STG_LAUNCH_CK();
    // level 1 encoder
    STG_TRY(relu_grad(N, st, N.G1cat + 4 * c, 6 * c, N.cat1 + 4 * c, 6 * c, 2 * c, n1));
    STG_TRY(conv_dw(N, st, 3, N.a1, 2 * c, n1));
    STG_TRY(conv_dx(N, st, 3, N.G1a, 2 * c, n1));
    STG_TRY(relu_grad(N, st, N.G1a, 2 * c, N.a1, 2 * c, 2 * c, n1));
    STG_TRY(conv_dw(N, st, 2, N.p0, c, n1));
    STG_TRY(conv_dx(N, st, 2, N.G1b, c, n1));
    k_pool_bwd<<<nb(V0 * c / 4), TPB, 0, st>>>(N.G1b, c, c, N.G0cat + 2 * c, 3 * c, n1);
    STG_LAUNCH_CK();
    // level 0 encoder
    STG_TRY(relu_grad(N, st, N.G0cat + 2 * c, 3 * c, N.cat0 + 2 * c, 3 * c, c, n));
    STG_TRY(conv_dw(N, st, 1, N.a0, c, n));
    STG_TRY(conv_dx(N, st, 1, N.G0a, c, n));
    STG_TRY(relu_grad(N, st, N.G0a, c, N.a0, c, c, n));
    STG_TRY(conv_dw(N, st, 0, N.in0, IN_CH, n));
    return STG_OK;
}

// loss = mean (out - tgt)^2 into N.dloss (device) and dout
int net_loss(NetState& N, cudaStream_t st, int n) {
    const long long cnt = vox3(n) * OUT_CH;
    k_sumsq<<<NPART, TPB, 0, st>>>(vox3(n), reinterpret_cast<const float4*>(N.tgt), N.part);
    STG_LAUNCH_CK();
    STG_TRY(reduce_parts(st, N.part, NPART, N.dt2));
    const int blocks = (int)std::min<long long>(NPART, (cnt + TPB - 1) / TPB);
    k_mse<<<blocks, TPB, 0, st>>>(N.out, N.tgt, cnt, N.dt2, N.dout, N.part);
    STG_LAUNCH_CK();
    return reduce_parts(st, N.part, blocks, N.dloss);
}

int net_adam(NetState& N, cudaStream_t st, double lr) {
    N.adam_t++;
    const double b1 = 0.9, b2 = 0.999;
    const float c1 = (float)(1.0 - std::pow(b1, N.adam_t)), c2 = (float)(1.0 - std::pow(b2, N.adam_t));
    const long long cnt = N.kappa_off;  // kappa is not trained
    k_adam<<<nb(cnt), TPB, 0, st>>>(cnt, N.p, N.g, N.m1, N.m2, (float)lr, (float)b1, (float)b2, c1, c2, 1e-8f, N.p16);
    STG_LAUNCH_CK();
    for (int l = 0; l < NCONV; l++) STG_TRY(conv3_flip_weights(st, N.p16 + N.woff[l], N.cout[l], N.cin[l], N.wf + N.woff[l]));
    return STG_OK;
}

// squared norm of a fine slot vector into N.dsum[0], then the network scales into N.sc
int net_scales(NetState& N, cudaStream_t st, const Geom& g, const float4* r, int n) {
    k_sumsq<<<NPART, TPB, 0, st>>>(g.nslot, r, N.part);
    STG_LAUNCH_CK();
    STG_TRY(reduce_parts(st, N.part, NPART, N.dsum));
    k_scales<<<1, 1, 0, st>>>(N.dsum, (double)vox3(n) * OUT_CH, N.p + N.kappa_off, N.sc);
    STG_LAUNCH_CK();
    return STG_OK;
}

int net_pack(stg_t* h, NetState& N, const float4* r1) {
    Level& F = fine(h);
    const int n = h->n;
    STG_TRY(net_scales(N, h->st, F.g, r1, n));
    k_pack_input<<<nb(vox3(n)), TPB, 0, h->st>>>(F.g, n, h->phys_used, F.P32, (float)(6.0 * F.vol), r1, N.sc, N.in0);
    STG_LAUNCH_CK();
    return STG_OK;
}

bool net_grid_ok(int n) { return n >= 8 && n % 4 == 0; }

}  // namespace

// z += NN(r1): the learned correction of a V-cycle result (3D, the handle's finest grid)
int net_correct(stg_t* h, const float4* r1, float4* z) {
    NetState& N = *h->net;
    const int n = h->n;
    STG_TRY(net_buffers(N, n, false));
    STG_TRY(net_pack(h, N, r1));
    STG_TRY(net_forward(N, h->st, n));
    k_unpack_output<<<nb(vox3(n)), TPB, 0, h->st>>>(fine(h).g, n, N.out, N.sc, fine(h).m, z);
    STG_LAUNCH_CK();
    return STG_OK;
}

void net_free(stg_t* h) {
    delete h->net;
    h->net = nullptr;
}

// One training pair on the handle's operator A and V-cycle M: e = M(noise), r = A e,
// z = M(r); input r1 = r - A z, target e - z (= A^-1 r1).
int net_pair(stg_t* h, NetState& N, uint64_t seed) {
    Level& F = fine(h);
    const Geom& g = F.g;
    if (!N.s_e) {
        STG_TRY(N.sbuf.get(&N.s_e, g.nslot));
        STG_TRY(N.sbuf.get(&N.s_r, g.nslot));
        STG_TRY(N.sbuf.get(&N.s_z, g.nslot));
        STG_TRY(N.sbuf.get(&N.s_r1, g.nslot));
        for (float4* p : {N.s_e, N.s_r, N.s_z, N.s_r1}) STG_CK(cudaMemsetAsync(p, 0, sizeof(float4) * g.nslot, h->st));
    }
    k_noise_slots<<<nb(g.box()), TPB, 0, h->st>>>(g, F.m, seed, N.s_r);
    STG_LAUNCH_CK();
    STG_TRY(precond3(h, N.s_r, N.s_e));
    STG_TRY(apply3(h, N.s_e, N.s_r));
    STG_TRY(precond3(h, N.s_r, N.s_z));
    STG_TRY(resid32(h->st, g, (float)F.vol, N.s_r, N.s_z, F.m, F.P32, N.s_r1, fast(h, F)));
    STG_TRY(net_pack(h, N, N.s_r1));
    const double* pm = nullptr;
    if (h->closed) {
        k_pmean<<<NPART, TPB, 0, h->st>>>(g, h->n, N.s_e, N.s_z, F.m, N.part);
        STG_LAUNCH_CK();
        STG_TRY(reduce_parts(h->st, N.part, NPART, N.dsum));
        STG_TRY(reduce_parts(h->st, N.part + NPART, NPART, N.dsum + 1));
        pm = N.dsum;
    }
    k_pack_target<<<nb(vox3(h->n)), TPB, 0, h->st>>>(g, h->n, N.s_e, N.s_z, N.sc, pm, F.m, N.tgt);
    STG_LAUNCH_CK();
    return STG_OK;
}

}  // namespace stg

namespace {
int net_check(stg_t* h) {
    if (!h) return stg::set_error("null handle"), STG_E_INVALID;
    if (!h->net) return stg::set_error("no network: call stg_net_init first"), STG_E_INVALID;
    return STG_OK;
}
}  // namespace

extern "C" {

int stg_net_init(stg_t* h, uint64_t seed) {
    if (!h) return stg::set_error("null handle"), STG_E_INVALID;
    if (!h->net) {
        h->net = new NetState();
        STG_TRY(stg::net_layout(*h->net, 16));
        if (int rc = stg::net_alloc_params(*h->net)) {
            stg::net_free(h);
            return rc;
        }
    }
    STG_TRY(stg::net_init_params(*h->net, h->st, seed));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_net_num_params(const stg_t* h, int64_t* count) {
    if (!h || !h->net || !count) return stg::set_error("no network or null argument"), STG_E_INVALID;
    *count = h->net->nparam;
    return STG_OK;
}

int stg_net_get_params(stg_t* h, float* out, int64_t count) {
    STG_TRY(net_check(h));
    NetState& N = *h->net;
    if (!out || count != N.nparam) return stg::set_error("stg_net_get_params: count %lld != %lld", (long long)count, N.nparam), STG_E_INVALID;
    STG_CK(cudaMemcpyAsync(out, N.p, sizeof(float) * N.nparam, cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_net_set_params(stg_t* h, const float* in, int64_t count) {
    STG_TRY(net_check(h));
    NetState& N = *h->net;
    if (!in || count != N.nparam) return stg::set_error("stg_net_set_params: count %lld != %lld", (long long)count, N.nparam), STG_E_INVALID;
    STG_CK(cudaMemcpyAsync(N.p, in, sizeof(float) * N.nparam, cudaMemcpyHostToDevice, h->st));
    N.kappa = in[N.kappa_off];
    STG_TRY(stg::reset_adam(N, h->st));
    STG_TRY(stg::refresh_working(N, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_net_forward_backward(stg_t* h, int n, const float* in, const float* target, float* out, float* grad, double* loss) {
    STG_TRY(net_check(h));
    NetState& N = *h->net;
    if (!in || !stg::net_grid_ok(n)) return stg::set_error("stg_net_forward_backward: n %d (needs n >= 8, n %% 4 == 0)", n), STG_E_INVALID;
    const bool train = target != nullptr;
    STG_TRY(stg::net_buffers(N, n, train));
    const long long V = (long long)n * n * n;
    std::vector<__nv_bfloat16> x((size_t)V * stg::IN_CH, __float2bfloat16(0.f));
    for (long long v = 0; v < V; v++)
        for (int c = 0; c < stg::IN_USED; c++) x[v * stg::IN_CH + c] = __float2bfloat16(in[v * stg::IN_USED + c]);
    STG_CK(cudaMemcpyAsync(N.in0, x.data(), sizeof(__nv_bfloat16) * x.size(), cudaMemcpyHostToDevice, h->st));
    STG_TRY(stg::net_forward(N, h->st, n));
    if (train) {
        STG_CK(cudaMemcpyAsync(N.tgt, target, sizeof(float) * V * stg::OUT_CH, cudaMemcpyHostToDevice, h->st));
        STG_TRY(stg::net_loss(N, h->st, n));
        STG_TRY(stg::net_backward(N, h->st, n));
        if (loss) STG_CK(cudaMemcpyAsync(loss, N.dloss, sizeof(double), cudaMemcpyDeviceToHost, h->st));
        if (grad) STG_CK(cudaMemcpyAsync(grad, N.g, sizeof(float) * N.nparam, cudaMemcpyDeviceToHost, h->st));
    }
    if (out) STG_CK(cudaMemcpyAsync(out, N.out, sizeof(float) * V * stg::OUT_CH, cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    return stg::tc_check(h->st);
}

int stg_net_adam_step(stg_t* h, double lr) {
    STG_TRY(net_check(h));
    STG_TRY(stg::net_adam(*h->net, h->st, lr));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_net_train(stg_t* h, int steps, double lr, uint64_t seed, float* losses) {
    STG_TRY(net_check(h));
    if (h->dim != 3) return stg::set_error("stg_net_train: 3D handles only"), STG_E_INVALID;
    if (!h->have_boundary || !h->have_penalty) return stg::set_error("stg_net_train: boundary and penalty (or density) first"), STG_E_INVALID;
    if (!stg::net_grid_ok(h->n)) return stg::set_error("stg_net_train: grid %d (needs n >= 8, n %% 4 == 0)", h->n), STG_E_INVALID;
    if (steps < 0) return stg::set_error("stg_net_train: steps < 0"), STG_E_INVALID;
    NetState& N = *h->net;
    STG_TRY(stg::ensure_setup(h, false));
    STG_TRY(stg::net_buffers(N, h->n, true));
    std::vector<double> dl(steps > 0 ? steps : 1);
    double* d_losses = nullptr;
    STG_TRY(stg::dalloc(&d_losses, dl.size()));
    int rc = STG_OK;
    for (int s = 0; s < steps && rc == STG_OK; s++) {
        const uint64_t sd = seed * 0x100000001B3ull + (uint64_t)s;
        if (N.kappa == 0.f) {
            // output scale: rms(e - z) / rms(r1) of the first pair
            const float one = 1.f;
            if ((rc = stg::cuda_ck(cudaMemcpyAsync(N.p + N.kappa_off, &one, sizeof(float), cudaMemcpyHostToDevice, h->st)))) break;
            if ((rc = stg::net_pair(h, N, sd))) break;
            float sc[2];
            double tsum = 0;
            if ((rc = stg::cuda_ck(cudaMemcpyAsync(sc, N.sc, sizeof(sc), cudaMemcpyDeviceToHost, h->st)))) break;
            std::vector<float> t((size_t)stg::vox3(h->n) * stg::OUT_CH);
            if ((rc = stg::cuda_ck(cudaMemcpyAsync(t.data(), N.tgt, sizeof(float) * t.size(), cudaMemcpyDeviceToHost, h->st)))) break;
            if ((rc = stg::cuda_ck(cudaStreamSynchronize(h->st)))) break;
            for (float q : t) tsum += (double)q * q;
            // tgt = (e - z) / sc[1] with sc[1] = rms(r1) at kappa 1
            const double k = std::sqrt(tsum / (double)t.size());
            N.kappa = k > 0 ? (float)k : 1.f;
            if ((rc = stg::cuda_ck(cudaMemcpyAsync(N.p + N.kappa_off, &N.kappa, sizeof(float), cudaMemcpyHostToDevice, h->st)))) break;
        }
        if ((rc = stg::net_pair(h, N, sd))) break;
        if ((rc = stg::net_forward(N, h->st, h->n))) break;
        if ((rc = stg::net_loss(N, h->st, h->n))) break;
        if ((rc = stg::net_backward(N, h->st, h->n))) break;
        if ((rc = stg::net_adam(N, h->st, lr))) break;
        if ((rc = stg::cuda_ck(cudaMemcpyAsync(d_losses + s, N.dloss, sizeof(double), cudaMemcpyDeviceToDevice, h->st)))) break;
    }
    if (rc == STG_OK && steps > 0) {
        rc = stg::cuda_ck(cudaMemcpyAsync(dl.data(), d_losses, sizeof(double) * steps, cudaMemcpyDeviceToHost, h->st));
        if (rc == STG_OK) rc = stg::cuda_ck(cudaStreamSynchronize(h->st));
        if (rc == STG_OK && losses)
            for (int s = 0; s < steps; s++) losses[s] = (float)dl[s];
    }
    cudaFree(d_losses);
    if (rc == STG_OK) rc = stg::tc_check(h->st);
    return rc;
}

}  // extern "C"
