// Kernels of the learned preconditioner (a 3D U-Net; no counterpart in the reference).
//
// Activations are channel-last BF16 arrays [voxel][ld] over an n^3 cell grid (voxel
// v = (i n + j) n + k), weights of a 3x3x3 convolution are BF16 [tap][C_out][C_in] with
// tap t = 9 (di+1) + 3 (dj+1) + (dk+1). Convolutions are implicit GEMMs on the tensor
// cores (mma.sync m16n8k16, BF16 inputs, FP32 accumulation):
//   forward          out[v][co] = act(bias[co] + sum_{t,ci} in[v + o_t][ci] W[t][co][ci]), zero padding;
//   backward data    the forward with the flipped, transposed weights Wf[t][ci][co] = W[26-t][co][ci];
//   backward weights dW[t][co][ci] += sum_v dy[v][co] x[v + o_t][ci] (FP32, per-warp partials
//                    over voxel chunks added with atomics), db[co] = sum_v dy[v][co].
// A warp owns 16 voxels (the M side) and all output channels (N = C_out <= 64).
#include <cuda_bf16.h>

#include "internal.cuh"

namespace stg {

namespace {

constexpr int WPB = 4;  // warps per block

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void vox(int n, int v, int& i, int& j, int& k) {
    k = v % n;
    j = (v / n) % n;
    i = v / (n * n);
}

// forward 3x3x3 convolution; CIN multiple of 16, COUT multiple of 8 (<= 64); F32: FP32
// output (used for gradients), else BF16
template <int COUT, bool F32>
__global__ void __launch_bounds__(32 * WPB) k_conv3_fwd(const __nv_bfloat16* __restrict__ in, int cin, int ldin,
                                                        const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias,
                                                        void* __restrict__ outp, int ldout, int n, int relu, int wtap) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gid = lane >> 2, tig = lane & 3;
    const int V = n * n * n;
    const int v0 = (blockIdx.x * WPB + warp) * 16;
    if (v0 >= V) return;
    const int vr0 = v0 + gid, vr1 = v0 + gid + 8;
    const bool in0 = vr0 < V, in1 = vr1 < V;  // rows past the grid (V not a multiple of 16) stay zero
    int i0, j0, k0, i1, j1, k1;
    vox(n, vr0, i0, j0, k0);
    vox(n, vr1, i1, j1, k1);
    constexpr int NF = COUT / 8;
    float acc[NF][4];
#pragma unroll
    for (int f = 0; f < NF; f++) acc[f][0] = acc[f][1] = acc[f][2] = acc[f][3] = 0.f;
    for (int t = 0; t < 27; t++) {
        const int di = t / 9 - 1, dj = (t / 3) % 3 - 1, dk = t % 3 - 1;
        const int a0i = i0 + di, a0j = j0 + dj, a0k = k0 + dk, a1i = i1 + di, a1j = j1 + dj, a1k = k1 + dk;
        const bool ok0 = in0 && a0i >= 0 && a0j >= 0 && a0k >= 0 && a0i < n && a0j < n && a0k < n;
        const bool ok1 = in1 && a1i >= 0 && a1j >= 0 && a1k >= 0 && a1i < n && a1j < n && a1k < n;
        const __nv_bfloat16* p0 = in + (size_t)(ok0 ? (a0i * n + a0j) * n + a0k : 0) * ldin;
        const __nv_bfloat16* p1 = in + (size_t)(ok1 ? (a1i * n + a1j) * n + a1k : 0) * ldin;
        const __nv_bfloat16* wt = w + (size_t)t * wtap;
        for (int c0 = 0; c0 < cin; c0 += 16) {
            uint32_t a[4];
            a[0] = ok0 ? ld_pair(p0 + c0 + 2 * tig) : 0u;
            a[1] = ok1 ? ld_pair(p1 + c0 + 2 * tig) : 0u;
            a[2] = ok0 ? ld_pair(p0 + c0 + 8 + 2 * tig) : 0u;
            a[3] = ok1 ? ld_pair(p1 + c0 + 8 + 2 * tig) : 0u;
#pragma unroll
            for (int f = 0; f < NF; f++) {
                const __nv_bfloat16* wp = wt + (size_t)(f * 8 + gid) * cin + c0 + 2 * tig;
                uint32_t b[2] = {ld_pair(wp), ld_pair(wp + 8)};
                mma16816(acc[f], a, b);
            }
        }
    }
#pragma unroll
    for (int f = 0; f < NF; f++) {
        const int co = f * 8 + 2 * tig;
        const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
        float y00 = acc[f][0] + b0, y01 = acc[f][1] + b1, y10 = acc[f][2] + b0, y11 = acc[f][3] + b1;
        if (relu) {
            y00 = fmaxf(y00, 0.f);
            y01 = fmaxf(y01, 0.f);
            y10 = fmaxf(y10, 0.f);
            y11 = fmaxf(y11, 0.f);
        }
        if (F32) {
            float* out = static_cast<float*>(outp);
            if (in0) *reinterpret_cast<float2*>(out + (size_t)vr0 * ldout + co) = make_float2(y00, y01);
            if (in1) *reinterpret_cast<float2*>(out + (size_t)vr1 * ldout + co) = make_float2(y10, y11);
        } else {
            __nv_bfloat16* out = static_cast<__nv_bfloat16*>(outp);
            if (in0) *reinterpret_cast<__nv_bfloat162*>(out + (size_t)vr0 * ldout + co) = __floats2bfloat162_rn(y00, y01);
            if (in1) *reinterpret_cast<__nv_bfloat162*>(out + (size_t)vr1 * ldout + co) = __floats2bfloat162_rn(y10, y11);
        }
    }
}

// dW[t][co][ci] += sum over a voxel chunk of dy[v][co] x[v + o_t][ci]. One warp: one tap,
// one 16-row block of output channels, all CIN (<= 64) input channels, one voxel chunk.
template <int CIN>
__global__ void __launch_bounds__(32 * WPB) k_conv3_dw(const __nv_bfloat16* __restrict__ x, int ldx, const __nv_bfloat16* __restrict__ dy,
                                                       int cout, int lddy, float* __restrict__ dw, int n, int chunk) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gid = lane >> 2, tig = lane & 3;
    const int V = n * n * n;
    const int t = blockIdx.y, co0 = blockIdx.z * 16;
    const int vbeg = (blockIdx.x * WPB + warp) * chunk;
    if (vbeg >= V) return;
    const int vend = min(vbeg + chunk, V);
    const int di = t / 9 - 1, dj = (t / 3) % 3 - 1, dk = t % 3 - 1;
    constexpr int NF = CIN / 8;
    float acc[NF][4];
#pragma unroll
    for (int f = 0; f < NF; f++) acc[f][0] = acc[f][1] = acc[f][2] = acc[f][3] = 0.f;
    const __nv_bfloat16 z = __float2bfloat16(0.f);
    for (int vb = vbeg; vb < vend; vb += 16) {
        // A (16 co x 16 v): rows co0 + gid (+8), columns v = vb + 2 tig (+1, +8, +9)
        // B (16 v x 8 ci):  rows v = vb + 2 tig (+1, +8, +9), column ci = f*8 + gid
        const int vs[4] = {vb + 2 * tig, vb + 2 * tig + 1, vb + 2 * tig + 8, vb + 2 * tig + 9};
        int nb[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int i, j, k;
            vox(n, vs[q], i, j, k);
            i += di;
            j += dj;
            k += dk;
            nb[q] = (vs[q] < vend && i >= 0 && j >= 0 && k >= 0 && i < n && j < n && k < n) ? (i * n + j) * n + k : -1;
        }
        __nv_bfloat16 av[2][4];
#pragma unroll
        for (int r = 0; r < 2; r++)
#pragma unroll
            for (int q = 0; q < 4; q++) av[r][q] = vs[q] < vend ? dy[(size_t)vs[q] * lddy + co0 + gid + 8 * r] : z;
        uint32_t a[4] = {pack2(av[0][0], av[0][1]), pack2(av[1][0], av[1][1]), pack2(av[0][2], av[0][3]),
                         pack2(av[1][2], av[1][3])};
#pragma unroll
        for (int f = 0; f < NF; f++) {
            const int ci = f * 8 + gid;
            __nv_bfloat16 bv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) bv[q] = nb[q] >= 0 ? x[(size_t)nb[q] * ldx + ci] : z;
            uint32_t b[2] = {pack2(bv[0], bv[1]), pack2(bv[2], bv[3])};
            mma16816(acc[f], a, b);
        }
    }
    // D (16 co x 8 ci): rows co0 + gid (+8), columns f*8 + 2 tig (+1)
#pragma unroll
    for (int f = 0; f < NF; f++) {
        const int ci = f * 8 + 2 * tig;
        float* d0 = dw + ((size_t)t * cout + co0 + gid) * CIN + ci;
        float* d1 = dw + ((size_t)t * cout + co0 + gid + 8) * CIN + ci;
        atomicAdd(d0, acc[f][0]);
        atomicAdd(d0 + 1, acc[f][1]);
        atomicAdd(d1, acc[f][2]);
        atomicAdd(d1 + 1, acc[f][3]);
    }
}

// db[co] += sum_v dy[v][co] (one block per 32 channels x voxel chunk)
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ dy, int cout, int lddy, float* __restrict__ db, int V, int chunk) {
    const int co = blockIdx.y * 32 + (threadIdx.x & 31);
    if (co >= cout) return;
    const int vbeg = blockIdx.x * chunk, vend = min(vbeg + chunk, V);
    float s = 0.f;
    for (int v = vbeg + (threadIdx.x >> 5); v < vend; v += blockDim.x >> 5) s += __bfloat162float(dy[(size_t)v * lddy + co]);
    atomicAdd(db + co, s);
}

// Wf[t][ci][co] = W[26 - t][co][ci]  (BF16 working weights for the backward-data pass)
__global__ void k_flip_weights(const __nv_bfloat16* __restrict__ w, int cout, int cin, __nv_bfloat16* __restrict__ wf) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 27 * cout * cin) return;
    const int ci = e % cin, co = (e / cin) % cout, t = e / (cin * cout);
    wf[((size_t)(26 - t) * cin + ci) * cout + co] = w[e];
}

template <int C>
void launch_fwd(int nblk, cudaStream_t st, const __nv_bfloat16* in, int cin, int ldin, const __nv_bfloat16* w, const float* bias,
                void* out, int ldout, int n, int relu, bool f32, int wtap) {
    if (f32)
        k_conv3_fwd<C, true><<<nblk, 32 * WPB, 0, st>>>(in, cin, ldin, w, bias, out, ldout, n, relu, wtap);
    else
        k_conv3_fwd<C, false><<<nblk, 32 * WPB, 0, st>>>(in, cin, ldin, w, bias, out, ldout, n, relu, wtap);
}
template <int C>
void launch_dw(dim3 grid, cudaStream_t st, const __nv_bfloat16* x, int ldx, const __nv_bfloat16* dy, int cout, int lddy, float* dw,
               int n, int chunk) {
    k_conv3_dw<C><<<grid, 32 * WPB, 0, st>>>(x, ldx, dy, cout, lddy, dw, n, chunk);
}

}  // namespace

int conv3_forward(cudaStream_t st, const __nv_bfloat16* in, int cin, int ldin, const __nv_bfloat16* w, const float* bias,
                  void* out, int cout, int ldout, int n, int relu, bool f32_out, int wtap) {
    // wtap: elements between taps of w (0: cout * cin, the dense layout; larger when w is a
    // block of output channels of a wider weight tensor)
    if (wtap == 0) wtap = cout * cin;
    if (n < 1 || cin < 16 || cin % 16 || cout < 8 || cout % 8 || cout > 64 || ldin < cin || ldout < cout || ldin % 2 || ldout % 2 ||
        wtap < cout * cin) {
        set_error("conv3_forward: unsupported shape (cin %d, cout %d, ld %d/%d, n %d)", cin, cout, ldin, ldout, n);
        return STG_E_INVALID;
    }
    const long long V = (long long)n * n * n;
    const int nblk = (int)((V / 16 + WPB - 1) / WPB);
    switch (cout) {
        case 8: launch_fwd<8>(nblk, st, in, cin, ldin, w, bias, out, ldout, n, relu, f32_out, wtap); break;
        case 16: launch_fwd<16>(nblk, st, in, cin, ldin, w, bias, out, ldout, n, relu, f32_out, wtap); break;
        case 24: launch_fwd<24>(nblk, st, in, cin, ldin, w, bias, out, ldout, n, relu, f32_out, wtap); break;
        case 32: launch_fwd<32>(nblk, st, in, cin, ldin, w, bias, out, ldout, n, relu, f32_out, wtap); break;
        case 40: launch_fwd<40>(nblk, st, in, cin, ldin, w, bias, out, ldout, n, relu, f32_out, wtap); break;
        case 48: launch_fwd<48>(nblk, st, in, cin, ldin, w, bias, out, ldout, n, relu, f32_out, wtap); break;
        case 56: launch_fwd<56>(nblk, st, in, cin, ldin, w, bias, out, ldout, n, relu, f32_out, wtap); break;
        default: launch_fwd<64>(nblk, st, in, cin, ldin, w, bias, out, ldout, n, relu, f32_out, wtap); break;
    }
    STG_LAUNCH_CK();
    return STG_OK;
}

int conv3_backward_weights(cudaStream_t st, const __nv_bfloat16* x, int cin, int ldx, const __nv_bfloat16* dy, int cout, int lddy,
                           float* dw, float* db, int n) {
    if (n < 1 || cin % 8 || cin < 8 || (cin > 64 && cin != 96) || cout % 16 || cout < 16 || ldx % 2 || lddy % 2) {
        set_error("conv3_backward_weights: unsupported shape (cin %d, cout %d)", cin, cout);
        return STG_E_INVALID;
    }
    const int V = n * n * n;
    const int chunk = 1024;  // voxels per warp
    const int nchunk = (V + chunk - 1) / chunk;
    dim3 grid((nchunk + WPB - 1) / WPB, 27, cout / 16);
    switch (cin) {
        case 8: launch_dw<8>(grid, st, x, ldx, dy, cout, lddy, dw, n, chunk); break;
        case 16: launch_dw<16>(grid, st, x, ldx, dy, cout, lddy, dw, n, chunk); break;
        case 24: launch_dw<24>(grid, st, x, ldx, dy, cout, lddy, dw, n, chunk); break;
        case 32: launch_dw<32>(grid, st, x, ldx, dy, cout, lddy, dw, n, chunk); break;
        case 40: launch_dw<40>(grid, st, x, ldx, dy, cout, lddy, dw, n, chunk); break;
        case 48: launch_dw<48>(grid, st, x, ldx, dy, cout, lddy, dw, n, chunk); break;
        case 56: launch_dw<56>(grid, st, x, ldx, dy, cout, lddy, dw, n, chunk); break;
        case 64: launch_dw<64>(grid, st, x, ldx, dy, cout, lddy, dw, n, chunk); break;
        default: launch_dw<96>(grid, st, x, ldx, dy, cout, lddy, dw, n, chunk); break;
    }
    STG_LAUNCH_CK();
    if (db) {
        const int bchunk = 4096;
        dim3 g2((V + bchunk - 1) / bchunk, (cout + 31) / 32);
        k_bias_grad<<<g2, 256, 0, st>>>(dy, cout, lddy, db, V, bchunk);
        STG_LAUNCH_CK();
    }
    return STG_OK;
}

int conv3_flip_weights(cudaStream_t st, const __nv_bfloat16* w, int cout, int cin, __nv_bfloat16* wf) {
    const int e = 27 * cout * cin;
    k_flip_weights<<<(e + 255) / 256, 256, 0, st>>>(w, cout, cin, wf);
    STG_LAUNCH_CK();
    return STG_OK;
}

}  // namespace stg
