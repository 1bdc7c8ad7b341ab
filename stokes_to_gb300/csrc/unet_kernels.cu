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

#include <algorithm>

#include "internal.cuh"

namespace stg {

extern bool g_conv_tc;

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

// ---------------------------------------------------------------- tcgen05 forward
// The same convolution on the 5th-generation tensor cores, as an implicit GEMM (M voxels,
// N = C_out, K = 27 taps x C_in). A CTA owns J consecutive j-lines (all k) of P
// consecutive i-planes and marches along i. For each 16-channel slice of the input it
// streams the P + 2 halo planes ((J+2) lines x (n+2) cells each) through a ring of five
// shared-memory slots, as K-major core matrices without swizzle: in a slot, row
// r = jj (n+2) + kk holds the 16 bytes of channels [8g, 8g+8) at (g R + r) 16,
// R = (J+2)(n+2). In this layout a tap (di,dj,dk) is a uniform row shift within the slot
// of plane i + di, so one shared-memory descriptor per tap and M-tile addresses the A
// operand (128 consecutive rows; rows on halo columns are computed and discarded). The
// slice's weights sit beside the ring as [g][tap][C_out] rows. One thread issues
// tcgen05.mma (M 128, N C_out, K 16, BF16 in, FP32 accumulators in tensor memory, one
// accumulator block per plane and M-tile) for plane i while the copies of plane i + 3 and
// the MMAs of plane i - 1 are in flight, and commits to one of two mbarriers; at the end
// the four warps read the accumulators with tcgen05.ld for the bias / ReLU / store
// epilogue.
namespace tc {

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, no swizzle; lbo = byte stride between core
// matrices along K, sbo = byte stride between 8-row core matrices along M/N
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int nn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(nn >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void cp16(uint32_t dst, const void* src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

// waits for the mbarrier phase of the given parity; false after about a second
__device__ __forceinline__ bool wait_parity(uint32_t bar, uint32_t parity) {
    uint64_t t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        uint64_t t1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        if (t1 - t0 > 1000000000ull) return false;
    }
}

__device__ __forceinline__ void ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

}  // namespace tc

// Tile plan of the tcgen05 kernel for an n^3 grid: J lines and P planes per CTA, T
// M-tiles per plane, tensor-memory columns and dynamic shared memory.
struct TcPlan {
    int J = 0, T = 0, P = 0, ncols = 0;
    size_t smem = 0;
};

constexpr int TC_RING = 5;

template <int COUT, bool F32>
__global__ void __launch_bounds__(128) k_conv3_tc(const __nv_bfloat16* __restrict__ in, int cin, int ldin,
                                                  const __nv_bfloat16* __restrict__ w, int wtap, const float* __restrict__ bias,
                                                  void* __restrict__ outp, int ldout, int n, int relu, int J, int T, int P,
                                                  int ncols, int* __restrict__ err) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int Hk = n + 2, R = (J + 2) * Hk;
    const uint32_t slot_bytes = 32u * (uint32_t)R;
    uint8_t* sB = smem + (size_t)TC_RING * slot_bytes;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sB + 864 * COUT);  // two mbarriers: commits alternate
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int i0 = blockIdx.x * P, j0 = blockIdx.y * J;
    const int np = min(P, n - i0);
    const uint32_t bar_a = tc::saddr(bar);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tc::saddr(tslot)), "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_a) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_a + 8u) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tbase = *tslot;
    const uint32_t a0 = tc::saddr(smem), b0 = tc::saddr(sB);
    const uint32_t lbo_a = 16u * (uint32_t)R, lbo_b = 432u * COUT;
    constexpr uint32_t ID = tc::idesc_bf16(128, COUT);
    const int rlast = (J + 1) * Hk - 2 - 127;
    // commit c goes to mbarrier c & 1 and completes its phase (c >> 1) & 1; a wait is only
    // ever made for the latest commit of its barrier, so the parity is unambiguous
    uint32_t ncommit = 0;
    auto commit_done = [&](uint32_t c) { return tc::wait_parity(bar_a + 8u * (c & 1u), (c >> 1) & 1u); };
    int bad = 0;

    // halo plane hp (i = i0 - 1 + hp) of channel slice c0 into ring slot hp % 4: line by
    // line, consecutive threads on consecutive 16-byte pieces
    auto load_plane = [&](int hp, int c0) {
        const int gi = i0 - 1 + hp;
        const uint32_t sbase = a0 + (uint32_t)(hp % TC_RING) * slot_bytes;
        for (int jj = 0; jj < J + 2; jj++) {
            const int gj = j0 - 1 + jj;
            const bool line_ok = gi >= 0 && gi < n && gj >= 0 && gj < n;
            const __nv_bfloat16* lsrc = line_ok ? in + (size_t)(gi * n + gj) * n * ldin + c0 : in;
            const uint32_t dst = sbase + 16u * (uint32_t)(jj * Hk);
            for (int x = tid; x < 2 * Hk; x += 128) {
                const int kk = x >> 1, g = x & 1;
                const bool ok = line_ok && kk >= 1 && kk <= n;
                tc::cp16(dst + 16u * (uint32_t)(g * R + kk), ok ? lsrc + (size_t)(kk - 1) * ldin + 8 * g : in, ok ? 16 : 0);
            }
        }
    };
    const int nchunk = cin / 16;
    for (int ch = 0; ch < nchunk && !bad; ch++) {
        const int c0 = ch * 16;
        // every MMA issued so far reads the ring or the weights: wait before refilling them
        if (ncommit) {
            bad = __syncthreads_or(!(commit_done(ncommit - 1) && (ncommit < 2 || commit_done(ncommit - 2))));
            if (bad) break;
        }
        for (int e = tid; e < 54 * COUT; e += 128) {
            const int g = e / (27 * COUT), rem = e - g * 27 * COUT, t = rem / COUT, co = rem - t * COUT;
            tc::cp16(b0 + 16u * e, w + (size_t)t * wtap + (size_t)co * cin + c0 + 8 * g, 16);
        }
        for (int hp = 0; hp < 3; hp++) {
            load_plane(hp, c0);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
        for (int ip = 0; ip < np; ip++) {
            // halo plane ip + 3 takes the slot of plane ip - 2, which output planes ip - 3
            // and ip - 2 read: wait for the commit of ip - 2 (output ip - 1 may still run)
            if (ip >= 2) {
                bad = __syncthreads_or(!commit_done(ncommit - 2));
                if (bad) break;
            }
            if (ip + 3 <= np + 1) load_plane(ip + 3, c0);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // halo planes <= ip + 2 have landed
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            __syncthreads();
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                for (int t = 0; t < 27; t++) {
                    const int di = t / 9 - 1, dj = (t / 3) % 3 - 1, dk = t % 3 - 1;
                    const uint64_t bd = tc::sdesc(b0 + 16u * (uint32_t)(t * COUT), lbo_b, 128);
                    const uint32_t sb = a0 + (uint32_t)((ip + 1 + di) % TC_RING) * slot_bytes;
                    for (int q = 0; q < T; q++) {
                        const int r0 = q < T - 1 ? Hk + 1 + 128 * q : rlast;
                        const uint32_t row = (uint32_t)(r0 + dj * Hk + dk);
                        tc::mma(tbase + (uint32_t)((ip * T + q) * COUT), tc::sdesc(sb + 16u * row, lbo_a, 128), bd, ID,
                                (ch > 0 || t > 0) ? 1u : 0u);
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 bar_a + 8u * (ncommit & 1u))
                             : "memory");
            }
            ncommit++;
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if (!bad && ncommit) bad = __syncthreads_or(!(commit_done(ncommit - 1) && (ncommit < 2 || commit_done(ncommit - 2))));
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (!bad) {
        for (int ip = 0; ip < np; ip++) {
            for (int q = 0; q < T; q++) {
                const int r = (q < T - 1 ? Hk + 1 + 128 * q : rlast) + warp * 32 + lane;
                const int jj = r / Hk, kk = r - jj * Hk;
                const int gj = j0 - 1 + jj;
                const bool valid = jj >= 1 && jj <= J && kk >= 1 && kk <= n && gj < n;
                const size_t v = ((size_t)(i0 + ip) * n + gj) * n + (kk - 1);
#pragma unroll
                for (int cb = 0; cb < COUT; cb += 16) {
                    uint32_t x[16];
                    tc::ld16(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)((ip * T + q) * COUT + cb), x);
                    if (valid) {
                        float y[16];
#pragma unroll
                        for (int u = 0; u < 16; u++) {
                            y[u] = __uint_as_float(x[u]) + (bias ? bias[cb + u] : 0.f);
                            if (relu) y[u] = fmaxf(y[u], 0.f);
                        }
                        if (F32) {
                            float4* o = reinterpret_cast<float4*>(static_cast<float*>(outp) + v * ldout + cb);
#pragma unroll
                            for (int u = 0; u < 4; u++) o[u] = make_float4(y[4 * u], y[4 * u + 1], y[4 * u + 2], y[4 * u + 3]);
                        } else {
                            __align__(16) __nv_bfloat162 hh[8];
#pragma unroll
                            for (int u = 0; u < 8; u++) hh[u] = __floats2bfloat162_rn(y[2 * u], y[2 * u + 1]);
                            uint4* o = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(outp) + v * ldout + cb);
                            o[0] = reinterpret_cast<const uint4*>(hh)[0];
                            o[1] = reinterpret_cast<const uint4*>(hh)[1];
                        }
                    }
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(ncols) : "memory");
}

constexpr size_t TC_SMEM_MAX = 227 * 1024;
constexpr size_t TC_SMEM_TWO = 110 * 1024;  // at most this much: two CTAs per SM
// requests at least this much so that no more than two (tier 0) or one (tier 1) CTAs share
// an SM's 512 tensor-memory columns (an SM has 228 KB of shared memory, 1 KB kept per CTA)
constexpr size_t TC_FLOOR_TWO = 78 * 1024, TC_FLOOR_ONE = 118 * 1024;

// J with the most useful rows per M-tile row, then as many planes per CTA as the tensor
// memory holds (256 columns with two CTAs per SM, 512 with one); J = 0 when no plan fits
// (small grids use the mma.sync kernel)
TcPlan tc_plan(int n, int cout) {
    TcPlan best;
    for (int tier = 0; tier < 2 && !best.J; tier++) {
        const size_t budget = tier == 0 ? TC_SMEM_TWO : TC_SMEM_MAX;
        const int max_cols = tier == 0 ? 256 : 512;
        double best_eff = 0;
        for (int J = 1; J <= n; J++) {
            const int Hk = n + 2, rows = J * Hk - 2;
            if (rows < 128) continue;
            const int T = (rows + 127) / 128;
            const size_t smem = (size_t)TC_RING * 32 * (J + 2) * Hk + 864 * (size_t)cout + 32;
            if (smem > budget || T * cout > max_cols) break;
            const double eff = (double)J * n / (128.0 * T);
            if (eff > best_eff + 1e-9) {
                best_eff = eff;
                best.J = J;
                best.T = T;
                best.P = std::min(n, max_cols / (T * cout));
                // one CTA per SM in the second tier: ask for more than half the SM's memory
                best.smem = std::max(smem, tier == 0 ? TC_FLOOR_TWO : TC_FLOOR_ONE);
            }
        }
    }
    if (best.J) {
        int c = 32;
        while (c < best.P * best.T * cout) c <<= 1;
        best.ncols = c;
    }
    return best;
}

template <int C, bool F32>
int launch_tc(const TcPlan& P, cudaStream_t st, const __nv_bfloat16* in, int cin, int ldin, const __nv_bfloat16* w, int wtap,
              const float* bias, void* out, int ldout, int n, int relu, int* err) {
    static bool attr[MAX_DEVICES] = {};
    const int dev = device_slot();
    if (dev >= 0 && !attr[dev]) {
        STG_CK(cudaFuncSetAttribute(k_conv3_tc<C, F32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM_MAX));
        attr[dev] = true;
    }
    dim3 grid((n + P.P - 1) / P.P, (n + P.J - 1) / P.J);
    k_conv3_tc<C, F32><<<grid, 128, P.smem, st>>>(in, cin, ldin, w, wtap, bias, out, ldout, n, relu, P.J, P.T, P.P, P.ncols, err);
    return STG_OK;
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

// tensor-core convolutions on (default) or the mma.sync kernel for every shape; the
// error flag of the tcgen05 kernel's bounded waits, per device (0 = no timeout)
bool g_conv_tc = true;
static int* g_tc_err[MAX_DEVICES] = {};

int conv3_tc_status(cudaStream_t st, int* timed_out) {
    *timed_out = 0;
    const int dev = device_slot();
    if (dev < 0 || !g_tc_err[dev]) return STG_OK;
    STG_CK(cudaMemcpyAsync(timed_out, g_tc_err[dev], sizeof(int), cudaMemcpyDeviceToHost, st));
    STG_CK(cudaStreamSynchronize(st));
    return STG_OK;
}

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
    // tensor-core path: C_out a multiple of 16, 16-byte aligned rows and weight slices
    if (g_conv_tc && cout % 16 == 0 && ldin % 8 == 0 && wtap % 8 == 0 && ((uintptr_t)in & 15) == 0 && ((uintptr_t)w & 15) == 0 &&
        ((uintptr_t)out & 15) == 0 && ldout % 8 == 0) {
        const TcPlan P = tc_plan(n, cout);
        const int dev = device_slot();
        if (P.J && dev >= 0) {
            if (!g_tc_err[dev]) {
                STG_CK(cudaMalloc((void**)&g_tc_err[dev], sizeof(int)));
                STG_CK(cudaMemset(g_tc_err[dev], 0, sizeof(int)));
            }
            int* const err = g_tc_err[dev];
            int rc = STG_OK;
            switch (cout) {
                case 16: rc = f32_out ? launch_tc<16, true>(P, st, in, cin, ldin, w, wtap, bias, out, ldout, n, relu, err)
                                      : launch_tc<16, false>(P, st, in, cin, ldin, w, wtap, bias, out, ldout, n, relu, err); break;
                case 32: rc = f32_out ? launch_tc<32, true>(P, st, in, cin, ldin, w, wtap, bias, out, ldout, n, relu, err)
                                      : launch_tc<32, false>(P, st, in, cin, ldin, w, wtap, bias, out, ldout, n, relu, err); break;
                case 48: rc = f32_out ? launch_tc<48, true>(P, st, in, cin, ldin, w, wtap, bias, out, ldout, n, relu, err)
                                      : launch_tc<48, false>(P, st, in, cin, ldin, w, wtap, bias, out, ldout, n, relu, err); break;
                default: rc = f32_out ? launch_tc<64, true>(P, st, in, cin, ldin, w, wtap, bias, out, ldout, n, relu, err)
                                      : launch_tc<64, false>(P, st, in, cin, ldin, w, wtap, bias, out, ldout, n, relu, err); break;
            }
            STG_TRY(rc);
            STG_LAUNCH_CK();
            return STG_OK;
        }
    }
    const int nblk = (int)(((V + 15) / 16 + WPB - 1) / WPB);
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
